// CTA-wide dense k x k routines on shared-memory matrices (row-major,
// leading dimension lda).  Every thread of the block must call them; they
// synchronise internally and return block-uniform results.
//
// These replace the Eigen calls of ETKF.hpp:150-159 and LETKF.hpp:215-224:
//   inverse()        -> Cholesky factor + triangular inverse (A is SPD)
//   llt().matrixL()  -> cta_cholesky
// and, for the symmetric square root of the Hunt et al. (2007) transform,
// a parallel two-sided Jacobi eigen-solver: round-robin (circle method)
// ordering, k/2 disjoint rotations per round, rows then columns, with the
// rotated 2 x 2 block written in closed form.
#pragma once

#include <cuda_runtime.h>

namespace mg {

template <typename T>
__device__ __forceinline__ T dsqrt(T x);
template <>
__device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }

// In-place lower Cholesky factor (upper triangle zeroed).  Returns false if
// a pivot is not positive and finite.
template <typename T>
__device__ bool cta_cholesky(T* A, int k, int lda, int* sflag) {
  if (threadIdx.x == 0) *sflag = 1;
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    if (threadIdx.x == 0) {
      const T d = A[j * lda + j];
      if (!(d > T(0)) || !(d < T(3.0e38))) *sflag = 0;
      A[j * lda + j] = dsqrt<T>(d > T(0) ? d : T(1));
    }
    __syncthreads();
    const T ljj = A[j * lda + j];
    for (int i = j + 1 + threadIdx.x; i < k; i += blockDim.x) A[i * lda + j] = A[i * lda + j] / ljj;
    __syncthreads();
    const int m = k - j - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = j + 1 + e / m, l = j + 1 + e % m;
      if (l <= i) A[i * lda + l] -= A[i * lda + j] * A[l * lda + j];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e / k, l = e % k;
    if (l > i) A[i * lda + l] = T(0);
  }
  __syncthreads();
  return *sflag != 0;
}

// Li = L^-1 for lower-triangular L (row by row; columns in parallel).
template <typename T>
__device__ void cta_lower_inverse(const T* L, T* Li, int k, int lda) {
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) Li[(e / k) * lda + e % k] = T(0);
  __syncthreads();
  for (int i = 0; i < k; ++i) {
    for (int c = threadIdx.x; c <= i; c += blockDim.x) {
      T s = (c == i) ? T(1) : T(0);
      for (int m = c; m < i; ++m) s -= L[i * lda + m] * Li[m * lda + c];
      Li[i * lda + c] = s / L[i * lda + i];
    }
    __syncthreads();
  }
}

// Ainv = Li^T Li (the inverse of A = L L^T), full symmetric matrix.
template <typename T>
__device__ void cta_gram_of_lower(const T* Li, T* Ainv, int k, int lda) {
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e / k, j = e % k;
    const int m0 = i > j ? i : j;
    T s = T(0);
    for (int m = m0; m < k; ++m) s += Li[m * lda + i] * Li[m * lda + j];
    Ainv[i * lda + j] = s;
  }
  __syncthreads();
}

// Parallel cyclic Jacobi: A (kp x kp, kp even, symmetric) is diagonalised in
// place, V receives the eigenvectors as columns (A_in = V diag(A_out) V^T).
// Round-robin (circle method) ordering: each round rotates kp/2 disjoint
// pairs at once.  Because the pairs partition the indices, J^T A J splits
// into independent 2 x 2 blocks (rows of pair b) x (columns of pair c): one
// thread updates a whole block from its four inputs, so a round is one
// rotation phase and one block phase (two barriers).  Diagonal blocks are
// written in closed form (a_pp - t a_pq, a_qq + t a_pq, 0).  A rotation is
// skipped when |a_pq| <= tol sqrt(|a_pp a_qq|).  init_v = false continues
// from the basis already in V.  Scratch: rot (4 per pair), pair (2 per pair).
// Returns the sweeps run (max_sweeps + 1 if it had not converged).
template <typename T>
__device__ int cta_jacobi(T* A, T* V, int kp, int lda, T tol, int max_sweeps, T* rot, int* pair,
                          bool init_v = true) {
  if (init_v) {
    for (int e = threadIdx.x; e < kp * kp; e += blockDim.x) {
      const int i = e / kp, j = e % kp;
      V[i * lda + j] = (i == j) ? T(1) : T(0);
    }
  }
  __syncthreads();
  const int h = kp >> 1, m = kp - 1;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int rotated = 0;
    for (int r = 0; r < m; ++r) {
      for (int i = threadIdx.x; i < h; i += blockDim.x) {
        int p, q;
        if (i == 0) {
          p = r;
          q = m;
        } else {
          p = (r + i) % m;
          q = (r - i + m) % m;
        }
        if (p > q) { const int t = p; p = q; q = t; }
        const T app = A[p * lda + p], aqq = A[q * lda + q], apq = A[p * lda + q];
        T c = T(1), s = T(0), t = T(0);
        // Threshold test in the working precision (no FP64 on the FP32 path).
        if (apq != T(0) && fabs(apq) > tol * dsqrt<T>(fabs(app) * fabs(aqq))) {
          const T theta = (aqq - app) / (T(2) * apq);
          t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + dsqrt<T>(theta * theta + T(1)));
          c = T(1) / dsqrt<T>(t * t + T(1));
          s = t * c;
          rotated = 1;
        }
        pair[2 * i] = p;
        pair[2 * i + 1] = q;
        rot[4 * i + 0] = c;
        rot[4 * i + 1] = s;
        rot[4 * i + 2] = app - t * apq;  // new a_pp
        rot[4 * i + 3] = aqq + t * apq;  // new a_qq
      }
      __syncthreads();
      // 2 x 2 blocks of A: rows (p_b, q_b) x columns (p_c, q_c).
      for (int e = threadIdx.x; e < h * h; e += blockDim.x) {
        const int b = e / h, c2 = e - b * h;
        const T sb = rot[4 * b + 1], sc = rot[4 * c2 + 1];
        if (sb == T(0) && sc == T(0)) continue;
        const int pb = pair[2 * b], qb = pair[2 * b + 1];
        const int pc = pair[2 * c2], qc = pair[2 * c2 + 1];
        if (b == c2) {
          A[pb * lda + pb] = rot[4 * b + 2];
          A[qb * lda + qb] = rot[4 * b + 3];
          A[pb * lda + qb] = T(0);
          A[qb * lda + pb] = T(0);
          continue;
        }
        const T cb = rot[4 * b + 0], cc = rot[4 * c2 + 0];
        const T a00 = A[pb * lda + pc], a01 = A[pb * lda + qc];
        const T a10 = A[qb * lda + pc], a11 = A[qb * lda + qc];
        const T m00 = cb * a00 - sb * a10, m01 = cb * a01 - sb * a11;  // rows: J_b^T A
        const T m10 = sb * a00 + cb * a10, m11 = sb * a01 + cb * a11;
        A[pb * lda + pc] = cc * m00 - sc * m01;  // columns: (.) J_c
        A[pb * lda + qc] = sc * m00 + cc * m01;
        A[qb * lda + pc] = cc * m10 - sc * m11;
        A[qb * lda + qc] = sc * m10 + cc * m11;
      }
      // Columns (p_c, q_c) of V.
      for (int e = threadIdx.x; e < kp * h; e += blockDim.x) {
        const int row = e / h, c2 = e - row * h;
        const T sc = rot[4 * c2 + 1];
        if (sc == T(0)) continue;
        const T cc = rot[4 * c2 + 0];
        const int pc = pair[2 * c2], qc = pair[2 * c2 + 1];
        const T va = V[row * lda + pc], vb = V[row * lda + qc];
        V[row * lda + pc] = cc * va - sc * vb;
        V[row * lda + qc] = sc * va + cc * vb;
      }
      __syncthreads();
    }
    if (!__syncthreads_or(rotated)) break;
  }
  return sweep + 1;
}

// cta_jacobi with compile-time bounds (KMAX >= kp, NT threads): the 2 x 2
// blocks and V column pairs a thread updates are the same in every round, so
// their (b, c) coordinates are computed once instead of by an integer
// division per element per round.  Same ordering, rotations and results as
// cta_jacobi.
template <typename T, int KMAX, int NT>
__device__ int cta_jacobi_fast(T* A, T* V, int kp, int lda, T tol, int max_sweeps, T* rot, int* pair,
                               bool init_v = true) {
  constexpr int HMAX = KMAX / 2;
  constexpr int NB = (HMAX * HMAX + NT - 1) / NT;  // A blocks per thread
  constexpr int NV = (KMAX * HMAX + NT - 1) / NT;  // V column pairs per thread
  const int tid = threadIdx.x;
  const int h = kp >> 1, m = kp - 1;
  if (init_v) {
    for (int e = tid; e < kp * kp; e += NT) {
      const int i = e / kp, j = e % kp;
      V[i * lda + j] = (i == j) ? T(1) : T(0);
    }
  }
  short bb[NB], bc[NB], vr[NV], vc[NV];
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int e = tid + u * NT;
    bb[u] = (short)(e < h * h ? e / h : -1);
    bc[u] = (short)(e < h * h ? e % h : 0);
  }
#pragma unroll
  for (int u = 0; u < NV; ++u) {  // rows fastest: a warp touches 32 consecutive rows (distinct banks)
    const int e = tid + u * NT;
    vr[u] = (short)(e < kp * h ? e % kp : -1);
    vc[u] = (short)(e < kp * h ? e / kp : 0);
  }
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int rotated = 0;
    for (int r = 0; r < m; ++r) {
      for (int i = tid; i < h; i += NT) {
        int p, q;
        if (i == 0) {
          p = r;
          q = m;
        } else {
          p = r + i;
          if (p >= m) p -= m;
          q = r - i;
          if (q < 0) q += m;
        }
        if (p > q) { const int x = p; p = q; q = x; }
        const T app = A[p * lda + p], aqq = A[q * lda + q], apq = A[p * lda + q];
        T c = T(1), s = T(0), t = T(0);
        if (apq != T(0) && fabs(apq) > tol * dsqrt<T>(fabs(app) * fabs(aqq))) {
          const T theta = (aqq - app) / (T(2) * apq);
          t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + dsqrt<T>(theta * theta + T(1)));
          c = T(1) / dsqrt<T>(t * t + T(1));
          s = t * c;
          rotated = 1;
        }
        pair[2 * i] = p;
        pair[2 * i + 1] = q;
        rot[4 * i + 0] = c;
        rot[4 * i + 1] = s;
        rot[4 * i + 2] = app - t * apq;
        rot[4 * i + 3] = aqq + t * apq;
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const int b = bb[u], c2 = bc[u];
        if (b < 0) continue;
        const T sb = rot[4 * b + 1], s_c = rot[4 * c2 + 1];
        if (sb == T(0) && s_c == T(0)) continue;
        const int pb = pair[2 * b], qb = pair[2 * b + 1];
        if (b == c2) {
          A[pb * lda + pb] = rot[4 * b + 2];
          A[qb * lda + qb] = rot[4 * b + 3];
          A[pb * lda + qb] = T(0);
          A[qb * lda + pb] = T(0);
          continue;
        }
        const int pc = pair[2 * c2], qc = pair[2 * c2 + 1];
        const T cb = rot[4 * b + 0], c_c = rot[4 * c2 + 0];
        const T a00 = A[pb * lda + pc], a01 = A[pb * lda + qc];
        const T a10 = A[qb * lda + pc], a11 = A[qb * lda + qc];
        const T m00 = cb * a00 - sb * a10, m01 = cb * a01 - sb * a11;
        const T m10 = sb * a00 + cb * a10, m11 = sb * a01 + cb * a11;
        A[pb * lda + pc] = c_c * m00 - s_c * m01;
        A[pb * lda + qc] = s_c * m00 + c_c * m01;
        A[qb * lda + pc] = c_c * m10 - s_c * m11;
        A[qb * lda + qc] = s_c * m10 + c_c * m11;
      }
#pragma unroll
      for (int u = 0; u < NV; ++u) {
        const int row = vr[u], c2 = vc[u];
        if (row < 0) continue;
        const T s_c = rot[4 * c2 + 1];
        if (s_c == T(0)) continue;
        const T c_c = rot[4 * c2 + 0];
        const int pc = pair[2 * c2], qc = pair[2 * c2 + 1];
        const T va = V[row * lda + pc], vb = V[row * lda + qc];
        V[row * lda + pc] = c_c * va - s_c * vb;
        V[row * lda + qc] = s_c * va + c_c * vb;
      }
      __syncthreads();
    }
    if (!__syncthreads_or(rotated)) break;
  }
  return sweep + 1;
}

// ---- FP32 Jacobi with the symmetric matrix kept as its upper triangle ----
//
// Same round-robin ordering and closed-form 2 x 2 updates as
// cta_jacobi_fast, arranged for shared-memory bandwidth, the limit of the
// analysis kernel: pairs come arithmetically from the round number (slot 0
// pairs (r, m), slot i >= 1 pairs ((r + i) mod m, (r - i) mod m), m = kp - 1),
// only the blocks (b <= c) of the upper triangle are updated (every entry at
// [min][max]), and the eigenvectors are kept transposed (Vt, one row per
// eigenvector) so that a rotation of two eigenvectors is two float4 row
// streams.

__device__ __forceinline__ void jacobi_pair(int s, int r, int m, int& p, int& q) {
  if (s == 0) {
    p = r;
    q = m;
  } else {
    p = r + s;
    if (p >= m) p -= m;
    q = r - s;
    if (q < 0) q += m;
  }
}

// Rotation (c, s) zeroing apq, and the two rotated diagonal entries, for
// the loose first stage only: the angle comes from the hardware reciprocal
// square root and approximate division (its error only changes how far the
// rotation zeroes apq), and c is refined by one Newton step so that
// c^2 + s^2 = 1 to FP32 rounding (the eigenvector rows stay orthonormal; the
// Newton-Schulz step after the Jacobi removes the rest).
__device__ __forceinline__ float4 jacobi_rot(float app, float aqq, float apq, float tol) {
  float c = 1.0f, s = 0.0f, t = 0.0f;
  if (apq != 0.0f && apq * apq > tol * tol * fabsf(app * aqq)) {
    const float tau = __fdividef(aqq - app, 2.0f * apq);
    const float q = fmaf(tau, tau, 1.0f);
    t = copysignf(__fdividef(1.0f, fabsf(tau) + q * rsqrtf(q)), tau);
    const float u = fmaf(t, t, 1.0f);
    const float c0 = rsqrtf(u);
    c = c0 * fmaf(-0.5f * u * c0, c0, 1.5f);
    s = t * c;
  }
  return make_float4(c, s, app - t * apq, aqq + t * apq);
}

// Diagonalises A (kp x kp, kp even, lda; read and written in its upper
// triangle only) to the off-diagonal threshold tol.  Vt (rows of ldv
// floats, ldv % 4 == 0, ldv >= 4 ceil(kp / 4), 16-byte aligned) receives the
// eigenvectors as rows: Vt[j * ldv + i] = V_ij.  rot holds kp/2 float4
// (16-byte aligned).  Returns the sweeps run.
template <int KMAX, int NT>
__device__ int cta_jacobi_tri(float* A, int lda, float* Vt, int ldv, int kp, float tol, int max_sweeps,
                              float4* rot) {
  constexpr int HM = KMAX / 2;
  constexpr int NB = (HM * (HM + 1) / 2 + NT - 1) / NT;     // upper-triangle blocks per thread
  constexpr int NVI = (HM * ((KMAX + 3) / 4) + NT - 1) / NT;  // (pair, 4-row chunk) items per thread
  const int tid = threadIdx.x, h = kp >> 1, m = kp - 1, nch = (kp + 3) >> 2;
  for (int e = tid; e < kp * 4 * nch; e += NT) {
    const int j = e / (4 * nch), i = e - j * (4 * nch);
    Vt[j * ldv + i] = (i == j) ? 1.0f : 0.0f;
  }
  int blk[NB];  // b << 8 | c with b <= c, or -1
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    int e = tid + u * NT, b = 0;
    if (e >= h * (h + 1) / 2) {
      blk[u] = -1;
      continue;
    }
    while (e >= h - b) {
      e -= h - b;
      ++b;
    }
    blk[u] = (b << 8) | (b + e);
  }
  __syncthreads();
  int sweep = 0;
  while (sweep < max_sweeps) {
    int rotated = 0;
    for (int r = 0; r < m; ++r) {
      for (int i = tid; i < h; i += NT) {
        int p, q;
        jacobi_pair(i, r, m, p, q);
        const float4 R = jacobi_rot(A[p * lda + p], A[q * lda + q], A[min(p, q) * lda + max(p, q)], tol);
        rot[i] = R;
        rotated |= (R.y != 0.0f);
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        if (blk[u] < 0) continue;
        const int b = blk[u] >> 8, c = blk[u] & 0xff;
        const float4 pb = rot[b];
        if (b == c) {
          if (pb.y == 0.0f) continue;
          int p, q;
          jacobi_pair(b, r, m, p, q);
          A[p * lda + p] = pb.z;
          A[q * lda + q] = pb.w;
          A[min(p, q) * lda + max(p, q)] = 0.0f;
          continue;
        }
        const float4 pc = rot[c];
        if (pb.y == 0.0f && pc.y == 0.0f) continue;
        int r0, r1, c0, c1;
        jacobi_pair(b, r, m, r0, r1);
        jacobi_pair(c, r, m, c0, c1);
        const int i00 = min(r0, c0) * lda + max(r0, c0), i01 = min(r0, c1) * lda + max(r0, c1);
        const int i10 = min(r1, c0) * lda + max(r1, c0), i11 = min(r1, c1) * lda + max(r1, c1);
        const float a00 = A[i00], a01 = A[i01], a10 = A[i10], a11 = A[i11];
        const float m00 = pb.x * a00 - pb.y * a10, m01 = pb.x * a01 - pb.y * a11;
        const float m10 = pb.y * a00 + pb.x * a10, m11 = pb.y * a01 + pb.x * a11;
        A[i00] = pc.x * m00 - pc.y * m01;
        A[i01] = pc.y * m00 + pc.x * m01;
        A[i10] = pc.x * m10 - pc.y * m11;
        A[i11] = pc.y * m10 + pc.x * m11;
      }
#pragma unroll
      for (int u = 0; u < NVI; ++u) {
        const int e = tid + u * NT;
        const int sl = e / nch, ch = e - sl * nch;
        if (sl >= h) break;
        const float4 ps = rot[sl];
        if (ps.y == 0.0f) continue;
        int p, q;
        jacobi_pair(sl, r, m, p, q);
        float4* vp = reinterpret_cast<float4*>(Vt + p * ldv) + ch;
        float4* vq = reinterpret_cast<float4*>(Vt + q * ldv) + ch;
        const float4 a = *vp, bq = *vq;
        *vp = make_float4(ps.x * a.x - ps.y * bq.x, ps.x * a.y - ps.y * bq.y, ps.x * a.z - ps.y * bq.z,
                          ps.x * a.w - ps.y * bq.w);
        *vq = make_float4(ps.y * a.x + ps.x * bq.x, ps.y * a.y + ps.x * bq.y, ps.y * a.z + ps.x * bq.z,
                          ps.y * a.w + ps.x * bq.w);
      }
      __syncthreads();
    }
    ++sweep;
    if (!__syncthreads_or(rotated)) break;
    // A sweep that rotated may still have left every pair under the
    // threshold: test all pairs at once (one barrier) instead of running a
    // further sweep whose rounds would only confirm it.
    int open = 0;
    for (int i = tid >> 5; i < kp - 1; i += NT / 32) {
      const float aii = A[i * lda + i];
      for (int j = i + 1 + (tid & 31); j < kp; j += 32) {
        const float aij = A[i * lda + j];
        open |= (aij != 0.0f && aij * aij > tol * tol * fabsf(aii * A[j * lda + j]));
      }
    }
    if (!__syncthreads_or(open)) break;
  }
  return sweep;
}

// One Newton-Schulz step towards the orthogonal polar factor of V (k x k):
// V <- V (3I - V^T V) / 2.  Rotations accumulated in FP32 leave V about
// sweeps * k * eps away from orthogonal; one step squares that deviation.
// M (k x lda) is scratch; tmp holds `rows` rows of KMAX values.
template <typename T, int KMAX>
__device__ void cta_reorthonormalize(T* V, int k, int lda, T* M, T* tmp, int rows) {
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e / k, j = e - i * k;
    T s = T(0);
    for (int m = 0; m < k; ++m) s += V[m * lda + i] * V[m * lda + j];
    M[i * lda + j] = ((i == j) ? T(1.5) : T(0)) - T(0.5) * s;
  }
  __syncthreads();
  for (int r0 = 0; r0 < k; r0 += rows) {
    const int nr = (k - r0 < rows) ? k - r0 : rows;
    for (int e = threadIdx.x; e < nr * k; e += blockDim.x) {
      const int r = e / k, j = e - r * k;
      tmp[r * KMAX + j] = V[(r0 + r) * lda + j];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nr * k; e += blockDim.x) {
      const int r = e / k, j = e - r * k;
      T s = T(0);
      for (int m = 0; m < k; ++m) s += tmp[r * KMAX + m] * M[m * lda + j];
      V[(r0 + r) * lda + j] = s;
    }
    __syncthreads();
  }
}

// A <- V^T A V in place (k x k), using tmp (at least rows x lda values of T,
// rows >= 1) as a staging buffer: first A <- A V row block by row block, then
// A <- V^T A column block by column block.
template <typename T>
__device__ void cta_similarity(T* A, const T* V, int k, int lda, T* tmp, int rows) {
  for (int r0 = 0; r0 < k; r0 += rows) {
    const int nr = (k - r0 < rows) ? k - r0 : rows;
    for (int e = threadIdx.x; e < nr * k; e += blockDim.x) tmp[(e / k) * lda + e % k] = A[(r0 + e / k) * lda + e % k];
    __syncthreads();
    for (int e = threadIdx.x; e < nr * k; e += blockDim.x) {
      const int r = e / k, j = e - r * k;
      T s = T(0);
      for (int m = 0; m < k; ++m) s += tmp[r * lda + m] * V[m * lda + j];
      A[(r0 + r) * lda + j] = s;
    }
    __syncthreads();
  }
  for (int c0 = 0; c0 < k; c0 += rows) {
    const int nc = (k - c0 < rows) ? k - c0 : rows;
    for (int e = threadIdx.x; e < nc * k; e += blockDim.x) tmp[(e / k) * lda + e % k] = A[(e % k) * lda + c0 + e / k];
    __syncthreads();
    for (int e = threadIdx.x; e < nc * k; e += blockDim.x) {
      const int c = e % nc, i = e / nc;
      T s = T(0);
      for (int m = 0; m < k; ++m) s += V[m * lda + i] * tmp[c * lda + m];
      A[i * lda + c0 + c] = s;
    }
    __syncthreads();
  }
}

// The k x k part of one ensemble-space analysis.  On entry A holds
// diag * I + Y'^T R^-1 Y' (k x k, padded to kp with a decoupled unit
// diagonal when k is odd) and b = Y'^T R^-1 d.  On exit A holds W (k x k) and
// wa the mean weights, so that
//   compat square root (use_chol): W = sqrt(k-1) chol_L(Pa), Pa = A^-1 (x rho
//     when infl_compat) -- ETKF.hpp:150-159, LETKF.hpp:215-224;
//   symmetric (Hunt): A = V diag(lam) V^T, Pa = sc V diag(1/lam) V^T,
//     W = V diag(sqrt((k-1) sc / lam)) V^T, sc = rho when infl_compat else 1;
//   wa = Pa b in both.
// Scratch: V (kp x lda), lam, uvec (k), rot (2 kp), pairbuf (kp ints),
// misc (4 ints).  Returns false if the system was not positive definite.
template <typename T, int KMAX, int NT>
__device__ bool solve_transform(T* A, T* V, const T* bvec, T* wa, T* lam, T* uvec, T* rot,
                                int* pairbuf, int* misc, int k, int kp, int lda, bool use_chol,
                                bool infl_compat, double rho, T tol, int sweep_cap, int* sweeps,
                                bool warm = false, T* tmp = nullptr, int tmp_rows = 0) {
  const int tid = threadIdx.x, nt = blockDim.x;
  bool ok = true;
  *sweeps = 0;
  if (use_chol) {
    ok = cta_cholesky<T>(A, k, lda, misc);
    cta_lower_inverse<T>(A, V, k, lda);
    cta_gram_of_lower<T>(V, A, k, lda);
    if (infl_compat)
      for (int e = tid; e < k * k; e += nt) A[(e / k) * lda + e % k] *= (T)rho;
    __syncthreads();
    for (int i = tid; i < k; i += nt) {
      T s = T(0);
      for (int j = 0; j < k; ++j) s += A[i * lda + j] * bvec[j];
      wa[i] = s;
    }
    __syncthreads();
    ok = cta_cholesky<T>(A, k, lda, misc) && ok;
    const T sqk = (T)sqrt((double)(k - 1));
    for (int e = tid; e < k * k; e += nt) A[(e / k) * lda + e % k] *= sqk;
    __syncthreads();
    return ok;
  }
  if (tid == 0) misc[1] = 0;
  // Warm start: V holds the eigenvectors of a nearby system; rotate A into
  // that basis and let the sweeps continue from it.
  if (warm) cta_similarity<T>(A, V, kp, lda, tmp, tmp_rows);
  *sweeps = cta_jacobi_fast<T, KMAX, NT>(A, V, kp, lda, tol, sweep_cap, rot, pairbuf, !warm);
  const T sc = infl_compat ? (T)rho : T(1);
  for (int i = tid; i < k; i += nt) {
    const T l = A[i * lda + i];
    lam[i] = l;
    if (!(l > T(0)) || !(l < T(3.0e38))) misc[1] = 1;
  }
  __syncthreads();
  ok = misc[1] == 0;
  for (int i = tid; i < k; i += nt) {  // u = diag(sc / lam) V^T b
    T s = T(0);
    for (int j = 0; j < k; ++j) s += V[j * lda + i] * bvec[j];
    uvec[i] = s * sc / lam[i];
  }
  __syncthreads();
  for (int i = tid; i < k; i += nt) {  // wa = V u
    T s = T(0);
    for (int m = 0; m < k; ++m) s += V[i * lda + m] * uvec[m];
    wa[i] = s;
  }
  __syncthreads();
  for (int i = tid; i < k; i += nt) uvec[i] = dsqrt<T>(T(k - 1) * sc / lam[i]);
  __syncthreads();
  for (int e = tid; e < k * k; e += nt) {
    const int i = e / k, j = e - i * k;
    T s = T(0);
    for (int m = 0; m < k; ++m) s += V[i * lda + m] * uvec[m] * V[j * lda + m];
    A[i * lda + j] = s;
  }
  __syncthreads();
  return ok;
}

}  // namespace mg
