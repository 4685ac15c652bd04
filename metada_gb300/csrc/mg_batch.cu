// Many independent global ETKF analyses (ETKF.hpp:100-179 each) of uneven
// sizes in one pass: the uneven-batch configuration (hundreds of cases with
// different state sizes, member counts and obs counts).
//
// A plan flattens every case into work items of fixed shape and runs five
// kernels over the item tables:
//   prep_state   (case, 256-state tile)  mean and perturbations (member order, bit-exact mean)
//   prep_obs     (case, 8-obs tile)      H (identity-interpolation gather or given HX), ym, Y', d, 1/sigma^2
//   gram<KMAX>   (case, obs chunk)       partial k x k Gram and b, one launch per member-count bucket
//   solve        (case)                  FP64 sum of partials, (k-1)/rho I or (k-1) I, transform T
//   update       (case, 32-state tile)   Xa = xm + X' T; the last tile of a case stamps its finish time
// The mixed-precision path with the symmetric square root (Hunt et al.
// 2007) replaces the FP64 Gram and solve by the scheme of the batched
// LETKF: an FP32 Gram, a loose FP32 Jacobi with one Newton-Schulz
// re-orthonormalisation (solve1), the Gram rebuilt from the factor
// B = R^-1/2 Y' V1 (rebuild), and a first-order Daleckii-Krein evaluation of
// A2^-1/2 and A2^-1 in that basis (solve2).  It touches no FP64 element with
// the FP64 pipe, which GB300 runs at about 1/64 of the FP32 rate:
//   prep_obs_mixed (case, 32 obs)     Y', d, 1/sigma^2 in FP32 (FP64 values as FP32 pairs)
//   update_mixed   (case, 512 states) member mean, X', Xa = m + X' T and the FP64
//                                     write-back in one pass (no prep_state, no X' buffer)
// Items are ordered largest first within each kernel.  The same sequence of
// launches is captured once into a CUDA graph and replayed.  The obs chunk
// of the Gram items and the member-count bucket boundaries are chosen by an
// autotuner that times the candidate plans on the actual batch.
#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "mg_dense.cuh"
#include "mg_ffloat.cuh"
#include "mg_update.cuh"
#include "mg_internal.h"

struct DevCase {
  double* X;
  int64_t n, ld;
  int k, kclass;
  const double* HX;        // p x k, or null
  const int64_t* obs_node; // p state indices (identity interpolation), or null
  const double* yo;
  const double* rvar;
  int64_t p;
  double rho;
  double* mean_out;
  // workspace
  double* mean;
  void* Xp;
  double* Y;
  double* d;
  double* rinv;
  double* Gpart;  // nchunk x k x k
  double* bpart;  // nchunk x k
  double* T;      // k x k
  // mixed path with the symmetric square root (FP32 throughout), else null
  float* Y32;     // p x k Y'
  float* d32;     // p innovations
  float* rinv32;  // p 1/sigma^2
  float* Gp32;    // nchunk x k x k partial Grams
  float* bp32;    // nchunk x k partial b
  float* V1;      // k x k stage-1 basis
  float* T32;     // k x k transform
  int64_t nchunk;
  int64_t ntiles;  // update items of the case
};

struct WorkItem {
  int32_t c;    // case
  int32_t pad;
  int64_t a, b;  // range [a, b) (states, obs or chunk index)
};

struct mg_etkf_batch {
  int ncases = 0;
  int flags = 0;
  int precision = MG_PREC_FP64;
  int gram_chunk = 512;
  int kclass_mode = 0;  // 0: {32, 64, 128}; 1: {64, 128}; 2: {128}
  std::vector<mg_etkf_case> host_cases;
  DevCase* dcases = nullptr;
  WorkItem* items = nullptr;  // all item tables, back to back
  int64_t n_state_items = 0, n_obs_items = 0, n_update_items = 0;
  int64_t gram_off[3] = {0, 0, 0}, gram_cnt[3] = {0, 0, 0};
  int64_t state_off = 0, obs_off = 0, update_off = 0;
  int maxk = 0;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  unsigned long long* counters = nullptr;  // per-case finished update tiles
  unsigned long long* times = nullptr;     // [0] start, [1 + c] case finish (ns)
  int* status = nullptr;
  const int* order = nullptr;  // case indices, largest k first (one CTA per case kernels)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

constexpr int kThreads = 256;
constexpr int kStateTile = 256;
constexpr int kObsTile = 8;
constexpr int kUpdTile = 32;

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename TE>
__global__ void __launch_bounds__(kThreads) batch_prep_state_kernel(const DevCase* __restrict__ cases,
                                                                    const WorkItem* __restrict__ items,
                                                                    unsigned long long* times) {
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  if (blockIdx.x == 0 && threadIdx.x == 0) times[0] = globaltimer();
  const int64_t s = it.a + threadIdx.x;
  if (s >= it.b) return;
  const double inv_k = 1.0 / (double)c.k;
  double m = 0.0;
  for (int i = 0; i < c.k; ++i) m = __dadd_rn(m, c.X[(int64_t)i * c.ld + s]);
  m = __dmul_rn(m, inv_k);
  c.mean[s] = m;
  TE* Xp = static_cast<TE*>(c.Xp);
  for (int i = 0; i < c.k; ++i) Xp[(int64_t)i * c.n + s] = (TE)__dsub_rn(c.X[(int64_t)i * c.ld + s], m);
}

__global__ void __launch_bounds__(kThreads) batch_prep_obs_kernel(const DevCase* __restrict__ cases,
                                                                  const WorkItem* __restrict__ items) {
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  const int lane = threadIdx.x & 31;
  const int64_t o = it.a + (threadIdx.x >> 5);
  if (o >= it.b) return;
  const int k = c.k;
  double h[4];
  double s = 0.0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = lane + 32 * t;
    h[t] = 0.0;
    if (i < k) {
      h[t] = c.HX ? c.HX[o * k + i] : c.X[(int64_t)i * c.ld + c.obs_node[o]];
      s += h[t];
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  const double ym = s / (double)k;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = lane + 32 * t;
    if (i < k) {
      c.Y[o * k + i] = h[t] - ym;
    }
  }
  if (lane == 0) {
    c.d[o] = c.yo[o] - ym;
    c.rinv[o] = 1.0 / c.rvar[o];
  }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// Mixed path: Y', d and 1/sigma^2 in FP32 for kObsWarp obs per warp, all
// their member values gathered before any is used.  The FP64 values enter
// as FP32 pairs (split_double); the member mean is taken twice (of the pairs,
// then of the residuals), so Y' keeps full FP32 accuracy however large the
// values are against their spread.
constexpr int kObsWarp = 4;
constexpr int kObsItem = kObsWarp * (kThreads / 32);

__global__ void __launch_bounds__(kThreads) batch_prep_obs_mixed_kernel(const DevCase* __restrict__ cases,
                                                                        const WorkItem* __restrict__ items,
                                                                        unsigned long long* times) {
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  if (blockIdx.x == 0 && threadIdx.x == 0) times[0] = globaltimer();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = c.k;
  const int64_t ob = it.a + (int64_t)warp * kObsWarp;
  double hv[kObsWarp][4];
#pragma unroll
  for (int u = 0; u < kObsWarp; ++u) {
    const int64_t o = ob + u;
    const bool valid = o < it.b;
    const int64_t node = (valid && !c.HX) ? c.obs_node[o] : 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = lane + 32 * t;
      hv[u][t] = 0.0;
      if (valid && i < k) hv[u][t] = c.HX ? c.HX[o * k + i] : c.X[(int64_t)i * c.ld + node];
    }
  }
  const float inv_k = 1.0f / (float)k;
#pragma unroll
  for (int u = 0; u < kObsWarp; ++u) {
    const int64_t o = ob + u;
    float hh[4], hl[4], s = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      mg::split_double(hv[u][t], hh[t], hl[t]);
      s += hh[t] + hl[t];
    }
    const float m1 = warp_sum(s) * inv_k;
    float pv[4], s2 = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      pv[t] = (lane + 32 * t < k) ? __fadd_rn(__fsub_rn(hh[t], m1), hl[t]) : 0.0f;
      s2 += pv[t];
    }
    const float m2 = warp_sum(s2) * inv_k;
    if (o < it.b) {
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = lane + 32 * t;
        if (i < k) c.Y32[o * k + i] = pv[t] - m2;
      }
      if (lane == 0) {  // FP32 pairs again: no FP64 instruction per obs
        float yh, yl, vh, vl;
        mg::split_double(c.yo[o], yh, yl);
        mg::split_double(c.rvar[o], vh, vl);
        c.d32[o] = __fsub_rn(__fadd_rn(__fsub_rn(yh, m1), yl), m2);
        c.rinv32[o] = 1.0f / __fadd_rn(vh, vl);
      }
    }
  }
}

// Mixed path update (mg_update.cuh): items of kUpdItemS states, the
// transform staged once per item.
constexpr int kUpdItemS = 512;

__global__ void __launch_bounds__(kThreads, 2) batch_update_mixed_kernel(const DevCase* __restrict__ cases,
                                                                         const WorkItem* __restrict__ items,
                                                                         int maxk, unsigned long long* counters,
                                                                         unsigned long long* times) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  float bg = 0.0f, an = 0.0f;
  mg::update_mixed<false>(c.X, c.ld, c.k, it.a, it.b, c.T32, c.mean_out, reinterpret_cast<float*>(smem_raw), maxk,
                          bg, an);
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(&counters[it.c], 1ull) + 1ull;
    if ((int64_t)done == c.ntiles) times[1 + it.c] = globaltimer();
  }
}

template <typename TE, int KMAX>
__global__ void __launch_bounds__(kThreads) batch_gram_kernel(const DevCase* __restrict__ cases,
                                                              const WorkItem* __restrict__ items) {
  constexpr int CH = (KMAX * 8 > 512) ? 32 : 64, R = KMAX / 16;
  __shared__ TE Ys[CH * KMAX];
  __shared__ TE sr[CH], sd[CH];
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  const int k = c.k;
  const int tid = threadIdx.x, ti = tid / 16, tj = tid % 16;
  // it.pad = chunk index within the case, [it.a, it.b) = its obs range
  const int64_t o0 = it.a, o1 = it.b;
  TE acc[R][R];
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) acc[a][b] = TE(0);
  TE bacc = TE(0);
  for (int64_t c0 = o0; c0 < o1; c0 += CH) {
    const int cnt = (int)(o1 - c0 < CH ? o1 - c0 : CH);
    for (int e = tid; e < cnt * KMAX; e += kThreads) {
      const int r = e / KMAX, j = e - r * KMAX;
      TE v = TE(0);
      if (j < k) {
        if constexpr (sizeof(TE) == 4)
          v = c.Y32[(c0 + r) * k + j];
        else
          v = c.Y[(c0 + r) * k + j];
      }
      Ys[e] = v;
    }
    if (tid < cnt) {
      if constexpr (sizeof(TE) == 4) {
        sr[tid] = c.rinv32[c0 + tid];
        sd[tid] = c.d32[c0 + tid];
      } else {
        sr[tid] = c.rinv[c0 + tid];
        sd[tid] = c.d[c0 + tid];
      }
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      const TE w = sr[r];
      TE av[R], bv[R];
#pragma unroll
      for (int a = 0; a < R; ++a) av[a] = Ys[r * KMAX + ti + 16 * a] * w;
#pragma unroll
      for (int b = 0; b < R; ++b) bv[b] = Ys[r * KMAX + tj + 16 * b];
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] += av[a] * bv[b];
    }
    if (tid < k)
      for (int r = 0; r < cnt; ++r) bacc += (Ys[r * KMAX + tid] * sr[r]) * sd[r];
    __syncthreads();
  }
  const int64_t chunk = it.pad;
  // partials in the element type (FP32 partials are summed in FP32)
  TE* G = (sizeof(TE) == 4) ? (TE*)c.Gp32 + chunk * k * k : (TE*)c.Gpart + chunk * k * k;
  TE* bp = (sizeof(TE) == 4) ? (TE*)c.bp32 : (TE*)c.bpart;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = ti + 16 * a, j = tj + 16 * b;
      if (i < k && j < k) G[i * k + j] = acc[a][b];
    }
  if (tid < k) bp[chunk * k + tid] = bacc;
}

// ---- mixed path with the symmetric square root (FP32, k <= 112) ----
constexpr float kStage1Tol = 3e-4f;  // off-diagonal threshold of the loose Jacobi

__host__ __device__ constexpr int mix_lda(int kp) { return kp + 1; }
__host__ __device__ constexpr int mix_ldv(int kp) { return ((kp + 3) & ~3) + 4; }
__host__ __device__ constexpr int round4(int x) { return (x + 3) & ~3; }
__host__ __device__ constexpr size_t solve1_floats(int kp) {
  return (size_t)round4(kp * mix_lda(kp)) + (size_t)kp * mix_ldv(kp) + 32 * 128 + 4 * 64;
}
__host__ __device__ constexpr size_t solve2_floats(int kp) { return 3 * (size_t)kp * mix_lda(kp) + 5 * (size_t)kp; }

// Stage 1 of one case: A = (k-1)/rho I + G (FP32 from the partials), loose
// Jacobi, V1 back to orthogonal, V1 to global memory.
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) batch_solve1_kernel(const DevCase* __restrict__ cases,
                                                                const int* __restrict__ order, int flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DevCase& c = cases[order[blockIdx.x]];
  const int k = c.k, kp = k + (k & 1), lda = mix_lda(kp), ldv = mix_ldv(kp);
  float* A = reinterpret_cast<float*>(smem_raw);
  float* Vt = A + round4(kp * lda);
  float* tmp = Vt + kp * ldv;
  float4* rot = reinterpret_cast<float4*>(tmp + 32 * 128);
  const int tid = threadIdx.x;
  const float diagf = (flags & MG_INFL_COMPAT) ? (float)(k - 1) : (float)(k - 1) / (float)c.rho;
  for (int e = tid; e < kp * kp; e += NT) {
    const int i = e / kp, j = e - i * kp;
    float s = 0.0f;
    if (i < k && j < k) {
      for (int64_t b = 0; b < c.nchunk; ++b) s += c.Gp32[b * k * k + i * k + j];
      if (i == j) s += diagf;
    } else if (i == j) {
      s = 1.0f;
    }
    A[i * lda + j] = s;
  }
  __syncthreads();
  mg::cta_jacobi_tri<128, NT>(A, lda, Vt, ldv, kp, kStage1Tol, 30, rot);
  for (int e = tid; e < kp * kp; e += NT) {  // eigenvector rows -> row-major V1 in the A region
    const int j = e / kp, i = e - j * kp;
    A[i * lda + j] = Vt[j * ldv + i];
  }
  __syncthreads();
  mg::cta_reorthonormalize<float, 128>(A, kp, lda, Vt, tmp, 32);
  for (int e = tid; e < k * k; e += NT) c.V1[e] = A[(e / k) * lda + e % k];
}

// Gram of the factor B = diag(sqrt(1/sigma^2)) Y' V1 over one obs chunk:
// the rebuilt A2 - (k-1)/rho I = V1^T G V1 with errors relative to the
// column norms of B.
template <int KMAX>
__global__ void __launch_bounds__(kThreads) batch_rebuild_kernel(const DevCase* __restrict__ cases,
                                                                 const WorkItem* __restrict__ items) {
  constexpr int CH = 32, R = KMAX / 16, LDW = KMAX + 1;
  constexpr int RW = CH / (kThreads / 32), CW = KMAX / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* V1s = reinterpret_cast<float*>(smem_raw);  // KMAX x LDW
  float* Ys = V1s + KMAX * LDW;                      // CH x KMAX
  float* Bc = Ys + CH * KMAX;                        // CH x KMAX
  __shared__ float sw[CH];
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  const int k = c.k;
  const int tid = threadIdx.x, ti = tid / 16, tj = tid % 16, wrp = tid >> 5, ln = tid & 31;
  for (int e = tid; e < KMAX * KMAX; e += kThreads) {
    const int i = e / KMAX, j = e - i * KMAX;
    V1s[i * LDW + j] = (i < k && j < k) ? c.V1[i * k + j] : 0.0f;
  }
  float acc[R][R];
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) acc[a][b] = 0.0f;
  for (int64_t c0 = it.a; c0 < it.b; c0 += CH) {
    const int cnt = (int)(it.b - c0 < CH ? it.b - c0 : CH);
    for (int e = tid; e < cnt * KMAX; e += kThreads) {
      const int r = e / KMAX, j = e - r * KMAX;
      Ys[e] = (j < k) ? c.Y32[(c0 + r) * k + j] : 0.0f;
    }
    if (tid < cnt) sw[tid] = sqrtf(c.rinv32[c0 + tid]);
    __syncthreads();
    float sacc[RW][CW];
#pragma unroll
    for (int x = 0; x < RW; ++x)
#pragma unroll
      for (int q = 0; q < CW; ++q) sacc[x][q] = 0.0f;
    for (int m0 = 0; m0 < k; m0 += 4) {  // rows of Ys and V1s are zero from k to KMAX
      float4 yv[RW];
#pragma unroll
      for (int x = 0; x < RW; ++x) yv[x] = *reinterpret_cast<const float4*>(Ys + (wrp * RW + x) * KMAX + m0);
#pragma unroll
      for (int mm = 0; mm < 4; ++mm) {
        float vv[CW];
#pragma unroll
        for (int q = 0; q < CW; ++q) vv[q] = V1s[(m0 + mm) * LDW + ln + 32 * q];
#pragma unroll
        for (int x = 0; x < RW; ++x) {
          const float y = mm == 0 ? yv[x].x : (mm == 1 ? yv[x].y : (mm == 2 ? yv[x].z : yv[x].w));
#pragma unroll
          for (int q = 0; q < CW; ++q) sacc[x][q] += y * vv[q];
        }
      }
    }
#pragma unroll
    for (int x = 0; x < RW; ++x) {
      const int r = wrp * RW + x;
      if (r < cnt)
#pragma unroll
        for (int q = 0; q < CW; ++q) Bc[r * KMAX + ln + 32 * q] = sacc[x][q] * sw[r];
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      float av[R], bv[R];
#pragma unroll
      for (int a = 0; a < R; ++a) av[a] = Bc[r * KMAX + ti + 16 * a];
#pragma unroll
      for (int b = 0; b < R; ++b) bv[b] = Bc[r * KMAX + tj + 16 * b];
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] += av[a] * bv[b];
    }
    __syncthreads();
  }
  float* G = c.Gp32 + (int64_t)it.pad * k * k;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = ti + 16 * a, j = tj + 16 * b;
      if (i < k && j < k) G[i * k + j] = acc[a][b];
    }
}

// Stage 2 of one case: A2 = (k-1)/rho I + sum of the rebuilt partials is
// nearly diagonal, so W = c V1 (A2^-1/2) V1^T and wa = V1 (A2^-1) V1^T b come
// from the first-order Daleckii-Krein formula (closed-form divided
// differences -1/(s_i s_j (s_i + s_j)), s = sqrt(d), and -1/(d_i d_j)).
__global__ void __launch_bounds__(kThreads) batch_solve2_kernel(const DevCase* __restrict__ cases,
                                                                const int* __restrict__ order, int flags,
                                                                int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ci = order[blockIdx.x];
  const DevCase& c = cases[ci];
  const int k = c.k, kp = k + (k & 1), lda = mix_lda(kp);
  float* V = reinterpret_cast<float*>(smem_raw);  // k x k (lda)
  float* A2 = V + kp * lda;
  float* Tm = A2 + kp * lda;
  float* bv = Tm + kp * lda;
  float* uv = bv + kp;
  float* gv = uv + kp;
  float* wa = gv + kp;
  float* lam = wa + kp;
  const int tid = threadIdx.x;
  const bool compat_infl = flags & MG_INFL_COMPAT;
  const float diag = compat_infl ? (float)(k - 1) : (float)(k - 1) / (float)c.rho;
  for (int e = tid; e < k * k; e += kThreads) {
    const int i = e / k, j = e - i * k;
    V[i * lda + j] = c.V1[e];
    float s = 0.0f;
    for (int64_t b = 0; b < c.nchunk; ++b) s += c.Gp32[b * k * k + e];
    if (i == j) s += diag;
    A2[i * lda + j] = s;
  }
  for (int i = tid; i < k; i += kThreads) {
    float s = 0.0f;
    for (int64_t b = 0; b < c.nchunk; ++b) s += c.bp32[b * k + i];
    bv[i] = s;
  }
  __syncthreads();
  for (int i = tid; i < k; i += kThreads) {
    const float l = A2[i * lda + i];
    lam[i] = l;
    if (!(l > 0.0f) || !(l < 3.0e38f)) atomicExch(status, 1 + ci);
    float s = 0.0f;  // u = V1^T b
    for (int j = 0; j < k; ++j) s += V[j * lda + i] * bv[j];
    uv[i] = s;
  }
  __syncthreads();
  for (int i = tid; i < k; i += kThreads) {  // g = (x^-1)(A2) u
    float s = uv[i];
    for (int j = 0; j < k; ++j)
      if (j != i) s -= A2[i * lda + j] * (uv[j] / lam[j]);
    gv[i] = s / lam[i];
  }
  __syncthreads();
  for (int i = tid; i < k; i += kThreads) {  // wa = V1 g
    float s = 0.0f;
    for (int m = 0; m < k; ++m) s += V[i * lda + m] * gv[m];
    wa[i] = s;
  }
  const float cw = sqrtf((float)(k - 1));
  for (int e = tid; e < k * k; e += kThreads) {  // A2 <- Wb = (c x^-1/2)(A2)
    const int i = e / k, j = e - i * k;
    const float si = sqrtf(lam[i]);
    if (i == j) {
      A2[i * lda + i] = cw / si;
    } else {
      const float sj = sqrtf(lam[j]);
      A2[i * lda + j] = -cw * A2[i * lda + j] / (si * sj * (si + sj));
    }
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += kThreads) {  // Tm = V1 Wb
    const int i = e / k, j = e - i * k;
    float s = 0.0f;
    for (int m = 0; m < k; ++m) s += V[i * lda + m] * A2[m * lda + j];
    Tm[i * lda + j] = s;
  }
  __syncthreads();
  const float scale = compat_infl ? (float)c.rho : 1.0f;
  for (int e = tid; e < k * k; e += kThreads) {  // T[j][i] = scale (wa_j + W_ji), W = Tm V1^T
    const int j = e / k, i = e - j * k;
    float s = 0.0f;
    for (int m = 0; m < k; ++m) s += Tm[j * lda + m] * V[i * lda + m];
    c.T32[j * k + i] = scale * (wa[j] + s);
  }
}

// One CTA per case: sum the partials, solve, write T (FP64; the case's
// k x k system is its only O(k^3) work).
__global__ void __launch_bounds__(kThreads) batch_solve_kernel(const DevCase* __restrict__ cases,
                                                               const int* __restrict__ order, int flags,
                                                               int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ci = order[blockIdx.x];
  const DevCase& c = cases[ci];
  const int k = c.k, kp = k + (k & 1), lda = kp + 1;
  double* A = reinterpret_cast<double*>(smem_raw);
  double* V = A + kp * lda;
  double* bvec = V + kp * lda;
  double* wa = bvec + kp;
  double* lam = wa + kp;
  double* uvec = lam + kp;
  double* rot = uvec + kp;
  int* pairbuf = reinterpret_cast<int*>(rot + 2 * kp);
  int* misc = pairbuf + kp;
  const int tid = threadIdx.x;
  const bool compat_infl = flags & MG_INFL_COMPAT;
  const double diag = compat_infl ? (double)(k - 1) : (double)(k - 1) / c.rho;
  for (int e = tid; e < kp * kp; e += kThreads) {
    const int i = e / kp, j = e % kp;
    double s = 0.0;
    if (i < k && j < k) {
      for (int64_t b = 0; b < c.nchunk; ++b) s += c.Gpart[b * k * k + i * k + j];
      if (i == j) s += diag;
    } else if (i == j) {
      s = 1.0;
    }
    A[i * lda + j] = s;
  }
  for (int i = tid; i < k; i += kThreads) {
    double s = 0.0;
    for (int64_t b = 0; b < c.nchunk; ++b) s += c.bpart[b * k + i];
    bvec[i] = s;
  }
  __syncthreads();
  int sweeps = 0;
  const bool ok = mg::solve_transform<double, 128, kThreads>(A, V, bvec, wa, lam, uvec, rot, pairbuf, misc, k, kp,
                                                              lda, flags & MG_SQRT_CHOLESKY, false, c.rho, 1e-14,
                                                              30, &sweeps);
  const double scale = compat_infl ? c.rho : 1.0;
  for (int e = tid; e < k * k; e += kThreads) {
    const int j = e / k, i = e - j * k;
    c.T[j * k + i] = scale * (wa[j] + A[j * lda + i]);
  }
  if (tid == 0 && !ok) atomicExch(status, 1 + ci);
}

template <typename TE>
__global__ void __launch_bounds__(kThreads) batch_update_kernel(const DevCase* __restrict__ cases,
                                                                const WorkItem* __restrict__ items,
                                                                unsigned long long* counters,
                                                                unsigned long long* times) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const WorkItem it = items[blockIdx.x];
  const DevCase& c = cases[it.c];
  const int k = c.k;
  TE* Ts = reinterpret_cast<TE*>(smem_raw);  // k x k
  TE* Xt = Ts + k * k;                       // 32 x (k + 1)
  const TE* Xp = static_cast<const TE*>(c.Xp);
  for (int e = threadIdx.x; e < k * k; e += kThreads) Ts[e] = (TE)c.T[e];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t s0 = it.a;
  for (int j = warp; j < k; j += kThreads / 32) {
    const int64_t s = s0 + lane;
    Xt[lane * (k + 1) + j] = (s < it.b) ? Xp[(int64_t)j * c.n + s] : TE(0);
  }
  __syncthreads();
  const int64_t s = s0 + lane;
  if (s < it.b) {
    const double m = c.mean[s];
    for (int i = warp; i < k; i += kThreads / 32) {
      TE acc = TE(0);
      for (int j = 0; j < k; ++j) acc += Xt[lane * (k + 1) + j] * Ts[j * k + i];
      c.X[(int64_t)i * c.ld + s] = m + (double)acc;
    }
    if (c.mean_out && warp == 0) c.mean_out[s] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(&counters[it.c], 1ull) + 1ull;
    if ((int64_t)done == c.ntiles) times[1 + it.c] = globaltimer();
  }
}

int kclass_of(int k, int mode) {
  if (mode == 0) return k <= 32 ? 0 : (k <= 64 ? 1 : 2);
  if (mode == 1) return k <= 64 ? 1 : 2;
  return 2;
}

// The mixed path with the symmetric square root runs the FP32 two-stage
// solve; with the Cholesky square root it keeps the FP64 Gram and solve.
bool mixed_hunt(const mg_etkf_batch* b) {
  return b->precision == MG_PREC_MIXED && !(b->flags & MG_SQRT_CHOLESKY);
}

// Builds the item tables and workspace for the current tuning.
int build(mg_context* ctx, mg_etkf_batch* b) {
  const bool f64 = b->precision == MG_PREC_FP64;
  const bool mh = mixed_hunt(b);
  const size_t te = f64 ? 8 : 4;
  std::vector<DevCase> dc(b->ncases);
  std::vector<WorkItem> st_items, ob_items, up_items, gr_items[3];
  mg::Carver cv;
  b->maxk = 0;
  for (int i = 0; i < b->ncases; ++i) {
    const mg_etkf_case& h = b->host_cases[i];
    DevCase& c = dc[i];
    c.X = h.X;
    c.n = h.n;
    c.ld = h.ld;
    c.k = h.k;
    c.kclass = kclass_of(h.k, b->kclass_mode);
    c.HX = h.HX;
    c.obs_node = h.obs_node;
    c.yo = h.yo;
    c.rvar = h.rvar;
    c.p = h.p;
    c.rho = h.rho;
    c.mean_out = h.mean_out;
    c.nchunk = (h.p + b->gram_chunk - 1) / b->gram_chunk;
    b->maxk = std::max(b->maxk, h.k);
    if (mh) {  // FP32 workspace only; the update reads and writes the members in place
      const int64_t upd = kUpdItemS;
      c.ntiles = (h.n + upd - 1) / upd;
      cv.reserve<float>((size_t)h.p * h.k);
      cv.reserve<float>(h.p);
      cv.reserve<float>(h.p);
      cv.reserve<float>((size_t)c.nchunk * h.k * h.k);
      cv.reserve<float>((size_t)c.nchunk * h.k);
      cv.reserve<float>((size_t)h.k * h.k);
      cv.reserve<float>((size_t)h.k * h.k);
      for (int64_t o = 0; o < h.p; o += kObsItem) ob_items.push_back({i, 0, o, std::min<int64_t>(h.p, o + kObsItem)});
      for (int64_t s = 0; s < h.n; s += upd) up_items.push_back({i, 0, s, std::min<int64_t>(h.n, s + upd)});
    } else {
      c.ntiles = (h.n + kUpdTile - 1) / kUpdTile;
      cv.reserve<double>(h.n);
      cv.reserve<char>((size_t)h.n * h.k * te);
      cv.reserve<double>((size_t)h.p * h.k);
      cv.reserve<double>(h.p);
      cv.reserve<double>(h.p);
      cv.reserve<double>((size_t)c.nchunk * h.k * h.k);
      cv.reserve<double>((size_t)c.nchunk * h.k);
      cv.reserve<double>((size_t)h.k * h.k);
      for (int64_t s = 0; s < h.n; s += kStateTile)
        st_items.push_back({i, 0, s, std::min<int64_t>(h.n, s + kStateTile)});
      for (int64_t o = 0; o < h.p; o += kObsTile) ob_items.push_back({i, 0, o, std::min<int64_t>(h.p, o + kObsTile)});
      for (int64_t s = 0; s < h.n; s += kUpdTile) up_items.push_back({i, 0, s, std::min<int64_t>(h.n, s + kUpdTile)});
    }
    for (int64_t ch = 0; ch < c.nchunk; ++ch) {
      const int64_t o0 = ch * b->gram_chunk;
      gr_items[c.kclass].push_back({i, (int32_t)ch, o0, std::min<int64_t>(h.p, o0 + b->gram_chunk)});
    }
  }
  // Largest first (work per item ~ k^2 x its length for the Gram and the update).
  auto by_k = [&](const WorkItem& x, const WorkItem& y) {
    const int64_t wx = (int64_t)dc[x.c].k * dc[x.c].k * (x.b - x.a), wy = (int64_t)dc[y.c].k * dc[y.c].k * (y.b - y.a);
    return wx > wy;
  };
  for (auto& g : gr_items) std::stable_sort(g.begin(), g.end(), by_k);
  if (mh) {
    // Mixed update items (all of one size) run shortest case first, a case's
    // items together, so that small cases finish early in the batch.
    auto work = [&](int ci) { return (double)dc[ci].n * dc[ci].k * dc[ci].k; };
    std::stable_sort(up_items.begin(), up_items.end(), [&](const WorkItem& x, const WorkItem& y) {
      if (work(x.c) != work(y.c)) return work(x.c) < work(y.c);
      return x.c != y.c ? x.c < y.c : x.a < y.a;
    });
  } else {
    std::stable_sort(up_items.begin(), up_items.end(), by_k);
  }
  std::vector<WorkItem> all;
  b->state_off = (int64_t)all.size();
  all.insert(all.end(), st_items.begin(), st_items.end());
  b->obs_off = (int64_t)all.size();
  all.insert(all.end(), ob_items.begin(), ob_items.end());
  for (int g = 0; g < 3; ++g) {
    b->gram_off[g] = (int64_t)all.size();
    b->gram_cnt[g] = (int64_t)gr_items[g].size();
    all.insert(all.end(), gr_items[g].begin(), gr_items[g].end());
  }
  b->update_off = (int64_t)all.size();
  all.insert(all.end(), up_items.begin(), up_items.end());
  b->n_state_items = (int64_t)st_items.size();
  b->n_obs_items = (int64_t)ob_items.size();
  b->n_update_items = (int64_t)up_items.size();
  cv.reserve<DevCase>(b->ncases);
  cv.reserve<WorkItem>(all.size());
  cv.reserve<unsigned long long>(b->ncases);
  cv.reserve<unsigned long long>(b->ncases + 1);
  cv.reserve<int>(4);
  cv.reserve<int>(b->ncases);
  if (cv.off > b->ws_bytes) {
    if (b->ws) cudaFree(b->ws);
    b->ws = nullptr;
    b->ws_bytes = 0;
    if (cudaMalloc(&b->ws, cv.off) != cudaSuccess) {
      cudaGetLastError();
      return mg::fail(ctx, MG_ERR_NOMEM, "mg_etkf_batch: workspace allocation failed");
    }
    b->ws_bytes = cv.off;
  }
  cv = mg::Carver{static_cast<char*>(b->ws), 0};
  for (int i = 0; i < b->ncases; ++i) {
    const mg_etkf_case& h = b->host_cases[i];
    DevCase& c = dc[i];
    if (mh) {
      c.mean = nullptr;
      c.Xp = nullptr;
      c.Y = c.d = c.rinv = c.Gpart = c.bpart = c.T = nullptr;
      c.Y32 = cv.take<float>((size_t)h.p * h.k);
      c.d32 = cv.take<float>(h.p);
      c.rinv32 = cv.take<float>(h.p);
      c.Gp32 = cv.take<float>((size_t)c.nchunk * h.k * h.k);
      c.bp32 = cv.take<float>((size_t)c.nchunk * h.k);
      c.V1 = cv.take<float>((size_t)h.k * h.k);
      c.T32 = cv.take<float>((size_t)h.k * h.k);
    } else {
      c.mean = cv.take<double>(h.n);
      c.Xp = cv.take<char>((size_t)h.n * h.k * te);
      c.Y = cv.take<double>((size_t)h.p * h.k);
      c.d = cv.take<double>(h.p);
      c.rinv = cv.take<double>(h.p);
      c.Gpart = cv.take<double>((size_t)c.nchunk * h.k * h.k);
      c.bpart = cv.take<double>((size_t)c.nchunk * h.k);
      c.T = cv.take<double>((size_t)h.k * h.k);
      c.Y32 = c.d32 = c.rinv32 = c.Gp32 = c.bp32 = c.V1 = c.T32 = nullptr;
    }
  }
  b->dcases = cv.take<DevCase>(b->ncases);
  b->items = cv.take<WorkItem>(all.size());
  b->counters = cv.take<unsigned long long>(b->ncases);
  b->times = cv.take<unsigned long long>(b->ncases + 1);
  b->status = cv.take<int>(4);
  int* order = cv.take<int>(b->ncases);
  b->order = order;
  std::vector<int> ord(b->ncases);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return dc[x].k > dc[y].k; });
  MG_TRY_CUDA(cudaMemcpy(b->dcases, dc.data(), sizeof(DevCase) * dc.size(), cudaMemcpyHostToDevice));
  MG_TRY_CUDA(cudaMemcpy(b->items, all.data(), sizeof(WorkItem) * all.size(), cudaMemcpyHostToDevice));
  MG_TRY_CUDA(cudaMemcpy(order, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice));
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  return MG_OK;
}


constexpr size_t rebuild_bytes(int kmax) { return sizeof(float) * ((size_t)kmax * (kmax + 1) + 2 * 32 * (size_t)kmax); }

// Enqueues the batch (no allocation, no host synchronisation: capturable).
int enqueue(mg_context* ctx, mg_etkf_batch* b) {
  cudaStream_t s = ctx->stream;
  const bool f64 = b->precision == MG_PREC_FP64;
  MG_TRY_CUDA(cudaMemsetAsync(b->counters, 0, sizeof(unsigned long long) * b->ncases, s));
  MG_TRY_CUDA(cudaMemsetAsync(b->status, 0, sizeof(int) * 4, s));
  if (b->n_state_items) {
    if (f64)
      batch_prep_state_kernel<double><<<(unsigned)b->n_state_items, kStateTile, 0, s>>>(b->dcases, b->items + b->state_off, b->times);
    else
      batch_prep_state_kernel<float><<<(unsigned)b->n_state_items, kStateTile, 0, s>>>(b->dcases, b->items + b->state_off, b->times);
    MG_COUNT_LAUNCH();
  }
  const bool mh = mixed_hunt(b);
  if (b->n_obs_items) {
    if (mh)
      batch_prep_obs_mixed_kernel<<<(unsigned)b->n_obs_items, kThreads, 0, s>>>(b->dcases, b->items + b->obs_off,
                                                                                 b->times);
    else
      batch_prep_obs_kernel<<<(unsigned)b->n_obs_items, kObsTile * 32, 0, s>>>(b->dcases, b->items + b->obs_off);
    MG_COUNT_LAUNCH();
  }
  const int kp = b->maxk + (b->maxk & 1);
  if (mh) {
    if (b->gram_cnt[0]) {
      batch_gram_kernel<float, 32><<<(unsigned)b->gram_cnt[0], kThreads, 0, s>>>(b->dcases, b->items + b->gram_off[0]);
      MG_COUNT_LAUNCH();
    }
    if (b->gram_cnt[1]) {
      batch_gram_kernel<float, 64><<<(unsigned)b->gram_cnt[1], kThreads, 0, s>>>(b->dcases, b->items + b->gram_off[1]);
      MG_COUNT_LAUNCH();
    }
    if (b->gram_cnt[2]) {
      batch_gram_kernel<float, 128><<<(unsigned)b->gram_cnt[2], kThreads, 0, s>>>(b->dcases,
                                                                                  b->items + b->gram_off[2]);
      MG_COUNT_LAUNCH();
    }
    if (b->maxk > 64)  // more threads per rotation round for the large cases
      batch_solve1_kernel<512><<<(unsigned)b->ncases, 512, sizeof(float) * solve1_floats(kp), s>>>(b->dcases, b->order,
                                                                                              b->flags);
    else
      batch_solve1_kernel<kThreads><<<(unsigned)b->ncases, kThreads, sizeof(float) * solve1_floats(kp), s>>>(
          b->dcases, b->order, b->flags);
    MG_COUNT_LAUNCH();
    if (b->gram_cnt[0]) {
      batch_rebuild_kernel<32><<<(unsigned)b->gram_cnt[0], kThreads, rebuild_bytes(32), s>>>(b->dcases,
                                                                                          b->items + b->gram_off[0]);
      MG_COUNT_LAUNCH();
    }
    if (b->gram_cnt[1]) {
      batch_rebuild_kernel<64><<<(unsigned)b->gram_cnt[1], kThreads, rebuild_bytes(64), s>>>(b->dcases,
                                                                                          b->items + b->gram_off[1]);
      MG_COUNT_LAUNCH();
    }
    if (b->gram_cnt[2]) {
      batch_rebuild_kernel<128><<<(unsigned)b->gram_cnt[2], kThreads, rebuild_bytes(128), s>>>(
          b->dcases, b->items + b->gram_off[2]);
      MG_COUNT_LAUNCH();
    }
    batch_solve2_kernel<<<(unsigned)b->ncases, kThreads, sizeof(float) * solve2_floats(kp), s>>>(b->dcases, b->order, b->flags,
                                                                                                b->status);
    MG_COUNT_LAUNCH();
    batch_update_mixed_kernel<<<(unsigned)b->n_update_items, kThreads, mg::upd_bytes(b->maxk), s>>>(
        b->dcases, b->items + b->update_off, b->maxk, b->counters, b->times);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
    return MG_OK;
  }
  if (b->gram_cnt[0]) {
    batch_gram_kernel<double, 32><<<(unsigned)b->gram_cnt[0], kThreads, 0, s>>>(b->dcases, b->items + b->gram_off[0]);
    MG_COUNT_LAUNCH();
  }
  if (b->gram_cnt[1]) {
    batch_gram_kernel<double, 64><<<(unsigned)b->gram_cnt[1], kThreads, 0, s>>>(b->dcases, b->items + b->gram_off[1]);
    MG_COUNT_LAUNCH();
  }
  if (b->gram_cnt[2]) {
    batch_gram_kernel<double, 128><<<(unsigned)b->gram_cnt[2], kThreads, 0, s>>>(b->dcases, b->items + b->gram_off[2]);
    MG_COUNT_LAUNCH();
  }
  const size_t smem = sizeof(double) * (2 * (size_t)kp * (kp + 1) + 6 * (size_t)kp) + sizeof(int) * (kp + 8) + 64;
  batch_solve_kernel<<<(unsigned)b->ncases, kThreads, smem, s>>>(b->dcases, b->order, b->flags, b->status);
  MG_COUNT_LAUNCH();
  const size_t te = f64 ? 8 : 4;
  const size_t usmem = te * ((size_t)b->maxk * b->maxk + 32 * (size_t)(b->maxk + 1));
  if (f64)
    batch_update_kernel<double><<<(unsigned)b->n_update_items, kThreads, usmem, s>>>(b->dcases, b->items + b->update_off,
                                                                                     b->counters, b->times);
  else
    batch_update_kernel<float><<<(unsigned)b->n_update_items, kThreads, usmem, s>>>(b->dcases, b->items + b->update_off,
                                                                                    b->counters, b->times);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int set_attributes(mg_context* ctx, const mg_etkf_batch* b) {
  const int kp = b->maxk + (b->maxk & 1);
  const size_t smem = sizeof(double) * (2 * (size_t)kp * (kp + 1) + 6 * (size_t)kp) + sizeof(int) * (kp + 8) + 64;
  const size_t te = b->precision == MG_PREC_FP64 ? 8 : 4;
  const size_t usmem = te * ((size_t)b->maxk * b->maxk + 32 * (size_t)(b->maxk + 1));
  if (smem > 227 * 1024 || usmem > 227 * 1024) return mg::fail(ctx, MG_ERR_ARG, "mg_etkf_batch: k too large");
  MG_TRY_CUDA(cudaFuncSetAttribute(batch_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (mixed_hunt(b)) {
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_solve1_kernel<kThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(float) * solve1_floats(kp))));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_solve1_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(float) * solve1_floats(kp))));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_solve2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(float) * solve2_floats(kp))));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_rebuild_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)rebuild_bytes(32)));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_rebuild_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)rebuild_bytes(64)));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_rebuild_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)rebuild_bytes(128)));
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_update_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)mg::upd_bytes(b->maxk)));
    return MG_OK;
  }
  if (te == 8)
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_update_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)usmem));
  else
    MG_TRY_CUDA(cudaFuncSetAttribute(batch_update_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)usmem));
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_etkf_batch_create(mg_context* ctx, const mg_etkf_case* cases, int32_t ncases, int32_t flags,
                         int32_t precision, mg_etkf_batch** out) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(cases && ncases > 0 && out, "mg_etkf_batch_create: bad arguments");
  MG_CHECK_ARG(precision == MG_PREC_FP64 || precision == MG_PREC_MIXED, "mg_etkf_batch_create: bad precision");
  for (int i = 0; i < ncases; ++i) {
    const mg_etkf_case& c = cases[i];
    MG_CHECK_ARG(c.X && c.n > 0 && c.ld >= c.n && c.k >= 2 && c.k <= 112 && c.p >= 1 && (c.HX || c.obs_node) &&
                     c.yo && c.rvar && c.rho > 0.0,
                 "mg_etkf_batch_create: bad case " + std::to_string(i) + " (k must be 2..112, p >= 1)");
  }
  auto b = std::make_unique<mg_etkf_batch>();
  b->ncases = ncases;
  b->flags = flags;
  b->precision = precision;
  b->host_cases.assign(cases, cases + ncases);
  int rc = build(ctx, b.get());
  if (rc != MG_OK) return rc;
  rc = set_attributes(ctx, b.get());
  if (rc != MG_OK) return rc;
  *out = b.release();
  return MG_OK;
}

void mg_etkf_batch_destroy(mg_etkf_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ws) cudaFree(b->ws);
  delete b;
}

int mg_etkf_batch_run(mg_context* ctx, mg_etkf_batch* b) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(b != nullptr, "mg_etkf_batch_run: null batch");
  return enqueue(ctx, b);
}

int mg_etkf_batch_launch_graph(mg_context* ctx, mg_etkf_batch* b) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(b != nullptr, "mg_etkf_batch_launch_graph: null batch");
  if (!b->exec) {
    // Capture on a private stream so the caller's stream stays uncaptured.
    cudaStream_t cap = nullptr;
    MG_TRY_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaStream_t saved = ctx->stream;
    ctx->stream = cap;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? enqueue(ctx, b) : MG_ERR_CUDA;
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
    ctx->stream = saved;
    cudaStreamDestroy(cap);
    if (e != cudaSuccess || e2 != cudaSuccess || rc != MG_OK) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return rc != MG_OK ? rc : mg::fail(ctx, MG_ERR_CUDA, "mg_etkf_batch: graph capture failed");
    }
    b->graph = g;
    MG_TRY_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
  }
  MG_TRY_CUDA(cudaGraphLaunch(b->exec, ctx->stream));
  return MG_OK;
}

int mg_etkf_batch_finish(mg_context* ctx, mg_etkf_batch* b, double* case_ms) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(b != nullptr, "mg_etkf_batch_finish: null batch");
  int st = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&st, b->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<unsigned long long> t(b->ncases + 1);
  if (case_ms)
    MG_TRY_CUDA(cudaMemcpyAsync(t.data(), b->times, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  if (case_ms)
    for (int i = 0; i < b->ncases; ++i) case_ms[i] = (double)(t[1 + i] - t[0]) * 1e-6;
  if (st) return mg::fail(ctx, MG_ERR_NUMERIC, "mg_etkf_batch: case " + std::to_string(st - 1) +
                                                   " k x k system was not positive definite");
  return MG_OK;
}

int mg_etkf_batch_autotune(mg_context* ctx, mg_etkf_batch* b, int32_t* gram_chunk, int32_t* bucket_mode) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(b != nullptr, "mg_etkf_batch_autotune: null batch");
  // The batch runs in place: keep the members and restore them between trials.
  std::vector<std::pair<double*, size_t>> saved;
  std::vector<void*> copies;
  for (const auto& c : b->host_cases) {
    void* p = nullptr;
    const size_t bytes = sizeof(double) * (size_t)((c.k - 1) * c.ld + c.n);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      for (void* q : copies) cudaFree(q);
      return mg::fail(ctx, MG_ERR_NOMEM, "mg_etkf_batch_autotune: no room to keep the members");
    }
    copies.push_back(p);
    saved.push_back({c.X, bytes});
    MG_TRY_CUDA(cudaMemcpyAsync(p, c.X, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  auto restore = [&]() {
    for (size_t i = 0; i < saved.size(); ++i)
      cudaMemcpyAsync(saved[i].first, copies[i], saved[i].second, cudaMemcpyDeviceToDevice, ctx->stream);
  };
  const int chunks[] = {128, 256, 512, 1024, 2048};
  const int modes[] = {0, 1, 2};
  float best = 1e30f;
  int best_chunk = b->gram_chunk, best_mode = b->kclass_mode;
  cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1];
  int rc = MG_OK;
  for (int mode : modes) {
    for (int ch : chunks) {
      b->gram_chunk = ch;
      b->kclass_mode = mode;
      if ((rc = build(ctx, b)) != MG_OK) break;
      restore();
      if ((rc = enqueue(ctx, b)) != MG_OK) break;  // warm
      restore();
      cudaEventRecord(e0, ctx->stream);
      if ((rc = enqueue(ctx, b)) != MG_OK) break;
      cudaEventRecord(e1, ctx->stream);
      cudaStreamSynchronize(ctx->stream);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        best_chunk = ch;
        best_mode = mode;
      }
    }
    if (rc != MG_OK) break;
  }
  restore();
  cudaStreamSynchronize(ctx->stream);
  for (void* q : copies) cudaFree(q);
  if (rc != MG_OK) return rc;
  b->gram_chunk = best_chunk;
  b->kclass_mode = best_mode;
  rc = build(ctx, b);
  if (rc != MG_OK) return rc;
  if (gram_chunk) *gram_chunk = best_chunk;
  if (bucket_mode) *bucket_mode = best_mode;
  return MG_OK;
}

}  // extern "C"
