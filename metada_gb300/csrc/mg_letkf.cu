// Batched LETKF local analyses (replaces LETKF.hpp:101 grid loop and
// updateGridPoint :152-243) and the sequential reference-order LETKF.
//
// One CTA (256 threads) runs one local analysis at a time, inside a
// persistent grid that pulls analysis points from a work counter in the
// grid's column order (neighbouring columns at the same time, so their
// shared candidates stay in L2); with thousands of points per CTA the
// uneven local-observation counts balance across SMs without any
// device-side wait.
//
// Per analysis: the column's candidate list is filtered (vertical support)
// and weighted (Gaspari-Cohn x 1/sigma^2, or 1 for the reference's R = I),
// the local rows of Y' are gathered chunk by chunk into shared memory and
// the k x k Gram Y'^T R^-1 Y' accumulated in a 16 x 16 grid of register
// tiles; the k x k transform comes from a Cholesky path (reference) or the
// parallel Jacobi eigen-solver (Hunt), and the update is applied to every
// variable of the point.
//
// TE is the arithmetic type of the Gram, eigen-solve and update: double for
// the FP64 path, float for the mixed path (means, innovations and outputs
// stay double).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mg_dense.cuh"
#include "mg_internal.h"
#include "mg_letkf.cuh"

namespace {

using mg::LetkfParams;
using mg::gaspari_cohn;

constexpr int kThreads = 256;
constexpr int kNVarMax = 8;
// Off-diagonal threshold of the loose first Jacobi stage (relative to
// sqrt(a_pp a_qq)); the second-order finish below leaves a remainder of
// order k^2 kStage1Tol^3.
constexpr double kStage1Tol = 1e-3;

// a / b by the hardware reciprocal for FP32 (a few ulp), exact for FP64.
__device__ __forceinline__ float fast_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fast_div(double a, double b) { return a / b; }

// Shared-memory plan of one CTA: A and V (k x k, padded rows), one chunk of
// gathered Y' rows (Ys) and, for the FP32 two-stage eigen-solve (k <= 96),
// one chunk of rotated rows (Bc); 32-row chunks keep the FP32 plan near
// 54 KB so four CTAs share an SM.
template <typename TE, int KMAX>
struct Plan {
  static constexpr bool TWO_STAGE = sizeof(TE) == 4 && KMAX <= 96;
  static constexpr int LDA = KMAX + 1;
  // The two-stage path's first Jacobi keeps its eigenvectors as float4 rows
  // (cta_jacobi_tri), so the V region has rows of LDV (multiple of 4).
  static constexpr int LDV = TWO_STAGE ? KMAX + 4 : LDA;
  static constexpr int CH = 32;                    // list chunk rows
  static constexpr int NCHUNK = TWO_STAGE ? 2 : 1;  // Ys (, Bc)
  static constexpr size_t te_count() {
    return (size_t)KMAX * LDA + (size_t)KMAX * LDV + (size_t)NCHUNK * CH * KMAX + 2 * CH + 4 * KMAX + 2 * KMAX +
           kNVarMax * KMAX;
  }
  static constexpr size_t bytes() {
    return sizeof(TE) * te_count() + sizeof(double) * (2 * kNVarMax) + sizeof(int) * (CH + KMAX + 16) + 64;
  }
};

// Walks the candidate list of column `col` for analysis level `lev` in
// chunks of CH entries: filters by vertical support, weights (Gaspari-Cohn x
// 1/sigma^2, or 1 for R = I), compacts the kept entries and gathers their Y'
// rows into Ys (zero-padded to KMAX columns); then calls body(cnt) with the
// chunk ready in shared memory.  Returns the number of local obs.
template <typename TE, int KMAX, int CH, typename Body>
__device__ int for_each_chunk(const LetkfParams& prm, int64_t e0, int64_t e1, int lev, TE* Ys, int* sel_o,
                              TE* sel_r, TE* sel_d, int* wcnt, Body&& body) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k = prm.k;
  const TE* Y = static_cast<const TE*>(prm.Y);
  const bool r_identity = prm.flags & MG_R_IDENTITY;
  const TE hc = (TE)(0.5 * prm.hsupport), vc = (TE)(0.5 * prm.vsupport), vs = (TE)prm.vsupport;
  int nloc = 0;
  for (int64_t c0 = e0; c0 < e1; c0 += CH) {
    bool keep = false;
    int o = 0;
    TE rw = TE(0), dd = TE(0);
    if (tid < CH && c0 + tid < e1) {
      const int64_t e = c0 + tid;
      o = prm.loc_idx[e];
      TE w = TE(1);
      keep = true;
      if (prm.obs_lev) {
        const TE dl = fabs((TE)lev - (TE)prm.obs_lev[o]);
        if (dl > vs) keep = false;
        else if (!r_identity) w *= gaspari_cohn<TE>(dl / vc);
      }
      if (keep && !r_identity) {
        if (prm.loc_dist) w *= gaspari_cohn<TE>((TE)prm.loc_dist[e] / hc);
        w *= (TE)prm.rinv[o];
        if (!(w > TE(0))) keep = false;
      }
      rw = w;
      dd = (TE)prm.dinn[o];
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcnt[warp] = __popc(bal);
    __syncthreads();
    int wbase = 0, cnt = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
      if (w < warp) wbase += wcnt[w];
      cnt += wcnt[w];
    }
    if (keep) {
      const int pos = wbase + __popc(bal & ((1u << lane) - 1u));
      sel_o[pos] = o;
      sel_r[pos] = rw;
      sel_d[pos] = dd;
    }
    __syncthreads();
    for (int e = tid; e < cnt * KMAX; e += kThreads) {
      const int r = e / KMAX, j = e - r * KMAX;
      Ys[e] = (j < k) ? Y[(int64_t)sel_o[r] * k + j] : TE(0);
    }
    __syncthreads();
    body(cnt);
    nloc += cnt;
    __syncthreads();
  }
  return nloc;
}

// acc[a][b] += sum_r w_r M[r, ti + 16a] M[r, tj + 16b] over the rows of a
// chunk (interleaved tiles: a warp's loads hit consecutive words).
template <typename TE, int KMAX, int R>
__device__ __forceinline__ void gram_rows(TE (&acc)[R][R], const TE* M, const TE* w, int cnt, int ti, int tj) {
  for (int r = 0; r < cnt; ++r) {
    const TE wr = w ? w[r] : TE(1);
    TE av[R], bv[R];
#pragma unroll
    for (int a = 0; a < R; ++a) av[a] = M[r * KMAX + ti + 16 * a] * wr;
#pragma unroll
    for (int b = 0; b < R; ++b) bv[b] = M[r * KMAX + tj + 16 * b];
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
      for (int b = 0; b < R; ++b) acc[a][b] += av[a] * bv[b];
  }
}

template <typename TE, int KMAX>
__global__ void __launch_bounds__(kThreads, (sizeof(TE) == 4 && KMAX <= 64) ? 4 : ((sizeof(TE) == 4 && KMAX <= 96) ? 2 : 1))
    letkf_batched_kernel(LetkfParams prm) {
  using P = Plan<TE, KMAX>;
  constexpr int LDA = P::LDA, CH = P::CH, R = KMAX / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TE* const A0 = reinterpret_cast<TE*>(smem_raw);
  TE* const V0 = A0 + KMAX * LDA;            // KMAX x LDV
  TE* Ys = V0 + KMAX * P::LDV;               // CH x KMAX
  TE* Bc = Ys + CH * KMAX;                   // two-stage only: CH x KMAX
  TE* sel_r = Ys + P::NCHUNK * CH * KMAX;    // CH
  TE* sel_d = sel_r + CH;                    // CH
  TE* bvec = sel_d + CH;                     // KMAX
  TE* wa = bvec + KMAX;                      // KMAX
  TE* uvec = wa + KMAX;                      // KMAX
  TE* lam = uvec + KMAX;                     // KMAX
  TE* rot = lam + KMAX;                      // 2*KMAX (4 per pair)
  TE* Xs = rot + 2 * KMAX;                   // kNVarMax x KMAX
  double* xm = reinterpret_cast<double*>(Xs + kNVarMax * KMAX);  // kNVarMax
  double* red = xm + kNVarMax;                                   // kNVarMax
  int* sel_o = reinterpret_cast<int*>(red + kNVarMax);           // CH
  int* pairbuf = sel_o + CH;                                     // KMAX
  int* misc = pairbuf + KMAX;                                    // 16
  __shared__ long long s_item;
  __shared__ int wcnt[kThreads / 32];

  const int tid = threadIdx.x;
  const int k = prm.k, kp = prm.kp;
  const TE* Xp = static_cast<const TE*>(prm.Xp);
  const int ti = tid / 16, tj = tid % 16;
  const bool use_chol = prm.flags & MG_SQRT_CHOLESKY;
  const bool infl_compat = prm.flags & MG_INFL_COMPAT;
  const bool upd_compat = prm.flags & MG_UPDATE_COMPAT;
  const bool rtps = prm.flags & MG_RTPS;
  const bool two_stage = P::TWO_STAGE && !use_chol;

  // Cold: one work item per (column, level).  Warm start: one item per
  // column, its levels analysed in sequence by this CTA, each eigen-solve
  // starting from the previous level's eigenvectors (kept in V).
  const bool warm_mode = prm.warm_start != 0 && !use_chol;
  const long long nitems = warm_mode ? prm.ncol : prm.npoints;
  long long item = 0;
  int lev = prm.nlev;
  bool have_basis = false;
  for (;;) {
    if (!warm_mode || lev + 1 >= prm.nlev) {
      if (tid == 0) s_item = (long long)atomicAdd(prm.next, 1ull);
      __syncthreads();
      item = s_item;
      __syncthreads();
      if (item >= nitems) break;
      lev = warm_mode ? 0 : (int)(item % prm.nlev);
      have_basis = false;
    } else {
      ++lev;
    }
    // The two-stage path may exchange the roles of the A and V regions.
    TE* A = A0;
    TE* V = V0;
    int64_t col;
    if (prm.redo_in) {
      const int32_t pt = prm.redo_in[item];
      col = pt / prm.nlev;
      lev = pt % prm.nlev;
    } else {
      col = warm_mode ? prm.order[item] : prm.order[item / prm.nlev];
    }
    const int64_t base = prm.col_base[col] + (int64_t)lev * prm.lev_stride;
    const int64_t e0 = prm.loc_off[col], e1 = prm.loc_off[col + 1];

    // ---- Gram G = Y'^T R^-1 Y' and b = Y'^T R^-1 d ----
    TE acc[R][R];
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
      for (int b = 0; b < R; ++b) acc[a][b] = TE(0);
    TE bacc = TE(0);
    const int nloc = for_each_chunk<TE, KMAX, CH>(prm, e0, e1, lev, Ys, sel_o, sel_r, sel_d, wcnt, [&](int cnt) {
      gram_rows<TE, KMAX, R>(acc, Ys, sel_r, cnt, ti, tj);
      if (tid < k)
        for (int r = 0; r < cnt; ++r) bacc += (Ys[r * KMAX + tid] * sel_r[r]) * sel_d[r];
    });

    if (nloc == 0) {
      // LETKF.hpp:167-190: no local obs, x' *= sqrt(rho) (RTPS: unchanged).
      const double sr = rtps ? 1.0 : sqrt(prm.rho);
      for (int e = tid; e < prm.n_var * k; e += kThreads) {
        const int v = e / k, i = e - v * k;
        const int64_t s = base + (int64_t)v * prm.var_stride;
        mg::letkf_store(prm, s * k + i, prm.xmean[s] + (double)Xp[s * k + i] * sr);
      }
      if (tid == 0) atomicAdd(prm.n_empty, 1ull);
      __syncthreads();
      continue;
    }

    // ---- k x k system ----
    const TE diag = (infl_compat || rtps) ? TE(k - 1) : TE((double)(k - 1) / prm.rho);
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
      for (int b = 0; b < R; ++b) {
        const int i = ti + 16 * a, j = tj + 16 * b;
        if (i < kp && j < kp) {
          TE v = (i < k && j < k) ? acc[a][b] : TE(0);
          if (i == j) v += (i < k) ? diag : TE(1);
          A[i * LDA + j] = v;
        }
      }
    if (tid < k) bvec[tid] = bacc;
    __syncthreads();

    int sweeps = 0;
    bool ok = true;
    if (!two_stage) {
      ok = mg::solve_transform<TE, KMAX, kThreads>(A, V, bvec, wa, lam, uvec, rot, pairbuf, misc, k, kp, LDA, use_chol,
                                   infl_compat, prm.rho, (TE)prm.tol, prm.sweep_cap, &sweeps,
                                   warm_mode && have_basis, Ys, CH - 1);
      have_basis = !use_chol;
    } else {
      // Stage 1: loose Jacobi on A = diag I + G gives a basis V1 in which A
      // is nearly diagonal.
      const bool warm = warm_mode && have_basis;
      if constexpr (P::TWO_STAGE) {
        static_assert((KMAX * LDA + KMAX * P::LDV + P::NCHUNK * CH * KMAX + 2 * CH + 2 * KMAX) % 4 == 0,
                      "rotation buffer must be 16-byte aligned");
        if (!warm_mode) {
          sweeps = mg::cta_jacobi_tri<KMAX, kThreads>(A, LDA, V, P::LDV, kp, (float)kStage1Tol, prm.sweep_cap,
                                                      reinterpret_cast<float4*>(uvec));
          // Eigenvector rows -> row-major V in the A region (A is not needed
          // any more), then the regions exchange roles.
          for (int e = tid; e < kp * kp; e += kThreads) {
            const int j = e / kp, i = e - j * kp;
            A[i * LDA + j] = V[j * P::LDV + i];
          }
          __syncthreads();
          TE* t = A;
          A = V;
          V = t;
        } else {
          if (warm) mg::cta_similarity<TE>(A, V, kp, LDA, Ys, CH - 1);
          sweeps = mg::cta_jacobi_fast<TE, KMAX, kThreads>(A, V, kp, LDA, TE(kStage1Tol), prm.sweep_cap, rot,
                                                           pairbuf, !warm);
        }
      } else {
        if (warm) mg::cta_similarity<TE>(A, V, kp, LDA, Ys, CH - 1);
        sweeps = mg::cta_jacobi_fast<TE, KMAX, kThreads>(A, V, kp, LDA, TE(kStage1Tol), prm.sweep_cap, rot, pairbuf,
                                                         !warm);
      }
      // V1 back to orthogonal (A is free until the rebuild below).
      mg::cta_reorthonormalize<TE, KMAX>(V, kp, LDA, A, Ys, CH);
      // Stage 2: rebuild A2 = V1^T A V1 from the factor, diag I + B^T B with
      // B = R^-1/2 Y' V1, chunk by chunk.  Entries of B^T B carry errors
      // relative to the column norms of B, so the small eigenvalues keep
      // their relative accuracy (no eps * cond(A) loss from rounding A).
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] = TE(0);
      for_each_chunk<TE, KMAX, CH>(prm, e0, e1, lev, Ys, sel_o, sel_r, sel_d, wcnt, [&](int cnt) {
        {  // Bc = diag(sqrt w) Ys V: warp w owns rows 4w..4w+3, lane the columns lane + 32c
          constexpr int RW = CH / (kThreads / 32), CW = KMAX / 32;
          const int wrp = tid >> 5, ln = tid & 31;
          TE sacc[RW][CW];
#pragma unroll
          for (int x = 0; x < RW; ++x)
#pragma unroll
            for (int c = 0; c < CW; ++c) sacc[x][c] = TE(0);
          for (int m = 0; m < k; ++m) {
            TE yv[RW], vv[CW];
#pragma unroll
            for (int x = 0; x < RW; ++x) yv[x] = Ys[(wrp * RW + x) * KMAX + m];
#pragma unroll
            for (int c = 0; c < CW; ++c) vv[c] = V[m * LDA + ln + 32 * c];
#pragma unroll
            for (int x = 0; x < RW; ++x)
#pragma unroll
              for (int c = 0; c < CW; ++c) sacc[x][c] += yv[x] * vv[c];
          }
#pragma unroll
          for (int x = 0; x < RW; ++x) {
            const int r = wrp * RW + x;
            if (r < cnt) {
              const TE sw = sqrt(sel_r[r]);
#pragma unroll
              for (int c = 0; c < CW; ++c) {
                const int j = ln + 32 * c;
                Bc[r * KMAX + j] = (j < k) ? sacc[x][c] * sw : TE(0);
              }
            }
          }
        }
        __syncthreads();
        gram_rows<TE, KMAX, R>(acc, Bc, nullptr, cnt, ti, tj);
      });
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
          const int i = ti + 16 * a, j = tj + 16 * b;
          if (i < kp && j < kp) {
            TE v = (i < k && j < k) ? acc[a][b] : TE(0);
            if (i == j) v += (i < k) ? diag : TE(1);
            A[i * LDA + j] = v;
          }
        }
      __syncthreads();
      // Stage 3: A2 = D + E is nearly diagonal (|E_ij| <= kStage1Tol
      // sqrt(d_i d_j) after stage 1, V1 orthonormal to FP32 rounding), so
      // f(A2) for f = x^-1/2 and x^-1 is taken to second order by the
      // Daleckii-Krein expansion
      //   f(D + E)_ij = f(d_i) delta_ij + f[d_i, d_j] E_ij
      //                 + sum_m f[d_i, d_m, d_j] E_im E_mj + O(|E|^3),
      // with the divided differences in closed form (no cancellation),
      // s = sqrt(d):
      //   x^-1/2: f[a,b] = -1 / (s_a s_b (s_a + s_b)),
      //           f[a,b,c] = (s_a + s_b + s_c) / (s_a s_b s_c (s_a + s_b) (s_b + s_c) (s_a + s_c));
      //   x^-1:   f[a,b] = -1 / (a b),  f[a,b,c] = 1 / (a b c).
      // For x^-1/2 the second-order sum splits by partial fractions into
      //   h_ij S_ij,  h_ij = 1 / (s_i s_j (s_i + s_j)),
      //   S_ij = sum_m [P_im E_mj + E_im P_mj] / s_m - P_im P_mj,  P_im = E_im / (s_i + s_m),
      // two k^3 products, run register-tiled (no eigen-sweep barriers).
      for (int i = tid; i < k; i += kThreads) {
        const TE l = A[i * LDA + i];
        lam[i] = l;
        if (!(l > TE(0)) || !(l < TE(3.0e38))) atomicExch(prm.status, 1);
      }
      __syncthreads();
      have_basis = true;
      const TE sc = infl_compat ? (TE)prm.rho : TE(1);
      TE* gvec = rot;        // k values; the Jacobi rotation buffer is free now
      TE* sv = rot + KMAX;   // s = sqrt(d)
      TE* yv = Bc;           // D^-1 u; the rebuild buffer is free now
      TE* zv = Bc + KMAX;    // z = E D^-1 u
      TE* zq = Bc + 2 * KMAX;  // D^-1 z
      for (int i = tid; i < k; i += kThreads) {  // u = V1^T b
        TE s = TE(0);
        for (int j = 0; j < k; ++j) s += V[j * LDA + i] * bvec[j];
        uvec[i] = s;
        yv[i] = s / lam[i];
        sv[i] = mg::dsqrt<TE>(lam[i]);
      }
      __syncthreads();
      for (int i = tid; i < k; i += kThreads) {
        TE z = TE(0);
        for (int j = 0; j < k; ++j)
          if (j != i) z += A[i * LDA + j] * yv[j];
        zv[i] = z;
        zq[i] = z / lam[i];
      }
      __syncthreads();
      for (int i = tid; i < k; i += kThreads) {  // g = (sc x^-1)(A2) u = sc D^-1 (u - z + E D^-1 z)
        TE w = TE(0);
        for (int m = 0; m < k; ++m)
          if (m != i) w += A[i * LDA + m] * zq[m];
        gvec[i] = (uvec[i] - zv[i] + w) * sc / lam[i];
      }
      __syncthreads();
      for (int i = tid; i < k; i += kThreads) {  // wa = V1 g
        TE s = TE(0);
        for (int m = 0; m < k; ++m) s += V[i * LDA + m] * gvec[m];
        wa[i] = s;
      }
      {
        // S (second-order sum) for the thread's R x R block: rows
        // i = ti + 16 a, columns j = tj + 16 b, as the Gram tiles.
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
          for (int b = 0; b < R; ++b) acc[a][b] = TE(0);
        TE si_[R], sj_[R];
#pragma unroll
        for (int a = 0; a < R; ++a) {
          const int i = ti + 16 * a, j = tj + 16 * a;
          si_[a] = i < k ? sv[i] : TE(1);
          sj_[a] = j < k ? sv[j] : TE(1);
        }
        // (approximate divisions: these scale a correction of order
        // kStage1Tol^2, a few ulp of it is far below the result's rounding)
        for (int m = 0; m < k; ++m) {
          const TE sm = sv[m], ism = fast_div(TE(1), sm);
          TE emj[R], pmj[R];
#pragma unroll
          for (int b = 0; b < R; ++b) {
            const int j = tj + 16 * b;
            emj[b] = (j < k && j != m) ? A[m * LDA + j] : TE(0);
            pmj[b] = fast_div(emj[b], sm + sj_[b]);
          }
#pragma unroll
          for (int a = 0; a < R; ++a) {
            const int i = ti + 16 * a;
            const TE eim = (i < k && i != m) ? A[i * LDA + m] : TE(0);
            const TE pim = fast_div(eim, si_[a] + sm);
#pragma unroll
            for (int b = 0; b < R; ++b) acc[a][b] += (pim * emj[b] + eim * pmj[b]) * ism - pim * pmj[b];
          }
        }
        __syncthreads();  // every read of E done
        // A <- Wb = (c x^-1/2)(A2), c = sqrt((k-1) sc); W = V1 Wb V1^T is
        // never formed: the update applies X' V1, then Wb, then V1^T.
        const TE cw = mg::dsqrt<TE>(TE(k - 1) * sc);
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
          for (int b = 0; b < R; ++b) {
            const int i = ti + 16 * a, j = tj + 16 * b;
            if (i < k && j < k) {
              const TE h = TE(1) / (si_[a] * sj_[b] * (si_[a] + sj_[b]));
              const TE first = (i == j) ? TE(1) / si_[a] : -A[i * LDA + j] * h;
              A[i * LDA + j] = cw * (first + acc[a][b] * h);
            }
          }
      }
      __syncthreads();
      if (upd_compat) {  // row sums of W = V1 Wb V1^T 1, kept in uvec
        for (int i = tid; i < k; i += kThreads) {
          TE s = TE(0);
          for (int m = 0; m < k; ++m) s += V[m * LDA + i];
          gvec[i] = s;  // V1^T 1
        }
        __syncthreads();
        for (int i = tid; i < k; i += kThreads) {
          TE s = TE(0);
          for (int m = 0; m < k; ++m) s += A[i * LDA + m] * gvec[m];
          lam[i] = s;  // Wb V1^T 1 (lam is not needed any more)
        }
        __syncthreads();
        for (int i = tid; i < k; i += kThreads) {
          TE s = TE(0);
          for (int m = 0; m < k; ++m) s += V[i * LDA + m] * lam[m];
          uvec[i] = s;
        }
        __syncthreads();
      }
    }
    if (!ok && tid == 0) atomicExch(prm.status, 1);

    // ---- update every variable of the point, kNVarMax at a time ----
    for (int v0 = 0; v0 < prm.n_var; v0 += kNVarMax) {
    const int nv = (prm.n_var - v0 < kNVarMax) ? prm.n_var - v0 : kNVarMax;
    for (int e = tid; e < nv * k; e += kThreads) {
      const int v = e / k, i = e - v * k;
      Xs[v * KMAX + i] = Xp[(base + (int64_t)(v0 + v) * prm.var_stride) * k + i];
    }
    if (tid < nv) xm[tid] = prm.xmean[base + (int64_t)(v0 + tid) * prm.var_stride];
    __syncthreads();
    if (two_stage) {  // P = ((X' V1) Wb) V1^T, two nv x KMAX buffers in Bc
      TE* P1 = Bc;
      TE* P2 = Bc + kNVarMax * KMAX;
      if (!upd_compat) {
        for (int e = tid; e < nv * k; e += kThreads) {
          const int v = e / k, j = e - v * k;
          TE s = TE(0);
          for (int m = 0; m < k; ++m) s += Xs[v * KMAX + m] * V[m * LDA + j];
          P1[v * KMAX + j] = s;
        }
        __syncthreads();
        for (int e = tid; e < nv * k; e += kThreads) {
          const int v = e / k, j = e - v * k;
          TE s = TE(0);
          for (int m = 0; m < k; ++m) s += P1[v * KMAX + m] * A[m * LDA + j];
          P2[v * KMAX + j] = s;
        }
        __syncthreads();
      }
      for (int e = tid; e < nv * k; e += kThreads) {
        const int v = e / k, i = e - v * k;
        const TE* x = Xs + v * KMAX;
        double out;
        if (upd_compat) {  // xa_i = (xm + x'_i wa_i) + x'_i sum_j W_ij, LETKF.hpp:232-238
          const TE xp = x[i];
          out = (xm[v] + (double)(xp * wa[i])) + (double)(xp * uvec[i]);
        } else {
          TE inc = TE(0), s2 = TE(0);
          for (int j = 0; j < k; ++j) inc += x[j] * wa[j];
          for (int m = 0; m < k; ++m) s2 += P2[v * KMAX + m] * V[i * LDA + m];
          out = (xm[v] + (double)inc) + (double)s2;
          if (rtps) Ys[v * KMAX + i] = s2;  // analysis perturbation for the spread
        }
        mg::letkf_store(prm, (base + (int64_t)(v0 + v) * prm.var_stride) * k + i, out);
      }
    } else
    for (int e = tid; e < nv * k; e += kThreads) {
      const int v = e / k, i = e - v * k;
      const TE* x = Xs + v * KMAX;
      double out;
      if (upd_compat) {  // xa_i = (xm + x'_i wa_i) + sum_j x'_i W_ij, LETKF.hpp:232-238
        const TE xp = x[i];
        TE rs = TE(0);
        for (int j = 0; j < k; ++j) rs += xp * A[i * LDA + j];
        out = (xm[v] + (double)(xp * wa[i])) + (double)rs;
      } else {  // xa_i = xm + sum_j x'_j (wa_j + W_ji)
        TE inc = TE(0), s2 = TE(0);
        for (int j = 0; j < k; ++j) {
          inc += x[j] * wa[j];
          s2 += x[j] * A[j * LDA + i];
        }
        out = (xm[v] + (double)inc) + (double)s2;
        if (rtps) Ys[v * KMAX + i] = s2;  // analysis perturbation for the spread
      }
      mg::letkf_store(prm, (base + (int64_t)(v0 + v) * prm.var_stride) * k + i, out);
    }
    if (rtps && !upd_compat) {
      __syncthreads();
      if (tid < nv) {
        double sb = 0.0, sa = 0.0;
        for (int i = 0; i < k; ++i) {
          const double xb = (double)Xs[tid * KMAX + i], xa = (double)Ys[tid * KMAX + i];
          sb += xb * xb;
          sa += xa * xa;
        }
        sb = sqrt(sb / (k - 1));
        sa = sqrt(sa / (k - 1));
        red[tid] = (sa > 0.0) ? prm.rho * (sb - sa) / sa : 0.0;  // factor - 1
      }
      __syncthreads();
      for (int e = tid; e < nv * k; e += kThreads) {
        const int v = e / k, i = e - v * k;
        mg::letkf_add(prm, (base + (int64_t)(v0 + v) * prm.var_stride) * k + i, red[v] * (double)Ys[v * KMAX + i]);
      }
    }
    __syncthreads();
    }
    if (tid == 0) {
      atomicAdd(prm.total_local, (unsigned long long)nloc);
      atomicAdd(prm.total_sweeps, (unsigned long long)sweeps);
      atomicMax(prm.max_local, nloc);
      atomicMax(prm.max_sweeps, sweeps);
    }
    __syncthreads();
  }
}

// Per-observation FP32 pack for the tensor-core kernel: (level, 1/sigma^2,
// innovation, 0), one 16-byte gather per candidate instead of three.
__global__ void obs_pack_kernel(const double* __restrict__ obs_lev, const double* __restrict__ rinv,
                                const double* __restrict__ dinn, int64_t p, float4* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p; o += stride)
    out[o] = make_float4(obs_lev ? (float)obs_lev[o] : 0.0f, (float)rinv[o], (float)dinn[o], 0.0f);
}

// Level bucket of each observation for the tensor-core path's sorted lists:
// floor(level) clamped to [0, nlev - 1] (non-finite levels to 0; the
// analyses that use the buckets drop them with a zero weight anyway).
__global__ void obs_bucket_kernel(const double* __restrict__ obs_lev, int64_t p, int nlev,
                                  uint8_t* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p; o += stride) {
    const double l = obs_lev[o];
    int b = 0;
    if (l == l) {
      const double f = floor(l);
      b = (f <= 0.0) ? 0 : ((f >= (double)(nlev - 1)) ? nlev - 1 : (int)f);
    }
    out[o] = (uint8_t)b;
  }
}

// Stable counting sort of each column's candidate list by level bucket, one
// warp per column: counts per bucket (lanes of one bucket found with
// match_any, the lowest of them adds the group's size), the bucket starts
// (relative to the column's start) to boff, then the entries scattered in
// list order within each bucket.  nlev <= kBucketMaxLev.
constexpr int kBucketMaxLev = 64;
__global__ void __launch_bounds__(256) level_bucket_kernel(const int64_t* __restrict__ off,
                                                           const int32_t* __restrict__ idx,
                                                           const double* __restrict__ dist,
                                                           const uint8_t* __restrict__ obkt, int nlev, int64_t ncol,
                                                           int32_t* __restrict__ idx2, double* __restrict__ dist2,
                                                           int32_t* __restrict__ boff) {
  __shared__ int cur[8][kBucketMaxLev];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int* c = cur[w];
  const int64_t nwarps = (int64_t)gridDim.x * 8;
  for (int64_t col = (int64_t)blockIdx.x * 8 + w; col < ncol; col += nwarps) {
    const int64_t e0 = off[col], e1 = off[col + 1];
    for (int b = lane; b < nlev; b += 32) c[b] = 0;
    __syncwarp();
    for (int64_t e = e0; e < e1; e += 32) {
      const bool v = e + lane < e1;
      const int b = v ? (int)obkt[idx[e + lane]] : 255;  // 255: no bucket
      const unsigned m = __match_any_sync(0xffffffffu, b);
      if (v && lane == __ffs(m) - 1) c[b] += __popc(m);
      __syncwarp();
    }
    if (lane == 0) {
      int run = 0;
      int32_t* bo = boff + col * (int64_t)(nlev + 1);
      for (int b = 0; b < nlev; ++b) {
        bo[b] = run;
        const int t = c[b];
        c[b] = run;
        run += t;
      }
      bo[nlev] = run;
    }
    __syncwarp();
    for (int64_t e = e0; e < e1; e += 32) {
      const bool v = e + lane < e1;
      const int o = v ? idx[e + lane] : 0;
      const int b = v ? (int)obkt[o] : 255;
      const unsigned m = __match_any_sync(0xffffffffu, b);
      const int pos = v ? c[b] + __popc(m & ((1u << lane) - 1u)) : 0;
      __syncwarp();
      if (v) {
        idx2[e0 + pos] = o;
        if (dist) dist2[e0 + pos] = dist[e + lane];
        if (lane == __ffs(m) - 1) c[b] += __popc(m);
      }
      __syncwarp();
    }
  }
}

// Work order of the columns: the grid's own order, so the CTAs that run at
// the same time analyse neighbouring columns, whose candidate obs (and
// their Y' rows) overlap and stay in L2.  Every CTA analyses thousands of
// points, so the persistent grid needs no longest-first order to balance
// its tail (measured: 1.2 % faster than longest first on the 2.6M-value
// configuration).
__global__ void column_order_kernel(int64_t ncol, int32_t* __restrict__ order) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncol) order[c] = (int32_t)c;
}

template <typename TE, int KMAX>
int launch_batched(mg_context* ctx, LetkfParams& prm) {
  const size_t smem = Plan<TE, KMAX>::bytes();
  if (smem > 227 * 1024) return mg::fail(ctx, MG_ERR_ARG, "mg_letkf_batched: k too large for this precision");
  MG_TRY_CUDA(cudaFuncSetAttribute(letkf_batched_kernel<TE, KMAX>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  MG_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, letkf_batched_kernel<TE, KMAX>,
                                                            kThreads, smem));
  if (per_sm < 1) return mg::fail(ctx, MG_ERR_ARG, "mg_letkf_batched: kernel does not fit on an SM");
  int64_t grid = (int64_t)per_sm * ctx->num_sms;
  if (grid > prm.npoints) grid = prm.npoints;
  if (grid < 1) grid = 1;
  letkf_batched_kernel<TE, KMAX><<<(unsigned)grid, kThreads, smem, ctx->stream>>>(prm);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

// ------------------------------------------------------------------------
// Sequential LETKF in the reference's order (LETKF.hpp:101), one CTA.
// ------------------------------------------------------------------------
struct CompatSeqParams {
  double* X;
  int k, nx, ny;
  int64_t ld;
  const int32_t* obs_xy;
  const uint8_t* valid;
  const double* yo;
  const int64_t* loc_off;
  const int32_t* loc_idx;
  double rho;
  int* status;
};

__device__ __forceinline__ double idw4_seq(const double* x, int nx, int ny, int ox, int oy) {
  const double xx = fmax(0.0, fmin((double)(nx - 1), (double)ox));
  const double yy = fmax(0.0, fmin((double)(ny - 1), (double)oy));
  const long long i0 = (long long)floor(xx), j0 = (long long)floor(yy);
  const long long i1 = min(i0 + 1, (long long)nx - 1), j1 = min(j0 + 1, (long long)ny - 1);
  const long long ii[4] = {i0, i1, i0, i1}, jj[4] = {j0, j0, j1, j1};
  double ws = 0.0, wsum = 0.0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const double dx = __dsub_rn(xx, (double)ii[t]), dy = __dsub_rn(yy, (double)jj[t]);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    const double w = (dist == 0.0) ? 1e12 : __ddiv_rn(1.0, dist);
    ws = __dadd_rn(ws, __dmul_rn(w, x[jj[t] * nx + ii[t]]));
    wsum = __dadd_rn(wsum, w);
  }
  return __ddiv_rn(ws, wsum);
}

template <int KMAX>
__global__ void __launch_bounds__(kThreads) letkf_compat_seq_kernel(CompatSeqParams prm) {
  constexpr int LDA = KMAX + 1, CH = 64;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* A = reinterpret_cast<double*>(smem_raw);
  double* V = A + KMAX * LDA;
  double* Ys = V + KMAX * LDA;  // CH x KMAX
  double* dd = Ys + CH * KMAX;  // CH
  double* bvec = dd + CH;       // KMAX
  double* wa = bvec + KMAX;     // KMAX
  double* xb = wa + KMAX;       // KMAX
  int* misc = reinterpret_cast<int*>(xb + KMAX);
  __shared__ double s_xm;
  const int tid = threadIdx.x, k = prm.k;
  const int npt = prm.nx * prm.ny;
  const double sqk = sqrt((double)(k - 1));
  for (int g = 0; g < npt; ++g) {
    const int64_t e0 = prm.loc_off[g], e1 = prm.loc_off[g + 1];
    double acc[KMAX / 16][KMAX / 16];
    constexpr int R = KMAX / 16;
    const int ti = tid / 16, tj = tid % 16;
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
      for (int b = 0; b < R; ++b) acc[a][b] = 0.0;
    double bacc = 0.0;
    for (int64_t c0 = e0; c0 < e1; c0 += CH) {
      const int cnt = (int)(e1 - c0 < (int64_t)CH ? e1 - c0 : (int64_t)CH);
      // H_local rows from the CURRENT members (LETKF.hpp:197-206).
      for (int e = tid; e < cnt * KMAX; e += kThreads) {
        const int r = e / KMAX, j = e - r * KMAX;
        double v = 0.0;
        if (j < k) {
          const int o = prm.loc_idx[c0 + r];
          if (!prm.valid || prm.valid[o])
            v = idw4_seq(prm.X + (int64_t)j * prm.ld, prm.nx, prm.ny, prm.obs_xy[2 * o],
                         prm.obs_xy[2 * o + 1]);
        }
        Ys[e] = v;
      }
      __syncthreads();
      if (tid < cnt) {  // row mean, anomalies, innovation (:209-211)
        double s = 0.0;
        for (int j = 0; j < k; ++j) s += Ys[tid * KMAX + j];
        const double ym = s / (double)k;
        for (int j = 0; j < k; ++j) Ys[tid * KMAX + j] -= ym;
        dd[tid] = prm.yo[prm.loc_idx[c0 + tid]] - ym;
      }
      __syncthreads();
      for (int r = 0; r < cnt; ++r) {
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
          for (int b = 0; b < R; ++b)
            acc[a][b] += Ys[r * KMAX + ti + 16 * a] * Ys[r * KMAX + tj + 16 * b];
      }
      if (tid < k)
        for (int r = 0; r < cnt; ++r) bacc += Ys[r * KMAX + tid] * dd[r];
      __syncthreads();
    }
    if (tid < k) xb[tid] = prm.X[(int64_t)tid * prm.ld + g];
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s += xb[i];
      s_xm = s / (double)k;
    }
    __syncthreads();
    const double xm = s_xm;
    if (e1 == e0) {  // LETKF.hpp:167-190
      const double sr = sqrt(prm.rho);
      if (tid < k) prm.X[(int64_t)tid * prm.ld + g] = xm + (xb[tid] - xm) * sr;
      __syncthreads();
      continue;
    }
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
      for (int b = 0; b < R; ++b) {
        const int i = ti + 16 * a, j = tj + 16 * b;
        if (i < k && j < k) A[i * LDA + j] = acc[a][b] + (i == j ? (double)(k - 1) : 0.0);
      }
    if (tid < k) bvec[tid] = bacc;
    __syncthreads();
    bool ok = mg::cta_cholesky<double>(A, k, LDA, misc);
    mg::cta_lower_inverse<double>(A, V, k, LDA);
    mg::cta_gram_of_lower<double>(V, A, k, LDA);
    for (int e = tid; e < k * k; e += kThreads) A[(e / k) * LDA + e % k] *= prm.rho;
    __syncthreads();
    if (tid < k) {
      double s = 0.0;
      for (int j = 0; j < k; ++j) s += A[tid * LDA + j] * bvec[j];
      wa[tid] = s;
    }
    __syncthreads();
    ok = mg::cta_cholesky<double>(A, k, LDA, misc) && ok;
    if (!ok && tid == 0) atomicExch(prm.status, 1);
    if (tid < k) {  // :227-242, in place
      const double xp = xb[tid] - xm;
      double rs = 0.0;
      for (int j = 0; j < k; ++j) rs += xp * (sqk * A[tid * LDA + j]);
      prm.X[(int64_t)tid * prm.ld + g] = (xm + xp * wa[tid]) + rs;
    }
    __syncthreads();
  }
}

}  // namespace

extern "C" {

int mg_letkf_batched(mg_context* ctx, const mg_letkf_desc* d) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(d != nullptr, "mg_letkf_batched: null descriptor");
  MG_CHECK_ARG(d->X && d->n > 0 && d->ld >= d->n && d->k >= 2 && d->k <= 128 && d->n_var >= 1 &&
                   d->nlev >= 1 && d->ncol >= 1 && d->col_base &&
                   d->p >= 0 && d->loc_off && (d->p == 0 || (d->HX && d->yo && d->rvar)) &&
                   d->rho > 0.0,
               "mg_letkf_batched: bad descriptor");
  MG_CHECK_ARG(d->precision == MG_PREC_FP64 || d->precision == MG_PREC_MIXED,
               "mg_letkf_batched: bad precision");
  MG_CHECK_ARG(!(d->flags & MG_RTPS) || !(d->flags & MG_UPDATE_COMPAT),
               "mg_letkf_batched: RTPS needs the Hunt update");
  const bool fp64 = d->precision == MG_PREC_FP64;
  const int k = d->k;
  MG_CHECK_ARG(!fp64 || k <= 96, "mg_letkf_batched: FP64 path supports k <= 96");
  MG_CHECK_ARG(d->x_dtype == MG_DTYPE_F64 || d->x_dtype == MG_DTYPE_F32, "mg_letkf_batched: bad x_dtype");
  // Members stored as FP32: the mixed path only, analysis written over the
  // FP32 perturbations (no FP64 point-major copy) and back as FP32.
  const bool x32 = d->x_dtype == MG_DTYPE_F32;
  MG_CHECK_ARG(!x32 || !fp64, "mg_letkf_batched: FP32 members need the mixed precision path");
  const int64_t n = d->n, p = d->p;
  const int64_t npoints = d->ncol * d->nlev;
  const size_t te = fp64 ? sizeof(double) : sizeof(float);
  // Level-bucketed candidate lists for the tensor-core path (it filters by
  // obs level with Gaspari-Cohn weights, so candidates outside the vertical
  // support never count): an analysis then walks about (2 vsupport + 1) /
  // nlev of its column's list instead of all of it.
  const bool bucket = !fp64 && !(d->flags & (MG_SOLVE_SIMT | MG_R_IDENTITY | MG_SQRT_CHOLESKY | MG_UPDATE_COMPAT |
                                             MG_WARM_START)) &&
                      k <= 96 && d->obs_lev && p > 0 && d->nlev >= 2 && d->nlev <= kBucketMaxLev &&
                      std::isfinite(d->vsupport) && d->vsupport >= 0.0;
  int64_t n_entries = 0;
  if (bucket) {
    MG_TRY_CUDA(cudaMemcpyAsync(&n_entries, d->loc_off + d->ncol, sizeof(n_entries), cudaMemcpyDeviceToHost,
                                ctx->stream));
    MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    MG_CHECK_ARG(n_entries >= 0, "mg_letkf_batched: bad candidate offsets");
  }
  mg::Carver cv;
  cv.reserve<char>((size_t)n * k * te);            // Xp
  cv.reserve<double>((size_t)n);                   // mean
  cv.reserve<double>(x32 ? 1 : (size_t)n * k);     // Xa (FP64 members only)
  cv.reserve<char>((size_t)(p + 1) * k * te);      // Y
  cv.reserve<double>((size_t)p + 1);               // d
  cv.reserve<double>((size_t)p + 1);               // rinv
  cv.reserve<int32_t>((size_t)d->ncol);            // column order
  cv.reserve<unsigned long long>(8);               // counters
  cv.reserve<int32_t>((size_t)npoints);            // points handed back by the tensor-core path
  cv.reserve<float4>((size_t)p + 1);               // per-obs FP32 pack (tensor-core path)
  cv.reserve<uint8_t>(bucket ? (size_t)p + 1 : 1);                          // obs level buckets
  cv.reserve<int32_t>(bucket ? (size_t)d->ncol * (d->nlev + 1) : 1);       // bucket starts
  cv.reserve<int32_t>(bucket ? (size_t)n_entries + 1 : 1);                 // sorted obs indices
  cv.reserve<double>(bucket && d->loc_dist ? (size_t)n_entries + 1 : 1);   // sorted distances
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  void* Xp = cv.take<char>((size_t)n * k * te);
  double* mean = cv.take<double>((size_t)n);
  double* Xa = cv.take<double>(x32 ? 1 : (size_t)n * k);
  void* Y = cv.take<char>((size_t)(p + 1) * k * te);
  double* dinn = cv.take<double>((size_t)p + 1);
  double* rinv = cv.take<double>((size_t)p + 1);
  int32_t* order = cv.take<int32_t>((size_t)d->ncol);
  auto* cnt = cv.take<unsigned long long>(8);
  int32_t* redo = cv.take<int32_t>((size_t)npoints);
  float4* opack = cv.take<float4>((size_t)p + 1);
  uint8_t* obkt = cv.take<uint8_t>(bucket ? (size_t)p + 1 : 1);
  int32_t* lev_boff = cv.take<int32_t>(bucket ? (size_t)d->ncol * (d->nlev + 1) : 1);
  int32_t* bidx = cv.take<int32_t>(bucket ? (size_t)n_entries + 1 : 1);
  double* bdist = cv.take<double>(bucket && d->loc_dist ? (size_t)n_entries + 1 : 1);
  cudaStream_t s = ctx->stream;

  MG_TRY_CUDA(cudaEventRecord(ctx->ev[0], s));
  // Point-major perturbations and means (Ensemble.hpp:105-151).
  if (x32)
    MG_TRY_CUDA(mg::launch_to_point_major_f32(static_cast<const float*>(d->X), n, k, d->ld, mean, (float*)Xp, s));
  else
    MG_TRY_CUDA(mg::launch_to_point_major(static_cast<const double*>(d->X), n, k, d->ld, mean,
                                          fp64 ? (double*)Xp : nullptr, fp64 ? nullptr : (float*)Xp, s));
  // Obs-space prior from the background (snapshot).
  if (p > 0)
    MG_TRY_CUDA(mg::launch_obs_prior(d->HX, d->yo, d->rvar, p, k, fp64 ? (double*)Y : nullptr,
                                     fp64 ? nullptr : (float*)Y, dinn, rinv, s));
  // Column order of the work (grid order).
  column_order_kernel<<<(unsigned)((d->ncol + 255) / 256), 256, 0, s>>>(d->ncol, order);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  MG_TRY_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 8, s));

  LetkfParams prm{};
  prm.k = k;
  prm.kp = k + (k & 1);
  prm.n_var = d->n_var;
  prm.nlev = d->nlev;
  prm.ncol = d->ncol;
  prm.npoints = npoints;
  prm.col_base = d->col_base;
  prm.lev_stride = d->lev_stride;
  prm.var_stride = d->var_stride;
  prm.Xp = Xp;
  prm.xmean = mean;
  prm.Xa = x32 ? nullptr : Xa;
  prm.Xa32 = x32 ? static_cast<float*>(Xp) : nullptr;
  prm.Y = Y;
  prm.dinn = dinn;
  prm.rinv = rinv;
  prm.obs_lev = d->obs_lev;
  prm.loc_off = d->loc_off;
  prm.loc_idx = d->loc_idx;
  prm.loc_dist = d->loc_dist;
  prm.hsupport = d->hsupport;
  prm.vsupport = d->vsupport;
  prm.rho = d->rho;
  prm.flags = d->flags;
  prm.order = order;
  prm.next = cnt + 0;
  prm.n_empty = cnt + 1;
  prm.total_local = cnt + 2;
  prm.max_local = reinterpret_cast<int*>(cnt + 3);
  prm.max_sweeps = reinterpret_cast<int*>(cnt + 3) + 1;
  prm.status = reinterpret_cast<int*>(cnt + 4);
  prm.total_sweeps = cnt + 5;
  prm.tol = fp64 ? 1e-14 : 1e-6;
  prm.sweep_cap = fp64 ? 30 : 20;
  prm.warm_start = (d->flags & MG_WARM_START) ? 1 : 0;
  prm.redo_out = redo;
  prm.n_redo = cnt + 6;
  prm.max_resid_bits = reinterpret_cast<unsigned*>(cnt + 7);
  prm.redo_in = nullptr;
  MG_TRY_CUDA(cudaEventRecord(ctx->ev[1], s));
  int rc;
  const bool tensor = !fp64 && !(d->flags & MG_SOLVE_SIMT) && mg::letkf_tc_supported(prm);
  int64_t n_fallback = 0;
  int tc_ctas = 0;
  if (tensor) {
    // Tensor-core local analyses; the few whose residual test fails are
    // re-run by the SIMT kernel over the list the first kernel wrote.
    if (p > 0) {
      const unsigned pb = (unsigned)std::min<int64_t>((p + 255) / 256, (int64_t)ctx->num_sms * 16);
      obs_pack_kernel<<<pb, 256, 0, s>>>(d->obs_lev, rinv, dinn, p, opack);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
    }
    prm.opack = opack;
    if (bucket) {
      const unsigned pb = (unsigned)std::min<int64_t>((p + 255) / 256, (int64_t)ctx->num_sms * 16);
      obs_bucket_kernel<<<pb, 256, 0, s>>>(d->obs_lev, p, d->nlev, obkt);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
      const unsigned cbk = (unsigned)std::min<int64_t>((d->ncol + 7) / 8, (int64_t)ctx->num_sms * 8);
      level_bucket_kernel<<<cbk, 256, 0, s>>>(d->loc_off, d->loc_idx, d->loc_dist, obkt, d->nlev, d->ncol, bidx,
                                             d->loc_dist ? bdist : nullptr, lev_boff);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
      prm.lev_boff = lev_boff;
      prm.bidx = bidx;
      prm.bdist = d->loc_dist ? bdist : nullptr;
    }
    const int e = mg::letkf_tc_launch(prm, ctx->num_sms, s, &tc_ctas);
    if (e != 0)
      return mg::fail(ctx, MG_ERR_CUDA, std::string("letkf_tc_kernel: ") + cudaGetErrorString((cudaError_t)e));
    unsigned long long hr = 0;
    MG_TRY_CUDA(cudaMemcpyAsync(&hr, cnt + 6, sizeof(hr), cudaMemcpyDeviceToHost, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
    n_fallback = (int64_t)hr;
    rc = MG_OK;
    if (n_fallback > 0) {
      LetkfParams fb = prm;
      fb.redo_in = redo;
      fb.npoints = n_fallback;
      fb.warm_start = 0;
      fb.next = cnt + 6;  // reused as the work counter of the re-run
      fb.lev_boff = nullptr;  // the SIMT kernel walks the column lists as given
      MG_TRY_CUDA(cudaMemsetAsync(cnt + 6, 0, sizeof(unsigned long long), s));
      rc = (k <= 64) ? launch_batched<float, 64>(ctx, fb) : launch_batched<float, 96>(ctx, fb);
    }
  } else if (fp64) {
    if (k <= 32) rc = launch_batched<double, 32>(ctx, prm);
    else if (k <= 64) rc = launch_batched<double, 64>(ctx, prm);
    else rc = launch_batched<double, 96>(ctx, prm);
  } else {
    if (k <= 32) rc = launch_batched<float, 32>(ctx, prm);
    else if (k <= 64) rc = launch_batched<float, 64>(ctx, prm);
    else if (k <= 96) rc = launch_batched<float, 96>(ctx, prm);
    else rc = launch_batched<float, 128>(ctx, prm);
  }
  if (rc != MG_OK) return rc;
  MG_TRY_CUDA(cudaEventRecord(ctx->ev[2], s));
  // Write back member-major; the analysis mean as LETKF.hpp:116 recomputes it.
  if (x32) {
    MG_TRY_CUDA(mg::launch_point_major_to_members_f32(static_cast<const float*>(Xp), n, k,
                                                      static_cast<float*>(d->X), d->ld, s));
    if (d->mean_out)
      MG_TRY_CUDA(mg::launch_mean_members_f32(static_cast<const float*>(d->X), n, k, d->ld, d->mean_out, s));
  } else {
    MG_TRY_CUDA(mg::launch_point_major_to_members(Xa, n, k, static_cast<double*>(d->X), d->ld, s));
    if (d->mean_out)
      MG_TRY_CUDA(mg::launch_mean_pert_members(static_cast<const double*>(d->X), n, k, d->ld, d->mean_out, nullptr,
                                               nullptr, 0, s));
  }
  MG_TRY_CUDA(cudaEventRecord(ctx->ev[3], s));
  unsigned long long host_cnt[8];
  MG_TRY_CUDA(cudaMemcpyAsync(host_cnt, cnt, sizeof(host_cnt), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  float ms[3] = {0.f, 0.f, 0.f};
  for (int i = 0; i < 3; ++i) MG_TRY_CUDA(cudaEventElapsedTime(&ms[i], ctx->ev[i], ctx->ev[i + 1]));
  ctx->stats.ms_prepare = ms[0];
  ctx->stats.ms_analysis = ms[1];
  ctx->stats.ms_writeback = ms[2];
  ctx->stats.n_points = npoints;
  ctx->stats.n_empty = (int64_t)host_cnt[1];
  ctx->stats.total_local = (int64_t)host_cnt[2];
  ctx->stats.max_local = (int32_t)(host_cnt[3] & 0xffffffffull);
  ctx->stats.max_sweeps = (int32_t)(host_cnt[3] >> 32);
  ctx->stats.total_sweeps = (int64_t)host_cnt[5];
  ctx->stats.n_fallback = n_fallback;
  {
    const unsigned bits = (unsigned)(host_cnt[7] & 0xffffffffull);
    float r;
    memcpy(&r, &bits, sizeof(r));
    ctx->stats.max_residual = tensor ? (double)r : 0.0;
  }
  ctx->stats.tensor_path = tensor ? 1 : 0;
  ctx->stats.tensor_ctas = tc_ctas;
  if ((int)(host_cnt[4] & 0xffffffffull) == 2)
    return mg::fail(ctx, MG_ERR_TIMEOUT, "mg_letkf_batched: a bounded tensor-core wait gave up");
  if ((int)(host_cnt[4] & 0xffffffffull) != 0)
    return mg::fail(ctx, MG_ERR_NUMERIC, "mg_letkf_batched: a local k x k system was not positive definite");
  return MG_OK;
}

int mg_letkf_compat_grid(mg_context* ctx, double* X, int32_t k, int64_t ld, int32_t nx, int32_t ny,
                         const int32_t* obs_xy, const uint8_t* valid, const double* yo, int64_t p,
                         double radius, double rho, double* mean_out) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && k >= 2 && k <= 64 && nx > 0 && ny > 0 && ld >= (int64_t)nx * ny && p >= 0 &&
                   (p == 0 || (obs_xy && yo)) && rho > 0.0,
               "mg_letkf_compat_grid: bad arguments (k must be 2..64)");
  const int64_t npt = (int64_t)nx * ny;
  // Local lists by grid distance (independent of the in-place updates).
  // mg_select_grid uses the context workspace, so these live apart from it.
  int64_t total = 0;
  int64_t* off_tmp = nullptr;
  int32_t* idx = nullptr;
  int* status = nullptr;
  MG_TRY_CUDA(cudaMalloc(&off_tmp, sizeof(int64_t) * (npt + 1)));
  int rc = mg_select_grid(ctx, nx, ny, obs_xy, p, radius, off_tmp, nullptr, 0, &total);
  if (rc != MG_OK && rc != MG_ERR_CAPACITY) {
    cudaFree(off_tmp);
    return rc;
  }
  if (cudaMalloc(&idx, sizeof(int32_t) * (total + 1)) != cudaSuccess ||
      cudaMalloc(&status, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(off_tmp);
    cudaFree(idx);
    return mg::fail(ctx, MG_ERR_NOMEM, "mg_letkf_compat_grid: allocation failed");
  }
  rc = mg_select_grid(ctx, nx, ny, obs_xy, p, radius, off_tmp, idx, total, &total);
  if (rc == MG_OK) {
    MG_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
    CompatSeqParams prm{X, k, nx, ny, ld, obs_xy, valid, yo, off_tmp, idx, rho, status};
    const int kmax = k <= 32 ? 32 : 64;
    const size_t smem = sizeof(double) * (2 * (size_t)kmax * (kmax + 1) + 64 * (size_t)kmax + 64 +
                                          3 * (size_t)kmax) + 64;
    cudaError_t e;
    if (kmax == 32) {
      e = cudaFuncSetAttribute(letkf_compat_seq_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess) letkf_compat_seq_kernel<32><<<1, kThreads, smem, ctx->stream>>>(prm);
      if (e == cudaSuccess) MG_COUNT_LAUNCH();
    } else {
      e = cudaFuncSetAttribute(letkf_compat_seq_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess) letkf_compat_seq_kernel<64><<<1, kThreads, smem, ctx->stream>>>(prm);
      if (e == cudaSuccess) MG_COUNT_LAUNCH();
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) rc = mg::fail(ctx, MG_ERR_CUDA, std::string("letkf_compat_seq: ") + cudaGetErrorString(e));
    if (rc == MG_OK && mean_out) {
      e = mg::launch_mean_pert_members(X, npt, k, ld, mean_out, nullptr, nullptr, 0, ctx->stream);
      if (e != cudaSuccess) rc = mg::fail(ctx, MG_ERR_CUDA, cudaGetErrorString(e));
    }
    int hs = 0;
    if (rc == MG_OK) {
      e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = mg::fail(ctx, MG_ERR_CUDA, cudaGetErrorString(e));
      else if (hs != 0)
        rc = mg::fail(ctx, MG_ERR_NUMERIC, "mg_letkf_compat_grid: a local k x k system was not positive definite");
    }
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(idx);
  cudaFree(status);
  cudaFree(off_tmp);
  return rc;
}

}  // extern "C"
