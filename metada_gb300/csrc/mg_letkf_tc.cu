// Batched LETKF local analyses on the tensor cores (mixed precision, Hunt
// transform, k <= 96): the k x k Gram Y'^T R^-1 Y', the products of the
// symmetric inverse square root and the update X' W all run as tcgen05.mma
// kind::tf32 products with an error-compensated 3-pass split
// (hi*hi + hi*lo + lo*hi, hi = x rounded to TF32, lo = x - hi), accumulated in
// FP32 in tensor memory.  Replaces the grid loop of LETKF::Analyse
// (LETKF.hpp:101) and the solve and update of updateGridPoint
// (LETKF.hpp:214-238) in the Hunt et al. (2007) form with Gaspari-Cohn
// R-localisation.
//
// Two instantiations by member slots KP:
//  * KP = 64 (k <= 64): 256 threads, two CTAs per SM (256 TMEM columns each);
//    Z and Y are stacked as the 128 rows of one operand, so [Z; Y] T is one
//    M = 128 product.
//  * KP = 96 (64 < k <= 96, the high-resolution configuration's k = 80): 384
//    threads, one CTA per SM with all 512 TMEM columns and 216 KB of
//    operands; Z, Y and T are separate 96-row operands and [Z; Y] T is two
//    products.
//
// Per local analysis (one CTA, persistent, points pulled in the grid's
// column order from a work counter):
//  1. Gram: the candidate list is filtered and weighted, the kept rows
//     sqrt(w) Y'_o are gathered 64 at a time into a K-major, 128-byte
//     swizzled operand (members x obs) with sqrt(w) d_o as an extra row, and
//     [G | b] = B^T [B | sqrt(w) d] accumulates in TMEM (two rotating
//     buffers; each chunk's rows are loaded while the previous one's MMAs run).
//  2. A = (k-1)/rho I + G.  The ensemble-mean direction 1 is an exact
//     eigenvector of A (Y' 1 = 0, eigenvalue delta) that never reaches the
//     outputs (X' 1 = 0, 1^T b = 0), so the iteration runs on
//     M = P A P / s + 1 1^T / k (P = I - 1 1^T / k), which puts that mode at 1;
//     s = min(||A||_inf, ||PAP||_F) >= lambda_max keeps M's spectrum in (0, 1].
//  3. Coupled Newton-Schulz with scaled steps: T = a I - b Z Y (a, b from
//     ns_coeffs: the classic (3I - Z Y)/2 after scaling Z and Y by sqrt(mu),
//     mu from the known spectrum bounds [delta/s, 1]), [Z; Y] <- [Z; Y] T; it
//     stops once max |Z Y - I| < 0.05 (one more step squares that error).
//     Z -> M^-1/2, and A^-1/2 = (Z - 1 1^T / k) / sqrt(s) on the complement
//     of 1.
//  4. First-order finish from the matrix itself: C = Z^T A Z, F = C - P,
//     W = sqrt((k-1) c) Z (I - F/2), wa = c Z (P - F) Z^T b (c = rho for the
//     reference's inflation placement, else 1).  max |F| is the per-analysis
//     residual.  Analyses whose conditioning bound s / delta is above
//     kMaxCond, whose iteration does not converge or leaves its basin, whose
//     residual is above the gates (kResidMax, kCondResid delta / s) or whose
//     values are not finite are listed and re-run by the SIMT Jacobi kernel.
//  5. Update: D = W^T X'^T (members x variables) on the tensor core, then
//     x_a = x_mean + X' wa + D (+ RTPS relaxation), written in FP64 (or FP32
//     storage).  Points with at most kPre variables take the short finish:
//     E = Z^T X'^T is issued beside the finish's first product and
//     W^T X'^T = cw (E - F^T E / 2), so W is never formed.
// Every mbarrier wait is bounded in time; a wait that gives up makes the CTA
// set the status word, drain its own MMAs (bounded) and free its TMEM.
#include <cuda_runtime.h>

#include "mg_internal.h"
#include "mg_letkf.cuh"
#include "mg_tcgen05.cuh"
#include "mg_tf32op.cuh"

namespace {

using namespace mg::t5;

constexpr int kChunk = 64;      // obs per Gram chunk: two 128-byte swizzle atoms of TF32
constexpr int kNBuf = 2;        // Gram chunk buffers
constexpr int kSelRing = 512;   // selected-entry ring (a candidate block + carry-over < kChunk)
constexpr int kMaxIt = 14;      // Newton-Schulz iterations before an analysis is handed back
constexpr float kStop = 0.05f;  // max |Z Y - I| that ends the iteration (after one more step)
constexpr float kResidMax = 5e-3f;  // max |F| accepted from the first-order finish
// Accuracy gates.  A is formed in FP32 from the Gram, a backward error of
// about eps32 ||A||, so the symmetric inverse square root carries a relative
// error of about eps32 kappa along the smallest eigenvalues (kappa =
// lambda_max / lambda_min of P A P on the complement of 1); on the GPU,
// analyses with kappa near 300 reached 1.8e-5 against FP64, those below 150
// stayed under 2.2e-6.  The first-order finish adds about 1e-4 (kappa
// max|F|)^2 (CPU model of this kernel's arithmetic).  s / delta >= kappa is
// known before the iteration (s >= lambda_max, lambda_min >= delta), so an
// analysis runs here only when s / delta <= kMaxCond, and its finish is
// accepted only when max|F| <= kCondResid delta / s as well as kResidMax; the
// others go to the SIMT kernel, whose factor rebuild keeps the small
// eigenvalues' relative accuracy.
constexpr float kMaxCond = 100.0f;
constexpr float kCondResid = 0.1f;
// max |Z Y - I| above which the iteration has left its basin (a convergent
// iterate stays below 1); the analysis is handed back at once.
constexpr float kDiverged = 4.0f;
constexpr int kVarTile = 16;    // variables per update MMA (N): two 8-column TMEM loads
constexpr int kPre = 4;         // variables whose X' rows and means are prefetched during the finish

// Shared and tensor memory of one CTA, by member slots KP (a multiple of 32).
// Every operand is K-major with the 128-byte swizzle: a slab holds 32 TF32
// columns of all its rows (128 bytes per row), with a hi and a lo copy.
//   KP = 64: STACK (Z in rows 0-63, Y in rows 64-127; 16 KB slabs) and T
//   (64 rows, 8 KB slabs): 96 KB.
//   KP = 96: Z, Y and T, each 96 rows in 12 KB slabs: 216 KB.  As a 128-row
//   A operand, Z's and Y's last 32 rows read the following 4 KB (the lo copy
//   or the next operand); those products land in TMEM lanes 96-127, never read.
// Gram view of the same region: two chunk buffers of KP + 16 rows (KP
// members, the innovation row, 15 unused), then the selected-entry ring.
template <int KP>
struct Lay {
  static_assert(KP == 64 || KP == 96, "member slots");
  static constexpr int NG = KP / 32;          // 32-column groups = TMEM lane quadrants holding rows
  static constexpr int kThreads = 128 * NG;   // four lane quadrants x NG column groups of warps
  static constexpr int kWarps = kThreads / 32;
  static constexpr bool kStack = KP == 64;    // [Z; Y] as one 128-row operand
  static constexpr int kMinBlocks = kStack ? 2 : 1;
  static constexpr uint32_t ZR = kStack ? 128u : (uint32_t)KP;  // rows per slab of Z and Y
  static constexpr uint32_t TR = KP;                            // rows per slab of T
  static constexpr uint32_t kSlabZ = ZR * 128u;
  static constexpr uint32_t kSlabT = TR * 128u;
  static constexpr uint32_t OFF_Z_HI = 0;
  static constexpr uint32_t OFF_Z_LO = NG * kSlabZ;
  static constexpr uint32_t OFF_Y_HI = kStack ? OFF_Z_HI + KP * 128u : 2 * NG * kSlabZ;
  static constexpr uint32_t OFF_Y_LO = kStack ? OFF_Z_LO + KP * 128u : 3 * NG * kSlabZ;
  static constexpr uint32_t OFF_T_HI = (kStack ? 2 : 4) * NG * kSlabZ;
  static constexpr uint32_t OFF_T_LO = OFF_T_HI + NG * kSlabT;
  static constexpr uint32_t kRegion = OFF_T_LO + NG * kSlabT;
  static constexpr int kGramRows = KP + 16;
  static constexpr int kGramN = KP + 16;      // Gram MMA N: members, the innovation row, 15 unused
  static constexpr uint32_t kGramSlab = kGramRows * 128u;
  static constexpr uint32_t kGramBuf = 4 * kGramSlab;  // hi (2 slabs), lo (2 slabs)
  static constexpr uint32_t OFF_SEL = kNBuf * kGramBuf + (128 - kGramRows) * 128u;
  static constexpr uint32_t kSelBytes = kSelRing * 12u;  // obs index, sqrt(w), sqrt(w) d
  // Tensor memory: product scratch at column 0 (and a second product at
  // kTmB for KP = 96), the Gram at kTmGram.
  static constexpr uint32_t kTmemCols = kStack ? 256u : 512u;
  static constexpr uint32_t kTmB = 128;
  static constexpr uint32_t kTmE = KP;  // E = Z^T X'^T (16 columns) beside the products
  static constexpr uint32_t kTmGram = kStack ? 128u : 256u;
  static_assert(kGramSlab % 1024 == 0 && kSlabZ % 1024 == 0 && kSlabT % 1024 == 0,
                "swizzle atoms are 1024-byte aligned");
  static_assert(OFF_SEL + kSelBytes <= kRegion, "Gram buffers, A-operand overhang and the ring");
  static_assert(kStack || (kTmB + KP <= kTmGram && kTmGram + kGramN <= kTmemCols), "tensor memory");
  static_assert(kSelRing >= kThreads + kChunk, "ring holds a candidate block and the carry-over");
};

// Vectors after the operand region.
template <int KP>
struct Vecs {
  static constexpr int NG = KP / 32;
  float b[KP], r[KP], u[KP], v[KP], wa[KP];
  float part[2 * NG][KP];
  float red[32];
  float xsq[kVarTile], inc[kVarTile], fac[kVarTile], one[kVarTile];
  float ssa[NG][kVarTile];
  double xm[kVarTile];
  double xmpre[kPre];
  float xpre[kPre][KP];
  int wcnt[Lay<KP>::kWarps];
};

template <int KP>
constexpr size_t smem_bytes() {
  return 1024 + Lay<KP>::kRegion + sizeof(Vecs<KP>);
}
static_assert(smem_bytes<96>() + 1024 <= 233472, "one KP = 96 CTA fits the SM's shared memory");

// Scaled Newton-Schulz step.  The spectrum of Z Y lies in [l, 1] (l = delta / s
// at the start: P A P >= delta on the complement of 1, s >= lambda_max).  The
// step scales Z and Y by sqrt(mu) before T = (3I - mu Z Y)/2, i.e.
// T = a I - b Z Y with a = 1.5 sqrt(mu), b = 0.5 mu^1.5, where mu equalises
// the map h(e) = e (3 - e)^2 / 4 at both ends of [mu l, mu]:
// mu = 3 (1 - sqrt l) / (1 - l^1.5).  The new interval is [h(mu l), 1].  The
// iteration keeps its fixed point (Z -> M^-1/2) and needs about 4 steps
// instead of 6 at the configurations' conditioning.
__device__ __forceinline__ void ns_coeffs(float& l, float& a, float& b) {
  float mu = 1.0f;
  if (l < 1.0f) {
    const float sl = sqrtf(l);
    mu = fmaxf(3.0f * (1.0f - sl) / (1.0f - l * sl), 1.0f);
  }
  const float smu = sqrtf(mu);
  a = 1.5f * smu;
  b = 0.5f * mu * smu;
  const float ml = fminf(mu * l, 1.0f);
  l = ml * (3.0f - ml) * (3.0f - ml) * 0.25f;
}

// Maximum that a NaN poisons (fmaxf would drop it): NaN -> +inf.
__device__ __forceinline__ float nan_max(float m, float x) { return (x != x) ? __int_as_float(0x7f800000) : fmaxf(m, x); }

// Asynchronous global -> shared copies (no registers held while in flight).
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// FP64 decision for a candidate whose FP32 vertical distance is within 1e-4
// of the support (kept out of line: a predicated FP64 instruction would
// occupy the FP64 pipe for every candidate).
__device__ __noinline__ bool vertical_keep_fp64(int lev, double obs_lev, double vsupport) {
  return fabs((double)lev - obs_lev) <= vsupport;
}

template <int KP>
__global__ void __launch_bounds__(Lay<KP>::kThreads, Lay<KP>::kMinBlocks) letkf_tc_kernel(mg::LetkfParams prm) {
  using L = Lay<KP>;
  constexpr int NG = L::NG;
  constexpr int kThreads = L::kThreads;
  constexpr uint32_t ZR = L::ZR, TR = L::TR;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* R = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  Vecs<KP>& V = *reinterpret_cast<Vecs<KP>*>(R + L::kRegion);
  unsigned char* const ZH = R + L::OFF_Z_HI;
  unsigned char* const ZL = R + L::OFF_Z_LO;
  unsigned char* const YH = R + L::OFF_Y_HI;
  unsigned char* const YL = R + L::OFF_Y_LO;
  unsigned char* const TH = R + L::OFF_T_HI;
  unsigned char* const TL = R + L::OFF_T_LO;
  int* const sel_o = reinterpret_cast<int*>(R + L::OFF_SEL);
  float* const sel_sw = reinterpret_cast<float*>(R + L::OFF_SEL + 4 * kSelRing);
  float* const sel_sd = reinterpret_cast<float*>(R + L::OFF_SEL + 8 * kSelRing);
  __shared__ uint64_t mma_bar;
  __shared__ uint64_t buf_bar[kNBuf];
  __shared__ uint32_t tmem_s;
  __shared__ long long s_item;
  __shared__ unsigned s_flag[4];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = warp & 3, g = warp >> 2;  // TMEM lane quadrant, 32-column group
  const int k = prm.k;
  const float ik = 1.0f / (float)k;
  const float* __restrict__ Y = static_cast<const float*>(prm.Y);
  const float* __restrict__ Xp = static_cast<const float*>(prm.Xp);
  const bool r_identity = prm.flags & MG_R_IDENTITY;
  const bool infl_compat = prm.flags & MG_INFL_COMPAT;
  const bool rtps = prm.flags & MG_RTPS;
  const float delta = (infl_compat || rtps) ? (float)(k - 1) : (float)((double)(k - 1) / prm.rho);
  const float sc = infl_compat ? (float)prm.rho : 1.0f;
  const float cw = sqrtf((float)(k - 1) * sc);
  const float hc = (float)(0.5 * prm.hsupport), vc = (float)(0.5 * prm.vsupport), vs = (float)prm.vsupport;
  const bool vec4 = (k & 3) == 0;

  if (tid == 0) {
    mbar_init(&mma_bar, 1);
    for (int b = 0; b < kNBuf; ++b) mbar_init(&buf_bar[b], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(&tmem_s, L::kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_s;
  const uint32_t tm_row = ((uint32_t)(32 * q) << 16);  // this warp's TMEM lanes
  const uint32_t sR = smem_u32(R);
  const uint32_t sZH = sR + L::OFF_Z_HI, sZL = sR + L::OFF_Z_LO;
  const uint32_t sYH = sR + L::OFF_Y_HI, sYL = sR + L::OFF_Y_LO;
  const uint32_t sTH = sR + L::OFF_T_HI, sTL = sR + L::OFF_T_LO;
  const uint32_t idescK = idesc_tf32_f32(128, KP);
  const uint32_t idescG = idesc_tf32_f32(128, L::kGramN);
  const uint32_t idescU = idesc_tf32_f32(128, kVarTile);

  uint32_t mma_ph = 0;      // parity of the next mma_bar phase
  uint32_t gchunk = 0;      // Gram chunks issued by this CTA (buffer rotation)
  bool alive = true;

  for (;;) {
    cp_async_wait_all();  // a handed-back analysis may leave its prefetch in flight
    if (tid == 0) s_item = (long long)atomicAdd(prm.next, 1ull);
    __syncthreads();
    const long long item = s_item;
    __syncthreads();
    if (item >= prm.npoints) break;
    const int lev = (int)(item % prm.nlev);
    const int64_t col = prm.order[item / prm.nlev];
    const int64_t base = prm.col_base[col] + (int64_t)lev * prm.lev_stride;
    int64_t e0 = prm.loc_off[col], e1 = prm.loc_off[col + 1];
    const int32_t* lidx = prm.loc_idx;
    const double* ldist = prm.loc_dist;
    if (prm.lev_boff) {  // only the level buckets that can reach this level
      const int32_t* bo = prm.lev_boff + col * (int64_t)(prm.nlev + 1);
      const double fl = floor((double)lev - prm.vsupport), fh = floor((double)lev + prm.vsupport);
      const int lo = (fl <= 0.0) ? 0 : (int)fl;
      const int hi = (fh >= (double)(prm.nlev - 1)) ? prm.nlev - 1 : (int)fh;
      e1 = e0 + bo[hi + 1];
      e0 = e0 + bo[lo];
      lidx = prm.bidx;
      ldist = prm.bdist;
    }

    // ---------------- 1. selection and Gram ----------------
    // Rounds: compact candidates into the ring (up to kSelRing - kThreads
    // entries), then emit its chunks; each chunk's rows are loaded into
    // registers while the previous chunk is stored and its MMAs issued.
    int64_t cpos = e0;
    int nloc = 0, nch = 0, head = 0, nsel = 0;
    const int slot = tid & (kChunk - 1), m0 = (tid / kChunk) * 16;  // gather: obs slot x 16 members
    auto load_rows = [&](int pos, int cnt, float (&x)[16], float& sd) {
      if (slot < cnt) {
        const int e = (pos + slot) & (kSelRing - 1);
        const int o = sel_o[e];
        const float sw = sel_sw[e];
        sd = sel_sd[e];
        const float* yr = Y + (int64_t)o * k;
        if (vec4 && m0 + 16 <= k) {
#pragma unroll
          for (int q4 = 0; q4 < 4; ++q4) {
            const float4 a4 = *reinterpret_cast<const float4*>(yr + m0 + 4 * q4);
            x[4 * q4 + 0] = a4.x * sw; x[4 * q4 + 1] = a4.y * sw; x[4 * q4 + 2] = a4.z * sw; x[4 * q4 + 3] = a4.w * sw;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) x[j] = (m0 + j < k) ? yr[m0 + j] * sw : 0.0f;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = 0.0f;
        sd = 0.0f;
      }
    };
    while (alive) {
      while (cpos < e1 && nsel <= kSelRing - kThreads) {
        bool keep = false;
        int o = 0;
        float sw = 0.0f, sd = 0.0f;
        if (cpos + tid < e1) {
          const int64_t e = cpos + tid;
          o = lidx[e];
          const float4 pk = prm.opack[o];  // (level, 1/sigma^2, innovation, 0) as FP32
          float w = 1.0f;
          keep = true;
          if (prm.obs_lev) {
            const float dl = fabsf((float)lev - pk.x);
            if (dl > vs + 1e-4f) keep = false;
            else if (dl >= vs - 1e-4f) keep = vertical_keep_fp64(lev, prm.obs_lev[o], prm.vsupport);
            if (keep && !r_identity) w *= mg::gaspari_cohn<float>(dl / vc);
          }
          if (keep && !r_identity) {
            if (ldist) w *= mg::gaspari_cohn<float>((float)ldist[e] / hc);
            w *= pk.y;
            if (!(w > 0.0f)) keep = false;
          }
          if (keep) {
            sw = sqrtf(w);
            sd = sw * pk.z;
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) V.wcnt[warp] = __popc(bal);
        __syncthreads();
        int wb = 0, cnt = 0;
#pragma unroll
        for (int w = 0; w < L::kWarps; ++w) {
          if (w < warp) wb += V.wcnt[w];
          cnt += V.wcnt[w];
        }
        if (keep) {
          const int pos = (head + nsel + wb + __popc(bal & ((1u << lane) - 1u))) & (kSelRing - 1);
          sel_o[pos] = o;
          sel_sw[pos] = sw;
          sel_sd[pos] = sd;
        }
        __syncthreads();
        nsel += cnt;
        nloc += cnt;
        cpos += kThreads;
      }
      const bool done = cpos >= e1;
      const int nchunks = done ? (nsel + kChunk - 1) / kChunk : nsel / kChunk;
      float x[16], sdv;
      if (nchunks > 0) load_rows(head, nsel < kChunk ? nsel : kChunk, x, sdv);
      for (int c = 0; c < nchunks; ++c) {
        const int b = (int)(gchunk % kNBuf);
        const uint32_t use = gchunk / kNBuf;
        if (use > 0 && !wait_all(&buf_bar[b], (use - 1) & 1u)) { alive = false; break; }
        unsigned char* bh = R + b * L::kGramBuf;
        unsigned char* bl = bh + 2 * L::kGramSlab;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const uint32_t off = sw_off(m0 + j, slot, L::kGramRows);
          float h, l;
          split(x[j], h, l);
          *reinterpret_cast<float*>(bh + off) = h;
          *reinterpret_cast<float*>(bl + off) = l;
        }
        if (m0 == 0) {  // the innovation row
          const uint32_t off = sw_off(KP, slot, L::kGramRows);
          float h, l;
          split(sdv, h, l);
          *reinterpret_cast<float*>(bh + off) = h;
          *reinterpret_cast<float*>(bl + off) = l;
        }
        if (c + 1 < nchunks) {  // next chunk's rows in flight during the barrier and the MMAs
          const int rem = nsel - (c + 1) * kChunk;
          load_rows(head + (c + 1) * kChunk, rem < kChunk ? rem : kChunk, x, sdv);
        }
        operands_ready();
        if (warp == 0) {
          tc_fence_after();
          const uint32_t a = sR + b * L::kGramBuf;
          issue3(tmem + L::kTmGram, a, a + 2 * L::kGramSlab, L::kGramSlab, a, a + 2 * L::kGramSlab, L::kGramSlab, 2,
                 idescG, nch > 0);
          mma_commit_elect(&buf_bar[b]);
        }
        ++gchunk;
        ++nch;
      }
      if (!alive) break;
      head = (head + nchunks * kChunk) & (kSelRing - 1);
      nsel = (nsel > nchunks * kChunk) ? nsel - nchunks * kChunk : 0;
      if (done) break;
    }
    if (!alive) break;

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
    if (warp == 0) mma_commit_elect(&mma_bar);
    if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
    mma_ph ^= 1u;

    // ---------------- 2. A, b, deflation and scaling ----------------
    // Warps of quadrants 0 .. NG-1 hold rows 0 .. KP-1 (their TMEM lanes),
    // column group g; each walks its 32 columns 8 at a time.
    const bool rowwarp = q < NG;
    const int row = 32 * q + lane;
    const int cb = 32 * g;
    if (rowwarp) {
      float rs = 0.0f, as = 0.0f, fa = 0.0f;
#pragma unroll 1
      for (int c0 = cb; c0 < cb + 32; c0 += 8) {
        uint32_t v[8];
        tmem_ld8(tmem + tm_row + L::kTmGram + c0, v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = c0 + j;
          const float x = __uint_as_float(v[j]) + ((c == row) ? delta : 0.0f);
          if (row < k && c < k) {
            rs += x;
            as += fabsf(x);
            fa += x * x;
          }
        }
      }
      V.part[g][row] = rs;
      V.part[NG + g][row] = as;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) fa += __shfl_xor_sync(0xffffffffu, fa, off);
      if (lane == 0) V.red[3 * NG + q * NG + g] = fa;  // ||A||_F^2, by warp
      if (g == 0) {
        const uint32_t bv = tmem_ld1(tmem + tm_row + L::kTmGram + KP);
        tmem_wait_ld();
        V.b[row] = (row < k) ? __uint_as_float(bv) : 0.0f;
      }
    }
    __syncthreads();
    if (warp < NG) {  // row means r, grand mean c, infinity norm
      const int i = tid;
      float r = 0.0f, ab = 0.0f;
      if (i < k) {
#pragma unroll
        for (int gg = 0; gg < NG; ++gg) {
          r += V.part[gg][i];
          ab += V.part[NG + gg][i];
        }
        r *= ik;
      }
      V.r[i] = r;
      float sr = r, mx = ab, s2 = r * r;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, off);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
      }
      if (lane == 0) {
        V.red[warp] = sr;
        V.red[NG + warp] = mx;
        V.red[2 * NG + warp] = s2;
      }
    }
    __syncthreads();
    float cbar = 0.0f, ninf = 0.0f;
#pragma unroll
    for (int gg = 0; gg < NG; ++gg) {
      cbar += V.red[gg];
      ninf = fmaxf(ninf, V.red[NG + gg]);
    }
    cbar *= ik;
    // Row `row` of P A P, columns c0 .. c0+7, from the Gram in TMEM (zero
    // outside the member block).
    auto pap8 = [&](int c0, float (&x)[8]) {
      uint32_t v[8];
      tmem_ld8(tmem + tm_row + L::kTmGram + c0, v);
      tmem_wait_ld();
      const float ri = V.r[row];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = c0 + j;
        const float av = __uint_as_float(v[j]) + ((c == row) ? delta : 0.0f);
        x[j] = (row < k && c < k) ? (av - ri - V.r[c] + cbar) : 0.0f;
      }
    };
    // Frobenius norm of P A P from the same pass (A symmetric, A 1 = k r):
    // ||P A P||_F^2 = ||A||_F^2 - 2 k sum r_i^2 + k^2 cbar^2.  With A 1 =
    // delta 1 up to rounding the subtracted part is about delta^2, at most
    // 1/k of ||A||_F^2 >= k delta^2, so the difference keeps FP32 accuracy
    // (and s only has to bound lambda_max).
    float fa2 = 0.0f, sr2 = 0.0f;
#pragma unroll
    for (int e = 0; e < NG * NG; ++e) fa2 += V.red[3 * NG + e];
#pragma unroll
    for (int gg = 0; gg < NG; ++gg) sr2 += V.red[2 * NG + gg];
    const float kf = (float)k;
    const float fro = sqrtf(fmaxf(fa2 - 2.0f * kf * sr2 + kf * kf * cbar * cbar, 0.0f));
    const float s = fmaxf(fminf(ninf, fro), 1e-30f);
    const float is = 1.0f / s;
    float lsp = fminf(delta * is, 1.0f);  // lower end of the spectrum of Z Y (upper end 1)
    // Points handed to the SIMT Jacobi kernel: nothing is written for them here.
    auto hand_back = [&]() {
      if (tid == 0) {
        const unsigned long long slot = atomicAdd(prm.n_redo, 1ull);
        prm.redo_out[slot] = (int32_t)(col * prm.nlev + lev);
      }
      __syncthreads();
    };
    const float l0 = lsp;  // delta / s, at most 1 / kappa
    if (!(l0 * kMaxCond >= 1.0f)) {
      hand_back();
      continue;
    }
    float nsa, nsb;
    ns_coeffs(lsp, nsa, nsb);
    // M = PAP / s + 1 1^T / k (identity on unused member slots); Z <- I,
    // Y <- M (row-major), T <- T0 = a I - b M stored transposed.
    if (rowwarp) {
#pragma unroll 1
      for (int c0 = cb; c0 < cb + 32; c0 += 8) {
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = (row == c0 + j) ? 1.0f : 0.0f;
        put_row8(ZH, ZL, row, c0, ZR, x);
        pap8(c0, x);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = c0 + j;
          x[j] = (row < k && c < k) ? x[j] * is + ik : ((row == c) ? 1.0f : 0.0f);
        }
        put_row8(YH, YL, row, c0, ZR, x);
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = ((row == c0 + j) ? nsa : 0.0f) - nsb * x[j];
        put_col8(TH, TL, row, c0, TR, x);
      }
    }

    // X' rows and means of the first kPre variables, in flight during the
    // Newton-Schulz iteration (members beyond k read as zero).
    const int npre = (prm.n_var < kPre) ? prm.n_var : kPre;
    for (int e = tid; e < kPre * KP; e += kThreads) {
      const int vv = e / KP, m = e - vv * KP;
      if (vv < npre && m < k) cp_async4(&V.xpre[vv][m], Xp + (base + (int64_t)vv * prm.var_stride) * k + m);
      else V.xpre[vv][m] = 0.0f;
    }
    if (tid < npre) cp_async8(&V.xmpre[tid], prm.xmean + base + (int64_t)tid * prm.var_stride);
    // Points with at most kPre variables take the short finish: E = Z^T X'^T
    // is computed beside Q, and X' W = cw (E - F^T E / 2), so W itself is
    // never formed (one dependent product and two epilogues fewer).
    const bool fast = prm.n_var <= kPre;

    // ---------------- 3. coupled Newton-Schulz ----------------
    int its = 0;
    bool stop = false;  // decided from max |Z Y - I| of the current iterate
    bool conv = false;
    bool diverged = false;
    for (;;) {
      // [Z; Y] <- [Z; Y] T
      operands_ready();
      if (warp == 0) {
        tc_fence_after();
        if constexpr (L::kStack) {
          issue3(tmem, sZH, sZL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescK, false);
        } else {
          issue3(tmem, sZH, sZL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescK, false);
          issue3(tmem + L::kTmB, sYH, sYL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescK, false);
        }
        mma_commit_elect(&mma_bar);
      }
      ++its;
      const bool last = stop || its >= kMaxIt;
      conv = stop;
      if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
      mma_ph ^= 1u;
      if (!last) {
        if constexpr (L::kStack) {  // all warps: rows 0-63 Z, 64-127 Y
#pragma unroll 1
          for (int c0 = cb; c0 < cb + 32; c0 += 8) {
            uint32_t v[8];
            tmem_ld8(tmem + tm_row + c0, v);
            tmem_wait_ld();
            float x[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = __uint_as_float(v[j]);
            put_row8(ZH, ZL, 32 * q + lane, c0, ZR, x);
          }
        } else if (rowwarp) {  // Z from the first product, Y from the second
#pragma unroll 1
          for (int c0 = cb; c0 < cb + 32; c0 += 8) {
            uint32_t v[8];
            float x[8];
            tmem_ld8(tmem + tm_row + c0, v);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = __uint_as_float(v[j]);
            put_row8(ZH, ZL, row, c0, ZR, x);
            tmem_ld8(tmem + tm_row + L::kTmB + c0, v);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = __uint_as_float(v[j]);
            put_row8(YH, YL, row, c0, ZR, x);
          }
        }
      } else if (rowwarp) {
        // Final Z -> (Z - 1 1^T / k) / sqrt(s) on the member block, 0 elsewhere,
        // stored transposed (Z's operand holds Z^T); Y's operand <- P A P (from
        // the Gram in TMEM) for the finish.
        const float isq = rsqrtf(s);
#pragma unroll 1
        for (int c0 = cb; c0 < cb + 32; c0 += 8) {
          uint32_t v[8];
          tmem_ld8(tmem + tm_row + c0, v);
          tmem_wait_ld();
          float x[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = c0 + j;
            x[j] = (row < k && c < k) ? (__uint_as_float(v[j]) - ik) * isq : 0.0f;
          }
          put_col8(ZH, ZL, row, c0, ZR, x);
          pap8(c0, x);
          put_row8(YH, YL, row, c0, ZR, x);
        }
      }
      if (last) break;
      // P = Z Y (Y as stored), T = a I - b P (scaled step) -> T transposed.
      operands_ready();
      if (warp == 0) {
        tc_fence_after();
        issue3(tmem, sZH, sZL, L::kSlabZ, sYH, sYL, L::kSlabZ, NG, idescK, false);
        mma_commit_elect(&mma_bar);
      }
      if (tid == 0) s_flag[0] = 0u;
      ns_coeffs(lsp, nsa, nsb);
      if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
      mma_ph ^= 1u;
      if (rowwarp) {
        float emax = 0.0f;
#pragma unroll 1
        for (int c0 = cb; c0 < cb + 32; c0 += 8) {
          uint32_t v[8];
          tmem_ld8(tmem + tm_row + c0, v);
          tmem_wait_ld();
          float t[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = c0 + j;
            const float d = __uint_as_float(v[j]) - ((row == c) ? 1.0f : 0.0f);
            emax = nan_max(emax, fabsf(d));
            t[j] = ((row == c) ? nsa - nsb : 0.0f) - nsb * d;  // a I - b P, P = I + d
          }
          put_col8(TH, TL, row, c0, TR, t);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, off));
        if (lane == 0 && !(emax < kStop)) atomicOr(&s_flag[0], 1u);
        if (lane == 0 && !(emax < kDiverged)) atomicOr(&s_flag[0], 2u);
      }
      __syncthreads();
      const unsigned fl = s_flag[0];
      stop = fl == 0u;
      if (fl & 2u) {
        diverged = true;
        break;
      }
    }
    if (!alive) break;
    if (diverged) {
      hand_back();
      continue;
    }

    // ---------------- 4. finish ----------------
    // The iterate is Z = p(M) up to rounding errors that the coupled
    // iteration leaves as right factors, so the finish takes C = Z^T A Z:
    // Q = (P A P) Z (A operand: Y's rows = P A P; B operand: Z^T rows), then
    // C = Z^T Q; A^-1 = Z C^-1 Z^T, A^-1/2 ~ Z C^-1/2.
    if (fast) {  // X' rows -> T rows 0..15 (B operand of E; T is free here)
      cp_async_wait_all();
      __syncthreads();
      for (int e = tid; e < kVarTile * KP; e += kThreads) {
        const int vv = e / KP, m = e - vv * KP;
        const uint32_t off = sw_off(vv, m, TR);
        float h, l;
        split((vv < npre) ? V.xpre[vv][m] : 0.0f, h, l);
        *reinterpret_cast<float*>(TH + off) = h;
        *reinterpret_cast<float*>(TL + off) = l;
      }
    }
    operands_ready();
    if (warp == 0) {
      tc_fence_after();
      issue3(tmem, sYH, sYL, L::kSlabZ, sZH, sZL, L::kSlabZ, NG, idescK, false);
      if (fast) issue3(tmem + L::kTmE, sZH, sZL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescU, false);
      mma_commit_elect(&mma_bar);
    }
    if (tid < KP) {  // u = Z^T b (row tid of Z^T)
      float acc = 0.0f;
#pragma unroll 1
      for (int c0 = 0; c0 < KP; c0 += 8) {
        float z[8];
        get_row8(ZH, ZL, tid, c0, ZR, z);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc += z[j] * V.b[c0 + j];
      }
      V.u[tid] = acc;
    }
    if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
    mma_ph ^= 1u;
    if (rowwarp) {  // Q -> T transposed
#pragma unroll 1
      for (int c0 = cb; c0 < cb + 32; c0 += 8) {
        uint32_t v[8];
        tmem_ld8(tmem + tm_row + c0, v);
        tmem_wait_ld();
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = __uint_as_float(v[j]);
        put_col8(TH, TL, row, c0, TR, x);
      }
    }
    // C = Z^T Q
    operands_ready();
    if (warp == 0) {
      tc_fence_after();
      issue3(tmem, sZH, sZL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescK, false);
      mma_commit_elect(&mma_bar);
      if (lane == 0) s_flag[1] = 0u;
    }
    if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
    mma_ph ^= 1u;
    // F = C - P (residual, partial F u) -> T transposed (B operand of Z F);
    // Z rows, read from the columns of Z^T, -> Y's operand row-major (A
    // operand of Z F; P A P there is not read any more).  Short finish:
    // F^T -> Y's operand (A operand of F^T E) and E -> T rows 0..15 (its B
    // operand).
    if (rowwarp) {
      float fu = 0.0f, fm = 0.0f;
#pragma unroll 1
      for (int c0 = cb; c0 < cb + 32; c0 += 8) {
        uint32_t v[8];
        tmem_ld8(tmem + tm_row + c0, v);
        tmem_wait_ld();
        float f[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = c0 + j;
          const float pij = (row < k && c < k) ? (((row == c) ? 1.0f : 0.0f) - ik) : 0.0f;
          const float x = (row < k && c < k) ? __uint_as_float(v[j]) - pij : 0.0f;
          f[j] = x;
          fm = nan_max(fm, fabsf(x));
          fu += x * V.u[c];
        }
        if (fast) {
          put_col8(YH, YL, row, c0, ZR, f);
        } else {
          put_col8(TH, TL, row, c0, TR, f);
          get_col8(ZH, ZL, row, c0, ZR, f);
          put_row8(YH, YL, row, c0, ZR, f);
        }
      }
      if (fast && g == 0) {
        uint32_t v[8];
#pragma unroll 1
        for (int c0 = 0; c0 < kVarTile; c0 += 8) {
          tmem_ld8(tmem + tm_row + L::kTmE + c0, v);
          tmem_wait_ld();
          float e8[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) e8[j] = __uint_as_float(v[j]);
          put_col8(TH, TL, row, c0, TR, e8);
        }
      }
      V.part[g][row] = fu;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) fm = fmaxf(fm, __shfl_xor_sync(0xffffffffu, fm, off));
      // NaN or Inf residuals map to the maximum (positive floats order as integers)
      if (lane == 0) atomicMax(&s_flag[1], (fm == fm && fm < 3.0e38f) ? __float_as_uint(fm) : 0x7f800000u);
    }
    // W = cw Z (I - F/2): D = Z F (short finish: D = F^T E, 16 columns)
    operands_ready();
    if (warp == 0) {
      tc_fence_after();
      if (fast) issue3(tmem, sYH, sYL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescU, false);
      else issue3(tmem, sYH, sYL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescK, false);
      mma_commit_elect(&mma_bar);
    }
    const float resid = __uint_as_float(s_flag[1]);
    if (tid < KP) {
      float fu = 0.0f;
#pragma unroll
      for (int gg = 0; gg < NG; ++gg) fu += V.part[gg][tid];
      V.v[tid] = (tid < k) ? V.u[tid] - fu : 0.0f;
    }
    __syncthreads();
    if (tid < KP) {  // wa = c Z v (row tid of Z: in Y's operand, or column tid of Z^T)
      float acc = 0.0f;
#pragma unroll 1
      for (int c0 = 0; c0 < KP; c0 += 8) {
        float z[8];
        if (fast) get_col8(ZH, ZL, tid, c0, ZR, z);
        else get_row8(YH, YL, tid, c0, ZR, z);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc += z[j] * V.v[c0 + j];
      }
      V.wa[tid] = sc * acc;
    }
    if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
    mma_ph ^= 1u;
    const bool redo = !conv || !(resid <= fminf(kResidMax, kCondResid * l0));
    if (redo) {
      hand_back();
      continue;
    }
    if (!fast && rowwarp) {  // W rows -> U^T = W^T into Z's operand (A operand of the update)
#pragma unroll 1
      for (int c0 = cb; c0 < cb + 32; c0 += 8) {
        uint32_t v[8];
        tmem_ld8(tmem + tm_row + c0, v);
        tmem_wait_ld();
        float w[8];
        get_row8(YH, YL, row, c0, ZR, w);
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = cw * (w[j] - 0.5f * __uint_as_float(v[j]));
        put_col8(ZH, ZL, row, c0, ZR, w);
      }
    }

    // ---------------- 5. update ----------------
    const float c1 = cw * rsqrtf(delta);  // W's eigenvalue on the mean direction
    cp_async_wait_all();
    __syncthreads();  // the prefetched rows visible to every thread
    if (fast) {
      // X' W = cw (E - D / 2), D = F^T E, from TMEM; X' wa, the mean of X'
      // and sum of X'^2 from the prefetched rows (one warp per variable).
      const int nv = prm.n_var;
      for (int vv = warp; vv < nv; vv += L::kWarps) {
        float dw = 0.0f, sx = 0.0f, sq = 0.0f;
#pragma unroll
        for (int gg = 0; gg < NG; ++gg) {
          const int m = lane + 32 * gg;
          const float x0 = V.xpre[vv][m];
          dw += x0 * V.wa[m];
          sx += x0;
          sq += x0 * x0;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          dw += __shfl_xor_sync(0xffffffffu, dw, off);
          sx += __shfl_xor_sync(0xffffffffu, sx, off);
          sq += __shfl_xor_sync(0xffffffffu, sq, off);
        }
        if (lane == 0) {
          V.one[vv] = c1 * sx * ik;
          V.inc[vv] = dw;
          V.xsq[vv] = sq;
          V.xm[vv] = V.xmpre[vv];
        }
      }
      __syncthreads();
      float dv[kPre];
      if (rowwarp && g == 0) {
        uint32_t dd[8], ee[8];
        tmem_ld8(tmem + tm_row, dd);
        tmem_ld8(tmem + tm_row + L::kTmE, ee);
        tmem_wait_ld();
#pragma unroll
        for (int vv = 0; vv < kPre; ++vv)
          dv[vv] = cw * (__uint_as_float(ee[vv]) - 0.5f * __uint_as_float(dd[vv])) + V.one[vv];
        if (rtps) {
#pragma unroll
          for (int vv = 0; vv < kPre; ++vv) {
            float s2 = (row < k && vv < nv) ? dv[vv] * dv[vv] : 0.0f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off);
            if (lane == 0) V.ssa[q][vv] = s2;
          }
        }
      }
      if (rtps) {
        __syncthreads();
        if (tid < nv) {
          float s2 = 0.0f;
#pragma unroll
          for (int qq = 0; qq < NG; ++qq) s2 += V.ssa[qq][tid];
          const float sb = sqrtf(V.xsq[tid] / (float)(k - 1));
          const float sa = sqrtf(s2 / (float)(k - 1));
          V.fac[tid] = (sa > 0.0f) ? (float)prm.rho * (sb - sa) / sa : 0.0f;  // factor - 1
        }
        __syncthreads();
      }
      if (rowwarp && g == 0 && row < k) {
#pragma unroll
        for (int vv = 0; vv < kPre; ++vv) {
          if (vv < nv) {
            const float a2 = rtps ? dv[vv] * (1.0f + V.fac[vv]) : dv[vv];
            mg::letkf_store(prm, (base + (int64_t)vv * prm.var_stride) * k + row,
                            (V.xm[vv] + (double)V.inc[vv]) + (double)a2);
          }
        }
      }
      __syncthreads();
    }
    for (int v0 = 0; !fast && v0 < prm.n_var; v0 += kVarTile) {
      const int nv = (prm.n_var - v0 < kVarTile) ? prm.n_var - v0 : kVarTile;
      // X' rows of the variables -> T rows 0..15 (B operand, K = members);
      // one warp per variable: X' wa, the mean of X', sum of X'^2.
      for (int vv = warp; vv < kVarTile; vv += L::kWarps) {
        const bool pre = v0 == 0 && vv < npre;
        const float* xr = (vv < nv && !pre) ? Xp + (base + (int64_t)(v0 + vv) * prm.var_stride) * k : nullptr;
        float dw = 0.0f, sx = 0.0f, sq = 0.0f;
#pragma unroll
        for (int gg = 0; gg < NG; ++gg) {
          const int m = lane + 32 * gg;
          const float x0 = pre ? V.xpre[vv][m] : ((xr && m < k) ? xr[m] : 0.0f);
          const uint32_t o0 = sw_off(vv, m, TR);
          float h, l;
          split(x0, h, l);
          *reinterpret_cast<float*>(TH + o0) = h;
          *reinterpret_cast<float*>(TL + o0) = l;
          dw += x0 * V.wa[m];
          sx += x0;
          sq += x0 * x0;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          dw += __shfl_xor_sync(0xffffffffu, dw, off);
          sx += __shfl_xor_sync(0xffffffffu, sx, off);
          sq += __shfl_xor_sync(0xffffffffu, sq, off);
        }
        if (lane == 0) {
          V.one[vv] = c1 * sx * ik;  // X' W on the mean direction (X' 1 is zero up to rounding)
          V.inc[vv] = dw;
          V.xsq[vv] = sq;
          V.xm[vv] = pre ? V.xmpre[vv] : ((vv < nv) ? prm.xmean[base + (int64_t)(v0 + vv) * prm.var_stride] : 0.0);
        }
      }
      operands_ready();
      if (warp == 0) {
        tc_fence_after();
        issue3(tmem, sZH, sZL, L::kSlabZ, sTH, sTL, L::kSlabT, NG, idescU, false);
        mma_commit_elect(&mma_bar);
      }
      if (!wait_all(&mma_bar, mma_ph)) { alive = false; break; }
      mma_ph ^= 1u;
      float dv[kVarTile];
      if (rowwarp && g == 0) {
        uint32_t v[8], v2[8];
        tmem_ld8(tmem + tm_row, v);
        tmem_ld8(tmem + tm_row + 8, v2);
        tmem_wait_ld();
#pragma unroll
        for (int vv = 0; vv < 8; ++vv) {
          dv[vv] = __uint_as_float(v[vv]) + V.one[vv];
          dv[8 + vv] = __uint_as_float(v2[vv]) + V.one[8 + vv];
        }
        if (rtps) {  // analysis spread per variable (members = rows 0 .. KP-1)
#pragma unroll
          for (int vv = 0; vv < kVarTile; ++vv) {
            float s2 = (row < k) ? dv[vv] * dv[vv] : 0.0f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off);
            if (lane == 0) V.ssa[q][vv] = s2;
          }
        }
      }
      if (rtps) {
        __syncthreads();
        if (tid < kVarTile) {
          float s2 = 0.0f;
#pragma unroll
          for (int qq = 0; qq < NG; ++qq) s2 += V.ssa[qq][tid];
          const float sb = sqrtf(V.xsq[tid] / (float)(k - 1));
          const float sa = sqrtf(s2 / (float)(k - 1));
          V.fac[tid] = (sa > 0.0f) ? (float)prm.rho * (sb - sa) / sa : 0.0f;  // factor - 1
        }
        __syncthreads();
      }
      if (rowwarp && g == 0 && row < k) {
        for (int vv = 0; vv < nv; ++vv) {
          const float a2 = rtps ? dv[vv] * (1.0f + V.fac[vv]) : dv[vv];
          mg::letkf_store(prm, (base + (int64_t)(v0 + vv) * prm.var_stride) * k + row,
                          (V.xm[vv] + (double)V.inc[vv]) + (double)a2);
        }
      }
      __syncthreads();  // T and the vectors are rewritten by the next tile
    }
    if (!alive) break;
    if (tid == 0) {
      atomicAdd(prm.total_local, (unsigned long long)nloc);
      atomicAdd(prm.total_sweeps, (unsigned long long)its);
      atomicMax(prm.max_local, nloc);
      atomicMax(prm.max_sweeps, its);
      atomicMax(prm.max_resid_bits, s_flag[1]);
    }
  }

  if (!alive) {
    // A bounded wait gave up: record it, drain this CTA's MMAs (bounded).
    if (tid == 0) {
      atomicExch(prm.status, 2);
      mma_commit(&mma_bar);
      mbar_wait(&mma_bar, mma_ph);
    }
  }
  cp_async_wait_all();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, L::kTmemCols);
}

template <int KP>
int launch_tc(const mg::LetkfParams& prm, int num_sms, void* stream, int* ctas) {
  using L = Lay<KP>;
  constexpr size_t kSmem = smem_bytes<KP>();
  auto kern = letkf_tc_kernel<KP>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e != cudaSuccess) return (int)e;
  // The whole unified L1/shared array as shared memory (two KP = 64 CTAs or
  // one KP = 96 CTA per SM).
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return (int)e;
  // CTAs per SM from the SM's shared memory and register file, at most the
  // design point (which also divides the SM's 512 TMEM columns evenly).
  cudaFuncAttributes fa{};
  e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return (int)e;
  int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess)
    return (int)e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
    return (int)e;
  if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess)
    return (int)e;
  const size_t per_cta = kSmem + fa.sharedSizeBytes + (size_t)reserved;
  int per_sm = (int)((size_t)smem_sm / per_cta);
  const int by_regs = fa.numRegs > 0 ? regs_sm / (fa.numRegs * L::kThreads) : L::kMinBlocks;
  if (by_regs < per_sm) per_sm = by_regs;
  if (per_sm > L::kMinBlocks) per_sm = L::kMinBlocks;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  int64_t grid = (int64_t)per_sm * num_sms;
  if (grid > prm.npoints) grid = prm.npoints;
  if (grid < 1) grid = 1;
  if (ctas) *ctas = (int)grid;
  kern<<<(unsigned)grid, L::kThreads, kSmem, static_cast<cudaStream_t>(stream)>>>(prm);
  MG_COUNT_LAUNCH();
  return (int)cudaGetLastError();
}

}  // namespace

namespace mg {

bool letkf_tc_supported(const LetkfParams& prm) {
  const bool chol = prm.flags & MG_SQRT_CHOLESKY, upd = prm.flags & MG_UPDATE_COMPAT;
  return prm.k >= 2 && prm.k <= 96 && !chol && !upd && !prm.warm_start && prm.redo_out && prm.n_redo;
}

int letkf_tc_launch(const LetkfParams& prm, int num_sms, void* stream, int* ctas) {
  return prm.k <= 64 ? launch_tc<64>(prm, num_sms, stream, ctas) : launch_tc<96>(prm, num_sms, stream, ctas);
}

}  // namespace mg
