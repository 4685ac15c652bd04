// Parameters of the batched local analyses, shared by the SIMT kernels
// (mg_letkf.cu) and the tensor-core kernel (mg_letkf_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mg {

struct LetkfParams {
  int k, kp, n_var, nlev;
  int64_t ncol, npoints;
  const int64_t* col_base;
  int64_t lev_stride, var_stride;
  const void* Xp;        // point-major perturbations, TE, [s*k + i]
  const double* xmean;   // n
  double* Xa;            // point-major analysis, [s*k + i]
  float* Xa32;           // or, for members stored as FP32, the FP32 analysis (may be Xp itself:
                         // each point's rows are read before they are written)
  const void* Y;         // obs anomalies, TE, [o*k + i]
  const double* dinn;    // innovation
  const double* rinv;    // 1 / error variance
  const double* obs_lev; // or null
  const float4* opack;    // tensor-core path: per obs (level, 1/sigma^2, innovation, 0) in FP32
  const int64_t* loc_off;
  const int32_t* loc_idx;
  const double* loc_dist;  // or null
  double hsupport, vsupport, rho;
  int flags;
  const int32_t* order;  // columns in work order (the grid's order)
  unsigned long long* next;
  unsigned long long* n_empty;
  unsigned long long* total_local;
  unsigned long long* total_sweeps;
  int* max_local;
  int* max_sweeps;
  int* status;
  double tol;
  int sweep_cap;
  int warm_start;  // levels of a column run in sequence, each Jacobi warm-started
  // Tensor-core path: analyses it hands back (points col * nlev + lev) and
  // their count; the largest first-order residual seen (float bits).
  int32_t* redo_out;
  unsigned long long* n_redo;
  unsigned* max_resid_bits;
  // SIMT path: when set, item i is the point redo_in[i] (col * nlev + lev)
  // instead of the column work order.
  const int32_t* redo_in;
  // Tensor-core path: when set, each column's candidates sorted by obs level
  // bucket (stable; bucket = floor(obs level) clamped to the grid's levels):
  // lev_boff[col * (nlev + 1) + b] is bucket b's start within the column's
  // range of loc_off, and bidx / bdist the sorted entries (same index space
  // as loc_idx / loc_dist).  An analysis at level l walks only the buckets
  // floor(l - vsupport) .. floor(l + vsupport).
  const int32_t* lev_boff;
  const int32_t* bidx;
  const double* bdist;
};

// Analysis value of point-major element idx, in the output's precision.
__device__ __forceinline__ void letkf_store(const LetkfParams& prm, int64_t idx, double v) {
  if (prm.Xa32) prm.Xa32[idx] = (float)v;
  else prm.Xa[idx] = v;
}
__device__ __forceinline__ void letkf_add(const LetkfParams& prm, int64_t idx, double dv) {
  if (prm.Xa32) prm.Xa32[idx] = (float)((double)prm.Xa32[idx] + dv);
  else prm.Xa[idx] += dv;
}

// Gaspari-Cohn (1999, eq. 4.10) fifth-order compactly supported function of
// z = distance / (support / 2).  FP64 evaluates the published polynomials
// in the oracle's operation order (the FP64 path's local lists are
// bit-identical to the oracle's).  In FP32 the outer polynomial cancels
// near z = 2, where the function vanishes to fourth order, and rounds to
// zero or below for z within about 1 % of the support, dropping candidates
// that FP64 keeps with tiny weights; FP32 uses the exact factored form
// z f(z) = (2 - z)^4 (z^2 + 2z - 1/2) / 12 instead (2 - z is exact for
// 1 <= z <= 2), which is positive for every z < 2.
template <typename T>
__device__ __forceinline__ T gaspari_cohn(T z) {
  z = fabs(z);
  if (z >= T(2)) return T(0);
  if (z <= T(1))
    return (((T(-0.25) * z + T(0.5)) * z + T(0.625)) * z - T(5.0 / 3.0)) * z * z + T(1);
  if constexpr (sizeof(T) == sizeof(float)) {
    const T t = T(2) - z;
    const T t2 = t * t;
    return (t2 * t2) * ((z + T(2)) * z - T(0.5)) / (T(12) * z);
  } else {
    return ((((z / T(12) - T(0.5)) * z + T(0.625)) * z + T(5.0 / 3.0)) * z - T(5)) * z + T(4) -
           T(2) / (T(3) * z);
  }
}

// Tensor-core local analyses (mixed precision, Hunt transform, k <= 96):
// true when this build and the parameters take that path.
bool letkf_tc_supported(const LetkfParams& prm);
// Launches them on `stream` as a persistent grid (two CTAs per SM for
// k <= 64, one for 64 < k <= 96); returns a cudaError_t value (0 on success)
// and the CTA count.
int letkf_tc_launch(const LetkfParams& prm, int num_sms, void* stream, int* ctas);

}  // namespace mg
