// Observation operators (HX) and the obs-space prior (mean, anomalies,
// innovation).  Arithmetic that must be bit-identical to the reference uses
// explicitly rounded intrinsics so the compiler cannot contract a multiply
// and an add into one FMA.
#include "mg_internal.h"

namespace {

// IdentityObsOperator.hpp:594-617 (2-D branch) and :643-676 for an obs at
// integer grid coordinates (ox, oy) on member x.
__device__ __forceinline__ double idw4(const double* __restrict__ x, int nx, int ny, int ox,
                                       int oy) {
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
    ws = __dadd_rn(ws, __dmul_rn(w, __ldg(x + jj[t] * nx + ii[t])));
    wsum = __dadd_rn(wsum, w);
  }
  return __ddiv_rn(ws, wsum);
}

__global__ void hx_idw4_kernel(const double* __restrict__ X, int k, int64_t ld, int nx, int ny,
                               const int32_t* __restrict__ obs_xy, const uint8_t* __restrict__ valid,
                               int64_t p, double* __restrict__ HX) {
  const int64_t total = p * k;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int64_t o = e / k;
    const int i = (int)(e - o * k);
    double v = 0.0;
    if (!valid || valid[o]) v = idw4(X + (int64_t)i * ld, nx, ny, obs_xy[2 * o], obs_xy[2 * o + 1]);
    HX[e] = v;
  }
}

// Bilinear in (lon, lat), linear in level; the operation order matches the
// oracle's restatement exactly.
// TX: the members' storage type (FP64, or FP32 widened to FP64 on load).
//
// Each warp takes 32 obs.  Lane j first computes obs j's grid geometry
// (fractional indices, weights, plane offsets: about 30 FP64 operations,
// which GB300 runs at 1/64 of the FP32 rate) and leaves it in shared memory;
// then the warp walks the 32 obs with its lanes over the members, so the
// geometry is computed once per obs instead of once per (obs, member).
struct LatLonGeom {
  double ax, fx, ay, fy, az, fz;
  int64_t lo, hi;  // offsets of the two level planes from the member's start
  int64_t r0, r1;  // j0 nlon, (j0 + 1) nlon
  int32_t i0, i1;
  int32_t valid;
};

template <typename TX>
__global__ void __launch_bounds__(256) hx_latlon_kernel(const TX* __restrict__ X, int k, int64_t ld, int nlon,
                                                        int nlat, int nlev, const double* __restrict__ olat,
                                                        const double* __restrict__ olon,
                                                        const double* __restrict__ olev,
                                                        const int32_t* __restrict__ ovar, int64_t p,
                                                        double* __restrict__ HX) {
  __shared__ LatLonGeom geo[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t plane = (int64_t)nlat * nlon;
  const int64_t nwarps = (int64_t)gridDim.x * 8;
  for (int64_t o0 = ((int64_t)blockIdx.x * 8 + w) * 32; o0 < p; o0 += nwarps * 32) {
    {
      const int64_t o = o0 + lane;
      LatLonGeom g{};
      // Reads stay inside member m: the variable must fit within the member
      // stride and the coordinates must be finite; otherwise the value is NaN.
      if (o < p && isfinite(olon[o]) && isfinite(olat[o]) && isfinite(olev[o]) && ovar[o] >= 0 &&
          ((int64_t)ovar[o] + 1) * nlev * plane <= ld) {
        // Fractional grid indices: lon_i = (i + 0.5) dlon, lat_j = -90 + (j + 0.5) dlat.
        const double dlon = 360.0 / (double)nlon, dlat = 180.0 / (double)nlat;
        const double gx = __dsub_rn(__ddiv_rn(olon[o], dlon), 0.5);
        const double fxl = floor(gx);
        const double fx = __dsub_rn(gx, fxl);
        long long i0 = (long long)fxl % nlon;
        if (i0 < 0) i0 += nlon;
        const long long i1 = (i0 + 1) % nlon;
        double gy = __dsub_rn(__ddiv_rn(__dadd_rn(olat[o], 90.0), dlat), 0.5);
        gy = fmax(0.0, fmin((double)(nlat - 1), gy));
        long long j0 = (long long)floor(gy);
        if (j0 > nlat - 2) j0 = nlat - 2;
        const double fy = __dsub_rn(gy, (double)j0);
        const double gz = fmax(0.0, fmin((double)(nlev - 1), olev[o]));
        long long l0 = (long long)floor(gz);
        if (l0 > nlev - 2) l0 = nlev - 2;
        if (l0 < 0) l0 = 0;
        const double fz = (nlev > 1) ? __dsub_rn(gz, (double)l0) : 0.0;
        const long long l1 = (nlev > 1) ? l0 + 1 : l0;
        const int64_t vb = (int64_t)ovar[o] * nlev * plane;
        g.ax = __dsub_rn(1.0, fx);
        g.fx = fx;
        g.ay = __dsub_rn(1.0, fy);
        g.fy = fy;
        g.az = __dsub_rn(1.0, fz);
        g.fz = fz;
        g.lo = vb + l0 * plane;
        g.hi = vb + l1 * plane;
        g.r0 = (int64_t)j0 * nlon;
        g.r1 = (int64_t)(j0 + 1) * nlon;
        g.i0 = (int32_t)i0;
        g.i1 = (int32_t)i1;
        g.valid = 1;
      }
      geo[w][lane] = g;
    }
    __syncwarp();
    const int nob = (p - o0 < 32) ? (int)(p - o0) : 32;
    for (int j = 0; j < nob; ++j) {
      const LatLonGeom& g = geo[w][j];
      const int64_t o = o0 + j;
      for (int m = lane; m < k; m += 32) {
        const int64_t e = o * k + m;
        if (!g.valid) {
          HX[e] = __longlong_as_double(0x7ff8000000000000LL);
          continue;
        }
        const TX* lo = X + (int64_t)m * ld + g.lo;
        const TX* hi = X + (int64_t)m * ld + g.hi;
        const double l00 = (double)lo[g.r0 + g.i0], l01 = (double)lo[g.r0 + g.i1];
        const double l10 = (double)lo[g.r1 + g.i0], l11 = (double)lo[g.r1 + g.i1];
        const double h00 = (double)hi[g.r0 + g.i0], h01 = (double)hi[g.r0 + g.i1];
        const double h10 = (double)hi[g.r1 + g.i0], h11 = (double)hi[g.r1 + g.i1];
        const double b0 = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(l00, g.ax), __dmul_rn(l01, g.fx)), g.ay),
                                    __dmul_rn(__dadd_rn(__dmul_rn(l10, g.ax), __dmul_rn(l11, g.fx)), g.fy));
        const double b1 = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(h00, g.ax), __dmul_rn(h01, g.fx)), g.ay),
                                    __dmul_rn(__dadd_rn(__dmul_rn(h10, g.ax), __dmul_rn(h11, g.fx)), g.fy));
        HX[e] = __dadd_rn(__dmul_rn(b0, g.az), __dmul_rn(b1, g.fz));
      }
    }
    __syncwarp();
  }
}

// One warp per observation: ym = (sum_i HX[o,i]) / k (rowwise().mean()),
// Y' = HX - ym, d = yo - ym, rinv = 1 / rvar.
__global__ void obs_prior_kernel(const double* __restrict__ HX, const double* __restrict__ yo,
                                 const double* __restrict__ rvar, int64_t p, int k,
                                 double* __restrict__ Y64, float* __restrict__ Y32,
                                 double* __restrict__ d, double* __restrict__ rinv) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t o = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); o < p; o += warps) {
    const double* h = HX + o * k;
    double s = 0.0;
    for (int i = lane; i < k; i += 32) s += h[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const double ym = s / (double)k;
    for (int i = lane; i < k; i += 32) {
      const double v = h[i] - ym;
      if (Y64) Y64[o * k + i] = v;
      if (Y32) Y32[o * k + i] = (float)v;
    }
    if (lane == 0) {
      if (d) d[o] = yo[o] - ym;
      if (rinv) rinv[o] = 1.0 / rvar[o];
    }
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 64) b = 152 * 64;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

namespace mg {

cudaError_t launch_obs_prior(const double* HX, const double* yo, const double* rvar, int64_t p,
                             int k, double* Y64, float* Y32, double* d, double* rinv,
                             cudaStream_t s) {
  if (p <= 0) return cudaSuccess;
  obs_prior_kernel<<<grid_for(p * 32, 256), 256, 0, s>>>(HX, yo, rvar, p, k, Y64, Y32, d, rinv);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

}  // namespace mg

extern "C" {

int mg_hx_idw4(mg_context* ctx, const double* X, int32_t k, int64_t ld, int32_t nx, int32_t ny,
               const int32_t* obs_xy, const uint8_t* valid, int64_t p, double* HX) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && obs_xy && HX && k > 0 && nx > 0 && ny > 0 && p >= 0 && ld >= (int64_t)nx * ny,
               "mg_hx_idw4: bad arguments");
  if (p == 0) return MG_OK;
  hx_idw4_kernel<<<grid_for(p * k, 256), 256, 0, ctx->stream>>>(X, k, ld, nx, ny, obs_xy, valid, p,
                                                                HX);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_hx_latlon(mg_context* ctx, const double* X, int32_t k, int64_t ld, int32_t nlon,
                 int32_t nlat, int32_t nlev, const double* obs_lat, const double* obs_lon,
                 const double* obs_lev, const int32_t* obs_var, int64_t p, double* HX) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && obs_lat && obs_lon && obs_lev && obs_var && HX && k > 0 && nlon > 0 &&
                   nlat > 1 && nlev > 0 && p >= 0,
               "mg_hx_latlon: bad arguments");
  if (p == 0) return MG_OK;
  hx_latlon_kernel<double><<<grid_for((p + 31) / 32 * 32, 256), 256, 0, ctx->stream>>>(X, k, ld, nlon, nlat, nlev,
                                                                          obs_lat, obs_lon, obs_lev,
                                                                          obs_var, p, HX);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_hx_latlon_f32(mg_context* ctx, const float* X, int32_t k, int64_t ld, int32_t nlon,
                     int32_t nlat, int32_t nlev, const double* obs_lat, const double* obs_lon,
                     const double* obs_lev, const int32_t* obs_var, int64_t p, double* HX) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && obs_lat && obs_lon && obs_lev && obs_var && HX && k > 0 && nlon > 0 &&
                   nlat > 1 && nlev > 0 && p >= 0,
               "mg_hx_latlon_f32: bad arguments");
  if (p == 0) return MG_OK;
  hx_latlon_kernel<float><<<grid_for((p + 31) / 32 * 32, 256), 256, 0, ctx->stream>>>(X, k, ld, nlon, nlat, nlev,
                                                                         obs_lat, obs_lon, obs_lev,
                                                                         obs_var, p, HX);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // extern "C"
