// Local observation search (LETKF.hpp:159-165 with Location::distance_to).
//
// Grid coordinates: exact integer distances, one warp per grid point, obs
// scanned in order and compacted with warp ballots so every list comes out
// in obs order, as the reference builds it.
//
// Geographic coordinates: a device-built spatial hash of 1 x 1 degree cells.
// Each query column visits only the cells its radius can reach (latitude
// band bound plus a longitude bound from the haversine inequality
// a >= cos(lat_c) cos(lat_o) sin^2(dlon/2)); the reachable cells of one
// latitude band are one or two contiguous runs of the cell-sorted obs, which
// the whole CTA sweeps after one warp has planned them (a lane per band).  The test on a candidate is the squared chord
// |u_c - u_o|^2 between unit vectors (u_o stored with the hash), compared
// with the chord of the radius: haversine <= r  <=>  chord^2 <= 4 sin^2(r/2R),
// with an absolute error near 1e-16 against a band of 2e-9 relative in
// chord^2 (radii of 50 km or more; smaller radii evaluate the reference
// haversine instead).  Lists are sorted by obs index in shared memory.
// Pairs within 1e-9 relative of the radius are re-decided on the host with
// the reference expression (glibc libm), so the selection is bit-exact
// whatever the device's transcendental rounding.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mg_internal.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEarthKm = 6371.0;
constexpr int kNBand = 180, kNLonCell = 360, kNCell = kNBand * kNLonCell;
constexpr int kMaxList = 32768;   // longest per-column list sorted in shared memory (128 KB)
constexpr int kBorderCap = 65536; // near-threshold pairs re-decided on the host
constexpr double kBorderRel = 1e-9;

struct BorderRec {
  int64_t col;
  int64_t obs;
  double clat, clon, olat, olon;
};

// ---------------------------------------------------------------- grid ----
__global__ void select_grid_kernel(int nx, int ny, const int32_t* __restrict__ obs_xy, int64_t p,
                                   double radius, const int64_t* __restrict__ offsets,
                                   int64_t* __restrict__ counts, int32_t* __restrict__ idx) {
  const int lane = threadIdx.x & 31;
  const int64_t npt = (int64_t)nx * ny;
  const int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (g >= npt) return;
  const int gx = (int)(g % nx), gy = (int)(g / nx);
  int64_t w = offsets ? offsets[g] : 0;
  for (int64_t o0 = 0; o0 < p; o0 += 32) {
    const int64_t o = o0 + lane;
    bool in = false;
    if (o < p) {
      const double dx = (double)(gx - obs_xy[2 * o]);
      const double dy = (double)(gy - obs_xy[2 * o + 1]);
      in = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy))) <= radius;
    }
    const unsigned b = __ballot_sync(0xffffffffu, in);
    if (idx && in) idx[w + __popc(b & ((1u << lane) - 1u))] = (int32_t)o;
    w += __popc(b);
  }
  if (!offsets && lane == 0) counts[g] = w;
}

// ----------------------------------------------------------- geographic ---
__device__ __forceinline__ int cell_of(double lat, double lon) {
  int band = (int)floor(lat + 90.0);
  band = band < 0 ? 0 : (band >= kNBand ? kNBand - 1 : band);
  double l = lon - 360.0 * floor(lon / 360.0);
  int c = (int)floor(l);
  c = c < 0 ? 0 : (c >= kNLonCell ? kNLonCell - 1 : c);
  return band * kNLonCell + c;
}

// Location::haversine (Location.hpp:349-357) with the device's libm.
__device__ __forceinline__ double haversine_dev(double lat1, double lon1, double lat2, double lon2) {
  const double dlat = (lat2 - lat1) * kPi / 180.0;
  const double dlon = (lon2 - lon1) * kPi / 180.0;
  const double s1 = sin(dlat / 2), s2 = sin(dlon / 2);
  const double a = s1 * s1 + cos(lat1 * kPi / 180.0) * cos(lat2 * kPi / 180.0) * s2 * s2;
  return kEarthKm * (2 * atan2(sqrt(a), sqrt(1 - a)));
}

__global__ void cell_count_kernel(const double* __restrict__ lat, const double* __restrict__ lon,
                                  int64_t p, unsigned long long* __restrict__ cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p; o += stride)
    atomicAdd(&cnt[cell_of(lat[o], lon[o])], 1ull);
}

__device__ __forceinline__ double3 unit_vec(double lat, double lon) {
  double sa, ca, so, co;
  sincos(lat * kPi / 180.0, &sa, &ca);
  sincos(lon * kPi / 180.0, &so, &co);
  return make_double3(ca * co, ca * so, sa);
}

// Cell-sorted obs: index, latitude, longitude and unit vector.
struct CellObs {
  int32_t* obs;
  double* lat;
  double* lon;
  double* ux;
  double* uy;
  double* uz;
};

// Obs into their cells (positions from the cell starts), with unit vectors
// both cell-sorted and in obs order (the latter for the list distances).
__global__ void cell_scatter_kernel(const double* __restrict__ lat, const double* __restrict__ lon,
                                    int64_t p, const int64_t* __restrict__ start,
                                    unsigned long long* __restrict__ cursor, CellObs co, double* __restrict__ oux,
                                    double* __restrict__ ouy, double* __restrict__ ouz) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p; o += stride) {
    const int c = cell_of(lat[o], lon[o]);
    const int64_t pos = start[c] + (int64_t)atomicAdd(&cursor[c], 1ull);
    co.obs[pos] = (int32_t)o;
    co.lat[pos] = lat[o];
    co.lon[pos] = lon[o];
    const double3 u = unit_vec(lat[o], lon[o]);
    co.ux[pos] = u.x;
    co.uy[pos] = u.y;
    co.uz[pos] = u.z;
    oux[o] = u.x;
    ouy[o] = u.y;
    ouz[o] = u.z;
  }
}

// Search plan of one column in shared memory, made by warp 0: the chord
// thresholds, the column's unit vector, and per reachable latitude band the
// one or two contiguous runs of cell-sorted obs its longitude window covers
// (slots 2 b and 2 b + 1, the second empty where one run suffices).  The
// FP64 transcendentals run once per band on one lane, not on every thread
// of the CTA (GB300's FP64 pipe does about 2 operations per clock per SM).
constexpr int kMaxRuns = 2 * kNBand;

struct ColPlan {
  double la, lo, rlo, rhi, c2lo, c2hi, ux, uy, uz;
  int chord, nrun;
};

__device__ void plan_column(double la, double lo, double radius_km, const int64_t* __restrict__ start,
                            ColPlan& pl, int64_t* run_lo, int64_t* run_hi) {
  const int lane = threadIdx.x & 31;
  const double theta = radius_km / kEarthKm;  // radians
  const double theta_deg = theta * 180.0 / kPi;
  int b0 = (int)floor(la + 90.0 - theta_deg - 1e-6);
  int b1 = (int)floor(la + 90.0 + theta_deg + 1e-6);
  b0 = b0 < 0 ? 0 : b0;
  b1 = b1 >= kNBand ? kNBand - 1 : b1;
  if (lane == 0) {
    const double rlo = radius_km * (1.0 - kBorderRel), rhi = radius_km * (1.0 + kBorderRel);
    const double slo = sin(0.5 * rlo / kEarthKm), shi = sin(0.5 * rhi / kEarthKm);
    const double3 uc = unit_vec(la, lo);
    pl.la = la;
    pl.lo = lo;
    pl.rlo = rlo;
    pl.rhi = rhi;
    pl.c2lo = 4.0 * slo * slo;
    pl.c2hi = 4.0 * shi * shi;
    pl.ux = uc.x;
    pl.uy = uc.y;
    pl.uz = uc.z;
    pl.chord = radius_km >= 50.0;
    pl.nrun = 2 * (b1 - b0 + 1);
  }
  const double sh = sin(0.5 * theta);
  const double a_r = sh * sh;
  const double cosc = cos(la * kPi / 180.0);
  for (int band = b0 + lane; band <= b1; band += 32) {
    const double e0 = (double)band - 90.0, e1 = e0 + 1.0;
    const double emax = fmax(fabs(e0), fabs(e1));
    const double cmin = cos(emax * kPi / 180.0);
    const double denom = cosc * cmin;
    int c0 = 0, c1 = kNLonCell - 1;
    if (denom > a_r * (1.0 + 1e-6)) {
      const double sarg = sqrt(a_r / denom) * (1.0 + 1e-9);
      if (sarg < 1.0) {
        const double dl = 2.0 * asin(sarg) * 180.0 / kPi + 1e-6;
        if (2.0 * dl + 2.0 < 360.0) {
          c0 = (int)floor(lo - dl);
          c1 = (int)floor(lo + dl);
        }
      }
    }
    // The cells c0..c1 (mod 360) as at most two contiguous runs of obs.
    const int bb = band * kNLonCell, slot = 2 * (band - b0);
    run_lo[slot + 1] = run_hi[slot + 1] = 0;
    if (c1 - c0 + 1 >= kNLonCell) {
      run_lo[slot] = start[bb];
      run_hi[slot] = start[bb + kNLonCell];
    } else {
      const int a0 = ((c0 % kNLonCell) + kNLonCell) % kNLonCell;
      const int a1 = ((c1 % kNLonCell) + kNLonCell) % kNLonCell;
      if (a0 <= a1) {
        run_lo[slot] = start[bb + a0];
        run_hi[slot] = start[bb + a1 + 1];
      } else {
        run_lo[slot] = start[bb + a0];
        run_hi[slot] = start[bb + kNLonCell];
        run_lo[slot + 1] = start[bb];
        run_hi[slot + 1] = start[bb + a1 + 1];
      }
    }
  }
}

// Visits every candidate obs of a planned column with the whole CTA and
// calls f(t, cls) for the candidates at cell-sorted position t with
// cls = +1 (inside) or 0 (within 1e-9 relative of the radius).
template <typename F>
__device__ void visit_candidates(const ColPlan& pl, const int64_t* run_lo, const int64_t* run_hi,
                                 const CellObs& co, F&& f) {
  const int nrun = pl.nrun;
  const bool chord = pl.chord;
  const double ux = pl.ux, uy = pl.uy, uz = pl.uz, c2lo = pl.c2lo, c2hi = pl.c2hi;
  for (int r = 0; r < nrun; ++r) {
    const int64_t hi = run_hi[r];
    for (int64_t t = run_lo[r] + threadIdx.x; t < hi; t += blockDim.x) {
      if (chord) {
        const double dx = co.ux[t] - ux, dy = co.uy[t] - uy, dz = co.uz[t] - uz;
        const double c2 = dx * dx + dy * dy + dz * dz;
        if (c2 <= c2lo) f(t, 1);
        else if (c2 <= c2hi) f(t, 0);
      } else {
        const double d = haversine_dev(pl.la, pl.lo, co.lat[t], co.lon[t]);
        if (d <= pl.rlo) f(t, 1);
        else if (d <= pl.rhi) f(t, 0);
      }
    }
  }
}

// asin(h) for a half chord 0 <= h <= 1.  Up to h = 0.05 (great-circle
// distances up to about 640 km) by its Maclaurin series
// asin h = sum_n (2n)! / (4^n (n!)^2 (2n + 1)) h^(2n+1), through n = 5: the
// first omitted term, 231/13312 h^13, is below 1e-18 of h there, so the
// result is the correctly rounded value to within a few units in the last
// place, at six FP64 multiply-adds (FP64 runs at 1/64 of the FP32 rate);
// larger h take the library asin.
__device__ __forceinline__ double asin_half_chord(double h) {
  if (h > 0.05) return asin(h < 1.0 ? h : 1.0);
  const double h2 = h * h;
  double q = 63.0 / 2816.0;
  q = fma(q, h2, 35.0 / 1152.0);
  q = fma(q, h2, 5.0 / 112.0);
  q = fma(q, h2, 3.0 / 40.0);
  q = fma(q, h2, 1.0 / 6.0);
  return fma(h * h2, q, h);
}

__device__ __forceinline__ bool key_rejected(const unsigned long long* rej, int nrej,
                                             unsigned long long key) {
  int lo = 0, hi = nrej;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (rej[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo < nrej && rej[lo] == key;
}

__global__ void __launch_bounds__(256) geo_count_kernel(
    const double* __restrict__ col_lat, const double* __restrict__ col_lon, int64_t ncol,
    double radius_km, const int64_t* __restrict__ start, CellObs co, int64_t* __restrict__ counts,
    BorderRec* __restrict__ border, unsigned long long* __restrict__ nborder) {
  __shared__ unsigned long long scount;
  __shared__ ColPlan pl;
  __shared__ int64_t run_lo[kMaxRuns], run_hi[kMaxRuns];
  const int64_t col = blockIdx.x;
  if (threadIdx.x == 0) scount = 0;
  const double la = col_lat[col], lo = col_lon[col];
  if (threadIdx.x < 32) plan_column(la, lo, radius_km, start, pl, run_lo, run_hi);
  __syncthreads();
  unsigned long long mine = 0;
  visit_candidates(pl, run_lo, run_hi, co, [&](int64_t t, int cls) {
    ++mine;
    if (cls == 0) {
      const unsigned long long slot = atomicAdd(nborder, 1ull);
      if (slot < (unsigned long long)kBorderCap)
        border[slot] = BorderRec{col, (int64_t)co.obs[t], la, lo, co.lat[t], co.lon[t]};
    }
  });
  atomicAdd(&scount, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    counts[col] = (int64_t)scount;
    atomicMax(nborder + 1, scount);  // the longest list sizes the fill pass's shared memory
  }
}

__global__ void apply_rejections_kernel(const unsigned long long* __restrict__ rej, int nrej,
                                        int64_t* __restrict__ counts) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nrej) atomicAdd(reinterpret_cast<unsigned long long*>(&counts[rej[t] >> 32]),
                          (unsigned long long)-1ll);
}

__global__ void __launch_bounds__(256) geo_fill_kernel(
    const double* __restrict__ col_lat, const double* __restrict__ col_lon, int64_t ncol,
    double radius_km, const int64_t* __restrict__ start, CellObs co,
    const int64_t* __restrict__ offsets, const unsigned long long* __restrict__ rej, int nrej,
    const double* __restrict__ obs_lat, const double* __restrict__ obs_lon, const double* __restrict__ oux,
    const double* __restrict__ ouy, const double* __restrict__ ouz, int32_t* __restrict__ idx,
    double* __restrict__ dist, int* __restrict__ overflow, int list_cap) {
  extern __shared__ int32_t slist[];  // list_cap entries, a power of two
  __shared__ int scount;
  __shared__ ColPlan pl;
  __shared__ int64_t run_lo[kMaxRuns], run_hi[kMaxRuns];
  const int64_t col = blockIdx.x;
  const int64_t base = offsets[col];
  const int64_t n = offsets[col + 1] - base;
  if (n == 0) return;
  if (n > list_cap) {
    if (threadIdx.x == 0) atomicExch(overflow, 1);
    return;
  }
  if (threadIdx.x == 0) scount = 0;
  const double la = col_lat[col], lo = col_lon[col];
  if (threadIdx.x < 32) plan_column(la, lo, radius_km, start, pl, run_lo, run_hi);
  __syncthreads();
  visit_candidates(pl, run_lo, run_hi, co, [&](int64_t t, int cls) {
    const int32_t o = co.obs[t];
    if (cls == 0 && nrej > 0 && key_rejected(rej, nrej, ((unsigned long long)col << 32) | (unsigned)o)) return;
    const int pos = atomicAdd(&scount, 1);
    if (pos < list_cap) slist[pos] = o;
  });
  __syncthreads();
  const int cnt = scount;
  if (cnt != (int)n) {  // count and fill passes disagree: report, write nothing
    if (threadIdx.x == 0) atomicExch(overflow, 2);
    return;
  }
  int m = 1;
  while (m < cnt) m <<= 1;
  for (int t = cnt + threadIdx.x; t < m; t += blockDim.x) slist[t] = 0x7fffffff;
  __syncthreads();
  // Bitonic sort by obs index (obs order, as LETKF.hpp:160-165).
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < (m >> 1); t += blockDim.x) {
        const int lo_i = 2 * t - (t & (stride - 1));
        const int hi_i = lo_i + stride;
        const bool up = ((lo_i & size) == 0);
        const int a = slist[lo_i], b = slist[hi_i];
        if ((a > b) == up) {
          slist[lo_i] = b;
          slist[hi_i] = a;
        }
      }
      __syncthreads();
    }
  }
  const bool chord = pl.chord;
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int o = slist[t];
    idx[base + t] = o;
    if (dist) {
      if (chord) {  // d = 2R asin(chord / 2): well conditioned for chords up to the radius
        const double dx = oux[o] - pl.ux, dy = ouy[o] - pl.uy, dz = ouz[o] - pl.uz;
        const double h = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
        dist[base + t] = 2.0 * kEarthKm * asin_half_chord(h);
      } else {
        dist[base + t] = haversine_dev(la, lo, obs_lat[o], obs_lon[o]);
      }
    }
  }
}

// Host-side reference predicate for near-threshold pairs (Location.hpp:349-357).
double haversine_host(double lat1, double lon1, double lat2, double lon2) {
  auto deg2rad = [](double deg) { return deg * kPi / 180.0; };
  const double dlat = deg2rad(lat2 - lat1);
  const double dlon = deg2rad(lon2 - lon1);
  const double a = std::sin(dlat / 2) * std::sin(dlat / 2) +
                   std::cos(deg2rad(lat1)) * std::cos(deg2rad(lat2)) * std::sin(dlon / 2) *
                       std::sin(dlon / 2);
  const double c = 2 * std::atan2(std::sqrt(a), std::sqrt(1 - a));
  return kEarthKm * c;
}

}  // namespace

extern "C" {

int mg_select_grid(mg_context* ctx, int32_t nx, int32_t ny, const int32_t* obs_xy, int64_t p,
                   double radius, int64_t* offsets, int32_t* idx, int64_t cap, int64_t* total) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(nx > 0 && ny > 0 && p >= 0 && offsets && total && (p == 0 || obs_xy),
               "mg_select_grid: bad arguments");
  const int64_t npt = (int64_t)nx * ny;
  const size_t tmpb = mg::scan_temp_bytes(npt);
  mg::Carver cv;
  cv.reserve<int64_t>(npt + 1);
  cv.reserve<char>(tmpb);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  int64_t* counts = cv.take<int64_t>(npt + 1);
  void* tmp = cv.take<char>(tmpb);
  const unsigned blocks = (unsigned)((npt + 7) / 8);
  MG_TRY_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t) * (npt + 1), ctx->stream));
  select_grid_kernel<<<blocks, 256, 0, ctx->stream>>>(nx, ny, obs_xy, p, radius, nullptr, counts,
                                                      nullptr);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  MG_TRY_CUDA(mg::exclusive_scan(counts, offsets, npt, tmp, tmpb, ctx->stream));
  MG_TRY_CUDA(cudaMemcpyAsync(total, offsets + npt, sizeof(int64_t), cudaMemcpyDeviceToHost,
                              ctx->stream));
  MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
  if (*total > cap || (*total > 0 && !idx))
    return mg::fail(ctx, MG_ERR_CAPACITY, "mg_select_grid: index buffer too small");
  if (*total > 0) {
    select_grid_kernel<<<blocks, 256, 0, ctx->stream>>>(nx, ny, obs_xy, p, radius, offsets, nullptr,
                                                        idx);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
  }
  return MG_OK;
}

int mg_select_geo(mg_context* ctx, const double* col_lat, const double* col_lon, int64_t ncol,
                  const double* obs_lat, const double* obs_lon, int64_t p, double radius_km,
                  int64_t* offsets, int32_t* idx, double* dist_km, int64_t cap, int64_t* total) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(col_lat && col_lon && ncol > 0 && p >= 0 && offsets && total && radius_km >= 0 &&
                   (p == 0 || (obs_lat && obs_lon)),
               "mg_select_geo: bad arguments");
  MG_CHECK_ARG(radius_km < 0.5 * kPi * kEarthKm, "mg_select_geo: radius must be below a quarter great circle");
  const size_t tmp_cells = mg::scan_temp_bytes(kNCell);
  const size_t tmp_cols = mg::scan_temp_bytes(ncol);
  const size_t tmpb = std::max(tmp_cells, tmp_cols);
  mg::Carver cv;
  cv.reserve<unsigned long long>(kNCell + 1);  // cell counts, then cursor
  cv.reserve<unsigned long long>(kNCell + 1);
  cv.reserve<int64_t>(kNCell + 1);             // cell start
  cv.reserve<int32_t>(p + 1);
  for (int a = 0; a < 8; ++a) cv.reserve<double>(p + 1);  // lat, lon, unit vector; unit vector in obs order
  cv.reserve<int64_t>(ncol + 1);               // column counts
  cv.reserve<BorderRec>(kBorderCap);
  cv.reserve<unsigned long long>(kBorderCap);  // rejected keys
  cv.reserve<unsigned long long>(2);           // n_border
  cv.reserve<int>(2);                          // overflow flag
  cv.reserve<char>(tmpb);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  auto* ccount = cv.take<unsigned long long>(kNCell + 1);
  auto* ccursor = cv.take<unsigned long long>(kNCell + 1);
  auto* cstart = cv.take<int64_t>(kNCell + 1);
  CellObs co;
  co.obs = cv.take<int32_t>(p + 1);
  co.lat = cv.take<double>(p + 1);
  co.lon = cv.take<double>(p + 1);
  co.ux = cv.take<double>(p + 1);
  co.uy = cv.take<double>(p + 1);
  co.uz = cv.take<double>(p + 1);
  double* oux = cv.take<double>(p + 1);
  double* ouy = cv.take<double>(p + 1);
  double* ouz = cv.take<double>(p + 1);
  auto* counts = cv.take<int64_t>(ncol + 1);
  auto* border = cv.take<BorderRec>(kBorderCap);
  auto* rej = cv.take<unsigned long long>(kBorderCap);
  auto* nborder = cv.take<unsigned long long>(2);
  auto* overflow = cv.take<int>(2);
  void* tmp = cv.take<char>(tmpb);
  cudaStream_t s = ctx->stream;

  // Spatial hash: counting sort of obs into cells.
  MG_TRY_CUDA(cudaMemsetAsync(ccount, 0, sizeof(unsigned long long) * (kNCell + 1), s));
  MG_TRY_CUDA(cudaMemsetAsync(ccursor, 0, sizeof(unsigned long long) * (kNCell + 1), s));
  MG_TRY_CUDA(cudaMemsetAsync(nborder, 0, sizeof(unsigned long long) * 2, s));
  MG_TRY_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int) * 2, s));
  MG_TRY_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t) * (ncol + 1), s));
  if (p > 0) {
    const unsigned gb = (unsigned)std::min<int64_t>((p + 255) / 256, 152 * 16);
    cell_count_kernel<<<gb, 256, 0, s>>>(obs_lat, obs_lon, p, ccount);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
    MG_TRY_CUDA(mg::exclusive_scan(reinterpret_cast<const int64_t*>(ccount), cstart, kNCell, tmp,
                                   tmpb, s));
    cell_scatter_kernel<<<gb, 256, 0, s>>>(obs_lat, obs_lon, p, cstart, ccursor, co, oux, ouy, ouz);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
  } else {
    MG_TRY_CUDA(cudaMemsetAsync(cstart, 0, sizeof(int64_t) * (kNCell + 1), s));
  }
  // Pass 1: counts (near-threshold pairs counted and recorded).
  geo_count_kernel<<<(unsigned)ncol, 256, 0, s>>>(col_lat, col_lon, ncol, radius_km, cstart, co, counts, border,
                                                  nborder);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  unsigned long long nbm[2] = {0, 0};
  MG_TRY_CUDA(cudaMemcpyAsync(nbm, nborder, sizeof(nbm), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  const unsigned long long nb = nbm[0], longest = nbm[1];
  if (longest > (unsigned long long)kMaxList)
    return mg::fail(ctx, MG_ERR_CAPACITY, "mg_select_geo: a local list exceeds 32768 obs");
  if (nb > (unsigned long long)kBorderCap)
    return mg::fail(ctx, MG_ERR_CAPACITY, "mg_select_geo: too many near-threshold pairs");
  int nrej = 0;
  if (nb > 0) {
    std::vector<BorderRec> recs(nb);
    MG_TRY_CUDA(cudaMemcpy(recs.data(), border, sizeof(BorderRec) * nb, cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> keys;
    for (const auto& r : recs)
      if (!(haversine_host(r.clat, r.clon, r.olat, r.olon) <= radius_km))
        keys.push_back(((unsigned long long)r.col << 32) | (unsigned long long)(uint32_t)r.obs);
    std::sort(keys.begin(), keys.end());
    nrej = (int)keys.size();
    if (nrej > 0) {
      MG_TRY_CUDA(cudaMemcpy(rej, keys.data(), sizeof(unsigned long long) * nrej,
                             cudaMemcpyHostToDevice));
      apply_rejections_kernel<<<(nrej + 255) / 256, 256, 0, s>>>(rej, nrej, counts);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
    }
  }
  MG_TRY_CUDA(mg::exclusive_scan(counts, offsets, ncol, tmp, tmpb, s));
  MG_TRY_CUDA(cudaMemcpyAsync(total, offsets + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  if (*total > cap || (*total > 0 && !idx))
    return mg::fail(ctx, MG_ERR_CAPACITY, "mg_select_geo: index buffer too small");
  if (*total == 0) return MG_OK;
  // Pass 2: fill, sort each list by obs index, distances.
  int smem_entries = 32;
  while ((unsigned long long)smem_entries < longest) smem_entries <<= 1;
  const size_t smem = sizeof(int32_t) * smem_entries;
  MG_TRY_CUDA(cudaFuncSetAttribute(geo_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  geo_fill_kernel<<<(unsigned)ncol, 256, smem, s>>>(col_lat, col_lon, ncol, radius_km, cstart, co, offsets, rej,
                                                    nrej, obs_lat, obs_lon, oux, ouy, ouz, idx, dist_km, overflow,
                                                    smem_entries);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  int ovf = 0;
  MG_TRY_CUDA(cudaMemcpyAsync(&ovf, overflow, sizeof(int), cudaMemcpyDeviceToHost, s));
  MG_TRY_CUDA(cudaStreamSynchronize(s));
  if (ovf == 1) return mg::fail(ctx, MG_ERR_CAPACITY, "mg_select_geo: a local list exceeds its sort buffer");
  if (ovf == 2) return mg::fail(ctx, MG_ERR_NUMERIC, "mg_select_geo: count and fill passes disagree");
  return MG_OK;
}

}  // extern "C"
