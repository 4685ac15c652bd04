// Nearest grid node of geographic observations on a curvilinear grid: the
// search of IdentityObsOperator::convertGeographicToGrid
// (src/backends/common/obsoperator/IdentityObsOperator.hpp:470-505) with a
// device spatial hash instead of a scan of every node per observation.
//
// The reference takes, over the nodes in index order, the first minimum of
//     dist = sqrt((lon - lon_n)^2 + (lat - lat_n)^2)
// (Euclidean in degrees, no wrap-around), i.e. the lexicographic minimum of
// (dist, index).  Here the nodes are bucketed on a uniform grid of cells
// over their bounding box (about four nodes per cell); one thread per
// observation visits the rings of cells around its own cell, keeping the
// (dist, index) minimum, and stops once no unvisited cell can hold a node at
// a distance <= the best (a tie with a lower index is then impossible).
// Distances use explicit round-to-nearest operations, so they and the
// chosen nodes equal the reference's bit for bit.  The square root is taken
// only near the running best: sqrt_rn maps s' and s to one value only if
// s' <= s (1 + 2^-51), so a node whose sum of squares exceeds the best one's
// times (1 + 2^-50), rounded up, is strictly farther and is skipped without
// it.  The vertical index is
// the first z minimising |level - vcoord[z]| (:491-500).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "mg_internal.h"

namespace {

constexpr int kThreads = 256;

struct NodeHash {
  double x0, y0, w, h;  // origin and cell size (lon, lat)
  int cx, cy;           // cells per axis
};

__device__ __forceinline__ int cell_x(const NodeHash& g, double x) {
  int c = (int)floor((x - g.x0) / g.w);
  return c < 0 ? 0 : (c >= g.cx ? g.cx - 1 : c);
}
__device__ __forceinline__ int cell_y(const NodeHash& g, double y) {
  int c = (int)floor((y - g.y0) / g.h);
  return c < 0 ? 0 : (c >= g.cy ? g.cy - 1 : c);
}

__global__ void node_count_kernel(const double* __restrict__ lat, const double* __restrict__ lon, int64_t nn,
                                  NodeHash g, unsigned long long* __restrict__ cnt) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[(int64_t)cell_y(g, lat[t]) * g.cx + cell_x(g, lon[t])], 1ull);
}

__global__ void node_scatter_kernel(const double* __restrict__ lat, const double* __restrict__ lon, int64_t nn,
                                    NodeHash g, const int64_t* __restrict__ start,
                                    unsigned long long* __restrict__ cursor, int64_t* __restrict__ sidx,
                                    double* __restrict__ slat, double* __restrict__ slon) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = (int64_t)cell_y(g, lat[t]) * g.cx + cell_x(g, lon[t]);
    const int64_t pos = start[c] + (int64_t)atomicAdd(&cursor[c], 1ull);
    sidx[pos] = t;
    slat[pos] = lat[t];
    slon[pos] = lon[t];
  }
}

// Bounding box of the nodes: per-CTA (min lon, max lon, min lat, max lat,
// non-finite count), then one CTA over the CTAs.
constexpr int kBoxBlocks = 152 * 4;

__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double2hiint(x) >> 20) & 0x7ff) != 0x7ff;
}

__global__ void __launch_bounds__(kThreads) node_box_kernel(const double* __restrict__ lat,
                                                            const double* __restrict__ lon, int64_t nn,
                                                            double* __restrict__ part) {
  __shared__ double red[5][kThreads / 32];
  double v[5] = {INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0};
  for (int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x; t < nn; t += (int64_t)gridDim.x * kThreads) {
    const double x = lon[t], y = lat[t];
    if (!finite_bits(x) || !finite_bits(y)) {
      v[4] += 1.0;
      continue;
    }
    v[0] = fmin(v[0], x);
    v[1] = fmax(v[1], x);
    v[2] = fmin(v[2], y);
    v[3] = fmax(v[3], y);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v[0] = fmin(v[0], __shfl_xor_sync(0xffffffffu, v[0], off));
    v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], off));
    v[2] = fmin(v[2], __shfl_xor_sync(0xffffffffu, v[2], off));
    v[3] = fmax(v[3], __shfl_xor_sync(0xffffffffu, v[3], off));
    v[4] += __shfl_xor_sync(0xffffffffu, v[4], off);
  }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 5; ++q) red[q][warp] = v[q];
  __syncthreads();
  if (threadIdx.x < 5) {
    const int q = threadIdx.x;
    double r = red[q][0];
    for (int w = 1; w < kThreads / 32; ++w)
      r = (q == 0 || q == 2) ? fmin(r, red[q][w]) : (q == 4 ? r + red[q][w] : fmax(r, red[q][w]));
    part[(int64_t)blockIdx.x * 5 + q] = r;
  }
}

// One warp per quantity: lanes stride over the partials, then a shuffle
// tree (the sum is of small integer counts, exact in any order).
__global__ void node_box_final_kernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= 5) return;
  auto op = [q](double a, double b) { return (q == 0 || q == 2) ? fmin(a, b) : (q == 4 ? a + b : fmax(a, b)); };
  double r = (q == 0 || q == 2) ? INFINITY : (q == 4 ? 0.0 : -INFINITY);
  for (int b = lane; b < nb; b += 32) r = op(r, part[(int64_t)b * 5 + q]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) r = op(r, __shfl_xor_sync(0xffffffffu, r, off));
  if (lane == 0) out[q] = r;
}

// dx^2 + dy^2 with the reference's roundings; the distance is its sqrt_rn.
__device__ __forceinline__ double node_dist2(double lat, double lon, double glat, double glon) {
  const double dx = __dsub_rn(lon, glon), dy = __dsub_rn(lat, glat);
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

__global__ void __launch_bounds__(kThreads) nearest_kernel(const double* __restrict__ olat,
                                                           const double* __restrict__ olon, int64_t p, NodeHash g,
                                                           const int64_t* __restrict__ start,
                                                           const int64_t* __restrict__ sidx,
                                                           const double* __restrict__ slat,
                                                           const double* __restrict__ slon, int32_t nx,
                                                           const double* __restrict__ vcoord, int32_t nz,
                                                           const double* __restrict__ olev,
                                                           int32_t* __restrict__ out_xy, int32_t* __restrict__ out_k) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= p) return;
  const double la = olat[o], lo = olon[o];
  const int cx0 = cell_x(g, lo), cy0 = cell_y(g, la);
  double best = INFINITY, thr = INFINITY;  // thr: sums of squares above it cannot reach best
  int64_t bidx = INT64_MAX;
  const int rmax = g.cx > g.cy ? g.cx : g.cy;
  for (int r = 0; r <= rmax; ++r) {
    const int x_lo = cx0 - r, x_hi = cx0 + r, y_lo = cy0 - r, y_hi = cy0 + r;
    for (int cyy = y_lo; cyy <= y_hi; ++cyy) {
      if (cyy < 0 || cyy >= g.cy) continue;
      const bool edge_row = (cyy == y_lo || cyy == y_hi);
      for (int cxx = x_lo; cxx <= x_hi; cxx += (edge_row ? 1 : (x_hi - x_lo > 0 ? x_hi - x_lo : 1))) {
        if (cxx < 0 || cxx >= g.cx) continue;
        const int64_t c = (int64_t)cyy * g.cx + cxx;
        for (int64_t t = start[c]; t < start[c + 1]; ++t) {
          const double s2 = node_dist2(la, lo, slat[t], slon[t]);
          if (!(s2 <= thr)) continue;  // strictly farther (or NaN, which the scan never takes)
          const double d = __dsqrt_rn(s2);
          const int64_t id = sidx[t];
          if (d < best || (d == best && id < bidx)) {
            best = d;
            bidx = id;
            thr = __dadd_ru(__dmul_ru(s2, 1.0 + 0x1p-50), 0x1p-1000);
          }
        }
      }
    }
    // Distance from the observation to the outside of the visited block of
    // cells; sides that reach the end of the grid have nothing beyond them.
    double bound = INFINITY;
    if (x_lo > 0) bound = fmin(bound, lo - (g.x0 + (double)x_lo * g.w));
    if (x_hi < g.cx - 1) bound = fmin(bound, (g.x0 + (double)(x_hi + 1) * g.w) - lo);
    if (y_lo > 0) bound = fmin(bound, la - (g.y0 + (double)y_lo * g.h));
    if (y_hi < g.cy - 1) bound = fmin(bound, (g.y0 + (double)(y_hi + 1) * g.h) - la);
    // (a margin covers the rounding of the cell boundaries)
    if (bidx != INT64_MAX && best < bound * (1.0 - 1e-12)) break;
    if (x_lo <= 0 && y_lo <= 0 && x_hi >= g.cx - 1 && y_hi >= g.cy - 1) break;  // every cell visited
  }
  if (bidx == INT64_MAX) bidx = 0;  // no finite distance (NaN coordinates): the scan keeps node 0
  out_xy[2 * o] = (int32_t)(bidx % nx);
  out_xy[2 * o + 1] = (int32_t)(bidx / nx);
  if (out_k) {
    int kb = 0;
    double bd = INFINITY;
    for (int z = 0; z < nz; ++z) {
      const double d = fabs(olev[o] - vcoord[z]);
      if (d < bd) {
        bd = d;
        kb = z;
      }
    }
    out_k[o] = kb;
  }
}

}  // namespace

extern "C" int mg_nearest_node(mg_context* ctx, const double* node_lat, const double* node_lon, int32_t nx,
                               int32_t ny, const double* obs_lat, const double* obs_lon, int64_t p,
                               const double* vcoord, int32_t nz, const double* obs_level, int32_t* out_xy,
                               int32_t* out_k) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(node_lat && node_lon && nx > 0 && ny > 0 && p >= 0 && (p == 0 || (obs_lat && obs_lon && out_xy)),
               "mg_nearest_node: bad arguments");
  MG_CHECK_ARG(!out_k || (vcoord && nz > 0 && obs_level), "mg_nearest_node: vertical index needs vcoord and levels");
  if (p == 0) return MG_OK;
  const int64_t nn = (int64_t)nx * ny;
  cudaStream_t s = ctx->stream;
  // Bounding box of the nodes (device reduction, five values back).
  const int nbox = (int)std::min<int64_t>(kBoxBlocks, (nn + kThreads - 1) / kThreads);
  double box[5];
  {
    void* wsb = mg::workspace(ctx, sizeof(double) * (5 * (size_t)nbox + 8));
    if (!wsb) return MG_ERR_NOMEM;
    double* part = static_cast<double*>(wsb);
    double* dbox = part + 5 * (size_t)nbox;
    node_box_kernel<<<nbox, kThreads, 0, s>>>(node_lat, node_lon, nn, part);
    MG_COUNT_LAUNCH();
    node_box_final_kernel<<<1, 5 * 32, 0, s>>>(part, nbox, dbox);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
    MG_TRY_CUDA(cudaMemcpyAsync(box, dbox, sizeof(box), cudaMemcpyDeviceToHost, s));
    MG_TRY_CUDA(cudaStreamSynchronize(s));
  }
  if (box[4] != 0.0) return mg::fail(ctx, MG_ERR_ARG, "mg_nearest_node: node coordinates must be finite");
  const double xmin = box[0], xmax = box[1], ymin = box[2], ymax = box[3];
  NodeHash g;
  const double span_x = std::max(xmax - xmin, 1e-9), span_y = std::max(ymax - ymin, 1e-9);
  const double cells = std::max(1.0, (double)nn / 4.0);
  const double aspect = span_x / span_y;
  g.cx = (int)std::max(1.0, std::min(4096.0, std::floor(std::sqrt(cells * aspect))));
  g.cy = (int)std::max(1.0, std::min(4096.0, std::floor(cells / g.cx)));
  g.w = span_x / g.cx * (1.0 + 1e-12);
  g.h = span_y / g.cy * (1.0 + 1e-12);
  g.x0 = xmin;
  g.y0 = ymin;
  const int64_t ncell = (int64_t)g.cx * g.cy;
  const size_t tmpb = mg::scan_temp_bytes(ncell);
  mg::Carver cv;
  cv.reserve<unsigned long long>(ncell + 1);
  cv.reserve<unsigned long long>(ncell + 1);
  cv.reserve<int64_t>(ncell + 1);
  cv.reserve<int64_t>(nn);
  cv.reserve<double>(nn);
  cv.reserve<double>(nn);
  cv.reserve<char>(tmpb);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  auto* cnt = cv.take<unsigned long long>(ncell + 1);
  auto* cur = cv.take<unsigned long long>(ncell + 1);
  auto* start = cv.take<int64_t>(ncell + 1);
  auto* sidx = cv.take<int64_t>(nn);
  auto* slat = cv.take<double>(nn);
  auto* slon = cv.take<double>(nn);
  void* tmp = cv.take<char>(tmpb);
  MG_TRY_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (ncell + 1), s));
  MG_TRY_CUDA(cudaMemsetAsync(cur, 0, sizeof(unsigned long long) * (ncell + 1), s));
  const unsigned gb = (unsigned)std::min<int64_t>((nn + kThreads - 1) / kThreads, 152 * 16);
  node_count_kernel<<<gb, kThreads, 0, s>>>(node_lat, node_lon, nn, g, cnt);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(mg::exclusive_scan(reinterpret_cast<const int64_t*>(cnt), start, ncell, tmp, tmpb, s));
  node_scatter_kernel<<<gb, kThreads, 0, s>>>(node_lat, node_lon, nn, g, start, cur, sidx, slat, slon);
  MG_COUNT_LAUNCH();
  nearest_kernel<<<(unsigned)((p + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      obs_lat, obs_lon, p, g, start, sidx, slat, slon, nx, vcoord, nz, obs_level, out_xy, out_k);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}
