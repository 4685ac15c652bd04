// CPU oracle for the METADA ensemble Kalman analysis path.
//
// TEST INFRASTRUCTURE ONLY: restates the reference algorithms on the host so
// that tests, the smoke check and the CPU-baseline leg of the benchmark can
// check the GPU library.  The product never links or calls this file.
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -shared -fPIC.
// Citations are file:line in the open-x-da/metada tree.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Dense k x k helpers (row-major).  These restate the Eigen 3.4.0 operations
// the reference calls: MatrixXd::inverse() (PartialPivLU) and
// LLT<MatrixXd>::matrixL() (lower Cholesky factor).
// ---------------------------------------------------------------------------

// Inverse by LU with partial pivoting (row interchanges on the largest
// |pivot|, first one on ties), then forward/back substitution per unit
// column.  Returns false on an exactly singular pivot.
bool lu_inverse(const double* A, int k, double* Ainv) {
  std::vector<double> LU(A, A + (size_t)k * k);
  std::vector<int> perm(k);
  for (int i = 0; i < k; ++i) perm[i] = i;
  for (int c = 0; c < k; ++c) {
    int piv = c;
    double best = std::fabs(LU[(size_t)c * k + c]);
    for (int r = c + 1; r < k; ++r) {
      double v = std::fabs(LU[(size_t)r * k + c]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) return false;
    if (piv != c) {
      for (int j = 0; j < k; ++j) std::swap(LU[(size_t)c * k + j], LU[(size_t)piv * k + j]);
      std::swap(perm[c], perm[piv]);
    }
    const double d = LU[(size_t)c * k + c];
    for (int r = c + 1; r < k; ++r) {
      double l = LU[(size_t)r * k + c] / d;
      LU[(size_t)r * k + c] = l;
      for (int j = c + 1; j < k; ++j) LU[(size_t)r * k + j] -= l * LU[(size_t)c * k + j];
    }
  }
  std::vector<double> col(k);
  for (int e = 0; e < k; ++e) {
    // Solve L U x = P e_e.
    for (int i = 0; i < k; ++i) col[i] = (perm[i] == e) ? 1.0 : 0.0;
    for (int i = 0; i < k; ++i) {
      double s = col[i];
      for (int j = 0; j < i; ++j) s -= LU[(size_t)i * k + j] * col[j];
      col[i] = s;
    }
    for (int i = k - 1; i >= 0; --i) {
      double s = col[i];
      for (int j = i + 1; j < k; ++j) s -= LU[(size_t)i * k + j] * col[j];
      col[i] = s / LU[(size_t)i * k + i];
    }
    for (int i = 0; i < k; ++i) Ainv[(size_t)i * k + e] = col[i];
  }
  return true;
}

// Lower Cholesky factor from the lower triangle of A.  Returns false if A is
// not positive definite (LLT reports NumericalIssue; the reference ignores
// it, the oracle reports it).
bool cholesky_lower(const double* A, int k, double* L) {
  std::fill(L, L + (size_t)k * k, 0.0);
  for (int j = 0; j < k; ++j) {
    double s = A[(size_t)j * k + j];
    for (int m = 0; m < j; ++m) s -= L[(size_t)j * k + m] * L[(size_t)j * k + m];
    if (!(s > 0.0)) return false;
    const double ljj = std::sqrt(s);
    L[(size_t)j * k + j] = ljj;
    for (int i = j + 1; i < k; ++i) {
      double t = A[(size_t)i * k + j];
      for (int m = 0; m < j; ++m) t -= L[(size_t)i * k + m] * L[(size_t)j * k + m];
      L[(size_t)i * k + j] = t / ljj;
    }
  }
  return true;
}

// Cyclic Jacobi eigen-solver (Rutishauser's rotation formulas), FP64.
int jacobi_eig(double* A, int k, double* w, double* V) {
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) V[(size_t)i * k + j] = (i == j) ? 1.0 : 0.0;
  int sweep = 0;
  for (; sweep < 64; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < k; ++p) {
      diag += A[(size_t)p * k + p] * A[(size_t)p * k + p];
      for (int q = p + 1; q < k; ++q) off += A[(size_t)p * k + q] * A[(size_t)p * k + q];
    }
    if (off <= 1e-32 * diag) break;
    for (int p = 0; p < k - 1; ++p) {
      for (int q = p + 1; q < k; ++q) {
        const double apq = A[(size_t)p * k + q];
        if (apq == 0.0) continue;
        const double app = A[(size_t)p * k + p], aqq = A[(size_t)q * k + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int j = 0; j < k; ++j) {  // rows p, q
          const double a = A[(size_t)p * k + j], b = A[(size_t)q * k + j];
          A[(size_t)p * k + j] = c * a - s * b;
          A[(size_t)q * k + j] = s * a + c * b;
        }
        for (int i = 0; i < k; ++i) {  // columns p, q
          const double a = A[(size_t)i * k + p], b = A[(size_t)i * k + q];
          A[(size_t)i * k + p] = c * a - s * b;
          A[(size_t)i * k + q] = s * a + c * b;
        }
        for (int i = 0; i < k; ++i) {
          const double a = V[(size_t)i * k + p], b = V[(size_t)i * k + q];
          V[(size_t)i * k + p] = c * a - s * b;
          V[(size_t)i * k + q] = s * a + c * b;
        }
      }
    }
  }
  for (int i = 0; i < k; ++i) w[i] = A[(size_t)i * k + i];
  return sweep;
}

// IDW4 at an integer grid node, IdentityObsOperator.hpp:594-617 (2-D branch,
// nz == 1) and :643-676.
inline double idw4_at(const double* x, int nx, int ny, int ox, int oy) {
  double xx = std::max(0.0, std::min((double)(nx - 1), (double)ox));
  double yy = std::max(0.0, std::min((double)(ny - 1), (double)oy));
  const long i0 = (long)std::floor(xx), j0 = (long)std::floor(yy);
  const long i1 = std::min(i0 + 1, (long)nx - 1), j1 = std::min(j0 + 1, (long)ny - 1);
  const long ii[4] = {i0, i1, i0, i1}, jj[4] = {j0, j0, j1, j1};
  double ws = 0.0, wsum = 0.0;
  for (int t = 0; t < 4; ++t) {
    const double dx = xx - (double)ii[t], dy = yy - (double)jj[t];
    const double dist = std::sqrt(dx * dx + dy * dy);
    const double w = (dist == 0.0) ? 1e12 : 1.0 / dist;
    ws += w * x[jj[t] * nx + ii[t]];
    wsum += w;
  }
  return ws / wsum;
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_ens_mean(const double* X, int64_t n, int32_t k, int64_t ld, double* mean) {
  const double inv = 1.0 / static_cast<double>(k);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n; ++s) {
    double m = 0.0;
    for (int i = 0; i < k; ++i) m += X[(int64_t)i * ld + s];
    mean[s] = m * inv;
  }
}

void orc_ens_mean_pert(const double* X, int64_t n, int32_t k, int64_t ld, double* mean,
                       double* Xp, int64_t ldp) {
  orc_ens_mean(X, n, k, ld, mean);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n; ++s)
    for (int i = 0; i < k; ++i) Xp[(int64_t)i * ldp + s] = X[(int64_t)i * ld + s] - mean[s];
}

void orc_hx_idw4(const double* X, int32_t k, int64_t ld, int32_t nx, int32_t ny,
                 const int32_t* obs_xy, const uint8_t* valid, int64_t p, double* HX) {
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < p; ++o) {
    for (int i = 0; i < k; ++i) {
      HX[o * k + i] = (valid && !valid[o])
                          ? 0.0
                          : idw4_at(X + (int64_t)i * ld, nx, ny, obs_xy[2 * o], obs_xy[2 * o + 1]);
    }
  }
}

void orc_hx_latlon(const double* X, int32_t k, int64_t ld, int32_t nlon, int32_t nlat,
                   int32_t nlev, const double* obs_lat, const double* obs_lon,
                   const double* obs_lev, const int32_t* obs_var, int64_t p, double* HX) {
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < p; ++o) {
    // Horizontal: periodic in longitude, clamped in latitude.
    const double dlon = 360.0 / (double)nlon, dlat = 180.0 / (double)nlat;
    const double gx = obs_lon[o] / dlon - 0.5;
    const double fxl = std::floor(gx);
    const double fx = gx - fxl;
    long i0 = (long)fxl % nlon;
    if (i0 < 0) i0 += nlon;
    const long i1 = (i0 + 1) % nlon;
    double gy = (obs_lat[o] + 90.0) / dlat - 0.5;
    gy = std::max(0.0, std::min((double)(nlat - 1), gy));
    long j0 = (long)std::floor(gy);
    if (j0 > nlat - 2) j0 = nlat - 2;
    const double fy = gy - (double)j0;
    double gz = std::max(0.0, std::min((double)(nlev - 1), obs_lev[o]));
    long l0 = (long)std::floor(gz);
    if (l0 > nlev - 2) l0 = nlev - 2;
    if (l0 < 0) l0 = 0;
    const double fz = (nlev > 1) ? gz - (double)l0 : 0.0;
    const long l1 = (nlev > 1) ? l0 + 1 : l0;
    const int64_t plane = (int64_t)nlat * nlon;
    const int64_t vb = (int64_t)obs_var[o] * nlev * plane;
    const double ax = 1.0 - fx, ay = 1.0 - fy, az = 1.0 - fz;
    for (int m = 0; m < k; ++m) {
      const double* x = X + (int64_t)m * ld + vb;
      const double* lo = x + l0 * plane;
      const double* hi = x + l1 * plane;
      const double b0 = (lo[j0 * nlon + i0] * ax + lo[j0 * nlon + i1] * fx) * ay +
                        (lo[(j0 + 1) * nlon + i0] * ax + lo[(j0 + 1) * nlon + i1] * fx) * fy;
      const double b1 = (hi[j0 * nlon + i0] * ax + hi[j0 * nlon + i1] * fx) * ay +
                        (hi[(j0 + 1) * nlon + i0] * ax + hi[(j0 + 1) * nlon + i1] * fx) * fy;
      HX[o * k + m] = b0 * az + b1 * fz;
    }
  }
}

double orc_grid_distance(int32_t i1, int32_t j1, int32_t i2, int32_t j2) {
  const double dx = static_cast<double>(i1 - i2);
  const double dy = static_cast<double>(j1 - j2);
  return std::sqrt(dx * dx + dy * dy);
}

double orc_haversine_km(double lat1, double lon1, double lat2, double lon2) {
  const double pi = 3.14159265358979323846;
  auto deg2rad = [pi](double deg) { return deg * pi / 180.0; };
  const double dlat = deg2rad(lat2 - lat1);
  const double dlon = deg2rad(lon2 - lon1);
  const double a = std::sin(dlat / 2) * std::sin(dlat / 2) +
                   std::cos(deg2rad(lat1)) * std::cos(deg2rad(lat2)) * std::sin(dlon / 2) *
                       std::sin(dlon / 2);
  const double c = 2 * std::atan2(std::sqrt(a), std::sqrt(1 - a));
  return 6371.0 * c;
}

double orc_gaspari_cohn(double z) {
  z = std::fabs(z);
  if (z >= 2.0) return 0.0;
  if (z <= 1.0)
    return (((-0.25 * z + 0.5) * z + 0.625) * z - 5.0 / 3.0) * z * z + 1.0;
  return ((((z / 12.0 - 0.5) * z + 0.625) * z + 5.0 / 3.0) * z - 5.0) * z + 4.0 -
         2.0 / (3.0 * z);
}

int64_t orc_select_grid(int32_t nx, int32_t ny, const int32_t* obs_xy, int64_t p,
                        double radius, int64_t* offsets, int32_t* idx, int64_t cap) {
  const int64_t npt = (int64_t)nx * ny;
  std::vector<int64_t> cnt(npt, 0);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < npt; ++g) {
    const int gx = (int)(g % nx), gy = (int)(g / nx);
    int64_t c = 0;
    for (int64_t o = 0; o < p; ++o)
      if (orc_grid_distance(gx, gy, obs_xy[2 * o], obs_xy[2 * o + 1]) <= radius) ++c;
    cnt[g] = c;
  }
  offsets[0] = 0;
  for (int64_t g = 0; g < npt; ++g) offsets[g + 1] = offsets[g] + cnt[g];
  const int64_t total = offsets[npt];
  if (idx && total <= cap) {
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < npt; ++g) {
      const int gx = (int)(g % nx), gy = (int)(g / nx);
      int64_t w = offsets[g];
      for (int64_t o = 0; o < p; ++o)
        if (orc_grid_distance(gx, gy, obs_xy[2 * o], obs_xy[2 * o + 1]) <= radius)
          idx[w++] = (int32_t)o;
    }
  }
  return total;
}

int64_t orc_select_geo(const double* col_lat, const double* col_lon, int64_t ncol,
                       const double* obs_lat, const double* obs_lon, int64_t p,
                       double radius_km, int64_t* offsets, int32_t* idx, double* dist_km,
                       int64_t cap) {
  // Candidates are pruned by latitude only, with a margin far above any
  // rounding in the distance; the decision itself is the reference predicate.
  std::vector<int64_t> order(p);
  for (int64_t o = 0; o < p; ++o) order[o] = o;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return obs_lat[a] < obs_lat[b] || (obs_lat[a] == obs_lat[b] && a < b);
  });
  std::vector<double> slat(p);
  for (int64_t t = 0; t < p; ++t) slat[t] = obs_lat[order[t]];
  const double dlat_deg = radius_km / 6371.0 * 180.0 / 3.14159265358979323846 + 1e-6;
  std::vector<std::vector<int32_t>> lists(ncol);
  std::vector<std::vector<double>> dists(ncol);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t c = 0; c < ncol; ++c) {
    const double la = col_lat[c], lo = col_lon[c];
    const int64_t b = std::lower_bound(slat.begin(), slat.end(), la - dlat_deg) - slat.begin();
    const int64_t e = std::upper_bound(slat.begin(), slat.end(), la + dlat_deg) - slat.begin();
    std::vector<int32_t>& L = lists[c];
    std::vector<double>& D = dists[c];
    for (int64_t t = b; t < e; ++t) {
      const int64_t o = order[t];
      const double d = orc_haversine_km(la, lo, obs_lat[o], obs_lon[o]);
      if (d <= radius_km) { L.push_back((int32_t)o); D.push_back(d); }
    }
    // Obs order, as LETKF.hpp:160-165 builds it.
    std::vector<size_t> perm(L.size());
    for (size_t i = 0; i < perm.size(); ++i) perm[i] = i;
    std::sort(perm.begin(), perm.end(), [&](size_t a, size_t b2) { return L[a] < L[b2]; });
    std::vector<int32_t> L2(L.size());
    std::vector<double> D2(L.size());
    for (size_t i = 0; i < perm.size(); ++i) { L2[i] = L[perm[i]]; D2[i] = D[perm[i]]; }
    L.swap(L2);
    D.swap(D2);
  }
  offsets[0] = 0;
  for (int64_t c = 0; c < ncol; ++c) offsets[c + 1] = offsets[c] + (int64_t)lists[c].size();
  const int64_t total = offsets[ncol];
  if (idx && total <= cap) {
    for (int64_t c = 0; c < ncol; ++c) {
      std::copy(lists[c].begin(), lists[c].end(), idx + offsets[c]);
      if (dist_km) std::copy(dists[c].begin(), dists[c].end(), dist_km + offsets[c]);
    }
  }
  return total;
}

int orc_etkf_compat(double* X, int64_t n, int32_t k, int64_t ld, const double* HX,
                    const double* yo, const double* rvar, int64_t p, double rho,
                    double* mean_out) {
  // (1) mean and perturbations, Ensemble.hpp:105-151; X' *= rho, ETKF.hpp:125.
  std::vector<double> mean(n), Xp((size_t)n * k);
  orc_ens_mean(X, n, k, ld, mean.data());
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n; ++s)
    for (int i = 0; i < k; ++i) Xp[(size_t)i * n + s] = (X[(int64_t)i * ld + s] - mean[s]) * rho;
  // (2) obs-space mean (rowwise().mean() = sum / k), anomalies, innovation.
  std::vector<double> Yp((size_t)p * k), d(p), rinv(p);
  for (int64_t o = 0; o < p; ++o) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += HX[o * k + i];
    const double ym = s / (double)k;
    for (int i = 0; i < k; ++i) Yp[o * k + i] = HX[o * k + i] - ym;
    d[o] = yo[o] - ym;
    rinv[o] = 1.0 / rvar[o];  // diagonal R.inverse(), ETKF.hpp:147-150
  }
  // (3) A = Y'^T R^-1 Y' + (k-1) I; Pa = A^-1; wa = Pa Y'^T R^-1 d.
  std::vector<double> A((size_t)k * k, 0.0), Pa((size_t)k * k), b(k, 0.0), wa(k, 0.0);
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      for (int64_t o = 0; o < p; ++o) s += Yp[o * k + i] * rinv[o] * Yp[o * k + j];
      A[(size_t)i * k + j] = s + (i == j ? (double)(k - 1) : 0.0);
    }
  for (int i = 0; i < k; ++i) {
    double s = 0.0;
    for (int64_t o = 0; o < p; ++o) s += Yp[o * k + i] * rinv[o] * d[o];
    b[i] = s;
  }
  if (!lu_inverse(A.data(), k, Pa.data())) return -1;
  for (int i = 0; i < k; ++i) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += Pa[(size_t)i * k + j] * b[j];
    wa[i] = s;
  }
  // (4) W = sqrt(k-1) chol_L(Pa), ETKF.hpp:158-159.
  std::vector<double> L((size_t)k * k);
  if (!cholesky_lower(Pa.data(), k, L.data())) return -1;
  const double sq = std::sqrt((double)(k - 1));
  for (auto& v : L) v *= sq;
  // (5) Xa = (xm + X' wa) 1^T + X' W, ETKF.hpp:163-176.
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < n; ++s) {
    double xm = 0.0;
    for (int j = 0; j < k; ++j) xm += Xp[(size_t)j * n + s] * wa[j];
    xm += mean[s];
    for (int i = 0; i < k; ++i) {
      double t = 0.0;
      for (int j = 0; j < k; ++j) t += Xp[(size_t)j * n + s] * L[(size_t)j * k + i];
      X[(int64_t)i * ld + s] = xm + t;
    }
  }
  if (mean_out) std::memcpy(mean_out, mean.data(), sizeof(double) * n);
  return 0;
}

int orc_letkf_compat_grid(double* X, int32_t k, int64_t ld, int32_t nx, int32_t ny,
                          const int32_t* obs_xy, const uint8_t* valid, const double* yo,
                          int64_t p, double radius, double rho, double* mean_out) {
  std::vector<int32_t> local;
  std::vector<double> H, A((size_t)k * k), Pa((size_t)k * k), L((size_t)k * k), wa(k), xb(k),
      ym, dl;
  const double sqk = std::sqrt((double)(k - 1));
  int status = 0;
  for (int gy = 0; gy < ny; ++gy) {
    for (int gx = 0; gx < nx; ++gx) {
      const int64_t g = (int64_t)gy * nx + gx;
      local.clear();
      for (int64_t o = 0; o < p; ++o)
        if (orc_grid_distance(gx, gy, obs_xy[2 * o], obs_xy[2 * o + 1]) <= radius)
          local.push_back((int32_t)o);
      double xs = 0.0;
      for (int i = 0; i < k; ++i) { xb[i] = X[(int64_t)i * ld + g]; xs += xb[i]; }
      const double xm = xs / (double)k;
      if (local.empty()) {  // LETKF.hpp:167-190
        const double sr = std::sqrt(rho);
        for (int i = 0; i < k; ++i) X[(int64_t)i * ld + g] = xm + (xb[i] - xm) * sr;
        continue;
      }
      const int pl = (int)local.size();
      H.assign((size_t)pl * k, 0.0);
      ym.assign(pl, 0.0);
      dl.assign(pl, 0.0);
      for (int r = 0; r < pl; ++r) {  // LETKF.hpp:197-206, current members
        const int o = local[r];
        for (int j = 0; j < k; ++j)
          H[(size_t)r * k + j] = (valid && !valid[o]) ? 0.0
                                 : idw4_at(X + (int64_t)j * ld, nx, ny, obs_xy[2 * o],
                                           obs_xy[2 * o + 1]);
        double s = 0.0;
        for (int j = 0; j < k; ++j) s += H[(size_t)r * k + j];
        ym[r] = s / (double)k;
        for (int j = 0; j < k; ++j) H[(size_t)r * k + j] -= ym[r];
        dl[r] = yo[o] - ym[r];
      }
      for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
          double s = 0.0;
          for (int r = 0; r < pl; ++r) s += H[(size_t)r * k + i] * H[(size_t)r * k + j];
          A[(size_t)i * k + j] = s + (i == j ? (double)(k - 1) : 0.0);
        }
      if (!lu_inverse(A.data(), k, Pa.data())) { status = -1; continue; }
      for (auto& v : Pa) v *= rho;  // LETKF.hpp:219
      for (int i = 0; i < k; ++i) {  // wa = Pa Y'^T d, LETKF.hpp:221-222
        double s = 0.0;
        for (int j = 0; j < k; ++j) {
          double t = 0.0;
          for (int r = 0; r < pl; ++r) t += H[(size_t)r * k + j] * dl[r];
          s += Pa[(size_t)i * k + j] * t;
        }
        wa[i] = s;
      }
      if (!cholesky_lower(Pa.data(), k, L.data())) { status = -1; continue; }
      for (int i = 0; i < k; ++i) {  // LETKF.hpp:227-242
        const double xp = xb[i] - xm;
        double rs = 0.0;
        for (int j = 0; j < k; ++j) rs += xp * (sqk * L[(size_t)i * k + j]);
        X[(int64_t)i * ld + g] = (xm + xp * wa[i]) + rs;
      }
    }
  }
  if (mean_out) orc_ens_mean(X, (int64_t)nx * ny, k, ld, mean_out);  // LETKF.hpp:116
  return status;
}

int orc_letkf_points(const double* X, int32_t k, int64_t ld, const int64_t* pt_base,
                     int32_t n_var, int64_t var_stride, int64_t npt, const double* HX,
                     const double* yo, const double* rvar, int64_t p, const int64_t* loc_off,
                     const int32_t* loc_idx, const double* loc_w, double rho, int32_t flags,
                     double* out) {
  (void)p;
  // Obs-space mean, anomalies and innovation from the background (snapshot).
  std::vector<double> ym(p), Yp((size_t)p * k);
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < p; ++o) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += HX[o * k + i];
    ym[o] = s / (double)k;
    for (int i = 0; i < k; ++i) Yp[o * k + i] = HX[o * k + i] - ym[o];
  }
  const bool r_id = flags & ORC_R_IDENTITY, chol = flags & ORC_SQRT_CHOLESKY;
  const bool infl_c = flags & ORC_INFL_COMPAT, upd_c = flags & ORC_UPDATE_COMPAT;
  const bool rtps = flags & ORC_RTPS;
  int status = 0;
#pragma omp parallel
  {
    std::vector<double> A((size_t)k * k), Pa((size_t)k * k), W((size_t)k * k),
        V((size_t)k * k), ev(k), b(k), wa(k), xb(k), xa(k), T((size_t)k * k);
#pragma omp for schedule(dynamic, 8)
    for (int64_t t = 0; t < npt; ++t) {
      const int64_t o0 = loc_off[t], o1 = loc_off[t + 1];
      const int pl = (int)(o1 - o0);
      double* dst = out + (size_t)t * n_var * k;
      if (pl == 0) {  // LETKF.hpp:167-190 (multiplicative); RTPS leaves x' as is
        const double sr = rtps ? 1.0 : std::sqrt(rho);
        for (int v = 0; v < n_var; ++v) {
          const int64_t s = pt_base[t] + v * var_stride;
          double xs = 0.0;
          for (int i = 0; i < k; ++i) { xb[i] = X[(int64_t)i * ld + s]; xs += xb[i]; }
          const double xm = xs / (double)k;
          for (int i = 0; i < k; ++i) dst[v * k + i] = xm + (xb[i] - xm) * sr;
        }
        continue;
      }
      // A = diag term + Y'^T R^-1 Y', b = Y'^T R^-1 d.
      const double diag = (infl_c || rtps) ? (double)(k - 1) : (double)(k - 1) / rho;
      std::fill(A.begin(), A.end(), 0.0);
      std::fill(b.begin(), b.end(), 0.0);
      for (int64_t e = o0; e < o1; ++e) {
        const int o = loc_idx[e];
        const double ri = r_id ? 1.0 : (loc_w ? loc_w[e] : 1.0) / rvar[o];
        const double* y = &Yp[(size_t)o * k];
        const double dd = yo[o] - ym[o];
        for (int i = 0; i < k; ++i) {
          const double yi = y[i] * ri;
          b[i] += yi * dd;
          for (int j = 0; j < k; ++j) A[(size_t)i * k + j] += yi * y[j];
        }
      }
      for (int i = 0; i < k; ++i) A[(size_t)i * k + i] += diag;
      if (chol) {
        if (!lu_inverse(A.data(), k, Pa.data())) { status = -1; continue; }
        if (infl_c) for (auto& v : Pa) v *= rho;
        if (!cholesky_lower(Pa.data(), k, W.data())) { status = -1; continue; }
        const double sq = std::sqrt((double)(k - 1));
        for (auto& v : W) v *= sq;
      } else {
        std::copy(A.begin(), A.end(), Pa.begin());
        jacobi_eig(Pa.data(), k, ev.data(), V.data());
        // Pa = V diag(1/ev) V^T (times rho in compat inflation), W = sqrt((k-1) Pa).
        const double sc = infl_c ? rho : 1.0;
        for (int i = 0; i < k; ++i)
          for (int j = 0; j < k; ++j) {
            double s1 = 0.0, s2 = 0.0;
            for (int m = 0; m < k; ++m) {
              const double vv = V[(size_t)i * k + m] * V[(size_t)j * k + m];
              s1 += vv / ev[m];
              s2 += vv / std::sqrt(ev[m]);
            }
            Pa[(size_t)i * k + j] = sc * s1;
            W[(size_t)i * k + j] = std::sqrt((double)(k - 1) * sc) * s2;
          }
      }
      for (int i = 0; i < k; ++i) {
        double s = 0.0;
        for (int j = 0; j < k; ++j) s += Pa[(size_t)i * k + j] * b[j];
        wa[i] = s;
      }
      for (int v = 0; v < n_var; ++v) {
        const int64_t s = pt_base[t] + v * var_stride;
        double xs = 0.0;
        for (int i = 0; i < k; ++i) { xb[i] = X[(int64_t)i * ld + s]; xs += xb[i]; }
        const double xm = xs / (double)k;
        if (upd_c) {
          for (int i = 0; i < k; ++i) {
            const double xp = xb[i] - xm;
            double rs = 0.0;
            for (int j = 0; j < k; ++j) rs += xp * W[(size_t)i * k + j];
            dst[v * k + i] = (xm + xp * wa[i]) + rs;
          }
        } else {
          double inc = 0.0;
          for (int j = 0; j < k; ++j) inc += (xb[j] - xm) * wa[j];
          for (int i = 0; i < k; ++i) {
            double s2 = 0.0;
            for (int j = 0; j < k; ++j) s2 += (xb[j] - xm) * W[(size_t)j * k + i];
            xa[i] = s2;
          }
          if (rtps) {  // Whitaker & Hamill (2012) relaxation to prior spread
            double sb = 0.0, sa = 0.0;
            for (int i = 0; i < k; ++i) {
              sb += (xb[i] - xm) * (xb[i] - xm);
              sa += xa[i] * xa[i];
            }
            sb = std::sqrt(sb / (k - 1));
            sa = std::sqrt(sa / (k - 1));
            const double f = (sa > 0.0) ? rho * (sb - sa) / sa + 1.0 : 1.0;
            for (int i = 0; i < k; ++i) xa[i] *= f;
          }
          for (int i = 0; i < k; ++i) dst[v * k + i] = (xm + inc) + xa[i];
        }
      }
    }
  }
  return status;
}

// Stochastic EnKF, EnKF.hpp:139-254, in the reference's dense form:
// perturbations inflated by sqrt(rho) (applyInflation :322-335), Yb from the
// raw members, S = Y'Y'^T/(k-1) + R (p x p, :193-196), K = X'Y'^T S^-1/(k-1)
// (:199, S^-1 by LU with partial pivoting as MatrixXd::inverse()),
// xa_i = xm + X'_i + K (yo + eps_i - Yb_i) (:215-224) with the obs
// perturbations eps given (the reference draws them from an unseeded
// generator, :336-352), then the mean recomputed (:237).  diag3 = {||d||,
// background spread, analysis spread} (:184, :334, :240-253); gain2 = {max,
// min} of K (:201-202), may be NULL.
int orc_enkf(double* X, int64_t n, int32_t k, int64_t ld, const double* HX, const double* yo,
             const double* rvar, const double* eps, int64_t p, double rho, double* mean_out, double* diag3,
             double* gain2) {
  std::vector<double> mean(n), Xp((size_t)n * k);
  orc_ens_mean(X, n, k, ld, mean.data());
  const double sr = std::sqrt(rho);
  double bss = 0.0;
  for (int64_t s = 0; s < n; ++s)
    for (int i = 0; i < k; ++i) {
      const double v = (X[(int64_t)i * ld + s] - mean[s]) * sr;
      Xp[(size_t)i * n + s] = v;
      bss += v * v;
    }
  std::vector<double> Yp((size_t)p * k), d(p);
  double dn = 0.0;
  for (int64_t o = 0; o < p; ++o) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += HX[o * k + i];
    const double ym = s / (double)k;
    for (int i = 0; i < k; ++i) Yp[o * k + i] = HX[o * k + i] - ym;
    d[o] = yo[o] - ym;
    dn += d[o] * d[o];
  }
  std::vector<double> S((size_t)p * p), Si((size_t)p * p);
  for (int64_t a = 0; a < p; ++a)
    for (int64_t b = 0; b < p; ++b) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s += Yp[a * k + i] * Yp[b * k + i];
      S[(size_t)a * p + b] = s / (double)(k - 1) + (a == b ? rvar[a] : 0.0);
    }
  if (!lu_inverse(S.data(), (int)p, Si.data())) return -1;
  // M = Y'^T S^-1 (k x p); K = X' M / (k - 1) (n x p).
  std::vector<double> M((size_t)k * p, 0.0);
  for (int i = 0; i < k; ++i)
    for (int64_t b = 0; b < p; ++b) {
      double s = 0.0;
      for (int64_t a = 0; a < p; ++a) s += Yp[a * k + i] * Si[(size_t)a * p + b];
      M[(size_t)i * p + b] = s;
    }
  double kmax = -1e300, kmin = 1e300;
  std::vector<double> Krow(p), Xa((size_t)n * k);
  for (int64_t s = 0; s < n; ++s) {
    for (int64_t b = 0; b < p; ++b) {
      double v = 0.0;
      for (int i = 0; i < k; ++i) v += Xp[(size_t)i * n + s] * M[(size_t)i * p + b];
      v /= (double)(k - 1);
      Krow[b] = v;
      kmax = std::max(kmax, v);
      kmin = std::min(kmin, v);
    }
    for (int i = 0; i < k; ++i) {
      double inc = 0.0;
      for (int64_t b = 0; b < p; ++b) inc += Krow[b] * ((yo[b] + eps[b * k + i]) - HX[b * k + i]);
      Xa[(size_t)i * n + s] = mean[s] + (Xp[(size_t)i * n + s] + inc);
    }
  }
  for (int i = 0; i < k; ++i)
    for (int64_t s = 0; s < n; ++s) X[(int64_t)i * ld + s] = Xa[(size_t)i * n + s];
  std::vector<double> am(n);
  orc_ens_mean(X, n, k, ld, am.data());
  double ass = 0.0;
  for (int i = 0; i < k; ++i)
    for (int64_t s = 0; s < n; ++s) {
      const double v = X[(int64_t)i * ld + s] - am[s];
      ass += v * v;
    }
  if (mean_out) std::memcpy(mean_out, am.data(), sizeof(double) * n);
  if (diag3) {
    diag3[0] = std::sqrt(dn);
    diag3[1] = std::sqrt(bss / ((double)n * k));
    diag3[2] = std::sqrt(ass / ((double)k * n));
  }
  if (gain2) {
    gain2[0] = kmax;
    gain2[1] = kmin;
  }
  return 0;
}

// IdentityObsOperator::convertGeographicToGrid with 2-D coordinates
// (IdentityObsOperator.hpp:470-505): scan every node in index order, keep
// the first strict minimum of the Euclidean degree distance; vertical index
// likewise over vcoord.
void orc_nearest_node(const double* node_lat, const double* node_lon, int32_t nx, int32_t ny,
                      const double* obs_lat, const double* obs_lon, int64_t p, const double* vcoord, int32_t nz,
                      const double* obs_level, int32_t* out_xy, int32_t* out_k) {
  const int64_t nn = (int64_t)nx * ny;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t o = 0; o < p; ++o) {
    double min_dist = std::numeric_limits<double>::max();
    int64_t min_idx = 0;
    for (int64_t idx = 0; idx < nn; ++idx) {
      const double dist = std::sqrt((obs_lon[o] - node_lon[idx]) * (obs_lon[o] - node_lon[idx]) +
                                    (obs_lat[o] - node_lat[idx]) * (obs_lat[o] - node_lat[idx]));
      if (dist < min_dist) {
        min_dist = dist;
        min_idx = idx;
      }
    }
    out_xy[2 * o] = (int32_t)(min_idx % nx);
    out_xy[2 * o + 1] = (int32_t)(min_idx / nx);
    if (out_k) {
      double md = std::numeric_limits<double>::max();
      int kb = 0;
      for (int z = 0; z < nz; ++z) {
        const double d = std::abs(obs_level[o] - vcoord[z]);
        if (d < md) {
          md = d;
          kb = z;
        }
      }
      out_k[o] = kb;
    }
  }
}

int orc_sym_eig(double* A, int32_t k, double* w, double* V) { return jacobi_eig(A, k, w, V); }

// Metrics<double>::CalculateAll (Metrics.hpp:74-94) and the functions it
// calls, in their order: mean by member-order sums then a division by k
// (:108-121), spread sqrt(sum (x - mean)^2 / (k - 1)) (:137-150), RMSE
// (:265-273), bias (:166-173), correlation by the single-pass sums formula
// (:189-206), CRPS with the O(k^2) pair sum per element (:232-252), average
// spread (:286-293).  Sequential sums over the state, as the reference.
void orc_ens_metrics(const double* X, int64_t n, int32_t k, int64_t ld, const double* truth, double* mean,
                     double* spread, double* out5) {
  for (int64_t i = 0; i < n; ++i) mean[i] = 0.0;
  for (int j = 0; j < k; ++j)
    for (int64_t i = 0; i < n; ++i) mean[i] += X[(int64_t)j * ld + i];
  for (int64_t i = 0; i < n; ++i) mean[i] /= (double)k;
  for (int64_t i = 0; i < n; ++i) spread[i] = 0.0;
  for (int j = 0; j < k; ++j)
    for (int64_t i = 0; i < n; ++i) {
      const double d = X[(int64_t)j * ld + i] - mean[i];
      spread[i] += d * d;
    }
  for (int64_t i = 0; i < n; ++i) spread[i] = std::sqrt(spread[i] / (double)(k - 1));
  double rmse = 0.0, bias = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double d = mean[i] - truth[i];
    rmse += d * d;
  }
  rmse = std::sqrt(rmse / (double)n);
  for (int64_t i = 0; i < n; ++i) bias += mean[i] - truth[i];
  bias /= (double)n;
  double sx = 0.0, sy = 0.0, sxy = 0.0, sx2 = 0.0, sy2 = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    sx += mean[i];
    sy += truth[i];
    sxy += mean[i] * truth[i];
    sx2 += mean[i] * mean[i];
    sy2 += truth[i] * truth[i];
  }
  const double nn = (double)n;
  const double corr = (nn * sxy - sx * sy) / std::sqrt((nn * sx2 - sx * sx) * (nn * sy2 - sy * sy));
  double crps = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double sd = 0.0, st = 0.0;
    for (int j = 0; j < k; ++j)
      for (int l = 0; l < k; ++l) sd += std::fabs(X[(int64_t)j * ld + i] - X[(int64_t)l * ld + i]);
    for (int j = 0; j < k; ++j) st += std::fabs(X[(int64_t)j * ld + i] - truth[i]);
    crps += st / (double)k - sd / (2.0 * k * k);
  }
  crps /= (double)n;
  double avg = 0.0;
  for (int64_t i = 0; i < n; ++i) avg += spread[i];
  avg /= (double)n;
  out5[0] = rmse;
  out5[1] = bias;
  out5[2] = corr;
  out5[3] = crps;
  out5[4] = avg;
}

void orc_column_op(const float* T, const float* q, int64_t ncol, int32_t nlev, const float* w,
                   const float* tau, int32_t nch, float* y) {
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ncol; ++c) {
    for (int ch = 0; ch < nch; ++ch) {
      double cq = 0.0, acc = 0.0;
      for (int l = 0; l < nlev; ++l) {
        cq += (double)q[c * nlev + l];
        const double t = (double)T[c * nlev + l];
        acc += (double)w[ch * nlev + l] * std::exp(-(double)tau[ch] * cq) * (t * t) * (t * t) / 1e8;
      }
      y[c * nch + ch] = (float)acc;
    }
  }
}

// SimpleState.hpp:255-261: getline, then `iss >> value` until it fails.
int64_t orc_parse_values(const char* text, int64_t nbytes, double* out, int64_t cap) {
  std::istringstream file(std::string(text, (size_t)nbytes));
  std::string line;
  int64_t n = 0;
  while (std::getline(file, line)) {
    std::istringstream iss(line);
    double value;
    while (iss >> value) {
      if (n < cap) out[n] = value;
      ++n;
    }
  }
  return n;
}

}  // extern "C"
