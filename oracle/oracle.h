/*
 * CPU oracle for the ensemble Kalman analysis path of METADA.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C++ on the host,
 * the reference algorithms that the GPU library replaces, so that tests, the
 * smoke check and the CPU-baseline leg of the benchmark have something to
 * compare against.  Nothing in the product (the CUDA library, its C-ABI, the
 * C++ host layer, the Python mirror) links or calls this code.
 *
 * Every function names the reference file:line it follows (paths are relative
 * to the open-x-da/metada source tree).  The dense linear algebra the
 * reference delegates to Eigen 3.4.0 (a third-party dependency that is not
 * vendored in the reference tree) is restated from its published algorithms:
 * LU with partial pivoting for MatrixXd::inverse(), and the
 * Cholesky-Banachiewicz factorisation for LLT::matrixL().
 *
 * Parity of this oracle is pinned against the reference's own headers
 * (ETKF.hpp, LETKF.hpp, Ensemble.hpp, IdentityObsOperator.hpp, Location.hpp,
 * SimpleState.hpp, GridObservation.hpp) compiled here against an
 * Eigen-subset restatement (oracle/eigen_subset), on the tutorial data and
 * on seeded inputs; the resulting golden vectors live in tests/golden.
 *
 * Arithmetic: compiled with -ffp-contract=off so that every multiply and add
 * rounds separately, as in the reference built for x86-64 without -mfma.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flag bits for orc_letkf_points: the reference (compat) semantics versus the
 * Hunt et al. (2007) formulation used for the large batched configurations. */
enum {
  ORC_R_IDENTITY = 1,    /* R_local = I, LETKF.hpp:214 */
  ORC_SQRT_CHOLESKY = 2, /* W = sqrt(k-1) chol_L(Pa), LETKF.hpp:223-224 */
  ORC_INFL_COMPAT = 4,   /* Pa *= rho, LETKF.hpp:219 */
  ORC_UPDATE_COMPAT = 8, /* xa_i = xm + x'_i wa_i + x'_i sum_j W_ij, LETKF.hpp:232-238 */
  ORC_COMPAT = 15,
  ORC_RTPS = 16          /* relaxation to prior spread (uses rho as alpha) */
};

/* Ensemble::RecomputeMean, Ensemble.hpp:105-114: member-order sum, then a
 * multiply by the reciprocal 1.0/k.  Member i starts at X + i*ld. */
void orc_ens_mean(const double* X, int64_t n, int32_t k, int64_t ld,
                  double* mean);

/* Ensemble::RecomputePerturbations, Ensemble.hpp:142-151. */
void orc_ens_mean_pert(const double* X, int64_t n, int32_t k, int64_t ld,
                       double* mean, double* Xp, int64_t ldp);

/* IdentityObsOperator::apply (IdentityObsOperator.hpp:154-180) for grid
 * observations on a 2-D SimpleState (row-major y*nx+x, SimpleState.hpp:73-80):
 * find4NearestGridPoints (:594-617) + idw4Interpolation (:643-676).
 * obs_xy holds (x, y) integer grid coordinates per observation; valid may be
 * NULL (all valid).  HX is p x k, row-major: HX[o*k + i] = H(member i)_o. */
void orc_hx_idw4(const double* X, int32_t k, int64_t ld, int32_t nx,
                 int32_t ny, const int32_t* obs_xy, const uint8_t* valid,
                 int64_t p, double* HX);

/* Bilinear-horizontal / linear-vertical interpolation on a regular lat-lon
 * grid with cell-centred nodes (lon_i = (i+0.5) 360/nlon deg,
 * lat_j = -90 + (j+0.5) 180/nlat deg) and
 * integer level coordinates.  State layout ((v*nlev + l)*nlat + j)*nlon + i.
 * This operator has no counterpart in the reference (it is the one the
 * lat-lon configurations name); it is fixed here so GPU and oracle agree
 * bit for bit. */
void orc_hx_latlon(const double* X, int32_t k, int64_t ld, int32_t nlon,
                   int32_t nlat, int32_t nlev, const double* obs_lat,
                   const double* obs_lon, const double* obs_lev,
                   const int32_t* obs_var, int64_t p, double* HX);

/* Location::distance_to for GRID locations, Location.hpp:205-211. */
double orc_grid_distance(int32_t i1, int32_t j1, int32_t i2, int32_t j2);

/* Location::haversine, Location.hpp:349-357 (km, R = 6371). */
double orc_haversine_km(double lat1, double lon1, double lat2, double lon2);

/* Gaspari & Cohn (1999) eq. 4.10 compactly supported 5th-order piecewise
 * rational function, argument z = distance / c (zero for z >= 2). */
double orc_gaspari_cohn(double z);

/* LETKF local search on a 2-D grid, LETKF.hpp:159-165 with the GRID branch
 * of distance_to: for grid point g (row-major, SimpleGeometry.hpp:49-54) the
 * local list is every obs o, in obs order, with distance <= radius.  Returns
 * the total entry count; writes offsets[nx*ny+1] and idx[] (up to cap). */
int64_t orc_select_grid(int32_t nx, int32_t ny, const int32_t* obs_xy,
                        int64_t p, double radius, int64_t* offsets,
                        int32_t* idx, int64_t cap);

/* The same search with the GEOGRAPHIC branch (haversine, Location.hpp:212-216)
 * for a list of query columns.  dist_km receives each entry's distance. */
int64_t orc_select_geo(const double* col_lat, const double* col_lon,
                       int64_t ncol, const double* obs_lat,
                       const double* obs_lon, int64_t p, double radius_km,
                       int64_t* offsets, int32_t* idx, double* dist_km,
                       int64_t cap);

/* Global ETKF, ETKF.hpp:100-179, in place on the members.  HX is the p x k
 * row-major obs-space ensemble of the RAW background members
 * (ETKF.hpp:128-132); rvar the obs error variances (ETKF.hpp:144-147; +inf
 * for invalid obs).  mean_out (optional) receives the background mean that
 * the reference leaves in Ensemble::Mean() and saves (ETKF.hpp:190-191).
 * Returns 0, or -1 if the k x k matrix is not positive definite. */
int orc_etkf_compat(double* X, int64_t n, int32_t k, int64_t ld,
                    const double* HX, const double* yo, const double* rvar,
                    int64_t p, double rho, double* mean_out);

/* LETKF exactly as LETKF.hpp:63-119,152-243 on a 2-D grid: grid points in
 * row-major order, local obs by grid distance, H by IDW4 from the CURRENT
 * (partly analysed) members, R_local = I, Pa *= rho, Cholesky square root,
 * the reference's per-member scalar update, written in place; then the
 * mean recomputed (LETKF.hpp:116) into mean_out (optional). */
int orc_letkf_compat_grid(double* X, int32_t k, int64_t ld, int32_t nx,
                          int32_t ny, const int32_t* obs_xy,
                          const uint8_t* valid, const double* yo, int64_t p,
                          double radius, double rho, double* mean_out);

/* One local analysis per point with the obs-space prior taken from the
 * background (snapshot), for a subset of npt analysis points.  Point t
 * updates state entries pt_base[t] + v*var_stride, v < n_var, of every
 * member; its local obs are loc_idx[loc_off[t] .. loc_off[t+1]) with
 * localisation weights loc_w (NULL = 1).  HX is p x k row-major (raw).
 * out receives npt x n_var x k analysis values.  flags: ORC_* above. */
int orc_letkf_points(const double* X, int32_t k, int64_t ld,
                     const int64_t* pt_base, int32_t n_var,
                     int64_t var_stride, int64_t npt, const double* HX,
                     const double* yo, const double* rvar, int64_t p,
                     const int64_t* loc_off, const int32_t* loc_idx,
                     const double* loc_w, double rho, int32_t flags,
                     double* out);

/* Stochastic EnKF, EnKF.hpp:139-254, dense p x p form, in place on the
 * members; eps (p x k row-major) are the obs perturbations the reference
 * would draw.  mean_out: analysis mean; diag3 = {||yo - ym||, background
 * spread, analysis spread}; gain2 = {max, min} of the gain (may be NULL).
 * Returns 0, or -1 if S is singular. */
int orc_enkf(double* X, int64_t n, int32_t k, int64_t ld, const double* HX, const double* yo,
             const double* rvar, const double* eps, int64_t p, double rho, double* mean_out, double* diag3,
             double* gain2);

/* Nearest node of geographic obs on a curvilinear grid by the reference's
 * scan (IdentityObsOperator.hpp:470-505); out_k may be NULL. */
void orc_nearest_node(const double* node_lat, const double* node_lon, int32_t nx, int32_t ny,
                      const double* obs_lat, const double* obs_lon, int64_t p, const double* vcoord, int32_t nz,
                      const double* obs_level, int32_t* out_xy, int32_t* out_k);

/* SimpleState::readFromFile (SimpleState.hpp:248-263): every double that
 * std::istringstream extracts from each line, in order.  Writes at most cap
 * values and returns the count found. */
int64_t orc_parse_values(const char* text, int64_t nbytes, double* out, int64_t cap);

/* Symmetric eigen-decomposition by cyclic Jacobi (FP64), A = V diag(w) V^T.
 * A (k x k, row-major) is overwritten.  Returns the number of sweeps. */
int orc_sym_eig(double* A, int32_t k, double* w, double* V);

/* Column observation operator of the learned-operator configuration:
 * y_c = sum_l w[c,l] exp(-tau[c] sum_{m<=l} q_m) T_l^4 / 1e8 for nlev levels
 * and nch channels; T and q are ncol x nlev row-major, y ncol x nch. */
void orc_column_op(const float* T, const float* q, int64_t ncol, int32_t nlev,
                   const float* w, const float* tau, int32_t nch, float* y);

/* Ensemble diagnostics, Metrics<double>::CalculateAll (Metrics.hpp:74-94):
 * mean and spread per state element (n each), and out5 = {RMSE, bias,
 * correlation, CRPS, average spread}.  Members start at X + j*ld. */
void orc_ens_metrics(const double* X, int64_t n, int32_t k, int64_t ld, const double* truth, double* mean,
                     double* spread, double* out5);

/* Number of OpenMP threads the oracle uses. */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
