/*
 * metada_gb300 — GB300-native (sm_103a) ensemble Kalman analysis for METADA.
 *
 * C-ABI of the CUDA library libmetada_gb300.so.  This is the boundary the
 * C++ host layer (include/metada_gb300/*.hpp, mirroring METADA's backend
 * traits and algorithm policies) and any other FFI caller bind.  Each entry
 * point names the reference member function (open-x-da/metada tree,
 * file:line) whose work it replaces.
 *
 * Conventions
 *  - Every function returns an int status: MG_OK (0) or an MG_ERR_* code;
 *    no C++ exception and no CUDA error crosses this boundary.  The message
 *    for the last failure on a context is mg_last_error(ctx).
 *  - Array arguments are DEVICE pointers owned by the caller unless a
 *    comment says "host".  Work is enqueued on the context's stream
 *    (mg_set_stream); entry points that return a host-visible count
 *    synchronise that stream.
 *  - Ensembles are member-major as in the reference (k separate state
 *    vectors, SimpleState.hpp:265): member i starts at X + i*ld.
 *  - Obs-space ensembles are p x k row-major: HX[o*k + i] = H(member i)_o.
 *  - A context is not re-entrant; use one per host thread.
 */
#ifndef METADA_GB300_H
#define METADA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define MG_OK 0
#define MG_ERR_ARG 1      /* invalid argument (sizes, null pointers, flags) */
#define MG_ERR_CUDA 2     /* a CUDA runtime call failed */
#define MG_ERR_NOMEM 3    /* device workspace could not be allocated */
#define MG_ERR_NUMERIC 4  /* k x k matrix not positive definite / not finite */
#define MG_ERR_TIMEOUT 5  /* a bounded device-side wait gave up */
#define MG_ERR_CAPACITY 6 /* caller's output buffer too small; *total says how large */

/* Analysis semantics (bit flags).  MG_COMPAT reproduces the reference:
 * LETKF.hpp:214 (R_local = I), :219 (Pa *= rho), :223-224 (Cholesky square
 * root), :232-238 (per-member scalar update).  Without them the Hunt et al.
 * (2007) LETKF is used: R^-1 = w/sigma^2 with Gaspari-Cohn weights w,
 * Pa = [(k-1)/rho I + Y'^T R^-1 Y']^-1, symmetric square root from a Jacobi
 * eigen-decomposition, Xa = xm + X'(wa 1^T + W). */
#define MG_R_IDENTITY 1
#define MG_SQRT_CHOLESKY 2
#define MG_INFL_COMPAT 4
#define MG_UPDATE_COMPAT 8
#define MG_COMPAT 15
#define MG_RTPS 16 /* relaxation to prior spread with alpha = rho (no multiplicative inflation) */
#define MG_WARM_START 32 /* batched LETKF: the levels of a column run in sequence, each
                            eigen-solve warm-started from the previous level's eigenvectors
                            (default: every eigen-solve starts from the identity) */
#define MG_SOLVE_SIMT 64 /* batched LETKF, mixed precision: the SIMT Jacobi solve instead of
                            the tensor-core Newton-Schulz route (which serves k <= 96 with the
                            Hunt transform and update) */

/* Arithmetic of the analysis. */
#define MG_PREC_FP64 0  /* every step in IEEE double */
#define MG_PREC_MIXED 1 /* FP64 means/innovations; FP32 anomalies, Gram, eigen-solve, update */

typedef struct mg_context mg_context;

/* Context: device, stream, device workspace, last error.
 * Replaces nothing in the reference (its analysis is host code); it owns the
 * GPU resources the algorithm policies need. */
int mg_create(mg_context** ctx, int device);
void mg_destroy(mg_context* ctx);
int mg_set_stream(mg_context* ctx, void* cuda_stream);
int mg_synchronize(mg_context* ctx);
const char* mg_last_error(const mg_context* ctx);
/* Library version string (static). */
const char* mg_version(void);

/* Ensemble::RecomputeMean, src/framework/adapters/Ensemble.hpp:105-114:
 * mean = (sum over members in member order) * (1.0/k).  Bit-exact. */
int mg_ens_mean(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld,
                double* mean);

/* Ensemble::RecomputePerturbations, Ensemble.hpp:142-151: mean as above and
 * Xp_i = X_i - mean (member-major, member i at Xp + i*ldp).  Bit-exact. */
int mg_ens_mean_pert(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld,
                     double* mean, double* Xp, int64_t ldp);

/* IdentityObsOperator::apply, src/backends/common/obsoperator/
 * IdentityObsOperator.hpp:154-180 with find4NearestGridPoints (:594-617)
 * and idw4Interpolation (:643-676), for grid observations on the 2-D
 * SimpleState (row-major y*nx + x).  obs_xy: p (x, y) int32 pairs; valid:
 * p bytes or NULL (invalid obs give 0, :165-167).  Bit-exact. */
int mg_hx_idw4(mg_context* ctx, const double* X, int32_t k, int64_t ld, int32_t nx,
               int32_t ny, const int32_t* obs_xy, const uint8_t* valid, int64_t p,
               double* HX);

/* Bilinear-horizontal / linear-vertical H on a cell-centred lat-lon grid
 * (lon_i = (i+0.5) 360/nlon deg, lat_j = -90 + (j+0.5) 180/nlat deg, integer
 * levels), state layout
 * ((v*nlev + l)*nlat + j)*nlon + i.  No reference counterpart (the reference
 * has only IDW4); used for the lat-lon configurations.  Bit-exact with the
 * oracle's fixed operation order. */
int mg_hx_latlon(mg_context* ctx, const double* X, int32_t k, int64_t ld, int32_t nlon,
                 int32_t nlat, int32_t nlev, const double* obs_lat, const double* obs_lon,
                 const double* obs_lev, const int32_t* obs_var, int64_t p, double* HX);
/* The same operator on members stored as FP32 (widened to FP64 on load;
 * the high-resolution configuration keeps its 80 members in FP32). */
int mg_hx_latlon_f32(mg_context* ctx, const float* X, int32_t k, int64_t ld, int32_t nlon,
                     int32_t nlat, int32_t nlev, const double* obs_lat, const double* obs_lon,
                     const double* obs_lev, const int32_t* obs_var, int64_t p, double* HX);

/* LETKF::updateGridPoint local search, src/framework/algorithms/
 * LETKF.hpp:159-165 with Location::distance_to GRID branch
 * (src/framework/base/Location.hpp:205-211): for each grid point of an
 * nx*ny SimpleGeometry (row-major), the obs with distance <= radius, in obs
 * order.  Writes offsets[nx*ny+1] (device) and idx[] (device, capacity cap);
 * *total (host) receives the entry count.  Bit-exact. */
int mg_select_grid(mg_context* ctx, int32_t nx, int32_t ny, const int32_t* obs_xy,
                   int64_t p, double radius, int64_t* offsets, int32_t* idx, int64_t cap,
                   int64_t* total);

/* The same search with the GEOGRAPHIC branch (haversine km,
 * Location.hpp:212-216, :349-357) over a device-built lat-lon spatial hash,
 * for ncol query columns.  Lists are in obs order; dist_km (device, may be
 * NULL) receives each entry's distance.  Pairs whose GPU distance lies within
 * 1e-9 relative of the radius are re-decided on the host with the reference
 * expression, so counts and lists are bit-exact. */
int mg_select_geo(mg_context* ctx, const double* col_lat, const double* col_lon,
                  int64_t ncol, const double* obs_lat, const double* obs_lon, int64_t p,
                  double radius_km, int64_t* offsets, int32_t* idx, double* dist_km,
                  int64_t cap, int64_t* total);

/* ETKF::Analyse, src/framework/algorithms/ETKF.hpp:100-179, in place on the
 * members X.  HX: obs-space ensemble of the raw background members
 * (ETKF.hpp:128-132); yo, rvar: obs values and error variances (+inf for
 * invalid obs).  flags: MG_COMPAT (X' *= rho, Cholesky W, ETKF.hpp:125,158)
 * or 0 (Hunt: symmetric W, (k-1)/rho prior).  mean_out (device, may be
 * NULL) receives the background mean the reference leaves in
 * Ensemble::Mean().  precision: MG_PREC_*. */
int mg_etkf(mg_context* ctx, double* X, int64_t n, int32_t k, int64_t ld, const double* HX,
            const double* yo, const double* rvar, int64_t p, double rho, int32_t flags,
            int32_t precision, double* mean_out);

/* LETKF::Analyse exactly as the reference runs it, LETKF.hpp:63-119 and
 * :152-243, on a 2-D SimpleState grid: grid points in row-major order, each
 * analysed with the obs-space prior of the CURRENT, partly analysed members
 * (IDW4 H), R_local = I, Pa *= rho, Cholesky W, the per-member scalar update,
 * written in place; then Ensemble::RecomputeMean into mean_out (may be
 * NULL).  Sequential by construction; for parity on small grids. */
int mg_letkf_compat_grid(mg_context* ctx, double* X, int32_t k, int64_t ld, int32_t nx,
                         int32_t ny, const int32_t* obs_xy, const uint8_t* valid,
                         const double* yo, int64_t p, double radius, double rho,
                         double* mean_out);

/* Allocation-free variant of mg_etkf, for callers that cannot allocate device
 * memory when they run the analysis: real-time assimilation loops whose
 * device memory is fixed at start-up (an allocation in the cycle could fail
 * or stall it), and host frameworks that own every device allocation through
 * their own pool (a cudaMalloc behind their back breaks their accounting, or
 * fails because the pool already holds the memory).  No counterpart in the
 * reference (its analysis is host code).
 *  - Same arguments and results as mg_etkf, but no context: work goes on
 *    `cuda_stream` (a cudaStream_t, NULL = default stream) of the current
 *    device.  The call copies its status word to the host and waits for the
 *    stream before it returns the status code.
 *  - Scratch comes from one fixed 32 MiB array that the library reserves on
 *    every GPU it is loaded on, until the process exits; the call performs no
 *    cudaMalloc, cudaFree or other allocating call.  A problem needs about
 *    8*n + s*n*k + 8*(p+1)*(k+2) + 8*B*k*(k+1) + 8*k*k bytes (s = 8 for FP64,
 *    4 for mixed; B = min(ceil(p/256), 2 x SM count)); larger problems return
 *    MG_ERR_CAPACITY before any GPU work.
 *  - The first call on a device looks up the array's device address (once
 *    per device, with that device current); make that first call before any
 *    stream capture begins.
 *  - Every call shares the one array, which keeps the last call's contents:
 *    calls that overlap on the GPU (other streams, other host threads) race
 *    and must be serialised by the caller.
 *  - k <= 112. */
int mg_etkf_noalloc(void* cuda_stream, double* X, int64_t n, int32_t k, int64_t ld,
                    const double* HX, const double* yo, const double* rvar, int64_t p,
                    double rho, int32_t flags, int32_t precision, double* mean_out);

/* Batched LETKF over columns x levels with the obs-space prior of the
 * background (all local analyses independent). */
/* Storage type of the members in mg_letkf_desc.X. */
#define MG_DTYPE_F64 0
#define MG_DTYPE_F32 1 /* mixed precision only: FP64 means from the widened values, the analysis
                          rounded to FP32 on write-back */

typedef struct mg_letkf_desc {
  void* X;               /* members, member-major (x_dtype), updated in place */
  int64_t n;             /* state values per member */
  int64_t ld;            /* member stride (>= n) */
  int32_t k;             /* members, 2..128 */
  int32_t n_var;         /* variables sharing one analysis point */
  int32_t nlev;          /* levels per column */
  int32_t precision;     /* MG_PREC_* */
  int64_t ncol;          /* horizontal columns */
  const int64_t* col_base; /* device, ncol: state index of (col, lev 0, var 0) */
  int64_t lev_stride;    /* state index step between levels */
  int64_t var_stride;    /* state index step between variables */
  int64_t p;             /* observations */
  const double* HX;      /* device p x k: H(raw background members) */
  const double* yo;      /* device p */
  const double* rvar;    /* device p: error variance */
  const double* obs_lev; /* device p or NULL: vertical coordinate (level units) */
  const int64_t* loc_off;  /* device ncol+1: per-column candidate lists */
  const int32_t* loc_idx;  /* device: obs index */
  const double* loc_dist;  /* device or NULL: horizontal distance of each entry */
  double hsupport;       /* horizontal Gaspari-Cohn support (weight 0 beyond) */
  double vsupport;       /* vertical support in levels (obs with |dl| > vsupport dropped) */
  double rho;            /* inflation (MG_RTPS: relaxation alpha) */
  int32_t flags;         /* MG_* semantics bits */
  int32_t x_dtype;       /* MG_DTYPE_F64 or MG_DTYPE_F32 */
  double* mean_out;      /* device n or NULL: analysis ensemble mean */
} mg_letkf_desc;

/* Batched local analyses: replaces the serial grid-point loop of
 * LETKF::Analyse (LETKF.hpp:101) and updateGridPoint (:152-243) with one
 * local analysis per (column, level), all sharing the background obs-space
 * prior.  With MG_COMPAT flags each analysis follows updateGridPoint's
 * arithmetic; without them, the Hunt et al. (2007) LETKF with Gaspari-Cohn
 * R-localisation.  Points are scheduled in the grid's column order. */
int mg_letkf_batched(mg_context* ctx, const mg_letkf_desc* desc);

/* One case of an uneven batch of global ETKF analyses (see mg_etkf_batch_*). */
typedef struct mg_etkf_case {
  double* X;               /* members, member-major, updated in place */
  int64_t n;               /* state values per member */
  int64_t ld;              /* member stride (>= n) */
  int32_t k;               /* members, 2..112 */
  int32_t reserved;
  const double* HX;        /* p x k obs-space ensemble of the raw members, or NULL */
  const int64_t* obs_node; /* identity interpolation: state index of each obs (used when HX is NULL) */
  const double* yo;        /* p */
  const double* rvar;      /* p */
  int64_t p;               /* observations */
  double rho;              /* inflation */
  double* mean_out;        /* n (background mean) or NULL */
} mg_etkf_case;

typedef struct mg_etkf_batch mg_etkf_batch;

/* Many independent ETKF::Analyse calls (ETKF.hpp:100-179) of uneven sizes
 * in one pass.  create() flattens the cases (host array; device pointers
 * inside) into work-item tables and a workspace; run() only enqueues kernels
 * (no allocation, no host synchronisation: capturable); launch_graph()
 * captures run() once into a CUDA graph and replays it; finish() waits,
 * checks the status and returns each case's completion time after the batch
 * start in ms (case_ms: host array of ncases, or NULL).  autotune() times
 * candidate obs chunks for the Gram items and member-count bucket boundaries
 * on this batch (restoring the members between trials) and keeps the fastest;
 * it reports the choice (either pointer may be NULL).  flags / precision as
 * for mg_etkf; cases are analysed in place. */
int mg_etkf_batch_create(mg_context* ctx, const mg_etkf_case* cases, int32_t ncases, int32_t flags,
                         int32_t precision, mg_etkf_batch** batch);
int mg_etkf_batch_autotune(mg_context* ctx, mg_etkf_batch* batch, int32_t* gram_chunk,
                           int32_t* bucket_mode);
int mg_etkf_batch_run(mg_context* ctx, mg_etkf_batch* batch);
int mg_etkf_batch_launch_graph(mg_context* ctx, mg_etkf_batch* batch);
int mg_etkf_batch_finish(mg_context* ctx, mg_etkf_batch* batch, double* case_ms);
void mg_etkf_batch_destroy(mg_etkf_batch* batch);

/* ---- Learned column observation operator (no reference counterpart) ----
 * Plain operator: nlev-level columns of T (K) and q to nch channels,
 *   y_c = sum_l w[c,l] exp(-tau_c sum_{m<=l} q_m) T_l^4 / 1e8   (nch <= 32).
 * T, q: ncol x nlev row-major; w: nch x nlev; y: ncol x nch (all FP32). */
int mg_column_op(mg_context* ctx, const float* T, const float* q, int64_t ncol, int32_t nlev,
                 const float* w, const float* tau, int32_t nch, float* y);
/* MLP input features of columns: [(T_l - 255)/30, 100 q_l, 0 pad]
 * (ncol x nin, nin >= 2 nlev). */
int mg_column_features(mg_context* ctx, const float* T, const float* q, int64_t ncol, int32_t nlev,
                       int32_t nin, float* X);
/* H of column observations on a member-major state laid out
 * ((v*nlev + l)*ncol + col), v = 0: T (K), v = 1: ln q.  Obs o observes
 * channel obs_ch[o] of column obs_col[o]; HX is p x k (FP64). */
int mg_hx_column(mg_context* ctx, const double* X, int32_t k, int64_t ld, int64_t ncol, int32_t nlev,
                 const int64_t* obs_col, const int32_t* obs_ch, int64_t p, const float* w,
                 const float* tau, int32_t nch, double* HX);

/* Surrogate MLP nin -> nh -> nh -> nout, SiLU, BF16 weights and FP32
 * accumulation, FP32 master parameters trained by Adam on the mean squared
 * error of standardised outputs ((y - out_shift)/out_scale).  Parameters are
 * one FP32 vector [W1 (nh x nin), b1, W2 (nh x nh), b2, W3 (nout x nh), b3]. */
typedef struct mg_mlp mg_mlp;
int mg_mlp_create(mg_context* ctx, int32_t nin, int32_t nh, int32_t nout, mg_mlp** mlp);
void mg_mlp_destroy(mg_mlp* mlp);
int64_t mg_mlp_num_params(const mg_mlp* mlp);
/* params (device, num_params); out_shift/out_scale (device, nout) or NULL.
 * Resets the Adam state. */
int mg_mlp_set_params(mg_context* ctx, mg_mlp* mlp, const float* params, const float* out_shift,
                      const float* out_scale);
/* FP32 master parameters, or (bf16_rounded != 0) the BF16 working copy. */
int mg_mlp_get_params(mg_context* ctx, const mg_mlp* mlp, float* params, int32_t bf16_rounded);
/* Y (B x nout, standardised) = MLP(X (B x nin)). */
int mg_mlp_forward(mg_context* ctx, mg_mlp* mlp, const float* X, int64_t B, float* Y);
/* Gradients of the loss for targets Yt (B x nout, physical units) into grad
 * (device, num_params, may be NULL); *loss (host, may be NULL). */
int mg_mlp_gradients(mg_context* ctx, mg_mlp* mlp, const float* X, const float* Yt, int64_t B,
                     float* grad, float* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on a batch; *loss as above. */
int mg_mlp_train_step(mg_context* ctx, mg_mlp* mlp, const float* X, const float* Yt, int64_t B,
                      float lr, float* loss);
/* mg_hx_column with the surrogate in place of the plain operator. */
int mg_hx_column_mlp(mg_context* ctx, mg_mlp* mlp, const double* X, int32_t k, int64_t ld,
                     int64_t ncol, int32_t nlev, const int64_t* obs_col, const int32_t* obs_ch,
                     int64_t p, double* HX);

/* C (M x N, FP32, row-major) = A (M x K) B^T + bias, then SiLU if silu != 0;
 * A and B are BF16 row-major (K contiguous) device arrays, 16-byte aligned,
 * 1 <= N <= 256, K a multiple of 8; bias (N) may be NULL.  Runs on the
 * tensor cores (tcgen05, TMA-staged tiles, FP32 accumulation in tensor
 * memory); the surrogate's inference layers use the same kernel.  No
 * counterpart in the reference. */
int mg_gemm_bf16_tc(mg_context* ctx, const void* A, const void* B, int32_t M, int32_t N, int32_t K,
                    const float* bias, int32_t silu, float* C);

/* Self-test of the kernel's bounded waits: the same GEMM with one k-block
 * of every CTA's first tile never loaded, so a wait runs out (after about a
 * second) and the kernel returns instead of hanging.  *observed receives the
 * status the launch reports (MG_ERR_TIMEOUT when the waits work); returns
 * MG_OK when the kernel came back.  C is scratch.  No counterpart in the
 * reference. */
int mg_gemm_bf16_tc_wait_selftest(mg_context* ctx, const void* A, const void* B, int32_t M, int32_t N,
                                  int32_t K, float* C, int32_t* observed);

/* Text I/O of the analysis path on the device (text and output buffers
 * on the host; parsed arrays on the device).
 *
 * mg_parse_grid_obs replaces GridObservation::loadFromFile
 * (src/backends/common/observation/GridObservation.hpp:395-474) for the
 * "Time Z Y X ZNU XLONG_U XLAT_U Value" format: data lines after the first
 * separator line following a header line, read as int x4, double x4 with
 * std::istream rules, kept unless Value == missing_value, in file order.
 * xyz (count x 3: x, y, z) and vals (count x 4: znu, xlong_u, xlat_u,
 * value); *count receives the number kept (MG_ERR_CAPACITY if > cap).
 *
 * mg_parse_values replaces SimpleState::readFromFile (SimpleState.hpp:248-263):
 * every double of every line, up to the first failed extraction of a line.
 *
 * mg_format_state replaces SimpleState::saveToFile (SimpleState.hpp:160-188):
 * ny rows of nx "%12.6f" values joined by one space; *nbytes receives the
 * text length (MG_ERR_CAPACITY, without writing, if out is NULL or cap is
 * smaller).
 *
 * Numbers are converted exactly as strtod/printf do.  The device reads
 * every number whose result is a normal double (Clinger's fast path, else
 * Eisel-Lemire; more than 19 significant digits when the two 19-digit
 * bounds round alike) and writes every value below 2^53 in magnitude; the
 * rest (subnormal or overflowing results, the rare long mantissas whose
 * bounds round apart, large or non-finite values to write) goes through
 * the host's std::istringstream / std::ostream, the reference's own
 * conversions.  mg_last_io_host_items gives how many lines (parsers) or
 * values (writer) of the last such call on the context went that way.  No
 * counterpart for the device placement in the reference. */
int mg_parse_grid_obs(mg_context* ctx, const char* text, int64_t nbytes, double missing_value, int32_t* xyz,
                      double* vals, int64_t cap, int64_t* count);
int mg_parse_values(mg_context* ctx, const char* text, int64_t nbytes, double* out, int64_t cap, int64_t* count);
int mg_format_state(mg_context* ctx, const double* values, int32_t nx, int32_t ny, char* out, int64_t cap,
                    int64_t* nbytes);
int mg_last_io_host_items(mg_context* ctx, int64_t* count);

/* Nearest grid node of geographic observations on a curvilinear nx x ny
 * grid (node n = j*nx + i at node_lat[n], node_lon[n], degrees), replacing
 * the per-observation scan of IdentityObsOperator::convertGeographicToGrid
 * (src/backends/common/obsoperator/IdentityObsOperator.hpp:470-505): the
 * first node in index order minimising sqrt((lon - lon_n)^2 + (lat - lat_n)^2),
 * found through a device spatial hash, bit-identical to the scan.  out_xy
 * (p x 2 int32, device) receives (i, j), the format mg_hx_idw4 reads;
 * with out_k (p, may be NULL) also the first z minimising
 * |obs_level - vcoord[z]| (:491-500).  All arrays on the device. */
int mg_nearest_node(mg_context* ctx, const double* node_lat, const double* node_lon, int32_t nx, int32_t ny,
                    const double* obs_lat, const double* obs_lon, int64_t p, const double* vcoord, int32_t nz,
                    const double* obs_level, int32_t* out_xy, int32_t* out_k);

/* Stochastic EnKF with perturbed observations, replacing EnKF::Analyse
 * (src/framework/algorithms/EnKF.hpp:139-254), in place on the members.
 * HX (p x k row-major) is H of the raw members; obs_pert (p x k row-major)
 * the observation perturbations eps_i (the reference draws them inside,
 * from an unseeded generator, chol_L(R) z with z ~ N(0, 1), :336-352; here
 * the caller supplies them, so runs are reproducible).  The perturbations
 * are inflated by sqrt(inflation) for every inflation method (:322-335).
 * Computed in the k-dimensional form (no p x p matrix).  mean_out: the
 * recomputed analysis mean (device, n, may be NULL); diag (host, may be
 * NULL): ||yo - mean(HX)||, background and analysis spread.  MG_PREC_MIXED
 * runs the O(n k^2) update in FP32.  2 <= k <= 112. */
typedef struct mg_enkf_diag {
  double innovation_norm;
  double background_spread;
  double analysis_spread;
} mg_enkf_diag;
int mg_enkf(mg_context* ctx, double* X, int64_t n, int32_t k, int64_t ld, const double* HX, const double* yo,
            const double* rvar, const double* obs_pert, int64_t p, double inflation, int32_t precision,
            double* mean_out, mg_enkf_diag* diag);

/* Ensemble diagnostics, replacing Metrics<double>::CalculateAll
 * (src/framework/algorithms/Metrics.hpp:74-94): for members X (k x n,
 * member i at X + i*ld, device) against truth (n, device), the ensemble mean
 * and spread per element (device, n each, may be NULL; the mean is the
 * member-order sum divided by k, the spread sqrt(sum (x - mean)^2 / (k-1)),
 * both as the reference computes them) and, on the host, RMSE and bias of
 * the mean, its correlation with the truth (single-pass sums formula),
 * CRPS (pair-sum form) and the average spread.  2 <= k <= 256. */
typedef struct mg_ens_metrics_t {
  double rmse;
  double bias;
  double correlation;
  double crps;
  double avg_spread;
} mg_ens_metrics_t;
int mg_ens_metrics(mg_context* ctx, const double* X, int64_t n, int32_t k, int64_t ld, const double* truth,
                   double* mean_out, double* spread_out, mg_ens_metrics_t* out);

/* Statistics of the last mg_letkf_batched call (host). */
typedef struct mg_letkf_stats {
  int64_t n_points;      /* local analyses run */
  int64_t n_empty;       /* analyses with no local obs */
  int64_t total_local;   /* sum of local obs counts */
  int32_t max_local;     /* largest local obs count */
  int32_t max_sweeps;    /* Jacobi sweeps of the slowest analysis */
  double ms_prepare;     /* device time: perturbations, obs prior, ordering */
  double ms_analysis;    /* device time of the local-analysis kernel */
  double ms_writeback;   /* device time: write-back to members and mean */
  int64_t total_sweeps;  /* Jacobi sweeps (tensor-core path: Newton-Schulz iterations)
                            summed over all analyses */
  int64_t n_fallback;    /* tensor-core path: analyses whose residual test failed and
                            that the SIMT Jacobi kernel re-ran */
  double max_residual;   /* tensor-core path: largest max |Z A Z - P| accepted */
  int32_t tensor_path;   /* 1 when the tensor-core kernel ran the analyses */
  int32_t tensor_ctas;   /* CTAs of its persistent grid */
} mg_letkf_stats;
int mg_letkf_last_stats(const mg_context* ctx, mg_letkf_stats* stats);

/* State vector arithmetic on the device, for the device-resident state
 * backend (SimpleState::add / subtract / multiply / dot, SimpleState.hpp:96-140):
 * y[i] += x[i] (subtract = 0) or y[i] -= x[i] (subtract != 0), and
 * y[i] *= a, one IEEE operation per element, so the results equal the
 * reference's host loops bit for bit.  mg_vec_dot sums in a fixed
 * (deterministic) order that differs from the reference's sequential one;
 * *result is host memory and the call synchronises the stream. */
int mg_vec_update(mg_context* ctx, double* y, const double* x, int64_t n, int32_t subtract);
int mg_vec_scale(mg_context* ctx, double* y, int64_t n, double a);
int mg_vec_dot(mg_context* ctx, const double* x, const double* y, int64_t n, double* result);

/* Number of kernels this context has launched since creation (host). */
int64_t mg_kernel_launches(const mg_context* ctx);

#ifdef __cplusplus
}
#endif

#endif /* METADA_GB300_H */
