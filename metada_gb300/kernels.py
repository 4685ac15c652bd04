"""Thin tensor-level wrappers over the C-ABI.

Every function takes CUDA tensors (torch is used only for device memory and
streams), checks shapes/dtypes, and calls the corresponding ``mg_*`` entry
point on the current torch stream.  Nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_int64, c_void_p

import torch

from . import _lib
from ._lib import Context, LetkfDesc, LetkfStats

_contexts: dict[int, Context] = {}


def context(device: int | None = None) -> Context:
    """Per-device context bound to torch's current stream."""
    if device is None:
        device = torch.cuda.current_device()
    ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        _contexts[device] = ctx
    ctx.set_stream(torch.cuda.current_stream(device).cuda_stream)
    return ctx


def _ptr(t: torch.Tensor | None) -> c_void_p:
    if t is None:
        return c_void_p(0)
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return c_void_p(t.data_ptr())


def _need(t: torch.Tensor, dtype: torch.dtype, name: str) -> None:
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {t.dtype}")


def ens_mean(X: torch.Tensor) -> torch.Tensor:
    """Ensemble mean of members X (k x n, float64), member-order sum * (1/k)."""
    _need(X, torch.float64, "X")
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    context(X.device.index).call("mg_ens_mean", _ptr(X), n, k, n, _ptr(mean))
    return mean


def ens_mean_pert(X: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    _need(X, torch.float64, "X")
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    Xp = torch.empty_like(X)
    context(X.device.index).call("mg_ens_mean_pert", _ptr(X), n, k, n, _ptr(mean), _ptr(Xp), n)
    return mean, Xp


# Outputs sized by an upper bound up to this many bytes take one call; larger
# ones are sized by a counting call first.
_ONE_CALL_BYTES = 1 << 30


def _trim(t: torch.Tensor, n: int) -> torch.Tensor:
    """The first n rows, in their own allocation when the bound was loose."""
    return t[:n].clone() if 2 * n < t.shape[0] else t[:n]


def parse_grid_obs(text: bytes, missing_value: float = -999.0,
                   device: int = 0) -> tuple[torch.Tensor, torch.Tensor]:
    """GridObservation text -> (xyz int32 p x 3: x, y, z; vals float64 p x 4:
    znu, xlong_u, xlat_u, value) on the device."""
    ctx = context(device)
    dev = torch.device("cuda", device)
    count = c_int64(0)
    # A data line holds 8 numbers with a non-digit between each two: at least
    # 15 characters and its newline.
    bound = (len(text) + 1) // 16 + 1
    cap = bound if 44 * bound <= _ONE_CALL_BYTES else 0
    xyz = torch.empty((max(cap, 1), 3), dtype=torch.int32, device=dev)
    vals = torch.empty((max(cap, 1), 4), dtype=torch.float64, device=dev)
    rc = ctx.lib.mg_parse_grid_obs(ctx.handle, text, len(text), float(missing_value), _ptr(xyz), _ptr(vals), cap,
                                   byref(count))
    if rc == _lib.MG_ERR_CAPACITY:
        xyz = torch.empty((max(count.value, 1), 3), dtype=torch.int32, device=dev)
        vals = torch.empty((max(count.value, 1), 4), dtype=torch.float64, device=dev)
        ctx.call("mg_parse_grid_obs", text, len(text), float(missing_value), _ptr(xyz), _ptr(vals), count.value,
                 byref(count))
    else:
        ctx.check(rc)
    return _trim(xyz, count.value), _trim(vals, count.value)


def parse_values(text: bytes, device: int = 0) -> torch.Tensor:
    """SimpleState text -> its values (float64) on the device."""
    ctx = context(device)
    dev = torch.device("cuda", device)
    count = c_int64(0)
    # Two extracted values need a non-digit between their digits.
    bound = (len(text) + 1) // 2
    cap = bound if 8 * bound <= _ONE_CALL_BYTES else 0
    out = torch.empty(max(cap, 1), dtype=torch.float64, device=dev)
    rc = ctx.lib.mg_parse_values(ctx.handle, text, len(text), _ptr(out), cap, byref(count))
    if rc == _lib.MG_ERR_CAPACITY:
        out = torch.empty(max(count.value, 1), dtype=torch.float64, device=dev)
        ctx.call("mg_parse_values", text, len(text), _ptr(out), count.value, byref(count))
    else:
        ctx.check(rc)
    return _trim(out, count.value)


def format_state(values: torch.Tensor, nx: int, ny: int) -> bytes:
    """SimpleState::saveToFile text of ny rows of nx values ("%12.6f")."""
    _need(values, torch.float64, "values")
    ctx = context(values.device.index)
    nbytes = c_int64(0)
    # A value the device formats (|v| < 2^53) takes at most 24 characters and
    # its separator; others are formatted on the host and may need a second
    # call.  The text lands in pinned memory (the host allocator reuses it).
    cap = 25 * nx * ny + 1
    if cap > _ONE_CALL_BYTES:  # too much pinned memory for a bound: count first
        rc = ctx.lib.mg_format_state(ctx.handle, _ptr(values), nx, ny, c_void_p(0), 0, byref(nbytes))
        if rc != _lib.MG_ERR_CAPACITY:
            ctx.check(rc)
        cap = max(nbytes.value, 1)
    buf = torch.empty(cap, dtype=torch.uint8, pin_memory=True)
    rc = ctx.lib.mg_format_state(ctx.handle, _ptr(values), nx, ny, c_void_p(buf.data_ptr()), cap, byref(nbytes))
    if rc == _lib.MG_ERR_CAPACITY:
        buf = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, pin_memory=True)
        ctx.call("mg_format_state", _ptr(values), nx, ny, c_void_p(buf.data_ptr()), nbytes.value, byref(nbytes))
    else:
        ctx.check(rc)
    return buf[: nbytes.value].numpy().tobytes()


def last_io_host_items(device: int = 0) -> int:
    """Lines (parsers) or values (writer) of the last text I/O call on the
    device's context that were converted on the host."""
    n = c_int64(0)
    context(device).call("mg_last_io_host_items", byref(n))
    return n.value


def nearest_node(node_lat: torch.Tensor, node_lon: torch.Tensor, nx: int, ny: int, obs_lat: torch.Tensor,
                 obs_lon: torch.Tensor, vcoord: torch.Tensor | None = None,
                 obs_level: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor | None]:
    """Nearest node (i, j) of each geographic observation on a curvilinear
    grid (and the nearest vertical index when vcoord/obs_level are given)."""
    for t, nm in ((node_lat, "node_lat"), (node_lon, "node_lon"), (obs_lat, "obs_lat"), (obs_lon, "obs_lon")):
        _need(t, torch.float64, nm)
    p = obs_lat.shape[0]
    xy = torch.empty((p, 2), dtype=torch.int32, device=obs_lat.device)
    kk = torch.empty(p, dtype=torch.int32, device=obs_lat.device) if vcoord is not None else None
    context(obs_lat.device.index).call("mg_nearest_node", _ptr(node_lat), _ptr(node_lon), nx, ny, _ptr(obs_lat),
                                       _ptr(obs_lon), p, _ptr(vcoord), vcoord.shape[0] if vcoord is not None else 0,
                                       _ptr(obs_level), _ptr(xy), _ptr(kk))
    return xy, kk


def enkf(X: torch.Tensor, HX: torch.Tensor, yo: torch.Tensor, rvar: torch.Tensor, obs_pert: torch.Tensor,
         inflation: float, precision: int = _lib.MG_PREC_FP64) -> tuple[torch.Tensor, dict]:
    """Stochastic EnKF in place on X (k x n); returns (analysis mean, diagnostics)."""
    _need(X, torch.float64, "X")
    k, n = X.shape
    p = yo.shape[0]
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    d = _lib.EnkfDiag()
    context(X.device.index).call("mg_enkf", _ptr(X), n, k, n, _ptr(HX), _ptr(yo), _ptr(rvar), _ptr(obs_pert), p,
                                 float(inflation), precision, _ptr(mean), byref(d))
    return mean, {f: getattr(d, f) for f, _ in d._fields_}


def ens_metrics(X: torch.Tensor, truth: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, dict]:
    """Ensemble diagnostics of members X (k x n, float64) against truth (n):
    (mean, spread, {rmse, bias, correlation, crps, avg_spread})."""
    _need(X, torch.float64, "X")
    _need(truth, torch.float64, "truth")
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    spread = torch.empty(n, dtype=torch.float64, device=X.device)
    out = _lib.EnsMetrics()
    context(X.device.index).call("mg_ens_metrics", _ptr(X), n, k, n, _ptr(truth), _ptr(mean), _ptr(spread),
                                 byref(out))
    return mean, spread, {f: getattr(out, f) for f, _ in out._fields_}


def hx_idw4(X: torch.Tensor, nx: int, ny: int, obs_xy: torch.Tensor,
            valid: torch.Tensor | None = None) -> torch.Tensor:
    """IDW4 obs operator for grid obs; returns HX (p x k)."""
    _need(X, torch.float64, "X")
    _need(obs_xy, torch.int32, "obs_xy")
    k, n = X.shape
    p = obs_xy.shape[0]
    HX = torch.empty((p, k), dtype=torch.float64, device=X.device)
    if valid is not None:
        _need(valid, torch.uint8, "valid")
    context(X.device.index).call("mg_hx_idw4", _ptr(X), k, n, nx, ny, _ptr(obs_xy), _ptr(valid), p, _ptr(HX))
    return HX


def hx_latlon(X: torch.Tensor, nlon: int, nlat: int, nlev: int, obs_lat: torch.Tensor,
              obs_lon: torch.Tensor, obs_lev: torch.Tensor, obs_var: torch.Tensor) -> torch.Tensor:
    if X.dtype != torch.float32:
        _need(X, torch.float64, "X")
    else:
        _need(X, torch.float32, "X")
    _need(obs_var, torch.int32, "obs_var")
    k, n = X.shape
    p = obs_lat.shape[0]
    HX = torch.empty((p, k), dtype=torch.float64, device=X.device)
    fn = "mg_hx_latlon_f32" if X.dtype == torch.float32 else "mg_hx_latlon"
    context(X.device.index).call(fn, _ptr(X), k, n, nlon, nlat, nlev, _ptr(obs_lat),
                                 _ptr(obs_lon), _ptr(obs_lev), _ptr(obs_var), p, _ptr(HX))
    return HX


def select_grid(nx: int, ny: int, obs_xy: torch.Tensor, radius: float) -> tuple[torch.Tensor, torch.Tensor]:
    """Local obs lists for every grid point (CSR: offsets, idx)."""
    _need(obs_xy, torch.int32, "obs_xy")
    dev = obs_xy.device
    ctx = context(dev.index)
    p = obs_xy.shape[0]
    offsets = torch.empty(nx * ny + 1, dtype=torch.int64, device=dev)
    total = c_int64(0)
    rc = ctx.lib.mg_select_grid(ctx.handle, nx, ny, _ptr(obs_xy), p, float(radius), _ptr(offsets), c_void_p(0),
                                0, byref(total))
    if rc not in (_lib.MG_OK, _lib.MG_ERR_CAPACITY):
        ctx.check(rc)
    idx = torch.empty(max(total.value, 1), dtype=torch.int32, device=dev)
    ctx.call("mg_select_grid", nx, ny, _ptr(obs_xy), p, float(radius), _ptr(offsets), _ptr(idx), idx.numel(),
             byref(total))
    return offsets, idx[: total.value]


# Last list length per (device, ncol, p, radius): repeated searches of the
# same shape pass it as the capacity, so the search runs once instead of a
# sizing call followed by the filling call.
_GEO_CAP: dict[tuple, int] = {}


def select_geo(col_lat: torch.Tensor, col_lon: torch.Tensor, obs_lat: torch.Tensor, obs_lon: torch.Tensor,
               radius_km: float, cap: int | None = None) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Local obs lists for every query column (haversine <= radius_km)."""
    for t, nm in ((col_lat, "col_lat"), (col_lon, "col_lon"), (obs_lat, "obs_lat"), (obs_lon, "obs_lon")):
        _need(t, torch.float64, nm)
    dev = col_lat.device
    ctx = context(dev.index)
    ncol = col_lat.shape[0]
    p = obs_lat.shape[0]
    key = (dev.index, ncol, p, float(radius_km))
    offsets = torch.empty(ncol + 1, dtype=torch.int64, device=dev)
    total = c_int64(0)
    if cap is None:
        cap = _GEO_CAP.get(key, 0)
    for _ in range(2):
        idx = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
        dist = torch.empty(max(cap, 1), dtype=torch.float64, device=dev)
        rc = ctx.lib.mg_select_geo(ctx.handle, _ptr(col_lat), _ptr(col_lon), ncol, _ptr(obs_lat), _ptr(obs_lon), p,
                                   float(radius_km), _ptr(offsets), _ptr(idx) if cap > 0 else c_void_p(0),
                                   _ptr(dist) if cap > 0 else c_void_p(0), cap, byref(total))
        if rc == _lib.MG_ERR_CAPACITY and total.value > cap:
            cap = total.value
            continue
        ctx.check(rc)
        break
    _GEO_CAP[key] = total.value
    return offsets, idx[: total.value], dist[: total.value]


def etkf(X: torch.Tensor, HX: torch.Tensor, yo: torch.Tensor, rvar: torch.Tensor, rho: float,
         flags: int = _lib.MG_COMPAT, precision: int = _lib.MG_PREC_FP64) -> torch.Tensor:
    """Global ETKF in place on X (k x n); returns the background mean."""
    _need(X, torch.float64, "X")
    k, n = X.shape
    p = HX.shape[0]
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    context(X.device.index).call("mg_etkf", _ptr(X), n, k, n, _ptr(HX), _ptr(yo), _ptr(rvar), p, float(rho),
                                 int(flags), int(precision), _ptr(mean))
    return mean


def letkf_compat_grid(X: torch.Tensor, nx: int, ny: int, obs_xy: torch.Tensor, yo: torch.Tensor,
                      radius: float, rho: float, valid: torch.Tensor | None = None) -> torch.Tensor:
    """Reference-order LETKF in place on X; returns the recomputed mean."""
    _need(X, torch.float64, "X")
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    context(X.device.index).call("mg_letkf_compat_grid", _ptr(X), k, n, nx, ny, _ptr(obs_xy), _ptr(valid),
                                 _ptr(yo), obs_xy.shape[0], float(radius), float(rho), _ptr(mean))
    return mean


def letkf_batched(X: torch.Tensor, *, col_base: torch.Tensor, nlev: int, n_var: int, lev_stride: int,
                  var_stride: int, HX: torch.Tensor, yo: torch.Tensor, rvar: torch.Tensor,
                  loc_off: torch.Tensor, loc_idx: torch.Tensor, loc_dist: torch.Tensor | None = None,
                  obs_lev: torch.Tensor | None = None, hsupport: float = 0.0, vsupport: float = 0.0,
                  rho: float = 1.0, flags: int = 0, precision: int = _lib.MG_PREC_FP64,
                  want_mean: bool = True) -> tuple[torch.Tensor | None, LetkfStats]:
    """Batched LETKF in place on X (k x n, float64, or float32 with the mixed
    precision path)."""
    if X.dtype == torch.float32:
        if precision != _lib.MG_PREC_MIXED:
            raise TypeError("X: float32 members need precision=MG_PREC_MIXED")
    else:
        _need(X, torch.float64, "X")
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device) if want_mean else None
    d = LetkfDesc()
    d.X = X.data_ptr()
    d.x_dtype = _lib.MG_DTYPE_F32 if X.dtype == torch.float32 else _lib.MG_DTYPE_F64
    d.n = n
    d.ld = n
    d.k = k
    d.n_var = n_var
    d.nlev = nlev
    d.precision = precision
    d.ncol = col_base.shape[0]
    d.col_base = _ptr(col_base).value
    d.lev_stride = lev_stride
    d.var_stride = var_stride
    d.p = HX.shape[0]
    d.HX = _ptr(HX).value
    d.yo = _ptr(yo).value
    d.rvar = _ptr(rvar).value
    d.obs_lev = _ptr(obs_lev).value
    d.loc_off = _ptr(loc_off).value
    d.loc_idx = _ptr(loc_idx).value if loc_idx.numel() else None
    d.loc_dist = _ptr(loc_dist).value if (loc_dist is not None and loc_dist.numel()) else None
    d.hsupport = hsupport
    d.vsupport = vsupport
    d.rho = rho
    d.flags = flags
    d.mean_out = _ptr(mean).value
    ctx = context(X.device.index)
    ctx.call("mg_letkf_batched", ctypes.byref(d))
    st = LetkfStats()
    ctx.call("mg_letkf_last_stats", ctypes.byref(st))
    return mean, st


class EtkfBatch:
    """An uneven batch of global ETKF analyses (mg_etkf_batch_*), in place on
    the members.  `cases` is a list of dicts with keys X (k x n float64 CUDA
    tensor), yo, rvar (p), and HX (p x k) or obs_node (p int64), rho."""

    def __init__(self, cases, flags: int = _lib.MG_COMPAT, precision: int = _lib.MG_PREC_FP64,
                 want_mean: bool = False):
        import numpy as np

        self.cases = cases
        dev = cases[0]["X"].device
        self.ctx = context(dev.index)
        arr = (_lib.EtkfCase * len(cases))()
        self.means = []
        for i, c in enumerate(cases):
            X = c["X"]
            _need(X, torch.float64, "X")
            k, n = X.shape
            a = arr[i]
            a.X = X.data_ptr()
            a.n = n
            a.ld = n
            a.k = k
            a.HX = _ptr(c.get("HX")).value
            a.obs_node = _ptr(c.get("obs_node")).value
            a.yo = _ptr(c["yo"]).value
            a.rvar = _ptr(c["rvar"]).value
            a.p = c["yo"].shape[0]
            a.rho = float(c.get("rho", 1.0))
            m = torch.empty(n, dtype=torch.float64, device=dev) if want_mean else None
            self.means.append(m)
            a.mean_out = _ptr(m).value
        self._arr = arr
        h = c_void_p()
        self.ctx.call("mg_etkf_batch_create", ctypes.cast(arr, c_void_p), len(cases), int(flags), int(precision),
                      byref(h))
        self.handle = h
        self.case_ms = np.zeros(len(cases))

    def autotune(self) -> tuple[int, int]:
        ch, mode = ctypes.c_int32(0), ctypes.c_int32(0)
        self.ctx.call("mg_etkf_batch_autotune", self.handle, byref(ch), byref(mode))
        return ch.value, mode.value

    def run(self, graph: bool = True) -> None:
        self.ctx.call("mg_etkf_batch_launch_graph" if graph else "mg_etkf_batch_run", self.handle)

    def finish(self):
        import numpy as np

        buf = (ctypes.c_double * len(self.cases))()
        self.ctx.call("mg_etkf_batch_finish", self.handle, ctypes.cast(buf, c_void_p))
        self.case_ms = np.frombuffer(buf, dtype=np.float64).copy()
        return self.case_ms

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.mg_etkf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------ tensor-core GEMM ----
def gemm_bf16_tc(A: torch.Tensor, B: torch.Tensor, bias: torch.Tensor | None = None,
                 silu: bool = False) -> torch.Tensor:
    """C = A B^T (+ bias, SiLU) on the tensor cores: A (M x K) and B (N x K)
    BF16, C FP32."""
    _need(A, torch.bfloat16, "A")
    _need(B, torch.bfloat16, "B")
    M, K = A.shape
    N = B.shape[0]
    C = torch.empty((M, N), dtype=torch.float32, device=A.device)
    context(A.device.index).call("mg_gemm_bf16_tc", _ptr(A), _ptr(B), M, N, K, _ptr(bias), int(silu), _ptr(C))
    return C


def gemm_bf16_tc_wait_selftest(A: torch.Tensor, B: torch.Tensor) -> int:
    """Runs the tensor-core GEMM with one k-block never loaded; returns the
    status its bounded waits report (MG_ERR_TIMEOUT when they work)."""
    _need(A, torch.bfloat16, "A")
    _need(B, torch.bfloat16, "B")
    M, K = A.shape
    N = B.shape[0]
    C = torch.empty((M, N), dtype=torch.float32, device=A.device)
    obs = ctypes.c_int32(-1)
    context(A.device.index).call("mg_gemm_bf16_tc_wait_selftest", _ptr(A), _ptr(B), M, N, K, _ptr(C), byref(obs))
    return obs.value


# ----------------------------------------------------- column operator ----
def column_op(T: torch.Tensor, q: torch.Tensor, w: torch.Tensor, tau: torch.Tensor) -> torch.Tensor:
    """Plain column operator: T, q (ncol x nlev float32) -> y (ncol x nch)."""
    ncol, nlev = T.shape
    nch = tau.shape[0]
    y = torch.empty((ncol, nch), dtype=torch.float32, device=T.device)
    context(T.device.index).call("mg_column_op", _ptr(T), _ptr(q), ncol, nlev, _ptr(w), _ptr(tau), nch, _ptr(y))
    return y


def column_features(T: torch.Tensor, q: torch.Tensor, nin: int = 64) -> torch.Tensor:
    ncol, nlev = T.shape
    X = torch.empty((ncol, nin), dtype=torch.float32, device=T.device)
    context(T.device.index).call("mg_column_features", _ptr(T), _ptr(q), ncol, nlev, nin, _ptr(X))
    return X


def hx_column(X: torch.Tensor, ncol: int, nlev: int, obs_col: torch.Tensor, obs_ch: torch.Tensor, w: torch.Tensor,
              tau: torch.Tensor) -> torch.Tensor:
    """Plain H of column obs on a member-major (T, ln q) state; HX p x k."""
    _need(X, torch.float64, "X")
    k, n = X.shape
    p = obs_col.shape[0]
    HX = torch.empty((p, k), dtype=torch.float64, device=X.device)
    context(X.device.index).call("mg_hx_column", _ptr(X), k, n, ncol, nlev, _ptr(obs_col), _ptr(obs_ch), p, _ptr(w),
                                 _ptr(tau), tau.shape[0], _ptr(HX))
    return HX


class MLP:
    """The surrogate network (mg_mlp_*): nin -> nh -> nh -> nout, SiLU, BF16
    weights, FP32 accumulation and master parameters, Adam."""

    def __init__(self, nin: int = 64, nh: int = 256, nout: int = 16, device: int = 0):
        self.ctx = context(device)
        self.nin, self.nh, self.nout = nin, nh, nout
        h = c_void_p()
        self.ctx.call("mg_mlp_create", nin, nh, nout, byref(h))
        self.handle = h
        self.nparam = int(self.ctx.lib.mg_mlp_num_params(h))
        self.device = torch.device("cuda", device)

    def init_params(self, seed: int = 0) -> torch.Tensor:
        """Seeded uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases."""
        import numpy as np

        g = np.random.Generator(np.random.PCG64(seed))
        parts = []
        for fan_out, fan_in in ((self.nh, self.nin), (self.nh, self.nh), (self.nout, self.nh)):
            bound = 1.0 / np.sqrt(fan_in)
            parts.append(g.uniform(-bound, bound, fan_out * fan_in))
            parts.append(np.zeros(fan_out))
        P = torch.tensor(np.concatenate(parts), dtype=torch.float32, device=self.device)
        self.set_params(P)
        return P

    def set_params(self, P: torch.Tensor, out_shift: torch.Tensor | None = None,
                   out_scale: torch.Tensor | None = None) -> None:
        self.ctx.call("mg_mlp_set_params", self.handle, _ptr(P), _ptr(out_shift), _ptr(out_scale))

    def params(self, bf16_rounded: bool = False) -> torch.Tensor:
        P = torch.empty(self.nparam, dtype=torch.float32, device=self.device)
        self.ctx.call("mg_mlp_get_params", self.handle, _ptr(P), int(bf16_rounded))
        return P

    def forward(self, X: torch.Tensor) -> torch.Tensor:
        Y = torch.empty((X.shape[0], self.nout), dtype=torch.float32, device=X.device)
        self.ctx.call("mg_mlp_forward", self.handle, _ptr(X), X.shape[0], _ptr(Y))
        return Y

    def gradients(self, X: torch.Tensor, Yt: torch.Tensor) -> tuple[torch.Tensor, float]:
        G = torch.empty(self.nparam, dtype=torch.float32, device=X.device)
        loss = ctypes.c_float(0.0)
        self.ctx.call("mg_mlp_gradients", self.handle, _ptr(X), _ptr(Yt), X.shape[0], _ptr(G), byref(loss))
        return G, loss.value

    def train_step(self, X: torch.Tensor, Yt: torch.Tensor, lr: float, want_loss: bool = False) -> float:
        loss = ctypes.c_float(0.0)
        self.ctx.call("mg_mlp_train_step", self.handle, _ptr(X), _ptr(Yt), X.shape[0], ctypes.c_float(lr),
                      byref(loss) if want_loss else None)
        return loss.value

    def hx_column(self, X: torch.Tensor, ncol: int, nlev: int, obs_col: torch.Tensor,
                  obs_ch: torch.Tensor) -> torch.Tensor:
        _need(X, torch.float64, "X")
        k, n = X.shape
        p = obs_col.shape[0]
        HX = torch.empty((p, k), dtype=torch.float64, device=X.device)
        self.ctx.call("mg_hx_column_mlp", self.handle, _ptr(X), k, n, ncol, nlev, _ptr(obs_col), _ptr(obs_ch), p,
                      _ptr(HX))
        return HX

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.mg_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
