"""ctypes binding of the CPU oracle (oracle.h).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  The product never imports
this module.  Arrays are numpy arrays (C-contiguous).
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

ORC_R_IDENTITY = 1
ORC_SQRT_CHOLESKY = 2
ORC_INFL_COMPAT = 4
ORC_UPDATE_COMPAT = 8
ORC_COMPAT = 15
ORC_RTPS = 16

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            import sys

            sys.path.insert(0, str(HERE.parent))
            from metada_gb300.build import build_oracle

            build_oracle()
        lib = ctypes.CDLL(str(LIB))
        vp = c_void_p
        sig = {
            "orc_ens_mean": ([vp, c_int64, c_int32, c_int64, vp], None),
            "orc_ens_mean_pert": ([vp, c_int64, c_int32, c_int64, vp, vp, c_int64], None),
            "orc_hx_idw4": ([vp, c_int32, c_int64, c_int32, c_int32, vp, vp, c_int64, vp], None),
            "orc_hx_latlon": ([vp, c_int32, c_int64, c_int32, c_int32, c_int32, vp, vp, vp, vp, c_int64, vp], None),
            "orc_grid_distance": ([c_int32, c_int32, c_int32, c_int32], c_double),
            "orc_haversine_km": ([c_double] * 4, c_double),
            "orc_gaspari_cohn": ([c_double], c_double),
            "orc_select_grid": ([c_int32, c_int32, vp, c_int64, c_double, vp, vp, c_int64], c_int64),
            "orc_select_geo": ([vp, vp, c_int64, vp, vp, c_int64, c_double, vp, vp, vp, c_int64], c_int64),
            "orc_etkf_compat": ([vp, c_int64, c_int32, c_int64, vp, vp, vp, c_int64, c_double, vp], ctypes.c_int),
            "orc_letkf_compat_grid": ([vp, c_int32, c_int64, c_int32, c_int32, vp, vp, vp, c_int64, c_double,
                                       c_double, vp], ctypes.c_int),
            "orc_letkf_points": ([vp, c_int32, c_int64, vp, c_int32, c_int64, c_int64, vp, vp, vp, c_int64, vp, vp,
                                  vp, c_double, c_int32, vp], ctypes.c_int),
            "orc_sym_eig": ([vp, c_int32, vp, vp], ctypes.c_int),
            "orc_column_op": ([vp, vp, c_int64, c_int32, vp, vp, c_int32, vp], None),
            "orc_ens_metrics": ([vp, c_int64, c_int32, c_int64, vp, vp, vp, vp], None),
            "orc_nearest_node": ([vp, vp, c_int32, c_int32, vp, vp, c_int64, vp, c_int32, vp, vp, vp], None),
            "orc_enkf": ([vp, c_int64, c_int32, c_int64, vp, vp, vp, vp, c_int64, c_double, vp, vp, vp], ctypes.c_int),
            "orc_parse_values": ([ctypes.c_char_p, c_int64, vp, c_int64], c_int64),
            "orc_num_threads": ([], ctypes.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def _p(a: np.ndarray | None) -> c_void_p:
    if a is None:
        return c_void_p(0)
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return c_void_p(a.ctypes.data)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def ens_mean(X: np.ndarray) -> np.ndarray:
    X = _f64(X)
    k, n = X.shape
    mean = np.empty(n)
    load().orc_ens_mean(_p(X), n, k, n, _p(mean))
    return mean


def ens_mean_pert(X: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    X = _f64(X)
    k, n = X.shape
    mean = np.empty(n)
    Xp = np.empty_like(X)
    load().orc_ens_mean_pert(_p(X), n, k, n, _p(mean), _p(Xp), n)
    return mean, Xp


def hx_idw4(X: np.ndarray, nx: int, ny: int, obs_xy: np.ndarray, valid: np.ndarray | None = None) -> np.ndarray:
    X = _f64(X)
    obs_xy = np.ascontiguousarray(obs_xy, dtype=np.int32)
    k, n = X.shape
    p = obs_xy.shape[0]
    HX = np.empty((p, k))
    v = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
    load().orc_hx_idw4(_p(X), k, n, nx, ny, _p(obs_xy), _p(v), p, _p(HX))
    return HX


def hx_latlon(X, nlon, nlat, nlev, obs_lat, obs_lon, obs_lev, obs_var) -> np.ndarray:
    X = _f64(X)
    k, n = X.shape
    obs_lat, obs_lon, obs_lev = _f64(obs_lat), _f64(obs_lon), _f64(obs_lev)
    obs_var = np.ascontiguousarray(obs_var, dtype=np.int32)
    p = obs_lat.shape[0]
    HX = np.empty((p, k))
    load().orc_hx_latlon(_p(X), k, n, nlon, nlat, nlev, _p(obs_lat), _p(obs_lon), _p(obs_lev), _p(obs_var), p,
                         _p(HX))
    return HX


def haversine_km(lat1, lon1, lat2, lon2) -> float:
    return load().orc_haversine_km(lat1, lon1, lat2, lon2)


def gaspari_cohn(z: float) -> float:
    return load().orc_gaspari_cohn(z)


def select_grid(nx: int, ny: int, obs_xy: np.ndarray, radius: float) -> tuple[np.ndarray, np.ndarray]:
    obs_xy = np.ascontiguousarray(obs_xy, dtype=np.int32)
    p = obs_xy.shape[0]
    off = np.empty(nx * ny + 1, dtype=np.int64)
    total = load().orc_select_grid(nx, ny, _p(obs_xy), p, radius, _p(off), c_void_p(0), 0)
    idx = np.empty(max(total, 1), dtype=np.int32)
    load().orc_select_grid(nx, ny, _p(obs_xy), p, radius, _p(off), _p(idx), idx.size)
    return off, idx[:total]


def select_geo(col_lat, col_lon, obs_lat, obs_lon, radius_km: float):
    col_lat, col_lon, obs_lat, obs_lon = map(_f64, (col_lat, col_lon, obs_lat, obs_lon))
    ncol, p = col_lat.shape[0], obs_lat.shape[0]
    off = np.empty(ncol + 1, dtype=np.int64)
    total = load().orc_select_geo(_p(col_lat), _p(col_lon), ncol, _p(obs_lat), _p(obs_lon), p, radius_km, _p(off),
                                  c_void_p(0), c_void_p(0), 0)
    idx = np.empty(max(total, 1), dtype=np.int32)
    dist = np.empty(max(total, 1))
    load().orc_select_geo(_p(col_lat), _p(col_lon), ncol, _p(obs_lat), _p(obs_lon), p, radius_km, _p(off), _p(idx),
                          _p(dist), idx.size)
    return off, idx[:total], dist[:total]


def etkf_compat(X: np.ndarray, HX: np.ndarray, yo: np.ndarray, rvar: np.ndarray, rho: float):
    """Returns (analysis members, background mean)."""
    Xa = _f64(X).copy()
    k, n = Xa.shape
    HX, yo, rvar = _f64(HX), _f64(yo), _f64(rvar)
    mean = np.empty(n)
    rc = load().orc_etkf_compat(_p(Xa), n, k, n, _p(HX), _p(yo), _p(rvar), HX.shape[0], rho, _p(mean))
    if rc != 0:
        raise RuntimeError("oracle ETKF: matrix not positive definite")
    return Xa, mean


def letkf_compat_grid(X, nx, ny, obs_xy, yo, radius, rho, valid=None):
    Xa = _f64(X).copy()
    k, n = Xa.shape
    obs_xy = np.ascontiguousarray(obs_xy, dtype=np.int32)
    yo = _f64(yo)
    v = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
    mean = np.empty(n)
    rc = load().orc_letkf_compat_grid(_p(Xa), k, n, nx, ny, _p(obs_xy), _p(v), _p(yo), obs_xy.shape[0], radius,
                                      rho, _p(mean))
    if rc != 0:
        raise RuntimeError("oracle LETKF: matrix not positive definite")
    return Xa, mean


def letkf_points(X, pt_base, n_var, var_stride, HX, yo, rvar, loc_off, loc_idx, loc_w, rho, flags) -> np.ndarray:
    """Analysis (npt x n_var x k) of the given points (snapshot semantics)."""
    X = _f64(X)
    k, n = X.shape
    pt_base = np.ascontiguousarray(pt_base, dtype=np.int64)
    HX, yo, rvar = _f64(HX), _f64(yo), _f64(rvar)
    loc_off = np.ascontiguousarray(loc_off, dtype=np.int64)
    loc_idx = np.ascontiguousarray(loc_idx, dtype=np.int32)
    w = None if loc_w is None else _f64(loc_w)
    npt = pt_base.shape[0]
    out = np.empty((npt, n_var, k))
    rc = load().orc_letkf_points(_p(X), k, n, _p(pt_base), n_var, var_stride, npt, _p(HX), _p(yo), _p(rvar),
                                 HX.shape[0], _p(loc_off), _p(loc_idx if loc_idx.size else None), _p(w), rho,
                                 flags, _p(out))
    if rc != 0:
        raise RuntimeError("oracle LETKF points: matrix not positive definite")
    return out


def sym_eig(A: np.ndarray):
    A = _f64(A).copy()
    k = A.shape[0]
    w = np.empty(k)
    V = np.empty((k, k))
    sweeps = load().orc_sym_eig(_p(A), k, _p(w), _p(V))
    return w, V, sweeps


def column_op(T, q, w, tau):
    T = np.ascontiguousarray(T, dtype=np.float32)
    q = np.ascontiguousarray(q, dtype=np.float32)
    w = np.ascontiguousarray(w, dtype=np.float32)
    tau = np.ascontiguousarray(tau, dtype=np.float32)
    ncol, nlev = T.shape
    nch = tau.shape[0]
    y = np.empty((ncol, nch), dtype=np.float32)
    load().orc_column_op(_p(T), _p(q), ncol, nlev, _p(w), _p(tau), nch, _p(y))
    return y


def ens_metrics(X, truth):
    """Metrics<double>::CalculateAll: (mean, spread, {rmse, bias, correlation,
    crps, avg_spread}) of members X (k x n)."""
    X = _f64(X)
    truth = _f64(truth)
    k, n = X.shape
    mean = np.empty(n)
    spread = np.empty(n)
    out = np.empty(5)
    load().orc_ens_metrics(_p(X), n, k, n, _p(truth), _p(mean), _p(spread), _p(out))
    return mean, spread, dict(zip(("rmse", "bias", "correlation", "crps", "avg_spread"), out.tolist()))


def nearest_node(node_lat, node_lon, nx, ny, obs_lat, obs_lon, vcoord=None, obs_level=None):
    node_lat, node_lon, obs_lat, obs_lon = map(_f64, (node_lat, node_lon, obs_lat, obs_lon))
    p = obs_lat.shape[0]
    xy = np.empty((p, 2), dtype=np.int32)
    kk = np.empty(p, dtype=np.int32) if vcoord is not None else None
    vc = _f64(vcoord) if vcoord is not None else None
    lev = _f64(obs_level) if obs_level is not None else None
    load().orc_nearest_node(_p(node_lat), _p(node_lon), nx, ny, _p(obs_lat), _p(obs_lon), p, _p(vc),
                            0 if vc is None else vc.shape[0], _p(lev), _p(xy), _p(kk))
    return xy, kk


def enkf(X, HX, yo, rvar, eps, rho):
    """Dense-form stochastic EnKF: (analysed members, analysis mean,
    {innovation_norm, background_spread, analysis_spread}, (max, min) gain)."""
    X = np.array(X, dtype=np.float64, order="C", copy=True)
    HX, yo, rvar, eps = _f64(HX), _f64(yo), _f64(rvar), _f64(eps)
    k, n = X.shape
    p = yo.shape[0]
    mean = np.empty(n)
    diag = np.empty(3)
    gain = np.empty(2)
    rc = load().orc_enkf(_p(X), n, k, n, _p(HX), _p(yo), _p(rvar), _p(eps), p, float(rho), _p(mean), _p(diag),
                         _p(gain))
    if rc != 0:
        raise RuntimeError("orc_enkf: S is singular")
    return X, mean, dict(zip(("innovation_norm", "background_spread", "analysis_spread"), diag.tolist())), \
        tuple(gain.tolist())


def num_threads() -> int:
    return load().orc_num_threads()


def parse_values(text: bytes) -> np.ndarray:
    """SimpleState::readFromFile: the doubles std::istringstream extracts from
    each line of the text."""
    lib = load()
    cap = max(1, text.count(b" ") + text.count(b"\n") + text.count(b"\t") + 1)
    out = np.empty(cap)
    n = lib.orc_parse_values(text, len(text), _p(out), cap)
    if n > cap:
        out = np.empty(n)
        n = lib.orc_parse_values(text, len(text), _p(out), n)
    return out[:n]
