"""ctypes binding of the C-ABI declared in include/metada_gb300.h.

Loading fails loudly when the CUDA library has not been built: there is no
CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, Structure, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p

from .build import LIB_PATH

MG_OK = 0
MG_ERR_ARG = 1
MG_ERR_CUDA = 2
MG_ERR_NOMEM = 3
MG_ERR_NUMERIC = 4
MG_ERR_TIMEOUT = 5
MG_ERR_CAPACITY = 6

MG_R_IDENTITY = 1
MG_SQRT_CHOLESKY = 2
MG_INFL_COMPAT = 4
MG_UPDATE_COMPAT = 8
MG_COMPAT = 15
MG_RTPS = 16
MG_WARM_START = 32
MG_SOLVE_SIMT = 64

MG_PREC_FP64 = 0
MG_PREC_MIXED = 1

MG_DTYPE_F64 = 0
MG_DTYPE_F32 = 1

_ERR_NAMES = {
    MG_ERR_ARG: "invalid argument",
    MG_ERR_CUDA: "CUDA error",
    MG_ERR_NOMEM: "out of device memory",
    MG_ERR_NUMERIC: "numerical failure",
    MG_ERR_TIMEOUT: "device wait timed out",
    MG_ERR_CAPACITY: "buffer too small",
}


class MgError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERR_NAMES.get(code, 'error')} ({code}): {message}")
        self.code = code


class LetkfDesc(Structure):
    _fields_ = [
        ("X", c_void_p),
        ("n", c_int64),
        ("ld", c_int64),
        ("k", c_int32),
        ("n_var", c_int32),
        ("nlev", c_int32),
        ("precision", c_int32),
        ("ncol", c_int64),
        ("col_base", c_void_p),
        ("lev_stride", c_int64),
        ("var_stride", c_int64),
        ("p", c_int64),
        ("HX", c_void_p),
        ("yo", c_void_p),
        ("rvar", c_void_p),
        ("obs_lev", c_void_p),
        ("loc_off", c_void_p),
        ("loc_idx", c_void_p),
        ("loc_dist", c_void_p),
        ("hsupport", c_double),
        ("vsupport", c_double),
        ("rho", c_double),
        ("flags", c_int32),
        ("x_dtype", c_int32),
        ("mean_out", c_void_p),
    ]


class EtkfCase(Structure):
    _fields_ = [
        ("X", c_void_p),
        ("n", c_int64),
        ("ld", c_int64),
        ("k", c_int32),
        ("reserved", c_int32),
        ("HX", c_void_p),
        ("obs_node", c_void_p),
        ("yo", c_void_p),
        ("rvar", c_void_p),
        ("p", c_int64),
        ("rho", c_double),
        ("mean_out", c_void_p),
    ]


class LetkfStats(Structure):
    _fields_ = [
        ("n_points", c_int64),
        ("n_empty", c_int64),
        ("total_local", c_int64),
        ("max_local", c_int32),
        ("max_sweeps", c_int32),
        ("ms_prepare", c_double),
        ("ms_analysis", c_double),
        ("ms_writeback", c_double),
        ("total_sweeps", c_int64),
        ("n_fallback", c_int64),
        ("max_residual", c_double),
        ("tensor_path", c_int32),
        ("tensor_ctas", c_int32),
    ]


class EnkfDiag(Structure):
    """mg_enkf_diag."""
    _fields_ = [("innovation_norm", c_double), ("background_spread", c_double), ("analysis_spread", c_double)]


class EnsMetrics(Structure):
    """mg_ens_metrics_t."""
    _fields_ = [("rmse", c_double), ("bias", c_double), ("correlation", c_double), ("crps", c_double),
                ("avg_spread", c_double)]


# name -> argtypes (every function returns int unless listed in _RESTYPES)
_SIGNATURES = {
    "mg_create": [POINTER(c_void_p), c_int],
    "mg_destroy": [c_void_p],
    "mg_set_stream": [c_void_p, c_void_p],
    "mg_synchronize": [c_void_p],
    "mg_last_error": [c_void_p],
    "mg_version": [],
    "mg_ens_mean": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p],
    "mg_ens_mean_pert": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p, c_void_p, c_int64],
    "mg_hx_idw4": [c_void_p, c_void_p, c_int32, c_int64, c_int32, c_int32, c_void_p, c_void_p, c_int64,
                   c_void_p],
    "mg_hx_latlon": [c_void_p, c_void_p, c_int32, c_int64, c_int32, c_int32, c_int32, c_void_p, c_void_p,
                     c_void_p, c_void_p, c_int64, c_void_p],
    "mg_hx_latlon_f32": [c_void_p, c_void_p, c_int32, c_int64, c_int32, c_int32, c_int32, c_void_p, c_void_p,
                         c_void_p, c_void_p, c_int64, c_void_p],
    "mg_select_grid": [c_void_p, c_int32, c_int32, c_void_p, c_int64, c_double, c_void_p, c_void_p, c_int64,
                       POINTER(c_int64)],
    "mg_select_geo": [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_double, c_void_p,
                      c_void_p, c_void_p, c_int64, POINTER(c_int64)],
    "mg_etkf": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_double,
                c_int32, c_int32, c_void_p],
    "mg_letkf_compat_grid": [c_void_p, c_void_p, c_int32, c_int64, c_int32, c_int32, c_void_p, c_void_p,
                             c_void_p, c_int64, c_double, c_double, c_void_p],
    "mg_letkf_batched": [c_void_p, POINTER(LetkfDesc)],
    "mg_letkf_last_stats": [c_void_p, POINTER(LetkfStats)],
    "mg_kernel_launches": [c_void_p],
    "mg_vec_update": [c_void_p, c_void_p, c_void_p, c_int64, c_int32],
    "mg_vec_scale": [c_void_p, c_void_p, c_int64, c_double],
    "mg_vec_dot": [c_void_p, c_void_p, c_void_p, c_int64, POINTER(c_double)],
    "mg_etkf_batch_create": [c_void_p, c_void_p, c_int32, c_int32, c_int32, POINTER(c_void_p)],
    "mg_etkf_batch_autotune": [c_void_p, c_void_p, POINTER(c_int32), POINTER(c_int32)],
    "mg_etkf_batch_run": [c_void_p, c_void_p],
    "mg_etkf_batch_launch_graph": [c_void_p, c_void_p],
    "mg_etkf_batch_finish": [c_void_p, c_void_p, c_void_p],
    "mg_etkf_batch_destroy": [c_void_p],
    "mg_column_op": [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_int32, c_void_p],
    "mg_column_features": [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p],
    "mg_hx_column": [c_void_p, c_void_p, c_int32, c_int64, c_int64, c_int32, c_void_p, c_void_p, c_int64, c_void_p,
                     c_void_p, c_int32, c_void_p],
    "mg_mlp_create": [c_void_p, c_int32, c_int32, c_int32, POINTER(c_void_p)],
    "mg_mlp_destroy": [c_void_p],
    "mg_mlp_num_params": [c_void_p],
    "mg_mlp_set_params": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "mg_mlp_get_params": [c_void_p, c_void_p, c_void_p, c_int32],
    "mg_mlp_forward": [c_void_p, c_void_p, c_void_p, c_int64, c_void_p],
    "mg_mlp_gradients": [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, POINTER(ctypes.c_float)],
    "mg_mlp_train_step": [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, ctypes.c_float, POINTER(ctypes.c_float)],
    "mg_hx_column_mlp": [c_void_p, c_void_p, c_void_p, c_int32, c_int64, c_int64, c_int32, c_void_p, c_void_p, c_int64,
                         c_void_p],
    "mg_parse_grid_obs": [c_void_p, c_char_p, c_int64, c_double, c_void_p, c_void_p, c_int64, POINTER(c_int64)],
    "mg_parse_values": [c_void_p, c_char_p, c_int64, c_void_p, c_int64, POINTER(c_int64)],
    "mg_format_state": [c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_int64, POINTER(c_int64)],
    "mg_last_io_host_items": [c_void_p, POINTER(c_int64)],
    "mg_nearest_node": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_int64, c_void_p,
                        c_int32, c_void_p, c_void_p, c_void_p],
    "mg_enkf": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_int64,
                c_double, c_int32, c_void_p, POINTER(EnkfDiag)],
    "mg_ens_metrics": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p, c_void_p, c_void_p,
                       POINTER(EnsMetrics)],
    "mg_gemm_bf16_tc": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_int32, c_void_p],
    "mg_gemm_bf16_tc_wait_selftest": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p],
    "mg_etkf_noalloc": [c_void_p, c_void_p, c_int64, c_int32, c_int64, c_void_p, c_void_p, c_void_p, c_int64,
                        c_double, c_int32, c_int32, c_void_p],
}
_RESTYPES = {"mg_destroy": None, "mg_etkf_batch_destroy": None, "mg_mlp_destroy": None,
             "mg_mlp_num_params": c_int64, "mg_last_error": c_char_p, "mg_version": c_char_p, "mg_kernel_launches": c_int64}

# Entry points the header declares; the CPU tests check every one is exported.
EXPORTED = tuple(_SIGNATURES)

_lib = None


def load() -> ctypes.CDLL:
    """Load libmetada_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(there is no CPU fallback)"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, c_int)
    _lib = lib
    return lib


class Context:
    """Owns one mg_context (device, stream binding, workspace)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        h = c_void_p()
        rc = self.lib.mg_create(ctypes.byref(h), device)
        if rc != MG_OK:
            raise MgError(rc, f"mg_create(device={device}) failed")
        self.handle = h
        if stream is not None:
            self.set_stream(stream)

    def set_stream(self, stream: int) -> None:
        self.check(self.lib.mg_set_stream(self.handle, c_void_p(stream)))

    def check(self, rc: int) -> None:
        if rc != MG_OK:
            msg = self.lib.mg_last_error(self.handle)
            raise MgError(rc, msg.decode() if msg else "")

    def call(self, name: str, *args) -> None:
        self.check(getattr(self.lib, name)(self.handle, *args))

    def launches(self) -> int:
        return int(self.lib.mg_kernel_launches(self.handle))

    def synchronize(self) -> None:
        self.check(self.lib.mg_synchronize(self.handle))

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.mg_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass
