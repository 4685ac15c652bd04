"""GPU test of mg_etkf_noalloc, the entry point for callers that cannot
allocate device memory while they run the analysis (a real-time loop whose
device memory is fixed at start-up, a framework that owns every device
allocation through its own pool).  Its output must match mg_etkf's, call after call: the
shared scratch array keeps the previous call's contents and must not leak
into the next result.  This file is collected last so that a failure here
stops a `-x` run only after every other test has run."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import GOLDEN, rel_err

from metada_gb300 import _lib
from metada_gb300 import kernels as K

pytestmark = pytest.mark.gpu

TOL = {_lib.MG_PREC_FP64: 1e-10, _lib.MG_PREC_MIXED: 1e-5}


def _noalloc(X, HX, yo, rvar, rho, flags, precision):
    lib = _lib.load()
    k, n = X.shape
    mean = torch.empty(n, dtype=torch.float64, device=X.device)
    stream = torch.cuda.current_stream(X.device).cuda_stream
    rc = lib.mg_etkf_noalloc(ctypes.c_void_p(stream), ctypes.c_void_p(X.data_ptr()), n, k, n,
                             ctypes.c_void_p(HX.data_ptr()), ctypes.c_void_p(yo.data_ptr()),
                             ctypes.c_void_p(rvar.data_ptr()), HX.shape[0], rho, flags, precision,
                             ctypes.c_void_p(mean.data_ptr()))
    return rc, mean


@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
@pytest.mark.parametrize("flags", [_lib.MG_COMPAT, 0])
def test_noalloc_matches_etkf_on_two_calls_in_a_row(dev, precision, flags):
    g = np.load(GOLDEN / "etkf_grid64.npz")
    X0 = torch.tensor(g["X"], device=dev)
    xy = torch.tensor(g["obs_xy"], device=dev)
    HX = K.hx_idw4(X0, 64, 64, xy)
    yo = torch.tensor(g["yo"], device=dev)
    rvar = torch.full_like(yo, float(g["sigma"]) ** 2)
    rho = float(g["rho"])
    Xref = X0.clone()
    mref = K.etkf(Xref, HX, yo, rvar, rho, flags=flags, precision=precision)
    for _ in range(2):  # two calls in a row share the static scratch
        X = X0.clone()
        rc, mean = _noalloc(X, HX, yo, rvar, rho, flags, precision)
        assert rc == _lib.MG_OK
        torch.cuda.synchronize()
        assert rel_err(X.cpu().numpy(), Xref.cpu().numpy()) <= TOL[precision]
        assert rel_err(mean.cpu().numpy(), mref.cpu().numpy()) <= TOL[precision]
    if flags == _lib.MG_COMPAT and precision == _lib.MG_PREC_FP64:
        assert rel_err(X.cpu().numpy(), g["members"]) <= TOL[precision]  # and the reference's own result


def test_noalloc_rejects_problems_beyond_its_scratch(dev):
    n, k, p = 200_000, 64, 1000  # n*k*8 alone is ~100 MB, above the 32 MiB array
    X = torch.zeros((k, n), dtype=torch.float64, device=dev)
    HX = torch.zeros((p, k), dtype=torch.float64, device=dev)
    yo = torch.zeros(p, dtype=torch.float64, device=dev)
    rvar = torch.ones(p, dtype=torch.float64, device=dev)
    rc, _ = _noalloc(X, HX, yo, rvar, 1.0, 0, _lib.MG_PREC_FP64)
    assert rc == _lib.MG_ERR_CAPACITY
