"""GPU: the uneven batch of global ETKF analyses (many cases of different
sizes in one pass, CUDA-graph replay, autotuned chunking) against the
single-case path and the oracle."""
import numpy as np
import pytest
import torch

from conftest import rel_err

import oracle.bind as ob
from metada_gb300 import _lib
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _device_cases(cases, dev, with_hx=False):
    out = []
    for c in cases:
        X = torch.tensor(c.X, device=dev)
        d = {"X": X, "yo": torch.tensor(c.yo, device=dev),
             "rvar": torch.full((len(c.yo),), c.sigma_o ** 2, dtype=torch.float64, device=dev), "rho": c.rho}
        if with_hx:
            d["HX"] = X[:, torch.tensor(c.obs_node, device=dev)].T.contiguous()
        else:
            d["obs_node"] = torch.tensor(c.obs_node, device=dev)
        out.append(d)
    return out


@pytest.fixture(scope="module")
def cases():
    return syn.uneven_batch(ncases=40, n_range=(1_000, 20_000), p_range=(100, 5_000), case=55)


@pytest.mark.parametrize("flags", [_lib.MG_COMPAT, 0])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_fp64_matches_single_case_path(dev, cases, flags, graph):
    dc = _device_cases(cases, dev)
    ref = []
    for c in dc:  # single-case mg_etkf on a copy, HX by the same gather
        X = c["X"].clone()
        HX = X[:, c["obs_node"]].T.contiguous()
        K.etkf(X, HX, c["yo"], c["rvar"], c["rho"], flags=flags, precision=_lib.MG_PREC_FP64)
        ref.append(X.cpu().numpy())
    b = K.EtkfBatch(dc, flags=flags, precision=_lib.MG_PREC_FP64)
    b.run(graph=graph)
    ms = b.finish()
    for c, r in zip(dc, ref):
        assert rel_err(c["X"].cpu().numpy(), r) <= 1e-10
    assert np.all(ms > 0)


def test_batch_reference_semantics_match_oracle(dev, cases):
    sub = cases[:6]
    dc = _device_cases(sub, dev, with_hx=True)
    b = K.EtkfBatch(dc, flags=_lib.MG_COMPAT, precision=_lib.MG_PREC_FP64)
    b.run(graph=False)
    b.finish()
    for c, d in zip(sub, dc):
        HX = c.X[:, c.obs_node].T.copy()
        want, _ = ob.etkf_compat(c.X, HX, c.yo, np.full(len(c.yo), c.sigma_o ** 2), c.rho)
        assert rel_err(d["X"].cpu().numpy(), want) <= 1e-10


def test_batch_mixed_within_tolerance_and_graph_replays(dev, cases):
    d64 = _device_cases(cases, dev)
    b64 = K.EtkfBatch(d64, flags=0, precision=_lib.MG_PREC_FP64)
    b64.run(graph=False)
    b64.finish()
    dmx = _device_cases(cases, dev)
    X0 = [c["X"].clone() for c in dmx]
    bmx = K.EtkfBatch(dmx, flags=0, precision=_lib.MG_PREC_MIXED)
    chunk, mode = bmx.autotune()
    assert chunk in (128, 256, 512, 1024, 2048) and mode in (0, 1, 2)
    for rep in range(2):  # replay the captured graph twice from the same background
        for c, x0 in zip(dmx, X0):
            c["X"].copy_(x0)
        bmx.run(graph=True)
        bmx.finish()
        for c, r in zip(dmx, d64):
            a, w = c["X"].cpu().numpy(), r["X"].cpu().numpy()
            ma, mw = a.mean(0), w.mean(0)
            assert rel_err(ma, mw) <= 1e-5
            assert rel_err(a - ma, w - mw) <= 1e-5


def test_batch_mixed_large_offset_values(dev):
    """Members and obs around 280 with unit spread (temperatures in K): the
    mixed path's FP32 perturbations must keep 1e-5 of the spread, which
    rounding the FP64 values to FP32 alone would not."""
    sub = syn.uneven_batch(ncases=12, n_range=(2_000, 30_000), p_range=(200, 4_000), case=91)
    for c in sub:
        c.X += 280.0
        c.yo += 280.0
    d64 = _device_cases(sub, dev)
    b64 = K.EtkfBatch(d64, flags=0, precision=_lib.MG_PREC_FP64)
    b64.run(graph=False)
    b64.finish()
    dmx = _device_cases(sub, dev)
    bmx = K.EtkfBatch(dmx, flags=0, precision=_lib.MG_PREC_MIXED)
    bmx.run(graph=False)
    bmx.finish()
    for c, r in zip(dmx, d64):
        a, w = c["X"].cpu().numpy(), r["X"].cpu().numpy()
        ma, mw = a.mean(0), w.mean(0)
        assert rel_err(ma, mw) <= 1e-5
        assert rel_err(a - ma, w - mw) <= 1e-5


def test_batch_at_the_configuration_extremes(dev):
    """Cases at the uneven-batch configuration's limits: n up to 200k, p up
    to 50k (more obs than states in one case), k from 20 to 100.  FP64
    batch against the single-case path at 1e-10, mixed against FP64 at
    1e-5, and the oracle on the smallest case."""
    g = np.random.default_rng(20261203 + 500 + 7)
    shapes = [(200_000, 100, 50_000), (180_000, 64, 40_000), (1_000, 20, 100), (40_000, 48, 50_000),
              (200_000, 32, 100), (5_000, 100, 30_000)]
    cases = []
    for n, k, p in shapes:
        truth = g.standard_normal(n).astype(np.float32)
        X = (truth[None, :] + g.standard_normal((k, n)).astype(np.float32)).astype(np.float64)
        nodes = g.choice(n, size=p, replace=p > n).astype(np.int64)
        yo = truth[nodes].astype(np.float64) + g.standard_normal(p)
        cases.append(syn.UnevenCase(X, nodes, yo, 1.0, syn.float_config(1.05)))
    d64 = _device_cases(cases, dev)
    ref = []
    for c in d64:
        X = c["X"].clone()
        K.etkf(X, X[:, c["obs_node"]].T.contiguous(), c["yo"], c["rvar"], c["rho"], flags=0,
               precision=_lib.MG_PREC_FP64)
        ref.append(X.cpu().numpy())
    b64 = K.EtkfBatch(d64, flags=0, precision=_lib.MG_PREC_FP64)
    b64.run(graph=True)
    b64.finish()
    for c, r in zip(d64, ref):
        assert rel_err(c["X"].cpu().numpy(), r) <= 1e-10
    dmx = _device_cases(cases, dev)
    bmx = K.EtkfBatch(dmx, flags=0, precision=_lib.MG_PREC_MIXED)
    bmx.autotune()
    bmx.run(graph=True)
    bmx.finish()
    for c, r in zip(dmx, d64):
        a, w = c["X"].cpu().numpy(), r["X"].cpu().numpy()
        ma, mw = a.mean(0), w.mean(0)
        assert rel_err(ma, mw) <= 1e-5
        assert rel_err(a - ma, w - mw) <= 1e-5
    c = cases[2]
    pts = np.arange(c.X.shape[1])
    HX = c.X[:, c.obs_node].T.copy()
    p = len(c.yo)
    want = ob.letkf_points(c.X, pts, 1, 0, HX, c.yo, np.full(p, 1.0), np.arange(len(pts) + 1, dtype=np.int64) * p,
                           np.tile(np.arange(p, dtype=np.int32), len(pts)), None, c.rho, 0)[:, 0, :].T
    assert rel_err(d64[2]["X"].cpu().numpy(), want) <= 1e-10
