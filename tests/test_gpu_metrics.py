"""GPU: ensemble diagnostics (Metrics<double>::CalculateAll) against the
reference's known answers and the oracle."""
import numpy as np
import pytest
import torch

import oracle.bind as ob
from metada_gb300 import algorithms as A
from metada_gb300 import kernels as K
from test_oracle import METRICS_MEMBERS, METRICS_TRUTH, METRICS_UNCORRELATED

pytestmark = pytest.mark.gpu


def _gpu(X, truth, dev):
    return K.ens_metrics(torch.tensor(X, device=dev), torch.tensor(truth, device=dev))


def test_metrics_known_answers(dev):
    mean, spread, m = _gpu(METRICS_MEMBERS, METRICS_TRUTH, dev)
    np.testing.assert_allclose(mean.cpu().numpy(), METRICS_TRUTH, atol=1e-6)
    np.testing.assert_allclose(spread.cpu().numpy(), 0.1, atol=1e-6)
    assert abs(m["crps"] - 0.022222222222222227) <= 1e-6
    assert abs(m["correlation"] - 1.0) <= 1e-6 and abs(m["bias"]) <= 1e-6 and abs(m["rmse"]) <= 1e-6
    assert abs(m["avg_spread"] - 0.1) <= 1e-6
    _, _, b = _gpu(METRICS_MEMBERS + 0.5, METRICS_TRUTH, dev)
    assert abs(b["bias"] - 0.5) <= 1e-6 and abs(b["rmse"] - 0.5) <= 1e-6
    _, _, u = _gpu(METRICS_UNCORRELATED, METRICS_TRUTH, dev)
    assert abs(u["correlation"] - 0.34105511573854358) <= 1e-6


@pytest.mark.parametrize("n,k", [(1, 2), (31, 3), (100_003, 64), (20_000, 100), (7_001, 200)])
def test_metrics_match_oracle(dev, n, k):
    g = np.random.default_rng(n + k)
    truth = g.standard_normal(n) * 3.0 + 1.0
    X = truth[None] + 0.7 * g.standard_normal((k, n)) + 0.2
    mean, spread, m = _gpu(X, truth, dev)
    wmean, wspread, wm = ob.ens_metrics(X, truth)
    # per element: the reference's operations in its order, bit for bit
    assert np.array_equal(mean.cpu().numpy(), wmean)
    assert np.array_equal(spread.cpu().numpy(), wspread)
    for key in ("rmse", "bias", "crps", "avg_spread"):
        assert abs(m[key] - wm[key]) <= 1e-12 * max(1.0, abs(wm[key])), key
    if n > 2:
        assert abs(m["correlation"] - wm["correlation"]) <= 1e-9


def test_metrics_python_mirror(dev):
    geom = A.SimpleGeometry(4, 1)
    ens = A.Ensemble(METRICS_MEMBERS, geom, device=dev)
    r = A.Metrics.CalculateAll(ens, METRICS_TRUTH, state_dim=4, ens_size=3)
    assert abs(r["crps"] - 0.022222222222222227) <= 1e-6
    np.testing.assert_allclose(r["spread"], 0.1, atol=1e-6)


def test_metrics_ties_and_shared_key_halves(dev):
    """Members on a coarse grid (many exact ties) and members a few ulp
    apart (same top 32 bits of the order key): the CRPS ranks take the exact
    recount, and the result still matches the pairwise sum."""
    g = np.random.default_rng(3)
    n, k = 4_099, 48
    truth = g.standard_normal(n)
    X = np.round(truth[None] + g.standard_normal((k, n)), 1)
    X[5:9] = X[4] + np.arange(1, 5)[:, None] * np.spacing(X[4])  # a few ulp above member 4
    mean, spread, m = _gpu(X, truth, dev)
    wmean, wspread, wm = ob.ens_metrics(X, truth)
    assert np.array_equal(mean.cpu().numpy(), wmean)
    assert np.array_equal(spread.cpu().numpy(), wspread)
    for key in ("rmse", "bias", "crps", "avg_spread"):
        assert abs(m[key] - wm[key]) <= 1e-12 * max(1.0, abs(wm[key])), key
