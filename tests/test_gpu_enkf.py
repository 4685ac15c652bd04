"""GPU: the stochastic EnKF (perturbed observations) in the k-dimensional
form against the oracle's dense p x p restatement of EnKF.hpp, for given
observation perturbations."""
import numpy as np
import pytest
import torch

from conftest import rel_err

import oracle.bind as ob
from metada_gb300 import _lib
from metada_gb300 import algorithms as A
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _case(k, p, seed):
    c = syn.global_etkf_grid(nx=48, ny=40, k=k, p=p, case=60 + seed)
    HX = ob.hx_idw4(c.X, 48, 40, c.obs_xy)
    z = np.random.default_rng(seed).standard_normal((p, k))
    eps = c.sigma_o * z
    return c, HX, eps


@pytest.mark.parametrize("k,p", [(9, 60), (32, 300), (64, 500), (100, 200)])
@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
def test_enkf_matches_dense_oracle(dev, k, p, precision):
    c, HX, eps = _case(k, p, k + p)
    rvar = c.rvar
    want, wmean, wdiag, _ = ob.enkf(c.X, HX, c.yo, rvar, eps, c.rho)
    X = torch.tensor(c.X, device=dev)
    mean, diag = K.enkf(X, torch.tensor(HX, device=dev), torch.tensor(c.yo, device=dev),
                        torch.tensor(rvar, device=dev), torch.tensor(eps, device=dev), c.rho, precision=precision)
    tol = 1e-10 if precision == _lib.MG_PREC_FP64 else 1e-5
    assert rel_err(X.cpu().numpy(), want) <= tol
    assert rel_err(mean.cpu().numpy(), wmean) <= tol
    for key in wdiag:
        assert abs(diag[key] - wdiag[key]) <= (1e-10 if precision == _lib.MG_PREC_FP64 else 1e-5) * wdiag[key], key


def test_enkf_mirror_reproducible_and_reduces_error(dev):
    c = syn.global_etkf_grid(nx=64, ny=64, k=32, p=1024, case=70)
    geom = A.SimpleGeometry(64, 64)
    out = []
    for _ in range(2):
        ens = A.Ensemble(c.X, geom, device=dev)
        obs = A.Observation(c.yo, c.sigma_o, grid_xy=c.obs_xy, device=dev)
        f = A.EnKF(ens, obs, A.ObsOperator(), {"inflation": 1.05, "seed": 3})
        f.Analyse()
        out.append((ens.X.cpu().numpy(), f.getAnalysisResults()))
    assert np.array_equal(out[0][0], out[1][0])  # seeded perturbations: identical analyses
    rb = np.sqrt(np.mean((c.X.mean(0) - c.truth) ** 2))
    ra = np.sqrt(np.mean((out[0][0].mean(0) - c.truth) ** 2))
    assert ra < rb
    r = out[0][1]
    assert r["analysis_spread"] < r["background_spread"]


@pytest.mark.parametrize("which", ["tut", "c1"])
def test_enkf_matches_reference_golden(dev, which):
    """The k-dimensional GPU EnKF against the reference's own EnKF.hpp
    (header harness, seeded generator; tests/golden/enkf.npz)."""
    from conftest import GOLDEN

    g = np.load(GOLDEN / "enkf.npz")
    X, xy, yo = g[f"{which}_X"], g[f"{which}_obs_xy"], g[f"{which}_yo"]
    nx, ny = (int(g["nx"]), int(g["ny"])) if which == "tut" else (int(g["c1_nx"]), int(g["c1_ny"]))
    s = float(g[f"{which}_sigma"])
    rho = 1.0 if which == "tut" else float(g["c1_rho"])
    Xd = torch.tensor(X, device=dev)
    HX = K.hx_idw4(Xd, nx, ny, torch.tensor(xy, device=dev))
    mean, diag = K.enkf(Xd, HX, torch.tensor(yo, device=dev), torch.full((len(yo),), s * s, dtype=torch.float64,
                                                                          device=dev),
                        torch.tensor(g[f"{which}_eps"], device=dev), rho)
    assert rel_err(Xd.cpu().numpy(), g[f"{which}_members"]) <= 1e-10
    assert rel_err(mean.cpu().numpy(), g[f"{which}_mean"]) <= 1e-10
    want = g[f"{which}_diag"]
    np.testing.assert_allclose([diag["innovation_norm"], diag["background_spread"], diag["analysis_spread"]],
                               want[:3], rtol=1e-10)
