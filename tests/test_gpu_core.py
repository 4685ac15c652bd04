"""GPU parity: ensemble mean/perturbations, observation operators and local
observation search, bit-exact against the oracle and the golden vectors."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN

import oracle.bind as ob
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("k,n", [(1, 5), (9, 648), (32, 4096), (64, 100_003), (100, 777)])
def test_mean_and_perturbations_bit_exact(dev, k, n):
    X = np.random.default_rng(k * 7 + n).standard_normal((k, n)) * 300.0
    mean = K.ens_mean(T(X, dev)).cpu().numpy()
    assert np.array_equal(mean, ob.ens_mean(X))
    m2, Xp = K.ens_mean_pert(T(X, dev))
    wm, wXp = ob.ens_mean_pert(X)
    assert np.array_equal(m2.cpu().numpy(), wm) and np.array_equal(Xp.cpu().numpy(), wXp)


def test_mean_matches_reference_golden(dev):
    g = np.load(GOLDEN / "etkf_grid64.npz")
    assert np.array_equal(K.ens_mean(T(g["X"], dev)).cpu().numpy(), g["mean"])


@pytest.mark.parametrize("case", ["tutorial", "grid64", "edges"])
def test_idw4_bit_exact(dev, case):
    if case == "tutorial":
        g = np.load(GOLDEN / "tutorial.npz")
        X, nx, ny, xy, valid = g["X"], int(g["nx"]), int(g["ny"]), g["obs_xy"], None
    elif case == "grid64":
        g = np.load(GOLDEN / "etkf_grid64.npz")
        X, nx, ny, xy, valid = g["X"], 64, 64, g["obs_xy"], None
    else:
        r = np.random.default_rng(1)
        nx, ny, p = 13, 7, 500
        X = r.standard_normal((5, nx * ny))
        xy = np.stack([r.integers(-3, nx + 3, p), r.integers(-3, ny + 3, p)], 1).astype(np.int32)
        valid = (r.uniform(size=p) > 0.1).astype(np.uint8)
    HX = K.hx_idw4(T(X, dev), nx, ny, T(xy, dev), None if valid is None else T(valid, dev)).cpu().numpy()
    assert np.array_equal(HX, ob.hx_idw4(X, nx, ny, xy, valid))


def test_latlon_operator_bit_exact(dev):
    r = np.random.default_rng(2)
    nlon, nlat, nlev, nvar, k, p = 36, 18, 4, 3, 6, 20_000
    X = r.standard_normal((k, nvar * nlev * nlat * nlon))
    lat = np.concatenate([np.rad2deg(np.arcsin(r.uniform(-1, 1, p - 6))), [90.0, -90.0, 89.99, -89.99, 0.0, 0.0]])
    lon = np.concatenate([r.uniform(-30, 400, p - 6), [0.0, 359.999, 180.0, 0.0, 359.5, 0.5]])
    lev = np.concatenate([r.uniform(-0.5, nlev - 0.5, p - 6), [0.0, 3.0, 2.5, 1.0, 0.0, 3.0]])
    var = r.integers(0, nvar, p).astype(np.int32)
    HX = K.hx_latlon(T(X, dev), nlon, nlat, nlev, T(lat, dev), T(lon, dev), T(lev, dev), T(var, dev)).cpu().numpy()
    want = ob.hx_latlon(X, nlon, nlat, nlev, lat, lon, lev, var)
    assert np.array_equal(HX, want)
    # and the synthetic generator's numpy restatement agrees to rounding
    np.testing.assert_allclose(HX[:, 0], syn.trilinear_h(X[0], nlon, nlat, nlev, lat, lon, lev, var), rtol=0,
                               atol=1e-12)


@pytest.mark.parametrize("case", ["tutorial", "letkf_grid24", "letkf_grid20", "random"])
def test_select_grid_bit_exact(dev, case):
    if case == "random":
        r = np.random.default_rng(3)
        nx, ny, p = 64, 48, 2000
        xy = np.stack([r.integers(-5, nx + 5, p), r.integers(-5, ny + 5, p)], 1).astype(np.int32)
        radius = syn.float_config(6.5)
    else:
        g = np.load(GOLDEN / f"{case}.npz")
        nx, ny, xy, radius = int(g["nx"]), int(g["ny"]), g["obs_xy"], float(g["radius"])
    off, idx = K.select_grid(nx, ny, T(xy, dev), radius)
    woff, widx = ob.select_grid(nx, ny, xy, radius)
    assert np.array_equal(off.cpu().numpy(), woff)
    assert np.array_equal(idx.cpu().numpy(), widx)


def test_select_grid_no_obs(dev):
    xy = torch.zeros((0, 2), dtype=torch.int32, device=dev)
    off, idx = K.select_grid(5, 4, xy, 3.0)
    assert idx.numel() == 0 and int(off[-1]) == 0


@pytest.mark.parametrize("radius", [500.0, 1234.5])
def test_select_geo_bit_exact(dev, radius):
    r = np.random.default_rng(4)
    p = 40_000
    olat = np.rad2deg(np.arcsin(r.uniform(-1, 1, p)))
    olon = r.uniform(0, 360, p)
    # a few obs exactly at the poles and on the date line
    olat[:4] = [90.0, -90.0, 45.0, -45.0]
    olon[:4] = [0.0, 123.0, 0.0, 360.0]
    la = -89.0 + 2.0 * np.arange(90)
    lo = 1.0 + 2.0 * np.arange(180)
    clat, clon = (a.reshape(-1).copy() for a in np.meshgrid(la, lo, indexing="ij"))
    off, idx, dist = K.select_geo(T(clat, dev), T(clon, dev), T(olat, dev), T(olon, dev), radius)
    woff, widx, wdist = ob.select_geo(clat, clon, olat, olon, radius)
    assert np.array_equal(off.cpu().numpy(), woff)
    assert np.array_equal(idx.cpu().numpy(), widx)
    np.testing.assert_allclose(dist.cpu().numpy(), wdist, rtol=1e-13, atol=1e-9)


def test_select_geo_threshold_pairs_decided_by_reference_expression(dev):
    """Obs placed at (numerically) exactly the radius from a column."""
    clat = np.array([10.0, -33.0])
    clon = np.array([20.0, 200.0])
    radius = 500.0
    # points due north at exactly radius / R radians, plus tiny offsets either side
    dlat = np.rad2deg(radius / 6371.0)
    olat = np.array([10.0 + dlat, 10.0 + dlat * (1 + 1e-13), 10.0 + dlat * (1 - 1e-13), -33.0 - dlat])
    olon = np.array([20.0, 20.0, 20.0, 200.0])
    off, idx, _ = K.select_geo(T(clat, dev), T(clon, dev), T(olat, dev), T(olon, dev), radius)
    woff, widx, _ = ob.select_geo(clat, clon, olat, olon, radius)
    assert np.array_equal(off.cpu().numpy(), woff)
    assert np.array_equal(idx.cpu().numpy(), widx)
