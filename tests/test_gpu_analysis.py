"""GPU parity of the analyses: global ETKF and LETKF (reference order and
batched), FP64 against the reference golden vectors and the oracle at
1e-10 relative, mixed precision at 1e-5 relative."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN, rel_err
from oracle.lists import point_lists

import oracle.bind as ob
from metada_gb300 import _lib
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-5


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


# ------------------------------------------------------------ global ETKF --
@pytest.mark.parametrize("name", ["tutorial", "etkf_grid64"])
def test_etkf_reference_semantics_match_golden(dev, name):
    g = np.load(GOLDEN / f"{name}.npz")
    if name == "tutorial":
        X, nx, ny, want, wmean, rho = g["X"], int(g["nx"]), int(g["ny"]), g["etkf_members"], g["etkf_mean"], 1.0
    else:
        X, nx, ny, want, wmean, rho = g["X"], 64, 64, g["members"], g["mean"], float(g["rho"])
    s = float(g["sigma"])
    Xd = T(X, dev)
    HX = K.hx_idw4(Xd, nx, ny, T(g["obs_xy"], dev))
    yo = T(g["yo"], dev)
    mean = K.etkf(Xd, HX, yo, torch.full_like(yo, s * s), rho, flags=_lib.MG_COMPAT, precision=_lib.MG_PREC_FP64)
    assert rel_err(Xd.cpu().numpy(), want) <= FP64_TOL
    assert np.array_equal(mean.cpu().numpy(), wmean)


def _global_oracle_hunt(X, HX, yo, rvar, rho, pts):
    p = HX.shape[0]
    npt = len(pts)
    off = np.arange(npt + 1, dtype=np.int64) * p
    idx = np.tile(np.arange(p, dtype=np.int32), npt)
    return ob.letkf_points(X, pts, 1, 0, HX, yo, rvar, off, idx, None, rho, 0)[:, 0, :].T


@pytest.mark.parametrize("k", [9, 32, 64, 100])
@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
def test_etkf_hunt_matches_oracle(dev, k, precision):
    c = syn.global_etkf_grid(48, 40, k, 700, case=21)
    Xd = T(c.X, dev)
    HX = K.hx_idw4(Xd, c.nx, c.ny, T(c.obs_xy, dev))
    yo = T(c.yo, dev)
    rvar = torch.full_like(yo, c.sigma_o ** 2)
    K.etkf(Xd, HX, yo, rvar, c.rho, flags=0, precision=precision)
    pts = np.random.default_rng(k).choice(c.nx * c.ny, 64, replace=False)
    want = _global_oracle_hunt(c.X, HX.cpu().numpy(), c.yo, c.rvar, c.rho, pts)
    got = Xd.cpu().numpy()[:, pts]
    tol = FP64_TOL if precision == _lib.MG_PREC_FP64 else MIXED_TOL
    assert rel_err(got, want) <= tol


def test_etkf_reference_semantics_mixed(dev):
    g = np.load(GOLDEN / "etkf_grid64.npz")
    Xd = T(g["X"], dev)
    HX = K.hx_idw4(Xd, 64, 64, T(g["obs_xy"], dev))
    yo = T(g["yo"], dev)
    K.etkf(Xd, HX, yo, torch.full_like(yo, float(g["sigma"]) ** 2), float(g["rho"]), flags=_lib.MG_COMPAT,
           precision=_lib.MG_PREC_MIXED)
    assert rel_err(Xd.cpu().numpy(), g["members"]) <= MIXED_TOL


# ----------------------------------------------------- reference-order LETKF --
@pytest.mark.parametrize("name,rho_key", [("tutorial", "rho"), ("tutorial", "rho11"), ("letkf_grid24", "rho"),
                                          ("letkf_grid20", "rho")])
def test_letkf_reference_order_matches_golden(dev, name, rho_key):
    g = np.load(GOLDEN / f"{name}.npz")
    if name == "tutorial":
        suffix = "letkf" if rho_key == "rho" else "letkf_rho11"
        want, wmean = g[f"{suffix}_members"], g[f"{suffix}_mean"]
    else:
        want, wmean = g["members"], g["mean"]
    Xd = T(g["X"], dev)
    mean = K.letkf_compat_grid(Xd, int(g["nx"]), int(g["ny"]), T(g["obs_xy"], dev), T(g["yo"], dev),
                               float(g["radius"]), float(g[rho_key]))
    assert rel_err(Xd.cpu().numpy(), want) <= FP64_TOL
    assert rel_err(mean.cpu().numpy(), wmean) <= FP64_TOL


# ------------------------------------------------------------ batched LETKF --
def _grid_batched(dev, g, rho, flags, precision):
    nx, ny = int(g["nx"]), int(g["ny"])
    X = g["X"]
    s = float(g["sigma"])
    Xd = T(X, dev)
    xy = T(g["obs_xy"], dev)
    HX = K.hx_idw4(Xd, nx, ny, xy)
    yo = T(g["yo"], dev)
    rvar = torch.full_like(yo, s * s)
    off, idx = K.select_grid(nx, ny, xy, float(g["radius"]))
    K.letkf_batched(Xd, col_base=torch.arange(nx * ny, dtype=torch.int64, device=dev), nlev=1, n_var=1,
                    lev_stride=0, var_stride=0, HX=HX, yo=yo, rvar=rvar, loc_off=off, loc_idx=idx, rho=rho,
                    flags=flags, precision=precision)
    offc, idxc = ob.select_grid(nx, ny, g["obs_xy"], float(g["radius"]))
    want = ob.letkf_points(X, np.arange(nx * ny), 1, 0, HX.cpu().numpy(), g["yo"], np.full(len(g["yo"]), s * s),
                           offc, idxc, None, rho, flags)[:, 0, :].T
    return Xd.cpu().numpy(), want


@pytest.mark.parametrize("name", ["tutorial", "letkf_grid24", "letkf_grid20"])
@pytest.mark.parametrize("flags", [_lib.MG_COMPAT, 0, _lib.MG_RTPS])
@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
def test_letkf_batched_grid_matches_oracle(dev, name, flags, precision):
    g = np.load(GOLDEN / f"{name}.npz")
    rho = 0.5 if flags == _lib.MG_RTPS else float(g["rho"]) if name != "tutorial" else 1.1
    got, want = _grid_batched(dev, g, rho, flags, precision)
    tol = FP64_TOL if precision == _lib.MG_PREC_FP64 else MIXED_TOL
    assert rel_err(got, want) <= tol


def _latlon_case(nlon, nlat, nlev, nvar, k, p, T_, case):
    return syn.latlon_letkf_case(nlon=nlon, nlat=nlat, nlev=nlev, nvar=nvar, k=k, p=p, T=T_, case=case)


def _run_latlon(dev, c, precision, flags=0, sample=None):
    Xd = T(c.X, dev)
    olat, olon, olev = T(c.obs_lat, dev), T(c.obs_lon, dev), T(c.obs_lev, dev)
    HX = K.hx_latlon(Xd, c.nlon, c.nlat, c.nlev, olat, olon, olev, T(c.obs_var, dev))
    clat, clon = c.col_lat_lon()
    off, idx, dist = K.select_geo(T(clat, dev), T(clon, dev), olat, olon, c.hsupport_km)
    yo = T(c.yo, dev)
    rvar = torch.full_like(yo, c.sigma_o ** 2)
    _, st = K.letkf_batched(Xd, col_base=T(c.col_base(), dev), nlev=c.nlev, n_var=c.nvar,
                            lev_stride=c.lev_stride, var_stride=c.var_stride, HX=HX, yo=yo, rvar=rvar,
                            loc_off=off, loc_idx=idx, loc_dist=dist, obs_lev=olev, hsupport=c.hsupport_km,
                            vsupport=c.vsupport, rho=c.rho, flags=flags, precision=precision, want_mean=False)
    return Xd, HX, off.cpu().numpy(), idx.cpu().numpy(), dist.cpu().numpy(), st


def _oracle_latlon(c, HX, off, idx, dist, cols, flags=0):
    pts, poff, pidx, pw = point_lists(cols, c.nlev, off, idx, dist, c.obs_lev, c.hsupport_km, c.vsupport,
                                      compat=bool(flags & ob.ORC_R_IDENTITY))
    base = c.col_base()[pts[:, 0]] + pts[:, 1] * c.lev_stride
    out = ob.letkf_points(c.X, base, c.nvar, c.var_stride, HX, c.yo, c.rvar, poff, pidx, pw, c.rho, flags)
    return base, out


@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
@pytest.mark.parametrize("k", [16, 64])
def test_letkf_latlon_small_matches_oracle(dev, precision, k):
    c = _latlon_case(72, 36, 5, 2, k, 20_000, 20, case=31)
    Xd, HX, off, idx, dist, st = _run_latlon(dev, c, precision)
    cols = np.arange(c.nlat * c.nlon)
    base, want = _oracle_latlon(c, HX.cpu().numpy(), off, idx, dist, cols)
    got = Xd.cpu().numpy()
    gv = np.stack([got[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)  # npt x nvar x k
    tol = FP64_TOL if precision == _lib.MG_PREC_FP64 else MIXED_TOL
    assert rel_err(gv, want) <= tol
    assert st.n_points == c.nlat * c.nlon * c.nlev
    assert st.total_local > 0 and st.max_local > 0


@pytest.mark.parametrize("precision", [_lib.MG_PREC_FP64, _lib.MG_PREC_MIXED])
def test_letkf_highres_shape_rtps_k80(dev, precision):
    """The high-resolution configuration's analysis at reduced size: k = 80
    (the k <= 96 kernels), 60 % of the obs in 20 Gaussian patches (strongly
    uneven local counts), 300 km support, RTPS with alpha = 0.9; against the
    oracle on a sample of columns."""
    c = syn.latlon_letkf_case(nlon=144, nlat=72, nlev=6, nvar=4, k=80, p=40_000, T=40, hsupport_km=300.0,
                              rho=0.9, case=33, clustered=0.6)
    Xd, HX, off, idx, dist, st = _run_latlon(dev, c, precision, flags=_lib.MG_RTPS)
    counts = np.diff(off)
    assert counts.max() > 8 * max(1.0, np.median(counts))  # the patches make the counts uneven
    cols = np.random.default_rng(3).choice(c.nlat * c.nlon, 300, replace=False)
    base, want = _oracle_latlon(c, HX.cpu().numpy(), off, idx, dist, cols, flags=ob.ORC_RTPS)
    got = Xd.cpu().numpy()
    gv = np.stack([got[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)
    tol = FP64_TOL if precision == _lib.MG_PREC_FP64 else MIXED_TOL
    assert rel_err(gv, want) <= tol


@pytest.mark.parametrize("k", [2, 33, 47])
def test_letkf_mixed_odd_member_counts(dev, k):
    """Member counts that pad the k x k system (odd k) or leave lanes idle."""
    c = _latlon_case(72, 36, 4, 2, k, 15_000, 20, case=34)
    Xd, HX, off, idx, dist, st = _run_latlon(dev, c, _lib.MG_PREC_MIXED)
    cols = np.arange(c.nlat * c.nlon)
    base, want = _oracle_latlon(c, HX.cpu().numpy(), off, idx, dist, cols)
    got = Xd.cpu().numpy()
    gv = np.stack([got[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)
    assert rel_err(gv, want) <= MIXED_TOL


@pytest.mark.slow
def test_letkf_latlon_full_size_sampled(dev):
    """The 360 x 180 x 10 x 4, 64-member, 500k-obs configuration, on the
    benchmarked inputs:
    * local selection (LETKF.hpp:159-165 with Location.hpp:349-357) of 240
      sampled columns against the oracle's own search over all 500k obs:
      lists and counts bit-exact, distances to 1e-13;
    * H(X) rows of every obs in those lists against the oracle's operator:
      bit-exact;
    * the FP64 analysis of those columns against the oracle run on its own
      lists and H(X) (nothing of the GPU's fed in) at 1e-10;
    * mixed against FP64 everywhere at 1e-5."""
    c = syn.latlon_letkf_case()
    X64, HX, off, idx, dist, st64 = _run_latlon(dev, c, _lib.MG_PREC_FP64)
    cols = np.sort(np.random.default_rng(7).choice(c.nlat * c.nlon, 240, replace=False))
    clat, clon = c.col_lat_lon()
    offc, idxc, distc = ob.select_geo(clat[cols], clon[cols], c.obs_lat, c.obs_lon, c.hsupport_km)
    for j, col in enumerate(cols):
        e0, e1 = int(off[col]), int(off[col + 1])
        assert e1 - e0 == int(offc[j + 1] - offc[j]), f"column {col}: count differs"
        assert np.array_equal(idx[e0:e1], idxc[offc[j]:offc[j + 1]]), f"column {col}: list differs"
        # distances come from device sin/cos/asin: equal to the host expression to rounding
        np.testing.assert_allclose(dist[e0:e1], distc[offc[j]:offc[j + 1]], rtol=1e-13, atol=1e-9)
    assert offc[-1] > 100 * len(cols)  # the sample holds a realistic share of the lists
    need = np.unique(idxc)
    HXc = ob.hx_latlon(c.X, c.nlon, c.nlat, c.nlev, c.obs_lat[need], c.obs_lon[need], c.obs_lev[need],
                       c.obs_var[need])
    assert np.array_equal(HX.cpu().numpy()[need], HXc)
    # oracle analysis of the sampled columns from its own lists and H(X)
    HXo = np.zeros((c.yo.size, HXc.shape[1]))
    HXo[need] = HXc
    offo = np.zeros(c.nlat * c.nlon + 1, dtype=np.int64)
    offo[cols + 1] = np.diff(offc)
    offo = np.cumsum(offo)
    base, want = _oracle_latlon(c, HXo, offo, idxc, distc, cols)
    a64 = X64.cpu().numpy()
    del X64
    gv = np.stack([a64[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)
    assert rel_err(gv, want) <= FP64_TOL
    Xmx, _, _, _, _, stmx = _run_latlon(dev, c, _lib.MG_PREC_MIXED)
    amx = Xmx.cpu().numpy()
    del Xmx
    # mean and perturbation errors of the mixed path against FP64
    m64, mmx = a64.mean(0), amx.mean(0)
    assert rel_err(mmx, m64) <= MIXED_TOL
    assert rel_err(amx - mmx, a64 - m64) <= MIXED_TOL
    # every analysis point of the configuration has local observations
    assert st64.n_points == c.nlat * c.nlon * c.nlev and st64.n_empty == stmx.n_empty == 0


def test_letkf_latlon_warm_start_fp64_matches_oracle(dev):
    """Levels of a column in sequence, each Jacobi warm-started from the
    previous level's eigenvectors: same analysis to 1e-10."""
    c = _latlon_case(72, 36, 5, 2, 32, 20_000, 20, case=32)
    Xd, HX, off, idx, dist, st = _run_latlon(dev, c, _lib.MG_PREC_FP64, flags=_lib.MG_WARM_START)
    base, want = _oracle_latlon(c, HX.cpu().numpy(), off, idx, dist, np.arange(c.nlat * c.nlon))
    got = Xd.cpu().numpy()
    gv = np.stack([got[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)
    assert rel_err(gv, want) <= FP64_TOL
