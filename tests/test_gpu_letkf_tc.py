"""GPU parity of the tensor-core local analyses (mixed precision, Hunt
transform, k <= 96; two kernel layouts, k <= 64 and 64 < k <= 96): the Gram, the Newton-Schulz inverse square root and the
update X' W on tcgen05 kind::tf32 with 3-pass products.  Each case checks that
the tensor-core kernel ran (stats.tensor_path), compares it with the oracle
(FP64, Jacobi eigen-solve) at 1e-5 relative, and with the SIMT Jacobi path."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle.lists import point_lists

import oracle.bind as ob
from metada_gb300 import _lib
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _run(dev, c, flags=0):
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
                            vsupport=c.vsupport, rho=c.rho, flags=flags, precision=_lib.MG_PREC_MIXED,
                            want_mean=False)
    return Xd.cpu().numpy(), HX.cpu().numpy(), off.cpu().numpy(), idx.cpu().numpy(), dist.cpu().numpy(), st


def _oracle(c, HX, off, idx, dist, cols, flags):
    pts, poff, pidx, pw = point_lists(cols, c.nlev, off, idx, dist, c.obs_lev, c.hsupport_km, c.vsupport,
                                      compat=bool(flags & ob.ORC_R_IDENTITY))
    base = c.col_base()[pts[:, 0]] + pts[:, 1] * c.lev_stride
    return base, ob.letkf_points(c.X, base, c.nvar, c.var_stride, HX, c.yo, c.rvar, poff, pidx, pw, c.rho, flags)


def _gather(X, c, base):
    return np.stack([X[:, base + v * c.var_stride].T for v in range(c.nvar)], axis=1)


@pytest.mark.parametrize("k", [4, 9, 16, 33, 47, 64, 65, 80, 96])
def test_tensor_path_matches_oracle_and_simt(dev, k):
    c = syn.latlon_letkf_case(nlon=72, nlat=36, nlev=5, nvar=2, k=k, p=20_000, T=20, case=41)
    got, HX, off, idx, dist, st = _run(dev, c)
    assert st.tensor_path == 1 and st.tensor_ctas >= torch.cuda.get_device_properties(dev).multi_processor_count
    assert st.n_fallback <= st.n_points // 1000 and 0.0 < st.max_residual < 5e-3
    assert st.total_sweeps > 0 and st.max_sweeps <= 14
    cols = np.arange(c.nlat * c.nlon)
    base, want = _oracle(c, HX, off, idx, dist, cols, 0)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL
    simt, _, _, _, _, st2 = _run(dev, c, flags=_lib.MG_SOLVE_SIMT)
    assert st2.tensor_path == 0
    assert rel_err(got, simt) <= MIXED_TOL


@pytest.mark.parametrize("k", [32, 80])
@pytest.mark.parametrize("flags", [_lib.MG_RTPS, _lib.MG_INFL_COMPAT, _lib.MG_R_IDENTITY])
def test_tensor_path_semantics_flags(dev, flags, k):
    """RTPS relaxation, the reference's inflation placement (Pa *= rho) and
    R = I on the tensor-core path (both layouts), against the oracle."""
    c = syn.latlon_letkf_case(nlon=72, nlat=36, nlev=4, nvar=3, k=k, p=15_000, T=20, case=42,
                              rho=0.8 if flags == _lib.MG_RTPS else 1.05)
    got, HX, off, idx, dist, st = _run(dev, c, flags)
    assert st.tensor_path == 1
    base, want = _oracle(c, HX, off, idx, dist, np.arange(c.nlat * c.nlon), flags)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL


@pytest.mark.parametrize("k", [24, 72])
def test_tensor_path_many_variables_per_point(dev, k):
    """More variables per analysis point than one update tile (16) holds,
    and more than the four whose update rows are prefetched."""
    c = syn.latlon_letkf_case(nlon=48, nlat=24, nlev=2, nvar=37, k=k, p=6_000, T=12, case=43)
    got, HX, off, idx, dist, st = _run(dev, c)
    assert st.tensor_path == 1
    cols = np.random.default_rng(0).choice(c.nlat * c.nlon, 200, replace=False)
    base, want = _oracle(c, HX, off, idx, dist, cols, 0)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL


@pytest.mark.parametrize("k", [64, 80])
def test_tensor_path_uneven_clustered_lists(dev, k):
    """Clustered obs: lists from a handful to thousands of candidates per
    column, so the Gram runs from one to many chunks (both kernel layouts)."""
    c = syn.latlon_letkf_case(nlon=120, nlat=60, nlev=4, nvar=2, k=k, p=60_000, T=30, hsupport_km=600.0,
                              case=44, clustered=0.7, n_patches=6)
    got, HX, off, idx, dist, st = _run(dev, c)
    counts = np.diff(off)
    assert counts.max() > 1000 and st.max_local > 500
    assert st.tensor_path == 1 and st.n_fallback <= st.n_points // 1000
    cols = np.concatenate([np.argsort(counts)[-60:], np.random.default_rng(1).choice(c.nlat * c.nlon, 60)])
    base, want = _oracle(c, HX, off, idx, dist, cols, 0)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL


@pytest.mark.parametrize("k", [64, 80])
def test_fp32_member_storage_highres_shape(dev, k):
    """The high-resolution configuration's analysis at reduced size with the
    members stored as FP32: 60 % of the obs in Gaussian patches, 300 km
    support, RTPS 0.9; both run the tensor-core kernel (k = 80 in its
    96-slot layout).  H(X) of the FP32 members is bit-identical to the
    oracle's on the widened values; the analysis of sampled columns (the longest lists among
    them) matches the oracle run on its own lists and H(X)."""
    c = syn.latlon_letkf_case(nlon=144, nlat=72, nlev=6, nvar=3, k=k, p=60_000, T=40, hsupport_km=300.0,
                              rho=0.9, case=45, clustered=0.6)
    X32 = T(c.X, dev).float().contiguous()
    Xw = X32.double().cpu().numpy()  # the background the FP32 path sees
    olat, olon, olev = T(c.obs_lat, dev), T(c.obs_lon, dev), T(c.obs_lev, dev)
    HX = K.hx_latlon(X32, c.nlon, c.nlat, c.nlev, olat, olon, olev, T(c.obs_var, dev))
    clat, clon = c.col_lat_lon()
    off, idx, dist = K.select_geo(T(clat, dev), T(clon, dev), olat, olon, c.hsupport_km)
    yo = T(c.yo, dev)
    _, st = K.letkf_batched(X32, col_base=T(c.col_base(), dev), nlev=c.nlev, n_var=c.nvar,
                            lev_stride=c.lev_stride, var_stride=c.var_stride, HX=HX, yo=yo,
                            rvar=torch.full_like(yo, c.sigma_o ** 2), loc_off=off, loc_idx=idx, loc_dist=dist,
                            obs_lev=olev, hsupport=c.hsupport_km, vsupport=c.vsupport, rho=c.rho,
                            flags=_lib.MG_RTPS, precision=_lib.MG_PREC_MIXED, want_mean=False)
    assert X32.dtype == torch.float32
    assert st.tensor_path == 1 and st.n_fallback <= st.n_points // 100
    counts = np.diff(off.cpu().numpy())
    assert counts.max() > 8 * max(1.0, np.median(counts))
    cols = np.unique(np.concatenate([np.argsort(counts)[-20:],
                                     np.random.default_rng(2).choice(c.nlat * c.nlon, 100, replace=False)]))
    offc, idxc, distc = ob.select_geo(clat[cols], clon[cols], c.obs_lat, c.obs_lon, c.hsupport_km)
    need = np.unique(idxc)
    HXc = ob.hx_latlon(Xw, c.nlon, c.nlat, c.nlev, c.obs_lat[need], c.obs_lon[need], c.obs_lev[need],
                       c.obs_var[need])
    assert np.array_equal(HX.cpu().numpy()[need], HXc)
    HXo = np.zeros((c.yo.size, k))
    HXo[need] = HXc
    offo = np.zeros(c.nlat * c.nlon + 1, dtype=np.int64)
    offo[cols + 1] = np.diff(offc)
    offo = np.cumsum(offo)
    pts, poff, pidx, pw = point_lists(cols, c.nlev, offo, idxc, distc, c.obs_lev, c.hsupport_km, c.vsupport)
    base = c.col_base()[pts[:, 0]] + pts[:, 1] * c.lev_stride
    want = ob.letkf_points(Xw, base, c.nvar, c.var_stride, HXo, c.yo, c.rvar, poff, pidx, pw, c.rho, ob.ORC_RTPS)
    got = X32.double().cpu().numpy()
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL


@pytest.mark.parametrize("sigma_o,k", [(0.2, 64), (0.01, 64), (0.2, 80)])
def test_ill_conditioned_points_go_to_the_simt_kernel(dev, sigma_o, k):
    """Accurate obs over a wide support make the deflated local matrix far
    worse conditioned than 3-pass TF32 products resolve.  Such points (a lower
    spectrum bound below the threshold, an iteration that leaves its basin,
    a finish residual above the bar) are re-run by the SIMT kernel: no
    non-finite value reaches the output, and every point matches the
    SIMT-only run (the re-run points bit for bit, since the SIMT kernel
    treats each point alone) and, on sampled columns, the oracle."""
    c = syn.latlon_letkf_case(nlon=72, nlat=36, nlev=4, nvar=2, k=k, p=40_000, T=20, sigma_o=sigma_o,
                              hsupport_km=900.0, case=46)
    got, HX, off, idx, dist, st = _run(dev, c)
    print(f"sigma_o {sigma_o}: {st.n_fallback} of {st.n_points} points re-run, max residual {st.max_residual:.2e}")
    assert st.tensor_path == 1 and st.n_fallback > 0
    assert np.isfinite(got).all()
    simt, _, _, _, _, st2 = _run(dev, c, flags=_lib.MG_SOLVE_SIMT)
    assert st2.tensor_path == 0
    assert rel_err(got, simt) <= MIXED_TOL
    cols = np.random.default_rng(3).choice(c.nlat * c.nlon, 80, replace=False)
    base, want = _oracle(c, HX, off, idx, dist, cols, 0)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL


def test_tensor_path_level_bucket_edges(dev):
    """The tensor-core kernel walks only the obs-level buckets (floor of the
    level, clamped to the grid) that can reach each analysis level.  Obs
    levels below level 0 and above the top level, levels at exact integers
    and a non-integer vertical support (1.5) sit at the bucket bounds; the
    localisation levels differ from the levels H interpolates at, so H(X)
    stays inside the grid.  Against the oracle on every column and against
    the SIMT kernel, which walks the unsorted lists."""
    c = syn.latlon_letkf_case(nlon=72, nlat=36, nlev=6, nvar=2, k=48, p=20_000, T=20, case=47)
    rng = np.random.default_rng(5)
    lev = c.obs_lev.copy()
    u = rng.random(lev.size)
    lo, hi, ints = u < 0.1, (u >= 0.1) & (u < 0.2), (u >= 0.2) & (u < 0.35)
    lev[lo] = -rng.uniform(0.0, 1.6, lo.sum())
    lev[hi] = (c.nlev - 1) + rng.uniform(0.0, 1.6, hi.sum())
    lev[ints] = rng.integers(0, c.nlev, ints.sum())
    vsupport = 1.5
    Xd = T(c.X, dev)
    olat, olon = T(c.obs_lat, dev), T(c.obs_lon, dev)
    HX = K.hx_latlon(Xd, c.nlon, c.nlat, c.nlev, olat, olon, T(c.obs_lev, dev), T(c.obs_var, dev))
    clat, clon = c.col_lat_lon()
    off, idx, dist = K.select_geo(T(clat, dev), T(clon, dev), olat, olon, c.hsupport_km)
    yo = T(c.yo, dev)
    rvar = torch.full_like(yo, c.sigma_o ** 2)

    def run(flags):
        X = Xd.clone()
        _, st = K.letkf_batched(X, col_base=T(c.col_base(), dev), nlev=c.nlev, n_var=c.nvar,
                                lev_stride=c.lev_stride, var_stride=c.var_stride, HX=HX, yo=yo, rvar=rvar,
                                loc_off=off, loc_idx=idx, loc_dist=dist, obs_lev=T(lev, dev), hsupport=c.hsupport_km,
                                vsupport=vsupport, rho=c.rho, flags=flags, precision=_lib.MG_PREC_MIXED,
                                want_mean=False)
        return X.cpu().numpy(), st

    got, st = run(0)
    assert st.tensor_path == 1 and st.n_fallback <= st.n_points // 100
    cols = np.arange(c.nlat * c.nlon)
    offh, idxh, disth = off.cpu().numpy(), idx.cpu().numpy(), dist.cpu().numpy()
    pts, poff, pidx, pw = point_lists(cols, c.nlev, offh, idxh, disth, lev, c.hsupport_km, vsupport)
    # the same candidates kept: a bucket bound that dropped one level's obs
    # would lose thousands; a few differ at the support's edge, where the
    # oracle's FP64 polynomial cancels to zero and the FP32 factored form
    # stays positive
    assert abs(st.total_local - poff[-1]) <= poff[-1] // 1000
    base = c.col_base()[pts[:, 0]] + pts[:, 1] * c.lev_stride
    want = ob.letkf_points(c.X, base, c.nvar, c.var_stride, HX.cpu().numpy(), c.yo, c.rvar, poff, pidx, pw, c.rho, 0)
    assert rel_err(_gather(got, c, base), want) <= MIXED_TOL
    simt, st2 = run(_lib.MG_SOLVE_SIMT)
    assert st2.tensor_path == 0 and st2.total_local == st.total_local
    assert rel_err(got, simt) <= MIXED_TOL
