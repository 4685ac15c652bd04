"""CPU tests: the oracle against the reference's golden vectors and against
independent restatements (numpy / scipy), plus the synthetic generators."""
import math

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

import oracle.bind as ob
from metada_gb300 import synthetic as syn


@pytest.fixture(scope="module")
def tut():
    return np.load(GOLDEN / "tutorial.npz")


def test_tutorial_etkf_matches_reference(built, tut):
    X, nx, ny, s = tut["X"], int(tut["nx"]), int(tut["ny"]), float(tut["sigma"])
    HX = ob.hx_idw4(X, nx, ny, tut["obs_xy"])
    Xa, mean = ob.etkf_compat(X, HX, tut["yo"], np.full(len(tut["yo"]), s * s), float(tut["rho"]))
    assert rel_err(Xa, tut["etkf_members"]) < 1e-12
    assert np.array_equal(mean, tut["etkf_mean"])  # stale background mean, bit-exact


@pytest.mark.parametrize("which,rho_key", [("letkf", "rho"), ("letkf_rho11", "rho11")])
def test_tutorial_letkf_matches_reference(built, tut, which, rho_key):
    X, nx, ny = tut["X"], int(tut["nx"]), int(tut["ny"])
    Xa, mean = ob.letkf_compat_grid(X, nx, ny, tut["obs_xy"], tut["yo"], float(tut["radius"]), float(tut[rho_key]))
    assert rel_err(Xa, tut[f"{which}_members"]) < 1e-12
    assert rel_err(mean, tut[f"{which}_mean"]) < 1e-12


def test_grid64_etkf_matches_reference(built):
    g = np.load(GOLDEN / "etkf_grid64.npz")
    HX = ob.hx_idw4(g["X"], 64, 64, g["obs_xy"])
    Xa, mean = ob.etkf_compat(g["X"], HX, g["yo"], np.full(len(g["yo"]), float(g["sigma"]) ** 2), float(g["rho"]))
    assert rel_err(Xa, g["members"]) < 1e-12
    assert np.array_equal(mean, g["mean"])


@pytest.mark.parametrize("name", ["letkf_grid24", "letkf_grid20"])
def test_small_letkf_matches_reference(built, name):
    g = np.load(GOLDEN / f"{name}.npz")
    Xa, mean = ob.letkf_compat_grid(g["X"], int(g["nx"]), int(g["ny"]), g["obs_xy"], g["yo"], float(g["radius"]),
                                    float(g["rho"]))
    assert rel_err(Xa, g["members"]) < 1e-12
    assert rel_err(mean, g["mean"]) < 1e-12
    off, _ = ob.select_grid(int(g["nx"]), int(g["ny"]), g["obs_xy"], float(g["radius"]))
    assert np.any(np.diff(off) == 0), "fixture should contain points without local obs"


def test_ensemble_mean_is_member_order_sum_times_reciprocal(built):
    X = np.random.default_rng(0).standard_normal((7, 1001)) * 1e3
    m = ob.ens_mean(X)
    want = np.zeros(1001)
    for i in range(7):
        want = want + X[i]
    want = want * (1.0 / 7)
    assert np.array_equal(m, want)
    m2, Xp = ob.ens_mean_pert(X)
    assert np.array_equal(m2, want) and np.array_equal(Xp, X - want)


def test_idw4_at_nodes_and_edges(built):
    nx, ny = 5, 4
    x = np.arange(nx * ny, dtype=np.float64)[None, :] ** 1.5
    obs = np.array([[0, 0], [4, 3], [2, 1], [7, -2]], dtype=np.int32)  # last one clamps to (4, 0)
    HX = ob.hx_idw4(x, nx, ny, obs, np.array([1, 1, 1, 1], dtype=np.uint8))

    def idw(ox, oy):
        xx, yy = min(max(ox, 0), nx - 1), min(max(oy, 0), ny - 1)
        i1, j1 = min(xx + 1, nx - 1), min(yy + 1, ny - 1)
        ws = wsum = 0.0
        for ii, jj in ((xx, yy), (i1, yy), (xx, j1), (i1, j1)):
            d = math.sqrt((xx - ii) ** 2 + (yy - jj) ** 2)
            w = 1e12 if d == 0 else 1.0 / d
            ws += w * x[0, jj * nx + ii]
            wsum += w
        return ws / wsum

    for o, (ox, oy) in enumerate(obs):
        assert HX[o, 0] == idw(ox, oy)
    HXv = ob.hx_idw4(x, nx, ny, obs, np.array([1, 0, 1, 1], dtype=np.uint8))
    assert HXv[1, 0] == 0.0  # invalid obs give 0 (IdentityObsOperator.hpp:165-167)


def test_haversine_and_gaspari_cohn_known_values(built):
    # one degree of longitude at the equator on the R = 6371 km sphere
    assert abs(ob.haversine_km(0, 0, 0, 1) - 6371.0 * math.pi / 180) < 1e-9
    assert abs(ob.haversine_km(-90, 0, 90, 0) - 6371.0 * math.pi) < 1e-6
    assert ob.gaspari_cohn(0.0) == 1.0
    assert abs(ob.gaspari_cohn(1.0) - 5.0 / 24.0) < 1e-15
    assert ob.gaspari_cohn(2.0) == 0.0 and ob.gaspari_cohn(3.0) == 0.0
    z = np.linspace(0, 2, 41)
    g = np.array([ob.gaspari_cohn(v) for v in z])
    assert np.all(np.diff(g) <= 1e-15)  # monotone non-increasing


def test_select_grid_matches_bruteforce(built):
    g = np.random.default_rng(3)
    nx, ny, p = 17, 11, 40
    obs = np.stack([g.integers(-2, nx + 2, p), g.integers(-2, ny + 2, p)], axis=1).astype(np.int32)
    r = syn.float_config(4.3)
    off, idx = ob.select_grid(nx, ny, obs, r)
    for gp in range(nx * ny):
        gx, gy = gp % nx, gp // nx
        want = [o for o in range(p) if math.sqrt((gx - obs[o, 0]) ** 2 + (gy - obs[o, 1]) ** 2) <= r]
        assert list(idx[off[gp]:off[gp + 1]]) == want


def test_select_geo_matches_bruteforce(built):
    g = np.random.default_rng(4)
    p = 3000
    olat = np.rad2deg(np.arcsin(g.uniform(-1, 1, p)))
    olon = g.uniform(0, 360, p)
    clat = np.array([0.0, 45.5, -89.5, 89.5, 10.0, -60.25])
    clon = np.array([0.5, 359.5, 180.0, 0.5, 180.0, 90.0])
    off, idx, dist = ob.select_geo(clat, clon, olat, olon, 1500.0)
    for c in range(len(clat)):
        want = [o for o in range(p) if ob.haversine_km(clat[c], clon[c], olat[o], olon[o]) <= 1500.0]
        assert list(idx[off[c]:off[c + 1]]) == want
        assert np.all(dist[off[c]:off[c + 1]] <= 1500.0)


def test_sym_eig_reconstructs(built):
    g = np.random.default_rng(5)
    B = g.standard_normal((40, 24))
    A = B.T @ B + 23.0 * np.eye(24)
    w, V, sweeps = ob.sym_eig(A)
    assert sweeps < 20
    assert rel_err(V @ np.diag(w) @ V.T, A) < 1e-13
    assert rel_err(np.sort(w), np.linalg.eigvalsh(A)) < 1e-13


def test_letkf_points_hunt_equals_dense_formula(built):
    """Hunt LETKF of the oracle against a numpy restatement for one point."""
    g = np.random.default_rng(6)
    k, p, n = 10, 25, 3
    X = g.standard_normal((k, n))
    HX = g.standard_normal((p, k))
    yo = g.standard_normal(p)
    rvar = g.uniform(0.5, 2.0, p)
    w = g.uniform(0.1, 1.0, p)
    rho = 1.1
    out = ob.letkf_points(X, np.array([1]), 1, 0, HX, yo, rvar, np.array([0, p]), np.arange(p), w, rho, 0)
    ym = HX.mean(axis=1)
    Yp = HX - ym[:, None]
    Rinv = np.diag(w / rvar)
    A = (k - 1) / rho * np.eye(k) + Yp.T @ Rinv @ Yp
    ev, V = np.linalg.eigh(A)
    Pa = V @ np.diag(1 / ev) @ V.T
    W = V @ np.diag(np.sqrt((k - 1) / ev)) @ V.T
    wa = Pa @ Yp.T @ Rinv @ (yo - ym)
    xb = X[:, 1]
    xm = xb.mean()
    xa = xm + (xb - xm) @ (wa[:, None] + W)
    assert rel_err(out[0, 0], xa) < 1e-12


def test_synthetic_generators_are_seeded():
    a = syn.global_etkf_grid(16, 16, 4, 20)
    b = syn.global_etkf_grid(16, 16, 4, 20)
    assert np.array_equal(a.X, b.X) and np.array_equal(a.yo, b.yo)
    assert len(np.unique(a.obs_xy[:, 0] + 16 * a.obs_xy[:, 1])) == 20  # distinct cells
    f = syn.sh_random_fields(64, 18, 36, 8, -3.0, syn.rng(99))
    assert f.shape == (64, 18, 36)
    assert 0.6 < f.var() < 1.4  # unit point variance on average


def test_column_operator_formula(built):
    g = np.random.default_rng(7)
    T = g.uniform(200, 310, (5, 30)).astype(np.float32)
    q = np.exp(g.uniform(np.log(1e-6), np.log(2e-2), (5, 30))).astype(np.float32)
    w = g.uniform(0, 1, (16, 30)).astype(np.float32)
    tau = g.uniform(0.5, 5, 16).astype(np.float32)
    y = ob.column_op(T, q, w, tau)
    c, ch = 3, 7
    cq = np.cumsum(q[c].astype(np.float64))
    want = np.sum(w[ch].astype(np.float64) * np.exp(-float(tau[ch]) * cq) * T[c].astype(np.float64) ** 4 / 1e8)
    assert abs(y[c, ch] - want) <= 1e-6 * abs(want)


# Known-answer tests of Metrics<double>::CalculateAll, from the reference's
# own tests (tests/framework/algorithms/MetricsTest.cpp:28-42 fixture,
# expectations at :64-200): truth [1, 2, 3, 4]; members truth + 0.1,
# truth - 0.1, truth.
METRICS_TRUTH = np.array([1.0, 2.0, 3.0, 4.0])
METRICS_MEMBERS = np.array([[1.1, 2.1, 3.1, 4.1], [0.9, 1.9, 2.9, 3.9], [1.0, 2.0, 3.0, 4.0]])
METRICS_UNCORRELATED = np.array([[10.0, 2.0, 300.0, 4.0], [4.0, 3.0, 20.0, 1.0], [2.0, 30.0, 1.0, 43.0]])


def test_metrics_match_reference_known_answers(built):
    mean, spread, m = ob.ens_metrics(METRICS_MEMBERS, METRICS_TRUTH)
    np.testing.assert_allclose(mean, METRICS_TRUTH, atol=1e-6)
    np.testing.assert_allclose(spread, 0.1, atol=1e-6)
    assert abs(m["bias"]) <= 1e-6
    assert abs(m["correlation"] - 1.0) <= 1e-6
    assert abs(m["crps"] - 0.022222222222222227) <= 1e-6 and m["crps"] > 0
    assert abs(m["rmse"]) <= 1e-6
    assert abs(m["avg_spread"] - 0.1) <= 1e-6
    _, _, b = ob.ens_metrics(METRICS_MEMBERS + 0.5, METRICS_TRUTH)
    assert abs(b["bias"] - 0.5) <= 1e-6 and abs(b["rmse"] - 0.5) <= 1e-6 and abs(b["correlation"] - 1.0) <= 1e-6
    _, _, u = ob.ens_metrics(METRICS_UNCORRELATED, METRICS_TRUTH)
    assert abs(u["correlation"] - 0.34105511573854358) <= 1e-6
    assert u["rmse"] > 1.0 and u["crps"] > 1.0


@pytest.mark.parametrize("which", ["tut", "c1"])
def test_enkf_matches_reference(built, which):
    """The dense EnKF restatement against the reference's own EnKF.hpp, run by
    the header harness with a seeded generator (tests/golden/enkf.npz)."""
    g = np.load(GOLDEN / "enkf.npz")
    X, xy, yo = g[f"{which}_X"], g[f"{which}_obs_xy"], g[f"{which}_yo"]
    nx, ny = (int(g["nx"]), int(g["ny"])) if which == "tut" else (int(g["c1_nx"]), int(g["c1_ny"]))
    s = float(g[f"{which}_sigma"])
    rho = 1.0 if which == "tut" else float(g["c1_rho"])
    HX = ob.hx_idw4(X, nx, ny, xy)
    Xa, mean, diag, gain = ob.enkf(X, HX, yo, np.full(len(yo), s * s), g[f"{which}_eps"], rho)
    assert rel_err(Xa, g[f"{which}_members"]) <= 1e-10
    assert rel_err(mean, g[f"{which}_mean"]) <= 1e-10
    want = g[f"{which}_diag"]
    got = [diag["innovation_norm"], diag["background_spread"], diag["analysis_spread"], gain[0], gain[1]]
    np.testing.assert_allclose(got, want, rtol=1e-10)


def test_nearest_node_scan_matches_numpy(built):
    """The restated scan of IdentityObsOperator::convertGeographicToGrid
    (first strict minimum in node order) against numpy's argmin."""
    g = np.random.default_rng(4)
    nx, ny = 30, 20
    lon, lat = np.meshgrid(np.linspace(100.0, 130.0, nx), np.linspace(10.0, 30.0, ny))
    lon = lon + 0.3 * np.sin(lat / 5.0)
    ol, oa = g.uniform(95, 135, 500), g.uniform(5, 35, 500)
    xy, _ = ob.nearest_node(lat.ravel(), lon.ravel(), nx, ny, oa, ol)
    d = np.sqrt((ol[:, None] - lon.ravel()[None]) ** 2 + (oa[:, None] - lat.ravel()[None]) ** 2)
    idx = np.argmin(d, axis=1)  # first minimum, as the scan
    assert np.array_equal(xy[:, 0], idx % nx) and np.array_equal(xy[:, 1], idx // nx)


def test_parse_values_is_the_istringstream_loop(built):
    """SimpleState::readFromFile: a line's extraction stops at the first
    token that is not a double; the next line starts afresh."""
    text = b"  1.5 2.25\n-3e2\t4.000000\nbad 5\n7 .5 8x 9\n\n+.25e1 -0.0\n"
    got = ob.parse_values(text)
    assert np.array_equal(got, [1.5, 2.25, -300.0, 4.0, 7.0, 0.5, 8.0, 2.5, -0.0])
    assert np.signbit(got[-1])


@pytest.mark.parametrize("case", ["curv", "reg"])
def test_nearest_node_matches_reference(case):
    """The oracle's nearest-node scan against the reference's own
    IdentityObsOperator geographic branch (IdentityObsOperator.hpp:484-520),
    run by the header harness (tests/golden/nearest.npz): nodes and levels
    identical, including exact ties (the first minimum wins) and obs outside
    the grid."""
    g = np.load(GOLDEN / "nearest.npz")
    c = lambda k: g[f"{case}_{k}"]  # noqa: E731
    xy, kk = ob.nearest_node(c("lat"), c("lon"), int(c("nx")), int(c("ny")), c("olat"), c("olon"), c("vc"), c("olev"))
    ijk = c("ijk")
    assert np.array_equal(xy[:, 0], ijk[:, 0]) and np.array_equal(xy[:, 1], ijk[:, 1])
    assert np.array_equal(kk, ijk[:, 2])
