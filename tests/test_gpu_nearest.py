"""GPU: nearest-node search of geographic obs on a curvilinear grid (spatial
hash) against the reference's scan restated in the oracle: bit-identical
node choice, including ties, obs outside the grid and the vertical index."""
import math

import numpy as np
import pytest
import torch

import oracle.bind as ob
from metada_gb300 import kernels as K

pytestmark = pytest.mark.gpu


def _grid(nx, ny, seed):
    g = np.random.default_rng(seed)
    lon, lat = np.meshgrid(np.linspace(70.0, 140.0, nx), np.linspace(5.0, 55.0, ny))
    lon = lon + 0.8 * np.sin(np.deg2rad(lat) * 3.0) + 0.05 * g.standard_normal(lon.shape)
    lat = lat + 0.4 * np.cos(np.deg2rad(lon) * 2.0)
    return np.ascontiguousarray(lat.ravel()), np.ascontiguousarray(lon.ravel())


@pytest.mark.parametrize("nx,ny,p", [(40, 30, 2000), (300, 200, 20000)])
def test_nearest_node_matches_scan(dev, nx, ny, p):
    lat, lon = _grid(nx, ny, nx)
    g = np.random.default_rng(p)
    oa = g.uniform(0.0, 60.0, p)    # some obs outside the grid
    ol = g.uniform(60.0, 150.0, p)
    # exact ties: obs at the midpoint of two nodes, and on nodes
    oa[:50], ol[:50] = 0.5 * (lat[:50] + lat[1:51]), 0.5 * (lon[:50] + lon[1:51])
    oa[50:100], ol[50:100] = lat[200:250], lon[200:250]
    vc = np.array([1000.0, 925.0, 850.0, 700.0, 500.0, 300.0, 100.0])
    lev = g.uniform(50.0, 1050.0, p)
    lev[:20] = 0.5 * (1000.0 + 925.0)  # ties between two levels: the first wins
    want_xy, want_k = ob.nearest_node(lat, lon, nx, ny, oa, ol, vc, lev)
    T = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    xy, kk = K.nearest_node(T(lat), T(lon), nx, ny, T(oa), T(ol), T(vc), T(lev))
    assert np.array_equal(xy.cpu().numpy(), want_xy)
    assert np.array_equal(kk.cpu().numpy(), want_k)


def test_nearest_node_feeds_idw4(dev):
    """(i, j) from the search is the grid-obs input of the IDW4 operator."""
    nx, ny = 50, 40
    lat, lon = _grid(nx, ny, 3)
    g = np.random.default_rng(9)
    X = g.standard_normal((6, nx * ny))
    oa, ol = g.uniform(10, 50, 300), g.uniform(75, 135, 300)
    T = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    xy, _ = K.nearest_node(T(lat), T(lon), nx, ny, T(oa), T(ol))
    HX = K.hx_idw4(T(X), nx, ny, xy).cpu().numpy()
    wxy, _ = ob.nearest_node(lat, lon, nx, ny, oa, ol)
    assert np.array_equal(HX, ob.hx_idw4(X, nx, ny, wxy))


def _collapsed_pairs(n, seed):
    """n obs, each with two nodes whose sums of squares dx^2 + dy^2 differ
    while their rounded square roots are equal: the scan keeps the lower
    index, which is given to the node with the larger sum."""
    g = np.random.default_rng(seed)

    def s_of(la, lo, gla, glo):
        dx, dy = lo - glo, la - gla
        return dx * dx + dy * dy

    def step(x, k):
        for _ in range(abs(k)):
            x = float(np.nextafter(x, np.inf if k > 0 else -np.inf))
        return x

    lat, lon, oa, ol = np.empty(2 * n), np.empty(2 * n), np.empty(n), np.empty(n)
    for j in range(n):
        ola, olo, found = 0.0, 16.0 * j, None
        while found is None:
            t = g.uniform(0.0, 2.0 * np.pi)
            A = (ola + 0.3 * math.sin(t), olo + 0.3 * math.cos(t))
            sA = s_of(ola, olo, *A)
            for a in range(-3, 4):
                for b in range(-3, 4):
                    B = (step(A[0], a), step(A[1], b))
                    sB = s_of(ola, olo, *B)
                    if sA != sB and math.sqrt(sA) == math.sqrt(sB):
                        found = (A, B) if sA > sB else (B, A)
                        break
                if found is not None:
                    break
        (lat[2 * j], lon[2 * j]), (lat[2 * j + 1], lon[2 * j + 1]) = found
        oa[j], ol[j] = ola, olo
    return lat, lon, oa, ol


def test_nearest_node_ties_of_rounded_square_roots(dev):
    n = 200
    lat, lon, oa, ol = _collapsed_pairs(n, 11)
    want, _ = ob.nearest_node(lat, lon, 2, n, oa, ol)
    assert np.all(want[:, 0] == 0) and np.array_equal(want[:, 1], np.arange(n))
    T = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    xy, _ = K.nearest_node(T(lat), T(lon), 2, n, T(oa), T(ol))
    assert np.array_equal(xy.cpu().numpy(), want)


@pytest.mark.parametrize("case", ["curv", "reg"])
def test_nearest_node_matches_reference_golden(dev, case):
    """Against the reference's own IdentityObsOperator geographic branch
    (IdentityObsOperator.hpp:484-520, run by the header harness): nodes and
    levels identical, ties and obs outside the grid included."""
    from conftest import GOLDEN

    g = np.load(GOLDEN / "nearest.npz")
    c = lambda k: g[f"{case}_{k}"]  # noqa: E731
    T = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)  # noqa: E731
    xy, kk = K.nearest_node(T(c("lat")), T(c("lon")), int(c("nx")), int(c("ny")), T(c("olat")), T(c("olon")),
                            T(c("vc")), T(c("olev")))
    ijk = c("ijk")
    assert np.array_equal(xy.cpu().numpy()[:, 0], ijk[:, 0]) and np.array_equal(xy.cpu().numpy()[:, 1], ijk[:, 1])
    assert np.array_equal(kk.cpu().numpy(), ijk[:, 2])
