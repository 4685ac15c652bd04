"""Host checks of the closed forms the mixed kernels rely on (no GPU):

* the second-order Daleckii-Krein finish of the LETKF's two-stage solve:
  f(D + E) for f = x^-1/2 and x^-1 from first and second divided differences
  in closed form, with the second-order sum for x^-1/2 split by partial
  fractions into two matrix products (the form the kernel evaluates);
* the sorted form of the CRPS pair sum used by the diagnostics kernel,
  sum_j sum_l |x_j - x_l| = 2 sum_j (2 r_j - k + 1) x_j with ties broken by
  member index.
"""
import numpy as np
import pytest


def _nearly_diagonal(k, tol, seed):
    g = np.random.default_rng(seed)
    d = np.exp(g.uniform(np.log(60.0), np.log(6e3), k))
    E = g.uniform(-1.0, 1.0, (k, k))
    E = (E + E.T) / 2
    np.fill_diagonal(E, 0.0)
    E *= tol * np.sqrt(d[:, None] * d[None, :])
    return d, E


def _exact(d, E, p):
    lam, V = np.linalg.eigh(np.diag(d) + E)
    return V @ np.diag(lam ** p) @ V.T


def _dk(d, E, order):
    s = np.sqrt(d)
    si, sj = s[:, None], s[None, :]
    h = 1.0 / (si * sj * (si + sj))
    W = np.diag(1.0 / s) - E * h
    G = np.diag(1.0 / d) - E / (d[:, None] * d[None, :])
    if order == 2:
        P = E / (si + sj)
        M = P @ (E / s[:, None])          # sum_m P_im E_mj / s_m
        S = M + M.T - P @ P               # M^T = sum_m E_im P_mj / s_m (E, P symmetric)
        W = W + h * S
        G = G + (E @ (E / d[:, None])) / (d[:, None] * d[None, :])
    return W, G


@pytest.mark.parametrize("k,tol", [(32, 1e-3), (64, 1e-3), (64, 3e-4), (96, 1e-3)])
def test_second_order_daleckii_krein(k, tol):
    d, E = _nearly_diagonal(k, tol, seed=k)
    Wx, Gx = _exact(d, E, -0.5), _exact(d, E, -1.0)
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()  # noqa: E731
    W1, G1 = _dk(d, E, 1)
    W2, G2 = _dk(d, E, 2)
    # the second-order remainder is third order in E
    assert rel(W2, Wx) <= 1e-2 * rel(W1, Wx) + 1e-15
    assert rel(G2, Gx) <= 1e-2 * rel(G1, Gx) + 1e-15
    assert rel(W2, Wx) <= k * k * tol ** 3


def test_partial_fraction_split_equals_second_divided_difference():
    k = 12
    d, E = _nearly_diagonal(k, 1e-2, seed=3)
    s = np.sqrt(d)
    want = np.zeros((k, k))
    for i in range(k):
        for j in range(k):
            for m in range(k):
                f3 = (s[i] + s[m] + s[j]) / (s[i] * s[m] * s[j] * (s[i] + s[m]) * (s[m] + s[j]) * (s[i] + s[j]))
                want[i, j] += f3 * E[i, m] * E[m, j]
    got = _dk(d, E, 2)[0] - _dk(d, E, 1)[0]
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_crps_pair_sum_in_sorted_form(seed):
    g = np.random.default_rng(seed)
    k = 64
    x = np.round(g.standard_normal(k), 1)  # coarse grid: many ties
    x[5:8] = x[4] + np.arange(1, 4) * np.spacing(x[4])
    pair = np.abs(x[:, None] - x[None, :]).sum()
    # rank by (value, member index), as the kernel counts it
    order = np.lexsort((np.arange(k), x))
    r = np.empty(k, dtype=np.int64)
    r[order] = np.arange(k)
    sorted_form = 2.0 * np.sum((2 * r - k + 1) * x)
    assert abs(sorted_form - pair) <= 1e-12 * pair
