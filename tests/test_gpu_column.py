"""GPU: the learned column observation operator — plain operator against
the oracle, surrogate MLP gradients against the numpy oracle, training on
operator-labelled columns, and the surrogate inside an LETKF."""
import numpy as np
import pytest
import torch

from conftest import rel_err

import oracle.bind as ob
import oracle.mlp as om
from metada_gb300 import _lib
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def op():
    return syn.column_operator()


def test_column_operator_matches_oracle(dev, op):
    T, q = syn.random_columns(20_000)
    y = K.column_op(torch.tensor(T, device=dev), torch.tensor(q, device=dev), torch.tensor(op.w, device=dev),
                    torch.tensor(op.tau, device=dev)).cpu().numpy()
    want = ob.column_op(T, q, op.w, op.tau)
    assert rel_err(y, want) <= 1e-5


def test_hx_column_plain_matches_oracle(dev, op):
    c = syn.column_letkf_case(nlon=24, nlat=12, nlev=30, k=8, p=500, T_trunc=8)
    X = torch.tensor(c.X, device=dev)
    HX = K.hx_column(X, c.ncol, c.nlev, torch.tensor(c.obs_col, device=dev), torch.tensor(c.obs_ch, device=dev),
                     torch.tensor(c.op.w, device=dev), torch.tensor(c.op.tau, device=dev)).cpu().numpy()
    want = np.empty_like(HX)
    for i in range(c.X.shape[0]):
        T, q = syn.column_state_to_Tq(c.X[i], c.nlev, c.ncol)
        y = ob.column_op(T[c.obs_col], q[c.obs_col], c.op.w, c.op.tau)
        want[:, i] = y[np.arange(len(c.obs_col)), c.obs_ch]
    assert rel_err(HX, want) <= 1e-5


def test_mlp_gradients_match_oracle(dev):
    mlp = K.MLP(64, 256, 16)
    P = mlp.init_params(seed=3)
    g = np.random.default_rng(1)
    B = 300
    X = g.standard_normal((B, 64)).astype(np.float32)
    X[:, 60:] = 0.0
    Yt = (g.standard_normal((B, 16)) * 3.0 + 1.0).astype(np.float32)
    shift = np.full(16, 1.0, np.float32)
    scale = np.full(16, 3.0, np.float32)
    mlp.set_params(P, torch.tensor(shift, device=dev), torch.tensor(scale, device=dev))
    G, loss = mlp.gradients(torch.tensor(X, device=dev), torch.tensor(Yt, device=dev))
    # the oracle uses the same BF16-rounded weights (biases stay FP32)
    Pw = mlp.params(bf16_rounded=True).cpu().numpy().astype(np.float64)
    Pm = mlp.params().cpu().numpy().astype(np.float64)
    W1, b1, W2, b2, W3, b3 = om.unpack(np.arange(len(Pm)), 64, 256, 16)
    for bias in (b1, b2, b3):
        Pw[bias.astype(int)] = Pm[bias.astype(int)]
    want, wloss = om.gradients(Pw, X, Yt, shift, scale, 64, 256, 16)
    assert rel_err(G.cpu().numpy(), want) <= 1e-4
    assert abs(loss - wloss) <= 1e-4 * wloss
    # forward too
    Y = mlp.forward(torch.tensor(X, device=dev)).cpu().numpy()
    wY, _ = om.forward(Pw, X, 64, 256, 16)
    assert rel_err(Y, wY) <= 1e-4


def _train(dev, op, ncol=200_000, steps=4000, batch=4096, seed=7):
    T, q = syn.random_columns(ncol, stream=seed)
    Td, qd = torch.tensor(T, device=dev), torch.tensor(q, device=dev)
    w, tau = torch.tensor(op.w, device=dev), torch.tensor(op.tau, device=dev)
    Y = K.column_op(Td, qd, w, tau)
    Xf = K.column_features(Td, qd, 64)
    shift, scale = Y.mean(0), Y.std(0)
    mlp = K.MLP(64, 256, 16)
    P = mlp.init_params(seed=seed)
    mlp.set_params(P, shift, scale)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    losses = []
    for s in range(steps):
        idx = torch.randint(0, ncol, (batch,), device=dev, generator=gen)
        lr = 2e-3 * 0.5 * (1 + np.cos(np.pi * s / steps)) + 1e-5
        loss = mlp.train_step(Xf[idx].contiguous(), Y[idx].contiguous(), lr, want_loss=(s % 100 == 0))
        if s % 100 == 0:
            losses.append(loss)
    return mlp, losses, (shift, scale)


def test_mlp_training_beats_linear_surrogate(dev, op):
    """The trained network against the method without it: a linear
    least-squares map from the same features."""
    mlp, losses, (shift, scale) = _train(dev, op)
    assert losses[-1] < 0.05 * losses[0]
    T, q = syn.random_columns(20_000, stream=99)
    Td, qd = torch.tensor(T, device=dev), torch.tensor(q, device=dev)
    y = K.column_op(Td, qd, torch.tensor(op.w, device=dev), torch.tensor(op.tau, device=dev)).cpu().numpy()
    Xf = K.column_features(Td, qd, 64)
    ynet = (mlp.forward(Xf) * scale + shift).cpu().numpy()
    T2, q2 = syn.random_columns(200_000, stream=7)
    X2 = K.column_features(torch.tensor(T2, device=dev), torch.tensor(q2, device=dev), 64).cpu().numpy()
    y2 = ob.column_op(T2, q2, op.w, op.tau)
    A = np.hstack([X2[:, :60], np.ones((len(X2), 1), np.float32)]).astype(np.float64)
    coef, *_ = np.linalg.lstsq(A, y2.astype(np.float64), rcond=None)
    ylin = np.hstack([Xf.cpu().numpy()[:, :60], np.ones((len(T), 1))]) @ coef
    err_net = np.sqrt(np.mean((ynet - y) ** 2)) / np.sqrt(np.mean(y ** 2))
    err_lin = np.sqrt(np.mean((ylin - y) ** 2)) / np.sqrt(np.mean(y ** 2))
    assert err_net < 0.02
    assert err_net < 0.5 * err_lin


def test_surrogate_letkf_gains_over_background(dev, op):
    """Column obs assimilated through the trained surrogate reduce the
    analysis error against the truth, close to the plain operator's."""
    c = syn.column_letkf_case(nlon=72, nlat=36, nlev=30, k=32, p=4000, T_trunc=12, hsupport_km=1500.0)
    mlp, _, _ = _train(dev, c.op)
    Xb = torch.tensor(c.X, device=dev)
    oc, och = torch.tensor(c.obs_col, device=dev), torch.tensor(c.obs_ch, device=dev)
    w, tau = torch.tensor(c.op.w, device=dev), torch.tensor(c.op.tau, device=dev)
    la, lo = c.col_lat_lon()
    off, idx, dist = K.select_geo(torch.tensor(la, device=dev), torch.tensor(lo, device=dev),
                                  torch.tensor(la[c.obs_col], device=dev), torch.tensor(lo[c.obs_col], device=dev),
                                  c.hsupport_km)
    yo = torch.tensor(c.yo, device=dev)
    rvar = torch.full_like(yo, c.sigma_o ** 2)
    out = {}
    for name in ("plain", "surrogate"):
        X = Xb.clone()
        HX = K.hx_column(X, c.ncol, c.nlev, oc, och, w, tau) if name == "plain" else mlp.hx_column(X, c.ncol, c.nlev, oc, och)
        K.letkf_batched(X, col_base=torch.arange(c.ncol, dtype=torch.int64, device=dev), nlev=1, n_var=2 * c.nlev,
                        lev_stride=0, var_stride=c.ncol, HX=HX, yo=yo, rvar=rvar, loc_off=off, loc_idx=idx,
                        loc_dist=dist, hsupport=c.hsupport_km, rho=c.rho, flags=0, precision=_lib.MG_PREC_MIXED,
                        want_mean=False)
        out[name] = X.mean(0).cpu().numpy()
    nT = c.nlev * c.ncol
    rmse = lambda a: float(np.sqrt(np.mean((a[:nT] - c.truth[:nT]) ** 2)))  # noqa: E731
    rb, rp, rs = rmse(c.X.mean(0)), rmse(out["plain"]), rmse(out["surrogate"])
    assert rp < rb and rs < rb  # both analyses improve on the background temperature
    assert rs < rb - 0.5 * (rb - rp)  # the surrogate keeps at least half the plain operator's gain
