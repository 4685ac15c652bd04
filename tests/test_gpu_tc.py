"""GPU: the tensor-core (tcgen05 + TMA) BF16 GEMM against an FP64 product of
the same BF16 values, its argument checks, and the surrogate's tensor-core
inference path against the SIMT forward pass."""
import numpy as np
import pytest
import torch

from conftest import rel_err

from metada_gb300 import _lib
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

# (M, N, K): ragged row tiles, every N tile width (16 ... 256), N below and
# between tile widths (zero-filled B rows), K tails inside a 64-wide block.
SHAPES = [(128, 16, 64), (77, 1, 16), (300, 48, 72), (129, 200, 8), (1000, 256, 256),
          (4096, 128, 512), (513, 32, 136), (2000, 64, 64)]


def _ref(A, B, bias, silu):
    C = A.double().cpu() @ B.double().cpu().T
    if bias is not None:
        C = C + bias.double().cpu()
    if silu:
        C = C / (1.0 + torch.exp(-C))
    return C.numpy()


@pytest.mark.parametrize("M,N,Kd", SHAPES)
@pytest.mark.parametrize("epi", ["plain", "bias_silu"])
def test_tc_gemm_matches_fp64(dev, M, N, Kd, epi):
    g = torch.Generator().manual_seed(M * 7 + N * 3 + Kd)
    A = torch.randn(M, Kd, generator=g).to(torch.bfloat16).to(dev)
    B = torch.randn(N, Kd, generator=g).to(torch.bfloat16).to(dev)
    bias = torch.randn(N, generator=g).to(dev) if epi != "plain" else None
    C = K.gemm_bf16_tc(A, B, bias, silu=(epi != "plain")).cpu().numpy()
    want = _ref(A, B, bias, epi != "plain")
    # FP32 accumulation of exact BF16 products: relative error ~ sqrt(K) 2^-24.
    assert rel_err(C, want) <= 1e-5
    assert np.isfinite(C).all()


def test_tc_gemm_back_to_back(dev):
    """Two launches in a row on the same context give identical results."""
    g = torch.Generator().manual_seed(5)
    A = torch.randn(3000, 256, generator=g).to(torch.bfloat16).to(dev)
    B = torch.randn(256, 256, generator=g).to(torch.bfloat16).to(dev)
    C1 = K.gemm_bf16_tc(A, B)
    C2 = K.gemm_bf16_tc(A, B)
    assert torch.equal(C1, C2)


@pytest.mark.parametrize("M,N,Kd,offset", [(128, 0, 64, 0), (128, 257, 64, 0), (128, 64, 12, 0),
                                            (128, 64, 64, 1)])
def test_tc_gemm_rejects_bad_arguments(dev, M, N, Kd, offset):
    A = torch.zeros(M * Kd + 8, dtype=torch.bfloat16, device=dev)[offset:offset + M * Kd].view(M, Kd)
    B = torch.zeros(max(N, 1), Kd, dtype=torch.bfloat16, device=dev)[:N]
    with pytest.raises(_lib.MgError) as e:
        K.gemm_bf16_tc(A, B)
    assert e.value.code == _lib.MG_ERR_ARG


def test_surrogate_tensor_core_path_matches_simt_forward(dev):
    """mg_hx_column_mlp (tensor-core inference, BF16 activations) against the
    SIMT forward pass (FP32 activations) on the same columns and weights."""
    c = syn.column_letkf_case(nlon=24, nlat=12, nlev=30, k=8, p=3000, T_trunc=8)
    mlp = K.MLP(64, 256, 16)
    P = mlp.init_params(seed=11)
    shift = torch.linspace(1.0, 4.0, 16, device=dev)
    scale = torch.linspace(0.5, 2.0, 16, device=dev)
    mlp.set_params(P, shift, scale)
    X = torch.tensor(c.X, device=dev)
    oc, och = torch.tensor(c.obs_col, device=dev), torch.tensor(c.obs_ch, device=dev)
    HX = mlp.hx_column(X, c.ncol, c.nlev, oc, och).cpu().numpy()
    want = np.empty_like(HX)
    for i in range(c.X.shape[0]):
        T, q = syn.column_state_to_Tq(c.X[i], c.nlev, c.ncol)
        F = K.column_features(torch.tensor(T[c.obs_col], device=dev), torch.tensor(q[c.obs_col], device=dev), 64)
        Y = (mlp.forward(F) * scale + shift).cpu().numpy()
        want[:, i] = Y[np.arange(len(c.obs_col)), c.obs_ch]
    # BF16 rounding of the features and hidden activations (2^-9 relative).
    assert rel_err(HX, want) <= 1e-2
    assert np.isfinite(HX).all()


def test_tc_gemm_bounded_wait_gives_up_and_context_stays_usable(dev):
    """A wait that can never complete (one k-block never loaded) runs out and
    the kernel returns MG_ERR_TIMEOUT instead of hanging; the next GEMM on
    the same context is correct."""
    from metada_gb300 import _lib

    g = torch.Generator().manual_seed(11)
    A = torch.randn(2048, 128, generator=g).to(torch.bfloat16).to(dev)
    B = torch.randn(256, 128, generator=g).to(torch.bfloat16).to(dev)
    assert K.gemm_bf16_tc_wait_selftest(A, B) == _lib.MG_ERR_TIMEOUT
    C = K.gemm_bf16_tc(A, B).cpu().numpy()
    assert rel_err(C, _ref(A, B, None, False)) <= 1e-5
