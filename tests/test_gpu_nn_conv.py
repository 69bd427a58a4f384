"""The learned preconditioner's 3x3 convolution on the tcgen05 tensor cores
(BF16 operands, FP32 accumulation in TMEM, TMA-staged operand tiles) and its
weight gradient, through the C ABI, against PyTorch's FP32 convolution of the
same BF16-rounded operands.

Tolerances: the FP32 outputs within 1e-5 (normwise relative: only the
summation order of exact BF16 x BF16 products differs); the BF16 outputs
within 1e-2 (one BF16 rounding, 2^-8); the FP32 weight gradient within 1e-4
(sums over thousands of pixels in a different order)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402

SHAPES = [  # (B, H, W, Cin, Cout)
    (1, 8, 128, 16, 16),
    (2, 16, 32, 32, 64),
    (1, 4, 256, 64, 128),
    (1, 8, 128, 128, 32),
    (2, 32, 64, 128, 128),
    (1, 16, 16, 16, 32),
]


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _rel(a, b):
    return float((a - b).norm() / b.norm())


def _operands(B, H, W, Cin, Cout, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((B, H, W, Cin), generator=g, device="cuda").to(torch.bfloat16)
    w = (torch.randn((Cout, 9, Cin), generator=g, device="cuda") / (3 * Cin ** 0.5)).to(torch.bfloat16)
    bias = torch.randn((Cout,), generator=g, device="cuda")
    return x, w, bias


def _torch_conv(x, w, bias, relu):
    B, H, W, Cin = x.shape
    Cout = w.shape[0]
    wt = w.float().view(Cout, 3, 3, Cin).permute(0, 3, 1, 2)
    y = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), wt, bias, padding=1)
    if relu:
        y = torch.relu(y)
    return y.permute(0, 2, 3, 1).contiguous()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("relu", [0, 1])
def test_conv3x3_matches_torch(shape, relu):
    B, H, W, Cin, Cout = shape
    x, w, bias = _operands(B, H, W, Cin, Cout, seed=sum(shape) + relu)
    y = torch.empty((B, H, W, Cout), dtype=torch.bfloat16, device="cuda")
    y32 = torch.empty((B, H, W, Cout), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = xc.lib().xc_nn_conv3x3(_p(x), _p(w), _p(bias), _p(y), _p(y32), B, H, W, Cin, Cout, relu, None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    ref = _torch_conv(x, w, bias, relu)
    assert _rel(y32, ref) <= 1e-5
    assert _rel(y.float(), ref) <= 1e-2
    # the edge rows and columns (zero padding) in particular
    for sl in (np.s_[:, 0], np.s_[:, -1], np.s_[:, :, 0], np.s_[:, :, -1]):
        assert _rel(y32[sl], ref[sl]) <= 1e-5


@pytest.mark.parametrize("shape", SHAPES)
def test_conv3x3_wgrad_matches_torch(shape):
    B, H, W, Cin, Cout = shape
    x, w, _ = _operands(B, H, W, Cin, Cout, seed=7 * sum(shape))
    g = torch.Generator(device="cuda").manual_seed(11)
    dy = torch.randn((B, H, W, Cout), generator=g, device="cuda").to(torch.bfloat16)
    dw = torch.empty((Cout, 9, Cin), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = xc.lib().xc_nn_conv3x3_wgrad(_p(x), _p(dy), _p(dw), B, H, W, Cin, Cout, None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    ref = torch.nn.grad.conv2d_weight(x.float().permute(0, 3, 1, 2), (Cout, Cin, 3, 3),
                                      dy.float().permute(0, 3, 1, 2), padding=1)
    ref = ref.permute(0, 2, 3, 1).reshape(Cout, 9, Cin)
    assert _rel(dw, ref) <= 1e-4


def test_conv3x3_rejects_untileable_shapes():
    x = torch.zeros((1, 8, 100, 16), dtype=torch.bfloat16, device="cuda")
    w = torch.zeros((16, 9, 16), dtype=torch.bfloat16, device="cuda")
    y = torch.zeros((1, 8, 100, 16), dtype=torch.bfloat16, device="cuda")
    rc = xc.lib().xc_nn_conv3x3(_p(x), _p(w), None, _p(y), None, 1, 8, 100, 16, 16, 0, None)
    assert rc == xc.XC_BAD_ARG
    rc = xc.lib().xc_nn_conv3x3(_p(x), _p(w), None, _p(y), None, 1, 8, 128, 24, 16, 0, None)
    assert rc == xc.XC_BAD_ARG
