"""The learned preconditioner's U-Net (BF16 tcgen05 convolutions, FP32
accumulation) trained by its own GPU forward and backward kernels: the loss
and every layer's gradient against PyTorch CPU autograd of the same network in
FP32 (same BF16-rounded weights and inputs), and a short training run.

Tolerance of the gradient check: the GPU keeps activations and activation
gradients in BF16 (8-bit mantissa) between layers, so each layer's weight
and bias gradient is held to 2e-2 relative (normwise) and to a cosine
similarity of at least 0.9995 with the FP32 gradient; the loss to 2e-2
(measured on a GB300: at most 6.5e-3 relative, cosine at least 0.99998)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402

LAYERS = ["c0a", "c0b", "c1a", "c1b", "c2a", "c2b", "c3a", "c3b", "c3u", "c2d", "c2u", "c1d", "c1u", "c0d", "cout"]


class Net:
    def __init__(self, H, W, B, cin=4, cout=3, seed=1):
        h = ctypes.c_void_p()
        rc = xc.lib().xc_nn_create(H, W, B, cin, cout, seed, ctypes.byref(h))
        assert rc == xc.XC_OK, xc.lib().xc_last_error()
        self.h, self.H, self.W, self.B, self.cin, self.cout = h, H, W, B, cin, cout
        self.n = xc.lib().xc_nn_param_count(h)
        wo, bo = (ctypes.c_longlong * 15)(), (ctypes.c_longlong * 15)()
        sp = (ctypes.c_int * 60)()
        assert xc.lib().xc_nn_layout(h, wo, bo, sp) == xc.XC_OK
        self.woff, self.boff = list(wo), list(bo)
        self.spec = [tuple(sp[4 * k:4 * k + 4]) for k in range(15)]

    def params(self):
        out = np.empty(self.n, dtype=np.float32)
        assert xc.lib().xc_nn_get_params(self.h, out.ctypes.data) == xc.XC_OK
        return out

    def grads(self):
        out = np.empty(self.n, dtype=np.float32)
        assert xc.lib().xc_nn_get_grads(self.h, out.ctypes.data) == xc.XC_OK
        return out

    def layer(self, flat, k):
        cin, cout = self.spec[k][0], self.spec[k][1]
        w = flat[self.woff[k]:self.woff[k] + 9 * cin * cout].reshape(cout, 9, cin)
        b = flat[self.boff[k]:self.boff[k] + cout]
        return w, b

    def close(self):
        xc.lib().xc_nn_destroy(self.h)


def _bf16(a):
    return torch.as_tensor(a).to(torch.bfloat16).float()


def torch_unet(net, flat, x):
    """The same U-Net in PyTorch (NCHW, FP32), weights rounded to BF16."""
    P = {}
    for k, name in enumerate(LAYERS):
        w, b = net.layer(flat, k)
        cout, _, cin = w.shape
        wt = _bf16(w).view(cout, 3, 3, cin).permute(0, 3, 1, 2).contiguous().requires_grad_(True)
        bt = torch.as_tensor(b.copy()).requires_grad_(True)
        P[name] = (wt, bt)

    def c(name, t, relu):
        y = torch.nn.functional.conv2d(t, P[name][0], P[name][1], padding=1)
        return torch.relu(y) if relu else y

    pool = lambda t: torch.nn.functional.avg_pool2d(t, 2)  # noqa: E731
    up = lambda t: torch.nn.functional.interpolate(t, scale_factor=2, mode="nearest")  # noqa: E731
    x16 = torch.zeros((x.shape[0], 16, x.shape[2], x.shape[3]))
    x16[:, :x.shape[1]] = _bf16(x)
    a0 = c("c0a", x16, 1); x0 = c("c0b", a0, 1)
    a1 = c("c1a", pool(x0), 1); x1 = c("c1b", a1, 1)
    a2 = c("c2a", pool(x1), 1); x2 = c("c2b", a2, 1)
    a3 = c("c3a", pool(x2), 1); x3 = c("c3b", a3, 1)
    y2 = c("c2d", up(c("c3u", x3, 0)) + x2, 1)
    y1 = c("c1d", up(c("c2u", y2, 0)) + x1, 1)
    y0 = c("c0d", up(c("c1u", y1, 0)) + x0, 1)
    return c("cout", y0, 0), P


def _inputs(B, H, W, cin, cout, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.randn((B, H, W, cin), generator=g)
    # a smooth target so the loss gradient is not noise
    t = torch.nn.functional.avg_pool2d(torch.randn((B, cout, H, W), generator=g), 5, 1, 2).permute(0, 2, 3, 1)
    return x.contiguous(), t.contiguous()


def test_unet_gradients_match_torch_autograd():
    B, H, W = 2, 128, 128
    net = Net(H, W, B)
    x, t = _inputs(B, H, W, net.cin, net.cout, seed=3)
    xd, td = x.cuda(), t.cuda()
    loss = ctypes.c_float()
    torch.cuda.synchronize()
    rc = xc.lib().xc_nn_loss_grad(net.h, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(td.data_ptr()),
                                  ctypes.byref(loss), None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    flat, g = net.params(), net.grads()
    out, P = torch_unet(net, flat, x.permute(0, 3, 1, 2))
    ref_loss = ((out[:, :net.cout] - t.permute(0, 3, 1, 2)) ** 2).sum(1).mean()
    ref_loss.backward()
    assert abs(loss.value - ref_loss.item()) <= 2e-2 * ref_loss.item(), (loss.value, ref_loss.item())
    report = {}
    for k, name in enumerate(LAYERS):
        gw, gb = net.layer(g, k)
        cout, _, cin = gw.shape
        rw = P[name][0].grad.permute(0, 2, 3, 1).reshape(cout, 9, cin).numpy()
        rb = P[name][1].grad.numpy()
        rel = np.linalg.norm(gw - rw) / np.linalg.norm(rw)
        cos = float((gw * rw).sum() / (np.linalg.norm(gw) * np.linalg.norm(rw)))
        relb = np.linalg.norm(gb - rb) / max(np.linalg.norm(rb), 1e-30)
        report[name] = (round(float(rel), 4), round(cos, 5), round(float(relb), 4))
        assert rel <= 2e-2 and cos >= 0.9995 and relb <= 2e-2, (name, report[name])
    print("U-Net gradient check (rel weight, cosine, rel bias):", report)
    net.close()


def test_unet_forward_matches_torch():
    B, H, W = 1, 256, 256
    net = Net(H, W, B, seed=5)
    x, _ = _inputs(B, H, W, net.cin, net.cout, seed=9)
    xd = x.cuda()
    out = torch.empty((B, H, W, net.cout), device="cuda")
    torch.cuda.synchronize()
    rc = xc.lib().xc_nn_forward(net.h, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    ref, _ = torch_unet(net, net.params(), x.permute(0, 3, 1, 2))
    ref = ref[:, :net.cout].permute(0, 2, 3, 1).detach()
    rel = float((out.cpu() - ref).norm() / ref.norm())
    assert rel <= 3e-2, rel
    net.close()


def test_unet_training_reduces_the_loss():
    """Fit a fixed smoothing of the input (a linear, local map): 300 Adam steps
    on one batch must cut the loss by at least 10x (150 steps gave 8.9x)."""
    B, H, W = 4, 128, 128
    net = Net(H, W, B, seed=2)
    g = torch.Generator().manual_seed(4)
    x = torch.randn((B, H, W, net.cin), generator=g)
    t = torch.nn.functional.avg_pool2d(x.permute(0, 3, 1, 2)[:, :net.cout], 3, 1, 1).permute(0, 2, 3, 1)
    xd, td = x.contiguous().cuda(), t.contiguous().cuda()
    loss = ctypes.c_float()
    losses = []
    for it in range(300):
        rc = xc.lib().xc_nn_train_step(net.h, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(td.data_ptr()),
                                       ctypes.c_float(2e-3), ctypes.byref(loss), None)
        assert rc == xc.XC_OK, xc.lib().xc_last_error()
        losses.append(loss.value)
    print("U-Net training loss:", losses[0], "->", losses[-1])
    assert losses[-1] <= losses[0] / 10, (losses[0], losses[-1])
    net.close()
