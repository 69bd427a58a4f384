"""The learned preconditioner of the Stokes solve: data, training and use.

The network (a 4-level U-Net of BF16 tcgen05 convolutions, include/xcore_gb300.h
``xc_nn_*``) maps a vector of the scaled saddle system of fluidmech!
(src/fluidmech.jl:491-523) -- seen as an Nz x Nx image of its W, U, P
components, plus log10(eta / etam0) -- to the direction of the system's
inverse applied to it.  Training pairs come from the plain FP64 solver
(FGMRES with the multigrid preconditioner, ``xc_learned_sample``) on
viscosity fields injected as in the reference's MMS test
(test/test_mms.jl:27-33): eta = etam0 * exp(ln(C) s), s a smoothed random
field in [0, 1], contrast C drawn log-uniformly.  Inside the mixed solver the
network either replaces the multigrid V-cycle of the FP32 inner FGMRES (the
multigrid redoing any inner solve it fails) or corrects what the V-cycle
leaves (``xc_solver_opts.learned`` 1 / 2); the FP64 residual of the
refinement judges the result either way.

    python xcore.jl_gb300/learned.py --out weights.npz [--N 256] [--samples 2048]
                                     [--steps 3000] [--seed 0]
trains a network on the GPU and writes its parameters.
"""
from __future__ import annotations

import ctypes
import math
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import xcore_gb300 as xc  # noqa: E402
else:
    import xcore_gb300 as xc  # noqa: E402

IN_CH, OUT_CH = 4, 3
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_stokes.npz")


class Network:
    """A U-Net of the library (xc_nn) for batches of H x W images."""

    def __init__(self, H, W, batch, seed=0):
        h = ctypes.c_void_p()
        xc._check(xc.lib().xc_nn_create(int(H), int(W), int(batch), IN_CH, OUT_CH, int(seed), ctypes.byref(h)))
        self.h, self.H, self.W, self.batch = h, H, W, batch
        self.nparams = int(xc.lib().xc_nn_param_count(h))

    def close(self):
        if getattr(self, "h", None):
            xc.lib().xc_nn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        xc._check(xc.lib().xc_nn_get_params(self.h, out.ctypes.data))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError(f"{p.size} parameters for a network of {self.nparams}")
        xc._check(xc.lib().xc_nn_set_params(self.h, p.ctypes.data))

    def train_step(self, inp, tgt, lr) -> float:
        """One Adam step on a batch (device FP32 tensors [batch][H][W][4] and
        [batch][H][W][3]); returns the batch loss."""
        loss = ctypes.c_float()
        xc._check(xc.lib().xc_nn_train_step(self.h, ctypes.c_void_p(inp.data_ptr()), ctypes.c_void_p(tgt.data_ptr()),
                                            ctypes.c_float(lr), ctypes.byref(loss), None))
        return loss.value

    def forward(self, inp, out):
        xc._check(xc.lib().xc_nn_forward(self.h, ctypes.c_void_p(inp.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                         None))


def save_params(path, params, meta=None):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, dtype=np.float32), **(meta or {}))


def load_params(path=WEIGHTS) -> np.ndarray:
    with np.load(path) as z:
        return np.asarray(z["params"], dtype=np.float32)


def use(state: "xc.State", params=None):
    """Give a State's Stokes solver the learned preconditioner (the committed
    weights by default); select it per solve with learned=1 or 2."""
    p = load_params() if params is None else np.ascontiguousarray(params, dtype=np.float32)
    xc._check(xc.lib().xc_set_learned_preconditioner(state._h, p.ctypes.data, ctypes.c_longlong(p.size)))


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def vector_layout(Nz, Nx):
    """Length and block sizes of the scaled system's vector: W (Nz+1, Nx+2),
    U (Nz+2, Nx+1), P (Nz+2, Nx+2), each column-major."""
    NW, NU, NP = (Nz + 1) * (Nx + 2), (Nz + 2) * (Nx + 1), (Nz + 2) * (Nx + 2)
    return NW + NU + NP, NW, NU, NP


def smooth_field(torch, gen, shape, width, device):
    """Standard-normal noise smoothed by a Gaussian of `width` cells
    (periodic, through the FFT) and scaled to unit RMS."""
    z = torch.randn(shape, generator=gen, device=device, dtype=torch.float32)
    if width > 0:
        ky = torch.fft.fftfreq(shape[-2], device=device).view(-1, 1)
        kx = torch.fft.fftfreq(shape[-1], device=device).view(1, -1)
        g = torch.exp(-2.0 * (math.pi * width) ** 2 * (ky * ky + kx * kx))
        z = torch.fft.ifft2(torch.fft.fft2(z) * g).real
    return z / z.pow(2).mean().sqrt().clamp_min(1e-30)


def staggered_vector(torch, gen, Nz, Nx, device, width):
    """A random vector of the scaled system: W, U, P components smoothed over
    `width` cells plus a little white noise, unit norm."""
    parts = []
    for rows, cols in ((Nz + 1, Nx + 2), (Nz + 2, Nx + 1), (Nz + 2, Nx + 2)):
        f = smooth_field(torch, gen, (cols, rows), width, device)      # column-major as [col][row]
        f = f + 0.05 * torch.randn((cols, rows), generator=gen, device=device)
        parts.append(f.reshape(-1))
    v = torch.cat(parts)
    return v / v.norm()


def inject_viscosity(state: "xc.State", contrast, rng):
    """eta = etam0 exp(ln(C) s) with s a smoothed random field in [0, 1]
    (test/test_mms.jl:27-33) on the cells, and the corner viscosities as the
    geometric mean of the four cells around each corner (x periodic, z
    repeated at the walls, as update! forms etaco)."""
    g = state.grid
    Nz, Nx = g.Nz, g.Nx
    z = rng.standard_normal((Nz, Nx))
    k = np.fft.fftfreq(Nz)[:, None] ** 2 + np.fft.fftfreq(Nx)[None, :] ** 2
    width = rng.uniform(2.0, Nz / 8)
    s = np.fft.ifft2(np.fft.fft2(z) * np.exp(-2.0 * (math.pi * width) ** 2 * k)).real
    s = (s - s.min()) / max(s.max() - s.min(), 1e-300)
    eta = state.par.etam0 * np.exp(math.log(contrast) * s)
    le = np.log(eta)
    ext = np.concatenate([le[:, -1:], le, le[:, :1]], axis=1)          # periodic x
    ext = np.concatenate([ext[:1], ext, ext[-1:]], axis=0)             # repeated z
    etaco = np.exp(0.25 * (ext[:-1, :-1] + ext[1:, :-1] + ext[:-1, 1:] + ext[1:, 1:]))
    state["eta"] = eta
    state["etaco"] = etaco[:Nz + 1, :Nx + 1]
    return eta


def workload_state(N, seed=0, etacntr=1e4):
    """A State of the 1024^2 mixed-precision workload's physics at N^2
    (lognormal crystal fraction, viscosity contrast cap etacntr), initialised,
    one phsevo! done so every Stokes input is populated."""
    D = 10.0
    h = D / N
    par = xc.Parameters(D=D, N=N, L=D, etam0=10.0, x0=0.1, Da=0.0, L0=3 * h, l0=3 * h, etacntr=float(etacntr),
                        ADVN="weno5", TINT="bd2im")
    st = xc.State(par)
    rng = np.random.default_rng(seed)
    x0 = np.clip(np.exp(np.log(0.1) + 0.5 * rng.standard_normal((N, N))), 0.0, 0.4)
    st.initialize(x0, rng.standard_normal((N, N)), rng.standard_normal((N, N)))
    coefs = xc.time_coefs("bd2im", 1)
    st.store_previous()
    st.store_noise()
    st.snapshot()
    st.phsevo(coefs, st.scales["dt0"])
    return st, coefs, st.scales["dt0"]


def generate(N=256, count=1024, per_field=16, contrasts=(1e2, 1e5), seed=0, rtol=1e-6, after_vcycle=True,
             log=None):
    """Training pairs (inputs [count][N][N][4], targets [count][N][N][3],
    device FP32): `count / per_field` injected viscosity fields, `per_field`
    random vectors each; with after_vcycle the right-hand side is the residual
    one multigrid V-cycle leaves of the vector (what the network corrects in
    learned mode 2), else the vector itself (mode 1); targets the plain FP64
    solver's solutions normalised to unit RMS (the network predicts the
    direction; FGMRES and the hybrid's least-squares step fix the scale)."""
    import torch
    dev = torch.device("cuda")
    st, coefs, dt = workload_state(N, seed)
    rng = np.random.default_rng(seed + 1)
    gen = torch.Generator(device=dev).manual_seed(seed + 2)
    inputs = torch.empty((count, N, N, IN_CH), device=dev)
    targets = torch.empty((count, N, N, OUT_CH), device=dev)
    iters = ctypes.c_int()
    t0 = time.time()
    total_its = 0
    for k in range(count):
        if k % per_field == 0:
            C = math.exp(rng.uniform(math.log(contrasts[0]), math.log(contrasts[1])))
            inject_viscosity(st, C, rng)
            # the operator of this viscosity (an FP64 solve sets up its multigrid)
            st.fluidmech(coefs, dt, solver="fgmres64", rtol=1e-6, maxit=600)
        v = staggered_vector(torch, gen, N, N, dev, float(np.exp(rng.uniform(0.0, math.log(N / 4)))))
        xc._check(xc.lib().xc_learned_sample(st._h, ctypes.c_void_p(v.data_ptr()), int(bool(after_vcycle)),
                                             ctypes.c_void_p(inputs[k].data_ptr()),
                                             ctypes.c_void_p(targets[k].data_ptr()), float(rtol), 600,
                                             ctypes.byref(iters)))
        total_its += iters.value
        if log and (k + 1) % max(1, count // 8) == 0:
            log(f"samples {k + 1}/{count} ({time.time() - t0:.0f} s, {total_its / (k + 1):.1f} FP64 iterations each)")
    rms = targets.pow(2).mean(dim=(1, 2, 3), keepdim=True).sqrt().clamp_min(1e-30)
    targets /= rms
    st.close()
    return inputs, targets


def train(net: Network, inputs, targets, steps=2000, lr=2e-3, seed=0, log=None):
    """Adam on random mini-batches of the pairs, cosine-decayed rate; returns
    the loss history."""
    import torch
    gen = torch.Generator(device=inputs.device).manual_seed(seed)
    B = net.batch
    losses = []
    t0 = time.time()
    for it in range(steps):
        idx = torch.randint(0, inputs.shape[0], (B,), generator=gen, device=inputs.device)
        xb, yb = inputs[idx].contiguous(), targets[idx].contiguous()
        rate = lr * 0.5 * (1.0 + math.cos(math.pi * it / steps))
        losses.append(net.train_step(xb, yb, rate))
        if log and (it + 1) % max(1, steps // 10) == 0:
            log(f"step {it + 1}/{steps} loss {np.mean(losses[-50:]):.4f} ({time.time() - t0:.0f} s)")
    return losses


SOLVE = dict(solver="mixed", rtol=1e-9, maxit=600, inner_rtol=5e-2, inner_maxit=30, pressure_sweeps=1)


def evaluate(params, N, seed=7, modes=(0, 1, 2), repeats=3, contrast=None):
    """The mixed solve of one Stokes system of the workload at N^2 with each
    preconditioner mode: inner iterations, learned fallbacks, final FP64
    residual and the device time of the solve (median of `repeats` after one
    untimed solve that captures the graphs).  contrast: the viscosity replaced
    by a smoothed random field of that contrast (inject_viscosity, the form of
    the training pairs) instead of the workload's rheology."""
    st, coefs, dt = workload_state(N, seed)
    if contrast is not None:
        inject_viscosity(st, contrast, np.random.default_rng(seed))
    use(st, params)
    snap = {k: st[k] for k in ("W", "U", "P", "MFS", "drhodt")}
    out = {}
    for mode in modes:
        secs = []
        info = None
        for r in range(repeats + 1):
            for k, v in snap.items():
                st[k] = v
            try:
                info = st.fluidmech(coefs, dt, learned=mode, **SOLVE)
            except xc.XcoreError as e:
                info = {"error": str(e)}
                break
            if r > 0:
                secs.append(info["seconds"])
        if secs:
            info["median_ms"] = 1e3 * float(np.median(secs))
        out[mode] = info
    st.close()
    return out


# (input channels, output channels, level) of the 15 convolutions
LAYERS = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 128, 3),
          (128, 128, 3), (128, 64, 3), (64, 64, 2), (64, 32, 2), (32, 32, 1), (32, 16, 1), (16, 16, 0), (16, 16, 0)]


def forward_flops(H, W):
    """Multiply-add flops of one forward pass (2 per multiply-add)."""
    return sum(2.0 * 9 * ci * co * (H >> lv) * (W >> lv) for ci, co, lv in LAYERS)


def bench_forward(N, iters=20):
    """Device time of one forward pass of the network at N^2 (CUDA events on
    the network's stream, after a warm-up pass) and its convolution flop
    rate."""
    import torch
    net = Network(N, N, 1, seed=0)
    inp = torch.randn((1, N, N, IN_CH), device="cuda")
    out = torch.empty((1, N, N, OUT_CH), device="cuda")
    net.forward(inp, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        net.forward(inp, out)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / iters
    net.close()
    return {"N": N, "ms_per_forward": ms, "conv_tflops": forward_flops(N, N) / (ms * 1e-3) / 1e12}


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--bench-forward", type=int, default=None, metavar="N",
                    help="only time the network's forward pass at N^2 and exit")
    ap.add_argument("--evaluate", type=int, default=None, metavar="N",
                    help="only evaluate the saved network (--out) at N^2 against the multigrid and exit")
    ap.add_argument("--contrast", type=float, default=None,
                    help="--evaluate with a smoothed random viscosity of this contrast instead of the workload's")
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--samples", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    xc.build()
    log = lambda m: print(m, flush=True)  # noqa: E731
    if a.bench_forward:
        import json
        log(json.dumps(bench_forward(a.bench_forward)))
        return
    if a.evaluate:
        import json
        rep = evaluate(load_params(a.out), a.evaluate, contrast=a.contrast)
        keep = ("iterations", "refinements", "rel_residual", "converged", "learned_fallbacks", "median_ms", "error")
        log(json.dumps({"N": a.evaluate, "contrast": a.contrast,
                        "modes": {str(m): {k: v for k, v in r.items() if k in keep} for m, r in rep.items()}}))
        return
    inputs, targets = generate(a.N, a.samples, seed=a.seed, after_vcycle=True, log=log)
    # the loss of predicting zero, for reference: the targets have unit RMS
    zero_loss = float(targets.pow(2).sum(dim=3).mean())
    net = Network(a.N, a.N, a.batch, seed=a.seed)
    losses = train(net, inputs, targets, steps=a.steps, lr=a.lr, seed=a.seed, log=log)
    params = net.params()
    net.close()
    del inputs, targets
    import json
    report = {n: evaluate(params, n) for n in (a.N, 1024)}
    log("evaluation: " + json.dumps(report))
    # the mode the bench uses: the fastest at 1024^2 (0 = the multigrid alone)
    times = {m: r.get("median_ms", float("inf")) for m, r in report[1024].items()}
    best = min(times, key=times.get)
    save_params(a.out, params, {"N": np.int64(a.N), "samples": np.int64(a.samples), "steps": np.int64(a.steps),
                                "loss_first": np.float64(np.mean(losses[:50])),
                                "loss_last": np.float64(np.mean(losses[-50:])), "loss_zero": np.float64(zero_loss),
                                "best_mode": np.int64(best),
                                **{f"ms_1024_mode{m}": np.float64(t if math.isfinite(t) else -1.0)
                                   for m, t in times.items()},
                                **{f"iterations_1024_mode{m}": np.int64(r.get("iterations", -1))
                                   for m, r in report[1024].items()}})
    log(f"wrote {a.out}: loss {np.mean(losses[:50]):.4f} -> {np.mean(losses[-50:]):.4f} (zero predictor "
        f"{zero_loss:.4f}); best mode at 1024^2: {best}")


if __name__ == "__main__":
    main()
