"""Generate the golden fixtures in this directory from the CPU oracle.

Seeded inputs (initial crystal fraction, white-noise draws) and the oracle's
fields after each of three time steps of a 16 x 12 grid (WENO5, BD2, three
Picard sweeps), plus single-kernel fixtures (WENO5 / QUICK advect-with-flux,
diffusion, the FFT noise filter).  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
import xcore_oracle as O  # noqa: E402
from gpu_helpers import oracle_params  # noqa: E402

STEP_FIELDS = ("X", "M", "x", "W", "U", "P", "eta", "etaco", "MFS", "Wx", "Ux", "psie", "xie", "kx", "rho")


def make_steps():
    par = oracle_params(16, 12)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(2024)
    x0 = rng.uniform(0.02, 0.10, (g.Nz, g.Nx))
    draws = rng.standard_normal((4, 2, g.Nz, g.Nx))
    st = O.initialize(g, par, sc, ns, x0, draws[0, 0], draws[0, 1])
    out = {"x0": x0, "draws": draws}
    dt = sc["dt0"]
    dts = [dt]
    for step in range(1, 4):
        dt, norms = O.timestep(st, g, par, sc, ns, step, dt, draws[step, 0], draws[step, 1])
        dts.append(dt)
        for f in STEP_FIELDS:
            out[f"s{step}_{f}"] = getattr(st, f).copy()
        out[f"s{step}_resnorm"] = np.array([n[0] for n in norms])
    out["dts"] = np.array(dts)
    np.savez_compressed(os.path.join(HERE, "steps_16x12.npz"), **out)


def make_kernels():
    rng = np.random.default_rng(77)
    Nz, Nx, h = 11, 9, 0.3
    f = rng.random((Nz, Nx)) * 2 + rng.standard_normal((Nz, Nx)) ** 3
    u = rng.standard_normal((Nz, Nx + 1))
    w = rng.standard_normal((Nz + 1, Nx))
    k = rng.random((Nz, Nx)) + 0.5
    out = {"f": f, "u": u, "w": w, "k": k, "h": np.array(h)}
    for s in ("weno5", "quick"):
        adv, qx, qz = O.advect_centered_with_flux(f, u, w, h, s)
        out[f"{s}_adv"], out[f"{s}_qx"], out[f"{s}_qz"] = adv, qx, qz
    out["dff"], out["dqx"], out["dqz"] = O.diffus_centered_with_flux(f, k, h)
    Gk = O.make_gaussian_filter(Nz + 4, Nx, h, 2 * h)
    out["filtered"] = O.fft_filter(f, Gk, 4)
    np.savez_compressed(os.path.join(HERE, "kernels_11x9.npz"), **out)


if __name__ == "__main__":
    make_steps()
    make_kernels()
    print("golden fixtures written to", HERE)
