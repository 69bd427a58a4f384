"""Committed golden fixtures (tests/golden/, generated by make_golden.py from
the oracle on seeded inputs): the oracle must keep reproducing them, and the
GPU path must match them through the C ABI."""
import os

import numpy as np
import pytest

import xcore_oracle as O
from gpu_helpers import oracle_params, rel_err

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STEP_FIELDS = ("X", "M", "x", "W", "U", "P", "eta", "etaco", "MFS", "Wx", "Ux", "psie", "xie", "kx", "rho")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def test_oracle_reproduces_kernel_fixtures():
    z = _load("kernels_11x9.npz")
    f, u, w, k, h = z["f"], z["u"], z["w"], z["k"], float(z["h"])
    for s in ("weno5", "quick"):
        adv, qx, qz = O.advect_centered_with_flux(f, u, w, h, s)
        assert np.array_equal(adv, z[f"{s}_adv"]) and np.array_equal(qx, z[f"{s}_qx"])
        assert np.array_equal(qz, z[f"{s}_qz"])
    dff, dqx, dqz = O.diffus_centered_with_flux(f, k, h)
    assert np.array_equal(dff, z["dff"]) and np.array_equal(dqx, z["dqx"]) and np.array_equal(dqz, z["dqz"])
    flt = O.fft_filter(f, O.make_gaussian_filter(f.shape[0] + 4, f.shape[1], h, 2 * h), 4)
    assert rel_err(flt, z["filtered"]) <= 1e-13


def _oracle_run(z):
    par = oracle_params(16, 12)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    d = z["draws"]
    st = O.initialize(g, par, sc, ns, z["x0"], d[0, 0], d[0, 1])
    return par, g, sc, ns, st


def test_oracle_reproduces_step_fixtures():
    z = _load("steps_16x12.npz")
    par, g, sc, ns, st = _oracle_run(z)
    dt = sc["dt0"]
    for step in range(1, 4):
        dt, _ = O.timestep(st, g, par, sc, ns, step, dt, z["draws"][step, 0], z["draws"][step, 1])
        for f in STEP_FIELDS:
            assert rel_err(getattr(st, f), z[f"s{step}_{f}"]) <= 1e-11, (step, f)
    assert dt == pytest.approx(z["dts"][3], rel=1e-12)


@pytest.mark.gpu
def test_gpu_matches_step_fixtures():
    pytest.importorskip("torch")
    from gpu_helpers import device_state
    z = _load("steps_16x12.npz")
    par, g, sc, ns, st = _oracle_run(z)
    ds = device_state(par, g, sc)
    d = z["draws"]
    ds.initialize(z["x0"], d[0, 0], d[0, 1])
    dt = sc["dt0"]
    for step in range(1, 4):
        info = ds.step(step, dt, d[step, 0], d[step, 1], sweeps=3, rtol=1e-11)
        dt = info["dt_next"]
        for f in STEP_FIELDS:
            e = rel_err(ds[f], z[f"s{step}_{f}"])
            assert e <= 1e-8, (step, f, e)
    assert dt == pytest.approx(z["dts"][3], rel=1e-8)
