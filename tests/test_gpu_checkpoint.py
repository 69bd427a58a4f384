"""Checkpoint interop (src/restart.jl:53-127): a GPU run saved with the
reference's dataset names and resumed in a fresh context continues exactly as
the uninterrupted run does."""
import numpy as np
import pytest

from gpu_helpers import device_state, realistic_state

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402


def test_resume_from_checkpoint_is_exact(tmp_path):
    par, g, sc, ns, st, dt, rng = realistic_state(N=32, Nx=40, steps=1)
    run = device_state(par, g, sc, st)
    draws = [(rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))) for _ in range(3)]
    info = run.step(2, dt, *draws[0], sweeps=3, solver="mixed", rtol=1e-9)
    dt = info["dt_next"]
    path = tmp_path / "run_cont.npz"
    run.save_checkpoint(path, time=1.5, dt=dt, step=2)

    resumed = device_state(par, g, sc)            # a fresh context: nothing uploaded
    t, dt_r, step = resumed.load_checkpoint(path)
    assert (t, dt_r, step) == (1.5, dt, 2)
    for k, v in resumed.checkpoint().items():
        np.testing.assert_array_equal(v, run[k.split("/", 1)[1]], err_msg=k)

    for n, (re, rs) in enumerate(draws[1:], start=3):
        a = run.step(n, dt, re, rs, sweeps=3, solver="mixed", rtol=1e-9)
        b = resumed.step(n, dt, re, rs, sweeps=3, solver="mixed", rtol=1e-9)
        assert a == b
        dt = a["dt_next"]
    ca, cb = run.checkpoint(), resumed.checkpoint()
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k], err_msg=k)
