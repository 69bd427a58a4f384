"""Several outer time steps of run! (src/run.jl:204-275) on the GPU against the
oracle, fed identical white-noise draws each step, for both advection schemes
of the path (WENO5 and QUICK).  The Stokes solve is iterative (FP64 FGMRES to
1e-11 here), so the fields follow the oracle's sparse-LU path within a
tolerance that grows with the steps: 1e-7 relative (normwise) after four
steps."""
import pytest

import xcore_oracle as O
from gpu_helpers import device_state, realistic_state, rel_err

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

FIELDS = ("X", "x", "M", "m", "W", "U", "P", "eta", "rho", "MFS", "psie", "psix", "psis", "xie", "Wx", "Ux", "kx")


@pytest.mark.parametrize("scheme", ["weno5", "quick"])
def test_four_steps_follow_the_oracle(scheme):
    par, g, sc, ns, st, dt, rng = realistic_state(N=32, Nx=40, steps=1, ADVN=scheme)
    ds = device_state(par, g, sc, st)
    dt_g = dt
    for step in range(2, 6):
        re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
        dt_o, _ = O.timestep(st, g, par, sc, ns, step, dt, re, rs)
        info = ds.step(step, dt_g, re, rs, sweeps=3, rtol=1e-11, maxit=1500)
        assert info["dt_next"] == pytest.approx(dt_o, rel=1e-7), step
        bad = {k: rel_err(ds[k], getattr(st, k)) for k in FIELDS}
        bad = {k: v for k, v in bad.items() if not v <= 1e-7}
        assert not bad, (step, bad)
        dt, dt_g = dt_o, info["dt_next"]
