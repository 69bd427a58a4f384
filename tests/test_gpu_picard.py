"""The time step's Picard loop and its failure reporting, on the GPU against
the oracle (src/run.jl:204-275):

* xc_step_converge runs the reference's while-loop -- at least 3 sweeps, then
  on while resnorm/resnorm0 >= rtol, resnorm >= atol and fewer than maxit
  sweeps ran, resnorm0 raised when a sweep's norm grows (run.jl:220-249) --
  and stops after the same number of sweeps as the oracle's loop;
* a Stokes solve held to one iteration surfaces as XC_NOT_CONVERGED after a
  completed step (the reference's direct solve never leaves an unconverged
  iterate, so the library says so instead of moving on silently);
* a NaN planted on the host travels as Julia's minimum / maximum carry it:
  NaN eta cap, NaN time step, NaN statistics;
* print_step!'s statistics (src/diagnose.jl:92-182) match the oracle."""
import math

import numpy as np
import pytest

import xcore_oracle as O
from gpu_helpers import device_state, realistic_state, rel_err

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402


def test_convergence_loop_runs_the_oracles_sweeps():
    par, g, sc, ns, st, dt, rng = realistic_state(N=32, Nx=40, steps=1)
    ds = device_state(par, g, sc, st)
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    rtol, atol, maxit = 1e-3, 1e-12, 12
    dt_o, norms, r0 = O.timestep_converge(st, g, par, sc, ns, 2, dt, re, rs, rtol=rtol, atol=atol, maxit=maxit)
    info = ds.step_converge(2, dt, re, rs, picard_rtol=rtol, picard_atol=atol, picard_maxit=maxit,
                            rtol=1e-12, maxit=1500)
    assert 3 <= len(norms) <= maxit
    assert info["sweeps"] == len(norms), (info["resnorm"], norms)
    np.testing.assert_allclose(info["resnorm"][:3], norms[:3], rtol=1e-6)
    assert info["dt_next"] == pytest.approx(dt_o, rel=1e-7)
    assert info["picard_converged"] == (norms[-1] / r0 < rtol or norms[-1] < atol)
    for k in ("X", "W", "U", "P", "eta"):
        assert rel_err(ds[k], getattr(st, k)) <= 1e-7, k


def test_convergence_loop_minimum_three_sweeps():
    """With rtol = atol = inf the while-condition is false after one sweep,
    but `|| iter < 3` keeps three."""
    par, g, sc, ns, st, dt, rng = realistic_state(N=24, Nx=20, steps=1)
    ds = device_state(par, g, sc, st)
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    info = ds.step_converge(2, dt, re, rs, picard_rtol=math.inf, picard_atol=math.inf, picard_maxit=15)
    assert info["sweeps"] == 3 and info["picard_converged"]
    info = ds.step_converge(3, dt, re, rs, picard_rtol=0.0, picard_atol=0.0, picard_maxit=5)
    assert info["sweeps"] == 5 and not info["picard_converged"]


def test_capped_stokes_solve_is_reported_after_a_completed_step():
    par, g, sc, ns, st, dt, rng = realistic_state(N=24, Nx=20, steps=1)
    ds = device_state(par, g, sc, st)
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    with pytest.raises(xc.NotConverged) as ei:
        ds.step(2, dt, re, rs, sweeps=3, rtol=1e-12, maxit=1)
    info = ei.value.info
    assert info["unconverged_solves"] == 3 and info["sweeps"] == 3
    assert info["solver_rel_residual"] > 1e-12
    assert math.isfinite(info["dt_next"]) and info["dt_next"] > 0
    # the same step with a converging solve reports nothing
    ds2 = device_state(par, g, sc, st)
    ok = ds2.step(2, dt, re, rs, sweeps=3, rtol=1e-10, maxit=1500)
    assert ok["unconverged_solves"] == 0


def test_nan_propagates_like_julia():
    par, g, sc, ns, st, dt, rng = realistic_state(N=24, Nx=20, steps=1)
    # a NaN crystal fraction in one cell: minimum(etai) is NaN, so the
    # harmonic cap makes every eta NaN (update.jl:330-335)
    st.x = st.x.copy()
    st.x[5, 7] = np.nan
    ds = device_state(par, g, sc, st)
    O.update(st, g, par, sc)
    ds.update()
    for k in ("eta", "etas", "kx", "Rc"):
        assert np.array_equal(np.isnan(ds[k]), np.isnan(getattr(st, k))), k
    assert np.isnan(st.eta).all()
    # a NaN phase speed gives a NaN time step (update.jl:497-501)
    par2, g2, sc2, ns2, st2, dt2, _ = realistic_state(N=24, Nx=20, steps=1)
    st2.Um = st2.Um.copy()
    st2.Um[3, 4] = np.nan
    ds2 = device_state(par2, g2, sc2, st2)
    assert math.isnan(O.update_dt(st2, g2, par2, dt2))
    assert math.isnan(ds2.update_dt(dt2))
    # and NaN statistics
    assert math.isnan(ds.history_stats()["eta_min"])


def test_print_step_stats_match_oracle():
    par, g, sc, ns, st, dt, rng = realistic_state(N=40, Nx=36, steps=2)
    ds = device_state(par, g, sc, st)
    got = ds.print_step_stats()
    ref = O.print_step_stats(st)
    assert set(got) == set(ref)
    for k, v in ref.items():
        assert got[k] == pytest.approx(v, rel=1e-12, abs=1e-300), k
