"""xc_update_dt_noalloc -- the CFL step for callers that cannot let the library
allocate device memory (a Julia process whose CUDA.jl pool owns the device
memory, or a framework with its own caching allocator).  It must give the same
time step as xc_update_dt on the same state, call after call, while its block
partials live in a static device array instead of allocated scratch.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from gpu_helpers import device_state, realistic_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402


def _noalloc_dt(ds, dt_prev, out):
    g, p = ds.grid, ds.par
    ptr = [ctypes.c_void_p(ds.device_ptr(n)) for n in ("kx", "Wx", "Wm", "Ux", "Um")]
    torch.cuda.synchronize()
    rc = xc.lib().xc_update_dt_noalloc(*ptr, g.Nz, g.Nx, g.h, p.CFL, p.dtmax, float(dt_prev),
                                       ctypes.c_void_p(out.data_ptr()), None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    torch.cuda.synchronize()
    return float(out.item())


def test_noalloc_dt_matches_update_dt_twice():
    par, g, sc, ns, st, dt, rng = realistic_state(N=48, Nx=40, steps=1)
    ds = device_state(par, g, sc, st)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    # first call: the state as the oracle left it
    ref1 = ds.update_dt(dt)
    got1 = _noalloc_dt(ds, dt, out)
    assert got1 == ref1
    # second call on changed fields: a faster phase velocity and a larger kx
    ds["Wx"] = st.Wx * 3.0
    ds["kx"] = st.kx * 1.7
    ref2 = ds.update_dt(dt * 0.5)
    got2 = _noalloc_dt(ds, dt * 0.5, out)
    assert got2 == ref2
    assert got1 != got2


def test_noalloc_dt_rejects_grids_beyond_the_static_scratch():
    """Checked on the host before any launch: nothing is read from the
    (deliberately null-free but unused) pointers."""
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = xc.lib().xc_update_dt_noalloc(p, p, p, p, p, 4000, 4000, 0.1, 0.5, 1e32, 1.0, p, None)
    assert rc == xc.XC_BAD_ARG
    assert b"static scratch" in xc.lib().xc_last_error()
