"""xc_update_dt_noalloc -- the CFL step for callers that cannot let the library
allocate device memory (a Julia process whose CUDA.jl pool owns the device
memory, or a framework with its own caching allocator).  It must give the same
time step as xc_update_dt on the same state, call after call, while its block
partials live in a static device array instead of allocated scratch.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test."""
import ctypes
from types import SimpleNamespace

import numpy as np
import pytest

import xcore_oracle as O
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


def _raw_noalloc_dt(arrs, Nz, Nx, h, CFL, dtmax, dt_prev, out):
    ptr = [ctypes.c_void_p(a.data_ptr()) for a in arrs]
    torch.cuda.synchronize()
    rc = xc.lib().xc_update_dt_noalloc(*ptr, Nz, Nx, h, CFL, dtmax, float(dt_prev),
                                       ctypes.c_void_p(out.data_ptr()), None)
    assert rc == xc.XC_OK, xc.lib().xc_last_error()
    torch.cuda.synchronize()
    return float(out.item())


def _random_fields(Nz, Nx, seed):
    """kx (Nz,Nx), Wx, Wm (Nz+1,Nx+2), Ux, Um (Nz+2,Nx+1) as device tensors
    holding the column-major bytes, with the extremes planted far from the
    first CTA's chunk so the cross-CTA combine decides them."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    shapes = [(Nz, Nx), (Nz + 1, Nx + 2), (Nz + 1, Nx + 2), (Nz + 2, Nx + 1), (Nz + 2, Nx + 1)]
    arrs = []
    for k, (r, c) in enumerate(shapes):
        t = torch.rand((c, r), dtype=torch.float64, device="cuda", generator=g)
        # small diffusivities, so the advective (CFL) bound is the binding one
        t = t * 1e-6 if k == 0 else t * 2.0 - 1.0
        flat = t.view(-1)
        flat[flat.numel() - 1 - 97 * k] = (3.0 + k) * (1 if k % 2 else -1) if k else 5e-6
        arrs.append(t)
    return arrs


def _oracle_dt(arrs, h, CFL, dtmax, dt_prev):
    host = [a.cpu().numpy().T for a in arrs]
    st = SimpleNamespace(kx=host[0], Wx=host[1], Wm=host[2], Ux=host[3], Um=host[4])
    return O.update_dt(st, SimpleNamespace(h=h), SimpleNamespace(CFL=CFL, dtmax=dtmax), dt_prev)


@pytest.mark.parametrize("shape", [(300, 200), (400, 400), (2890, 2890)])
def test_noalloc_dt_many_ctas_per_array(shape):
    """Grids whose arrays span many CTAs of unequal counts (40 for the
    400^2 faces, about 2040 near the 8,388,608-element limit at 2890^2), so
    the scratch stride per array, the -inf partials of CTAs past a shorter
    array's end and the combine over many partials all decide the result;
    two calls in a row, each bit-identical to the oracle's update_dt."""
    Nz, Nx = shape
    h, CFL, dtmax = 10.0 / Nz, 0.5, 1e32
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    arrs = _random_fields(Nz, Nx, seed=Nz + Nx)
    got1 = _raw_noalloc_dt(arrs, Nz, Nx, h, CFL, dtmax, 1.0, out)
    assert got1 == _oracle_dt(arrs, h, CFL, dtmax, 1.0)
    arrs[3].view(-1)[arrs[3].numel() // 2] = -40.0   # a faster U phase speed mid-array
    got2 = _raw_noalloc_dt(arrs, Nz, Nx, h, CFL, dtmax, 1.0, out)
    assert got2 == _oracle_dt(arrs, h, CFL, dtmax, 1.0)
    assert got2 < got1


def test_noalloc_dt_nan_gives_nan_like_update_dt():
    """Julia's maximum propagates NaN, so a NaN speed gives a NaN step (CUDA's
    fmax would have dropped it)."""
    Nz, Nx = 96, 80
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    arrs = _random_fields(Nz, Nx, seed=3)
    arrs[2].view(-1)[777] = float("nan")
    got = _raw_noalloc_dt(arrs, Nz, Nx, 0.1, 0.5, 1e32, 1.0, out)
    assert np.isnan(got) and np.isnan(_oracle_dt(arrs, 0.1, 0.5, 1e32, 1.0))
