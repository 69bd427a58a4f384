"""Helpers for the GPU parity tests: build a realistic oracle state, mirror it
into a device context, and compare fields."""
import numpy as np

import xcore_oracle as O
import xcore_gb300 as xc


def oracle_params(N=24, Nx=20, **kw):
    D = 10.0
    h = D / N
    base = dict(D=D, N=N, L=Nx * h, etam0=10.0, x0=0.05, dxr=0.1, Da=0.01, TINT="bd2im", ADVN="weno5",
                alpha=0.5, L0=3 * h, l0=3 * h, etacntr=1e3)
    base.update(kw)
    return O.Params(**base)


def product_params(op: O.Params) -> xc.Parameters:
    keys = [k for k in xc.Parameters.__dataclass_fields__ if hasattr(op, k)]
    return xc.Parameters(**{k: getattr(op, k) for k in keys})


def realistic_state(N=24, Nx=20, steps=2, seed=7, **kw):
    """Oracle state after initialize! and `steps` time steps."""
    par = oracle_params(N, Nx, **kw)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(seed)
    x0 = np.clip(rng.uniform(0.02, 0.10, (g.Nz, g.Nx)), 0, 1)
    st = O.initialize(g, par, sc, ns, x0, rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx)))
    dt = sc["dt0"]
    for step in range(1, steps + 1):
        dt, _ = O.timestep(st, g, par, sc, ns, step, dt, rng.standard_normal((g.Nz, g.Nx)),
                           rng.standard_normal((g.Nz, g.Nx)))
    return par, g, sc, ns, st, dt, rng


def device_state(par, g, sc, st=None, **kw):
    s = xc.State(product_params(par), grid=xc.Grid(Nx=g.Nx, Nz=g.Nz, h=g.h, D=g.D, L=g.L), scales=sc, **kw)
    if st is not None:
        upload_all(s, st)
    return s


def upload_all(ds, st):
    for name in xc.field_names():
        if name.startswith("res_"):
            continue
        if hasattr(st, name):
            ds[name] = getattr(st, name)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def assert_fields(ds, st, names, exact=False, tol=1e-12):
    bad = []
    for n in names:
        got = ds[n]
        ref = getattr(st, n)
        if exact:
            if not np.array_equal(got, ref):
                bad.append((n, float(np.abs(got - ref).max()), rel_err(got, ref)))
        else:
            e = rel_err(got, ref)
            if not e <= tol:
                bad.append((n, e))
    assert not bad, bad
