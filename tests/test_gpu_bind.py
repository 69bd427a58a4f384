"""xc_field_bind: the library working in place on the caller's device arrays
(the zero-copy form of the drop-in, e.g. CuArrays of the reference's
FluidState / PhaseState).  A context whose fields are bound to torch tensors
must step bit-identically to one that keeps its own copies, and the results
must land in the caller's tensors."""
import numpy as np
import pytest

import xcore_oracle as O  # noqa: F401  (conftest path)
from gpu_helpers import device_state, realistic_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402

BOUND = ("W", "U", "P", "eta", "etaco", "rho", "X", "M", "x", "m", "kx", "Wx", "Ux", "hasx", "psie", "MFS")


def _tensor_of(ds, name):
    a = ds[name]
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.uint8 if a.dtype == bool else np.float64).T))
    return t.cuda()


def test_bound_fields_step_like_own_copies():
    par, g, sc, ns, st, dt, rng = realistic_state(N=32, Nx=40, steps=1)
    own = device_state(par, g, sc, st)
    bound = device_state(par, g, sc, st)
    tensors = {n: _tensor_of(bound, n) for n in BOUND}
    for n, t in tensors.items():
        bound.bind(n, t)
    draws = [(rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))) for _ in range(2)]
    for k, (re, rs) in enumerate(draws):
        a = own.step(2 + k, dt, re, rs, sweeps=3, rtol=1e-11, maxit=1500)
        b = bound.step(2 + k, dt, re, rs, sweeps=3, rtol=1e-11, maxit=1500)
        assert a["dt_next"] == b["dt_next"] and a["resnorm"] == b["resnorm"]
    for n, t in tensors.items():
        got = t.cpu().numpy().T
        ref = own[n]
        assert np.array_equal(got.astype(ref.dtype) if ref.dtype == bool else got, ref), n
        assert np.array_equal(bound[n], ref), n   # downloads read the bound array too
    # unbinding returns to the context's own (stale) copy
    bound.bind("W", None)
    assert not np.array_equal(bound["W"], own["W"])


def test_bind_rejects_bad_pointers():
    par, g, sc, ns, st, dt, rng = realistic_state(N=24, Nx=20, steps=0)
    ds = device_state(par, g, sc, st)
    host = torch.zeros((22, 25), dtype=torch.float64)
    with pytest.raises(ValueError):
        ds.bind("W", torch.zeros((3, 3), dtype=torch.float64, device="cuda"))
    with pytest.raises(xc.XcoreError):
        xc._check(xc.lib().xc_field_bind(ds._h, xc.field_names().index("W"), xc.ctypes.c_void_p(host.data_ptr())))
