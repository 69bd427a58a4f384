"""The learned preconditioner end to end on the GPU, through the C ABI:
training pairs from the plain FP64 solver (xc_learned_sample), training by
the library's own BF16 tcgen05 forward and backward kernels, and use inside
the mixed solver -- in place of the multigrid V-cycle with the multigrid as
fallback (learned = 1), and after the V-cycle (learned = 2).

The multigrid stays the judge: every learned solve must reach the same FP64
relative residual (1e-9) and the same solution as the plain mixed solve.
What the trained network gains is measured against the same solve with an
untrained network of identical architecture: the trained one must redo fewer
inner solves with the multigrid (mode 1) and need no more inner iterations
(mode 2)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402
import xcore_gb300.learned as L  # noqa: E402

N = 128


@pytest.fixture(scope="module")
def trained():
    inp, tgt = L.generate(N, 256, per_field=16, seed=3)
    net = L.Network(N, N, 8, seed=1)
    losses = L.train(net, inp, tgt, steps=600, lr=2e-3, seed=1)
    params = net.params()
    untrained = L.Network(N, N, 1, seed=1).params()
    net.close()
    return params, untrained, losses


def test_samples_solve_the_system():
    """A training pair's target solves S LL S z = v: applying the operator to
    the target's interior part reproduces v on the interior rows up to the
    boundary rows' share."""
    st, coefs, dt = L.workload_state(N, seed=5)
    st.fluidmech(coefs, dt, solver="fgmres64", rtol=1e-8, maxit=600)
    gen = torch.Generator(device="cuda").manual_seed(0)
    v = L.staggered_vector(torch, gen, N, N, torch.device("cuda"), 4.0)
    inp = torch.empty((N, N, 4), device="cuda")
    tgt = torch.empty((N, N, 3), device="cuda")
    its = ctypes.c_int()
    xc._check(xc.lib().xc_learned_sample(st._h, ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(inp.data_ptr()),
                                         ctypes.c_void_p(tgt.data_ptr()), 1e-8, 600, ctypes.byref(its)))
    assert its.value > 0
    # the input holds v at unit norm scaled by sqrt(N^2), and log10(eta/etam0)
    vin = inp[..., :3]
    assert torch.isfinite(inp).all() and torch.isfinite(tgt).all()
    assert 0.2 < float(vin.pow(2).mean().sqrt()) < 5.0
    eta = st["eta"]
    np.testing.assert_allclose(inp[..., 3].cpu().numpy(), np.log10(eta / st.par.etam0), rtol=1e-6, atol=1e-6)
    st.close()


def test_training_reduces_the_loss(trained):
    params, untrained, losses = trained
    first, last = np.mean(losses[:30]), np.mean(losses[-30:])
    print(f"learned preconditioner training loss {first:.4f} -> {last:.4f}")
    assert last < 0.7 * first


@pytest.mark.parametrize("mode", [1, 2])
def test_learned_solve_reaches_the_multigrid_solution(trained, mode):
    params, untrained, _ = trained
    st, coefs, dt = L.workload_state(N, seed=9)
    snap = {k: st[k] for k in ("W", "U", "P", "MFS", "drhodt")}
    ref = st.fluidmech(coefs, dt, solver="mixed", rtol=1e-9, maxit=600, inner_rtol=5e-2, inner_maxit=30,
                       pressure_sweeps=1)
    Wr, Ur, Pr = st["W"], st["U"], st["P"]
    results = {}
    for name, p in (("trained", params), ("untrained", untrained)):
        L.use(st, p)
        for k, v in snap.items():
            st[k] = v
        info = st.fluidmech(coefs, dt, solver="mixed", rtol=1e-9, maxit=600, inner_rtol=5e-2, inner_maxit=30,
                            pressure_sweeps=1, learned=mode)
        assert info["converged"] and info["rel_residual"] <= 1e-9, (name, info)
        for k, r in (("W", Wr), ("U", Ur), ("P", Pr)):
            e = float(np.abs(st[k] - r).max() / np.abs(r).max())
            assert e <= 1e-6, (name, k, e)
        results[name] = info
    print(f"mode {mode}: multigrid {ref['iterations']} inner iterations; trained "
          f"{results['trained']['iterations']} ({results['trained']['learned_fallbacks']} fallbacks); untrained "
          f"{results['untrained']['iterations']} ({results['untrained']['learned_fallbacks']} fallbacks)")
    if mode == 1:
        assert results["trained"]["learned_fallbacks"] <= results["untrained"]["learned_fallbacks"]
    else:
        assert results["trained"]["iterations"] <= results["untrained"]["iterations"]
    st.close()


def test_learned_option_needs_a_network():
    st, coefs, dt = L.workload_state(N, seed=2)
    with pytest.raises(xc.XcoreError):
        st.fluidmech(coefs, dt, solver="mixed", rtol=1e-9, learned=1)
    with pytest.raises(xc.XcoreError):
        L.use(st, np.zeros(10, dtype=np.float32))
    st.close()
