"""The learned preconditioner end to end on the GPU, through the C ABI:
training pairs from the plain FP64 solver (xc_learned_sample), training by
the library's own BF16 tcgen05 forward and backward kernels, and use inside
the mixed solver -- in place of the multigrid V-cycle (learned = 1) and after
it (learned = 2).

The multigrid stays fallback and judge: a learned inner solve that misses its
reduction is redone with the multigrid, a learned refinement pass that does
not halve the FP64 residual is undone and the multigrid takes the rest of the
solve, and every solve must reach the same FP64 relative residual (1e-9) and
the same solution as the multigrid-preconditioned one.  What training gains
is measured on held-out pairs: the trained network's correction points along
the plain solver's (cosine) better than an untrained network of the same
architecture."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402
import xcore_gb300.learned as L  # noqa: E402

N = 128


@pytest.fixture(scope="module")
def pairs():
    inp, tgt = L.generate(N, 320, per_field=16, seed=3, after_vcycle=True)
    return inp[:256].contiguous(), tgt[:256].contiguous(), inp[256:].contiguous(), tgt[256:].contiguous()


@pytest.fixture(scope="module")
def trained(pairs):
    inp, tgt, _, _ = pairs
    net = L.Network(N, N, 8, seed=1)
    losses = L.train(net, inp, tgt, steps=800, lr=2e-3, seed=1)
    params = net.params()
    net.close()
    untrained = L.Network(N, N, 1, seed=1)
    p0 = untrained.params()
    untrained.close()
    return params, p0, losses


@pytest.mark.parametrize("after_vcycle", [0, 1])
def test_samples(after_vcycle):
    """A pair's input holds the right-hand side at unit norm (times sqrt(N^2))
    and log10(eta / etam0); the target is finite and not zero."""
    st, coefs, dt = L.workload_state(N, seed=5)
    st.fluidmech(coefs, dt, solver="fgmres64", rtol=1e-8, maxit=600)
    gen = torch.Generator(device="cuda").manual_seed(0)
    v = L.staggered_vector(torch, gen, N, N, torch.device("cuda"), 4.0)
    inp = torch.empty((N, N, 4), device="cuda")
    tgt = torch.empty((N, N, 3), device="cuda")
    its = ctypes.c_int()
    xc._check(xc.lib().xc_learned_sample(st._h, ctypes.c_void_p(v.data_ptr()), after_vcycle,
                                         ctypes.c_void_p(inp.data_ptr()), ctypes.c_void_p(tgt.data_ptr()), 1e-8,
                                         600, ctypes.byref(its)))
    assert its.value > 0
    assert torch.isfinite(inp).all() and torch.isfinite(tgt).all() and tgt.abs().max() > 0
    assert 0.2 < float(inp[..., :3].pow(2).mean().sqrt()) < 5.0
    np.testing.assert_allclose(inp[..., 3].cpu().numpy(), np.log10(st["eta"] / st.par.etam0), rtol=1e-6,
                               atol=1e-6)
    st.close()


def _cosine(params, inp, tgt):
    net = L.Network(N, N, inp.shape[0], seed=0)
    net.set_params(params)
    out = torch.empty_like(tgt)
    net.forward(inp, out)
    net.close()
    a, b = out.reshape(out.shape[0], -1), tgt.reshape(tgt.shape[0], -1)
    return float(((a * b).sum(1) / (a.norm(dim=1) * b.norm(dim=1)).clamp_min(1e-30)).mean())


def test_training_gains_over_the_untrained_network(trained, pairs):
    params, p0, losses = trained
    _, _, hin, htg = pairs
    first, last = np.mean(losses[:30]), np.mean(losses[-30:])
    c_trained, c_untrained = _cosine(params, hin, htg), _cosine(p0, hin, htg)
    print(f"learned preconditioner: training loss {first:.4f} -> {last:.4f} (predicting zero: 3.0); held-out "
          f"cosine with the plain solver's correction: trained {c_trained:.3f}, untrained {c_untrained:.3f}")
    assert last < first
    assert c_trained > c_untrained + 0.05


@pytest.mark.parametrize("mode", [1, 2])
def test_learned_solve_reaches_the_multigrid_solution(trained, mode):
    params, p0, _ = trained
    st, coefs, dt = L.workload_state(N, seed=9)
    snap = {k: st[k] for k in ("W", "U", "P", "MFS", "drhodt")}
    ref = st.fluidmech(coefs, dt, **L.SOLVE)
    Wr, Ur, Pr = st["W"], st["U"], st["P"]
    results = {}
    for name, p in (("trained", params), ("untrained", p0)):
        L.use(st, p)
        for k, v in snap.items():
            st[k] = v
        info = st.fluidmech(coefs, dt, learned=mode, **L.SOLVE)
        assert info["converged"] and info["rel_residual"] <= 1e-9, (name, info)
        for k, r in (("W", Wr), ("U", Ur), ("P", Pr)):
            e = float(np.abs(st[k] - r).max() / np.abs(r).max())
            assert e <= 1e-6, (name, k, e)
        results[name] = info
    print(f"mode {mode}: multigrid {ref['iterations']} inner iterations; trained "
          f"{results['trained']['iterations']} ({results['trained']['learned_fallbacks']} fallbacks); untrained "
          f"{results['untrained']['iterations']} ({results['untrained']['learned_fallbacks']} fallbacks)")
    st.close()


def test_learned_option_needs_a_network():
    st, coefs, dt = L.workload_state(N, seed=2)
    with pytest.raises(xc.XcoreError):
        st.fluidmech(coefs, dt, learned=1, **{k: v for k, v in L.SOLVE.items()})
    with pytest.raises(xc.XcoreError):
        L.use(st, np.zeros(10, dtype=np.float32))
    st.close()
