"""Ensemble of independent instances (uneven grid sizes, separate seeds)
stepped together -- one host thread and one CUDA stream per member, or one
CUDA graph launch per explicit stage for all members with the Stokes solves
on a pool of host threads: every member ends bit-identical to the same
instance stepped alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402

SIZES = [(32, 1), (48, 2), (40, 3), (64, 4), (24, 5), (56, 6)]
SOLVER = dict(sweeps=3, solver="mixed", rtol=1e-9)


def _member(N, seed):
    D = 10.0
    par = xc.Parameters(D=D, N=N, L=D, etam0=10.0, x0=0.1, Da=0.0, L0=3 * D / N, l0=3 * D / N, etacntr=1e3,
                        Xi=1e-3 * seed)
    st = xc.State(par)
    rng = np.random.default_rng(seed)
    x0 = np.clip(rng.uniform(0.02, 0.10, (N, N)), 0.0, 1.0)
    st.initialize(x0, rng.standard_normal((N, N)), rng.standard_normal((N, N)))
    draws = [(rng.standard_normal((N, N)), rng.standard_normal((N, N))) for _ in range(2)]
    return st, draws


@pytest.mark.parametrize("graphs,threads", [(False, None), (True, None), (True, 2)])
def test_ensemble_matches_members_stepped_alone(graphs, threads):
    solo = []
    for N, seed in SIZES:
        st, draws = _member(N, seed)
        dt = st.scales["dt0"]
        for k, (re, rs) in enumerate(draws):
            dt = st.step(k + 1, dt, re, rs, **SOLVER)["dt_next"]
        solo.append((st.checkpoint(), dt))
        st.close()

    members, draws = zip(*[_member(N, seed) for N, seed in SIZES])
    ens = xc.Ensemble(members, threads=threads, graphs=graphs)
    dts = [m.scales["dt0"] for m in members]
    for k in range(2):
        infos = ens.step([k + 1] * len(members), dts, [d[k] for d in draws], **SOLVER)
        dts = [i["dt_next"] for i in infos]
        assert all(i["sweeps"] == SOLVER["sweeps"] and i["solver_iterations"] > 0 for i in infos)
    for m, dt, (ref, dt_ref) in zip(members, dts, solo):
        assert dt == dt_ref
        got = m.checkpoint()
        for key, v in ref.items():
            np.testing.assert_array_equal(got[key], v, err_msg=f"N={m.grid.Nz} {key}")
    ens.close()
