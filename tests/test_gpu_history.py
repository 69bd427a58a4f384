"""record_history! field statistics on the device (src/history.jl:183-222)
against the oracle."""
import pytest

import xcore_oracle as O
from gpu_helpers import device_state, realistic_state

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")


def test_history_stats_match_oracle():
    par, g, sc, ns, st, dt, rng = realistic_state(N=40, Nx=36, steps=2)
    ds = device_state(par, g, sc, st)
    got = ds.history_stats()
    ref = O.history_stats(st)
    assert set(got) == set(ref)
    for k, v in ref.items():
        assert got[k] == pytest.approx(v, rel=1e-12, abs=1e-300), k
