"""The checkpoint groups name fields the library holds, once each, in the
reference's groups (src/restart.jl:53-83; FluidState src/state.jl:74-122,
PhaseState src/state.jl:165-258, noise_dynamic_fields src/restart.jl:25-28)."""
import xcore_gb300 as xc


def test_checkpoint_groups_are_registry_fields():
    reg = set(xc.field_names())
    seen = []
    for group, names in xc.CHECKPOINT_GROUPS.items():
        assert set(names) <= reg, (group, sorted(set(names) - reg))
        seen += names
    assert len(seen) == len(set(seen))
    assert {g: len(n) for g, n in xc.CHECKPOINT_GROUPS.items()} == {"fluid": 19, "phase": 76, "noise": 17}
    # everything else the context holds is derived scratch of one step
    assert sorted(reg - set(seen)) == ["res_MFSo", "res_Po", "res_Uo", "res_Wo", "res_Xo"]
