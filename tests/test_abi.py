"""The C-ABI library (built on CPU here) loads, exports every entry point the
header declares, and reports errors without a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

import xcore_gb300 as xc
import xcore_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xcore_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xc_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    xc.build()
    return xc.lib()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", xc.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (xc_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_field_registry_matches_reference_state(lib):
    names = xc.field_names()
    shapes = O.field_shapes(8, 6)
    for n in shapes:
        assert n in names, n
    assert len(set(names)) == len(names)
    assert lib.xc_field_id(b"W") == names.index("W")
    assert lib.xc_field_id(b"nope") == -1


def test_time_coefs_through_abi():
    for tint in ("be1im", "bd2im", "cn2si", "bd2si"):
        for step in (1, 2, 3, 7):
            assert xc.time_coefs(tint, step) == O.time_coefs(tint, step)
    out = (ctypes.c_double * 6)()
    assert xc.lib().xc_time_coefs(9, 1, out) == xc.XC_BAD_ARG


def test_context_creation_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(xc.XcoreError) as e:
        xc.State(xc.Parameters(N=16))
    assert e.value.status == xc.XC_NO_DEVICE


def test_bad_parameters_rejected_before_any_device_work():
    with pytest.raises(xc.XcoreError) as e:
        xc.State(xc.Parameters(N=2))
    assert e.value.status == xc.XC_BAD_ARG


def test_ensemble_arguments_rejected_before_any_device_work(lib):
    out = ctypes.c_void_p()
    assert lib.xc_ensemble_create(None, 0, 0, ctypes.byref(out)) == xc.XC_BAD_ARG
    members = (ctypes.c_void_p * 2)(None, None)
    assert lib.xc_ensemble_create(members, 2, 0, ctypes.byref(out)) == xc.XC_BAD_ARG
    assert b"null" in lib.xc_last_error()
    assert lib.xc_ensemble_create(members, 2, -1, ctypes.byref(out)) == xc.XC_BAD_ARG
    steps, dts = (ctypes.c_int * 1)(1), (ctypes.c_double * 1)(1e-3)
    assert lib.xc_ensemble_step(None, steps, dts, 3, None, None, None, None) == xc.XC_BAD_ARG
    assert lib.xc_ensemble_destroy(None) == xc.XC_OK


def _registry_shapes(Nz, Nx):
    """The library's field registry (the XC_FIELDS table of its internal
    header) as {name: (rows, cols)} for an Nz x Nx grid."""
    src = open(os.path.join(ROOT, "xcore.jl_gb300", "csrc", "xc_internal.cuh")).read()
    body = src[src.index("#define XC_FIELDS(F)"):src.index("enum FieldId")]
    dims = {"SH_C": (0, 0), "SH_ZF": (1, 0), "SH_XF": (0, 1), "SH_W": (1, 2), "SH_U": (2, 1), "SH_CO": (1, 1),
            "SH_P": (2, 2)}
    out = {}
    for name, code, _eb in re.findall(r"F\((\w+), (SH_\w+), (\d)\)", body):
        dz, dx = dims[code]
        out[name] = (Nz + dz, Nx + dx)
    return out


def test_registry_sizes_are_the_reference_sizes():
    """Every field the library allocates has the reference's size: the
    oracle's table of FluidState / PhaseState / NoiseState (state.jl:101-122,
    218-258; noise.jl:82-92), the StepResidual buffers of
    test/test_diagnose.jl:18-33 and the NoiseState sizes of
    test/test_noise.jl:21-43."""
    Nz, Nx = 10, 7
    reg = _registry_shapes(Nz, Nx)
    assert len(reg) == len(xc.field_names())
    ref = O.field_shapes(Nz, Nx)
    for name, shp in ref.items():
        assert reg[name] == shp, name
    residual = {"res_Wo": (Nz + 1, Nx + 2), "res_Uo": (Nz + 2, Nx + 1), "res_Po": (Nz + 2, Nx + 2),
                "res_Xo": (Nz, Nx), "res_MFSo": (Nz, Nx)}
    noise = {"psie": (Nz, Nx), "psieo": (Nz, Nx), "re": (Nz, Nx), "rs": (Nz, Nx), "xiew": (Nz + 1, Nx + 2),
             "xieu": (Nz + 2, Nx + 1), "xixw": (Nz + 1, Nx + 2), "xixu": (Nz + 2, Nx + 1),
             "xisw": (Nz + 1, Nx + 2), "xisu": (Nz + 2, Nx + 1), "xie": (Nz, Nx), "xix": (Nz, Nx),
             "xis": (Nz, Nx)}
    for name, shp in {**residual, **noise}.items():
        assert reg[name] == shp, name
