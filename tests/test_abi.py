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
