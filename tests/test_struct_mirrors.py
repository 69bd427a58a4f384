"""The structs of the C ABI and their mirrors agree: the Python ctypes classes
(field names, order, offsets and size, against a C probe compiled with gcc
from the header) and the Julia binding's structs (field names, order and
types, and the short SolverOpts constructor's zero padding)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

import xcore_gb300 as xc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xcore_gb300.h")
JULIA = os.path.join(ROOT, "xcore.jl_gb300", "julia", "XcoreGPU.jl")
BUILD = os.path.join(ROOT, "xcore.jl_gb300", "_build")

# C typedef name -> (ctypes class, Julia struct name or None)
MIRRORS = {
    "xc_params": (xc._Params, "XcParams"),
    "xc_solver_opts": (xc.SolverOpts, "SolverOpts"),
    "xc_solver_stats": (xc.SolverStats, "SolverStats"),
    "xc_step_stats": (xc.StepStats, "StepStats"),
}


def c_fields(name):
    """[(field, ctype, count)] of `typedef struct name {...} name;` in the header."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for k, v in re.findall(r"^#define (\w+) (\d+)$", src, flags=re.M):
        src = re.sub(r"\b%s\b" % k, v, src)
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S)
    assert m, name
    out = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        for item in names.split(","):
            item = item.strip()
            a = re.match(r"(\w+)(?:\[(\d+)\])?$", item)
            assert a, item
            out.append((a.group(1), ctype, int(a.group(2) or 1)))
    return out


@pytest.fixture(scope="module")
def c_layout():
    """sizeof and offsetof of every mirrored struct, from gcc on the header."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    os.makedirs(BUILD, exist_ok=True)
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "xcore_gb300.h"', "int main(void) {"]
    for name in MIRRORS:
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f, _, _ in c_fields(name):
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines += ["  return 0;", "}"]
    probe = os.path.join(BUILD, "struct_probe.c")
    exe = os.path.join(BUILD, "struct_probe")
    with open(probe, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), probe, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    layout = {}
    for line in out.splitlines():
        s, f, v = line.split()
        layout[(s, f)] = int(v)
    return layout


@pytest.mark.parametrize("name", list(MIRRORS))
def test_ctypes_mirror_matches_the_header(name, c_layout):
    cls = MIRRORS[name][0]
    fields = c_fields(name)
    assert [f for f, _, _ in fields] == [f for f, _ in cls._fields_]
    for f, _, _ in fields:
        assert getattr(cls, f).offset == c_layout[(name, f)], (name, f)
    assert ctypes.sizeof(cls) == c_layout[(name, "size")], name


def julia_fields(struct):
    src = re.sub(r"#.*", "", open(JULIA).read())
    m = re.search(r"^(?:mutable )?struct %s\s*\n(.*?)^end" % struct, src, flags=re.S | re.M)
    assert m, struct
    out = []
    for item in re.split(r"[;\n]", m.group(1)):
        item = item.strip()
        if item:
            f, t = item.split("::")
            out.append((f.strip(), t.strip()))
    return out


@pytest.mark.parametrize("name", [n for n, (_, j) in MIRRORS.items() if j])
def test_julia_mirror_matches_the_header(name):
    jl = julia_fields(MIRRORS[name][1])
    want = []
    for f, ctype, count in c_fields(name):
        base = {"int": "Cint", "double": "Cdouble"}[ctype]
        want.append((f, base if count == 1 else "NTuple{%d,%s}" % (count, base)))
    assert jl == want


def test_julia_short_solver_opts_constructor_pads_every_field():
    src = open(JULIA).read()
    m = re.search(r"SolverOpts\(kind, rtol, maxit, restart, inner_rtol, inner_maxit\) =\s*\n\s*SolverOpts\((.*?)\)\n",
                  src)
    assert m
    args = [a.strip() for a in m.group(1).split(",")]
    assert len(args) == len(c_fields("xc_solver_opts"))


def test_julia_solver_opts_calls_have_six_or_all_arguments():
    """Every SolverOpts(...) call of the binding passes the 6 leading fields
    (the short constructor) or every field of xc_solver_opts."""
    src = re.sub(r"#.*", "", open(JULIA).read())
    n = len(c_fields("xc_solver_opts"))
    calls = re.findall(r"SolverOpts\(([^()]*)\)", src)
    assert calls
    for args in calls:
        k = len([a for a in args.split(",") if a.strip()])
        assert k in (6, n), (k, args)


def _julia_extension_methods():
    """(name, positional arguments) of every method the binding adds to a
    function of the xcore module (`function xcore.f(...)` or `xcore.f(...) =`)."""
    src = re.sub(r"#.*", "", open(JULIA).read())
    out = []
    for m in re.finditer(r"(?:^function\s+|^)xcore\.(\w+!?)\(", src, flags=re.M):
        depth, k = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(src[k], 0)
            k += 1
        args = src[m.end():k - 1].split(";")[0]
        out.append((m.group(1), [a.strip() for a in args.split(",") if a.strip()]))
    return out


def test_julia_gpu_methods_type_every_positional_argument():
    """A GPU method that leaves a positional argument untyped ties with the
    reference's own method (which types every one) and makes the call
    ambiguous; each must be strictly more specific."""
    methods = _julia_extension_methods()
    assert {n for n, _ in methods} >= {"store_previous!", "snapshot!", "phsevo!", "fluidmech!", "noise!",
                                       "update_phase_velocities!", "update!", "compute_resnorm", "update_dt",
                                       "record_history!"}
    for name, args in methods:
        assert args, name
        for a in args:
            assert "::" in a, (name, a)
        assert any(a.endswith(("::GPUPhase", "::GPUFluid")) for a in args), name
