"""Julia's Float64 max / min semantics, which the device helpers (jmax / jmin
of the library's internal header) and the oracle both follow: a NaN argument
gives NaN, and -0.0 < +0.0, so max(0.0, -0.0) is +0.0 and min(0.0, -0.0) is
-0.0 in either argument order (noise.jl:166-183 `max(zero(T), ...)`,
update.jl:134, store.jl:65, the superbee limiter of kernels/advect.jl:279)."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

import xcore_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAN, INF = float("nan"), float("inf")

# (a, b, max(a, b), min(a, b)) as Julia gives them
CASES = [
    (0.0, -0.0, 0.0, -0.0),
    (-0.0, 0.0, 0.0, -0.0),
    (-0.0, -0.0, -0.0, -0.0),
    (0.0, 0.0, 0.0, 0.0),
    (1.0, 2.0, 2.0, 1.0),
    (2.0, 1.0, 2.0, 1.0),
    (NAN, 1.0, NAN, NAN),
    (1.0, NAN, NAN, NAN),
    (INF, INF, INF, INF),
    (-INF, 1.0, 1.0, -INF),
    (-1.0, -0.0, -0.0, -1.0),
    (0.0, -1e-300, 0.0, -1e-300),
]


def same(x, y):
    """Equal as Julia's isequal: NaN equals NaN, -0.0 differs from +0.0."""
    x, y = float(x), float(y)
    if math.isnan(x) or math.isnan(y):
        return math.isnan(x) and math.isnan(y)
    return x == y and math.copysign(1.0, x) == math.copysign(1.0, y)


@pytest.mark.parametrize("a,b,mx,mn", CASES)
def test_oracle_max_min_follow_julia(a, b, mx, mn):
    assert same(O.jl_max(a, b), mx)
    assert same(O.jl_min(a, b), mn)
    assert same(O.jmax(a, b), mx)
    assert same(O.jmin(a, b), mn)


def test_oracle_max_min_broadcast():
    a = np.array([0.0, -0.0, 3.0, NAN, -2.0])
    got = O.jl_max(0.0, a)
    for g, w in zip(got, [0.0, 0.0, 3.0, NAN, 0.0]):
        assert same(g, w)
    got = O.jl_min(a, -0.0)
    for g, w in zip(got, [-0.0, -0.0, -0.0, NAN, -2.0]):
        assert same(g, w)


def test_oracle_array_reductions_follow_julia():
    assert same(O.jl_maximum(np.array([-0.0, 0.0, -0.0])), 0.0)
    assert same(O.jl_maximum(np.array([-0.0, -0.0])), -0.0)
    assert same(O.jl_minimum(np.array([0.0, -0.0, 0.0])), -0.0)
    assert same(O.jl_minimum(np.array([0.0, 0.0])), 0.0)
    assert same(O.jl_maximum(np.array([1.0, NAN, 2.0])), NAN)
    assert same(O.jl_minimum(np.array([1.0, NAN, 2.0])), NAN)
    assert same(O.jl_maximum(np.array([-3.0, 7.5, 2.0])), 7.5)
    assert same(O.jl_minimum(np.array([-3.0, 7.5, 2.0])), -3.0)


PROBE = r"""
#include <cstdio>
#include <cstring>
#include "xc_internal.cuh"
static unsigned long long bits(double v) { unsigned long long u; std::memcpy(&u, &v, 8); return u; }
int main(int argc, char** argv) {
  for (int k = 1; k + 1 < argc; k += 2) {
    double a, b;
    unsigned long long ua = std::strtoull(argv[k], nullptr, 16), ub = std::strtoull(argv[k + 1], nullptr, 16);
    std::memcpy(&a, &ua, 8);
    std::memcpy(&b, &ub, 8);
    std::printf("%016llx %016llx\n", bits(jmax(a, b)), bits(jmin(a, b)));
  }
  return 0;
}
"""


def _bits(v):
    return "%016x" % np.array([v], dtype=np.float64).view(np.uint64)[0]


def _from_bits(h):
    return float(np.array([int(h, 16)], dtype=np.uint64).view(np.float64)[0])


def test_library_helpers_follow_julia(tmp_path):
    """The library's jmax / jmin, compiled for the host from the same header
    the kernels include (the device build differs only in how it reads the
    sign bit)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "minmax_probe.cu"
    src.write_text(PROBE)
    exe = tmp_path / "minmax_probe"
    csrc = os.path.join(ROOT, "xcore.jl_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "-I", csrc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    args = [h for a, b, _, _ in CASES for h in (_bits(a), _bits(b))]
    out = subprocess.run([str(exe)] + args, check=True, capture_output=True, text=True).stdout.split("\n")
    for (a, b, mx, mn), line in zip(CASES, out):
        gmx, gmn = line.split()
        assert same(_from_bits(gmx), mx), (a, b)
        assert same(_from_bits(gmn), mn), (a, b)
