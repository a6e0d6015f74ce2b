"""The float-float arithmetic of the complex128 fast path (ff.cuh) on the
host: tests/ff_host/ff_check.cpp is compiled with g++ (contraction off) and
compared with long double on seeded operands.  The bounds are what the 1e-12
complex128 parity bar rests on: about 2^-45 per float-float step, so a few
thousand gate applications stay far below 1e-12.  The packed f32x2 policy
runs these operation sequences lane by lane; its results are checked against
the oracle on the GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "ff_host", "ff_check.cpp")

BOUNDS = {
    "from_double": 2.0 ** -47,  # lo keeps 24 of the 29 low bits
    "mul": 2.0 ** -45,
    "dot2": 2.0 ** -44,
    "add": 2.0 ** -45,
}


def test_float_float_error_bounds(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ff_check")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", SRC, "-o", exe, "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "200000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in r.stdout.split("\n"):
        if line.strip():
            k, v = line.split()
            got[k] = float(v)
    assert got["to_double_mismatches"] == 0
    for k, bound in BOUNDS.items():
        assert 0 < got[k] <= bound, (k, got[k], bound)
