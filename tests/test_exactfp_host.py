"""The integer-pipe IEEE routines of rebound_gb300/csrc/exactfp.cuh (non-negative
add, multiply, square, divide, square root, and the power-of-two
scaled comparison of the tree opening test), compiled for the host and compared
bit for bit with the host's IEEE double arithmetic over random operands in six
classes: wide exponents, cancellation, sparse significands (exact and tie
cases), exponent gaps near the significand width, range ends (zeros,
subnormals, overflow, infinities, NaN) and the tree walk's coordinate ranges.
The device build of the same source is checked against the GPU's own FP64
instructions by rgpu_selftest_exactfp (tests/test_gravity_gpu.py)."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO


@pytest.mark.parametrize("seed", [1, 20260])
def test_exactfp_matches_host_ieee(tmp_path, seed):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "exactfp_host")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                           "-I" + os.path.join(REPO, "rebound_gb300", "csrc"),
                           os.path.join(REPO, "tests", "exactfp", "exactfp_host.cpp"), "-o", exe])
    out = subprocess.run([exe, "1000000", str(seed)], capture_output=True, text=True, timeout=300)
    rows = {}
    for ln in out.stdout.splitlines():
        f = ln.split()
        if len(f) == 3 and f[1].isdigit():
            rows[f[0]] = (int(f[1]), int(f[2]))
    assert set(rows) == {"add_pos_rn", "mul_rn", "sqr_rn", "div_rn", "sqrt_rn",
                         "gt_scaled_pow2"}, out.stdout
    for name, (n, bad) in rows.items():
        assert n >= 5_000_000 and bad == 0, (name, n, bad, out.stdout)
    assert out.returncode == 0
