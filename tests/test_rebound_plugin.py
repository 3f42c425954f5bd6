"""The REBOUND-side plugin (rebound_gb300/plugin/rgpu_rebound.c), compiled against
REBOUND's own header and linked with REBOUND's own library.

The reference's C core is built into oracle/_ref/ by oracle/ref.mk from the
sources named by the REBOUND_REFERENCE environment variable or recorded in
oracle/_ref/reference_path by the build step; without them these tests skip.

* With a test double of the C ABI (tests/plugin/fake_rgpu.c) whose "device" is a
  private REBOUND simulation running REBOUND's built-in integrators, the plugin
  must reproduce the built-in integrator bit for bit through REBOUND's own
  integrate and steps loops: leapfrog with a shortened last step, modified /
  added / removed particles and a periodic boundary the plugin holds for the
  device and hands back; WHFast on the outer solar system (its synchronize on
  exit and before the shortened last step).
* Linked with the real librebound_gb300: on a machine without a GPU,
  reb_simulation_integrate must end with REB_STATUS_GENERIC_ERROR and the
  library's error in REBOUND's message list (no crash); with a GPU it must track
  the built-in leapfrog.
"""
import glob
import os
import subprocess

import pytest

from conftest import REPO

REB_STATUS_SUCCESS, REB_STATUS_GENERIC_ERROR = 0, 1


def reference_src():
    path = os.environ.get("REBOUND_REFERENCE")
    if not path:
        rec = os.path.join(REPO, "oracle", "_ref", "reference_path")
        if os.path.exists(rec):
            path = open(rec).read().strip()
    if not path or not os.path.exists(os.path.join(path, "src", "rebound.h")):
        pytest.skip("REBOUND's sources are not available on this machine")
    return os.path.join(path, "src")


def reference_lib():
    libs = [p for p in glob.glob(os.path.join(REPO, "oracle", "_ref", "librebound*.so"))
            if not p.endswith(("_omp.so", "_quad.so"))]
    if not libs:
        pytest.skip("the reference library has not been built (oracle/ref.mk)")
    return libs[0]


def build_driver(tmp_path, backend):
    src = reference_src()
    lib = reference_lib()
    exe = str(tmp_path / "driver")
    cmd = ["gcc", "-std=c99", "-O1", "-D_GNU_SOURCE", "-Wall", "-Werror=implicit-function-declaration",
           "-I" + src, "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(REPO, "rebound_gb300", "plugin"),
           os.path.join(REPO, "tests", "plugin", "plugin_driver.c"),
           os.path.join(REPO, "rebound_gb300", "plugin", "rgpu_rebound.c")] + backend + [
           lib, "-lm", "-o", exe]
    subprocess.check_call(cmd)
    return exe


def run(exe, *args):
    env = dict(os.environ)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    env["LD_LIBRARY_PATH"] = os.path.join(cuda, "lib64") + ":" + env.get("LD_LIBRARY_PATH", "")
    out = subprocess.run([exe, *args], capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout.splitlines()


def parse(lines):
    status, diff, extra = {}, {}, {}
    for ln in lines:
        f = ln.split()
        if f[0] == "STATUS":
            status[f[1]] = (int(f[2]), int(f[3]))
        elif f[0] == "DIFF":
            diff[f[1]] = (float(f[2]), float(f[3]))
        else:
            extra[f[0]] = f[1:]
    return status, diff, extra


def test_plugin_reproduces_builtin_leapfrog_through_rebound_loops(tmp_path):
    exe = build_driver(tmp_path, [os.path.join(REPO, "tests", "plugin", "fake_rgpu.c")])
    status, diff, extra = parse(run(exe))
    assert "DONE" in extra, (status, diff, extra)
    for phase in ("integrate", "modified", "added", "removed", "steps", "periodic", "builtin_again"):
        assert status[phase] == (REB_STATUS_SUCCESS, REB_STATUS_SUCCESS) or phase == "steps", (phase, status[phase])
        assert diff[phase] == (0.0, 0.0), (phase, diff[phase])
    # the plugin held the periodic boundary for the device and gave it back
    assert extra["HELD"] == ["0", "2"]
    assert extra["RETURNED"] == ["2"]


def test_plugin_reproduces_builtin_whfast(tmp_path):
    # the WHFast plugin (safe_mode 1, Jacobi) through REBOUND's integrate loop, its
    # synchronize called on exit and before the shortened last step
    exe = build_driver(tmp_path, [os.path.join(REPO, "tests", "plugin", "fake_rgpu.c")])
    status, diff, extra = parse(run(exe, "whfast"))
    assert "DONE" in extra, (status, diff, extra)
    for phase in ("whfast_integrate", "whfast_modified"):
        assert status[phase] == (REB_STATUS_SUCCESS, REB_STATUS_SUCCESS), (phase, status[phase])
        assert diff[phase] == (0.0, 0.0), (phase, diff[phase])
    ea, eb = map(float, extra["ENERGY"])
    assert ea == eb


def test_plugin_with_gpu_library(tmp_path):
    lib = os.path.join(REPO, "rebound_gb300", "librebound_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("librebound_gb300.so has not been built")
    exe = build_driver(tmp_path, [lib, "-Wl,-rpath," + os.path.dirname(lib)])
    lines = run(exe)
    status, diff, extra = parse(lines)
    if status["integrate"][1] == REB_STATUS_GENERIC_ERROR:
        # no usable GPU: the library's error reaches REBOUND's message list
        assert any(ln.startswith("ERROR rgpu: rgpu_sim_create failed") for ln in lines), lines
    else:
        assert "DONE" in extra, lines
        for phase, (dx, dt) in diff.items():
            assert dx <= 1e-12 and abs(dt) <= 1e-15, (phase, dx, dt)
