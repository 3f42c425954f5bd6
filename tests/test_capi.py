"""The C-ABI library loads and exports every entry point include/*.h declares.

No compute calls are made here (this file runs without a GPU); the host-side
workload generators are checked against the reference's own draws.
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import REPO, golden


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(rgpu_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("rgpu_sim_create", "rgpu_update_acceleration", "rgpu_collision_search", "rgpu_steps",
                 "rgpu_integrate", "rgpu_energy", "rgpu_sim_set_particles", "rgpu_sim_get_particles"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import rebound_gb300
    lib = rebound_gb300.load()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_reference():
    from rebound_gb300._lib import PARTICLE_DTYPE, COLLISION_DTYPE, Config
    assert PARTICLE_DTYPE.itemsize == 112       # struct reb_particle on LP64
    assert COLLISION_DTYPE.itemsize == 72       # struct reb_collision
    assert ctypes.sizeof(Config) % 8 == 0


def test_plummer_generator_matches_reference_draws():
    import rebound_gb300 as R
    g = golden("gravity_plummer.npz")
    p = R.ics.plummer(4096, seed=int(g["plummer_seed"]))
    ref = g["particles"]
    # host libm (pow, sin, cos) may differ by an ulp between machines; the draw
    # sequence itself must match, so the bar is a few ulps of the largest value
    for f in ("x", "y", "z", "vx", "vy", "vz", "m"):
        np.testing.assert_allclose(p[f], ref[f], rtol=1e-14, atol=1e-14)
    raw = R.ics.plummer(64, seed=int(g["plummer_seed"]), rmax=1e300)
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_allclose(raw[f], g["plummer_raw"][f], rtol=1e-14, atol=1e-15)


def test_ring_patch_generator_shape():
    import rebound_gb300 as R
    p = R.ics.ring_patch(200.0, seed=7)
    ref = golden("ring_patch.npz")["particles"]
    assert len(p) == len(ref)
    for f in ("x", "y", "z", "vx", "vy", "vz", "m", "r"):
        np.testing.assert_allclose(p[f], ref[f], rtol=1e-13, atol=1e-16)


def test_planetary_generator_shape():
    import rebound_gb300 as R
    systems, periods = R.ics.planetary_systems(32, seed=3)
    for s, P in zip(systems, periods):
        k = len(s) - 1
        assert 2 <= k <= 10 and P > 0
        com = [np.sum(s["m"] * s[f]) / np.sum(s["m"]) for f in ("x", "y", "z", "vx", "vy", "vz")]
        assert np.max(np.abs(com)) < 1e-12
        assert np.all(s["m"][1:] >= 1e-7) and np.all(s["m"][1:] <= 1e-3)


def test_no_gpu_create_fails_loudly():
    import torch
    if torch.cuda.is_available():
        return
    import rebound_gb300 as R
    try:
        R.Simulation()
    except R.RGPUError as e:
        assert e.code == 2
    else:
        raise AssertionError("creating a simulation without a GPU must raise")


def _c_layout(tmp_path, struct, names):
    """Size and field offsets of a struct of include/rebound_gb300.h, from a compiled probe."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / ("%s.c" % struct)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rebound_gb300.h"', 'int main(void) {',
             '  printf("size %%zu\\n", sizeof(%s));' % struct]
    lines += ['  printf("%s %%zu\\n", offsetof(%s, %s));' % (n, struct, n) for n in names]
    lines += ['  return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / struct
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.check_call([cc, "-I", inc, str(src), "-o", str(exe)])
    return {k: int(v) for k, v in (line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())}


@pytest.mark.parametrize("struct", ["rgpu_config", "rgpu_server_config", "rgpu_server_stats"])
def test_struct_layout_matches_header(tmp_path, struct):
    # the ctypes mirrors must have the C header's size and field offsets
    from rebound_gb300 import _lib
    cls = {"rgpu_config": _lib.Config, "rgpu_server_config": _lib.ServerConfig,
           "rgpu_server_stats": _lib.ServerStats}[struct]
    names = [f[0] for f in cls._fields_]
    out = _c_layout(tmp_path, struct, names)
    assert out["size"] == ctypes.sizeof(cls)
    for n in names:
        assert out[n] == getattr(cls, n).offset, n


def test_collision_record_matches_header(tmp_path):
    # the numpy record used for pair lists is struct rgpu_collision (and reb_collision)
    from rebound_gb300._lib import COLLISION_DTYPE
    out = _c_layout(tmp_path, "rgpu_collision", ["p1", "p2", "gb", "ri"])
    assert out["size"] == COLLISION_DTYPE.itemsize
    for n in ("p1", "p2", "gb", "ri"):
        assert out[n] == COLLISION_DTYPE.fields[n][1], n
