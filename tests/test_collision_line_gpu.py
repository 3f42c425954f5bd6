"""LINE and LINETREE collision searches on the GPU (src/collision.c:125-196,
270-330, 506-572): pairs whose straight paths over the last step come within the
sum of the radii, in the reference's discovery order.

Inputs, the state after the step and the reference's pair lists come from
tests/golden/collision_line.npz (made from the reference by
tests/golden/make_golden.py): a shearing-sheet patch after one SEI + tree-gravity
step, and a periodic box of fast particles after one leapfrog drift.  The search
returns pairs in discovery order; the test applies the reference's rand_r shuffle
from the recorded seed and then requires the reference's list entry for entry.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")


def ring(gpu, g, start):
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]
    sim = gpu.Simulation()
    sim.G, sim.OMEGA, sim.softening, sim.dt, sim.t = G, OM, soft, dt, t
    sim.configure_box(rs, int(nx), int(ny), int(nz))
    sim.configure_ghostboxes(int(gx), int(gy), int(gz))
    sim.opening_angle2 = oa2
    sim.boundary = "shear"
    sim.gravity = "tree"
    sim.integrator = "sei"
    sim.add(start)
    return sim


def box(gpu, start):
    sim = gpu.Simulation()
    sim.integrator = "leapfrog"
    sim.gravity = "none"
    sim.boundary = "periodic"
    sim.configure_box(10.)
    sim.configure_ghostboxes(1, 1, 1)
    sim.dt = 0.3
    sim.add(start)
    return sim


def shuffled(pairs, seed):
    """The reference's post-search shuffle (src/collision.c:336-342): swap entry i with
    entry rand_r(&seed) % n, i = 0..n-1, using the C library's rand_r."""
    libc = ctypes.CDLL(None)
    libc.rand_r.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    out = pairs.copy()
    s = ctypes.c_uint(int(seed))
    n = len(out)
    for i in range(n):
        j = libc.rand_r(ctypes.byref(s)) % n
        tmp = out[i].copy()
        out[i] = out[j]
        out[j] = tmp
    return out


def same_pairs(got, ref, with_root):
    assert len(got) == len(ref) > 0
    assert np.array_equal(got["p1"], ref["p1"]) and np.array_equal(got["p2"], ref["p2"])
    assert np.array_equal(got["gb"], ref["gb"])
    if with_root:
        assert np.array_equal(got["ri"], ref["ri"])


@pytest.mark.parametrize("scene", ["ring", "box"])
@pytest.mark.parametrize("mode", ["line", "linetree", "direct"])
def test_line_searches_match_reference(gpu, scene, mode):
    g = golden("collision_line.npz")
    key = "%s_pairs_%s" % (scene, mode)
    if key not in g.files:
        pytest.skip("no reference list for this combination")
    sim = ring(gpu, golden("ring_patch.npz"), g["ring_start"]) if scene == "ring" else box(gpu, g["box_start"])
    sim.steps(1)                                          # sets dt_last_done
    p = sim.particles
    for f in XV:
        assert np.array_equal(p[f], g[scene + "_after1"][f]), f
    sim.collision = mode
    got = shuffled(sim.collision_search(), g["%s_seed_%s" % (scene, mode)])   # discovery order, then shuffled
    same_pairs(got, g[key], with_root=(mode == "linetree"))


def test_line_finds_crossings_the_overlap_test_misses(gpu):
    # paths that crossed during the step but no longer overlap: LINE reports them
    g = golden("collision_line.npz")
    sim = box(gpu, g["box_start"])
    sim.steps(1)
    sim.collision = "direct"
    direct = {(int(a), int(b)) for a, b in zip(*[sim.collision_search()[k] for k in ("p1", "p2")])}
    sim.collision = "line"
    line = {(int(a), int(b)) for a, b in zip(*[sim.collision_search()[k] for k in ("p1", "p2")])}
    assert len(line) > len(direct) // 2
    assert any(((a, b) not in direct and (b, a) not in direct) for a, b in line)
