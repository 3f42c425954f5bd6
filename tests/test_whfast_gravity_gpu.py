"""WHFast with the simulation's own gravity mode, and the collision exit.

The reference's WHFast evaluates whatever r->gravity names, so a WHFast run with
gravity = "compensated" sums its kicks with Kahan-compensated pair forces and one
with gravity = "none" kicks only with the Jacobi / star terms.  Inputs and the
reference's own end states come from tests/golden/whfast_gravity.npz (made from the
reference by tests/golden/make_golden.py).  The collision tests restate
rebound/tests/test_collisions.py:8-101: with collision_resolve = "halt", integrate
raises Collision when the LINE / LINETREE search finds the pair.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")


def same(a, b):
    for f in XV:
        assert np.array_equal(a[f], b[f]), f


def test_testparticle_whfast_compensated_type0(gpu):
    # rebound/tests/test_gravity.py:55-68: a massive test particle of type 0 leaves
    # the star where it was
    g = golden("whfast_gravity.npz")
    sim = gpu.Simulation()
    sim.gravity = "compensated"
    sim.integrator = "whfast"
    sim.testparticle_type = 0
    sim.dt = float(g["comp0_dt"])
    sim.add(g["comp0_start"])
    sim.N_active = 1
    sim.integrate(10.)
    p = sim.particles
    assert p["x"][0] == 0.
    same(p, g["comp0_end"])


def test_testparticle_whfast_compensated_type1(gpu):
    # rebound/tests/test_gravity.py:70-94: type 1 moves the star; the planet agrees
    # with the reference's IAS15 run to 1e-9
    g = golden("whfast_gravity.npz")
    sim = gpu.Simulation()
    sim.gravity = "compensated"
    sim.integrator = "whfast"
    sim.dt = 1e-4
    sim.testparticle_type = 1
    sim.add(g["comp1_start"])
    sim.N_active = 2
    sim.integrate(10.)
    p = sim.particles
    assert p["x"][0] != 0.
    assert abs(g["comp1_end_ias15"]["x"][1] - p["x"][1]) < 1e-9
    same(p, g["comp1_end_whfast"])


@pytest.mark.parametrize("gravity", ["compensated", "none"])
@pytest.mark.parametrize("coords", ["jacobi", "democraticheliocentric", "whds", "barycentric"])
def test_whfast_gravity_modes_bit_exact(gpu, gravity, coords):
    g = golden("whfast_gravity.npz")
    sim = gpu.Simulation()
    sim.add(g["oss"])
    sim.gravity = gravity
    sim.integrator = "whfast"
    sim.ri_whfast.coordinates = coords
    sim.ri_whfast.safe_mode = 0
    sim.dt = 0.5
    sim.steps(100)
    sim.synchronize()
    same(sim.particles, g["oss_%s_%s" % (gravity, coords)])


def test_whfast_rejects_other_gravity(gpu):
    g = golden("whfast_gravity.npz")
    sim = gpu.Simulation()
    sim.add(g["oss"])
    sim.integrator = "whfast"
    sim.gravity = "mixed"
    sim.dt = 0.5
    with pytest.raises(gpu.RGPUError, match="BASIC, COMPENSATED or NONE"):
        sim.steps(1)


def two_bodies(gpu, mode, x2, vx2):
    sim = gpu.Simulation()
    sim.integrator = "leapfrog"
    sim.gravity = "none"
    sim.collision = mode
    sim.configure_box(100.)
    sim.dt = 10
    sim.add(r=1, x=0)
    sim.add(r=1, x=x2, vx=vx2)
    return sim


@pytest.mark.parametrize("mode", ["line", "linetree"])
@pytest.mark.parametrize("x2", [3., 1., 11.])          # through, overlapping at t=0, overlapping at the end
def test_line_finds_collision(gpu, mode, x2):
    sim = two_bodies(gpu, mode, x2, -1.)
    with pytest.raises(gpu.Collision):
        sim.integrate(10)


@pytest.mark.parametrize("mode", ["line", "linetree"])
def test_line_miss(gpu, mode):
    sim = two_bodies(gpu, mode, 2.1, 1.)
    sim.integrate(10)
    assert sim.t == 10.
