"""The reference's own unit-test scenarios for this path, run on the GPU.

Each test restates a scenario of REBOUND's test suite with the same inputs and
the same bar, and where the reference's own result is in the fixture
(tests/golden/reference_cases.npz, made by tests/golden/make_golden.py from the
reference itself) it also holds the GPU to that result:

  rebound/tests/test_leapfrog.py:14-22      leapfrog, outer solar system, |dE/E| < 1e-3
  rebound/tests/test_whfast.py:20-29        WHFast Jacobi, outer solar system, < 2.4e-8
  rebound/tests/test_whfast.py:31-41        WHFast, very hyperbolic test particle, one step
  rebound/tests/test_whfast.py:43-54        WHFast, hyperbolic orbit, < 1e-14
  rebound/tests/test_whfast.py:56-69        WHFast, two planets, < 1.2e-8
  rebound/tests/test_whfast.py:307-345      WHFast forward then backward: back to the start
  rebound/tests/test_boundary.py:18-34      periodic box: exact wrapped positions
  rebound/tests/test_shearingsheet.py:8-58  shearing sheet: > 1000 collisions per orbit
"""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs((a - b) / b)


def whfast_sim(gpu, particles, dt):
    sim = gpu.Simulation()
    sim.integrator = "whfast"
    sim.dt = dt
    sim.add(particles)
    return sim


def test_leapfrog_outer_solar_system(gpu):
    g = golden("reference_cases.npz")
    sim = gpu.Simulation()
    sim.integrator = "leapfrog"
    sim.gravity = "basic"
    sim.dt = 1.0
    sim.add(g["oss"])
    e0 = sim.energy()
    sim.integrate(1e3)
    err = rel(e0, sim.energy())
    assert err < 1e-3
    assert err <= 2 * float(g["oss_leapfrog_err"]), (err, float(g["oss_leapfrog_err"]))


def test_whfast_outer_solar_system(gpu):
    g = golden("reference_cases.npz")
    sim = whfast_sim(gpu, g["oss_raw"], 0.005 * 12. * 2. * 3.1415)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    err = rel(e0, sim.energy())
    assert err < 2.4e-8
    assert err <= 2 * float(g["oss_whfast_err"]), (err, float(g["oss_whfast_err"]))


def test_whfast_very_hyperbolic_test_particle(gpu):
    p = np.zeros(2, dtype=gpu.PARTICLE_DTYPE)
    p["m"] = [1.0, 0.0]
    p["x"][1] = 1.0
    p["vy"][1] = 100000.0
    sim = whfast_sim(gpu, p, 1.234567)
    sim.steps(1)
    sim.synchronize()
    ys = 1.234567 * 100000.
    assert abs((sim.particles["y"][1] - ys) / ys) <= 1e-15


def test_whfast_hyperbolic_orbit(gpu):
    g = golden("reference_cases.npz")
    yr = float(g["hyper_yr"])
    sim = whfast_sim(gpu, g["hyper"], 0.00512 * yr)
    e0 = sim.energy()
    sim.integrate(1e2 * yr)
    err = rel(e0, sim.energy())
    assert err < 1e-14
    assert err <= max(2 * float(g["hyper_err"]), 1e-14)


def test_whfast_two_planets(gpu):
    g = golden("reference_cases.npz")
    jupyr = 2. * math.pi
    sim = whfast_sim(gpu, g["two"], 0.005123 * jupyr)
    e0 = sim.energy()
    sim.integrate(1e3 * jupyr)
    err = rel(e0, sim.energy())
    assert err < 1.2e-8
    assert err <= 2 * float(g["two_err"]), (err, float(g["two_err"]))


@pytest.mark.parametrize("case,bar", [("bf_hyper", 1e-14), ("bf_ecc", 1e-13)])
def test_whfast_forward_then_backward(gpu, case, bar):
    g = golden("reference_cases.npz")
    p0 = g[case]
    dt = float(g[case + "_dt"])
    sim = whfast_sim(gpu, p0, dt)
    e0 = sim.energy()
    sim.steps(100)
    sim.dt = -dt
    sim.steps(100)
    sim.synchronize()
    end = sim.particles
    assert rel(e0, sim.energy()) < bar
    assert rel(p0["x"][1], end["x"][1]) < bar
    assert rel(p0["vx"][1], end["vx"][1]) < bar
    # and the same end state as the reference's own run
    ref = g[case + "_end"]
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.allclose(end[f], ref[f], rtol=1e-14, atol=0), f


def test_periodic_box_exact_positions(gpu):
    # two massless particles in a periodic box of side 10 (free motion, wrapped)
    sim = gpu.Simulation()
    sim.boundary = "periodic"
    sim.root_size = 10.0
    sim.integrator = "leapfrog"
    sim.dt = 0.125
    sim.add(m=0.0, x=1., vx=5.0, vy=15.1, vz=26.)
    sim.add(m=0.0, x=-1., vx=-5.0, vy=-15.1, vz=-26.)
    sim.integrate(1.)
    p = sim.particles
    assert abs(p["x"][0] - (-4)) <= 1e-16 and abs(p["y"][0] - (-4.9)) <= 1e-14 and abs(p["z"][0] - (-4.0)) <= 1e-16
    assert abs(p["x"][1] - 4) <= 1e-16
    sim.integrate(2.)
    p = sim.particles
    assert abs(p["x"][0] - 1) <= 1e-16 and abs(p["y"][0] - 0.2) <= 1e-14 and abs(p["z"][0] - 2.0) <= 1e-16
    assert abs(p["x"][1] - (-1)) <= 1e-16


def test_shearing_sheet_collision_rate(gpu):
    # Saturn's-rings patch of 50 m, SEI + shear + tree gravity + tree collisions +
    # hardsphere; particle radii power law (slope -3, 1..4 m), 400 kg/m^3, until
    # the surface density reaches 400 kg/m^2.  One orbit gives over 1000 collisions.
    rng = np.random.default_rng(2024)
    OMEGA, box = 0.00013143527, 50.
    rows = []
    total = 0.
    while total < 400. * box * box:
        y = rng.random()
        r = ((4. ** -2 - 1.) * y + 1.) ** (1. / -2)
        m = 400. * 4. / 3. * math.pi * r ** 3
        x = rng.uniform(-box / 2, box / 2)
        z = rng.normal(0., 1.)
        while abs(z) >= box / 2:
            z = rng.normal(0., 1.)
        rows.append((x, rng.uniform(-box / 2, box / 2), z, 0., -1.5 * x * OMEGA, 0., m, r))
        total += m
    p = np.zeros(len(rows), dtype=gpu.PARTICLE_DTYPE)
    for k, f in enumerate(("x", "y", "z", "vx", "vy", "vz", "m", "r")):
        p[f] = [row[k] for row in rows]
    assert len(p) > 50
    sim = gpu.Simulation()
    sim.OMEGA = OMEGA
    sim.G = 6.67428e-11
    sim.dt = 1e-3 * 2. * math.pi / OMEGA
    sim.softening = 0.2
    sim.root_size = box
    sim.N_ghost_x = 2
    sim.N_ghost_y = 2
    sim.integrator = "sei"
    sim.boundary = "shear"
    sim.gravity = "tree"
    sim.collision = "tree"
    sim.collision_resolve = "hardsphere"
    sim.coefficient_of_restitution = 0.5
    sim.add(p)
    sim.integrate(2. * math.pi / OMEGA)
    assert sim.collisions_log_n > 1000
