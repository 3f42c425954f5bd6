"""WHFast in democratic heliocentric coordinates on the GPU plain path.

Bar: the trajectory is the reference's bit for bit (same operation order,
--fmad=false), and the scenarios of rebound/tests/test_whfast.py:212-305 meet the
reference's bars and stay within 2x of the reference's own energy error
(tests/golden/whfast_dh.npz, made from the reference by tests/golden/make_golden.py).
"""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")


def dh_sim(gpu, particles, dt, safe_mode=1):
    sim = gpu.Simulation()
    sim.integrator = "whfast"
    sim.ri_whfast.coordinates = "democraticheliocentric"
    sim.ri_whfast.safe_mode = safe_mode
    sim.dt = dt
    sim.add(particles)
    return sim


def rel(a, b):
    return abs((a - b) / b)


@pytest.mark.parametrize("safe_mode", [1, 0])
def test_two_planets_100_steps_bit_exact(gpu, safe_mode):
    g = golden("whfast_dh.npz")
    sim = dh_sim(gpu, g["two"], 0.005123 * 2. * math.pi, safe_mode)
    sim.steps(100)
    sim.synchronize()
    out, ref = sim.particles, g["two_after100_safe%d" % safe_mode]
    for f in XV:
        assert np.array_equal(out[f], ref[f]), f


def test_outer_solar_system(gpu):
    g = golden("whfast_dh.npz")
    sim = dh_sim(gpu, g["oss"], 0.005 * 12. * 2. * 3.1415)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    err = rel(e0, sim.energy())
    assert err < 1.5e-8
    assert err <= 2 * float(g["oss_err"])


def test_very_hyperbolic_test_particle(gpu):
    p = np.zeros(2, dtype=gpu.PARTICLE_DTYPE)
    p["m"] = [1.0, 0.0]
    p["x"][1] = 1.0
    p["vy"][1] = 100000.0
    sim = dh_sim(gpu, p, 1.234567)
    sim.steps(1)
    ys = 1.234567 * 100000.
    assert abs((sim.particles["y"][1] - ys) / ys) <= 1e-15


def test_hyperbolic_orbit(gpu):
    g = golden("whfast_dh.npz")
    yr = float(g["hyper_yr"])
    sim = dh_sim(gpu, g["hyper"], 0.00512 * yr)
    e0 = sim.energy()
    sim.integrate(1e2 * yr)
    err = rel(e0, sim.energy())
    assert err < 4.5e-8
    assert err <= 2 * float(g["hyper_err"])


@pytest.mark.parametrize("safe_mode", [1, 0])
def test_two_planets_energy(gpu, safe_mode):
    g = golden("whfast_dh.npz")
    jupyr = 2. * math.pi
    sim = dh_sim(gpu, g["two"], 0.005123 * jupyr, safe_mode)
    e0 = sim.energy()
    sim.integrate(1e3 * jupyr)
    err = rel(e0, sim.energy())
    assert err < 2.9e-8
    assert err <= 2 * float(g["two_err_safe%d" % safe_mode])


def test_order_of_planets_does_not_matter(gpu):
    g = golden("whfast_dh.npz")
    jupyr = 2. * math.pi
    ends = {}
    for tag in ("order12", "order21"):
        sim = dh_sim(gpu, g[tag], 0.005123 * jupyr)
        sim.integrate(1e0 * jupyr)
        ends[tag] = sim.particles
        for f in XV:                       # and each run is the reference's own, bit for bit
            assert np.array_equal(ends[tag][f], g[tag + "_end"][f]), (tag, f)
    a, b = ends["order12"], ends["order21"]
    for f in ("x", "y"):
        assert abs(a[f][1] - b[f][2]) <= 1e-14 and abs(a[f][2] - b[f][1]) <= 1e-14


@pytest.mark.parametrize("coords", ["jacobi", "democraticheliocentric"])
def test_safe_mode_off_synchronize_mid_run(gpu, coords):
    # safe_mode 0: 50 steps, synchronize, 50 more steps from the synchronized
    # coordinates, synchronize: the reference's own trajectory bit for bit
    g = golden("whfast_dh.npz")
    sim = dh_sim(gpu, g["two"], 0.005123 * 2. * math.pi, 0)
    sim.ri_whfast.coordinates = coords
    sim.steps(50)
    sim.synchronize()
    sim.steps(50)
    sim.synchronize()
    out, ref = sim.particles, g["two_sync_mid_" + coords]
    for f in XV:
        assert np.array_equal(out[f], ref[f]), f


def test_dh_ensemble_bit_exact(gpu):
    # the batched democratic heliocentric kernels (the WHFast512 splitting) follow the
    # reference's own 100-step run and, for 200 generated systems, the plain path
    from rebound_gb300.ensemble import Ensemble
    g = golden("whfast_dh.npz")
    ens = Ensemble([g["two"]], [0.005123 * 2. * math.pi], coordinates="democraticheliocentric")
    ens.steps(100)
    p = ens.particles()[0]
    for f in XV:
        assert np.array_equal(p[f], g["two_after100_safe1"][f]), f
    systems, periods = gpu.ics.planetary_systems(200, seed=5)
    dts = periods / 20.0
    ens = Ensemble(systems, dts, coordinates="democraticheliocentric")
    ens.autotune(probe_steps=2, max_steps_per_launch=16)
    ens = Ensemble(systems, dts, coordinates="democraticheliocentric")
    ens.set_launch(64, 7)                      # ragged chunks must not change results
    ens.steps(50)
    out = ens.particles()
    for s in (0, 17, 99, 199):
        sim = dh_sim(gpu, systems[s], dts[s])
        sim.steps(50)
        q = sim.particles
        for f in XV:
            assert np.array_equal(q[f], out[s][f]), (s, f)
