"""Leapfrog on the GPU: orders 2, 4, 6, 8 (src/integrator_leapfrog.c:97-203), and configuration 1 (Plummer N=4,096, softening
0.01, dt=1e-3, 1,000 steps, BASIC, FP64) against the reference.

Bar: the relative energy error after 1,000 steps is within 2x of the
reference's (src/tools.c:108 energy, unsoftened), and the first 10 steps track
the reference trajectory to 1e-12 relative (the summation order differs, so not
bit for bit).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def make(R, p, gravity="basic"):
    sim = R.Simulation()
    sim.softening = 0.01
    sim.dt = 1e-3
    sim.gravity = gravity
    sim.integrator = "leapfrog"
    sim.add(p)
    return sim


def test_first_steps_track_reference(gpu):
    g = golden("gravity_plummer.npz")
    sim = make(gpu, g["particles"])
    sim.steps(10)
    p, ref = sim.particles, g["after10"]
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        scale = np.abs(ref[f]).max()
        assert np.abs(p[f] - ref[f]).max() <= 1e-12 * scale, f
    assert abs(sim.t - 0.01) < 1e-15


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
def test_energy_error_1000_steps_within_2x(gpu, gravity):
    g = golden("gravity_plummer.npz")
    e0 = g["energy0"]
    ref_err = abs((g["energy1000"] - e0) / e0)
    sim = make(gpu, g["particles"], gravity)
    assert abs(sim.energy() - e0) <= 1e-13 * abs(e0)
    sim.steps(1000)
    err = abs((sim.energy() - e0) / e0)
    assert err <= 2 * ref_err, (err, ref_err)


def test_mixed_energy_drift_reported(gpu):
    # The mixed form's drift is a stated number, bounded loosely here.
    g = golden("gravity_plummer.npz")
    e0 = g["energy0"]
    sim = make(gpu, g["particles"], "mixed")
    sim.steps(1000)
    err = abs((sim.energy() - e0) / e0)
    ref_err = abs((g["energy1000"] - e0) / e0)
    assert err <= 10 * ref_err + 1e-6, (err, ref_err)


def test_integrate_exact_finish_time(gpu):
    # reb_simulation_integrate with exact_finish_time = 1 (src/simulation.c:291-354,
    # 455-458): full steps while t + dt < tmax, one shortened step of tmax - t, exit
    # once |t - tmax| < 1e-12 tmax, dt back to the last full step.  Each leapfrog
    # step advances t by two half steps, so t ends where that sum rounds
    # (0.010499999999999999, which the reference's own run reports as well).
    g = golden("gravity_plummer.npz")
    sim = make(gpu, g["particles"][:256])
    sim.integrate(0.0105)
    t, dt = 0.0, 1e-3
    while t + dt < 0.0105:
        t += dt / 2.
        t += dt / 2.
    last = 0.0105 - t
    t += last / 2.
    t += last / 2.
    assert sim.t == t and abs(sim.t - 0.0105) < 1e-12 * 0.0105
    assert sim.dt == 1e-3


@pytest.mark.parametrize("order", [4, 6, 8])
def test_higher_orders_track_reference(gpu, order):
    # 20 steps of the reference's composition schemes on a softened 128-body sphere
    g = golden("leapfrog_orders.npz")
    sim = make(gpu, g["particles"])
    sim.leapfrog_order = order
    sim.steps(20)
    p, ref = sim.particles, g["after20_o%d" % order]
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        scale = np.abs(ref[f]).max()
        assert np.abs(p[f] - ref[f]).max() <= 1e-12 * scale, (order, f)
    assert sim.t == float(g["t_o%d" % order])      # the same sequence of drift lengths


@pytest.mark.parametrize("order,bar", [(4, 3e-6), (6, 1e-9), (8, 1e-9)])
def test_higher_orders_outer_solar_system(gpu, order, bar):
    # rebound/tests/test_leapfrog.py:24-56: integrate to t = 1e3 with dt = 1, one more step
    g = golden("reference_cases.npz")
    ref_err = float(golden("leapfrog_orders.npz")["oss_err_o%d" % order])
    sim = gpu.Simulation()
    sim.integrator = "leapfrog"
    sim.leapfrog_order = order
    sim.dt = 1.0
    sim.add(g["oss"])
    e0 = sim.energy()
    sim.integrate(1e3)
    sim.steps(1)
    err = abs((e0 - sim.energy()) / sim.energy())
    assert err < bar
    assert err <= max(2 * ref_err, 1e-13), (err, ref_err)


def test_unsupported_order_is_an_error(gpu):
    sim = make(gpu, golden("leapfrog_orders.npz")["particles"])
    sim.leapfrog_order = 3
    with pytest.raises(gpu.RGPUError):
        sim.steps(1)
