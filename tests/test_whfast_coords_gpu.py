"""WHFast in WHDS and barycentric coordinates, and test particles in every
coordinate system, on the GPU plain path.

Inputs and the reference's own end states come from tests/golden/whfast_coords.npz
(made from the reference by tests/golden/make_golden.py); every run is held to the
reference's end state bit for bit and to the bars of rebound/tests/test_whfast.py:9-19
and rebound/tests/test_whfast_testparticles.py.
"""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")
COORDS = ("jacobi", "democraticheliocentric", "whds", "barycentric")


def run(gpu, arr, coords, dt, safe=1, N_active=-1, tp_type=0, corrector=0):
    sim = gpu.Simulation()
    sim.testparticle_type = tp_type
    sim.add(arr)
    if N_active > 0:
        sim.N_active = N_active
    sim.integrator = "whfast"
    sim.ri_whfast.coordinates = coords
    sim.ri_whfast.safe_mode = safe
    sim.ri_whfast.corrector = corrector
    sim.dt = dt
    return sim


def same(a, b):
    for f in XV:
        assert np.array_equal(a[f], b[f]), f


def close(a, b, eps):
    for f in ("x", "vx", "y", "vy"):
        assert np.max(np.abs(a[f] - b[f])) < eps, f


def test_whds_outer_solar_system(gpu):
    g = golden("whfast_coords.npz")
    sim = run(gpu, g["oss"], "whds", 0.005 * 12. * 2. * 3.1415)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    e1 = sim.energy()
    err = abs((e0 - e1) / e1)
    assert err < 2.4e-8 and err <= 2 * float(g["whds_oss_err"])
    same(sim.particles, g["whds_oss_end"])


@pytest.mark.parametrize("coords", ["whds", "barycentric"])
@pytest.mark.parametrize("safe", [1, 0])
def test_two_planets_100_steps(gpu, coords, safe):
    g = golden("whfast_coords.npz")
    sim = run(gpu, g["two"], coords, 0.005123 * 2. * math.pi, safe)
    sim.steps(100)
    sim.synchronize()
    same(sim.particles, g["two_%s_safe%d" % (coords, safe)])


@pytest.mark.parametrize("order,safe,n", [(5, 0, 50), (17, 1, 10)])
def test_barycentric_correctors(gpu, order, safe, n):
    g = golden("whfast_coords.npz")
    sim = run(gpu, g["two"], "barycentric", 0.005123 * 2. * math.pi, safe, corrector=order)
    sim.steps(n)
    sim.synchronize()
    same(sim.particles, g["two_barycentric_c%d" % order])


@pytest.mark.parametrize("coords", COORDS)
@pytest.mark.parametrize("N", [1, 2])
def test_test_particles(gpu, coords, N):
    # create_whfast_testparticle: one orbit of period 1 comes back to 2e-14, and
    # setting N_active changes nothing (1e-16)
    g = golden("whfast_coords.npz")
    start = g["tp_N%d" % N]
    ref_run = run(gpu, start, coords, 1e-1)
    ref_run.integrate(1)
    for na in [-1] + list(range(1, N + 2)):
        sim2 = run(gpu, start, coords, 1e-1, N_active=na)
        sim2.integrate(1)
        p2 = sim2.particles
        close(start, p2, 2e-14)
        close(ref_run.particles, p2, 1e-16)
        same(p2, g["tp_N%d_%s_na%d" % (N, coords, na)])


@pytest.mark.parametrize("coords", COORDS)
@pytest.mark.parametrize("N", [1, 2])
def test_test_particles_with_planets(gpu, coords, N):
    g = golden("whfast_coords.npz")
    start = g["tpp_N%d" % N]
    sim = run(gpu, start, coords, 1e-3)
    sim.integrate(1)
    for na in [-1] + list(range(3, N + 4)):
        sim2 = run(gpu, start, coords, 1e-3, N_active=na)
        sim2.integrate(1)
        close(sim.particles, sim2.particles, 1e-13)
        same(sim2.particles, g["tpp_N%d_%s_na%d" % (N, coords, na)])


@pytest.mark.parametrize("coords", COORDS)
@pytest.mark.parametrize("N", [1, 2])
def test_massive_test_particles(gpu, coords, N):
    # test particles with mass (N_active = 2) move like massless ones (2e-13)
    g = golden("whfast_coords.npz")
    start = g["mtp_N%d" % N]
    sim = run(gpu, start, coords, 1e-3)
    sim.integrate(1)
    heavy = start.copy()
    heavy["m"][2:] = 1.
    sim2 = run(gpu, heavy, coords, 1e-3, N_active=2)
    sim2.integrate(1)
    close(sim.particles, sim2.particles, 2e-13)
    same(sim.particles, g["mtp_N%d_%s_massless" % (N, coords)])
    same(sim2.particles, g["mtp_N%d_%s_massive" % (N, coords)])


@pytest.mark.parametrize("coords", COORDS)
def test_testparticle_type_one(gpu, coords):
    # testparticle_type 1: N_active does not change the transforms (1e-16)
    g = golden("whfast_coords.npz")
    for start, nas in (("tp1", (-1, 1)), ("tp1p", (-1, 3))):
        sim = run(gpu, g[start], coords, 1e-3, tp_type=1)
        sim.integrate(1)
        for na in nas:
            sim2 = run(gpu, g[start], coords, 1e-3, N_active=na, tp_type=1)
            sim2.integrate(1)
            close(sim.particles, sim2.particles, 1e-16)
            same(sim2.particles, g["%s_%s_na%d" % (start, coords, na)])


def test_corrector_needs_jacobi_or_barycentric(gpu):
    g = golden("whfast_coords.npz")
    sim = run(gpu, g["two"], "whds", 0.01, corrector=3)
    with pytest.raises(gpu.RGPUError, match="only compatible with Jacobi and Barycentric"):
        sim.steps(1)
