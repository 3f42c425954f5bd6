"""WHFast symplectic correctors and kernels on the GPU plain path.

The scenarios of rebound/tests/test_whfast_advanced.py (outer solar system,
dt = 0.0123235235 P_1, corrector orders 3-17, the second corrector, kernels
MODIFIEDKICK, COMPOSITION and LAZY) with the reference's bars, and each run held
to the reference's own end state bit for bit (tests/golden/whfast_advanced.npz,
made from the reference by tests/golden/make_golden.py).
"""

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")
KERNELS = ("default", "modifiedkick", "composition", "lazy")
# rebound/tests/test_whfast_advanced.py:5-21: (corrector, corrector2, kernel) -> energy bar
ENERGY_BAR = {(0, 0, "default"): 2e-7, (3, 0, "default"): 1e-9, (5, 0, "default"): 1e-9,
              (7, 0, "default"): 1e-9, (11, 0, "default"): 1e-9, (17, 0, "default"): 1e-9,
              (0, 0, "modifiedkick"): 2e-7, (3, 0, "modifiedkick"): 1e-9, (5, 0, "modifiedkick"): 1e-11,
              (7, 0, "modifiedkick"): 1e-12, (11, 0, "modifiedkick"): 1e-12, (17, 0, "modifiedkick"): 1e-12,
              (17, 0, "composition"): 1e-12, (17, 0, "lazy"): 1e-12, (11, 1, "modifiedkick"): 1e-12}
# rows of the reference's second table only (:23-30: 3/composition, 3/lazy, 3+2nd/lazy)
# run its back-and-forth test; here they also run the bit-exact trajectory test


def cases():
    g = golden("whfast_advanced.npz")
    return [(int(c), int(c2), KERNELS[int(k)]) for c, c2, k in g["settings"]]


def table1():
    # the rows the reference runs its energy, notcom and compias tests on
    return [k for k in cases() if k in ENERGY_BAR]


def make(gpu, g, c, c2, kernel, shift=0.0, safe=None):
    sim = gpu.Simulation()
    p = g["oss"].copy()
    p["vx"] += shift
    sim.add(p)
    sim.integrator = "whfast"
    sim.ri_whfast.corrector = c
    sim.ri_whfast.corrector2 = c2
    sim.ri_whfast.kernel = kernel
    if safe is not None:
        sim.ri_whfast.safe_mode = safe
    sim.dt = float(g["dt"])
    return sim


def same(a, b):
    for f in XV:
        assert np.array_equal(a[f], b[f]), f


def com(p):
    m = p["m"]
    return np.array([np.sum(m * p[f]) / np.sum(m) for f in XV])


@pytest.mark.parametrize("c,c2,kernel", table1())
def test_energy(gpu, c, c2, kernel):
    g = golden("whfast_advanced.npz")
    tag = "c%d_c2%d_%s" % (c, c2, kernel)
    sim = make(gpu, g, c, c2, kernel, safe=False)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    e1 = sim.energy()
    err = abs((e0 - e1) / e1)
    assert err < ENERGY_BAR[(c, c2, kernel)]
    assert err <= 2 * float(g["energy_err_" + tag])
    same(sim.particles, g["energy_end_" + tag])


@pytest.mark.parametrize("c,c2,kernel", table1())
def test_energy_notcom(gpu, c, c2, kernel):
    g = golden("whfast_advanced.npz")
    tag = "c%d_c2%d_%s" % (c, c2, kernel)
    sim = make(gpu, g, c, c2, kernel, shift=1.0)
    c0 = com(sim.particles)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    e1 = sim.energy()
    assert abs((e0 - e1) / e1) < ENERGY_BAR[(c, c2, kernel)]
    c1 = com(sim.particles)
    t = sim.t
    assert abs((c0[0] + c0[3] * t - c1[0]) / (c1[0] + c1[1])) < 1e-12
    assert abs((c0[1] + c0[4] * t - c1[1]) / (c1[0] + c1[1])) < 1e-12
    same(sim.particles, g["notcom_end_" + tag])


@pytest.mark.parametrize("c,c2,kernel", table1())
def test_compare_with_ias15(gpu, c, c2, kernel):
    # rebound/tests/test_whfast_advanced.py:70-92; the IAS15 solution is the
    # reference's own, at the WHFast run's end time
    g = golden("whfast_advanced.npz")
    tag = "c%d_c2%d_%s" % (c, c2, kernel)
    sim = make(gpu, g, c, c2, kernel, shift=1050.)
    sim.integrate(13.21415, exact_finish_time=False)
    assert sim.t == float(g["compias_t_" + tag]) == float(g["compias_ias15_t"])
    p, ias = sim.particles, g["compias_ias15"]
    bar = 1e-8 if c else 1.2e-6
    assert np.max(np.abs(ias["x"] - p["x"])) < bar
    same(p, g["compias_end_" + tag])


@pytest.mark.parametrize("c,c2,kernel", [(0, 0, "default"), (3, 0, "modifiedkick"), (3, 0, "composition"),
                                         (3, 0, "default"), (3, 0, "lazy"), (3, 1, "lazy")])
def test_back_and_forth(gpu, c, c2, kernel):
    g = golden("whfast_advanced.npz")
    tag = "c%d_c2%d_%s" % (c, c2, kernel)
    sim = make(gpu, g, c, c2, kernel, shift=1.0)
    p0 = sim.particles.copy()
    sim.steps(10)
    sim.dt = -sim.dt
    sim.steps(10)
    p = sim.particles
    if c:
        assert np.max(np.abs(p0["x"] - p["x"])) < 2e-11
    same(p, g["bf_end_" + tag])


@pytest.mark.parametrize("c,c2,kernel", cases())
def test_trajectory_bit_exact(gpu, c, c2, kernel):
    g = golden("whfast_advanced.npz")
    sim = make(gpu, g, c, c2, kernel, safe=False)
    sim.steps(20)
    sim.synchronize()
    same(sim.particles, g["traj_c%d_c2%d_%s" % (c, c2, kernel)])


@pytest.mark.parametrize("c", [0, 5])
def test_keep_unsynchronized(gpu, c):
    g = golden("whfast_advanced.npz")
    sim = make(gpu, g, c, 0, "default", safe=False)
    sim.ri_whfast.keep_unsynchronized = 1
    sim.steps(10)
    sim.synchronize()
    same(sim.particles, g["keep_mid_c%d" % c])
    sim.steps(10)
    sim.synchronize()
    same(sim.particles, g["keep_end_c%d" % c])


@pytest.mark.parametrize("setting,msg", [
    (dict(corrector=4), "only available in the following orders"),
    (dict(corrector=3, coordinates="democraticheliocentric"), "only compatible with Jacobi"),
    (dict(kernel="lazy", coordinates="democraticheliocentric"), "requires Jacobi"),
    (dict(kernel=7), "Kernel method must be"),
    (dict(keep_unsynchronized=1), "not compatible with safe_mode"),
])
def test_configuration_errors(gpu, setting, msg):
    # reb_integrator_whfast_init's checks (src/integrator_whfast.c:909-928)
    g = golden("whfast_advanced.npz")
    sim = make(gpu, g, 0, 0, "default")
    for k, v in setting.items():
        setattr(sim.ri_whfast, k, v)
    with pytest.raises(gpu.RGPUError, match=msg):
        sim.steps(1)


@pytest.mark.parametrize("c", [0, 5])
def test_reading_mid_run_does_not_change_the_trajectory(gpu, c):
    # safe_mode 0: reading particles or the energy between steps shows synchronized
    # values but the run continues exactly as without the reads (the reference's
    # sim.particles does not synchronize)
    g = golden("whfast_advanced.npz")
    a = make(gpu, g, c, 0, "default", safe=False)
    b = make(gpu, g, c, 0, "default", safe=False)
    for _ in range(4):
        a.steps(5)
        b.steps(5)
        pa = a.particles
        a.energy()
        assert np.all(np.isfinite(pa["x"]))
    a.synchronize()
    b.synchronize()
    same(a.particles, b.particles)
    same(b.particles, g["traj_c%d_c20_default" % c])
