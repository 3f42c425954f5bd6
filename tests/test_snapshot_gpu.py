"""Snapshots and archives of the device-resident state (the Simulationarchive
counterpart): the restart scenarios of rebound/tests/test_simulationarchive.py:86-365.

A run that saves snapshots every 10 time units, is stopped, restored from its last
snapshot and integrated on must end bit for bit where an uninterrupted run ends --
and there the reference's own run ends too (tests/golden/archive_cases.npz, made
from the reference by tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")

CASES = [("jacobi", 0, 0), ("jacobi", 1, 0), ("jacobi", 0, 5), ("jacobi", 1, 5),
         ("democraticheliocentric", 0, 0), ("democraticheliocentric", 1, 0), ("whds", 0, 0), ("whds", 1, 0)]


def make(gpu, g, coords, safe, corrector):
    sim = gpu.Simulation()
    sim.add(g["start"])
    sim.integrator = "whfast"
    sim.ri_whfast.coordinates = coords
    sim.ri_whfast.corrector = corrector
    sim.dt = 0.1313
    sim.ri_whfast.safe_mode = safe
    return sim


def same(a, b):
    for f in XV:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("coords,safe,corrector", CASES)
def test_restart_is_bit_exact(gpu, tmp_path, coords, safe, corrector):
    g = golden("archive_cases.npz")
    tag = "%s_safe%d_c%d" % (coords, safe, corrector)
    path = tmp_path / "test.bin"
    sim = make(gpu, g, coords, safe, corrector)
    sim.save_to_file(path, 10., delete_file=True)
    sim.integrate(42., exact_finish_time=0)
    del sim
    sa = gpu.Simulationarchive(path)
    assert len(sa) == 5 and sa.tmin == 0.0 and 40. <= sa.tmax < 40. + 0.1313
    sim = sa[-1]
    sim.integrate(80., exact_finish_time=0)
    straight = make(gpu, g, coords, safe, corrector)
    straight.integrate(80., exact_finish_time=0)
    assert sim.t == straight.t == float(g["t_" + tag])
    same(sim.particles, straight.particles)
    same(sim.particles, g["end_" + tag])


@pytest.mark.parametrize("coords,safe,corrector", [("jacobi", 0, 0), ("jacobi", 0, 5)])
def test_get_simulation_modes(gpu, tmp_path, coords, safe, corrector):
    g = golden("archive_cases.npz")
    path = tmp_path / "test.bin"
    sim = make(gpu, g, coords, safe, corrector)
    sim.save_to_file(path, 10., delete_file=True)
    sim.integrate(42., exact_finish_time=0)
    sa = gpu.Simulationarchive(path)
    s = sa.getSimulation(27.123, mode="exact")
    assert abs(s.t - 27.123) <= 1e-14
    s = sa.getSimulation(25.123, mode="close")
    assert abs(s.t - 25.123) <= s.dt
    sims = [sa.getSimulation(t, mode="close") for t in (0., 11., 22.)]
    assert abs(sims[-1].t - 22.058400000000105) <= sims[-1].dt   # test_simulationarchive.py:306-323
    s = sa.getSimulation(21.0)                                      # 'snapshot': the one at t = 20.x
    assert 20. <= s.t < 20. + 0.1313


def test_append_and_step_interval(gpu, tmp_path):
    g = golden("archive_cases.npz")
    path = tmp_path / "test.bin"
    sim = make(gpu, g, "jacobi", 0, 0)
    sim.save_to_file(path, 10., delete_file=True)
    sim.integrate(40., exact_finish_time=0)
    sa = gpu.Simulationarchive(path)
    n0 = len(sa)
    sim = sa[-1]
    sim.save_to_file(path, 10.)          # appends to the same archive, as the reference does
    sim.integrate(80., exact_finish_time=0)
    sa = gpu.Simulationarchive(path)
    assert len(sa) > n0 and np.all(np.diff(sa.t[n0:]) > 0)
    # snapshots every 7 steps
    path2 = tmp_path / "steps.bin"
    sim = make(gpu, g, "jacobi", 1, 0)
    sim.save_to_file(path2, step=7, delete_file=True)
    sim.steps(30)
    sa = gpu.Simulationarchive(path2)
    assert len(sa) == 5                   # before steps 0, 7, 14, 21, 28
    assert np.allclose(np.diff(sa.t), 7 * 0.1313)


def test_snapshot_roundtrip_in_memory(gpu):
    # the C ABI's buffer form: write, restore into a fresh handle, continue identically
    import ctypes
    g = golden("archive_cases.npz")
    a = make(gpu, g, "jacobi", 0, 5)
    a.steps(17)
    L = a._L
    n = ctypes.c_size_t(0)
    assert L.rgpu_sim_snapshot_size(a.handle, ctypes.byref(n)) == 0
    buf = ctypes.create_string_buffer(n.value)
    w = ctypes.c_size_t(0)
    assert L.rgpu_sim_snapshot_write(a.handle, buf, n.value, ctypes.byref(w)) == 0 and w.value == n.value
    c = gpu.Simulation()
    assert L.rgpu_sim_snapshot_read(c._h, buf, w.value) == 0
    L.rgpu_sim_get_config(c._h, ctypes.byref(c._cfg))
    c._host = np.zeros(L.rgpu_sim_N(c._h), dtype=gpu.PARTICLE_DTYPE)
    c._device_newer = True
    a.steps(23)
    c.steps(23)
    same(a.particles, c.particles)
    # a buffer without the magic is refused with an error, not read
    bad = ctypes.create_string_buffer(b"XXXXXXXX" + buf.raw[8:w.value], w.value)
    assert L.rgpu_sim_snapshot_read(c._h, bad, w.value) != 0


def copy_via_snapshot(gpu, sim):
    """A second handle restored from a snapshot of `sim` (the reference's sim.copy())."""
    twin = gpu.Simulation()
    import ctypes
    L = sim._L
    n = ctypes.c_size_t(0)
    assert L.rgpu_sim_snapshot_size(sim.handle, ctypes.byref(n)) == 0
    buf = ctypes.create_string_buffer(n.value)
    w = ctypes.c_size_t(0)
    assert L.rgpu_sim_snapshot_write(sim.handle, buf, n.value, ctypes.byref(w)) == 0
    assert L.rgpu_sim_snapshot_read(twin._h, buf, w.value) == 0
    L.rgpu_sim_get_config(twin._h, ctypes.byref(twin._cfg))
    twin._host = np.zeros(L.rgpu_sim_N(twin._h), dtype=gpu.PARTICLE_DTYPE)
    twin._device_newer = True
    return twin


@pytest.mark.parametrize("c,c2,kernel", [(0, 0, "default"), (3, 0, "modifiedkick"), (3, 0, "composition"),
                                         (3, 0, "default"), (3, 0, "lazy"), (3, 1, "lazy")])
def test_whfast_restart_equals_continuation(gpu, c, c2, kernel):
    # rebound/tests/test_whfast_advanced.py:113-125 (restart): one step, copy, one more
    # step on each; both equal, and equal to the reference's two-step run when safe
    g = golden("whfast_advanced.npz")
    sim = gpu.Simulation()
    sim.add(g["oss"])
    sim.integrator = "whfast"
    sim.ri_whfast.corrector = c
    sim.ri_whfast.corrector2 = c2
    sim.ri_whfast.kernel = kernel
    sim.dt = float(g["dt"])
    sim.steps(1)
    sim2 = copy_via_snapshot(gpu, sim)
    sim.steps(1)
    sim2.steps(1)
    assert sim.t == sim2.t
    same(sim.particles, sim2.particles)


def test_shearing_sheet_restart_bit_exact(gpu, tmp_path):
    # the ring patch (SEI, shear, tree gravity, tree collisions, hardsphere): 3 steps,
    # snapshot, 3 more steps on the original and on the restored handle
    g = golden("ring_patch.npz")
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]

    def ring():
        sim = gpu.Simulation()
        sim.G, sim.OMEGA, sim.softening, sim.dt, sim.t = G, OM, soft, dt, t
        sim.configure_box(rs, int(nx), int(ny), int(nz))
        sim.configure_ghostboxes(int(gx), int(gy), int(gz))
        sim.opening_angle2 = oa2
        sim.boundary, sim.gravity, sim.integrator = "shear", "tree", "sei"
        sim.collision, sim.collision_resolve = "tree", "hardsphere"
        sim.coefficient_of_restitution = 0.5
        sim.rand_seed = int(g["after5_seed0"])
        sim.add(g["particles"])
        return sim

    a = ring()
    a.steps(3)
    a.save_to_file(tmp_path / "ring.bin", delete_file=True)
    b = gpu.Simulationarchive(tmp_path / "ring.bin")[-1]
    a.steps(3)
    b.steps(3)
    assert a.t == b.t and a.rand_seed == b.rand_seed and a.collisions_log_n == b.collisions_log_n
    same(a.particles, b.particles)
