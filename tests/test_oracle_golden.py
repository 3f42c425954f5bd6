"""Pin the CPU oracle against golden vectors of the unmodified reference.

The fixtures in tests/golden/ were produced by REBOUND 5.0.0's own C core
(serial, -ffp-contract=off) through its own Python package; see
tests/golden/make_golden.py.  The oracle must reproduce them bit for bit.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

XV = ("x", "y", "z", "vx", "vy", "vz")


def max_diff(a, b, fields=XV):
    return max(float(np.abs(a[f] - b[f]).max()) for f in fields)


def test_oracle_basic_compensated_plummer():
    g = golden("gravity_plummer.npz")
    s = O.Sim(g["particles"], softening=0.01)
    assert np.array_equal(s.gravity("basic"), g["acc_basic"])
    assert np.array_equal(s.gravity("basic_omp"), g["acc_basic"])   # gather order gives the same bits
    assert np.array_equal(s.gravity("compensated"), g["acc_compensated"])
    assert s.energy() == g["energy0"]


def test_oracle_leapfrog_trajectory():
    g = golden("gravity_plummer.npz")
    s = O.Sim(g["particles"], softening=0.01, dt=1e-3)
    s.leapfrog(10)
    assert max_diff(s.p, g["after10"]) == 0.0


@pytest.mark.parametrize("order", [4, 6, 8])
def test_oracle_leapfrog_orders(order):
    # src/integrator_leapfrog.c:97-203, bit for bit with the reference's own run
    g = golden("leapfrog_orders.npz")
    s = O.Sim(g["particles"], softening=0.01, dt=1e-3)
    s.leapfrog(20, order=order)
    assert max_diff(s.p, g["after20_o%d" % order]) == 0.0
    assert s.s.t == float(g["t_o%d" % order])


@pytest.mark.parametrize("case", ["plain", "testp0", "testp1", "ignore01", "ignore0", "ghost", "single", "two"])
def test_oracle_gravity_cases(case):
    g = golden("gravity_cases.npz")
    n, na, tp, ign, ghost, soft = g[case + "_meta"]
    for mode in ("basic", "compensated"):
        key = f"{case}_acc_{mode}"
        if key not in g:
            continue
        s = O.Sim(g[case + "_particles"], softening=soft / 1e6, N_active=None if na < 0 else int(na),
                  testparticle_type=int(tp), boundary="periodic" if ghost else "none",
                  root_size=2.0 if ghost else -1.0, N_ghost=(1, 1, 1) if ghost else (0, 0, 0))
        s.s.gravity_ignore_terms = int(ign)
        assert np.array_equal(s.gravity(mode), g[key]), (case, mode)


def ring_sim(g):
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]
    return O.Sim(g["particles"], G=G, softening=soft, dt=dt, boundary="shear", root_size=rs,
                 N_root=(int(nx), int(ny), int(nz)), N_ghost=(int(gx), int(gy), int(gz)), OMEGA=OM,
                 opening_angle2=oa2, t=t)


@pytest.mark.parametrize("case", ["binary_wide", "cluster_far", "plummer_binary"])
def test_oracle_gravity_hierarchical(case):
    # small coordinates far below the largest one (the inputs of the fixed-point guard)
    g = golden("gravity_hierarchical.npz")
    s = O.Sim(g[case + "_particles"], softening=float(g[case + "_softening"]))
    for mode in ("basic", "compensated"):
        assert np.array_equal(s.gravity(mode), g[f"{case}_acc_{mode}"]), (case, mode)


def test_oracle_tree_cells_and_gravity():
    g = golden("ring_patch.npz")
    s = ring_sim(g)
    cells, ref = s.tree_cells(), g["cells"]
    assert len(cells) == len(ref)
    for f in ref.dtype.names:
        assert np.array_equal(cells[f], ref[f]), f
    assert np.array_equal(s.gravity("tree"), g["acc_tree"])
    assert np.array_equal(ring_sim(g).gravity("basic"), g["acc_basic"])


def pair_key(p):
    return sorted(zip(p["p1"].tolist(), p["p2"].tolist(), map(tuple, p["gb"].tolist())))


@pytest.mark.parametrize("mode", ["direct", "tree"])
def test_oracle_collision_pairs(mode):
    g = golden("ring_patch.npz")
    pr = ring_sim(g).collisions(mode)
    assert len(pr) == len(g["pairs_" + mode]) > 0
    assert pair_key(pr) == pair_key(g["pairs_" + mode])


def test_oracle_tree_search_threads_keep_the_serial_order():
    # the OpenMP split of the tree search returns the serial list entry for entry
    g = golden("ring_patch.npz")
    s = ring_sim(g)
    a, b = s.collisions("tree"), s.collisions("tree_omp")
    assert len(a) == len(b) > 0 and a.tobytes() == b.tobytes()


def test_oracle_kepler_solver():
    g = golden("whfast.npz")
    k = g["kepler_in"].copy()
    for i in range(len(k)):
        O.lib().orc_whfast_kepler_solver(k[i:i + 1].ctypes.data, g["kepler_mu"][i], g["kepler_dt"][i])
    assert max_diff(k, g["kepler_out"]) == 0.0


def test_oracle_whfast_systems():
    g = golden("whfast.npz")
    for s in range(8):
        dt, e0, e1 = g[f"sys{s}_meta"]
        sim = O.Sim(g[f"sys{s}_p0"], dt=dt)
        sim.whfast(100)
        assert max_diff(sim.p, g[f"sys{s}_p100"]) == 0.0
        sim.whfast(900)
        assert max_diff(sim.p, g[f"sys{s}_p1000"]) == 0.0
        assert sim.energy() == e1


def test_oracle_sei_shear_trajectory():
    g = golden("sei_shear.npz")
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, t = g["meta"]
    s = O.Sim(g["particles"], G=G, softening=soft, dt=dt, boundary="shear", root_size=rs,
              N_root=(int(nx), int(ny), int(nz)), N_ghost=(int(gx), int(gy), int(gz)), OMEGA=OM, t=t)
    for _ in range(20):
        O.lib().orc_sei_step(s.ref, 1)
        O.lib().orc_boundary_check(s.ref)
    assert max_diff(s.p, g["after20"]) == 0.0


def test_oracle_energy_after_1000_leapfrog_steps_recorded():
    # The reference's relative energy error after 1000 steps at N=4096 is the
    # bar for the GPU path (within 2x); it must be a sane small number.
    g = golden("gravity_plummer.npz")
    err = abs((g["energy1000"] - g["energy0"]) / g["energy0"])
    assert 0 < err < 1e-2


KERNELS = ("default", "modifiedkick", "composition", "lazy")


def advanced_cases():
    g = golden("whfast_advanced.npz")
    return [(int(c), int(c2), KERNELS[int(k)]) for c, c2, k in g["settings"]]


def advanced_sim(g, c, c2, kernel, shift=0.0, safe=1, keep=0):
    p = g["oss"].copy()
    p["vx"] += shift
    return O.Sim(p, dt=float(g["dt"]), safe_mode=safe, corrector=c, corrector2=c2, kernel=kernel,
                 keep_unsynchronized=keep)


@pytest.mark.parametrize("c,c2,kernel", advanced_cases())
def test_oracle_whfast_correctors_and_kernels(c, c2, kernel):
    # WHFast correctors / kernels against the reference's own runs of
    # rebound/tests/test_whfast_advanced.py, bit for bit
    g = golden("whfast_advanced.npz")
    tag = "c%d_c2%d_%s" % (c, c2, kernel)
    s = advanced_sim(g, c, c2, kernel, safe=0)
    s.whfast(20)
    s.whfast_synchronize()
    assert max_diff(s.p, g["traj_" + tag]) == 0.0
    s = advanced_sim(g, c, c2, kernel, safe=0)
    e0 = s.energy()
    s.whfast_integrate(1000. * 2. * 3.1415)
    assert max_diff(s.p, g["energy_end_" + tag]) == 0.0
    assert abs((e0 - s.energy()) / s.energy()) == float(g["energy_err_" + tag])
    s = advanced_sim(g, c, c2, kernel, shift=1.0)
    s.whfast_integrate(1000. * 2. * 3.1415)
    assert max_diff(s.p, g["notcom_end_" + tag]) == 0.0
    s = advanced_sim(g, c, c2, kernel, shift=1050.)
    s.whfast_integrate(13.21415, exact_finish_time=0)
    assert max_diff(s.p, g["compias_end_" + tag]) == 0.0 and s.s.t == float(g["compias_t_" + tag])
    s = advanced_sim(g, c, c2, kernel, shift=1.0)
    s.whfast(10)
    s.s.dt *= -1
    s.whfast(10)
    assert max_diff(s.p, g["bf_end_" + tag]) == 0.0


@pytest.mark.parametrize("c", [0, 5])
def test_oracle_whfast_keep_unsynchronized(c):
    g = golden("whfast_advanced.npz")
    s = advanced_sim(g, c, 0, "default", safe=0, keep=1)
    s.whfast(10)
    s.whfast_synchronize()
    assert max_diff(s.p, g["keep_mid_c%d" % c]) == 0.0
    s.whfast(10)
    s.whfast_synchronize()
    assert max_diff(s.p, g["keep_end_c%d" % c]) == 0.0


def coords_cases():
    g = golden("whfast_coords.npz")
    cases = []
    for N in (1, 2):
        cases += [("tp_N%d" % N, "tp_N%d_jacobi_na%d" % (N, na), 1e-1, na, 0) for na in [-1] + list(range(1, N + 2))]
        cases += [("tpp_N%d" % N, "tpp_N%d_jacobi_na%d" % (N, na), 1e-3, na, 0) for na in [-1] + list(range(3, N + 4))]
    cases += [("tp1", "tp1_jacobi_na%d" % na, 1e-3, na, 1) for na in (-1, 1)]
    cases += [("tp1p", "tp1p_jacobi_na%d" % na, 1e-3, na, 1) for na in (-1, 3)]
    return cases


@pytest.mark.parametrize("start,end,dt,na,tp", coords_cases())
def test_oracle_whfast_test_particles(start, end, dt, na, tp):
    # rebound/tests/test_whfast_testparticles.py, Jacobi coordinates: the reference's
    # own end states, bit for bit (N_active as WHFast reads it for testparticle_type 1)
    g = golden("whfast_coords.npz")
    s = O.Sim(g[start], dt=dt, N_active=None if na < 0 else na, testparticle_type=tp)
    s.whfast_integrate(1.0)
    assert max_diff(s.p, g[end]) == 0.0


@pytest.mark.parametrize("theta2", [0.25, 0.5])
def test_oracle_tree_quadrupole(theta2):
    # the tree with quadrupole moments against the reference built with -DQUADRUPOLE
    gq = golden("tree_quadrupole.npz")
    g = golden("ring_patch.npz")
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]
    s = O.Sim(gq["particles"], G=G, softening=soft, dt=dt, boundary="shear", root_size=rs,
              N_root=(int(nx), int(ny), int(nz)), N_ghost=(int(gx), int(gy), int(gz)), OMEGA=OM,
              opening_angle2=theta2, t=t, quadrupole=1)
    acc = s.gravity("tree")
    assert np.array_equal(acc, gq["acc_quad_t%g" % theta2])
    s.s.tree_quadrupole = 0
    assert np.array_equal(s.gravity("tree"), gq["acc_mono_t%g" % theta2])


COORDS = ("jacobi", "democraticheliocentric", "whds", "barycentric")


@pytest.mark.parametrize("coords,safe", [(c, s) for c in ("democraticheliocentric", "whds", "barycentric")
                                         for s in (1, 0)])
def test_oracle_whfast_other_coordinates(coords, safe):
    # 100-step two-planet runs of the reference in each coordinate system, bit for bit
    import math
    name, key = ("whfast_dh.npz", "two_after100_safe%d" % safe) if coords == "democraticheliocentric" \
        else ("whfast_coords.npz", "two_%s_safe%d" % (coords, safe))
    g = golden(name)
    s = O.Sim(g["two"], dt=0.005123 * 2. * math.pi, safe_mode=safe, coordinates=coords)
    s.whfast(100)
    s.whfast_synchronize()
    assert max_diff(s.p, g[key]) == 0.0


@pytest.mark.parametrize("order,safe,n", [(5, 0, 50), (17, 1, 10)])
def test_oracle_whfast_barycentric_correctors(order, safe, n):
    import math
    g = golden("whfast_coords.npz")
    s = O.Sim(g["two"], dt=0.005123 * 2. * math.pi, safe_mode=safe, coordinates="barycentric", corrector=order)
    s.whfast(n)
    s.whfast_synchronize()
    assert max_diff(s.p, g["two_barycentric_c%d" % order]) == 0.0


def test_oracle_whds_outer_solar_system():
    g = golden("whfast_coords.npz")
    s = O.Sim(g["oss"], dt=0.005 * 12. * 2. * 3.1415, coordinates="whds")
    s.whfast_integrate(1000. * 2. * 3.1415)
    assert max_diff(s.p, g["whds_oss_end"]) == 0.0


@pytest.mark.parametrize("coords", COORDS)
def test_oracle_test_particles_every_coordinate_system(coords):
    # rebound/tests/test_whfast_testparticles.py scenarios, the reference's end states
    g = golden("whfast_coords.npz")
    for N in (1, 2):
        for start, dt, nas in (("tp_N%d" % N, 0.1, [-1] + list(range(1, N + 2))),
                               ("tpp_N%d" % N, 1e-3, [-1] + list(range(3, N + 4)))):
            for na in nas:
                s = O.Sim(g[start], dt=dt, N_active=None if na < 0 else na, coordinates=coords)
                s.whfast_integrate(1.0)
                assert max_diff(s.p, g["%s_%s_na%d" % (start, coords, na)]) == 0.0, (start, na)


@pytest.mark.parametrize("gravity", ["compensated", "none"])
@pytest.mark.parametrize("coords", COORDS)
def test_oracle_whfast_gravity_modes(gravity, coords):
    g = golden("whfast_gravity.npz")
    s = O.Sim(g["oss"], dt=0.5, safe_mode=0, coordinates=coords, whfast_gravity=gravity)
    s.whfast(100)
    s.whfast_synchronize()
    assert max_diff(s.p, g["oss_%s_%s" % (gravity, coords)]) == 0.0


def test_oracle_whfast_compensated_test_particles():
    # rebound/tests/test_gravity.py:55-94 runs, the reference's own end states
    g = golden("whfast_gravity.npz")
    s = O.Sim(g["comp0_start"], dt=float(g["comp0_dt"]), N_active=1, whfast_gravity="compensated")
    s.whfast_integrate(10.)
    assert max_diff(s.p, g["comp0_end"]) == 0.0 and s.p["x"][0] == 0.0
    s = O.Sim(g["comp1_start"], dt=1e-4, N_active=2, testparticle_type=1, whfast_gravity="compensated")
    s.whfast_integrate(10.)
    assert max_diff(s.p, g["comp1_end_whfast"]) == 0.0


def shuffled_like_reference(pairs, seed):
    """The post-search rand_r shuffle of src/collision.c:336-342 (C library rand_r)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.rand_r.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    out = pairs.copy()
    s = ctypes.c_uint(int(seed))
    for i in range(len(out)):
        j = libc.rand_r(ctypes.byref(s)) % len(out)
        tmp = out[i].copy()
        out[i] = out[j]
        out[j] = tmp
    return out


@pytest.mark.parametrize("scene", ["ring", "box"])
@pytest.mark.parametrize("mode", ["line", "linetree"])
def test_oracle_line_searches(scene, mode):
    # LINE / LINETREE on the reference's post-step states: the reference's lists entry
    # for entry after its shuffle
    g = golden("collision_line.npz")
    if scene == "ring":
        G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = golden("ring_patch.npz")["meta"]
        s = O.Sim(g["ring_after1"], G=G, softening=soft, dt=dt, boundary="shear", root_size=rs,
                  N_root=(int(nx), int(ny), int(nz)), N_ghost=(int(gx), int(gy), int(gz)), OMEGA=OM,
                  t=t + dt)                                  # one step in: the shear offset moves with t
    else:
        dt = 0.3
        s = O.Sim(g["box_after1"], dt=dt, boundary="periodic", root_size=10., N_ghost=(1, 1, 1))
    got = shuffled_like_reference(s.collisions(mode, dt_last_done=dt), g["%s_seed_%s" % (scene, mode)])
    ref = g["%s_pairs_%s" % (scene, mode)]
    assert len(got) == len(ref) > 0
    assert np.array_equal(got["p1"], ref["p1"]) and np.array_equal(got["p2"], ref["p2"])
    assert np.array_equal(got["gb"], ref["gb"])
    if mode == "linetree":
        assert np.array_equal(got["ri"], ref["ri"])


def test_oracle_reference_unit_scenarios():
    # the reference's own unit-test runs (rebound/tests/test_leapfrog.py:14-22,
    # test_whfast.py:20-69, 307-345): the oracle reaches the reference's energy
    # errors exactly and its forward-backward end states bit for bit
    import math
    g = golden("reference_cases.npz")

    def rel(a, b):
        return abs((a - b) / b)

    s = O.Sim(g["oss"], dt=1.0)
    e0 = s.energy()
    s.leapfrog(1000)
    assert rel(e0, s.energy()) == float(g["oss_leapfrog_err"])
    for start, dt, tmax, key in (("oss_raw", 0.005 * 12. * 2. * 3.1415, 1000. * 2. * 3.1415, "oss_whfast_err"),
                                 ("hyper", 0.00512 * float(g["hyper_yr"]), 1e2 * float(g["hyper_yr"]), "hyper_err"),
                                 ("two", 0.005123 * 2. * math.pi, 1e3 * 2. * math.pi, "two_err")):
        s = O.Sim(g[start], dt=dt)
        e0 = s.energy()
        s.whfast_integrate(tmax)
        assert rel(e0, s.energy()) == float(g[key]), start
    for name in ("bf_hyper", "bf_ecc"):
        s = O.Sim(g[name], dt=float(g[name + "_dt"]))
        s.whfast(100)
        s.s.dt *= -1
        s.whfast(100)
        s.whfast_synchronize()
        assert max_diff(s.p, g[name + "_end"]) == 0.0, name


@pytest.mark.parametrize("coords,safe,corrector", [("jacobi", 0, 0), ("jacobi", 1, 0), ("jacobi", 0, 5),
                                                   ("jacobi", 1, 5), ("democraticheliocentric", 0, 0),
                                                   ("democraticheliocentric", 1, 0), ("whds", 0, 0),
                                                   ("whds", 1, 0)])
def test_oracle_archive_scenarios(coords, safe, corrector):
    # the uninterrupted runs of rebound/tests/test_simulationarchive.py:86-365 to
    # t = 80 with exact_finish_time = 0: the reference's end state and time
    g = golden("archive_cases.npz")
    tag = "%s_safe%d_c%d" % (coords, safe, corrector)
    s = O.Sim(g["start"], dt=0.1313, safe_mode=safe, coordinates=coords, corrector=corrector)
    s.whfast_integrate(80., exact_finish_time=0)
    assert max_diff(s.p, g["end_" + tag]) == 0.0 and s.s.t == float(g["t_" + tag])


def test_oracle_sim_layout_matches_header(tmp_path):
    # the checker's own ctypes mirror of orc_sim must match oracle/oracle.h
    import ctypes
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = [f[0] for f in O.OrcSim._fields_]
    src = tmp_path / "orc.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "oracle.h"', 'int main(void) {',
             '  printf("size %zu\\n", sizeof(orc_sim));']
    lines += ['  printf("%s %%zu\\n", offsetof(orc_sim, %s));' % (n, n) for n in names]
    lines += ['  return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "orc"
    subprocess.check_call([cc, "-I", os.path.dirname(os.path.abspath(O.__file__)), str(src), "-o", str(exe)])
    out = {k: int(v) for k, v in (l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())}
    assert out["size"] == ctypes.sizeof(O.OrcSim)
    for n in names:
        assert out[n] == getattr(O.OrcSim, n).offset, n
