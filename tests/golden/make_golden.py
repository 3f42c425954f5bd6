"""Generate golden fixtures from the UNMODIFIED reference (REBOUND 5.0.0).

Run in a container that has the reference sources (it reads them where they
lie and never copies them):

    make -f oracle/ref.mk REF=<reference checkout>      # builds oracle/_ref/ (incl. the -DQUADRUPOLE build)
    python tests/golden/make_golden.py <reference checkout>

The reference's own Python package is imported from the checkout and loads the
serial, -ffp-contract=off build of its C core from oracle/_ref/.  Each fixture
stores the input state next to the reference's outputs so that tests replay
identical inputs through the oracle and the CUDA path on any machine.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if len(sys.argv) < 2 and not os.environ.get("REBOUND_REF"):
    sys.exit("usage: make_golden.py <reference checkout> [fixture ...]  (or set REBOUND_REF)")
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ["REBOUND_REF"]
sys.dont_write_bytecode = True
sys.path[:0] = [os.path.join(REPO, "oracle", "_ref"), REF, REPO]

import rebound  # noqa: E402  (the reference package)
from rebound import clibrebound  # noqa: E402

from oracle.oracle import PARTICLE_DTYPE, COLLISION_DTYPE, CELL_DTYPE  # noqa: E402

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m", "r")
clibrebound.reb_simulation_add_plummer.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_double]
clibrebound.reb_random_uniform.restype = ctypes.c_double
clibrebound.reb_random_normal.restype = ctypes.c_double
clibrebound.reb_random_powerlaw.restype = ctypes.c_double
clibrebound.reb_random_rayleigh.restype = ctypes.c_double
clibrebound.reb_simulation_energy.restype = ctypes.c_double


def state(sim):
    """Copy the reference's particle array (struct reb_particle AoS) into our dtype."""
    n = sim.N
    buf = (ctypes.c_char * (112 * n)).from_address(ctypes.addressof(sim.particles[0]))
    arr = np.frombuffer(bytes(buf), dtype=PARTICLE_DTYPE).copy()
    arr["name"] = 0
    arr["ap"] = 0
    arr["sim"] = 0
    return arr


def load(sim, arr):
    for p in arr:
        sim.add(m=float(p["m"]), r=float(p["r"]), x=float(p["x"]), y=float(p["y"]), z=float(p["z"]),
                vx=float(p["vx"]), vy=float(p["vy"]), vz=float(p["vz"]))


def accel(sim):
    clibrebound.reb_simulation_update_acceleration(ctypes.byref(sim))
    s = state(sim)
    return np.stack([s["ax"], s["ay"], s["az"]], axis=1)


def energy(sim):
    return clibrebound.reb_simulation_energy(ctypes.byref(sim))


def plummer_truncated(n, seed, rmax=10.0):
    """reb_simulation_add_plummer (src/tools.c:463-502), keeping r <= rmax in order."""
    scratch = rebound.Simulation()
    scratch.rand_seed = seed
    clibrebound.reb_simulation_add_plummer(ctypes.byref(scratch), int(n * 1.05) + 64, 1.0, 1.0)
    s = state(scratch)
    rr = np.sqrt(s["x"] ** 2 + s["y"] ** 2 + s["z"] ** 2)
    s = s[rr <= rmax][:n].copy()
    s["m"] = 1.0 / n
    return s


def fixture_gravity_plummer():
    n, seed = 4096, 11
    raw = rebound.Simulation()
    raw.rand_seed = seed
    clibrebound.reb_simulation_add_plummer(ctypes.byref(raw), 64, 1.0, 1.0)
    plummer_raw = state(raw)                      # first 64 untruncated draws, for the IC generator
    p0 = plummer_truncated(n, seed)
    out = {"plummer_raw": plummer_raw, "plummer_seed": np.int64(seed), "particles": p0}
    for mode in ("basic", "compensated"):
        sim = rebound.Simulation()
        sim.softening = 0.01
        sim.gravity = mode
        load(sim, p0)
        out["acc_" + mode] = accel(sim)
    sim = rebound.Simulation()
    sim.softening = 0.01
    sim.gravity = "basic"
    sim.integrator = "leapfrog"
    sim.dt = 1e-3
    load(sim, p0)
    out["energy0"] = np.float64(energy(sim))
    sim.steps(10)
    out["after10"] = state(sim)
    sim.steps(990)
    out["after1000"] = state(sim)
    out["energy1000"] = np.float64(energy(sim))
    np.savez_compressed(os.path.join(HERE, "gravity_plummer.npz"), **out)


def fixture_gravity_cases():
    """Edge cases of src/gravity.c: test particles, ignore terms, ghost boxes, no softening."""
    rng = np.random.default_rng(5)
    out = {}
    for name, n, n_active, tp, ign, ghost, soft in (
            ("plain", 37, None, 0, 0, 0, 0.0),
            ("testp0", 41, 29, 0, 0, 0, 0.02),
            ("testp1", 41, 29, 1, 0, 0, 0.02),
            ("ignore01", 23, None, 0, 1, 0, 0.0),
            ("ignore0", 23, None, 0, 2, 0, 0.0),
            ("ghost", 19, None, 0, 0, 1, 0.05),
            ("single", 1, None, 0, 0, 0, 0.0),
            ("two", 2, None, 0, 0, 0, 0.0)):
        p = np.zeros(n, dtype=PARTICLE_DTYPE)
        for k in ("x", "y", "z"):
            p[k] = rng.uniform(-0.9, 0.9, n)
        for k in ("vx", "vy", "vz"):
            p[k] = rng.normal(0, 0.1, n)
        p["m"] = rng.uniform(0.1, 1.0, n) / n
        for mode in ("basic", "compensated"):
            if ghost and mode == "compensated":
                continue                          # COMPENSATED has no ghost-box loop (src/gravity.c:284-531)
            sim = rebound.Simulation()
            sim.softening = soft
            sim.gravity = mode
            if ghost:
                sim.root_size = 2.0
                sim.boundary = "periodic"
                sim.N_ghost_x = sim.N_ghost_y = sim.N_ghost_z = 1
            load(sim, p)
            if n_active is not None:
                sim.N_active = n_active
            sim.testparticle_type = tp
            sim.gravity_ignore = ign
            out[f"{name}_particles"] = p
            out[f"{name}_acc_{mode}"] = accel(sim)
        out[f"{name}_meta"] = np.array([n, -1 if n_active is None else n_active, tp, ign, ghost, soft * 1e6],
                                       dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "gravity_cases.npz"), **out)


def fixture_gravity_hierarchical():
    """BASIC and COMPENSATED accelerations of hierarchical systems, whose small
    coordinates lie far below the largest one: a tight binary near the origin in
    a wide system, a cluster at the origin beside a distant body, and the
    configuration-1 Plummer sphere with a tight binary at its centre."""
    rng = np.random.default_rng(21)
    cases = {}
    # tight binary (separation ~3.7e-7) at ~4e-4 from the origin, 30 field bodies out to ~1e2, one body at 1e3
    p = np.zeros(33, dtype=PARTICLE_DTYPE)
    c = np.array([1e-4, -2e-4, 3e-4])
    h = np.array([3e-7, 1e-7, -2e-7]) * 0.5
    p[0]["x"], p[0]["y"], p[0]["z"] = c + h
    p[1]["x"], p[1]["y"], p[1]["z"] = c - h
    r = 10 ** rng.uniform(-2, 2, 30)
    u = rng.normal(size=(30, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    for k, f in enumerate(("x", "y", "z")):
        p[f][2:32] = r * u[:, k]
    p[32]["x"] = 1e3
    p["m"] = rng.uniform(0.5, 1.5, 33) * 1e-3
    cases["binary_wide"] = (p, 0.0)
    # cluster of 2048 at the origin (sigma 1e-2) beside one body at 1e3
    n = 2048
    q = np.zeros(n, dtype=PARTICLE_DTYPE)
    q["x"], q["y"], q["z"] = rng.standard_normal((3, n)) * 1e-2
    q["x"][0] = 1e3
    q["m"] = 1.0 / n
    cases["cluster_far"] = (q, 0.0)
    # the N=4,096 Plummer sphere with a tight binary (separation 2e-6) near its centre
    pl = plummer_truncated(4096, 11)
    b = np.zeros(2, dtype=PARTICLE_DTYPE)
    cb = np.array([2.5e-3, -1.5e-3, 1e-3])
    hb = np.array([1e-6, -5e-7, 5e-7])
    b[0]["x"], b[0]["y"], b[0]["z"] = cb + hb
    b[1]["x"], b[1]["y"], b[1]["z"] = cb - hb
    b["m"] = 1.0 / 4096
    cases["plummer_binary"] = (np.concatenate([pl, b]), 0.0)
    out = {}
    for name, (arr, soft) in cases.items():
        out[name + "_particles"] = arr
        out[name + "_softening"] = np.float64(soft)
        for mode in ("basic", "compensated"):
            sim = rebound.Simulation()
            sim.softening = soft
            sim.gravity = mode
            load(sim, arr)
            out[f"{name}_acc_{mode}"] = accel(sim)
    np.savez_compressed(os.path.join(HERE, "gravity_hierarchical.npz"), **out)


def ring_patch(L, seed, omega=1.3143527e-4, surface_density=400., rho=400.):
    """Config-3 style shearing-sheet patch (examples/shearing_sheet/problem.c pattern)."""
    sim = rebound.Simulation()
    sim.rand_seed = seed
    sim.OMEGA = omega
    sim.G = 6.674e-11
    sim.softening = 0.1
    sim.dt = 1e-3 * 2. * np.pi / omega
    sim.integrator = "sei"
    sim.boundary = "shear"
    sim.gravity = "tree"
    sim.collision = "tree"
    sim.collision_resolve = "hardsphere"
    sim.root_size = 20.0
    sim.N_root_x = int(L / 20)
    sim.N_root_y = int(L / 20)
    sim.N_root_z = 1
    sim.N_ghost_x = 2
    sim.N_ghost_y = 2
    sim.N_ghost_z = 0
    sim.opening_angle2 = 0.25
    sp = ctypes.byref(sim)
    total = 0.0
    lx = ly = L
    while total < surface_density * lx * ly:
        rad = clibrebound.reb_random_powerlaw(sp, ctypes.c_double(1.), ctypes.c_double(4.), ctypes.c_double(-3.))
        x = clibrebound.reb_random_uniform(sp, ctypes.c_double(-lx / 2), ctypes.c_double(lx / 2))
        y = clibrebound.reb_random_uniform(sp, ctypes.c_double(-ly / 2), ctypes.c_double(ly / 2))
        while True:
            z = clibrebound.reb_random_normal(sp, ctypes.c_double(25.0))   # variance = sigma^2, sigma = 5 m
            if abs(z) < 10.0:
                break
        vx = clibrebound.reb_random_normal(sp, ctypes.c_double(0.0005 ** 2))
        vy = -1.5 * x * omega + clibrebound.reb_random_normal(sp, ctypes.c_double(0.0005 ** 2))
        vz = clibrebound.reb_random_normal(sp, ctypes.c_double(0.0005 ** 2))
        m = rho * 4. / 3. * np.pi * rad ** 3
        sim.add(m=m, r=rad, x=x, y=y, z=z, vx=vx, vy=vy, vz=vz)
        total += m
    return sim


class TreeCellC(ctypes.Structure):
    pass


TreeCellC._fields_ = [(k, ctypes.c_double) for k in ("x", "y", "z", "w", "m", "mx", "my", "mz")] + [
    ("oct", ctypes.POINTER(TreeCellC) * 8), ("pt", ctypes.c_int), ("remote", ctypes.c_int)]


def export_tree(sim):
    """Walk the reference's pointer octree (src/tree.h:81-103) depth-first, octants 0..7."""
    sp = ctypes.byref(sim)
    clibrebound.reb_tree_construct(sp)
    clibrebound.reb_tree_calculate_gravity_data(sp)
    nroot = sim.N_root_x * sim.N_root_y * sim.N_root_z
    roots = ctypes.cast(sim._tree_root, ctypes.POINTER(ctypes.POINTER(TreeCellC) * nroot)).contents
    cells = []

    def rec(c, root, depth, path):
        cells.append((root, depth, path, c.x, c.y, c.z, c.w, c.m, c.mx, c.my, c.mz, c.pt))
        for o in range(8):
            if c.oct[o]:
                rec(c.oct[o].contents, root, depth + 1, (path << 3) | o)

    for i in range(nroot):
        if roots[i]:
            rec(roots[i].contents, i, 0, 0)
    clibrebound.reb_tree_delete(sp)
    return np.array(cells, dtype=CELL_DTYPE)


NOOP_RESOLVE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_byte * 72)(lambda s, c: 0)


def collision_pairs(sim, mode):
    """reb_collision_search (src/collision.c:49) with a no-op resolver; returns the stored pair list."""
    sim.collision = mode
    sim._collision_resolve = ctypes.cast(NOOP_RESOLVE, type(sim._collision_resolve))
    clibrebound.reb_collision_search(ctypes.byref(sim))
    n = sim.N_collisions
    if n == 0:
        return np.zeros(0, dtype=COLLISION_DTYPE)
    buf = (ctypes.c_char * (72 * n)).from_address(sim.collisions)
    return np.frombuffer(bytes(buf), dtype=COLLISION_DTYPE).copy()


def fixture_ring():
    sim = ring_patch(200.0, seed=7)
    out = {"particles": state(sim),
           "meta": np.array([sim.G, sim.OMEGA, sim.softening, sim.dt, sim.root_size, sim.N_root_x,
                             sim.N_root_y, sim.N_root_z, 2, 2, 0, sim.opening_angle2, sim.t], dtype=np.float64)}
    out["cells"] = export_tree(sim)
    out["acc_tree"] = accel(sim)
    sim.gravity = "basic"
    out["acc_basic"] = accel(sim)
    sim.gravity = "tree"
    out["pairs_direct"] = collision_pairs(sim, "direct")
    out["pairs_tree"] = collision_pairs(sim, "tree")
    # A few full SEI + tree gravity + tree collision + hardsphere steps.
    sim2 = ring_patch(200.0, seed=7)
    sim2.coefficient_of_restitution = lambda s, v: 0.5
    out["after5_seed0"] = np.int64(sim2.rand_seed)       # shuffle seed when stepping starts
    sim2.steps(5)
    out["after5"] = state(sim2)
    out["after5_t"] = np.float64(sim2.t)
    out["after5_seed"] = np.int64(sim2.rand_seed)
    out["after5_collisions_log_n"] = np.int64(sim2.collisions_log_n)
    out["after5_collisions_plog"] = np.float64(sim2.collisions_plog)
    # The same five steps with the velocity-dependent restitution coefficient of the
    # reference's own shearing-sheet test (rebound/tests/test_shearingsheet.py:26-32).
    sim3 = ring_patch(200.0, seed=7)

    def cor_bridges(r, v):
        eps = 0.32 * pow(abs(v) * 100., -0.234)
        return min(1., max(0., eps))
    sim3.coefficient_of_restitution = cor_bridges
    sim3.steps(5)
    out["bridges_after5"] = state(sim3)
    out["bridges_after5_seed"] = np.int64(sim3.rand_seed)
    out["bridges_after5_collisions_log_n"] = np.int64(sim3.collisions_log_n)
    out["bridges_after5_collisions_plog"] = np.float64(sim3.collisions_plog)
    np.savez_compressed(os.path.join(HERE, "ring_patch.npz"), **out)


def planetary_system(sim, k, seed_sim):
    """Config-4 style system: star + k planets (log-uniform m, a; Rayleigh e, i)."""
    sp = ctypes.byref(seed_sim)
    U = lambda a, b: clibrebound.reb_random_uniform(sp, ctypes.c_double(a), ctypes.c_double(b))
    R = lambda s: clibrebound.reb_random_rayleigh(sp, ctypes.c_double(s))
    sim.add(m=1.0)
    while True:
        ms = np.exp([U(np.log(1e-7), np.log(1e-3)) for _ in range(k)])
        a = np.sort(np.exp([U(np.log(0.5), np.log(30.)) for _ in range(k)]))
        rh = ((ms[:-1] + ms[1:]) / 3.) ** (1. / 3.) * (a[:-1] + a[1:]) / 2.
        if np.all(np.diff(a) >= 3. * rh):
            break
    for j in range(k):
        sim.add(m=float(ms[j]), a=float(a[j]), e=float(R(0.02)), inc=float(R(0.01)),
                Omega=U(0, 2 * np.pi), omega=U(0, 2 * np.pi), f=U(0, 2 * np.pi))
    sim.move_to_com()
    return 2 * np.pi * np.sqrt(a[0] ** 3)


def fixture_whfast():
    seeder = rebound.Simulation()
    seeder.rand_seed = 3
    systems = []
    for s in range(8):
        k = 2 + (s % 9)
        sim = rebound.Simulation()
        p_inner = planetary_system(sim, k, seeder)
        sim.integrator = "whfast"
        sim.dt = p_inner / 20.
        p0 = state(sim)
        e0 = energy(sim)
        sim.steps(100)
        p100 = state(sim)
        sim.steps(900)
        systems.append((p0, p100, state(sim), sim.dt, e0, energy(sim)))
    out = {}
    for s, (p0, p100, p1000, dt, e0, e1) in enumerate(systems):
        out[f"sys{s}_p0"] = p0
        out[f"sys{s}_p100"] = p100
        out[f"sys{s}_p1000"] = p1000
        out[f"sys{s}_meta"] = np.array([dt, e0, e1])
    # Kepler solver cases (src/integrator_whfast.c:241), elliptic and hyperbolic, incl. steps > 1 period.
    rng = np.random.default_rng(9)
    ks = np.zeros(64, dtype=PARTICLE_DTYPE)
    for k in ("x", "y", "z"):
        ks[k] = rng.normal(size=64)
    for k in ("vx", "vy", "vz"):
        ks[k] = rng.normal(size=64) * np.where(np.arange(64) % 4 == 0, 2.0, 0.7)
    mus = rng.uniform(0.5, 2.0, 64)
    dts = rng.uniform(-3.0, 3.0, 64) * np.where(np.arange(64) % 5 == 0, 10.0, 0.1)
    clibrebound.reb_integrator_whfast_kepler_solver.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    kout = ks.copy()
    for i in range(64):
        clibrebound.reb_integrator_whfast_kepler_solver(kout[i:i + 1].ctypes.data, mus[i], dts[i], None)
    out["kepler_in"] = ks
    out["kepler_mu"] = mus
    out["kepler_dt"] = dts
    out["kepler_out"] = kout
    np.savez_compressed(os.path.join(HERE, "whfast.npz"), **out)


def fixture_sei_periodic():
    """SEI + BASIC gravity + shear boundary without collisions (trajectory parity)."""
    sim = ring_patch(100.0, seed=21)
    sim.collision = "none"
    sim.gravity = "basic"
    p0 = state(sim)
    meta = np.array([sim.G, sim.OMEGA, sim.softening, sim.dt, sim.root_size,
                     sim.N_root_x, sim.N_root_y, sim.N_root_z, 2, 2, 0, sim.t])
    sim.steps(20)
    np.savez_compressed(os.path.join(HERE, "sei_shear.npz"), particles=p0, after20=state(sim), meta=meta)


def fixture_reference_cases():
    """Scenarios of the reference's own unit tests for this path (leapfrog and
    WHFast energy thresholds, forward/backward reversibility), with the inputs the
    reference builds (its "outer solar system" data set, orbital elements) and
    the errors the reference itself reaches on them."""
    import math
    out = {}

    def rel(a, b):
        return abs((a - b) / b)

    # outer solar system, moved to the centre of mass (rebound/tests/test_leapfrog.py:7-9)
    sim = rebound.Simulation()
    sim.add("outer solar system")
    sim.move_to_com()
    out["oss"] = state(sim)
    sim.integrator = "leapfrog"
    sim.dt = 1.
    e0 = sim.energy()
    sim.integrate(1e3)
    out["oss_leapfrog_err"] = rel(e0, sim.energy())          # test_leapfrog.py:14-22 (bar 1e-3)
    sim = rebound.Simulation()
    sim.add("outer solar system")
    sim.integrator = "whfast"
    sim.dt = 0.005 * 12. * 2. * 3.1415
    out["oss_raw"] = state(sim)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    out["oss_whfast_err"] = rel(e0, sim.energy())            # test_whfast.py:20-29 (bar 2.4e-8)
    # hyperbolic orbit (test_whfast.py:43-54, bar 1e-14)
    sim = rebound.Simulation()
    sim.add(m=1.)
    sim.add(m=1e-3, a=-1., e=2.5)
    out["hyper"] = state(sim)
    yr = -sim.particles[1].P
    out["hyper_yr"] = yr
    sim.integrator = "whfast"
    sim.dt = 0.00512 * yr
    e0 = sim.energy()
    sim.integrate(1e2 * yr)
    out["hyper_err"] = rel(e0, sim.energy())
    # two planets (test_whfast.py:56-69, bar 1.2e-8)
    sim = rebound.Simulation()
    sim.add(m=1.)
    sim.add(m=1e-3, a=1., e=.1)
    sim.add(m=1e-3, a=3., e=0.1)
    out["two"] = state(sim)
    sim.integrator = "whfast"
    sim.dt = 0.005123 * 2. * math.pi
    e0 = sim.energy()
    sim.integrate(1e3 * 2. * math.pi)
    out["two_err"] = rel(e0, sim.energy())
    # forward then backward (test_whfast.py:307-345, bars 1e-14 and 1e-13)
    for name, kw, per_sign in (("bf_hyper", dict(a=-1., e=2.5, omega=0.3, Omega=0.4, inc=0.1), -1.),
                               ("bf_ecc", dict(a=1.4, e=0.0125, omega=0.3, Omega=0.4, inc=0.1), 1.)):
        sim = rebound.Simulation()
        sim.add(m=1.)
        sim.add(m=1e-3, **kw)
        out[name] = state(sim)
        yr = per_sign * sim.particles[1].P
        sim.integrator = "whfast"
        sim.dt = 0.0512 * yr
        out[name + "_dt"] = sim.dt
        sim.steps(100)
        sim.dt *= -1
        sim.steps(100)
        out[name + "_end"] = state(sim)
    np.savez_compressed(os.path.join(HERE, "reference_cases.npz"), **out)


def fixture_leapfrog_orders():
    """Leapfrog orders 4, 6, 8 (src/integrator_leapfrog.c:97-203): 20 steps of a
    softened 128-body Plummer sphere with BASIC gravity, and the outer-solar-system
    energy errors of rebound/tests/test_leapfrog.py:24-56 (integrate(1e3), steps(1))."""
    out = {}
    p0 = plummer_truncated(128, seed=21)
    out["particles"] = p0
    for order in (4, 6, 8):
        sim = rebound.Simulation()
        load(sim, p0)
        sim.softening = 0.01
        sim.integrator = "leapfrog"
        sim.integrator.order = order
        sim.dt = 1e-3
        sim.steps(20)
        out["after20_o%d" % order] = state(sim)
        out["t_o%d" % order] = sim.t
        sim = rebound.Simulation()
        sim.add("outer solar system")
        sim.move_to_com()
        sim.integrator = "leapfrog"
        sim.integrator.order = order
        sim.dt = 1
        e0 = sim.energy()
        sim.integrate(1e3)
        sim.steps(1)
        out["oss_err_o%d" % order] = abs((e0 - sim.energy()) / sim.energy())
    np.savez_compressed(os.path.join(HERE, "leapfrog_orders.npz"), **out)


def fixture_whfast_dh():
    """WHFast in democratic heliocentric coordinates (src/integrator_whfast.c with
    coordinates = DEMOCRATICHELIOCENTRIC): the scenarios of
    rebound/tests/test_whfast.py:212-305 with the reference's own errors, and a
    100-step trajectory of the two-planet system (safe_mode 1 and 0)."""
    import math
    out = {}

    def rel(a, b):
        return abs((a - b) / b)

    def dh(sim, dt, safe=1):
        sim.integrator = "whfast"
        sim.integrator.coordinates = "democraticheliocentric"
        sim.integrator.safe_mode = safe
        sim.dt = dt

    sim = rebound.Simulation()
    sim.add("outer solar system")
    out["oss"] = state(sim)
    dh(sim, 0.005 * 12. * 2. * 3.1415)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    out["oss_err"] = rel(e0, sim.energy())                   # bar 1.5e-8
    sim = rebound.Simulation()
    sim.add(m=1.)
    sim.add(m=1e-3, a=-1., e=2.5)
    out["hyper"] = state(sim)
    yr = -sim.particles[1].P
    out["hyper_yr"] = yr
    dh(sim, 0.00512 * yr)
    e0 = sim.energy()
    sim.integrate(1e2 * yr)
    out["hyper_err"] = rel(e0, sim.energy())                 # bar 4.5e-8
    jupyr = 2. * math.pi
    for safe in (1, 0):
        sim = rebound.Simulation()
        sim.add(m=1.)
        sim.add(m=1e-3, a=1., e=.1)
        sim.add(m=1e-3, a=3., e=0.1)
        out["two"] = state(sim)
        dh(sim, 0.005123 * jupyr, safe)
        e0 = sim.energy()
        sim.integrate(1e3 * jupyr)
        out["two_err_safe%d" % safe] = rel(e0, sim.energy())  # bar 2.9e-8
        sim = rebound.Simulation()
        load(sim, out["two"])
        dh(sim, 0.005123 * jupyr, safe)
        sim.steps(100)
        if not safe:
            sim.integrator.synchronize() if hasattr(sim.integrator, "synchronize") else sim.synchronize()
        out["two_after100_safe%d" % safe] = state(sim)
    # safe_mode 0: steps, synchronize, more steps from the synchronized coordinates
    for coords in ("jacobi", "democraticheliocentric"):
        sim = rebound.Simulation()
        load(sim, out["two"])
        dh(sim, 0.005123 * jupyr, 0)
        sim.integrator.coordinates = coords
        sim.steps(50)
        sim.synchronize()
        sim.steps(50)
        sim.synchronize()
        out["two_sync_mid_" + coords] = state(sim)
    for tag, order in (("order12", (1., 3.)), ("order21", (3., 1.))):
        sim = rebound.Simulation()
        sim.add(m=1.)
        for a in order:
            sim.add(m=1e-3, a=a, e=0.1, primary=sim.particles[0])
        out[tag] = state(sim)
        dh(sim, 0.005123 * jupyr)
        sim.integrate(1e0 * jupyr)
        out[tag + "_end"] = state(sim)
    np.savez_compressed(os.path.join(HERE, "whfast_dh.npz"), **out)


def fixture_whfast_advanced():
    """WHFast symplectic correctors and kernels (src/integrator_whfast.c:653-785,
    1113-1259): the scenarios of rebound/tests/test_whfast_advanced.py with the
    reference's own errors and end states, short trajectories for bit-exact replay,
    and the reference's IAS15 positions for the comparison of its compias test."""
    out = {}

    def rel(a, b):
        return abs((a - b) / b)

    settings = [(0, 0, "default"), (3, 0, "default"), (5, 0, "default"), (7, 0, "default"),
                (11, 0, "default"), (17, 0, "default"), (0, 0, "modifiedkick"), (3, 0, "modifiedkick"),
                (5, 0, "modifiedkick"), (7, 0, "modifiedkick"), (11, 0, "modifiedkick"),
                (17, 0, "modifiedkick"), (17, 0, "composition"), (17, 0, "lazy"), (11, 1, "modifiedkick"),
                (3, 0, "composition"), (3, 0, "lazy"), (3, 1, "lazy")]
    sim = rebound.Simulation()
    sim.add("outer solar system")
    out["oss"] = state(sim)
    out["dt"] = 0.0123235235 * sim.particles[1].P
    out["settings"] = np.array([(c, c2, ["default", "modifiedkick", "composition", "lazy"].index(k))
                                for c, c2, k in settings], dtype=np.int32)

    def make(c, c2, k, shift=0.0, safe=None):
        sim = rebound.Simulation()
        load(sim, out["oss"])
        for p in sim.particles:
            p.vx += shift
        sim.integrator = "whfast"
        sim.integrator.corrector = c
        sim.integrator.corrector2 = c2
        sim.integrator.kernel = k
        if safe is not None:
            sim.integrator.safe_mode = safe
        sim.dt = float(out["dt"])
        return sim

    for c, c2, k in settings:
        tag = "c%d_c2%d_%s" % (c, c2, k)
        sim = make(c, c2, k, safe=False)                         # energy (test_whfast_advanced.py:35-48)
        e0 = sim.energy()
        sim.integrate(1000. * 2. * 3.1415)
        out["energy_err_" + tag] = rel(e0, sim.energy())
        out["energy_end_" + tag] = state(sim)
        sim = make(c, c2, k, shift=1.0)                          # energy_notcom (:50-68), safe_mode 1
        e0 = sim.energy()
        sim.integrate(1000. * 2. * 3.1415)
        out["notcom_err_" + tag] = rel(e0, sim.energy())
        out["notcom_end_" + tag] = state(sim)
        sim = make(c, c2, k, shift=1050.)                        # compias (:70-92)
        sim.integrate(13.21415, exact_finish_time=False)
        out["compias_end_" + tag] = state(sim)
        out["compias_t_" + tag] = sim.t
        sim = make(c, c2, k, shift=1.0)                          # backandforth (:94-111)
        sim.steps(10)
        sim.dt *= -1
        sim.steps(10)
        out["bf_end_" + tag] = state(sim)
        sim = make(c, c2, k, safe=False)                         # 20 steps, synchronize (bit-exact replay)
        sim.steps(20)
        sim.synchronize()
        out["traj_" + tag] = state(sim)
    # the IAS15 reference solution of the compias test at the WHFast runs' end time
    t_end = float(out["compias_t_c3_c20_default"])
    simi = rebound.Simulation()
    simi.integrator = "ias15"
    load(simi, out["oss"])
    for p in simi.particles:
        p.vx += 1050.
    simi.integrate(t_end, exact_finish_time=True)
    out["compias_ias15"] = state(simi)
    out["compias_ias15_t"] = simi.t
    # keep_unsynchronized: steps, synchronize without leaving the drift, more steps
    for c in (0, 5):
        sim = make(c, 0, "default", safe=False)
        sim.integrator.keep_unsynchronized = 1
        sim.steps(10)
        sim.synchronize()
        out["keep_mid_c%d" % c] = state(sim)
        sim.steps(10)
        sim.synchronize()
        out["keep_end_c%d" % c] = state(sim)
    np.savez_compressed(os.path.join(HERE, "whfast_advanced.npz"), **out)


def fixture_whfast_coords():
    """WHFast in WHDS and barycentric coordinates and the test-particle scenarios of
    rebound/tests/test_whfast_testparticles.py in all four coordinate systems: the
    inputs the reference builds from orbital elements and the reference's own end
    states."""
    import math
    out = {}
    coords = ("jacobi", "democraticheliocentric", "whds", "barycentric")

    def run(arr, coordinates, dt, safe=1, N_active=-1, tp_type=0, corrector=0):
        sim = rebound.Simulation()
        sim.testparticle_type = tp_type
        load(sim, arr)
        if N_active > 0:
            sim.N_active = N_active
        sim.integrator = "whfast"
        sim.integrator.coordinates = coordinates
        sim.integrator.safe_mode = safe
        sim.integrator.corrector = corrector
        sim.dt = dt
        return sim

    # WHDS outer solar system (rebound/tests/test_whfast.py:9-19)
    sim = rebound.Simulation()
    sim.add("outer solar system")
    out["oss"] = state(sim)
    sim = run(out["oss"], "whds", 0.005 * 12. * 2. * 3.1415)
    e0 = sim.energy()
    sim.integrate(1000. * 2. * 3.1415)
    out["whds_oss_err"] = abs((e0 - sim.energy()) / sim.energy())
    out["whds_oss_end"] = state(sim)
    # two planets, 100 steps in each safe mode
    sim = rebound.Simulation()
    sim.add(m=1.)
    sim.add(m=1e-3, a=1., e=.1)
    sim.add(m=1e-3, a=3., e=0.1)
    out["two"] = state(sim)
    jupyr = 2. * math.pi
    for c in ("whds", "barycentric"):
        for safe in (1, 0):
            sim = run(out["two"], c, 0.005123 * jupyr, safe)
            sim.steps(100)
            sim.synchronize()
            out["two_%s_safe%d" % (c, safe)] = state(sim)
    for order, safe, n in ((5, 0, 50), (17, 1, 10)):
        sim = run(out["two"], "barycentric", 0.005123 * jupyr, safe, corrector=order)
        sim.steps(n)
        sim.synchronize()
        out["two_barycentric_c%d" % order] = state(sim)
    # test particles (rebound/tests/test_whfast_testparticles.py)
    for N in (1, 2):
        sim = rebound.Simulation()
        sim.add(m=1)
        for i in range(N):
            sim.add(m=0, P=1, e=0.1, f=i)
        out["tp_N%d" % N] = state(sim)
        sim = rebound.Simulation()
        sim.add(m=1)
        sim.add(m=1e-3, P=0.4)
        sim.add(m=1e-3, P=0.7)
        for i in range(N):
            sim.add(m=0, P=1, e=0.1, f=i)
        out["tpp_N%d" % N] = state(sim)
        sim = rebound.Simulation()
        sim.add(m=1)
        sim.add(m=1e-3, P=0.4)
        for i in range(N):
            sim.add(m=0, P=1, e=0.1, f=i)
        out["mtp_N%d" % N] = state(sim)
        for c in coords:
            for na in [-1] + list(range(1, N + 2)):
                sim = run(out["tp_N%d" % N], c, 1e-1, N_active=na)
                sim.integrate(1)
                out["tp_N%d_%s_na%d" % (N, c, na)] = state(sim)
            for na in [-1] + list(range(3, N + 4)):
                sim = run(out["tpp_N%d" % N], c, 1e-3, N_active=na)
                sim.integrate(1)
                out["tpp_N%d_%s_na%d" % (N, c, na)] = state(sim)
            sim = run(out["mtp_N%d" % N], c, 1e-3)
            sim.integrate(1)
            out["mtp_N%d_%s_massless" % (N, c)] = state(sim)
            heavy = out["mtp_N%d" % N].copy()
            heavy["m"][2:] = 1.
            sim = run(heavy, c, 1e-3, N_active=2)
            sim.integrate(1)
            out["mtp_N%d_%s_massive" % (N, c)] = state(sim)
    sim = rebound.Simulation()
    sim.add(m=1)
    sim.add(m=1e-3, P=1, e=0.1)
    out["tp1"] = state(sim)
    sim = rebound.Simulation()
    sim.add(m=1)
    sim.add(m=1e-3, P=0.4)
    sim.add(m=1e-3, P=0.7, e=0.1)
    sim.add(m=1e-3, P=1.0)
    out["tp1p"] = state(sim)
    for c in coords:
        for na in (-1, 1):
            sim = run(out["tp1"], c, 1e-3, N_active=na, tp_type=1)
            sim.integrate(1)
            out["tp1_%s_na%d" % (c, na)] = state(sim)
        for na in (-1, 3):
            sim = run(out["tp1p"], c, 1e-3, N_active=na, tp_type=1)
            sim.integrate(1)
            out["tp1p_%s_na%d" % (c, na)] = state(sim)
    np.savez_compressed(os.path.join(HERE, "whfast_coords.npz"), **out)


def fixture_archive_cases():
    """Restart scenarios of rebound/tests/test_simulationarchive.py:86-365: the
    three-body input the reference builds from orbital elements and the reference's
    own state at t = 80 (exact_finish_time = 0) for each integrator setting."""
    out = {}
    sim = rebound.Simulation()
    sim.add(m=1)
    sim.add(m=1e-3, a=1, e=0.1, omega=0.1, M=0.1, inc=0.1, Omega=0.1)
    sim.add(m=1e-3, a=-2, e=1.1, omega=0.1, M=0.1, inc=0.1, Omega=0.1)
    out["start"] = state(sim)
    for coords in ("jacobi", "democraticheliocentric", "whds"):
        for safe in (0, 1):
            for corrector in ((0, 5) if coords == "jacobi" else (0,)):
                sim = rebound.Simulation()
                load(sim, out["start"])
                sim.integrator = "whfast"
                sim.integrator.coordinates = coords
                sim.integrator.corrector = corrector
                sim.dt = 0.1313
                sim.integrator.safe_mode = safe
                sim.integrate(80., exact_finish_time=0)
                out["end_%s_safe%d_c%d" % (coords, safe, corrector)] = state(sim)
                out["t_%s_safe%d_c%d" % (coords, safe, corrector)] = sim.t
    np.savez_compressed(os.path.join(HERE, "archive_cases.npz"), **out)


def fixture_collision_line():
    """LINE and LINETREE collision searches (src/collision.c:125-196, 270-330,
    506-572) after one step, so that dt_last_done is set: the shearing-sheet patch
    after one SEI + tree-gravity step, and a periodic box of fast particles after one
    leapfrog drift; the reference's pair lists after its rand_r shuffle (src/collision.c:
    336-342), with the shuffle seed each search started from."""
    out = {}
    sim = ring_patch(200.0, seed=7)
    out["ring_start"] = state(sim)
    sim.collision = "none"
    sim.steps(1)
    out["ring_after1"] = state(sim)
    for mode in ("line", "linetree"):
        out["ring_seed_" + mode] = np.int64(sim.rand_seed)        # the search ends with the rand_r shuffle
        out["ring_pairs_" + mode] = collision_pairs(sim, mode)
    sim = rebound.Simulation()
    sim.rand_seed = 11
    sim.integrator = "leapfrog"
    sim.gravity = "none"
    sim.boundary = "periodic"
    sim.root_size = 10.
    sim.N_ghost_x = sim.N_ghost_y = sim.N_ghost_z = 1
    sim.dt = 0.3
    sp = ctypes.byref(sim)
    for _ in range(500):
        u = lambda a, b: clibrebound.reb_random_uniform(sp, ctypes.c_double(a), ctypes.c_double(b))
        nrm = lambda: clibrebound.reb_random_normal(sp, ctypes.c_double(1.0))
        sim.add(m=0.0, r=u(0.2, 0.4), x=u(-5., 5.), y=u(-5., 5.), z=u(-5., 5.), vx=nrm(), vy=nrm(), vz=nrm())
    out["box_start"] = state(sim)
    sim.steps(1)
    out["box_after1"] = state(sim)
    for mode in ("line", "linetree", "direct"):
        out["box_seed_" + mode] = np.int64(sim.rand_seed)
        out["box_pairs_" + mode] = collision_pairs(sim, mode)
    np.savez_compressed(os.path.join(HERE, "collision_line.npz"), **out)


def fixture_tree_quadrupole():
    """Tree gravity with quadrupole moments (src/tree.c:147-207, 273-320 with
    QUADRUPOLE defined; src/Makefile.defs:90-91): the reference built with
    -DQUADRUPOLE (oracle/_ref/librebound_quad.so, from oracle/ref.mk) evaluates the
    shearing-sheet patch; its accelerations next to the monopole build's."""
    qlib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "librebound_quad.so"))
    qlib.reb_simulation_create.restype = ctypes.c_void_p
    qlib.reb_simulation_add.argtypes = [ctypes.c_void_p, rebound.Particle]
    qlib.reb_simulation_update_acceleration.argtypes = [ctypes.c_void_p]
    out = {}
    for L, theta2 in ((200.0, 0.25), (200.0, 0.5)):
        src = ring_patch(L, seed=7)
        src.opening_angle2 = theta2
        qptr = qlib.reb_simulation_create()
        Q = ctypes.cast(qptr, ctypes.POINTER(rebound.Simulation)).contents
        for f in ("G", "softening", "dt", "OMEGA", "root_size", "N_root_x", "N_root_y", "N_root_z",
                  "N_ghost_x", "N_ghost_y", "N_ghost_z", "opening_angle2"):
            setattr(Q, f, getattr(src, f))
        Q.gravity = "tree"
        Q.boundary = "shear"
        for i in range(src.N):
            qlib.reb_simulation_add(qptr, src.particles[i])
        qlib.reb_simulation_update_acceleration(qptr)
        tag = "t%g" % theta2
        out["particles"] = state(src)
        out["acc_quad_" + tag] = np.stack([state(Q)[k] for k in ("ax", "ay", "az")], axis=1)
        out["acc_mono_" + tag] = accel(src)
    np.savez_compressed(os.path.join(HERE, "tree_quadrupole.npz"), **out)


def fixture_whfast_gravity():
    """WHFast with the simulation's gravity set to COMPENSATED or NONE (the
    reference's WHFast evaluates r->gravity): the scenarios of
    rebound/tests/test_gravity.py:55-94 with the reference's own end states and its
    IAS15 value, and 100-step outer-solar-system runs per coordinate system."""
    out = {}
    sim = rebound.Simulation()
    sim.gravity = "compensated"
    sim.integrator = "whfast"
    sim.testparticle_type = 0
    sim.add(m=1.)
    sim.add(m=1e-3, a=1.)
    out["comp0_start"] = state(sim)
    out["comp0_dt"] = sim.dt
    sim.N_active = 1
    sim.integrate(10.)
    out["comp0_end"] = state(sim)
    for integ in ("whfast", "ias15"):
        sim = rebound.Simulation()
        sim.gravity = "compensated"
        sim.integrator = integ
        if integ == "whfast":
            sim.dt = 1e-4
        sim.testparticle_type = 1
        sim.add(m=1.)
        sim.add(m=1e-3, a=1.)
        sim.add(m=1e-3, a=1.4)
        out["comp1_start"] = state(sim)
        sim.N_active = 2
        sim.integrate(10.)
        out["comp1_end_" + integ] = state(sim)
    sim = rebound.Simulation()
    sim.add("outer solar system")
    out["oss"] = state(sim)
    for gravity in ("compensated", "none"):
        for coords in ("jacobi", "democraticheliocentric", "whds", "barycentric"):
            sim = rebound.Simulation()
            load(sim, out["oss"])
            sim.gravity = gravity
            sim.integrator = "whfast"
            sim.integrator.coordinates = coords
            sim.integrator.safe_mode = 0
            sim.dt = 0.5
            sim.steps(100)
            sim.synchronize()
            out["oss_%s_%s" % (gravity, coords)] = state(sim)
    np.savez_compressed(os.path.join(HERE, "whfast_gravity.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[2:] or ["gravity_cases", "ring", "whfast", "sei", "gravity_plummer", "reference_cases",
                             "leapfrog_orders", "whfast_dh", "whfast_advanced", "whfast_coords",
                             "archive_cases", "collision_line", "tree_quadrupole",
                             "whfast_gravity", "gravity_hierarchical"]
    for w in which:
        print("generating", w, flush=True)
        globals()["fixture_" + w]() if w != "sei" else fixture_sei_periodic()
