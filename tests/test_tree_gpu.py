"""Octree gravity, tree/direct collision search, SEI and the shear boundary on
the GPU against the reference's golden vectors and the oracle.

Bars: octree cell membership, cell centres and centres of mass bit-exact; tree
accelerations bit-exact (the walk keeps the reference's order); collision pair
sets bit-exact and in the reference's discovery order; SEI + shear trajectories
tracked to round-off; error conditions raise like the reference.
"""
import numpy as np
import pytest

from conftest import golden, rel_err_vec
from oracle import oracle as O

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")


def ring_gpu(R, g, particles=None):
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]
    sim = R.Simulation()
    sim.G, sim.OMEGA, sim.softening, sim.dt, sim.t = G, OM, soft, dt, t
    sim.configure_box(rs, int(nx), int(ny), int(nz))
    sim.configure_ghostboxes(int(gx), int(gy), int(gz))
    sim.opening_angle2 = oa2
    sim.boundary = "shear"
    sim.gravity = "tree"
    sim.integrator = "sei"
    sim.add(g["particles"] if particles is None else particles)
    return sim


def ring_oracle(g, particles=None):
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, oa2, t = g["meta"]
    return O.Sim(g["particles"] if particles is None else particles, G=G, softening=soft, dt=dt, boundary="shear",
                 root_size=rs, N_root=(int(nx), int(ny), int(nz)), N_ghost=(int(gx), int(gy), int(gz)), OMEGA=OM,
                 opening_angle2=oa2, t=t)


def test_tree_cells_bit_exact(gpu):
    g = golden("ring_patch.npz")
    cells = ring_gpu(gpu, g).tree_cells()
    ref = g["cells"]
    assert len(cells) == len(ref)
    for f in ref.dtype.names:
        assert np.array_equal(cells[f], ref[f]), f


def test_tree_gravity_bit_exact(gpu):
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.update_acceleration()
    assert np.array_equal(gpu.accelerations(sim), g["acc_tree"])


def test_tree_error_statistics_match_reference(gpu):
    # |a_tree - a_direct| / |a_direct| at opening angle 0.5: same distribution.
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.update_acceleration()
    a_tree = gpu.accelerations(sim)
    sim2 = ring_gpu(gpu, g)
    sim2.gravity = "basic"
    sim2.update_acceleration()
    a_dir = gpu.accelerations(sim2)
    e_gpu = rel_err_vec(a_tree, a_dir)
    e_ref = rel_err_vec(g["acc_tree"], g["acc_basic"])
    for q in (0.5, 0.99, 1.0):
        assert abs(np.quantile(e_gpu, q) - np.quantile(e_ref, q)) <= 1e-9 * max(1e-12, np.quantile(e_ref, q))


@pytest.mark.parametrize("mode", ["direct", "tree"])
def test_collision_pairs_bit_exact_and_ordered(gpu, mode):
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.collision = mode
    pairs = sim.collision_search()
    ref = g["pairs_" + mode]
    key = lambda p: sorted(zip(p["p1"].tolist(), p["p2"].tolist(), map(tuple, p["gb"].tolist())))
    assert len(pairs) == len(ref) > 0
    assert key(pairs) == key(ref)
    # discovery order equals the reference's serial order (oracle restatement)
    orc = ring_oracle(g).collisions(mode)
    assert np.array_equal(pairs["p1"], orc["p1"]) and np.array_equal(pairs["p2"], orc["p2"])
    assert np.array_equal(pairs["gb"], orc["gb"])


def test_sei_tree_collisions_hardsphere_trajectory(gpu):
    # 5 full steps: SEI, tree gravity, shear boundary, tree collision search,
    # rand_r shuffle and hardsphere (epsilon 0.5), against the reference.
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.collision = "tree"
    sim.collision_resolve = "hardsphere"
    sim.coefficient_of_restitution = 0.5
    sim.rand_seed = int(g["after5_seed0"])
    sim.steps(5)
    p, ref = sim.particles, g["after5"]
    assert sim.t == g["after5_t"]
    assert sim.collisions_log_n == g["after5_collisions_log_n"]
    assert sim.rand_seed == g["after5_seed"]
    # y-momentum transferred by the collisions (src/collision.c:655-662)
    assert abs(sim.collisions_plog - g["after5_collisions_plog"]) <= 1e-10 * abs(g["after5_collisions_plog"])
    for f in XV:
        scale = np.abs(ref[f]).max()
        assert np.abs(p[f] - ref[f]).max() <= 1e-12 * scale, f


def test_velocity_dependent_restitution(gpu):
    # The reference's shearing-sheet restitution law (rebound/tests/test_shearingsheet.py:26-32),
    # called on the host for each collision as REBOUND calls r->coefficient_of_restitution.
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.collision = "tree"
    sim.collision_resolve = "hardsphere"
    calls = []

    def cor_bridges(r, v):
        calls.append(v)
        eps = 0.32 * pow(abs(v) * 100., -0.234)
        return min(1., max(0., eps))
    sim.coefficient_of_restitution = cor_bridges
    sim.rand_seed = int(g["after5_seed0"])
    sim.steps(5)
    p, ref = sim.particles, g["bridges_after5"]
    assert sim.collisions_log_n == g["bridges_after5_collisions_log_n"] == len(calls)
    assert sim.rand_seed == g["bridges_after5_seed"]
    assert abs(sim.collisions_plog - g["bridges_after5_collisions_plog"]) <= 1e-10 * abs(g["bridges_after5_collisions_plog"])
    for f in XV:
        scale = np.abs(ref[f]).max()
        assert np.abs(p[f] - ref[f]).max() <= 1e-12 * scale, f
    ms, n = sim.resolve_time()
    assert 1 <= n <= 5 and ms > 0


def test_sei_basic_shear_trajectory(gpu):
    g = golden("sei_shear.npz")
    G, OM, soft, dt, rs, nx, ny, nz, gx, gy, gz, t = g["meta"]
    sim = gpu.Simulation()
    sim.G, sim.OMEGA, sim.softening, sim.dt, sim.t = G, OM, soft, dt, t
    sim.configure_box(rs, int(nx), int(ny), int(nz))
    sim.configure_ghostboxes(int(gx), int(gy), int(gz))
    sim.boundary = "shear"
    sim.gravity = "basic"
    sim.integrator = "sei"
    sim.add(g["particles"])
    sim.steps(20)
    p, ref = sim.particles, g["after20"]
    for f in XV:
        scale = np.abs(ref[f]).max()
        assert np.abs(p[f] - ref[f]).max() <= 1e-11 * scale, f


def test_tree_rejects_duplicate_positions(gpu):
    # rebound/tests/test_gravity.py:96-104: two particles at the same position.
    sim = gpu.Simulation()
    sim.configure_box(10.0)
    sim.gravity = "tree"
    sim.add(m=1.0, x=1.0, y=1.0)
    sim.add(m=1.0, x=1.0, y=1.0)
    sim.add(m=1.0, x=-1.0, y=1.0)
    with pytest.raises(gpu.RGPUError) as e:
        sim.update_acceleration()
    assert e.value.code == 7


@pytest.mark.parametrize("bad,code", [((1e6, 0.0, 0.0), 6), ((np.nan, 0.0, 0.0), 6)])
def test_tree_rejects_bad_particles(gpu, bad, code):
    sim = gpu.Simulation()
    sim.configure_box(10.0)
    sim.gravity = "tree"
    sim.add(m=1.0, x=0.5)
    sim.add(m=1.0, x=bad[0], y=bad[1], z=bad[2])
    with pytest.raises(gpu.RGPUError) as e:
        sim.update_acceleration()
    # NaN fails the in-box comparison first in the reference's order as well
    assert e.value.code in (5, 6)


def test_full_size_ring_patch(gpu):
    # Configuration-3 size (2,300 m box, 115 x 115 roots, N ~ 197k): cell
    # membership against the oracle's insertion tree, tree accelerations of a
    # sample of particles bit-exact, and the tree pair set equal to an exact
    # neighbour search.
    R = gpu
    p = R.ics.ring_patch(2300.0, seed=7)
    meta = dict(G=6.674e-11, OMEGA=1.3143527e-4, softening=0.1)
    sim = R.Simulation()
    sim.G, sim.OMEGA, sim.softening = meta["G"], meta["OMEGA"], meta["softening"]
    sim.configure_box(20.0, 115, 115, 1)
    sim.configure_ghostboxes(2, 2, 0)
    sim.boundary = "shear"
    sim.gravity = "tree"
    sim.collision = "tree"
    sim.add(p)
    cells = sim.tree_cells()
    orc = O.Sim(p, G=meta["G"], softening=0.1, boundary="shear", root_size=20.0, N_root=(115, 115, 1),
                N_ghost=(2, 2, 0), OMEGA=meta["OMEGA"])
    ref = orc.tree_cells()
    assert len(cells) == len(ref)
    for f in ("root", "depth", "path", "pt", "x", "y", "z", "w", "m", "mx", "my", "mz"):
        assert np.array_equal(cells[f], ref[f]), f
    sim.update_acceleration()
    a = R.accelerations(sim)
    rows = np.arange(0, len(p), len(p) // 24)[:24]
    for i in rows:
        O.lib().orc_gravity_tree_rows(orc.ref, int(i), int(i) + 1)
    assert np.array_equal(a[rows], orc.acc()[rows])
    pairs = sim.collision_search()
    assert len(pairs) > 0
    # exact neighbour search: candidate pairs from a KD-tree, then the reference's test
    scipy = pytest.importorskip("scipy.spatial")
    q = sim.particles
    pos = np.stack([q["x"], q["y"], q["z"]], 1)
    kd = scipy.cKDTree(pos)
    cand = kd.query_pairs(2 * q["r"].max() + 1e-6, output_type="ndarray")
    cand = np.concatenate([cand, cand[:, ::-1]])
    i, j = cand[:, 0], cand[:, 1]
    dx, dy, dz = q["x"][i] - q["x"][j], q["y"][i] - q["y"][j], q["z"][i] - q["z"][j]
    sr = q["r"][i] + q["r"][j]
    ok = (dx * dx + dy * dy + dz * dz) <= sr * sr
    dv = (q["vx"][i] - q["vx"][j]) * dx + (q["vy"][i] - q["vy"][j]) * dy + (q["vz"][i] - q["vz"][j]) * dz
    ok &= ~(dv > 0)
    inner = pairs[np.all(pairs["gb"] == 0, axis=1)]
    got = set(zip(inner["p1"].tolist(), inner["p2"].tolist()))
    exp = set(zip(i[ok].tolist(), j[ok].tolist()))
    assert got == exp
    # the whole list, ghost-box pairs included, entry for entry in the reference's
    # serial discovery order (the oracle's search, its particle loop split over
    # OpenMP threads and joined in order)
    ref_pairs = orc.collisions("tree_omp")
    assert len(pairs) == len(ref_pairs)
    assert np.any(np.any(ref_pairs["gb"] != 0, axis=1))
    for f in ("p1", "p2", "gb"):
        assert np.array_equal(pairs[f], ref_pairs[f]), f


def test_tree_split_mode_matches_exact_walk(gpu):
    # 800 m patch (40 x 40 roots, ~25k particles, 25 ghost boxes): the split
    # mode walks the roots within ceil(1/theta)+1 root widths exactly and sums
    # all others as monopoles in mixed precision.  Against the exact walk the
    # per-particle difference stays at FP32 round-off of the far field, orders
    # of magnitude below the tree's own error, whose distribution is unchanged.
    R = gpu
    p = R.ics.ring_patch(800.0, seed=11)

    def accel(mode):
        sim = R.Simulation()
        sim.G, sim.OMEGA, sim.softening = 6.674e-11, 1.3143527e-4, 0.1
        sim.configure_box(20.0, 40, 40, 1)
        sim.configure_ghostboxes(2, 2, 0)
        sim.boundary = "shear"
        sim.gravity = mode
        sim.add(p)
        sim.update_acceleration()
        return R.accelerations(sim)

    a_exact, a_split, a_direct = accel("tree"), accel("tree_split"), accel("basic")
    d = rel_err_vec(a_split, a_exact)
    assert np.median(d) <= 1e-7 and d.max() <= 1e-4, (np.median(d), d.max())
    e_exact, e_split = rel_err_vec(a_exact, a_direct), rel_err_vec(a_split, a_direct)
    for q in (0.5, 0.9, 0.99):
        qe, qs = np.quantile(e_exact, q), np.quantile(e_split, q)
        assert abs(qs - qe) <= 1e-2 * qe, (q, qe, qs)


@pytest.mark.parametrize("theta2", [0.3, 0.7, 0.125])
def test_tree_gravity_bit_exact_any_opening_angle(gpu, theta2):
    # opening_angle2 = 2^k turns the walk's opening test into an integer
    # comparison; any other value takes the FP64 comparison.  Both must give the
    # oracle's tree accelerations bit for bit (0.125 = 2^-3 is the integer path).
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g)
    sim.opening_angle2 = theta2
    sim.update_acceleration()
    orc = ring_oracle(g)
    orc.s.opening_angle2 = theta2
    assert np.array_equal(gpu.accelerations(sim), orc.gravity("tree"))


@pytest.mark.parametrize("theta2", [0.25, 0.5])
def test_tree_quadrupole_bit_exact(gpu, theta2):
    # mass quadrupoles in the cells and the quadrupole far-cell term, against the
    # reference built with -DQUADRUPOLE (tests/golden/tree_quadrupole.npz)
    gq = golden("tree_quadrupole.npz")
    g = golden("ring_patch.npz")
    sim = ring_gpu(gpu, g, gq["particles"])
    sim.opening_angle2 = theta2
    sim.tree_quadrupole = 1
    sim.update_acceleration()
    assert np.array_equal(gpu.accelerations(sim), gq["acc_quad_t%g" % theta2])
    sim.tree_quadrupole = 0
    sim.update_acceleration()
    assert np.array_equal(gpu.accelerations(sim), gq["acc_mono_t%g" % theta2])
    sim.tree_quadrupole = 1
    sim.gravity = "tree_split"
    with pytest.raises(gpu.RGPUError, match="monopoles"):
        sim.update_acceleration()
