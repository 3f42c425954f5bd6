"""Direct-sum gravity on the GPU against the oracle and the reference's golden vectors.

Tolerances (per-particle vector-norm relative error |a_gpu - a_ref| / |a_ref|):
  FP64 BASIC and COMPENSATED: <= 1e-14 against the reference's own result.
  MIXED / MIXED_SPLIT: median <= 1e-6 against FP64, max <= 1e-3.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden, rel_err_vec
from oracle import oracle as O

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-14


def gpu_accel(R, particles, gravity, **cfg):
    sim = R.Simulation()
    sim.gravity = gravity
    for k, v in cfg.items():
        setattr(sim, k, v)
    sim.add(particles)
    sim.update_acceleration()
    return R.accelerations(sim)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_basic_plummer_4096_matches_reference(gpu, variant):
    # m/r^3 variants with the FP64-subtraction displacement
    L = gpu.load()
    assert L.rgpu_set_kernel_variant(variant, 1) == 0
    assert L.rgpu_set_displacement_mode(0) == 0
    try:
        g = golden("gravity_plummer.npz")
        a = gpu_accel(gpu, g["particles"], "basic", softening=0.01)
        err = rel_err_vec(a, g["acc_basic"])
        assert err.max() <= FP64_TOL, err.max()
        # and against the compensated (most accurate) reference sum
        assert rel_err_vec(a, g["acc_compensated"]).max() <= FP64_TOL
    finally:
        L.rgpu_set_kernel_variant(3, 0)
        L.rgpu_set_displacement_mode(2)


@pytest.mark.parametrize("disp", [1, 2])
@pytest.mark.parametrize("gravity", ["basic", "compensated"])
def test_fixed_point_forms_match_reference(gpu, gravity, disp):
    # 1: int64 fixed-point positions, displacement converted on the integer pipe;
    # 2 (default): also r^2 and (r^2+eps^2)^(-3/2) on the integer pipes
    L = gpu.load()
    assert L.rgpu_set_displacement_mode(disp) == 0
    try:
        g = golden("gravity_plummer.npz")
        a = gpu_accel(gpu, g["particles"], gravity, softening=0.01)
        assert rel_err_vec(a, g["acc_" + gravity]).max() <= FP64_TOL
        assert rel_err_vec(a, g["acc_compensated"]).max() <= FP64_TOL
    finally:
        L.rgpu_set_displacement_mode(2)


def _two_modes(gpu, parts, gravity, mode_a, mode_b, **cfg):
    L = gpu.load()
    out = []
    try:
        for m in (mode_a, mode_b):
            assert L.rgpu_set_displacement_mode(m) == 0
            out.append(gpu_accel(gpu, parts, gravity, **cfg))
    finally:
        L.rgpu_set_displacement_mode(2)
    return out


def _shell_box(n, offset, seed):
    # coordinates in +-[4, 8] (scaled and shifted for an offset cluster)
    rng = np.random.default_rng(seed)
    parts = np.zeros(n, dtype=O.PARTICLE_DTYPE)
    mag = 4.0 + 4.0 * rng.random((n, 3))
    pos = np.where(rng.random((n, 3)) < 0.5, -mag, mag)
    if offset:
        pos = offset + pos * (abs(offset) * 1e-3 if abs(offset) > 1 else 1.0)
    parts["x"], parts["y"], parts["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    parts["m"] = rng.random(n) / n
    return parts


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
@pytest.mark.parametrize("offset", [0.0, 1e6, -3.5e-3])
def test_fixed_point_displacement_is_the_fp64_subtraction(gpu, gravity, offset):
    # Every coordinate within a factor 2^8 of the largest is exact in the fixed-point
    # form, so the integer-pipe displacement equals the FP64 subtraction bit for bit
    # and the whole sum is bit-identical.
    parts = _shell_box(3000, offset, 11)
    a_fix, a_sub = _two_modes(gpu, parts, gravity, 1, 0, softening=0.0)
    assert np.array_equal(a_fix, a_sub)


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
@pytest.mark.parametrize("offset,soft", [(0.0, 0.0), (0.0, 0.3), (1e6, 0.0), (-3.5e-3, 1e-4), (0.0, 40.0)])
def test_integer_pair_factor_matches_fp64(gpu, gravity, offset, soft):
    # (r^2 + eps^2)^(-3/2) on the integer pipes against the FP64 form, including a
    # softening larger than the whole box (the fixed-point scale then follows eps).
    # Error measured against each particle's force scale sum_j m_j / (r^2+eps^2)
    # (the net force of a box interior nearly cancels): each pair factor is good to
    # about one ulp, so the difference stays within a few ulps of that scale.
    parts = _shell_box(3000, offset, 13)
    a_int, a_fp = _two_modes(gpu, parts, gravity, 2, 0, softening=soft)
    pos = np.stack([parts["x"], parts["y"], parts["z"]], axis=1)
    d = pos[None, :, :] - pos[:, None, :]
    r2 = (d * d).sum(axis=2) + soft * soft
    np.fill_diagonal(r2, np.inf)
    scale = (parts["m"][None, :] / r2).sum(axis=1)
    err = np.linalg.norm(a_int - a_fp, axis=1) / scale
    assert err.max() <= 4e-15, err.max()
    # and per particle against its own force |a| (where the box interior cancels)
    assert rel_err_vec(a_int, a_fp).max() <= FP64_TOL, rel_err_vec(a_int, a_fp).max()


@pytest.mark.parametrize("soft", [0.01, 0.0])
@pytest.mark.parametrize("offset", [0.0, 1e6])
def test_mixed_forms_far_from_origin(gpu, offset, soft):
    # The two-float split keeps the displacement exact to ~2^-48 of the coordinates,
    # also for a box shifted by 1e6 (the high halves cancel exactly); with zero
    # softening the kernel skips the self pair explicitly.  Both mixed forms against
    # FP64 at the mixed-precision budget, and against each other (they differ only
    # in the accumulation: FP64 for MIXED, a compensated FP32 pair for MIXED_SPLIT).
    parts = _shell_box(3001, offset, 17)
    a64 = gpu_accel(gpu, parts, "basic", softening=soft)
    a_m = gpu_accel(gpu, parts, "mixed", softening=soft)
    a_s = gpu_accel(gpu, parts, "mixed_split", softening=soft)
    for a in (a_m, a_s):
        assert np.all(np.isfinite(a))
        err = rel_err_vec(a, a64)
        assert np.median(err) <= 1e-6 and err.max() <= 1e-3, (np.median(err), err.max())
    assert np.median(rel_err_vec(a_m, a_s)) <= 1e-7


def _guarded(gpu, parts, gravity, disp=2, **cfg):
    """Accelerations through displacement mode `disp` and the guard's counters."""
    L = gpu.load()
    assert L.rgpu_set_displacement_mode(disp) == 0
    try:
        sim = gpu.Simulation()
        sim.gravity = gravity
        for k, v in cfg.items():
            setattr(sim, k, v)
        sim.add(parts)
        sim.update_acceleration()
        return gpu.accelerations(sim), sim.guard_stats()
    finally:
        L.rgpu_set_displacement_mode(2)


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
def test_fixed_point_displacement_small_coordinates(gpu, gravity):
    # Coordinates far below the largest are off the fixed-point grid: a cluster at the
    # origin next to one distant body.  The exactness guard sends every particle to
    # the FP64 kernel, so the default mode and mode 1 meet the FP64 bar.
    rng = np.random.default_rng(12)
    n = 2048
    parts = np.zeros(n, dtype=O.PARTICLE_DTYPE)
    parts["x"], parts["y"], parts["z"] = (rng.standard_normal((3, n)) * 1e-2)
    parts["x"][0] = 1e3
    parts["m"] = 1.0 / n
    ref = O.Sim(parts, softening=0.0).gravity("compensated")
    a_sub = _two_modes(gpu, parts, gravity, 0, 0, softening=0.0)[0]
    for disp in (2, 1):
        a_fix, (n_inexact, n_redo) = _guarded(gpu, parts, gravity, disp, softening=0.0)
        assert n_inexact > n // 4 and n_redo == n, (disp, n_inexact, n_redo)
        assert rel_err_vec(a_fix, ref).max() <= FP64_TOL, (disp, rel_err_vec(a_fix, ref).max())
        assert rel_err_vec(a_fix, a_sub).max() <= FP64_TOL


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
@pytest.mark.parametrize("case", ["binary_wide", "cluster_far", "plummer_binary"])
def test_hierarchical_systems_match_reference(gpu, gravity, case):
    # The reference's own accelerations of hierarchical inputs (a tight binary in a
    # wide system, a cluster beside a distant body, a Plummer sphere with a tight
    # central binary) through the default fixed-point mode: per particle within 1e-14.
    g = golden("gravity_hierarchical.npz")
    parts = g[case + "_particles"]
    a, (n_inexact, n_redo) = _guarded(gpu, parts, gravity, softening=float(g[case + "_softening"]))
    assert n_inexact > 0 and n_redo > 0, (n_inexact, n_redo)
    if case == "plummer_binary":
        # only some bodies are off the grid: the guard recomputes a subset
        assert n_inexact < len(parts) // 4 and n_redo < len(parts), (n_inexact, n_redo)
    err = rel_err_vec(a, g[f"{case}_acc_{gravity}"])
    assert err.max() <= FP64_TOL, err.max()
    assert rel_err_vec(a, g[f"{case}_acc_compensated"]).max() <= FP64_TOL


def test_guard_recomputes_few_on_plummer(gpu):
    # On a Plummer sphere a few percent of the bodies have coordinates below 2^-8 of
    # the largest, and the bound keeps nearly all of them on the fixed-point path.
    g = golden("gravity_plummer.npz")
    a, (n_inexact, n_redo) = _guarded(gpu, g["particles"], "basic", softening=0.01)
    assert 0 < n_inexact < 4096 // 8 and n_redo < 16, (n_inexact, n_redo)
    assert rel_err_vec(a, g["acc_compensated"]).max() <= FP64_TOL


@pytest.mark.parametrize("gravity", ["basic", "compensated"])
@pytest.mark.parametrize("n_box,n_cluster", [(3000, 500), (12000, 2900)])
def test_guard_recompute_regimes(gpu, gravity, n_box, n_cluster):
    # A box of bodies with coordinates on the grid plus a compact cluster at the
    # origin whose coordinates are not: the guard recomputes the cluster in FP64,
    # one warp per particle for a short list (500) and in 256-particle tiles for a
    # long one (2,900 > 2,048), without sending every particle there.
    rng = np.random.default_rng(n_cluster)
    box = _shell_box(n_box, 0.0, 29)
    cl = np.zeros(n_cluster, dtype=O.PARTICLE_DTYPE)
    cl["x"], cl["y"], cl["z"] = rng.standard_normal((3, n_cluster)) * 1e-3
    cl["m"] = 1.0 / n_box
    parts = np.concatenate([box, cl])
    a, (n_inexact, n_redo) = _guarded(gpu, parts, gravity, softening=0.0)
    assert n_cluster <= n_inexact < len(parts) // 4, n_inexact
    # most of the cluster is recomputed (its bounds exceed 5e-15 |a|), not the box
    assert n_cluster // 2 <= n_redo < n_cluster + n_box // 10, n_redo
    assert (n_redo > 2048) == (n_cluster > 2048), n_redo        # the regime under test
    ref = O.Sim(parts, softening=0.0).gravity("compensated")
    assert rel_err_vec(a, ref).max() <= FP64_TOL, rel_err_vec(a, ref).max()


def test_guard_non_finite_body(gpu):
    # A NaN coordinate: the reference's sums give NaN on every particle it touches;
    # the guard sends those particles to the FP64 kernel, which does the same.
    parts = _shell_box(300, 0.0, 5)
    parts["x"][7] = np.nan
    a, _ = _guarded(gpu, parts, "basic", softening=0.01)
    ref = O.Sim(parts, softening=0.01).gravity("basic")
    assert np.array_equal(np.isnan(a), np.isnan(ref))


def test_compensated_plummer_4096_matches_reference(gpu):
    g = golden("gravity_plummer.npz")
    a = gpu_accel(gpu, g["particles"], "compensated", softening=0.01)
    err = rel_err_vec(a, g["acc_compensated"])
    assert err.max() <= FP64_TOL, err.max()


@pytest.mark.parametrize("mode", ["mixed", "mixed_split"])
def test_mixed_precision_error_budget(gpu, mode):
    g = golden("gravity_plummer.npz")
    a = gpu_accel(gpu, g["particles"], mode, softening=0.01)
    err = rel_err_vec(a, g["acc_compensated"])
    assert np.median(err) <= 1e-6, np.median(err)
    assert err.max() <= 1e-3, err.max()


@pytest.mark.parametrize("case", ["plain", "testp0", "testp1", "ignore01", "ignore0", "ghost", "single", "two"])
def test_gravity_edge_cases(gpu, case):
    g = golden("gravity_cases.npz")
    n, na, tp, ign, ghost, soft = g[case + "_meta"]
    for mode in ("basic", "compensated"):
        key = f"{case}_acc_{mode}"
        if key not in g:
            continue
        sim = gpu.Simulation()
        sim.gravity = mode
        sim.softening = soft / 1e6
        if ghost:
            sim.boundary = "periodic"
            sim.configure_box(2.0)
            sim.configure_ghostboxes(1, 1, 1)
        sim.add(g[case + "_particles"])
        sim.N_active = None if na < 0 else int(na)
        sim.testparticle_type = int(tp)
        sim.gravity_ignore_terms = int(ign)
        sim.update_acceleration()
        a = gpu.accelerations(sim)
        ref = g[key]
        if n == 1:
            assert np.all(a == 0)
            continue
        err = rel_err_vec(a, ref)
        assert err.max() <= FP64_TOL, (case, mode, err.max())


def test_empty_simulation(gpu):
    sim = gpu.Simulation()
    sim.update_acceleration()
    sim.steps(3)
    assert sim.N == 0
    assert sim.energy() == 0.0


def test_ragged_sizes_against_oracle(gpu):
    # sizes that are not multiples of the 256-body tile, including j-splits
    rng = np.random.default_rng(3)
    for n in (3, 255, 257, 1000, 5000):
        p = np.zeros(n, dtype=O.PARTICLE_DTYPE)
        for f in ("x", "y", "z"):
            p[f] = rng.normal(size=n)
        p["m"] = rng.uniform(0.5, 1.5, n) / n
        ref = O.Sim(p, softening=0.02).gravity("compensated")
        for mode in ("basic", "compensated"):
            a = gpu_accel(gpu, p, mode, softening=0.02)
            assert rel_err_vec(a, ref).max() <= FP64_TOL, (n, mode)


def test_full_size_262144_properties(gpu):
    # Configuration-2 size: BASIC vs COMPENSATED agree to 1e-14 on every
    # particle, and the mixed form's error budget holds against FP64.
    p = gpu.ics.plummer(262144, seed=11)
    a_b = gpu_accel(gpu, p, "basic", softening=0.005)
    a_c = gpu_accel(gpu, p, "compensated", softening=0.005)
    err = rel_err_vec(a_b, a_c)
    assert err.max() <= FP64_TOL, err.max()
    # Newton's third law: total force vanishes relative to the force scale.
    f = (p["m"][:, None] * a_c).sum(axis=0)
    scale = np.abs(p["m"][:, None] * a_c).sum()
    assert np.abs(f).max() / scale < 1e-12
    for mode in ("mixed", "mixed_split"):
        a_m = gpu_accel(gpu, p, mode, softening=0.005)
        e = rel_err_vec(a_m, a_c)
        assert np.median(e) <= 1e-6 and e.max() <= 1e-3, (mode, np.median(e), e.max())
    # Rows checked against the oracle's compensated gather: the first 48 and
    # the 48 most central particles (largest cancellation).
    s = O.Sim(p, softening=0.005)
    r2 = p["x"] ** 2 + p["y"] ** 2 + p["z"] ** 2
    central = np.argsort(r2)[:48]
    O.lib().orc_gravity_compensated_omp_rows(s.ref, 0, 48)
    ref_rows = s.acc()[:48].copy()
    for a in (a_b, a_c):
        assert rel_err_vec(a[:48], ref_rows).max() <= FP64_TOL
    full = O.Sim(p, softening=0.005)
    for i in central[:16]:
        O.lib().orc_gravity_compensated_omp_rows(full.ref, int(i), int(i) + 1)
    ref_c = full.acc()[central[:16]]
    for a in (a_b, a_c):
        assert rel_err_vec(a[central[:16]], ref_c).max() <= FP64_TOL


def test_energy_matches_oracle(gpu):
    g = golden("gravity_plummer.npz")
    sim = gpu.Simulation()
    sim.softening = 0.01
    sim.add(g["particles"])
    e = sim.energy()
    assert abs(e - g["energy0"]) <= 1e-13 * abs(g["energy0"])


def test_fp64_routine_probes(gpu):
    # throughput probes of the walk's integer-pipe routines and the hardware FP64
    # forms (rgpu_probe_rate 5-12): every class runs and reports a finite rate;
    # the integer-pipe division and square root beat the hardware sequences
    L = gpu.load()
    rates = {}
    for which in range(5, 13):
        r = ctypes.c_double(0.)
        assert L.rgpu_probe_rate(which, ctypes.byref(r)) == 0
        assert 0 < r.value < 1e15
        rates[which] = r.value
    assert rates[5] > rates[10] and rates[6] > rates[11]
    bad = ctypes.c_double(0.)
    assert L.rgpu_probe_rate(13, ctypes.byref(bad)) != 0


def test_integer_pipe_ieee_arithmetic_matches_hardware(gpu):
    # the exact tree walk's division, square root, non-negative addition,
    # multiplication and square, bit for bit against the GPU's own IEEE
    # operations on 2e7 operand sets (normal range, edge mantissas, signs)
    L = gpu.load()
    bad = ctypes.c_longlong(-1)
    assert L.rgpu_selftest_exactfp(20_000_000, 12345, ctypes.byref(bad)) == 0
    assert bad.value == 0
