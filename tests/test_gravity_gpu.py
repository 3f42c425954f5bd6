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
    L = gpu.load()
    assert L.rgpu_set_kernel_variant(variant, 1) == 0
    try:
        g = golden("gravity_plummer.npz")
        a = gpu_accel(gpu, g["particles"], "basic", softening=0.01)
        err = rel_err_vec(a, g["acc_basic"])
        assert err.max() <= FP64_TOL, err.max()
        # and against the compensated (most accurate) reference sum
        assert rel_err_vec(a, g["acc_compensated"]).max() <= FP64_TOL
    finally:
        L.rgpu_set_kernel_variant(3, 0)


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
