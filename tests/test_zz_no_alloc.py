"""Allocation-free direct summation (rgpu_direct_accel_noalloc) through the C ABI.

The entry point serves callers that cannot allocate device memory when they
need forces (a framework that owns all device allocations, a locked-down
embedding allocator): the caller passes device arrays for positions, masses and
accelerations, and the library's scratch is a fixed device array inside the
library.  Its results must agree with the allocating entry point
(rgpu_update_acceleration) to the FP64 tolerance used by the other gravity
tests, on two calls in a row with different inputs (the second reuses the
scratch left by the first).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err_vec

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-14
BASIC, COMPENSATED = 1, 2
MIXED, MIXED_SPLIT = 64, 65
NAMES = {BASIC: "basic", COMPENSATED: "compensated", MIXED: "mixed", MIXED_SPLIT: "mixed_split"}


def noalloc_accel(R, torch, p, gravity, softening):
    L = R.load()
    n = len(p)
    inputs = [torch.tensor(np.ascontiguousarray(p[f]), dtype=torch.float64, device="cuda") for f in ("x", "y", "z", "m")]
    outputs = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3)]
    stream = torch.cuda.current_stream()
    rc = L.rgpu_direct_accel_noalloc(*[t.data_ptr() for t in inputs], *[t.data_ptr() for t in outputs], n, 1.0,
                                     softening, gravity, ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    return np.stack([t.cpu().numpy() for t in outputs], axis=1)


def allocating_accel(R, p, gravity, softening):
    sim = R.Simulation()
    sim.gravity = NAMES[gravity]
    sim.softening = softening
    sim.add(p)
    sim.update_acceleration()
    return R.accelerations(sim)


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    R = gpu
    first = R.ics.plummer(4096, seed=21)
    second = R.ics.plummer(3001, seed=22)          # smaller and different: stale scratch must not leak
    for p, gravity in ((first, BASIC), (second, BASIC), (second, COMPENSATED)):
        a = noalloc_accel(R, torch, p, gravity, 0.01)
        ref = allocating_accel(R, p, gravity, 0.01)
        assert np.all(np.isfinite(a))
        err = rel_err_vec(a, ref)
        assert err.max() <= FP64_TOL, (len(p), gravity, err.max())


def test_noalloc_mixed_forms_twice(gpu):
    # MIXED_SPLIT keeps its float split in its own region of the scratch array;
    # both mixed forms against the allocating path at the mixed-precision budget
    # of the other gravity tests (median <= 1e-6, max <= 1e-3), two calls in a row.
    torch = pytest.importorskip("torch")
    R = gpu
    for p in (R.ics.plummer(4096, seed=23), R.ics.plummer(2999, seed=24)):
        for gravity in (MIXED, MIXED_SPLIT):
            a = noalloc_accel(R, torch, p, gravity, 0.01)
            ref = allocating_accel(R, p, BASIC, 0.01)
            err = rel_err_vec(a, ref)
            assert np.median(err) <= 1e-6 and err.max() <= 1e-3, (len(p), gravity, np.median(err), err.max())


def test_noalloc_rejects_sizes_beyond_its_maximum(gpu):
    torch = pytest.importorskip("torch")
    L = gpu.load()
    buf = torch.zeros(1, dtype=torch.float64, device="cuda")
    ptr = buf.data_ptr()
    rc = L.rgpu_direct_accel_noalloc(ptr, ptr, ptr, ptr, ptr, ptr, ptr, 65537, 1.0, 0.0, BASIC, None)
    assert rc == 10     # RGPU_ERR_CAPACITY, checked on the host before any launch
