"""Serving engine: continuous batching of mixed WHFast / Plummer-cluster requests.

Bar: every request's result is the same alone and in the mix (bit for bit:
per-request kernels do not depend on their batch neighbours); WHFast results
track the plain per-simulation path to 1e-9 relative and clusters to 1e-6
relative (the two paths differ in FMA contraction and summation split only);
admission respects the HBM budget; a host-side wait times out without
disturbing the request.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
XV = ("x", "y", "z", "vx", "vy", "vz")


def small_stream(R, n=24):
    from rebound_gb300.serve import make_stream
    return make_stream(n, seed=13, t_end_periods=(5.0, 60.0), cluster_n=(256, 700), cluster_steps=(20, 60))


def same(a, b):
    return all(np.array_equal(a[f], b[f]) for f in XV)


def test_results_identical_alone_and_in_the_mix(gpu):
    from rebound_gb300.serve import Server, run_stream
    reqs = small_stream(gpu)
    lat, mixed, makespan, st = run_stream(reqs, rate=400.0)
    assert st["completed"] == len(reqs)
    assert np.all(lat > 0)
    for q in (0, 3, 7, 11, len(reqs) - 1):
        srv = Server()
        out, _ = srv.wait(srv.submit(*reqs[q]))
        srv.close()
        assert same(out, mixed[q]), q


def test_time_sliced_ticks_give_the_same_results(gpu):
    # tick_ns > 0: each warp steps its system for a device-time budget per tick
    # instead of a fixed chunk; results are the same step sequence, so bit for
    # bit the fixed-chunk results
    from rebound_gb300.serve import Server, run_stream
    reqs = small_stream(gpu, 16)
    fixed = Server(tick_ns=0)
    _, res_fixed, _, st_fixed = run_stream(reqs, rate=1000.0, server=fixed)
    fixed.close()
    sliced = Server(tick_ns=200_000)
    _, res_sliced, _, st_sliced = run_stream(reqs, rate=1000.0, server=sliced)
    sliced.close()
    assert st_sliced["completed"] == st_fixed["completed"] == len(reqs)
    for q in range(len(reqs)):
        assert same(res_fixed[q], res_sliced[q]), q


def test_time_sliced_config_is_checked(gpu):
    from rebound_gb300 import _lib
    from rebound_gb300.serve import Server
    with pytest.raises(_lib.RGPUError):
        Server(tick_ns=-1)
    with pytest.raises(_lib.RGPUError):
        Server(tick_ns=2_000_000_000)
    with pytest.raises(_lib.RGPUError):
        Server(steps_per_launch=1 << 40)


@pytest.mark.parametrize("thread_per_system", [0, 1])
def test_results_track_plain_path(gpu, thread_per_system):
    # 0: warp per WHFast system (lanes = bodies, prefix-sum Jacobi transforms);
    # 1: thread per system (the serial restatement)
    from rebound_gb300.serve import Server, run_stream, WHFAST
    reqs = small_stream(gpu, 12)
    srv = Server(thread_per_system=thread_per_system)
    _, res, _, _ = run_stream(reqs, rate=1000.0, server=srv)
    srv.close()
    checked = {1: 0, 2: 0}
    for (kind, p, dt, steps, G, soft), out in zip(reqs, res):
        sim = gpu.Simulation()
        sim.dt = dt
        sim.softening = soft
        if kind == WHFAST:
            sim.integrator = "whfast"
            tol = 1e-9
        else:
            sim.integrator = "leapfrog"
            sim.gravity = "mixed_split"
            tol = 1e-6
        sim.add(p)
        sim.steps(steps)
        ref = sim.particles
        for f in ("x", "y", "z"):
            scale = np.abs(ref[f]).max()
            assert np.abs(out[f] - ref[f]).max() <= tol * scale, (kind, f)
        checked[kind] += 1
    assert checked[1] > 0 and checked[2] > 0


def test_admission_respects_budget(gpu):
    # A budget that holds one cluster at a time: requests queue, all complete.
    from rebound_gb300.serve import Server, CLUSTER
    p = gpu.ics.plummer(512, seed=3)
    srv = Server(hbm_budget_bytes=512 * 112 + 1024)
    ids = [srv.submit(CLUSTER, p, 1e-3, 30, 1.0, 0.01) for _ in range(4)]
    outs = [srv.wait(i)[0] for i in ids]
    srv.close()
    for o in outs[1:]:
        assert same(o, outs[0])


def test_wait_timeout_leaves_request_running(gpu):
    from rebound_gb300.serve import Server, WHFAST
    systems, periods = gpu.ics.planetary_systems(1, seed=4)
    srv = Server()
    rid = srv.submit(WHFAST, systems[0], periods[0] / 20, 200000)
    with pytest.raises(gpu.RGPUError) as e:
        srv.wait(rid, timeout=0.0)
    assert e.value.code == 11
    out, lat = srv.wait(rid, timeout=600.0)
    srv.close()
    assert np.all(np.isfinite(out["x"])) and lat > 0
