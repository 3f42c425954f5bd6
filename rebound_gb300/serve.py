"""Serving: continuous batching of integrate requests on one GPU.

`Server` wraps the C++ request loop of librebound_gb300 (rgpu_server_*): requests
are queued from any thread, admitted against an HBM budget, advanced in batched
kernels tick by tick, and returned with their submit-to-finish latency.
`bench_summary` drives it with a Poisson stream shaped like the reference's
served-request configuration and reports p50/p99 latency and throughput beside
the plain one-simulation-per-call GPU path.
"""
import ctypes
import threading
import time

import numpy as np

from . import _lib
from ._lib import PARTICLE_DTYPE, RGPUError, ServerConfig, ServerStats

WHFAST, CLUSTER = 1, 2


class Server:
    def __init__(self, hbm_budget_bytes=None, steps_per_launch=None, slots_per_bucket=None, pool_particles=None,
                 cluster_steps_per_tick=None, thread_per_system=None, tick_ns=None):
        self._L = _lib.load()
        cfg = ServerConfig()
        self._L.rgpu_server_config_default(ctypes.byref(cfg))
        for k, v in dict(hbm_budget_bytes=hbm_budget_bytes, steps_per_launch=steps_per_launch,
                         slots_per_bucket=slots_per_bucket, pool_particles=pool_particles,
                         cluster_steps_per_tick=cluster_steps_per_tick, thread_per_system=thread_per_system,
                         tick_ns=tick_ns).items():
            if v is not None:
                setattr(cfg, k, v)
        h = ctypes.c_void_p()
        rc = self._L.rgpu_server_create(ctypes.byref(h), ctypes.byref(cfg))
        if rc:
            raise RGPUError(rc, "server create")
        self._h = h
        self._n = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.rgpu_server_free(self._h)
            self._h = ctypes.c_void_p()

    __del__ = close

    def submit(self, kind, particles, dt, n_steps, G=1.0, softening=0.0):
        p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
        rid = ctypes.c_int64(0)
        rc = self._L.rgpu_server_submit(self._h, kind, p.ctypes.data, len(p), PARTICLE_DTYPE.itemsize, float(dt),
                                        int(n_steps), float(G), float(softening), ctypes.byref(rid))
        if rc:
            raise RGPUError(rc, "submit")
        self._n[rid.value] = p.copy()
        return rid.value

    def wait(self, rid, timeout=600.0):
        out = self._n[rid]
        lat = ctypes.c_double(0)
        rc = self._L.rgpu_server_wait(self._h, rid, out.ctypes.data, PARTICLE_DTYPE.itemsize, float(timeout),
                                      ctypes.byref(lat))
        if rc:
            raise RGPUError(rc, f"request {rid}")
        del self._n[rid]
        return out, lat.value

    def stats(self):
        st = ServerStats()
        self._L.rgpu_server_get_stats(self._h, ctypes.byref(st))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}


def make_stream(n_requests, seed=5, frac_whfast=0.8, t_end_periods=(1e2, 1e5), cluster_n=(256, 8192),
                cluster_steps=(100, 2000)):
    """Requests shaped like the served-stream configuration: 80% planetary
    systems (k in [2, 10], end time log-uniform in inner orbital periods,
    WHFast at dt = P_inner/20) and 20% Plummer clusters (N log-uniform,
    leapfrog dt = 1e-3, softening 0.01, mixed precision)."""
    from . import ics
    rng = np.random.default_rng(seed)
    kinds = rng.random(n_requests) < frac_whfast
    n_wh = int(kinds.sum())
    systems, periods = ics.planetary_systems(max(n_wh, 1), seed=seed)
    reqs = []
    w = 0
    for q in range(n_requests):
        if kinds[q]:
            P = periods[w]
            t_end = np.exp(rng.uniform(np.log(t_end_periods[0]), np.log(t_end_periods[1]))) * P
            dt = P / 20.0
            reqs.append((WHFAST, systems[w], dt, int(np.ceil(t_end / dt)), 1.0, 0.0))
            w += 1
        else:
            n = int(np.exp(rng.uniform(np.log(cluster_n[0]), np.log(cluster_n[1]))))
            p = ics.plummer(n, seed=int(rng.integers(1, 2**31)))
            reqs.append((CLUSTER, p, 1e-3, int(rng.integers(cluster_steps[0], cluster_steps[1] + 1)), 1.0, 0.01))
    return reqs


def run_stream(reqs, rate, seed=9, server=None, deadline_s=900.0):
    """Submit `reqs` with Poisson arrivals at `rate` per second; return latencies and results.
    Waits are bounded: a request still running after `deadline_s` raises instead of blocking."""
    srv = server or Server()
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    ids = [None] * len(reqs)
    results = [None] * len(reqs)
    lat = np.zeros(len(reqs))
    errors = []
    done = threading.Event()
    t_start = time.perf_counter()

    def collector():
        try:
            for q in range(len(reqs)):
                while ids[q] is None:
                    if time.perf_counter() - t_start > deadline_s:
                        raise TimeoutError("submission stalled")
                    time.sleep(0.0005)
                while True:
                    try:
                        results[q], lat[q] = srv.wait(ids[q], timeout=1.0)
                        break
                    except RGPUError as e:
                        if e.code != 11 or time.perf_counter() - t_start > deadline_s:
                            raise
        except Exception as e:  # surfaced to the caller below
            errors.append(e)
        finally:
            done.set()

    th = threading.Thread(target=collector, daemon=True)
    t0 = time.perf_counter()
    th.start()
    next_t = t0
    for q, r in enumerate(reqs):
        next_t += gaps[q]
        d = next_t - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids[q] = srv.submit(*r)
    done.wait(timeout=deadline_s + 60.0)
    makespan = time.perf_counter() - t0
    if errors or not done.is_set():
        if server is None:
            srv.close()
        raise RuntimeError(f"stream did not complete: {errors[:1] or 'deadline'}")
    st = srv.stats()
    if server is None:
        srv.close()
    return lat, results, makespan, st


def run_stream_bounded(reqs, rate, wall_s, seed=9, **server_kw):
    """Submit `reqs` with Poisson arrivals at `rate` per second and stop waiting
    `wall_s` seconds after the first submission.  Returns the server-side latency
    of every request that finished by then (NaN for the others), the number still
    in flight, the elapsed time and the server's counters.  `server_kw` configure
    the Server."""
    srv = Server(**server_kw)
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    ids = []
    t0 = time.perf_counter()
    next_t = t0
    for r, g in zip(reqs, gaps):
        next_t += g
        d = next_t - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids.append(srv.submit(*r))
    lat = np.full(len(reqs), np.nan)
    pending = list(range(len(reqs)))
    while pending and time.perf_counter() - t0 < wall_s:
        still = []
        for q in pending:
            try:
                _, lat[q] = srv.wait(ids[q], timeout=0.05)
            except RGPUError as e:
                if e.code != 11:
                    srv.close()
                    raise
                still.append(q)
        pending = still
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return lat, len(pending), elapsed, st


def plain_rate(reqs, max_whfast=8, steps_cap=400, clusters=2, cluster_steps_cap=20):
    """System-steps/s and pair-int/s of the plain path (one rgpu_sim per request,
    one C-ABI call per step) on a sample of the stream with capped steps."""
    from .simulation import Simulation
    L = _lib.load()
    wh_steps, wh_time, pairs, cl_time = 0, 0.0, 0.0, 0.0
    for kind, p, dt, n_steps, G, soft in [r for r in reqs if r[0] == WHFAST][:max_whfast]:
        sim = Simulation()
        sim.dt, sim.integrator = dt, "whfast"
        sim.add(p)
        h = sim.handle
        steps = min(n_steps, steps_cap)
        t0 = time.perf_counter()
        for _ in range(steps):
            L.rgpu_steps(h, 1)
        wh_time += time.perf_counter() - t0
        wh_steps += steps
    for kind, p, dt, n_steps, G, soft in [r for r in reqs if r[0] == CLUSTER][:clusters]:
        sim = Simulation()
        sim.dt, sim.softening, sim.gravity, sim.integrator = dt, soft, "mixed_split", "leapfrog"
        sim.add(p)
        h = sim.handle
        steps = min(n_steps, cluster_steps_cap)
        t0 = time.perf_counter()
        for _ in range(steps):
            L.rgpu_steps(h, 1)
        cl_time += time.perf_counter() - t0
        pairs += steps * len(p) * (len(p) - 1.0)
    return {"whfast_system_steps_per_s": wh_steps / wh_time if wh_time else None,
            "cluster_pair_int_per_s": pairs / cl_time if cl_time else None}


def bench_summary(quick=False, n_requests=240, rates=(100.0,), t_end_periods=(1e2, 1e5), wall_s=90.0,
                  **server_kw):
    """Served stream of the configuration: 80 % WHFast systems with end times
    log-uniform in [1e2, 1e5] inner periods (2e3 to 2e6 steps each), 20 % Plummer
    clusters, Poisson arrivals.  The run is bounded by the request count and by
    `wall_s` seconds of wall time: p50 / p99 are over the requests that finished,
    and the number still in flight at the end is reported beside them."""
    if quick:
        n_requests, t_end_periods, wall_s = 60, (1e2, 1e3), 60.0
    reqs = make_stream(n_requests, t_end_periods=t_end_periods)
    wh_steps = sum(r[3] for r in reqs if r[0] == WHFAST)
    cl_pairs = sum(r[3] * len(r[1]) * (len(r[1]) - 1.0) for r in reqs if r[0] == CLUSTER)
    out = {"requests": n_requests, "whfast_requests": sum(r[0] == WHFAST for r in reqs),
           "t_end_inner_periods": list(t_end_periods), "whfast_system_steps": wh_steps,
           "cluster_pair_interactions": cl_pairs, "runs": []}
    kinds = np.array([r[0] for r in reqs])
    steps = np.array([r[3] for r in reqs], dtype=np.float64)
    for rate in rates:
        lat, in_flight, elapsed, st = run_stream_bounded(reqs, rate, wall_s, **server_kw)
        ok = np.isfinite(lat)
        q = lambda m, f: float(np.quantile(lat[ok & m], f)) if np.any(ok & m) else None
        out["runs"].append({"rate_per_s": rate, "completed": int(ok.sum()), "in_flight_at_end": int(in_flight),
                            "wall_s": elapsed, "p50_latency_s": q(ok, 0.5), "p99_latency_s": q(ok, 0.99),
                            "p50_latency_whfast_s": q(kinds == WHFAST, 0.5),
                            "p99_latency_whfast_s": q(kinds == WHFAST, 0.99),
                            "p50_latency_cluster_s": q(kinds == CLUSTER, 0.5),
                            "max_steps_completed": float(steps[ok].max()) if ok.any() else 0.0,
                            "system_steps_per_s": st["system_steps"] / elapsed,
                            "pair_int_per_s": st["pair_interactions"] / elapsed,
                            "ticks": st["ticks"]})
    plain = plain_rate(reqs)
    out["plain_path"] = plain
    best = max(r["system_steps_per_s"] for r in out["runs"])
    if plain["whfast_system_steps_per_s"]:
        out["whfast_speedup_vs_plain"] = best / plain["whfast_system_steps_per_s"]
        out["plain_path_serial_seconds_est"] = wh_steps / plain["whfast_system_steps_per_s"]
    return out
