#!/usr/bin/env python
"""Benchmark: FP64 direct-sum leapfrog steps on a Plummer sphere, N = 262,144.

Workload (the reference's large direct-sum configuration): seeded Plummer
sphere truncated at r = 10, softening 0.005, leapfrog (order 2) with
dt = 1e-4, REB_GRAVITY_BASIC in FP64.  One step = drift + O(N^2) force
evaluation + kick/drift on the device.  Metric: Gpair-int/s = N (N-1) per step
/ step time.  The same line reports COMPENSATED and the mixed-precision forms,
their accuracy against FP64, the roofline of the dominant kernel against the
FP64 pipe peak measured live on this GPU, and an end-to-end figure through the
C ABI with host buffers.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Inputs are already resident in HBM for `value`; between timed steps L2 is
flushed by writing 512 MB of scratch on the stream (the j-data of one step is
only 8 MB and stays L2-resident within a step by design).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_DEFAULT = 262144
SOFTENING = 0.005
DT = 1e-4
SEED = 11
FLOPS_PER_PAIR = 20          # 3 sub, 6 for r^2+eps^2, sqrt, 2 mul, div, mul by m, 6 accumulate
L2_FLUSH_BYTES = 512 << 20
METRIC = "Gpair-int/s FP64 vs mixed, N=262k; ensemble steps/s; p50/p99 latency"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, dist, device):
    """Max of a per-rank time over all ranks: the job is as slow as its slowest rank."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank_step, steps, world, total_ms):
    """Whole-job throughput: every rank processes its own units (replicas, weak
    scaling), so the job's units over the slowest rank's time."""
    return units_per_rank_step * steps * world / (total_ms * 1e-3)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        smax = max([num(r[2]) for r in rows if num(r[2])] or [0])
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(n)
        load = [x for x in sm if x > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows)}


def oracle_cpu_rate(particles, seconds=10.0, label="sample"):
    """Oracle (port of the reference's OpenMP BASIC gather, src/gravity.c:215-233)
    on all host cores: time a bounded block of i-rows against all N j-bodies."""
    from oracle import oracle as O
    n = len(particles)
    s = O.Sim(particles, softening=SOFTENING)
    T = O.lib_timing()
    rows = 512
    t0 = time.perf_counter()
    T.orc_gravity_basic_omp_rows(s.ref, 0, rows)
    dt = time.perf_counter() - t0
    rows = int(min(n, max(512, rows * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    T.orc_gravity_basic_omp_rows(s.ref, 0, rows)
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return rows * (n - 1) / dt / 1e9, cores, f"{rows} of {n} i-rows x {n} j-bodies, FP64 BASIC gather ({dt:.1f} s)"


def config_block(n, world):
    return {"workload": f"Plummer N={n}, softening {SOFTENING}, leapfrog dt={DT}, REB_GRAVITY_BASIC FP64",
            "N": n, "softening": SOFTENING, "dt": DT, "seed": SEED, "gravity": "basic", "integrator": "leapfrog",
            "parallelism": f"replicas{world}" if world > 1 else "single-gpu",
            "l2": "flushed between timed steps (512 MB scratch write)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    import numpy as np
    # Inputs from the reference's own Plummer construction (restated in the oracle harness).
    p = plummer_oracle(args.n)
    s = O.Sim(p, softening=SOFTENING)
    L = O.lib_timing()
    n = args.n
    rows = 256
    t0 = time.perf_counter()
    L.orc_gravity_basic_omp_rows(s.ref, 0, rows)
    dt = time.perf_counter() - t0
    rows = int(min(n, max(256, rows * args.ref_seconds / max(dt, 1e-6))))
    times = []
    for k in range(args.warmup + args.steps):
        r0 = (k * rows) % max(1, n - rows)
        t0 = time.perf_counter()
        L.orc_gravity_basic_omp_rows(s.ref, r0, r0 + rows)
        el = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(el)
    rate = rows * (n - 1) * len(times) / sum(times) / 1e9
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = (f"{rows} of {n} i-rows x {n} j-bodies per step (oracle port of the OpenMP BASIC gather, "
              f"src/gravity.c:215-233, timing build); the reference's own C is not on the GPU machine")
    # ms_per_step is the time of one sampled step (what this run spent per step);
    # a full N^2 evaluation at the same rate is given beside it.
    out = {"metric": METRIC, "value": rate, "unit": "Gpair-int/s", "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
           "ms_per_full_step_est": 1e3 * n * (n - 1) / (rate * 1e9), "sample_fraction": rows / n,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded Plummer sphere)", "config": config_block(n, 1),
           "cpu_baseline": {"value": rate, "unit": "Gpair-int/s", "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": rate, "unit": "Gpair-int/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def plummer_oracle(n):
    """Seeded Plummer sphere for the reference arm without the product library."""
    import numpy as np
    from oracle import oracle as O
    out = np.zeros(n, dtype=O.PARTICLE_DTYPE)
    O.lib().orc_ic_plummer(SEED, n, 1.0, 1.0, 10.0, out.ctypes.data)
    return out


def run_gb300(args):
    rank, world, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import rebound_gb300 as R
    L = R.load()
    n = args.n
    p = R.ics.plummer(n, seed=SEED)

    def make(gravity):
        sim = R.Simulation()
        sim.softening = SOFTENING
        sim.dt = DT
        sim.gravity = gravity
        sim.integrator = "leapfrog"
        sim.add(p)
        return sim

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    sim = make("basic")
    h = sim.handle
    ms = ctypes.c_double(0.)
    for _ in range(args.warmup):
        R._lib.check(L.rgpu_sim_time_steps(h, 1, ctypes.byref(ms)), h)
    L.rgpu_sim_kernel_timer(h, 1)
    clocks = Clocks(local)
    launches0 = L.rgpu_launch_count()
    barrier()
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        R._lib.check(L.rgpu_l2_flush(h, L2_FLUSH_BYTES), h)
        R._lib.check(L.rgpu_sim_time_steps(h, 1, ctypes.byref(ms)), h)
        total_ms += ms.value
    barrier()
    clk = clocks.stop()
    launches = L.rgpu_launch_count() - launches0
    kms, kn = ctypes.c_double(0.), ctypes.c_int64(0)
    L.rgpu_sim_kernel_time(h, ctypes.byref(kms), ctypes.byref(kn))
    total_ms = max_over_ranks(total_ms, dist, "cuda")
    pairs = n * (n - 1)
    value = job_rate(pairs, args.steps, world, total_ms) / 1e9
    ms_step = total_ms / args.steps
    kernel_ms = kms.value / max(1, kn.value)

    # FP64 pipe: nominal issue rate at the sampled clock, and the live DFMA probe
    # (lane-ops/s x 2 flops); FP32 and integer-ALU probes.
    rate = ctypes.c_double(0.)
    L.rgpu_probe_rate(0, ctypes.byref(rate))
    fp64_probe = 2 * rate.value / 1e12
    L.rgpu_probe_rate(1, ctypes.byref(rate))
    fp32_peak = 2 * rate.value / 1e12
    L.rgpu_probe_rate(4, ctypes.byref(rate))
    alu_peak = rate.value / 1e12
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    fp64_nominal = nominal_fp64_tflops(sm_count, (clk or {}).get("sm_mhz"))
    pair_rate = pairs / (kernel_ms * 1e-3)
    counts = profiled_counts()
    fp64_equiv = FLOPS_PER_PAIR * pair_rate / 1e12

    # Accuracy and speed of the other forms (force evaluation at step 0).
    forms = {}
    form_list = () if args.lite else ("basic", "compensated", "mixed", "mixed_split")
    ref_sim = make("compensated") if form_list else None
    if ref_sim is None:
        a_ref = None
    else:
        ref_sim.update_acceleration()
        a_ref = R.accelerations(ref_sim)
        del ref_sim
    for form in form_list:
        fs = make(form)
        fh = fs.handle
        R._lib.check(L.rgpu_sim_time_steps(fh, 1, ctypes.byref(ms)), fh)       # warm
        fs.set_particles_array(p)
        fs.update_acceleration()
        a = R.accelerations(fs)
        den = np.linalg.norm(a_ref, axis=1)
        err = np.linalg.norm(a - a_ref, axis=1) / np.where(den > 0, den, 1)
        fh = fs.handle
        L.rgpu_sim_kernel_timer(fh, 1)
        steps_f = 2
        tf = 0.0
        for _ in range(steps_f):
            L.rgpu_l2_flush(fh, L2_FLUSH_BYTES)
            R._lib.check(L.rgpu_sim_time_steps(fh, 1, ctypes.byref(ms)), fh)
            tf += ms.value
        fk, fkn = ctypes.c_double(0.), ctypes.c_int64(0)
        L.rgpu_sim_kernel_time(fh, ctypes.byref(fk), ctypes.byref(fkn))
        forms[form] = {"gpair_per_s": pairs * steps_f / (tf * 1e-3) / 1e9, "ms_per_step": tf / steps_f,
                       "kernel_ms": fk.value / max(1, fkn.value),
                       "median_rel_err_vs_compensated": float(np.median(err)),
                       "max_rel_err_vs_compensated": float(err.max())}
        del fs
    if form_list:
        forms["mixed_speedup_vs_fp64"] = forms["mixed"]["gpair_per_s"] / forms["basic"]["gpair_per_s"]
        forms["mixed_split_speedup_vs_fp64"] = forms["mixed_split"]["gpair_per_s"] / forms["basic"]["gpair_per_s"]

    # End to end through the C ABI: pinned host AoS in, step, AoS out.
    host = torch.empty(n * 112, dtype=torch.uint8, pin_memory=True)
    hv = host.numpy().view(R.PARTICLE_DTYPE)
    hv[:] = p
    e2e_steps = max(2, min(args.steps, 3))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        R._lib.check(L.rgpu_sim_set_particles(h, host.data_ptr(), n, 112), h)
        R._lib.check(L.rgpu_steps(h, 1), h)
        R._lib.check(L.rgpu_sim_get_particles(h, host.data_ptr(), n, 112), h)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e = {"value": job_rate(pairs, e2e_steps, world, e2e_s * 1e3) / 1e9, "unit": "Gpair-int/s",
           "h2d_bytes_per_step": n * 112, "d2h_bytes_per_step": n * 88}

    extra = {}
    if args.precision and rank == 0 and not args.lite:
        for key, fn in (("c1", lambda: c1_summary(cpu_seconds=2.0 if args.quick else 8.0)),
                        ("c2_drift", lambda: c2_drift_summary(steps=10 if args.quick else 100)),
                        ("c5_cluster_drift", lambda: c5_cluster_drift(steps=200 if args.quick else 1000))):
            try:
                extra[key] = fn()
            except Exception as ex:
                extra[key] = {"error": repr(ex)}
    if args.ensemble and rank == 0 and not args.lite:
        try:
            from rebound_gb300 import ensemble as E
            extra["ensemble"] = E.bench_summary(quick=args.quick)
            extra["ensemble"]["cpu_baseline"] = ensemble_cpu_baseline(seconds=2.0 if args.quick else 8.0)
            extra["ensemble"]["roofline"] = ensemble_roofline(extra["ensemble"]["system_steps_per_s"], sm_count,
                                                              (clk or {}).get("sm_mhz"))
        except Exception as ex:  # reported, not hidden
            extra["ensemble"] = {"error": repr(ex)}
    if args.tree and rank == 0 and not args.lite:
        try:
            extra["tree"] = tree_summary(quick=args.quick, sm_count=sm_count, sm_mhz=(clk or {}).get("sm_mhz"))
        except Exception as ex:
            extra["tree"] = {"error": repr(ex)}
    if args.serve and rank == 0 and not args.lite:
        import importlib.util
        if importlib.util.find_spec("rebound_gb300.serve") is not None:
            from rebound_gb300 import serve as S
            try:
                extra["serving"] = S.bench_summary(quick=args.quick)
            except Exception as ex:
                extra["serving"] = {"error": repr(ex)}

    if rank == 0:
        cpu_val, cores, sample = oracle_cpu_rate(p, seconds=args.cpu_seconds)
        out = {"metric": METRIC, "value": value, "unit": "Gpair-int/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Plummer sphere)",
               "config": config_block(n, world),
               "e2e": e2e, "gpu_launches": int(launches),
               "roofline": roofline_block(counts, pair_rate, alu_peak, fp64_probe, fp64_nominal, fp32_peak,
                                          fp64_equiv, kernel_ms),
               "forms": forms,
               "cpu_baseline": {"value": cpu_val, "unit": "Gpair-int/s", "cores": cores, "kind": "port",
                                "sample": sample},
               "clocks": clk}
        out.update(extra)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


TREE_COUNTS_FILE = os.path.join(REPO, "profiles", "tree_walk_counts.json")


def tree_summary(quick=False, steps=2, sm_count=None, sm_mhz=None):
    """Configuration-3 ring patch: SEI, tree gravity (opening angle 0.5, 25 ghost
    boxes), shear boundary, tree collision search + hardsphere (epsilon 0.5).
    Device-timed full steps, a split of gravity / collision time, and the oracle
    (port of the reference's OpenMP tree walk) on a row sample of the same
    particles for the CPU baseline."""
    import numpy as np
    import rebound_gb300 as R
    from oracle import oracle as O
    L = R.load()
    box = 400.0 if quick else 2300.0
    p = R.ics.ring_patch(box, seed=7)
    n_root = int(box / 20.0)
    omega = 1.3143527e-4

    def make():
        sim = R.Simulation()
        sim.G, sim.OMEGA, sim.softening = 6.674e-11, omega, 0.1
        sim.dt = 1e-3 * 2 * np.pi / omega
        sim.configure_box(20.0, n_root, n_root, 1)
        sim.configure_ghostboxes(2, 2, 0)
        sim.opening_angle2 = 0.25
        sim.boundary, sim.gravity, sim.integrator = "shear", "tree", "sei"
        sim.collision, sim.collision_resolve = "tree", "hardsphere"
        sim.coefficient_of_restitution = 0.5
        sim.add(p)
        return sim

    sim = make()
    h = sim.handle
    ms = ctypes.c_double(0)
    R._lib.check(L.rgpu_sim_time_steps(h, 1, ctypes.byref(ms)), h)        # warm-up
    times = []
    for _ in range(steps):
        R._lib.check(L.rgpu_sim_time_steps(h, 1, ctypes.byref(ms)), h)
        times.append(ms.value)
    step_s = sum(times) / len(times) / 1e3
    R._lib.check(L.rgpu_sim_get_config(h, ctypes.byref(sim._cfg)), h)     # counters advanced by the steps
    rms, rcalls = sim.resolve_time()
    resolve = {"host_ms_per_step": rms / max(1, steps + 1), "share_of_step": rms / max(1, steps + 1) / (1e3 * step_s),
               "collisions_per_step": sim.collisions_log_n / (steps + 1)}
    g = make()
    g.collision = "none"
    t0 = time.perf_counter()
    g.update_acceleration()                 # returns after the device status is read (synchronous)
    grav_s = time.perf_counter() - t0
    # split mode: exact near-window walk + mixed-precision far-root sweep
    sp = make()
    sp.gravity = "tree_split"
    sp.collision = "none"
    sp.update_acceleration()
    t0 = time.perf_counter()
    sp.update_acceleration()
    split_s = time.perf_counter() - t0
    a_split = R.accelerations(sp)
    a_exact = R.accelerations(g)
    den = np.linalg.norm(a_exact, axis=1)
    split_err = np.linalg.norm(a_split - a_exact, axis=1) / np.where(den > 0, den, 1)
    sp2 = make()
    sp2.gravity = "tree_split"
    h2 = sp2.handle
    R._lib.check(L.rgpu_sim_time_steps(h2, 1, ctypes.byref(ms)), h2)
    split_step = []
    for _ in range(steps):
        R._lib.check(L.rgpu_sim_time_steps(h2, 1, ctypes.byref(ms)), h2)
        split_step.append(ms.value)
    split_step_s = sum(split_step) / len(split_step) / 1e3
    c = make()
    ch = c.handle
    n = ctypes.c_size_t(0)
    out = np.zeros(max(1024, 4 * len(p)), dtype=R.COLLISION_DTYPE)
    t0 = time.perf_counter()
    R._lib.check(L.rgpu_collision_search(ch, out.ctypes.data, len(out), ctypes.byref(n)), ch)
    coll_s = time.perf_counter() - t0
    # CPU baseline: oracle tree walk (OpenMP over particles) on a row sample
    orc = O.Sim(p, G=6.674e-11, softening=0.1, boundary="shear", root_size=20.0, N_root=(n_root, n_root, 1),
                N_ghost=(2, 2, 0), OMEGA=omega, opening_angle2=0.25)
    rows = 64 if quick else 256
    t0 = time.perf_counter()
    O.lib_timing().orc_gravity_tree_rows(orc.ref, 0, rows)
    cpu_rows_s = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    cpu_grav_step_s = cpu_rows_s / rows * len(p)
    # Roofline of the exact walk.  The committed ncu counts (valid while tree.cu and
    # exactfp.cuh hash to the recorded digest) give, per (particle, ghost box, root)
    # visit, the FP64-pipe lane instructions and the warp instructions issued on all
    # pipes; times the visits of one walk / the walk's time, against the nominal FP64
    # pipe rate (0.5 lanes/clock/SMSP) and the issue rate (one warp instruction per
    # clock per SMSP) at the sampled clock.  The bound is the larger fraction.
    roof = {"kernel": "walk_exact"}
    try:
        with open(TREE_COUNTS_FILE) as f:
            rec = json.load(f)
        if sources_digest(rec["sources"]) == rec["sha256"]:
            visits = len(p) * 25 * n_root * n_root
            clk = sm_mhz * 1e6 if sm_mhz else None
            fp64_ach = rec["fp64_lane_inst_per_root_visit"] * visits / grav_s
            fp64_peak = FP64_LANES_PER_CLK_PER_SMSP * 4 * sm_count * clk if clk and sm_count else None
            iss_ach = rec["warp_inst_per_root_visit"] * visits / grav_s if "warp_inst_per_root_visit" in rec else None
            iss_peak = 4 * sm_count * clk if clk and sm_count else None
            fr64 = fp64_ach / fp64_peak if fp64_peak else None
            friss = iss_ach / iss_peak if (iss_ach and iss_peak) else None
            bound = "issue" if (friss or 0) > (fr64 or 0) else "fp64"
            roof.update({"bound": bound, "frac": friss if bound == "issue" else fr64,
                         "fp64": {"achieved": fp64_ach / 1e12, "peak": fp64_peak / 1e12 if fp64_peak else None,
                                  "unit": "T lane-inst/s", "frac": fr64,
                                  "inst_per_visit": rec["fp64_lane_inst_per_root_visit"]},
                         "issue": {"achieved": iss_ach / 1e12 if iss_ach else None,
                                   "peak": iss_peak / 1e12 if iss_peak else None,
                                   "unit": "T warp-inst/s", "frac": friss,
                                   "inst_per_visit": rec.get("warp_inst_per_root_visit")},
                         "visits_per_walk": visits,
                         "peak_source": "nominal rates at the sampled SM clock"})
        else:
            roof["counts"] = "tree sources changed since the ncu capture (sha256 mismatch)"
    except (OSError, ValueError, KeyError) as ex:
        roof["counts"] = repr(ex)
    # Throughput of each FP64 routine of a visit alone (rgpu_probe_rate 5-12), as
    # SM-sub-partition clocks per warp operation at the sampled clock.
    if sm_mhz and sm_count:
        names = {5: "int_div", 6: "int_sqrt", 7: "int_square", 8: "int_product", 9: "int_nonneg_sum",
                 10: "hw_div", 11: "hw_sqrt", 12: "hw_add"}
        clocks = {}
        for which, name in names.items():
            r = ctypes.c_double(0.)
            if L.rgpu_probe_rate(which, ctypes.byref(r)) == 0 and r.value > 0:
                clocks[name] = round(4 * sm_count * sm_mhz * 1e6 * 32 / r.value, 1)
        roof["routine_clocks_per_warp_op"] = clocks
    return {"workload": f"ring patch {box:.0f} m box, N={len(p)}, 25 ghost boxes, {n_root * n_root} roots",
            "N": len(p), "gpu_step_s": step_s, "gpu_tree_gravity_s": grav_s, "gpu_collision_search_s": coll_s,
            "roofline": roof, "resolve": resolve,
            "split_mode": {"gpu_step_s": split_step_s, "gpu_tree_gravity_s": split_s,
                           "steps_per_s": 1.0 / split_step_s,
                           "median_rel_diff_vs_exact_walk": float(np.median(split_err)),
                           "max_rel_diff_vs_exact_walk": float(split_err.max())},
            "pairs_found": int(n.value), "steps_per_s": 1.0 / step_s,
            "cpu_baseline": {"tree_gravity_s_per_step_est": cpu_grav_step_s, "cores": cores, "kind": "port",
                             "sample": f"{rows} of {len(p)} particles walked (oracle tree, OpenMP), scaled to N"},
            "gravity_speedup_vs_cpu": cpu_grav_step_s / grav_s,
            "split_gravity_speedup_vs_cpu": cpu_grav_step_s / split_s}


def form_drift(p, softening, dt, steps, forms=("basic", "compensated", "mixed", "mixed_split")):
    """Each force form integrated `steps` leapfrog steps from the same state:
    relative energy error (REBOUND's unsoftened energy, src/tools.c:108-162),
    device time per step, and for the mixed forms the final energy against the
    FP64 BASIC run's."""
    import rebound_gb300 as R
    L = R.load()
    out, e_final, e0 = {}, {}, None
    for form in forms:
        sim = R.Simulation()
        sim.softening, sim.dt, sim.gravity, sim.integrator = softening, dt, form, "leapfrog"
        sim.add(p)
        e_start = sim.energy()
        e0 = e_start if e0 is None else e0
        h = sim.handle
        ms = ctypes.c_double(0.)
        R._lib.check(L.rgpu_sim_time_steps(h, steps, ctypes.byref(ms)), h)
        e1 = sim.energy()
        e_final[form] = e1
        n = len(p)
        out[form] = {"energy_rel_err": abs((e1 - e_start) / e_start), "ms_per_step": ms.value / steps,
                     "gpair_per_s": n * (n - 1.0) * steps / (ms.value * 1e-3) / 1e9}
        del sim
    for form in forms:
        if form.startswith("mixed") and "basic" in e_final:
            out[form]["energy_vs_fp64"] = abs(e_final[form] - e_final["basic"]) / abs(e0)
    return out


def c1_summary(cpu_seconds=10.0):
    """Configuration 1: Plummer N = 4,096, softening 0.01, leapfrog dt = 1e-3,
    1,000 steps.  GPU forms with their energy errors; the CPU baseline is the
    oracle's port of the reference's OpenMP BASIC leapfrog on every host core,
    run over all 1,000 steps when that fits `cpu_seconds`, else over a prefix."""
    import rebound_gb300 as R
    from oracle import oracle as O
    n, soft, dt, steps = 4096, 0.01, 1e-3, 1000
    p = R.ics.plummer(n, seed=SEED)
    forms = form_drift(p, soft, dt, steps)
    T = O.lib_timing()
    s = O.Sim(p, softening=soft, dt=dt)
    e0 = T.orc_energy(s.ref)
    t0 = time.perf_counter()
    T.orc_leapfrog_step_order(s.ref, O.GRAVITY["basic_omp"], 2)
    one = time.perf_counter() - t0
    cpu_steps = int(max(1, min(steps - 1, cpu_seconds / max(one, 1e-6)))) + 1
    t0 = time.perf_counter()
    for _ in range(cpu_steps - 1):
        T.orc_leapfrog_step_order(s.ref, O.GRAVITY["basic_omp"], 2)
    el = one + time.perf_counter() - t0
    cpu = {"s_per_step": el / cpu_steps, "steps": cpu_steps, "cores": os.cpu_count() or 1, "kind": "port",
           "gpair_per_s": n * (n - 1.0) * cpu_steps / el / 1e9}
    if cpu_steps == steps:
        cpu["energy_rel_err"] = abs((T.orc_energy(s.ref) - e0) / e0)
    gpu_s = forms["basic"]["ms_per_step"] * 1e-3
    return {"workload": f"Plummer N={n}, softening {soft}, leapfrog dt={dt}, {steps} steps", "forms": forms,
            "cpu_baseline": cpu, "basic_speedup_vs_cpu": cpu["s_per_step"] / gpu_s}


def c2_drift_summary(steps=100):
    """Configuration 2 over its 100 steps: energy error of FP64 BASIC, COMPENSATED
    and the mixed forms from the same Plummer N = 262,144 state."""
    import rebound_gb300 as R
    p = R.ics.plummer(N_DEFAULT, seed=SEED)
    return {"workload": f"Plummer N={N_DEFAULT}, softening {SOFTENING}, leapfrog dt={DT}, {steps} steps",
            "forms": form_drift(p, SOFTENING, DT, steps, forms=("basic", "mixed", "mixed_split"))}


def c5_cluster_drift(steps=1000):
    """Served-stream clusters (Plummer, N in [256, 8192], softening 0.01, leapfrog
    dt = 1e-3) under the mixed forms against FP64 BASIC."""
    import rebound_gb300 as R
    out = {}
    for n in (256, 1024, 4096, 8192):
        p = R.ics.plummer(n, seed=1000 + n)
        out[str(n)] = form_drift(p, 0.01, 1e-3, steps, forms=("basic", "mixed", "mixed_split"))
    return {"steps": steps, "clusters": out}


def whfast_plain_summary(steps=200):
    """The plain one-simulation-per-call WHFast path (what the REBOUND plugin
    drives): a 5-body system of the configuration-4 generator, `steps` steps of
    P_inner / 20, one C-ABI call (one program launch) per step."""
    import rebound_gb300 as R
    L = R.load()
    systems, periods = R.ics.planetary_systems(64, seed=3)
    k = next(q for q, s in enumerate(systems) if len(s) == 5)
    sim = R.Simulation()
    sim.dt, sim.integrator = float(periods[k]) / 20.0, "whfast"
    sim.add(systems[k])
    h = sim.handle
    for _ in range(3):
        R._lib.check(L.rgpu_steps(h, 1), h)
    ms = ctypes.c_double(0.)
    R._lib.check(L.rgpu_sim_time_steps(h, steps, ctypes.byref(ms)), h)
    return {"bodies": 5, "steps": steps, "us_per_step": 1e3 * ms.value / steps}


def tree_patch_summary(box=800.0, gravity="tree"):
    """One tree-gravity evaluation and one tree collision search of a ring patch
    (configuration-3 physics, `box` metres square): the small case of the tree
    kernels' ncu summaries.  gravity "tree_split" runs the split mode."""
    import rebound_gb300 as R
    L = R.load()
    p = R.ics.ring_patch(box, seed=11)
    n_root = int(box / 20.0)
    sim = R.Simulation()
    sim.G, sim.OMEGA, sim.softening = 6.674e-11, 1.3143527e-4, 0.1
    sim.configure_box(20.0, n_root, n_root, 1)
    sim.configure_ghostboxes(2, 2, 0)
    sim.boundary, sim.gravity, sim.collision = "shear", gravity, "tree"
    sim.add(p)
    t0 = time.perf_counter()
    sim.update_acceleration()
    grav = time.perf_counter() - t0
    t0 = time.perf_counter()
    pairs = sim.collision_search()
    return {"N": len(p), "roots": n_root * n_root, "gravity": gravity, "tree_gravity_s": grav,
            "collision_search_s": time.perf_counter() - t0, "pairs": int(len(pairs))}


def ensemble_only(args):
    from rebound_gb300 import ensemble as E
    import numpy as np
    systems, periods = __import__("rebound_gb300").ics.planetary_systems(args.ens_systems, seed=3)
    ens = E.Ensemble(systems, periods / 20.0, exact=bool(args.ens_exact))
    ens.set_launch(args.ens_block, args.ens_steps)
    ms = ens.time_steps(args.ens_steps)
    return {"systems": args.ens_systems, "steps": args.ens_steps, "block": args.ens_block,
            "system_steps_per_s": args.ens_systems * args.ens_steps / (ms * 1e-3)}


def ensemble_cpu_baseline(seconds=8.0, seed=3, steps=10000):
    """The oracle's port of the reference's single-simulation WHFast step
    (src/integrator_whfast.c:1113-1259) on every host core, one system per thread
    at a time: the first systems of the configuration-4 ensemble (same generator,
    same dt = P_inner / 20), each advanced by the same 10^4 steps as on the GPU, as
    many systems as fit the time budget.  ctypes releases the GIL during each
    foreign call, so the threads run in parallel."""
    import concurrent.futures as cf
    from oracle import oracle as O
    from rebound_gb300 import ics
    O.build()
    L = O.lib_timing()
    cores = os.cpu_count() or 1
    probe = 2 * cores
    systems, periods = ics.planetary_systems(probe, seed=seed)
    sims = [O.Sim(systems[q], dt=float(periods[q]) / 20.0) for q in range(probe)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(lambda q: L.orc_whfast_steps(sims[q].ref, 2000), range(probe)))
    per_step = max((time.perf_counter() - t0) * cores / (probe * 2000), 1e-8)   # thread-seconds per system-step
    n_sys = int(min(65536, max(cores, seconds * cores / (steps * per_step))))
    systems, periods = ics.planetary_systems(n_sys, seed=seed)
    sims = [O.Sim(systems[q], dt=float(periods[q]) / 20.0) for q in range(n_sys)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(lambda q: L.orc_whfast_steps(sims[q].ref, steps), range(n_sys)))
    el = time.perf_counter() - t0
    return {"value": n_sys * steps / el, "unit": "system-steps/s", "cores": cores, "kind": "port",
            "sample": f"the first {n_sys} of the 65,536 systems (k in [2, 10]) x {steps} steps each, oracle WHFast, "
                      f"one thread per core ({el:.1f} s)"}


COUNTS_FILE = os.path.join(REPO, "profiles", "direct_kernel_counts.json")
ENSEMBLE_COUNTS_FILE = os.path.join(REPO, "profiles", "ensemble_kernel_counts.json")


def ensemble_roofline(rate, sm_count, sm_mhz):
    """FP64-pipe roofline of the thread-per-system ensemble kernel: FP64-pipe lane
    instructions per system-step from the committed ncu count (valid while the
    kernel's sources hash to the recorded digest) x the measured system-steps/s,
    against the nominal FP64 pipe rate (0.5 lanes/clock/SMSP) at the sampled clock."""
    roof = {"kernel": "ens_fast::persistent_kernel", "bound": "fp64"}
    try:
        with open(ENSEMBLE_COUNTS_FILE) as f:
            rec = json.load(f)
        if sources_digest(rec["sources"]) != rec["sha256"]:
            roof["counts"] = "ensemble sources changed since the ncu capture (sha256 mismatch)"
            return roof
        ach = rec["fp64_lane_inst_per_system_step"] * rate
        peak = FP64_LANES_PER_CLK_PER_SMSP * 4 * sm_count * sm_mhz * 1e6 if (sm_count and sm_mhz) else None
        roof.update({"achieved": ach / 1e12, "peak": peak / 1e12 if peak else None, "unit": "T lane-inst/s",
                     "frac": ach / peak if peak else None,
                     "inst_per_system_step": rec["fp64_lane_inst_per_system_step"],
                     "peak_source": "nominal FP64 pipe rate at the sampled SM clock"})
    except (OSError, ValueError, KeyError) as ex:
        roof["counts"] = repr(ex)
    return roof


def sources_digest(paths):
    import hashlib
    h = hashlib.sha256()
    for rel in paths:
        with open(os.path.join(REPO, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def profiled_counts():
    """Per-launch DRAM bytes and per-pair instruction counts of the dominant kernel,
    measured by ncu and recorded with the SHA-256 of the kernel's sources.  When the
    sources have changed since the capture the counts no longer describe the kernel:
    every count is then None and `stale` says so."""
    try:
        with open(COUNTS_FILE) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return {"stale": "no counts file"}
    if sources_digest(rec["sources"]) != rec["sha256"]:
        return {"stale": "kernel sources changed since the ncu capture (sha256 mismatch)"}
    return {k: rec.get(k) for k in ("traffic_bytes_per_launch", "alu_inst_per_pair", "inst_per_pair",
                                    "fp64_inst_per_pair")}


# FP64 pipe issue rate of GB300 (ncu's peak for sm__pipe_fp64_cycles_active):
# 0.5 lanes per clock per SM sub-partition, 4 sub-partitions per SM.
FP64_LANES_PER_CLK_PER_SMSP = 0.5


def nominal_fp64_tflops(sm_count, sm_mhz):
    """DFMA-equivalent TFLOP/s of the FP64 pipe at the sampled SM clock."""
    if not sm_count or not sm_mhz:
        return None
    return 2 * FP64_LANES_PER_CLK_PER_SMSP * 4 * sm_count * sm_mhz * 1e6 / 1e12


def roofline_block(counts, pair_rate, alu_peak, fp64_probe, fp64_nominal, fp32_peak, fp64_equiv, kernel_ms):
    """Roofline of the FP64 pair kernel against the pipe that binds it.  The kernel
    issues fp64_inst_per_pair FP64 instructions and alu_inst_per_pair integer-ALU
    instructions per pair (ncu counts, size-independent, valid only while the
    kernel's sources hash to the recorded digest); each pipe's achieved rate is that
    count times the live pair rate.  The FP64 pipe's peak is its nominal issue rate
    at the sampled clock (0.5 lanes/clock/SMSP x 4 x SMs); the live DFMA probe
    (rgpu_probe_rate 0) sustains less and is reported beside it.  FP64 rates are
    DFMA-equivalent TFLOP/s (2 flops per pipe instruction).  The plain-FP64 view
    (20 flops per pair at the FP64 peak) rides alongside."""
    fp64_ipp, alu_ipp = counts.get("fp64_inst_per_pair"), counts.get("alu_inst_per_pair")
    traffic = counts.get("traffic_bytes_per_launch")
    pipes = {}
    fp64_peak = fp64_nominal or fp64_probe
    if fp64_ipp and fp64_peak:
        a = 2 * fp64_ipp * pair_rate / 1e12
        pipes["fp64"] = {"achieved": a, "peak": fp64_peak, "unit": "TFLOP/s (DFMA-equivalent)",
                         "frac": a / fp64_peak, "inst_per_pair": fp64_ipp,
                         "peak_source": ("nominal FP64 pipe rate at the sampled SM clock" if fp64_nominal else
                                         "live DFMA probe (no clock sample)"),
                         "probe_peak": fp64_probe, "frac_of_probe": a / fp64_probe if fp64_probe else None}
    if alu_ipp and alu_peak:
        a = alu_ipp * pair_rate / 1e12
        pipes["alu"] = {"achieved": a, "peak": alu_peak, "unit": "Tinst/s (integer ALU lane-ops)",
                        "frac": a / alu_peak, "inst_per_pair": alu_ipp,
                        "peak_source": "live integer-ALU probe (rgpu_probe_rate 4)"}
    plain = {"flops_per_pair": FLOPS_PER_PAIR, "equivalent_tflops": fp64_equiv, "fp64_peak_tflops": fp64_peak,
             "equivalent_over_peak": fp64_equiv / fp64_peak if fp64_peak else None,
             "fp64_probe_tflops": fp64_probe}
    kernel = "direct_kernel<BASIC> (int64 fixed-point pair, FP64 accumulate)"
    if not pipes:
        return {"bound": "fp64", "achieved": None, "peak": fp64_peak, "unit": "TFLOP/s", "frac": None,
                "traffic": traffic, "kernel": kernel, "kernel_ms": kernel_ms, "pair_rate_per_s": pair_rate,
                "counts": counts.get("stale", "missing"), "plain_fp64_view": plain, "fp32_peak_tflops": fp32_peak}
    bound = max(pipes, key=lambda k: pipes[k]["frac"])
    b = pipes[bound]
    return {"bound": bound, "achieved": b["achieved"], "peak": b["peak"], "unit": b["unit"], "frac": b["frac"],
            "traffic": traffic, "kernel": kernel, "kernel_ms": kernel_ms, "pair_rate_per_s": pair_rate,
            "pipes": pipes, "plain_fp64_view": plain, "fp32_peak_tflops": fp32_peak}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=3.0)
    ap.add_argument("--no-ensemble", dest="ensemble", action="store_false")
    ap.add_argument("--no-serve", dest="serve", action="store_false")
    ap.add_argument("--no-tree", dest="tree", action="store_false")
    ap.add_argument("--no-precision", dest="precision", action="store_false",
                    help="skip configuration 1 and the energy drift of every form (configurations 1, 2, 5)")
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--only", choices=["tree", "ensemble", "ensemble_full", "serve", "whfast_plain", "tree_patch"],
                    default=None, help="run one secondary workload alone and print its summary (also the small "
                                       "workloads the committed ncu summaries were captured on)")
    ap.add_argument("--patch", type=float, default=800.0, help="ring-patch box size (m) for --only tree_patch")
    ap.add_argument("--tree-gravity", default="tree", choices=["tree", "tree_split"],
                    help="gravity mode for --only tree_patch")
    ap.add_argument("--ens-systems", type=int, default=8192)
    ap.add_argument("--ens-steps", type=int, default=20)
    ap.add_argument("--ens-block", type=int, default=128)
    ap.add_argument("--ens-exact", type=int, default=0)
    ap.add_argument("--lite", action="store_true",
                    help="headline FP64 step only (no other forms, ensemble or serving), for profiling runs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.only == "tree":
            print(json.dumps({"tree": tree_summary(quick=args.quick)}), flush=True)
        elif args.only == "ensemble":
            print(json.dumps({"ensemble": ensemble_only(args)}), flush=True)
        elif args.only == "ensemble_full":
            from rebound_gb300 import ensemble as E
            print(json.dumps({"ensemble": E.bench_summary(quick=args.quick)}), flush=True)
        elif args.only == "whfast_plain":
            print(json.dumps({"whfast_plain": whfast_plain_summary(args.steps)}), flush=True)
        elif args.only == "tree_patch":
            print(json.dumps({"tree_patch": tree_patch_summary(args.patch, args.tree_gravity)}), flush=True)
        else:
            from rebound_gb300 import serve as S
            print(json.dumps({"serving": S.bench_summary(quick=args.quick)}), flush=True)
        return 0
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
