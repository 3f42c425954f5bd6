"""Batched WHFast ensembles: many independent small planetary systems on one GPU.

Each system is what the reference runs as one `rebound.Simulation` with
`integrator = "whfast"` (Jacobi coordinates, DEFAULT kernel, safe_mode = 1,
src/integrator_whfast.c).  `Ensemble` packs them into the batched kernel of
librebound_gb300 (thread or warp per system, systems grouped by body count,
chunks of steps captured in CUDA graphs, autotuned mapping and launch shape).
"""
import ctypes
import time

import numpy as np

from . import _lib
from ._lib import PARTICLE_DTYPE, RGPUError


class Ensemble:
    """coordinates="democraticheliocentric" runs the WHFast512 splitting (always
    bit-exact: no FMA contraction)."""

    def __init__(self, systems, dts, G=1.0, exact=False, coordinates="jacobi"):
        if coordinates not in ("jacobi", "democraticheliocentric"):
            raise ValueError("coordinates: jacobi or democraticheliocentric")
        mode = 2 if coordinates == "democraticheliocentric" else int(bool(exact))
        self._L = _lib.load()
        self.sizes = np.array([len(s) for s in systems], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.records = np.ascontiguousarray(np.concatenate(systems).astype(PARTICLE_DTYPE))
        self.dts = np.ascontiguousarray(np.asarray(dts, dtype=np.float64))
        h = ctypes.c_void_p()
        rc = self._L.rgpu_ensemble_create(ctypes.byref(h), self.records.ctypes.data, PARTICLE_DTYPE.itemsize,
                                          self.offsets.ctypes.data, len(systems), self.dts.ctypes.data,
                                          float(G), mode)
        if rc:
            raise RGPUError(rc, "ensemble create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.rgpu_ensemble_free(self._h)
            self._h = ctypes.c_void_p()

    def _check(self, rc):
        if rc:
            raise RGPUError(rc, (self._L.rgpu_ensemble_last_error(self._h) or b"").decode())

    def set_launch(self, block=128, steps_per_launch=256):
        self._check(self._L.rgpu_ensemble_set_launch(self._h, block, steps_per_launch))

    MAPPINGS = {"thread": 0, "warp": 1}

    def set_mapping(self, mapping):
        """"thread": one thread per system (throughput); "warp": one warp per system (latency)."""
        self._check(self._L.rgpu_ensemble_set_mapping(self._h, self.MAPPINGS[mapping]))

    def launch(self):
        """(mapping, CTA size, steps per launch) in effect."""
        m, b, spl = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int64(0)
        self._check(self._L.rgpu_ensemble_get_launch(self._h, ctypes.byref(m), ctypes.byref(b), ctypes.byref(spl)))
        return {v: k for k, v in self.MAPPINGS.items()}[m.value], b.value, spl.value

    def autotune(self, probe_steps=16, max_steps_per_launch=512):
        """Time every mapping x CTA size, then the steps per launch, on this ensemble
        (advancing it) and keep the fastest; returns (CTA size, ms per step)."""
        b = ctypes.c_int(0)
        ms = ctypes.c_double(0)
        self._check(self._L.rgpu_ensemble_autotune(self._h, probe_steps, max_steps_per_launch,
                                                   ctypes.byref(b), ctypes.byref(ms)))
        return b.value, ms.value

    def steps(self, n):
        self._check(self._L.rgpu_ensemble_steps(self._h, int(n)))

    def time_steps(self, n):
        ms = ctypes.c_double(0)
        self._check(self._L.rgpu_ensemble_time_steps(self._h, int(n), ctypes.byref(ms)))
        return ms.value

    def particles(self):
        out = self.records.copy()
        self._check(self._L.rgpu_ensemble_get_particles(self._h, out.ctypes.data, PARTICLE_DTYPE.itemsize))
        return [out[a:b] for a, b in zip(self.offsets[:-1], self.offsets[1:])]

    def energies(self):
        e = np.zeros(len(self.sizes))
        self._check(self._L.rgpu_ensemble_energy(self._h, e.ctypes.data))
        return e

    def times(self):
        t = np.zeros(len(self.sizes))
        self._check(self._L.rgpu_ensemble_times(self._h, t.ctypes.data))
        return t


def energy_host(p, G=1.0):
    """Energy of one system on the host (src/tools.c:108-162), for initial values."""
    ek = 0.5 * np.sum(p["m"] * (p["vx"] ** 2 + p["vy"] ** 2 + p["vz"] ** 2))
    ep = 0.0
    for i in range(len(p)):
        for j in range(i + 1, len(p)):
            d = np.sqrt((p["x"][i] - p["x"][j]) ** 2 + (p["y"][i] - p["y"][j]) ** 2 + (p["z"][i] - p["z"][j]) ** 2)
            ep -= G * p["m"][j] * p["m"][i] / d
    return ek + ep


def plain_path_rate(systems, dts, steps, G=1.0):
    """System-steps/s of the plain path: one rgpu_sim per system, one C-ABI call
    (one kernel launch) per step, as a REBOUND integrator plugin drives it."""
    from .simulation import Simulation
    L = _lib.load()
    total_steps = 0
    t0 = time.perf_counter()
    energies = []
    for p, dt in zip(systems, dts):
        sim = Simulation()
        sim.G = G
        sim.dt = dt
        sim.gravity = "basic"
        sim.integrator = "whfast"
        sim.add(p)
        h = sim.handle
        for _ in range(steps):
            rc = L.rgpu_steps(h, 1)
            if rc:
                raise RGPUError(rc, "plain whfast step")
        total_steps += steps
        energies.append(sim.energy())
    el = time.perf_counter() - t0
    return total_steps / el, np.array(energies)


def bench_summary(quick=False, n_systems=65536, steps=10000, seed=3):
    """Configuration-4 ensemble: 65,536 systems, k in [2,10], dt = P_inner/20,
    10^4 steps; compared with the plain per-simulation GPU path and reported with
    the energy-error distribution."""
    from . import ics
    if quick:
        n_systems, steps = 4096, 500
    systems, periods = ics.planetary_systems(n_systems, seed=seed)
    dts = periods / 20.0
    e0 = np.array([energy_host(p) for p in systems[:512]])
    # Autotune (mapping, CTA size, steps per launch) on a scratch copy of the same
    # systems (its probe steps advance the state), then run the tuned shape.
    scratch = Ensemble(systems, dts)
    scratch.autotune(probe_steps=8, max_steps_per_launch=500)
    mapping, block, spl = scratch.launch()
    del scratch
    ens = Ensemble(systems, dts)
    ens.set_mapping(mapping)
    ens.set_launch(block, spl)
    ms = ens.time_steps(steps)
    rate = n_systems * steps / (ms * 1e-3)
    e1 = ens.energies()[:512]
    rel = np.abs((e1 - e0) / e0)
    # Plain path on a sample of systems, and the energy error of both paths on
    # that sample after the same number of steps (the batched run repeated for
    # the sample alone, so both start from the same state).
    sample = min(32, n_systems)
    plain_steps = 500 if not quick else 50
    plain_rate, e_plain = plain_path_rate(systems[:sample], dts[:sample], plain_steps)
    e0s = e0[:sample]
    small = Ensemble(systems[:sample], dts[:sample])
    small.set_mapping(mapping)
    small.set_launch(block, spl)
    small.steps(plain_steps)
    rel_plain = np.abs((e_plain - e0s) / e0s)
    rel_batched = np.abs((small.energies() - e0s) / e0s)
    return {"systems": n_systems, "steps": steps, "k_range": [2, 10], "mapping": mapping, "block": block,
            "steps_per_launch": spl, "launch_chosen_by": "rgpu_ensemble_autotune",
            "system_steps_per_s": rate, "seconds": ms * 1e-3,
            "energy_rel_err_median": float(np.median(rel)), "energy_rel_err_p99": float(np.quantile(rel, 0.99)),
            "energy_sample": int(len(rel)),
            "plain_path_system_steps_per_s": plain_rate,
            "plain_path_sample": f"{sample} systems x {plain_steps} steps, one C-ABI call per step",
            "matching_energy_error": {"systems": sample, "steps": plain_steps,
                                      "plain_median": float(np.median(rel_plain)),
                                      "plain_max": float(rel_plain.max()),
                                      "batched_median": float(np.median(rel_batched)),
                                      "batched_max": float(rel_batched.max())},
            "speedup_vs_plain": rate / plain_rate}
