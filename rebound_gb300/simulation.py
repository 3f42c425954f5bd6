"""Host-side mirror of REBOUND's Simulation interface for the GPU hot path.

`rebound_gb300.Simulation` follows the reference's Python API
(rebound/simulation.py of REBOUND 5.0.0): modes are set by string
(`sim.gravity = "basic"`, `sim.integrator = "whfast"`, `sim.collision = "tree"`,
`sim.boundary = "shear"`), particles are added with `sim.add(...)`, and
`sim.integrate(tmax)` / `sim.steps(n)` advance the state.  Everything below
the attribute layer is one C-ABI call into librebound_gb300.so; particle state
lives on the GPU between calls and is copied back only when `particles` is
read (the synchronize-on-read protocol of the reference's WHFast, where the
device copy is authoritative between steps).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import PARTICLE_DTYPE, COLLISION_DTYPE, Config, check

_CFG_FLOATS = ("G", "softening", "dt", "t", "OMEGA", "OMEGAZ", "root_size", "opening_angle2",
               "coefficient_of_restitution", "minimum_collision_velocity")
_CFG_INTS = ("testparticle_type", "N_root_x", "N_root_y", "N_root_z", "N_ghost_x", "N_ghost_y",
             "N_ghost_z", "rand_seed", "gravity_ignore_terms", "leapfrog_order", "tree_quadrupole",
             "exact_finish_time")


_RESTITUTION_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_void_p, ctypes.c_double)


class Collision(Exception):
    """An integration stopped because two particles collided and collision_resolve
    is "halt" (rebound's Collision exception)."""


class WHFastSettings:
    """rebound's ri_whfast on the GPU path: safe_mode, coordinates, correctors, kernel,
    keep_unsynchronized (src/integrator_whfast.h:28-50)."""

    COORDINATES = {"jacobi": 0, "democraticheliocentric": 1, "whds": 2, "barycentric": 3}

    def __init__(self, sim):
        self._sim = sim

    @property
    def safe_mode(self):
        return self._sim._cfg.whfast_safe_mode

    @safe_mode.setter
    def safe_mode(self, v):
        self._sim._cfg.whfast_safe_mode = int(v)

    @property
    def coordinates(self):
        c = self._sim._cfg.whfast_coordinates
        return next(k for k, v in self.COORDINATES.items() if v == c)

    @coordinates.setter
    def coordinates(self, name):
        self._sim._cfg.whfast_coordinates = self.COORDINATES[name]

    # symplectic correctors and kernels (src/integrator_whfast.h:29-37)
    KERNELS = {"default": 0, "modifiedkick": 1, "composition": 2, "lazy": 3}

    @property
    def corrector(self):
        return self._sim._cfg.whfast_corrector

    @corrector.setter
    def corrector(self, order):
        self._sim._cfg.whfast_corrector = int(order)

    @property
    def corrector2(self):
        return self._sim._cfg.whfast_corrector2

    @corrector2.setter
    def corrector2(self, v):
        self._sim._cfg.whfast_corrector2 = int(v)

    @property
    def kernel(self):
        k = self._sim._cfg.whfast_kernel
        return next((n for n, v in self.KERNELS.items() if v == k), k)

    @kernel.setter
    def kernel(self, name):
        self._sim._cfg.whfast_kernel = self.KERNELS[name] if isinstance(name, str) else int(name)

    @property
    def keep_unsynchronized(self):
        return self._sim._cfg.whfast_keep_unsynchronized

    @keep_unsynchronized.setter
    def keep_unsynchronized(self, v):
        self._sim._cfg.whfast_keep_unsynchronized = int(v)


class Simulation:
    def __init__(self):
        self._L = _lib.load()
        h = ctypes.c_void_p()
        check(self._L.rgpu_sim_create(ctypes.byref(h)))
        self._h = h
        self._cfg = Config()
        self._L.rgpu_config_default(ctypes.byref(self._cfg))
        self._host = np.zeros(0, dtype=PARTICLE_DTYPE)
        self._host_dirty = False      # host particles changed since the last upload
        self._host_seen = None        # copy of the array handed out by `particles`
        self._device_newer = False    # device stepped since the last download
        self.ri_whfast = WHFastSettings(self)

    def __del__(self):
        try:
            if getattr(self, "_h", None) and self._h.value:
                self._L.rgpu_sim_free(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # ---- scalar settings ---------------------------------------------------
    def __getattr__(self, name):
        if name in _CFG_FLOATS or name in _CFG_INTS:
            return getattr(self.__dict__["_cfg"], name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name == "coefficient_of_restitution" and callable(value):
            # velocity-dependent restitution, called as value(sim, v) for each resolved
            # pair (rebound/simulation.py: sim.coefficient_of_restitution = f)
            cb = _RESTITUTION_FN(lambda _user, v: float(value(self, v)))
            object.__setattr__(self, "_eps_cb", cb)
            check(self._L.rgpu_sim_set_restitution_fn(self._h, ctypes.cast(cb, ctypes.c_void_p), None), self._h)
            return
        if name == "coefficient_of_restitution" and self.__dict__.get("_eps_cb") is not None:
            check(self._L.rgpu_sim_set_restitution_fn(self._h, None, None), self._h)
            object.__setattr__(self, "_eps_cb", None)
        if name in _CFG_FLOATS:
            setattr(self._cfg, name, float(value))
        elif name in _CFG_INTS:
            setattr(self._cfg, name, int(value))
        else:
            object.__setattr__(self, name, value)

    def _enum(field, table):
        def get(self):
            v = getattr(self._cfg, field)
            return next(k for k, x in table.items() if x == v)

        def set_(self, value):
            setattr(self._cfg, field, table[value.lower()] if isinstance(value, str) else int(value))
        return property(get, set_)

    gravity = _enum("gravity", _lib.GRAVITY)
    collision = _enum("collision", _lib.COLLISION)
    boundary = _enum("boundary", _lib.BOUNDARY)
    integrator = _enum("integrator", _lib.INTEGRATOR)
    collision_resolve = _enum("collision_resolve", _lib.RESOLVE)
    del _enum

    @property
    def N_active(self):
        v = self._cfg.N_active
        return self.N if v < 0 else v

    @N_active.setter
    def N_active(self, v):
        self._cfg.N_active = -1 if v is None else int(v)

    @property
    def status(self):
        return self._cfg.status

    @property
    def collisions_log_n(self):
        return self._cfg.collisions_log_n

    @property
    def collisions_plog(self):
        """Y-momentum transferred by hardsphere collisions (src/collision.c:655-662)."""
        return self._cfg.collisions_plog

    def resolve_time(self):
        """(host milliseconds spent resolving collisions, number of resolves)."""
        ms, n = ctypes.c_double(0.), ctypes.c_int64(0)
        check(self._L.rgpu_sim_resolve_time(self._h, ctypes.byref(ms), ctypes.byref(n)), self._h)
        return ms.value, n.value

    def configure_box(self, root_size, N_root_x=1, N_root_y=1, N_root_z=1):
        self._cfg.root_size = float(root_size)
        self._cfg.N_root_x, self._cfg.N_root_y, self._cfg.N_root_z = int(N_root_x), int(N_root_y), int(N_root_z)

    def configure_ghostboxes(self, N_ghost_x=0, N_ghost_y=0, N_ghost_z=0):
        self._cfg.N_ghost_x, self._cfg.N_ghost_y, self._cfg.N_ghost_z = int(N_ghost_x), int(N_ghost_y), int(N_ghost_z)

    # ---- particles ---------------------------------------------------------
    @property
    def N(self):
        return len(self._host)

    def add(self, particles=None, **kw):
        """Add one particle by keyword (m, r, x, y, z, vx, vy, vz) or an array of records."""
        self._pull()
        if particles is not None:
            arr = np.asarray(particles)
            if arr.dtype != PARTICLE_DTYPE:
                rec = np.zeros(len(arr), dtype=PARTICLE_DTYPE)
                for f in arr.dtype.names:
                    if f in PARTICLE_DTYPE.names:
                        rec[f] = arr[f]
                arr = rec
            self._host = np.concatenate([self._host, arr])
        else:
            rec = np.zeros(1, dtype=PARTICLE_DTYPE)
            for k, v in kw.items():
                rec[k] = v
            self._host = np.concatenate([self._host, rec])
        self._host_dirty = True

    @property
    def particles(self):
        """Host copy of the particle array (synchronized from the GPU).  Changes the
        caller makes to it are uploaded by the next call that runs on the GPU; a
        read alone leaves the integrator state as it is (as reading
        sim.particles does in the reference)."""
        self._pull()
        self._host_seen = self._host.copy()
        return self._host

    def set_particles_array(self, arr):
        self._host = np.ascontiguousarray(arr, dtype=PARTICLE_DTYPE).copy()
        self._host_dirty = True
        self._device_newer = False

    def _push(self):
        check(self._L.rgpu_sim_configure(self._h, ctypes.byref(self._cfg)), self._h)
        seen = self.__dict__.get("_host_seen")
        if seen is not None:
            if not self._host_dirty and (len(seen) != len(self._host) or
                                         not np.array_equal(seen.view(np.uint8), self._host.view(np.uint8))):
                self._host_dirty = True
            self._host_seen = None
        if self._host_dirty:
            check(self._L.rgpu_sim_set_particles(self._h, self._host.ctypes.data, len(self._host),
                                                 PARTICLE_DTYPE.itemsize), self._h)
            self._host_dirty = False

    def _pull(self):
        if self._device_newer:
            if self._cfg.integrator == _lib.INTEGRATOR["whfast"]:
                # A read shows synchronized values but leaves the integrator where it was,
                # as reading sim.particles does in the reference: with safe_mode 0 the
                # synchronize runs as keep_unsynchronized (src/integrator_whfast.c:1060-1104).
                dev = Config()
                check(self._L.rgpu_sim_get_config(self._h, ctypes.byref(dev)))
                if dev.whfast_safe_mode == 0 and not dev.whfast_keep_unsynchronized:
                    tmp = Config.from_buffer_copy(dev)
                    tmp.whfast_keep_unsynchronized = 1
                    check(self._L.rgpu_sim_configure(self._h, ctypes.byref(tmp)), self._h)
                    try:
                        check(self._L.rgpu_synchronize(self._h), self._h)
                    finally:
                        check(self._L.rgpu_sim_configure(self._h, ctypes.byref(dev)), self._h)
                else:
                    check(self._L.rgpu_synchronize(self._h), self._h)
            check(self._L.rgpu_sim_get_particles(self._h, self._host.ctypes.data, len(self._host),
                                                 PARTICLE_DTYPE.itemsize), self._h)
            self._device_newer = False

    def _after(self, rc):
        check(self._L.rgpu_sim_get_config(self._h, ctypes.byref(self._cfg)))
        self._device_newer = True
        check(rc, self._h)

    # ---- hot path ----------------------------------------------------------
    def update_acceleration(self):
        """reb_simulation_update_acceleration (src/simulation.c:640)."""
        self._push()
        self._after(self._L.rgpu_update_acceleration(self._h))

    def steps(self, n):
        """reb_simulation_steps (src/simulation.c:500)."""
        self._push()
        self._after(self._L.rgpu_steps(self._h, int(n)))

    def integrate(self, tmax, exact_finish_time=1):
        """reb_simulation_integrate (src/simulation.c:465); exact_finish_time as rebound's
        Simulation.integrate sets it (1: the last step is shortened to land on tmax)."""
        self._cfg.exact_finish_time = int(exact_finish_time)
        self._push()
        self._after(self._L.rgpu_integrate(self._h, float(tmax)))
        if self._cfg.status == 7:                # REB_STATUS_COLLISION (rebound/simulation.py:1324)
            raise Collision("Two particles collided (d < r1+r2)")

    def collision_search(self):
        """Pair list of the search half of reb_collision_search (src/collision.c:49)."""
        self._push()
        n = ctypes.c_size_t(0)
        cap = max(1024, 4 * self.N)
        while True:
            out = np.zeros(cap, dtype=COLLISION_DTYPE)
            rc = self._L.rgpu_collision_search(self._h, out.ctypes.data, cap, ctypes.byref(n))
            if rc == 9 and n.value > cap:
                cap = int(n.value)
                continue
            self._after(rc)
            return out[:n.value]

    def tree_cells(self):
        """Octree cells (depth-first) for the current positions."""
        self._push()
        n = ctypes.c_size_t(0)
        cap = 4 * self.N + 1024
        while True:
            out = np.zeros(cap, dtype=_lib.CELL_DTYPE)
            rc = self._L.rgpu_tree_export(self._h, out.ctypes.data, cap, ctypes.byref(n))
            if rc == 9 and n.value > cap:
                cap = int(n.value)
                continue
            check(rc, self._h)
            return out[:n.value]

    def energy(self):
        """reb_simulation_energy (src/tools.c:108)."""
        self._push()
        e = ctypes.c_double(0.)
        check(self._L.rgpu_energy(self._h, ctypes.byref(e)), self._h)
        return e.value

    def synchronize(self):
        self._push()
        self._after(self._L.rgpu_synchronize(self._h))

    def last_kernel_ms(self):
        return self._L.rgpu_sim_last_kernel_ms(self._h)

    def guard_stats(self):
        """(bodies off the fixed-point grid, particles recomputed in FP64) of the last
        BASIC / COMPENSATED fixed-point force evaluation; (-1, -1) before one."""
        a, b = ctypes.c_int64(0), ctypes.c_int64(0)
        check(self._L.rgpu_sim_guard_stats(self._h, ctypes.byref(a), ctypes.byref(b)), self._h)
        return a.value, b.value

    # ---- snapshots (Simulationarchive counterpart) --------------------------
    def save_to_file(self, filename, interval=None, step=None, delete_file=False):
        """rebound's Simulation.save_to_file (rebound/simulation.py:1166): one snapshot
        now, or automatic snapshots every `interval` of time / every `step` steps
        during later steps and integrations.  Snapshots keep the unsynchronized
        integrator state, so a run restarted from one continues bit for bit."""
        self._push()
        check(self._L.rgpu_sim_save_to_file(self._h, str(filename).encode(), float(interval or 0.),
                                            int(step or 0), int(bool(delete_file))), self._h)

    @classmethod
    def from_file(cls, filename, index=-1):
        """A new simulation restored from snapshot `index` of an archive file."""
        sim = cls()
        check(sim._L.rgpu_sim_load_from_file(sim._h, str(filename).encode(), int(index)), sim._h)
        check(sim._L.rgpu_sim_get_config(sim._h, ctypes.byref(sim._cfg)))
        sim._host = np.zeros(sim._L.rgpu_sim_N(sim._h), dtype=PARTICLE_DTYPE)
        sim._host_dirty = False
        sim._device_newer = True
        return sim

    @property
    def handle(self):
        self._push()
        return self._h


def accelerations(sim):
    p = sim.particles
    return np.stack([p["ax"], p["ay"], p["az"]], axis=1)


class Simulationarchive:
    """rebound's Simulationarchive (rebound/simulationarchive.py) over an archive
    written by Simulation.save_to_file: len(), indexing (a new Simulation per
    snapshot), tmin / tmax and getSimulation(t, mode)."""

    def __init__(self, filename):
        self.filename = str(filename)
        L = _lib.load()
        n = ctypes.c_size_t(0)
        rc = L.rgpu_archive_scan(self.filename.encode(), None, None, 0, ctypes.byref(n))
        if rc not in (0, 9):
            raise _lib.RGPUError(rc, "cannot read archive " + self.filename)
        self.t = np.zeros(n.value)
        self.offsets = np.zeros(n.value, dtype=np.int64)
        if n.value:
            check(L.rgpu_archive_scan(self.filename.encode(), self.t.ctypes.data, self.offsets.ctypes.data,
                                      n.value, ctypes.byref(n)))

    def __len__(self):
        return len(self.t)

    def __getitem__(self, key):
        if not isinstance(key, (int, np.integer)):
            raise AttributeError("Must access individual simulations with integer index.")
        if key < 0:
            key += len(self)
        if key >= len(self) or key < 0:
            raise IndexError("Index out of range, number of snapshots stored in binary: %d." % len(self))
        return Simulation.from_file(self.filename, int(key))

    @property
    def tmin(self):
        return float(self.t[0])

    @property
    def tmax(self):
        return float(self.t[-1])

    def _snapshot_index(self, t):
        """Index of the last snapshot at or before t (rebound/simulationarchive.py:159-177)."""
        if t > self.tmax or t < self.tmin:
            raise ValueError("Requested time outside of baseline stored in binary file.")
        lo, hi = 0, len(self)
        while True:
            bi = lo + (hi - lo) // 2
            if self.t[bi] > t:
                hi = bi
            else:
                lo = bi
            if hi - 1 <= lo:
                return lo

    def getSimulation(self, t, mode="snapshot", keep_unsynchronized=1):
        """rebound/simulationarchive.py:179-241: the snapshot before t, integrated to
        t ('exact'), past it by at most one step ('close'), or as stored ('snapshot')."""
        if mode not in ("snapshot", "close", "exact"):
            raise AttributeError("Unknown mode.")
        sim = self[self._snapshot_index(t)]
        if sim.integrator == "whfast":
            if sim.ri_whfast.safe_mode == 1 or mode == "exact":
                keep_unsynchronized = 0
            sim.ri_whfast.keep_unsynchronized = keep_unsynchronized
        if mode == "snapshot":
            sim.synchronize()
        elif mode == "close":
            sim.integrate(t, exact_finish_time=0)
        else:
            sim.integrate(t, exact_finish_time=1)
        return sim
