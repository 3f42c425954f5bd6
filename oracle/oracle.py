"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, never by the rebound_gb300 package.  The oracle
restates REBOUND 5.0.0's hot path (src/gravity.c, src/tree.c, src/collision.c,
src/boundary.c, src/integrator_{leapfrog,sei,whfast}.c, src/transformations.c,
src/tools.c) and is pinned against golden vectors of the unmodified reference.
"""
import ctypes
import math
import os
import subprocess
import sysconfig

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

# Same layout as struct reb_particle (src/rebound.h:86-104), 112 bytes.
PARTICLE_DTYPE = np.dtype([
    ("x", "f8"), ("y", "f8"), ("z", "f8"), ("vx", "f8"), ("vy", "f8"), ("vz", "f8"),
    ("ax", "f8"), ("ay", "f8"), ("az", "f8"), ("m", "f8"), ("r", "f8"),
    ("name", "u8"), ("ap", "u8"), ("sim", "u8")])
COLLISION_DTYPE = np.dtype([("p1", "u8"), ("p2", "u8"), ("gb", "f8", 6), ("ri", "u8")])
CELL_DTYPE = np.dtype([("root", "i4"), ("depth", "i4"), ("path", "u8"),
                       ("x", "f8"), ("y", "f8"), ("z", "f8"), ("w", "f8"),
                       ("m", "f8"), ("mx", "f8"), ("my", "f8"), ("mz", "f8"), ("pt", "i8")])
SIZE_MAX = 2**64 - 1


class OrcSim(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("t", "G", "softening", "dt", "OMEGA", "OMEGAZ", "root_size", "opening_angle2")] + [
        ("N", ctypes.c_size_t), ("N_active", ctypes.c_size_t),
        ("testparticle_type", ctypes.c_int), ("gravity_ignore_terms", ctypes.c_int),
        ("N_root_x", ctypes.c_int), ("N_root_y", ctypes.c_int), ("N_root_z", ctypes.c_int),
        ("N_ghost_x", ctypes.c_int), ("N_ghost_y", ctypes.c_int), ("N_ghost_z", ctypes.c_int),
        ("boundary", ctypes.c_int), ("whfast_safe_mode", ctypes.c_int),
        ("whfast_is_synchronized", ctypes.c_int), ("whfast_did_modify", ctypes.c_int),
        ("rand_seed", ctypes.c_uint), ("error", ctypes.c_int),
        ("particles", ctypes.c_void_p), ("p_jh", ctypes.c_void_p), ("cs", ctypes.c_void_p),
        ("sei_lastdt", ctypes.c_double), ("sei_sindt", ctypes.c_double), ("sei_tandt", ctypes.c_double),
        ("sei_sindtz", ctypes.c_double), ("sei_tandtz", ctypes.c_double),
        ("whfast_corrector", ctypes.c_int), ("whfast_corrector2", ctypes.c_int),
        ("whfast_kernel", ctypes.c_int), ("whfast_keep_unsynchronized", ctypes.c_int),
        ("tree_quadrupole", ctypes.c_int), ("whfast_coordinates", ctypes.c_int),
        ("whfast_gravity", ctypes.c_int), ("reserved0", ctypes.c_int)]


def _elf_matches_host(path):
    import platform
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    return head[:4] == b"\x7fELF" and want is not None and int.from_bytes(head[18:20], "little") == want


# Timing build: the compiler's default floating-point contraction (FMA where the
# target has it), as the reference's own OpenMP build is compiled.  Used only for
# the CPU-baseline timings; every parity check uses LIB (no contraction).
LIB_TIMING = os.path.join(HERE, "liboracle_timing.so")


def _build_one(out, contract_off, force):
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if not force and _elf_matches_host(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return out
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-std=gnu99", "-O3", "-fPIC", "-shared"] + (["-ffp-contract=off"] if contract_off else []) + [
        "-fopenmp", "-D_GNU_SOURCE", src, "-o", out + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build(force=False):
    """Compile oracle.c into liboracle.so (serial + OpenMP, no FP contraction: the
    parity build) and liboracle_timing.so (default contraction: the CPU-baseline build)."""
    _build_one(LIB_TIMING, False, force)
    return _build_one(LIB, True, force)


_lib = None
_lib_timing = None


def lib_timing():
    """The oracle compiled with default contraction, for CPU-baseline timing only."""
    global _lib_timing
    if _lib_timing is None:
        build()
        _lib_timing = _bind(ctypes.CDLL(LIB_TIMING))
    return _lib_timing


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = _bind(ctypes.CDLL(LIB))
    return _lib


def _bind(L):
    """Argument and result types of the oracle's entry points."""
    P = ctypes.POINTER(OrcSim)
    for name in ("orc_gravity_basic_serial", "orc_gravity_basic_omp", "orc_gravity_compensated_serial",
                 "orc_gravity_compensated_omp", "orc_gravity_tree", "orc_boundary_check",
                 "orc_whfast_step", "orc_whfast_synchronize"):
        getattr(L, name).argtypes = [P]
        getattr(L, name).restype = None
    L.orc_gravity_basic_omp_rows.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    L.orc_gravity_compensated_omp_rows.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    L.orc_gravity_tree_rows.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    L.orc_whfast_steps.argtypes = [P, ctypes.c_long]
    L.orc_whfast_steps.restype = None
    L.orc_leapfrog_step.argtypes = [P, ctypes.c_int]
    L.orc_leapfrog_step_order.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.orc_leapfrog_step_order.restype = ctypes.c_int
    L.orc_sei_step.argtypes = [P, ctypes.c_int]
    L.orc_collision_search_direct.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t]
    L.orc_collision_search_direct.restype = ctypes.c_size_t
    L.orc_collision_search_tree.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t]
    L.orc_collision_search_tree.restype = ctypes.c_size_t
    L.orc_collision_search_tree_omp.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t]
    L.orc_collision_search_tree_omp.restype = ctypes.c_size_t
    for name in ("orc_collision_search_line", "orc_collision_search_linetree"):
        getattr(L, name).argtypes = [P, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t]
        getattr(L, name).restype = ctypes.c_size_t
    L.orc_tree_export.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.orc_tree_export.restype = ctypes.c_int
    L.orc_energy.argtypes = [P]
    L.orc_energy.restype = ctypes.c_double
    L.orc_whfast_kepler_solver.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
    L.orc_ic_plummer.argtypes = [ctypes.c_uint, ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_void_p]
    L.orc_collision_resolve_hardsphere.argtypes = [P, ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
    return L


GRAVITY = {"none": 0, "basic": 1, "compensated": 2, "tree": 3, "basic_omp": 101, "compensated_omp": 102}
BOUNDARY = {"none": 0, "open": 1, "periodic": 2, "shear": 3}
WHFAST_KERNEL = {"default": 0, "modifiedkick": 1, "composition": 2, "lazy": 3}
WHFAST_COORDINATES = {"jacobi": 0, "democraticheliocentric": 1, "whds": 2, "barycentric": 3}


class Sim:
    """A reference-shaped simulation held in host memory and stepped by the oracle."""

    def __init__(self, particles, G=1.0, softening=0.0, dt=0.0, t=0.0, N_active=None,
                 testparticle_type=0, boundary="none", root_size=-1.0, N_root=(1, 1, 1),
                 N_ghost=(0, 0, 0), OMEGA=0.0, OMEGAZ=-1.0, opening_angle2=0.25, safe_mode=1,
                 corrector=0, corrector2=0, kernel=0, keep_unsynchronized=0, quadrupole=0,
                 coordinates="jacobi", whfast_gravity="basic"):
        self.p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE).copy()
        n = len(self.p)
        self.pj = np.zeros(n, dtype=PARTICLE_DTYPE)
        self.cs = np.zeros(3 * max(n, 1), dtype=np.float64)
        s = OrcSim()
        s.t, s.G, s.softening, s.dt = t, G, softening, dt
        s.OMEGA, s.OMEGAZ, s.root_size, s.opening_angle2 = OMEGA, OMEGAZ, root_size, opening_angle2
        s.N = n
        s.N_active = SIZE_MAX if N_active is None else N_active
        s.testparticle_type = testparticle_type
        s.N_root_x, s.N_root_y, s.N_root_z = N_root
        s.N_ghost_x, s.N_ghost_y, s.N_ghost_z = N_ghost
        s.boundary = BOUNDARY[boundary] if isinstance(boundary, str) else boundary
        s.whfast_safe_mode = safe_mode
        s.whfast_is_synchronized = 1
        s.whfast_did_modify = 1
        s.whfast_corrector, s.whfast_corrector2 = corrector, corrector2
        s.whfast_kernel = WHFAST_KERNEL[kernel] if isinstance(kernel, str) else kernel
        s.whfast_keep_unsynchronized = keep_unsynchronized
        s.tree_quadrupole = quadrupole
        s.whfast_coordinates = WHFAST_COORDINATES[coordinates] if isinstance(coordinates, str) else coordinates
        s.whfast_gravity = {"basic": 0, "compensated": 1, "none": 2}[whfast_gravity]
        s.particles = self.p.ctypes.data
        s.p_jh = self.pj.ctypes.data
        s.cs = self.cs.ctypes.data
        self.s = s

    @property
    def ref(self):
        return ctypes.byref(self.s)

    def acc(self):
        return np.stack([self.p["ax"], self.p["ay"], self.p["az"]], axis=1)

    def gravity(self, mode="basic"):
        L = lib()
        fn = {"basic": L.orc_gravity_basic_serial, "basic_omp": L.orc_gravity_basic_omp,
              "compensated": L.orc_gravity_compensated_serial,
              "compensated_omp": L.orc_gravity_compensated_omp, "tree": L.orc_gravity_tree}[mode]
        fn(self.ref)
        return self.acc()

    def leapfrog(self, steps, gravity="basic", order=2):
        for _ in range(steps):
            if lib().orc_leapfrog_step_order(self.ref, GRAVITY[gravity], order):
                raise ValueError("leapfrog order must be 2, 4, 6 or 8")

    def sei(self, steps, gravity="tree"):
        for _ in range(steps):
            lib().orc_sei_step(self.ref, GRAVITY[gravity])

    def whfast(self, steps):
        for _ in range(steps):
            lib().orc_whfast_step(self.ref)

    def whfast_synchronize(self):
        lib().orc_whfast_synchronize(self.ref)

    def whfast_integrate(self, tmax, exact_finish_time=1):
        """reb_simulation_integrate (src/simulation.c:372-464) with the exit test of
        reb_check_exit (:291-354), for WHFast."""
        s = self.s
        if tmax != s.t:
            s.dt = math.copysign(s.dt, 1.0 if tmax > s.t else -1.0)
        last_full_dt, dt_last_done, last_step = s.dt, 0.0, False
        while True:
            sign = math.copysign(1.0, s.dt)
            if exact_finish_time:
                if (s.t + s.dt) * sign >= tmax * sign:
                    if s.t == tmax:
                        break
                    if last_step:
                        tscale = 1e-12 * abs(tmax)
                        if tscale < 1e-200:
                            tscale = 1e-12
                        if abs(s.t - tmax) < tscale:
                            break
                        self.whfast_synchronize()
                        s.dt = tmax - s.t
                    else:
                        last_step = True
                        self.whfast_synchronize()
                        if dt_last_done != 0.0:
                            last_full_dt = dt_last_done
                        s.dt = tmax - s.t
                else:
                    last_step = False
            elif s.t * sign >= tmax * sign:
                break
            lib().orc_whfast_step(self.ref)
            dt_last_done = s.dt
        self.whfast_synchronize()
        if exact_finish_time:
            s.dt = last_full_dt

    def energy(self):
        return lib().orc_energy(self.ref)

    def collisions(self, mode="direct", cap=None, dt_last_done=0.0):
        """Pairs in discovery order; "line" / "linetree" test the paths over the last
        step of length dt_last_done."""
        L = lib()
        cap = cap or max(1024, 64 * len(self.p))
        out = np.zeros(cap, dtype=COLLISION_DTYPE)
        if mode in ("line", "linetree"):
            fn = L.orc_collision_search_line if mode == "line" else L.orc_collision_search_linetree
            n = fn(self.ref, float(dt_last_done), out.ctypes.data, cap)
        else:
            fn = {"direct": L.orc_collision_search_direct, "tree": L.orc_collision_search_tree,
                  "tree_omp": L.orc_collision_search_tree_omp}[mode]
            n = fn(self.ref, out.ctypes.data, cap)
        if n > cap:
            return self.collisions(mode, cap=int(n), dt_last_done=dt_last_done)
        return out[:n]

    def tree_cells(self):
        cap = 4 * len(self.p) + 16
        out = np.zeros(cap, dtype=CELL_DTYPE)
        n = ctypes.c_size_t(0)
        err = lib().orc_tree_export(self.ref, out.ctypes.data, cap, ctypes.byref(n))
        if err:
            raise RuntimeError(f"oracle tree build failed with code {err}")
        return out[:n.value]
