"""Seeded synthetic inputs with the reference benchmark configurations' shapes.

Thin wrappers over the host-side generators in librebound_gb300.so, which draw
with the reference's random-number conventions (glibc rand_r streams as in
src/tools.c:64-105).  Loading the library does not need a GPU.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import PARTICLE_DTYPE, check


def plummer(n, seed=11, M=1.0, R=1.0, rmax=10.0):
    """Plummer sphere of n equal masses M/n, truncated at r <= rmax (src/tools.c:463-502)."""
    out = np.zeros(n, dtype=PARTICLE_DTYPE)
    check(_lib.load().rgpu_ic_plummer(seed, n, M, R, rmax, out.ctypes.data, PARTICLE_DTYPE.itemsize))
    return out


RING_DEFAULTS = dict(OMEGA=1.3143527e-4, surface_density=400., particle_density=400., rmin=1., rmax=4.,
                     sigma_z=5., sigma_v=0.0005, Lz=20.)


def ring_patch(L, seed=7, **kw):
    """Shearing-sheet ring patch of L x L x 20 m (examples/shearing_sheet/problem.c shape)."""
    p = dict(RING_DEFAULTS, **kw)
    n = ctypes.c_size_t(0)
    L_ = _lib.load()
    args = (seed, L, L, p["Lz"], p["OMEGA"], p["surface_density"], p["particle_density"], p["rmin"],
            p["rmax"], p["sigma_z"], p["sigma_v"])
    check(L_.rgpu_ic_ring_patch(*args, None, PARTICLE_DTYPE.itemsize, 0, ctypes.byref(n)))
    out = np.zeros(n.value, dtype=PARTICLE_DTYPE)
    check(L_.rgpu_ic_ring_patch(*args, out.ctypes.data, PARTICLE_DTYPE.itemsize, n.value, ctypes.byref(n)))
    return out


def planetary_systems(n_systems, seed=3, kmin=2, kmax=10, G=1.0):
    """Star + k planets per system, k uniform in [kmin, kmax] (configuration-4 shape).

    Returns (list of particle arrays, array of inner periods)."""
    L_ = _lib.load()
    state = ctypes.c_uint(seed)
    rng = np.random.default_rng(seed)
    ks = rng.integers(kmin, kmax + 1, size=n_systems)
    systems, periods = [], np.zeros(n_systems)
    for s, k in enumerate(ks):
        out = np.zeros(int(k) + 1, dtype=PARTICLE_DTYPE)
        p = ctypes.c_double(0.)
        check(L_.rgpu_ic_planetary(ctypes.byref(state), int(k), G, 1e-7, 1e-3, 0.5, 30., 0.02, 0.01, 3.0,
                                   out.ctypes.data, PARTICLE_DTYPE.itemsize, ctypes.byref(p)))
        systems.append(out)
        periods[s] = p.value
    return systems, periods
