"""CPU oracle (test infrastructure only).

ctypes wrapper of ``liborc.so``, the plain-C FP64 restatement of the
reference's force-and-integrate path in this folder.  Only the tests, the
smoke check and the benchmark's CPU-baseline leg import this package.
Parity status: unpinned (the reference has no tests or golden vectors and
cannot be compiled here).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

TERM_NEAR, TERM_FAR, TERM_VALENCE, TERM_DIHEDRAL, TERM_BERENDSEN = 1, 2, 4, 8, 16
TERM_INTERNAL, TERM_SUBTRACT, TERM_WALL, TERM_GRAPHITE, TERM_ALL = 32, 64, 128, 256, 511
TERM_BOND = 512          # harmonic chain bonds (configuration preset)
TERM_ALL_CFG = 1023


def threads() -> int:
    """OpenMP threads the oracle's pair kernels and FMA passes use."""
    return int(lib().orc_threads())


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_int] * 5 + [dp, dp, ctypes.c_int, dp, ctypes.c_int]
        for name in ["orc_destroy", "orc_move_a_api", "orc_move_b_api", "orc_init_accel_api"]:
            getattr(L, name).argtypes = [P]
        L.orc_force.argtypes = [P, ctypes.c_int]
        L.orc_threads.restype = ctypes.c_int
        L.orc_force_terms.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_step.argtypes = [P, ctypes.c_int]
        L.orc_run.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_get.argtypes = [P, ctypes.c_int, dp]
        L.orc_set.argtypes = [P, ctypes.c_int, dp]
        L.orc_get_eta.restype = ctypes.c_double
        L.orc_get_eta.argtypes = [P]
        L.orc_set_eta.argtypes = [P, ctypes.c_double]
        L.orc_temperature_api.restype = ctypes.c_double
        L.orc_temperature_api.argtypes = [P]
        L.orc_fail_count.restype = ctypes.c_int
        L.orc_fail_count.argtypes = [P]
        L.orc_pair_counts.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        L.orc_get_key.argtypes = [P, ip, ip]
        L.orc_get_fma.argtypes = [P, ctypes.c_int, dp]
        L.orc_located.argtypes = [P, ip]
        L.orc_near_generic.argtypes = [P, dp, dp]
        L.orc_energies.argtypes = [P, dp]
        L.orc_constants.argtypes = [dp]
        # configuration preset (orc_cfg.c)
        L.ocf_create.restype = P
        L.ocf_create.argtypes = [ctypes.c_int] * 5 + [dp, dp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double,
                                                      ctypes.c_double, ctypes.c_double]
        for name in ["ocf_destroy", "ocf_move_a", "ocf_move_b", "ocf_init_accel"]:
            getattr(L, name).argtypes = [P]
        L.ocf_force_terms.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.ocf_step.argtypes = [P, ctypes.c_int]
        L.ocf_run.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.ocf_get.argtypes = [P, ctypes.c_int, dp]
        L.ocf_set.argtypes = [P, ctypes.c_int, dp]
        L.ocf_get_eta.restype = ctypes.c_double
        L.ocf_get_eta.argtypes = [P]
        L.ocf_set_eta.argtypes = [P, ctypes.c_double]
        L.ocf_temperature.restype = ctypes.c_double
        L.ocf_temperature.argtypes = [P]
        L.ocf_fail_count.restype = ctypes.c_int
        L.ocf_fail_count.argtypes = [P]
        L.ocf_pair_counts.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        L.ocf_energies.argtypes = [P, dp]
        L.ocf_direct_far.argtypes = [P, dp]
        L.ocf_graphite_layer.restype = ctypes.c_int
        L.ocf_graphite_layer.argtypes = [P]
        L.ocf_type_tables.argtypes = [dp, dp]
        L.orc_legendre.restype = ctypes.c_double
        L.orc_legendre.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One system in the oracle; mirrors the reference driver's call surface.
    A system of the configuration preset (``system.preset == 1``) gets a
    :class:`ConfigOracle` instead."""

    def __new__(cls, system, *a, **kw):
        if cls is Oracle and getattr(system, "preset", 0) == 1:
            return super().__new__(ConfigOracle)
        return super().__new__(cls)

    def __init__(self, system):
        L = lib()
        self.sys = system
        pos = np.ascontiguousarray(system.pos, dtype=np.float64)
        vel = np.ascontiguousarray(system.vel, dtype=np.float64)
        carb = np.ascontiguousarray(system.carbons, dtype=np.float64).reshape(-1, 3)
        if carb.size == 0:
            carb = np.zeros((1, 3))
            nc = 0
        else:
            nc = carb.shape[0]
        ncx, ncy, ncz = system.cells
        self._h = L.orc_create(system.n_water, system.n_surf, ncx, ncy, ncz, _dp(pos), _dp(vel), nc, _dp(carb),
                               int(system.graphite_on))
        if not self._h:
            raise ValueError("oracle rejected the system (cell counts must be positive multiples of 4)")
        self.n = system.n_sites

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def force(self, rebuild=True, terms=TERM_ALL):
        lib().orc_force_terms(self._h, int(rebuild), int(terms))
        return self.get(3)

    def move_a(self):
        lib().orc_move_a_api(self._h)

    def move_b(self):
        lib().orc_move_b_api(self._h)

    def init_accel(self):
        lib().orc_init_accel_api(self._h)

    def step(self, kb):
        lib().orc_step(self._h, int(kb))

    def run(self, kb0, nsteps):
        lib().orc_run(self._h, int(kb0), int(nsteps))

    def get(self, which):
        out = np.empty((self.n, 3))
        lib().orc_get(self._h, int(which), _dp(out))
        return out

    def set(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().orc_set(self._h, int(which), _dp(a))

    @property
    def eta(self):
        return lib().orc_get_eta(self._h)

    @eta.setter
    def eta(self, v):
        lib().orc_set_eta(self._h, float(v))

    def temperature(self):
        return lib().orc_temperature_api(self._h)

    def fail_count(self):
        return lib().orc_fail_count(self._h)

    def pair_counts(self):
        out = (ctypes.c_int64 * 2)()
        lib().orc_pair_counts(self._h, out)
        return int(out[0]), int(out[1])

    def keys(self):
        nm = self.sys.n_water + self.sys.n_surf
        key = np.empty(nm, dtype=np.int32)
        w1 = np.empty(nm, dtype=np.int32)
        lib().orc_get_key(self._h, key.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          w1.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return key, w1

    def located(self):
        loc = np.empty(self.n, dtype=np.int32)
        lib().orc_located(self._h, loc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return loc

    def fma(self, which):
        ncell = int(np.prod(self.sys.cells))
        out = np.empty((ncell, 25, 2))
        lib().orc_get_fma(self._h, int(which), _dp(out))
        return out[..., 0] + 1j * out[..., 1]

    def near_generic(self):
        f = np.empty((self.n, 3))
        e = np.empty(2)
        lib().orc_near_generic(self._h, _dp(f), _dp(e))
        return f, e

    def energies(self):
        out = np.empty(8)
        lib().orc_energies(self._h, _dp(out))
        return out


class ConfigOracle(Oracle):
    """A system of the configuration preset in the oracle (orc_cfg.c): the same
    call surface as :class:`Oracle`."""

    def __init__(self, system, tr=None, tau_steps=None, tol=None):
        from surfactant_enhanced_spreading_gb300 import config_preset as C
        L = lib()
        self.sys = system
        pos = np.ascontiguousarray(system.pos, dtype=np.float64)
        vel = np.ascontiguousarray(system.vel, dtype=np.float64)
        carb = np.ascontiguousarray(system.carbons, dtype=np.float64).reshape(-1, 3)
        nc = carb.shape[0]
        if nc == 0:
            carb = np.zeros((1, 3))
        ncx, ncy, ncz = system.cells
        self._h = L.ocf_create(system.n_water, system.n_surf, ncx, ncy, ncz, _dp(pos), _dp(vel), nc, _dp(carb),
                               int(system.graphite_on), float(C.TR if tr is None else tr),
                               float(C.TAU_STEPS if tau_steps is None else tau_steps),
                               float(C.SHAKE_TOL if tol is None else tol))
        if not self._h:
            raise ValueError("oracle rejected the system (cells: multiples of 4, at least 8 in x and y)")
        self.n = system.n_sites

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ocf_destroy(self._h)
            self._h = None

    def force(self, rebuild=True, terms=TERM_ALL_CFG):
        lib().ocf_force_terms(self._h, int(rebuild), int(terms))
        return self.get(3)

    def move_a(self):
        lib().ocf_move_a(self._h)

    def move_b(self):
        lib().ocf_move_b(self._h)

    def init_accel(self):
        lib().ocf_init_accel(self._h)

    def step(self, kb):
        lib().ocf_step(self._h, int(kb))

    def run(self, kb0, nsteps):
        lib().ocf_run(self._h, int(kb0), int(nsteps))

    def get(self, which):
        out = np.empty((self.n, 3))
        lib().ocf_get(self._h, int(which), _dp(out))
        return out

    def set(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().ocf_set(self._h, int(which), _dp(a))

    @property
    def eta(self):
        return lib().ocf_get_eta(self._h)

    @eta.setter
    def eta(self, v):
        lib().ocf_set_eta(self._h, float(v))

    def temperature(self):
        return lib().ocf_temperature(self._h)

    def fail_count(self):
        return lib().ocf_fail_count(self._h)

    def pair_counts(self):
        out = (ctypes.c_int64 * 2)()
        lib().ocf_pair_counts(self._h, out)
        return int(out[0]), int(out[1])

    def energies(self):
        out = np.empty(8)
        lib().ocf_energies(self._h, _dp(out))
        return out

    def direct_far(self):
        """Coulomb of the 3 x 3 image supercell minus the near field, by direct
        summation (what the far field plus its intramolecular correction
        approximates); O(N^2)."""
        out = np.empty((self.n, 3))
        lib().ocf_direct_far(self._h, _dp(out))
        return out

    def graphite_layer(self):
        return int(lib().ocf_graphite_layer(self._h))


def config_type_tables():
    """Charges and masses (reduced) of the configuration preset's 14 site kinds."""
    q, m = np.empty(14), np.empty(14)
    lib().ocf_type_tables(_dp(q), _dp(m))
    return q, m


def legendre(l, m, x):
    return float(lib().orc_legendre(int(l), int(m), float(x)))


def constants():
    out = np.empty(8)
    lib().orc_constants(_dp(out))
    return dict(sigma=out[0], epsilon=out[1], rc=out[2], rs=out[3], xpi=out[4], dt=out[5])
