"""Host side of the GB300 engine: a ctypes binding of ``libsesp.so``.

It mirrors the reference driver's call surface (src/mybox.f90): the force
section (``force``), the velocity-Verlet halves (``move_a`` / ``move_b``, which
stand for move_surfactant_a + move_w1_a + move_w2_a and their ``_b``
counterparts), ``init_accel`` and ``temperature``, plus the step loop.  There
is no CPU fallback: constructing an :class:`Engine` without the compiled
library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsesp.so")

PLAIN_FP64 = 0
MIXED = 1          # FP32 force arithmetic, FP64 constraint iterations
MIXED_FP32C = 2    # MIXED with FP32 constraint iterations
MIXED_COMP = 3     # MIXED with compensated FP32 sums in the pair field
# warning bits of Engine.checks (sesp_check_flags)
CHECK_MOLECULES_LOST, CHECK_CHARGE, CHECK_OH_RATIO, CHECK_MISSING_OXYGEN = 1, 2, 4, 8
RESCALE_TARGET = 3.9   # target of the reference's temperature-rescaling variant

T_NEAR, T_FAR, T_VALENCE, T_DIHEDRAL, T_BERENDSEN = 1, 2, 4, 8, 16
T_INTERNAL, T_SUBTRACT, T_WALL, T_GRAPHITE = 32, 64, 128, 256
T_BOND = 512       # harmonic chain bonds (configuration preset)
T_ALL = 1023
PRESET_REFERENCE, PRESET_CONFIG = 0, 1

ERRORS = {1: "EINVAL", 2: "ECUDA", 3: "ENOMEM", 4: "ESTATE", 5: "ECAPACITY", 6: "ESHAKE", 7: "EBUDGET"}

# exported symbols of include/sesp.h
SYMBOLS = ["sesp_abi_version", "sesp_last_error", "sesp_default_params", "sesp_create", "sesp_destroy",
           "sesp_upload_state", "sesp_download_state", "sesp_set_state", "sesp_force", "sesp_force_terms",
           "sesp_download_forces", "sesp_init_accel", "sesp_move_a", "sesp_move_b", "sesp_step", "sesp_run",
           "sesp_run_async", "sesp_sync", "sesp_temperature", "sesp_get_eta", "sesp_set_eta", "sesp_energies",
           "sesp_counters", "sesp_kernel_times", "sesp_enable_timing", "sesp_run_timed", "sesp_pair_counts",
           "sesp_upload_batch", "sesp_replica_count", "sesp_get_eta_batch", "sesp_set_eta_batch", "sesp_failures_batch", "sesp_query", "sesp_device_bytes",
           "sesp_energies_static", "sesp_autotune", "sesp_tuning", "sesp_set_tuning", "sesp_checks",
           "sesp_check_flags", "sesp_rescale_temperature", "sesp_set_constraint_tuning", "sesp_constraint_tuning",
           "sesp_default_config_params", "sesp_fp32_peak"]


class SespError(RuntimeError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int * 3), ("precision", ctypes.c_int), ("rebuild_interval", ctypes.c_int),
                ("graphite_on", ctypes.c_int), ("tr", ctypes.c_double), ("tau_steps", ctypes.c_double),
                ("shake_tol", ctypes.c_double), ("shake_maxit", ctypes.c_int), ("device", ctypes.c_int),
                ("max_cell_sites", ctypes.c_int), ("preset", ctypes.c_int)]


_lib = None


def load(path: str = LIB_PATH):
    """Load the engine library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SespError(f"engine library not built: {path} (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    L.sesp_abi_version.restype = ctypes.c_int
    L.sesp_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.sesp_default_params.argtypes = [ctypes.POINTER(Params)]
    L.sesp_default_config_params.argtypes = [ctypes.POINTER(Params)]
    L.sesp_fp32_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    L.sesp_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(P)]
    L.sesp_destroy.argtypes = [P]
    L.sesp_upload_state.argtypes = [P, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, dp]
    L.sesp_download_state.argtypes = [P, dp, dp, dp]
    L.sesp_set_state.argtypes = [P, dp, dp, dp, ctypes.c_double]
    L.sesp_force.argtypes = [P, ctypes.c_int]
    L.sesp_force_terms.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.sesp_download_forces.argtypes = [P, dp]
    for n in ["sesp_init_accel", "sesp_move_a", "sesp_move_b", "sesp_sync"]:
        getattr(L, n).argtypes = [P]
    L.sesp_step.argtypes = [P, ctypes.c_int]
    L.sesp_run.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.sesp_run_async.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.sesp_temperature.argtypes = [P, dp]
    L.sesp_get_eta.argtypes = [P, dp]
    L.sesp_set_eta.argtypes = [P, ctypes.c_double]
    L.sesp_energies.argtypes = [P, dp]
    L.sesp_counters.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.sesp_kernel_times.argtypes = [P, dp, ctypes.c_int]
    L.sesp_enable_timing.argtypes = [P, ctypes.c_int]
    L.sesp_run_timed.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.sesp_pair_counts.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    ip = ctypes.POINTER(ctypes.c_int)
    L.sesp_upload_batch.argtypes = [P, ctypes.c_int, ip, ip, ip, dp, dp, ip, dp]
    L.sesp_replica_count.argtypes = [P]
    L.sesp_get_eta_batch.argtypes = [P, dp]
    L.sesp_set_eta_batch.argtypes = [P, dp]
    L.sesp_failures_batch.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.sesp_query.argtypes = [P]
    L.sesp_device_bytes.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.sesp_energies_static.argtypes = [P, dp]
    L.sesp_autotune.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    L.sesp_tuning.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    L.sesp_set_tuning.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.sesp_set_constraint_tuning.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.sesp_constraint_tuning.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    L.sesp_checks.argtypes = [P, dp]
    L.sesp_check_flags.argtypes = [dp]
    L.sesp_rescale_temperature.argtypes = [P, ctypes.c_double, dp]
    _lib = L
    return L


def fp32_peak(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device (TFLOP/s)."""
    v = ctypes.c_double()
    _check(load().sesp_fp32_peak(int(device), ctypes.byref(v)))
    return v.value


def check_flags(counts) -> int:
    """Warning bits of one replica's counts (first 7 values of a checks row);
    host code of the library, no GPU needed."""
    c = np.ascontiguousarray(counts, dtype=np.float64)[:7]
    if c.size != 7:
        raise ValueError("check_flags needs 7 counts")
    return int(load().sesp_check_flags(_dp(c)))


def _check(rc: int):
    if rc != 0:
        buf = ctypes.create_string_buffer(512)
        _lib.sesp_last_error(buf, 512)
        raise SespError(f"{ERRORS.get(rc, rc)}: {buf.value.decode(errors='replace')}")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_params(cells=(12, 12, 12), precision=PLAIN_FP64, preset=PRESET_REFERENCE, **kw) -> Params:
    """The engine's parameters for a force field (``preset``): the reference's
    settings, or the configuration preset's (300 K, 0.1 ps thermostat, SHAKE
    tolerance 1e-8); keywords override single fields."""
    L = load()
    p = Params()
    if preset == PRESET_CONFIG:
        _check(L.sesp_default_config_params(ctypes.byref(p)))
    else:
        _check(L.sesp_default_params(ctypes.byref(p)))
    for a in range(3):
        p.n_cells[a] = int(cells[a])
    p.precision = int(precision)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Engine:
    """One system on one GPU, driven through the C ABI."""

    def __init__(self, system, precision=PLAIN_FP64, device=0, **kw):
        L = load()
        if isinstance(system, (list, tuple)):
            self._init_batch(list(system), precision, device, **kw)
            return
        self.system = system
        p = default_params(system.cells, precision, preset=getattr(system, "preset", 0), device=device,
                           graphite_on=int(system.graphite_on), **kw)
        h = ctypes.c_void_p()
        _check(L.sesp_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        self.n = system.n_sites
        pos = np.ascontiguousarray(system.pos, dtype=np.float64)
        vel = np.ascontiguousarray(system.vel, dtype=np.float64)
        carb = np.ascontiguousarray(system.carbons, dtype=np.float64).reshape(-1, 3)
        nc = carb.shape[0]
        if nc == 0:
            carb = np.zeros((1, 3))
        _check(L.sesp_upload_state(self._h, system.n_water, system.n_surf, _dp(pos), _dp(vel), nc, _dp(carb)))

    def _init_batch(self, systems, precision, device, **kw):
        """Several replica systems advanced together by every launch."""
        L = _lib
        self.systems = systems
        self.system = systems[0]
        graphite = int(any(s.graphite_on for s in systems))
        presets = {getattr(s, "preset", 0) for s in systems}
        if len(presets) != 1:
            raise ValueError("replicas of one context share one force field (preset)")
        p = default_params(systems[0].cells, precision, preset=presets.pop(), device=device, graphite_on=graphite, **kw)
        h = ctypes.c_void_p()
        _check(L.sesp_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        nw = (ctypes.c_int * len(systems))(*[s.n_water for s in systems])
        ns = (ctypes.c_int * len(systems))(*[s.n_surf for s in systems])
        cells = (ctypes.c_int * (3 * len(systems)))(*[int(c) for s in systems for c in s.cells])
        ncarb = (ctypes.c_int * len(systems))(*[s.carbons.reshape(-1, 3).shape[0] for s in systems])
        pos = np.ascontiguousarray(np.concatenate([s.pos for s in systems]), dtype=np.float64)
        vel = np.ascontiguousarray(np.concatenate([s.vel for s in systems]), dtype=np.float64)
        carb = np.ascontiguousarray(np.concatenate([s.carbons.reshape(-1, 3) for s in systems] + [np.zeros((1, 3))]),
                                    dtype=np.float64)
        _check(L.sesp_upload_batch(self._h, len(systems), nw, ns, cells, _dp(pos), _dp(vel), ncarb, _dp(carb)))
        self.n = pos.shape[0]
        self.offsets = np.cumsum([0] + [s.n_sites for s in systems])

    def replica_count(self):
        return int(_lib.sesp_replica_count(self._h))

    def etas(self):
        out = np.empty(self.replica_count())
        _check(_lib.sesp_get_eta_batch(self._h, _dp(out)))
        return out

    def failures(self):
        """SHAKE / RATTLE non-convergences per replica since upload."""
        out = (ctypes.c_int64 * self.replica_count())()
        _check(_lib.sesp_failures_batch(self._h, out))
        return np.array(out[:], dtype=np.int64)

    def set_etas(self, etas):
        v = np.ascontiguousarray(etas, dtype=np.float64)
        if v.shape != (self.replica_count(),):
            raise ValueError("one eta per replica")
        _check(_lib.sesp_set_eta_batch(self._h, _dp(v)))

    def close(self):
        if getattr(self, "_h", None):
            _lib.sesp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference driver surface
    def force(self, rebuild=True, terms=T_ALL):
        _check(_lib.sesp_force_terms(self._h, int(rebuild), int(terms)))
        return self.forces()

    def forces(self):
        f = np.empty((self.n, 3))
        _check(_lib.sesp_download_forces(self._h, _dp(f)))
        return f

    def init_accel(self):
        _check(_lib.sesp_init_accel(self._h))

    def move_a(self):
        _check(_lib.sesp_move_a(self._h))

    def move_b(self):
        _check(_lib.sesp_move_b(self._h))

    def step(self, kb):
        _check(_lib.sesp_step(self._h, int(kb)))

    def run(self, kb0, nsteps):
        _check(_lib.sesp_run(self._h, int(kb0), int(nsteps)))

    def run_async(self, kb0, nsteps):
        _check(_lib.sesp_run_async(self._h, int(kb0), int(nsteps)))

    def sync(self):
        _check(_lib.sesp_sync(self._h))

    def busy(self) -> bool:
        """True while work launched on this context is still running (non-blocking)."""
        rc = _lib.sesp_query(self._h)
        if rc < 0:
            _check(-rc)
        return rc == 1

    def device_bytes(self) -> int:
        v = ctypes.c_int64()
        _check(_lib.sesp_device_bytes(self._h, ctypes.byref(v)))
        return v.value

    def state(self, out=None):
        """(pos, vel, acc) as (n, 3) float64 arrays; ``out``: three such
        C-contiguous arrays to fill instead (e.g. pinned host buffers)."""
        if out is None:
            pos, vel, acc = (np.empty((self.n, 3)) for _ in range(3))
        else:
            pos, vel, acc = out
            for a in out:
                if a.shape != (self.n, 3) or a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError("state(out=...) needs three C-contiguous (n, 3) float64 arrays")
        _check(_lib.sesp_download_state(self._h, _dp(pos), _dp(vel), _dp(acc)))
        return pos, vel, acc

    def set_state(self, pos=None, vel=None, acc=None, eta=0.0):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (pos, vel, acc)]
        ptrs = [None if a is None else _dp(a) for a in arrs]
        _check(_lib.sesp_set_state(self._h, *ptrs, float(eta)))

    def temperature(self):
        t = ctypes.c_double()
        _check(_lib.sesp_temperature(self._h, ctypes.byref(t)))
        return t.value

    @property
    def eta(self):
        v = ctypes.c_double()
        _check(_lib.sesp_get_eta(self._h, ctypes.byref(v)))
        return v.value

    @eta.setter
    def eta(self, v):
        _check(_lib.sesp_set_eta(self._h, float(v)))

    def energies(self):
        out = np.empty(8)
        _check(_lib.sesp_energies(self._h, _dp(out)))
        return out

    def autotune(self):
        """Pick the pair field's launch shape by timing the candidates on the
        current state (results do not depend on it); returns
        (tile, ctas_per_sm, largest ctas_per_sm)."""
        out = (ctypes.c_int * 3)()
        _check(_lib.sesp_autotune(self._h, out))
        return tuple(out)

    def tuning(self):
        out = (ctypes.c_int * 3)()
        _check(_lib.sesp_tuning(self._h, out))
        return tuple(out)

    def set_tuning(self, tile, ctas_per_sm):
        _check(_lib.sesp_set_tuning(self._h, int(tile), int(ctas_per_sm)))

    def constraint_tuning(self):
        """(surfactant warps per CTA, surfactants per warp, largest of each) of
        the mixed constraint halves."""
        out = (ctypes.c_int * 4)()
        _check(_lib.sesp_constraint_tuning(self._h, out))
        return tuple(out)

    def set_constraint_tuning(self, surf_warps, mols_per_warp=1):
        _check(_lib.sesp_set_constraint_tuning(self._h, int(surf_warps), int(mols_per_warp)))

    def checks(self):
        """The reference's consistency checks per replica (rows of 8): molecules
        located whole, molecules uploaded, total charge in the cells, water O
        and H in the cells, waters uploaded, sites in no cell, warning bits
        (CHECK_* constants)."""
        out = np.empty((self.replica_count(), 8))
        _check(_lib.sesp_checks(self._h, _dp(out)))
        return out

    def rescale_temperature(self, target=RESCALE_TARGET):
        """Scale the velocities to the temperature `target` (the reference's
        rescaling variant uses 3.9); returns the temperature before."""
        t = ctypes.c_double()
        _check(_lib.sesp_rescale_temperature(self._h, float(target), ctypes.byref(t)))
        return t.value

    def energies_static(self):
        """The same eight energies through sesp_energies_static: no device
        allocation, so a loop that shares the GPU with other runs can call it
        without the device-wide wait of cudaFree (at most 131,072 sites and
        4,096 surfactants per context)."""
        out = np.empty(8)
        _check(_lib.sesp_energies_static(self._h, _dp(out)))
        return out

    def counters(self):
        out = (ctypes.c_int64 * 8)()
        _check(_lib.sesp_counters(self._h, out))
        return list(out)

    def enable_timing(self, on=True):
        _check(_lib.sesp_enable_timing(self._h, int(on)))

    def run_timed(self, kb0, nsteps, flush_l2=True):
        """Per-step device times (ms) from CUDA events on the engine's stream."""
        out = np.empty(int(nsteps))
        _check(_lib.sesp_run_timed(self._h, int(kb0), int(nsteps), int(flush_l2), _dp(out)))
        return out

    def pair_counts(self):
        out = (ctypes.c_int64 * 2)()
        _check(_lib.sesp_pair_counts(self._h, out))
        return int(out[0]), int(out[1])

    def kernel_times(self, reset=False):
        out = np.empty(8)
        _check(_lib.sesp_kernel_times(self._h, _dp(out), int(reset)))
        return out


def mybox_start(engine: Engine):
    """Start-up force evaluation and accelerations (src/mybox.f90:65-128)."""
    engine.force(rebuild=True)
    engine.init_accel()


def mybox_loop(engine: Engine, kb0: int, nsteps: int):
    """The step loop src/mybox.f90:130-241 (rebuild every 10th kb)."""
    engine.run(kb0, nsteps)
