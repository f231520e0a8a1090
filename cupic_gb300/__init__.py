"""cupic_gb300: the per-step electrostatic PIC cycle of cupic on one GB300.

Python mirror of the C-ABI in include/cupic_gpu.h.  ``Sim`` exposes the
reference's host entry points under their own names (charge_deposition,
poisson_solver, field_solver, particle_mover, cc -- src/mesh.cu,
src/particles.cu, src/cc.cu of AntonioTejero/cupic) over the CUDA library
``_build/libcupic_gpu.so``.  There is no CPU fallback: when the library or a
GPU is missing, every call raises.
"""
import ctypes
import os

import numpy as np

from .params import Params, StepStats, workload_params

__all__ = ["Sim", "Params", "StepStats", "workload_params", "load_library", "library_path",
           "CupicError", "params_from_input_data", "SPECIES", "FLAGS", "EXPORTED",
           "write_particles_file", "read_particles_file", "write_mesh_file",
           "write_bookmarks_file", "write_bins_file", "rewrite_input_data", "driver_path",
           "Batch", "reserve"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

SPECIES = {"electrons": 0, "ions": 1}
FLAGS = {"cfl": 1, "capacity": 2, "stage": 4, "nonfinite": 8, "timeout": 16, "xrange": 32}

# every symbol declared in include/cupic_gpu.h
EXPORTED = [
    "cupic_params_default", "cupic_params_from_input_data", "cupic_params_finalize",
    "cupic_create", "cupic_destroy", "cupic_strerror", "cupic_init_plasma",
    "cupic_load_particles", "cupic_set_time", "cupic_get_time",
    "cupic_charge_deposition", "cupic_poisson_solver", "cupic_field_solver",
    "cupic_particle_mover", "cupic_cc", "cupic_step", "cupic_sync", "cupic_step_timed",
    "cupic_get_counts", "cupic_store_particles", "cupic_store_particles_f32",
    "cupic_get_bookmarks", "cupic_get_rho", "cupic_get_rho_fixed", "cupic_get_phi",
    "cupic_set_phi", "cupic_get_field", "cupic_get_phi_f32", "cupic_get_field_f32",
    "cupic_get_stats", "cupic_get_flags", "cupic_clear_flags", "cupic_poisson_solver_static",
    "cupic_init_mesh", "cupic_get_params", "cupic_get_solver_plan", "cupic_write_particles_file",
    "cupic_read_particles_file", "cupic_write_mesh_file", "cupic_write_bookmarks_file",
    "cupic_write_bins_file", "cupic_rewrite_input_data", "cupic_particles_snapshot",
    "cupic_mesh_snapshot", "cupic_save_bm", "cupic_save_bins", "cupic_load_particles_file",
    "cupic_batch_create", "cupic_batch_set", "cupic_batch_step", "cupic_batch_sync",
    "cupic_batch_plan", "cupic_batch_destroy", "cupic_probe_current", "cupic_density_profile",
    "cupic_test_bounded_wait", "cupic_init_plasma_nowait", "cupic_reserve",
]


class CupicError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} (status {status})")


def library_path():
    return os.path.join(_HERE, "_build", "libcupic_gpu.so")


def driver_path():
    """The drop-in program (the reference's main, src/main.cu:26-117)."""
    return os.path.join(_HERE, "_build", "cupic_run")


def load_library(build_if_missing=False):
    """Load libcupic_gpu.so (built by cupic_gb300/build.py)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run `python -m cupic_gb300.build`")
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    c_i, c_i32, c_i64, c_d = ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "cupic_params_default": [P(Params)],
        "cupic_params_from_input_data": [ctypes.c_char_p, P(Params)],
        "cupic_params_finalize": [P(Params)],
        "cupic_create": [P(Params), c_i, P(vp)],
        "cupic_destroy": [vp],
        "cupic_init_plasma": [vp],
        "cupic_init_plasma_nowait": [vp],
        "cupic_reserve": [c_i, ctypes.c_uint64, c_i32],
        "cupic_load_particles": [vp, c_i, P(c_d), c_i64],
        "cupic_set_time": [vp, c_i64, c_d, c_d, c_d],
        "cupic_get_time": [vp, P(c_i64), P(c_d), P(c_d), P(c_d)],
        "cupic_charge_deposition": [vp],
        "cupic_poisson_solver": [vp, c_d, c_i32, c_i32, c_i32],
        "cupic_field_solver": [vp],
        "cupic_particle_mover": [vp],
        "cupic_cc": [vp, c_d],
        "cupic_step": [vp, c_i32],
        "cupic_sync": [vp],
        "cupic_step_timed": [vp, c_i32, P(ctypes.c_float), c_i32, P(ctypes.c_float)],
        "cupic_get_counts": [vp, P(c_i64), P(c_i64)],
        "cupic_store_particles": [vp, c_i, P(c_d), c_i64, P(c_i64)],
        "cupic_store_particles_f32": [vp, c_i, P(ctypes.c_float), c_i64, P(c_i64)],
        "cupic_get_bookmarks": [vp, c_i, P(c_i32)],
        "cupic_get_rho": [vp, c_i, P(c_d)],
        "cupic_get_rho_fixed": [vp, c_i, P(c_i64)],
        "cupic_get_phi": [vp, P(c_d)],
        "cupic_set_phi": [vp, P(c_d)],
        "cupic_get_field": [vp, P(c_d), P(c_d)],
        "cupic_get_phi_f32": [vp, P(ctypes.c_float)],
        "cupic_get_field_f32": [vp, P(ctypes.c_float), P(ctypes.c_float)],
        "cupic_get_stats": [vp, P(StepStats), c_i32],
        "cupic_get_flags": [vp, P(ctypes.c_uint32)],
        "cupic_clear_flags": [vp],
        "cupic_poisson_solver_static": [P(Params), ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, c_d, c_i32, c_i32, c_i32,
                                        ctypes.c_void_p, P(c_i32), P(ctypes.c_float)],
        "cupic_init_mesh": [vp],
        "cupic_get_params": [vp, P(Params)],
        "cupic_get_solver_plan": [vp, P(c_i32), P(c_i32), P(c_i32)],
        "cupic_write_particles_file": [ctypes.c_char_p, P(c_d), c_i64, ctypes.c_char_p],
        "cupic_read_particles_file": [ctypes.c_char_p, P(c_d), c_i64, P(c_i64)],
        "cupic_write_mesh_file": [ctypes.c_char_p, P(c_d), c_i32, c_i32],
        "cupic_write_bookmarks_file": [ctypes.c_char_p, P(c_i32), c_i32],
        "cupic_write_bins_file": [ctypes.c_char_p, P(c_d), c_i64, c_d],
        "cupic_rewrite_input_data": [ctypes.c_char_p, c_i32],
        "cupic_particles_snapshot": [vp, c_i, ctypes.c_char_p],
        "cupic_mesh_snapshot": [vp, c_i, ctypes.c_char_p],
        "cupic_save_bm": [vp, c_i, ctypes.c_char_p],
        "cupic_save_bins": [vp, c_i, ctypes.c_char_p],
        "cupic_load_particles_file": [vp, c_i, ctypes.c_char_p],
        "cupic_batch_create": [c_i, P(vp)],
        "cupic_batch_set": [vp, P(vp), c_i32],
        "cupic_batch_step": [vp, c_i32],
        "cupic_batch_sync": [vp],
        "cupic_batch_plan": [vp, P(c_i32), P(c_i32), P(c_i32)],
        "cupic_batch_destroy": [vp],
        "cupic_probe_current": [vp, c_i32, P(c_d)],
        "cupic_density_profile": [vp, c_i, P(c_d)],
        "cupic_test_bounded_wait": [vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = c_i
    L.cupic_strerror.argtypes = [c_i]
    L.cupic_strerror.restype = ctypes.c_char_p
    _LIB = L
    return L


def strerror(status):
    try:
        return load_library().cupic_strerror(status).decode()
    except Exception:
        return "unknown"


def _ok(rc, what):
    if rc != 0:
        raise CupicError(rc, what)


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def write_particles_file(path, xyvv, header=None):
    """particles_snapshot's format (diagnostic.cu:76-79); `header` adds one
    "# ..." line first."""
    a = np.ascontiguousarray(xyvv, dtype=np.float64).reshape(-1, 4)
    _ok(load_library().cupic_write_particles_file(
        os.fsencode(path), _ptr(a, ctypes.c_double), a.shape[0],
        None if header is None else header.encode()), "write_particles_file")


def read_particles_file(path):
    """Every line holding four numbers, as an (n, 4) float64 array."""
    L = load_library()
    n = ctypes.c_int64()
    _ok(L.cupic_read_particles_file(os.fsencode(path), None, 0, ctypes.byref(n)),
        "read_particles_file")
    out = np.empty((max(n.value, 1), 4))
    got = ctypes.c_int64()
    _ok(L.cupic_read_particles_file(os.fsencode(path), _ptr(out, ctypes.c_double), n.value,
                                    ctypes.byref(got)), "read_particles_file")
    return out[:got.value]


def write_mesh_file(path, m):
    """mesh_snapshot's format (diagnostic.cu:118-125); m is (nny, nnx)."""
    a = np.ascontiguousarray(m, dtype=np.float64)
    _ok(load_library().cupic_write_mesh_file(os.fsencode(path), _ptr(a, ctypes.c_double),
                                             a.shape[1], a.shape[0]), "write_mesh_file")


def write_bookmarks_file(path, bm):
    a = np.ascontiguousarray(bm, dtype=np.int32).ravel()
    _ok(load_library().cupic_write_bookmarks_file(os.fsencode(path), _ptr(a, ctypes.c_int32),
                                                  a.size // 2), "write_bookmarks_file")


def write_bins_file(path, xyvv, ds):
    a = np.ascontiguousarray(xyvv, dtype=np.float64).reshape(-1, 4)
    _ok(load_library().cupic_write_bins_file(os.fsencode(path), _ptr(a, ctypes.c_double),
                                             a.shape[0], ds), "write_bins_file")


def rewrite_input_data(path, n_ini):
    """main.cu:98-113: line 1 of input_data becomes "n_ini = <n_ini>;"."""
    _ok(load_library().cupic_rewrite_input_data(os.fsencode(path), n_ini), "rewrite_input_data")


def reserve(nbytes, contexts=0, device=0):
    """Grows the device memory pool the contexts allocate from to at least
    nbytes and the kept streams to `contexts` contexts' worth (see
    cupic_reserve)."""
    _ok(load_library().cupic_reserve(device, int(nbytes), int(contexts)), "reserve")


def params_from_input_data(path):
    """Parse the reference's input_data file (init.cu:424-789)."""
    p = Params()
    _ok(load_library().cupic_params_from_input_data(os.fsencode(path), ctypes.byref(p)),
        "cupic_params_from_input_data")
    return p


class Sim:
    """One plasma slab on one GPU, driven through the C-ABI."""

    def __init__(self, params, device=0):
        self.L = load_library()
        self.p = params.copy()
        h = ctypes.c_void_p()
        _ok(self.L.cupic_create(ctypes.byref(self.p), device, ctypes.byref(h)), "cupic_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.cupic_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def nnodes(self):
        return self.p.nnx * self.p.nny

    # ---- setup ------------------------------------------------------------
    def init_plasma(self, wait=True):
        """init_sim (init.cu:57-83); wait=False only enqueues it on the
        context's stream (call sync() before reading results)."""
        if wait:
            _ok(self.L.cupic_init_plasma(self.h), "init_plasma")
        else:
            _ok(self.L.cupic_init_plasma_nowait(self.h), "init_plasma_nowait")

    def load(self, species, xyvv):
        a = np.ascontiguousarray(xyvv, dtype=np.float64).reshape(-1, 4)
        _ok(self.L.cupic_load_particles(self.h, species, _ptr(a, ctypes.c_double), a.shape[0]),
            "load_particles")

    def init_mesh(self):
        """initialize_mesh after a load (init.cu:84-93): linear phi, deposit,
        initial solve and field, clock at step n_ini+1."""
        _ok(self.L.cupic_init_mesh(self.h), "init_mesh")

    def solver_plan(self):
        """(CTAs, rows per CTA, halo depth) of the Jacobi solver."""
        g, b, k = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _ok(self.L.cupic_get_solver_plan(self.h, ctypes.byref(g), ctypes.byref(b), ctypes.byref(k)),
            "get_solver_plan")
        return g.value, b.value, k.value

    def load_file(self, species, path):
        _ok(self.L.cupic_load_particles_file(self.h, species, os.fsencode(path)),
            "load_particles_file")

    def set_time(self, step, t, tin_e=-1.0, tin_i=-1.0):
        _ok(self.L.cupic_set_time(self.h, step, t, tin_e, tin_i), "set_time")

    def get_time(self):
        s, t, a, b = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _ok(self.L.cupic_get_time(self.h, ctypes.byref(s), ctypes.byref(t), ctypes.byref(a),
                                  ctypes.byref(b)), "get_time")
        return s.value, t.value, a.value, b.value

    # ---- the cycle, by the reference's names --------------------------------
    def charge_deposition(self):
        _ok(self.L.cupic_charge_deposition(self.h), "charge_deposition")

    def poisson_solver(self, max_error=None, min_sweeps=None, max_sweeps=None, check_every=1):
        if max_error is None:
            _ok(self.L.cupic_poisson_solver(self.h, -1.0, 0, 0, 0), "poisson_solver")
            return
        mn = self.p.nnx if min_sweeps is None else min_sweeps
        mx = 1000000 if max_sweeps is None else max_sweeps
        _ok(self.L.cupic_poisson_solver(self.h, max_error, mn, mx, check_every), "poisson_solver")

    def field_solver(self):
        _ok(self.L.cupic_field_solver(self.h), "field_solver")

    def particle_mover(self):
        _ok(self.L.cupic_particle_mover(self.h), "particle_mover")

    def cc(self, t):
        _ok(self.L.cupic_cc(self.h, t), "cc")

    def step(self, n=1, sync=True):
        _ok(self.L.cupic_step(self.h, n), "step")
        if sync:
            self.sync()

    PHASES = ("solve", "zero", "push", "arrive", "inject", "final")

    def step_timed(self, n):
        """n cycles with device timing per phase: (total_ms, {phase: ms})."""
        ph = (ctypes.c_float * len(self.PHASES))()
        tot = ctypes.c_float()
        _ok(self.L.cupic_step_timed(self.h, n, ph, len(self.PHASES), ctypes.byref(tot)),
            "step_timed")
        return tot.value, dict(zip(self.PHASES, list(ph)))

    def sync(self):
        _ok(self.L.cupic_sync(self.h), "sync")

    # ---- results ------------------------------------------------------------
    def counts(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _ok(self.L.cupic_get_counts(self.h, ctypes.byref(a), ctypes.byref(b)), "get_counts")
        return a.value, b.value

    def particles(self, species, f32=False):
        n = self.counts()[species]
        got = ctypes.c_int64()
        if f32:
            out = np.empty((n, 4), dtype=np.float32)
            _ok(self.L.cupic_store_particles_f32(self.h, species, _ptr(out, ctypes.c_float), n,
                                                 ctypes.byref(got)), "store_particles_f32")
        else:
            out = np.empty((n, 4), dtype=np.float64)
            _ok(self.L.cupic_store_particles(self.h, species, _ptr(out, ctypes.c_double), n,
                                             ctypes.byref(got)), "store_particles")
        return out

    def bookmarks(self, species):
        out = np.empty(2 * self.p.ncy, dtype=np.int32)
        _ok(self.L.cupic_get_bookmarks(self.h, species, _ptr(out, ctypes.c_int32)), "bookmarks")
        return out

    def row_counts(self, species):
        bm = self.bookmarks(species).reshape(-1, 2)
        return np.where(bm[:, 0] >= 0, bm[:, 1] - bm[:, 0] + 1, 0).astype(np.int32)

    def rho(self, which=0):
        o = np.empty(self.nnodes)
        _ok(self.L.cupic_get_rho(self.h, which, _ptr(o, ctypes.c_double)), "get_rho")
        return o.reshape(self.p.nny, self.p.nnx)

    def rho_fixed(self, which=0):
        o = np.empty(self.nnodes, dtype=np.int64)
        _ok(self.L.cupic_get_rho_fixed(self.h, which, _ptr(o, ctypes.c_int64)), "get_rho_fixed")
        return o.reshape(self.p.nny, self.p.nnx)

    def phi(self):
        o = np.empty(self.nnodes, dtype=np.float32)
        _ok(self.L.cupic_get_phi_f32(self.h, _ptr(o, ctypes.c_float)), "get_phi")
        return o.reshape(self.p.nny, self.p.nnx)

    def phi64(self):
        """The potential as doubles: the FP64 potential of the precision form
        (refine_every > 0), else the FP32 one widened."""
        o = np.empty(self.nnodes)
        _ok(self.L.cupic_get_phi(self.h, _ptr(o, ctypes.c_double)), "get_phi")
        return o.reshape(self.p.nny, self.p.nnx)

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, dtype=np.float64).ravel()
        _ok(self.L.cupic_set_phi(self.h, _ptr(a, ctypes.c_double)), "set_phi")

    def efield(self):
        ex = np.empty(self.nnodes, dtype=np.float32)
        ey = np.empty(self.nnodes, dtype=np.float32)
        _ok(self.L.cupic_get_field_f32(self.h, _ptr(ex, ctypes.c_float), _ptr(ey, ctypes.c_float)),
            "get_field")
        return ex.reshape(self.p.nny, self.p.nnx), ey.reshape(self.p.nny, self.p.nnx)

    def stats(self, count=1):
        arr = (StepStats * count)()
        _ok(self.L.cupic_get_stats(self.h, arr, count), "get_stats")
        return [s.as_dict() for s in arr]

    def probe_current(self, window):
        """Net charge absorbed by the probe per step over the last `window` steps."""
        v = ctypes.c_double()
        _ok(self.L.cupic_probe_current(self.h, window, ctypes.byref(v)), "probe_current")
        return v.value

    def density_profile(self, species):
        """Particles per unit volume in each cell row (ncy values)."""
        o = np.empty(self.p.ncy)
        _ok(self.L.cupic_density_profile(self.h, species, _ptr(o, ctypes.c_double)),
            "density_profile")
        return o

    def flags(self):
        f = ctypes.c_uint32()
        _ok(self.L.cupic_get_flags(self.h, ctypes.byref(f)), "get_flags")
        return f.value

    def clear_flags(self):
        _ok(self.L.cupic_clear_flags(self.h), "clear_flags")

    # ---- the reference's files ---------------------------------------------
    MESH = {"rho": 0, "rho_last": 1, "phi": 2, "ex": 3, "ey": 4}

    def particles_snapshot(self, species, path):
        _ok(self.L.cupic_particles_snapshot(self.h, species, os.fsencode(path)),
            "particles_snapshot")

    def mesh_snapshot(self, what, path):
        w = self.MESH[what] if isinstance(what, str) else what
        _ok(self.L.cupic_mesh_snapshot(self.h, w, os.fsencode(path)), "mesh_snapshot")

    def save_bm(self, species, path):
        _ok(self.L.cupic_save_bm(self.h, species, os.fsencode(path)), "save_bm")

    def save_bins(self, species, path):
        _ok(self.L.cupic_save_bins(self.h, species, os.fsencode(path)), "save_bins")


class Batch:
    """Many contexts stepped together (cupic_batch_*): one launch per kernel
    for all members.  Step members only through the batch while they are
    members, and sync before reading them."""

    def __init__(self, sims=(), device=0):
        self.L = load_library()
        h = ctypes.c_void_p()
        _ok(self.L.cupic_batch_create(device, ctypes.byref(h)), "cupic_batch_create")
        self.h = h
        self.sims = []
        if sims:
            self.set(sims)

    def set(self, sims):
        sims = list(sims)
        arr = (ctypes.c_void_p * max(len(sims), 1))(*[s.h.value for s in sims])
        _ok(self.L.cupic_batch_set(self.h, arr, len(sims)), "batch_set")
        self.sims = sims

    def step(self, n=1, sync=True):
        _ok(self.L.cupic_batch_step(self.h, n), "batch_step")
        if sync:
            self.sync()

    def sync(self):
        _ok(self.L.cupic_batch_sync(self.h), "batch_sync")

    def plan(self):
        """The batched solve's layout: (halo depth cap, CTA multiple, CTAs)."""
        d, m, n = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _ok(self.L.cupic_batch_plan(self.h, ctypes.byref(d), ctypes.byref(m), ctypes.byref(n)),
            "batch_plan")
        return d.value, m.value, n.value

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.cupic_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
