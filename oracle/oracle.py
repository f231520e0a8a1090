"""ctypes binding of the CPU oracle (oracle/pic_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, never by the product package.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

from cupic_gb300.params import Params, StepStats

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib = None


def build(force=False):
    """Compile liboracle.so with the Makefile beside this file (again when
    the existing build came from another host architecture)."""
    stamp = os.path.join(_HERE, "build", ".arch")
    old = open(stamp).read().strip() if os.path.exists(stamp) else ""
    if old != platform.machine():
        force = True
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-C", _HERE, "-s", "-B"], check=True)
        with open(stamp, "w") as f:
            f.write(platform.machine())
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        L.ora_create.restype = vp
        L.ora_create.argtypes = [P(Params), ctypes.c_int]
        L.ora_destroy.argtypes = [vp]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        L.ora_params_from_input_data.argtypes = [ctypes.c_char_p, P(Params)]
        L.ora_params_default.argtypes = [P(Params)]
        for name in ("ora_init_plasma", "ora_deposit", "ora_field"):
            getattr(L, name).argtypes = [vp]
        L.ora_load.argtypes = [vp, ctypes.c_int, P(ctypes.c_double), ctypes.c_int64]
        L.ora_set_time.argtypes = [vp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double]
        L.ora_get_time.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_double),
                                   P(ctypes.c_double), P(ctypes.c_double)]
        L.ora_solve.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_int32, P(ctypes.c_int32), P(ctypes.c_double)]
        L.ora_push.argtypes = [vp, ctypes.c_int]
        L.ora_inject.argtypes = [vp, ctypes.c_double]
        L.ora_step.argtypes = [vp, ctypes.c_int32]
        L.ora_get_counts.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_int64)]
        L.ora_get_particles.argtypes = [vp, ctypes.c_int, P(ctypes.c_double)]
        L.ora_get_row_counts.argtypes = [vp, ctypes.c_int, P(ctypes.c_int32)]
        L.ora_gather.argtypes = [vp, ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double)]
        L.ora_get_phi.argtypes = [vp, P(ctypes.c_double)]
        L.ora_set_phi.argtypes = [vp, P(ctypes.c_double)]
        L.ora_get_field.argtypes = [vp, P(ctypes.c_double), P(ctypes.c_double)]
        L.ora_get_rho.argtypes = [vp, ctypes.c_int, P(ctypes.c_double)]
        L.ora_get_rho_fixed.argtypes = [vp, P(ctypes.c_int64)]
        L.ora_get_stats.argtypes = [vp, P(StepStats)]
        L.ora_get_flags.argtypes = [vp]
        L.ora_get_flags.restype = ctypes.c_uint32
        L.ora_philox4x32_10.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint32),
                                        P(ctypes.c_uint32)]
        L.ora_log.argtypes = [ctypes.c_double]
        L.ora_log.restype = ctypes.c_double
        L.ora_sincos2pi.argtypes = [ctypes.c_double, P(ctypes.c_double), P(ctypes.c_double)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def set_threads(n):
    lib().ora_set_threads(int(n))


def params_from_input_data(path):
    p = Params()
    _check(lib().ora_params_from_input_data(os.fsencode(path), ctypes.byref(p)), "parse")
    return p


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().ora_philox4x32_10(c, k, o)
    return list(o)


def olog(x):
    return lib().ora_log(float(x))


def osincos2pi(u):
    s, c = ctypes.c_double(), ctypes.c_double()
    lib().ora_sincos2pi(float(u), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


class Oracle:
    """One simulation instance of the oracle (fp64=True: precision oracle,
    fp64=False: bit-level model of the GPU kernels)."""

    def __init__(self, params, fp64=False):
        self.p = params.copy()
        self.fp64 = fp64
        self.L = lib()
        self.h = self.L.ora_create(ctypes.byref(self.p), 1 if fp64 else 0)
        if not self.h:
            raise ValueError("oracle rejected the parameters")

    def close(self):
        if self.h:
            self.L.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nnodes(self):
        return self.p.nnx * self.p.nny

    def init_plasma(self):
        _check(self.L.ora_init_plasma(self.h), "init")

    def load(self, species, xyvv):
        a = np.ascontiguousarray(xyvv, dtype=np.float64).reshape(-1, 4)
        _check(self.L.ora_load(self.h, species, _dp(a), a.shape[0]), "load")

    def set_time(self, step, t, tin_e=-1.0, tin_i=-1.0):
        _check(self.L.ora_set_time(self.h, step, t, tin_e, tin_i), "set_time")

    def get_time(self):
        s, t, a, b = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.L.ora_get_time(self.h, ctypes.byref(s), ctypes.byref(t), ctypes.byref(a),
                            ctypes.byref(b))
        return s.value, t.value, a.value, b.value

    def deposit(self):
        _check(self.L.ora_deposit(self.h), "deposit")

    def solve(self, tol, min_sweeps, max_sweeps, check_every=1):
        sw, res = ctypes.c_int32(), ctypes.c_double()
        _check(self.L.ora_solve(self.h, tol, min_sweeps, max_sweeps, check_every,
                                ctypes.byref(sw), ctypes.byref(res)), "solve")
        return sw.value, res.value

    def field(self):
        _check(self.L.ora_field(self.h), "field")

    def push(self, mode=0):
        _check(self.L.ora_push(self.h, mode), "push")

    def inject(self, t):
        _check(self.L.ora_inject(self.h, t), "inject")

    def step(self, n=1):
        _check(self.L.ora_step(self.h, n), "step")

    def counts(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self.L.ora_get_counts(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def particles(self, species):
        n = self.counts()[species]
        out = np.empty((n, 4), dtype=np.float64)
        if n:
            _check(self.L.ora_get_particles(self.h, species, _dp(out)), "particles")
        return out

    def gather(self, species):
        """E interpolated at every particle of a species (the push's CIC
        gather), in row order: (ex, ey)."""
        n = self.counts()[species]
        ex, ey = np.empty(n), np.empty(n)
        if n:
            _check(self.L.ora_gather(self.h, species, _dp(ex), _dp(ey)), "gather")
        return ex, ey

    def row_counts(self, species):
        out = np.empty(self.p.ncy, dtype=np.int32)
        self.L.ora_get_row_counts(self.h, species,
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return out

    def phi(self):
        o = np.empty(self.nnodes)
        self.L.ora_get_phi(self.h, _dp(o))
        return o.reshape(self.p.nny, self.p.nnx)

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, dtype=np.float64).ravel()
        self.L.ora_set_phi(self.h, _dp(a))

    def efield(self):
        ex, ey = np.empty(self.nnodes), np.empty(self.nnodes)
        self.L.ora_get_field(self.h, _dp(ex), _dp(ey))
        return ex.reshape(self.p.nny, self.p.nnx), ey.reshape(self.p.nny, self.p.nnx)

    def rho(self, which=0):
        o = np.empty(self.nnodes)
        self.L.ora_get_rho(self.h, which, _dp(o))
        return o.reshape(self.p.nny, self.p.nnx)

    def rho_fixed(self):
        o = np.empty(self.nnodes, dtype=np.int64)
        _check(self.L.ora_get_rho_fixed(self.h, o.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
               "rho_fixed")
        return o.reshape(self.p.nny, self.p.nnx)

    def stats(self):
        s = StepStats()
        self.L.ora_get_stats(self.h, ctypes.byref(s))
        return s.as_dict()

    def flags(self):
        return self.L.ora_get_flags(self.h)
