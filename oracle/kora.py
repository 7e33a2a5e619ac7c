"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
legs, always as the checker or the timed CPU baseline, never by the product
package.  The oracle restates the reference Kuramoto DP45 program
(znicolaou/kuramoto: kuramoto.cu, dp45.cu and their FP64 twins); see
``kora_core.hpp`` for the file:line of each piece.
"""
import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


class _Spec(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64), ("k", ctypes.c_int32), ("onthefly", ctypes.c_int32), ("seed", ctypes.c_int32),
        ("fp64", ctypes.c_int32),
        ("c1", ctypes.c_double), ("t0", ctypes.c_double), ("t1", ctypes.c_double), ("dt", ctypes.c_double),
        ("h0", ctypes.c_double), ("atol", ctypes.c_double), ("rtol", ctypes.c_double),
        ("fixed", ctypes.c_int32), ("dense", ctypes.c_int32), ("initial_record", ctypes.c_int32),
        ("threads", ctypes.c_int32), ("max_attempts", ctypes.c_int64),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(BUILD, "libkora.so")
        if not os.path.exists(path):
            from oracle import build_oracle
            build_oracle.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.kora_run.restype = ctypes.c_void_p
        L.kora_run.argtypes = [ctypes.POINTER(_Spec), dp, dp, dp]
        L.kora_result_size.restype = ctypes.c_int64
        L.kora_result_size.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.kora_result_copy.argtypes = [ctypes.c_void_p, ctypes.c_int32, dp]
        L.kora_result_scalars.argtypes = [ctypes.c_void_p, dp, dp, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]
        L.kora_result_free.argtypes = [ctypes.c_void_p]
        L.kora_rhs.argtypes = [ctypes.POINTER(_Spec), dp, dp, dp, dp, dp]
        L.kora_philox_stream_word.restype = ctypes.c_uint32
        L.kora_philox_stream_word.argtypes = [ctypes.c_int32, ctypes.c_uint64]
        L.kora_volcano_factor.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
        L.kora_volcano_adjacency_f32.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
        L.kora_volcano_adjacency_f64.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
        L.kora_host_random_inputs.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                              ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_void_p]
        L.kora_set_threads.argtypes = [ctypes.c_int32]
        L.kora_max_threads.restype = ctypes.c_int32
        L.kora_philox4x32_10.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.kora_model_create.restype = ctypes.c_void_p
        L.kora_model_create.argtypes = [ctypes.POINTER(_Spec), dp, dp]
        L.kora_model_run.restype = ctypes.c_void_p
        L.kora_model_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Spec), dp]
        L.kora_model_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, np.uint32); k = np.asarray(key, np.uint32); o = np.zeros(4, np.uint32)
    lib().kora_philox4x32_10(c.ctypes.data, k.ctypes.data, o.ctypes.data)
    return o


def volcano_factor(seed, n, k):
    u = np.zeros(k * n, np.int8)
    lib().kora_volcano_factor(seed, n, k, u.ctypes.data)
    return u.reshape(k, n)


def volcano_adjacency(seed, n, k, fp64=False):
    a = np.zeros((n, n), np.float64 if fp64 else np.float32)
    (lib().kora_volcano_adjacency_f64 if fp64 else lib().kora_volcano_adjacency_f32)(seed, n, k, a.ctypes.data)
    return a


def host_random_inputs(seed, n, init=0.0, freq=1.0, normal=False, gen_theta=True, gen_omega=True):
    th = np.zeros(n, np.float32); om = np.zeros(n, np.float32)
    lib().kora_host_random_inputs(seed, n, init, freq, int(normal), int(gen_theta), int(gen_omega),
                                  th.ctypes.data, om.ctypes.data)
    return th, om


def max_threads():
    return lib().kora_max_threads()


@dataclass
class Result:
    order: np.ndarray
    thetas: np.ndarray
    couplings: np.ndarray
    times: np.ndarray
    steph: np.ndarray
    final_theta: np.ndarray
    final_coupling: np.ndarray
    final_t: float
    final_h: float
    steps: int
    attempts: int
    status: int


def _spec(n, k, c1, onthefly, seed, fp64, t0, t1, dt, h0, atol, rtol, fixed, dense, initial_record, threads,
          max_attempts):
    s = _Spec()
    s.n, s.k, s.onthefly, s.seed, s.fp64 = n, k, int(onthefly), seed, int(fp64)
    s.c1, s.t0, s.t1, s.dt = c1, t0, t1, dt
    s.h0 = dt / 100 if h0 is None else h0
    s.atol, s.rtol = atol, rtol
    s.fixed, s.dense, s.initial_record, s.threads = int(fixed), dense, int(initial_record), threads
    s.max_attempts = -1 if max_attempts is None else max_attempts
    return s


def run(theta0, omega, *, k=5, c1=3.0, adj=None, onthefly=False, seed=1, fp64=True, t0=0.0, t1=100.0, dt=1.0,
        h0=None, atol=1e-6, rtol=0.0, fixed=False, dense=0, initial_record=True, threads=0, max_attempts=None):
    """One reference-semantics run.  ``adj`` (row-major N x N) overrides the volcano rule."""
    theta0 = np.ascontiguousarray(theta0, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    n = theta0.size
    a = None if adj is None else np.ascontiguousarray(adj, np.float64)
    s = _spec(n, k, c1, onthefly, seed, fp64, t0, t1, dt, h0, atol, rtol, fixed, dense, initial_record, threads,
              max_attempts)
    L = lib()
    return _result(L, L.kora_run(ctypes.byref(s), _dptr(theta0), _dptr(omega), _dptr(a)), n)


class Model:
    """A network kept between runs: its adjacency (dense, built once: 4 N^2 bytes in float for a
    large N) or rank-K factor, and its frequencies.  ``run`` integrates one trajectory from theta0
    with the given coupling constant and horizon, as ``run()`` above does."""

    def __init__(self, omega, *, k=5, adj=None, onthefly=False, seed=1, fp64=True, threads=0):
        omega = np.ascontiguousarray(omega, np.float64)
        self.n = omega.size
        a = None if adj is None else np.ascontiguousarray(adj, np.float64)
        self.base = dict(k=k, onthefly=onthefly, seed=seed, fp64=fp64, threads=threads)
        s = _spec(self.n, k, 0.0, onthefly, seed, fp64, 0.0, 1.0, 1.0, None, 1e-6, 0.0, False, 0, True, threads, None)
        self.h = lib().kora_model_create(ctypes.byref(s), _dptr(omega), _dptr(a))

    def run(self, theta0, *, c1=3.0, t0=0.0, t1=100.0, dt=1.0, h0=None, atol=1e-6, rtol=0.0, fixed=False, dense=0,
            initial_record=True, max_attempts=None):
        theta0 = np.ascontiguousarray(theta0, np.float64)
        b = self.base
        s = _spec(self.n, b["k"], c1, b["onthefly"], b["seed"], b["fp64"], t0, t1, dt, h0, atol, rtol, fixed, dense,
                  initial_record, b["threads"], max_attempts)
        L = lib()
        return _result(L, L.kora_model_run(self.h, ctypes.byref(s), _dptr(theta0)), self.n)

    def close(self):
        if getattr(self, "h", None):
            lib().kora_model_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _result(L, r, n):
    try:
        def get(which):
            m = L.kora_result_size(r, which)
            out = np.zeros(m, np.float64)
            if m:
                L.kora_result_copy(r, which, _dptr(out))
            return out
        ft = ctypes.c_double(); fh = ctypes.c_double(); st = ctypes.c_int64(); at = ctypes.c_int64()
        stat = ctypes.c_int32()
        L.kora_result_scalars(r, ctypes.byref(ft), ctypes.byref(fh), ctypes.byref(st), ctypes.byref(at),
                              ctypes.byref(stat))
        return Result(order=get(0), thetas=get(1).reshape(-1, n), couplings=get(2).reshape(-1, 2 * n),
                      times=get(3), steph=get(4), final_theta=get(5), final_coupling=get(6),
                      final_t=ft.value, final_h=fh.value, steps=st.value, attempts=at.value, status=stat.value)
    finally:
        L.kora_result_free(r)


def rhs(y, omega, *, k=5, c1=3.0, adj=None, onthefly=False, seed=1, fp64=True):
    """RHS dtheta/dt and the couplings [A cos, A sin] interleaved (kuramoto.cu:104-126)."""
    y = np.ascontiguousarray(y, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    n = y.size
    a = None if adj is None else np.ascontiguousarray(adj, np.float64)
    s = _spec(n, k, c1, onthefly, seed, fp64, 0, 1, 1, None, 1e-6, 0, 0, 0, 1, 0, None)
    f = np.zeros(n, np.float64); cp = np.zeros(2 * n, np.float64)
    lib().kora_rhs(ctypes.byref(s), _dptr(omega), _dptr(a), _dptr(y), _dptr(f), _dptr(cp))
    return f, cp


def cli_path(fp64=False):
    return os.path.join(BUILD, "kuramoto_oracle_64" if fp64 else "kuramoto_oracle")
