"""ctypes binding of libkura (include/kura.h).

``Network`` wraps one handle: a network (oscillators, frequencies, dense or
regenerated volcano adjacency) and a batch of trajectories integrated together
by the persistent DP45 kernel.  Method names follow the C entry points; each
C entry point cites the reference code it replaces.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(PKG, "_build")

COUPLING_DENSE = 0
COUPLING_VOLCANO = 1
ENGINE_AUTO = 0
ENGINE_PERSISTENT = 1
ENGINE_TENSOR = 2
ADJ_F32 = 0
ADJ_I8 = 1

ERRORS = {
    -1: "KURA_ERR_INVALID", -2: "KURA_ERR_CUDA", -3: "KURA_ERR_NOMEM", -4: "KURA_ERR_BARRIER_TIMEOUT",
    -5: "KURA_ERR_STEP_UNDERFLOW", -6: "KURA_ERR_NONFINITE", -7: "KURA_ERR_UNSUPPORTED", -8: "KURA_ERR_CALLBACK",
}


class KuraError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64), ("k", ctypes.c_int32), ("coupling", ctypes.c_int32), ("batch", ctypes.c_int32),
        ("seed", ctypes.c_int32), ("atol", ctypes.c_double), ("rtol", ctypes.c_double),
        ("fixed_step", ctypes.c_int32), ("device", ctypes.c_int32), ("dense_level", ctypes.c_int32),
        ("engine", ctypes.c_int32), ("stream", ctypes.c_void_p), ("adj_storage", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("accepted", ctypes.c_int64), ("rejected", ctypes.c_int64), ("launches", ctypes.c_int64),
        ("barriers", ctypes.c_int64), ("kernel_ms", ctypes.c_double), ("grid", ctypes.c_int32),
        ("block", ctypes.c_int32), ("coupling_ms", ctypes.c_double), ("coupling_launches", ctypes.c_int64),
    ]


class Instance(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("k", ctypes.c_int32), ("seed", ctypes.c_int32), ("c", ctypes.c_float),
                ("reserved", ctypes.c_int32)]


class MultiStats(ctypes.Structure):
    _fields_ = [
        ("kernel_ms", ctypes.c_double), ("osc_steps", ctypes.c_double), ("tune_ms", ctypes.c_double),
        ("accepted", ctypes.c_int64), ("rejected", ctypes.c_int64), ("cluster_size", ctypes.c_int32),
        ("block_threads", ctypes.c_int32), ("grid", ctypes.c_int32), ("heavy", ctypes.c_int32),
    ]


STEP_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                           ctypes.c_int64)
OUTPUT_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                             ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float))
CHUNK_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                            ctypes.POINTER(ctypes.c_float))


class Callbacks(ctypes.Structure):
    _fields_ = [("user", ctypes.c_void_p), ("on_step", STEP_CB), ("on_output", OUTPUT_CB), ("on_chunk", CHUNK_CB)]


_lib = None


def lib_path():
    return os.path.join(BUILD, "libkura.so")


def cli_path():
    return os.path.join(BUILD, "kuramoto")


def lib():
    """Load libkura.so; raises if it has not been built (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError("libkura.so is not built (run __graft_entry__.build()): %s" % path)
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    fp = ctypes.POINTER(ctypes.c_float)
    i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "kura_create": (i32, [ctypes.POINTER(Config), ctypes.POINTER(P)]),
        "kura_destroy": (None, [P]),
        "kura_last_error": (ctypes.c_char_p, []),
        "kura_memory_required": (i32, [ctypes.POINTER(Config), ctypes.POINTER(i64)]),
        "kura_set_frequencies": (i32, [P, fp, i64]),
        "kura_set_adjacency": (i32, [P, fp, i64]),
        "kura_generate_adjacency": (i32, [P]),
        "kura_get_adjacency": (i32, [P, fp, i64]),
        "kura_set_coupling": (i32, [P, i32, ctypes.c_float]),
        "kura_set_state": (i32, [P, i32, fp, f64, f64]),
        "kura_set_state_device": (i32, [P, i32, P, f64, f64]),
        "kura_set_horizon": (i32, [P, f64, f64, i32]),
        "kura_run": (i32, [P, ctypes.POINTER(Callbacks)]),
        "kura_advance": (i32, [P, ctypes.POINTER(Callbacks), i64, ctypes.POINTER(i32)]),
        "kura_get_state": (i32, [P, i32, fp, ctypes.POINTER(f64), ctypes.POINTER(f64)]),
        "kura_get_order": (i32, [P, i32, fp, i64, ctypes.POINTER(i64)]),
        "kura_final_record": (i32, [P, i32, fp, fp, ctypes.POINTER(f64), ctypes.POINTER(f64)]),
        "kura_rhs": (i32, [P, i32, fp, fp, fp]),
        "kura_get_stats": (i32, [P, ctypes.POINTER(Stats)]),
        "kura_set_launch_attempts": (i32, [P, i64]),
        "kura_random_inputs": (i32, [i32, i64, ctypes.c_float, ctypes.c_float, i32, i32, i32, fp, fp]),
        "kura_volcano_factor": (i32, [i32, i64, i32, ctypes.c_void_p]),
        "kura_multi_create": (i32, [ctypes.POINTER(Instance), i32, f64, f64, f64, f64, f64, i32, i32, i32,
                                    ctypes.POINTER(P)]),
        "kura_multi_destroy": (None, [P]),
        "kura_multi_integrate": (i32, [P, fp, fp, fp, fp, ctypes.POINTER(i64)]),
        "kura_multi_get_stats": (i32, [P, ctypes.POINTER(MultiStats)]),
        "kura_mlp_create": (i32, [i32, i32, i32, i32, ctypes.c_uint64, i32, ctypes.POINTER(P)]),
        "kura_mlp_destroy": (None, [P]),
        "kura_mlp_param_count": (i32, [P, ctypes.POINTER(i64)]),
        "kura_mlp_get_params": (i32, [P, fp, i64]),
        "kura_mlp_set_params": (i32, [P, fp, i64]),
        "kura_mlp_forward": (i32, [P, fp, i64, fp]),
        "kura_mlp_gradients": (i32, [P, fp, fp, i64, fp, fp]),
        "kura_mlp_train": (i32, [P, fp, fp, i64, i32, ctypes.c_float, ctypes.c_float, ctypes.c_uint64, fp,
                                 ctypes.POINTER(f64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise KuraError(rc, lib().kura_last_error().decode(errors="replace"))


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def random_inputs(seed, n, init=0.0, freq=1.0, normal=False, gen_theta=True, gen_omega=True):
    """theta0 and omega from glibc rand() as the reference draws them (kuramoto.cu:416, 495-541)."""
    th = np.zeros(n, np.float32)
    om = np.zeros(n, np.float32)
    _check(lib().kura_random_inputs(seed, n, init, freq, int(normal), int(gen_theta), int(gen_omega), _fptr(th),
                                    _fptr(om)))
    return th, om


def volcano_factor(seed, n, k):
    """+/-1 volcano factor u[m, i] from the device Philox stream (kuramoto.cu:62-101, 128-135)."""
    u = np.zeros((k, n), np.int8)
    _check(lib().kura_volcano_factor(seed, n, k, u.ctypes.data))
    return u


class Network:
    def __init__(self, n, k=6, coupling=COUPLING_DENSE, batch=1, seed=1, atol=1e-6, rtol=0.0, fixed_step=False,
                 device=0, dense_level=0, stream=None, engine=0, adj_storage=ADJ_F32):
        c = Config()
        c.n, c.k, c.coupling, c.batch, c.seed, c.engine = n, k, coupling, batch, seed, engine
        c.adj_storage = adj_storage
        c.atol, c.rtol, c.fixed_step, c.device, c.dense_level = atol, rtol, int(fixed_step), device, dense_level
        c.stream = stream
        self.cfg = c
        self.n = n
        self.batch = batch
        self.dense_level = dense_level
        h = ctypes.c_void_p()
        _check(lib().kura_create(ctypes.byref(c), ctypes.byref(h)))
        self.h = h

    @staticmethod
    def memory_required(n, k=6, coupling=COUPLING_DENSE, batch=1, dense_level=0, engine=0, adj_storage=ADJ_F32):
        c = Config()
        c.n, c.k, c.coupling, c.batch, c.atol, c.dense_level, c.engine = n, k, coupling, batch, 1e-6, dense_level, engine
        c.adj_storage = adj_storage
        b = ctypes.c_int64()
        _check(lib().kura_memory_required(ctypes.byref(c), ctypes.byref(b)))
        return b.value

    def close(self):
        if getattr(self, "h", None):
            lib().kura_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_frequencies(self, omega):
        om = np.ascontiguousarray(omega, np.float32)
        _check(lib().kura_set_frequencies(self.h, _fptr(om), om.size))

    def set_adjacency(self, adj):
        a = np.ascontiguousarray(adj, np.float32)
        _check(lib().kura_set_adjacency(self.h, _fptr(a), self.n))

    def generate_adjacency(self):
        _check(lib().kura_generate_adjacency(self.h))

    def adjacency(self):
        a = np.zeros((self.n, self.n), np.float32)
        _check(lib().kura_get_adjacency(self.h, _fptr(a), self.n))
        return a

    def set_coupling(self, traj, c):
        _check(lib().kura_set_coupling(self.h, traj, float(c)))

    def set_state(self, traj, theta, t=0.0, h=0.01):
        th = np.ascontiguousarray(theta, np.float32)
        _check(lib().kura_set_state(self.h, traj, _fptr(th), float(t), float(h)))

    def set_state_device(self, traj, theta_ptr, t=0.0, h=0.01):
        _check(lib().kura_set_state_device(self.h, traj, ctypes.c_void_p(theta_ptr), float(t), float(h)))

    def set_horizon(self, t1, dt, initial_record=True):
        _check(lib().kura_set_horizon(self.h, float(t1), float(dt), int(initial_record)))

    def run(self, on_step=None, on_output=None, on_chunk=None):
        """Integrate to the horizon.  Optional Python observers receive
        on_step(traj, t, h, step), on_output(traj, index, t_eval, r, theta, couplings)
        and on_chunk(traj, t, h, theta); arrays are copies."""
        cb, keep = self._callbacks(on_step, on_output, on_chunk)
        _check(lib().kura_run(self.h, ctypes.byref(cb) if keep else None))

    def advance(self, attempts, on_step=None, on_output=None, on_chunk=None):
        """At most ``attempts`` step attempts of every unfinished trajectory (kura_advance);
        returns the number of trajectories still short of the horizon's end."""
        cb, keep = self._callbacks(on_step, on_output, on_chunk)
        running = ctypes.c_int32(0)
        _check(lib().kura_advance(self.h, ctypes.byref(cb) if keep else None, int(attempts), ctypes.byref(running)))
        return running.value

    def _callbacks(self, on_step, on_output, on_chunk):
        n = self.n
        cb = Callbacks()
        keep = []
        if on_step:
            f = STEP_CB(lambda u, b, t, h, s: int(bool(on_step(b, t, h, s))))
            cb.on_step = f
            keep.append(f)
        if on_output:
            def _o(u, b, idx, te, r, th, cp):
                tha = np.ctypeslib.as_array(th, (n,)).copy() if th else None
                cpa = np.ctypeslib.as_array(cp, (2 * n,)).copy() if cp else None
                return int(bool(on_output(b, idx, te, r, tha, cpa)))
            f = OUTPUT_CB(_o)
            cb.on_output = f
            keep.append(f)
        if on_chunk:
            f = CHUNK_CB(lambda u, b, t, h, th: int(bool(on_chunk(b, t, h, np.ctypeslib.as_array(th, (n,)).copy()))))
            cb.on_chunk = f
            keep.append(f)
        self._keep = keep  # the C callbacks live until the next call
        return cb, keep

    def state(self, traj=0, out=None):
        """(theta, t, h) of a trajectory; theta is written into ``out`` when given (a
        contiguous float32 array of n values, e.g. in pinned memory)."""
        if out is None:
            th = np.zeros(self.n, np.float32)
        else:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.size == self.n
                    and out.flags["C_CONTIGUOUS"] and out.flags["WRITEABLE"]):
                raise ValueError("out must be a writeable contiguous float32 array of %d values" % self.n)
            th = out
        t = ctypes.c_double()
        h = ctypes.c_double()
        _check(lib().kura_get_state(self.h, traj, _fptr(th), ctypes.byref(t), ctypes.byref(h)))
        return th, t.value, h.value

    def order(self, traj=0):
        cnt = ctypes.c_int64()
        _check(lib().kura_get_order(self.h, traj, None, 0, ctypes.byref(cnt)))
        r = np.zeros(cnt.value, np.float32)
        _check(lib().kura_get_order(self.h, traj, _fptr(r), r.size, ctypes.byref(cnt)))
        return r

    def final_record(self, traj=0):
        th = np.zeros(self.n, np.float32)
        cp = np.zeros(2 * self.n, np.float32)
        t = ctypes.c_double()
        h = ctypes.c_double()
        _check(lib().kura_final_record(self.h, traj, _fptr(th), _fptr(cp), ctypes.byref(t), ctypes.byref(h)))
        return th, cp, t.value, h.value

    def rhs(self, traj, theta):
        th = np.ascontiguousarray(theta, np.float32)
        f = np.zeros(self.n, np.float32)
        cp = np.zeros(2 * self.n, np.float32)
        _check(lib().kura_rhs(self.h, traj, _fptr(th), _fptr(f), _fptr(cp)))
        return f, cp

    def set_launch_attempts(self, attempts):
        _check(lib().kura_set_launch_attempts(self.h, attempts))

    def stats(self):
        s = Stats()
        _check(lib().kura_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}


class MultiNetworks:
    """Independent regenerated-volcano networks of uneven size integrated together, each
    with its own adaptive step, by one persistent launch (kura_multi_* in kura.h).

    ``ns``, ``ks``, ``seeds`` and ``cs`` give each network's size, volcano rank (0..8),
    Philox seed and coupling constant; all share t1, dt, h0 (default dt/100, the
    reference's first step), atol and rtol.  ``cluster_size`` / ``block_threads`` fix the
    launch shape (0: autotuned at the first integration)."""

    def __init__(self, ns, ks, seeds, cs, t1, dt, h0=None, atol=1e-6, rtol=0.0, device=0, cluster_size=0,
                 block_threads=0):
        count = len(ns)
        if not (len(ks) == len(seeds) == len(cs) == count):
            raise ValueError("ns, ks, seeds and cs must have the same length")
        arr = (Instance * count)()
        for i in range(count):
            arr[i].n, arr[i].k, arr[i].seed, arr[i].c = int(ns[i]), int(ks[i]), int(seeds[i]), float(cs[i])
        self.ns = np.asarray(ns, np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.ns)])
        self.count = count
        self.records = int(np.float32(t1) / np.float32(dt)) + 1
        h = ctypes.c_void_p()
        _check(lib().kura_multi_create(arr, count, float(t1), float(dt), float(dt / 100 if h0 is None else h0),
                                       float(atol), float(rtol), device, cluster_size, block_threads,
                                       ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().kura_multi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def integrate(self, omega, theta0, want_theta=True):
        """omega, theta0: the networks' oscillators back to back (or lists of per-network
        arrays).  Returns (order [count, records], final phases per network or None,
        accepted steps per network)."""
        if isinstance(omega, (list, tuple)):
            omega = np.concatenate(omega)
        if isinstance(theta0, (list, tuple)):
            theta0 = np.concatenate(theta0)
        om = np.ascontiguousarray(omega, np.float32)
        th = np.ascontiguousarray(theta0, np.float32)
        if om.size != self.offsets[-1] or th.size != self.offsets[-1]:
            raise ValueError("omega and theta0 need %d values" % self.offsets[-1])
        order = np.zeros((self.count, self.records), np.float32)
        fin = np.zeros(th.size, np.float32) if want_theta else None
        acc = np.zeros(self.count, np.int64)
        _check(lib().kura_multi_integrate(self.h, _fptr(om), _fptr(th), _fptr(order),
                                          _fptr(fin) if want_theta else None,
                                          acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        thetas = None
        if want_theta:
            thetas = [fin[self.offsets[i]:self.offsets[i + 1]] for i in range(self.count)]
        return order, thetas, acc

    def stats(self):
        s = MultiStats()
        _check(lib().kura_multi_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in MultiStats._fields_}


class MLP:
    """The order-parameter surrogate network (kura_mlp_* in kura.h): in_dim -> hidden ->
    hidden -> hidden -> out_dim with SiLU, BF16 weights and FP32 accumulation, trained and
    evaluated by libkura's tensor-core kernels."""

    def __init__(self, in_dim, out_dim, hidden=256, batch=512, seed=1, device=0):
        self.in_dim, self.out_dim, self.hidden, self.batch = in_dim, out_dim, hidden, batch
        h = ctypes.c_void_p()
        _check(lib().kura_mlp_create(in_dim, hidden, out_dim, batch, seed, device, ctypes.byref(h)))
        self.h = h
        c = ctypes.c_int64()
        _check(lib().kura_mlp_param_count(self.h, ctypes.byref(c)))
        self.param_count = c.value

    def close(self):
        if getattr(self, "h", None):
            lib().kura_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self):
        p = np.zeros(self.param_count, np.float32)
        _check(lib().kura_mlp_get_params(self.h, _fptr(p), p.size))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(lib().kura_mlp_set_params(self.h, _fptr(p), p.size))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.in_dim)
        y = np.zeros((x.shape[0], self.out_dim), np.float32)
        _check(lib().kura_mlp_forward(self.h, _fptr(x), x.shape[0], _fptr(y)))
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.in_dim)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, self.out_dim)
        g = np.zeros(self.param_count, np.float32)
        loss = ctypes.c_float()
        _check(lib().kura_mlp_gradients(self.h, _fptr(x), _fptr(t), x.shape[0], _fptr(g), ctypes.byref(loss)))
        return loss.value, g

    def train(self, x, t, epochs, lr=1e-3, lr_final=None, seed=1):
        """Adam on minibatches of `batch` rows; returns (loss per epoch, device ms)."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.in_dim)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, self.out_dim)
        losses = np.zeros(epochs, np.float32)
        ms = ctypes.c_double()
        _check(lib().kura_mlp_train(self.h, _fptr(x), _fptr(t), x.shape[0], epochs, lr,
                                    lr if lr_final is None else lr_final, seed, _fptr(losses), ctypes.byref(ms)))
        return losses, ms.value
