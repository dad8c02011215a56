"""ctypes binding of libdvmh_gb.so (the dvmh_* C ABI and its extensions) and of
the workload programs in libdvmhgb_workloads.so, for tests and bench.py.

Everything here calls the C ABI; the compute runs in the CUDA library.  Loading
fails loudly when the library is missing -- there is no fallback.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")
RUNTIME = os.path.join(LIB_DIR, "libdvmh_gb.so")
WORKLOADS = os.path.join(LIB_DIR, "libdvmhgb_workloads.so")

MODES = {"plain": 0, "async": 1, "batched": 2}

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)


class JacobiParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_long), ("iters", ctypes.c_long), ("seed", ctypes.c_uint64)]


class SorParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_long), ("sweeps", ctypes.c_long), ("omega", ctypes.c_double),
                ("seed", ctypes.c_uint64)]


class HeatParams(ctypes.Structure):
    _fields_ = [("count", ctypes.c_long), ("side_lo", ctypes.c_long), ("side_hi", ctypes.c_long),
                ("steps", ctypes.c_long), ("coef", ctypes.c_double), ("seed", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_long) for n in (
        "loops_performed", "handler_calls", "fused_pairs", "batched_groups", "graphs_captured", "graph_replays",
        "flushes", "h2d_bytes", "d2h_bytes", "kernel_launches", "relayouts")]

    def asdict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_rt = None
_wl = None
_inited = False


def built():
    return os.path.exists(RUNTIME) and os.path.exists(WORKLOADS)


def runtime():
    """The runtime library (ABI symbols only; no GPU needed to load it)."""
    global _rt
    if _rt is None:
        if not os.path.exists(RUNTIME):
            raise RuntimeError("libdvmh_gb.so is not built (run __graft_entry__.build())")
        _rt = ctypes.CDLL(RUNTIME, mode=ctypes.RTLD_GLOBAL)
        _rt.dvmhgb_get_mode.restype = ctypes.c_int
        _rt.dvmhgb_stream.restype = ctypes.c_void_p
        _rt.dvmh_wtime.restype = ctypes.c_double
    return _rt


def workloads():
    global _wl
    if _wl is None:
        runtime()
        _wl = ctypes.CDLL(WORKLOADS)
        for p in ("jac2d", "jac3d"):
            getattr(_wl, "wl_%s_setup" % p).argtypes = [ctypes.POINTER(JacobiParams)]
            getattr(_wl, "wl_%s_run" % p).argtypes = [ctypes.c_long, _dp]
            getattr(_wl, "wl_%s_fetch" % p).argtypes = [_dp, _dp]
            getattr(_wl, "wl_%s_step" % p).restype = ctypes.c_double
        _wl.wl_jac3d_load.argtypes = [_dp, _dp]
        _wl.wl_sor3d_setup.argtypes = [ctypes.POINTER(SorParams)]
        _wl.wl_sor3d_run.argtypes = [ctypes.c_long, _dp]
        _wl.wl_sor3d_fetch.argtypes = [_dp]
        _wl.wl_sor3d_step.restype = ctypes.c_double
        _wl.wl_heat_setup.argtypes = [ctypes.POINTER(HeatParams), _lp]
        _wl.wl_heat_run.argtypes = [ctypes.c_long, _dp, _dp, _ip]
        _wl.wl_heat_fetch.argtypes = [ctypes.c_long, _dp]
        _wl.wl_heat_total_cells.restype = ctypes.c_long
    return _wl


def init():
    """dvmh_init_C once per process (needs a CUDA GPU)."""
    global _inited
    if not _inited:
        workloads()
        argc = ctypes.c_int(0)
        argv = ctypes.POINTER(ctypes.c_char_p)()
        runtime().dvmh_init_C(0, ctypes.byref(argc), ctypes.byref(argv))
        _inited = True
    return runtime()


def set_mode(mode):
    init().dvmhgb_set_mode(MODES[mode] if isinstance(mode, str) else int(mode))


def force_variant(v):
    """Every loop variant query returns v from now on (v < 0: tuning / defaults again)."""
    init().dvmhgb_force_variant(int(v))


def set_deferral(on):
    """Whether queued loops that start a fusion rule may wait for the next loop (dvmhgb_set_deferral)."""
    init().dvmhgb_set_deferral(1 if on else 0)


def sync():
    init().dvmhgb_sync()


def stats():
    s = Stats()
    init().dvmhgb_get_stats(ctypes.byref(s))
    return s.asdict()


def reset_stats():
    init().dvmhgb_reset_stats()


def P(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class Jacobi:
    """The Jacobi program (rank 2 or 3) driven through its C entry points."""

    def __init__(self, rank, n, seed):
        init()
        self.rank, self.n = rank, n
        self.w = workloads()
        self.p = "jac%dd" % rank
        prm = JacobiParams(n, 0, seed)
        getattr(self.w, "wl_%s_setup" % self.p)(ctypes.byref(prm))

    def run(self, iters):
        eps = np.zeros(iters)
        getattr(self.w, "wl_%s_run" % self.p)(iters, P(eps))
        return eps

    def step(self):
        return getattr(self.w, "wl_%s_step" % self.p)()

    def fetch(self):
        cells = self.n ** self.rank
        A, B = np.zeros(cells), np.zeros(cells)
        getattr(self.w, "wl_%s_fetch" % self.p)(P(A), P(B))
        return A, B

    def load(self, A, B):
        assert self.rank == 3
        self.w.wl_jac3d_load(P(A) if A is not None else None, P(B) if B is not None else None)

    def push(self):
        """Host copies of A and B declared current: the next step uploads them (3-D only)."""
        self.w.wl_jac3d_push()

    def pull(self):
        """A and B made current on the host again (get_actual, 3-D only)."""
        self.w.wl_jac3d_pull()

    def close(self):
        getattr(self.w, "wl_%s_teardown" % self.p)()


class Sor:
    def __init__(self, n, omega, seed):
        init()
        self.n = n
        self.w = workloads()
        self.w.wl_sor3d_setup(ctypes.byref(SorParams(n, 0, omega, seed)))

    def run(self, sweeps):
        s = np.zeros(sweeps)
        self.w.wl_sor3d_run(sweeps, P(s))
        return s

    def fetch(self):
        A = np.zeros(self.n ** 3)
        self.w.wl_sor3d_fetch(P(A))
        return A

    def close(self):
        self.w.wl_sor3d_teardown()


class Heat:
    def __init__(self, count, lo, hi, coef, seed):
        init()
        self.w = workloads()
        self.count = count
        sides = np.zeros(count, dtype=np.int64)
        self.w.wl_heat_setup(ctypes.byref(HeatParams(count, lo, hi, 0, coef, seed)), sides.ctypes.data_as(_lp))
        self.sides = [int(s) for s in sides]

    def cells(self):
        return int(self.w.wl_heat_total_cells())

    def run(self, steps):
        sums = np.zeros(steps * self.count)
        mins = np.zeros(steps * self.count)
        locs = np.zeros(steps * self.count * 2, dtype=np.int32)
        self.w.wl_heat_run(steps, P(sums), P(mins), locs.ctypes.data_as(_ip))
        return sums.reshape(steps, self.count), mins.reshape(steps, self.count), locs.reshape(steps, self.count, 2)

    def fetch(self, k):
        u = np.zeros(self.sides[k] ** 2)
        self.w.wl_heat_fetch(k, P(u))
        return u

    def close(self):
        self.w.wl_heat_teardown()
