"""ACROSS loops with a handler in the shape cdvmh generates in its basic mode:
one thread walks the loop nest in the source order (converter_main.cpp isOneThread),
the block forced to 1x1x1 after dvmh_loop_cuda_get_config_C, a single reduction
slot.  A 2-D Gauss-Seidel sweep with a SUM of the new values
(workloads/gs2d*.c/cu), bit-exact against the sequential loop restated here,
in every execution mode."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc

pytestmark = pytest.mark.gpu


def sequential(n, sweeps, seed):
    L = orc.lib()
    a = np.zeros((n, n))
    for i in range(1, n - 1):
        for j in range(1, n - 1):
            a[i, j] = L.orc_u01(seed, 13, i * n + j)
    sums = []
    for _ in range(sweeps):
        s = -0.0  # the thread's private SUM starts at the identity
        for i in range(1, n - 1):
            for j in range(1, n - 1):
                a[i, j] = (((a[i - 1, j] + a[i + 1, j]) + a[i, j - 1]) + a[i, j + 1]) * 0.25
                s = s + a[i, j]
        sums.append((0.0 + s) + 0.0)  # one slot: (start + fold) + the initial value 0
    return np.array(sums), a


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    yield g
    g.set_mode("batched")


@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
def test_generated_across_one_thread(g, mode):
    g.set_mode(mode)
    n, sweeps, seed = 30, 3, 99
    w = g.workloads()
    w.wl_gs2d_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double)]
    s = np.zeros(sweeps)
    a = np.zeros(n * n)
    assert w.wl_gs2d_run(n, sweeps, seed, orc.P(s), orc.P(a)) == 0
    s_ref, a_ref = sequential(n, sweeps, seed)
    assert np.array_equal(a.reshape(n, n), a_ref), mode
    assert np.array_equal(s, s_ref), mode
