"""The reference's FP32 Jacobi benchmarks (examples/Performance/jac3d_perf.c,
jac2d_perf.c) through handlers in cdvmh's generated shape
(workloads/jacperf*.c/cu): the arrays initialised by a device loop, MAX with
one slot per launched thread, the programs' cuda_block clauses.  Checked bit
for bit against the reference runtime's own outputs (tests/golden), and the
full configurations against the examples' own verification values
(jac3d_perf.c:92: eps 5.058044 +- 1e-4 at 384^3 after 100 iterations;
jac2d_perf.c:89: 58.37598 +- 1e-3 at 8000^2)."""
import ctypes
import hashlib

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu

KNOWN_ANSWERS = {(3, 384, 100): (5.058044, 1e-4), (2, 8000, 100): (58.37598, 1e-3)}


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    w = g.workloads()
    fp = ctypes.POINTER(ctypes.c_float)
    w.wl_jacperf_run.restype = ctypes.c_long
    w.wl_jacperf_run.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long, fp, fp, fp]
    yield g
    g.set_mode("batched")


def sha32(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f4").tobytes()).hexdigest()


@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
def test_golden(g, golden, mode):
    g.set_mode(mode)
    fp = ctypes.POINTER(ctypes.c_float)
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "jacperf"]
    assert {tuple(c["params"]) for _, c in cases} >= set(KNOWN_ANSWERS)
    for name, c in cases:
        rank, L, itmax = c["params"]
        if mode == "async" and L > 100:
            continue  # the full configurations run in plain and batched mode
        eps = np.zeros(itmax, dtype=np.float32)
        a = np.zeros(L ** rank, dtype=np.float32)
        b = np.zeros(L ** rank, dtype=np.float32)
        its = g.workloads().wl_jacperf_run(rank, L, itmax, eps.ctypes.data_as(fp), a.ctypes.data_as(fp),
                                           b.ctypes.data_as(fp))
        assert its == c["its"], (name, mode)
        assert [float(x).hex() for x in eps[:its]] == c["eps"], (name, mode)
        assert sha32(a) == c["A_sha256"] and sha32(b) == c["B_sha256"], (name, mode)
        ka = KNOWN_ANSWERS.get((rank, L, itmax))
        if ka:
            assert abs(float(eps[its - 1]) - ka[0]) < ka[1], (name, mode)
