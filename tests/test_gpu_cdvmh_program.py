"""A program exactly as cdvmh converts it (workloads/cdvh2d.c with its CUDA
handlers and module initialiser) links unchanged against this runtime and
gives the reference runtime's results bit for bit: the library-entry
dvmh_init_lib_C, dynamic DVM arrays (dvmh_array_declare_C /
dvmh_array_alloc_C / dvmh_array_free_C / dvmh_forget_header_), regular memory
from dvmh_malloc_C / dvmh_free_C, a global regular array entered by the
module initialiser, implicit data regions around each region
(dvmh_data_enter_C / dvmh_data_exit_C with the save flag), regular arrays
registered through dvmh_variable_gen_header_C and handed to the handlers as
dvmh_variable_get_header_C, and own-element writes
(dvmh_get_own_element_addr_C) in sequential code."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc
from tests.util import sha, unhex

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prog():
    ge.build()
    _, g = ge.package()
    g.init()
    w = g.workloads()
    w.wl_cdvh2d_run.restype = ctypes.c_int
    w.wl_cdvh2d_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double)]

    def run(n, iters, seed):
        eps, B = np.zeros(iters), np.zeros(n * n)
        assert w.wl_cdvh2d_run(n, iters, seed, orc.P(eps), orc.P(B)) == 0
        return eps, B
    yield g, run
    g.set_mode("batched")


@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
def test_reference_golden(prog, golden, mode):
    g, run = prog
    g.set_mode(mode)
    cases = [k for k, v in golden.items() if v["prog"] == "cdvh2d"]
    assert cases
    for k in cases:
        c = golden[k]
        n, it, seed = c["params"]
        for _ in range(2):  # twice: every regular variable and dynamic array left the runtime cleanly
            eps, B = run(n, it, seed)
            assert [float(x).hex() for x in eps] == c["eps"], (k, mode)
            assert sha(B) == c["B_sha256"], (k, mode)
            if "B" in c:
                assert np.array_equal(B, unhex(c["B"])), (k, mode)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_larger_than_the_goldens(prog, mode):
    g, run = prog
    g.set_mode(mode)
    n, it, seed = 1030, 7, 20261214
    e_ref, B_ref = orc.cdvh2d_run(n, it, seed)
    eps, B = run(n, it, seed)
    assert np.array_equal(eps, e_ref) and np.array_equal(B, B_ref), mode
