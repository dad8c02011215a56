"""The drop-in boundary: the runtime library loads without a GPU and exports
every function the public headers (include/*.h) declare.

Only symbol lookup happens here (no call into the library), so the test runs
on machines without a CUDA device; the GPU tests exercise the same entry
points with data."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = ["dvmhlib2.h", "dvmh_gb.h", "dvmh_gb_kernels.h"]
# a declaration: a return type, then the function name and "(" -- at the start of a line
DECL = re.compile(r"^\s*(?!typedef|#|return\b)[A-Za-z_][\w\s\*]*?\b((?:dvmh|dvmhgb)_\w+)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # comments may hold example calls
    text = re.sub(r"//[^\n]*", "", text)
    return sorted(set(DECL.findall(text)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    return g.runtime()


@pytest.mark.parametrize("header", HEADERS)
def test_header_symbols_exported(lib, header):
    names = declared(header)
    assert len(names) > 10, header  # the parser found the declarations
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, (header, missing)


def test_parser_sees_known_entry_points():
    assert "dvmh_loop_cuda_red_prepare_C" in declared("dvmhlib2.h")
    assert "dvmhgb_sor3d_sweep" in declared("dvmh_gb_kernels.h")
    assert "dvmhgb_jac3d_update_noalloc" in declared("dvmh_gb_kernels.h")
    assert "dvmhgb_force_variant" in declared("dvmh_gb.h")


def test_workload_handlers_exported():
    """The CUDA handlers of the example programs (what cdvmh would emit) live
    in the workload library, linked against the runtime."""
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    w = ctypes.CDLL(g.WORKLOADS)
    for name in ["loop_jac3d_upd_cuda", "loop_jac3d_stn_cuda", "loop_sor3d_cuda", "loop_heat_cuda",
                 "loop_heat_batch_cuda", "wl_jac3d_setup", "wl_sor3d_run", "wl_heat_step",
                 # handlers in cdvmh's generated shapes
                 "loop_gen3d_cuda", "loop_genred_cuda", "loop_gs2d_cuda", "loop_gsd2d_cuda", "loop_gsd3d_cuda",
                 "loop_rec2d_cuda", "loop_sor3d_gen_cuda", "loop_jac3d_upd_gen_cuda", "loop_jac3d_stn_gen_cuda",
                 "loop_jacperf3_upd_cuda", "loop_jacperf2_stn_cuda", "wl_jacperf_run", "wl_genred_run_data"]:
        assert hasattr(w, name), name


@pytest.mark.parametrize("pattern", [0, 1, 2])
def test_edge_value_patterns_match_the_oracle(pattern):
    """The edge-value inputs of the reductions program (wl_genred_pattern,
    host C in the workload library; the reference driver compiles the same
    source to make the golden cases) are the ones the oracle's own copy
    (orc_genred_pattern) builds when it checks those goldens."""
    import numpy as np

    import __graft_entry__ as ge
    from oracle import orc
    ge.build()
    _, g = ge.package()
    w = ctypes.CDLL(g.WORKLOADS)
    D, I = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    w.wl_genred_pattern.argtypes = [ctypes.c_int, ctypes.c_long, D, I]
    n = 10007
    x = np.zeros(n)
    v = np.zeros(n, dtype=np.int32)
    assert w.wl_genred_pattern(pattern, n, x.ctypes.data_as(D), v.ctypes.data_as(I)) == 0
    xo, vo = orc.genred_pattern(pattern, n)
    assert x.tobytes() == xo.tobytes() and np.array_equal(v, vo)
