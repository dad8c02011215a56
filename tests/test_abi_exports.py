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
                 "loop_heat_batch_cuda", "wl_jac3d_setup", "wl_sor3d_run", "wl_heat_step"]:
        assert hasattr(w, name), name
