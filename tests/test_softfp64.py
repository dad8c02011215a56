"""Integer-pipe FP64 arithmetic (csrc/kernels/softfp64.cuh) is bit-identical
to IEEE binary64 round-to-nearest: on the host FPU (CPU) and on the GB300
FP64 unit (GPU self-test through the C-ABI)."""
import ctypes
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def hostlib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("sf") / "libsfcheck.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC", "-shared",
                           os.path.join(HERE, "softfp64_check.cpp"), "-o", out])
    L = ctypes.CDLL(out)
    L.softfp64_check.argtypes = [ctypes.c_long, ctypes.c_uint64, ctypes.POINTER(ctypes.c_long)]
    return L


@pytest.mark.parametrize("seed", [1, 20261203])
def test_softfp64_matches_host_fpu(hostlib, seed):
    bad = (ctypes.c_long * 4)()
    hostlib.softfp64_check(4_000_000, seed, bad)
    assert list(bad) == [0, 0, 0, 0], "mismatches add/sub/mul/div6: %s" % list(bad)


@pytest.mark.parametrize("seed", [3, 20261204])
def test_add_pos_matches_host_fpu(hostlib, seed):
    """The non-negative-operand addition of the stencil kernels, on its whole domain."""
    hostlib.softfp64_check_pos.restype = ctypes.c_long
    hostlib.softfp64_check_pos.argtypes = [ctypes.c_long, ctypes.c_uint64]
    assert hostlib.softfp64_check_pos(4_000_000, seed) == 0


def test_scale_up_and_pos_small(hostlib):
    """The exact x * 4.0 of the heat kernel and the range test of its integer SUM tree."""
    hostlib.softfp64_check_scale.restype = ctypes.c_long
    hostlib.softfp64_check_scale.argtypes = [ctypes.c_long, ctypes.c_uint64]
    assert hostlib.softfp64_check_scale(2_000_000, 11) == 0


@pytest.mark.gpu
def test_softfp64_matches_gb300_fp64_unit():
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    g.init()
    bad = (ctypes.c_long * 4)()
    assert g.runtime().dvmhgb_selftest_softfp64(ctypes.c_long(1 << 30), ctypes.c_ulonglong(7), bad) == 0
    assert list(bad) == [0, 0, 0, 0], "mismatches add/sub/mul/div6: %s" % list(bad)


@pytest.mark.parametrize("seed", [3, 20261204])
def test_div6_fma_matches_host_division(hostlib, seed):
    """RN(x / 6) from one multiply and two FMAs (Markstein's correction) equals
    the host FPU's division on stencil sums and on normal doubles of both signs
    across the exponent range the method covers."""
    hostlib.softfp64_check_div6_fma.restype = ctypes.c_long
    hostlib.softfp64_check_div6_fma.argtypes = [ctypes.c_long, ctypes.c_uint64]
    assert hostlib.softfp64_check_div6_fma(4_000_000, seed) == 0


@pytest.mark.parametrize("seed", [5, 20261205])
def test_q61_chain_matches_host_fpu(hostlib, seed):
    """The fixed-point form of the Jacobi stencil: five additions and the division by 6."""
    hostlib.softfp64_check_q61.restype = ctypes.c_long
    hostlib.softfp64_check_q61.argtypes = [ctypes.c_long, ctypes.c_uint64]
    assert hostlib.softfp64_check_q61(2_000_000, seed) == 0
