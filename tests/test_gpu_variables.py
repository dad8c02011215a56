"""Scalars registered in regions live in the runtime's variable registry by
host address.  A program may free such memory and later register a new
variable that overlaps an old one (another program's reduction buffer, a
temporary): the old registration is forgotten -- with its device copy and any
cached graph that named it -- instead of being reported as a conflict, as long
as its host copy is current.  An old variable whose only current value is on
the device is never dropped silently: that registration is an error, as a
changed or overlapping regular variable is in the reference
(rts/dvmh/dvmh2.cpp:1794-1830)."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu

INTENT_INOUT, DEVICE_TYPE_CUDA = 3, 2


@pytest.fixture(scope="module")
def rt():
    ge.build()
    _, g = ge.package()
    g.init()
    rt = g.runtime()
    rt.dvmh_region_create_C.restype = ctypes.c_long
    rt.dvmh_region_create_C.argtypes = [ctypes.c_long]
    rt.dvmh_region_register_scalar_C.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_void_p, ctypes.c_long,
                                                 ctypes.c_char_p]
    rt.dvmh_region_execute_on_targets_C.argtypes = [ctypes.c_long, ctypes.c_long]
    rt.dvmh_region_end_C.argtypes = [ctypes.c_long]
    rt.dvmh_actual_variable2_.argtypes = [ctypes.c_void_p]
    rt.dvmh_get_actual_variable2_.argtypes = [ctypes.c_void_p]
    return rt


def region_with(rt, addr, size, name):
    r = rt.dvmh_region_create_C(0)
    rt.dvmh_region_register_scalar_C(r, INTENT_INOUT, addr, size, name)
    rt.dvmh_region_execute_on_targets_C(r, DEVICE_TYPE_CUDA)
    rt.dvmh_region_end_C(r)


def test_overlapping_variables_from_earlier_regions(rt):
    buf = np.arange(16, dtype=np.float64)
    p = buf.ctypes.data
    region_with(rt, p, 32, b"old")            # doubles 0..3
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p))
    region_with(rt, p + 16, 32, b"shifted")   # doubles 2..5: overlaps the old one
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p + 16))
    region_with(rt, p + 8, 64, b"wider")      # doubles 1..8: overlaps the shifted one
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p + 8))
    region_with(rt, p, 128, b"whole")         # all of them
    # the surviving registration round-trips the host values through the device
    rt.dvmh_actual_variable2_(ctypes.c_void_p(p))
    region_with(rt, p, 128, b"whole")
    before = buf.copy()
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p))
    assert np.array_equal(buf, before)


def test_smaller_variable_at_a_known_address(rt):
    # a new, smaller variable where an earlier region registered a larger one (an
    # allocation reused): reading it back copies only its own bytes, never the old size
    buf = np.full(24, 1.0)
    p = buf.ctypes.data
    region_with(rt, p, 192, b"old")
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p))
    buf[:] = 2.0
    rt.dvmh_actual_variable2_(ctypes.c_void_p(p))
    region_with(rt, p, 128, b"new")      # doubles 0..15; the device copy is newer afterwards
    buf[16:] = 9.0                       # the program's memory beyond the new variable
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p))
    assert np.array_equal(buf[:16], np.full(16, 2.0))
    assert np.array_equal(buf[16:], np.full(8, 9.0))
    # and growing again at the same address from a later region
    buf[:] = 3.0
    rt.dvmh_actual_variable2_(ctypes.c_void_p(p))
    region_with(rt, p, 192, b"grown")
    buf[:] = -1.0
    rt.dvmh_get_actual_variable2_(ctypes.c_void_p(p))
    assert np.array_equal(buf, np.full(24, 3.0))


CHILD = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, %r)
    import __graft_entry__ as ge
    _, g = ge.package()
    g.init()
    rt = g.runtime()
    rt.dvmh_region_create_C.restype = ctypes.c_long
    rt.dvmh_region_create_C.argtypes = [ctypes.c_long]
    rt.dvmh_region_register_scalar_C.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_void_p, ctypes.c_long,
                                                 ctypes.c_char_p]
    rt.dvmh_region_execute_on_targets_C.argtypes = [ctypes.c_long, ctypes.c_long]
    rt.dvmh_region_end_C.argtypes = [ctypes.c_long]
    buf = np.full(8, 1.0)
    p = buf.ctypes.data
    def region(addr, size):
        r = rt.dvmh_region_create_C(0)
        rt.dvmh_region_register_scalar_C(r, 3, addr, size, b"v")
        rt.dvmh_region_execute_on_targets_C(r, 2)
        rt.dvmh_region_end_C(r)
    region(p, 64)       # INOUT: afterwards the device copy is the current one
    region(p, %d)       # the same address with another extent, nothing read back
    print("not refused")
""")


@pytest.mark.parametrize("size", [32, 128])
def test_device_newer_variable_is_not_dropped_silently(size):
    """A shrink or a growth of a variable whose only current value is on the
    device, from a later region and without get_actual: the runtime reports it
    (exit status 1, the reference's user-error convention) instead of dropping
    the value.  Run in a child process."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", CHILD % (root, size)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "only current value on the device" in r.stderr, r.stderr
    assert "not refused" not in r.stdout
