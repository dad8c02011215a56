"""The wavefront's bounded waits: a wait that runs out makes the kernel return
with the timeout code in the runtime's status word and the hand-out counter
stopped, and the runtime reports it at its next synchronisation with the
reference's user-error convention (exit status 1).  The wait is made to run
out without any fault: the sweep's hand-out starts at tile 1, so tile 0 is
never computed and the flags its successors wait for are never set; the poll
limit is 1000 instead of 2^24.  Run in a child process, which that report ends."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

CHILD = textwrap.dedent("""
    import ctypes, sys
    import torch
    sys.path.insert(0, %r)
    import __graft_entry__ as ge
    _, g = ge.package()
    g.init()
    L = g.runtime()
    L.dvmhgb_sor3d_items.restype = ctypes.c_long
    L.dvmhgb_sor3d_scratch_bytes.restype = ctypes.c_long
    L.dvmhgb_status_word.restype = ctypes.c_void_p
    L.dvmhgb_sor3d_sweep_bounded.restype = ctypes.c_int
    variant = %d
    n = 40
    LA = ctypes.c_long * 3
    st, ext, lo, hi = LA(n * n, n, 1), LA(n, n, n), LA(1, 1, 1), LA(n - 2, n - 2, n - 2)
    A = torch.rand(n, n, n, dtype=torch.float64, device="cuda")
    w = torch.tensor([1.5], dtype=torch.float64, device="cuda")
    items = torch.empty(L.dvmhgb_sor3d_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    scratch = torch.zeros(L.dvmhgb_sor3d_scratch_bytes(lo, hi, variant) // 4, dtype=torch.int32, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = L.dvmhgb_sor3d_sweep_bounded(vp(A), st, ext, lo, hi, vp(w), vp(items), vp(scratch),
                                      ctypes.c_void_p(L.dvmhgb_status_word()), variant,
                                      ctypes.c_void_p(L.dvmhgb_stream()), ctypes.c_long(1000), ctypes.c_long(1))
    print("launch", rc, flush=True)
    torch.cuda.synchronize()  # the kernel has returned
    counter = int(scratch[0].item()) & 0xFFFFFFFF
    print("counter-stopped", bool(counter & 0x80000000), flush=True)
    L.dvmhgb_sync()           # the runtime reads its status word here
    print("not reported", flush=True)
""")


@pytest.mark.parametrize("variant", [1, 3, 4, 5])
def test_expired_wait_is_reported(variant):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", CHILD % (root, variant)], capture_output=True, text=True, timeout=600)
    assert "launch 0" in r.stdout, (r.stdout, r.stderr)
    assert "counter-stopped True" in r.stdout, (r.stdout, r.stderr)
    assert "not reported" not in r.stdout, (r.stdout, r.stderr)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "gave up waiting" in r.stderr and "0x50520001" in r.stderr, r.stderr


def test_default_limit_sweep_unaffected():
    """The same launcher with the default limit and hand-out from tile 0
    (what dvmhgb_sor3d_sweep runs) completes and reports nothing."""
    import ctypes
    import torch
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    g.init()
    L = g.runtime()
    L.dvmhgb_sor3d_items.restype = ctypes.c_long
    L.dvmhgb_sor3d_scratch_bytes.restype = ctypes.c_long
    L.dvmhgb_status_word.restype = ctypes.c_void_p
    n, variant = 40, 1
    LA = ctypes.c_long * 3
    st, ext, lo, hi = LA(n * n, n, 1), LA(n, n, n), LA(1, 1, 1), LA(n - 2, n - 2, n - 2)
    A = torch.rand(n, n, n, dtype=torch.float64, device="cuda")
    w = torch.tensor([1.5], dtype=torch.float64, device="cuda")
    items = torch.empty(L.dvmhgb_sor3d_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    scratch = torch.zeros(L.dvmhgb_sor3d_scratch_bytes(lo, hi, variant) // 4, dtype=torch.int32, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    assert L.dvmhgb_sor3d_sweep_bounded(vp(A), st, ext, lo, hi, vp(w), vp(items), vp(scratch),
                                        ctypes.c_void_p(L.dvmhgb_status_word()), variant,
                                        ctypes.c_void_p(L.dvmhgb_stream()), ctypes.c_long(1 << 24),
                                        ctypes.c_long(0)) == 0
    torch.cuda.synchronize()
    assert int(scratch[0].item()) & 0x80000000 == 0
    g.sync()  # no report
