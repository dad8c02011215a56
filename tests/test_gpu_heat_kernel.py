"""The heat kernels directly through the C ABI, on data that takes every path.

The example program's data (uniform [0, 1)) only ever takes the integer-pipe
paths of the heat kernel (the exact 4.0 * x, the SUM tree on sf::add_pos).
Here one array holds negative values, zeros, a subnormal and a huge value,
which force the FP64-unit fallbacks, and another holds ordinary values.  Both
go through dvmhgb_heat (one loop) and dvmhgb_heat_many (the batched table).
The array, the SUM (items folded by the canonical pairwise tree) and the
MINLOC (value and location) are compared bit for bit with the oracle's
restatement of the loop (oracle/restate.c: orc_heat_step)."""
import ctypes

import numpy as np
import pytest

from oracle import orc

pytestmark = pytest.mark.gpu


class HeatDesc(ctypes.Structure):
    _fields_ = [("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("s0", ctypes.c_long),
                ("lo0", ctypes.c_long), ("hi0", ctypes.c_long), ("lo1", ctypes.c_long), ("hi1", ctypes.c_long),
                ("coef", ctypes.c_void_p), ("c0", ctypes.c_long), ("nck", ctypes.c_long), ("units", ctypes.c_long),
                ("unitBase", ctypes.c_long), ("sr", ctypes.c_long), ("strips", ctypes.c_long),
                ("stripBase", ctypes.c_long), ("sumItems", ctypes.c_void_p), ("minItems", ctypes.c_void_p),
                ("locItems", ctypes.c_void_p)]


def pairwise(items):
    """The reduction engine's fold: pairwise by item index, padded with -0.0 to a power of two."""
    v = [float(x) for x in items]
    m = 1
    while m < len(v):
        m *= 2
    v += [-0.0] * (m - len(v))
    while len(v) > 1:
        v = [v[2 * q] + v[2 * q + 1] for q in range(len(v) // 2)]
    return v[0]


def arrays():
    rng = np.random.default_rng(3)
    n1 = 131
    a = rng.random((n1, n1))
    a[10:20, :] -= 0.5          # negative values: the native SUM tree
    a[40, 70] = 5e-310          # subnormal: the native 4.0 * x
    a[50:52, 5:60] = 0.0
    a[90, 100] = 1e300          # huge: outside the integer tree's range
    n2 = 200
    b = rng.random((n2, n2))    # ordinary values: the integer-pipe paths
    return [a, b]


def oracle(src, c):
    n = src.shape[0]
    s = np.ascontiguousarray(src)
    dst = np.zeros_like(s)
    ss, sc, mn = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    loc = (ctypes.c_int * 2)()
    orc.lib().orc_heat_step(ctypes.c_long(n), ctypes.c_double(c), orc.P(s), orc.P(dst), ctypes.byref(ss),
                            ctypes.byref(sc), ctypes.byref(mn), loc)
    return dst, sc.value, mn.value, (loc[0], loc[1])


@pytest.mark.parametrize("batched", [False, True])
def test_heat_kernel_all_paths(batched):
    import torch
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    L = g.runtime()
    c = 0.2
    coef = torch.tensor([c], dtype=torch.float64, device="cuda")
    srcs = arrays()
    descs, keep = [], []
    for a in srcs:
        n = a.shape[0]
        w = n + (n & 1)  # even row stride: 16-byte aligned rows
        S = torch.zeros(n, w, dtype=torch.float64, device="cuda")
        S[:, :n] = torch.from_numpy(a).cuda()
        D = torch.zeros_like(S)
        d = HeatDesc()
        lo, hi = (ctypes.c_long * 2)(1, 1), (ctypes.c_long * 2)(n - 2, n - 2)
        assert L.dvmhgb_heat_desc_fill(ctypes.byref(d), ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(D.data_ptr()),
                                       ctypes.c_long(w), lo, hi, ctypes.c_void_p(coef.data_ptr())) == 0
        si = torch.empty(d.units, dtype=torch.float64, device="cuda")
        mi = torch.empty(d.units, dtype=torch.float64, device="cuda")
        li = torch.empty(2 * d.units, dtype=torch.int32, device="cuda")
        d.sumItems, d.minItems, d.locItems = si.data_ptr(), mi.data_ptr(), li.data_ptr()
        descs.append(d)
        keep.append((S, D, si, mi, li, n))
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if batched:
        table = (HeatDesc * len(descs))(*descs)
        total = units = 0
        for q in range(len(descs)):
            table[q].stripBase, table[q].unitBase = total, units
            total += table[q].strips
            units += table[q].units
        dev = torch.empty(ctypes.sizeof(table), dtype=torch.uint8, device="cuda")
        dev.copy_(torch.frombuffer(bytearray(table), dtype=torch.uint8))
        assert L.dvmhgb_heat_many(ctypes.c_void_p(dev.data_ptr()), len(descs), ctypes.c_long(total), sp) == 0
    else:
        for d in descs:
            assert L.dvmhgb_heat(ctypes.byref(d), sp) == 0
    torch.cuda.synchronize()
    for a, (S, D, si, mi, li, n) in zip(srcs, keep):
        dst, sc, mn, loc = oracle(a, c)
        got = D.cpu().numpy()[:, :n]
        assert np.array_equal(got[1:-1, 1:-1], dst[1:-1, 1:-1]), n
        assert (0.0 + pairwise(si.cpu().numpy())) + 0.0 == sc, n
        mins = mi.cpu().numpy()
        k = int(np.argmin(mins))  # the first smallest item: loop order
        assert mins[k] == mn, n
        assert tuple(li.cpu().numpy()[2 * k:2 * k + 2]) == loc, n
