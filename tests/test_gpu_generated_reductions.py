"""Loop normalisation, signed steps and every reduction operation through a
handler in the exact generated shape (workloads/genred*.c/cu).

A 1-D loop `for i = start; i <=/>= end; i += step` carries eight reductions:
SUM and PROD of doubles, MIN / AND / OR / XOR of ints, MAX of a float and
MINLOC of a double.  Each launched thread fills one slot per reduction.

The expected results emulate what the runtime defines:

- normalised bounds end = start + floor((end-start)/step)*step (loop.cpp:556-565);
- SUM / PROD slots folded pairwise by slot index (identity padding), then
  combined as (start (+) fold) (+) initial value (dvmh2.cpp:3848-3851, 3950-3953);
- MIN / MAX / MINLOC strict, the earliest slot winning ties (loop.cpp:117-118);
- bitwise operations exact.

An empty loop leaves every variable at its initial value."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    yield g
    g.set_mode("batched")


def fold(slots, op, ident):
    v = np.asarray(slots, dtype=np.float64)
    m = 1
    while m < len(v):
        m *= 2
    v = np.concatenate([v, np.full(m - len(v), ident)])
    while len(v) > 1:
        v = op(v[0::2], v[1::2])
    return float(v[0])


def expected(n, start, end, step, seed, bx, init):
    L = orc.lib()
    x = np.array([L.orc_u01(seed, 11, i) for i in range(n)])
    v = np.array([int(L.orc_u01(seed, 12, i) * 2147483647.0) - 1073741824 for i in range(n)], dtype=np.int64)
    ds0, dp0, dml0, imn0, ia0, io0, ix0, fmx0, lc0 = init
    cnt = (end - start) // step + 1
    if cnt <= 0:
        return dict(ds=ds0, dp=dp0, dml=dml0, imn=imn0, ia=ia0, io=io0, ix=ix0, fmx=fmx0, lc=lc0)
    pts = start + step * np.arange(cnt)
    xs, vs = x[pts], v[pts]
    nslots = -(-cnt // bx) * bx
    ss = np.full(nslots, -0.0)
    ss[:cnt] = -0.0 + xs
    sp = np.full(nslots, 1.0)
    sp[:cnt] = 1.0 * (1.0 + xs / 65536.0)
    ds = (0.0 + fold(ss, np.add, -0.0)) + ds0
    dp = (1.0 * fold(sp, np.multiply, 1.0)) * dp0
    ia, io, ix = ia0, io0, 0
    for q in vs:
        ia &= int(q) | 0x0F0F0F0F
        io |= int(q) & 0x00FF00FF
        ix ^= int(q)
    ix ^= ix0
    k = int(np.argmin(xs))
    dml, lc = (xs[k], int(pts[k])) if xs[k] < dml0 else (dml0, lc0)
    fmx = max(np.float32(fmx0), np.float32(xs.astype(np.float32).max()))
    return dict(ds=ds, dp=dp, dml=dml, imn=min(imn0, int(vs.min())), ia=ia, io=io, ix=ix, fmx=float(fmx), lc=lc)


CASES = [(1000, 3, 990, 7, 128), (5000, 4990, 2, -13, 64), (300000, 0, 299999, 1, 256), (100, 50, 10, 1, 32),
         (777, 776, 0, -1, 0)]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
def test_generated_reductions(g, case, mode):
    g.set_mode(mode)
    n, start, end, step, bx = case
    seed = 17 + n
    init = (0.125, 1.5, 0.75, 123, -1, 0x100, 0x5A5A5A5A, -2.0, -9)
    w = g.workloads()
    w.wl_genred_run.argtypes = [ctypes.c_long] * 4 + [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float),
                                                      ctypes.POINTER(ctypes.c_long)]
    d3 = (ctypes.c_double * 3)(init[0], init[1], init[2])
    i4 = (ctypes.c_int * 4)(init[3], init[4], init[5], init[6])
    f1 = (ctypes.c_float * 1)(init[7])
    lc = (ctypes.c_long * 1)(init[8])
    assert w.wl_genred_run(n, start, end, step, seed, bx, d3, i4, f1, lc) == 0
    blk = bx if bx else 256  # the runtime's default block for rank 1
    e = expected(n, start, end, step, seed, blk, init)
    got = dict(ds=d3[0], dp=d3[1], dml=d3[2], imn=i4[0], ia=i4[1], io=i4[2], ix=i4[3], fmx=f1[0], lc=lc[0])
    for k in e:
        want = e[k]
        if k in ("ia", "io", "ix"):  # compare as 32-bit patterns
            assert (got[k] & 0xFFFFFFFF) == (want & 0xFFFFFFFF), (k, mode, case)
        else:
            assert got[k] == want, (k, mode, case, got[k], want)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_reference_golden(g, golden, mode):
    """The reference runtime's own results (its host handler, loop order):
    MIN / MAX / AND / OR / XOR / MINLOC and the location bit for bit; SUM and
    PROD, which the generated handler folds per thread, within the forward
    error bound of the reference's sequential value (n additions: n * 2^-53 *
    sum |x|; n multiplications by factors near 1: 2n * 2^-53 * |product|)."""
    g.set_mode(mode)
    w = g.workloads()
    w.wl_genred_run.argtypes = [ctypes.c_long] * 4 + [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float),
                                                      ctypes.POINTER(ctypes.c_long)]
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "genred"]
    assert cases
    u = 2.0 ** -53
    for name, c in cases:
        n, start, end, step, seed = c["params"][:5]
        init = c["params"][5:]
        d3 = (ctypes.c_double * 3)(*init[0:3])
        i4 = (ctypes.c_int * 4)(*init[3:7])
        f1 = (ctypes.c_float * 1)(init[7])
        lc = (ctypes.c_long * 1)(init[8])
        assert w.wl_genred_run(n, start, end, step, seed, 0, d3, i4, f1, lc) == 0
        ref_d = [float.fromhex(x) for x in c["d3"]]
        cnt = max(0, (end - start) // step + 1)
        assert abs(d3[0] - ref_d[0]) <= cnt * u * (abs(ref_d[0]) + abs(init[0])) + 0.0, name
        assert abs(d3[1] - ref_d[1]) <= 2 * cnt * u * abs(ref_d[1]), name
        assert float(d3[2]).hex() == c["d3"][2], name
        assert list(i4) == c["i4"], name
        assert float(f1[0]).hex() == c["f1"][0], name
        assert lc[0] == c["lc"], name


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_edge_values_reference_golden(g, golden, mode):
    """Signed zeros, subnormals, infinities, NaN and ties (wl_genred_pattern),
    against the reference runtime's results: MAX of signed zeros and MINLOC
    ties go to the first in loop order (the fold keeps the lower slot on ties,
    slots follow loop order), MIN / AND / OR / XOR exact; SUM and PROD exact
    where the reference's value is NaN or infinite, else within the error bound."""
    g.set_mode(mode)
    w = g.workloads()
    D, I, F, Lp = (ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float),
                   ctypes.POINTER(ctypes.c_long))
    w.wl_genred_pattern.argtypes = [ctypes.c_int, ctypes.c_long, D, I]
    w.wl_genred_run_data.argtypes = [ctypes.c_long] * 4 + [D, I, ctypes.c_int, D, I, F, Lp]
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "genredx"]
    assert len(cases) >= 5
    u = 2.0 ** -53
    for name, c in cases:
        n, start, end, step, pattern = c["params"][:5]
        init = c["params"][5:]
        x = np.zeros(n)
        v = np.zeros(n, dtype=np.int32)
        assert w.wl_genred_pattern(pattern, n, x.ctypes.data_as(D), v.ctypes.data_as(I)) == 0
        d3 = (ctypes.c_double * 3)(*init[0:3])
        i4 = (ctypes.c_int * 4)(*init[3:7])
        f1 = (ctypes.c_float * 1)(init[7])
        lc = (ctypes.c_long * 1)(init[8])
        assert w.wl_genred_run_data(n, start, end, step, x.ctypes.data_as(D), v.ctypes.data_as(I), 0, d3, i4, f1,
                                    lc) == 0
        cnt = max(0, (end - start) // step + 1)
        for k, bound in ((0, lambda ref: cnt * u * (cnt * 0.5 + abs(init[0]))), (1, lambda ref: 2 * cnt * u * abs(ref))):
            ref = float.fromhex(c["d3"][k])
            if ref != ref or ref in (float("inf"), float("-inf")):
                assert float(d3[k]).hex() == c["d3"][k], (name, k)
            else:
                assert abs(d3[k] - ref) <= bound(ref), (name, k, d3[k], ref)
        assert float(d3[2]).hex() == c["d3"][2], name
        assert list(i4) == c["i4"], name
        assert float(f1[0]).hex() == c["f1"][0], name
        assert lc[0] == c["lc"], name
