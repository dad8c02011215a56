"""Handlers in the exact shape cdvmh generates run unmodified on this runtime.

gen3d_cuda.cu is a CUDA handler written to the generated template
(cdvmh/src/converter_main.cpp:2132-2401, kernel :1861-2130), knowing nothing
of this runtime:

- the block comes from dvmh_loop_cuda_get_config_C;
- the block counts blocksS[d] are products over the inner axes;
- red_prepare gets one slot per launched thread;
- launches are at most 65535 blocks with a block offset;
- the kernel runs one loop point per thread and writes every thread's private
  reduction values to its slot.

The runtime must give it correct headers, bounds, device scalars and
reduction buffers, and fold its per-thread slots.  The array must be
bit-exact and MAXLOC (value, location) exact.  The SUM must be bit-exact
against the fold the runtime defines: pairwise over slot indices, padded
with -0.0, then (+0.0 + T) + the initial value.  These checks run for user
blocks of every rank, the default block, and all three modes."""
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


def init_a(n0, n1, n2, seed):
    L = orc.lib()
    return np.array([L.orc_u01(seed, 7, x) for x in range(n0 * n1 * n2)]).reshape(n0, n1, n2)


def pairwise(v):
    m = 1
    while m < len(v):
        m *= 2
    v = np.concatenate([v, np.full(m - len(v), -0.0)])
    while len(v) > 1:
        v = v[0::2] + v[1::2]
    return float(v[0])


def expected_sum(b, block, s_init):
    """The handler's per-thread slots, folded as the runtime folds them."""
    bx, by, bz = block
    n0, n1, n2 = (x - 2 for x in b.shape)
    s2 = -(-n2 // bx)
    s1 = s2 * -(-n1 // by)
    s0 = s1 * -(-n0 // bz)
    blk = np.repeat(np.arange(s0), bx * by * bz)
    t = np.tile(np.arange(bx * by * bz), s0)
    tx, ty, tz = t % bx, (t // bx) % by, t // (bx * by)
    cb0 = blk // s1
    rem = blk - cb0 * s1
    cb1 = rem // s2
    cb2 = rem - cb1 * s2
    i, j, k = 1 + cb0 * bz + tz, 1 + cb1 * by + ty, 1 + cb2 * bx + tx
    ok = (i <= n0) & (j <= n1) & (k <= n2)
    slots = np.full(len(t), -0.0)
    slots[ok] = -0.0 + b[i[ok], j[ok], k[ok]]  # the private SUM starts at the identity -0.0
    return (0.0 + pairwise(slots)) + s_init


@pytest.mark.parametrize("shape,block", [
    ((20, 37, 70), (32, 4, 2)),
    ((20, 37, 70), (16, 8, 1)),
    ((9, 130, 33), (64, 2, 2)),
    ((33, 5, 200), (128, 1, 1)),
    ((17, 19, 23), (0, 0, 0)),  # the runtime's default block for rank 3
])
@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
def test_generated_shape_handler(g, shape, block, mode):
    g.set_mode(mode)
    n0, n1, n2 = shape
    seed = 31 + n0 + n1 + n2
    w = g.workloads()
    w.wl_gen3d_run.argtypes = [ctypes.c_long] * 3 + [ctypes.c_uint64] + [ctypes.c_int] * 3 + [
        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_long),
        ctypes.POINTER(ctypes.c_double)]
    s, mx, lc = ctypes.c_double(0.25), ctypes.c_double(0.5), ctypes.c_long(-7)
    bout = np.zeros(n0 * n1 * n2)
    assert w.wl_gen3d_run(n0, n1, n2, seed, *block, ctypes.byref(s), ctypes.byref(mx), ctypes.byref(lc),
                          bout.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    a = init_a(n0, n1, n2, seed)
    b = np.zeros_like(a)
    b[1:-1, 1:-1, 1:-1] = a[:-2, 1:-1, 1:-1] + 0.5 * a[1:-1, 1:-1, 2:]
    assert np.array_equal(bout.reshape(shape), b), (mode, shape, block)
    inner = b[1:-1, 1:-1, 1:-1]
    q = np.unravel_index(int(np.argmax(inner)), inner.shape)
    vmax = inner[q]
    assert mx.value == max(vmax, 0.5)
    assert lc.value == (((q[0] + 1) * n1 + q[1] + 1) * n2 + q[2] + 1 if vmax > 0.5 else -7)
    blk = block if block[0] else (32, 4, 2)
    assert s.value == expected_sum(b, blk, 0.25), (mode, shape, block)


@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("block", [(0, 0, 0), (64, 2, 1)])
def test_reference_golden(g, golden, mode, block):
    """The reference runtime's own results (host handler, loop order): B and
    MAXLOC bit for bit; SUM, folded per thread here, within n * 2^-53 * sum |b|
    of the reference's sequential value (all terms positive)."""
    import hashlib
    g.set_mode(mode)
    w = g.workloads()
    w.wl_gen3d_run.argtypes = [ctypes.c_long] * 3 + [ctypes.c_uint64] + [ctypes.c_int] * 3 + [
        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_long),
        ctypes.POINTER(ctypes.c_double)]
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "gen3d"]
    assert cases
    for name, c in cases:
        n0, n1, n2, seed, s0, mx0, lc0 = c["params"]
        s, mx, lc = ctypes.c_double(s0), ctypes.c_double(mx0), ctypes.c_long(lc0)
        bout = np.zeros(n0 * n1 * n2)
        assert w.wl_gen3d_run(n0, n1, n2, seed, *block, ctypes.byref(s), ctypes.byref(mx), ctypes.byref(lc),
                              bout.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        assert hashlib.sha256(bout.astype("<f8").tobytes()).hexdigest() == c["B_sha256"], name
        assert mx.value.hex() == c["s_mx"][1] and lc.value == c["lc"], name
        ref_s = float.fromhex(c["s_mx"][0])
        cnt = max(0, (n0 - 2) * (n1 - 2) * (n2 - 2))
        assert abs(s.value - ref_s) <= cnt * 2.0 ** -53 * (float(np.abs(bout).sum()) + abs(s0)), name
