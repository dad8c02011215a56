"""The reduction fold's tree, modelled on the CPU.

The runtime folds reduction partials by a fixed pairwise tree over item
indices: item a is combined with item a + w (a a multiple of 2w), the lower
index as the destination, with the operation's identity beyond the last item.
The shared-memory kernel does it in passes over aligned spans of 1024 items,
the bandwidth-bound kernels (rt_device.cu kFold2 / kFoldSeg*) over aligned
spans of 2048.  A larger span only adds levels that combine a node with the
identity, which leaves it unchanged for SUM, PROD, MIN, MAX, AND, OR, XOR and
the LOC pairs, signed zeros, infinities and NaN included.  This model checks
that claim on such data, with the combine rules of loop.cpp:116-238 (strict
compares, the lower index winning ties, identity slots never winning)."""
import numpy as np
import pytest

SUM, PROD, MAX, MIN, AND, OR, XOR, MINLOC, MAXLOC = range(9)


def identity(op, dtype):
    if op == SUM:
        return dtype.type(-0.0) if dtype.kind == "f" else dtype.type(0)
    if op == PROD:
        return dtype.type(1)
    if op in (MAX, MAXLOC):
        return dtype.type(-np.inf) if dtype.kind == "f" else np.iinfo(dtype).min
    if op in (MIN, MINLOC):
        return dtype.type(np.inf) if dtype.kind == "f" else np.iinfo(dtype).max
    if op == AND:
        return dtype.type(-1)
    return dtype.type(0)


def level(op, d, s, di, si):
    """one tree level: d (+)= s elementwise; returns values and indices"""
    if op == SUM:
        return d + s, di
    if op == PROD:
        return d * s, di
    if op == MAX:
        return np.where(d < s, s, d), di
    if op == MIN:
        return np.where(d > s, s, d), di
    if op == AND:
        return d & s, di
    if op == OR:
        return d | s, di
    if op == XOR:
        return d ^ s, di
    better = (d < s) if op == MAXLOC else (d > s)
    take = ((di < 0) & (si >= 0)) | ((si >= 0) & better)
    return np.where(take, s, d), np.where(take, si, di)


def fold(v, op, span):
    """multi-pass fold over aligned spans of `span` items, as the kernels run it"""
    v = np.asarray(v)
    vi = np.arange(len(v), dtype=np.int64)
    ident = identity(op, v.dtype)
    while True:
        n = len(v)
        blocks = max(1, -(-n // span))
        pad = blocks * span - n
        pv = np.concatenate([v, np.full(pad, ident, dtype=v.dtype)])
        pi = np.concatenate([vi, np.full(pad, -1, dtype=np.int64)])
        w = 1
        while w < span:
            # pairs (a, a + w) for a a multiple of 2w, inside each span
            d, s = pv[0::2 * w], pv[w::2 * w]
            di, si = pi[0::2 * w], pi[w::2 * w]
            with np.errstate(all="ignore"):  # inf * 0, inf - inf, NaN compares: IEEE results wanted
                nv, ni = level(op, d, s, di, si)
            pv, pi = pv.copy(), pi.copy()
            pv[0::2 * w], pi[0::2 * w] = nv, ni
            w *= 2
        v, vi = pv[0::span], pi[0::span]
        if n <= span:
            return v[0], vi[0]


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        return (np.isnan(a) and np.isnan(b)) or a.tobytes() == b.tobytes()
    return a == b


def data(kind, n, rng):
    if kind == "f8" or kind == "f4":
        dt = np.float64 if kind == "f8" else np.float32
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324 if kind == "f8" else 1e-45, 1.0, -1.0],
                            dtype=dt)
        v = rng.standard_normal(n).astype(dt)
        mask = rng.random(n) < 0.3
        v[mask] = specials[rng.integers(0, len(specials), mask.sum())]
        return v
    return rng.integers(-2 ** 31, 2 ** 31, n, dtype=np.int64).astype(np.int32)


SIZES = [1, 2, 7, 1023, 1024, 1025, 2047, 2048, 2049, 5000, 1024 * 1024 + 3, 2048 * 2048 + 5]


@pytest.mark.parametrize("op", [SUM, PROD, MAX, MIN, MINLOC, MAXLOC])
@pytest.mark.parametrize("kind", ["f8", "f4"])
def test_span_2048_equals_span_1024_float(op, kind):
    rng = np.random.default_rng(op * 10 + len(kind))
    for n in SIZES:
        v = data(kind, n, rng)
        a, ai = fold(v, op, 1024)
        b, bi = fold(v, op, 2048)
        assert same(a, b), (op, kind, n, a, b)
        if op in (MINLOC, MAXLOC):
            assert ai == bi, (op, kind, n)


@pytest.mark.parametrize("op", [SUM, MAX, MIN, AND, OR, XOR, MINLOC])
def test_span_2048_equals_span_1024_int(op):
    rng = np.random.default_rng(100 + op)
    for n in SIZES[:10]:
        v = data("i4", n, rng)
        a, ai = fold(v, op, 1024)
        b, bi = fold(v, op, 2048)
        assert a == b, (op, n)
        if op == MINLOC:
            assert ai == bi, (op, n)


def test_signed_zero_max_keeps_the_first():
    # the lower index wins a tie: MAX over [-0, +0, -0] is the first zero, as in loop order
    v = np.array([-0.0, 0.0, -0.0] * 700)
    r, _ = fold(v, MAX, 2048)
    assert np.signbit(r)
    r, _ = fold(v[1:], MAX, 2048)
    assert not np.signbit(r)


def test_minloc_ties_take_the_lowest_index():
    v = np.full(5000, 0.5)
    v[[17, 4000, 4999]] = 0.25
    r, ri = fold(v, MINLOC, 2048)
    assert r == 0.25 and ri == 17
