"""Transformed device layouts (the reference's autotransform) through a
program whose ACROSS loop has two dependences and a handler in the shape cdvmh
generates with automatic transforms (workloads/gsd2d*.c/cu): one launch per
diagonal, the array indexed through the header the runtime fills.  With
transforms on, the runtime stores the array diagonalised (slash orientation
when the loop runs its two axes in opposite directions); a mirror loop whose
handler does not ask for transforms reads the array in the natural layout in
between.  Everything is checked bit for bit against the sequential loop."""
import ctypes
import hashlib

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
    w = g.workloads()
    w.wl_gsd2d_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_uint64, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    yield g
    g.set_mode("batched")
    g.runtime().dvmhgb_set_autotransform(1)
    g.runtime().dvmhgb_set_tuning(0)


def run(g, n0, n1, sweeps, seed, dirs=(1, 1), read_each=1, mirror=0):
    m = np.zeros(sweeps)
    a = np.zeros(n0 * n1)
    b = np.zeros(n0 * n1)
    g.reset_stats()
    assert g.workloads().wl_gsd2d_run(n0, n1, sweeps, seed, dirs[0], dirs[1], read_each, mirror, orc.P(m), orc.P(a),
                                      orc.P(b)) == 0
    return m, a, b, g.stats()


def check(m, a, b, n0, n1, sweeps, seed, dirs, read_each, mirror):
    m_ref, a_ref = orc.gsd2d_run(n0, n1, sweeps, seed, dirs[0], dirs[1])
    assert np.array_equal(a, a_ref)
    if read_each:
        assert np.array_equal(m, m_ref)
    else:
        assert m[0] == m_ref[-1]
    if mirror:
        assert np.array_equal(b, a_ref * 2.0)


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x, dtype="<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
def test_golden(g, golden, mode, tfm):
    """The reference runtime's own outputs (its host handlers, sequential
    order) for the program, with and without transformed layouts."""
    g.set_mode(mode)
    g.runtime().dvmhgb_set_autotransform(tfm)
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "gsd2d"]
    assert cases
    for name, c in cases:
        n0, n1, sw, seed, d0, d1, mirror = c["params"]
        m, a, b, _ = run(g, n0, n1, sw, seed, dirs=(d0, d1), read_each=1, mirror=mirror)
        assert [float(x).hex() for x in m] == c["m"], name
        assert sha(a) == c["A_sha256"], name
        if mirror:
            assert sha(b) == c["B_sha256"], name


@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
@pytest.mark.parametrize("prog", ["rec2d", "gsd3d", "gs2d"])
def test_golden_other_programs(g, golden, mode, tfm, prog):
    """The reference runtime's outputs for the one-dependence recurrence
    (permuted layout), the rank-3 program (diagonal plane under an outer
    axis) and the one-thread Gauss-Seidel handler."""
    g.set_mode(mode)
    g.runtime().dvmhgb_set_autotransform(tfm)
    w = g.workloads()
    D, U, L = ctypes.POINTER(ctypes.c_double), ctypes.c_uint64, ctypes.c_long
    w.wl_rec2d_run.argtypes = [L, L, L, U, D, D]
    w.wl_gsd3d_run.argtypes = [L, L, L, L, U, D, D]
    w.wl_gs2d_run.argtypes = [L, L, U, D, D]
    cases = [(k, c) for k, c in golden.items() if c["prog"] == prog]
    assert cases
    for name, c in cases:
        p = c["params"]
        sw = p[{"rec2d": 2, "gsd3d": 3, "gs2d": 1}[prog]]
        cells = {"rec2d": p[0] * p[1], "gsd3d": p[0] * p[1] * p[2], "gs2d": p[0] * p[0]}[prog]
        r = np.zeros(sw)
        a = np.zeros(cells)
        assert getattr(w, "wl_%s_run" % prog)(*p, orc.P(r), orc.P(a)) == 0
        assert [float(x).hex() for x in r] == c["r"], name
        assert sha(a) == c["A_sha256"], name


@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
def test_modes_and_switch(g, mode, tfm):
    g.set_mode(mode)
    g.runtime().dvmhgb_set_autotransform(tfm)
    n0, n1, sweeps, seed = 40, 40, 3, 11
    m, a, b, s = run(g, n0, n1, sweeps, seed, read_each=1, mirror=1)
    check(m, a, b, n0, n1, sweeps, seed, (1, 1), 1, 1)
    if tfm:
        # every sweep diagonalises A, every mirror loop makes it natural again (counted when
        # run or captured; a replayed graph repeats them without counting)
        assert s["relayouts"] >= (2 * sweeps if mode != "batched" else 2), s
    else:
        assert s["relayouts"] == 0, s


@pytest.mark.parametrize("dirs", [(1, 1), (-1, 1), (1, -1), (-1, -1)])
@pytest.mark.parametrize("shape", [(23, 23), (17, 41), (41, 17)])
def test_directions_and_shapes(g, dirs, shape):
    g.set_mode("batched")
    g.runtime().dvmhgb_set_autotransform(1)
    n0, n1 = shape
    m, a, b, s = run(g, n0, n1, 4, 5, dirs=dirs, read_each=0, mirror=0)
    check(m, a, b, n0, n1, 4, 5, dirs, 0, 0)
    # one relayout to the diagonal layout for the whole time loop, one back for get_actual
    assert s["relayouts"] == 2, s


def test_graph_replays_keep_layouts(g):
    # the same queue replayed: captured relayouts and swaps are replayed with their layouts
    g.set_mode("batched")
    g.runtime().dvmhgb_set_autotransform(1)
    n0, n1, sweeps, seed = 33, 26, 6, 3
    m, a, b, s = run(g, n0, n1, sweeps, seed, dirs=(-1, 1), read_each=1, mirror=1)
    check(m, a, b, n0, n1, sweeps, seed, (-1, 1), 1, 1)
    assert s["graph_replays"] > 0, s


def test_larger_grid_int_and_long_index(g):
    g.set_mode("batched")
    g.runtime().dvmhgb_set_autotransform(1)
    n0, n1, sweeps, seed = 300, 257, 2, 8
    m, a, b, s = run(g, n0, n1, sweeps, seed, dirs=(1, -1), read_each=1, mirror=0)
    check(m, a, b, n0, n1, sweeps, seed, (1, -1), 1, 0)


def test_tuner_chooses_layout(g):
    # tuning on: the loop runs twice transformed, twice natural, then keeps the faster layout;
    # the results stay exact whichever layout each sweep ran in
    rt, w = g.runtime(), g.workloads()
    rt.dvmhgb_tuner_layout.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    rt.dvmhgb_tuner_layout.restype = ctypes.c_int
    handler = ctypes.cast(w.loop_gsd2d_cuda, ctypes.c_void_p)
    g.set_mode("plain")
    rt.dvmhgb_set_autotransform(1)
    rt.dvmhgb_set_tuning(1)
    try:
        n0, n1, sweeps, seed = 64, 48, 7, 21
        m, a, b, s = run(g, n0, n1, sweeps, seed, dirs=(1, -1), read_each=1, mirror=0)
        check(m, a, b, n0, n1, sweeps, seed, (1, -1), 1, 0)
        best = (ctypes.c_double * 2)()
        choice = rt.dvmhgb_tuner_layout(handler, best)
        assert choice in (0, 1), (choice, list(best))
        assert best[0] > 0 and best[1] > 0
        # transformed for two sweeps, natural for two, then the choice (plus get_actual)
        assert s["relayouts"] >= 2, s
    finally:
        rt.dvmhgb_set_tuning(0)
        g.set_mode("batched")


def rec2d_sequential(n0, n1, sweeps, seed):
    L = orc.lib()
    a = np.array([[L.orc_u01(seed, 19, i * n1 + j) for j in range(n1)] for i in range(n0)])
    los = []
    for _ in range(sweeps):
        for j in range(1, n1):
            a[:, j] = a[:, j] * 0.5 + a[:, j - 1] * 0.25
        los.append(min(a[:, 1:].min(), 1.0))  # MIN of the loop, then the initial value 1.0
    return np.array(los), a


@pytest.mark.parametrize("mode", ["plain", "async", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
def test_one_dependence_permuted(g, mode, tfm):
    # a recurrence along j over independent rows: with transforms the rows' axis is stored
    # innermost (a permuted layout, header state 1), so the threads of one launch are adjacent
    g.set_mode(mode)
    rt, w = g.runtime(), g.workloads()
    rt.dvmhgb_set_autotransform(tfm)
    w.wl_rec2d_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_uint64,
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    n0, n1, sweeps, seed = 37, 52, 3, 4
    lo = np.zeros(sweeps)
    a = np.zeros(n0 * n1)
    g.reset_stats()
    assert w.wl_rec2d_run(n0, n1, sweeps, seed, orc.P(lo), orc.P(a)) == 0
    s = g.stats()
    lo_ref, a_ref = rec2d_sequential(n0, n1, sweeps, seed)
    assert np.array_equal(a.reshape(n0, n1), a_ref)
    assert np.array_equal(lo, lo_ref)
    # transposed once for the time loop, back once for get_actual
    assert s["relayouts"] == (2 if tfm else 0), s


@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
def test_two_dependences_with_an_outer_axis(g, mode, tfm):
    # rank 3: the two dependent axes diagonalised as one plane, the independent outer axis
    # striding over whole planes; every plane is the 2-D program with its own seed
    g.set_mode(mode)
    rt, w = g.runtime(), g.workloads()
    rt.dvmhgb_set_autotransform(tfm)
    w.wl_gsd3d_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_uint64,
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    n0, n1, n2, sweeps, seed = 5, 19, 27, 3, 40
    m = np.zeros(sweeps)
    a = np.zeros(n0 * n1 * n2)
    g.reset_stats()
    assert w.wl_gsd3d_run(n0, n1, n2, sweeps, seed, orc.P(m), orc.P(a)) == 0
    s = g.stats()
    planes = [orc.gsd2d_run(n1, n2, sweeps, seed + k) for k in range(n0)]
    assert np.array_equal(a.reshape(n0, n1 * n2), np.stack([p[1] for p in planes]))
    assert np.array_equal(m, np.max(np.stack([p[0] for p in planes]), axis=0))
    assert s["relayouts"] == (2 if tfm else 0), s


@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("tfm", [1, 0])
@pytest.mark.parametrize("reduce", [0, 1])
@pytest.mark.parametrize("shape,moved", [((3, 30), True), ((30, 3), False), ((3, 3), False)])
def test_dispatcher_single_iteration_axes(g, mode, tfm, reduce, shape, moved):
    # a dependent axis with one iteration keeps its dependence (the reference's default) and
    # the generated handler's dispatcher takes the two-dependence case; with dependences
    # reduced it has none, the dispatcher counts one and takes the one-dependence case, and
    # with the rows' axis the only independent one (3 x n) the reference's rule stores it
    # innermost (a transposed layout).  The results are the sequential loop's either way.
    rt = g.runtime()
    g.set_mode(mode)
    rt.dvmhgb_set_autotransform(tfm)
    rt.dvmhgb_set_reduce_dependences(reduce)
    try:
        n0, n1 = shape
        m, a, b, s = run(g, n0, n1, 3, 6, dirs=(1, -1), read_each=1, mirror=1)
        check(m, a, b, n0, n1, 3, 6, (1, -1), 1, 1)
        if not tfm:
            assert s["relayouts"] == 0, s
        elif not reduce or moved:
            # two dependences: the array's plane is diagonalised; one: the rows' axis goes innermost
            assert s["relayouts"] >= 2, s
        else:
            # one dependence, and the array's innermost axis already follows the independent loop axis
            assert s["relayouts"] == 0, s
    finally:
        rt.dvmhgb_set_reduce_dependences(0)


def test_freed_arrays_leave_no_cached_graphs(g):
    # a program run twice: the second run's arrays reuse the first run's descriptors and
    # (pooled) device buffers, but graphs recorded for the freed arrays are not replayed
    g.set_mode("batched")
    g.runtime().dvmhgb_set_autotransform(1)
    n0, n1, sweeps, seed = 24, 20, 3, 12
    for rep in range(2):
        m, a, b, s = run(g, n0, n1, sweeps, seed, dirs=(1, 1), read_each=1, mirror=1)
        check(m, a, b, n0, n1, sweeps, seed, (1, 1), 1, 1)
        assert s["graphs_captured"] >= 1, (rep, s)
