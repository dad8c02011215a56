"""Jacobi 2-D/3-D through the dvmh_* C ABI on the GPU, against the reference's
golden outputs and the CPU oracle, bit for bit, in every execution mode."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc
from tests.util import J3_FUSED, J3_IN_PLACE, J3_ONE_PASS_Q, J3_STENCILS, J3_STNUPD, sha, unhex

pytestmark = pytest.mark.gpu

MODES = ["plain", "async", "batched"]


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    yield g
    g.set_mode("batched")


@pytest.mark.parametrize("mode", MODES)
def test_jacobi_golden(g, golden, mode):
    g.set_mode(mode)
    for name, c in golden.items():
        if c["prog"] not in ("jac2d", "jac3d") or c["params"][0] > 200:
            continue
        rank = 2 if c["prog"] == "jac2d" else 3
        n, it, seed = c["params"]
        j = g.Jacobi(rank, n, seed)
        eps = j.run(it)
        A, B = j.fetch()
        j.close()
        assert np.array_equal(eps, unhex(c["eps"])), (name, mode)
        assert sha(A) == c["A_sha256"] and sha(B) == c["B_sha256"], (name, mode)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_jacobi3d_generated_handlers_golden(g, golden, mode):
    """The FP64 Jacobi-3D program through cdvmh's generated one-point-per-thread
    handlers (jacperf_cuda.cu: one MAX slot per launched thread) instead of the
    library's kernels: the same golden outputs, bit for bit."""
    import ctypes
    g.set_mode(mode)
    w = g.workloads()
    w.wl_jac3d_use_generated.argtypes = [ctypes.c_int]
    w.wl_jac3d_use_generated(1)
    try:
        for name, c in golden.items():
            if c["prog"] != "jac3d" or c["params"][0] > 200:
                continue
            n, it, seed = c["params"]
            j = g.Jacobi(3, n, seed)
            eps = j.run(it)
            A, B = j.fetch()
            j.close()
            assert np.array_equal(eps, unhex(c["eps"])), (name, mode)
            assert sha(A) == c["A_sha256"] and sha(B) == c["B_sha256"], (name, mode)
    finally:
        w.wl_jac3d_use_generated(0)


def test_jacobi2d_cpu_config_golden(g, golden):
    """The reference's CPU configuration (1024^2, 100 iterations) on the GPU path."""
    c = golden["jac2d_n1024_it100"]
    n, it, seed = c["params"]
    g.set_mode("batched")
    j = g.Jacobi(2, n, seed)
    eps = j.run(it)
    A, B = j.fetch()
    j.close()
    assert np.array_equal(eps, unhex(c["eps"]))
    assert sha(A) == c["A_sha256"] and sha(B) == c["B_sha256"]


@pytest.mark.parametrize("rank,n,iters", [(3, 5, 2), (3, 33, 4), (3, 66, 3), (3, 129, 2), (2, 5, 3), (2, 6, 3),
                                          (2, 7, 2), (2, 11, 4), (2, 65, 6), (2, 300, 5), (2, 1027, 2)])
def test_jacobi_vs_oracle_sizes(g, rank, n, iters):
    """Ragged sizes: extents around the 64-element tiles and the 2-D kernels' row chunks
    (4 rows at the least: interiors of 3, 4, 5, 9 and 1025 rows)."""
    seed = 1000 + n
    e_ref, A_ref, B_ref = orc.jacobi_run(rank, n, iters, seed, threads=8)
    for mode in MODES:
        g.set_mode(mode)
        j = g.Jacobi(rank, n, seed)
        eps = j.run(iters)
        A, B = j.fetch()
        j.close()
        assert np.array_equal(eps, e_ref), (mode, n)
        assert np.array_equal(A, A_ref) and np.array_equal(B, B_ref), (mode, n)


def test_jacobi3d_512_matches_oracle(g):
    """Full-size grid of the 3-D configuration, 3 iterations, against the CPU oracle."""
    n, iters, seed = 512, 3, 20261203
    e_ref, A_ref, B_ref = orc.jacobi_run(3, n, iters, seed, threads=16)
    g.set_mode("batched")
    j = g.Jacobi(3, n, seed)
    eps = j.run(iters)
    A, B = j.fetch()
    j.close()
    assert np.array_equal(eps, e_ref)
    assert np.array_equal(A, A_ref) and np.array_equal(B, B_ref)


def test_batched_mode_fuses_and_replays(g):
    g.set_mode("batched")
    j = g.Jacobi(3, 40, 5)
    g.reset_stats()
    j.run(6)
    s = g.stats()
    j.close()
    assert s["loops_performed"] == 12
    assert s["fused_pairs"] >= 1
    # one group per step: the first step's update alone, then each step's stencil with the next step's update
    # (deferral); the first pair allocates A's second buffer, afterwards the two buffers of A alternate
    assert s["graphs_captured"] <= 4
    assert s["graphs_captured"] + s["graph_replays"] == 6 and s["graph_replays"] >= 2


def test_plain_mode_no_fusion(g):
    g.set_mode("plain")
    j = g.Jacobi(3, 40, 5)
    g.reset_stats()
    j.run(3)
    s = g.stats()
    j.close()
    g.set_mode("batched")
    assert s["fused_pairs"] == 0 and s["graphs_captured"] == 0 and s["handler_calls"] == 6


@pytest.mark.parametrize("variant", list(range(J3_FUSED)))
def test_jacobi3d_variants_vs_oracle(g, variant):
    """Every kernel variant of the 3-D loops (rows per thread x additions on the
    FP64 unit, the rest on the integer pipe; the fixed-point stencils; the
    unfused and overlapped pairs) through the program, plain (separate update
    and stencil loops) and batched (the fused loop: deferral off, so that each
    step's update and stencil meet in one flush)."""
    try:
        g.set_deferral(False)
        g.force_variant(variant)
        for n, iters in ((19, 4), (66, 3), (131, 2)):
            e_ref, A_ref, B_ref = orc.jacobi_run(3, n, iters, 900 + n)
            for mode in ("plain", "batched"):
                g.set_mode(mode)
                j = g.Jacobi(3, n, 900 + n)
                eps = j.run(iters)
                A, B = j.fetch()
                j.close()
                assert np.array_equal(eps, e_ref), (variant, n, mode)
                assert np.array_equal(A, A_ref) and np.array_equal(B, B_ref), (variant, n, mode)
    finally:
        g.force_variant(-1)
        g.set_deferral(True)


@pytest.mark.parametrize("variant", [-1] + list(range(J3_STNUPD)))
def test_jacobi3d_stencil_then_next_update(g, variant):
    """Batched mode with deferral (the default): each step's stencil, naming
    arrays only, waits past its region for the next step's update loop, and the
    fusion rule runs the two as one pass (dvmhgb_jac3d_stnupd: |B - A| and
    A = B on the new B, A's second buffer swapped in).  eps of every step and
    the final A, B bit-exact against the oracle; one such pair (run, or its
    captured graph replayed) per step after the first."""
    try:
        g.force_variant(variant)
        for n, iters in ((19, 4), (66, 5), (131, 3)):
            e_ref, A_ref, B_ref = orc.jacobi_run(3, n, iters, 700 + n)
            g.set_mode("batched")
            j = g.Jacobi(3, n, 700 + n)
            g.reset_stats()
            eps = j.run(iters)
            st = g.stats()
            A, B = j.fetch()
            j.close()
            assert np.array_equal(eps, e_ref), (variant, n)
            assert np.array_equal(A, A_ref) and np.array_equal(B, B_ref), (variant, n)
            # every step after the first is one group (a captured graph, replayed once it repeats): the pair
            assert st["fused_pairs"] >= 1 and st["fused_pairs"] + st["graph_replays"] == iters - 1, (variant, n, st)
    finally:
        g.force_variant(-1)


def test_deferred_stencil_meets_other_programs(g):
    """Batched mode with deferral, the 3-D and 2-D Jacobi programs stepping in
    turn: the 3-D step's stencil waits in the queue, the 2-D step's loops
    (which start no deferrable rule) come after it and its region's end runs
    the queue through them, so the 3-D stencil runs alone there and the next
    3-D update runs alone too.  Every eps and the final arrays of both
    programs bit-exact against the oracle; then a mode change and the arrays'
    fetch run whatever is still queued."""
    e3, A3, B3 = orc.jacobi_run(3, 40, 4, 71)
    e2, A2, B2 = orc.jacobi_run(2, 70, 4, 72)
    g.set_mode("batched")
    j3 = g.Jacobi(3, 40, 71)
    j2 = g.Jacobi(2, 70, 72)
    got3, got2 = [], []
    try:
        for _ in range(4):
            got3.append(j3.run(1)[0])
            got2.append(j2.run(1)[0])
        g.set_mode("async")  # a mode change runs the 3-D stencil still queued
        g.set_mode("batched")
        A, B = j3.fetch()
        a, b = j2.fetch()
    finally:
        j3.close()
        j2.close()
    assert np.array_equal(np.array(got3), e3) and np.array_equal(np.array(got2), e2)
    assert np.array_equal(A, A3) and np.array_equal(B, B3)
    assert np.array_equal(a, A2) and np.array_equal(b, B2)


@pytest.mark.parametrize("variant", list(range(J3_STNUPD)))
def test_jacobi3d_stnupd_kernel_sub_box(g, variant):
    """dvmhgb_jac3d_stnupd through the C ABI over a box with array cells
    outside it on every side: B = stencil(A) inside the box (outside untouched),
    eps = max |B_new - A| over the box, Aalt = B_new inside the box and A's
    values outside it; values mostly in the fixed-point range, a few outside
    (planes on the FP64 unit).  Bit-exact against float64 on the CPU."""
    import ctypes
    import torch
    L = g.runtime()
    L.dvmhgb_jac3d_stnupd_items.restype = ctypes.c_long
    n0, n1, n2 = 30, 45, 202
    LA = ctypes.c_long * 3
    lo_, hi_ = (3, 5, 7), (25, 38, 190)
    st, ext, lo, hi = LA(n1 * n2, n2, 1), LA(n0, n1, n2), LA(*lo_), LA(*hi_)
    gen = torch.Generator().manual_seed(500 + variant)
    A = 0.25 + 0.5 * torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B = torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    A[17, 20, 100], A[9, 30, 60], A[2, 10, 50] = -0.5, 3.0, 1.25  # outside the range
    # in range, but the new B of cell (10, 20, 100) falls below it: 2^-9 / 6 (|B - A| on the FP64 unit)
    A[9, 20, 100], A[11, 20, 100], A[10, 19, 100], A[10, 21, 100], A[10, 20, 99], A[10, 20, 101] = \
        2.0 ** -9, 0.0, 0.0, 0.0, 0.0, 0.0
    Ad, Bd = A.cuda(), B.cuda()
    Aalt = torch.full_like(Ad, 7.0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    items = torch.empty(L.dvmhgb_jac3d_stnupd_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.dvmhgb_jac3d_stnupd(vp(Ad), vp(Aalt), vp(Bd), st, ext, lo, hi, vp(items), variant, sp) == 0
    torch.cuda.synchronize()
    box = tuple(slice(a, b + 1) for a, b in zip(lo_, hi_))
    inner = tuple(slice(a - 1, b) for a, b in zip(lo_, hi_))
    s_ref, _ = _stencil_ref(A)
    Bw = B.clone()
    Bw[box] = s_ref[inner]
    Aw = A.clone()
    Aw[box] = s_ref[inner]
    eps_ref = (s_ref[inner] - A[box]).abs().max().item()
    assert torch.equal(Bd.cpu().view(torch.int64), Bw.view(torch.int64)), variant
    assert torch.equal(Aalt.cpu().view(torch.int64), Aw.view(torch.int64)), variant
    assert torch.equal(Ad.cpu(), A), variant  # the source is only read
    assert items.max().item() == eps_ref, variant


def _stencil_ref(A):
    """(A[i-1]+A[j-1]+A[k-1]+A[k+1]+A[j+1]+A[i+1]) / 6 over the interior, float64
    on the CPU, one IEEE operation at a time in the source order."""
    c = A[1:-1, 1:-1, 1:-1]
    t = A[:-2, 1:-1, 1:-1] + A[1:-1, :-2, 1:-1]
    t = t + A[1:-1, 1:-1, :-2]
    t = t + A[1:-1, 1:-1, 2:]
    t = t + A[1:-1, 2:, 1:-1]
    t = t + A[2:, 1:-1, 1:-1]
    return t / 6.0, c


@pytest.mark.parametrize("variant", list(range(J3_STENCILS)) + J3_ONE_PASS_Q)
def test_jacobi3d_kernels_signs_and_tiny_values(g, variant):
    """The kernels directly through the C ABI on values that take every path:
    negative values (no integer-pipe additions for that CTA), values below
    2^-12 and zeros (the FP64-unit fallback of the fixed-point MAX), and
    ordinary [0, 1) values; A, Bnew and eps bit-exact against float64 on the CPU."""
    import ctypes
    import torch
    L = g.runtime()
    L.dvmhgb_jac3d_fused_items.restype = ctypes.c_long
    n0, n1, n2 = 23, 37, 150  # row pitch 150: 16-byte aligned rows
    LA = ctypes.c_long * 3
    st, ext, lo, hi = LA(n1 * n2, n2, 1), LA(n0, n1, n2), LA(1, 1, 1), LA(n0 - 2, n1 - 2, n2 - 2)
    gen = torch.Generator().manual_seed(variant)
    A = torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B = torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B[3:9, :, :40] -= 0.5  # negative values in some tiles
    B[12:, 20:, 64:90] *= 2.0 ** -20  # tiny values
    A[12:, 20:, 64:70] = 0.0
    B[5, 5, 100], A[5, 5, 100] = 0.999, 2.0 ** -40  # the largest |B - A|: A below the fixed-point range
    Ad, Bd = A.cuda(), B.cuda()
    Bnew = torch.full_like(Bd, 7.0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    items = torch.empty(L.dvmhgb_jac3d_fused_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.dvmhgb_jac3d_fused(vp(Ad), vp(Bd), vp(Bnew), st, ext, lo, hi, vp(items), variant, sp) == 0
    Bs = torch.full_like(Bd, 7.0)
    sv = variant if variant < J3_STENCILS else 14  # the one-pass fixed-point pair has no stencil-only form
    assert L.dvmhgb_jac3d_stencil(vp(Bd), vp(Bs), st, ext, lo, hi, sv, sp) == 0
    torch.cuda.synchronize()
    # reference: update on the interior, then the stencil of the updated A
    An = A.clone()
    An[1:-1, 1:-1, 1:-1] = B[1:-1, 1:-1, 1:-1]
    eps_ref = (B[1:-1, 1:-1, 1:-1] - A[1:-1, 1:-1, 1:-1]).abs().max().item()
    s_ref, _ = _stencil_ref(An)
    assert items.max().item() == eps_ref, variant
    assert torch.equal(Ad.cpu(), An), variant
    assert torch.equal(Bnew.cpu()[1:-1, 1:-1, 1:-1], s_ref), variant
    assert torch.equal(Bnew.cpu()[0], B[0]), variant  # outside the box: B's values
    s2, _ = _stencil_ref(B)
    assert torch.equal(Bs.cpu()[1:-1, 1:-1, 1:-1], s2), variant


@pytest.mark.parametrize("variant", list(range(J3_FUSED)))
def test_jacobi3d_fused_sub_box(g, variant):
    """The update and stencil loops over a box that leaves several planes,
    rows and columns of the array outside it on every side (A != B there), as
    one fused call: A = B and eps inside the box only; the stencil's source is
    B inside the box and A outside it; the next B holds the stencil inside the
    box and B's values outside it.  Values mostly in the fixed-point range, a
    few outside it.  Bit-exact against float64 on the CPU."""
    import ctypes
    import torch
    L = g.runtime()
    L.dvmhgb_jac3d_fused_items.restype = ctypes.c_long
    n0, n1, n2 = 30, 45, 202  # row pitch 202: 16-byte aligned rows
    LA = ctypes.c_long * 3
    lo_, hi_ = (3, 5, 7), (25, 38, 190)
    st, ext, lo, hi = LA(n1 * n2, n2, 1), LA(n0, n1, n2), LA(*lo_), LA(*hi_)
    gen = torch.Generator().manual_seed(300 + variant)
    A = 0.25 + 0.5 * torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B = 0.25 + 0.5 * torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B[17, 20, 100], A[9, 30, 60], A[2, 10, 50] = -0.5, 3.0, 1.25  # outside the range: planes on the FP64 unit
    Ad, Bd = A.cuda(), B.cuda()
    in_place = variant in J3_IN_PLACE  # the two-kernel pairs write the next B over B
    Bnew = Bd if in_place else torch.full_like(Bd, 7.0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    items = torch.empty(L.dvmhgb_jac3d_fused_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.dvmhgb_jac3d_fused(vp(Ad), vp(Bd), vp(Bnew), st, ext, lo, hi, vp(items), variant, sp) == 0
    torch.cuda.synchronize()
    box = tuple(slice(a, b + 1) for a, b in zip(lo_, hi_))
    An = A.clone()
    An[box] = B[box]
    eps_ref = (B[box] - A[box]).abs().max().item()
    s_ref, _ = _stencil_ref(An)
    inner = tuple(slice(a - 1, b) for a, b in zip(lo_, hi_))  # the box in _stencil_ref's interior coordinates
    want = B.clone()
    want[box] = s_ref[inner]
    assert items.max().item() == eps_ref, variant
    assert torch.equal(Ad.cpu(), An), variant
    assert torch.equal(Bnew.cpu().view(torch.int64), want.view(torch.int64)), variant


@pytest.mark.parametrize("native", [0, 1, 2])
def test_jacobi3d_update_kernel_all_paths(g, native):
    """The update loop through the C ABI: |B - A| on the integer pipe (0), the
    FP64 unit (1) and as exact fixed point with its FP64 fallback (2), on
    values that take every path; A and eps bit-exact against float64 on the CPU."""
    import ctypes
    import torch
    L = g.runtime()
    L.dvmhgb_jac3d_update_items.restype = ctypes.c_long
    n0, n1, n2 = 21, 33, 140
    LA = ctypes.c_long * 3
    st, lo, hi = LA(n1 * n2, n2, 1), LA(1, 1, 1), LA(n0 - 2, n1 - 2, n2 - 2)
    gen = torch.Generator().manual_seed(40 + native)
    A = torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B = torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    B[2:5, :, :30] -= 0.7   # negative values
    A[10:, 5:9, 40:70] *= 2.0 ** -30  # below the fixed-point range
    B[6, 7, 8] = 0.0
    B[12, 20, 50], A[12, 20, 50] = 0.9999, 2.0 ** -40  # the largest |B - A|, A out of the fixed-point range
    for case in range(2):
        if case == 1:  # the largest difference among ordinary values only
            A, B = A.abs() % 1.0, B.abs() % 1.0
        Ad, Bd = A.cuda(), B.cuda()
        items = torch.empty(L.dvmhgb_jac3d_update_items(lo, hi), dtype=torch.float64, device="cuda")
        vp = lambda t: ctypes.c_void_p(t.data_ptr())
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        assert L.dvmhgb_jac3d_update(vp(Ad), vp(Bd), st, lo, hi, vp(items), native, sp) == 0
        torch.cuda.synchronize()
        eps_ref = (B[1:-1, 1:-1, 1:-1] - A[1:-1, 1:-1, 1:-1]).abs().max().item()
        An = A.clone()
        An[1:-1, 1:-1, 1:-1] = B[1:-1, 1:-1, 1:-1]
        assert items.max().item() == eps_ref, (native, case)
        assert torch.equal(Ad.cpu(), An), (native, case)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_subarray_actuality(g, mode):
    """dvmh_get_actual_subarray_C brings exactly its box to the host (the rest of
    the host copy stays as it was); dvmh_actual_subarray_C sends a host box to the
    device, whose copy stays whole and current; the program continues from the
    mixed state exactly as the oracle does."""
    import ctypes
    g.set_mode(mode)
    w = g.workloads()
    LA = ctypes.c_long * 3
    n, seed = 20, 4242
    A, B = orc.jacobi_init(3, n, seed)
    A0 = A.copy()
    j = g.Jacobi(3, n, seed)
    j.run(1)
    orc.lib().orc_jacobi_step(3, n, orc.P(A), orc.P(B), 1)
    lo, hi = (2, 3, 4), (9, 7, 15)
    sl = tuple(slice(a, b + 1) for a, b in zip(lo, hi))
    box = np.zeros(int(np.prod([b - a + 1 for a, b in zip(lo, hi)])))
    assert w.wl_jac3d_box(0, 0, LA(*lo), LA(*hi), orc.P(box)) == 0
    A3, A03 = A.reshape(n, n, n), A0.reshape(n, n, n)
    assert np.array_equal(box.reshape(A3[sl].shape), A3[sl])
    peek = np.zeros(n ** 3)
    w.wl_jac3d_host_peek(0, orc.P(peek))
    peek = peek.reshape(n, n, n)
    inside = np.zeros((n, n, n), dtype=bool)
    inside[sl] = True
    assert np.array_equal(peek[inside], A3[inside]) and np.array_equal(peek[~inside], A03[~inside])
    # a host box of B, declared current, then one more step from the mixed state
    lo2, hi2 = (5, 1, 0), (12, 18, 19)
    sl2 = tuple(slice(a, b + 1) for a, b in zip(lo2, hi2))
    vals = np.random.default_rng(7).random(B.reshape(n, n, n)[sl2].shape)
    assert w.wl_jac3d_box(1, 1, LA(*lo2), LA(*hi2), orc.P(np.ascontiguousarray(vals).ravel())) == 0
    B.reshape(n, n, n)[sl2] = vals
    eps = j.run(1)
    e_ref = orc.lib().orc_jacobi_step(3, n, orc.P(A), orc.P(B), 1)
    Ag, Bg = j.fetch()
    j.close()
    assert np.array_equal(Ag, A) and np.array_equal(Bg, B), mode
    assert eps[0] == e_ref, mode


@pytest.mark.parametrize("variant", list(range(14, J3_STENCILS)))
def test_jacobi3d_fixed_point_stencil_range_edges(g, variant):
    """The fixed-point stencil computes a plane on the FP64 unit when any value
    its cells read lies outside +0 and [2^-9, 1).  Values on both sides of
    those limits are planted where each kind of load reads them: a CTA's own
    rows, the j-halo rows above and below it, the k-edge columns left and right
    of its 64-element chunk, the i-planes before and after a chunk of planes,
    and the array's first and last planes.  Bit-exact against float64 on the CPU."""
    import ctypes
    import torch
    L = g.runtime()
    n0, n1, n2 = 70, 41, 200  # row pitch 200: 16-byte aligned rows
    LA = ctypes.c_long * 3
    st, ext, lo, hi = LA(n1 * n2, n2, 1), LA(n0, n1, n2), LA(1, 1, 1), LA(n0 - 2, n1 - 2, n2 - 2)
    gen = torch.Generator().manual_seed(100 + variant)
    A = 0.5 + 0.5 * torch.rand(n0, n1, n2, dtype=torch.float64, generator=gen)
    inside = [2.0 ** -9, 0.9999999999999999, 0.0, 2.0 ** -9 * 1.5]
    outside = [2.0 ** -9 * 0.9999999999999999, 1.0, -0.25, 5e-324, -0.0, 2.0 ** -60, 1.5]
    rng = np.random.default_rng(variant)
    spots = [(1, 1, 1), (n0 - 2, n1 - 2, n2 - 2), (0, 5, 7), (n0 - 1, 9, 70)]
    spots += [(int(i), int(j), int(k)) for i, j, k in zip(rng.integers(0, n0, 40), rng.integers(0, n1, 40),
                                                            rng.integers(0, n2, 40))]
    spots += [(20, 8, 63), (21, 7, 64), (30, 16, 127), (31, 15, 128), (44, 24, 0), (45, 40, 199), (8, 0, 90)]
    for q, (i, j, k) in enumerate(spots):
        A[i, j, k] = (outside if q % 3 else inside)[q % 4 if q % 3 == 0 else q % 7]
    Ad = A.cuda()
    Bs = torch.full_like(Ad, 7.0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.dvmhgb_jac3d_stencil(vp(Ad), vp(Bs), st, ext, lo, hi, variant, sp) == 0
    torch.cuda.synchronize()
    s_ref, _ = _stencil_ref(A)
    got = Bs.cpu()
    assert torch.equal(got[1:-1, 1:-1, 1:-1].view(torch.int64), s_ref.view(torch.int64)), variant
    assert torch.equal(got[0], torch.full_like(got[0], 7.0))  # outside the box: untouched
