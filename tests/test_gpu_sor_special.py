"""The SOR wavefront kernel called directly on caller-owned device memory, on
edge values of IEEE binary64: subnormal, tiny normal and signed-zero cells
(and sums and updates that fall toward the subnormal range) must give the
sequential loop's bits, for every tile depth and for several omegas."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc

pytestmark = pytest.mark.gpu

L3 = ctypes.c_long * 3


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    rt = g.runtime()
    rt.dvmhgb_sor3d_items.restype = ctypes.c_long
    rt.dvmhgb_sor3d_scratch_bytes.restype = ctypes.c_long
    return g


def special_grid(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.random((n, n, n))
    A[0, :, :] = A[-1, :, :] = A[:, 0, :] = A[:, -1, :] = A[:, :, 0] = A[:, :, -1] = 0.0
    specials = [5e-324, -5e-324, 1e-310, 2.0 ** -1021, -(2.0 ** -1022), 0.0, -0.0, 2.0 ** -1020, 3e-308]
    for t, v in enumerate(specials):
        A[2 + t, 3, 4 + t] = v
    A[5:8, 5:8, 5:8] = 1e-308      # a block whose sums and updates fall toward the subnormal range
    A[9:11, 2:4, 12:14] = -2.2e-308
    return A.ravel().copy()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("omega", [1.5, 1.25, 1.0])
def test_sor_kernel_special_values(g, variant, omega):
    import torch
    n = 22
    A0 = special_grid(n, 7 + variant)
    ref = A0.copy()
    canon = np.zeros(1)
    orc.lib().orc_sor_sweep(n, omega, orc.P(ref), orc.P(canon))
    rt = g.runtime()
    lo, hi = L3(1, 1, 1), L3(n - 2, n - 2, n - 2)
    st, ext = L3(n * n, n, 1), L3(n, n, n)
    A = torch.tensor(A0, dtype=torch.float64, device="cuda")
    w = torch.tensor([omega], dtype=torch.float64, device="cuda")
    items = torch.zeros(rt.dvmhgb_sor3d_items(lo, hi, variant), dtype=torch.float64, device="cuda")
    scratch = torch.zeros(rt.dvmhgb_sor3d_scratch_bytes(lo, hi, variant) // 4 + 1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert rt.dvmhgb_sor3d_sweep(P(A), st, ext, lo, hi, P(w), P(items), P(scratch), P(status), variant, stream) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = A.cpu().numpy()
    assert np.array_equal(got.view(np.int64), ref.view(np.int64)), (variant, omega)


def _tree(leaves):
    """Pairwise sum over a power-of-two number of leaves, as the canonical SUM forms a part."""
    while len(leaves) > 1:
        leaves = [leaves[q] + leaves[q + 1] for q in range(0, len(leaves), 2)]
    return leaves[0]


def _sub_box_reference(A, lo, hi, omega, tk):
    """Sequential sweep of the loop box lo..hi (array A, modified) and the items the kernels write:
    per row (i, j) of the box and per tk-wide part of the 64-wide chunks its k range meets, the
    pairwise sum of (nv - old)^2 with -0.0 at positions outside the box."""
    c1, c2 = 1.0 - omega, omega / 6.0
    sq = {}
    for i in range(lo[0], hi[0] + 1):
        for j in range(lo[1], hi[1] + 1):
            for k in range(lo[2], hi[2] + 1):
                old = A[i, j, k]
                s = ((((A[i - 1, j, k] + A[i + 1, j, k]) + A[i, j - 1, k]) + A[i, j + 1, k]) + A[i, j, k - 1]) + \
                    A[i, j, k + 1]
                nv = c1 * old + c2 * s
                A[i, j, k] = nv
                d = nv - old
                sq[(i, j, k)] = d * d
    parts = 64 // tk
    kc0, nc = parts * (lo[2] // 64), parts * (hi[2] // 64 - lo[2] // 64 + 1)
    items = []
    for i in range(lo[0], hi[0] + 1):
        for j in range(lo[1], hi[1] + 1):
            for c in range(nc):
                kb = (kc0 + c) * tk
                items.append(_tree([sq[(i, j, k)] if lo[2] <= k <= hi[2] else -0.0 for k in range(kb, kb + tk)]))
    return np.array(items)


@pytest.mark.parametrize("variant", [1, 2, 4, 5])
@pytest.mark.parametrize("box", [((2, 3, 40), (9, 13, 121)), ((1, 1, 1), (6, 17, 5)), ((3, 1, 70), (3, 9, 71))])
def test_sor_kernel_sub_box(g, variant, box):
    """A loop box that is not the array's interior: k starting past the first 64-wide chunk, rows that
    fill no whole tile, a box one cell thick -- the array and every residual item bit-exact."""
    import torch
    lo, hi = box
    shape = (12, 19, 130)
    rng = np.random.default_rng(11 + variant)
    A0 = rng.random(shape) * 2.0 - 0.5
    ref = A0.copy()
    tk = {1: 16, 2: 8, 4: 8, 5: 8}[variant]
    want = _sub_box_reference(ref, lo, hi, 1.5, tk)
    rt = g.runtime()
    L_lo, L_hi = L3(*lo), L3(*hi)
    st, ext = L3(shape[1] * shape[2], shape[2], 1), L3(*shape)
    A = torch.tensor(A0.ravel(), dtype=torch.float64, device="cuda")
    w = torch.tensor([1.5], dtype=torch.float64, device="cuda")
    n_items = rt.dvmhgb_sor3d_items(L_lo, L_hi, variant)
    assert n_items == len(want)
    items = torch.full((n_items,), float("nan"), dtype=torch.float64, device="cuda")
    scratch = torch.zeros(rt.dvmhgb_sor3d_scratch_bytes(L_lo, L_hi, variant) // 4 + 1, dtype=torch.int32,
                          device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert rt.dvmhgb_sor3d_sweep(P(A), st, ext, L_lo, L_hi, P(w), P(items), P(scratch), P(status), variant,
                                 stream) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = A.cpu().numpy().reshape(shape)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64)), (variant, box)
    gi = items.cpu().numpy()
    assert np.array_equal(gi.view(np.int64), want.view(np.int64)), (variant, box)
