"""The allocation-free Jacobi-3D update entry point (dvmhgb_jac3d_update_noalloc).

It exists for callers that cannot allocate device memory -- code running
inside a global-mode stream capture, hosts whose allocator owns the whole
GPU, paths that must not block in the driver -- and keeps its partial maxima
in a static device array instead.  This test calls it through the C ABI twice
in a row, on different data, and checks A and eps bit for bit against the
allocating entry point (dvmhgb_jac3d_update with a caller buffer, partials
folded by max): the second call must not see anything of the first.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test; it also passes alone.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k_lo,k_hi", [(1, 129), (57, 57), (100, 130)])
def test_update_noalloc_matches_allocating_entry_point(k_lo, k_hi):
    """The whole interior; one column at an odd k (the pair's second element
    alone); a box ending on the row's last element, whose pair reaches into
    the row padding."""
    import torch

    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    L = g.runtime()
    L.dvmhgb_jac3d_update_items.restype = ctypes.c_long
    n = 131  # odd extent: ragged 64-wide segments; rows padded to an even length (16-byte aligned rows)
    w = n + 1
    LA = ctypes.c_long * 3
    st, lo, hi = LA(n * w, w, 1), LA(1, 1, k_lo), LA(n - 2, n - 2, k_hi)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    gen = torch.Generator(device="cuda").manual_seed(5)
    for call in range(2):
        A = torch.rand(n, n, w, dtype=torch.float64, device="cuda", generator=gen)
        B = torch.rand(n, n, w, dtype=torch.float64, device="cuda", generator=gen) * (call + 1)
        A1, A2 = A.clone(), A.clone()
        items = torch.empty(L.dvmhgb_jac3d_update_items(lo, hi), dtype=torch.float64, device="cuda")
        assert L.dvmhgb_jac3d_update(vp(A1), vp(B), st, lo, hi, vp(items), 1, sp) == 0
        eps_ref = items.max()
        eps = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        assert L.dvmhgb_jac3d_update_noalloc(vp(A2), vp(B), st, lo, hi, vp(eps), sp) == 0
        torch.cuda.synchronize()
        assert torch.equal(A1, A2), call
        assert eps.item() == eps_ref.item(), (call, eps.item(), eps_ref.item())
        # the loop ran: A is B's inside the box, untouched outside it
        assert torch.equal(A2[1:-1, 1:-1, k_lo:k_hi + 1], B[1:-1, 1:-1, k_lo:k_hi + 1])
        assert torch.equal(A2[1:-1, 1:-1, :k_lo], A[1:-1, 1:-1, :k_lo])
        assert torch.equal(A2[1:-1, 1:-1, k_hi + 1:], A[1:-1, 1:-1, k_hi + 1:])
        assert torch.equal(A2[0], A[0])
        assert eps_ref.item() == (B - A)[1:-1, 1:-1, k_lo:k_hi + 1].abs().max().item()


def test_update_noalloc_rejects_unaligned_rows():
    """An odd row stride would make the 128-bit accesses misaligned: rejected, nothing launched."""
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    L = g.runtime()
    LA = ctypes.c_long * 3
    st, lo, hi = LA(131 * 131, 131, 1), LA(1, 1, 1), LA(129, 129, 129)
    assert L.dvmhgb_jac3d_update_noalloc(ctypes.c_void_p(256), ctypes.c_void_p(256), st, lo, hi,
                                         ctypes.c_void_p(256), None) == -1


def test_update_noalloc_rejects_invalid_arguments():
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    L = g.runtime()
    LA = ctypes.c_long * 3
    st, lo, hi = LA(64, 8, 2), LA(1, 1, 1), LA(6, 6, 6)  # innermost stride must be 1
    assert L.dvmhgb_jac3d_update_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), st, lo, hi,
                                         ctypes.c_void_p(16), None) == -1
