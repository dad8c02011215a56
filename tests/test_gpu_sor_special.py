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


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
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
