"""Host-side sizes of the SOR wavefront (no GPU: the functions only compute sizes).

`dvmhgb_sor3d_items` gives one residual item per row and TK-wide part of each 64-wide chunk of k (TK = the tile
depth; 8 for the hyperplane tiles, one item per chunk for the streaming columns); `dvmhgb_sor3d_scratch_bytes`
gives, for the hyperplane tiles, the tile counter's line, one flag per (a, b, c) of the tile grid, the tile list
(8 bytes a tile) and the carried differences (7 doubles a row).  The tile set is restated here: column (a, b) of
tiles of ti x tj rows holds tiles c = cmin .. cmax, the hyperplanes its rows' cells lie on, 8 per tile."""
import ctypes

import pytest

L3 = ctypes.c_long * 3
TK = {0: 32, 1: 16, 2: 8, 3: 64, 4: 8, 5: 8}


@pytest.fixture(scope="module")
def rt():
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    r = g.runtime()
    r.dvmhgb_sor3d_items.restype = ctypes.c_long
    r.dvmhgb_sor3d_scratch_bytes.restype = ctypes.c_long
    return r


def hyp_scratch(lo, hi, ti, tj, G=8):
    na, nb, nk = (hi[0] - lo[0] + ti) // ti, (hi[1] - lo[1] + tj) // tj, hi[2] - lo[2] + 1
    cmin = lambda a, b: (ti * a + tj * b) // G
    cmax = lambda a, b: (ti * a + tj * b + ti + tj - 2 + nk - 1) // G
    ncg = cmax(na - 1, nb - 1) + 1
    ntiles = sum(cmax(a, b) - cmin(a, b) + 1 for a in range(na) for b in range(nb))
    rows = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1)
    table_off = (256 + 4 * na * nb * ncg + 15) // 16 * 16
    return table_off + 8 * ntiles + 8 * (G - 1) * rows


BOXES = [((1, 1, 1), (382, 382, 382)), ((1, 1, 1), (2, 2, 2)), ((2, 3, 40), (9, 13, 121)), ((3, 1, 70), (3, 9, 71)),
         ((1, 1, 1), (129, 5, 300))]


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("variant", sorted(TK))
def test_items(rt, box, variant):
    lo, hi = box
    rows = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1)
    chunks = hi[2] // 64 - lo[2] // 64 + 1
    assert rt.dvmhgb_sor3d_items(L3(*lo), L3(*hi), variant) == rows * (64 // TK[variant]) * chunks


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("variant,ti,tj", [(4, 4, 8), (5, 16, 8)])
def test_hyperplane_scratch(rt, box, variant, ti, tj):
    lo, hi = box
    assert rt.dvmhgb_sor3d_scratch_bytes(L3(*lo), L3(*hi), variant) == hyp_scratch(lo, hi, ti, tj)


def test_rejects(rt):
    lo, hi = L3(1, 1, 1), L3(10, 10, 10)
    for v in (-1, 6, 7):
        assert rt.dvmhgb_sor3d_items(lo, hi, v) == -1
        assert rt.dvmhgb_sor3d_scratch_bytes(lo, hi, v) == -1
    assert rt.dvmhgb_sor3d_scratch_bytes(L3(5, 1, 1), L3(4, 10, 10), 4) == -1  # empty box
