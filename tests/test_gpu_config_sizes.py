"""Parity at the benchmark configurations' own sizes and seeds, where the
wavefront's tile counts, plane offsets and resident-grid cap, the persistent
heat grid's strip search and the segmented fold all take their full-size
values:

  SOR 384^3, omega 1.5 (the configuration's 20 sweeps cut to 2), the default
  tile depth and the streaming-column variant, plain and batched;
  the batched heat configuration: 256 arrays with sides log-uniform in
  [64, 2048] (1.66e8 cells), 3 steps, plain and batched;
  Jacobi 3-D 512^3, 10 iterations, the default kernels and the fixed-point
  stencil, plain and batched.

Arrays, MAX, MIN and MINLOC bit-exact against the CPU restatement (itself
pinned to the reference runtime's outputs by tests/test_oracle.py); floating
SUMs bit-exact against the restatement of the canonical pairwise tree and
within gamma_n * sum|x| of the sequential order.  The seeds are the ones the
benchmark uses."""
import os

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc

pytestmark = pytest.mark.gpu
SEED = 20261203  # the benchmark's base seed: Jacobi SEED, SOR SEED + 2, heat SEED + 3


@pytest.fixture(scope="module")
def g():
    ge.build()
    _, g = ge.package()
    g.init()
    yield g
    g.force_variant(-1)
    g.set_mode("batched")


def gamma_close(a, b, absum, n):
    eps = 2.0 ** -53
    gamma = (n * eps) / (1 - n * eps)
    return np.all(np.abs(a - b) <= 2 * gamma * absum + 1e-300)


@pytest.fixture(scope="module")
def sor_ref():
    return orc.sor_run(384, 2, 1.5, SEED + 2)


@pytest.mark.parametrize("variant", [1, 3, 4, 5])
@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_sor_384(g, sor_ref, mode, variant):
    seq, canon, A_ref = sor_ref
    g.force_variant(variant)
    try:
        g.set_mode(mode)
        s = g.Sor(384, 1.5, SEED + 2)
        res = s.run(2)
        A = s.fetch()
        s.close()
    finally:
        g.force_variant(-1)
    assert np.array_equal(A, A_ref), (mode, variant)
    assert np.array_equal(res, canon), (mode, variant, res, canon)
    assert gamma_close(res, seq, seq, 382 ** 3), (res, seq)


@pytest.fixture(scope="module")
def heat_ref():
    return orc.heat_run(256, 64, 2048, 3, 0.2, SEED + 3)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_heat_256_arrays(g, heat_ref, mode):
    r = heat_ref
    g.set_mode(mode)
    h = g.Heat(256, 64, 2048, 0.2, SEED + 3)
    assert h.sides == r["sides"]
    assert max(h.sides) > 1500 and min(h.sides) < 80 and h.cells() > 1.2e8
    sums, mins, locs = h.run(3)
    for k in range(256):
        assert np.array_equal(np.ravel(h.fetch(k)), np.ravel(r["finals"][k])), (mode, k, h.sides[k])
    h.close()
    assert np.array_equal(np.ravel(mins), r["mins"].ravel()), mode
    assert np.ravel(locs).tolist() == r["locs"].ravel().tolist(), mode
    assert np.array_equal(np.ravel(sums), r["sums_canon"].ravel()), mode
    absum = np.array([[float(np.abs(f).sum()) for f in r["finals"]]] * 3)
    assert gamma_close(np.reshape(sums, (3, 256)), r["sums_seq"], absum, 2048 ** 2), mode


@pytest.fixture(scope="module")
def jac_ref():
    return orc.jacobi_run(3, 512, 10, SEED, threads=os.cpu_count() or 1)


@pytest.mark.parametrize("variant", [-1, 14, 16, 22, 25])
@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_jacobi3d_512_ten_iterations(g, jac_ref, mode, variant):
    e_ref, A_ref, B_ref = jac_ref
    g.force_variant(variant)
    try:
        g.set_mode(mode)
        j = g.Jacobi(3, 512, SEED)
        eps = j.run(10)
        A, B = j.fetch()
        j.close()
    finally:
        g.force_variant(-1)
    assert np.array_equal(eps, e_ref), (mode, variant)
    assert np.array_equal(A, A_ref) and np.array_equal(B, B_ref), (mode, variant)
