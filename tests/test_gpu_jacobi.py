"""Jacobi 2-D/3-D through the dvmh_* C ABI on the GPU, against the reference's
golden outputs and the CPU oracle, bit for bit, in every execution mode."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import orc
from tests.util import sha, unhex

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


@pytest.mark.parametrize("rank,n,iters", [(3, 5, 2), (3, 33, 4), (3, 66, 3), (3, 129, 2), (2, 5, 3), (2, 65, 6),
                                          (2, 300, 5)])
def test_jacobi_vs_oracle_sizes(g, rank, n, iters):
    """Ragged sizes: extents around the 64-element tiles and 16-row tiles."""
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
    # the first call allocates the alternate buffer; afterwards the two buffers of B alternate
    assert s["graphs_captured"] <= 3
    assert s["graphs_captured"] + s["graph_replays"] == 6 and s["graph_replays"] >= 3


def test_plain_mode_no_fusion(g):
    g.set_mode("plain")
    j = g.Jacobi(3, 40, 5)
    g.reset_stats()
    j.run(3)
    s = g.stats()
    j.close()
    g.set_mode("batched")
    assert s["fused_pairs"] == 0 and s["graphs_captured"] == 0 and s["handler_calls"] == 6
