"""SOR ACROSS (tiled wavefront) and the batched heat program on the GPU.

Arrays, MAX/MIN/MINLOC values and MINLOC locations: bit-exact against the
reference's own outputs (tests/golden) and the CPU oracle.  Floating SUM:
bit-exact against the oracle's restatement of the canonical pairwise tree
the GPU folds in (launch-configuration independent), and within the forward
error bound gamma_n * sum|x| of the reference's sequential order."""
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
    g.force_variant(-1)
    g.set_mode("batched")


@pytest.fixture(autouse=True)
def _no_forced_variant(g):
    yield
    g.force_variant(-1)


def close_sum(a, b, n):
    # |fl(sum) - sum| <= gamma_{n-1} * sum|x|; the residual terms are >= 0, so sum|x| = sum
    eps = 2.0 ** -53
    gamma = (n * eps) / (1 - n * eps)
    return np.all(np.abs(a - b) <= 2 * gamma * np.abs(b) + 1e-300)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("mode", MODES)
def test_sor_golden(g, golden, mode, variant):
    g.set_mode(mode)
    g.force_variant(variant)  # tile depth along k: 32, 16, 8; 3: streaming columns
    for name, c in golden.items():
        if c["prog"] != "sor3d":
            continue
        n, sw, omega, seed = c["params"]
        s = g.Sor(n, omega, seed)
        res = s.run(sw)
        A = s.fetch()
        s.close()
        assert sha(A) == c["A_sha256"], (name, mode)
        _, canon, _ = orc.sor_run(n, sw, omega, seed)
        assert np.array_equal(res, canon), (name, mode, res, canon)
        assert close_sum(res, unhex(c["s"]), (n - 2) ** 3), name


@pytest.mark.parametrize("tfm", [1, 0])
@pytest.mark.parametrize("mode", MODES)
def test_sor_generated_hyperplane_handler(g, golden, mode, tfm):
    """The same program through cdvmh's generated shape for three dependences
    (workloads/sor3d_gen_cuda.cu: one launch per hyperplane, a SUM slot per
    column prepared with fill = 1 and accumulated across the launches), with
    the runtime's transformed layout (the plane of the two fastest dependent
    axes diagonalised) or natural: the array bit for bit against the
    reference's goldens, the SUM bit for bit against the column-wise
    restatement and within the error bound of the reference's value."""
    import ctypes
    g.set_mode(mode)
    rt, w = g.runtime(), g.workloads()
    rt.dvmhgb_set_autotransform(tfm)
    w.wl_sor3d_use_generated.argtypes = [ctypes.c_int]
    w.wl_sor3d_use_generated(1)
    try:
        for name, c in golden.items():
            if c["prog"] != "sor3d":
                continue
            n, sw, omega, seed = c["params"]
            g.reset_stats()
            s = g.Sor(n, omega, seed)
            res = s.run(sw)
            A = s.fetch()
            s.close()
            st = g.stats()
            assert sha(A) == c["A_sha256"], (name, mode, tfm)
            cols, A_ref = orc.sor_run_columns(n, sw, omega, seed)
            assert np.array_equal(res, cols), (name, mode, tfm, res, cols)
            assert close_sum(res, unhex(c["s"]), (n - 2) ** 3), name
            if not tfm:
                assert st["relayouts"] == 0, st
    finally:
        w.wl_sor3d_use_generated(0)
        rt.dvmhgb_set_autotransform(1)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [4, 9, 17, 66, 75, 131])
def test_sor_sizes_vs_oracle(g, n, variant):
    seq, canon, A_ref = orc.sor_run(n, 3, 1.5, 77 + n)
    g.force_variant(variant)
    for mode in ("plain", "batched"):
        g.set_mode(mode)
        s = g.Sor(n, 1.5, 77 + n)
        res = s.run(3)
        A = s.fetch()
        s.close()
        assert np.array_equal(A, A_ref), (mode, n)
        assert np.array_equal(res, canon), (mode, n)


@pytest.mark.parametrize("mode", MODES)
def test_heat_golden(g, golden, mode):
    g.set_mode(mode)
    for name, c in golden.items():
        if c["prog"] != "heat":
            continue
        cnt, lo, hi, steps, coef, seed = c["params"]
        h = g.Heat(cnt, lo, hi, coef, seed)
        assert h.sides == c["sides"]
        sums, mins, locs = h.run(steps)
        finals = [h.fetch(k) for k in range(cnt)]
        h.close()
        assert np.array_equal(mins.ravel(), unhex(c["mins"])), (name, mode)
        assert locs.ravel().tolist() == c["locs"], (name, mode)
        for k in range(cnt):
            if "final" in c:
                assert np.array_equal(finals[k], unhex(c["final"][k])), (name, mode, k)
            else:
                assert sha(finals[k]) == c["final_sha256"][k], (name, mode, k)
        r = orc.heat_run(cnt, lo, hi, steps, coef, seed)
        assert np.array_equal(sums, r["sums_canon"]), (name, mode)
        ref = unhex(c["sums"]).reshape(steps, cnt)
        absum = np.array([[float(np.abs(f).sum()) for f in r["finals"]]] * steps)
        n = max(s * s for s in c["sides"])
        assert np.all(np.abs(sums - ref) <= 4 * n * 2.0 ** -53 * (absum + 1e-300) + 1e-300), name


def test_heat_batched_uses_batch_rule(g):
    g.set_mode("batched")
    h = g.Heat(16, 3, 200, 0.2, 11)
    g.reset_stats()
    h.run(3)
    s = g.stats()
    h.close()
    # src/dst alternate: two captured graphs (each running the batch rule once), then replays
    assert s["loops_performed"] == 48 and s["batched_groups"] == s["graphs_captured"] >= 1
    assert s["graphs_captured"] + s["graph_replays"] == 3
