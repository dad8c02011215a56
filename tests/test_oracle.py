"""The CPU restatement (oracle/restate.c) against outputs of the reference
runtime itself (tests/golden/golden.json, made by tests/golden/make_golden.py
from the reference's host handlers, sequential order)."""
import hashlib
import os

import numpy as np
import pytest

from oracle import orc


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def unhex(xs):
    return np.array([float.fromhex(x) for x in xs])


def jac_cases(golden):
    return [k for k, v in golden.items() if v["prog"] in ("jac2d", "jac3d") and v["params"][0] <= 130]


def test_golden_present(golden):
    progs = {v["prog"] for v in golden.values()}
    assert progs == {"jac2d", "jac3d", "sor3d", "heat", "gsd2d", "genred", "genredx", "rec2d", "gsd3d", "gs2d",
                     "gen3d", "jacperf", "cdvh2d"}


# the reference examples' own verification (examples/Performance/jac3d_perf.c:92, jac2d_perf.c:89)
KNOWN_ANSWERS = {(3, 384, 100): (5.058044, 1e-4), (2, 8000, 100): (58.37598, 1e-3)}


def sha32(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f4").tobytes()).hexdigest()


def test_jacperf_vs_reference(golden):
    """The reference's FP32 Jacobi benchmarks, including both full
    configurations (about 4 s each here) and an early stop at eps < 0.5."""
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "jacperf"]
    assert {tuple(c["params"]) for _, c in cases} >= set(KNOWN_ANSWERS)
    for name, c in cases:
        its, eps, A, B = orc.jacperf_run(*c["params"])
        assert its == c["its"], name
        assert [float(x).hex() for x in eps] == c["eps"], name
        assert sha32(A) == c["A_sha256"] and sha32(B) == c["B_sha256"], name
        ka = KNOWN_ANSWERS.get(tuple(c["params"]))
        if ka:
            assert abs(float(eps[-1]) - ka[0]) < ka[1], name


@pytest.mark.parametrize("rank", [2, 3])
def test_jacobi_vs_reference(golden, rank):
    for name, c in golden.items():
        if c["prog"] != "jac%dd" % rank or c["params"][0] > 130:
            continue
        n, it, seed = c["params"]
        eps, A, B = orc.jacobi_run(rank, n, it, seed)
        assert np.array_equal(eps, unhex(c["eps"])), name
        assert sha(A) == c["A_sha256"] and sha(B) == c["B_sha256"], name
        if "A" in c:
            assert np.array_equal(A, unhex(c["A"])) and np.array_equal(B, unhex(c["B"])), name


def test_jacobi2d_full_config_vs_reference(golden):
    """The CPU-runnable configuration: 1024^2, 100 iterations (about 1 s)."""
    c = golden["jac2d_n1024_it100"]
    n, it, seed = c["params"]
    eps, A, B = orc.jacobi_run(2, n, it, seed, threads=4)
    assert np.array_equal(eps, unhex(c["eps"]))
    assert sha(A) == c["A_sha256"] and sha(B) == c["B_sha256"]


def test_jacobi_thread_count_invariant():
    e1, A1, B1 = orc.jacobi_run(3, 21, 3, 99, threads=1)
    e4, A4, B4 = orc.jacobi_run(3, 21, 3, 99, threads=4)
    assert np.array_equal(e1, e4) and np.array_equal(A1, A4) and np.array_equal(B1, B4)


def test_sor_vs_reference(golden):
    for name, c in golden.items():
        if c["prog"] != "sor3d":
            continue
        n, sw, omega, seed = c["params"]
        seq, can, A = orc.sor_run(n, sw, omega, seed)
        assert np.array_equal(seq, unhex(c["s"])), name
        assert sha(A) == c["A_sha256"], name
        # canonical tree: same value up to the forward error bound of summation
        assert np.allclose(can, seq, rtol=1e-12, atol=0), name


def test_sor_columns_restatement(golden):
    """The column-wise SUM restatement (the hyperplane handler's slots) sweeps
    the same array as the reference and sums within its error bound."""
    u = 2.0 ** -53
    for name, c in golden.items():
        if c["prog"] != "sor3d":
            continue
        n, sw, omega, seed = c["params"]
        cols, A = orc.sor_run_columns(n, sw, omega, seed)
        assert sha(A) == c["A_sha256"], name
        ref = unhex(c["s"])
        assert np.all(np.abs(cols - ref) <= 2 * (n - 2) ** 3 * u * ref), name


def test_heat_vs_reference(golden):
    for name, c in golden.items():
        if c["prog"] != "heat":
            continue
        cnt, lo, hi, steps, coef, seed = c["params"]
        r = orc.heat_run(cnt, lo, hi, steps, coef, seed)
        assert r["sides"] == c["sides"], name
        assert np.array_equal(r["sums_seq"].ravel(), unhex(c["sums"])), name
        assert np.array_equal(r["mins"].ravel(), unhex(c["mins"])), name
        assert r["locs"].ravel().tolist() == c["locs"], name
        key = "final" if "final" in c else "final_sha256"
        for k, f in enumerate(r["finals"]):
            if key == "final":
                assert np.array_equal(f, unhex(c["final"][k])), name
            else:
                assert sha(f) == c["final_sha256"][k], name


def test_gsd2d_vs_reference(golden):
    """The two-dependence ACROSS loop in every direction, and the mirror loop
    B = 2 A run between sweeps."""
    for name, c in golden.items():
        if c["prog"] != "gsd2d":
            continue
        n0, n1, sw, seed, d0, d1, mirror = c["params"]
        m, A = orc.gsd2d_run(n0, n1, sw, seed, d0, d1)
        assert np.array_equal(m, unhex(c["m"])), name
        assert sha(A) == c["A_sha256"], name
        if "A" in c:
            assert np.array_equal(A, unhex(c["A"])), name
        if mirror:
            assert sha(A * 2.0) == c["B_sha256"], name


@pytest.mark.parametrize("prog", ["rec2d", "gsd3d", "gs2d"])
def test_across_programs_vs_reference(golden, prog):
    """One-dependence recurrence (MIN), a diagonal plane under an independent
    outer axis (MAX), one-thread Gauss-Seidel (SUM in loop order)."""
    run = {"rec2d": orc.rec2d_run, "gsd3d": orc.gsd3d_run, "gs2d": orc.gs2d_run}[prog]
    cases = [(k, c) for k, c in golden.items() if c["prog"] == prog]
    assert cases
    for name, c in cases:
        r, A = run(*c["params"])
        assert np.array_equal(r, unhex(c["r"])), name
        assert sha(A) == c["A_sha256"], name
        if "A" in c:
            assert np.array_equal(A, unhex(c["A"])), name


def test_gen3d_vs_reference(golden):
    """SUM in loop order and MAXLOC (strict >, initial value kept when never
    exceeded) of a 3-D parallel loop that reads a shadow edge."""
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "gen3d"]
    assert cases
    for name, c in cases:
        s, mx, lc, B = orc.gen3d_run(*c["params"])
        assert [s.hex(), mx.hex()] == c["s_mx"], name
        assert lc == c["lc"], name
        assert sha(B) == c["B_sha256"], name
        if "B" in c:
            assert np.array_equal(B, unhex(c["B"])), name


def test_genred_vs_reference(golden):
    """Eight reductions of four types with signed steps, an empty loop, and
    initial values that the loop never improves on."""
    for name, c in golden.items():
        if c["prog"] != "genred":
            continue
        n, start, end, step, seed = c["params"][:5]
        r = orc.genred_run(n, start, end, step, seed, c["params"][5:])
        assert [float(x).hex() for x in r[0:3]] == c["d3"], name
        assert list(r[3:7]) == c["i4"], name
        assert float(r[7]).hex() == c["f1"][0], name
        assert r[8] == c["lc"], name


def test_genred_edge_values_vs_reference(golden):
    """Signed zeros, subnormals, infinities, NaN and ties (wl_genred_pattern):
    MAX of signed zeros and MINLOC ties go to the first in loop order, NaN
    propagates through SUM and PROD and never wins a comparison."""
    cases = [(k, c) for k, c in golden.items() if c["prog"] == "genredx"]
    assert len(cases) >= 5
    for name, c in cases:
        n, start, end, step, pattern = c["params"][:5]
        x, v = orc.genred_pattern(pattern, n)
        r = orc.genred_run_data(n, start, end, step, x, v, c["params"][5:])
        assert [float(q).hex() for q in r[0:3]] == c["d3"], name
        assert list(r[3:7]) == c["i4"], name
        assert float(r[7]).hex() == c["f1"][0], name
        assert r[8] == c["lc"], name


def test_cdvh2d_vs_reference(golden):
    """The program in cdvmh's converted form (regular variables, dynamic arrays):
    eps per iteration and B bit-exact against the reference runtime."""
    cases = [k for k, v in golden.items() if v["prog"] == "cdvh2d"]
    assert len(cases) >= 4
    for k in cases:
        c = golden[k]
        n, it, seed = c["params"]
        eps, B = orc.cdvh2d_run(n, it, seed)
        assert [float(x).hex() for x in eps] == c["eps"], k
        assert sha(B) == c["B_sha256"], k
        if "B" in c:
            assert np.array_equal(B, unhex(c["B"])), k


def test_pairwise_tree_identity():
    """-0.0 padding is exact: a tree over n leaves equals the tree over the next power of two."""
    rng = np.random.default_rng(1)
    v = rng.standard_normal(37)
    a = orc.lib().orc_pairwise_sum(orc.P(v.copy()), 37)
    w = np.concatenate([v, np.full(27, -0.0)])
    b = orc.lib().orc_pairwise_sum(orc.P(w.copy()), 64)
    assert a == b
    z = np.array([-0.0, -0.0, -0.0])
    assert np.signbit(orc.lib().orc_pairwise_sum(orc.P(z), 3))


def test_canonical_chunking_matches_manual():
    rng = np.random.default_rng(2)
    rows, lo, hi = 5, 1, 130
    t = rng.standard_normal((rows, hi - lo + 1))
    got = orc.lib().orc_canon_sum(orc.P(t.copy()), rows, lo, hi)
    items = []
    for r in range(rows):
        for c in range(lo // 64, hi // 64 + 1):
            leaf = [t[r, k - lo] if lo <= k <= hi else -0.0 for k in range(64 * c, 64 * c + 64)]
            leaf = np.array(leaf)
            items.append(orc.lib().orc_pairwise_sum(orc.P(leaf), 64))
    items = np.array(items)
    assert got == orc.lib().orc_pairwise_sum(orc.P(items), len(items))


@pytest.mark.skipif(__import__("oracle.build", fromlist=["x"]).reference_source() is None,
                    reason="reference sources not present (GPU box)")
def test_reference_runtime_builds():
    from oracle import build
    drv = build.build_reference()
    assert drv and os.path.exists(drv)
