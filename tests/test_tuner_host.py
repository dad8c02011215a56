"""The tuner's host logic, without a GPU: the candidate enumeration and the
feature vectors the learned model sees (csrc/rt_tuner.cpp), on the seeded
synthetic loop family the tuner is trained on (tune.py).

Each candidate must be a launchable configuration of its loop (at most 1024
threads, accepted by the synthetic kernel's shape rules).  ACROSS loops keep
their dependent axis off threadIdx.x, as the reference's ACROSS handlers do.
Each loop gets 16..64 candidates, including the reference's default block
(rts/dvmh/loop.cpp:1464-1485).  Features are finite and deterministic."""
import ctypes
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def env():
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    spec = importlib.util.spec_from_file_location("tune", os.path.join(ROOT, "dvm-snapshot-r6603-fork_gb300", "tune.py"))
    tune = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tune)
    rt = g.runtime()
    rt.dvmhgb_synth_items.restype = ctypes.c_long
    rt.dvmhgb_tuner_candidates.restype = ctypes.c_int
    return rt, tune


def cands_of(rt, tune, L):
    arr = (tune.SynthCand * tune.MAXC)()
    n = rt.dvmhgb_tuner_candidates(ctypes.byref(L), arr, tune.MAXC)
    return [arr[q] for q in range(n)]


def test_candidates_are_launchable_and_complete(env):
    rt, tune = env
    loops = tune.draw_loops(300, 11)
    for L in loops:
        cs = cands_of(rt, tune, L)
        assert 16 <= len(cs) <= 64, (L.rank, L.across, len(cs))
        keys = set()
        for c in cs:
            assert c.bx * c.by * c.bz <= 1024 and min(c.bx, c.by, c.bz) >= 1
            assert rt.dvmhgb_synth_items(ctypes.byref(L), ctypes.byref(c)) >= 0
            if L.across or L.rank == 1:
                assert c.xinner == 1  # the dependent (outer) axis never goes on threadIdx.x
            keys.add((c.bx, c.by, c.bz, c.xinner, c.ept))
        assert len(keys) == len(cs)  # no duplicates
        want = {1: (256, 1, 1), 2: (32, 8, 1)}.get(L.rank, (32, 4, 2))
        dc = tune.SynthCand(*want, 1, 1)
        if rt.dvmhgb_synth_items(ctypes.byref(L), ctypes.byref(dc)) >= 0:  # launchable for this loop
            d = cs[tune.default_cand(L, cs)]
            assert (d.bx, d.by, d.bz, d.xinner, d.ept) == (*want, 1, 1)


def test_features_finite_and_deterministic(env):
    rt, tune = env
    loops = tune.draw_loops(50, 5)
    for L in loops:
        cs = cands_of(rt, tune, L)
        f = np.zeros((len(cs), 24), dtype=np.float32)
        for q, c in enumerate(cs):
            v = (ctypes.c_float * 24)()
            rt.dvmhgb_tuner_features(ctypes.byref(L), ctypes.byref(c), v)
            f[q] = np.frombuffer(v, dtype=np.float32)
        assert np.all(np.isfinite(f))
        assert f[:, 0].min() == f[:, 0].max() == L.rank  # loop features shared by its candidates
        assert len({tuple(r) for r in f}) == len(cs)       # candidates are distinguishable
    again = tune.draw_loops(50, 5)
    assert all(a.rank == b.rank and list(a.ext) == list(b.ext) and a.red == b.red for a, b in zip(loops, again))
