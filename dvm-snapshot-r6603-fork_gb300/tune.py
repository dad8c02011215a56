"""The tuner's training and evaluation pipeline on synthetic parallel loops.

1. Draw loops (seeded): rank 1-4, total extent log-uniform in [2^6, 2^24],
   stencil radius 0-3, fp32/fp64/int32, reduction none/sum/max/minloc,
   ACROSS on the outermost axis for some rank>=2 loops.
2. Exhaustive tuning: the runtime times every candidate (CUDA block, axis on
   threadIdx.x, elements per thread; 16-64 per loop) and records each timing
   in its database (dvmhgb_tuner_time_synth).
3. Training: the database's features and log-times (centred per loop, so the
   model learns the ranking) train the FP32 MLP on the GPU with the library's
   own kernels (dvmhgb_mlp_train).
4. Evaluation on held-out loops: the model ranks the candidates, the top k
   (about 10% of the candidates) are timed, the best of them is compared with
   the exhaustive best; the tuning time is the summed time of the candidates
   actually run.  Baselines: the reference's default block
   (rts/dvmh/loop.cpp:1464-1485) and k random candidates.
"""
import ctypes
import os
import math
import time

import numpy as np

MAXC = 64


class SynthLoop(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_int), ("radius", ctypes.c_int), ("across", ctypes.c_int), ("red", ctypes.c_int),
                ("esize", ctypes.c_int), ("isint", ctypes.c_int), ("ext", ctypes.c_long * 4)]


class SynthCand(ctypes.Structure):
    _fields_ = [("bx", ctypes.c_int), ("by", ctypes.c_int), ("bz", ctypes.c_int), ("xinner", ctypes.c_int),
                ("ept", ctypes.c_int)]


def draw_loops(count, seed, max_elems=1 << 25):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        rank = int(rng.integers(1, 5))
        total = 2.0 ** rng.uniform(6, 24)
        w = rng.dirichlet(np.ones(rank))
        ext = [max(2, int(round(total ** wi))) for wi in w]
        radius = int(rng.integers(0, 4))
        dt = int(rng.integers(0, 3))  # fp32, fp64, int32
        red = int(rng.integers(0, 4))
        across = int(rank >= 2 and rng.uniform() < 0.2)
        padded = 1
        for e in ext:
            padded *= e + 2 * radius
        if padded > max_elems:
            continue
        out.append(make_loop(rank, ext, radius, dt, red, across))
    return out


def make_loop(rank, ext, radius, dt, red, across):
    L = SynthLoop()
    L.rank, L.radius, L.across, L.red = rank, radius, across, red
    L.esize = 8 if dt == 1 else 4
    L.isint = 1 if dt == 2 else 0
    for a in range(4):
        L.ext[a] = ext[a] if a < rank else 0
    return L


def config_loops():
    """The workloads' loop shapes as synthetic loops: Jacobi-2D 1022^2 MAX,
    Jacobi-3D 510^3 MAX, SOR 382^3 SUM with ACROSS (fp64, radius 1)."""
    return {"jacobi2d_1024": make_loop(2, [1022, 1022], 1, 1, 2, 0),
            "jacobi3d_512": make_loop(3, [510, 510, 510], 1, 1, 2, 0),
            "sor3d_384": make_loop(3, [382, 382, 382], 1, 1, 1, 1)}


def default_cand(L, cands):
    """The reference's default block for the loop's rank: 256 / 32x8 / 32x4x2."""
    want = {1: (256, 1, 1), 2: (32, 8, 1)}.get(L.rank, (32, 4, 2))
    for i, c in enumerate(cands):
        if (c.bx, c.by, c.bz, c.xinner, c.ept) == (*want, 1, 1):
            return i
    return 0


class Tuner:
    def __init__(self, rt):
        self.rt = rt
        rt.dvmhgb_tuner_time_synth.restype = ctypes.c_double
        rt.dvmhgb_tuner_db_size.restype = ctypes.c_long
        rt.dvmhgb_tuner_db_export.restype = ctypes.c_long
        rt.dvmhgb_mlp_nparams.restype = ctypes.c_long

    def candidates(self, L):
        arr = (SynthCand * MAXC)()
        n = self.rt.dvmhgb_tuner_candidates(ctypes.byref(L), arr, MAXC)
        return [arr[i] for i in range(n)]

    def exhaustive(self, L, loop_id, reps=2):
        """Times every candidate; returns the seconds per candidate (recorded in the runtime's database)."""
        cands = self.candidates(L)
        arr = (SynthCand * len(cands))(*cands)
        ts = (ctypes.c_double * len(cands))()
        assert self.rt.dvmhgb_tuner_time_synth_all(ctypes.byref(L), arr, len(cands), ctypes.c_long(loop_id), reps,
                                                   ts) == 0
        return cands, np.array(ts)

    def features(self, L, cands):
        F = np.zeros((len(cands), 24), dtype=np.float32)
        row = (ctypes.c_float * 24)()
        for i, c in enumerate(cands):
            self.rt.dvmhgb_tuner_features(ctypes.byref(L), ctypes.byref(c), row)
            F[i] = np.frombuffer(row, dtype=np.float32)
        return F

    def train(self, X, y, epochs=200, batch=4096, lr=1e-3, seed=1):
        np_ = self.rt.dvmhgb_mlp_nparams()
        params = np.zeros(np_, dtype=np.float32)
        losses = np.zeros(epochs, dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        rc = self.rt.dvmhgb_mlp_train(X.ctypes.data_as(fp), y.ctypes.data_as(fp), ctypes.c_long(len(y)), epochs,
                                      ctypes.c_long(batch), ctypes.c_float(lr), ctypes.c_ulonglong(seed),
                                      params.ctypes.data_as(fp), losses.ctypes.data_as(fp))
        assert rc == 0, "training failed"
        return params, losses

    def install(self, params, mean, std):
        fp = ctypes.POINTER(ctypes.c_float)
        self.rt.dvmhgb_tuner_set_model(np.ascontiguousarray(params, np.float32).ctypes.data_as(fp),
                                       np.ascontiguousarray(mean, np.float32).ctypes.data_as(fp),
                                       np.ascontiguousarray(std, np.float32).ctypes.data_as(fp))

    def rank(self, L, cands):
        arr = (SynthCand * len(cands))(*cands)
        order = (ctypes.c_int * len(cands))()
        assert self.rt.dvmhgb_tuner_rank(ctypes.byref(L), arr, len(cands), order) == 0
        return list(order)


def run(rt, n_loops=2000, n_test=200, seed=20261207, reps=2, epochs=200, frac=0.10, log=print):
    """Returns a dict of the evaluation (the bench's TUNE line)."""
    tu = Tuner(rt)
    rt.dvmhgb_tuner_db_clear()
    loops = draw_loops(n_loops, seed)
    t0 = time.time()
    times = []
    cands_all = []
    for q, L in enumerate(loops):
        cands, ts = tu.exhaustive(L, q, reps)
        cands_all.append(cands)
        times.append(ts)
    t_collect = time.time() - t0
    n_train = n_loops - n_test
    # training set: the database rows of the first n_train loops, log-time centred per loop
    X, y = [], []
    for q in range(n_train):
        F = tu.features(loops[q], cands_all[q])
        lt = np.log(np.maximum(times[q], 1e-9))
        X.append(F)
        y.append(lt - lt.mean())
    X = np.concatenate(X)
    y = np.concatenate(y)
    mean, std = X.mean(0), X.std(0) + 1e-6
    t1 = time.time()
    params, losses = tu.train((X - mean) / std, y, epochs=epochs)
    t_train = time.time() - t1
    tu.install(params, mean, std)

    def evaluate(L, cands, ts, rng):
        nc = len(cands)
        k = max(1, int(math.floor(frac * nc)))
        order = tu.rank(L, cands)
        top = order[:k]
        best_model = ts[top].min()
        best = ts.min()
        rand = rng.choice(nc, size=k, replace=False)
        return {"k": k, "n": nc, "ratio": best_model / best, "tune_frac": ts[top].sum() / ts.sum(),
                "default_ratio": ts[default_cand(L, cands)] / best, "random_ratio": ts[rand].min() / best}

    rng = np.random.default_rng(seed + 1)
    res = [evaluate(loops[q], cands_all[q], times[q], rng) for q in range(n_train, n_loops)]
    cfg = {}
    for name, L in config_loops().items():
        cands, ts = tu.exhaustive(L, -1, reps)
        cfg[name] = evaluate(L, cands, ts, rng)
    r = np.array([x["ratio"] for x in res])
    out = {"loops": n_loops, "train": n_train, "test": n_test,
           "candidates_mean": float(np.mean([x["n"] for x in res])),
           "db_rows": int(rt.dvmhgb_tuner_db_size()),
           "within_5pct": float(np.mean(r <= 1.05)), "ratio_geomean": float(np.exp(np.mean(np.log(r)))),
           "ratio_p90": float(np.quantile(r, 0.9)),
           "tuning_time_frac_mean": float(np.mean([x["tune_frac"] for x in res])),
           "default_block_ratio_geomean": float(np.exp(np.mean(np.log([x["default_ratio"] for x in res])))),
           "random_k_ratio_geomean": float(np.exp(np.mean(np.log([x["random_ratio"] for x in res])))),
           "random_k_within_5pct": float(np.mean(np.array([x["random_ratio"] for x in res]) <= 1.05)),
           "configs": {k: {kk: float(vv) for kk, vv in v.items()} for k, v in cfg.items()},
           "loss_first_last": [float(losses[0]), float(losses[-1])],
           "seconds": {"collect": t_collect, "train": t_train}}
    return out


# ---------------------------------------------------------------- the configurations' own loops
#
# The hand-written handlers of the workload programs choose among kernel
# variants through dvmhgb_loop_variant_desc, describing each variant to the
# runtime.  Every timed execution goes into the runtime's variant database.
# Protocol, per program:
#   1. exhaustive tuning (mode 1) at a few training sizes: the runtime tries
#      every variant twice (DVMH_GB_TUNE_REPS), in successive steps, and
#      records each run;
#   2. the variant model (same MLP, same kernels) is trained on those records,
#      log-times centred per loop shape, and installed in the runtime;
#   3. at the configuration's own size (never seen in training): exhaustive
#      tuning again (the reference point: every variant's time, their sum the
#      exhaustive tuning time), then model-guided tuning (mode 2): the runtime
#      ranks the variants by the model, tries only the first floor(0.1 n)
#      (none: it keeps the model's first choice), and keeps the fastest tried.
# Reported: the kept variant's time over the exhaustive best, the model's
# tuning time over the exhaustive one, both variants.

def _programs(g, seed):
    """name -> (training sizes, configuration size, maker(size) -> object with run/close)."""
    return {
        "jacobi2d_1024": ([642, 770, 898, 962, 1090, 1154, 1282, 1538], 1024, lambda n: g.Jacobi(2, n, seed)),
        "jacobi3d_512": ([322, 386, 450, 578], 512, lambda n: g.Jacobi(3, n, seed)),
        "sor3d_384": ([258, 322, 354, 418, 450], 384, lambda n: g.Sor(n, 1.5, seed + 2)),
        "heat_256x2048": ([(128, 1024), (192, 1536), (320, 2048)], (256, 2048),
                          lambda p: g.Heat(p[0], 64, p[1], 0.2, seed + 3)),
    }


def _variant_runs(g, rt, mode, maker, size, steps_cap=200):
    """Tunes one program at one size in `mode`; returns the variant record of
    the program's main loop: the handler that ran the most tuned executions
    (the steps run back to back, as the program runs them, so that a loop the
    runtime defers to the next step meets it)."""
    rt.dvmhgb_tuner_reset()
    rt.dvmhgb_set_tuning(mode)
    w = maker(size)
    try:
        steps = 0
        while steps < steps_cap:
            w.run(1)
            steps += 1
            if not rt.dvmhgb_tuner_exploring():
                break
        w.run(2)  # the kept variant, as it then runs
        g.sync()
        info = _variant_info(rt)
    finally:
        rt.dvmhgb_set_tuning(0)
        w.close()
    return info


def _variant_info(rt):
    H = ctypes.c_void_p()
    nv, ch, ex = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    es = ctypes.c_double()
    best = (ctypes.c_double * 64)()
    out = None
    for i in range(int(rt.dvmhgb_tuner_variant_count())):
        rt.dvmhgb_tuner_variant_info(ctypes.c_long(i), ctypes.byref(H), ctypes.byref(nv), ctypes.byref(ch), best, 64,
                                     ctypes.byref(ex), ctypes.byref(es))
        rec = {"handler": H.value, "nvariants": nv.value, "chosen": ch.value,
               "best": [best[v] for v in range(nv.value)], "explored": ex.value, "explore_seconds": es.value}
        out = (out or []) + [rec]
    return out


def _main_record(recs, handler=None):
    """The record of `handler`, or (None) of the handler whose exhaustive search took the longest."""
    if handler is not None:
        return next(r for r in recs if r["handler"] == handler)
    return max(recs, key=lambda r: (r["explore_seconds"], r["nvariants"]))


def configs_eval(g, seed=20261203, epochs=300, log=print, reps=4):
    """The learned tuner on the configurations' own loops (the bench's configs.tune).  Every variant a
    tuning session tries runs `reps` times (the fastest counts) in the training runs, the exhaustive
    reference and the model-guided runs alike: the configurations' smallest loops take tens of
    microseconds, where two runs leave their order to chance."""
    old = os.environ.get("DVMH_GB_TUNE_REPS")
    os.environ["DVMH_GB_TUNE_REPS"] = str(reps)
    try:
        return _configs_eval(g, seed, epochs, log)
    finally:
        if old is None:
            os.environ.pop("DVMH_GB_TUNE_REPS", None)
        else:
            os.environ["DVMH_GB_TUNE_REPS"] = old


def _configs_eval(g, seed, epochs, log):
    rt = g.runtime()
    rt.dvmhgb_tuner_vdb_size.restype = ctypes.c_long
    rt.dvmhgb_tuner_vdb_export.restype = ctypes.c_long
    rt.dvmhgb_tuner_variant_count.restype = ctypes.c_long
    rt.dvmhgb_mlp_nparams.restype = ctypes.c_long
    g.set_mode("batched")
    progs = _programs(g, seed)
    rt.dvmhgb_tuner_vdb_clear()
    t0 = time.time()
    for name, (train, _, maker) in progs.items():
        for size in train:
            _variant_runs(g, rt, 1, maker, size)
    rows = int(rt.dvmhgb_tuner_vdb_size())
    X = np.zeros((rows, 24), dtype=np.float32)
    sec = np.zeros(rows)
    keys = np.zeros(rows, dtype=np.uint64)
    var = np.zeros(rows, dtype=np.int32)
    fp = ctypes.POINTER(ctypes.c_float)
    rt.dvmhgb_tuner_vdb_export(X.ctypes.data_as(fp), sec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                               keys.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)),
                               var.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.c_long(rows))
    # one row per (loop shape, variant): its fastest time; log-time centred per loop shape
    best = {}
    for i in range(rows):
        k = (int(keys[i]), int(var[i]))
        if k not in best or sec[i] < sec[best[k]]:
            best[k] = i
    idx = np.array(sorted(best.values()))
    Xt, lt = X[idx], np.log(np.maximum(sec[idx], 1e-9))
    kt = keys[idx]
    y = lt.copy()
    for k in np.unique(kt):
        m = kt == k
        y[m] = lt[m] - lt[m].mean()
    mean, std = Xt.mean(0), Xt.std(0) + 1e-6
    tu = Tuner(rt)
    params, losses = tu.train((Xt - mean) / std, y, epochs=epochs, batch=min(4096, len(y)), lr=2e-3)
    rt.dvmhgb_tuner_set_variant_model(np.ascontiguousarray(params, np.float32).ctypes.data_as(fp),
                                      np.ascontiguousarray(mean, np.float32).ctypes.data_as(fp),
                                      np.ascontiguousarray(std, np.float32).ctypes.data_as(fp))
    t_train = time.time() - t0
    out = {"protocol": "exhaustive at training sizes -> variant model -> at the configuration size: exhaustive "
                       "vs model-guided (top floor(0.1 n) tried)", "train_rows": int(len(y)),
           "loss_first_last": [float(losses[0]), float(losses[-1])], "train_seconds": t_train}
    for name, (train, size, maker) in progs.items():
        ex = _main_record(_variant_runs(g, rt, 1, maker, size))
        md = _main_record(_variant_runs(g, rt, 2, maker, size), ex["handler"])
        bests = np.array(ex["best"])
        vbest = int(np.argmin(np.where(bests >= 0, bests, np.inf)))
        pick = md["chosen"]
        out[name] = {"size": size if not isinstance(size, tuple) else list(size), "train_sizes": train,
                     "variants": ex["nvariants"], "exhaustive_best_variant": vbest,
                     "model_variant": pick, "model_tried": md["explored"],
                     "model_over_exhaustive_time": float(bests[pick] / bests[vbest]) if bests[pick] > 0 else None,
                     "tuning_time_frac": float(md["explore_seconds"] / ex["explore_seconds"])
                     if ex["explore_seconds"] > 0 else None,
                     "exhaustive_ms": {str(v): round(1e3 * b, 4) for v, b in enumerate(bests)},
                     "exhaustive_tuning_s": ex["explore_seconds"], "model_tuning_s": md["explore_seconds"]}
        log(name, out[name])
    rt.dvmhgb_tuner_reset()
    return out


if __name__ == "__main__":
    import argparse
    import json
    import os
    import sys
    ap = argparse.ArgumentParser(description="exhaustive + learned tuning of synthetic loops")
    ap.add_argument("--loops", type=int, default=2000)
    ap.add_argument("--test", type=int, default=200)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--out", default=None)
    ap.add_argument("--configs", action="store_true", help="the configurations' own loops (variants) only")
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    g.init()
    t0 = time.time()
    if a.configs:
        res = configs_eval(g)
    else:
        res = run(g.runtime(), n_loops=a.loops, n_test=a.test, reps=a.reps)
    res["wall_seconds"] = time.time() - t0
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")
    print(text)
