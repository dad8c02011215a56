"""Benchmark of the GB300 DVMH loop-execution path.

Headline workload (N=1): the 3-D 7-point Jacobi program, FP64, 512^3 grid with
shadow width 1 (510^3 interior cells), seeded uniform[0,1) interior, zero
boundary.  One step = one time step of the program through the dvmh_* C ABI:
the update loop (eps = max|B-A|, A = B) with its MAX reduction, shadow renew,
the stencil loop, get_actual(eps) -- in the batched mode (loops captured as a
cached CUDA graph, update+stencil fused).  --steps defaults to the
configuration's 50 iterations.

Printed as one JSON line:
  value      cell-updates/s, device-timed (CUDA events on the runtime's stream),
             arrays resident in HBM (2 x 1.07 GB, larger than L2: no flush needed)
  e2e        the same metric through the C ABI from host arrays: every run
             declares the program's pinned host copies of A and B current
             (dvmh_actual_array2_: uploaded by the first step), runs the steps,
             reads A and B back (dvmh_get_actual_array2_); bytes per step =
             those copies / steps
  roofline   dominant handler (the fused update+stencil pair): algorithmic
             bytes 32 per cell (A and B read once, written once) x 510^3 cells
             per launch / its average duration from the runtime's event timing
             over the timed region, against the measured HBM copy bandwidth
  roofline_fp64  the stencil's 5 FP64 additions per cell as if all ran on the
             FP64 unit, against that unit's measured addition rate: a fraction
             above 1 is work moved to the integer pipes (q61 fixed point)
  cpu_baseline  the CPU port of the same loops (oracle/restate.c, OpenMP,
             static schedule over the outermost loop like the reference host
             handlers) on this machine's host cores, bounded sample
  modes      the same step in plain (per-loop launches, per-loop synchronisation
             and reduction write-back, as the reference runtime) and async modes
  configs    SOR-3D ACROSS 384^3 x 20 sweeps and the batched uneven heat
             program (256 arrays, 64..2048, 200 steps), batched vs plain
`--impl reference` times the CPU port alone (the reference runtime itself
cannot be built on this machine: its sources are not present here).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 512
SEED = 20261203
BYTES_PER_CELL = 32  # A and B each read once and written once per step
FP64_ADDS_PER_CELL = 5  # the stencil's additions (mostly in q61 fixed point on the integer pipes)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.rows = []
        self.p = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            visible = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
            local = int(os.environ.get("LOCAL_RANK", "0"))
            gpu = visible[local] if local < len(visible) and visible[local] else str(local)  # this rank's GPU
            self.p = subprocess.Popen(["nvidia-smi", "-i", gpu,
                                       "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=2)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
                for k, nm in enumerate(names):
                    if r[3 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


class Replicas:
    """One process per GPU running an independent replica of the workload (the
    path does not shard).  A gloo group carries only timing: every timed region
    is bracketed by barriers and its time is the maximum over the ranks; the
    whole-job value is the units of all ranks divided by that time."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo", init_method="env://", rank=self.rank, world_size=self.world)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())


def cpu_port_rate(n, seconds=10.0, max_iters=40, threads=None):
    """Jacobi-3D steps of the CPU port on the host cores: (cell-updates/s, iters, threads)."""
    from oracle import orc
    L = orc.lib()
    threads = threads or L.orc_max_threads()
    A, B = orc.jacobi_init(3, n, SEED)
    L.orc_jacobi_step(3, n, orc.P(A), orc.P(B), threads)  # warm-up (first touch)
    it, t0 = 0, time.time()
    while it < max_iters and (it < 2 or time.time() - t0 < seconds):
        L.orc_jacobi_step(3, n, orc.P(A), orc.P(B), threads)
        it += 1
    dt = time.time() - t0
    return (n - 2) ** 3 * it / dt, it, threads


def run_reference(args):
    """The CPU port alone, on all host threads, same workload and metric."""
    from oracle import orc
    L = orc.lib()
    n = args.grid
    threads = L.orc_max_threads()
    A, B = orc.jacobi_init(3, n, SEED)
    for _ in range(args.warmup):
        L.orc_jacobi_step(3, n, orc.P(A), orc.P(B), threads)
    t0 = time.time()
    for _ in range(args.steps):
        L.orc_jacobi_step(3, n, orc.P(A), orc.P(B), threads)
    dt = time.time() - t0
    v = (n - 2) ** 3 * args.steps / dt
    line = {"impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "jacobi3d-7pt fp64 %d^3 (%d^3 interior), CPU port of the host handlers" % (n, n - 2),
                       "grid": n},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "sample": "%d steps of the %d^3 workload" % (args.steps, n)},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference runtime not buildable on this machine (its sources are absent); CPU port of its loops"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--grid", type=int, default=N_DEFAULT)
    ap.add_argument("--quick", action="store_true", help="headline only (no extra modes/configs/cpu leg)")
    ap.add_argument("--only", choices=["jacobi3d", "jacobi2d", "sor", "heat", "gsd2d", "jacperf"], default=None,
                    help="time one workload alone (small cases for profiling): --grid is its size "
                         "(heat: the largest side), --steps its steps or sweeps")
    ap.add_argument("--mode", choices=["batched", "async", "plain"], default="batched", help="with --only")
    ap.add_argument("--arrays", type=int, default=256, help="heat arrays, with --only heat")
    ap.add_argument("--variant", type=int, default=-1, help="force a kernel variant, with --only")
    ap.add_argument("--autotfm", type=int, default=1, help="layouts for ACROSS loops with --only gsd2d: 1 the "
                                                             "reference's transform, 0 natural, 2 chosen by the tuner")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))  # under torchrun; --impl reference runs on rank 0 only
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.gpus > 1:
        # one GPU per rank, independent replicas (the path does not shard: one process, one GPU)
        os.environ.setdefault("DVMH_GB_DEVICE", os.environ.get("LOCAL_RANK", "0"))

    import torch
    if args.gpus > 1:
        torch.cuda.set_device(int(os.environ["DVMH_GB_DEVICE"]))  # events on the runtime's device
    import __graft_entry__ as ge
    ge.build()
    _, g = ge.package()
    g.init()
    rt = g.runtime()
    stream = torch.cuda.ExternalStream(rt.dvmhgb_stream())
    if args.only:
        run_only(args, g, stream)
        return
    wl = g.workloads()
    n = args.grid
    cells = (n - 2) ** 3
    reps = Replicas()

    def timed_run(mode, steps, warmup, clocks=None):
        g.set_mode(mode)
        j = g.Jacobi(3, n, SEED)
        j.run(warmup)
        g.sync()
        g.reset_stats()
        rt.dvmhgb_timing_reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if clocks:
            clocks.start()
        torch.cuda.synchronize()
        reps.barrier()
        e0.record(stream)
        j.run(steps)
        e1.record(stream)
        g.sync()
        torch.cuda.synchronize()
        reps.barrier()
        ck = clocks.stop() if clocks else None
        ms = reps.max(e0.elapsed_time(e1) / steps)  # the slowest replica
        st = g.stats()
        j.close()
        return ms, st, ck

    # headline: batched mode with handler timing on (event nodes in the graph)
    rt.dvmhgb_set_timing(1)
    clocks = Clocks()
    ms, st, ck = timed_run("batched", args.steps, args.warmup, clocks)
    tot = ctypes.c_double()
    cnt = ctypes.c_long()
    # the step's pair: a step's stencil with the next step's update (the runtime's deferred pairing), else the
    # update with the stencil of the same step
    pair = "loop_jac3d_stnupd_cuda"
    rt.dvmhgb_timing_get(ctypes.cast(getattr(wl, pair), ctypes.c_void_p), ctypes.byref(tot), ctypes.byref(cnt))
    if cnt.value == 0:
        pair = "loop_jac3d_fused_cuda"
        rt.dvmhgb_timing_get(ctypes.cast(getattr(wl, pair), ctypes.c_void_p), ctypes.byref(tot), ctypes.byref(cnt))
    rt.dvmhgb_set_timing(0)
    kern_ms = tot.value / max(cnt.value, 1)
    peak, peak_kind = peaks()
    achieved = BYTES_PER_CELL * cells / (kern_ms * 1e-3) / 1e9
    value = reps.world * cells / (ms * 1e-3)  # whole job: every replica's cells
    # the stencil's five FP64 additions per cell against the measured FP64 addition rate
    rate = ctypes.c_double(0.0)
    fp64_peak = rate.value if rt.dvmhgb_fp64_add_rate(ctypes.byref(rate)) == 0 else None
    fp64_achieved = FP64_ADDS_PER_CELL * cells / (kern_ms * 1e-3)

    # e2e: host arrays in, host arrays out, through the C ABI
    e2e_runs = 2
    g.set_mode("batched")
    j = g.Jacobi(3, n, SEED)
    j.run(3)  # graphs captured
    j.pull()
    g.sync()
    torch.cuda.synchronize()
    reps.barrier()
    t0 = time.time()
    for _ in range(e2e_runs):
        j.push()  # the program's pinned host arrays are the input: uploaded by the first step
        j.run(args.steps)
        j.pull()  # and the output: get_actual of A and B
    dt = reps.max(time.time() - t0)
    j.close()
    e2e = {"value": reps.world * cells * args.steps * e2e_runs / dt, "unit": "cell-updates/s",
           "h2d_bytes_per_step": int((2 * 8 * n ** 3 + 8 * args.steps) / args.steps),
           "d2h_bytes_per_step": int((2 * 8 * n ** 3 + 8 * args.steps) / args.steps),
           "note": "per run: A,B uploaded from the program's pinned host arrays (actual), %d steps, "
                   "A,B read back (get_actual)" % args.steps}

    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: splitmix64-seeded uniform[0,1) interior, zero boundary",
            "config": {"workload": "jacobi3d-7pt fp64 %d^3 (%d^3 interior), update+MAX, renew, stencil per step"
                                   % (n, n - 2), "grid": n, "mode": "batched (one captured graph per step, loop pair through the fusion rule)",
                       "l2": "no flush: inputs 2 x %.2f GB > 129 MB L2" % (8 * n ** 3 / 1e9),
                       "parallelism": "replicas" if args.gpus > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": None,
                         "kernel": (pair + ": a step's stencil with the next step's update in one pass -- "
                                    "kStencil3T<3> (planes staged by TMA, q61 sums on the integer pipes, |B - A| on "
                                    "the FP64 unit, B and the new A written) -- in the step's captured graph")
                                   if pair == "loop_jac3d_stnupd_cuda" else
                                   (pair + ": the update+stencil pair of the fusion rule -- kUpdate (fixed-point "
                                    "MAX, A = B), then kStencil3T writing B in place -- in the step's captured graph"),
                         "bytes_per_launch": BYTES_PER_CELL * cells, "launch_ms": kern_ms,
                         "hbm_frac_of_step": BYTES_PER_CELL * cells / (ms * 1e-3) / 1e9 / peak},
            "roofline_fp64": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "FP64 add/s",
                              "frac": fp64_achieved / fp64_peak if fp64_peak else None,
                              "ops_per_cell": FP64_ADDS_PER_CELL,
                              "peak_kind": "measured (dvmhgb_fp64_add_rate: independent DADD chains on every SM)",
                              "note": "FP64-add equivalent: most additions run as q61 integer additions"},
            "clocks": ck, "e2e": e2e, "gpu_launches": st["kernel_launches"]}
    traffic = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic):
        try:
            tj = json.load(open(traffic))
            line["roofline"]["traffic"] = tj.get("jac3d_step_bytes_per_launch_512") if n == 512 else None
        except Exception:
            pass

    if not args.quick:
        # the other modes on every replica (collective timing, whole-job values)
        modes = {}
        for mode in ("plain", "async"):
            mms, _, _ = timed_run(mode, min(args.steps, 20), 2)
            modes[mode] = {"value": reps.world * cells / (mms * 1e-3), "ms_per_step": mms}
        modes["batched"] = {"value": value, "ms_per_step": ms}
        line["modes"] = modes
    if not args.quick and rank == 0:
        # secondary workloads and the CPU baseline: rank 0 alone, no collective
        line["configs"] = extra_configs(g, stream)
        v, it, thr = cpu_port_rate(n)
        line["cpu_baseline"] = {"value": v, "unit": "cell-updates/s", "cores": thr, "kind": "port",
                                "sample": "%d Jacobi-3D steps at %d^3 on the host cores" % (it, n)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_only(args, g, stream):
    """One workload alone, device-timed: the small cases the profiles are taken on."""
    import torch
    g.force_variant(args.variant)
    g.set_mode(args.mode)
    if args.only == "gsd2d":
        return run_gsd2d(args, g, stream)
    if args.only == "jacperf":
        return run_jacperf(args, g)
    if args.only == "jacobi3d":
        w = g.Jacobi(3, args.grid, SEED)
        cells, unit = (args.grid - 2) ** 3, "step"
    elif args.only == "jacobi2d":
        w = g.Jacobi(2, args.grid, SEED)
        cells, unit = (args.grid - 2) ** 2, "iteration"
    elif args.only == "sor":
        w = g.Sor(args.grid, 1.5, SEED + 2)
        cells, unit = (args.grid - 2) ** 3, "sweep"
    else:
        w = g.Heat(args.arrays, 64, args.grid, 0.2, SEED + 3)
        cells, unit = w.cells(), "step"
    w.run(args.warmup)
    g.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    w.run(args.steps)
    e1.record(stream)
    g.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    w.close()
    g.force_variant(-1)
    print(json.dumps({"workload": args.only, "grid": args.grid, "mode": args.mode, "variant": args.variant,
                      "steps": args.steps, "ms_per_" + unit: ms, "cell-updates/s": cells / (ms * 1e-3)}), flush=True)


def run_jacperf(args, g):
    """The FP32 Jacobi-3D benchmark program (--grid L, --steps iterations) once,
    after one warm-up run of --warmup iterations; wall time of the whole program."""
    import ctypes
    import numpy as np
    w = g.workloads()
    fp = ctypes.POINTER(ctypes.c_float)
    w.wl_jacperf_run.restype = ctypes.c_long
    w.wl_jacperf_run.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long, fp, fp, fp]
    eps = np.zeros(max(args.steps, args.warmup, 1), dtype=np.float32)
    w.wl_jacperf_run(3, args.grid, max(args.warmup, 1), eps.ctypes.data_as(fp), None, None)
    t0 = time.time()
    its = w.wl_jacperf_run(3, args.grid, args.steps, eps.ctypes.data_as(fp), None, None)
    dt = time.time() - t0
    print(json.dumps({"workload": "jacperf3d_fp32", "grid": args.grid, "mode": args.mode, "iterations": its,
                      "program_wall_ms": 1e3 * dt, "eps_last": float(eps[its - 1])}), flush=True)


def run_gsd2d(args, g, stream):
    """2-D Gauss-Seidel ACROSS (two dependences) through the generated-shape
    handler with one launch per diagonal: the array natural or diagonalised."""
    import ctypes
    import numpy as np
    import torch
    w = g.workloads()
    w.wl_gsd2d_setup.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64]
    w.wl_gsd2d_sweeps.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double)]
    rt = g.runtime()
    rt.dvmhgb_set_autotransform(1 if args.autotfm else 0)
    n, k = args.grid, args.steps
    m = np.zeros(max(k, 4))
    mp = m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    w.wl_gsd2d_setup(n, n, SEED + 4)
    g.reset_stats()
    tuned = None
    if args.autotfm == 2:
        # the tuner's exploration (immediate execution), then its choice in the timed mode
        rt.dvmhgb_set_tuning(1)
        g.set_mode("plain")
        w.wl_gsd2d_sweeps(5, 1, 1, 1, 0, mp)
        best = (ctypes.c_double * 2)()
        rt.dvmhgb_tuner_layout.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        choice = rt.dvmhgb_tuner_layout(ctypes.cast(w.loop_gsd2d_cuda, ctypes.c_void_p), best)
        tuned = {"choice": ["natural", "transformed"][choice] if choice >= 0 else None,
                 "best_ms_natural": best[0] * 1e3, "best_ms_transformed": best[1] * 1e3}
        g.set_mode(args.mode)
    for _ in range(2):  # the queue of k sweeps captured from each starting layout
        w.wl_gsd2d_sweeps(k, 1, 1, 0, 0, mp)
    g.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    w.wl_gsd2d_sweeps(k, 1, 1, 0, 0, mp)
    e1.record(stream)
    g.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / k
    st = g.stats()
    w.wl_gsd2d_free()
    rt.dvmhgb_set_autotransform(1)
    rt.dvmhgb_set_tuning(0)
    cells = (n - 2) ** 2
    print(json.dumps({"workload": "gsd2d", "grid": n, "mode": args.mode, "autotfm": args.autotfm, "sweeps": k,
                      "ms_per_sweep": ms, "cell-updates/s": cells / (ms * 1e-3), "relayouts": st["relayouts"],
                      "graph_replays": st["graph_replays"], "tuner": tuned}), flush=True)


def extra_configs(g, stream):
    import torch
    out = {}
    # SOR 3-D ACROSS 384^3, 20 sweeps
    n, sweeps = 384, 20
    res = {}
    for mode in ("batched", "plain"):
        g.set_mode(mode)
        s = g.Sor(n, 1.5, SEED + 2)
        s.run(2)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run(sweeps)
        e1.record(stream)
        g.sync()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / sweeps
        s.close()
        res[mode] = {"value": (n - 2) ** 3 / (ms * 1e-3), "ms_per_sweep": ms}
    # the same program through cdvmh's generated hyperplane handler (one launch per
    # hyperplane, 3n - 8 per sweep): the reference's own GPU execution shape
    import ctypes
    w = g.workloads()
    w.wl_sor3d_use_generated.argtypes = [ctypes.c_int]
    w.wl_sor3d_use_generated(1)
    try:
        for mode in ("batched", "plain"):
            g.set_mode(mode)
            s = g.Sor(n, 1.5, SEED + 2)
            s.run(2)
            g.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            k = 5
            e0.record(stream)
            s.run(k)
            e1.record(stream)
            g.sync()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / k
            s.close()
            res["generated_hyperplane_" + mode] = {"value": (n - 2) ** 3 / (ms * 1e-3), "ms_per_sweep": ms,
                                                   "launches_per_sweep": 3 * (n - 2) - 2}
    finally:
        w.wl_sor3d_use_generated(0)
        g.set_mode("batched")
    peak, _ = peaks()
    for r in res.values():
        r["hbm_frac"] = r["value"] * 16 / 1e9 / peak
    out["sor3d_across_384"] = {"unit": "cell-updates/s", "bytes_per_cell": 16, **res}
    # batched uneven heat: 256 arrays, sides log-uniform in [64, 2048], 200 steps
    res = {}
    for mode in ("batched", "plain"):
        g.set_mode(mode)
        h = g.Heat(256, 64, 2048, 0.2, SEED + 3)
        cells = h.cells()
        steps = 200 if mode == "batched" else 50
        h.run(3)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.time()
        e0.record(stream)
        h.run(steps)
        e1.record(stream)
        g.sync()
        torch.cuda.synchronize()
        wall = (time.time() - t0) / steps
        ms = e0.elapsed_time(e1) / steps
        h.close()
        res[mode] = {"value": cells / (ms * 1e-3), "ms_per_step": ms, "wall_ms_per_step": 1000 * wall, "steps": steps}
    for m in ("batched", "plain"):
        res[m]["hbm_frac"] = res[m]["value"] * 16 / 1e9 / peak
    res["batched_over_plain"] = res["batched"]["value"] / res["plain"]["value"]
    out["heat_batched_256"] = {"unit": "cell-updates/s", "bytes_per_cell": 16, "cells": cells, **res}
    g.set_mode("batched")
    out["gsd2d_layouts_2048"] = gsd2d_layouts(g, stream, 2048, 2)
    out["jacobi3d_512_generated_handlers"] = jacobi3d_generated(g, stream, 512, 20)
    out["jacobi2d_1024"] = jacobi2d(g, stream, 1024, 100)
    out["jacperf3d_fp32_384"] = jacperf(g, 3, 384, 5.058044, 1e-4)
    out["jacperf2d_fp32_8000"] = jacperf(g, 2, 8000, 58.37598, 1e-3)
    out["tune"] = tune_configs(g)
    return out


def tune_configs(g):
    """The learned tuner on the configurations' own loops (J2 1024^2, J3 512^3,
    SOR 384^3, heat 256 arrays): exhaustive variant tuning at smaller sizes
    trains the variant model; at the configuration's size, exhaustive tuning
    and model-guided tuning are run and compared (tune.configs_eval)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("dvmhgb_tune", os.path.join(ROOT, "dvm-snapshot-r6603-fork_gb300",
                                                                              "tune.py"))
    tune = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tune)
    try:
        return tune.configs_eval(g, seed=SEED, log=lambda *a: None)
    finally:
        g.set_mode("batched")


def jacperf(g, rank, L, answer, tol):
    """The reference's FP32 Jacobi benchmark programs (examples/Performance/
    jac3d_perf.c, jac2d_perf.c) as whole programs through handlers in cdvmh's
    generated shape: per iteration = (T(100 iterations) - T(10)) / 90 of the
    program's wall time, which cancels allocation, the device init loop and
    teardown; every iteration reads eps back as the program does.  verified =
    the example's own check on eps after 100 iterations."""
    import ctypes
    import numpy as np
    from oracle import orc
    w = g.workloads()
    fp = ctypes.POINTER(ctypes.c_float)
    w.wl_jacperf_run.restype = ctypes.c_long
    w.wl_jacperf_run.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long, fp, fp, fp]
    eps = np.zeros(100, dtype=np.float32)
    res = {}
    for mode in ("batched", "plain"):
        g.set_mode(mode)
        w.wl_jacperf_run(rank, L, 3, eps.ctypes.data_as(fp), None, None)
        t = {}
        for its in (10, 100):
            t0 = time.time()
            w.wl_jacperf_run(rank, L, its, eps.ctypes.data_as(fp), None, None)
            t[its] = time.time() - t0
        ms = 1e3 * (t[100] - t[10]) / 90
        res[mode] = {"ms_per_iteration": ms, "value": (L - 2) ** rank / (ms * 1e-3),
                     "eps_100": float(eps[99]), "verified": bool(abs(float(eps[99]) - answer) < tol)}
    g.set_mode("batched")
    peak, _ = peaks()
    for m in ("batched", "plain"):
        res[m]["hbm_frac"] = res[m]["value"] * 20 / 1e9 / peak
    # the CPU port (oracle restatement, every host thread), 10 iterations
    L_ = orc.lib()
    t0 = time.time()
    orc.jacperf_run(rank, L, 10)
    t10 = time.time() - t0
    t0 = time.time()
    orc.jacperf_run(rank, L, 1)
    t1 = time.time() - t0
    res["cpu_port"] = {"ms_per_iteration": 1e3 * (t10 - t1) / 9, "cores": L_.orc_max_threads()}
    res["cpu_port"]["value"] = (L - 2) ** rank / (res["cpu_port"]["ms_per_iteration"] * 1e-3)
    return {"unit": "cell-updates/s", "bytes_per_cell": 20, "dtype": "f32", "reference_check": [answer, tol], **res}


def jacobi3d_generated(g, stream, n, steps):
    """The headline program through cdvmh's generated one-point-per-thread
    handlers (the reference's GPU kernel shape: one MAX slot per launched
    thread, default 32 x 4 x 2 blocks) on this runtime, beside the library's
    kernels in the headline line."""
    import ctypes
    import torch
    w = g.workloads()
    w.wl_jac3d_use_generated.argtypes = [ctypes.c_int]
    w.wl_jac3d_use_generated(1)
    res = {}
    try:
        for mode in ("batched", "plain"):
            g.set_mode(mode)
            j = g.Jacobi(3, n, SEED)
            j.run(3)
            g.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            j.run(steps)
            e1.record(stream)
            g.sync()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            j.close()
            res[mode] = {"ms_per_step": ms, "value": (n - 2) ** 3 / (ms * 1e-3)}
    finally:
        w.wl_jac3d_use_generated(0)
        g.set_mode("batched")
    return {"unit": "cell-updates/s", "bytes_per_cell": 32, **res}


def jacobi2d(g, stream, n, iters):
    """The 2-D Jacobi configuration (1024^2, 100 iterations of update + renew + stencil
    with a MAX reduction each), on the GPU in every mode, beside the CPU port."""
    import torch
    from oracle import orc
    res = {}
    for mode in ("batched", "async", "plain"):
        g.set_mode(mode)
        j = g.Jacobi(2, n, SEED)
        j.run(3)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        j.run(iters)
        e1.record(stream)
        g.sync()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / iters
        j.close()
        res[mode] = {"ms_per_iteration": ms, "value": (n - 2) ** 2 / (ms * 1e-3)}
    g.set_mode("batched")
    L = orc.lib()
    threads = L.orc_max_threads()
    A, B = orc.jacobi_init(2, n, SEED)
    L.orc_jacobi_step(2, n, orc.P(A), orc.P(B), threads)
    t0 = time.time()
    for _ in range(iters):
        L.orc_jacobi_step(2, n, orc.P(A), orc.P(B), threads)
    dt = time.time() - t0
    res["cpu_port"] = {"value": (n - 2) ** 2 * iters / dt, "cores": threads,
                       "ms_per_iteration": 1e3 * dt / iters}
    return {"unit": "cell-updates/s", "bytes_per_cell": 32, **res}


def gsd2d_layouts(g, stream, n, k):
    """A generated two-dependence ACROSS handler (one launch per diagonal) with its
    array natural, diagonalised as the reference chooses, and as the tuner chooses."""
    import ctypes
    import numpy as np
    import torch
    w, rt = g.workloads(), g.runtime()
    w.wl_gsd2d_setup.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64]
    w.wl_gsd2d_sweeps.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double)]
    rt.dvmhgb_tuner_layout.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    m = np.zeros(8)
    mp = m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    res = {}
    for name, tfm, tune in (("natural", 0, 0), ("diagonal", 1, 0), ("tuned", 1, 1)):
        rt.dvmhgb_set_autotransform(tfm)
        w.wl_gsd2d_setup(n, n, SEED + 4)
        if tune:
            rt.dvmhgb_set_tuning(1)
            g.set_mode("plain")
            w.wl_gsd2d_sweeps(5, 1, 1, 1, 0, mp)  # the tuner's exploration
            g.set_mode("batched")
        for _ in range(2):
            w.wl_gsd2d_sweeps(k, 1, 1, 0, 0, mp)
        g.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.wl_gsd2d_sweeps(k, 1, 1, 0, 0, mp)
        e1.record(stream)
        g.sync()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        res[name] = {"ms_per_sweep": ms, "value": (n - 2) ** 2 / (ms * 1e-3)}
        if tune:
            choice = rt.dvmhgb_tuner_layout(ctypes.cast(w.loop_gsd2d_cuda, ctypes.c_void_p), None)
            res[name]["choice"] = ["natural", "diagonal"][choice] if choice >= 0 else None
            rt.dvmhgb_set_tuning(0)
        w.wl_gsd2d_free()
    rt.dvmhgb_set_autotransform(1)
    return {"unit": "cell-updates/s", "launches_per_sweep": 2 * n - 5, **res}


if __name__ == "__main__":
    main()
