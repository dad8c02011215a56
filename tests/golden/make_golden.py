"""Generate tests/golden/golden.json from the REFERENCE runtime.

Builds the reference DVM-system runtime from its sources (oracle/ref.mk, host
handlers only) together with the workload programs, runs each case with
DVMH_NUM_THREADS=1 (sequential loop order) and records the outputs: reduction
values as exact float.hex strings, final arrays as SHA-256 of their dense
little-endian float64 bytes (and in full for tiny cases).

Run here (needs the reference sources):  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.build import reference_source  # noqa: E402

REF = reference_source()
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# (name, program, params, keep full arrays)
CASES = [
    ("jac2d_n12_it4", "jac2d", [12, 4, 5], True),
    ("jac2d_n3_it2", "jac2d", [3, 2, 9], True),
    ("jac2d_n67_it7", "jac2d", [67, 7, 21], False),
    ("jac2d_n1024_it100", "jac2d", [1024, 100, 20261203], False),
    ("jac3d_n10_it3", "jac3d", [10, 3, 7], True),
    ("jac3d_n3_it2", "jac3d", [3, 2, 3], True),
    ("jac3d_n4_it3", "jac3d", [4, 3, 4], True),
    ("jac3d_n67_it3", "jac3d", [67, 3, 20261204], False),
    ("jac3d_n130_it2", "jac3d", [130, 2, 20261204], False),
    ("sor3d_n10_sw3", "sor3d", [10, 3, 1.5, 11], True),
    ("sor3d_n5_sw2", "sor3d", [5, 2, 1.5, 2], True),
    ("sor3d_n35_sw3", "sor3d", [35, 3, 1.5, 20261205], False),
    ("sor3d_n70_sw2", "sor3d", [70, 2, 1.5, 20261205], False),
    ("heat_c5_s3", "heat", [5, 5, 40, 3, 0.2, 13], True),
    ("heat_c24_s6", "heat", [24, 3, 150, 6, 0.2, 20261206], False),
    # genred: n start end step seed, then the initial values ds dp dml imn ia io ix fmx lc
    ("genred_n1000_s7", "genred", [1000, 3, 990, 7, 1017, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9], True),
    ("genred_n5000_sm13", "genred", [5000, 4990, 2, -13, 5017, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9],
     True),
    ("genred_n300000_s1", "genred", [300000, 0, 299999, 1, 300017, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0,
                                     -9], True),
    ("genred_empty", "genred", [100, 50, 10, 1, 117, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9], True),
    ("genred_n777_sm1", "genred", [777, 776, 0, -1, 794, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9], True),
    ("genred_n777_keep", "genred", [777, 0, 776, 3, 795, -3.5, 0.25, 0.0, -2147483648, 0, -1, 0, 2.0, 41], True),
    # genredx: genred on the edge-value patterns of wl_genred_pattern (the fifth parameter)
    ("genredx_p0_n5000", "genredx", [5000, 0, 4999, 1, 0, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9], True),
    ("genredx_p0_n3001_sm3", "genredx", [3001, 3000, 0, -3, 0, 0.0, -1.0, 1.0, 0, -1, 0, 0, -1.0, 5], True),
    ("genredx_p1_n4097", "genredx", [4097, 0, 4096, 1, 1, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9], True),
    ("genredx_p2_n70000", "genredx", [70000, 1, 69998, 2, 2, 0.125, 1.5, 0.75, 123, -1, 256, 1515870810, -2.0, -9],
     True),
    ("genredx_p2_n9000_sm1", "genredx", [9000, 8999, 0, -1, 2, 0.0, 1.0, 0.5, 7, -1, 0, 0, 0.5, 3], True),
    # jacperf: rank L itmax (the reference's FP32 benchmarks; the last two are their
    # full configurations, whose final eps the examples verify)
    ("jacperf3_L12_it5", "jacperf", [3, 12, 5], True),
    ("jacperf2_L20_it7", "jacperf", [2, 20, 7], True),
    ("jacperf2_L10_it100", "jacperf", [2, 10, 100], True),
    ("jacperf3_L67_it9", "jacperf", [3, 67, 9], False),
    ("jacperf3_L384_it100", "jacperf", [3, 384, 100], False),
    ("jacperf2_L8000_it100", "jacperf", [2, 8000, 100], False),
    # gen3d: n0 n1 n2 seed, then the initial values s mx lc
    ("gen3d_6x7x9", "gen3d", [6, 7, 9, 3, 0.5, -1.0, -5], True),
    ("gen3d_3x3x3", "gen3d", [3, 3, 3, 12, 0.0, -1.0, -1], True),
    ("gen3d_40x33x70_keep", "gen3d", [40, 33, 70, 20261210, -7.25, 5.0, 77], False),
    ("gen3d_64x64x64", "gen3d", [64, 64, 64, 20261211, 0.0, -1.0, -1], False),
    ("rec2d_5x9_sw2", "rec2d", [5, 9, 2, 3], True),
    ("rec2d_37x52_sw3", "rec2d", [37, 52, 3, 4], False),
    ("rec2d_1x40_sw2", "rec2d", [1, 40, 2, 8], True),
    ("gsd3d_3x6x7_sw2", "gsd3d", [3, 6, 7, 2, 4], True),
    ("gsd3d_5x19x27_sw3", "gsd3d", [5, 19, 27, 3, 40], False),
    ("gs2d_n8_sw2", "gs2d", [8, 2, 5], True),
    ("gs2d_n61_sw3", "gs2d", [61, 3, 20261209], False),
    ("gsd2d_9x7_fwd_mirror", "gsd2d", [9, 7, 3, 31, 1, 1, 1], True),
    ("gsd2d_6x11_slash", "gsd2d", [6, 11, 2, 32, 1, -1, 0], True),
    # The reference crashes (SIGSEGV in libdvm's across_) when an axis with a
    # single iteration runs backward, so the single-row case runs it forward.
    ("gsd2d_3x30_rowback", "gsd2d", [3, 30, 2, 33, 1, -1, 0], True),
    ("gsd2d_4x30_back", "gsd2d", [4, 30, 2, 34, -1, -1, 1], True),
    ("gsd2d_96x200_mixed", "gsd2d", [96, 200, 4, 20261207, -1, 1, 1], False),
    ("gsd2d_257x129_fwd", "gsd2d", [257, 129, 3, 20261208, 1, 1, 0], False),
    # cdvh2d: n iters seed (the program in cdvmh's converted form: regular variables, dynamic arrays)
    ("cdvh2d_n12_it3", "cdvh2d", [12, 3, 5], True),
    ("cdvh2d_n3_it2", "cdvh2d", [3, 2, 6], True),
    ("cdvh2d_n97_it5", "cdvh2d", [97, 5, 20261212], False),
    ("cdvh2d_n300_it4", "cdvh2d", [300, 4, 20261213], False),
]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def sha32(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f4").tobytes()).hexdigest()


def hx(a):
    return [float(x).hex() for x in np.asarray(a, dtype=np.float64).ravel()]


def build():
    if REF is None:
        sys.exit("make_golden: the reference sources are needed (set DVMH_REF_SRC)")
    subprocess.check_call(["make", "-s", "-f", "oracle/ref.mk", "-j8", "REF=" + REF], cwd=ROOT)


def run(prog, params):
    # one thread (loop order) except for the FP32 benchmarks, whose only
    # reduction is MAX: order-independent, so they may use every core
    threads = str(os.cpu_count()) if prog == "jacperf" else "1"
    if prog == "jacperf":
        params = list(params) + [1]
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        env = dict(os.environ, DVMH_NUM_THREADS=threads, OMP_SCHEDULE="static")
        subprocess.check_call([DRIVER, prog, out] + [str(p) for p in params], cwd=td, env=env,
                              stdout=subprocess.DEVNULL)
        return open(out, "rb").read()


def case(name, prog, params, full):
    raw = run(prog, params)
    rec = {"prog": prog, "params": params}
    if prog in ("jac2d", "jac3d"):
        n, it = params[0], params[1]
        cells = n ** (2 if prog == "jac2d" else 3)
        d = np.frombuffer(raw, dtype="<f8")
        rec["eps"] = hx(d[:it])
        A, B = d[it:it + cells], d[it + cells:it + 2 * cells]
        rec["A_sha256"], rec["B_sha256"] = sha(A), sha(B)
        if full:
            rec["A"], rec["B"] = hx(A), hx(B)
    elif prog == "sor3d":
        n, sw = params[0], params[1]
        d = np.frombuffer(raw, dtype="<f8")
        rec["s"] = hx(d[:sw])
        A = d[sw:sw + n ** 3]
        rec["A_sha256"] = sha(A)
        if full:
            rec["A"] = hx(A)
    elif prog in ("genred", "genredx"):
        rec["d3"] = hx(np.frombuffer(raw[0:24], dtype="<f8"))
        rec["i4"] = [int(x) for x in np.frombuffer(raw[24:40], dtype="<i4")]
        rec["f1"] = hx(np.frombuffer(raw[40:44], dtype="<f4"))
        rec["lc"] = int(np.frombuffer(raw[44:52], dtype="<i8")[0])
    elif prog == "jacperf":
        rank, L, itmax = params
        cells = L ** rank
        its = int(np.frombuffer(raw[0:8], dtype="<i8")[0])
        rec["its"] = its
        rec["eps"] = hx(np.frombuffer(raw[8:8 + 4 * its], dtype="<f4"))
        off = 8 + 4 * itmax
        A = np.frombuffer(raw[off:off + 4 * cells], dtype="<f4")
        B = np.frombuffer(raw[off + 4 * cells:off + 8 * cells], dtype="<f4")
        rec["A_sha256"], rec["B_sha256"] = sha32(A), sha32(B)
        if full:
            rec["A"], rec["B"] = hx(A), hx(B)
    elif prog == "gen3d":
        cells = params[0] * params[1] * params[2]
        rec["s_mx"] = hx(np.frombuffer(raw[0:16], dtype="<f8"))
        rec["lc"] = int(np.frombuffer(raw[16:24], dtype="<i8")[0])
        B = np.frombuffer(raw[24:24 + 8 * cells], dtype="<f8")
        rec["B_sha256"] = sha(B)
        if full:
            rec["B"] = hx(B)
    elif prog in ("rec2d", "gsd3d", "gs2d"):
        cells = {"rec2d": lambda p: p[0] * p[1], "gsd3d": lambda p: p[0] * p[1] * p[2],
                 "gs2d": lambda p: p[0] * p[0]}[prog](params)
        sw = params[{"rec2d": 2, "gsd3d": 3, "gs2d": 1}[prog]]
        d = np.frombuffer(raw, dtype="<f8")
        rec["r"] = hx(d[:sw])
        A = d[sw:sw + cells]
        rec["A_sha256"] = sha(A)
        if full:
            rec["A"] = hx(A)
    elif prog == "cdvh2d":
        n, it = params[0], params[1]
        d = np.frombuffer(raw, dtype="<f8")
        rec["eps"] = hx(d[:it])
        B = d[it:it + n * n]
        rec["B_sha256"] = sha(B)
        if full:
            rec["B"] = hx(B)
    elif prog == "gsd2d":
        n0, n1, sw, mirror = params[0], params[1], params[2], params[6]
        d = np.frombuffer(raw, dtype="<f8")
        rec["m"] = hx(d[:sw])
        A = d[sw:sw + n0 * n1]
        rec["A_sha256"] = sha(A)
        if full:
            rec["A"] = hx(A)
        if mirror:
            B = d[sw + n0 * n1:sw + 2 * n0 * n1]
            rec["B_sha256"] = sha(B)
            if full:
                rec["B"] = hx(B)
    else:
        cnt, steps = params[0], params[3]
        off = 0
        sides = np.frombuffer(raw[off:off + 8 * cnt], dtype="<i8")
        off += 8 * cnt
        sums = np.frombuffer(raw[off:off + 8 * cnt * steps], dtype="<f8")
        off += 8 * cnt * steps
        mins = np.frombuffer(raw[off:off + 8 * cnt * steps], dtype="<f8")
        off += 8 * cnt * steps
        locs = np.frombuffer(raw[off:off + 8 * cnt * steps], dtype="<i4")
        off += 8 * cnt * steps
        rec["sides"] = [int(s) for s in sides]
        rec["sums"], rec["mins"] = hx(sums), hx(mins)
        rec["locs"] = [int(x) for x in locs]
        finals = []
        for s in sides:
            a = np.frombuffer(raw[off:off + 8 * int(s) * int(s)], dtype="<f8")
            off += 8 * int(s) * int(s)
            finals.append(sha(a) if not full else hx(a))
        rec["final_sha256" if not full else "final"] = finals
    return rec


def main():
    """All cases, or (arguments given) only the cases whose names start with one
    of the arguments, kept beside the others already in golden.json."""
    build()
    path = os.path.join(ROOT, "tests", "golden", "golden.json")
    only = sys.argv[1:]
    if only and os.path.exists(path):
        out = json.load(open(path))
    else:
        out = {"generator": "tests/golden/make_golden.py", "runtime": "reference host handlers, DVMH_NUM_THREADS=1",
               "cases": {}}
    for name, prog, params, full in CASES:
        if only and not any(name.startswith(o) for o in only):
            continue
        print("case", name, file=sys.stderr)
        out["cases"][name] = case(name, prog, params, full)
    path = os.path.join(ROOT, "tests", "golden", "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print("wrote", path, os.path.getsize(path), "bytes", file=sys.stderr)


if __name__ == "__main__":
    main()
