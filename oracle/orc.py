"""ctypes binding of the CPU restatement (oracle/restate.c).

Test infrastructure only (checker and CPU-baseline port); never imported by
the product path.
"""
import ctypes
import os

import numpy as np

from . import build as _build  # noqa: F401  (package-relative when imported as oracle.orc)

_dp = ctypes.POINTER(ctypes.c_double)
_L = None


def lib():
    global _L
    if _L is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.orc_u01.restype = ctypes.c_double
        L.orc_u01.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_pairwise_sum.restype = ctypes.c_double
        L.orc_pairwise_sum.argtypes = [_dp, ctypes.c_long]
        L.orc_canon_sum.restype = ctypes.c_double
        L.orc_canon_sum.argtypes = [_dp, ctypes.c_long, ctypes.c_long, ctypes.c_long]
        L.orc_jacobi_init.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_uint64, _dp, _dp]
        L.orc_jacobi_step.restype = ctypes.c_double
        L.orc_jacobi_step.argtypes = [ctypes.c_int, ctypes.c_long, _dp, _dp, ctypes.c_int]
        L.orc_sor_init.argtypes = [ctypes.c_long, ctypes.c_uint64, _dp]
        L.orc_sor_sweep.restype = ctypes.c_double
        L.orc_sor_sweep.argtypes = [ctypes.c_long, ctypes.c_double, _dp, _dp]
        L.orc_sor_sweep_cols.argtypes = [ctypes.c_long, ctypes.c_double, _dp, _dp]
        L.orc_heat_side.restype = ctypes.c_long
        L.orc_heat_side.argtypes = [ctypes.c_uint64, ctypes.c_long, ctypes.c_long, ctypes.c_long]
        L.orc_heat_init.argtypes = [ctypes.c_long, ctypes.c_uint64, ctypes.c_long, _dp, _dp]
        L.orc_heat_step.argtypes = [ctypes.c_long, ctypes.c_double, _dp, _dp, _dp, _dp, _dp,
                                    ctypes.POINTER(ctypes.c_int)]
        L.orc_gsd2d_init.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64, _dp]
        L.orc_gsd2d_sweep.restype = ctypes.c_double
        L.orc_gsd2d_sweep.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_diag_index.restype = ctypes.c_long
        L.orc_diag_index.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_int]
        L.orc_genred.argtypes = [ctypes.c_long] * 4 + [ctypes.c_uint64, _dp, ctypes.POINTER(ctypes.c_int),
                                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_long)]
        L.orc_gs2d_init.argtypes = [ctypes.c_long, ctypes.c_uint64, _dp]
        L.orc_gs2d_sweep.restype = ctypes.c_double
        L.orc_gs2d_sweep.argtypes = [ctypes.c_long, _dp]
        L.orc_rec2d_init.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64, _dp]
        L.orc_rec2d_sweep.restype = ctypes.c_double
        L.orc_rec2d_sweep.argtypes = [ctypes.c_long, ctypes.c_long, _dp]
        L.orc_gen3d.argtypes = [ctypes.c_long] * 3 + [ctypes.c_uint64, _dp, _dp, ctypes.POINTER(ctypes.c_long), _dp]
        _ip = ctypes.POINTER(ctypes.c_int)
        L.orc_genred_data.argtypes = [ctypes.c_long] * 4 + [_dp, _ip, _dp, _ip, ctypes.POINTER(ctypes.c_float),
                                                            ctypes.POINTER(ctypes.c_long)]
        L.orc_genred_pattern.argtypes = [ctypes.c_int, ctypes.c_long, _dp, _ip]
        _fp = ctypes.POINTER(ctypes.c_float)
        L.orc_jacperf.restype = ctypes.c_long
        L.orc_jacperf.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long, _fp, _fp, _fp]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_cdvh2d.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_uint64, _dp, _dp]
        _L = L
    return _L


def P(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def jacobi_init(rank, n, seed):
    A = np.zeros(n ** rank)
    B = np.zeros(n ** rank)
    lib().orc_jacobi_init(rank, n, seed, P(A), P(B))
    return A, B


def jacobi_run(rank, n, iters, seed, threads=1):
    A, B = jacobi_init(rank, n, seed)
    eps = [lib().orc_jacobi_step(rank, n, P(A), P(B), threads) for _ in range(iters)]
    return np.array(eps), A, B


def cdvh2d_run(n, iters, seed):
    """The weighted Jacobi 2-D program of workloads/cdvh2d.c: (eps per iteration, B)."""
    eps, B = np.zeros(iters), np.zeros(n * n)
    lib().orc_cdvh2d(n, iters, seed, P(eps), P(B))
    return eps, B


def sor_run(n, sweeps, omega, seed):
    """Returns (sequential-order residuals, canonical-tree residuals, A)."""
    A = np.zeros(n ** 3)
    lib().orc_sor_init(n, seed, P(A))
    seq, can = [], []
    for _ in range(sweeps):
        c = ctypes.c_double()
        seq.append(lib().orc_sor_sweep(n, omega, P(A), ctypes.byref(c)))
        can.append(c.value)
    return np.array(seq), np.array(can), A


def pairwise(v, op=np.add, ident=-0.0):
    """the pairwise tree over slot indices, identity padding to a power of two"""
    v = np.asarray(v, dtype=np.float64)
    m = 1
    while m < len(v):
        m *= 2
    v = np.concatenate([v, np.full(m - len(v), ident)])
    while len(v) > 1:
        v = op(v[0::2], v[1::2])
    return float(v[0])


def sor_run_columns(n, sweeps, omega, seed):
    """SOR sweeps whose SUM is folded as the hyperplane handler folds it: per
    (i, j) column in k order, then the pairwise tree over the columns, then
    (0 + fold) + 0.  Returns (sums, A)."""
    A = np.zeros(n ** 3)
    lib().orc_sor_init(n, seed, P(A))
    cols = np.zeros((n - 2) ** 2)
    out = []
    for _ in range(sweeps):
        lib().orc_sor_sweep_cols(n, omega, P(A), P(cols))
        out.append((0.0 + pairwise(cols)) + 0.0)
    return np.array(out), A


def heat_sides(count, lo, hi, seed):
    return [int(lib().orc_heat_side(seed, k, lo, hi)) for k in range(count)]


def heat_run(count, lo, hi, steps, coef, seed):
    """Returns dict: sides, sums_seq, sums_canon, mins, locs ([steps][count]...), finals."""
    sides = heat_sides(count, lo, hi, seed)
    out = {"sides": sides, "sums_seq": np.zeros((steps, count)), "sums_canon": np.zeros((steps, count)),
           "mins": np.zeros((steps, count)), "locs": np.zeros((steps, count, 2), dtype=np.int32), "finals": []}
    for k, n in enumerate(sides):
        U = np.zeros(n * n)
        V = np.zeros(n * n)
        lib().orc_heat_init(n, seed, k, P(U), P(V))
        src, dst = U, V
        for t in range(steps):
            ss, sc, mn = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
            lc = (ctypes.c_int * 2)()
            lib().orc_heat_step(n, coef, P(src), P(dst), ctypes.byref(ss), ctypes.byref(sc), ctypes.byref(mn), lc)
            out["sums_seq"][t, k], out["sums_canon"][t, k], out["mins"][t, k] = ss.value, sc.value, mn.value
            out["locs"][t, k] = list(lc)
            src, dst = dst, src
        out["finals"].append(src)
    return out


def gsd2d_run(n0, n1, sweeps, seed, dir0=1, dir1=1):
    A = np.zeros(n0 * n1)
    L = lib()
    L.orc_gsd2d_init(n0, n1, seed, P(A))
    m = [L.orc_gsd2d_sweep(n0, n1, dir0, dir1, P(A)) for _ in range(sweeps)]
    return np.array(m), A


def gs2d_run(n, sweeps, seed):
    A = np.zeros(n * n)
    L = lib()
    L.orc_gs2d_init(n, seed, P(A))
    s = [L.orc_gs2d_sweep(n, P(A)) for _ in range(sweeps)]
    return np.array(s), A


def rec2d_run(n0, n1, sweeps, seed):
    A = np.zeros(n0 * n1)
    L = lib()
    L.orc_rec2d_init(n0, n1, seed, P(A))
    lo = [L.orc_rec2d_sweep(n0, n1, P(A)) for _ in range(sweeps)]
    return np.array(lo), A


def gsd3d_run(n0, n1, n2, sweeps, seed):
    """plane k is the 2-D program with seed + k; m = MAX over the planes per sweep"""
    planes = [gsd2d_run(n1, n2, sweeps, seed + k) for k in range(n0)]
    m = np.max(np.stack([p[0] for p in planes]), axis=0)
    return m, np.concatenate([p[1] for p in planes])


def gen3d_run(n0, n1, n2, seed, s, mx, lc):
    """returns (s, mx, lc, B) of the sequential loop; B dense n0*n1*n2"""
    B = np.zeros(n0 * n1 * n2)
    sv, mv = ctypes.c_double(s), ctypes.c_double(mx)
    lv = ctypes.c_long(lc)
    lib().orc_gen3d(n0, n1, n2, seed, ctypes.byref(sv), ctypes.byref(mv), ctypes.byref(lv), P(B))
    return sv.value, mv.value, lv.value, B


def jacperf_run(rank, L, itmax):
    """FP32 Jacobi benchmark: (iterations run, eps per iteration, A, B) as float32"""
    fp = ctypes.POINTER(ctypes.c_float)
    eps = np.zeros(itmax, dtype=np.float32)
    A = np.zeros(L ** rank, dtype=np.float32)
    B = np.zeros(L ** rank, dtype=np.float32)
    its = lib().orc_jacperf(rank, L, itmax, eps.ctypes.data_as(fp), A.ctypes.data_as(fp), B.ctypes.data_as(fp))
    return its, eps[:its], A, B


def genred_pattern(pattern, n):
    x = np.zeros(n)
    v = np.zeros(n, dtype=np.int32)
    lib().orc_genred_pattern(pattern, n, P(x), v.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return x, v


def genred_run_data(n, start, end, step, x, v, init):
    """genred_run on given inputs x (float64) and v (int32)"""
    d3 = np.array(init[0:3], dtype=np.float64)
    i4 = (ctypes.c_int * 4)(*[int(q) for q in init[3:7]])
    f1 = (ctypes.c_float * 1)(init[7])
    lc = (ctypes.c_long * 1)(int(init[8]))
    v = np.ascontiguousarray(v, dtype=np.int32)
    lib().orc_genred_data(n, start, end, step, P(np.ascontiguousarray(x, dtype=np.float64)),
                          v.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), P(d3), i4, f1, lc)
    return (float(d3[0]), float(d3[1]), float(d3[2]), i4[0], i4[1], i4[2], i4[3], f1[0], lc[0])


def genred_run(n, start, end, step, seed, init):
    """init = (ds, dp, dml, imn, ia, io, ix, fmx, lc); returns the results in the same order."""
    d3 = np.array(init[0:3], dtype=np.float64)
    i4 = (ctypes.c_int * 4)(*[int(x) for x in init[3:7]])
    f1 = (ctypes.c_float * 1)(init[7])
    lc = (ctypes.c_long * 1)(int(init[8]))
    lib().orc_genred(n, start, end, step, seed, P(d3), i4, f1, lc)
    return (float(d3[0]), float(d3[1]), float(d3[2]), i4[0], i4[1], i4[2], i4[3], f1[0], lc[0])
