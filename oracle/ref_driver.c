/*
 * Driver that runs a workload program (dvm-snapshot-r6603-fork_gb300/workloads/*.c,
 * compiled with WL_NO_CUDA) on the REFERENCE runtime built by oracle/ref.mk, and
 * writes its outputs as raw little-endian binary.  Test infrastructure only: it
 * generates the golden fixtures under tests/golden/ (tests/golden/make_golden.py).
 *
 * usage: ref_driver <prog> <out.bin> <params...>
 *   jac2d|jac3d  n iters seed          -> eps[iters], A[n^r], B[n^r]
 *   sor3d        n sweeps omega seed   -> s[sweeps], A[n^3]
 *   heat         count lo hi steps coef seed
 *                -> sides[count] (int64), then per step: sums[count], mins[count],
 *                   locs[count][2] (int32), then the final arrays in order
 *   genred       n start end step seed ds dp dml imn ia io ix fmx lc   (initial values)
 *                -> ds dp dml (f64), imn ia io ix (int32), fmx (f32), lc (int64)
 *   genredx      n start end step pattern ds dp dml imn ia io ix fmx lc
 *                -> as genred, on the inputs of wl_genred_pattern(pattern)
 *   gen3d        n0 n1 n2 seed s mx lc  -> s, mx (f64), lc (int64), B[n0*n1*n2]
 *   jacperf      rank L itmax full      -> iterations run (int64), eps[itmax] (f32, 0 past
 *                                          the last), then A, B (f32, L^rank) when full
 *   rec2d        n0 n1 sweeps seed      -> lo[sweeps], A[n0*n1]
 *   gsd3d        n0 n1 n2 sweeps seed   -> m[sweeps], A[n0*n1*n2]
 *   gs2d         n sweeps seed          -> s[sweeps], A[n*n]
 *   gsd2d        n0 n1 sweeps seed dir0 dir1 mirror
 *                -> m[sweeps] (read after every sweep), A[n0*n1], then B[n0*n1]
 *                   when mirror
 *   cdvh2d       n iters seed           -> eps[iters], B[n*n]
 * Run with DVMH_NUM_THREADS=1 for the sequential (order-exact) oracle.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

int wl_jac2d_setup(const wl_jacobi_params *p);
int wl_jac2d_run(long iters, double *eps_out);
int wl_jac2d_fetch(double *a_out, double *b_out);
int wl_jac3d_setup(const wl_jacobi_params *p);
int wl_jac3d_run(long iters, double *eps_out);
int wl_jac3d_fetch(double *a_out, double *b_out);
int wl_sor3d_setup(const wl_sor_params *p);
int wl_sor3d_run(long sweeps, double *s_out);
int wl_sor3d_fetch(double *a_out);
int wl_heat_setup(const wl_heat_params *p, long *sides_out);
int wl_heat_run(long steps, double *sums_out, double *mins_out, int *locs_out);
int wl_heat_fetch(long k, double *u_out);
int wl_genred_run(long n, long start, long end, long step, uint64_t seed, int bx, double *d3, int *i4, float *f1,
                  long *lc);
int wl_genred_pattern(int pattern, long n, double *x, int *v);
int wl_genred_run_data(long n, long start, long end, long step, const double *x, const int *v, int bx, double *d3,
                       int *i4, float *f1, long *lc);
int wl_gen3d_run(long n0, long n1, long n2, uint64_t seed, int bx, int by, int bz, double *s, double *mx, long *lc,
                 double *b_out);
long wl_jacperf_run(int rank, long L, long itmax, float *eps_out, float *a_out, float *b_out);
int wl_rec2d_run(long n0, long n1, long sweeps, uint64_t seed, double *lo_out, double *a_out);
int wl_gsd3d_run(long n0, long n1, long n2, long sweeps, uint64_t seed, double *m_out, double *a_out);
int wl_gs2d_run(long n, long sweeps, uint64_t seed, double *s_out, double *a_out);
int wl_gsd2d_run(long n0, long n1, long sweeps, uint64_t seed, int dir0, int dir1, int readEach, int mirror,
                 double *m_out, double *a_out, double *b_out);
int wl_cdvh2d_run(long n, long iters, unsigned long long seed, double *eps_out, double *b_out);

static void put(FILE *f, const void *p, size_t bytes) {
    if (fwrite(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "write failed\n");
        exit(2);
    }
}

int main(int argc, char **argv) {
    FILE *f;
    if (argc < 3) {
        fprintf(stderr, "usage: %s prog out.bin params...\n", argv[0]);
        return 2;
    }
    dvmh_init_C(0, &argc, &argv);
    f = fopen(argv[2], "wb");
    if (!f)
        return 2;
    if (!strcmp(argv[1], "jac2d") || !strcmp(argv[1], "jac3d")) {
        int r3 = !strcmp(argv[1], "jac3d");
        wl_jacobi_params p;
        size_t cells;
        double *e, *a, *b;
        p.n = atol(argv[3]);
        p.iters = atol(argv[4]);
        p.seed = strtoull(argv[5], 0, 10);
        cells = (size_t)p.n * p.n * (r3 ? p.n : 1);
        e = malloc(sizeof(double) * p.iters);
        a = malloc(sizeof(double) * cells);
        b = malloc(sizeof(double) * cells);
        if (r3) {
            wl_jac3d_setup(&p);
            wl_jac3d_run(p.iters, e);
            wl_jac3d_fetch(a, b);
        } else {
            wl_jac2d_setup(&p);
            wl_jac2d_run(p.iters, e);
            wl_jac2d_fetch(a, b);
        }
        put(f, e, sizeof(double) * p.iters);
        put(f, a, sizeof(double) * cells);
        put(f, b, sizeof(double) * cells);
    } else if (!strcmp(argv[1], "sor3d")) {
        wl_sor_params p;
        size_t cells;
        double *s, *a;
        p.n = atol(argv[3]);
        p.sweeps = atol(argv[4]);
        p.omega = atof(argv[5]);
        p.seed = strtoull(argv[6], 0, 10);
        cells = (size_t)p.n * p.n * p.n;
        s = malloc(sizeof(double) * p.sweeps);
        a = malloc(sizeof(double) * cells);
        wl_sor3d_setup(&p);
        wl_sor3d_run(p.sweeps, s);
        wl_sor3d_fetch(a);
        put(f, s, sizeof(double) * p.sweeps);
        put(f, a, sizeof(double) * cells);
    } else if (!strcmp(argv[1], "heat")) {
        wl_heat_params p;
        long *sides, k;
        double *sums, *mins, *u;
        int *locs;
        p.count = atol(argv[3]);
        p.side_lo = atol(argv[4]);
        p.side_hi = atol(argv[5]);
        p.steps = atol(argv[6]);
        p.coef = atof(argv[7]);
        p.seed = strtoull(argv[8], 0, 10);
        sides = malloc(sizeof(long) * p.count);
        sums = malloc(sizeof(double) * p.count * p.steps);
        mins = malloc(sizeof(double) * p.count * p.steps);
        locs = malloc(sizeof(int) * 2 * p.count * p.steps);
        wl_heat_setup(&p, sides);
        wl_heat_run(p.steps, sums, mins, locs);
        put(f, sides, sizeof(long) * p.count);
        put(f, sums, sizeof(double) * p.count * p.steps);
        put(f, mins, sizeof(double) * p.count * p.steps);
        put(f, locs, sizeof(int) * 2 * p.count * p.steps);
        for (k = 0; k < p.count; k++) {
            u = malloc(sizeof(double) * sides[k] * sides[k]);
            wl_heat_fetch(k, u);
            put(f, u, sizeof(double) * sides[k] * sides[k]);
            free(u);
        }
    } else if (!strcmp(argv[1], "genred") || !strcmp(argv[1], "genredx")) {
        long n = atol(argv[3]), start = atol(argv[4]), end = atol(argv[5]), step = atol(argv[6]);
        uint64_t seed = strtoull(argv[7], 0, 10);
        double *xs = 0;
        int *vs = 0;
        double d3[3] = {atof(argv[8]), atof(argv[9]), atof(argv[10])};
        int i4[4] = {atoi(argv[11]), (int)strtol(argv[12], 0, 0), (int)strtol(argv[13], 0, 0),
                     (int)strtol(argv[14], 0, 0)};
        float f1[1] = {(float)atof(argv[15])};
        long lc[1] = {atol(argv[16])};
        if (!strcmp(argv[1], "genredx")) {
            xs = malloc(sizeof(double) * n);
            vs = malloc(sizeof(int) * n);
            wl_genred_pattern((int)seed, n, xs, vs);
            wl_genred_run_data(n, start, end, step, xs, vs, 0, d3, i4, f1, lc);
        } else {
            wl_genred_run(n, start, end, step, seed, 0, d3, i4, f1, lc);
        }
        put(f, d3, sizeof(d3));
        put(f, i4, sizeof(i4));
        put(f, f1, sizeof(f1));
        put(f, lc, sizeof(lc));
    } else if (!strcmp(argv[1], "gen3d")) {
        long n0 = atol(argv[3]), n1 = atol(argv[4]), n2 = atol(argv[5]);
        uint64_t seed = strtoull(argv[6], 0, 10);
        double s = atof(argv[7]), mx = atof(argv[8]);
        long lc = atol(argv[9]);
        double *b = malloc(sizeof(double) * n0 * n1 * n2);
        wl_gen3d_run(n0, n1, n2, seed, 0, 0, 0, &s, &mx, &lc, b);
        put(f, &s, sizeof(s));
        put(f, &mx, sizeof(mx));
        put(f, &lc, sizeof(lc));
        put(f, b, sizeof(double) * n0 * n1 * n2);
    } else if (!strcmp(argv[1], "jacperf")) {
        int rank = atoi(argv[3]), full = atoi(argv[6]);
        long L = atol(argv[4]), itmax = atol(argv[5]), its, cells = rank == 3 ? L * L * L : L * L;
        float *e = calloc((size_t)itmax, sizeof(float)), *a = 0, *b = 0;
        if (full) {
            a = malloc(sizeof(float) * cells);
            b = malloc(sizeof(float) * cells);
        }
        its = wl_jacperf_run(rank, L, itmax, e, a, b);
        put(f, &its, sizeof(its));
        put(f, e, sizeof(float) * itmax);
        if (full) {
            put(f, a, sizeof(float) * cells);
            put(f, b, sizeof(float) * cells);
        }
    } else if (!strcmp(argv[1], "rec2d") || !strcmp(argv[1], "gs2d") || !strcmp(argv[1], "gsd3d")) {
        int r3 = !strcmp(argv[1], "gsd3d"), sq = !strcmp(argv[1], "gs2d");
        long n0 = atol(argv[3]), n1 = sq ? n0 : atol(argv[4]), n2 = r3 ? atol(argv[5]) : 1;
        long sweeps = atol(argv[sq ? 4 : (r3 ? 6 : 5)]);
        uint64_t seed = strtoull(argv[sq ? 5 : (r3 ? 7 : 6)], 0, 10);
        double *r = malloc(sizeof(double) * sweeps), *a = malloc(sizeof(double) * n0 * n1 * n2);
        if (r3)
            wl_gsd3d_run(n0, n1, n2, sweeps, seed, r, a);
        else if (sq)
            wl_gs2d_run(n0, sweeps, seed, r, a);
        else
            wl_rec2d_run(n0, n1, sweeps, seed, r, a);
        put(f, r, sizeof(double) * sweeps);
        put(f, a, sizeof(double) * n0 * n1 * n2);
    } else if (!strcmp(argv[1], "gsd2d")) {
        long n0 = atol(argv[3]), n1 = atol(argv[4]), sweeps = atol(argv[5]);
        uint64_t seed = strtoull(argv[6], 0, 10);
        int dir0 = atoi(argv[7]), dir1 = atoi(argv[8]), mirror = atoi(argv[9]);
        double *m = malloc(sizeof(double) * sweeps), *a = malloc(sizeof(double) * n0 * n1),
               *b = malloc(sizeof(double) * n0 * n1);
        wl_gsd2d_run(n0, n1, sweeps, seed, dir0, dir1, 1, mirror, m, a, b);
        put(f, m, sizeof(double) * sweeps);
        put(f, a, sizeof(double) * n0 * n1);
        if (mirror)
            put(f, b, sizeof(double) * n0 * n1);
    } else if (!strcmp(argv[1], "cdvh2d")) {
        long n = atol(argv[3]), iters = atol(argv[4]);
        uint64_t seed = strtoull(argv[5], 0, 10);
        double *e = malloc(sizeof(double) * iters), *b = malloc(sizeof(double) * n * n);
        wl_cdvh2d_run(n, iters, seed, e, b);
        put(f, e, sizeof(double) * iters);
        put(f, b, sizeof(double) * n * n);
    } else {
        fprintf(stderr, "unknown program %s\n", argv[1]);
        return 2;
    }
    fclose(f);
    dvmh_exit_C(0);
    return 0;
}
