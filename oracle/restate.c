/*
 * oracle/restate.c -- CPU restatement of the DVMH loop-execution path for the
 * workloads this repository runs.  TEST INFRASTRUCTURE ONLY: tests/, the smoke
 * check and bench.py's CPU-baseline leg load it as the checker / the timed
 * CPU port.  The GPU product never links or calls it.
 *
 * Pinned against the reference runtime itself: tests/golden/ holds outputs of
 * the same workload programs run on the reference's host handlers (built from
 * its sources by oracle/ref.mk, DVMH_NUM_THREADS=1), and tests/test_oracle.py
 * checks this file against those fixtures bit for bit.
 *
 * What it restates (reference file:line):
 *  - loop bodies: examples/Performance/jac3d_perf.c:56-73 (3-D Jacobi, FP64),
 *    examples/Jacobi/jac2d.c:49-64 (2-D Jacobi), examples/Sor/sor.c:45-53 made
 *    3-D with a sum-of-squares residual; the batched heat step is the body of
 *    dvm-snapshot-r6603-fork_gb300/workloads/heat.c.
 *  - reduction semantics: per-thread init (DvmhReduction::initValues,
 *    rts/dvmh/loop.cpp:37-100), combine rules incl. strict '<'/'>' for MAX/MIN
 *    so the first value in loop order wins a tie (RED_MAX/RED_MIN, loop.cpp:117-118),
 *    final result = (identity (+) loop value) (+) initial value
 *    (initGlobalValues + postValues + addInitialValues, rts/dvmh/dvmh2.cpp:3848-3851,3950-3953).
 *  - sequential order = the reference with one host thread.
 *
 * Canonical tree (the GPU's deterministic order for floating SUM/PROD, restated
 * here so GPU results can be checked bit for bit): the loop's iteration box is
 * cut into rows (all indices but the innermost) in loop order; each row into
 * 64-wide chunks aligned to multiples of 64 of the innermost ARRAY index.  A
 * chunk's value is the pairwise tree over its 64 positions (position p pairs
 * with p^1, then p^2, ...), with the identity (-0.0 for SUM, 1.0 for PROD) at
 * positions outside the loop.  Chunks, in row-major order, are then combined by
 * a pairwise tree over their indices padded with the identity to a power of two.
 *
 * Compile with -O2 -ffp-contract=off (no FMA contraction) so every cell's
 * arithmetic is the source program's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Max(a, b) ((a) > (b) ? (a) : (b))
#define CHUNK 64

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* splitmix64 stream `stream` of `seed`, element n, as a double in [0,1) */
double orc_u01(uint64_t seed, uint64_t stream, uint64_t n) {
    uint64_t s0 = seed ^ (0xD1B54A32D192ED03ULL * (stream + 1));
    return (double)(mix64(s0 + (n + 1) * 0x9E3779B97F4A7C15ULL) >> 11) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------ canonical tree */

/* pairwise sum of v[0..n) padded with -0.0 to a power of two (in place, destroys v) */
double orc_pairwise_sum(double *v, long n) {
    long p = 1, len, i;
    if (n <= 0)
        return -0.0;
    while (p < n)
        p <<= 1;
    for (len = p; len > 1; len >>= 1) {
        long half = len >> 1;
        for (i = 0; i < half; i++) {
            double a = (2 * i < n) ? v[2 * i] : -0.0;
            double b = (2 * i + 1 < n) ? v[2 * i + 1] : -0.0;
            v[i] = a + b;
        }
        n = half;
    }
    return v[0];
}

/*
 * Canonical SUM of terms over an iteration box.  terms is dense over the box
 * (row-major, innermost extent = hi_in - lo_in + 1); rows = number of rows;
 * the innermost loop index runs lo_in..hi_in (array index, step 1).
 */
double orc_canon_sum(const double *terms, long rows, long lo_in, long hi_in) {
    long c_lo = lo_in / CHUNK, c_hi = hi_in / CHUNK, nck = c_hi - c_lo + 1, w = hi_in - lo_in + 1;
    long nitems = rows * nck, r, c, p;
    double *items = malloc(sizeof(double) * (nitems > 0 ? nitems : 1));
    double leaf[CHUNK], res;
    for (r = 0; r < rows; r++) {
        const double *row = terms + r * w;
        for (c = 0; c < nck; c++) {
            long base = (c_lo + c) * CHUNK;
            for (p = 0; p < CHUNK; p++) {
                long k = base + p;
                leaf[p] = (k >= lo_in && k <= hi_in) ? row[k - lo_in] : -0.0;
            }
            items[r * nck + c] = orc_pairwise_sum(leaf, CHUNK);
        }
    }
    res = orc_pairwise_sum(items, nitems);
    free(items);
    return res;
}

/* ------------------------------------------------------------ Jacobi */

void orc_jacobi_init(int rank, long n, uint64_t seed, double *A, double *B) {
    long i, j, k;
    if (rank == 2) {
        for (i = 0; i < n; i++)
            for (j = 0; j < n; j++) {
                long lin = i * n + j;
                A[lin] = 0.0;
                B[lin] = (i == 0 || j == 0 || i == n - 1 || j == n - 1) ? 0.0 : orc_u01(seed, 1, (uint64_t)lin);
            }
    } else {
        for (i = 0; i < n; i++)
            for (j = 0; j < n; j++)
                for (k = 0; k < n; k++) {
                    long lin = (i * n + j) * n + k;
                    A[lin] = 0.0;
                    B[lin] = (i == 0 || j == 0 || k == 0 || i == n - 1 || j == n - 1 || k == n - 1)
                                 ? 0.0
                                 : orc_u01(seed, 1, (uint64_t)lin);
                }
    }
}

/*
 * One Jacobi time step: the update loop (eps = max |B-A|, A = B) then the
 * stencil loop, over the interior, with `nthreads` OpenMP threads (static
 * schedule over the outermost index, like the reference host handler with
 * OMP_SCHEDULE=static).  Returns eps = max(0.0 init, loop max); MAX is
 * order-independent so every thread count gives the sequential result.
 */
double orc_jacobi_step(int rank, long n, double *A, double *B, int nthreads) {
    double eps = 0.0;
    long i;
    if (nthreads < 1)
        nthreads = 1;
    if (rank == 2) {
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(max : eps)
        for (i = 1; i <= n - 2; i++) {
            long j;
            for (j = 1; j <= n - 2; j++) {
                long c = i * n + j;
                double tmp = fabs(B[c] - A[c]);
                eps = Max(tmp, eps);
                A[c] = B[c];
            }
        }
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (i = 1; i <= n - 2; i++) {
            long j;
            for (j = 1; j <= n - 2; j++) {
                long c = i * n + j;
                B[c] = (A[c - n] + A[c - 1] + A[c + 1] + A[c + n]) / 4.0;
            }
        }
    } else {
        long nn = n * n;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(max : eps)
        for (i = 1; i <= n - 2; i++) {
            long j, k;
            for (j = 1; j <= n - 2; j++)
                for (k = 1; k <= n - 2; k++) {
                    long c = (i * n + j) * n + k;
                    double tmp = fabs(B[c] - A[c]);
                    eps = Max(tmp, eps);
                    A[c] = B[c];
                }
        }
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (i = 1; i <= n - 2; i++) {
            long j, k;
            for (j = 1; j <= n - 2; j++)
                for (k = 1; k <= n - 2; k++) {
                    long c = (i * n + j) * n + k;
                    B[c] = (A[c - nn] + A[c - n] + A[c - 1] + A[c + 1] + A[c + n] + A[c + nn]) / 6.0;
                }
        }
    }
    /* (identity 0.0 max loop value) max initial value 0.0 */
    return Max(eps, 0.0);
}

/*
 * The weighted Jacobi 2-D program in cdvmh's converted form
 * (dvm-snapshot-r6603-fork_gb300/workloads/cdvh2d.c): row weights w[i] =
 * 0.5 + u(seed, 2, i) / 2, weights coef = {0.25, 0.125, 0.375, 0.25}; each
 * iteration eps = Max(|B - A|, eps), A = B over the interior, then
 * B = w[i] * (coef0 A[i-1][j] + coef1 A[i][j-1] + coef2 A[i][j+1] + coef3 A[i+1][j]),
 * every operation in the source order.  eps_out[iters], B[n*n].
 */
void orc_cdvh2d(long n, long iters, uint64_t seed, double *eps_out, double *B) {
    const double coef[4] = {0.25, 0.125, 0.375, 0.25};
    double *A = (double *)malloc(sizeof(double) * n * n), *w = (double *)malloc(sizeof(double) * n);
    long i, j, it;
    orc_jacobi_init(2, n, seed, A, B);
    for (i = 0; i < n; i++) w[i] = 0.5 + orc_u01(seed, 2, (uint64_t)i) / 2.0;
    for (it = 0; it < iters; it++) {
        double eps = 0.0;
        for (i = 1; i <= n - 2; i++)
            for (j = 1; j <= n - 2; j++) {
                long c = i * n + j;
                eps = Max(fabs(B[c] - A[c]), eps);
                A[c] = B[c];
            }
        for (i = 1; i <= n - 2; i++)
            for (j = 1; j <= n - 2; j++) {
                long c = i * n + j;
                B[c] = w[i] * (coef[0] * A[c - n] + coef[1] * A[c - 1] + coef[2] * A[c + 1] + coef[3] * A[c + n]);
            }
        eps_out[it] = Max(eps, 0.0);
    }
    free(A);
    free(w);
}

/* ------------------------------------------------------------ SOR (ACROSS) */

void orc_sor_init(long n, uint64_t seed, double *A) {
    long i, j, k;
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            for (k = 0; k < n; k++) {
                long lin = (i * n + j) * n + k;
                A[lin] = (i == 0 || j == 0 || k == 0 || i == n - 1 || j == n - 1 || k == n - 1)
                             ? 0.0
                             : orc_u01(seed, 1, (uint64_t)lin);
            }
}

/*
 * One SOR sweep in sequential loop order (the only order the ACROSS
 * dependences allow on one thread).  Returns the sequential-order residual
 * (0.0 + s_seq) + 0.0; *s_canon (may be NULL) receives the canonical-tree one.
 */
double orc_sor_sweep(long n, double w, double *A, double *s_canon) {
    long nn = n * n, m = n - 2, i, j, k, t = 0;
    double s = 0.0;
    double *terms = s_canon ? malloc(sizeof(double) * m * m * m) : 0;
    for (i = 1; i <= n - 2; i++)
        for (j = 1; j <= n - 2; j++)
            for (k = 1; k <= n - 2; k++) {
                long c = (i * n + j) * n + k;
                double old = A[c];
                double nv = (1.0 - w) * old + w / 6.0 * (A[c - nn] + A[c + nn] + A[c - n] + A[c + n] + A[c - 1] +
                                                         A[c + 1]);
                A[c] = nv;
                s += (nv - old) * (nv - old);
                if (terms)
                    terms[t++] = (nv - old) * (nv - old);
            }
    if (s_canon) {
        *s_canon = (0.0 + orc_canon_sum(terms, m * m, 1, n - 2)) + 0.0;
        free(terms);
    }
    return (0.0 + s) + 0.0;
}

/* One sweep with the residual terms summed per (i, j) column in k order, the
 * partial sums the hyperplane handler (workloads/sor3d_gen_cuda.cu) keeps in
 * its reduction slots: cols[(i-1)*(n-2) + (j-1)], starting from the identity
 * -0.0.  The array is the sequential sweep's. */
void orc_sor_sweep_cols(long n, double w, double *A, double *cols) {
    const long nn = n * n, m = n - 2;
    for (long i = 1; i <= n - 2; i++)
        for (long j = 1; j <= n - 2; j++) {
            double cs = -0.0;
            for (long k = 1; k <= n - 2; k++) {
                const long c = (i * n + j) * n + k;
                const double old = A[c];
                const double nv = (1.0 - w) * old + w / 6.0 * (A[c - nn] + A[c + nn] + A[c - n] + A[c + n] +
                                                               A[c - 1] + A[c + 1]);
                A[c] = nv;
                cs = cs + (nv - old) * (nv - old);
            }
            cols[(i - 1) * m + (j - 1)] = cs;
        }
}

/* ------------------------------------------------------------ batched heat */

long orc_heat_side(uint64_t seed, long k, long lo, long hi) {
    double u = orc_u01(seed, 1000, (uint64_t)k);
    long n = (long)floor((double)lo * pow((double)hi / (double)lo, u));
    if (n < 3)
        n = 3;
    if (n > hi)
        n = hi;
    return n;
}

void orc_heat_init(long n, uint64_t seed, long k, double *U, double *V) {
    long i, j;
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) {
            long lin = i * n + j;
            U[lin] = (i == 0 || j == 0 || i == n - 1 || j == n - 1) ? 0.0 : orc_u01(seed, 1 + (uint64_t)k, (uint64_t)lin);
            V[lin] = 0.0;
        }
}

/*
 * One heat step of one array: dst = src + c * lap5(src) over the interior.
 * Outputs: *sum_seq = (0.0 + sequential sum) + 0.0, *sum_canon = canonical-tree
 * sum, *mn / loc = MINLOC with init (1e300, {-1,-1}) and first-in-loop-order ties.
 */
void orc_heat_step(long n, double c, const double *src, double *dst, double *sum_seq, double *sum_canon, double *mn,
                   int loc[2]) {
    long m = n - 2, i, j, t = 0;
    double s = 0.0, best = 1e300;
    int l0 = -1, l1 = -1;
    double *terms = sum_canon ? malloc(sizeof(double) * (m > 0 ? m * m : 1)) : 0;
    for (i = 1; i <= n - 2; i++)
        for (j = 1; j <= n - 2; j++) {
            long q = i * n + j;
            double v = src[q] + c * (src[q - n] + src[q + n] + src[q - 1] + src[q + 1] - 4.0 * src[q]);
            dst[q] = v;
            s += v;
            if (terms)
                terms[t++] = v;
            if (v < best) {
                best = v;
                l0 = (int)i;
                l1 = (int)j;
            }
        }
    if (sum_seq)
        *sum_seq = (0.0 + s) + 0.0;
    if (sum_canon) {
        *sum_canon = (0.0 + orc_canon_sum(terms, m, 1, n - 2)) + 0.0;
        free(terms);
    }
    *mn = best;
    loc[0] = l0;
    loc[1] = l1;
}

/*
 * Gauss-Seidel over an n0 x n1 array with dependences on both axes
 * (dvm-snapshot-r6603-fork_gb300/workloads/gsd2d.c): the sequential loop, each axis
 * forward (dir > 0) or backward, interior only; returns MAX |new - old| of
 * the sweep combined with the initial value 0 (the reduction's result).
 */
void orc_gsd2d_init(long n0, long n1, uint64_t seed, double *A) {
    for (long i = 0; i < n0; i++)
        for (long j = 0; j < n1; j++)
            A[i * n1 + j] =
                (i == 0 || j == 0 || i == n0 - 1 || j == n1 - 1) ? 0.0 : orc_u01(seed, 17, (uint64_t)(i * n1 + j));
}

double orc_gsd2d_sweep(long n0, long n1, int dir0, int dir1, double *A) {
    double m = 0.0;  /* MAX identity of non-negative values; the initial value 0 is folded in last */
    for (long a = 0; a < n0 - 2; a++) {
        long i = dir0 > 0 ? 1 + a : n0 - 2 - a;
        for (long b = 0; b < n1 - 2; b++) {
            long j = dir1 > 0 ? 1 + b : n1 - 2 - b;
            double old = A[i * n1 + j];
            double v = (((A[(i - 1) * n1 + j] + A[(i + 1) * n1 + j]) + A[i * n1 + j - 1]) + A[i * n1 + j + 1]) * 0.25;
            A[i * n1 + j] = v;
            m = Max(m, fabs(v - old));
        }
    }
    return Max(m, 0.0);
}

/*
 * Gauss-Seidel over an n x n array, SUM of the new values
 * (dvm-snapshot-r6603-fork_gb300/workloads/gs2d.c): the sequential loop over the
 * interior; returns (0 + sum) + 0, the handler's sum combined with the
 * global start and the initial value 0 (rts/dvmh/loop.cpp:37-113).
 */
void orc_gs2d_init(long n, uint64_t seed, double *A) {
    for (long i = 0; i < n; i++)
        for (long j = 0; j < n; j++)
            A[i * n + j] = (i == 0 || j == 0 || i == n - 1 || j == n - 1) ? 0.0 : orc_u01(seed, 13, (uint64_t)(i * n + j));
}

double orc_gs2d_sweep(long n, double *A) {
    double s = 0.0;
    for (long i = 1; i < n - 1; i++)
        for (long j = 1; j < n - 1; j++) {
            A[i * n + j] = (((A[(i - 1) * n + j] + A[(i + 1) * n + j]) + A[i * n + j - 1]) + A[i * n + j + 1]) * 0.25;
            s = s + A[i * n + j];
        }
    return (0.0 + s) + 0.0;
}

/*
 * The recurrence A[i][j] = A[i][j] * 0.5 + A[i][j-1] * 0.25 along j over
 * independent rows, MIN of the new values with the initial value 1.0
 * (dvm-snapshot-r6603-fork_gb300/workloads/rec2d.c).
 */
void orc_rec2d_init(long n0, long n1, uint64_t seed, double *A) {
    for (long i = 0; i < n0; i++)
        for (long j = 0; j < n1; j++) A[i * n1 + j] = orc_u01(seed, 19, (uint64_t)(i * n1 + j));
}

double orc_rec2d_sweep(long n0, long n1, double *A) {
    double lo = 1.0;  /* MIN: the handler starts at the initial value */
    for (long i = 0; i < n0; i++)
        for (long j = 1; j < n1; j++) {
            A[i * n1 + j] = A[i * n1 + j] * 0.5 + A[i * n1 + j - 1] * 0.25;
            lo = A[i * n1 + j] < lo ? A[i * n1 + j] : lo;
        }
    return lo < 1.0 ? lo : 1.0;
}

/*
 * One pass of the 3-D loop B = A[i-1][j][k] + 0.5 * A[i][j][k+1] over the
 * interior with SUM and MAXLOC (dvm-snapshot-r6603-fork_gb300/workloads/gen3d.c),
 * in loop order; s, mx, lc: initial values in, results out, combined as the
 * reference's engine does (rts/dvmh/loop.cpp:37-113: SUM from the identity,
 * MAXLOC from the initial value, strict >).  B (dense) is 0 outside the loop.
 */
void orc_gen3d(long n0, long n1, long n2, uint64_t seed, double *s, double *mx, long *lc, double *B) {
    double acc = 0.0, m = *mx;
    long loc = *lc;
    const long cells = n0 * n1 * n2;
    double *A = (double *)malloc(sizeof(double) * (size_t)cells);
    for (long q = 0; q < cells; q++) {
        A[q] = orc_u01(seed, 7, (uint64_t)q);
        B[q] = 0.0;
    }
    for (long i = 1; i < n0 - 1; i++)
        for (long j = 1; j < n1 - 1; j++)
            for (long k = 1; k < n2 - 1; k++) {
                const long q = (i * n1 + j) * n2 + k;
                const double v = A[q - n1 * n2] + 0.5 * A[q + 1];
                B[q] = v;
                acc = acc + v;
                if (v > m) {
                    m = v;
                    loc = q;
                }
            }
    free(A);
    *s = (0.0 + acc) + *s;
    *mx = m;
    *lc = loc;
}

/*
 * The reference's FP32 Jacobi benchmarks (examples/Performance/jac2d_perf.c
 * and jac3d_perf.c; dvm-snapshot-r6603-fork_gb300/workloads/jacperf.c): A = 0,
 * B = c + sum of indices inside (c = 3 in 2-D, 4 in 3-D), then per iteration
 * eps = MAX |B - A|, A = B over the interior and B = (sum of the 2r
 * neighbours of A in the program's order) / (2r)f, stopping after the first
 * iteration with eps < 0.5.  All arithmetic in float.  eps_out[it] per
 * iteration; A, B dense L^rank.  Returns the iterations run.
 */
long orc_jacperf(int rank, long L, long itmax, float *eps_out, float *A, float *B) {
    const long n2 = L * L, planes = rank == 3 ? L : 1, rows = L;
    long it, done = 0;
    /* rank 2 is the 3-D walk with one plane and no plane neighbours */
    for (long i = 0; i < planes; i++)
        for (long j = 0; j < rows; j++)
            for (long k = 0; k < L; k++) {
                const long q = (i * L + j) * L + k;
                A[q] = 0.0f;
                if (rank == 3)
                    B[q] = (i == 0 || j == 0 || k == 0 || i == L - 1 || j == L - 1 || k == L - 1) ? 0.0f
                                                                                                  : (float)(4 + i + j + k);
                else
                    B[q] = (j == 0 || k == 0 || j == L - 1 || k == L - 1) ? 0.0f : (float)(3 + j + k);
            }
    const long i0 = rank == 3 ? 1 : 0, i1 = rank == 3 ? L - 2 : 0;
    for (it = 1; it <= itmax; it++) {
        float eps = 0.0f;
#pragma omp parallel for collapse(2) reduction(max : eps) schedule(static)
        for (long i = i0; i <= i1; i++)
            for (long j = 1; j <= L - 2; j++)
                for (long k = 1; k <= L - 2; k++) {
                    const long q = (i * L + j) * L + k;
                    float tmp = fabsf(B[q] - A[q]);
                    eps = tmp > eps ? tmp : eps;
                    A[q] = B[q];
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (long i = i0; i <= i1; i++)
            for (long j = 1; j <= L - 2; j++)
                for (long k = 1; k <= L - 2; k++) {
                    const long q = (i * L + j) * L + k;
                    if (rank == 3)
                        B[q] = (A[q - n2] + A[q - L] + A[q - 1] + A[q + 1] + A[q + L] + A[q + n2]) / 6.0f;
                    else
                        B[q] = (A[q - L] + A[q - 1] + A[q + 1] + A[q + L]) / 4.0f;
                }
        eps_out[it - 1] = eps;
        done = it;
        if (eps < 0.5f) break;
    }
    return done;
}

/*
 * The eight reductions of a 1-D loop with a signed step
 * (dvm-snapshot-r6603-fork_gb300/workloads/genred.c), in loop order, combined
 * as the reference's engine combines them (rts/dvmh/loop.cpp:37-113): the
 * handler's SUM, PROD and XOR start at the identity, MIN, MAX, AND, OR and
 * MINLOC at the variable's initial value; the global value starts the same
 * way, takes the handler's result, then the initial value once more.
 * d3 = {ds, dp, dml}, i4 = {imn, ia, io, ix}, f1 = {fmx}, lc: initial values
 * in, results out.
 */
static void genred_loop(long n, long start, long end, long step, const double *xs, const int *vs, uint64_t seed,
                        double *d3, int *i4, float *f1, long *lc);

void orc_genred(long n, long start, long end, long step, uint64_t seed, double *d3, int *i4, float *f1, long *lc) {
    genred_loop(n, start, end, step, 0, 0, seed, d3, i4, f1, lc);
}

/* the same loop on given inputs */
void orc_genred_data(long n, long start, long end, long step, const double *x, const int *v, double *d3, int *i4,
                     float *f1, long *lc) {
    genred_loop(n, start, end, step, x, v, 0, d3, i4, f1, lc);
}

/* the program's edge-value inputs (workloads/genred.c wl_genred_pattern): a
 * multiplicative hash of i + 1 picks one of five values; V is its high half */
void orc_genred_pattern(int pattern, long n, double *x, int *v) {
    const double p0[5] = {0.0, -0.0, -0.5, -1e-310, -INFINITY};
    const double p1[5] = {0.25, NAN, INFINITY, -0.0, 4.9406564584124654e-324};
    for (long i = 0; i < n; i++) {
        const uint64_t h = (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
        const int k = (int)((h >> 40) % 5);
        x[i] = pattern == 0 ? p0[k] : pattern == 1 ? p1[k] : 0.5;
        v[i] = pattern == 2 ? 7 : (int)(uint32_t)(h >> 32);
    }
}

static void genred_loop(long n, long start, long end, long step, const double *xs, const int *vs, uint64_t seed,
                        double *d3, int *i4, float *f1, long *lc) {
    double ds = 0.0, dp = 1.0, dml = d3[2];
    int imn = i4[0], ia = i4[1], io = i4[2], ix = 0;
    float fmx = f1[0];
    long loc = lc[0];
    if (step != 0)
        for (long i = start; step > 0 ? i <= end : i >= end; i += step) {
            if (i < 0 || i >= n) break;
            double x = xs ? xs[i] : orc_u01(seed, 11, (uint64_t)i);
            int v = vs ? vs[i] : (int)(orc_u01(seed, 12, (uint64_t)i) * 2147483647.0) - 1073741824;
            ds = ds + x;
            dp = dp * (1.0 + x / 65536.0);
            imn = v < imn ? v : imn;
            fmx = (float)x > fmx ? (float)x : fmx;
            ia &= v | 0x0F0F0F0F;
            io |= v & 0x00FF00FF;
            ix ^= v;
            if (x < dml) {
                dml = x;
                loc = i;
            }
        }
    /* global: identity (+) handler (+) initial, for the order-sensitive two */
    d3[0] = (0.0 + ds) + d3[0];
    d3[1] = (1.0 * dp) * d3[1];
    d3[2] = dml;
    i4[0] = imn;
    i4[1] = ia;
    i4[2] = io;
    i4[3] = (0 ^ ix) ^ i4[3];
    f1[0] = fmx;
    lc[0] = loc;
}

/* position of (x, y) in the diagonal numbering of an Rx x Ry plane
 * (rts/dvmh/util.cpp:1009-1055), by walking the diagonals: cells ordered by
 * d = x + y (slash: x + Ry - 1 - y), inside a diagonal along y when Rx < Ry
 * or (Rx == Ry and d < Rx), else along x.  Counting, not a closed form, so it
 * checks the runtime's closed form independently. */
long orc_diag_index(long x, long y, long Rx, long Ry, int slash) {
    long yy = slash ? Ry - 1 - y : y, d = x + yy, pos = 0;
    for (long e = 0; e < d; e++)
        for (long xx = 0; xx < Rx; xx++)
            if (e - xx >= 0 && e - xx < Ry) pos++;
    int alongY = Rx < Ry || (Rx == Ry && d < Rx);
    for (long xx = 0; xx < Rx; xx++) {
        long y2 = d - xx;
        if (y2 < 0 || y2 >= Ry) continue;
        if (alongY ? y2 < yy : xx < x) pos++;
    }
    return pos;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
