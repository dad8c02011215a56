/*
 * Jacobi 3-D 7-point, FP64 -- a C-DVMH program written out in the form cdvmh
 * converts it to: main code calling the dvmh_* ABI (cdvmh/src/converter_main.cpp
 * :2560-2960 for loops, :3013-3090 for regions) and OpenMP host handlers
 * (converter_main.cpp:1503-1859).  The CUDA handlers are in jac3d_cuda.cu.
 *
 * Source program (after examples/Performance/jac3d_perf.c:28-73, in FP64):
 *   A = 0 everywhere; B = seeded uniform[0,1) inside, 0 on the boundary
 *   repeat iters times:
 *     eps = 0
 *     region {
 *       parallel([i][j][k] on A[i][j][k]) reduction(max(eps)):
 *         tmp = fabs(B - A); eps = Max(tmp, eps); A = B          (interior)
 *       parallel([i][j][k] on B[i][j][k]) shadow_renew(A):
 *         B = (A[i-1]+A[j-1]+A[k-1]+A[k+1]+A[j+1]+A[i+1]) / 6.0 (interior)
 *     }
 *     get_actual(eps)
 *
 * Built against the reference runtime (oracle/_ref) with WL_NO_CUDA it is the
 * oracle; built against libdvmh_gb it runs the GPU path.  Same source.
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

#define Max(a, b) ((a) > (b) ? (a) : (b))

#ifdef _OPENMP
#define OMP_HANDLER_TYPE (HANDLER_TYPE_MASTER | HANDLER_TYPE_PARALLEL)
#else
#define OMP_HANDLER_TYPE 0
#endif

static DvmType A[64], B[64];
static double eps;
static wl_jacobi_params P;

#ifndef WL_NO_CUDA
void loop_jac3d_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr);
void loop_jac3d_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
void loop_jac3d_upd_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr);
void loop_jac3d_stn_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
#endif
static int useGenerated;

/* the CUDA handlers the loops register: 0 = jac3d_cuda.cu (the library's
 * kernels), 1 = cdvmh's generated one-point-per-thread shape (jacperf_cuda.cu) */
int wl_jac3d_use_generated(int on) {
    useGenerated = on;
    return 0;
}

/* ---------------------------------------------------------------- host handlers */

void loop_jac3d_upd_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (double (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    double (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (double (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3];
    int slotCount;
    (void)eps_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        double eps;
        DvmType i, j, k;
        dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
#pragma omp for schedule(runtime) nowait
        for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
            for (j = boundsLow[1]; j <= boundsHigh[1]; j++)
                for (k = boundsLow[2]; k <= boundsHigh[2]; k++) {
                    double tmp = fabs(b[i][j][k] - a[i][j][k]);
                    eps = Max(tmp, eps);
                    a[i][j][k] = b[i][j][k];
                }
        dvmh_loop_red_post_C(loop_ref, 1, &eps, 0);
    }
}

void loop_jac3d_stn_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (double (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    double (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (double (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3];
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j, k;
#pragma omp for schedule(runtime) nowait
        for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
            for (j = boundsLow[1]; j <= boundsHigh[1]; j++)
                for (k = boundsLow[2]; k <= boundsHigh[2]; k++)
                    b[i][j][k] = (a[i - 1][j][k] + a[i][j - 1][k] + a[i][j][k - 1] + a[i][j][k + 1] +
                                  a[i][j + 1][k] + a[i + 1][j][k]) / 6.0;
    }
}

/* ---------------------------------------------------------------- main code */

/* Creates and seeds the arrays on the host.  Returns 0. */
int wl_jac3d_setup(const wl_jacobi_params *p) {
    long n = p->n, i, j, k, st[3];
    double *a, *b;
    P = *p;
    dvmh_array_create_C(A, 3, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_distribute_C(A, 3, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2), dvmh_distribution_block_C(3));
    dvmh_array_create_C(B, 3, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_align_C(B, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                 dvmh_alignment_linear_C(3, 1, 0));
    a = (double *)dvmh_get_natural_base_C(0, A);
    b = (double *)dvmh_get_natural_base_C(0, B);
    wl_strides(A, 3, st);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            for (k = 0; k < n; k++) {
                long lin = (i * n + j) * n + k, q = i * st[0] + j * st[1] + k;
                a[q] = 0.0;
                if (i == 0 || j == 0 || k == 0 || i == n - 1 || j == n - 1 || k == n - 1)
                    b[q] = 0.0;
                else
                    b[q] = wl_u01(p->seed, 1, (uint64_t)lin);
            }
    dvmh_actual_array2_(A);
    dvmh_actual_array2_(B);
    return 0;
}

/* One time step of the source program.  Returns eps. */
double wl_jac3d_step(void) {
    long n = P.n;
    DvmType cur_region, cur_loop;
    eps = 0;
    dvmh_actual_variable2_(&eps);
    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, B, "B");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &eps, sizeof(eps), "eps");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);

    cur_loop = dvmh_loop_create_C(cur_region, 3, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L, 1L,
                                  (DvmType)(n - 2), 1L);
    dvmh_loop_map_C(cur_loop, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                    dvmh_alignment_linear_C(3, 1, 0));
    dvmh_loop_reduction_C(cur_loop, rf_MAX, &eps, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac3d_upd_host, 3, A, B, &eps));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)(useGenerated ? loop_jac3d_upd_gen_cuda
                                                                                   : loop_jac3d_upd_cuda),
                                                     3, A, B, &eps));
#endif
    dvmh_loop_perform_C(cur_loop);

    dvmh_shadow_renew_C(A, 0, 0);
    cur_loop = dvmh_loop_create_C(cur_region, 3, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L, 1L,
                                  (DvmType)(n - 2), 1L);
    dvmh_loop_map_C(cur_loop, B, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                    dvmh_alignment_linear_C(3, 1, 0));
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac3d_stn_host, 2, A, B));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)(useGenerated ? loop_jac3d_stn_gen_cuda
                                                                                   : loop_jac3d_stn_cuda),
                                                     2, A, B));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);

    dvmh_get_actual_variable2_(&eps);
    return eps;
}

/* Runs `iters` steps; eps_out (may be NULL) receives eps after each.  Returns 0. */
int wl_jac3d_run(long iters, double *eps_out) {
    long it;
    for (it = 0; it < iters; it++) {
        double e = wl_jac3d_step();
        if (eps_out)
            eps_out[it] = e;
    }
    return 0;
}

/* dense n^3 <-> the array's host layout; dir 0: array -> dense, 1: dense -> array */
static void jac3d_xfer(DvmType *D, double *dense, int dir) {
    long n = P.n, i, j, st[3];
    double *h = (double *)dvmh_get_natural_base_C(0, D);
    wl_strides(D, 3, st);
#pragma omp parallel for private(j) schedule(static)
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) {
            double *row = h + i * st[0] + j * st[1], *drow = dense + (i * n + j) * n;
            if (dir == 0)
                memcpy(drow, row, sizeof(double) * n);
            else
                memcpy(row, drow, sizeof(double) * n);
        }
}

/* Copies the current A and B (dense n^3 doubles each, may be NULL) to the caller. */
int wl_jac3d_fetch(double *a_out, double *b_out) {
    if (a_out) {
        dvmh_get_actual_array2_(A);
        jac3d_xfer(A, a_out, 0);
    }
    if (b_out) {
        dvmh_get_actual_array2_(B);
        jac3d_xfer(B, b_out, 0);
    }
    return 0;
}

/* Replaces A and B with caller data (NULL keeps an array) and marks the host
 * copies actual: every element is overwritten, so the old contents are not
 * fetched first. */
int wl_jac3d_load(const double *a_in, const double *b_in) {
    if (a_in) {
        jac3d_xfer(A, (double *)a_in, 1);
        dvmh_actual_array2_(A);
    }
    if (b_in) {
        jac3d_xfer(B, (double *)b_in, 1);
        dvmh_actual_array2_(B);
    }
    return 0;
}

/* The program's own host arrays as the data source and sink: declares the host
 * copies of A and B current (the next region uploads them) ... */
void wl_jac3d_push(void) {
    dvmh_actual_array2_(A);
    dvmh_actual_array2_(B);
}

/* ... and makes them current again from the device (get_actual). */
void wl_jac3d_pull(void) {
    dvmh_get_actual_array2_(A);
    dvmh_get_actual_array2_(B);
}

/* Box [lo, hi] of A (which = 0) or B (which = 1) and its dense copy box_io
 * (row-major, innermost last).  get: makes the box current on the host
 * (dvmh_get_actual_subarray_C) and copies it out; put: writes box_io into the
 * host array and declares the box current there (dvmh_actual_subarray_C). */
static DvmType *pick(int which) { return which ? B : A; }

int wl_jac3d_box(int which, int put, const long lo[3], const long hi[3], double *box_io) {
    DvmType *D = pick(which);
    double *h = (double *)dvmh_get_natural_base_C(0, D);
    long st[3], i, j, w = hi[2] - lo[2] + 1, q = 0;
    wl_strides(D, 3, st);
    if (!put) dvmh_get_actual_subarray_C(D, 3, (DvmType)lo[0], (DvmType)hi[0], (DvmType)lo[1], (DvmType)hi[1],
                                         (DvmType)lo[2], (DvmType)hi[2]);
    for (i = lo[0]; i <= hi[0]; i++)
        for (j = lo[1]; j <= hi[1]; j++, q += w) {
            double *row = h + i * st[0] + j * st[1] + lo[2];
            if (put)
                memcpy(row, box_io + q, sizeof(double) * w);
            else
                memcpy(box_io + q, row, sizeof(double) * w);
        }
    if (put) dvmh_actual_subarray_C(D, 3, (DvmType)lo[0], (DvmType)hi[0], (DvmType)lo[1], (DvmType)hi[1],
                                    (DvmType)lo[2], (DvmType)hi[2]);
    return 0;
}

/* The host copy of A or B as it is (dense n^3), without making it current. */
void wl_jac3d_host_peek(int which, double *out) { jac3d_xfer(pick(which), out, 0); }

void wl_jac3d_teardown(void) {
    dvmh_array_free_C(B);
    dvmh_array_free_C(A);
}
