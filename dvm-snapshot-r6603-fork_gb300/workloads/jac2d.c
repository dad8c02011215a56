/*
 * Jacobi 2-D 5-point, FP64 -- C-DVMH program in the form cdvmh converts it to
 * (main code: cdvmh/src/converter_main.cpp:2560-2960, :3013-3090; OpenMP host
 * handlers: converter_main.cpp:1503-1859).  CUDA handlers: jac2d_cuda.cu.
 *
 * Source program (examples/Jacobi/jac2d.c:24-67, seeded, fixed iteration count):
 *   A = 0 everywhere; B = seeded uniform[0,1) inside, 0 on the boundary
 *   repeat iters times:
 *     eps = 0
 *     region {
 *       parallel([i][j] on A[i][j]) reduction(max(eps)):
 *         tmp = fabs(B - A); eps = Max(tmp, eps); A = B            (interior)
 *       parallel([i][j] on B[i][j]) shadow_renew(A):
 *         B = (A[i-1][j] + A[i][j-1] + A[i][j+1] + A[i+1][j]) / 4.0 (interior)
 *     }
 *     get_actual(eps)
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
void loop_jac2d_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr);
void loop_jac2d_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
#endif

void loop_jac2d_upd_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    double (*b)[B_hdr[1]] = (double (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    int slotCount;
    (void)eps_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        double eps;
        DvmType i, j;
        dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
#pragma omp for schedule(runtime) nowait
        for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
            for (j = boundsLow[1]; j <= boundsHigh[1]; j++) {
                double tmp = fabs(b[i][j] - a[i][j]);
                eps = Max(tmp, eps);
                a[i][j] = b[i][j];
            }
        dvmh_loop_red_post_C(loop_ref, 1, &eps, 0);
    }
}

void loop_jac2d_stn_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    double (*b)[B_hdr[1]] = (double (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j;
#pragma omp for schedule(runtime) nowait
        for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
            for (j = boundsLow[1]; j <= boundsHigh[1]; j++)
                b[i][j] = (a[i - 1][j] + a[i][j - 1] + a[i][j + 1] + a[i + 1][j]) / 4.0;
    }
}

int wl_jac2d_setup(const wl_jacobi_params *p) {
    long n = p->n, i, j, st[2];
    double *a, *b;
    P = *p;
    dvmh_array_create_C(A, 2, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
    dvmh_array_create_C(B, 2, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_align_C(B, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    a = (double *)dvmh_get_natural_base_C(0, A);
    b = (double *)dvmh_get_natural_base_C(0, B);
    wl_strides(A, 2, st);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) {
            long lin = i * n + j, q = i * st[0] + j;
            a[q] = 0.0;
            if (i == 0 || j == 0 || i == n - 1 || j == n - 1)
                b[q] = 0.0;
            else
                b[q] = wl_u01(p->seed, 1, (uint64_t)lin);
        }
    dvmh_actual_array2_(A);
    dvmh_actual_array2_(B);
    return 0;
}

double wl_jac2d_step(void) {
    long n = P.n;
    DvmType cur_region, cur_loop;
    eps = 0;
    dvmh_actual_variable2_(&eps);
    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, B, "B");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &eps, sizeof(eps), "eps");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);

    cur_loop = dvmh_loop_create_C(cur_region, 2, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L);
    dvmh_loop_map_C(cur_loop, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    dvmh_loop_reduction_C(cur_loop, rf_MAX, &eps, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac2d_upd_host, 3, A, B, &eps));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac2d_upd_cuda, 3, A, B, &eps));
#endif
    dvmh_loop_perform_C(cur_loop);

    dvmh_shadow_renew_C(A, 0, 0);
    cur_loop = dvmh_loop_create_C(cur_region, 2, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L);
    dvmh_loop_map_C(cur_loop, B, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac2d_stn_host, 2, A, B));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_jac2d_stn_cuda, 2, A, B));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);

    dvmh_get_actual_variable2_(&eps);
    return eps;
}

int wl_jac2d_run(long iters, double *eps_out) {
    long it;
    for (it = 0; it < iters; it++) {
        double e = wl_jac2d_step();
        if (eps_out)
            eps_out[it] = e;
    }
    return 0;
}

static void jac2d_out(DvmType *D, double *dense) {
    long n = P.n, i, st[2];
    double *h = (double *)dvmh_get_natural_base_C(0, D);
    wl_strides(D, 2, st);
    for (i = 0; i < n; i++)
        memcpy(dense + i * n, h + i * st[0], sizeof(double) * n);
}

/* Copies the current A and B (dense n^2 doubles each, may be NULL) to the caller. */
int wl_jac2d_fetch(double *a_out, double *b_out) {
    if (a_out) {
        dvmh_get_actual_array2_(A);
        jac2d_out(A, a_out);
    }
    if (b_out) {
        dvmh_get_actual_array2_(B);
        jac2d_out(B, b_out);
    }
    return 0;
}

void wl_jac2d_teardown(void) {
    dvmh_array_free_C(B);
    dvmh_array_free_C(A);
}
