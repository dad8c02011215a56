/*
 * The reference's FP32 Jacobi benchmarks with their own verification values
 * (examples/Performance/jac3d_perf.c, 384^3, eps after 100 iterations
 * 5.058044 +- 1e-4, :92; examples/Performance/jac2d_perf.c, 8000^2,
 * 58.37598 +- 1e-3, :89), in the form cdvmh converts them to (main code:
 * cdvmh/src/converter_main.cpp:2560-2960).  Unlike jac2d.c / jac3d.c the
 * arrays are float, initialised by a parallel loop on the device, and the
 * CUDA handlers (jacperf_cuda.cu) have the generated shape: one loop point
 * per thread, one MAX slot per launched thread.
 *
 * Source program (rank r = 2 or 3, side L; c = 3 for r = 2, 4 for r = 3):
 *   region { parallel(on A) cuda_block(..): A = 0; B = boundary ? 0 : c + sum of indices }
 *   for it = 1..itmax:
 *     eps = 0
 *     region {
 *       parallel(on A) reduction(max(eps)): tmp = fabs(B - A); eps = Max(tmp, eps); A = B
 *       parallel(on B) shadow_renew(A): B = (sum of the 2r neighbours of A) / (2r)f
 *     }
 *     get_actual(eps); stop when eps < 0.5
 * cuda_block(32, 8) for r = 3, cuda_block(256) for r = 2, as the examples set.
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
static float eps;

#ifndef WL_NO_CUDA
void loop_jacperf2_init_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
void loop_jacperf2_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr);
void loop_jacperf2_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
void loop_jacperf3_init_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
void loop_jacperf3_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr);
void loop_jacperf3_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]);
#endif

/* ---- host handlers (OpenMP, schedule(runtime), as cdvmh emits them) ---- */

void loop_jacperf2_init_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1]] = (float (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1]] = (float (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[2], hi[2], st[2], L;
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    L = hi[0] + 1;
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j;
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++) {
                a[i][j] = 0;
                if (i == 0 || j == 0 || i == L - 1 || j == L - 1)
                    b[i][j] = 0;
                else
                    b[i][j] = 3 + i + j;
            }
    }
}

void loop_jacperf2_upd_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1]] = (float (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1]] = (float (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[2], hi[2], st[2];
    int slotCount;
    (void)eps_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        float eps;
        DvmType i, j;
        dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++) {
                float tmp = fabs(b[i][j] - a[i][j]);
                eps = Max(tmp, eps);
                a[i][j] = b[i][j];
            }
        dvmh_loop_red_post_C(loop_ref, 1, &eps, 0);
    }
}

void loop_jacperf2_stn_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1]] = (float (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1]] = (float (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[2], hi[2], st[2];
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j;
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++)
                b[i][j] = (a[i - 1][j] + a[i][j - 1] + a[i][j + 1] + a[i + 1][j]) / 4.0f;
    }
}

void loop_jacperf3_init_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (float (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (float (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[3], hi[3], st[3], L;
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    L = hi[0] + 1;
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j, k;
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++)
                for (k = lo[2]; k <= hi[2]; k++) {
                    a[i][j][k] = 0;
                    if (i == 0 || j == 0 || k == 0 || i == L - 1 || j == L - 1 || k == L - 1)
                        b[i][j][k] = 0;
                    else
                        b[i][j][k] = 4 + i + j + k;
                }
    }
}

void loop_jacperf3_upd_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (float (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (float (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[3], hi[3], st[3];
    int slotCount;
    (void)eps_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        float eps;
        DvmType i, j, k;
        dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++)
                for (k = lo[2]; k <= hi[2]; k++) {
                    float tmp = fabs(b[i][j][k] - a[i][j][k]);
                    eps = Max(tmp, eps);
                    a[i][j][k] = b[i][j][k];
                }
        dvmh_loop_red_post_C(loop_ref, 1, &eps, 0);
    }
}

void loop_jacperf3_stn_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    float (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (float (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    float (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (float (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType lo[3], hi[3], st[3];
    int slotCount;
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        DvmType i, j, k;
#pragma omp for schedule(runtime) nowait
        for (i = lo[0]; i <= hi[0]; i++)
            for (j = lo[1]; j <= hi[1]; j++)
                for (k = lo[2]; k <= hi[2]; k++)
                    b[i][j][k] = (a[i - 1][j][k] + a[i][j - 1][k] + a[i][j][k - 1] + a[i][j][k + 1] + a[i][j + 1][k] +
                                  a[i + 1][j][k]) /
                                 6.0f;
    }
}

/* ---- main code ---- */

static DvmType loopOver(DvmType region, int rank, long from, long to) {
    if (rank == 3)
        return dvmh_loop_create_C(region, 3, (DvmType)from, (DvmType)to, 1L, (DvmType)from, (DvmType)to, 1L,
                                  (DvmType)from, (DvmType)to, 1L);
    return dvmh_loop_create_C(region, 2, (DvmType)from, (DvmType)to, 1L, (DvmType)from, (DvmType)to, 1L);
}

static void mapOn(DvmType loop, DvmType *D, int rank) {
    if (rank == 3)
        dvmh_loop_map_C(loop, D, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                        dvmh_alignment_linear_C(3, 1, 0));
    else
        dvmh_loop_map_C(loop, D, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
}

static void blockOf(DvmType loop, int rank) {
    if (rank == 3)
        dvmh_loop_set_cuda_block_C(loop, 32, 8, 1);
    else
        dvmh_loop_set_cuda_block_C(loop, 256, 1, 1);
}

static void fetch(DvmType *D, int rank, long L, float *dense) {
    long i, j, st[3];
    float *h = (float *)dvmh_get_natural_base_C(0, D);
    dvmh_get_actual_array2_(D);
    wl_strides(D, rank, st);
    if (rank == 3) {
        for (i = 0; i < L; i++)
            for (j = 0; j < L; j++) memcpy(dense + (i * L + j) * L, h + i * st[0] + j * st[1], sizeof(float) * L);
    } else {
        for (i = 0; i < L; i++) memcpy(dense + i * L, h + i * st[0], sizeof(float) * L);
    }
}

/* The whole program on an L^rank grid: eps_out[it-1] = eps after iteration it;
 * a_out / b_out (dense L^rank floats) get A and B when non-null.  Returns the
 * number of iterations run (itmax unless eps fell below 0.5), -1 on a bad rank. */
long wl_jacperf_run(int rank, long L, long itmax, float *eps_out, float *a_out, float *b_out) {
    DvmType cur_region, cur_loop;
    long it, done = 0;
    if (rank != 2 && rank != 3) return -1;
    if (rank == 3) {
        dvmh_array_create_C(A, 3, -rt_FLOAT, (DvmType)L, 1L, 1L, (DvmType)L, 1L, 1L, (DvmType)L, 1L, 1L);
        dvmh_distribute_C(A, 3, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2),
                          dvmh_distribution_block_C(3));
        dvmh_array_create_C(B, 3, -rt_FLOAT, (DvmType)L, 0L, 0L, (DvmType)L, 0L, 0L, (DvmType)L, 0L, 0L);
        dvmh_align_C(B, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                     dvmh_alignment_linear_C(3, 1, 0));
    } else {
        dvmh_array_create_C(A, 2, -rt_FLOAT, (DvmType)L, 1L, 1L, (DvmType)L, 1L, 1L);
        dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
        dvmh_array_create_C(B, 2, -rt_FLOAT, (DvmType)L, 0L, 0L, (DvmType)L, 0L, 0L);
        dvmh_align_C(B, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    }

    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_OUT, A, "A");
    dvmh_region_register_array_C(cur_region, INTENT_OUT, B, "B");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
    cur_loop = loopOver(cur_region, rank, 0, L - 1);
    mapOn(cur_loop, A, rank);
    blockOf(cur_loop, rank);
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                 dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_init_host
                                                                                : loop_jacperf2_init_host),
                                                     2, A, B));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_init_cuda
                                                                                : loop_jacperf2_init_cuda),
                                                     2, A, B));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);

    for (it = 1; it <= itmax; it++) {
        eps = 0;
        dvmh_actual_variable2_(&eps);
        cur_region = dvmh_region_create_C(0);
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, B, "B");
        dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &eps, sizeof(eps), "eps");
        dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);

        cur_loop = loopOver(cur_region, rank, 1, L - 2);
        mapOn(cur_loop, A, rank);
        blockOf(cur_loop, rank);
        dvmh_loop_reduction_C(cur_loop, rf_MAX, &eps, rt_FLOAT, 1, 0, 0);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                     dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_upd_host
                                                                                    : loop_jacperf2_upd_host),
                                                         3, A, B, &eps));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_upd_cuda
                                                                                    : loop_jacperf2_upd_cuda),
                                                         3, A, B, &eps));
#endif
        dvmh_loop_perform_C(cur_loop);

        dvmh_shadow_renew_C(A, 0, 0);
        cur_loop = loopOver(cur_region, rank, 1, L - 2);
        mapOn(cur_loop, B, rank);
        blockOf(cur_loop, rank);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                     dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_stn_host
                                                                                    : loop_jacperf2_stn_host),
                                                         2, A, B));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)(rank == 3 ? loop_jacperf3_stn_cuda
                                                                                    : loop_jacperf2_stn_cuda),
                                                         2, A, B));
#endif
        dvmh_loop_perform_C(cur_loop);
        dvmh_region_end_C(cur_region);

        dvmh_get_actual_variable2_(&eps);
        eps_out[it - 1] = eps;
        done = it;
        if (eps < 0.5f) break;
    }
    if (a_out) fetch(A, rank, L, a_out);
    if (b_out) fetch(B, rank, L, b_out);
    dvmh_array_free_C(B);
    dvmh_array_free_C(A);
    return done;
}
