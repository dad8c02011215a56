/*
 * A 2-D ACROSS loop with one dependence (a recurrence along j, independent
 * rows) whose CUDA handler has the shape cdvmh generates for one dependence
 * when asked for automatic transforms (rec2d_cuda.cu: one launch per value of
 * the dependent index, the independent rows across the threads, the array
 * indexed through the header, which may describe a permuted layout).  Main
 * code in the form cdvmh converts a DVMH-C program to (converter_main.cpp:2560-2960).
 *
 * Source program (n0 x n1 array):
 *   A = seeded uniform[0,1)
 *   repeat sweeps times:
 *     region {
 *       parallel([i][j] on A[i][j]) across(A[0:0][1:0]) reduction(min(lo)):
 *         A[i][j] = A[i][j] * 0.5 + A[i][j-1] * 0.25;   lo = min(lo, A[i][j])
 *     }                                                  (i in 0..n0-1, j in 1..n1-1)
 *     get_actual(lo)
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64];

#ifndef WL_NO_CUDA
void loop_rec2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *lo_ptr);
#endif

/* the sequential host form, loop order */
void loop_rec2d_host(DvmType *pLoopRef, DvmType A_hdr[], double *lo_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    DvmType i, j;
    double lo;
    (void)lo_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &lo, 0);
    for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
        for (j = boundsLow[1]; j <= boundsHigh[1]; j++) {
            a[i][j] = a[i][j] * 0.5 + a[i][j - 1] * 0.25;
            lo = a[i][j] < lo ? a[i][j] : lo;
        }
    dvmh_loop_red_post_C(loop_ref, 1, &lo, 0);
}

/* lo_out[t] = lo after sweep t; a_out (n0*n1) = A */
int wl_rec2d_run(long n0, long n1, long sweeps, uint64_t seed, double *lo_out, double *a_out) {
    static double lo;
    long i, j, t, st[2];
    double *a;
    DvmType cur_region, cur_loop;
    dvmh_array_create_C(A, 2, -rt_DOUBLE, (DvmType)n0, 0L, 0L, (DvmType)n1, 1L, 0L);
    dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
    a = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 2, st);
    for (i = 0; i < n0; i++)
        for (j = 0; j < n1; j++) a[i * st[0] + j] = wl_u01(seed, 19, (uint64_t)(i * n1 + j));
    dvmh_actual_array2_(A);
    for (t = 0; t < sweeps; t++) {
        lo = 1.0;
        dvmh_actual_variable2_(&lo);
        cur_region = dvmh_region_create_C(0);
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
        dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &lo, sizeof(lo), "lo");
        dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
        cur_loop = dvmh_loop_create_C(cur_region, 2, 0L, (DvmType)(n0 - 1), 1L, 1L, (DvmType)(n1 - 1), 1L);
        dvmh_loop_map_C(cur_loop, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
        dvmh_loop_across_C(cur_loop, 0, A, 2, 0L, 0L, 1L, 0L);
        dvmh_loop_reduction_C(cur_loop, rf_MIN, &lo, rt_DOUBLE, 1, 0, 0);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_rec2d_host, 2, A, &lo));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_rec2d_cuda, 2, A, &lo));
#endif
        dvmh_loop_perform_C(cur_loop);
        dvmh_region_end_C(cur_region);
        dvmh_get_actual_variable2_(&lo);
        lo_out[t] = lo;
    }
    dvmh_get_actual_array2_(A);
    for (i = 0; i < n0; i++) memcpy(a_out + i * n1, a + i * st[0], sizeof(double) * n1);
    dvmh_array_free_C(A);
    return 0;
}
