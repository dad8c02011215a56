/*
 * A 2-D ACROSS loop (Gauss-Seidel with dependences (1:1, 1:1)) whose CUDA
 * handler has exactly the shape cdvmh generates for ACROSS loops in its basic
 * mode (gs2d_cuda.cu: one thread walks the loop nest in order,
 * cdvmh/src/converter_main.cpp:2138-2145 isOneThread).  Main code in the form
 * cdvmh converts a DVMH-C program to (converter_main.cpp:2560-2960).
 *
 * Source program:
 *   A = seeded uniform[0,1) inside, 0 on the boundary
 *   repeat sweeps times:
 *     s = 0
 *     region {
 *       parallel([i][j] on A[i][j]) across(A[1:1][1:1]) reduction(sum(s)):
 *         A[i][j] = (A[i-1][j] + A[i+1][j] + A[i][j-1] + A[i][j+1]) * 0.25;  s = s + A[i][j];
 *     }
 *     get_actual(s)
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64];

#ifndef WL_NO_CUDA
void loop_gs2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr);
#endif

/* the sequential host form, loop order */
void loop_gs2d_host(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    DvmType i, j;
    double s;
    (void)s_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
        for (j = boundsLow[1]; j <= boundsHigh[1]; j++) {
            a[i][j] = (a[i - 1][j] + a[i + 1][j] + a[i][j - 1] + a[i][j + 1]) * 0.25;
            s = s + a[i][j];
        }
    dvmh_loop_red_post_C(loop_ref, 1, &s, 0);
}

/* sweeps of the program on an n x n grid; s_out[t] = s after sweep t; a_out (n*n) = A */
int wl_gs2d_run(long n, long sweeps, uint64_t seed, double *s_out, double *a_out) {
    static double s;
    long i, j, t, st[2];
    double *a;
    DvmType cur_region, cur_loop;
    dvmh_array_create_C(A, 2, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
    a = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 2, st);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            a[i * st[0] + j] = (i == 0 || j == 0 || i == n - 1 || j == n - 1) ? 0.0 : wl_u01(seed, 13, (uint64_t)(i * n + j));
    dvmh_actual_array2_(A);
    for (t = 0; t < sweeps; t++) {
        s = 0;
        dvmh_actual_variable2_(&s);
        cur_region = dvmh_region_create_C(0);
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
        dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &s, sizeof(s), "s");
        dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
        cur_loop = dvmh_loop_create_C(cur_region, 2, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L);
        dvmh_loop_map_C(cur_loop, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
        dvmh_loop_across_C(cur_loop, 0, A, 2, 1L, 1L, 1L, 1L);
        dvmh_loop_reduction_C(cur_loop, rf_SUM, &s, rt_DOUBLE, 1, 0, 0);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gs2d_host, 2, A, &s));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gs2d_cuda, 2, A, &s));
#endif
        dvmh_loop_perform_C(cur_loop);
        dvmh_region_end_C(cur_region);
        dvmh_get_actual_variable2_(&s);
        s_out[t] = s;
    }
    dvmh_get_actual_array2_(A);
    for (i = 0; i < n; i++) memcpy(a_out + i * n, a + i * st[0], sizeof(double) * n);
    dvmh_array_free_C(A);
    return 0;
}
