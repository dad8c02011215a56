/*
 * A 3-D ACROSS loop with two dependences and one independent (outer) axis,
 * handler in the shape cdvmh generates with automatic transforms
 * (gsd3d_cuda.cu: one launch per diagonal of the two dependent axes, the
 * independent axis across the grid's y dimension).  With transforms the two
 * dependent axes form a diagonalised plane and the outer axis strides over
 * whole planes.  Main code in the form cdvmh converts a DVMH-C program to.
 *
 * Source program (n0 x n1 x n2 array; plane k is seeded as the 2-D program
 * gsd2d.c is with seed + k):
 *   repeat sweeps times:
 *     m = 0
 *     region {
 *       parallel([k][i][j] on A[k][i][j]) across(A[0:0][1:1][1:1]) reduction(max(m)):
 *         old = A[k][i][j];
 *         A[k][i][j] = (A[k][i-1][j] + A[k][i+1][j] + A[k][i][j-1] + A[k][i][j+1]) * 0.25;
 *         m = max(m, |A[k][i][j] - old|)
 *     }                                   (k in 0..n0-1, i in 1..n1-2, j in 1..n2-2)
 *     get_actual(m)
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64];

#ifndef WL_NO_CUDA
void loop_gsd3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr);
#endif

/* the sequential host form, loop order */
void loop_gsd3d_host(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (double (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3];
    DvmType i, j, k;
    double m;
    (void)m_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &m, 0);
    for (k = boundsLow[0]; k <= boundsHigh[0]; k++)
        for (i = boundsLow[1]; i <= boundsHigh[1]; i++)
            for (j = boundsLow[2]; j <= boundsHigh[2]; j++) {
                double old = a[k][i][j];
                a[k][i][j] = (a[k][i - 1][j] + a[k][i + 1][j] + a[k][i][j - 1] + a[k][i][j + 1]) * 0.25;
                m = fabs(a[k][i][j] - old) > m ? fabs(a[k][i][j] - old) : m;
            }
    dvmh_loop_red_post_C(loop_ref, 1, &m, 0);
}

/* m_out[t] = m after sweep t; a_out (n0*n1*n2) = A */
int wl_gsd3d_run(long n0, long n1, long n2, long sweeps, uint64_t seed, double *m_out, double *a_out) {
    static double m;
    long i, j, k, t, st[3];
    double *a;
    DvmType cur_region, cur_loop;
    dvmh_array_create_C(A, 3, -rt_DOUBLE, (DvmType)n0, 0L, 0L, (DvmType)n1, 1L, 1L, (DvmType)n2, 1L, 1L);
    dvmh_distribute_C(A, 3, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2), dvmh_distribution_block_C(3));
    a = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 3, st);
    for (k = 0; k < n0; k++)
        for (i = 0; i < n1; i++)
            for (j = 0; j < n2; j++)
                a[k * st[0] + i * st[1] + j] = (i == 0 || j == 0 || i == n1 - 1 || j == n2 - 1)
                                                   ? 0.0
                                                   : wl_u01(seed + (uint64_t)k, 17, (uint64_t)(i * n2 + j));
    dvmh_actual_array2_(A);
    for (t = 0; t < sweeps; t++) {
        m = 0;
        dvmh_actual_variable2_(&m);
        cur_region = dvmh_region_create_C(0);
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
        dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &m, sizeof(m), "m");
        dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
        cur_loop = dvmh_loop_create_C(cur_region, 3, 0L, (DvmType)(n0 - 1), 1L, 1L, (DvmType)(n1 - 2), 1L, 1L,
                                      (DvmType)(n2 - 2), 1L);
        dvmh_loop_map_C(cur_loop, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                        dvmh_alignment_linear_C(3, 1, 0));
        dvmh_loop_across_C(cur_loop, 0, A, 3, 0L, 0L, 1L, 1L, 1L, 1L);
        dvmh_loop_reduction_C(cur_loop, rf_MAX, &m, rt_DOUBLE, 1, 0, 0);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gsd3d_host, 2, A, &m));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gsd3d_cuda, 2, A, &m));
#endif
        dvmh_loop_perform_C(cur_loop);
        dvmh_region_end_C(cur_region);
        dvmh_get_actual_variable2_(&m);
        m_out[t] = m;
    }
    dvmh_get_actual_array2_(A);
    for (k = 0; k < n0; k++)
        for (i = 0; i < n1; i++) memcpy(a_out + (k * n1 + i) * n2, a + k * st[0] + i * st[1], sizeof(double) * n2);
    dvmh_array_free_C(A);
    return 0;
}
