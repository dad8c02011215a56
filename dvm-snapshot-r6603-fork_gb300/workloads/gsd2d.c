/*
 * A 2-D ACROSS loop with two dependences whose CUDA handler has the shape
 * cdvmh generates when asked for automatic transforms (gsd2d_cuda.cu: one
 * launch per diagonal, the array indexed through the header, which may
 * describe a diagonalised layout).  Main code in the form cdvmh converts a
 * DVMH-C program to (converter_main.cpp:2560-2960).
 *
 * Source program (n0 x n1 array; the loop runs each axis forward or backward):
 *   A = seeded uniform[0,1) inside, 0 on the boundary
 *   repeat sweeps times:
 *     m = 0
 *     region {
 *       parallel([i][j] on A[i][j]) across(A[1:1][1:1]) reduction(max(m)):
 *         old = A[i][j];
 *         A[i][j] = (A[i-1][j] + A[i+1][j] + A[i][j-1] + A[i][j+1]) * 0.25;
 *         m = max(m, |A[i][j] - old|)
 *     }
 *     get_actual(m)        (every sweep, or only after the last one)
 *     optionally (mirror):
 *     region { parallel([i][j] on B[i][j]): B[i][j] = A[i][j] * 2 }   (all of B)
 * The mirror loop's handler does not ask for transforms: the runtime gives it
 * A in the natural layout, between two sweeps that work on the transformed one.
 * The host handlers below are the sequential form (one slot); the reference
 * runtime runs them in loop order, which is the order the results are pinned to.
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64], B[64];

#ifndef WL_NO_CUDA
void loop_gsd2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr);
void loop_gsd2d_mirror_cuda(DvmType *pLoopRef, DvmType B_hdr[], DvmType A_hdr[]);
#endif

void loop_gsd2d_host(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    DvmType i, j;
    double m;
    (void)m_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &m, 0);
    for (i = boundsLow[0]; loopSteps[0] > 0 ? i <= boundsHigh[0] : i >= boundsHigh[0]; i += loopSteps[0])
        for (j = boundsLow[1]; loopSteps[1] > 0 ? j <= boundsHigh[1] : j >= boundsHigh[1]; j += loopSteps[1]) {
            double old = a[i][j];
            a[i][j] = (a[i - 1][j] + a[i + 1][j] + a[i][j - 1] + a[i][j + 1]) * 0.25;
            m = fabs(a[i][j] - old) > m ? fabs(a[i][j] - old) : m;
        }
    dvmh_loop_red_post_C(loop_ref, 1, &m, 0);
}

void loop_gsd2d_mirror_host(DvmType *pLoopRef, DvmType B_hdr[], DvmType A_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*b)[B_hdr[1]] = (double (*)[B_hdr[1]])dvmh_get_natural_base_C(device_num, B_hdr);
    double (*a)[A_hdr[1]] = (double (*)[A_hdr[1]])dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    DvmType i, j;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
        for (j = boundsLow[1]; j <= boundsHigh[1]; j++) b[i][j] = a[i][j] * 2.0;
}

static double m;
static long N0, N1;

/* A (n0 x n1) seeded, B (n0 x n1, aligned with A) */
int wl_gsd2d_setup(long n0, long n1, uint64_t seed) {
    long i, j, st[2];
    double *a;
    N0 = n0;
    N1 = n1;
    dvmh_array_create_C(A, 2, -rt_DOUBLE, (DvmType)n0, 1L, 1L, (DvmType)n1, 1L, 1L);
    dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
    dvmh_array_create_C(B, 2, -rt_DOUBLE, (DvmType)n0, 0L, 0L, (DvmType)n1, 0L, 0L);
    dvmh_align_C(B, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    a = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 2, st);
    for (i = 0; i < n0; i++)
        for (j = 0; j < n1; j++)
            a[i * st[0] + j] =
                (i == 0 || j == 0 || i == n0 - 1 || j == n1 - 1) ? 0.0 : wl_u01(seed, 17, (uint64_t)(i * n1 + j));
    dvmh_actual_array2_(A);
    return 0;
}

/* `sweeps` sweeps; m_out[t] = m after sweep t (readEach) or m_out[0] = m after
 * the last sweep.  dir0 / dir1: +1 forward, -1 backward loops. */
int wl_gsd2d_sweeps(long sweeps, int dir0, int dir1, int readEach, int mirror, double *m_out) {
    long t, n0 = N0, n1 = N1;
    DvmType cur_region, cur_loop;
    for (t = 0; t < sweeps; t++) {
        m = 0;
        dvmh_actual_variable2_(&m);
        cur_region = dvmh_region_create_C(0);
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
        dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &m, sizeof(m), "m");
        dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
        cur_loop = dvmh_loop_create_C(cur_region, 2, (DvmType)(dir0 > 0 ? 1 : n0 - 2), (DvmType)(dir0 > 0 ? n0 - 2 : 1),
                                      (DvmType)dir0, (DvmType)(dir1 > 0 ? 1 : n1 - 2),
                                      (DvmType)(dir1 > 0 ? n1 - 2 : 1), (DvmType)dir1);
        dvmh_loop_map_C(cur_loop, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
        dvmh_loop_across_C(cur_loop, 0, A, 2, 1L, 1L, 1L, 1L);
        dvmh_loop_reduction_C(cur_loop, rf_MAX, &m, rt_DOUBLE, 1, 0, 0);
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gsd2d_host, 2, A, &m));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_gsd2d_cuda, 2, A, &m));
#endif
        dvmh_loop_perform_C(cur_loop);
        dvmh_region_end_C(cur_region);
        if (mirror) {
            cur_region = dvmh_region_create_C(0);
            dvmh_region_register_array_C(cur_region, INTENT_IN, A, "A");
            dvmh_region_register_array_C(cur_region, INTENT_OUT, B, "B");
            dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
            cur_loop = dvmh_loop_create_C(cur_region, 2, 0L, (DvmType)(n0 - 1), 1L, 0L, (DvmType)(n1 - 1), 1L);
            dvmh_loop_map_C(cur_loop, B, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
            dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                         dvmh_handler_func_C((DvmHandlerFunc)loop_gsd2d_mirror_host, 2, B, A));
#ifndef WL_NO_CUDA
            dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                         dvmh_handler_func_C((DvmHandlerFunc)loop_gsd2d_mirror_cuda, 2, B, A));
#endif
            dvmh_loop_perform_C(cur_loop);
            dvmh_region_end_C(cur_region);
        }
        if (readEach || t == sweeps - 1) {
            dvmh_get_actual_variable2_(&m);
            m_out[readEach ? t : 0] = m;
        }
    }
    return 0;
}

/* a_out (n0*n1) = A; b_out (n0*n1) = B when non-null */
int wl_gsd2d_fetch(double *a_out, double *b_out) {
    long i, st[2];
    double *a = (double *)dvmh_get_natural_base_C(0, A), *b;
    dvmh_get_actual_array2_(A);
    wl_strides(A, 2, st);
    for (i = 0; i < N0; i++) memcpy(a_out + i * N1, a + i * st[0], sizeof(double) * N1);
    if (b_out) {
        dvmh_get_actual_array2_(B);
        b = (double *)dvmh_get_natural_base_C(0, B);
        wl_strides(B, 2, st);
        for (i = 0; i < N0; i++) memcpy(b_out + i * N1, b + i * st[0], sizeof(double) * N1);
    }
    return 0;
}

int wl_gsd2d_free(void) {
    dvmh_array_free_C(B);
    dvmh_array_free_C(A);
    return 0;
}

/* the whole program: setup, sweeps, fetch (b_out when mirror), free */
int wl_gsd2d_run(long n0, long n1, long sweeps, uint64_t seed, int dir0, int dir1, int readEach, int mirror,
                 double *m_out, double *a_out, double *b_out) {
    wl_gsd2d_setup(n0, n1, seed);
    wl_gsd2d_sweeps(sweeps, dir0, dir1, readEach, mirror, m_out);
    wl_gsd2d_fetch(a_out, mirror ? b_out : 0);
    return wl_gsd2d_free();
}
