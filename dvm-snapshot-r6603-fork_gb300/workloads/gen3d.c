/*
 * A 3-D loop whose CUDA handler has exactly the shape cdvmh generates
 * (gen3d_cuda.cu): the runtime's contract for unmodified generated handlers.
 * Main code in the form cdvmh converts a DVMH-C program to
 * (cdvmh/src/converter_main.cpp:2560-2960).
 *
 * Source program:
 *   A = seeded uniform[0,1), B = 0
 *   region {
 *     parallel([i][j][k] on B[i][j][k]) reduction(sum(s), maxloc(mx, lc)):
 *       B[i][j][k] = A[i-1][j][k] + 0.5 * A[i][j][k+1];
 *       s = s + B[i][j][k];
 *       if (B[i][j][k] > mx) { mx = B[i][j][k]; lc = (i * n1 + j) * n2 + k; }
 *   }                                                  (i, j, k over the interior)
 *   get_actual(s, mx, lc, B)
 */
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64], B[64];
static long n12v, n2v;  /* plane and row sizes, used by the loop body for lc */

#ifndef WL_NO_CUDA
void loop_gen3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], long *n12_ptr, long *n2_ptr, double *s_ptr,
                     double *mx_ptr, long *lc_ptr);
#endif

/* the sequential host form, loop order */
void loop_gen3d_host(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], long *n12_ptr, long *n2_ptr, double *s_ptr,
                     double *mx_ptr, long *lc_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (double (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    double (*b)[B_hdr[1] / B_hdr[2]][B_hdr[2]] =
        (double (*)[B_hdr[1] / B_hdr[2]][B_hdr[2]])dvmh_get_natural_base_C(device_num, B_hdr);
    long n12 = *n12_ptr, n2 = *n2_ptr;
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3];
    DvmType i, j, k;
    double s, mx;
    long lc;
    (void)s_ptr, (void)mx_ptr, (void)lc_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    dvmh_loop_red_init_C(loop_ref, 2, &mx, &lc);
    for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
        for (j = boundsLow[1]; j <= boundsHigh[1]; j++)
            for (k = boundsLow[2]; k <= boundsHigh[2]; k++) {
                b[i][j][k] = a[i - 1][j][k] + 0.5 * a[i][j][k + 1];
                s = s + b[i][j][k];
                if (b[i][j][k] > mx) {
                    mx = b[i][j][k];
                    lc = i * n12 + j * n2 + k;
                }
            }
    dvmh_loop_red_post_C(loop_ref, 1, &s, 0);
    dvmh_loop_red_post_C(loop_ref, 2, &mx, &lc);
}

/* One run of the program on an n0 x n1 x n2 grid.  A CUDA block (bx, by, bz) > 0
 * is set on the loop as the program's cuda_block clause would; 0 keeps the
 * runtime's choice.  s, mx and lc hold the reduction variables' initial values on
 * entry and their results on return; b_out (n0*n1*n2 doubles, dense) gets B. */
int wl_gen3d_run(long n0, long n1, long n2, uint64_t seed, int bx, int by, int bz, double *s, double *mx, long *lc,
                 double *b_out) {
    long i, j, k, st[3];
    double *a, *b;
    DvmType cur_region, cur_loop;
    dvmh_array_create_C(A, 3, -rt_DOUBLE, (DvmType)n0, 1L, 1L, (DvmType)n1, 1L, 1L, (DvmType)n2, 1L, 1L);
    dvmh_distribute_C(A, 3, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2), dvmh_distribution_block_C(3));
    dvmh_array_create_C(B, 3, -rt_DOUBLE, (DvmType)n0, 1L, 1L, (DvmType)n1, 1L, 1L, (DvmType)n2, 1L, 1L);
    dvmh_align_C(B, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                 dvmh_alignment_linear_C(3, 1, 0));
    a = (double *)dvmh_get_natural_base_C(0, A);
    b = (double *)dvmh_get_natural_base_C(0, B);
    wl_strides(A, 3, st);
    for (i = 0; i < n0; i++)
        for (j = 0; j < n1; j++)
            for (k = 0; k < n2; k++) {
                a[i * st[0] + j * st[1] + k] = wl_u01(seed, 7, (uint64_t)((i * n1 + j) * n2 + k));
                b[i * st[0] + j * st[1] + k] = 0.0;
            }
    dvmh_actual_array2_(A);
    dvmh_actual_array2_(B);
    n12v = n1 * n2;
    n2v = n2;
    dvmh_actual_variable2_(&n12v);
    dvmh_actual_variable2_(&n2v);
    dvmh_actual_variable2_(s);
    dvmh_actual_variable2_(mx);
    dvmh_actual_variable2_(lc);

    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_IN, A, "A");
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, B, "B");
    dvmh_region_register_scalar_C(cur_region, INTENT_IN, &n12v, sizeof(n12v), "n12");
    dvmh_region_register_scalar_C(cur_region, INTENT_IN, &n2v, sizeof(n2v), "n2");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, s, sizeof(*s), "s");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, mx, sizeof(*mx), "mx");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, lc, sizeof(*lc), "lc");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
    dvmh_shadow_renew_C(A, 0, 0);
    cur_loop = dvmh_loop_create_C(cur_region, 3, 1L, (DvmType)(n0 - 2), 1L, 1L, (DvmType)(n1 - 2), 1L, 1L,
                                  (DvmType)(n2 - 2), 1L);
    dvmh_loop_map_C(cur_loop, B, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                    dvmh_alignment_linear_C(3, 1, 0));
    if (bx > 0) dvmh_loop_set_cuda_block_C(cur_loop, bx, by, bz);
    dvmh_loop_reduction_C(cur_loop, rf_SUM, s, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_MAXLOC, mx, rt_DOUBLE, 1, lc, sizeof(*lc));
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_gen3d_host, 7, A, B, &n12v, &n2v, s, mx, lc));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_gen3d_cuda, 7, A, B, &n12v, &n2v, s, mx, lc));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);
    dvmh_get_actual_variable2_(s);
    dvmh_get_actual_variable2_(mx);
    dvmh_get_actual_variable2_(lc);
    dvmh_get_actual_array2_(B);
    for (i = 0; i < n0; i++)
        for (j = 0; j < n1; j++)
            memcpy(b_out + (i * n1 + j) * n2, b + i * st[0] + j * st[1], sizeof(double) * n2);
    dvmh_array_free_C(B);
    dvmh_array_free_C(A);
    return 0;
}
