/*
 * SOR / Gauss-Seidel 3-D, FP64, as an ACROSS loop -- C-DVMH program in the
 * form cdvmh converts it to (main code: cdvmh/src/converter_main.cpp:2560-2960,
 * across clause :2716-2723; host handler :1503-1859).  CUDA handler: sor3d_cuda.cu.
 *
 * Source program (after examples/Sor/sor.c:35-55, in 3-D FP64 with a SUM residual):
 *   A = seeded uniform[0,1) inside, 0 on the boundary
 *   repeat sweeps times:
 *     s = 0
 *     region {
 *       parallel([i][j][k] on A[i][j][k]) across(A[1:1][1:1][1:1]) reduction(sum(s)):
 *         old = A[i][j][k]
 *         nv  = (1 - w) * old + w / 6 * (A[i-1][j][k] + A[i+1][j][k] + A[i][j-1][k]
 *                                      + A[i][j+1][k] + A[i][j][k-1] + A[i][j][k+1])
 *         A[i][j][k] = nv;  s += (nv - old) * (nv - old)
 *     }
 *     get_actual(s)
 * The host handler below is the sequential form (one slot); with one thread the
 * reference runs it in loop order, which is the order every result is pinned to.
 */
#include <math.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType A[64];
static double s, w;
static wl_sor_params P;

#ifndef WL_NO_CUDA
void loop_sor3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr);
void loop_sor3d_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr);
#endif
static int useGenerated;

/* the CUDA handler the loop registers: 0 = sor3d_cuda.cu (the library's
 * wavefront kernel), 1 = sor3d_gen_cuda.cu (cdvmh's generated hyperplane shape) */
int wl_sor3d_use_generated(int on) {
    useGenerated = on;
    return 0;
}

void loop_sor3d_host(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A_hdr[1] / A_hdr[2]][A_hdr[2]] =
        (double (*)[A_hdr[1] / A_hdr[2]][A_hdr[2]])dvmh_get_natural_base_C(device_num, A_hdr);
    double w = *w_ptr;
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3];
    double s;
    DvmType i, j, k;
    (void)s_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
        for (j = boundsLow[1]; j <= boundsHigh[1]; j++)
            for (k = boundsLow[2]; k <= boundsHigh[2]; k++) {
                double old = a[i][j][k];
                double nv = (1.0 - w) * old + w / 6.0 * (a[i - 1][j][k] + a[i + 1][j][k] + a[i][j - 1][k] +
                                                         a[i][j + 1][k] + a[i][j][k - 1] + a[i][j][k + 1]);
                a[i][j][k] = nv;
                s += (nv - old) * (nv - old);
            }
    dvmh_loop_red_post_C(loop_ref, 1, &s, 0);
}

int wl_sor3d_setup(const wl_sor_params *p) {
    long n = p->n, i, j, k, st[3];
    double *a;
    P = *p;
    w = p->omega;
    dvmh_array_create_C(A, 3, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
    dvmh_distribute_C(A, 3, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2), dvmh_distribution_block_C(3));
    a = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 3, st);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            for (k = 0; k < n; k++) {
                long lin = (i * n + j) * n + k, q = i * st[0] + j * st[1] + k;
                if (i == 0 || j == 0 || k == 0 || i == n - 1 || j == n - 1 || k == n - 1)
                    a[q] = 0.0;
                else
                    a[q] = wl_u01(p->seed, 1, (uint64_t)lin);
            }
    dvmh_actual_array2_(A);
    return 0;
}

double wl_sor3d_step(void) {
    long n = P.n;
    DvmType cur_region, cur_loop;
    s = 0;
    dvmh_actual_variable2_(&s);
    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_INOUT, A, "A");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &s, sizeof(s), "s");
    dvmh_region_register_scalar_C(cur_region, INTENT_IN, &w, sizeof(w), "w");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);

    cur_loop = dvmh_loop_create_C(cur_region, 3, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L, 1L,
                                  (DvmType)(n - 2), 1L);
    dvmh_loop_map_C(cur_loop, A, 3, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0),
                    dvmh_alignment_linear_C(3, 1, 0));
    dvmh_loop_across_C(cur_loop, 0, A, 3, 1L, 1L, 1L, 1L, 1L, 1L);
    dvmh_loop_reduction_C(cur_loop, rf_SUM, &s, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_sor3d_host, 3, A, &s, &w));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)(useGenerated ? loop_sor3d_gen_cuda
                                                                                   : loop_sor3d_cuda),
                                                     3, A, &s, &w));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);

    dvmh_get_actual_variable2_(&s);
    return s;
}

int wl_sor3d_run(long sweeps, double *s_out) {
    long it;
    for (it = 0; it < sweeps; it++) {
        double r = wl_sor3d_step();
        if (s_out)
            s_out[it] = r;
    }
    return 0;
}

/* Copies the current A (dense n^3 doubles) to the caller. */
int wl_sor3d_fetch(double *a_out) {
    long n = P.n, i, j, st[3];
    double *h;
    dvmh_get_actual_array2_(A);
    h = (double *)dvmh_get_natural_base_C(0, A);
    wl_strides(A, 3, st);
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            memcpy(a_out + (i * n + j) * n, h + i * st[0] + j * st[1], sizeof(double) * n);
    return 0;
}

void wl_sor3d_teardown(void) {
    dvmh_array_free_C(A);
}
