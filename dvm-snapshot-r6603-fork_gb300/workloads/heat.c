/*
 * Batched uneven heat equation: `count` independent 2-D FP64 arrays of
 * log-uniform side, one explicit 5-point step each per time step, with a SUM
 * and a MINLOC reduction per array -- C-DVMH program in the form cdvmh converts
 * it to (main code: cdvmh/src/converter_main.cpp:2560-2960; OpenMP host
 * handler :1503-1859).  CUDA handlers: heat_cuda.cu.
 *
 * Source program, for each time step t (src/dst swap every step):
 *   sums[k] = 0; mins[k] = 1e300; locs[k] = {-1, -1}      (all k)
 *   region {
 *     for each array k:
 *       parallel([i][j] on dst_k[i][j]) reduction(sum(sums[k]), minloc(mins[k], locs[k])):
 *         dst[i][j] = src[i][j] + c * (src[i-1][j] + src[i+1][j] + src[i][j-1]
 *                                      + src[i][j+1] - 4.0 * src[i][j])     (interior)
 *         sums[k] += dst[i][j]
 *         if (dst[i][j] < mins[k]) { mins[k] = dst[i][j]; locs[k] = {i, j} }
 *   }
 *   get_actual(sums, mins, locs)
 * Sides: s_k = floor(lo * (hi/lo)^u_k), u_k from stream 1000 of the seed.
 * Array k interior = stream 1 + k, boundary 0 (both buffers).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dvmhlib2.h"
#include "wl_common.h"

#ifdef _OPENMP
#define OMP_HANDLER_TYPE (HANDLER_TYPE_MASTER | HANDLER_TYPE_PARALLEL)
#else
#define OMP_HANDLER_TYPE 0
#endif

static DvmType (*U)[64], (*V)[64];
static long *sides;
static double *sums, *mins;
static int (*locs)[2];
static double coef;
static long step_no;
static wl_heat_params P;

#ifndef WL_NO_CUDA
void loop_heat_cuda(DvmType *pLoopRef, DvmType S_hdr[], DvmType D_hdr[], double *sum_ptr, double *min_ptr,
                    int *loc_ptr, double *c_ptr);
#endif

void loop_heat_host(DvmType *pLoopRef, DvmType S_hdr[], DvmType D_hdr[], double *sum_ptr, double *min_ptr,
                    int *loc_ptr, double *c_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*src)[S_hdr[1]] = (double (*)[S_hdr[1]])dvmh_get_natural_base_C(device_num, S_hdr);
    double (*dst)[D_hdr[1]] = (double (*)[D_hdr[1]])dvmh_get_natural_base_C(device_num, D_hdr);
    double c = *c_ptr;
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    int slotCount;
    (void)sum_ptr;
    (void)min_ptr;
    (void)loc_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    slotCount = dvmh_loop_get_slot_count_C(loop_ref);
#pragma omp parallel num_threads(slotCount)
    {
        double sm, mn;
        int lc[2];
        DvmType i, j;
        dvmh_loop_red_init_C(loop_ref, 1, &sm, 0);
        dvmh_loop_red_init_C(loop_ref, 2, &mn, lc);
#pragma omp for schedule(runtime) nowait
        for (i = boundsLow[0]; i <= boundsHigh[0]; i++)
            for (j = boundsLow[1]; j <= boundsHigh[1]; j++) {
                dst[i][j] = src[i][j] + c * (src[i - 1][j] + src[i + 1][j] + src[i][j - 1] + src[i][j + 1] -
                                             4.0 * src[i][j]);
                sm += dst[i][j];
                if (dst[i][j] < mn) {
                    mn = dst[i][j];
                    lc[0] = (int)i;
                    lc[1] = (int)j;
                }
            }
        dvmh_loop_red_post_C(loop_ref, 1, &sm, 0);
        dvmh_loop_red_post_C(loop_ref, 2, &mn, lc);
    }
}

/* sides_out (may be NULL) receives the count array sides. */
int wl_heat_setup(const wl_heat_params *p, long *sides_out) {
    long k, i, j;
    P = *p;
    coef = p->coef;
    step_no = 0;
    U = calloc(p->count, sizeof(*U));
    V = calloc(p->count, sizeof(*V));
    sides = calloc(p->count, sizeof(long));
    sums = calloc(p->count, sizeof(double));
    mins = calloc(p->count, sizeof(double));
    locs = calloc(p->count, sizeof(*locs));
    for (k = 0; k < p->count; k++) {
        double u = wl_u01(p->seed, 1000, (uint64_t)k);
        long n = (long)floor((double)p->side_lo * pow((double)p->side_hi / (double)p->side_lo, u)), st[2];
        double *a, *b;
        if (n < 3)
            n = 3;
        if (n > p->side_hi)
            n = p->side_hi;
        sides[k] = n;
        dvmh_array_create_C(U[k], 2, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
        dvmh_distribute_C(U[k], 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
        dvmh_array_create_C(V[k], 2, -rt_DOUBLE, (DvmType)n, 1L, 1L, (DvmType)n, 1L, 1L);
        dvmh_align_C(V[k], U[k], 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
        a = (double *)dvmh_get_natural_base_C(0, U[k]);
        b = (double *)dvmh_get_natural_base_C(0, V[k]);
        wl_strides(U[k], 2, st);
        for (i = 0; i < n; i++)
            for (j = 0; j < n; j++) {
                long lin = i * n + j, q = i * st[0] + j;
                if (i == 0 || j == 0 || i == n - 1 || j == n - 1)
                    a[q] = 0.0;
                else
                    a[q] = wl_u01(p->seed, 1 + (uint64_t)k, (uint64_t)lin);
                b[q] = 0.0;
            }
        dvmh_actual_array2_(U[k]);
        dvmh_actual_array2_(V[k]);
    }
    if (sides_out)
        memcpy(sides_out, sides, sizeof(long) * p->count);
    return 0;
}

/* One time step over all arrays. */
void wl_heat_step(void) {
    long k, cnt = P.count;
    DvmType cur_region, cur_loop;
    DvmType (*S)[64] = (step_no % 2 == 0) ? U : V;
    DvmType (*D)[64] = (step_no % 2 == 0) ? V : U;
    for (k = 0; k < cnt; k++) {
        sums[k] = 0.0;
        mins[k] = 1e300;
        locs[k][0] = -1;
        locs[k][1] = -1;
    }
    dvmh_actual_variable2_(sums);
    dvmh_actual_variable2_(mins);
    dvmh_actual_variable2_(locs);
    cur_region = dvmh_region_create_C(0);
    for (k = 0; k < cnt; k++) {
        dvmh_region_register_array_C(cur_region, INTENT_IN, S[k], "src");
        dvmh_region_register_array_C(cur_region, INTENT_INOUT, D[k], "dst");
    }
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, sums, sizeof(double) * cnt, "sums");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, mins, sizeof(double) * cnt, "mins");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, locs, sizeof(int) * 2 * cnt, "locs");
    dvmh_region_register_scalar_C(cur_region, INTENT_IN, &coef, sizeof(coef), "coef");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
    for (k = 0; k < cnt; k++) {
        long n = sides[k];
        dvmh_shadow_renew_C(S[k], 0, 0);
        cur_loop = dvmh_loop_create_C(cur_region, 2, 1L, (DvmType)(n - 2), 1L, 1L, (DvmType)(n - 2), 1L);
        dvmh_loop_map_C(cur_loop, D[k], 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
        dvmh_loop_reduction_C(cur_loop, rf_SUM, &sums[k], rt_DOUBLE, 1, 0, 0);
        dvmh_loop_reduction_C(cur_loop, rf_MINLOC, &mins[k], rt_DOUBLE, 1, locs[k], sizeof(locs[k]));
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_heat_host, 6, S[k], D[k], &sums[k],
                                                         &mins[k], locs[k], &coef));
#ifndef WL_NO_CUDA
        dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                     dvmh_handler_func_C((DvmHandlerFunc)loop_heat_cuda, 6, S[k], D[k], &sums[k],
                                                         &mins[k], locs[k], &coef));
#endif
        dvmh_loop_perform_C(cur_loop);
    }
    dvmh_region_end_C(cur_region);
    dvmh_get_actual_variable2_(sums);
    dvmh_get_actual_variable2_(mins);
    dvmh_get_actual_variable2_(locs);
    step_no++;
}

/* Runs `steps` steps; per step the count sums/mins/locs go to the outputs (may be NULL). */
int wl_heat_run(long steps, double *sums_out, double *mins_out, int *locs_out) {
    long t, cnt = P.count;
    for (t = 0; t < steps; t++) {
        wl_heat_step();
        if (sums_out)
            memcpy(sums_out + t * cnt, sums, sizeof(double) * cnt);
        if (mins_out)
            memcpy(mins_out + t * cnt, mins, sizeof(double) * cnt);
        if (locs_out)
            memcpy(locs_out + 2 * t * cnt, locs, sizeof(int) * 2 * cnt);
    }
    return 0;
}

/* Copies array k's current state (the buffer written last) to u_out. */
int wl_heat_fetch(long k, double *u_out) {
    DvmType *cur = (step_no % 2 == 0) ? U[k] : V[k];
    long n = sides[k], i, st[2];
    double *h;
    dvmh_get_actual_array2_(cur);
    h = (double *)dvmh_get_natural_base_C(0, cur);
    wl_strides(cur, 2, st);
    for (i = 0; i < n; i++)
        memcpy(u_out + i * n, h + i * st[0], sizeof(double) * n);
    return 0;
}

long wl_heat_total_cells(void) {
    long k, t = 0;
    for (k = 0; k < P.count; k++)
        t += (sides[k] - 2) * (sides[k] - 2);
    return t;
}

void wl_heat_teardown(void) {
    long k;
    for (k = P.count - 1; k >= 0; k--) {
        dvmh_array_free_C(V[k]);
        dvmh_array_free_C(U[k]);
    }
    free(U);
    free(V);
    free(sides);
    free(sums);
    free(mins);
    free(locs);
}
