/*
 * A 1-D loop with a non-unit (possibly negative) step and eight reductions of
 * four types, whose CUDA handler has exactly the shape cdvmh generates
 * (genred_cuda.cu).  It exercises loop normalisation (rts/dvmh/loop.cpp:556-565),
 * signed steps in dvmh_loop_fill_bounds_C and the reduction engine's operations
 * (loop.cpp:116-238) through generated per-thread reduction slots.
 *
 * Source program:
 *   X = seeded uniform[0,1) (double), V = seeded integers (int)
 *   region {
 *     parallel([i] on X[i]) reduction(sum(ds), product(dp), min(imn), max(fmx),
 *                                     and(ia), or(io), xor(ix), minloc(dml, lc)):
 *       for i = start; i (step > 0 ? <= : >=) end; i += step:
 *         ds = ds + X[i];  dp = dp * (1.0 + X[i] / 65536.0);
 *         imn = Min(imn, V[i]);  fmx = Max(fmx, (float)X[i]);
 *         ia &= V[i] | 0x0F0F0F0F;  io |= V[i] & 0x00FF00FF;  ix ^= V[i];
 *         if (X[i] < dml) { dml = X[i]; lc = i; }
 *   }
 */
#include "dvmhlib2.h"
#include "wl_common.h"

static DvmType X[64], V[64];

#ifndef WL_NO_CUDA
void loop_genred_cuda(DvmType *pLoopRef, DvmType X_hdr[], DvmType V_hdr[], double *ds_ptr, double *dp_ptr,
                      int *imn_ptr, float *fmx_ptr, int *ia_ptr, int *io_ptr, int *ix_ptr, double *dml_ptr,
                      long *lc_ptr);
#endif

/* the sequential host form (cdvmh's host handler: reduction variables
 * initialised by the runtime, the loop in its own order, results posted) */
void loop_genred_host(DvmType *pLoopRef, DvmType X_hdr[], DvmType V_hdr[], double *ds_ptr, double *dp_ptr,
                      int *imn_ptr, float *fmx_ptr, int *ia_ptr, int *io_ptr, int *ix_ptr, double *dml_ptr,
                      long *lc_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *x = (double *)dvmh_get_natural_base_C(device_num, X_hdr);
    int *v = (int *)dvmh_get_natural_base_C(device_num, V_hdr);
    DvmType lo, hi, st, i;
    double ds, dp, dml;
    int imn, ia, io, ix;
    float fmx;
    long lc;
    (void)ds_ptr, (void)dp_ptr, (void)imn_ptr, (void)fmx_ptr, (void)ia_ptr, (void)io_ptr, (void)ix_ptr;
    (void)dml_ptr, (void)lc_ptr;
    dvmh_loop_fill_bounds_C(loop_ref, &lo, &hi, &st);
    dvmh_loop_red_init_C(loop_ref, 1, &ds, 0);
    dvmh_loop_red_init_C(loop_ref, 2, &dp, 0);
    dvmh_loop_red_init_C(loop_ref, 3, &imn, 0);
    dvmh_loop_red_init_C(loop_ref, 4, &fmx, 0);
    dvmh_loop_red_init_C(loop_ref, 5, &ia, 0);
    dvmh_loop_red_init_C(loop_ref, 6, &io, 0);
    dvmh_loop_red_init_C(loop_ref, 7, &ix, 0);
    dvmh_loop_red_init_C(loop_ref, 8, &dml, &lc);
    for (i = lo; st > 0 ? i <= hi : i >= hi; i += st) {
        ds = ds + x[i];
        dp = dp * (1.0 + x[i] / 65536.0);
        imn = v[i] < imn ? v[i] : imn;
        fmx = (float)x[i] > fmx ? (float)x[i] : fmx;
        ia &= v[i] | 0x0F0F0F0F;
        io |= v[i] & 0x00FF00FF;
        ix ^= v[i];
        if (x[i] < dml) {
            dml = x[i];
            lc = i;
        }
    }
    dvmh_loop_red_post_C(loop_ref, 1, &ds, 0);
    dvmh_loop_red_post_C(loop_ref, 2, &dp, 0);
    dvmh_loop_red_post_C(loop_ref, 3, &imn, 0);
    dvmh_loop_red_post_C(loop_ref, 4, &fmx, 0);
    dvmh_loop_red_post_C(loop_ref, 5, &ia, 0);
    dvmh_loop_red_post_C(loop_ref, 6, &io, 0);
    dvmh_loop_red_post_C(loop_ref, 7, &ix, 0);
    dvmh_loop_red_post_C(loop_ref, 8, &dml, &lc);
}

/* Deterministic edge-value inputs (the reductions' order-sensitive cases):
 *   0: +0, -0, -0.5, a subnormal, -inf (MAX of the float conversions is a
 *      signed zero: the first in loop order wins; MINLOC ties at -inf)
 *   1: 0.25, NaN, +inf, -0, the smallest subnormal (SUM and PROD are NaN; NaN
 *      never enters a MIN/MAX/MINLOC slot: its comparisons are false)
 *   2: every value 0.5 and every int 7 (MINLOC: the first in loop order)
 * V: a multiplicative hash of the index over the whole int range. */
int wl_genred_pattern(int pattern, long n, double *x, int *v) {
    static const double p0[5] = {0.0, -0.0, -0.5, -1e-310, -__builtin_inf()};
    static const double p1[5] = {0.25, __builtin_nan(""), __builtin_inf(), -0.0, 4.9406564584124654e-324};
    long i;
    for (i = 0; i < n; i++) {
        uint64_t h = (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
        int k = (int)((h >> 40) % 5);
        x[i] = pattern == 0 ? p0[k] : pattern == 1 ? p1[k] : 0.5;
        v[i] = pattern == 2 ? 7 : (int)(uint32_t)(h >> 32);
    }
    return 0;
}

static int genred(long n, long start, long end, long step, uint64_t seed, const double *xin, const int *vin, int bx,
                  double *d3, int *i4, float *f1, long *lc);

/* red: the eight reduction variables' initial values in, results out:
 * ds, dp, dml (double[3]), imn, ia, io, ix (int[4]), fmx (float[1]), lc (long[1]). */
int wl_genred_run(long n, long start, long end, long step, uint64_t seed, int bx, double *d3, int *i4, float *f1,
                  long *lc) {
    return genred(n, start, end, step, seed, 0, 0, bx, d3, i4, f1, lc);
}

/* the same program on given X (n doubles) and V (n ints) */
int wl_genred_run_data(long n, long start, long end, long step, const double *x, const int *v, int bx, double *d3,
                       int *i4, float *f1, long *lc) {
    return genred(n, start, end, step, 0, x, v, bx, d3, i4, f1, lc);
}

static int genred(long n, long start, long end, long step, uint64_t seed, const double *xin, const int *vin, int bx,
                  double *d3, int *i4, float *f1, long *lc) {
    static double ds, dp, dml;
    static int imn, ia, io, ix;
    static float fmx;
    static long lcv;
    long i;
    double *x;
    int *v;
    DvmType cur_region, cur_loop;
    ds = d3[0], dp = d3[1], dml = d3[2];
    imn = i4[0], ia = i4[1], io = i4[2], ix = i4[3];
    fmx = f1[0];
    lcv = lc[0];
    dvmh_array_create_C(X, 1, -rt_DOUBLE, (DvmType)n, 0L, 0L);
    dvmh_distribute_C(X, 1, dvmh_distribution_block_C(1));
    dvmh_array_create_C(V, 1, -rt_INT, (DvmType)n, 0L, 0L);
    dvmh_align_C(V, X, 1, dvmh_alignment_linear_C(1, 1, 0));
    x = (double *)dvmh_get_natural_base_C(0, X);
    v = (int *)dvmh_get_natural_base_C(0, V);
    for (i = 0; i < n; i++) {
        x[i] = xin ? xin[i] : wl_u01(seed, 11, (uint64_t)i);
        v[i] = vin ? vin[i] : (int)(wl_u01(seed, 12, (uint64_t)i) * 2147483647.0) - 1073741824;
    }
    dvmh_actual_array2_(X);
    dvmh_actual_array2_(V);
    dvmh_actual_variable2_(&ds);
    dvmh_actual_variable2_(&dp);
    dvmh_actual_variable2_(&dml);
    dvmh_actual_variable2_(&imn);
    dvmh_actual_variable2_(&ia);
    dvmh_actual_variable2_(&io);
    dvmh_actual_variable2_(&ix);
    dvmh_actual_variable2_(&fmx);
    dvmh_actual_variable2_(&lcv);

    cur_region = dvmh_region_create_C(0);
    dvmh_region_register_array_C(cur_region, INTENT_IN, X, "X");
    dvmh_region_register_array_C(cur_region, INTENT_IN, V, "V");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &ds, sizeof(ds), "ds");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &dp, sizeof(dp), "dp");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &imn, sizeof(imn), "imn");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &fmx, sizeof(fmx), "fmx");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &ia, sizeof(ia), "ia");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &io, sizeof(io), "io");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &ix, sizeof(ix), "ix");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &dml, sizeof(dml), "dml");
    dvmh_region_register_scalar_C(cur_region, INTENT_INOUT, &lcv, sizeof(lcv), "lc");
    dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);
    cur_loop = dvmh_loop_create_C(cur_region, 1, (DvmType)start, (DvmType)end, (DvmType)step);
    dvmh_loop_map_C(cur_loop, X, 1, dvmh_alignment_linear_C(1, 1, 0));
    if (bx > 0) dvmh_loop_set_cuda_block_C(cur_loop, bx, 1, 1);
    dvmh_loop_reduction_C(cur_loop, rf_SUM, &ds, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_PROD, &dp, rt_DOUBLE, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_MIN, &imn, rt_INT, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_MAX, &fmx, rt_FLOAT, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_AND, &ia, rt_INT, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_OR, &io, rt_INT, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_XOR, &ix, rt_INT, 1, 0, 0);
    dvmh_loop_reduction_C(cur_loop, rf_MINLOC, &dml, rt_DOUBLE, 1, &lcv, sizeof(lcv));
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_genred_host, 11, X, V, &ds, &dp, &imn, &fmx,
                                                     &ia, &io, &ix, &dml, &lcv));
#ifndef WL_NO_CUDA
    dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                 dvmh_handler_func_C((DvmHandlerFunc)loop_genred_cuda, 11, X, V, &ds, &dp, &imn, &fmx,
                                                     &ia, &io, &ix, &dml, &lcv));
#endif
    dvmh_loop_perform_C(cur_loop);
    dvmh_region_end_C(cur_region);
    dvmh_get_actual_variable2_(&ds);
    dvmh_get_actual_variable2_(&dp);
    dvmh_get_actual_variable2_(&dml);
    dvmh_get_actual_variable2_(&imn);
    dvmh_get_actual_variable2_(&ia);
    dvmh_get_actual_variable2_(&io);
    dvmh_get_actual_variable2_(&ix);
    dvmh_get_actual_variable2_(&fmx);
    dvmh_get_actual_variable2_(&lcv);
    d3[0] = ds, d3[1] = dp, d3[2] = dml;
    i4[0] = imn, i4[1] = ia, i4[2] = io, i4[3] = ix;
    f1[0] = fmx;
    lc[0] = lcv;
    dvmh_array_free_C(V);
    dvmh_array_free_C(X);
    return 0;
}
