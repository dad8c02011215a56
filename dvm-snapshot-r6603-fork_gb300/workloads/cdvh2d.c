/*
 * A weighted Jacobi 2-D program with regular (non-distributed) variables and
 * dynamic arrays, written out exactly as cdvmh converts it -- every call the
 * converter emits for these constructs, with the converter's own naming and
 * order -- so that it links unchanged against either runtime:
 *   - cdvmh's library-entry form (converter_main.cpp:901, 966-980): the entry
 *     function starts with dvmh_init_lib_C;
 *   - dynamic DVM arrays: dvmh_array_declare_C at the declaration (:721-735),
 *     malloc -> dvmh_array_alloc_C + dvmh_distribute_C / dvmh_align_C
 *     (:3385-3392), free -> dvmh_array_free_C (:3614-3640), dvmh_forget_header_ when
 *     the pointer goes out of scope (:742-749);
 *   - malloc / free of regular memory -> dvmh_malloc_C / dvmh_free_C
 *     (project_ctx.cpp:497-503);
 *   - a global regular array: data enter / exit in the module's init and
 *     finish functions (:866-872), registered by DvmhModuleInitializer
 *     (c_dvmh.cpp:204-222, in cdvh2d_init.cpp);
 *   - the implicit data region around a region: dvmh_data_enter_C of every
 *     regular variable it uses before dvmh_region_create_C, and
 *     dvmh_data_exit_C(..., 1) after dvmh_region_end_C (:3000-3010, 3094-3100);
 *     regular arrays registered through dvmh_variable_gen_header_C (file_ctx.cpp:297-316)
 *     and passed to handlers as dvmh_variable_get_header_C (:2797, file_ctx.cpp:318-328);
 *   - sequential code: an assignment to a DVM array element becomes an own
 *     computation through dvmh_get_own_element_addr_C (:3330-3345), a read
 *     goes through dvmh_get_element_addr_C (:3470-3500); get_actual -> :11-59.
 * CUDA handlers: cdvh2d_cuda.cu.
 *
 * Source program (C-DVMH):
 *
 *   double coef[4];                                  // stencil weights (global)
 *   int wl_cdvh2d_run(long n, long iters, unsigned long long seed,
 *                     double *eps_out, double *b_out) {
 *   #pragma dvm array distribute[block][block], shadow[1:1][1:1]
 *       double (*A)[n];
 *   #pragma dvm array align([i][j] with A[i][j]), shadow[1:1][1:1]
 *       double (*B)[n];
 *       double *w, eps;
 *       long i, j, it;
 *       A = malloc(n * n * sizeof(double));
 *       B = malloc(n * n * sizeof(double));
 *       w = malloc(n * sizeof(double));          // a weight per row
 *       coef[0] = 0.25; coef[1] = 0.125; coef[2] = 0.375; coef[3] = 0.25;
 *       for (i = 0; i < n; i++) w[i] = 0.5 + wl_u01(seed, 2, i) / 2.0;
 *       for (i = 0; i < n; i++)
 *           for (j = 0; j < n; j++) {
 *               A[i][j] = 0.0;
 *               B[i][j] = (i == 0 || j == 0 || i == n-1 || j == n-1) ? 0.0 : wl_u01(seed, 1, i*n+j);
 *           }
 *       for (it = 0; it < iters; it++) {
 *           eps = 0.0;
 *   #pragma dvm region
 *           {
 *   #pragma dvm parallel([i][j] on A[i][j]) reduction(max(eps))
 *               for (i = 1; i < n - 1; i++)
 *                   for (j = 1; j < n - 1; j++) {
 *                       eps = Max(fabs(B[i][j] - A[i][j]), eps);
 *                       A[i][j] = B[i][j];
 *                   }
 *   #pragma dvm parallel([i][j] on B[i][j]) shadow_renew(A)
 *               for (i = 1; i < n - 1; i++)
 *                   for (j = 1; j < n - 1; j++)
 *                       B[i][j] = w[i] * (coef[0] * A[i-1][j] + coef[1] * A[i][j-1]
 *                                         + coef[2] * A[i][j+1] + coef[3] * A[i+1][j]);
 *           }
 *   #pragma dvm get_actual(eps)
 *           eps_out[it] = eps;
 *       }
 *   #pragma dvm get_actual(B)
 *       for (i = 0; i < n; i++)
 *           for (j = 0; j < n; j++) b_out[i * n + j] = B[i][j];
 *       free(w);
 *       free(B);
 *       free(A);
 *       return 0;
 *   }
 */
#include <math.h>
#include <stdlib.h>

#include "dvmhlib2.h"
#include "wl_common.h"

#define dvm0c(n) ((DvmType)(n))
#define dvm0c0 dvm0c(0)
#define dvm0c1 dvm0c(1)
#define dvm0c2 dvm0c(2)

#define Max(a, b) ((a) > (b) ? (a) : (b))

#ifdef _OPENMP
#define OMP_HANDLER_TYPE (HANDLER_TYPE_MASTER | HANDLER_TYPE_PARALLEL)
#else
#define OMP_HANDLER_TYPE 0
#endif

/* Forward declaraions for the handlers for this file */
void loop_cdvh2d_c_110_host(DvmType *pLoopRef, DvmType A[], DvmType B[], double *eps);
void loop_cdvh2d_c_116_host(DvmType *pLoopRef, DvmType A[], DvmType B[], DvmType coef[], DvmType w[]);
#ifndef WL_NO_CUDA
void loop_cdvh2d_c_110_cuda(DvmType *pLoopRef, DvmType A[], DvmType B[], double *eps);
void loop_cdvh2d_c_116_cuda(DvmType *pLoopRef, DvmType A[], DvmType B[], DvmType coef[], DvmType w[]);
#endif

double coef[4];

void loop_cdvh2d_c_110_host(DvmType *pLoopRef, DvmType A[], DvmType B[], double *eps_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A[1]] = (double (*)[A[1]])dvmh_get_natural_base_C(device_num, A);
    double (*b)[B[1]] = (double (*)[B[1]])dvmh_get_natural_base_C(device_num, B);
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
                eps = Max(fabs(b[i][j] - a[i][j]), eps);
                a[i][j] = b[i][j];
            }
        dvmh_loop_red_post_C(loop_ref, 1, &eps, 0);
    }
}

void loop_cdvh2d_c_116_host(DvmType *pLoopRef, DvmType A[], DvmType B[], DvmType coef_hdr[], DvmType w_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double (*a)[A[1]] = (double (*)[A[1]])dvmh_get_natural_base_C(device_num, A);
    double (*b)[B[1]] = (double (*)[B[1]])dvmh_get_natural_base_C(device_num, B);
    double *coef = (double *)dvmh_get_natural_base_C(device_num, coef_hdr);
    double *w = (double *)dvmh_get_natural_base_C(device_num, w_hdr);
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
                b[i][j] = w[i] * (coef[0] * a[i - 1][j] + coef[1] * a[i][j - 1] + coef[2] * a[i][j + 1] +
                                  coef[3] * a[i + 1][j]);
    }
}

int wl_cdvh2d_run(long n, long iters, unsigned long long seed, double *eps_out, double *b_out) {
    dvmh_line_C(86, "cdvh2d.c");
#ifdef _OPENMP
    dvmh_init_lib_C(INITFLAG_OPENMP);
#else
    dvmh_init_lib_C(0);
#endif

    DvmType A[64];
    dvmh_array_declare_C(A, 2, -rt_DOUBLE, dvm0c0, dvm0c1, dvm0c1, dvm0c(n), dvm0c1, dvm0c1);
    DvmType B[64];
    dvmh_array_declare_C(B, 2, -rt_DOUBLE, dvm0c0, dvm0c1, dvm0c1, dvm0c(n), dvm0c1, dvm0c1);
    double *w, eps;
    long i, j, it;
    do {
        dvmh_line_C(93, "cdvh2d.c");
        dvmh_array_alloc_C(A, (n * n * sizeof(double)));
        dvmh_distribute_C(A, 2, dvmh_distribution_block_C(1), dvmh_distribution_block_C(2));
    } while (0);
    do {
        dvmh_line_C(94, "cdvh2d.c");
        dvmh_array_alloc_C(B, (n * n * sizeof(double)));
        dvmh_align_C(B, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
    } while (0);
    w = dvmh_malloc_C(n * sizeof(double));
    coef[0] = 0.25;
    coef[1] = 0.125;
    coef[2] = 0.375;
    coef[3] = 0.25;
    for (i = 0; i < n; i++) w[i] = 0.5 + wl_u01(seed, 2, (uint64_t)i) / 2.0;
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) {
            (dvmh_get_own_element_addr_C(A, 2, dvm0c(i), dvm0c(j)) ?
                 ((*(double *)dvmh_get_own_element_addr_C(A, 2, dvm0c(i), dvm0c(j))) = 0.0) : ((void)0));
            (dvmh_get_own_element_addr_C(B, 2, dvm0c(i), dvm0c(j)) ?
                 ((*(double *)dvmh_get_own_element_addr_C(B, 2, dvm0c(i), dvm0c(j))) =
                      (i == 0 || j == 0 || i == n - 1 || j == n - 1) ? 0.0 : wl_u01(seed, 1, (uint64_t)(i * n + j)))
                 : ((void)0));
        }
    for (it = 0; it < iters; it++) {
        eps = 0.0;
        {
            dvmh_line_C(106, "cdvh2d.c");
            dvmh_data_enter_C((const void *)coef, sizeof(coef));
            dvmh_data_enter_C((const void *)w, 0);
            DvmType cur_region = dvmh_region_create_C(0);
            DvmType cur_loop = 0;
            dvmh_region_register_array_C(cur_region, INTENT_IN | INTENT_OUT, A, "A");
            dvmh_region_register_array_C(cur_region, INTENT_IN | INTENT_OUT, B, "B");
            dvmh_region_register_array_C(cur_region, INTENT_IN,
                                         dvmh_variable_gen_header_C((const void *)coef, 1, -rt_DOUBLE, dvm0c(4)),
                                         "coef");
            dvmh_region_register_array_C(cur_region, INTENT_IN,
                                         dvmh_variable_gen_header_C((const void *)w, 1, -rt_DOUBLE, dvm0c0), "w");
            dvmh_region_execute_on_targets_C(cur_region, DEVICE_TYPE_HOST | DEVICE_TYPE_CUDA);

            dvmh_line_C(110, "cdvh2d.c");
            cur_loop = dvmh_loop_create_C(cur_region, 2, dvm0c1, dvm0c(n - 2), dvm0c1, dvm0c1, dvm0c(n - 2), dvm0c1);
            dvmh_loop_map_C(cur_loop, A, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
            dvmh_loop_reduction_C(cur_loop, rf_MAX, &eps, rt_DOUBLE, 1, 0, 0);
            dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                                         dvmh_handler_func_C((DvmHandlerFunc)loop_cdvh2d_c_110_host, 3, A, B, &eps));
#ifndef WL_NO_CUDA
            dvmh_loop_register_handler_C(cur_loop, DEVICE_TYPE_CUDA, 0,
                                         dvmh_handler_func_C((DvmHandlerFunc)loop_cdvh2d_c_110_cuda, 3, A, B, &eps));
#endif
            dvmh_loop_perform_C(cur_loop);
            cur_loop = 0;

            dvmh_line_C(116, "cdvh2d.c");
            dvmh_shadow_renew_C(A, 0, 0);
            cur_loop = dvmh_loop_create_C(cur_region, 2, dvm0c1, dvm0c(n - 2), dvm0c1, dvm0c1, dvm0c(n - 2), dvm0c1);
            dvmh_loop_map_C(cur_loop, B, 2, dvmh_alignment_linear_C(1, 1, 0), dvmh_alignment_linear_C(2, 1, 0));
            dvmh_loop_register_handler_C(
                cur_loop, DEVICE_TYPE_HOST, OMP_HANDLER_TYPE,
                dvmh_handler_func_C((DvmHandlerFunc)loop_cdvh2d_c_116_host, 4, A, B,
                                    dvmh_variable_get_header_C((const void *)coef),
                                    dvmh_variable_get_header_C((const void *)w)));
#ifndef WL_NO_CUDA
            dvmh_loop_register_handler_C(
                cur_loop, DEVICE_TYPE_CUDA, 0,
                dvmh_handler_func_C((DvmHandlerFunc)loop_cdvh2d_c_116_cuda, 4, A, B,
                                    dvmh_variable_get_header_C((const void *)coef),
                                    dvmh_variable_get_header_C((const void *)w)));
#endif
            dvmh_loop_perform_C(cur_loop);
            cur_loop = 0;

            dvmh_line_C(122, "cdvh2d.c");
            dvmh_region_end_C(cur_region);
            dvmh_data_exit_C((const void *)coef, 1);
            dvmh_data_exit_C((const void *)w, 1);
        }
        dvmh_line_C(123, "cdvh2d.c");
        dvmh_get_actual_variable2_((void *)&eps);

        eps_out[it] = eps;
    }
    dvmh_line_C(126, "cdvh2d.c");
    dvmh_get_actual_array2_(B);

    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) b_out[i * n + j] = (*(double *)dvmh_get_element_addr_C(B, 2, dvm0c(i), dvm0c(j)));
    dvmh_free_C(w);
    dvmh_line_C(131, "cdvh2d.c");
    dvmh_array_free_C(B);
    dvmh_line_C(132, "cdvh2d.c");
    dvmh_array_free_C(A);
    dvmh_forget_header_(B);
    dvmh_forget_header_(A);
    return 0;
}

/* the module's init and finish functions (the converter's tail, c_dvmh.cpp:204-210);
   the initialiser object that registers them is C++ (cdvh2d_init.cpp) */
void initCdvmhGlobals_cdvh2d_c(void) {
    dvmh_data_enter_C((const void *)coef, sizeof(coef));
}

void finishCdvmhGlobals_cdvh2d_c(void) {
    dvmh_data_exit_C((const void *)coef, 0);
}
