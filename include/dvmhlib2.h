/*
 * dvmhlib2.h -- C ABI of the GB300 loop-execution runtime (libdvmh_gb.so).
 *
 * This header declares the part of the DVMH runtime's C interface that
 * cdvmh-generated main code and loop handlers call on the parallel-loop path:
 * init/exit, distributed arrays, regions, actuality, shadow renew, parallel
 * loops (create/map/reduction/across/cuda_block/handlers/perform) and the
 * in-handler queries (bounds, CUDA config, reduction buffers).  Every entry
 * point keeps the reference's name, argument order, argument meaning and
 * varargs layout, so generated code compiles against this header and links
 * against this library unchanged.  Each declaration cites the reference
 * declaration it replaces (rts/dvmh/include/dvmhlib2.h:<line> unless noted).
 *
 * Errors keep the reference's observable convention: a user error prints a
 * message and exits with status 1; an internal inconsistency aborts
 * (rts/dvmh/dvmh_log.h:75-100).
 *
 * Device numbering follows the reference: device 0 is the host, device 1 is
 * the GPU.  Loops inside a region that targets CUDA run on the GPU only;
 * there is no host execution of parallel loops in this library.
 */
#ifndef DVMHLIB2_H
#define DVMHLIB2_H

#include <stdlib.h>

/* ---- types (rts/dvmh/include/dvmhlib_types.h:9-18) ---- */
#if defined(_WIN64)
typedef long long DvmType;
#else
typedef long DvmType;
#endif
#ifdef __cplusplus
typedef int (*DvmHandlerFunc)(...);
#else
typedef int (*DvmHandlerFunc)();
#endif

/* ---- constants: values are part of the ABI (rts/dvmh/include/dvmhlib_const.h:8-72) ---- */
#define INITFLAG_FORTRAN 1
#define INITFLAG_NOH 2
#define INITFLAG_SEQUENTIAL 4
#define INITFLAG_OPENMP 8
#define INITFLAG_DEBUG 16

#define rt_UNKNOWN (-1)
#define rt_CHAR 0
#define rt_INT 1
#define rt_LONG 2
#define rt_FLOAT 3
#define rt_DOUBLE 4
#define rt_FLOAT_COMPLEX 5
#define rt_DOUBLE_COMPLEX 6
#define rt_LOGICAL 7
#define rt_LLONG 8
#define rt_UCHAR 9
#define rt_UINT 10
#define rt_ULONG 11
#define rt_ULLONG 12
#define rt_SHORT 13
#define rt_USHORT 14
#define rt_POINTER 15

#define REGION_ASYNC 1
#define REGION_COMPARE_DEBUG 2

#define INTENT_IN 1
#define INTENT_OUT 2
#define INTENT_LOCAL 4
#define INTENT_INOUT 3
#define INTENT_INLOCAL 5
#define INTENT_USE 8

#define UNDEF_BOUND (-2147483648LL)

#define DEVICE_TYPE_HOST 1
#define DEVICE_TYPE_CUDA 2

#define HANDLER_TYPE_PARALLEL 1
#define HANDLER_TYPE_MASTER 2

#define rf_SUM 1
#define rf_PROD 2
#define rf_MULT 2
#define rf_MAX 3
#define rf_MIN 4
#define rf_AND 5
#define rf_OR 6
#define rf_XOR 7
#define rf_EQU 8
#define rf_NE 9
#define rf_EQ 10
#define rf_MAXLOC 11
#define rf_MINLOC 12

#pragma GCC visibility push(default)
#ifdef __cplusplus
extern "C" {
#endif

/* ---- init / exit ---- */
void dvmh_line_C(DvmType lineNumber, const char fileName[]);                 /* :19 */
void dvmh_init_C(DvmType flags, int *pArgc, char ***pArgv);                  /* :22 */
void dvmh_exit_C(DvmType exitCode);                                          /* :26 */
/* a translation unit other than main's: initialises once, later calls are ignored */
void dvmh_init_lib_C(DvmType flags);                                         /* :24 */
void dvmh_init_lib_(const DvmType *pFlags);                                  /* :25 */

/* ---- distributed arrays and templates ---- */
/* varargs: {axisSize, shadowLow, shadowHigh} x rank; typeSize < 0 means -rt_TYPE */
void dvmh_array_create_C(DvmType dvmDesc[], DvmType rank, DvmType typeSize, ...);          /* :30 */
void dvmh_template_create_C(DvmType dvmDesc[], DvmType rank, ...);                         /* :33 */
/* varargs: nParams handler parameters (pointers / descriptors) */
DvmType dvmh_handler_func_C(DvmHandlerFunc handlerFunc, DvmType customParamCount, ...);    /* :37 */
DvmType dvmh_distribution_replicated_(void);                                               /* :46 */
DvmType dvmh_distribution_block_C(DvmType mpsAxis);                                        /* :47 */
/* varargs: rank distribution helpers */
void dvmh_distribute_C(DvmType dvmDesc[], DvmType rank, ...);                              /* :61 */
void dvmh_redistribute_C(DvmType dvmDesc[], DvmType rank, ...);                            /* :63 */
DvmType dvmh_alignment_linear_C(DvmType axis, DvmType multiplier, DvmType summand);        /* :65 */
/* varargs: templRank alignment helpers */
void dvmh_align_C(DvmType dvmDesc[], const DvmType templDesc[], DvmType templRank, ...);   /* :67 */
void dvmh_array_free_C(DvmType dvmDesc[]);                                                 /* :77 */
void dvmh_delete_object_(DvmType dvmDesc[]);                                               /* :78 */
/* dynamic arrays: declared with the first size unknown (0), then allocated with
 * byteCount bytes (the first size = byteCount / (element size x other sizes)) */
void dvmh_array_declare_C(DvmType dvmDesc[], DvmType rank, DvmType typeSize, ...);         /* :29 */
void dvmh_array_alloc_C(DvmType dvmDesc[], DvmType byteCount);                             /* :35 */
void dvmh_forget_header_(DvmType dvmDesc[]);                                               /* :79 */

/* ---- regular (non-distributed) variables: data regions and their headers ---- */
/* varargs: rank axis sizes (the first may be 0 for an incomplete array) */
DvmType *dvmh_variable_gen_header_C(const void *addr, DvmType rank, DvmType typeSize, ...); /* :81 */
DvmType *dvmh_variable_get_header_C(const void *addr);                                     /* :86 */
void dvmh_data_enter_C(const void *addr, DvmType size);                                    /* :87 */
void dvmh_data_enter_(const void *addr, const DvmType *pSize);                             /* :88 */
void dvmh_data_exit_C(const void *addr, DvmType saveFlag);                                 /* :89 */
void dvmh_data_exit_(const void *addr, const DvmType *pSaveFlag);                          /* :90 */
void *dvmh_malloc_C(size_t size);                                                          /* :91 */
void *dvmh_calloc_C(size_t nmemb, size_t size);                                            /* :92 */
void *dvmh_realloc_C(void *ptr, size_t size);                                              /* :93 */
char *dvmh_strdup_C(const char *s);                                                        /* :94 */
void dvmh_free_C(void *ptr);                                                               /* :95 */

/* ---- addresses and headers ---- */
void *dvmh_get_natural_base_C(DvmType deviceNum, const DvmType dvmDesc[]);                 /* :103 */
void *dvmh_get_device_addr_C(DvmType deviceNum, const void *addr);                         /* :104 */
DvmType dvmh_fill_header_C(DvmType deviceNum, const void *baseAddr, const DvmType dvmDesc[],
                           DvmType devHeader[], DvmType extendedParams[]);                 /* :105 */
/* varargs: rank global indexes */
DvmType dvmh_calc_linear_C(const DvmType dvmDesc[], DvmType rank, ...);                    /* :137 */
void *dvmh_get_element_addr_C(const DvmType dvmDesc[], DvmType rank, ...);                 /* :140 */
/* the element's address if this process owns it, else NULL (one process owns all) */
void *dvmh_get_own_element_addr_C(const DvmType dvmDesc[], DvmType rank, ...);             /* :139 */

/* ---- actuality ---- */
void dvmh_get_actual_variable2_(void *addr);                                               /* :111 */
/* varargs: {indexLow, indexHigh} x rank; UNDEF_BOUND means the array bound */
void dvmh_get_actual_subarray_C(const DvmType dvmDesc[], DvmType rank, ...);               /* :112 */
void dvmh_get_actual_array2_(const DvmType dvmDesc[]);                                     /* :114 */
void dvmh_get_actual_all2_(void);                                                          /* :115 */
void dvmh_actual_variable2_(const void *addr);                                             /* :119 */
void dvmh_actual_subarray_C(const DvmType dvmDesc[], DvmType rank, ...);                   /* :120 */
void dvmh_actual_array2_(const DvmType dvmDesc[]);                                         /* :122 */
void dvmh_actual_all2_(void);                                                              /* :123 */

/* ---- shadow edges ---- */
/* varargs: {shadowLow, shadowHigh} x specifiedRank (0 = full declared widths) */
void dvmh_shadow_renew_C(const DvmType dvmDesc[], DvmType cornerFlag, DvmType specifiedRank, ...); /* :125 */

/* ---- regions ---- */
DvmType dvmh_region_create_C(DvmType regionFlags);                                         /* :142 */
void dvmh_region_register_subarray_C(DvmType curRegion, DvmType intent, const DvmType dvmDesc[],
                                     const char varName[], DvmType rank, ...);             /* :144 */
void dvmh_region_register_array_C(DvmType curRegion, DvmType intent, const DvmType dvmDesc[],
                                  const char varName[]);                                   /* :148 */
void dvmh_region_register_scalar_C(DvmType curRegion, DvmType intent, const void *addr,
                                   DvmType typeSize, const char varName[]);                /* :150 */
void dvmh_region_execute_on_targets_C(DvmType curRegion, DvmType deviceTypes);             /* :152 */
void dvmh_region_end_C(DvmType curRegion);                                                 /* :154 */

/* ---- parallel loops ---- */
/* varargs: {start, end, step} x rank; bounds inclusive, steps signed */
DvmType dvmh_loop_create_C(DvmType curRegion, DvmType rank, ...);                          /* :157 */
/* varargs: templRank alignment helpers */
void dvmh_loop_map_C(DvmType curLoop, const DvmType templDesc[], DvmType templRank, ...);   /* :159 */
void dvmh_loop_set_cuda_block_C(DvmType curLoop, DvmType xSize, DvmType ySize, DvmType zSize); /* :161 */
void dvmh_loop_set_stage_C(DvmType curLoop, DvmType stage);                                /* :163 */
void dvmh_loop_reduction_C(DvmType curLoop, DvmType redType, void *arrayAddr, DvmType varType,
                           DvmType arrayLength, void *locAddr, DvmType locSize);           /* :165 */
/* varargs: {shadowLow, shadowHigh} x rank */
void dvmh_loop_across_C(DvmType curLoop, DvmType isOut, const DvmType dvmDesc[], DvmType rank, ...); /* :168 */
void dvmh_loop_shadow_compute_C(DvmType curLoop, const DvmType templDesc[], DvmType specifiedRank, ...); /* :170 */
void dvmh_loop_register_handler_C(DvmType curLoop, DvmType deviceType, DvmType handlerType,
                                  DvmType handlerHelper);                                  /* :181 */
void dvmh_loop_perform_C(DvmType curLoop);                                                 /* :183 */

/* ---- queries from inside a handler (curLoop = the handler's loop reference) ---- */
DvmType dvmh_loop_get_dependency_mask_C(DvmType curLoop);                                  /* :185 */
DvmType dvmh_loop_get_device_num_C(DvmType curLoop);                                       /* :187 */
DvmType dvmh_loop_autotransform_C(DvmType curLoop, DvmType dvmDesc[]);                     /* :189 */
void dvmh_loop_fill_bounds_C(DvmType curLoop, DvmType boundsLow[], DvmType boundsHigh[],
                             DvmType loopSteps[]);                                         /* :191 */
DvmType dvmh_loop_get_slot_count_C(DvmType curLoop);                                       /* :193 */
/* part[2*i], part[2*i+1]: the array's local part on axis i+1 on the handler's device */
void dvmh_loop_fill_local_part_C(DvmType curLoop, const DvmType dvmDesc[], DvmType part[]);  /* :195 */
DvmType dvmh_loop_guess_index_type_C(DvmType curLoop);                                     /* :197 */
void dvmh_loop_cuda_register_red_C(DvmType curLoop, DvmType redIndex, void **arrayAddrPtr,
                                   void **locAddrPtr);                                     /* :202 */
void dvmh_loop_red_init_C(DvmType curLoop, DvmType redIndex, void *arrayAddr, void *locAddr); /* :203 */
void dvmh_loop_cuda_red_init_C(DvmType curLoop, DvmType redIndex, void **devArrayAddrPtr,
                               void **devLocAddrPtr);                                      /* :205 */
/* inOutThreads points to a dim3, outStream to a cudaStream_t */
void dvmh_loop_cuda_get_config_C(DvmType curLoop, DvmType sharedPerThread, DvmType regsPerThread,
                                 void *inOutThreads, void *outStream,
                                 DvmType *outSharedPerBlock);                              /* :206 */
void dvmh_loop_cuda_red_prepare_C(DvmType curLoop, DvmType redIndex, DvmType count,
                                  DvmType fillFlag);                                       /* :208 */
void dvmh_loop_cuda_red_finish_C(DvmType curLoop, DvmType redIndex);                       /* :211 */
void dvmh_loop_red_post_C(DvmType curLoop, DvmType redIndex, const void *arrayAddr,
                          const void *locAddr);                                            /* :212 */
void dvmh_change_filled_bounds_C(DvmType boundsLow[], DvmType boundsHigh[], DvmType loopSteps[],
                                 DvmType rank, DvmType depMask, DvmType idxPerm[]);        /* :229 */
void dvmh_change_filled_bounds2_C(DvmType boundsLow[], DvmType boundsHigh[], DvmType loopSteps[],
                                  DvmType rank, DvmType depMask, DvmType idxPerm[]);       /* :230 */

/* ---- misc (rts/dvmh/include/dvmh_runtime_api.h:14,35) ---- */
void dvmh_barrier(void);
double dvmh_wtime(void);

#ifdef __cplusplus
}

/* The module initialiser cdvmh emits for a translation unit with global
 * regular variables (cdvmh/src/c_dvmh.cpp:204-222): its init function (data
 * enter of the globals) runs when the runtime initialises, or at once if it
 * already has; its finish function at dvmh_exit_C.  Same class layout and
 * member signatures as the reference's, so generated code links unchanged.  (:236-247) */
class DvmhModuleInitializer {
public:
    explicit DvmhModuleInitializer(void (*fInit)(), void (*fFinish)() = 0);
    static void executeInit();
    static void executeFinish();
protected:
    static DvmhModuleInitializer *head;
    DvmhModuleInitializer *next;
    void (*funcInit)();
    void (*funcFinish)();
};
#endif
#pragma GCC visibility pop

#endif
