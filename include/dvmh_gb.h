/*
 * dvmh_gb.h -- entry points of libdvmh_gb.so that have no counterpart in the
 * reference's dvmhlib2.h: execution-mode control, loop batching/fusion rules
 * for generated CUDA handlers, runtime statistics, and the CUDA-block tuner.
 * Plain C, plain pointers and sizes.
 */
#ifndef DVMH_GB_H
#define DVMH_GB_H

#include "dvmhlib2.h"

#pragma GCC visibility push(default)
#ifdef __cplusplus
extern "C" {
#endif

/* ---- execution mode ------------------------------------------------------
 * 0 plain   : every loop launched when performed; reduction results written to
 *             the host variable with a stream synchronisation at loop end (the
 *             reference's model: DvmhLoopCuda::syncAfterHandlerExec,
 *             rts/dvmh/loop.cpp:2235-2240).
 * 1 async   : every loop launched when performed; reduction results stay on
 *             the device until get_actual; no per-loop synchronisation.
 * 2 batched : loops are queued and run at the next synchronisation point
 *             (get_actual, barrier, exit, dvmhgb_flush) as one CUDA graph that
 *             is cached by the queue's signature and replayed; fusion rules
 *             apply.  Default; environment DVMH_GB_MODE=plain|async|batched.
 * Changing the mode flushes queued work. */
void dvmhgb_set_mode(int mode);
int dvmhgb_get_mode(void);
void dvmhgb_flush(void);   /* run queued loops now (no host synchronisation) */
void dvmhgb_sync(void);    /* flush and wait for the GPU */

/* ---- fusion and batching rules for generated handlers ---------------------
 * A fusion rule says: when loop X with CUDA handler `first` is followed in the
 * queue by loop Y with handler `second` over the same region, run
 * fused(DvmType refs[2], <X's parameters>, <Y's parameters>) instead of the
 * two handlers.  The fused handler must compute exactly what X then Y compute.
 * A batch rule says: consecutive queued loops whose CUDA handler is `single`
 * and whose arrays are pairwise disjoint may run as one call of
 * batched(DvmType refs[], DvmType count); parameters of each loop are read
 * with dvmhgb_loop_param.  Both apply in batched mode only. */
void dvmhgb_register_fusion(DvmHandlerFunc first, DvmHandlerFunc second, DvmHandlerFunc fused);
void dvmhgb_register_batch(DvmHandlerFunc single, DvmHandlerFunc batched);
/* Deferred loops.  In batched mode a queued loop whose handler starts a fusion
 * rule, and whose parameters are all array descriptors (no variable, no other
 * address, no reduction), need not run when
 * a variable is read or written on the host or when its region ends: it waits
 * in the queue for the next loop, so that a time step's last loop and the next
 * step's first loop can meet in one flush (the region's end no longer forces
 * it: handler parameters that could die with the region are variables, and a
 * loop naming one is still run by then).  Every access to the loop's arrays,
 * freeing them, a mode change or dvmhgb_flush still runs it first.  On by
 * default; dvmhgb_set_deferral(0) or env DVMH_GB_DEFER=0 turns it off. */
void dvmhgb_set_deferral(int on);
void *dvmhgb_loop_param(DvmType loopRef, DvmType index);
/* Device base (natural base) of a second buffer with the same layout as the
 * array; when the loop ends the array's device buffer and this one swap. */
void *dvmhgb_loop_alt_buffer(DvmType loopRef, const DvmType dvmDesc[]);

/* Device scratch owned by this loop execution (pool memory; kept with a
 * captured graph, returned to the pool otherwise).  Contents undefined. */
void *dvmhgb_loop_scratch(DvmType loopRef, DvmType bytes);
/* Pinned host memory owned by this loop execution (for descriptor tables a
 * handler copies to the device on its stream); kept with a captured graph. */
void *dvmhgb_loop_host_scratch(DvmType loopRef, DvmType bytes);
/* Device address of the runtime's status word.  A kernel whose bounded wait
 * runs out writes a nonzero code there; the runtime reports it as a fatal
 * error at the next synchronisation. */
int *dvmhgb_status_word(void);

/* Kernel variant for this loop execution (0 <= result < nvariants): the
 * generated handler's alternatives -- here the number of FP64 operations per
 * cell executed on the FP64 unit rather than the integer pipe.  The tuner
 * chooses it with the CUDA block; `dflt` applies when tuning is off.
 * Environment DVMH_GB_VARIANT forces a value. */
int dvmhgb_loop_variant(DvmType loopRef, int nvariants, int dflt);
/* Force every later dvmhgb_loop_variant() to return v (clamped to the loop's
 * variant count); v < 0 restores tuning / defaults.  Overrides DVMH_GB_VARIANT. */
void dvmhgb_force_variant(int v);
/* dvmhgb_loop_variant with a description of each variant: desc[v * ndesc + d]
 * (ndesc <= DVMHGB_VARIANT_NDESC numbers per variant, the first one naming the
 * kernel family).  With model-guided tuning the runtime ranks the variants by
 * the variant model's predicted time for this loop and tries only the first
 * floor(0.1 x nvariants) of them (none: the model's first choice is taken as
 * it is); every timed execution is recorded with its features in the
 * runtime's variant database.  Exhaustive tuning tries every variant, as
 * dvmhgb_loop_variant does.  A variant counts as tried after two timed runs
 * (environment DVMH_GB_TUNE_REPS), its fastest kept; environment
 * DVMH_GB_TUNE_FRAC changes the 0.1.  In batched mode, flushes run without graph
 * capture while a loop's variants are being tried, then are captured with
 * the chosen one. */
#define DVMHGB_VARIANT_NDESC 16
int dvmhgb_loop_variant_desc(DvmType loopRef, int nvariants, int dflt, const float *desc, int ndesc);

/* Device layouts for ACROSS loops.  On (default; environment
 * DVMH_GB_AUTOTFM=0 turns it off), dvmh_loop_autotransform_C stores a loop's
 * array as the reference does: the array axis of the fastest independent loop
 * axis innermost (one dependence), or the two fastest dependent axes
 * numbered along the diagonal the loop sweeps (two or more).  Off, arrays
 * stay natural and autotransform reports 0.  Either way a device copy is
 * natural again before host copies and before any handler that did not ask
 * for the transform.  With tuning on (DVMH_OPT_PARAMS / dvmhgb_set_tuning),
 * the tuner times each loop shape with the transform and without (twice
 * each, in immediate execution) and keeps the faster. */
void dvmhgb_set_autotransform(int on);
int dvmhgb_get_autotransform(void);
/* The layout the tuner keeps for the latest loop shape of a handler: 0
 * natural, 1 transformed, -1 not yet measured both ways; best[0..1] (may be
 * null) = fastest seconds seen natural / transformed (-1 = none). */
int dvmhgb_tuner_layout(DvmHandlerFunc handler, double best[2]);
/* ACROSS dependences of loop axes with a single iteration: kept by default
 * (the reference's DVMH_REDUCE_DEPS=0); on (environment DVMH_REDUCE_DEPS=1),
 * such an axis gets no dependence bit unless no other axis has one. */
void dvmhgb_set_reduce_dependences(int on);
/* Online tuning of CUDA blocks, variants and layouts: 0 off, 1 exhaustive,
 * 2 model-guided (the same as DVMH_OPT_PARAMS at start-up). */
void dvmhgb_set_tuning(int mode);
/* Forget what the tuner learnt about variants and layouts (not its databases
 * or models). */
void dvmhgb_tuner_reset(void);
/* The variant tuning of each loop shape seen (index 0 .. count-1): the handler
 * that asked, its variant count, the variant kept (or about to be),
 * per-variant fastest seconds (-1 = never timed; best[] holds nvariants
 * entries, may be null), how many executions tried an untried variant and
 * their summed seconds (the tuning time).  0, or -1 for a bad index. */
long dvmhgb_tuner_variant_count(void);
/* 1 while some loop shape is still trying variants (its flushes run uncaptured) */
int dvmhgb_tuner_exploring(void);
int dvmhgb_tuner_variant_info(long index, DvmHandlerFunc *handler, int *nvariants, int *chosen, double *best,
                              int maxBest, int *explored, double *exploreSeconds);

/* Self-test of the integer-pipe FP64 operations against the FP64 unit on n
 * random operand pairs: mismatches[0..3] = add, sub, mul, division by 6. */
int dvmhgb_selftest_softfp64(long n, unsigned long long seed, long mismatches[4]);
/* Measured FP64 addition throughput of the current GPU (additions/s): the
 * FP64 roofline's denominator.  0 on success. */
int dvmhgb_fp64_add_rate(double *addsPerSecond);

/* ---- handler timing (the runtime's timing database) -----------------------
 * On: every handler execution is bracketed by CUDA events on the runtime
 * stream (recorded inside captured graphs too) and accumulated per handler at
 * each synchronisation.  dvmhgb_timing_get returns the total milliseconds and
 * the number of executions recorded for a handler (0 on success, -1 if none). */
void dvmhgb_set_timing(int on);
int dvmhgb_timing_get(DvmHandlerFunc handler, double *totalMs, long *count);
void dvmhgb_timing_reset(void);

/* ---- statistics --------------------------------------------------------- */
typedef struct {
    long loops_performed;   /* dvmh_loop_perform_C calls */
    long handler_calls;     /* CUDA handler invocations (captures count once) */
    long fused_pairs;       /* fusion-rule applications */
    long batched_groups;    /* batch-rule applications */
    long graphs_captured;
    long graph_replays;
    long flushes;
    long h2d_bytes, d2h_bytes;
    long kernel_launches;   /* launches issued by this library's launchers */
    long relayouts;         /* device copies moved between layouts (autotransform) */
} dvmhgb_stats_t;
void dvmhgb_get_stats(dvmhgb_stats_t *out);
void dvmhgb_reset_stats(void);
/* Launch counter, incremented by every launcher of this library (also the
 * kernels inside captured graphs, once per replay). */
void dvmhgb_count_launches(long n);

/* Host profile of the ABI entry points (DVMH_GB_HOSTPROF=1): calls and
 * inclusive wall time per entry point, printed to stderr at exit or now. */
void dvmhgb_hostprof_dump(void);
void dvmhgb_hostprof_reset(void);

/* Stream the runtime launches on (a cudaStream_t). */
void *dvmhgb_stream(void);

/* The CUDA block that dvmh_loop_cuda_get_config_C hands a handler, as a pure
 * function of the loop and the device's limits (the reference's
 * DvmhLoopCuda::pickBlock, rts/dvmh/loop.cpp:2134-2199, and its default
 * blocks, loop.cpp:1464-1485): the user's block (userBlock != 0) or the given
 * one (block[] >= 1) or the default for min(3, rank - (hasDeps != 0)) block
 * dimensions; then a block needing more shared memory (sharedPerThread per
 * thread) or registers (regsPerThread, 0 = the device's maximum per thread)
 * than one block can have is shrunk to one dimension of
 * max(1, roundDown(min(256, have / perThread), warpSize)) threads (1 for a
 * loop with no free block dimension).  Returns 0 with block[] set, or a user
 * error the reference reports: 1 more block dimensions than the loop has (one
 * fewer with dependences), 2 an axis above the device's limit, 3 more threads
 * than a block can have, 4 / 5 shared memory / registers insufficient for a
 * block the user fixed. */
typedef struct {
    int maxBlockSize[3];
    int maxThreadsPerBlock;
    long sharedPerBlock;   /* cudaDeviceProp::sharedMemPerBlock */
    long regsPerBlock;     /* cudaDeviceProp::regsPerBlock */
    int warpSize;
    int maxRegsPerThread;  /* 255 */
} dvmhgb_cuda_limits_t;
int dvmhgb_pick_block(int loopRank, int hasDeps, int userBlock, int block[3], long sharedPerThread,
                      long regsPerThread, const dvmhgb_cuda_limits_t *limits);

#ifdef __cplusplus
}
#endif
#pragma GCC visibility pop

#endif
