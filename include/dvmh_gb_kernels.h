/*
 * dvmh_gb_kernels.h -- launchers of the hand-written sm_103a loop kernels in
 * libdvmh_gb.so.  These are what cdvmh would emit as the body of a CUDA
 * handler (cdvmh/src/converter_main.cpp:1861-2401 for parallel loops,
 * cdvmh/src/across.cpp for ACROSS loops): the workload programs' CUDA
 * handlers call them after the dvmh_loop_* queries.
 *
 * Conventions: arrays are device natural bases (element (i,j,k) at
 * base[i*st[0] + j*st[1] + k*st[2]], strides in elements as returned by
 * dvmh_fill_header_C for device 1); lo/hi are the loop's inclusive bounds
 * (step 1); ext is the array extent per axis; stream is a cudaStream_t.
 * Reduction launchers write `items` partial values that
 * dvmh_loop_cuda_red_finish_C folds: *_items() gives the count to prepare.
 * `native` (0..ops per cell): how many of a cell's FP64 additions/subtractions
 * run on the FP64 unit; the others run bit-identically on the integer pipe
 * (GB300 issues 2 FP64 thread-ops per clock per SM against 128 integer ones).
 * Every launcher returns 0, or -1 on invalid arguments (nothing launched).
 */
#ifndef DVMH_GB_KERNELS_H
#define DVMH_GB_KERNELS_H

#pragma GCC visibility push(default)
#ifdef __cplusplus
extern "C" {
#endif

/* ---- Jacobi 3-D (examples/Performance/jac3d_perf.c:56-73, FP64) ---- */
/* loop 1: eps = max |B-A|, A = B over the box; MAX partials, one per CTA.
 * native: 0 = |B-A| on the integer pipe (general), 1 = on the FP64 unit, 2 =
 * exact 64-bit fixed point for values in [2^-12, 1) (FP64 unit otherwise) */
long dvmhgb_jac3d_update_items(const long lo[3], const long hi[3]);
int dvmhgb_jac3d_update(double *A, const double *B, const long st[3], const long lo[3], const long hi[3],
                        double *items, int native, void *stream);
/* loop 2: B = (A[i-1]+A[j-1]+A[k-1]+A[k+1]+A[j+1]+A[i+1]) / 6 over the box.
 * Variants (stencil and fused alike): v = 0..11: v = 6 * (rows per thread - 1)
 * + N, N = 0..5 additions of a cell on the FP64 unit (the others on the integer
 * pipe when the CTA's inputs are all +0 or positive normal, else all native);
 * v = 12, 13: all native, one row per thread, registers capped for 3 / 4 CTAs
 * per SM; v = 14..21: the sums in 61-bit fixed point on the integer pipe
 * (planes whose neighbourhood holds a value outside +0 and [2^-9, 1) on the
 * FP64 unit), with a share of the CTAs computing natively so that the FP64
 * unit works beside the integer pipe -- (CTAs per SM, native CTAs of every
 * den): 14 (4, 0/1), 15 (3, 0/1), 16 (4, 1/2), 17 (4, 1/3), 18 (4, 2/5),
 * 19 (3, 1/2), 20 (4, 1/4), 21 (4, 3/5); v = 22, 23: the fixed-point sums
 * with the source planes staged in shared memory by TMA box copies, a ring of
 * 6 / 4 planes per CTA (a copy that does not land within 2 s
 * writes DVMHGB_ERR_TMA_TIMEOUT to dvmhgb_status_word() and the CTA stops);
 * v = 24, 25, 26: ring of 6, with 1, 2, 3 of the CTA's 8 warps computing their
 * cells on the FP64 unit (division by 6 as one multiply and two FMAs);
 * -1 for v outside 0..DVMHGB_JAC3D_VARIANTS-1 */
#define DVMHGB_JAC3D_VARIANTS 27
#define DVMHGB_ERR_TMA_TIMEOUT 0x544D4101
int dvmhgb_jac3d_stencil(const double *A, double *B, const long st[3], const long ext[3], const long lo[3],
                         const long hi[3], int native, void *stream);
/* loops 1+2 fused (same box): reads A, B; writes A = B and Bnew = stencil(A_new)
 * into Bnew (a second buffer of B's layout), B's values outside the box copied
 * into Bnew; MAX partials, one per CTA (the count depends on the variant).
 * Variants 0..13 as above (one pass), 14..26 the update kernel and then the
 * fixed-point stencil of that variant, and DVMHGB_JAC3D_UNFUSED: the update
 * and the stencil kernels (variant 13) one after the other (Bnew may then be B
 * itself: the stencil reads only A; the one-pass variants reject Bnew == B) */
#define DVMHGB_JAC3D_UNFUSED DVMHGB_JAC3D_VARIANTS
/* DVMHGB_JAC3D_OVERLAP: the pair in 8 chunks of planes, the updates on
 * `stream`, the stencils on a second stream of the library (stencil chunk k
 * after update chunk k+1), joined back into `stream`, so that the HBM-bound
 * update runs beside the FP64-bound stencil; Bnew must be B */
#define DVMHGB_JAC3D_OVERLAP (DVMHGB_JAC3D_VARIANTS + 1)
/* DVMHGB_JAC3D_OVERLAP_Q: the same with the fixed-point stencil (variant 14) */
#define DVMHGB_JAC3D_OVERLAP_Q (DVMHGB_JAC3D_VARIANTS + 2)
/* DVMHGB_JAC3D_FUSED_Q (+ 1): the two loops in one pass with the fixed-point
 * sums (32 bytes per cell), registers capped for 4 (3) CTAs per SM; the update
 * of a plane is done as its values arrive; Bnew must not be B */
#define DVMHGB_JAC3D_FUSED_Q (DVMHGB_JAC3D_VARIANTS + 3)
/* DVMHGB_JAC3D_FUSED_T (+ 1): the two loops in one pass with the fixed-point
 * sums and the planes of B (A outside the box) and A's own cells staged by TMA
 * box copies, a ring of 5 (4) planes per CTA; Bnew must not be B */
#define DVMHGB_JAC3D_FUSED_T (DVMHGB_JAC3D_VARIANTS + 5)
#define DVMHGB_JAC3D_FUSED_VARIANTS (DVMHGB_JAC3D_VARIANTS + 7)
long dvmhgb_jac3d_fused_items(const long lo[3], const long hi[3], int native);
/* The other pairing of the same loops, across a time-step boundary: step n's
 * stencil loop B = (6 neighbours of A) / 6 followed by step n+1's update loop
 * eps = Max(|B - A|, eps); A = B over the same box.  B is written in place,
 * the new A into Aalt (a second buffer of A's layout, to become A: A is still
 * read while the pass runs; A's cells outside the box are copied over), MAX
 * partials into items (dvmhgb_jac3d_stnupd_items).  24 bytes a cell.  The
 * TMA-staged fixed-point stencil; variants (warps of 8 on the FP64 unit, warps
 * taking |B - A| as exact fixed-point differences on the integer pipe, the
 * rest on the FP64 unit): 0 (0, 0), 1 (1, 0), 2 (2, 0), 3 (1, 2), 4 (1, 4),
 * 5 (2, 3).  The runtime pairs the loops so when a program's time steps leave
 * the stencil queued past the step's end (deferred loops, dvmh_gb.h). */
#define DVMHGB_JAC3D_STNUPD_VARIANTS 6
long dvmhgb_jac3d_stnupd_items(const long lo[3], const long hi[3], int variant);
int dvmhgb_jac3d_stnupd(const double *A, double *Aalt, double *B, const long st[3], const long ext[3],
                        const long lo[3], const long hi[3], double *items, int variant, void *stream);
int dvmhgb_jac3d_fused(double *A, const double *B, double *Bnew, const long st[3], const long ext[3],
                       const long lo[3], const long hi[3], double *items, int native, void *stream);

/* ---- Jacobi 2-D (examples/Jacobi/jac2d.c:49-64, FP64) ---- */
long dvmhgb_jac2d_update_items(const long lo[2], const long hi[2]);
int dvmhgb_jac2d_update(double *A, const double *B, const long st[2], const long lo[2], const long hi[2],
                        double *items, int native, void *stream);
int dvmhgb_jac2d_stencil(const double *A, double *B, const long st[2], const long ext[2], const long lo[2],
                         const long hi[2], int native, void *stream);
long dvmhgb_jac2d_fused_items(const long lo[2], const long hi[2]);
int dvmhgb_jac2d_fused(double *A, const double *B, double *Bnew, const long st[2], const long ext[2],
                       const long lo[2], const long hi[2], double *items, int native, void *stream);

/* ---- SOR 3-D ACROSS (1:1,1:1,1:1), FP64: one sweep as a persistent tiled
 * wavefront of 4 x 8 x TK tiles, TK = 32, 16, 8 for variant 0, 1, 2, or
 * (variant 3) as 4 x 8-row columns streamed along k by one warp each, or
 * (variants 4, 5) as tiles cut along the hyperplanes i + j + k, 8
 * hyperplanes each, of 4 x 8 rows per warp (4) or 16 x 8 rows per CTA (5)
 * (a first launch lists the tiles); items = canonical partials of SUM
 * (nv-old)^2, one per row and TK-wide part of each 64-wide chunk (row, chunk,
 * part order; TK = 8 for variants 4, 5; one per row and chunk for variant 3);
 * wDev = device address of omega; scratch = dvmhgb_sor3d_scratch_bytes()
 * bytes; status = dvmhgb_status_word().  -1 for an unknown variant or invalid
 * arguments ---- */
#define DVMHGB_SOR3D_VARIANTS 6
long dvmhgb_sor3d_items(const long lo[3], const long hi[3], int variant);
long dvmhgb_sor3d_scratch_bytes(const long lo[3], const long hi[3], int variant);
int dvmhgb_sor3d_sweep(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3],
                       const double *wDev, double *items, void *scratch, int *status, int variant, void *stream);
/* The same sweep with its bounded waits made explicit.  Every wait for a
 * predecessor tile (column, variant 3) polls at most pollLimit times
 * (dvmhgb_sor3d_sweep: 2^24, about 1-4 s) before the kernel writes its timeout
 * code 0x50520001 to *status, sets the top bit of the hand-out counter (the
 * first word of scratch) so that no warp takes another tile, and returns; the
 * runtime reports a non-zero status word at its next synchronisation (exit
 * status 1).  firstIndex > 0 starts the hand-out at that tile: the tiles
 * before it are left to nobody, so their successors' waits run out -- how the
 * tests make a wait expire without a fault.  -1 for pollLimit < 1 or a
 * negative firstIndex. */
int dvmhgb_sor3d_sweep_bounded(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3],
                               const double *wDev, double *items, void *scratch, int *status, int variant,
                               void *stream, long pollLimit, long firstIndex);

/* ---- explicit 2-D heat step, FP64 (workloads/heat.c), with SUM and MINLOC:
 * per (row, 64-wide chunk) unit one SUM item (canonical pairwise tree), one
 * MINLOC value item and its location {i, j} (two ints).  The kernels walk
 * strips of sr rows of one chunk; dvmhgb_heat (one loop) shortens the strips
 * until they fill the GPU ---- */
#define DVMHGB_HEAT_STRIP 64
typedef struct {
    const double *src;
    double *dst;
    long s0;                 /* row stride of src and dst (elements, even) */
    long lo0, hi0, lo1, hi1; /* loop box */
    const double *coef;      /* device address of c */
    long c0, nck, units, unitBase;
    long sr;                 /* rows per strip (dvmhgb_heat_desc_fill: DVMHGB_HEAT_STRIP) */
    long strips, stripBase;  /* strips of this loop; prefix over a table (dvmhgb_heat_many) */
    double *sumItems, *minItems;
    int *locItems;
} dvmhgb_heat_desc;
int dvmhgb_heat_desc_fill(dvmhgb_heat_desc *d, const double *src, double *dst, long rowStride, const long lo[2],
                          const long hi[2], const double *coefDev);
int dvmhgb_heat(const dvmhgb_heat_desc *d, void *stream);
/* dDev: device array of n descriptors with unitBase / stripBase = prefix sums of
 * units / strips; totalStrips = the sum of strips */
int dvmhgb_heat_many(const dvmhgb_heat_desc *dDev, int n, long totalStrips, void *stream);
/* The strip geometry of the batched step, a tuner choice (results do not depend
 * on it: a strip's SUM and MINLOC items are per (row, chunk) whatever the
 * strip): variant v walks strips of DVMHGB_HEAT_ROWS(v) rows with a persistent
 * grid of DVMHGB_HEAT_CTAS(v) CTAs of 8 warps per SM.  dvmhgb_heat_desc_rows
 * sets a descriptor's rows per strip (and its strip count); -1 for sr < 1. */
#define DVMHGB_HEAT_VARIANTS 10
#define DVMHGB_HEAT_DEFAULT 2
#define DVMHGB_HEAT_ROWS(v) (16L << ((v) % 5))
#define DVMHGB_HEAT_CTAS(v) ((v) < 5 ? 8 : 4)
int dvmhgb_heat_desc_rows(dvmhgb_heat_desc *d, long sr);
int dvmhgb_heat_many_grid(const dvmhgb_heat_desc *dDev, int n, long totalStrips, int ctasPerSm, void *stream);

/* ---- no counterpart in the reference: the Jacobi-3D update loop for callers
 * that cannot allocate device memory (inside a stream capture in global mode,
 * under a host allocator that owns the whole GPU, on a path that must not
 * block in the driver).  Same work as dvmhgb_jac3d_update with native = 1,
 * then eps = max |B - A| over the box is written to epsDev (one double in
 * device memory).  Partial maxima go to a file-scope static __device__ array
 * of 4096 doubles (32 KB, held by every GPU that loads the library until the
 * process exits), not to a caller buffer: nothing is allocated and no
 * allocating library routine is called.  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept for
 * the life of the process: after cudaDeviceReset the array lives at a new
 * address, so a process that resets a device must not call this entry point
 * on that device again.  All calls share the array: calls whose GPU work
 * overlaps in time race.  Returns 0; -1 invalid
 * arguments; -2 the launch would need more than 4096 partial slots (message
 * on stderr); -3 CUDA error. ---- */
int dvmhgb_jac3d_update_noalloc(double *A, const double *B, const long st[3], const long lo[3], const long hi[3],
                                double *epsDev, void *stream);

/* ---- synthetic parallel loops (the tuner's training and evaluation set):
 * rank 1..4 star stencil of radius 0..3 over float/double/int arrays padded
 * by the radius, optional SUM/MAX/MINLOC reduction (1/2/3; one partial per
 * CTA into items, MINLOC offsets into locs), optional ACROSS on the outermost
 * axis; launch configuration = candidate (block, axis on x, elements per
 * thread) ---- */
typedef struct {
    int rank, radius, across, red, esize, isint;
    long ext[4];
} dvmhgb_synth_loop;
typedef struct {
    int bx, by, bz, xinner, ept;
} dvmhgb_synth_cand;
long dvmhgb_synth_elems(const dvmhgb_synth_loop *L);
long dvmhgb_synth_items(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C);
int dvmhgb_synth_run(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, const void *in, void *out, void *items,
                     long *locs, void *stream);

/* ---- the tuner's cost model: 3-layer FP32 MLP, DVMHGB_TUNE_NF -> 128 -> 128 -> 1
 * (ReLU), parameters packed W1,b1,W2,b2,W3,b3; trained on the GPU by these
 * kernels (MSE of log-time, Adam) ---- */
#define DVMHGB_TUNE_NF 24
long dvmhgb_mlp_nparams(void);
long dvmhgb_mlp_work_floats(long n);
int dvmhgb_mlp_init(float *params, unsigned long long seed, void *stream);
int dvmhgb_mlp_forward(const float *params, const float *X, long n, float *pred, float *work, void *stream);
int dvmhgb_mlp_loss_grad(const float *params, const float *X, const float *y, long n, float *grad, float *loss,
                         float *work, void *stream);
int dvmhgb_mlp_adam(float *params, const float *grad, float *m, float *v, long step, float lr, void *stream);
int dvmhgb_mlp_train(const float *X, const float *y, long n, int epochs, long batch, float lr,
                     unsigned long long seed, float *params, float *losses);

/* ---- the tuner (runtime): candidates and features of a synthetic loop, its
 * timing (recorded in the runtime's timing database), database export, and
 * ranking by the installed cost model ---- */
int dvmhgb_tuner_candidates(const dvmhgb_synth_loop *L, dvmhgb_synth_cand *out, int maxOut);
void dvmhgb_tuner_features(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, float *f);
double dvmhgb_tuner_time_synth(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, long loopId, int cand, int reps);
int dvmhgb_tuner_time_synth_all(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *cands, int n, long loopId,
                                int reps, double *times);
long dvmhgb_tuner_db_size(void);
long dvmhgb_tuner_db_export(float *X, double *seconds, long *loopIds, int *cands, long maxRows);
void dvmhgb_tuner_db_clear(void);
int dvmhgb_tuner_set_model(const float *params, const float *mean, const float *stdv);
int dvmhgb_tuner_rank(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *cands, int n, int *order);
/* The variant database (timed executions of variant-choosing handlers:
 * features of loop and variant, the loop shape's key, the variant, seconds),
 * and the variant model that ranks them (dvmhgb_loop_variant_desc); the model
 * has the cost model's shape and normalisation. */
long dvmhgb_tuner_vdb_size(void);
long dvmhgb_tuner_vdb_export(float *X, double *seconds, unsigned long long *keys, int *variants, long maxRows);
void dvmhgb_tuner_vdb_clear(void);
int dvmhgb_tuner_set_variant_model(const float *params, const float *mean, const float *stdv);

/* copy src -> dst for every element of the array outside the box (both arrays share st/ext) */
int dvmhgb_copy_outside_box(int rank, const double *src, double *dst, const long *st, const long *ext,
                            const long *lo, const long *hi, void *stream);

#ifdef __cplusplus
}
#endif
#pragma GCC visibility pop

#endif
