// CUDA handlers of the batched heat program (heat.c), in the shape cdvmh emits
// (cdvmh/src/converter_main.cpp:2132-2401): queries, reduction registration
// (SUM and MINLOC), launch of the hand-written kernel (csrc/kernels/heat.cu),
// reduction finish.
//
// loop_heat_batch_cuda is registered as the batch rule of loop_heat_cuda: in
// batched mode a run of these loops over pairwise distinct arrays (one per
// array of the time step) becomes one kernel over a table of all arrays, and
// the runtime folds all their reductions in one more launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "dvmhlib2.h"
#include "dvmh_gb.h"
#include "dvmh_gb_kernels.h"

namespace {

// the variants as the tuner's variant model sees them: family 4 (this program),
// log2 rows per strip, CTAs per SM, then the batch: log2 of its loops and of
// its cells, log2 of the largest loop's rows
constexpr int HEAT_NDESC = 6;
void heatVariantDesc(float *d, long loops, long cells, long maxRows) {
    for (int v = 0; v < DVMHGB_HEAT_VARIANTS; v++) {
        float *e = d + v * HEAT_NDESC;
        e[0] = 4;
        e[1] = (float)(4 + v % 5);
        e[2] = (float)DVMHGB_HEAT_CTAS(v);
        e[3] = (float)log2((double)loops);
        e[4] = (float)log2((double)(cells > 1 ? cells : 1));
        e[5] = (float)log2((double)(maxRows > 1 ? maxRows : 1));
    }
}

// everything a heat loop needs on the device, its reduction buffers prepared
void prepare(DvmType loop_ref, DvmType S_hdr[], DvmType D_hdr[], double *c_ptr, dvmhgb_heat_desc *d,
             cudaStream_t *stream) {
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *src = (double *)dvmh_get_natural_base_C(device_num, S_hdr);
    double *dst = (double *)dvmh_get_natural_base_C(device_num, D_hdr);
    DvmType sh[5], dh[5], bl[2], bh[2], bs[2];
    dvmh_fill_header_C(device_num, src, S_hdr, sh, 0);
    dvmh_fill_header_C(device_num, dst, D_hdr, dh, 0);
    dvmh_loop_fill_bounds_C(loop_ref, bl, bh, bs);
    long lo[2] = {(long)bl[0], (long)bl[1]}, hi[2] = {(long)bh[0], (long)bh[1]};
    if (sh[1] != dh[1] || sh[2] != 1 || bs[0] != 1 || bs[1] != 1 ||
        dvmhgb_heat_desc_fill(d, src, dst, (long)sh[1], lo, hi,
                              (const double *)dvmh_get_device_addr_C(device_num, c_ptr)) != 0) {
        fprintf(stderr, "heat handler: unsupported loop or array layout\n");
        exit(1);
    }
    dim3 threads(0, 0, 0);
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, stream, 0);
    double s, mn;
    int lc[2];
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&d->sumItems, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 2, (void **)&d->minItems, (void **)&d->locItems);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    dvmh_loop_red_init_C(loop_ref, 2, &mn, lc);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, d->units, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 2, d->units, 0);
}

}  // namespace

extern "C" void loop_heat_cuda(DvmType *pLoopRef, DvmType S_hdr[], DvmType D_hdr[], double *sum_ptr, double *min_ptr,
                               int *loc_ptr, double *c_ptr) {
    (void)sum_ptr;
    (void)min_ptr;
    (void)loc_ptr;
    DvmType loop_ref = *pLoopRef;
    dvmhgb_heat_desc d;
    cudaStream_t stream;
    prepare(loop_ref, S_hdr, D_hdr, c_ptr, &d, &stream);
    if (dvmhgb_heat(&d, stream) != 0) {
        fprintf(stderr, "loop_heat_cuda: kernel launch rejected its arguments\n");
        exit(1);
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
    dvmh_loop_cuda_red_finish_C(loop_ref, 2);
}

// refs: `count` loops whose CUDA handler is loop_heat_cuda, over distinct arrays.
// The strip geometry (rows per strip, CTAs per SM) is the tuner's variant.
extern "C" void loop_heat_batch_cuda(DvmType *refs, DvmType count) {
    dvmhgb_heat_desc *table =
        (dvmhgb_heat_desc *)dvmhgb_loop_host_scratch(refs[0], (DvmType)(sizeof(dvmhgb_heat_desc) * count));
    cudaStream_t stream = 0;
    long cells = 0, maxRows = 1;
    for (DvmType q = 0; q < count; q++) {
        DvmType ref = refs[q];
        prepare(ref, (DvmType *)dvmhgb_loop_param(ref, 0), (DvmType *)dvmhgb_loop_param(ref, 1),
                (double *)dvmhgb_loop_param(ref, 5), &table[q], &stream);
        const long rows = table[q].hi0 - table[q].lo0 + 1;
        cells += rows * (table[q].hi1 - table[q].lo1 + 1);
        if (rows > maxRows) maxRows = rows;
    }
    float desc[DVMHGB_HEAT_VARIANTS * HEAT_NDESC];
    heatVariantDesc(desc, (long)count, cells, maxRows);
    const int v = dvmhgb_loop_variant_desc(refs[0], DVMHGB_HEAT_VARIANTS, DVMHGB_HEAT_DEFAULT, desc, HEAT_NDESC);
    long total = 0, units = 0;
    for (DvmType q = 0; q < count; q++) {
        dvmhgb_heat_desc_rows(&table[q], DVMHGB_HEAT_ROWS(v));
        table[q].unitBase = units;
        table[q].stripBase = total;
        units += table[q].units;
        total += table[q].strips;
    }
    dvmhgb_heat_desc *dev =
        (dvmhgb_heat_desc *)dvmhgb_loop_scratch(refs[0], (DvmType)(sizeof(dvmhgb_heat_desc) * count));
    if (cudaMemcpyAsync(dev, table, sizeof(dvmhgb_heat_desc) * count, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        dvmhgb_heat_many_grid(dev, (int)count, total, DVMHGB_HEAT_CTAS(v), stream) != 0) {
        fprintf(stderr, "loop_heat_batch_cuda: launch failed\n");
        exit(1);
    }
    for (DvmType q = 0; q < count; q++) {
        dvmh_loop_cuda_red_finish_C(refs[q], 1);
        dvmh_loop_cuda_red_finish_C(refs[q], 2);
    }
}

namespace {
struct Rules {
    Rules() { dvmhgb_register_batch((DvmHandlerFunc)loop_heat_cuda, (DvmHandlerFunc)loop_heat_batch_cuda); }
} rules;
}  // namespace
