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

#include <cstdio>
#include <cstdlib>

#include "dvmhlib2.h"
#include "dvmh_gb.h"
#include "dvmh_gb_kernels.h"

namespace {

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

// refs: `count` loops whose CUDA handler is loop_heat_cuda, over distinct arrays
extern "C" void loop_heat_batch_cuda(DvmType *refs, DvmType count) {
    dvmhgb_heat_desc *table =
        (dvmhgb_heat_desc *)dvmhgb_loop_host_scratch(refs[0], (DvmType)(sizeof(dvmhgb_heat_desc) * count));
    cudaStream_t stream = 0;
    long total = 0, units = 0;
    for (DvmType q = 0; q < count; q++) {
        DvmType ref = refs[q];
        prepare(ref, (DvmType *)dvmhgb_loop_param(ref, 0), (DvmType *)dvmhgb_loop_param(ref, 1),
                (double *)dvmhgb_loop_param(ref, 5), &table[q], &stream);
        table[q].unitBase = units;
        table[q].stripBase = total;
        units += table[q].units;
        total += table[q].strips;
    }
    dvmhgb_heat_desc *dev =
        (dvmhgb_heat_desc *)dvmhgb_loop_scratch(refs[0], (DvmType)(sizeof(dvmhgb_heat_desc) * count));
    if (cudaMemcpyAsync(dev, table, sizeof(dvmhgb_heat_desc) * count, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        dvmhgb_heat_many(dev, (int)count, total, stream) != 0) {
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
