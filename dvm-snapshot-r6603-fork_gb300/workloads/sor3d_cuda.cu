// CUDA handler of the SOR ACROSS program (sor3d.c), in the shape cdvmh emits
// for ACROSS loops (cdvmh/src/across.cpp:2788-2894): dependency mask query,
// reduction registration, launch, reduction finish.  The launch is one
// persistent wavefront kernel per sweep (csrc/kernels/across.cu) instead of the
// reference's per-hyperplane launches.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "dvmhlib2.h"
#include "dvmh_gb.h"
#include "dvmh_gb_kernels.h"

#define SOR_DEFAULT_VARIANT 4

// the variants as the tuner's variant model sees them: family 3 (this program),
// the tile depth along k (64: streaming columns; hyperplanes per tile for the
// hyperplane tiles), tile kind (0 box, 1 streaming column, 2 / 3 hyperplane
// tile per warp / per CTA)
static const float sorDesc[6 * 3] = {3, 32, 0, 3, 16, 0, 3, 8, 0, 3, 64, 1, 3, 8, 2, 3, 8, 3};

extern "C" void loop_sor3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr) {
    (void)s_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    DvmType dep = dvmh_loop_get_dependency_mask_C(loop_ref);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType hdr[6], part[6], bl[3], bh[3], bs[3];
    dvmh_fill_header_C(device_num, A, A_hdr, hdr, 0);
    dvmh_loop_fill_local_part_C(loop_ref, A_hdr, part);
    dvmh_loop_fill_bounds_C(loop_ref, bl, bh, bs);
    long st[3], ext[3], lo[3], hi[3];
    for (int i = 0; i < 3; i++) {
        st[i] = (long)hdr[i + 1];
        ext[i] = (long)part[2 * i + 1] + 1;
        lo[i] = (long)bl[i];
        hi[i] = (long)bh[i];
    }
    if (dep != 7 || bs[0] != 1 || bs[1] != 1 || bs[2] != 1) {
        fprintf(stderr, "loop_sor3d_cuda: expects dependences on all three axes and unit steps\n");
        exit(1);
    }
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    double *w_dev = (double *)dvmh_get_device_addr_C(device_num, w_ptr);
    double s, *s_grid = 0;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&s_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    // tile shape: chosen by the runtime's variant tuner
    const int variant = dvmhgb_loop_variant_desc(loop_ref, DVMHGB_SOR3D_VARIANTS, SOR_DEFAULT_VARIANT, sorDesc, 3);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, dvmhgb_sor3d_items(lo, hi, variant), 0);
    void *scratch = dvmhgb_loop_scratch(loop_ref, dvmhgb_sor3d_scratch_bytes(lo, hi, variant));
    if (dvmhgb_sor3d_sweep(A, st, ext, lo, hi, w_dev, s_grid, scratch, dvmhgb_status_word(), variant, stream) != 0) {
        fprintf(stderr, "loop_sor3d_cuda: kernel launch rejected its arguments\n");
        exit(1);
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}
