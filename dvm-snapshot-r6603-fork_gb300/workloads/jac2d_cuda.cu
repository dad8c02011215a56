// CUDA handlers of the Jacobi 2-D program (jac2d.c), in the shape cdvmh emits
// (cdvmh/src/converter_main.cpp:2132-2401): loop queries through the dvmh_*
// ABI, then the launch -- here of this library's hand-written sm_103a kernels
// (csrc/kernels/jacobi.cu) -- and the reduction calls.
//
// The fused handler is registered as a fusion rule: in batched mode the update
// loop followed by the stencil loop over the same box runs as one kernel pass
// that reads A and B once and writes A and the new B once (32 bytes per cell
// instead of 40).  Its arithmetic per cell is that of the two loops.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "dvmhlib2.h"
#include "dvmh_gb.h"
#include "dvmh_gb_kernels.h"

#define R 2
// FP64 additions per cell of the stencil loop; default count on the FP64 unit
#define NOPS_STN 3
#define DEF_STN 3
#define DEF_FUSED 4

namespace {

// the variants as the tuner's variant model sees them: family 2 (this program),
// the handler (1 update, 2 stencil, 3 the fused pair), its variant number
constexpr int NDESC = 3;
const float *variantDesc(int handler) {
    static float d[3][(NOPS_STN + 2) * NDESC];
    static bool ready = false;
    if (!ready) {
        for (int h = 1; h <= 3; h++)
            for (int v = 0; v < NOPS_STN + 2; v++) {
                d[h - 1][v * NDESC] = 2, d[h - 1][v * NDESC + 1] = (float)h, d[h - 1][v * NDESC + 2] = (float)v;
            }
        ready = true;
    }
    return d[handler - 1];
}

struct ArrDev {
    double *base;
    long st[R];
    long ext[R];
};

ArrDev devArray(DvmType loop_ref, DvmType device_num, DvmType hdr[]) {
    ArrDev a;
    DvmType devHdr[R + 3], part[2 * R];
    a.base = (double *)dvmh_get_natural_base_C(device_num, hdr);
    dvmh_fill_header_C(device_num, a.base, hdr, devHdr, 0);
    dvmh_loop_fill_local_part_C(loop_ref, hdr, part);
    for (int i = 0; i < R; i++) {
        a.st[i] = (long)devHdr[i + 1];
        a.ext[i] = (long)(part[2 * i + 1] + 1);
    }
    return a;
}

void bounds(DvmType loop_ref, long lo[R], long hi[R]) {
    DvmType bl[R], bh[R], bs[R];
    dvmh_loop_fill_bounds_C(loop_ref, bl, bh, bs);
    for (int i = 0; i < R; i++) {
        lo[i] = (long)bl[i];
        hi[i] = (long)bh[i];
    }
}

void check(int rc, const char *what) {
    if (rc != 0) {
        fprintf(stderr, "%s: kernel launch rejected its arguments\n", what);
        exit(1);
    }
}

}  // namespace

extern "C" void loop_jac2d_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
    (void)eps_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    ArrDev A = devArray(loop_ref, device_num, A_hdr), B = devArray(loop_ref, device_num, B_hdr);
    long lo[R], hi[R];
    bounds(loop_ref, lo, hi);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    double eps, *eps_grid = 0;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, dvmhgb_jac2d_update_items(lo, hi), 0);
    check(dvmhgb_jac2d_update(A.base, B.base, A.st, lo, hi, eps_grid, dvmhgb_loop_variant_desc(loop_ref, 3, 2, variantDesc(1), NDESC), stream), "loop_jac2d_upd_cuda");
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

extern "C" void loop_jac2d_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    ArrDev A = devArray(loop_ref, device_num, A_hdr), B = devArray(loop_ref, device_num, B_hdr);
    long lo[R], hi[R];
    bounds(loop_ref, lo, hi);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    check(dvmhgb_jac2d_stencil(A.base, B.base, A.st, A.ext, lo, hi, dvmhgb_loop_variant_desc(loop_ref, NOPS_STN + 1, DEF_STN, variantDesc(2), NDESC), stream), "loop_jac2d_stn_cuda");
}

// refs[0]: the update loop (A_hdr, B_hdr, eps_ptr), refs[1]: the stencil loop (A2_hdr, B2_hdr)
extern "C" void loop_jac2d_fused_cuda(DvmType refs[2], DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr,
                                       DvmType A2_hdr[], DvmType B2_hdr[]) {
    DvmType upd = refs[0], stn = refs[1];
    long lo[R], hi[R], lo2[R], hi2[R];
    bounds(upd, lo, hi);
    bounds(stn, lo2, hi2);
    bool same = A_hdr == A2_hdr && B_hdr == B2_hdr;
    for (int i = 0; i < R; i++) same = same && lo[i] == lo2[i] && hi[i] == hi2[i];
    if (!same) {  // not the pattern the fused kernel implements: run the loops one after the other
        loop_jac2d_upd_cuda(&upd, A_hdr, B_hdr, eps_ptr);
        loop_jac2d_stn_cuda(&stn, A2_hdr, B2_hdr);
        return;
    }
    DvmType device_num = dvmh_loop_get_device_num_C(upd);
    ArrDev A = devArray(upd, device_num, A_hdr), B = devArray(upd, device_num, B_hdr);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(upd, 0, 0, &threads, &stream, 0);
    dvmh_loop_cuda_get_config_C(stn, 0, 0, &threads, &stream, 0);
    double eps, *eps_grid = 0;
    dvmh_loop_cuda_register_red_C(upd, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(upd, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(upd, 1, dvmhgb_jac2d_fused_items(lo, hi), 0);
    double *Bnew = (double *)dvmhgb_loop_alt_buffer(stn, B_hdr);
    check(dvmhgb_jac2d_fused(A.base, B.base, Bnew, A.st, A.ext, lo, hi, eps_grid,
                             dvmhgb_loop_variant_desc(upd, NOPS_STN + 2, DEF_FUSED, variantDesc(3), NDESC), stream),
          "loop_jac2d_fused_cuda");
    dvmh_loop_cuda_red_finish_C(upd, 1);
}

// module initialiser: the fusion rule (the role DvmhModuleInitializer plays for
// generated code, rts/dvmh/include/dvmhlib2.h:236-247)
namespace {
struct Rules {
    Rules() {
        dvmhgb_register_fusion((DvmHandlerFunc)loop_jac2d_upd_cuda, (DvmHandlerFunc)loop_jac2d_stn_cuda,
                               (DvmHandlerFunc)loop_jac2d_fused_cuda);
    }
} rules;
}  // namespace
