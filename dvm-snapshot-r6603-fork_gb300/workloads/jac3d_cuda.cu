// CUDA handlers of the Jacobi 3-D program (jac3d.c), in the shape cdvmh emits
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

#define R 3
// default kernel variants, the fastest measured on GB300 at 512^3 (ms per call): the stencil with its planes
// staged by TMA, sums in q61 fixed point on the integer pipes and 2 of the CTA's 8 warps on the FP64 unit
// (0.822; the TMA stencil without FP64-unit warps 0.884, the register-staged fixed-point stencil 1.213, all
// additions on the FP64 unit 1.464)
#define DEF_STN 25
// the pair: the update kernel, then that stencil into the second buffer (1.354 per step; the one-pass TMA pair
// 1.66, the update and the TMA stencil running at the same time 1.66, the register-staged one-pass pair 2.01)
#define DEF_FUSED 25
// a step's stencil with the next step's update in one pass (the pairing the runtime forms across steps)
#define DEF_STNUPD 5  // 2 FP64-unit warps, 3 warps with the integer-pipe |B - A| (1.092 against 1.130 ms for variant 1, same box)

namespace {

// The variants as the tuner's variant model sees them (dvmhgb_loop_variant_desc):
// family 1 (this program), the handler (1 update, 2 stencil, 3 the fused pair),
// then for stencils: fixed-point sums, FP64-unit additions per cell, rows per
// thread, CTAs per SM, share of CTAs on the FP64 unit, and for the pair how it
// runs (0 one pass, 1 update then stencil, 2 the two overlapped in chunks).
// (the fixed-point feature is 1 for the register-staged kernels and 1 + ring/6
// for the TMA-staged ones; the share on the FP64 unit is that of CTAs or of
// warps)
constexpr int NDESC = 8;
constexpr int V_Q = 14, V_T = 22;  // first fixed-point stencil variant, first TMA-staged one
void stencilDesc(int v, float *d) {
    static const int q[8][3] = {{4, 0, 1}, {3, 0, 1}, {4, 1, 2}, {4, 1, 3}, {4, 2, 5}, {3, 1, 2}, {4, 1, 4}, {4, 3, 5}};
    if (v < 12) {
        d[2] = 0, d[3] = (float)(v % 6), d[4] = (float)(1 + v / 6), d[5] = 2, d[6] = 1;
    } else if (v < V_Q) {
        d[2] = 0, d[3] = 5, d[4] = 1, d[5] = v == 12 ? 3.0f : 4.0f, d[6] = 1;
    } else if (v < V_T) {
        const int *c = q[v - V_Q];
        d[2] = 1, d[3] = 5, d[4] = 1, d[5] = (float)c[0], d[6] = (float)c[1] / (float)c[2];
    } else {  // TMA-staged: ring planes, warps (of 8) on the FP64 unit
        static const int t[5][2] = {{6, 0}, {4, 0}, {6, 1}, {6, 2}, {6, 3}};
        const int *c = t[v - V_T];
        d[2] = 1.0f + (float)c[0] / 6.0f, d[3] = 5, d[4] = 1, d[5] = 4, d[6] = (float)c[1] / 8.0f;
    }
}
const float *variantDesc(int handler) {
    static float upd[3 * NDESC], stn[DVMHGB_JAC3D_VARIANTS * NDESC], fus[DVMHGB_JAC3D_FUSED_VARIANTS * NDESC];
    static float su[DVMHGB_JAC3D_STNUPD_VARIANTS * NDESC];
    static bool ready = false;
    if (!ready) {
        static const int wq[DVMHGB_JAC3D_STNUPD_VARIANTS][2] = {{0, 0}, {1, 0}, {2, 0}, {1, 2}, {1, 4}, {2, 3}};
        for (int v = 0; v < DVMHGB_JAC3D_STNUPD_VARIANTS; v++) {  // handler 4: stencil then the next update, one pass
            float *d = su + v * NDESC;
            d[0] = 1, d[1] = 4;
            stencilDesc(V_T, d);
            d[6] = (float)wq[v][0] / 8.0f;  // warps on the FP64 unit
            d[7] = (float)wq[v][1] / 8.0f;  // warps with the integer-pipe |B - A|
        }
        for (int v = 0; v < 3; v++) upd[v * NDESC] = 1, upd[v * NDESC + 1] = 1, upd[v * NDESC + 2] = (float)v;
        for (int v = 0; v < DVMHGB_JAC3D_VARIANTS; v++) {
            float *d = stn + v * NDESC;
            d[0] = 1, d[1] = 2;
            stencilDesc(v, d);
        }
        for (int v = 0; v < DVMHGB_JAC3D_FUSED_VARIANTS; v++) {
            float *d = fus + v * NDESC;
            d[0] = 1, d[1] = 3;
            if (v >= DVMHGB_JAC3D_FUSED_T) {  // one pass, fixed point, TMA-staged (rings of 5, 4)
                stencilDesc(V_T, d);
                d[2] = v == DVMHGB_JAC3D_FUSED_T ? 1.0f + 5.0f / 6.0f : 1.0f + 4.0f / 6.0f;
                d[7] = 0;
                continue;
            }
            if (v >= DVMHGB_JAC3D_FUSED_Q) {  // one pass, fixed point
                stencilDesc(V_Q, d);
                d[5] = v == DVMHGB_JAC3D_FUSED_Q ? 4.0f : 3.0f;
                d[7] = 0;
                continue;
            }
            const int sv = v < DVMHGB_JAC3D_VARIANTS ? v : (v == DVMHGB_JAC3D_OVERLAP_Q ? V_Q : 13);
            stencilDesc(sv, d);
            d[7] = v < V_Q ? 0.0f : (v < DVMHGB_JAC3D_OVERLAP ? 1.0f : 2.0f);
        }
        ready = true;
    }
    return handler == 1 ? upd : (handler == 2 ? stn : (handler == 3 ? fus : su));
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

extern "C" void loop_jac3d_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
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
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, dvmhgb_jac3d_update_items(lo, hi), 0);
    check(dvmhgb_jac3d_update(A.base, B.base, A.st, lo, hi, eps_grid, dvmhgb_loop_variant_desc(loop_ref, 3, 2, variantDesc(1), NDESC), stream), "loop_jac3d_upd_cuda");
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

extern "C" void loop_jac3d_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    ArrDev A = devArray(loop_ref, device_num, A_hdr), B = devArray(loop_ref, device_num, B_hdr);
    long lo[R], hi[R];
    bounds(loop_ref, lo, hi);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    check(dvmhgb_jac3d_stencil(A.base, B.base, A.st, A.ext, lo, hi, dvmhgb_loop_variant_desc(loop_ref, DVMHGB_JAC3D_VARIANTS, DEF_STN, variantDesc(2), NDESC), stream), "loop_jac3d_stn_cuda");
}

// refs[0]: the update loop (A_hdr, B_hdr, eps_ptr), refs[1]: the stencil loop (A2_hdr, B2_hdr)
extern "C" void loop_jac3d_fused_cuda(DvmType refs[2], DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr,
                                       DvmType A2_hdr[], DvmType B2_hdr[]) {
    DvmType upd = refs[0], stn = refs[1];
    long lo[R], hi[R], lo2[R], hi2[R];
    bounds(upd, lo, hi);
    bounds(stn, lo2, hi2);
    bool same = A_hdr == A2_hdr && B_hdr == B2_hdr;
    for (int i = 0; i < R; i++) same = same && lo[i] == lo2[i] && hi[i] == hi2[i];
    if (!same) {  // not the pattern the fused kernel implements: run the loops one after the other
        loop_jac3d_upd_cuda(&upd, A_hdr, B_hdr, eps_ptr);
        loop_jac3d_stn_cuda(&stn, A2_hdr, B2_hdr);
        return;
    }
    DvmType device_num = dvmh_loop_get_device_num_C(upd);
    ArrDev A = devArray(upd, device_num, A_hdr), B = devArray(upd, device_num, B_hdr);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(upd, 0, 0, &threads, &stream, 0);
    dvmh_loop_cuda_get_config_C(stn, 0, 0, &threads, &stream, 0);
    // + the pair: unfused, overlapped (two stencils), one pass in fixed point (two)
    const int variant = dvmhgb_loop_variant_desc(upd, DVMHGB_JAC3D_FUSED_VARIANTS, DEF_FUSED, variantDesc(3), NDESC);
    double eps, *eps_grid = 0;
    dvmh_loop_cuda_register_red_C(upd, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(upd, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(upd, 1, dvmhgb_jac3d_fused_items(lo, hi, variant), 0);
    // a one-pass kernel writes the next B into a second buffer; the pairs of two kernels (the update, then a
    // stencil that reads only A) write B itself
    double *Bnew = (variant >= V_Q && variant < DVMHGB_JAC3D_FUSED_Q) ? B.base
                                                                       : (double *)dvmhgb_loop_alt_buffer(stn, B_hdr);
    check(dvmhgb_jac3d_fused(A.base, B.base, Bnew, A.st, A.ext, lo, hi, eps_grid, variant, stream),
          "loop_jac3d_fused_cuda");
    dvmh_loop_cuda_red_finish_C(upd, 1);
}

// refs[0]: a time step's stencil loop (A_hdr, B_hdr), refs[1]: the next step's
// update loop (A2_hdr, B2_hdr, eps_ptr) -- the pair the runtime forms when the
// stencil, naming arrays only, stays queued past its step's region (one pass:
// the update's |B - A| and A = B on the stencil's new values, 24 bytes a cell)
extern "C" void loop_jac3d_stnupd_cuda(DvmType refs[2], DvmType A_hdr[], DvmType B_hdr[], DvmType A2_hdr[],
                                        DvmType B2_hdr[], double *eps_ptr) {
    DvmType stn = refs[0], upd = refs[1];
    long lo[R], hi[R], lo2[R], hi2[R];
    bounds(stn, lo, hi);
    bounds(upd, lo2, hi2);
    bool same = A_hdr == A2_hdr && B_hdr == B2_hdr;
    for (int i = 0; i < R; i++) same = same && lo[i] == lo2[i] && hi[i] == hi2[i];
    if (!same) {  // not the pattern the one-pass kernel implements: the loops one after the other
        loop_jac3d_stn_cuda(&stn, A_hdr, B_hdr);
        loop_jac3d_upd_cuda(&upd, A2_hdr, B2_hdr, eps_ptr);
        return;
    }
    DvmType device_num = dvmh_loop_get_device_num_C(upd);
    ArrDev A = devArray(upd, device_num, A_hdr), B = devArray(upd, device_num, B_hdr);
    dim3 threads(0, 0, 0);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(stn, 0, 0, &threads, &stream, 0);
    dvmh_loop_cuda_get_config_C(upd, 0, 0, &threads, &stream, 0);
    const int variant =
        dvmhgb_loop_variant_desc(upd, DVMHGB_JAC3D_STNUPD_VARIANTS, DEF_STNUPD, variantDesc(4), NDESC);
    double eps, *eps_grid = 0;
    dvmh_loop_cuda_register_red_C(upd, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(upd, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(upd, 1, dvmhgb_jac3d_stnupd_items(lo, hi, variant), 0);
    // the new A goes into A's second buffer: A is read by the pass; the two swap when the pair ends
    double *Aalt = (double *)dvmhgb_loop_alt_buffer(upd, A_hdr);
    check(dvmhgb_jac3d_stnupd(A.base, Aalt, B.base, A.st, A.ext, lo, hi, eps_grid, variant, stream),
          "loop_jac3d_stnupd_cuda");
    dvmh_loop_cuda_red_finish_C(upd, 1);
}

// module initialiser: the fusion rules (the role DvmhModuleInitializer plays for
// generated code, rts/dvmh/include/dvmhlib2.h:236-247)
namespace {
struct Rules {
    Rules() {
        dvmhgb_register_fusion((DvmHandlerFunc)loop_jac3d_upd_cuda, (DvmHandlerFunc)loop_jac3d_stn_cuda,
                               (DvmHandlerFunc)loop_jac3d_fused_cuda);
        dvmhgb_register_fusion((DvmHandlerFunc)loop_jac3d_stn_cuda, (DvmHandlerFunc)loop_jac3d_upd_cuda,
                               (DvmHandlerFunc)loop_jac3d_stnupd_cuda);
    }
} rules;
}  // namespace
