// A second CUDA handler of sor3d.c, in the shape cdvmh generates for an ACROSS
// loop whose dependences cover three axes when asked for automatic transforms
// (cdvmh/src/across.cpp:848-1000 for the kernel, :2180-2480 for the case
// handler, :2811-2894 for the dispatcher), with no knowledge of this runtime:
//   * the dispatcher counts the bits of dvmh_loop_get_dependency_mask_C and
//     calls the case handler;
//   * dvmh_loop_autotransform_C (the runtime diagonalises the plane of the two
//     fastest dependent axes), the natural base, the header with the
//     transform's extended parameters;
//   * dvmh_loop_fill_bounds_C, dvmh_change_filled_bounds2_C (dependent axes
//     first), the block from dvmh_loop_cuda_get_config_C;
//   * one launch per hyperplane a + b + c = d of the normalised loop indices,
//     the hyperplane's (a, b) pairs on the grid's (y, x), c = d - a - b;
//   * a SUM slot per (a, b) column, prepared with fill = 1 and accumulated over
//     the hyperplanes (the column's cells in loop order), then red_finish.
// Every cell reads its -1 neighbours after their hyperplane and its +1
// neighbours before theirs, so the array is the sequential loop's bit for bit.
#include <cuda_runtime.h>

#include <cassert>
#include <cstdio>
#include <cstdlib>

#include "dvmh_gb_layout.h"
#include "dvmhlib2.h"

namespace {

// element (i, j, k) through the header: coefficients plus, when the plane of
// two axes is diagonalised, their position in the diagonal numbering
struct Arr3 {
    double *base;
    long c[3];
    int tfm, xAxis, yAxis;  // plane axes 1-based
    long Rx, Ry, xOff, yOff;
    __device__ double &operator()(long i, long j, long k) const {
        long off = i * c[0] + j * c[1] + k * c[2];
        if (tfm & 2) {
            const long idx[3] = {i, j, k};
            off += dvmhgb_diag_index(idx[xAxis - 1] - xOff, idx[yAxis - 1] - yOff, Rx, Ry, (tfm & 4) != 0);
        }
        return base[off];
    }
};

struct Box {
    long base[3], step[3], idxs[3];
    long M[3];
};

__global__ void loop_sor3d_gen_kernel_7_case(Arr3 A, const double *w_ptr, double s, double s_grid[], Box b, long d,
                                             long aLo, long aHi, long bLo, long bHi) {
    const long a = aLo + (long)blockIdx.y * blockDim.y + threadIdx.y;
    const long bb = bLo + (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a > aHi || bb > bHi) return;
    const long c = d - a - bb;
    if (c < 0 || c >= b.M[2]) return;
    long coords[3];
    coords[b.idxs[0]] = b.base[0] + a * b.step[0];
    coords[b.idxs[1]] = b.base[1] + bb * b.step[1];
    coords[b.idxs[2]] = b.base[2] + c * b.step[2];
    const long i = coords[0], j = coords[1], k = coords[2];
    const double w = *w_ptr;
    const double old = A(i, j, k);
    const double nv = (1.0 - w) * old + w / 6.0 * (A(i - 1, j, k) + A(i + 1, j, k) + A(i, j - 1, k) +
                                                   A(i, j + 1, k) + A(i, j, k - 1) + A(i, j, k + 1));
    A(i, j, k) = nv;
    s = s + (nv - old) * (nv - old);
    const long slot = a * b.M[1] + bb;
    s_grid[slot] = s_grid[slot] + s;
}

void loop_sor3d_gen_cuda_7_case(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr,
                                DvmType dependency_mask) {
    (void)s_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    dvmh_loop_autotransform_C(loop_ref, A_hdr);
    double *base = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[6], A_ext[7];
    DvmType tfm = dvmh_fill_header_C(device_num, base, A_hdr, A_devHdr, A_ext);
    assert(tfm == 0 || tfm == 1 || tfm == 2);
    Arr3 A;
    A.base = base;
    for (int q = 0; q < 3; q++) A.c[q] = A_devHdr[q + 1];
    A.tfm = (int)(tfm == 2 ? tfm + 4 * A_ext[6] : tfm);
    A.xAxis = tfm == 2 ? (int)A_ext[0] : 3;
    A.yAxis = tfm == 2 ? (int)A_ext[3] : 2;
    A.Rx = tfm == 2 ? A_ext[2] : 0;
    A.Ry = tfm == 2 ? A_ext[5] : 0;
    A.xOff = tfm == 2 ? A_ext[1] : 0;
    A.yOff = tfm == 2 ? A_ext[4] : 0;
    const double *w = (const double *)dvmh_get_device_addr_C(device_num, w_ptr);

    DvmType lo[3], hi[3], st[3], idxs[3];
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    dvmh_change_filled_bounds2_C(lo, hi, st, 3, dependency_mask, idxs);
    Box b;
    for (int q = 0; q < 3; q++) {
        b.base[q] = lo[q];
        b.step[q] = st[q];
        b.idxs[q] = idxs[q];
        b.M[q] = (hi[q] - lo[q]) / st[q] + 1;
    }
    dim3 threads(32, 8, 1);
    cudaStream_t stream;
    DvmType shared = 0;
    dvmh_loop_cuda_get_config_C(loop_ref, shared, 0, &threads, &stream, &shared);
    threads.z = 1;

    double s, *s_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&s_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, b.M[0] * b.M[1], 1);

    const long M0 = b.M[0], M1 = b.M[1], M2 = b.M[2];
    for (long d = 0; d <= M0 + M1 + M2 - 3; d++) {
        const long aLo = d - (M1 - 1) - (M2 - 1) > 0 ? d - (M1 - 1) - (M2 - 1) : 0;
        const long aHi = d < M0 - 1 ? d : M0 - 1;
        const long bLo = d - aHi - (M2 - 1) > 0 ? d - aHi - (M2 - 1) : 0;
        const long bHi = d - aLo < M1 - 1 ? d - aLo : M1 - 1;
        const dim3 blocks((unsigned)((bHi - bLo + 1 + threads.x - 1) / threads.x),
                          (unsigned)((aHi - aLo + 1 + threads.y - 1) / threads.y), 1);
        loop_sor3d_gen_kernel_7_case<<<blocks, threads, 0, stream>>>(A, w, s, s_grid, b, d, aLo, aHi, bLo, bHi);
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

}  // namespace

// The dispatcher: a hyperplane order over all three axes respects any subset
// of the dependences, so the three-dependence case serves every count here.
extern "C" void loop_sor3d_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr, double *w_ptr) {
    int dependency_mask = dvmh_loop_get_dependency_mask_C(*pLoopRef);
    int dependency_mask_tmp = dependency_mask, dependency_num = 0;
    while (dependency_mask_tmp) {
        dependency_mask_tmp &= (dependency_mask_tmp - 1);
        ++dependency_num;
    }
    if (dependency_num > 3) {
        fprintf(stderr, "loop_sor3d_gen_cuda: %d dependences in a 3-D loop\n", dependency_num);
        abort();
    }
    loop_sor3d_gen_cuda_7_case(pLoopRef, A_hdr, s_ptr, w_ptr, dependency_mask);
}
