// CUDA handlers of cdvh2d.c in the shape cdvmh generates them
// (cdvmh/src/converter_main.cpp:2132-2401 for the handler, :1861-2130 for the
// kernel): device bases and headers of the distributed arrays and of the
// regular arrays (`coef`, `w`, passed as dvmh_variable_get_header_C headers),
// the index type from dvmh_loop_guess_index_type_C, the block from
// dvmh_loop_cuda_get_config_C, one loop point per thread (loop axes y, x on
// the block's y, x), launches of at most 65535 blocks with a block offset,
// and one MAX reduction slot per launched thread.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

template <typename IndexT>
__global__ void loop_cdvh2d_c_110_cuda_kernel(double *A, IndexT A_hdr1, double *B, IndexT B_hdr1, IndexT lo1,
                                              IndexT hi1, IndexT lo2, IndexT hi2, IndexT blocksS_2, double eps,
                                              double eps_grid[], IndexT blockOffset) {
    IndexT restBlocks, curBlocks, i, j;
    restBlocks = blockIdx.x + blockOffset;
    curBlocks = restBlocks / blocksS_2;
    i = lo1 + (curBlocks * blockDim.y + threadIdx.y);
    if (i <= hi1) {
        restBlocks = restBlocks - curBlocks * blocksS_2;
        curBlocks = restBlocks;
        j = lo2 + (curBlocks * blockDim.x + threadIdx.x);
        if (j <= hi2) {
            const double d = fabs(B[i * B_hdr1 + j] - A[i * A_hdr1 + j]);
            eps = d > eps ? d : eps;
            A[i * A_hdr1 + j] = B[i * B_hdr1 + j];
        }
    }
    const IndexT slot = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * (blockIdx.x + blockOffset));
    eps_grid[slot] = eps;
}

template <typename IndexT>
__global__ void loop_cdvh2d_c_116_cuda_kernel(double *A, IndexT A_hdr1, double *B, IndexT B_hdr1, double *coef,
                                              double *w, IndexT lo1, IndexT hi1, IndexT lo2, IndexT hi2,
                                              IndexT blocksS_2, IndexT blockOffset) {
    IndexT restBlocks, curBlocks, i, j;
    restBlocks = blockIdx.x + blockOffset;
    curBlocks = restBlocks / blocksS_2;
    i = lo1 + (curBlocks * blockDim.y + threadIdx.y);
    if (i <= hi1) {
        restBlocks = restBlocks - curBlocks * blocksS_2;
        curBlocks = restBlocks;
        j = lo2 + (curBlocks * blockDim.x + threadIdx.x);
        if (j <= hi2)
            B[i * B_hdr1 + j] = w[i] * (coef[0] * A[(i - 1) * A_hdr1 + j] + coef[1] * A[i * A_hdr1 + (j - 1)] +
                                        coef[2] * A[i * A_hdr1 + (j + 1)] + coef[3] * A[(i + 1) * A_hdr1 + j]);
    }
}

namespace {

// index type, block, bounds and block counts of a 2-D loop (the generated preamble)
struct Launch2 {
    int indexT;
    dim3 threads;
    cudaStream_t stream;
    DvmType lo[2], hi[2], st[2], blocksS[2];
};

Launch2 preamble(DvmType loop_ref) {
    Launch2 L;
    L.indexT = dvmh_loop_guess_index_type_C(loop_ref);
    if (L.indexT == rt_LONG) L.indexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(L.indexT == rt_INT || L.indexT == rt_LLONG);
    L.threads = dim3(0, 0, 0);
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &L.threads, &L.stream, 0);
    dvmh_loop_fill_bounds_C(loop_ref, L.lo, L.hi, L.st);
    L.blocksS[1] = ((L.hi[1] - L.lo[1]) / L.st[1] + 1 + (L.threads.x - 1)) / L.threads.x;
    L.blocksS[0] = L.blocksS[1] * (((L.hi[0] - L.lo[0]) / L.st[0] + 1 + (L.threads.y - 1)) / L.threads.y);
    return L;
}

}  // namespace

extern "C" void loop_cdvh2d_c_110_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
    DvmType tmpVar;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, 0);
    assert(tmpVar == 0);
    double *B = (double *)dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType B_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, B, B_hdr, B_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    (void)eps_ptr;
    Launch2 L = preamble(loop_ref);
    double eps, *eps_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, L.blocksS[0] * L.threads.x * L.threads.y * L.threads.z, 0);
    dim3 blocks(1, 1, 1);
    DvmType restBlocks = L.blocksS[0];
    while (restBlocks > 0) {
        blocks.x = (restBlocks <= 65535 ? restBlocks : (restBlocks <= 65535 * 2 ? restBlocks / 2 : 65535));
        if (L.indexT == rt_INT)
            loop_cdvh2d_c_110_cuda_kernel<int><<<blocks, L.threads, 0, L.stream>>>(
                A, A_devHdr[1], B, B_devHdr[1], L.lo[0], L.hi[0], L.lo[1], L.hi[1], L.blocksS[1], eps, eps_grid,
                L.blocksS[0] - restBlocks);
        else
            loop_cdvh2d_c_110_cuda_kernel<long long><<<blocks, L.threads, 0, L.stream>>>(
                A, A_devHdr[1], B, B_devHdr[1], L.lo[0], L.hi[0], L.lo[1], L.hi[1], L.blocksS[1], eps, eps_grid,
                L.blocksS[0] - restBlocks);
        restBlocks -= blocks.x;
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

extern "C" void loop_cdvh2d_c_116_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], DvmType coef_hdr[],
                                       DvmType w_hdr[]) {
    DvmType tmpVar;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, 0);
    assert(tmpVar == 0);
    double *B = (double *)dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType B_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, B, B_hdr, B_devHdr, 0);
    assert(tmpVar == 0);
    double *coef = (double *)dvmh_get_natural_base_C(device_num, coef_hdr);
    DvmType coef_devHdr[4];
    tmpVar = dvmh_fill_header_C(device_num, coef, coef_hdr, coef_devHdr, 0);
    assert(tmpVar == 0);
    double *w = (double *)dvmh_get_natural_base_C(device_num, w_hdr);
    DvmType w_devHdr[4];
    tmpVar = dvmh_fill_header_C(device_num, w, w_hdr, w_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    Launch2 L = preamble(loop_ref);
    dim3 blocks(1, 1, 1);
    DvmType restBlocks = L.blocksS[0];
    while (restBlocks > 0) {
        blocks.x = (restBlocks <= 65535 ? restBlocks : (restBlocks <= 65535 * 2 ? restBlocks / 2 : 65535));
        if (L.indexT == rt_INT)
            loop_cdvh2d_c_116_cuda_kernel<int><<<blocks, L.threads, 0, L.stream>>>(
                A, A_devHdr[1], B, B_devHdr[1], coef, w, L.lo[0], L.hi[0], L.lo[1], L.hi[1], L.blocksS[1],
                L.blocksS[0] - restBlocks);
        else
            loop_cdvh2d_c_116_cuda_kernel<long long><<<blocks, L.threads, 0, L.stream>>>(
                A, A_devHdr[1], B, B_devHdr[1], coef, w, L.lo[0], L.hi[0], L.lo[1], L.hi[1], L.blocksS[1],
                L.blocksS[0] - restBlocks);
        restBlocks -= blocks.x;
    }
}
