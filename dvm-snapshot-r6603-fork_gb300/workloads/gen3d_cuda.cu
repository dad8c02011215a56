// CUDA handler of gen3d.c written exactly in the shape cdvmh generates for a
// parallel loop with reductions (cdvmh/src/converter_main.cpp:2132-2401 for
// the handler, :1861-2130 for the kernel), with no knowledge of this runtime:
//   * device base and header of every array (dvmh_get_natural_base_C,
//     dvmh_fill_header_C), addresses of scalars (dvmh_get_device_addr_C);
//   * the index type from dvmh_loop_guess_index_type_C, one kernel per type;
//   * the block from dvmh_loop_cuda_get_config_C, the loop bounds, the block
//     counts blocksS[d] as products over the inner axes;
//   * per reduction: register_red, red_init, red_prepare with one slot per
//     launched thread;
//   * launches of at most 65535 blocks with a block offset, then red_finish.
// The kernel runs one loop point per thread (loop axes z, y, x on the block's
// z, y, x) and writes every thread's private reduction values to its slot.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

template <typename IndexT>
__global__ void loop_gen3d_kernel(double *A, IndexT A_hdr1, IndexT A_hdr2, double *B, IndexT B_hdr1, IndexT B_hdr2,
                                  long *n12, long *n2, IndexT lo1, IndexT hi1, IndexT lo2, IndexT hi2,
                                  IndexT blocksS_2, IndexT lo3, IndexT hi3, IndexT blocksS_3, double s,
                                  double s_grid[], double mx, double mx_grid[], long lc, long lc_grid[],
                                  IndexT blockOffset) {
    IndexT restBlocks, curBlocks, i, j, k;
    restBlocks = blockIdx.x + blockOffset;
    curBlocks = restBlocks / blocksS_2;
    i = lo1 + (curBlocks * blockDim.z + threadIdx.z);
    if (i <= hi1) {
        restBlocks = restBlocks - curBlocks * blocksS_2;
        curBlocks = restBlocks / blocksS_3;
        j = lo2 + (curBlocks * blockDim.y + threadIdx.y);
        if (j <= hi2) {
            restBlocks = restBlocks - curBlocks * blocksS_3;
            curBlocks = restBlocks;
            k = lo3 + (curBlocks * blockDim.x + threadIdx.x);
            if (k <= hi3) {
                B[i * B_hdr1 + j * B_hdr2 + k] = A[(i - 1) * A_hdr1 + j * A_hdr2 + k] + 0.5 * A[i * A_hdr1 + j * A_hdr2 + (k + 1)];
                s = s + B[i * B_hdr1 + j * B_hdr2 + k];
                if (B[i * B_hdr1 + j * B_hdr2 + k] > mx) {
                    mx = B[i * B_hdr1 + j * B_hdr2 + k];
                    lc = i * *n12 + j * *n2 + k;
                }
            }
        }
    }
    const IndexT slot = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * (threadIdx.z + blockDim.z * (blockIdx.x + blockOffset)));
    s_grid[slot] = s;
    mx_grid[slot] = mx;
    lc_grid[slot] = lc;
}

extern "C" void loop_gen3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], long *n12_ptr, long *n2_ptr,
                                double *s_ptr, double *mx_ptr, long *lc_ptr) {
    DvmType tmpVar;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[6];
    tmpVar = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, 0);
    assert(tmpVar == 0);
    double *B = (double *)dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType B_devHdr[6];
    tmpVar = dvmh_fill_header_C(device_num, B, B_hdr, B_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    long *n12 = (long *)dvmh_get_device_addr_C(device_num, n12_ptr);
    long *n2 = (long *)dvmh_get_device_addr_C(device_num, n2_ptr);
    (void)s_ptr;
    (void)mx_ptr;
    (void)lc_ptr;
    DvmType boundsLow[3], boundsHigh[3], loopSteps[3], blocksS[3];
    DvmType restBlocks;
    dim3 blocks(1, 1, 1), threads(0, 0, 0);
    cudaStream_t stream;

    int kernelIndexT = dvmh_loop_guess_index_type_C(loop_ref);
    if (kernelIndexT == rt_LONG) kernelIndexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(kernelIndexT == rt_INT || kernelIndexT == rt_LLONG);
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);

    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    blocksS[2] = ((boundsHigh[2] - boundsLow[2]) / loopSteps[2] + 1 + (threads.x - 1)) / threads.x;
    blocksS[1] = blocksS[2] * (((boundsHigh[1] - boundsLow[1]) / loopSteps[1] + 1 + (threads.y - 1)) / threads.y);
    blocksS[0] = blocksS[1] * (((boundsHigh[0] - boundsLow[0]) / loopSteps[0] + 1 + (threads.z - 1)) / threads.z);

    double s, *s_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&s_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, blocksS[0] * threads.x * threads.y * threads.z, 0);
    double mx, *mx_grid;
    long lc, *lc_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 2, (void **)&mx_grid, (void **)&lc_grid);
    dvmh_loop_red_init_C(loop_ref, 2, &mx, &lc);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 2, blocksS[0] * threads.x * threads.y * threads.z, 0);

    restBlocks = blocksS[0];
    while (restBlocks > 0) {
        blocks.x = (restBlocks <= 65535 ? restBlocks : (restBlocks <= 65535 * 2 ? restBlocks / 2 : 65535));
        if (kernelIndexT == rt_INT)
            loop_gen3d_kernel<int><<<blocks, threads, 0, stream>>>(
                A, A_devHdr[1], A_devHdr[2], B, B_devHdr[1], B_devHdr[2], n12, n2, boundsLow[0], boundsHigh[0],
                boundsLow[1], boundsHigh[1], blocksS[1], boundsLow[2], boundsHigh[2], blocksS[2], s, s_grid, mx,
                mx_grid, lc, lc_grid, blocksS[0] - restBlocks);
        if (kernelIndexT == rt_LLONG)
            loop_gen3d_kernel<long long><<<blocks, threads, 0, stream>>>(
                A, A_devHdr[1], A_devHdr[2], B, B_devHdr[1], B_devHdr[2], n12, n2, boundsLow[0], boundsHigh[0],
                boundsLow[1], boundsHigh[1], blocksS[1], boundsLow[2], boundsHigh[2], blocksS[2], s, s_grid, mx,
                mx_grid, lc, lc_grid, blocksS[0] - restBlocks);
        restBlocks -= blocks.x;
    }

    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
    dvmh_loop_cuda_red_finish_C(loop_ref, 2);
}
