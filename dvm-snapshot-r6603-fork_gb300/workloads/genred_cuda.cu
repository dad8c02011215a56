// CUDA handler of genred.c in exactly the shape cdvmh generates for a 1-D
// parallel loop with reductions (cdvmh/src/converter_main.cpp:2132-2401, kernel
// :1861-2130): a signed step from dvmh_loop_fill_bounds_C, one loop point per
// thread, every thread's private reduction values written to its slot.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

template <typename IndexT>
__global__ void loop_genred_kernel(double *X, int *V, IndexT lo1, IndexT hi1, IndexT step1, double ds, double ds_grid[],
                                   double dp, double dp_grid[], int imn, int imn_grid[], float fmx, float fmx_grid[],
                                   int ia, int ia_grid[], int io, int io_grid[], int ix, int ix_grid[], double dml,
                                   double dml_grid[], long lc, long lc_grid[], IndexT blockOffset) {
    IndexT restBlocks, curBlocks, i;
    restBlocks = blockIdx.x + blockOffset;
    curBlocks = restBlocks;
    i = lo1 + step1 * (curBlocks * blockDim.x + threadIdx.x);
    if (step1 > 0 ? i <= hi1 : i >= hi1) {
        ds = ds + X[i];
        dp = dp * (1.0 + X[i] / 65536.0);
        imn = V[i] < imn ? V[i] : imn;
        fmx = (float)X[i] > fmx ? (float)X[i] : fmx;
        ia &= V[i] | 0x0F0F0F0F;
        io |= V[i] & 0x00FF00FF;
        ix ^= V[i];
        if (X[i] < dml) {
            dml = X[i];
            lc = i;
        }
    }
    const IndexT slot = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * (threadIdx.z + blockDim.z * (blockIdx.x + blockOffset)));
    ds_grid[slot] = ds;
    dp_grid[slot] = dp;
    imn_grid[slot] = imn;
    fmx_grid[slot] = fmx;
    ia_grid[slot] = ia;
    io_grid[slot] = io;
    ix_grid[slot] = ix;
    dml_grid[slot] = dml;
    lc_grid[slot] = lc;
}

extern "C" void loop_genred_cuda(DvmType *pLoopRef, DvmType X_hdr[], DvmType V_hdr[], double *ds_ptr, double *dp_ptr,
                                 int *imn_ptr, float *fmx_ptr, int *ia_ptr, int *io_ptr, int *ix_ptr, double *dml_ptr,
                                 long *lc_ptr) {
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *X = (double *)dvmh_get_natural_base_C(device_num, X_hdr);
    int *V = (int *)dvmh_get_natural_base_C(device_num, V_hdr);
    (void)ds_ptr, (void)dp_ptr, (void)imn_ptr, (void)fmx_ptr, (void)ia_ptr, (void)io_ptr, (void)ix_ptr, (void)dml_ptr,
        (void)lc_ptr;
    DvmType boundsLow[1], boundsHigh[1], loopSteps[1], blocksS[1];
    DvmType restBlocks;
    dim3 blocks(1, 1, 1), threads(0, 0, 0);
    cudaStream_t stream;
    int kernelIndexT = dvmh_loop_guess_index_type_C(loop_ref);
    if (kernelIndexT == rt_LONG) kernelIndexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(kernelIndexT == rt_INT || kernelIndexT == rt_LLONG);
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    blocksS[0] = ((boundsHigh[0] - boundsLow[0]) / loopSteps[0] + 1 + (threads.x - 1)) / threads.x;
    const DvmType slots = blocksS[0] * threads.x * threads.y * threads.z;

    double ds, *ds_grid, dp, *dp_grid, dml, *dml_grid;
    int imn, *imn_grid, ia, *ia_grid, io, *io_grid, ix, *ix_grid;
    float fmx, *fmx_grid;
    long lc, *lc_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&ds_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &ds, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 2, (void **)&dp_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 2, &dp, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 2, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 3, (void **)&imn_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 3, &imn, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 3, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 4, (void **)&fmx_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 4, &fmx, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 4, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 5, (void **)&ia_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 5, &ia, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 5, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 6, (void **)&io_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 6, &io, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 6, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 7, (void **)&ix_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 7, &ix, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 7, slots, 0);
    dvmh_loop_cuda_register_red_C(loop_ref, 8, (void **)&dml_grid, (void **)&lc_grid);
    dvmh_loop_red_init_C(loop_ref, 8, &dml, &lc);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 8, slots, 0);

    restBlocks = blocksS[0];
    while (restBlocks > 0) {
        blocks.x = (restBlocks <= 65535 ? restBlocks : (restBlocks <= 65535 * 2 ? restBlocks / 2 : 65535));
        if (kernelIndexT == rt_INT)
            loop_genred_kernel<int><<<blocks, threads, 0, stream>>>(
                X, V, boundsLow[0], boundsHigh[0], loopSteps[0], ds, ds_grid, dp, dp_grid, imn, imn_grid, fmx, fmx_grid,
                ia, ia_grid, io, io_grid, ix, ix_grid, dml, dml_grid, lc, lc_grid, blocksS[0] - restBlocks);
        if (kernelIndexT == rt_LLONG)
            loop_genred_kernel<long long><<<blocks, threads, 0, stream>>>(
                X, V, boundsLow[0], boundsHigh[0], loopSteps[0], ds, ds_grid, dp, dp_grid, imn, imn_grid, fmx, fmx_grid,
                ia, ia_grid, io, io_grid, ix, ix_grid, dml, dml_grid, lc, lc_grid, blocksS[0] - restBlocks);
        restBlocks -= blocks.x;
    }
    for (int r = 1; r <= 8; r++) dvmh_loop_cuda_red_finish_C(loop_ref, r);
}
