// CUDA handler of rec2d.c in the shape cdvmh generates for an ACROSS loop with
// one dependence when it is asked for automatic transforms
// (cdvmh/src/across.cpp:1393-1437, 1700-1940): dvmh_loop_autotransform_C,
// then the header (0 natural or 1 permuted: the coefficients say where every
// element is); the dependent axis comes first after
// dvmh_change_filled_bounds2_C and the host launches one kernel per value of
// it, the independent axis across the threads; each block folds its MIN into
// its own reduction slot, which accumulates over all launches.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

template <typename IndexT>
__global__ void loop_rec2d_kernel(double *A, IndexT c0, IndexT c1, double lo, double lo_grid[], IndexT num_elem_1,
                                  IndexT base_0, IndexT base_1, IndexT step_1, IndexT idxs_0, IndexT idxs_1) {
    extern __shared__ double lo_block[];
    const unsigned nt = blockDim.x * blockDim.y * blockDim.z;
    const unsigned t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const IndexT id = (IndexT)blockIdx.x * nt + t;
    if (id < num_elem_1) {
        IndexT coords[2];
        coords[idxs_0] = base_0;                 // the dependent index of this launch
        coords[idxs_1] = base_1 + id * step_1;   // the independent one
        const IndexT i = coords[0], j = coords[1];
        const double v = A[i * c0 + j * c1] * 0.5 + A[i * c0 + (j - 1) * c1] * 0.25;
        A[i * c0 + j * c1] = v;
        lo = v < lo ? v : lo;
    }
    lo_block[t] = lo;
    __syncthreads();
    for (unsigned s = 1; s < nt; s <<= 1) {
        if (t % (2 * s) == 0 && t + s < nt) lo_block[t] = lo_block[t + s] < lo_block[t] ? lo_block[t + s] : lo_block[t];
        __syncthreads();
    }
    if (t == 0) lo_grid[blockIdx.x] = lo_block[0] < lo_grid[blockIdx.x] ? lo_block[0] : lo_grid[blockIdx.x];
}

extern "C" void loop_rec2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *lo_ptr) {
    (void)lo_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    dvmh_loop_autotransform_C(loop_ref, A_hdr);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5], A_extendedParams[7];
    DvmType A_typeOfTransform = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, A_extendedParams);
    assert(A_typeOfTransform == 0 || A_typeOfTransform == 1);
    (void)A_typeOfTransform;

    DvmType boundsLow[2], boundsHigh[2], loopSteps[2], idxs[2];
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_change_filled_bounds2_C(boundsLow, boundsHigh, loopSteps, 2, dvmh_loop_get_dependency_mask_C(loop_ref),
                                 idxs);
    dim3 threads(256, 1, 1);
    cudaStream_t stream;
    DvmType shared = 8;
    dvmh_loop_cuda_get_config_C(loop_ref, shared, 0, &threads, &stream, &shared);
    const long nt = (long)threads.x * threads.y * threads.z;
    const long M0 = (boundsHigh[0] - boundsLow[0]) / loopSteps[0] + 1;  // the dependent axis
    const long M1 = (boundsHigh[1] - boundsLow[1]) / loopSteps[1] + 1;
    double lo, *lo_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&lo_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &lo, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, (M1 + nt - 1) / nt, 1);
    const dim3 blocks((unsigned)((M1 + nt - 1) / nt), 1, 1);
    for (long q = 0; q < M0; q++)
        loop_rec2d_kernel<long long><<<blocks, threads, shared, stream>>>(
            A, A_devHdr[1], A_devHdr[2], lo, lo_grid, M1, boundsLow[0] + q * loopSteps[0], boundsLow[1], loopSteps[1],
            idxs[0], idxs[1]);
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}
