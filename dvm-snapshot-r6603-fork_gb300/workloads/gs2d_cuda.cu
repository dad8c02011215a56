// CUDA handler of gs2d.c in the shape cdvmh generates for an ACROSS loop in
// its basic mode (cdvmh/src/converter_main.cpp:2132-2401 with isOneThread):
// the block is forced to one thread after dvmh_loop_cuda_get_config_C, the
// reduction has one slot, and the kernel walks the loop nest in the source
// order with the loop's own (signed) steps.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

template <typename IndexT>
__global__ void loop_gs2d_kernel(double *A, IndexT A_hdr1, IndexT lo1, IndexT hi1, IndexT st1, IndexT lo2, IndexT hi2,
                                 IndexT st2, double s, double s_grid[]) {
    IndexT i, j;
    for (i = lo1; st1 > 0 ? i <= hi1 : i >= hi1; i += st1)
        for (j = lo2; st2 > 0 ? j <= hi2 : j >= hi2; j += st2) {
            A[i * A_hdr1 + j] = (A[(i - 1) * A_hdr1 + j] + A[(i + 1) * A_hdr1 + j] + A[i * A_hdr1 + (j - 1)] +
                                 A[i * A_hdr1 + (j + 1)]) * 0.25;
            s = s + A[i * A_hdr1 + j];
        }
    s_grid[0] = s;
}

extern "C" void loop_gs2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *s_ptr) {
    DvmType tmpVar;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    (void)s_ptr;
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    dim3 blocks(1, 1, 1), threads(1, 1, 1);
    cudaStream_t stream;
    int kernelIndexT = dvmh_loop_guess_index_type_C(loop_ref);
    if (kernelIndexT == rt_LONG) kernelIndexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(kernelIndexT == rt_INT || kernelIndexT == rt_LLONG);
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    threads = dim3(1, 1, 1);
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    double s, *s_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&s_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &s, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, 1, 0);
    if (kernelIndexT == rt_INT)
        loop_gs2d_kernel<int><<<blocks, threads, 0, stream>>>(A, A_devHdr[1], boundsLow[0], boundsHigh[0], loopSteps[0],
                                                              boundsLow[1], boundsHigh[1], loopSteps[1], s, s_grid);
    if (kernelIndexT == rt_LLONG)
        loop_gs2d_kernel<long long><<<blocks, threads, 0, stream>>>(A, A_devHdr[1], boundsLow[0], boundsHigh[0],
                                                                    loopSteps[0], boundsLow[1], boundsHigh[1],
                                                                    loopSteps[1], s, s_grid);
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}
