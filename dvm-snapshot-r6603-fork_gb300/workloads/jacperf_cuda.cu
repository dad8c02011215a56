// CUDA handlers of jacperf.c (the reference's FP32 Jacobi benchmarks), and
// generated-shape handlers of jac3d.c's FP64 loops (wl_jac3d_use_generated),
// in the shape cdvmh generates for parallel loops (cdvmh/src/converter_main.cpp:
// 2132-2401 for the handler, :1861-2130 for the kernel), with no knowledge of
// this runtime: natural bases and headers (dvmh_get_natural_base_C,
// dvmh_fill_header_C), the index type from dvmh_loop_guess_index_type_C, the
// block from dvmh_loop_cuda_get_config_C (the program's cuda_block), block
// counts blocksS[d] as products over the inner axes, one MAX slot per launched
// thread (register_red, red_init, red_prepare, red_finish), launches of at most
// 65535 blocks with a block offset.  One loop point per thread: loop axes
// (i, j, k) on the block's (z, y, x), or (i, j) on (y, x).
#include <cuda_runtime.h>

#include <cassert>

#include "dvmhlib2.h"

#define Max(a, b) ((a) > (b) ? (a) : (b))

namespace {

// loop point of this thread from the block number; false past the bounds
template <typename IndexT, int R>
__device__ bool pointOf(IndexT restBlocks, const IndexT lo[R], const IndexT hi[R], const IndexT blocksS[R],
                        IndexT idx[R]) {
    const unsigned th[3] = {R == 3 ? threadIdx.z : threadIdx.y, R == 3 ? threadIdx.y : threadIdx.x, threadIdx.x};
    const unsigned bd[3] = {R == 3 ? blockDim.z : blockDim.y, R == 3 ? blockDim.y : blockDim.x, blockDim.x};
    for (int d = 0; d < R; d++) {
        const IndexT cur = d + 1 < R ? restBlocks / blocksS[d + 1] : restBlocks;
        idx[d] = lo[d] + (cur * (IndexT)bd[d] + (IndexT)th[d]);
        if (idx[d] > hi[d]) return false;
        if (d + 1 < R) restBlocks = restBlocks - cur * blocksS[d + 1];
    }
    return true;
}

template <typename IndexT, int R>
struct Geo {
    IndexT lo[R], hi[R], blocksS[R];
};

template <typename IndexT, int R>
__global__ void loop_jacperf_init_kernel(float *A, IndexT A_hdr1, IndexT A_hdr2, float *B, IndexT B_hdr1,
                                         IndexT B_hdr2, IndexT L, Geo<IndexT, R> g, IndexT blockOffset) {
    IndexT x[R];
    if (!pointOf<IndexT, R>((IndexT)blockIdx.x + blockOffset, g.lo, g.hi, g.blocksS, x)) return;
    if (R == 3) {
        const IndexT i = x[0], j = x[1], k = x[R - 1];
        A[i * A_hdr1 + j * A_hdr2 + k] = 0;
        if (i == 0 || j == 0 || k == 0 || i == L - 1 || j == L - 1 || k == L - 1)
            B[i * B_hdr1 + j * B_hdr2 + k] = 0;
        else
            B[i * B_hdr1 + j * B_hdr2 + k] = 4 + i + j + k;
    } else {
        const IndexT i = x[0], j = x[R - 1];
        A[i * A_hdr1 + j] = 0;
        if (i == 0 || j == 0 || i == L - 1 || j == L - 1)
            B[i * B_hdr1 + j] = 0;
        else
            B[i * B_hdr1 + j] = 3 + i + j;
    }
}

template <typename T, typename IndexT, int R>
__global__ void loop_jacperf_upd_kernel(T *A, IndexT A_hdr1, IndexT A_hdr2, T *B, IndexT B_hdr1, IndexT B_hdr2,
                                        Geo<IndexT, R> g, T eps, T eps_grid[], IndexT blockOffset) {
    IndexT x[R];
    if (pointOf<IndexT, R>((IndexT)blockIdx.x + blockOffset, g.lo, g.hi, g.blocksS, x)) {
        const IndexT qa = R == 3 ? x[0] * A_hdr1 + x[1] * A_hdr2 + x[R - 1] : x[0] * A_hdr1 + x[R - 1];
        const IndexT qb = R == 3 ? x[0] * B_hdr1 + x[1] * B_hdr2 + x[R - 1] : x[0] * B_hdr1 + x[R - 1];
        T tmp = fabs(B[qb] - A[qa]);
        eps = Max(tmp, eps);
        A[qa] = B[qb];
    }
    const IndexT slot = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * (threadIdx.z + blockDim.z *
                                                                                   ((IndexT)blockIdx.x + blockOffset)));
    eps_grid[slot] = eps;
}

template <typename T, typename IndexT, int R>
__global__ void loop_jacperf_stn_kernel(T *A, IndexT A_hdr1, IndexT A_hdr2, T *B, IndexT B_hdr1, IndexT B_hdr2,
                                        Geo<IndexT, R> g, IndexT blockOffset) {
    IndexT x[R];
    if (!pointOf<IndexT, R>((IndexT)blockIdx.x + blockOffset, g.lo, g.hi, g.blocksS, x)) return;
    if (R == 3) {
        const IndexT i = x[0], j = x[1], k = x[R - 1];
        B[i * B_hdr1 + j * B_hdr2 + k] =
            (A[(i - 1) * A_hdr1 + j * A_hdr2 + k] + A[i * A_hdr1 + (j - 1) * A_hdr2 + k] +
             A[i * A_hdr1 + j * A_hdr2 + (k - 1)] + A[i * A_hdr1 + j * A_hdr2 + (k + 1)] +
             A[i * A_hdr1 + (j + 1) * A_hdr2 + k] + A[(i + 1) * A_hdr1 + j * A_hdr2 + k]) /
            (T)6;
    } else {
        const IndexT i = x[0], j = x[R - 1];
        B[i * B_hdr1 + j] = (A[(i - 1) * A_hdr1 + j] + A[i * A_hdr1 + (j - 1)] + A[i * A_hdr1 + (j + 1)] +
                             A[(i + 1) * A_hdr1 + j]) /
                            (T)4;
    }
}

// The handler body every loop shares: headers, index type, block, bounds and
// block counts, then `launch(blocks, threads, stream, geometry, offset)` per
// chunk of at most 65535 blocks.
struct Prep {
    DvmType loop_ref, device_num;
    void *A, *B;
    DvmType A_devHdr[8], B_devHdr[8];
    DvmType lo[3], hi[3], steps[3], blocksS[3];
    dim3 threads;
    cudaStream_t stream;
    int indexT;
};

template <int R>
Prep prepare(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    Prep p;
    DvmType tmpVar;
    p.loop_ref = *pLoopRef;
    p.device_num = dvmh_loop_get_device_num_C(p.loop_ref);
    p.A = dvmh_get_natural_base_C(p.device_num, A_hdr);
    tmpVar = dvmh_fill_header_C(p.device_num, p.A, A_hdr, p.A_devHdr, 0);
    assert(tmpVar == 0);
    p.B = dvmh_get_natural_base_C(p.device_num, B_hdr);
    tmpVar = dvmh_fill_header_C(p.device_num, p.B, B_hdr, p.B_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    p.indexT = dvmh_loop_guess_index_type_C(p.loop_ref);
    if (p.indexT == rt_LONG) p.indexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(p.indexT == rt_INT || p.indexT == rt_LLONG);
    p.threads = dim3(0, 0, 0);
    dvmh_loop_cuda_get_config_C(p.loop_ref, 0, 0, &p.threads, &p.stream, 0);
    dvmh_loop_fill_bounds_C(p.loop_ref, p.lo, p.hi, p.steps);
    const unsigned per[3] = {R == 3 ? p.threads.z : p.threads.y, R == 3 ? p.threads.y : p.threads.x, p.threads.x};
    DvmType prod = 1;
    for (int d = R - 1; d >= 0; d--) {
        prod *= ((p.hi[d] - p.lo[d]) / p.steps[d] + 1 + (per[d] - 1)) / per[d];
        p.blocksS[d] = prod;
    }
    return p;
}

template <typename IndexT, int R>
Geo<IndexT, R> geo(const Prep &p) {
    Geo<IndexT, R> g;
    for (int d = 0; d < R; d++) {
        g.lo[d] = (IndexT)p.lo[d];
        g.hi[d] = (IndexT)p.hi[d];
        g.blocksS[d] = (IndexT)p.blocksS[d];
    }
    return g;
}

template <typename F>
void chunks(const Prep &p, F launch) {
    DvmType restBlocks = p.blocksS[0];
    dim3 blocks(1, 1, 1);
    while (restBlocks > 0) {
        blocks.x = (restBlocks <= 65535 ? restBlocks : (restBlocks <= 65535 * 2 ? restBlocks / 2 : 65535));
        launch(blocks, p.blocksS[0] - restBlocks);
        restBlocks -= blocks.x;
    }
}

template <int R>
void initHandler(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    Prep p = prepare<R>(pLoopRef, A_hdr, B_hdr);
    const DvmType L = p.hi[0] + 1;
    chunks(p, [&](dim3 blocks, DvmType off) {
        if (p.indexT == rt_INT)
            loop_jacperf_init_kernel<int, R><<<blocks, p.threads, 0, p.stream>>>(
                (float *)p.A, p.A_devHdr[1], p.A_devHdr[2], (float *)p.B, p.B_devHdr[1], p.B_devHdr[2], L,
                geo<int, R>(p), off);
        else
            loop_jacperf_init_kernel<long long, R><<<blocks, p.threads, 0, p.stream>>>(
                (float *)p.A, p.A_devHdr[1], p.A_devHdr[2], (float *)p.B, p.B_devHdr[1], p.B_devHdr[2], L,
                geo<long long, R>(p), off);
    });
}

template <typename T, int R>
void updHandler(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    Prep p = prepare<R>(pLoopRef, A_hdr, B_hdr);
    T eps, *eps_grid;
    dvmh_loop_cuda_register_red_C(p.loop_ref, 1, (void **)&eps_grid, 0);
    dvmh_loop_red_init_C(p.loop_ref, 1, &eps, 0);
    dvmh_loop_cuda_red_prepare_C(p.loop_ref, 1, p.blocksS[0] * p.threads.x * p.threads.y * p.threads.z, 0);
    chunks(p, [&](dim3 blocks, DvmType off) {
        if (p.indexT == rt_INT)
            loop_jacperf_upd_kernel<T, int, R><<<blocks, p.threads, 0, p.stream>>>(
                (T *)p.A, p.A_devHdr[1], p.A_devHdr[2], (T *)p.B, p.B_devHdr[1], p.B_devHdr[2], geo<int, R>(p), eps,
                eps_grid, off);
        else
            loop_jacperf_upd_kernel<T, long long, R><<<blocks, p.threads, 0, p.stream>>>(
                (T *)p.A, p.A_devHdr[1], p.A_devHdr[2], (T *)p.B, p.B_devHdr[1], p.B_devHdr[2], geo<long long, R>(p),
                eps, eps_grid, off);
    });
    dvmh_loop_cuda_red_finish_C(p.loop_ref, 1);
}

template <typename T, int R>
void stnHandler(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    Prep p = prepare<R>(pLoopRef, A_hdr, B_hdr);
    chunks(p, [&](dim3 blocks, DvmType off) {
        if (p.indexT == rt_INT)
            loop_jacperf_stn_kernel<T, int, R><<<blocks, p.threads, 0, p.stream>>>(
                (T *)p.A, p.A_devHdr[1], p.A_devHdr[2], (T *)p.B, p.B_devHdr[1], p.B_devHdr[2], geo<int, R>(p), off);
        else
            loop_jacperf_stn_kernel<T, long long, R><<<blocks, p.threads, 0, p.stream>>>(
                (T *)p.A, p.A_devHdr[1], p.A_devHdr[2], (T *)p.B, p.B_devHdr[1], p.B_devHdr[2], geo<long long, R>(p),
                off);
    });
}

}  // namespace

extern "C" void loop_jacperf2_init_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    initHandler<2>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jacperf2_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr) {
    (void)eps_ptr;
    updHandler<float, 2>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jacperf2_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    stnHandler<float, 2>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jacperf3_init_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    initHandler<3>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jacperf3_upd_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], float *eps_ptr) {
    (void)eps_ptr;
    updHandler<float, 3>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jacperf3_stn_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    stnHandler<float, 3>(pLoopRef, A_hdr, B_hdr);
}

// jac3d.c's FP64 loops (examples/Performance/jac3d_perf.c:56-73 in FP64) through
// the same generated shape, for comparison with the library's fused kernels
extern "C" void loop_jac3d_upd_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[], double *eps_ptr) {
    (void)eps_ptr;
    updHandler<double, 3>(pLoopRef, A_hdr, B_hdr);
}
extern "C" void loop_jac3d_stn_gen_cuda(DvmType *pLoopRef, DvmType A_hdr[], DvmType B_hdr[]) {
    stnHandler<double, 3>(pLoopRef, A_hdr, B_hdr);
}
