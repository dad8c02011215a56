// CUDA handler of gsd2d.c in the shape cdvmh generates for an ACROSS loop when
// it is asked for automatic transforms (cdvmh/src/across.cpp:2788-2894): the
// handler counts the loop's dependences (dvmh_loop_get_dependency_mask_C; a
// dependent axis with a single iteration has no dependence) and calls the
// case handler for that count.  The two-dependence case
// (cdvmh/src/across.cpp:1393-1437, 1960-2170):
//   - dvmh_loop_autotransform_C first, then the natural base and the header
//     with its extended parameters; the kernel indexes the array through the
//     header, so it runs on the natural, a permuted or a diagonalised layout;
//   - the host walks the loop's diagonals in order and launches one kernel per
//     diagonal; thread k of a launch takes the k-th cell of the diagonal,
//     from the largest index of the first loop axis down;
//   - each block folds its cells' MAX in shared memory and folds that into its
//     own reduction slot, which accumulates over all launches.
// The one-dependence case (cdvmh/src/across.cpp:1700-1940) launches once per
// value of the dependent index, the independent one across the threads.
#include <cuda_runtime.h>

#include <cassert>

#include "dvmh_gb_layout.h"
#include "dvmhlib2.h"

namespace {

// element (i, j) of a 2-D array through its header: coefficients per axis
// plus, when diagonalised, the position in the diagonal numbering
template <typename IndexT>
struct Arr2 {
    double *base;
    IndexT c0, c1;
    int tfm;      // 0 natural, 1 permuted, 2 diagonalised (+4: slash orientation)
    int xAxis;    // the diagonal plane's x axis (1 or 2)
    IndexT Rx, Ry, xOff, yOff;
    __device__ double &operator()(IndexT i, IndexT j) const {
        IndexT off = i * c0 + j * c1;
        if (tfm & 2) {
            const IndexT x = (xAxis == 1 ? i : j) - xOff, y = (xAxis == 1 ? j : i) - yOff;
            off += (IndexT)dvmhgb_diag_index(x, y, Rx, Ry, (tfm & 4) != 0);
        }
        return base[off];
    }
};

template <typename IndexT>
__global__ void loop_gsd2d_kernel(Arr2<IndexT> A, double m, double m_grid[], DvmType num_elem_across, IndexT base_0,
                                  IndexT base_1, IndexT step_0, IndexT step_1) {
    extern __shared__ double m_block[];
    const unsigned nt = blockDim.x * blockDim.y * blockDim.z;
    const unsigned t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const IndexT id = (IndexT)blockIdx.x * nt + t;
    if (id < num_elem_across) {
        const IndexT i = base_0 - id * step_0, j = base_1 + id * step_1;
        const double old = A(i, j);
        const double v = (((A(i - 1, j) + A(i + 1, j)) + A(i, j - 1)) + A(i, j + 1)) * 0.25;
        A(i, j) = v;
        const double d = fabs(v - old);
        m = d > m ? d : m;
    }
    m_block[t] = m;
    __syncthreads();
    for (unsigned s = 1; s < nt; s <<= 1) {
        if (t % (2 * s) == 0 && t + s < nt) m_block[t] = m_block[t + s] > m_block[t] ? m_block[t + s] : m_block[t];
        __syncthreads();
    }
    if (t == 0) m_grid[blockIdx.x] = m_block[0] > m_grid[blockIdx.x] ? m_block[0] : m_grid[blockIdx.x];
}

template <typename IndexT>
void sweep(DvmType loop_ref, const Arr2<IndexT> &A, const DvmType lo[2], const DvmType st[2], long M0, long M1,
           dim3 threads, cudaStream_t stream, DvmType shared) {
    double m, *m_grid;
    const long nt = (long)threads.x * threads.y * threads.z;
    const long longest = M0 < M1 ? M0 : M1;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&m_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &m, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, (longest + nt - 1) / nt, 1);
    for (long d = 0; d <= M0 + M1 - 2; d++) {
        const long aHi = d < M0 - 1 ? d : M0 - 1;          // first cell: the largest step index on axis 0
        const long aLo = d - (M1 - 1) > 0 ? d - (M1 - 1) : 0;
        const long cells = aHi - aLo + 1;
        const dim3 blocks((unsigned)((cells + nt - 1) / nt), 1, 1);
        loop_gsd2d_kernel<IndexT><<<blocks, threads, shared, stream>>>(
            A, m, m_grid, cells, (IndexT)(lo[0] + aHi * st[0]), (IndexT)(lo[1] + (d - aHi) * st[1]), (IndexT)st[0],
            (IndexT)st[1]);
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

template <typename IndexT>
Arr2<IndexT> arrayOf(double *base, const DvmType hdr[], DvmType tfm, const DvmType ext[7]) {
    Arr2<IndexT> A;
    A.base = base;
    A.c0 = (IndexT)hdr[1];
    A.c1 = (IndexT)hdr[2];
    A.tfm = (int)tfm;
    A.xAxis = tfm & 2 ? (int)ext[0] : 2;
    A.Rx = tfm & 2 ? (IndexT)ext[2] : 0;
    A.Ry = tfm & 2 ? (IndexT)ext[5] : 0;
    A.xOff = tfm & 2 ? (IndexT)ext[1] : 0;
    A.yOff = tfm & 2 ? (IndexT)ext[4] : 0;
    return A;
}

// one launch per value of the dependent index (coords[idxs_0]); the independent
// index runs across the threads
template <typename IndexT>
__global__ void loop_gsd2d_1_kernel(Arr2<IndexT> A, double m, double m_grid[], IndexT num_elem_1, IndexT base_0,
                                    IndexT base_1, IndexT step_1, IndexT idxs_0, IndexT idxs_1) {
    extern __shared__ double m_block[];
    const unsigned nt = blockDim.x * blockDim.y * blockDim.z;
    const unsigned t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const IndexT id = (IndexT)blockIdx.x * nt + t;
    if (id < num_elem_1) {
        IndexT coords[2];
        coords[idxs_0] = base_0;
        coords[idxs_1] = base_1 + id * step_1;
        const IndexT i = coords[0], j = coords[1];
        const double old = A(i, j);
        const double v = (((A(i - 1, j) + A(i + 1, j)) + A(i, j - 1)) + A(i, j + 1)) * 0.25;
        A(i, j) = v;
        const double d = fabs(v - old);
        m = d > m ? d : m;
    }
    m_block[t] = m;
    __syncthreads();
    for (unsigned s = 1; s < nt; s <<= 1) {
        if (t % (2 * s) == 0 && t + s < nt) m_block[t] = m_block[t + s] > m_block[t] ? m_block[t + s] : m_block[t];
        __syncthreads();
    }
    if (t == 0) m_grid[blockIdx.x] = m_block[0] > m_grid[blockIdx.x] ? m_block[0] : m_grid[blockIdx.x];
}

}  // namespace

extern "C" void loop_gsd2d_cuda_1_case(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr, int dependency_mask) {
    (void)m_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    dvmh_loop_autotransform_C(loop_ref, A_hdr);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5], A_extendedParams[7];
    DvmType A_typeOfTransform = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, A_extendedParams);
    assert(A_typeOfTransform == 0 || A_typeOfTransform == 1 || A_typeOfTransform == 2);
    if (A_typeOfTransform == 2) A_typeOfTransform += 4 * A_extendedParams[6];
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2], idxs[2];
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_change_filled_bounds2_C(boundsLow, boundsHigh, loopSteps, 2, dependency_mask, idxs);
    dim3 threads(256, 1, 1);
    cudaStream_t stream;
    DvmType shared = 8;
    dvmh_loop_cuda_get_config_C(loop_ref, shared, 0, &threads, &stream, &shared);
    const long nt = (long)threads.x * threads.y * threads.z;
    const long M0 = (boundsHigh[0] - boundsLow[0]) / loopSteps[0] + 1;  // the dependent axis
    const long M1 = (boundsHigh[1] - boundsLow[1]) / loopSteps[1] + 1;
    const Arr2<long long> Ah = arrayOf<long long>(A, A_devHdr, A_typeOfTransform, A_extendedParams);
    double m, *m_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&m_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &m, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, (M1 + nt - 1) / nt, 1);
    const dim3 blocks((unsigned)((M1 + nt - 1) / nt), 1, 1);
    for (long q = 0; q < M0; q++)
        loop_gsd2d_1_kernel<long long><<<blocks, threads, shared, stream>>>(
            Ah, m, m_grid, M1, boundsLow[0] + q * loopSteps[0], boundsLow[1], loopSteps[1], idxs[0], idxs[1]);
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}

extern "C" void loop_gsd2d_cuda_3_case(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr, int dependency_mask) {
    (void)m_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    dvmh_loop_autotransform_C(loop_ref, A_hdr);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5], A_extendedParams[7];
    DvmType A_typeOfTransform = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, A_extendedParams);
    assert(A_typeOfTransform == 0 || A_typeOfTransform == 1 || A_typeOfTransform == 2);
    if (A_typeOfTransform == 2) A_typeOfTransform += 4 * A_extendedParams[6];

    DvmType boundsLow[2], boundsHigh[2], loopSteps[2], idxs[2];
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dvmh_change_filled_bounds2_C(boundsLow, boundsHigh, loopSteps, 2, dependency_mask, idxs);
    int kernelIndexT = dvmh_loop_guess_index_type_C(loop_ref);
    if (kernelIndexT == rt_LONG) kernelIndexT = (sizeof(long) <= sizeof(int) ? rt_INT : rt_LLONG);
    assert(kernelIndexT == rt_INT || kernelIndexT == rt_LLONG);

    dim3 threads(256, 1, 1);
    cudaStream_t stream;
    DvmType shared = 8;
    dvmh_loop_cuda_get_config_C(loop_ref, shared, 0, &threads, &stream, &shared);
    const long M0 = (boundsHigh[0] - boundsLow[0]) / loopSteps[0] + 1;
    const long M1 = (boundsHigh[1] - boundsLow[1]) / loopSteps[1] + 1;
    if (kernelIndexT == rt_INT)
        sweep<int>(loop_ref, arrayOf<int>(A, A_devHdr, A_typeOfTransform, A_extendedParams), boundsLow, loopSteps, M0,
                   M1, threads, stream, shared);
    else
        sweep<long long>(loop_ref, arrayOf<long long>(A, A_devHdr, A_typeOfTransform, A_extendedParams), boundsLow,
                         loopSteps, M0, M1, threads, stream, shared);
}

// the handler: the case for the loop's number of dependences
extern "C" void loop_gsd2d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr) {
    int dependency_mask = (int)dvmh_loop_get_dependency_mask_C(*pLoopRef);
    int dependency_mask_tmp = dependency_mask;
    int dependency_num = 0;
    while (dependency_mask_tmp) {
        dependency_mask_tmp &= (dependency_mask_tmp - 1);
        ++dependency_num;
    }
    if (dependency_num == 1) loop_gsd2d_cuda_1_case(pLoopRef, A_hdr, m_ptr, dependency_mask);
    else if (dependency_num == 2) loop_gsd2d_cuda_3_case(pLoopRef, A_hdr, m_ptr, dependency_mask);
}

// The mirror loop B = 2 A over the whole array, in cdvmh's plain shape (no
// transforms asked for: the header must describe the natural layout).
template <typename IndexT>
__global__ void loop_gsd2d_mirror_kernel(double *B, IndexT B_hdr1, const double *A, IndexT A_hdr1, IndexT n0,
                                         IndexT n1) {
    const IndexT j = (IndexT)blockIdx.x * blockDim.x + threadIdx.x, i = (IndexT)blockIdx.y * blockDim.y + threadIdx.y;
    if (i < n0 && j < n1) B[i * B_hdr1 + j] = A[i * A_hdr1 + j] * 2.0;
}

extern "C" void loop_gsd2d_mirror_cuda(DvmType *pLoopRef, DvmType B_hdr[], DvmType A_hdr[]) {
    DvmType tmpVar;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    double *B = (double *)dvmh_get_natural_base_C(device_num, B_hdr);
    DvmType B_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, B, B_hdr, B_devHdr, 0);
    assert(tmpVar == 0);
    double *A = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[5];
    tmpVar = dvmh_fill_header_C(device_num, A, A_hdr, A_devHdr, 0);
    assert(tmpVar == 0);
    (void)tmpVar;
    DvmType boundsLow[2], boundsHigh[2], loopSteps[2];
    dvmh_loop_fill_bounds_C(loop_ref, boundsLow, boundsHigh, loopSteps);
    dim3 threads(32, 8, 1);
    cudaStream_t stream;
    dvmh_loop_cuda_get_config_C(loop_ref, 0, 0, &threads, &stream, 0);
    const long n0 = boundsHigh[0] + 1, n1 = boundsHigh[1] + 1;
    const dim3 blocks((unsigned)((n1 + threads.x - 1) / threads.x), (unsigned)((n0 + threads.y - 1) / threads.y), 1);
    const dim3 flat(threads.x, threads.y, 1);
    loop_gsd2d_mirror_kernel<long long><<<blocks, flat, 0, stream>>>(B, B_devHdr[1], A, A_devHdr[1], n0, n1);
}
