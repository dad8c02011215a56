// CUDA handler of gsd3d.c in the shape cdvmh generates for an ACROSS loop with
// two dependences and an independent axis when asked for automatic transforms
// (cdvmh/src/across.cpp:1393-1437, 1960-2170): after
// dvmh_change_filled_bounds2_C the two dependent axes come first; the host
// walks their diagonals and launches one kernel per diagonal, the diagonal's
// cells along x and the independent axis along the grid's y dimension.  The
// array is indexed through the header (natural, permuted or diagonalised).
#include <cuda_runtime.h>

#include <cassert>

#include "dvmh_gb_layout.h"
#include "dvmhlib2.h"

namespace {

// element (k, i, j) through the header: coefficients plus, when diagonalised,
// the position of the two plane axes in the diagonal numbering
struct Arr3 {
    double *base;
    long c[3];
    int tfm, xAxis, yAxis;  // plane axes 1-based
    long Rx, Ry, xOff, yOff;
    __device__ double &operator()(long k, long i, long j) const {
        long off = k * c[0] + i * c[1] + j * c[2];
        if (tfm & 2) {
            const long idx[3] = {k, i, j};
            off += dvmhgb_diag_index(idx[xAxis - 1] - xOff, idx[yAxis - 1] - yOff, Rx, Ry, (tfm & 4) != 0);
        }
        return base[off];
    }
};

__global__ void loop_gsd3d_kernel(Arr3 A, double m, double m_grid[], long num_elem_across, long num_elem_2,
                                  long base_0, long base_1, long base_2, long step_0, long step_1, long step_2,
                                  long idxs_0, long idxs_1, long idxs_2) {
    extern __shared__ double m_block[];
    const unsigned t = threadIdx.x;
    const long id = (long)blockIdx.x * blockDim.x + t, q = blockIdx.y;
    if (id < num_elem_across && q < num_elem_2) {
        long coords[3];
        coords[idxs_0] = base_0 - id * step_0;
        coords[idxs_1] = base_1 + id * step_1;
        coords[idxs_2] = base_2 + q * step_2;
        const long k = coords[0], i = coords[1], j = coords[2];
        const double old = A(k, i, j);
        const double v = (((A(k, i - 1, j) + A(k, i + 1, j)) + A(k, i, j - 1)) + A(k, i, j + 1)) * 0.25;
        A(k, i, j) = v;
        const double d = fabs(v - old);
        m = d > m ? d : m;
    }
    m_block[t] = m;
    __syncthreads();
    for (unsigned s = 1; s < blockDim.x; s <<= 1) {
        if (t % (2 * s) == 0 && t + s < blockDim.x)
            m_block[t] = m_block[t + s] > m_block[t] ? m_block[t + s] : m_block[t];
        __syncthreads();
    }
    const long slot = (long)blockIdx.y * gridDim.x + blockIdx.x;
    if (t == 0) m_grid[slot] = m_block[0] > m_grid[slot] ? m_block[0] : m_grid[slot];
}

}  // namespace

extern "C" void loop_gsd3d_cuda(DvmType *pLoopRef, DvmType A_hdr[], double *m_ptr) {
    (void)m_ptr;
    DvmType loop_ref = *pLoopRef;
    DvmType device_num = dvmh_loop_get_device_num_C(loop_ref);
    dvmh_loop_autotransform_C(loop_ref, A_hdr);
    double *base = (double *)dvmh_get_natural_base_C(device_num, A_hdr);
    DvmType A_devHdr[6], A_ext[7];
    DvmType tfm = dvmh_fill_header_C(device_num, base, A_hdr, A_devHdr, A_ext);
    assert(tfm == 0 || tfm == 1 || tfm == 2);
    Arr3 A;
    A.base = base;
    for (int a = 0; a < 3; a++) A.c[a] = A_devHdr[a + 1];
    A.tfm = (int)(tfm == 2 ? tfm + 4 * A_ext[6] : tfm);
    A.xAxis = tfm == 2 ? (int)A_ext[0] : 3;
    A.yAxis = tfm == 2 ? (int)A_ext[3] : 2;
    A.Rx = tfm == 2 ? A_ext[2] : 0;
    A.Ry = tfm == 2 ? A_ext[5] : 0;
    A.xOff = tfm == 2 ? A_ext[1] : 0;
    A.yOff = tfm == 2 ? A_ext[4] : 0;

    DvmType lo[3], hi[3], st[3], idxs[3];
    dvmh_loop_fill_bounds_C(loop_ref, lo, hi, st);
    dvmh_change_filled_bounds2_C(lo, hi, st, 3, dvmh_loop_get_dependency_mask_C(loop_ref), idxs);
    dim3 threads(128, 1, 1);
    cudaStream_t stream;
    DvmType shared = 8;
    dvmh_loop_cuda_get_config_C(loop_ref, shared, 0, &threads, &stream, &shared);
    threads = dim3(threads.x * threads.y * threads.z, 1, 1);  // the diagonal along x only
    shared = (DvmType)threads.x * 8;
    const long M0 = (hi[0] - lo[0]) / st[0] + 1, M1 = (hi[1] - lo[1]) / st[1] + 1;
    const long N2 = (hi[2] - lo[2]) / st[2] + 1;
    const long longest = M0 < M1 ? M0 : M1;
    const long bx = (longest + threads.x - 1) / threads.x;
    double m, *m_grid;
    dvmh_loop_cuda_register_red_C(loop_ref, 1, (void **)&m_grid, 0);
    dvmh_loop_red_init_C(loop_ref, 1, &m, 0);
    dvmh_loop_cuda_red_prepare_C(loop_ref, 1, bx * N2, 1);
    for (long d = 0; d <= M0 + M1 - 2; d++) {
        const long aHi = d < M0 - 1 ? d : M0 - 1;
        const long aLo = d - (M1 - 1) > 0 ? d - (M1 - 1) : 0;
        const long cells = aHi - aLo + 1;
        // blocks.x never exceeds bx, so every slot index stays below bx * N2
        const dim3 blocks((unsigned)((cells + threads.x - 1) / threads.x), (unsigned)N2, 1);
        loop_gsd3d_kernel<<<blocks, threads, shared, stream>>>(A, m, m_grid, cells, N2, lo[0] + aHi * st[0],
                                                               lo[1] + (d - aHi) * st[1], lo[2], st[0], st[1], st[2],
                                                               idxs[0], idxs[1], idxs[2]);
    }
    dvmh_loop_cuda_red_finish_C(loop_ref, 1);
}
