// ACROSS loop kernel for sm_103a: SOR / Gauss-Seidel 3-D with dependences
// (1:1, 1:1, 1:1), executed as a persistent tiled wavefront.
//
// The reference runs such a loop as one kernel launch per hyperplane from the
// host (cdvmh/src/across.cpp:2480-2760: three diagonal phases, ~3n launches per
// sweep).  Here one launch covers the sweep:
//   * the loop box is cut into 8 x 8 x 64 tiles (the 64-wide k range aligned to
//     multiples of 64 of the array index);
//   * a tile depends only on its three face predecessors (a-1,b,c), (a,b-1,c),
//     (a,b,c-1) -- the 7-point stencil touches face neighbours only;
//   * tiles are handed out by an atomic counter in diagonal order (a topological
//     order), the grid is no larger than the GPU holds at once, so every tile a
//     CTA waits for is already owned by a running CTA: progress is guaranteed;
//   * every wait is bounded: past the limit the CTA writes an error code to the
//     runtime's status word and returns, the host reports it at the next sync;
//   * inside a tile, thread (li, lj) owns row (i, j) and at step s updates
//     k = s - li - lj: cell (i,j,k) sees (i-1,j,k), (i,j-1,k), (i,j,k-1) already
//     updated and (i+1,j,k), (i,j+1,k), (i,j,k+1) not yet -- exactly the values
//     the sequential loop order gives it, so every cell is bit-identical.
// The residual SUM of (nv - old)^2 is kept per row chunk as the pairwise tree
// over the chunk's 64 positions (the canonical order the reduction engine
// folds), accumulated in registers as the row advances.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"

namespace {

constexpr int TI = 8, TJ = 8, TK = 64;
constexpr int NT = TI * TJ;              // threads per CTA: one per row of the tile
constexpr int SI = TI + 2, SJ = TJ + 2, SK = TK + 2;
constexpr size_t SMEM = sizeof(double) * SI * SJ * SK;
constexpr long SPIN_LIMIT = 1L << 24;    // ~1-4 s of polling before giving up
constexpr int ERR_SOR_TIMEOUT = 0x50520001;
constexpr long MAX_DIAGS = 2048;         // a + b diagonals (tile grid up to 1024 x 1024 in i, j)

struct Geo {
    long s0, s1;
    long e0, e1, e2;
    long lo0, lo1, lo2, hi0, hi1, hi2;
    long na, nb, nc;  // tiles per axis
    long kc0;         // first k chunk (lo2 / 64)
    long nj;          // rows per i in the item layout
};

__device__ __forceinline__ long tileLinear(const Geo &g, long a, long b, long c) { return (a * g.nb + b) * g.nc + c; }

// Tiles are handed out in the order (a + b, then c, then a): a topological
// order -- (a-1,b,c) and (a,b-1,c) lie on the previous a+b diagonal, (a,b,c-1)
// earlier on the same one -- that keeps whole 2-D diagonals in flight.
// pre[s] = number of tiles before diagonal s (shared memory, built per CTA).
__device__ __forceinline__ long diagLen(long s, long na, long nb) {  // #(a,b), a+b = s
    long amin = s - (nb - 1) > 0 ? s - (nb - 1) : 0;
    long amax = s < na - 1 ? s : na - 1;
    return amax >= amin ? amax - amin + 1 : 0;
}

__device__ void tileAt(const Geo &g, const long *pre, long ns, long idx, long &a, long &b, long &c) {
    long lo = 0, hi = ns - 1;  // last s with pre[s] <= idx
    while (lo < hi) {
        long mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    long sd = lo, len = diagLen(sd, g.na, g.nb), rem = idx - pre[sd];
    c = rem / len;
    long amin = sd - (g.nb - 1) > 0 ? sd - (g.nb - 1) : 0;
    a = amin + rem % len;
    b = sd - a;
}

__device__ __forceinline__ int ldAcquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void stRelease(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(NT) kSorWave(double *A, Geo g, const double *wPtr, int *done, unsigned *counter,
                                               double *items, int *status) {
    extern __shared__ double sm[];  // [SI][SJ][SK], then pre[ns + 1]
    __shared__ long sIdx;
    __shared__ int sFail;
    const int tid = threadIdx.x, li = tid / TJ, lj = tid % TJ;
    const long ntiles = g.na * g.nb * g.nc;
    const long ns = g.na + g.nb - 1;
    long *pre = (long *)(sm + SI * SJ * SK);
    if (tid == 0) {
        long acc = 0;
        for (long sd = 0; sd < ns; sd++) {
            pre[sd] = acc;
            acc += diagLen(sd, g.na, g.nb) * g.nc;
        }
        pre[ns] = acc;
    }
    __syncthreads();
    const double w = *wPtr;
    const double c1 = 1.0 - w, c2 = w / 6.0;  // loop invariants, rounded as in the source expression
    const long nck = g.nc;
    while (true) {
        if (tid == 0) {
            sIdx = (long)atomicAdd(counter, 1u);
            sFail = 0;
        }
        __syncthreads();
        const long idx = sIdx;
        if (idx >= ntiles) break;
        long a, b, c;
        tileAt(g, pre, ns, idx, a, b, c);
        // wait for the face predecessors (bounded)
        if (tid < 3) {
            long pa = a - (tid == 0), pb = b - (tid == 1), pc = c - (tid == 2);
            if (pa >= 0 && pb >= 0 && pc >= 0) {
                const int *f = done + tileLinear(g, pa, pb, pc);
                long n = 0;
                while (ldAcquire(f) == 0) {
                    if (++n > SPIN_LIMIT) {
                        atomicExch(status, ERR_SOR_TIMEOUT);
                        sFail = 1;
                        break;
                    }
                    __nanosleep(64);
                }
            }
        }
        __syncthreads();
        if (sFail) return;
        const long i0 = g.lo0 + a * TI, j0 = g.lo1 + b * TJ, kb = (g.kc0 + c) * TK;
        // stage tile + halo (reads through L2: producers are other SMs)
        for (int q = tid; q < SI * SJ * SK; q += NT) {
            int qk = q % SK, qj = (q / SK) % SJ, qi = q / (SK * SJ);
            long i = i0 - 1 + qi, j = j0 - 1 + qj, k = kb - 1 + qk;
            double v = 0.0;
            if (i >= 0 && i < g.e0 && j >= 0 && j < g.e1 && k >= 0 && k < g.e2) v = __ldcg(A + i * g.s0 + j * g.s1 + k);
            sm[q] = v;
        }
        __syncthreads();
        const long i = i0 + li, j = j0 + lj;
        const bool row = i <= g.hi0 && j <= g.hi1;
        double p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0, root = -0.0;  // pairwise-tree stack
        double *cen = sm + ((li + 1) * SJ + (lj + 1)) * SK + 1;              // k = kb at cen[0]
        for (int s = 0; s < TK + TI + TJ - 2; s++) {
            const int p = s - li - lj;
            if (row && p >= 0 && p < TK) {
                const long k = kb + p;
                double term = -0.0;  // identity of positions outside the loop
                if (k >= g.lo2 && k <= g.hi2) {
                    double *x = cen + p;
                    double old = x[0];
                    // A[i-1] + A[i+1] + A[j-1] + A[j+1] + A[k-1] + A[k+1], left to right
                    double sum = ((((x[-SJ * SK] + x[SJ * SK]) + x[-SK]) + x[SK]) + x[-1]) + x[1];
                    double nv = c1 * old + c2 * sum;
                    x[0] = nv;
                    double dlt = nv - old;
                    term = dlt * dlt;
                }
                // pairwise tree over positions 0..63 of the chunk, in order
                double v = term;
                if (p & 1) {
                    v = p0 + v;
                    if (p & 2) {
                        v = p1 + v;
                        if (p & 4) {
                            v = p2 + v;
                            if (p & 8) {
                                v = p3 + v;
                                if (p & 16) {
                                    v = p4 + v;
                                    if (p & 32) root = p5 + v;
                                    else p5 = v;
                                } else p4 = v;
                            } else p3 = v;
                        } else p2 = v;
                    } else p1 = v;
                } else p0 = v;
            }
            __syncthreads();
        }
        // write the tile's updated cells (coalesced along k)
        for (int q = tid; q < TI * TJ * TK; q += NT) {
            int qk = q % TK, qj = (q / TK) % TJ, qi = q / (TK * TJ);
            long ii = i0 + qi, jj = j0 + qj, k = kb + qk;
            if (ii <= g.hi0 && jj <= g.hi1 && k >= g.lo2 && k <= g.hi2)
                A[ii * g.s0 + jj * g.s1 + k] = sm[((qi + 1) * SJ + (qj + 1)) * SK + qk + 1];
        }
        if (row) items[((i - g.lo0) * g.nj + (j - g.lo1)) * nck + c] = root;
        __threadfence();
        __syncthreads();
        if (tid == 0) stRelease(done + tileLinear(g, a, b, c), 1);
    }
}

bool geo(const long st[3], const long ext[3], const long lo[3], const long hi[3], Geo &g) {
    if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2] || lo[2] < 0 || st[2] != 1) return false;
    g.s0 = st[0];
    g.s1 = st[1];
    g.e0 = ext[0];
    g.e1 = ext[1];
    g.e2 = ext[2];
    g.lo0 = lo[0];
    g.lo1 = lo[1];
    g.lo2 = lo[2];
    g.hi0 = hi[0];
    g.hi1 = hi[1];
    g.hi2 = hi[2];
    g.na = (hi[0] - lo[0] + TI) / TI;
    g.nb = (hi[1] - lo[1] + TJ) / TJ;
    g.kc0 = lo[2] / TK;
    g.nc = hi[2] / TK - g.kc0 + 1;
    g.nj = hi[1] - lo[1] + 1;
    return true;
}

}  // namespace

extern "C" {

long dvmhgb_sor3d_items(const long lo[3], const long hi[3]) {
    return (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] / TK - lo[2] / TK + 1);
}

long dvmhgb_sor3d_scratch_bytes(const long lo[3], const long hi[3]) {
    long ntiles = ((hi[0] - lo[0] + TI) / TI) * ((hi[1] - lo[1] + TJ) / TJ) * (hi[2] / TK - lo[2] / TK + 1);
    return (ntiles + 64) * (long)sizeof(int);
}

int dvmhgb_sor3d_sweep(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3],
                       const double *wDev, double *items, void *scratch, int *status, void *stream) {
    Geo g;
    if (!A || !wDev || !items || !scratch || !status || !geo(st, ext, lo, hi, g)) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    long ntiles = g.na * g.nb * g.nc;
    unsigned *counter = (unsigned *)scratch;
    int *done = (int *)scratch + 64;  // counter on its own 256-byte line
    const long ns = g.na + g.nb - 1;
    if (ns > MAX_DIAGS) return -1;
    const size_t smem = SMEM + sizeof(long) * (MAX_DIAGS + 1);
    if (cudaMemsetAsync(scratch, 0, (size_t)(ntiles + 64) * sizeof(int), s) != cudaSuccess) return -1;
    static int occ = 0, sms = 0;
    if (!occ) {
        cudaFuncSetAttribute(kSorWave, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kSorWave, NT, smem);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (occ < 1) occ = 1;
    }
    long grid = (long)occ * sms;  // all CTAs resident at once: waits always resolve
    if (grid > ntiles) grid = ntiles;
    kSorWave<<<(unsigned)grid, NT, smem, s>>>(A, g, wDev, done, counter, items, status);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // extern "C"
