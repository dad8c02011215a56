// ACROSS loop kernel for sm_103a: SOR / Gauss-Seidel 3-D with dependences
// (1:1, 1:1, 1:1), executed as a persistent tiled wavefront.
//
// The reference runs such a loop as one kernel launch per hyperplane from the
// host (cdvmh/src/across.cpp:2480-2760: three diagonal phases, ~3n launches per
// sweep).  Here one launch covers the sweep:
//   * the loop box is cut into 4 x 8 x TK tiles (TK = 32, 16 or 8: the loop
//     variant), the k ranges aligned to 64 / TK parts of the 64-wide chunks of
//     the array index; one warp works a tile (no CTA-wide barrier), several
//     tile-warps share a CTA;
//   * a tile depends only on its three face predecessors (a-1,b,c), (a,b-1,c),
//     (a,b,c-1) -- the 7-point stencil touches face neighbours only;
//   * tiles are handed out by an atomic counter plane by plane (a + b + c, a
//     topological order), the grid is no larger than the GPU holds at once, so
//     every tile a warp waits for is already owned by a running warp: progress
//     is guaranteed;
//   * every wait is bounded: past the limit the warp writes an error code to the
//     runtime's status word, stops the tile counter and returns; the host
//     reports it at the next sync;
//   * a tile stages its own cells and its +1 faces before it waits (no tile
//     writes them earlier), and the -1 faces once its predecessors are done,
//     each row with one coalesced load;
//   * inside a tile, lane (li, lj) owns row (i, j) and at step s updates
//     k = s - li - lj: cell (i,j,k) sees (i-1,j,k), (i,j-1,k), (i,j,k-1) already
//     updated and (i+1,j,k), (i,j+1,k), (i,j,k+1) not yet -- exactly the values
//     the sequential loop order gives it, so every cell is bit-identical.
// The critical path of a sweep is (tiles along i + j + k) x (TK + TI + TJ - 2)
// steps of a 7-deep FP64 chain; a smaller TK shortens it at the price of idle
// lanes in the skew.  Only the update runs on the skewed steps: the residual
// SUM of (nv - old)^2 of a row part (the pairwise tree over its TK positions)
// is formed after the tile has released its successors, from the saved old
// values.  Items are laid out (row, chunk, part), so the reduction engine's
// pairwise fold over items first joins the parts of each 64-position chunk:
// the result is the canonical chunk tree, then the canonical tree over chunks.
// The default tiles (variants 4 and 5, at the end of this file) are cut along
// the hyperplanes i + j + k instead, so that no lane idles on the skew.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"
#include "devinfo.cuh"

namespace {

// one warp works on one 4 x 8 x TK tile: lane (li, lj) owns row (i0+li, j0+lj)
constexpr int TI = 4, TJ = 8;
constexpr int WPB = 4;                   // independent tile-warps per CTA
constexpr int NT = 32 * WPB;
constexpr int SI = TI + 2, SJ = TJ + 2;
template <int TK>
struct Tile {
    static constexpr int SK = TK + 2;
    static constexpr int BOX = SI * SJ * SK;     // doubles of one warp's tile + halo
    static constexpr int OSTR = TK + 1;          // a lane's saved old values (padded: no bank conflicts)
    static constexpr int WSM = BOX + 32 * OSTR;  // doubles of shared memory per warp
    static constexpr size_t SMEM = sizeof(double) * WSM * WPB;
    static constexpr int RPL = 32 / TK;          // rows per warp load
    static constexpr int LOG = TK == 32 ? 5 : (TK == 16 ? 4 : 3);
};
constexpr long SPIN_LIMIT = 1L << 24;    // default polls before giving up: ~1-4 s

// How long a wavefront launch waits: every wait for a predecessor polls at
// most pollLimit times; the hand-out of tiles (columns) starts at firstIndex
// (0 in every sweep the runtime runs; tests start later so that a wait expires)
struct Bound {
    long pollLimit;
    unsigned firstIndex;
};
constexpr int ERR_SOR_TIMEOUT = 0x50520001;
constexpr int MAX_PLANES = 1536;         // a + b + c planes of the tile grid

struct Geo {
    long s0, s1;
    long e0, e1, e2;
    long lo0, lo1, lo2, hi0, hi1, hi2;
    long na, nb, nc;  // tiles per axis
    long kc0;         // first k tile (PARTS * (lo2 / 64): tiles are chunk parts)
    long nj;          // rows per i in the item layout
};

__device__ __forceinline__ long tileLinear(const Geo &g, long a, long b, long c) { return (a * g.nb + b) * g.nc + c; }

// Tiles are handed out plane by plane, d = a + b + c (a topological order: the
// three predecessors lie on plane d - 1), inside a plane by c, then a.  So the
// tiles held at any time are those of the current wavefront, all close to
// ready.  Plane sizes follow from inclusion-exclusion over the box
// [0,na) x [0,nb) x [0,nc):
//   #{x,y,z >= 0 : x+y+z = m} = (m+1)(m+2)/2,  #{... : x+y+z < m} = m(m+1)(m+2)/6.
__device__ __forceinline__ long long below3(long long m) { return m > 0 ? m * (m + 1) * (m + 2) / 6 : 0; }
__device__ __forceinline__ int on3(int m) { return m >= 0 ? (m + 1) * (m + 2) / 2 : 0; }

// number of box points with a + b + c < d
__device__ long long planesBefore(long long d, long long na, long long nb, long long nc) {
    return below3(d) - below3(d - na) - below3(d - nb) - below3(d - nc) + below3(d - na - nb) + below3(d - na - nc) +
           below3(d - nb - nc) - below3(d - na - nb - nc);
}

// number of points (a, b, c') of plane d with c' < c
__device__ __forceinline__ int onPlane(int d, int na, int nb, int c) {
    return on3(d) - on3(d - na) - on3(d - nb) - on3(d - c) + on3(d - na - nb) + on3(d - na - c) + on3(d - nb - c) -
           on3(d - na - nb - c);
}

// pre[d] = tiles before plane d (shared, built per CTA); all lanes of a warp call this
__device__ void tileAt(const Geo &g, const int *pre, int np, long idx, int lane, long &a, long &b, long &c) {
    int lo = 0, hi = np - 1;  // last plane with pre[d] <= idx
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    const int d = lo, rem = (int)(idx - pre[d]), na = (int)g.na, nb = (int)g.nb, nc = (int)g.nc;
    // c = the last c with onPlane(d, c) <= rem, 32 candidates per round
    int cc = 0;
    for (int c0 = 0; c0 < nc; c0 += 32) {
        const int cand = c0 + lane;
        const bool past = cand >= nc || onPlane(d, na, nb, cand + 1) > rem;
        const unsigned m = __ballot_sync(0xffffffffu, past);
        if (m) {
            cc = c0 + __ffs(m) - 1;
            break;
        }
    }
    c = cc;
    const long sd = d - cc, amin = sd - (g.nb - 1) > 0 ? sd - (g.nb - 1) : 0;
    a = amin + (rem - onPlane(d, na, nb, cc));
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

__device__ __forceinline__ double ldCell(const double *A, const Geo &g, long i, long j, long k) {
    return (i >= 0 && i < g.e0 && j >= 0 && j < g.e1 && k >= 0 && k < g.e2) ? __ldcg(A + i * g.s0 + j * g.s1 + k)
                                                                             : 0.0;
}

// Box rows (qi, qj) are TK + 2 doubles along k; a warp load brings the TK
// interior ones (k = kb + lane % TK) of 32 / TK rows, the k faces take one load
// per lane.  Before the wait: the own rows and the +i / +j face rows (qi, qj >=
// 1), and the +k face of the own rows -- no tile writes them before this one
// is done.
template <int TK>
__device__ __forceinline__ void stageOwn(double *box, const double *A, const Geo &g, long i0, long j0, long kb,
                                         int lane) {
    using T = Tile<TK>;
    constexpr int NR = (SI - 1) * (SJ - 1), NL = (NR + T::RPL - 1) / T::RPL;
    const int sub = lane / TK, kk = lane % TK;
    double v[NL];
#pragma unroll
    for (int u = 0; u < NL; u++) {
        const int r = u * T::RPL + sub, qi = 1 + r / (SJ - 1), qj = 1 + r % (SJ - 1);
        v[u] = r < NR ? ldCell(A, g, i0 - 1 + qi, j0 - 1 + qj, kb + kk) : 0.0;
    }
    const int li = lane / TJ, lj = lane % TJ;
    const double kf = ldCell(A, g, i0 + li, j0 + lj, kb + TK);
#pragma unroll
    for (int u = 0; u < NL; u++) {
        const int r = u * T::RPL + sub, qi = 1 + r / (SJ - 1), qj = 1 + r % (SJ - 1);
        if (r < NR) box[(qi * SJ + qj) * T::SK + 1 + kk] = v[u];
    }
    box[((li + 1) * SJ + lj + 1) * T::SK + T::SK - 1] = kf;
}

// After the wait: the -i, -j and -k faces, written by the predecessors.
template <int TK>
__device__ __forceinline__ void stageFaces(double *box, const double *A, const Geo &g, long i0, long j0, long kb,
                                           int lane) {
    using T = Tile<TK>;
    constexpr int NR = TJ + TI, NL = (NR + T::RPL - 1) / T::RPL;  // rows (0, 1..TJ), then (1..TI, 0)
    const int sub = lane / TK, kk = lane % TK;
    double v[NL];
#pragma unroll
    for (int u = 0; u < NL; u++) {
        const int r = u * T::RPL + sub, qi = r < TJ ? 0 : r - TJ + 1, qj = r < TJ ? r + 1 : 0;
        v[u] = r < NR ? ldCell(A, g, i0 - 1 + qi, j0 - 1 + qj, kb + kk) : 0.0;
    }
    const int li = lane / TJ, lj = lane % TJ;
    const double kf = ldCell(A, g, i0 + li, j0 + lj, kb - 1);
#pragma unroll
    for (int u = 0; u < NL; u++) {
        const int r = u * T::RPL + sub, qi = r < TJ ? 0 : r - TJ + 1, qj = r < TJ ? r + 1 : 0;
        if (r < NR) box[(qi * SJ + qj) * T::SK + 1 + kk] = v[u];
    }
    box[((li + 1) * SJ + lj + 1) * T::SK] = kf;
}

template <int TK>
__global__ void __launch_bounds__(NT) kSorWave(double *A, Geo g, const double *wPtr, int *done, unsigned *counter,
                                               double *items, int *status, Bound bound) {
    using T = Tile<TK>;
    constexpr int SK = T::SK;
    extern __shared__ double sm[];  // per warp: box [SI][SJ][SK] + olds [32][OSTR]; then pre[np + 1]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, li = lane / TJ, lj = lane % TJ;
    const long ntiles = g.na * g.nb * g.nc;
    const int np = (int)(g.na + g.nb + g.nc - 2);
    int *pre = (int *)(sm + (size_t)T::WSM * WPB);
    for (int d = threadIdx.x; d <= np; d += NT) pre[d] = (int)planesBefore(d, g.na, g.nb, g.nc);
    __syncthreads();  // the only CTA-wide barrier: from here every warp runs on its own
    double *box = sm + (size_t)T::WSM * warp;
    double *olds = box + T::BOX + lane * T::OSTR;
    const double w = *wPtr;
    const double c1 = 1.0 - w, c2 = w / 6.0;  // loop invariants, rounded as in the source expression
    const long nck = g.nc;
    while (true) {
        long idx = 0;
        if (lane == 0) idx = (long)atomicAdd(counter, 1u) + bound.firstIndex;  // >= 2^31 once a warp has failed
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= ntiles) break;
        long a, b, c;
        tileAt(g, pre, np, idx, lane, a, b, c);
        const long i0 = g.lo0 + a * TI, j0 = g.lo1 + b * TJ, kb = (g.kc0 + c) * TK;
        // 1. own cells and the +1 faces: nobody writes them before this tile is done
        stageOwn<TK>(box, A, g, i0, j0, kb, lane);
        // 2. wait for the face predecessors (bounded)
        int fail = 0;
        if (lane < 3) {
            long pa = a - (lane == 0), pb = b - (lane == 1), pc = c - (lane == 2);
            if (pa >= 0 && pb >= 0 && pc >= 0) {
                const int *f = done + tileLinear(g, pa, pb, pc);
                long n = 0;
                while (ldAcquire(f) == 0) {
                    if (++n > bound.pollLimit) {
                        atomicExch(status, ERR_SOR_TIMEOUT);
                        atomicOr(counter, 0x80000000u);  // no warp takes another tile
                        fail = 1;
                        break;
                    }
                    __nanosleep(64);
                }
            }
        }
        if (__any_sync(0xffffffffu, fail)) return;
        __syncwarp();  // orders the acquiring lanes' loads before every lane's face loads
        // 3. the -1 faces, written by the predecessors (through L2)
        stageFaces<TK>(box, A, g, i0, j0, kb, lane);
        __syncwarp();
        const long i = i0 + li, j = j0 + lj;
        const bool row = i <= g.hi0 && j <= g.hi1;
        double *cen = box + ((li + 1) * SJ + (lj + 1)) * SK + 1;  // k = kb at cen[0]
        // the dependent chain: only the update itself runs on the skewed steps
        for (int st = 0; st < TK + TI + TJ - 2; st++) {
            const int p = st - li - lj;
            const long k = kb + p;
            if (row && p >= 0 && p < TK && k >= g.lo2 && k <= g.hi2) {
                double *x = cen + p;
                double old = x[0];
                // A[i-1] + A[i+1] + A[j-1] + A[j+1] + A[k-1] + A[k+1], left to right
                double sum = ((((x[-SJ * SK] + x[SJ * SK]) + x[-SK]) + x[SK]) + x[-1]) + x[1];
                x[0] = c1 * old + c2 * sum;
                olds[p] = old;
            }
            __syncwarp();
        }
        // write the tile's updated cells (coalesced along k)
        for (int q = lane; q < TI * TJ * TK; q += 32) {
            int qk = q % TK, qj = (q / TK) % TJ, qi = q / (TK * TJ);
            long ii = i0 + qi, jj = j0 + qj, k = kb + qk;
            if (ii <= g.hi0 && jj <= g.hi1 && k >= g.lo2 && k <= g.hi2)
                A[ii * g.s0 + jj * g.s1 + k] = box[((qi + 1) * SJ + (qj + 1)) * SK + qk + 1];
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) stRelease(done + tileLinear(g, a, b, c), 1);
        // the residual, off the chain: successors already run.  Every lane is at
        // the same position p, so the pairwise tree over the TK positions of the
        // row part takes warp-uniform branches.
        double stk[T::LOG], root = -0.0;
#pragma unroll
        for (int p = 0; p < TK; p++) {
            const long k = kb + p;
            double v = -0.0;  // identity of positions outside the loop
            if (row && k >= g.lo2 && k <= g.hi2) {
                double dlt = cen[p] - olds[p];
                v = dlt * dlt;
            }
            // pairwise: position p closes the subtrees of its trailing one bits
#pragma unroll
            for (int l = 0; l < T::LOG; l++) {
                if (!((p >> l) & 1)) {
                    stk[l] = v;
                    break;
                }
                v = stk[l] + v;
            }
            if (p == TK - 1) root = v;
        }
        if (row) items[((i - g.lo0) * g.nj + (j - g.lo1)) * nck + c] = root;
        __syncwarp();  // the box and olds are reused by this warp's next tile
    }
}

bool geo(const long st[3], const long ext[3], const long lo[3], const long hi[3], int parts, Geo &g) {
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
    g.kc0 = parts * (lo[2] / 64);
    g.nc = parts * (hi[2] / 64 - lo[2] / 64 + 1);
    g.nj = hi[1] - lo[1] + 1;
    return true;
}

// variant -> TK: 0 -> 32, 1 -> 16, 2 -> 8; 3: streaming columns (items as for TK = 64: one per 64-wide chunk);
// 4, 5: hyperplane tiles of G = 8 hyperplanes, 4 x 8 rows per warp or 16 x 8 rows per CTA (items as for TK = 8)
int tkOf(int variant) {
    static const int tk[6] = {32, 16, 8, 64, 8, 8};
    return variant >= 0 && variant < 6 ? tk[variant] : 0;
}

template <int TK>
int sweepT(double *A, const Geo &g, const double *wDev, double *items, void *scratch, int *status, Bound bound,
           cudaStream_t s) {
    using T = Tile<TK>;
    const long ntiles = g.na * g.nb * g.nc;
    unsigned *counter = (unsigned *)scratch;
    int *done = (int *)scratch + 64;  // counter on its own 256-byte line
    if (g.na + g.nb + g.nc - 2 > MAX_PLANES || ntiles >= (1L << 30)) return -1;
    const size_t smem = T::SMEM + sizeof(int) * (MAX_PLANES + 1);  // one size for every launch (occupancy cached)
    if (cudaMemsetAsync(scratch, 0, (size_t)(ntiles + 64) * sizeof(int), s) != cudaSuccess) return -1;
    static std::atomic<int> occCache[gbdev::MAX_DEVICES];
    const int occ = gbdev::residentCtas(occCache, kSorWave<TK>, NT, smem);
    long grid = (long)occ * gbdev::smCount();  // all CTAs resident at once: waits always resolve
    long gridCap = (ntiles + WPB - 1) / WPB;
    if (grid > gridCap) grid = gridCap;
    kSorWave<TK><<<(unsigned)grid, NT, smem, s>>>(A, g, wDev, done, counter, items, status, bound);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------- streaming columns (variant 3)
//
// One warp owns a column of 4 x 8 rows (lane (li, lj) -> row (i0 + li, j0 + lj))
// and streams it along k: at step s lane (li, lj) updates position
// p = s - li - lj, so a cell sees its -i / -j / -k neighbours new and its
// +i / +j / +k neighbours old, the values the sequential order gives it.
// Neighbour rows inside the column come by warp shuffles: the new value a lane
// computed one step earlier (-i, -j) and the old value a lane holds one
// position ahead (+i, +j).  The column's -i / -j faces are the last rows of
// the predecessor columns (a-1, b) and (a, b-1), read through L2 once they are
// published; its +i / +j faces are old values.  Every SC steps a column
// publishes how many leading positions all its rows have stored (after a
// fence); a successor waits (bounded) for the positions it reads.  A column
// has one skew ramp for the whole sweep, where a tile has one per TK
// positions: on GB300 an FP64 warp instruction costs the same whatever its
// active lanes, so the ramps were a third of the tiles' update instructions.
// Residual: every lane keeps (nv - old)^2 of its recent positions in shared
// memory; after each group the positions all lanes have finished enter the
// canonical pairwise tree of their 64-wide chunk, with every lane at the same
// position (warp-uniform branches).  One item per row and 64-wide chunk.
constexpr int SC = 16;            // steps per group (publication granularity)
constexpr int SKEW = TI + TJ - 2;  // the last lane's lag behind lane 0
constexpr int SQR = 32;           // positions of squares kept per lane (>= SC + SKEW)
constexpr int SWPB = 4;           // column-warps per CTA
constexpr int SNT = 32 * SWPB;

struct SGeo {
    long s0, s1;
    long e0, e1, e2;
    long lo0, lo1, lo2, hi0, hi1, hi2;
    long na, nb, nk;  // columns along i and j; positions along k
    long nj;          // rows per i in the item layout
    long kc0, nch;    // first 64-wide chunk of k; chunks per row
};

// columns are handed out by diagonal d = a + b; #{(a, b) in box : a + b < d}
__device__ __forceinline__ long long below2(long long m) { return m > 0 ? m * (m + 1) / 2 : 0; }
__device__ __forceinline__ void colAt(const SGeo &g, long idx, long &a, long &b) {
    long lo = 0, hi = g.na + g.nb - 2;  // last d with count(< d) <= idx
    while (lo < hi) {
        const long mid = (lo + hi + 1) >> 1;
        const long long c = below2(mid) - below2(mid - g.na) - below2(mid - g.nb) + below2(mid - g.na - g.nb);
        if (c <= idx) lo = mid;
        else hi = mid - 1;
    }
    const long d = lo;
    const long long before = below2(d) - below2(d - g.na) - below2(d - g.nb) + below2(d - g.na - g.nb);
    const long amin = d - (g.nb - 1) > 0 ? d - (g.nb - 1) : 0;
    a = amin + (idx - (long)before);
    b = d - a;
}

__device__ __forceinline__ double ldAt(const double *A, const SGeo &g, long i, long j, long k) {
    return (i >= 0 && i < g.e0 && j >= 0 && j < g.e1 && k >= 0 && k < g.e2) ? __ldcg(A + i * g.s0 + j * g.s1 + k)
                                                                             : 0.0;
}

// bounded wait until *f >= want; false (status written, counter stopped) when it runs out
__device__ __forceinline__ bool waitProgress(const int *f, int want, int *status, unsigned *counter, long limit) {
    long n = 0;
    while (ldAcquire(f) < want) {
        if (++n > limit) {
            atomicExch(status, ERR_SOR_TIMEOUT);
            atomicOr(counter, 0x80000000u);
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

__global__ void __launch_bounds__(SNT) kSorStream(double *A, SGeo g, const double *wPtr, int *prog, unsigned *counter,
                                                  double *items, int *status, Bound bound) {
    __shared__ double sqs[SWPB][32][SQR + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, li = lane / TJ, lj = lane % TJ, sk = li + lj;
    double *sq = sqs[warp][lane];
    const double w = *wPtr;
    const double c1 = 1.0 - w, c2 = w / 6.0;  // loop invariants, rounded as in the source expression
    const long ncols = g.na * g.nb;
    const int nk = (int)g.nk;
    while (true) {
        long idx = 0;
        if (lane == 0) idx = (long)atomicAdd(counter, 1u) + bound.firstIndex;  // >= 2^31 once a warp has failed
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= ncols) break;
        long a, b;
        colAt(g, idx, a, b);
        const long i = g.lo0 + a * TI + li, j = g.lo1 + b * TJ + lj;
        const bool row = i <= g.hi0 && j <= g.hi1;
        // the faces a boundary lane reads: -i / +i (li = 0 / TI-1), -j / +j (lj = 0 / TJ-1)
        const long fi = li == 0 ? i - 1 : i + 1, fj = lj == 0 ? j - 1 : j + 1;
        const bool hasFi = li == 0 || li == TI - 1, hasFj = lj == 0 || lj == TJ - 1;
        const int *predI = a > 0 ? prog + (a - 1) * g.nb + b : nullptr;
        const int *predJ = b > 0 ? prog + a * g.nb + (b - 1) : nullptr;
        double res = ldAt(A, g, i, j, g.lo2 - 1);  // the value at the position before p: the k - 1 neighbour
        double stk[6];
#pragma unroll
        for (int l = 0; l < 6; l++) stk[l] = -0.0;
        int done = 0;  // positions whose squares have entered the trees
        const int G = (nk + SKEW + SC - 1) / SC;
        for (int gr = 0; gr < G; gr++) {
            const int p0 = gr * SC - sk;  // this lane's first position in the group
            // 1. the predecessors' rows up to the group's last position (lane (0, 0) reaches gr*SC + SC - 1)
            const int want = min(nk, gr * SC + SC);
            int fail = 0;
            if (lane == 0 && predI && !waitProgress(predI, want, status, counter, bound.pollLimit)) fail = 1;
            if (lane == 1 && predJ && !waitProgress(predJ, want, status, counter, bound.pollLimit)) fail = 1;
            if (__any_sync(0xffffffffu, fail)) return;
            __syncwarp();  // orders the acquiring lanes' loads before every lane's face loads
            // 2. the group's values: own row positions p0 .. p0 + SC (one ahead), the faces p0 .. p0 + SC - 1
            double own[SC + 1], fI[SC], fJ[SC];
#pragma unroll
            for (int u = 0; u <= SC; u++) own[u] = ldAt(A, g, i, j, g.lo2 + p0 + u);
#pragma unroll
            for (int u = 0; u < SC; u++) {
                fI[u] = hasFi ? ldAt(A, g, fi, j, g.lo2 + p0 + u) : 0.0;
                fJ[u] = hasFj ? ldAt(A, g, i, fj, g.lo2 + p0 + u) : 0.0;
            }
            // 3. the steps
#pragma unroll
            for (int u = 0; u < SC; u++) {
                const int p = p0 + u;
                const double cur = own[u], nxt = own[u + 1];
                const double upI = __shfl_up_sync(0xffffffffu, res, TJ), dnI = __shfl_down_sync(0xffffffffu, nxt, TJ);
                const double upJ = __shfl_up_sync(0xffffffffu, res, 1), dnJ = __shfl_down_sync(0xffffffffu, nxt, 1);
                const double xim = li == 0 ? fI[u] : upI, xip = li == TI - 1 ? fI[u] : dnI;
                const double xjm = lj == 0 ? fJ[u] : upJ, xjp = lj == TJ - 1 ? fJ[u] : dnJ;
                if (row && p >= 0 && p < nk) {
                    // A[i-1] + A[i+1] + A[j-1] + A[j+1] + A[k-1] + A[k+1], left to right
                    const double sum = ((((xim + xip) + xjm) + xjp) + res) + nxt;
                    const double nv = c1 * cur + c2 * sum;
                    A[i * g.s0 + j * g.s1 + g.lo2 + p] = nv;
                    const double dl = nv - cur;
                    sq[p & (SQR - 1)] = dl * dl;
                    res = nv;
                } else {
                    res = cur;
                }
            }
            // 4. publish the positions every row has stored
            const int fin = min(nk, max(0, gr * SC + SC - SKEW));
            __threadfence();
            __syncwarp();
            if (lane == 0) stRelease(prog + a * g.nb + b, gr == G - 1 ? nk : fin);
            // 5. the residual of the finished positions, every lane at the same position
            const int upto = gr == G - 1 ? nk : fin;
            for (; done < upto; done++) {
                const long k = g.lo2 + done;
                const int q = (int)(k & 63);
                double v = row ? sq[done & (SQR - 1)] : -0.0;
#pragma unroll
                for (int l = 0; l < 6; l++) {
                    if (!((q >> l) & 1)) {
                        stk[l] = v;
                        break;
                    }
                    v = stk[l] + v;
                }
                if (q == 63 || done == nk - 1) {
                    // the chunk's remaining positions are the identity: complete its tree
                    double root = v;
                    if (q != 63) {
                        root = -0.0;
                        for (int qq = q + 1; qq <= 63; qq++) {
                            double x = -0.0;
                            for (int l = 0; l < 6; l++) {
                                if (!((qq >> l) & 1)) {
                                    stk[l] = x;
                                    break;
                                }
                                x = stk[l] + x;
                            }
                            root = x;
                        }
                    }
                    if (row) items[((i - g.lo0) * g.nj + (j - g.lo1)) * g.nch + ((k >> 6) - g.kc0)] = root;
#pragma unroll
                    for (int l = 0; l < 6; l++) stk[l] = -0.0;
                }
            }
            __syncwarp();
        }
    }
}

int sweepStream(double *A, const Geo &g0, const double *wDev, double *items, void *scratch, int *status,
                Bound bound, cudaStream_t s) {
    SGeo g;
    g.s0 = g0.s0;
    g.s1 = g0.s1;
    g.e0 = g0.e0;
    g.e1 = g0.e1;
    g.e2 = g0.e2;
    g.lo0 = g0.lo0;
    g.lo1 = g0.lo1;
    g.lo2 = g0.lo2;
    g.hi0 = g0.hi0;
    g.hi1 = g0.hi1;
    g.hi2 = g0.hi2;
    g.na = g0.na;
    g.nb = g0.nb;
    g.nk = g0.hi2 - g0.lo2 + 1;
    g.nj = g0.nj;
    g.kc0 = g0.lo2 / 64;
    g.nch = g0.hi2 / 64 - g0.lo2 / 64 + 1;
    const long ncols = g.na * g.nb;
    if (ncols >= (1L << 30) || g.nk >= (1L << 30) || g.lo2 < 1) return -1;
    unsigned *counter = (unsigned *)scratch;
    int *prog = (int *)scratch + 64;  // counter on its own 256-byte line
    if (cudaMemsetAsync(scratch, 0, (size_t)(ncols + 64) * sizeof(int), s) != cudaSuccess) return -1;
    static std::atomic<int> occCache[gbdev::MAX_DEVICES];
    const int occ = gbdev::residentCtas(occCache, kSorStream, SNT, 0);
    long grid = (long)occ * gbdev::smCount();  // all CTAs resident at once: waits always resolve
    const long gridCap = (ncols + SWPB - 1) / SWPB;
    if (grid > gridCap) grid = gridCap;
    kSorStream<<<(unsigned)grid, SNT, 0, s>>>(A, g, wDev, prog, counter, items, status, bound);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------- hyperplane tiles (variants 4 and 5)
//
// The tiles above are boxes: inside one, lane (li, lj) starts li + lj steps
// late, so a 4 x 8 x TK tile takes TK + 10 steps for TK positions per lane, and
// on GB300 an FP64 warp instruction costs the same whatever its active lanes.
// Here a tile is cut along hyperplanes instead.  With (ri, rj, rk) the cell's
// offsets from the loop box's low corner and h = ri + rj + rk its hyperplane,
// tile (a, b, c) holds rows ri = 4a .. 4a + 3, rj = 8b .. 8b + 7 and the cells
// of those rows with h in [G c, G c + G).  Lane (li, lj) takes, at step t, the
// cell of its row on hyperplane G c + t: every lane is busy at every step
// (except where a row's window leaves the loop box), and the step order is the
// skewed order of the box tiles, so every cell sees exactly the values the
// sequential loop gives it.  A cell (ri, rj, rk) on hyperplane h reads the new
// values of (ri-1, rj, rk), (ri, rj-1, rk), (ri, rj, rk-1), all on h - 1: so
// tile (a, b, c) depends on (a-1, b, c), (a-1, b, c-1), (a, b-1, c),
// (a, b-1, c-1) and (a, b, c-1), all on plane a + b + c - 1 or lower.  Column
// (a, b) holds the tiles c = cmin .. cmax that meet the loop box; a small
// kernel lists them plane by plane (a + b + c, then c, then a) before the sweep,
// and the sweep hands them out in that order (topological: progress as above).
//
// Shared memory holds, per row of the tile and of its four face neighbours, a
// window of the row's positions h - ri - rj - 1 .. for h = G c - 1 .. G c + G:
// position p of the window is hyperplane G c - 1 + p of the row.  Row i - 1 is
// read at p = t, row i + 1 at p = t + 2 (the same for j), the row itself at
// t, t + 1, t + 2.
//
// Residual: the canonical tree wants, per row, the pairwise sum of every
// G-position part of the array index k (parts aligned to multiples of G,
// positions outside the loop -0.0).  A lane's window [k0, k0 + G) covers the
// tail of one part and the head of the next; the offset dl = k0 mod G is the
// same for every window of the row.  Each step keeps nv - old; the lane stores
// the differences of its last dl positions (the next part's head) for the
// row's next window before the tile releases its successors -- tile (a, b,
// c + 1) waits for this tile anyway and loads them with its -1 faces -- and,
// after the release, squares the carried and its own differences into the
// part it closes.  The first window of a row writes -0.0 for the parts before
// it, the last one closes the next part and writes -0.0 for the rest.

template <int G>
struct Hyp {
    static constexpr int SKP = G + 3;                  // window: positions 0 .. G + 1 (odd stride: banks)
    static constexpr int BOX = SI * SJ * SKP;
    static constexpr int SQS = 2 * G + 1;              // leaves of two parts per lane (padded)
    static constexpr int WSM = BOX + 32 * SQS;         // doubles of shared memory per warp
    static constexpr size_t SMEM = sizeof(double) * WSM * WPB;
    static constexpr int PARTS = 64 / G;
    static constexpr int LOG = G == 16 ? 4 : 3;
};

struct HGeo {
    long s0, s1;
    long e0, e1, e2;
    long lo0, lo1, lo2, hi0, hi1, hi2;
    long na, nb, nk;
    long ncg;         // tiles of the longest column: c < ncg
    long nj;          // rows per i in the item layout
    long kc0, nparts; // first part (of the whole array's k) with items; items per row
    long ntiles, nlev;
    long rows;        // rows of the loop box: (hi0 - lo0 + 1) * nj
    long ti, tj;      // rows of a tile along i and j
};

// the first and last tile of column (a, b): the hyperplanes its rows' cells lie on
template <int G>
__host__ __device__ __forceinline__ long hypCmin(const HGeo &g, long a, long b) {
    return (g.ti * a + g.tj * b) / G;
}
template <int G>
__host__ __device__ __forceinline__ long hypCmax(const HGeo &g, long a, long b) {
    return (g.ti * a + g.tj * b + g.ti + g.tj - 2 + g.nk - 1) / G;
}

__device__ __forceinline__ unsigned long long hypPack(long a, long b, long c) {
    return ((unsigned long long)a << 42) | ((unsigned long long)b << 21) | (unsigned long long)c;
}

// One CTA per plane d: the plane's first index (tiles on planes < d, summed
// over the columns in closed form) and its tiles in the order (c, then a).
// Thread u takes the diagonal s = a + b = smax - u of the plane (c = d - s:
// ascending with u), counts its tiles, and writes them, a ascending, at its
// place in the CTA's scan.
template <int G>
__global__ void __launch_bounds__(256) kHypTable(HGeo g, unsigned long long *table) {
    __shared__ long long part[8];
    const long d = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    long long before = 0;
    for (long q = tid; q < g.na * g.nb; q += 256) {
        const long a = q / g.nb, b = q % g.nb, c0 = hypCmin<G>(g, a, b), cnt = hypCmax<G>(g, a, b) - c0 + 1;
        const long x = d - a - b - c0;
        before += x <= 0 ? 0 : (x < cnt ? x : cnt);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    if (lane == 0) part[warp] = before;
    __syncthreads();
    long long pos = 0;
    for (int w = 0; w < 8; w++) pos += part[w];
    __syncthreads();  // part is reused by the scans below
    const long smax = g.na + g.nb - 2 < d ? g.na + g.nb - 2 : d;
    for (long s0 = smax; s0 >= 0; s0 -= 256) {
        const long s = s0 - tid, c = d - s;
        const long amin = s - (g.nb - 1) > 0 ? s - (g.nb - 1) : 0, amax = s < g.na - 1 ? s : g.na - 1;
        long long cnt = 0;
        if (s >= 0)
            for (long a = amin; a <= amax; a++) cnt += c >= hypCmin<G>(g, a, s - a) && c <= hypCmax<G>(g, a, s - a);
        // exclusive scan of cnt over the CTA's threads
        long long inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) part[warp] = inc;
        __syncthreads();
        long long off = inc - cnt, tot = 0;
        for (int w = 0; w < 8; w++) {
            off += w < warp ? part[w] : 0;
            tot += part[w];
        }
        if (s >= 0) {
            long long at = pos + off;
            for (long a = amin; a <= amax; a++)
                if (c >= hypCmin<G>(g, a, s - a) && c <= hypCmax<G>(g, a, s - a)) table[at++] = hypPack(a, s - a, c);
        }
        pos += tot;
        __syncthreads();  // part is rewritten by the next pass over the diagonals
    }
}

// bounded wait for *f >= want by one lane; false once the limit ran out (status written, counter stopped)
__device__ __forceinline__ bool hypWait(const int *f, int want, int *status, unsigned *counter, long limit) {
    long n = 0;
    while (ldAcquire(f) < want) {
        if (++n > limit) {
            atomicExch(status, ERR_SOR_TIMEOUT);
            atomicOr(counter, 0x80000000u);  // no warp takes another tile
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

__device__ __forceinline__ double ldH(const double *A, const HGeo &g, long i, long j, long k) {
    return (i >= 0 && i < g.e0 && j >= 0 && j < g.e1 && k >= 0 && k < g.e2) ? __ldcg(A + i * g.s0 + j * g.s1 + k)
                                                                             : 0.0;
}

// the multiple of G at or below x (x may be negative: a row's first windows start before the loop box)
template <int G>
__device__ __forceinline__ long hypFloor(long x) {
    return (x >= 0 ? x / G : -((-x + G - 1) / G)) * G;
}

// pairwise tree over the G leaves of the part starting at array index k = kf: leaf p is d[p]^2 where
// k = kf + p lies in the loop, -0.0 elsewhere (every lane at the same leaf: warp-uniform)
template <int G>
__device__ __forceinline__ double hypTree(const double *d, long kf, long lo2, long hi2) {
    double stk[Hyp<G>::LOG], v = 0.0;
#pragma unroll
    for (int p = 0; p < G; p++) {
        v = kf + p >= lo2 && kf + p <= hi2 ? d[p] * d[p] : -0.0;
#pragma unroll
        for (int l = 0; l < Hyp<G>::LOG; l++) {
            if (!((p >> l) & 1)) {
                stk[l] = v;
                break;
            }
            v = stk[l] + v;
        }
    }
    return v;
}

template <int G>
__global__ void __launch_bounds__(NT) kSorHyp(double *A, HGeo g, const double *wPtr, int *flags, unsigned *counter,
                                              const unsigned long long *table, double *carry, double *items,
                                              int *status, Bound bound) {
    using H = Hyp<G>;
    constexpr int SKP = H::SKP, RS = SJ * SKP;  // RS: one step of i in the window box
    extern __shared__ double sm[];              // per warp: box [SI][SJ][SKP], then leaves [32][SQS]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, li = lane / TJ, lj = lane % TJ;
    double *box = sm + (size_t)H::WSM * warp;
    double *sq = box + H::BOX + lane * H::SQS;
    const double w = *wPtr;
    const double c1 = 1.0 - w, c2 = w / 6.0;  // loop invariants, rounded as in the source expression
    const int nk = (int)g.nk;
    while (true) {
        long idx = 0;
        if (lane == 0) idx = (long)atomicAdd(counter, 1u) + bound.firstIndex;  // >= 2^31 once a warp has failed
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= g.ntiles) break;
        const unsigned long long tv = table[idx];
        const long a = (long)(tv >> 42), b = (long)((tv >> 21) & 0x1fffff), c = (long)(tv & 0x1fffff);
        const long ra = TI * a, rb = TJ * b, hc = G * c;  // hc: the tile's first hyperplane
        // 1. before the wait: rows qi 1..5, qj 1..9 (own rows and the +i / +j faces), positions 1 .. G+1 --
        //    old values that no tile writes before this one is done
        {
            constexpr int NV = (SI - 1) * (SJ - 1) * (G + 1), NL = (NV + 31) / 32;
            double v[NL];
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * 32 + lane, r = q / (G + 1), p = 1 + q % (G + 1);
                const int qi = 1 + r / (SJ - 1), qj = 1 + r % (SJ - 1);
                const long ri = ra - 1 + qi, rj = rb - 1 + qj;
                v[u] = q < NV ? ldH(A, g, g.lo0 + ri, g.lo1 + rj, g.lo2 + hc - ri - rj - 1 + p) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * 32 + lane, r = q / (G + 1), p = 1 + q % (G + 1);
                const int qi = 1 + r / (SJ - 1), qj = 1 + r % (SJ - 1);
                if (q < NV) box[(qi * SJ + qj) * SKP + p] = v[u];
            }
        }
        // 2. wait for the five predecessors (bounded)
        int fail = 0;
        if (lane < 5) {
            // lanes 0..4: (a-1,b,c), (a-1,b,c-1), (a,b-1,c), (a,b-1,c-1), (a,b,c-1)
            const long pa = a - (lane < 2), pb = b - (lane == 2 || lane == 3),
                       pc = c - (lane == 1 || lane == 3 || lane == 4);
            if (pa >= 0 && pb >= 0 && pc >= hypCmin<G>(g, pa, pb) && pc <= hypCmax<G>(g, pa, pb) &&
                !hypWait(flags + (pa * g.nb + pb) * g.ncg + pc, 1, status, counter, bound.pollLimit))
                fail = 1;
        }
        if (__any_sync(0xffffffffu, fail)) return;
        __syncwarp();  // orders the acquiring lanes' loads before every lane's face loads
        const long ri = ra + li, rj = rb + lj, i = g.lo0 + ri, j = g.lo1 + rj;
        const bool row = i <= g.hi0 && j <= g.hi1;
        const int rk0 = (int)(hc - ri - rj);                // the row's rk at step 0
        const long k0 = g.lo2 + rk0;                          // ... and its array index k
        const long m = hypFloor<G>(k0);                       // the part boundary at or below k0
        const int dl = (int)(k0 - m);                         // positions of the part before the window
        const long rowIdx = row ? (i - g.lo0) * g.nj + (j - g.lo1) : 0;
        const bool first = c == hypCmin<G>(g, a, b);
        const bool res = row && k0 <= g.hi2;                  // the row has a part to close here
        // 3. the -i face rows (0, 1..8) and -j face rows (1..4, 0) at positions 0 .. G-1, the own rows at 0,
        //    and the differences the row's previous window carried over (its last dl positions)
        double cin[G - 1];
        {
            constexpr int NV = (TI + TJ) * G, NL = (NV + 31) / 32;
            double v[NL];
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * 32 + lane, r = q / G, p = q % G;
                const int qi = r < TJ ? 0 : r - TJ + 1, qj = r < TJ ? r + 1 : 0;
                const long fi = ra - 1 + qi, fj = rb - 1 + qj;
                v[u] = q < NV ? ldH(A, g, g.lo0 + fi, g.lo1 + fj, g.lo2 + hc - fi - fj - 1 + p) : 0.0;
            }
            const double k0v = ldH(A, g, i, j, k0 - 1);
#pragma unroll
            for (int q = 0; q < G - 1; q++)
                cin[q] = res && !first && q < dl ? __ldcg(carry + q * g.rows + rowIdx) : 0.0;
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * 32 + lane, r = q / G, p = q % G;
                const int qi = r < TJ ? 0 : r - TJ + 1, qj = r < TJ ? r + 1 : 0;
                if (q < NV) box[(qi * SJ + qj) * SKP + p] = v[u];
            }
            box[((li + 1) * SJ + lj + 1) * SKP] = k0v;
        }
        __syncwarp();
        double *x = box + ((li + 1) * SJ + (lj + 1)) * SKP + 1;  // x[t]: position t + 1
        double dv[G];                                              // nv - old of each step
        // 4. the dependent chain: G steps, every lane on its own row
#pragma unroll
        for (int t = 0; t < G; t++) {
            const int rk = rk0 + t;
            dv[t] = 0.0;
            if (row && rk >= 0 && rk < nk) {
                const double old = x[t];
                // A[i-1] + A[i+1] + A[j-1] + A[j+1] + A[k-1] + A[k+1], left to right
                const double s = ((((x[t - RS - 1] + x[t + RS + 1]) + x[t - SKP - 1]) + x[t + SKP + 1]) + x[t - 1]) +
                                 x[t + 1];
                const double nv = c1 * old + c2 * s;
                x[t] = nv;
                dv[t] = nv - old;
            }
            __syncwarp();
        }
        // 5. store what the successors read -- the rows li = 3 and lj = 7, the last position of the others, and
        //    the differences of the row's last dl positions (the row's next window needs them) -- release the
        //    successors, then store the tile's other cells (read by no tile of this sweep)
        auto store = [&](int r, int p) {  // row r of the tile, window position p (1 .. G)
            const int qi = r / TJ, qj = r % TJ;
            const long ii = ra + qi, jj = rb + qj, rk = hc - ii - jj + p - 1;
            if (g.lo0 + ii <= g.hi0 && g.lo1 + jj <= g.hi1 && rk >= 0 && rk < nk)
                A[(g.lo0 + ii) * g.s0 + (g.lo1 + jj) * g.s1 + g.lo2 + rk] = box[((qi + 1) * SJ + qj + 1) * SKP + p];
        };
#pragma unroll
        for (int u = (TI - 1) * TJ * G / 32; u < TI * TJ * G / 32; u++) {  // rows li = 3
            const int q = u * 32 + lane;
            store(q / G, 1 + q % G);
        }
        {
            constexpr int NE = (TI - 1) * G + (TI - 1) * (TJ - 1);  // rows lj = 7 (li < 3), last positions
#pragma unroll
            for (int u = 0; u < (NE + 31) / 32; u++) {
                const int e = u * 32 + lane, f = e - (TI - 1) * G;
                if (e < (TI - 1) * G) store((e / G) * TJ + TJ - 1, 1 + e % G);
                else if (e < NE) store((f / (TJ - 1)) * TJ + f % (TJ - 1), G);
            }
        }
#pragma unroll
        for (int t = 1; t < G; t++)  // position t is leaf t - G + dl of the next part
            if (res && t - G + dl >= 0) carry[(t - G + dl) * g.rows + rowIdx] = dv[t];
        // the warp barrier orders every lane's stores before lane 0's release at GPU scope, which publishes
        // them (release cumulativity) without a sequentially consistent fence in every lane
        __syncwarp();
        if (lane == 0) stRelease(flags + (a * g.nb + b) * g.ncg + c, 1);
#pragma unroll
        for (int u = 0; u < (TI - 1) * TJ * G / 32; u++) {  // rows li < 3, lj < 7 at positions 1 .. G - 1
            const int q = u * 32 + lane, r = q / G, p = 1 + q % G;
            if (r % TJ < TJ - 1 && p < G) store(r, p);
        }
        // 6. the residual, off the chain: the leaves of the part [m, m + G) are the carried differences, then
        //    this window's; squared where k lies in the loop, -0.0 elsewhere
        if (res) {
#pragma unroll
            for (int q = 0; q < G - 1; q++)
                if (q < dl) sq[q] = cin[q];
#pragma unroll
            for (int t = 0; t < G; t++) sq[dl + t] = dv[t];
            const long P = m / G - g.kc0;  // m / G: exact, m is a multiple of G (possibly negative)
            double *it = items + rowIdx * g.nparts;
            if (first)
                for (long q = 0; q < P && q < g.nparts; q++) it[q] = -0.0;
            if (P >= 0 && P < g.nparts) it[P] = hypTree<G>(sq, m, g.lo2, g.hi2);
            if (k0 + G - 1 >= g.hi2) {  // the row ends in this window: the next part, then -0.0 to the end
                if (P + 1 >= 0 && P + 1 < g.nparts) it[P + 1] = hypTree<G>(sq + G, m + G, g.lo2, g.hi2);
                for (long q = P + 2 > 0 ? P + 2 : 0; q < g.nparts; q++) it[q] = -0.0;
            }
        }
        __syncwarp();  // the box and the leaves are reused by this warp's next tile
    }
}

// CTA tiles: TIc x TJc rows, one thread per row (TIc * TJc / 32 warps), one tile per CTA.  Fewer, larger
// tiles shorten the chain of tile planes (a + b + c) a sweep has to go through; the tile's warps take their
// steps in lockstep (a CTA barrier per step), each on its own SM sub-partition.
template <int G, int TIc, int TJc>
struct HypC {
    static constexpr int NTc = TIc * TJc;
    static constexpr int SIc = TIc + 2, SJc = TJc + 2;
    static constexpr int SKP = G + 3;  // window: positions 0 .. G + 1 (odd stride: banks)
    static constexpr int BOX = SIc * SJc * SKP;
    static constexpr int SQS = 2 * G + 1;
    static constexpr size_t SMEM = sizeof(double) * (BOX + NTc * SQS);
};

template <int G, int TIc, int TJc>
__global__ void __launch_bounds__(TIc * TJc, 4) kSorHypCta(double *A, HGeo g, const double *wPtr, int *flags,
                                                        unsigned *counter, const unsigned long long *table,
                                                        double *carry, double *items, int *status, Bound bound) {
    using H = HypC<G, TIc, TJc>;
    constexpr int SKP = H::SKP, SJc = H::SJc, RS = SJc * SKP, NTc = H::NTc;
    extern __shared__ double sm[];  // box [SIc][SJc][SKP], then leaves [NTc][SQS]
    __shared__ long tileIdx;
    const int tid = threadIdx.x, li = tid / TJc, lj = tid % TJc;
    double *box = sm;
    double *sq = sm + H::BOX + tid * H::SQS;
    const double w = *wPtr;
    const double c1 = 1.0 - w, c2 = w / 6.0;  // loop invariants, rounded as in the source expression
    const int nk = (int)g.nk;
    while (true) {
        if (tid == 0) tileIdx = (long)atomicAdd(counter, 1u) + bound.firstIndex;  // >= 2^31 once a CTA has failed
        __syncthreads();  // the index; and the previous tile's last box reads are done
        const long idx = tileIdx;
        if (idx >= g.ntiles) break;
        const unsigned long long tv = table[idx];
        const long a = (long)(tv >> 42), b = (long)((tv >> 21) & 0x1fffff), c = (long)(tv & 0x1fffff);
        const long ra = TIc * a, rb = TJc * b, hc = G * c;
        // 1. before the wait: rows qi 1..TIc+1, qj 1..TJc+1, positions 1 .. G+1 (old values)
        {
            constexpr int NV = (H::SIc - 1) * (SJc - 1) * (G + 1), NL = (NV + NTc - 1) / NTc;
            double v[NL];
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * NTc + tid, r = q / (G + 1), p = 1 + q % (G + 1);
                const int qi = 1 + r / (SJc - 1), qj = 1 + r % (SJc - 1);
                const long fi = ra - 1 + qi, fj = rb - 1 + qj;
                v[u] = q < NV ? ldH(A, g, g.lo0 + fi, g.lo1 + fj, g.lo2 + hc - fi - fj - 1 + p) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * NTc + tid, r = q / (G + 1), p = 1 + q % (G + 1);
                const int qi = 1 + r / (SJc - 1), qj = 1 + r % (SJc - 1);
                if (q < NV) box[(qi * SJc + qj) * SKP + p] = v[u];
            }
        }
        // 2. wait for the five predecessors (bounded); the barrier orders the acquiring threads' loads
        //    before every thread's face loads
        int fail = 0;
        if (tid < 5) {
            // threads 0..4: (a-1,b,c), (a-1,b,c-1), (a,b-1,c), (a,b-1,c-1), (a,b,c-1)
            const long pa = a - (tid < 2), pb = b - (tid == 2 || tid == 3), pc = c - (tid == 1 || tid == 3 || tid == 4);
            if (pa >= 0 && pb >= 0 && pc >= hypCmin<G>(g, pa, pb) && pc <= hypCmax<G>(g, pa, pb) &&
                !hypWait(flags + (pa * g.nb + pb) * g.ncg + pc, 1, status, counter, bound.pollLimit))
                fail = 1;
        }
        if (__syncthreads_or(fail)) return;
        const long ri = ra + li, rj = rb + lj, i = g.lo0 + ri, j = g.lo1 + rj;
        const bool row = i <= g.hi0 && j <= g.hi1;
        const int rk0 = (int)(hc - ri - rj);
        const long k0 = g.lo2 + rk0;
        const long m = hypFloor<G>(k0);                       // the part boundary at or below k0
        const int dl = (int)(k0 - m);
        const long rowIdx = row ? (i - g.lo0) * g.nj + (j - g.lo1) : 0;
        const bool first = c == hypCmin<G>(g, a, b);
        const bool res = row && k0 <= g.hi2;
        // 3. the -i face rows (0, 1..TJc), the -j face rows (1..TIc, 0) at positions 0 .. G-1, the own rows at
        //    0, and the carried differences
        double cin[G - 1];
        {
            constexpr int NV = (TIc + TJc) * G, NL = (NV + NTc - 1) / NTc;
            double v[NL];
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * NTc + tid, r = q / G, p = q % G;
                const int qi = r < TJc ? 0 : r - TJc + 1, qj = r < TJc ? r + 1 : 0;
                const long fi = ra - 1 + qi, fj = rb - 1 + qj;
                v[u] = q < NV ? ldH(A, g, g.lo0 + fi, g.lo1 + fj, g.lo2 + hc - fi - fj - 1 + p) : 0.0;
            }
            const double k0v = ldH(A, g, i, j, k0 - 1);
#pragma unroll
            for (int q = 0; q < G - 1; q++)
                cin[q] = res && !first && q < dl ? __ldcg(carry + q * g.rows + rowIdx) : 0.0;
#pragma unroll
            for (int u = 0; u < NL; u++) {
                const int q = u * NTc + tid, r = q / G, p = q % G;
                const int qi = r < TJc ? 0 : r - TJc + 1, qj = r < TJc ? r + 1 : 0;
                if (q < NV) box[(qi * SJc + qj) * SKP + p] = v[u];
            }
            box[((li + 1) * SJc + lj + 1) * SKP] = k0v;
        }
        __syncthreads();
        double *x = box + ((li + 1) * SJc + (lj + 1)) * SKP + 1;  // x[t]: position t + 1
        double dv[G];
        // 4. the dependent chain: G steps, one thread per row, the CTA in lockstep
#pragma unroll
        for (int t = 0; t < G; t++) {
            const int rk = rk0 + t;
            dv[t] = 0.0;
            if (row && rk >= 0 && rk < nk) {
                const double old = x[t];
                // A[i-1] + A[i+1] + A[j-1] + A[j+1] + A[k-1] + A[k+1], left to right
                const double s = ((((x[t - RS - 1] + x[t + RS + 1]) + x[t - SKP - 1]) + x[t + SKP + 1]) + x[t - 1]) +
                                 x[t + 1];
                const double nv = c1 * old + c2 * s;
                x[t] = nv;
                dv[t] = nv - old;
            }
            __syncthreads();
        }
        // 5. store what the successors read (rows li = TIc-1 and lj = TJc-1, the last position of the others,
        //    the carried differences), release the successors, then store the other cells
        auto store = [&](int r, int p) {
            const int qi = r / TJc, qj = r % TJc;
            const long ii = ra + qi, jj = rb + qj, rk = hc - ii - jj + p - 1;
            if (g.lo0 + ii <= g.hi0 && g.lo1 + jj <= g.hi1 && rk >= 0 && rk < nk)
                A[(g.lo0 + ii) * g.s0 + (g.lo1 + jj) * g.s1 + g.lo2 + rk] = box[((qi + 1) * SJc + qj + 1) * SKP + p];
        };
        {
            constexpr int N1 = TJc * G, N2 = N1 + (TIc - 1) * G, NE = N2 + (TIc - 1) * (TJc - 1);
#pragma unroll
            for (int u = 0; u < (NE + NTc - 1) / NTc; u++) {
                const int e = u * NTc + tid;
                if (e < N1) store((TIc - 1) * TJc + e / G, 1 + e % G);
                else if (e < N2) store(((e - N1) / G) * TJc + TJc - 1, 1 + (e - N1) % G);
                else if (e < NE) store(((e - N2) / (TJc - 1)) * TJc + (e - N2) % (TJc - 1), G);
            }
        }
#pragma unroll
        for (int t = 1; t < G; t++)  // position t is leaf t - G + dl of the next part
            if (res && t - G + dl >= 0) carry[(t - G + dl) * g.rows + rowIdx] = dv[t];
        // the CTA barrier orders every thread's stores before thread 0's release at GPU scope
        __syncthreads();
        if (tid == 0) stRelease(flags + (a * g.nb + b) * g.ncg + c, 1);
#pragma unroll
        for (int u = 0; u < G; u++) {  // rows li < TIc-1, lj < TJc-1 at positions 1 .. G-1
            const int q = u * NTc + tid, r = q / G, p = 1 + q % G;
            if (r / TJc < TIc - 1 && r % TJc < TJc - 1 && p < G) store(r, p);
        }
        // 6. the residual, off the chain (per thread, as in the warp tiles)
        if (res) {
#pragma unroll
            for (int q = 0; q < G - 1; q++)
                if (q < dl) sq[q] = cin[q];
#pragma unroll
            for (int t = 0; t < G; t++) sq[dl + t] = dv[t];
            const long P = m / G - g.kc0;
            double *it = items + rowIdx * g.nparts;
            if (first)
                for (long q = 0; q < P && q < g.nparts; q++) it[q] = -0.0;
            if (P >= 0 && P < g.nparts) it[P] = hypTree<G>(sq, m, g.lo2, g.hi2);
            if (k0 + G - 1 >= g.hi2) {
                if (P + 1 >= 0 && P + 1 < g.nparts) it[P + 1] = hypTree<G>(sq + G, m + G, g.lo2, g.hi2);
                for (long q = P + 2 > 0 ? P + 2 : 0; q < g.nparts; q++) it[q] = -0.0;
            }
        }
    }
}

template <int G>
bool hypGeo(const long st[3], const long ext[3], const long lo[3], const long hi[3], long ti, long tj, HGeo &g) {
    if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2] || lo[0] < 0 || lo[1] < 0 || lo[2] < 0 || (st && st[2] != 1))
        return false;
    if (ext && (hi[0] >= ext[0] || hi[1] >= ext[1] || hi[2] >= ext[2])) return false;  // cells stored in the array
    g.s0 = st ? st[0] : 0;
    g.s1 = st ? st[1] : 0;
    g.e0 = ext ? ext[0] : 0;
    g.e1 = ext ? ext[1] : 0;
    g.e2 = ext ? ext[2] : 0;
    g.lo0 = lo[0];
    g.lo1 = lo[1];
    g.lo2 = lo[2];
    g.hi0 = hi[0];
    g.hi1 = hi[1];
    g.hi2 = hi[2];
    g.ti = ti;
    g.tj = tj;
    g.na = (hi[0] - lo[0] + ti) / ti;
    g.nb = (hi[1] - lo[1] + tj) / tj;
    g.nk = hi[2] - lo[2] + 1;
    g.ncg = hypCmax<G>(g, g.na - 1, g.nb - 1) + 1;
    g.nj = hi[1] - lo[1] + 1;
    g.rows = (hi[0] - lo[0] + 1) * g.nj;
    g.kc0 = Hyp<G>::PARTS * (lo[2] / 64);
    g.nparts = Hyp<G>::PARTS * (hi[2] / 64 - lo[2] / 64 + 1);
    if (g.na >= (1L << 21) || g.nb >= (1L << 21) || g.ncg >= (1L << 21) || g.nk >= (1L << 30) ||
        g.na * g.nb * g.ncg >= (1L << 30))
        return false;
    long n = 0;
    for (long a = 0; a < g.na; a++)
        for (long b = 0; b < g.nb; b++) n += hypCmax<G>(g, a, b) - hypCmin<G>(g, a, b) + 1;
    g.ntiles = n;
    g.nlev = g.na + g.nb + g.ncg - 2;
    return true;
}

// scratch: the tile counter (own 256-byte line), one flag per (a, b, c < ncg), the hand-out table, the carries
struct HypScratch {
    size_t flagsOff, tableOff, carryOff, bytes;
};
template <int G>
HypScratch hypScratch(const HGeo &g) {
    HypScratch s;
    s.flagsOff = 256;
    s.tableOff = (s.flagsOff + sizeof(int) * (size_t)(g.na * g.nb * g.ncg) + 15) / 16 * 16;
    s.carryOff = s.tableOff + sizeof(unsigned long long) * (size_t)g.ntiles;
    s.bytes = s.carryOff + sizeof(double) * (G - 1) * (size_t)g.rows;
    return s;
}

// one hyperplane sweep: the tile list, then the persistent wavefront.  cta: tiles of CTA_TI x CTA_TJ rows, one
// per CTA (kSorHypCta); else tiles of 4 x 8 rows, one per warp (kSorHyp)
constexpr int CTA_TI = 16, CTA_TJ = 8;
template <int G>
int sweepHyp(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3], const double *wDev,
             double *items, void *scratch, int *status, Bound bound, bool cta, cudaStream_t s) {
    HGeo g;
    if (!hypGeo<G>(st, ext, lo, hi, cta ? CTA_TI : TI, cta ? CTA_TJ : TJ, g)) return -1;
    const HypScratch sc = hypScratch<G>(g);
    char *base = (char *)scratch;
    unsigned *counter = (unsigned *)base;
    int *flags = (int *)(base + sc.flagsOff);
    unsigned long long *table = (unsigned long long *)(base + sc.tableOff);
    double *carry = (double *)(base + sc.carryOff);
    if (cudaMemsetAsync(scratch, 0, sc.tableOff, s) != cudaSuccess) return -1;
    kHypTable<G><<<(unsigned)g.nlev, 256, 0, s>>>(g, table);
    long grid;
    if (cta) {
        using H = HypC<G, CTA_TI, CTA_TJ>;
        static std::atomic<int> occCache[gbdev::MAX_DEVICES];
        const int occ = gbdev::residentCtas(occCache, kSorHypCta<G, CTA_TI, CTA_TJ>, H::NTc, H::SMEM);
        grid = (long)occ * gbdev::smCount();  // all CTAs resident at once: waits always resolve
        if (grid > g.ntiles) grid = g.ntiles;
        kSorHypCta<G, CTA_TI, CTA_TJ><<<(unsigned)grid, H::NTc, H::SMEM, s>>>(A, g, wDev, flags, counter, table,
                                                                             carry, items, status, bound);
    } else {
        using H = Hyp<G>;
        static std::atomic<int> occCache[gbdev::MAX_DEVICES];
        const int occ = gbdev::residentCtas(occCache, kSorHyp<G>, NT, H::SMEM);
        grid = (long)occ * gbdev::smCount();
        const long gridCap = (g.ntiles + WPB - 1) / WPB;
        if (grid > gridCap) grid = gridCap;
        kSorHyp<G><<<(unsigned)grid, NT, H::SMEM, s>>>(A, g, wDev, flags, counter, table, carry, items, status,
                                                        bound);
    }
    dvmhgb_count_launches(2);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

extern "C" {

long dvmhgb_sor3d_items(const long lo[3], const long hi[3], int variant) {
    const int tk = tkOf(variant);
    if (!tk) return -1;
    return (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (64 / tk) * (hi[2] / 64 - lo[2] / 64 + 1);
}

long dvmhgb_sor3d_scratch_bytes(const long lo[3], const long hi[3], int variant) {
    const int tk = tkOf(variant);
    if (!tk) return -1;
    if (variant >= 4) {
        HGeo g;
        if (!hypGeo<8>(nullptr, nullptr, lo, hi, variant == 5 ? CTA_TI : TI, variant == 5 ? CTA_TJ : TJ, g))
            return -1;
        return (long)hypScratch<8>(g).bytes;
    }
    long ntiles = ((hi[0] - lo[0] + TI) / TI) * ((hi[1] - lo[1] + TJ) / TJ) * (64 / tk) * (hi[2] / 64 - lo[2] / 64 + 1);
    return (ntiles + 64) * (long)sizeof(int);
}

int dvmhgb_sor3d_sweep_bounded(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3],
                               const double *wDev, double *items, void *scratch, int *status, int variant,
                               void *stream, long pollLimit, long firstIndex) {
    const int tk = tkOf(variant);
    Geo g;
    if (!tk || !A || !wDev || !items || !scratch || !status || !geo(st, ext, lo, hi, 64 / tk, g)) return -1;
    if (pollLimit < 1 || firstIndex < 0 || firstIndex >= (1L << 30)) return -1;
    const Bound bound{pollLimit, (unsigned)firstIndex};
    cudaStream_t s = (cudaStream_t)stream;
    if (variant >= 4) return sweepHyp<8>(A, st, ext, lo, hi, wDev, items, scratch, status, bound, variant == 5, s);
    switch (tk) {
        case 64: return sweepStream(A, g, wDev, items, scratch, status, bound, s);
        case 32: return sweepT<32>(A, g, wDev, items, scratch, status, bound, s);
        case 16: return sweepT<16>(A, g, wDev, items, scratch, status, bound, s);
        default: return sweepT<8>(A, g, wDev, items, scratch, status, bound, s);
    }
}

int dvmhgb_sor3d_sweep(double *A, const long st[3], const long ext[3], const long lo[3], const long hi[3],
                       const double *wDev, double *items, void *scratch, int *status, int variant, void *stream) {
    return dvmhgb_sor3d_sweep_bounded(A, st, ext, lo, hi, wDev, items, scratch, status, variant, stream, SPIN_LIMIT,
                                      0);
}

}  // extern "C"
