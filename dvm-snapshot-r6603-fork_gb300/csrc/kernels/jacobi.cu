// Jacobi loop kernels (2-D 5-point and 3-D 7-point, FP64) for sm_103a.
//
// The loops are those of examples/Performance/jac3d_perf.c:56-73 and
// examples/Jacobi/jac2d.c:49-64 with FP64 data:
//   update : tmp = fabs(B-A); eps = Max(tmp, eps); A = B
//   stencil: B = (A[i-1][j][k] + A[i][j-1][k] + A[i][j][k-1] + A[i][j][k+1]
//                 + A[i][j+1][k] + A[i+1][j][k]) / 6.0          (3-D)
//            B = (A[i-1][j] + A[i][j-1] + A[i][j+1] + A[i+1][j]) / 4.0  (2-D)
// Sums are evaluated left to right exactly as written; the build uses
// -fmad=false so no product is contracted into an FMA.
//
// GB300 executes 2 FP64 thread-operations per clock per SM, so FP64 issue --
// not HBM -- bounds these loops when every operation is a native FP64 one.
// Here the division is done exactly on the integer pipe (sf::div3p2 /
// sf::scale_down), MAX compares bit patterns as integers, and `native` of a
// cell's FP64 additions run on the FP64 unit while the rest run on the
// integer pipe (sf::add), bit for bit the same (softfp64.cuh).  `native` is a
// launch parameter the tuner chooses.
//
// Layout: innermost axis contiguous, rows 16-byte aligned (the runtime pads
// device rows), so element pairs (2p, 2p+1) are loaded and stored as one
// 128-bit access.  The stencil kernels stream the outermost axis through
// registers (plane i-1, i, i+1 per thread) and stage plane i with its halo in
// shared memory (2.5-D blocking): every A element comes from HBM once.
#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"
#include "devinfo.cuh"
#include "softfp64.cuh"

namespace {

constexpr int UPD_THREADS = 256;
constexpr int UPD_CTAS_PER_SM = 8;

int smCount() { return gbdev::smCount(); }

__device__ __forceinline__ double2 ld2cs(const double *p) { return __ldcs(reinterpret_cast<const double2 *>(p)); }
__device__ __forceinline__ double2 ld2(const double *p) { return *reinterpret_cast<const double2 *>(p); }
__device__ __forceinline__ void st2(double *p, double2 v) { *reinterpret_cast<double2 *>(p) = v; }
__device__ __forceinline__ void st2cs(double *p, double2 v) { __stcs(reinterpret_cast<double2 *>(p), v); }

__device__ __forceinline__ double maxOf(double tmp, double eps) { return tmp > eps ? tmp : eps; }  // Max(tmp, eps)

// CTA-wide maximum (any order: MAX is order-independent); thread 0 gets it
__device__ __forceinline__ double ctaMax(double m, double *sh) {
    for (int o = 16; o > 0; o >>= 1) m = maxOf(__shfl_xor_sync(0xffffffffu, m, o), m);
    const int warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (blockDim.x * blockDim.y) >> 5;
    if (lane == 0) sh[warp] = m;
    __syncthreads();
    if (warp == 0) {
        m = lane < nw ? sh[lane] : -__builtin_huge_val();
        for (int o = 16; o > 0; o >>= 1) m = maxOf(__shfl_xor_sync(0xffffffffu, m, o), m);
    }
    return m;
}

// ---------------------------------------------------------------- update loop (2-D and 3-D)

// Rows are (i, j) pairs of the box (nj = 1 and s1 = 0 in 2-D); a warp handles
// 32 element pairs of one row per unit; units are strided over the grid.
__global__ void __launch_bounds__(UPD_THREADS) kUpdate(double *A, const double *__restrict__ B, long s0, long s1,
                                                       long lo0, long lo1, long lo2, long hi2, unsigned nj,
                                                       unsigned units, unsigned nseg, long p0, long p1,
                                                       double *items, int native) {
    __shared__ double sh[UPD_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t mb = 0, qmax = 0;  // FP64-unit / integer-pipe MAX parts (native == 2: the latter)
    bool seen = false;
    const unsigned wstride = gridDim.x * (UPD_THREADS / 32);
    // UNITS units per trip: all their loads are issued before any is used
    constexpr int UNITS = 4;
    for (unsigned u0 = blockIdx.x * (UPD_THREADS / 32) + warp; u0 < units; u0 += UNITS * wstride) {
        long off[UNITS], k0[UNITS];
        bool live[UNITS];
        double2 a[UNITS], b[UNITS];
#pragma unroll
        for (int q = 0; q < UNITS; q++) {
            unsigned u = u0 + q * wstride;
            unsigned row = u / nseg, seg = u - row * nseg;
            unsigned ri = row / nj, rj = row - ri * nj;
            long p = p0 + (long)seg * 32 + lane;
            live[q] = u < units && p <= p1;
            k0[q] = 2 * p;
            off[q] = (lo0 + ri) * s0 + (lo1 + rj) * s1 + k0[q];
            if (live[q]) {
                b[q] = ld2cs(B + off[q]);
                a[q] = ld2cs(A + off[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < UNITS; q++) {
            if (!live[q]) continue;
            bool in0 = k0[q] >= lo2 && k0[q] <= hi2, in1 = k0[q] + 1 >= lo2 && k0[q] + 1 <= hi2;
            bool ok = native == 2;
            if (ok) {
                // |B - A| exact as 64-bit fixed point for values in [2^-12, 1) (see kStencil3)
                const uint64_t b0 = sf::q64(b[q].x, ok), a0 = sf::q64(a[q].x, ok);
                const uint64_t b1 = sf::q64(b[q].y, ok), a1 = sf::q64(a[q].y, ok);
                const uint64_t d0 = b0 > a0 ? b0 - a0 : a0 - b0, d1 = b1 > a1 ? b1 - a1 : a1 - b1;
                if (ok && in0 && d0 > qmax) qmax = d0;  // only exact differences enter the maximum
                if (ok && in1 && d1 > qmax) qmax = d1;
            }
            if (!ok) {  // native 0 / 1, or a value outside the fixed-point range (rare)
                if (in0) mb = sf::absmax_bits(native ? sf::nadd(b[q].x, -a[q].x) : sf::sub(b[q].x, a[q].x), mb);
                if (in1) mb = sf::absmax_bits(native ? sf::nadd(b[q].y, -a[q].y) : sf::sub(b[q].y, a[q].y), mb);
            }
            seen = seen || in0 || in1;
            if (in0 && in1) st2cs(A + off[q], b[q]);
            else if (in0) A[off[q]] = b[q].x;
            else if (in1) A[off[q] + 1] = b[q].y;
        }
    }
    double m = -__builtin_huge_val();
    if (seen) {
        const double qd = __ull2double_rn(qmax) * 0x1p-64, f = sf::from(mb);  // RN(max |b - a|), then MAX
        m = qd > f ? qd : f;
    }
    m = ctaMax(m, sh);
    if (threadIdx.x == 0) items[blockIdx.x] = m;
}

// 128-bit accesses need 16-byte aligned rows: even outer strides, aligned bases
bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }
bool rows16(const long *st, int rank) {
    for (int i = 0; i < rank - 1; i++)
        if (st[i] & 1) return false;
    return st[rank - 1] == 1;
}

struct UpdGeom {
    unsigned units, nseg, nj;
    long p0, p1;
    long blocks;
    bool ok;
};

UpdGeom updGeom(long ni, long nj, long lo2, long hi2) {
    UpdGeom g{};
    g.p0 = lo2 >> 1;
    g.p1 = hi2 >> 1;
    long nseg = (g.p1 - g.p0 + 1 + 31) / 32;
    long units = ni * nj * nseg;
    g.ok = ni > 0 && nj > 0 && hi2 >= lo2 && lo2 >= 0 && units < (1L << 31);
    g.units = (unsigned)units;
    g.nseg = (unsigned)nseg;
    g.nj = (unsigned)nj;
    long want = (units + UPD_THREADS / 32 - 1) / (UPD_THREADS / 32);
    long cap = (long)smCount() * UPD_CTAS_PER_SM;
    g.blocks = want < cap ? want : cap;
    if (g.blocks < 1) g.blocks = 1;
    return g;
}

// ---------------------------------------------------------------- 3-D stencil / fused (2.5-D blocking)

constexpr int TX = 32;  // lanes: element pairs along k (64 elements)
constexpr int TY = 8;   // warps: rows along j

struct Box3 {
    long s0, s1;
    long e0, e1, e2;
    long lo0, lo1, lo2, hi0, hi1, hi2;
};

__device__ __forceinline__ bool inArr3(const Box3 &b, long i, long j, long k) {
    return i >= 0 && i < b.e0 && j >= 0 && j < b.e1 && k >= 0 && k < b.e2;
}
__device__ __forceinline__ bool inBox3(const Box3 &b, long i, long j, long k) {
    return i >= b.lo0 && i <= b.hi0 && j >= b.lo1 && j <= b.hi1 && k >= b.lo2 && k <= b.hi2;
}

// element pair (k, k+1), k even, guarded by the array bounds (0 outside)
__device__ __forceinline__ double2 ldPair(const double *X, const Box3 &b, long i, long j, long k) {
    double2 v = make_double2(0.0, 0.0);
    if (i < 0 || i >= b.e0 || j < 0 || j >= b.e1) return v;
    const double *p = X + i * b.s0 + j * b.s1 + k;
    if (k >= 0 && k + 1 < b.e2) return ld2(p);
    if (k >= 0 && k < b.e2) v.x = p[0];
    if (k + 1 >= 0 && k + 1 < b.e2) v.y = p[1];
    return v;
}
__device__ __forceinline__ double ldOne(const double *X, const Box3 &b, long i, long j, long k) {
    return inArr3(b, i, j, k) ? X[i * b.s0 + j * b.s1 + k] : 0.0;
}

// FUSED = false: plain stencil, source = A.
// FUSED = true : source of the stencil is A_new = (x in box ? B : A) (the update
// loop's A = B applied), own cells also update A and eps; output goes to Bnew.
// (((((a + b) + c) + d) + e) + f) / 6.0: the first N additions on the FP64
// unit, the others and the division on the integer pipe (fast paths)
template <int N>
__device__ __forceinline__ double stencil7(double a, double b, double c, double d, double e, double f, bool &spc) {
    if (N >= 5)  // all additions native: the division's rare native fallback is a real branch
        return sf::div3p2(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(a, b), c), d), e), f), 1);
    double t = N > 0 ? sf::nadd(a, b) : sf::add_fast(a, b, spc);
    t = N > 1 ? sf::nadd(t, c) : sf::add_fast(t, c, spc);
    t = N > 2 ? sf::nadd(t, d) : sf::add_fast(t, d, spc);
    t = N > 3 ? sf::nadd(t, e) : sf::add_fast(t, e, spc);
    t = N > 4 ? sf::nadd(t, f) : sf::add_fast(t, f, spc);
    return sf::div3p2_fast(t, 1, spc);
}

// (((a + b) + c) + d) / 4.0 likewise (x / 4.0 == x * 0.25 exactly)
template <int N>
__device__ __forceinline__ double stencil5(double a, double b, double c, double d, bool &spc) {
    double t = N > 0 ? sf::nadd(a, b) : sf::add_fast(a, b, spc);
    t = N > 1 ? sf::nadd(t, c) : sf::add_fast(t, c, spc);
    t = N > 2 ? sf::nadd(t, d) : sf::add_fast(t, d, spc);
    return sf::scale_down_fast(t, 2, spc);
}

// (((((a + b) + c) + d) + e) + f) / 6.0 for a tile whose inputs were all
// checked pos_ok: the first 5 - N additions on the integer pipe (sf::add_pos),
// the others on the FP64 unit, the division on the integer pipe.
template <int N>
__device__ __forceinline__ double stencil7pos(double a, double b, double c, double d, double e, double f, bool &spc) {
    double t = N > 4 ? sf::nadd(a, b) : sf::add_pos(a, b);
    t = N > 3 ? sf::nadd(t, c) : sf::add_pos(t, c);
    t = N > 2 ? sf::nadd(t, d) : sf::add_pos(t, d);
    t = N > 1 ? sf::nadd(t, e) : sf::add_pos(t, e);
    t = N > 0 ? sf::nadd(t, f) : sf::add_pos(t, f);
    return sf::div3p2_fast(t, 1, spc);
}

// The 3-D stencil loop (FUSED = false: Out = (6 neighbours of A) / 6) or the
// update and stencil loops fused (FUSED = true: eps = Max(|B - A|, eps); A = B
// over the box, then Out = (6 neighbours of A_new) / 6, A_new = B inside the
// box and A outside it).
//
// A CTA of TY warps covers 64 elements of k (lane l owns the pair k = kb + 2l,
// k + 1) and TJ = TY * JT rows of j (warp ty owns rows ty*JT .. ty*JT + JT-1),
// and streams the planes i of its chunk.  Per thread, the own pairs of planes
// i-1, i, i+1 are in registers and plane i+2 is in flight; plane i's rows are
// also in shared memory (two buffers, one barrier per plane) for the j
// neighbours owned by the next / previous warp; k neighbours come by shuffles,
// the chunk's edge columns kb-1 / kb+64 are loaded by lanes 0 / 31.  Every
// source element is read from HBM once.
//
// FP64 work per cell: the five additions (5 - NATIVE of them on the integer
// pipe once the CTA has seen only pos_ok inputs).  The division by 6 and, in
// the fused loop, the MAX of |B - A| run on the integer pipe: |B - A| of two
// values in [2^-12, 1) is exact as 64-bit fixed point (value * 2^64), its
// maximum is rounded once at the end -- RN is monotone and odd, so
// RN(max |b - a|) = max |RN(b - a)|.  Values outside that range take the FP64
// unit (a warp-uniform branch).
template <bool FUSED, int NATIVE, int JT, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB) kStencil3(double *A, const double *B, double *Out, Box3 b,
                                                                   long p0, int ichunk, double *items) {
    constexpr int TJ = TY * JT;
    __shared__ double2 sm[2][TJ + 2][TX];
    __shared__ double shr[TY];
    const int lane = threadIdx.x, ty = threadIdx.y;
    const long kb = 2 * (p0 + (long)blockIdx.x * TX);
    const long jb = b.lo1 + (long)blockIdx.y * TJ;
    const long ib = b.lo0 + (long)blockIdx.z * ichunk;
    const long ie = ib + ichunk - 1 < b.hi0 ? ib + ichunk - 1 : b.hi0;
    const long k = kb + 2 * lane;

    // per-thread constants: the lane's columns, its rows, its edge column and halo row
    const bool kA = k < b.e2, kA1 = k + 1 < b.e2;  // k >= 0 always
    const bool kI0 = k >= b.lo2 && k <= b.hi2, kI1 = k + 1 >= b.lo2 && k + 1 <= b.hi2;
    const bool edgeLane = lane == 0 || lane == TX - 1;
    const long hc = lane == 0 ? kb - 1 : kb + 2 * TX;
    const bool hcA = edgeLane && hc >= 0 && hc < b.e2, hcI = hc >= b.lo2 && hc <= b.hi2;
    long jo[JT];
    bool jA[JT], jI[JT];
#pragma unroll
    for (int r = 0; r < JT; r++) {
        const long j = jb + ty * JT + r;
        jo[r] = j * b.s1;
        jA[r] = j < b.e1;
        jI[r] = j <= b.hi1;
    }
    const bool haloWarp = ty == 0 || ty == TY - 1;
    const long hr = ty == 0 ? jb - 1 : jb + TJ;
    const bool hrA = haloWarp && hr >= 0 && hr < b.e1, hrI = hr >= b.lo1 && hr <= b.hi1;
    const long hro = hr * b.s1;
    const int hrIdx = ty == 0 ? 0 : TJ + 1;

    bool bad = false;  // this thread loaded a value outside pos_ok
    auto chk = [&](double x) {
        if (NATIVE < 5) bad |= !sf::pos_ok(x);
    };
    // the loop's source value at (ii, row, pair k)
    auto srcPair = [&](long ii, long joff, bool ja, bool ji) -> double2 {
        double2 v = make_double2(0.0, 0.0);
        if (ja && kA && ii >= 0 && ii < b.e0) {
            const long off = ii * b.s0 + joff + k;
            if (!FUSED) {
                v = ld2(A + off);
            } else {
                const bool iin = ii >= b.lo0 && ii <= b.hi0;
                const bool in0 = iin && ji && kI0, in1 = iin && ji && kI1;
                if (in0 && in1) {
                    v = ld2(B + off);
                } else {
                    v = ld2(A + off);
                    if (in0 || in1) {
                        const double2 w = ld2(B + off);
                        if (in0) v.x = w.x;
                        if (in1) v.y = w.y;
                    }
                }
            }
            if (!kA1) v.y = 0.0;
        }
        chk(v.x);
        chk(v.y);
        return v;
    };
    auto srcEdge = [&](long ii, long joff, bool ja, bool ji) -> double {
        double v = 0.0;
        if (ja && hcA && ii >= 0 && ii < b.e0) {
            const long off = ii * b.s0 + joff + hc;
            v = (FUSED && ii >= b.lo0 && ii <= b.hi0 && ji && hcI) ? B[off] : A[off];
        }
        chk(v);
        return v;
    };

    double2 pm[JT], pc[JT], pp[JT], pq[JT], ao[JT], aon[JT];
    double ec[JT], ep[JT], eq[JT];
    double2 hp = make_double2(0.0, 0.0), hq = hp;
#pragma unroll
    for (int r = 0; r < JT; r++) {
        pm[r] = srcPair(ib - 1, jo[r], jA[r], jI[r]);
        pc[r] = srcPair(ib, jo[r], jA[r], jI[r]);
        pp[r] = srcPair(ib + 1, jo[r], jA[r], jI[r]);
        ec[r] = srcEdge(ib, jo[r], jA[r], jI[r]);
        ep[r] = srcEdge(ib + 1, jo[r], jA[r], jI[r]);
        if (FUSED) ao[r] = (jA[r] && kA) ? ld2(A + ib * b.s0 + jo[r] + k) : make_double2(0.0, 0.0);
    }
    double2 hc0 = haloWarp ? srcPair(ib, hro, hrA, hrI) : make_double2(0.0, 0.0);
    if (haloWarp) hp = srcPair(ib + 1, hro, hrA, hrI);
#pragma unroll
    for (int r = 0; r < JT; r++) sm[0][1 + ty * JT + r][lane] = pc[r];
    if (haloWarp) sm[0][hrIdx][lane] = hc0;
    bool ctaBad = __syncthreads_or(bad) != 0;

    uint64_t mb = 0, qmax = 0;  // eps: FP64-unit part (bit pattern), fixed-point part
    bool seen = false;
    int cur = 0;
    for (long i = ib; i <= ie; i++) {
        // plane i+2 in flight, and A_old of plane i+1 for the update
#pragma unroll
        for (int r = 0; r < JT; r++) {
            pq[r] = srcPair(i + 2, jo[r], jA[r], jI[r]);
            eq[r] = srcEdge(i + 2, jo[r], jA[r], jI[r]);
            if (FUSED)
                aon[r] = (i + 1 <= ie && jA[r] && kA) ? ld2(A + (i + 1) * b.s0 + jo[r] + k) : make_double2(0.0, 0.0);
        }
        if (haloWarp) hq = srcPair(i + 2, hro, hrA, hrI);

        // plane i
        double v[JT][2];
        bool spc = false;
#pragma unroll
        for (int r = 0; r < JT; r++) {
            const double2 up = r > 0 ? pc[r - 1] : sm[cur][ty * JT + r][lane];
            const double2 dn = r < JT - 1 ? pc[r + 1] : sm[cur][ty * JT + r + 2][lane];
            double left = __shfl_up_sync(0xffffffffu, pc[r].y, 1), right = __shfl_down_sync(0xffffffffu, pc[r].x, 1);
            if (lane == 0) left = ec[r];
            if (lane == TX - 1) right = ec[r];
            if (NATIVE < 5 && !ctaBad) {
                v[r][0] = stencil7pos<NATIVE>(pm[r].x, up.x, left, pc[r].y, dn.x, pp[r].x, spc);
                v[r][1] = stencil7pos<NATIVE>(pm[r].y, up.y, pc[r].x, right, dn.y, pp[r].y, spc);
            } else {
                v[r][0] = stencil7<5>(pm[r].x, up.x, left, pc[r].y, dn.x, pp[r].x, spc);
                v[r][1] = stencil7<5>(pm[r].y, up.y, pc[r].x, right, dn.y, pp[r].y, spc);
            }
            if (__any_sync(0xffffffffu, spc)) {  // rare: an operand or result the fast division does not cover
                if (spc) {
                    v[r][0] = sf::ndiv(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(pm[r].x, up.x), left), pc[r].y),
                                                         dn.x), pp[r].x), 6.0);
                    v[r][1] = sf::ndiv(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(pm[r].y, up.y), pc[r].x), right),
                                                         dn.y), pp[r].y), 6.0);
                }
                spc = false;
            }
        }
#pragma unroll
        for (int r = 0; r < JT; r++) {
            if (!jI[r]) continue;
            const long off = i * b.s0 + jo[r] + k;
            if (FUSED) {
                // update loop on own cells: eps = Max(|B - A|, eps); A = B
                bool ok = true;
                const uint64_t b0 = sf::q64(pc[r].x, ok), a0 = sf::q64(ao[r].x, ok);
                const uint64_t b1 = sf::q64(pc[r].y, ok), a1 = sf::q64(ao[r].y, ok);
                const uint64_t d0 = b0 > a0 ? b0 - a0 : a0 - b0, d1 = b1 > a1 ? b1 - a1 : a1 - b1;
                if (ok && kI0 && d0 > qmax) qmax = d0;  // only exact differences enter the maximum
                if (ok && kI1 && d1 > qmax) qmax = d1;
                if (__any_sync(0xffffffffu, !ok) && !ok) {
                    if (kI0) mb = sf::absmax_bits(sf::nadd(pc[r].x, -ao[r].x), mb);
                    if (kI1) mb = sf::absmax_bits(sf::nadd(pc[r].y, -ao[r].y), mb);
                }
                seen = seen || kI0 || kI1;
                if (kI0 && kI1) st2cs(A + off, pc[r]);
                else if (kI0) A[off] = pc[r].x;
                else if (kI1) A[off + 1] = pc[r].y;
            }
            if (kI0 && kI1) st2cs(Out + off, make_double2(v[r][0], v[r][1]));
            else if (kI0) Out[off] = v[r][0];
            else if (kI1) Out[off + 1] = v[r][1];
        }
        // stage plane i+1, then rotate
#pragma unroll
        for (int r = 0; r < JT; r++) sm[cur ^ 1][1 + ty * JT + r][lane] = pp[r];
        if (haloWarp) sm[cur ^ 1][hrIdx][lane] = hp;
        ctaBad = (__syncthreads_or(bad) != 0) || ctaBad;
        cur ^= 1;
#pragma unroll
        for (int r = 0; r < JT; r++) {
            pm[r] = pc[r];
            pc[r] = pp[r];
            pp[r] = pq[r];
            ec[r] = ep[r];
            ep[r] = eq[r];
            if (FUSED) ao[r] = aon[r];
        }
        hp = hq;
    }
    if (FUSED) {
        // RN(max |b - a|) from the fixed-point part, then the MAX with the FP64-unit part
        double m = -__builtin_huge_val();
        if (seen) {
            const double q = __ull2double_rn(qmax) * 0x1p-64;
            const double f = sf::from(mb);
            m = q > f ? q : f;
        }
        m = ctaMax(m, shr);
        if (ty == 0 && lane == 0)
            items[blockIdx.x + gridDim.x * ((long)blockIdx.y + (long)gridDim.y * blockIdx.z)] = m;
    }
}

// The 3-D stencil loop, Out = (6 neighbours of A) / 6, with the sums in the
// q61 fixed-point form of softfp64.cuh: a double in [2^-9, 1) or +0 is an
// exact multiple of 2^-61, an FP64 addition of two such values is an integer
// addition plus a round-to-nearest-even of the sum to 53 significant bits,
// and the division by 6 rounds the sum straight to the double quotient.  Bit
// for bit the FP64 unit's results, on the integer pipe, which a GB300 SM runs
// far faster than its FP64 unit (2 FP64 thread-operations per clock):
// measured on GB300, 1.7e11 cells/s of the cell arithmetic alone against
// 7.1e10 for the five native additions.
//
// The integer pipe then bounds this kernel while the FP64 unit idles, so a
// fraction of the CTAs (nat of every den, by block index) computes its cells
// the native way -- five FP64 additions, the division on the integer pipe --
// and both pipes of an SM work at once.  Both forms give the same bits.
//
// Layout of the work as in kStencil3 with one row per thread: a CTA of TY
// warps covers 64 elements of k and TY rows of j and streams the planes i of
// its chunk; a thread keeps planes i-1, i, i+1 of its element pair in
// registers (q61 values, or the doubles' bits in a native CTA), plane i+2 in
// flight as doubles (converted one plane later, so the loads have a plane of
// work to arrive), and plane i's rows in double-buffered shared memory for
// the j neighbours; k neighbours come by shuffles, the chunk's edge columns
// by lanes 0 / 31.
//
// Range (fixed-point CTAs): every value the cells of a plane read must be
// q61_ok.  Each thread flags the values it converts; the flags of the CTA are
// OR-ed once per plane (the barrier the shared-memory rows need anyway) and
// kept for the last three planes.  A plane whose neighbourhood holds any
// other value (a negative value, one below 2^-9 or at least 1, a subnormal,
// an infinity or a NaN) is computed by the whole CTA on the FP64 unit from
// global memory (the arithmetic of stencil7<5>), so every input gives the
// FP64 unit's result.
template <bool Q>
__device__ __forceinline__ void planes3(const double *__restrict__ A, double *Out, const Box3 &b, long p0, int ichunk,
                                        ulonglong2 (*sm)[TY + 2][TX]) {
    const int lane = threadIdx.x, ty = threadIdx.y;
    const long kb = 2 * (p0 + (long)blockIdx.x * TX);
    const long jb = b.lo1 + (long)blockIdx.y * TY;
    const long ib = b.lo0 + (long)blockIdx.z * ichunk;
    const long ie = ib + ichunk - 1 < b.hi0 ? ib + ichunk - 1 : b.hi0;
    const long k = kb + 2 * lane;
    const bool kA = k < b.e2, kA1 = k + 1 < b.e2;  // k >= 0 always
    const bool kI0 = k >= b.lo2 && k <= b.hi2, kI1 = k + 1 >= b.lo2 && k + 1 <= b.hi2;
    const bool edgeLane = lane == 0 || lane == TX - 1;
    const long hc = lane == 0 ? kb - 1 : kb + 2 * TX;
    const bool hcA = edgeLane && hc >= 0 && hc < b.e2;
    const long j = jb + ty;
    const long jo = j * b.s1;
    const bool jA = j < b.e1, jI = j <= b.hi1;
    const bool haloWarp = ty == 0 || ty == TY - 1;
    const long hr = ty == 0 ? jb - 1 : jb + TY;
    const bool hrA = haloWarp && hr >= 0 && hr < b.e1;
    const long hro = hr * b.s1;
    const int hrIdx = ty == 0 ? 0 : TY + 1;
    // what this thread loads in every plane, and from where: its element pair,
    // its edge column (lanes 0 and 31), its halo row (warps 0 and TY-1)
    const bool ownOk = jA && kA, edgeOk = jA && hcA, haloOk = hrA && kA;
    const double *own = A + jo + k, *edge = A + jo + hc, *halo = A + hro + k;

    auto ldPair = [&](const double *p, bool ok) -> double2 {
        double2 v = make_double2(0.0, 0.0);
        if (ok) {
            v = ld2(p);
            if (!kA1) v.y = 0.0;
        }
        return v;
    };
    auto planeOk = [&](long ii) { return ii >= 0 && ii < b.e0; };
    // a loaded value in the CTA's representation (q61, or the double's bits)
    auto cv = [](double x, bool &bad) -> uint64_t {
        if (!Q) return sf::bits(x);
        bad |= !sf::q61_ok(x);
        return sf::q61(x);
    };
    // (((((a + b) + c) + d) + e) + f) / 6 in the CTA's representation
    auto cell = [](uint64_t a, uint64_t b2, uint64_t c, uint64_t d, uint64_t e, uint64_t f) -> double {
        if (Q) return sf::q61_div6(sf::q61_add(sf::q61_add(sf::q61_add(sf::q61_add(sf::q61_add(a, b2), c), d), e), f));
        return sf::div3p2(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::from(a), sf::from(b2)), sf::from(c)),
                                                     sf::from(d)), sf::from(e)), sf::from(f)), 1);
    };
    // the cell (i, j, kk) on the FP64 unit, its neighbours from global memory (0 outside the array)
    auto nativeCell = [&](long i, long kk) -> double {
        const double a = ldOne(A, b, i - 1, j, kk), bb = ldOne(A, b, i, j - 1, kk), c = ldOne(A, b, i, j, kk - 1);
        const double d = ldOne(A, b, i, j, kk + 1), e = ldOne(A, b, i, j + 1, kk), f = ldOne(A, b, i + 1, j, kk);
        return sf::div3p2(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(a, bb), c), d), e), f), 1);
    };

    // planes ib-1, ib, ib+1 (own pair), the edge column of ib and ib+1, the halo row of ib and ib+1
    bool bad = false;
    const long s0 = b.s0;
    double2 t = ldPair(own + (ib - 1) * s0, ownOk && planeOk(ib - 1));
    uint64_t pmx = cv(t.x, bad), pmy = cv(t.y, bad);
    t = ldPair(own + ib * s0, ownOk && planeOk(ib));
    uint64_t pcx = cv(t.x, bad), pcy = cv(t.y, bad);
    t = ldPair(own + (ib + 1) * s0, ownOk && planeOk(ib + 1));
    uint64_t ppx = cv(t.x, bad), ppy = cv(t.y, bad);
    uint64_t ec = cv(edgeOk && planeOk(ib) ? edge[ib * s0] : 0.0, bad);
    uint64_t ep = cv(edgeOk && planeOk(ib + 1) ? edge[(ib + 1) * s0] : 0.0, bad);
    uint64_t hpx = 0, hpy = 0;
    if (haloWarp) {
        t = ldPair(halo + ib * s0, haloOk && planeOk(ib));
        sm[0][hrIdx][lane] = make_ulonglong2(cv(t.x, bad), cv(t.y, bad));
        t = ldPair(halo + (ib + 1) * s0, haloOk && planeOk(ib + 1));
        hpx = cv(t.x, bad);
        hpy = cv(t.y, bad);
    }
    sm[0][1 + ty][lane] = make_ulonglong2(pcx, pcy);
    // flags of planes i-1, i, i+1 in bits 2, 1, 0 (the first three merged)
    unsigned flags = __syncthreads_or(bad) ? 7u : 0u;
    int cur = 0;
    // plane pointers of plane i+2 (loads) and plane i (stores), bumped by one plane per step;
    // plane i+2 exists for the first `nload` steps
    const int nplanes = (int)(ie - ib + 1);
    const int nload = (int)(b.e0 - (ib + 2) < (long)nplanes ? b.e0 - (ib + 2) : (long)nplanes);
    const double *qOwn = own + (ib + 2) * s0, *qEdge = edge + (ib + 2) * s0, *qHalo = halo + (ib + 2) * s0;
    double *out = Out + ib * s0 + jo + k;
    long i = ib;
    for (int step = 0; step < nplanes; step++, i++) {
        // plane i+2 in flight
        const bool more = step < nload;
        const double2 q = ldPair(qOwn, ownOk && more);
        const double eqd = (edgeOk && more) ? *qEdge : 0.0;
        double2 hq = make_double2(0.0, 0.0);
        if (haloWarp) hq = ldPair(qHalo, haloOk && more);
        qOwn += s0;
        qEdge += s0;
        qHalo += s0;

        // plane i
        double v0, v1;
        if (flags == 0) {
            const ulonglong2 up = sm[cur][ty][lane], dn = sm[cur][ty + 2][lane];
            uint64_t left = __shfl_up_sync(0xffffffffu, pcy, 1), right = __shfl_down_sync(0xffffffffu, pcx, 1);
            if (lane == 0) left = ec;
            if (lane == TX - 1) right = ec;
            // (((((A[i-1] + A[j-1]) + A[k-1]) + A[k+1]) + A[j+1]) + A[i+1]) / 6, left to right
            v0 = cell(pmx, up.x, left, pcy, dn.x, ppx);
            v1 = cell(pmy, up.y, pcx, right, dn.y, ppy);
        } else {  // rare: a value outside the fixed-point range near this plane
            v0 = (jI && kI0) ? nativeCell(i, k) : 0.0;
            v1 = (jI && kI1) ? nativeCell(i, k + 1) : 0.0;
        }
        if (jI) {
            if (kI0 && kI1) st2cs(out, make_double2(v0, v1));
            else if (kI0) out[0] = v0;
            else if (kI1) out[1] = v1;
        }
        out += s0;

        // plane i+2 converted; plane i+1 staged; one barrier; rotate
        bad = false;
        const uint64_t qx = cv(q.x, bad), qy = cv(q.y, bad), eq = cv(eqd, bad);
        uint64_t hqx = 0, hqy = 0;
        if (haloWarp) {
            hqx = cv(hq.x, bad);
            hqy = cv(hq.y, bad);
            sm[cur ^ 1][hrIdx][lane] = make_ulonglong2(hpx, hpy);
        }
        sm[cur ^ 1][1 + ty][lane] = make_ulonglong2(ppx, ppy);
        if (Q) flags = ((flags << 1) | (__syncthreads_or(bad) ? 1u : 0u)) & 7u;
        else __syncthreads();
        cur ^= 1;
        pmx = pcx, pmy = pcy;
        pcx = ppx, pcy = ppy;
        ppx = qx, ppy = qy;
        ec = ep, ep = eq;
        hpx = hqx, hpy = hqy;
    }
}

// The update and stencil loops in one pass with the fixed-point sums
// (kStencil3QF): eps = Max(|B - A|, eps); A = B over the box, then
// Bnew = (6 neighbours of A_new) / 6 with A_new = B inside the box and A
// outside it.  The stencil part is planes3's (q61 sums; planes whose
// neighbourhood leaves the fixed-point range on the FP64 unit).  The update
// of a plane of the chunk is done when that plane's values are converted:
// A_old, loaded beside B, enters |B - A_old| -- exact as a difference of q61
// values, rounded once at the end (RN is monotone and odd, so
// RN(max |b - a|) = max |RN(b - a)|), or on the FP64 unit for a value outside
// the range -- and B is stored into A.  Nothing reads A inside the box
// afterwards (the stencil's source there is B), so the early store is safe.
// 32 bytes per cell: A and B read, A and Bnew written.
template <int MINB>
__global__ void __launch_bounds__(TX *TY, MINB) kStencil3QF(double *A, const double *__restrict__ B, double *Out,
                                                              Box3 b, long p0, int ichunk, double *items) {
    __shared__ ulonglong2 sm[2][TY + 2][TX];
    __shared__ double shr[TY];
    const int lane = threadIdx.x, ty = threadIdx.y;
    const long kb = 2 * (p0 + (long)blockIdx.x * TX);
    const long jb = b.lo1 + (long)blockIdx.y * TY;
    const long ib = b.lo0 + (long)blockIdx.z * ichunk;
    const long ie = ib + ichunk - 1 < b.hi0 ? ib + ichunk - 1 : b.hi0;
    const long k = kb + 2 * lane;
    const bool kA = k < b.e2, kA1 = k + 1 < b.e2;  // k >= 0 always
    const bool kI0 = k >= b.lo2 && k <= b.hi2, kI1 = k + 1 >= b.lo2 && k + 1 <= b.hi2;
    const bool edgeLane = lane == 0 || lane == TX - 1;
    const long hc = lane == 0 ? kb - 1 : kb + 2 * TX;
    const bool hcA = edgeLane && hc >= 0 && hc < b.e2, hcI = hc >= b.lo2 && hc <= b.hi2;
    const long j = jb + ty;
    const long jo = j * b.s1;
    const bool jA = j < b.e1, jI = j <= b.hi1;  // j >= lo1 always
    const bool haloWarp = ty == 0 || ty == TY - 1;
    const long hr = ty == 0 ? jb - 1 : jb + TY;
    const bool hrA = haloWarp && hr >= 0 && hr < b.e1, hrI = hr >= b.lo1 && hr <= b.hi1;
    const long hro = hr * b.s1;
    const int hrIdx = ty == 0 ? 0 : TY + 1;
    const long s0 = b.s0;

    auto planeOk = [&](long ii) { return ii >= 0 && ii < b.e0; };
    auto planeIn = [&](long ii) { return ii >= b.lo0 && ii <= b.hi0; };
    // the stencil's source pair at plane ii, row offset roff: B inside the box, A outside (0 beyond the array)
    auto srcPair = [&](long ii, long roff, bool ok, bool rowIn) -> double2 {
        double2 v = make_double2(0.0, 0.0);
        if (ok && planeOk(ii)) {
            const long off = ii * s0 + roff + k;
            const bool iin = planeIn(ii) && rowIn;
            const bool in0 = iin && kI0, in1 = iin && kI1;
            if (in0 && in1) {
                v = ld2(B + off);
            } else {
                v = ld2(A + off);
                if (in0 || in1) {
                    const double2 w = ld2(B + off);
                    if (in0) v.x = w.x;
                    if (in1) v.y = w.y;
                }
            }
            if (!kA1) v.y = 0.0;
        }
        return v;
    };
    auto srcEdge = [&](long ii) -> double {
        if (!(jA && hcA && planeOk(ii))) return 0.0;
        const long off = ii * s0 + jo + hc;
        return (planeIn(ii) && jI && hcI) ? B[off] : A[off];
    };
    auto srcAt = [&](long i, long jj, long kk) -> double {
        if (!inArr3(b, i, jj, kk)) return 0.0;
        const long off = i * s0 + jj * b.s1 + kk;
        return inBox3(b, i, jj, kk) ? B[off] : A[off];
    };
    auto cv = [](double x, bool &bad) -> uint64_t {
        bad |= !sf::q61_ok(x);
        return sf::q61(x);
    };
    auto nativeCell = [&](long i, long kk) -> double {
        const double a = srcAt(i - 1, j, kk), bb = srcAt(i, j - 1, kk), c = srcAt(i, j, kk - 1);
        const double d = srcAt(i, j, kk + 1), e = srcAt(i, j + 1, kk), f = srcAt(i + 1, j, kk);
        return sf::div3p2(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(a, bb), c), d), e), f), 1);
    };
    // the update loop on the own pair of plane ii, a plane of this chunk (inside the box):
    // eps = Max(|B - A|, eps) and A = B for the pair's elements in the box
    uint64_t qmax = 0, mb = 0;  // eps: fixed-point part, FP64-unit part (bit pattern)
    bool seen = false;
    const bool ownUpd = jA && kA && jI && (kI0 || kI1);
    auto aOld = [&](long ii) -> double2 {
        return (ownUpd && ii >= ib && ii <= ie) ? ld2(A + ii * s0 + jo + k) : make_double2(0.0, 0.0);
    };
    auto update = [&](long ii, double2 bs, double2 ao) {
        if (!ownUpd || ii < ib || ii > ie) return;
        const bool ok0 = sf::q61_ok(bs.x) && sf::q61_ok(ao.x), ok1 = sf::q61_ok(bs.y) && sf::q61_ok(ao.y);
        const uint64_t b0 = sf::q61(bs.x), a0 = sf::q61(ao.x), b1 = sf::q61(bs.y), a1 = sf::q61(ao.y);
        const uint64_t d0 = b0 > a0 ? b0 - a0 : a0 - b0, d1 = b1 > a1 ? b1 - a1 : a1 - b1;
        if (kI0 && ok0 && d0 > qmax) qmax = d0;
        if (kI1 && ok1 && d1 > qmax) qmax = d1;
        if ((kI0 && !ok0) || (kI1 && !ok1)) {  // rare: a value outside the fixed-point range
            if (kI0 && !ok0) mb = sf::absmax_bits(sf::nadd(bs.x, -ao.x), mb);
            if (kI1 && !ok1) mb = sf::absmax_bits(sf::nadd(bs.y, -ao.y), mb);
        }
        seen = true;
        double *pa = A + ii * s0 + jo + k;
        if (kI0 && kI1) st2cs(pa, bs);
        else if (kI0) pa[0] = bs.x;
        else pa[1] = bs.y;
    };

    // planes ib-1, ib, ib+1 (own pair), the edge column of ib and ib+1, the halo row of ib and ib+1;
    // the update of planes ib and ib+1
    bool bad = false;
    double2 t = srcPair(ib - 1, jo, jA && kA, jI);
    uint64_t pmx = cv(t.x, bad), pmy = cv(t.y, bad);
    const double2 tc = srcPair(ib, jo, jA && kA, jI), ac = aOld(ib);
    const double2 tp = srcPair(ib + 1, jo, jA && kA, jI), ap = aOld(ib + 1);
    uint64_t pcx = cv(tc.x, bad), pcy = cv(tc.y, bad);
    uint64_t ppx = cv(tp.x, bad), ppy = cv(tp.y, bad);
    update(ib, tc, ac);
    update(ib + 1, tp, ap);
    uint64_t ec = cv(srcEdge(ib), bad), ep = cv(srcEdge(ib + 1), bad);
    uint64_t hpx = 0, hpy = 0;
    if (haloWarp) {
        t = srcPair(ib, hro, hrA && kA, hrI);
        sm[0][hrIdx][lane] = make_ulonglong2(cv(t.x, bad), cv(t.y, bad));
        t = srcPair(ib + 1, hro, hrA && kA, hrI);
        hpx = cv(t.x, bad);
        hpy = cv(t.y, bad);
    }
    sm[0][1 + ty][lane] = make_ulonglong2(pcx, pcy);
    unsigned flags = __syncthreads_or(bad) ? 7u : 0u;  // planes i-1, i, i+1 in bits 2, 1, 0
    int cur = 0;
    for (long i = ib; i <= ie; i++) {
        // plane i+2 in flight: the source, and A_old where it is a plane of this chunk
        const double2 q = srcPair(i + 2, jo, jA && kA, jI);
        const double2 aq = aOld(i + 2);
        const double eqd = srcEdge(i + 2);
        double2 hq = make_double2(0.0, 0.0);
        if (haloWarp) hq = srcPair(i + 2, hro, hrA && kA, hrI);

        // plane i
        double v0, v1;
        if (flags == 0) {
            const ulonglong2 up = sm[cur][ty][lane], dn = sm[cur][ty + 2][lane];
            uint64_t left = __shfl_up_sync(0xffffffffu, pcy, 1), right = __shfl_down_sync(0xffffffffu, pcx, 1);
            if (lane == 0) left = ec;
            if (lane == TX - 1) right = ec;
            // (((((A[i-1] + A[j-1]) + A[k-1]) + A[k+1]) + A[j+1]) + A[i+1]) / 6, left to right
            v0 = sf::q61_div6(sf::q61_add(
                sf::q61_add(sf::q61_add(sf::q61_add(sf::q61_add(pmx, up.x), left), pcy), dn.x), ppx));
            v1 = sf::q61_div6(sf::q61_add(
                sf::q61_add(sf::q61_add(sf::q61_add(sf::q61_add(pmy, up.y), pcx), right), dn.y), ppy));
        } else {  // rare: a value outside the fixed-point range near this plane
            v0 = (jI && kI0) ? nativeCell(i, k) : 0.0;
            v1 = (jI && kI1) ? nativeCell(i, k + 1) : 0.0;
        }
        if (jI) {
            double *out = Out + i * s0 + jo + k;
            if (kI0 && kI1) st2cs(out, make_double2(v0, v1));
            else if (kI0) out[0] = v0;
            else if (kI1) out[1] = v1;
        }

        // plane i+2: updated (when it is this chunk's) and converted; plane i+1 staged; one barrier; rotate
        update(i + 2, q, aq);
        bad = false;
        const uint64_t qx = cv(q.x, bad), qy = cv(q.y, bad), eq = cv(eqd, bad);
        uint64_t hqx = 0, hqy = 0;
        if (haloWarp) {
            hqx = cv(hq.x, bad);
            hqy = cv(hq.y, bad);
            sm[cur ^ 1][hrIdx][lane] = make_ulonglong2(hpx, hpy);
        }
        sm[cur ^ 1][1 + ty][lane] = make_ulonglong2(ppx, ppy);
        flags = ((flags << 1) | (__syncthreads_or(bad) ? 1u : 0u)) & 7u;
        cur ^= 1;
        pmx = pcx, pmy = pcy;
        pcx = ppx, pcy = ppy;
        ppx = qx, ppy = qy;
        ec = ep, ep = eq;
        hpx = hqx, hpy = hqy;
    }
    // RN(max |b - a|) from the fixed-point part, then the MAX with the FP64-unit part
    double m = -__builtin_huge_val();
    if (seen) {
        const double qd = __ull2double_rn(qmax) * 0x1p-61;
        const double f = sf::from(mb);
        m = qd > f ? qd : f;
    }
    m = ctaMax(m, shr);
    if (ty == 0 && lane == 0) items[blockIdx.x + gridDim.x * ((long)blockIdx.y + (long)gridDim.y * blockIdx.z)] = m;
}

#include "stencil_tma.cuh"

// CTAs started on each SM (any starting value: only its residue matters); the
// share of native CTAs is counted per SM, so that every SM runs both kinds at
// once -- a split by block index alone can put all native CTAs on some SMs
// (consecutive blocks of the same residue land on the same SM).  Launches that
// run at the same time share the counters; that only shifts the pattern.
__device__ unsigned ctaSlots[1024];

// nat of every den CTAs started on an SM native, the others fixed point (MIX =
// false: all fixed point, and only that path compiled)
template <int MINB, bool MIX>
__global__ void __launch_bounds__(TX *TY, MINB) kStencil3Q(const double *__restrict__ A, double *Out, Box3 b,
                                                             long p0, int ichunk, int nat, int den) {
    __shared__ ulonglong2 sm[2][TY + 2][TX];
    if (!MIX) {
        planes3<true>(A, Out, b, p0, ichunk, sm);
        return;
    }
    __shared__ int native;
    if (nat > 0) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            native = (int)(atomicAdd(&ctaSlots[smid & 1023u], 1u) % (unsigned)den) < nat;
        }
        __syncthreads();
    }
    if (nat > 0 && native) planes3<false>(A, Out, b, p0, ichunk, sm);
    else planes3<true>(A, Out, b, p0, ichunk, sm);
}

struct St3Geom {
    dim3 grid;
    long p0;
    int ichunk;
    bool ok;
};

St3Geom st3Geom(const long lo[3], const long hi[3], int TJ) {
    St3Geom g{};
    g.ok = hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2] && lo[2] >= 0;
    g.p0 = lo[2] >> 1;
    long p1 = hi[2] >> 1;
    long gx = (p1 - g.p0 + TX) / TX;
    long gy = (hi[1] - lo[1] + TJ) / TJ;
    long ni = hi[0] - lo[0] + 1;
    // split the streamed axis so the grid covers the GPU about four times
    long target = (long)smCount() * 4 * 4;
    long chunks = (target + gx * gy - 1) / (gx * gy);
    if (chunks < 1) chunks = 1;
    if (chunks > ni) chunks = ni;
    long ichunk = (ni + chunks - 1) / chunks;
    if (ichunk < 8 && ni >= 8) ichunk = 8;
    g.ichunk = (int)ichunk;
    long gz = (ni + ichunk - 1) / ichunk;
    g.ok = g.ok && gx < 65536 && gy < 65536 && gz < 65536;
    g.grid = dim3((unsigned)gx, (unsigned)gy, (unsigned)gz);
    return g;
}

// ---------------------------------------------------------------- 2-D stencil / fused (1.5-D blocking)

constexpr int T2Y = 8;  // independent column strips per CTA (one per warp)
constexpr int SW = 66;  // shared row: k = kb-1 .. kb+64

struct Box2 {
    long s0;
    long e0, e1;
    long lo0, lo1, hi0, hi1;
};

__device__ __forceinline__ double2 ldPair2(const double *X, const Box2 &b, long i, long k) {
    double2 v = make_double2(0.0, 0.0);
    if (i < 0 || i >= b.e0) return v;
    const double *p = X + i * b.s0 + k;
    if (k >= 0 && k + 1 < b.e1) return ld2(p);
    if (k >= 0 && k < b.e1) v.x = p[0];
    if (k + 1 >= 0 && k + 1 < b.e1) v.y = p[1];
    return v;
}
__device__ __forceinline__ double ldOne2(const double *X, const Box2 &b, long i, long k) {
    return (i >= 0 && i < b.e0 && k >= 0 && k < b.e1) ? X[i * b.s0 + k] : 0.0;
}
__device__ __forceinline__ bool inBox2(const Box2 &b, long i, long k) {
    return i >= b.lo0 && i <= b.hi0 && k >= b.lo1 && k <= b.hi1;
}

template <bool FUSED, int NATIVE>
__global__ void __launch_bounds__(TX *T2Y) kStencil2(double *A, const double *B, double *Out, Box2 b, long p0,
                                                      long nstrips, int ichunk, double *items) {
    __shared__ double sm[T2Y][SW];
    __shared__ double shr[T2Y];
    const int lane = threadIdx.x, ty = threadIdx.y;
    const long strip = (long)blockIdx.x * T2Y + ty;
    const bool active = strip < nstrips;
    const long kb = 2 * (p0 + strip * TX);
    const long ib = b.lo0 + (long)blockIdx.y * ichunk;
    long ie = ib + ichunk - 1;
    if (ie > b.hi0) ie = b.hi0;
    const long k = kb + 2 * lane;
    auto srcPair = [&](long i, long kk) -> double2 {
        if (!FUSED) return ldPair2(A, b, i, kk);
        double2 v = ldPair2(B, b, i, kk);
        bool x0 = inBox2(b, i, kk), x1 = inBox2(b, i, kk + 1);
        if (!(x0 && x1)) {
            double2 a = ldPair2(A, b, i, kk);
            if (!x0) v.x = a.x;
            if (!x1) v.y = a.y;
        }
        return v;
    };
    auto srcOne = [&](long i, long kk) -> double {
        if (!FUSED) return ldOne2(A, b, i, kk);
        return inBox2(b, i, kk) ? ldOne2(B, b, i, kk) : ldOne2(A, b, i, kk);
    };
    const long hcol = (lane == 0) ? kb - 1 : kb + 2 * TX;
    const bool ownsColHalo = (lane == 0) || (lane == TX - 1);
    double2 am = make_double2(0.0, 0.0), ac = am, ap = am;
    double hcc = 0.0, hcn = 0.0;
    if (active) {
        am = srcPair(ib - 1, k);
        ac = srcPair(ib, k);
        if (ownsColHalo) hcc = srcOne(ib, hcol);
    }
    uint64_t mb = 0;
    bool seen = false;
    for (long i = ib; i <= ie; i++) {
        double2 aold = make_double2(0.0, 0.0);
        if (active) {
            ap = srcPair(i + 1, k);
            if (ownsColHalo) hcn = srcOne(i + 1, hcol);
            if (FUSED) aold = ldPair2(A, b, i, k);
        }
        sm[ty][1 + 2 * lane] = ac.x;
        sm[ty][2 + 2 * lane] = ac.y;
        if (ownsColHalo) sm[ty][lane == 0 ? 0 : SW - 1] = hcc;
        __syncwarp();
        double v[2], dif[2];
        bool spc = false;
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int c = 1 + 2 * lane + e;
            double ame = e ? am.y : am.x, ape = e ? ap.y : ap.x;
            // (((A[i-1][j] + A[i][j-1]) + A[i][j+1]) + A[i+1][j]) / 4.0
            v[e] = stencil5<FUSED ? NATIVE - 1 : NATIVE>(ame, sm[ty][c - 1], sm[ty][c + 1], ape, spc);
            if (FUSED) {
                double bo = e ? ac.y : ac.x, ao = e ? aold.y : aold.x;
                dif[e] = NATIVE > 0 ? sf::nadd(bo, -ao) : sf::sub_fast(bo, ao, spc);
            }
        }
        if (__any_sync(0xffffffffu, spc)) {
            if (spc) {
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int c = 1 + 2 * lane + e;
                    double ame = e ? am.y : am.x, ape = e ? ap.y : ap.x;
                    v[e] = sf::ndiv(sf::nadd(sf::nadd(sf::nadd(ame, sm[ty][c - 1]), sm[ty][c + 1]), ape), 4.0);
                    if (FUSED) dif[e] = sf::nadd(e ? ac.y : ac.x, -(e ? aold.y : aold.x));
                }
            }
        }
        if (active) {
            bool in[2];
#pragma unroll
            for (int e = 0; e < 2; e++) in[e] = (k + e) >= b.lo1 && (k + e) <= b.hi1;
            const long off = i * b.s0 + k;
            if (FUSED) {
                if (in[0]) mb = sf::absmax_bits(dif[0], mb);
                if (in[1]) mb = sf::absmax_bits(dif[1], mb);
                seen = seen || in[0] || in[1];
                if (in[0] && in[1]) st2cs(A + off, ac);
                else if (in[0]) A[off] = ac.x;
                else if (in[1]) A[off + 1] = ac.y;
            }
            if (in[0] && in[1]) st2cs(Out + off, make_double2(v[0], v[1]));
            else if (in[0]) Out[off] = v[0];
            else if (in[1]) Out[off + 1] = v[1];
        }
        __syncwarp();
        am = ac;
        ac = ap;
        hcc = hcn;
    }
    if (FUSED) {
        double m = seen ? sf::from(mb) : -__builtin_huge_val();
        for (int o = 16; o > 0; o >>= 1) m = maxOf(__shfl_xor_sync(0xffffffffu, m, o), m);
        if (lane == 0) shr[ty] = m;
        __syncthreads();
        if (ty == 0 && lane == 0) {
            double r = shr[0];
            for (int w = 1; w < T2Y; w++) r = maxOf(shr[w], r);
            items[blockIdx.x + (long)gridDim.x * blockIdx.y] = r;
        }
    }
}

struct St2Geom {
    dim3 grid;
    long p0, nstrips;
    int ichunk;
    bool ok;
};

St2Geom st2Geom(const long lo[2], const long hi[2]) {
    St2Geom g{};
    g.ok = hi[0] >= lo[0] && hi[1] >= lo[1] && lo[1] >= 0;
    g.p0 = lo[1] >> 1;
    long p1 = hi[1] >> 1;
    g.nstrips = (p1 - g.p0 + TX) / TX;
    long gx = (g.nstrips + T2Y - 1) / T2Y;
    long ni = hi[0] - lo[0] + 1;
    long target = (long)smCount() * 8 * 4;
    long chunks = (target + gx - 1) / gx;
    if (chunks < 1) chunks = 1;
    if (chunks > ni) chunks = ni;
    long ichunk = (ni + chunks - 1) / chunks;
    if (ichunk < 4 && ni >= 4) ichunk = 4;  // halo rows cost 2 / ichunk extra reads
    g.ichunk = (int)ichunk;
    long gy = (ni + ichunk - 1) / ichunk;
    g.ok = g.ok && gx < (1L << 31) && gy < 65536;
    g.grid = dim3((unsigned)gx, (unsigned)gy, 1);
    return g;
}

// ---------------------------------------------------------------- copy outside a box

struct Slabs {
    int n;
    int rank;
    long lo[6][3], cnt[6][3];
    long start[7];
    long st[3];
};

__global__ void kCopyOutside(const double *__restrict__ src, double *__restrict__ dst, Slabs s) {
    long total = s.start[s.n];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int q = 0;
        while (t >= s.start[q + 1]) q++;
        long r = t - s.start[q], off = 0;
        for (int d = s.rank - 1; d >= 0; d--) {
            long c = r % s.cnt[q][d];
            r /= s.cnt[q][d];
            off += (s.lo[q][d] + c) * s.st[d];
        }
        dst[off] = src[off];
    }
}

// 3-D variants (stencil and fused alike): v < 12: v = 6 * (JT - 1) + N, N =
// additions of a cell on the FP64 unit (0..5, the others on the integer pipe),
// JT = rows per thread, two CTAs per SM; v = 12, 13: all additions native, one
// row per thread, registers capped for three / four CTAs per SM; v = 14..21:
// the q61 fixed-point stencil (kStencil3Q) with (CTAs per SM, native CTAs of
// every den): 14 (4, 0 of 1), 15 (3, 0 of 1), 16 (4, 1 of 2), 17 (4, 1 of 3),
// 18 (4, 2 of 5), 19 (3, 1 of 2), 20 (4, 1 of 4), 21 (4, 3 of 5); v = 22, 23:
// the q61 stencil with its planes staged by TMA (kStencil3T), a ring of 6 / 4
// plane slots, four CTAs per SM; v = 24, 25, 26: ring of 6 with 1, 2, 3 of the
// 8 warps on the FP64 unit (the fused entry point runs the update and then the
// stencil into the second buffer for v = 14..26)
constexpr int V3Q = 14, V3T = 22, V3 = 27;
int jtOf3(int v) { return (v >= 6 && v < 12) ? 2 : 1; }
bool isQ3(int v) { return v >= V3Q && v < V3; }
bool isT3(int v) { return v >= V3T && v < V3; }
// the fused entry point's extra variants: the two loops as two kernels (the
// update, then the stencil with variant UNFUSED_STN into the second buffer)
constexpr int V3_UNFUSED = V3, UNFUSED_STN = 13;
// ... and the pair overlapped (V3_OVERLAP, V3_OVERLAP_Q): the HBM-bound update
// and the stencil (variant 13, or the q61 stencil 14) in OVL_CHUNKS chunks of
// planes, the updates on the caller's stream, the stencils on a second stream
// of the library; stencil chunk q waits for update chunk q+1 (it reads A up to
// the first plane of the next chunk), and nothing an update reads is written
// by a stencil running beside it
constexpr int V3_OVERLAP = V3 + 1, V3_OVERLAP_Q = V3 + 2, OVL_CHUNKS = 8;
// ... and the one-pass fixed-point pair (kStencil3QF), registers capped for
// four / three CTAs per SM
constexpr int V3_QF = V3 + 3;
bool isQF(int v) { return v == V3_QF || v == V3_QF + 1; }
// ... and the one-pass pair with its planes staged by TMA (kStencil3T<true>),
// a ring of 5 / 4 planes, four CTAs per SM
constexpr int V3_TF = V3 + 5;
bool isTF(int v) { return v == V3_TF || v == V3_TF + 1; }

// the TMA-staged stencil alone (kStencil3T, M = 0) with NS slots and W
// FP64-unit warps; a launch above 48 KB of shared memory is opted in once per
// device
template <int NS, int W>
int launchT(const CUtensorMap &map, double *A, double *Out, const Box3 &b, const St3Geom &g, cudaStream_t s) {
    const int smem = tma::smemBytes(false, NS, W > 0);
    if (smem > 48 * 1024) {
        static std::atomic<unsigned long long> optedIn{0};
        const int dev = gbdev::current();
        if (dev < 0 || dev >= 64) return -1;
        if (!(optedIn.load() >> dev & 1ull)) {
            if (cudaFuncSetAttribute(kStencil3T<0, NS, 4, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                cudaSuccess)
                return -1;
            optedIn.fetch_or(1ull << dev);
        }
    }
    kStencil3T<0, NS, 4, W><<<g.grid, dim3(TX, TY), smem, s>>>(map, map, map, A, nullptr, Out, b, g.p0, g.ichunk,
                                                               nullptr, dvmhgb_status_word(), nullptr, 0);
    return 0;
}

template <bool FUSED>
void launch3(int variant, const St3Geom &g, double *A, const double *B, double *Out, const Box3 &b, double *items,
             cudaStream_t s) {
    dim3 blk(TX, TY);
    switch (variant) {
#define C3(V)                                                                                       \
    case V: kStencil3<FUSED, (V) % 6, 1 + (V) / 6, 2><<<g.grid, blk, 0, s>>>(A, B, Out, b, g.p0, g.ichunk, items); break;
        C3(0) C3(1) C3(2) C3(3) C3(4) C3(5) C3(6) C3(7) C3(8) C3(9) C3(10) C3(11)
#undef C3
    case 12: kStencil3<FUSED, 5, 1, 3><<<g.grid, blk, 0, s>>>(A, B, Out, b, g.p0, g.ichunk, items); break;
    case 13: kStencil3<FUSED, 5, 1, 4><<<g.grid, blk, 0, s>>>(A, B, Out, b, g.p0, g.ichunk, items); break;
#define CQ(V, M, N, D) \
    case V: if (!FUSED) kStencil3Q<M, (N > 0)><<<g.grid, blk, 0, s>>>(A, Out, b, g.p0, g.ichunk, N, D); break;
        CQ(14, 4, 0, 1) CQ(15, 3, 0, 1) CQ(16, 4, 1, 2) CQ(17, 4, 1, 3) CQ(18, 4, 2, 5) CQ(19, 3, 1, 2)
        CQ(20, 4, 1, 4) CQ(21, 4, 3, 5)
#undef CQ
    }
}

template <bool FUSED>
void launch2(int native, const St2Geom &g, double *A, const double *B, double *Out, const Box2 &b, double *items,
             cudaStream_t s) {
    const int n = FUSED ? 4 : 3;
    native = native < 0 ? 0 : (native > n ? n : native);
    dim3 blk(TX, T2Y);
    switch (native) {
#define C2(N)                                                                                          \
    case N: kStencil2<FUSED, (FUSED ? N : (N > 3 ? 3 : N))><<<g.grid, blk, 0, s>>>(A, B, Out, b, g.p0, g.nstrips, g.ichunk, items); break;
        C2(0) C2(1) C2(2) C2(3) C2(4)
#undef C2
    }
}

}  // namespace

extern "C" {

long dvmhgb_jac3d_update_items(const long lo[3], const long hi[3]) {
    return updGeom(hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, lo[2], hi[2]).blocks;
}

int dvmhgb_jac3d_update(double *A, const double *B, const long st[3], const long lo[3], const long hi[3],
                        double *items, int native, void *stream) {
    UpdGeom g = updGeom(hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, lo[2], hi[2]);
    if (!g.ok || !A || !B || !items || !rows16(st, 3) || !aligned16(A) || !aligned16(B)) return -1;
    kUpdate<<<(unsigned)g.blocks, UPD_THREADS, 0, (cudaStream_t)stream>>>(A, B, st[0], st[1], lo[0], lo[1], lo[2],
                                                                          hi[2], g.nj, g.units, g.nseg, g.p0, g.p1,
                                                                          items, native);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_jac3d_stencil(const double *A, double *B, const long st[3], const long ext[3], const long lo[3],
                         const long hi[3], int native, void *stream) {
    if (native < 0 || native >= V3) return -1;
    St3Geom g = st3Geom(lo, hi, TY * jtOf3(native));
    if (!g.ok || !A || !B || !rows16(st, 3) || !aligned16(A) || !aligned16(B)) return -1;
    Box3 b{st[0], st[1], ext[0], ext[1], ext[2], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
    if (isT3(native)) {
        CUtensorMap map;
        if (!encodeMap3(&map, A, ext, st, tma::BX, tma::BY)) return -1;
        cudaStream_t s = (cudaStream_t)stream;
        double *a = (double *)A;
        switch (native - V3T) {
#define CT(V, NS, W) \
    case V: if (launchT<NS, W>(map, a, B, b, g, s) != 0) return -1; break;
            CT(0, 6, 0) CT(1, 4, 0) CT(2, 6, 1) CT(3, 6, 2) CT(4, 6, 3)
#undef CT
        }
    } else {
        launch3<false>(native, g, (double *)A, nullptr, B, b, nullptr, (cudaStream_t)stream);
    }
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// plane range of chunk q of K over [lo0, hi0]
void ovlChunk(const long lo[3], const long hi[3], int q, int K, long clo[3], long chi[3]) {
    const long n = hi[0] - lo[0] + 1;
    for (int d = 0; d < 3; d++) clo[d] = lo[d], chi[d] = hi[d];
    clo[0] = lo[0] + n * q / K;
    chi[0] = lo[0] + n * (q + 1) / K - 1;
}

int ovlCount(const long lo[3], const long hi[3]) {
    const long n = hi[0] - lo[0] + 1;
    return (int)(n < OVL_CHUNKS ? n : OVL_CHUNKS);
}

long ovlItems(const long lo[3], const long hi[3]) {
    const int K = ovlCount(lo, hi);
    long total = 0;
    for (int q = 0; q < K; q++) {
        long clo[3], chi[3];
        ovlChunk(lo, hi, q, K, clo, chi);
        total += dvmhgb_jac3d_update_items(clo, chi);
    }
    return total;
}

// the second stream and the events of the overlapped pair, per device (created
// on the first use on that device)
constexpr int OVL_DEVICES = 64;
struct Ovl {
    bool ready = false;
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev[OVL_CHUNKS + 1] = {};
};
Ovl ovlState[OVL_DEVICES];

Ovl *ovlFor() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= OVL_DEVICES) return nullptr;
    Ovl &o = ovlState[dev];
    if (!o.ready) {
        if (cudaStreamCreateWithFlags(&o.s2, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        for (auto &e : o.ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        o.ready = true;
    }
    return &o;
}

int runOverlap(double *A, const double *B, const long st[3], const long ext[3], const long lo[3], const long hi[3],
               double *items, int stencilVariant, cudaStream_t s1) {
    Ovl *op = ovlFor();
    if (!op) return -1;
    Ovl &o = *op;
    const int K = ovlCount(lo, hi);
    long clo[OVL_CHUNKS][3], chi[OVL_CHUNKS][3];
    for (int q = 0; q < K; q++) ovlChunk(lo, hi, q, K, clo[q], chi[q]);
    double *it = items;
    for (int q = 0; q < K; q++) {  // the updates, in order, on the caller's stream
        if (dvmhgb_jac3d_update(A, B, st, clo[q], chi[q], it, 2, s1) != 0) return -1;
        it += dvmhgb_jac3d_update_items(clo[q], chi[q]);
        if (cudaEventRecord(o.ev[q], s1) != cudaSuccess) return -1;
    }
    for (int q = 0; q < K; q++) {  // the stencils on the second stream, each after the update it reads
        if (cudaStreamWaitEvent(o.s2, o.ev[q + 1 < K ? q + 1 : K - 1], 0) != cudaSuccess) return -1;
        if (dvmhgb_jac3d_stencil(A, (double *)B, st, ext, clo[q], chi[q], stencilVariant, o.s2) != 0) return -1;
    }
    if (cudaEventRecord(o.ev[OVL_CHUNKS], o.s2) != cudaSuccess) return -1;
    return cudaStreamWaitEvent(s1, o.ev[OVL_CHUNKS], 0) == cudaSuccess ? 0 : -1;  // join
}

long dvmhgb_jac3d_fused_items(const long lo[3], const long hi[3], int native) {
    if (native == V3_UNFUSED || isQ3(native)) return dvmhgb_jac3d_update_items(lo, hi);
    if (native == V3_OVERLAP || native == V3_OVERLAP_Q) return ovlItems(lo, hi);
    if (isQF(native) || isTF(native)) {
        St3Geom g = st3Geom(lo, hi, TY);
        return (long)g.grid.x * g.grid.y * g.grid.z;
    }
    if (native < 0 || native >= V3) return -1;
    St3Geom g = st3Geom(lo, hi, TY * jtOf3(native));
    return (long)g.grid.x * g.grid.y * g.grid.z;
}

int dvmhgb_jac3d_fused(double *A, const double *B, double *Bnew, const long st[3], const long ext[3],
                       const long lo[3], const long hi[3], double *items, int native, void *stream) {
    if (native == V3_UNFUSED || isQ3(native)) {
        if (dvmhgb_jac3d_update(A, B, st, lo, hi, items, 2, stream) != 0 ||
            dvmhgb_jac3d_stencil(A, Bnew, st, ext, lo, hi, isQ3(native) ? native : UNFUSED_STN, stream) != 0)
            return -1;
        // Bnew == B: the stencil wrote B in place of the second buffer (it reads only A)
        return Bnew == B ? 0 : dvmhgb_copy_outside_box(3, B, Bnew, st, ext, lo, hi, stream);
    }
    if (native == V3_OVERLAP || native == V3_OVERLAP_Q) {
        if (Bnew != B || !A || !B || !items || !rows16(st, 3) || !aligned16(A) || !aligned16(B)) return -1;
        return runOverlap(A, B, st, ext, lo, hi, items, native == V3_OVERLAP ? UNFUSED_STN : V3Q,
                          (cudaStream_t)stream);
    }
    if (Bnew == B) return -1;  // the fused kernel reads B while it writes the next B
    if (isTF(native)) {
        St3Geom g = st3Geom(lo, hi, TY);
        if (!g.ok || !A || !B || !Bnew || A == B || !items || !rows16(st, 3) || !aligned16(A) || !aligned16(B) ||
            !aligned16(Bnew))
            return -1;
        Box3 b{st[0], st[1], ext[0], ext[1], ext[2], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
        CUtensorMap mapB, mapA, mapT;
        if (!encodeMap3(&mapB, B, ext, st, tma::BX, tma::BY) || !encodeMap3(&mapA, A, ext, st, tma::BX, tma::BY) ||
            !encodeMap3(&mapT, A, ext, st, 2 * TX, TY))
            return -1;
        dim3 blk(TX, TY);
        cudaStream_t s = (cudaStream_t)stream;
        int *status = dvmhgb_status_word();
        if (native == V3_TF)
            kStencil3T<2, 5, 4, 0><<<g.grid, blk, tma::smemBytes(true, 5), s>>>(mapB, mapA, mapT, A, B, Bnew, b, g.p0,
                                                                                g.ichunk, items, status, nullptr, 0);
        else
            kStencil3T<2, 5, 3, 0><<<g.grid, blk, tma::smemBytes(true, 5), s>>>(mapB, mapA, mapT, A, B, Bnew, b, g.p0,
                                                                                g.ichunk, items, status, nullptr, 0);
        dvmhgb_count_launches(1);
        if (cudaGetLastError() != cudaSuccess) return -1;
        return dvmhgb_copy_outside_box(3, B, Bnew, st, ext, lo, hi, stream);
    }
    if (isQF(native)) {
        St3Geom g = st3Geom(lo, hi, TY);
        if (!g.ok || !A || !B || !Bnew || !items || !rows16(st, 3) || !aligned16(A) || !aligned16(B) ||
            !aligned16(Bnew))
            return -1;
        Box3 b{st[0], st[1], ext[0], ext[1], ext[2], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
        dim3 blk(TX, TY);
        if (native == V3_QF)
            kStencil3QF<4><<<g.grid, blk, 0, (cudaStream_t)stream>>>(A, B, Bnew, b, g.p0, g.ichunk, items);
        else
            kStencil3QF<3><<<g.grid, blk, 0, (cudaStream_t)stream>>>(A, B, Bnew, b, g.p0, g.ichunk, items);
        dvmhgb_count_launches(1);
        if (cudaGetLastError() != cudaSuccess) return -1;
        return dvmhgb_copy_outside_box(3, B, Bnew, st, ext, lo, hi, stream);
    }
    if (native < 0 || native >= V3) return -1;
    St3Geom g = st3Geom(lo, hi, TY * jtOf3(native));
    if (!g.ok || !A || !B || !Bnew || !items || !rows16(st, 3) || !aligned16(A) || !aligned16(B) || !aligned16(Bnew))
        return -1;
    Box3 b{st[0], st[1], ext[0], ext[1], ext[2], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
    launch3<true>(native, g, A, B, Bnew, b, items, (cudaStream_t)stream);
    dvmhgb_count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return -1;
    return dvmhgb_copy_outside_box(3, B, Bnew, st, ext, lo, hi, stream);
}

long dvmhgb_jac3d_stnupd_items(const long lo[3], const long hi[3], int variant) {
    if (variant < 0 || variant >= DVMHGB_JAC3D_STNUPD_VARIANTS) return -1;
    St3Geom g = st3Geom(lo, hi, TY);
    return (long)g.grid.x * g.grid.y * g.grid.z;
}

int dvmhgb_jac3d_stnupd(const double *A, double *Aalt, double *B, const long st[3], const long ext[3],
                        const long lo[3], const long hi[3], double *items, int variant, void *stream) {
    if (variant < 0 || variant >= DVMHGB_JAC3D_STNUPD_VARIANTS) return -1;
    St3Geom g = st3Geom(lo, hi, TY);
    if (!g.ok || !A || !Aalt || !B || !items || A == Aalt || A == B || Aalt == B || !rows16(st, 3) ||
        !aligned16(A) || !aligned16(Aalt) || !aligned16(B))
        return -1;
    Box3 b{st[0], st[1], ext[0], ext[1], ext[2], lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
    CUtensorMap map;
    if (!encodeMap3(&map, A, ext, st, tma::BX, tma::BY)) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    double *a = (double *)A;
    const int smem = tma::smemBytes(false, 6, true);  // above 48 KB: opted in once per device
    static std::atomic<unsigned long long> optedIn{0};
    const int dev = gbdev::current();
    if (dev < 0 || dev >= 64) return -1;
    if (!(optedIn.load() >> dev & 1ull)) {
        if (cudaFuncSetAttribute(kStencil3T<3, 6, 4, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(kStencil3T<3, 6, 4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(kStencil3T<3, 6, 4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                cudaSuccess)
            return -1;
        optedIn.fetch_or(1ull << dev);
    }
    int *status = dvmhgb_status_word();
    const dim3 blk(TX, TY);
    // (FP64-unit warps, warps with the integer-pipe |B - A|) of each variant
    static const int wq[DVMHGB_JAC3D_STNUPD_VARIANTS][2] = {{0, 0}, {1, 0}, {2, 0}, {1, 2}, {1, 4}, {2, 3}};
    const int w = wq[variant][0], qe = wq[variant][1];
    if (w == 0)
        kStencil3T<3, 6, 4, 0><<<g.grid, blk, smem, s>>>(map, map, map, a, nullptr, B, b, g.p0, g.ichunk, items, status,
                                                         Aalt, qe);
    else if (w == 1)
        kStencil3T<3, 6, 4, 1><<<g.grid, blk, smem, s>>>(map, map, map, a, nullptr, B, b, g.p0, g.ichunk, items, status,
                                                         Aalt, qe);
    else
        kStencil3T<3, 6, 4, 2><<<g.grid, blk, smem, s>>>(map, map, map, a, nullptr, B, b, g.p0, g.ichunk, items, status,
                                                         Aalt, qe);
    dvmhgb_count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return -1;
    return dvmhgb_copy_outside_box(3, A, Aalt, st, ext, lo, hi, stream);  // A's cells outside the box carry over
}

long dvmhgb_jac2d_update_items(const long lo[2], const long hi[2]) {
    return updGeom(hi[0] - lo[0] + 1, 1, lo[1], hi[1]).blocks;
}

int dvmhgb_jac2d_update(double *A, const double *B, const long st[2], const long lo[2], const long hi[2],
                        double *items, int native, void *stream) {
    UpdGeom g = updGeom(hi[0] - lo[0] + 1, 1, lo[1], hi[1]);
    if (!g.ok || !A || !B || !items || !rows16(st, 2) || !aligned16(A) || !aligned16(B)) return -1;
    kUpdate<<<(unsigned)g.blocks, UPD_THREADS, 0, (cudaStream_t)stream>>>(A, B, st[0], 0, lo[0], 0, lo[1], hi[1],
                                                                          g.nj, g.units, g.nseg, g.p0, g.p1, items, native);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_jac2d_stencil(const double *A, double *B, const long st[2], const long ext[2], const long lo[2],
                         const long hi[2], int native, void *stream) {
    St2Geom g = st2Geom(lo, hi);
    if (!g.ok || !A || !B || !rows16(st, 2) || !aligned16(A) || !aligned16(B)) return -1;
    Box2 b{st[0], ext[0], ext[1], lo[0], lo[1], hi[0], hi[1]};
    launch2<false>(native, g, (double *)A, nullptr, B, b, nullptr, (cudaStream_t)stream);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

long dvmhgb_jac2d_fused_items(const long lo[2], const long hi[2]) {
    St2Geom g = st2Geom(lo, hi);
    return (long)g.grid.x * g.grid.y;
}

int dvmhgb_jac2d_fused(double *A, const double *B, double *Bnew, const long st[2], const long ext[2],
                       const long lo[2], const long hi[2], double *items, int native, void *stream) {
    St2Geom g = st2Geom(lo, hi);
    if (!g.ok || !A || !B || !Bnew || !items || !rows16(st, 2) || !aligned16(A) || !aligned16(B) || !aligned16(Bnew))
        return -1;
    Box2 b{st[0], ext[0], ext[1], lo[0], lo[1], hi[0], hi[1]};
    launch2<true>(native, g, A, B, Bnew, b, items, (cudaStream_t)stream);
    dvmhgb_count_launches(1);
    if (cudaGetLastError() != cudaSuccess) return -1;
    return dvmhgb_copy_outside_box(2, B, Bnew, st, ext, lo, hi, stream);
}

}  // extern "C"

// ---------------------------------------------------------------- update loop without allocation
//
// For callers that cannot allocate device memory: code running while a CUDA
// stream is being captured into a graph in global capture mode (cudaMalloc is
// illegal there and would also synchronise the device), hosts whose own
// allocator owns all of the GPU's memory and forbids other allocations, or
// code on a latency-critical path that must not block in the driver.  The
// per-CTA partial maxima live in this file-scope array instead of a buffer the
// caller or the runtime allocates.  Every GPU that loads the library holds it
// (32 KB) until the process exits.  Every call uses the same array and leaves
// its partials there; nothing in it needs to start at zero, because each call
// writes every entry it later reads.  Calls whose GPU work overlaps in time
// (different streams, or host threads without ordering) race on the array.
namespace {

constexpr long NOALLOC_PARTIALS = 4096;  // maximum CTAs of one call
static __device__ __align__(256) double noallocPartials[NOALLOC_PARTIALS];

// eps = the largest partial (MAX is order-independent)
__global__ void __launch_bounds__(256) kMaxPartials(const double *partials, long n, double *eps) {
    __shared__ double sh[8];
    double m = -__builtin_huge_val();
    for (long i = threadIdx.x; i < n; i += blockDim.x) m = maxOf(partials[i], m);
    m = ctaMax(m, sh);
    if (threadIdx.x == 0) eps[0] = m;
}

// device address of noallocPartials on each device, looked up once per device
// (a lookup races harmlessly with another: both store the same address)
constexpr int MAX_DEVICES = 64;
std::atomic<double *> noallocAddr[MAX_DEVICES];

}  // namespace

extern "C" {

int dvmhgb_jac3d_update_noalloc(double *A, const double *B, const long st[3], const long lo[3], const long hi[3],
                                double *epsDev, void *stream) {
    if (!A || !B || !epsDev || !st || !lo || !hi || !rows16(st, 3) || !aligned16(A) || !aligned16(B)) return -1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return -3;
    double *partials = noallocAddr[dev].load(std::memory_order_acquire);
    if (!partials) {
        // first call on this device: take the array's address with the device current
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, noallocPartials);
        if (e != cudaSuccess) {
            fprintf(stderr, "dvmhgb_jac3d_update_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                    cudaGetErrorString(e));
            return -3;
        }
        partials = (double *)p;
        noallocAddr[dev].store(partials, std::memory_order_release);
    }
    UpdGeom g = updGeom(hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, lo[2], hi[2]);
    if (!g.ok) return -1;
    if (g.blocks > NOALLOC_PARTIALS) {
        fprintf(stderr,
                "dvmhgb_jac3d_update_noalloc: this launch needs %ld partial slots, the static array has %ld "
                "(use dvmhgb_jac3d_update with a caller-provided buffer)\n",
                g.blocks, NOALLOC_PARTIALS);
        return -2;
    }
    cudaStream_t s = (cudaStream_t)stream;
    kUpdate<<<(unsigned)g.blocks, UPD_THREADS, 0, s>>>(A, B, st[0], st[1], lo[0], lo[1], lo[2], hi[2], g.nj, g.units,
                                                       g.nseg, g.p0, g.p1, partials, 1);
    kMaxPartials<<<1, 256, 0, s>>>(partials, g.blocks, epsDev);
    dvmhgb_count_launches(2);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int dvmhgb_copy_outside_box(int rank, const double *src, double *dst, const long *st, const long *ext,
                            const long *lo, const long *hi, void *stream) {
    if (rank < 1 || rank > 3) return -1;
    Slabs s{};
    s.rank = rank;
    for (int d = 0; d < rank; d++) s.st[d] = st[d];
    s.start[0] = 0;
    // slab (d, side): axis d outside [lo_d, hi_d] on one side, axes < d inside, axes > d anything
    for (int d = 0; d < rank; d++)
        for (int side = 0; side < 2; side++) {
            long a = side == 0 ? 0 : hi[d] + 1, z = side == 0 ? lo[d] - 1 : ext[d] - 1;
            if (z < a) continue;
            int q = s.n;
            long cells = 1;
            for (int e = 0; e < rank; e++) {
                long l, h;
                if (e < d) { l = lo[e]; h = hi[e]; }
                else if (e == d) { l = a; h = z; }
                else { l = 0; h = ext[e] - 1; }
                s.lo[q][e] = l;
                s.cnt[q][e] = h - l + 1;
                cells *= h - l + 1;
            }
            s.start[q + 1] = s.start[q] + cells;
            s.n++;
        }
    if (s.n == 0) return 0;
    long total = s.start[s.n];
    long blocks = (total + 255) / 256;
    if (blocks > (long)smCount() * 8) blocks = (long)smCount() * 8;
    kCopyOutside<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(src, dst, s);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // extern "C"
