// Explicit 2-D heat step with SUM and MINLOC reductions, FP64, for sm_103a:
// the loop of dvm-snapshot-r6603-fork_gb300/workloads/heat.c
//   dst[i][j] = src[i][j] + c * (src[i-1][j] + src[i+1][j] + src[i][j-1] + src[i][j+1] - 4.0 * src[i][j])
//   sum += dst[i][j];  if (dst[i][j] < mn) { mn = dst[i][j]; loc = {i, j}; }
//
// A warp walks a strip: up to DVMHGB_HEAT_STRIP consecutive rows of one
// 64-wide chunk of j aligned to a multiple of 64 of the array index (lane l
// holds j = base+2l, base+2l+1 as one 128-bit access).  Rows i-1, i, i+1 roll
// through registers with row i+2 in flight, so every source row is read once
// per chunk; lanes 0 and 31 also fetch the chunk's edge columns.  Per row the
// warp writes one SUM item -- the pairwise tree over the chunk's 64 positions
// (pair sum, then xor-butterfly 1..16), the canonical order the reduction
// engine folds -- and one MINLOC item: the smallest value, ties to the
// smallest j, i.e. the first in loop order, as the strict '<' of the source
// gives.  Items are in row-major (row, chunk) order.
//
// The same strip code serves one array (plain per-loop launches) and a table
// of arrays of uneven sizes (batched mode): there the strips of all arrays
// form one index space that a persistent grid strides over (strip bases
// cached in shared memory), so small and large arrays share the GPU in a
// single launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"
#include "devinfo.cuh"
#include "softfp64.cuh"

namespace {

constexpr int HT = 256;  // threads per CTA (8 warps)

__device__ __forceinline__ uint64_t minKey(double v) {
    // IEEE order as unsigned order; -0 keyed as +0 (they compare equal); NaN last
    uint64_t b = (uint64_t)__double_as_longlong(v);
    if ((b & 0x7FFFFFFFFFFFFFFFull) == 0) b = 0;
    if ((b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return ~0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

constexpr int MAX_CACHED = 2048;  // strip bases cached in shared memory

__device__ __forceinline__ double2 ldRow(const double *row, long j, bool need) {
    return need ? *reinterpret_cast<const double2 *>(row + j) : make_double2(0.0, 0.0);
}

// strip `local` of loop d: chunk local / nrb, rows (local % nrb) * sr ...
__device__ __forceinline__ void heatStrip(const dvmhgb_heat_desc &d, long local) {
    const int lane = threadIdx.x & 31;
    const long nrows = d.hi0 - d.lo0 + 1;
    const long sr = d.sr;
    const unsigned nrb = (unsigned)((nrows + sr - 1) / sr);
    const unsigned ch = (unsigned)local / nrb, rb = (unsigned)local - ch * nrb;
    const long r0 = (long)rb * sr, r1 = r0 + sr < nrows ? r0 + sr : nrows;
    const long base = (d.c0 + ch) * 64;
    const long j = base + 2 * lane;
    const bool need = j <= d.hi1 + 1;  // the pair holds a cell of the loop or its right neighbour
    const bool in0 = j >= d.lo1 && j <= d.hi1, in1 = j + 1 >= d.lo1 && j + 1 <= d.hi1;
    // edge columns: lane 0 the left neighbour of j = base, lane 31 the right one of base + 63
    const long ej = lane == 0 ? j - 1 : j + 2;
    const bool eNeed = (lane == 0 && j >= 1) || (lane == 31 && j + 2 <= d.hi1 + 1);
    const double c = *d.coef;
    const long s0 = d.s0;
    const double *p = d.src + (d.lo0 + r0 - 1) * s0;  // row i-1 of the first row
    double2 up = ldRow(p, j, need), mid = ldRow(p + s0, j, need), dn = ldRow(p + 2 * s0, j, need);
    double emid = eNeed ? p[s0 + ej] : 0.0, edn = eNeed ? p[2 * s0 + ej] : 0.0;
    for (long r = r0; r < r1; r++) {
        const long i = d.lo0 + r;
        const double *pn = d.src + (i + 2) * s0;  // row i+2, in flight (exists while r + 1 < r1)
        const bool more = r + 1 < r1;
        const double2 dn2 = ldRow(pn, j, need && more);
        const double edn2 = (eNeed && more) ? pn[ej] : 0.0;
        double left = __shfl_up_sync(0xffffffffu, mid.y, 1), right = __shfl_down_sync(0xffffffffu, mid.x, 1);
        if (lane == 0) left = emid;
        if (lane == 31) right = emid;
        // 4.0 * mid is exact: an exponent increment on the integer pipe unless a
        // lane of the warp holds a subnormal, infinite or huge value
        double m4x, m4y;
        if (__all_sync(0xffffffffu, sf::scale_up_ok(mid.x, 2) && sf::scale_up_ok(mid.y, 2))) {
            m4x = sf::scale_up(mid.x, 2);
            m4y = sf::scale_up(mid.y, 2);
        } else {
            m4x = 4.0 * mid.x;
            m4y = 4.0 * mid.y;
        }
        const double v0 = mid.x + c * ((((up.x + dn.x) + left) + mid.y) - m4x);
        const double v1 = mid.y + c * ((((up.y + dn.y) + mid.x) + right) - m4y);
        double *out = d.dst + i * s0 + j;
        if (in0 && in1) *reinterpret_cast<double2 *>(out) = make_double2(v0, v1);
        else if (in0) out[0] = v0;
        else if (in1) out[1] = v1;
        // SUM: pairwise tree over the chunk's positions, -0.0 outside the loop.
        // When every value of the chunk is +0 or a positive normal below 2^1009
        // the levels above the pairs run on the integer pipe (sf::add_pos); the
        // positions outside the loop then count as +0, which gives the same
        // sum, since the chunk has a cell of the loop and no sum is negative.
        double s;
        if (__all_sync(0xffffffffu, (!in0 || sf::pos_small(v0)) && (!in1 || sf::pos_small(v1)))) {
            s = (in0 ? v0 : 0.0) + (in1 ? v1 : 0.0);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) s = sf::add_pos(s, __shfl_xor_sync(0xffffffffu, s, o));
        } else {
            s = (in0 ? v0 : -0.0) + (in1 ? v1 : -0.0);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
        }
        // MINLOC: smallest key, then smallest j; the value comes from the winning lane
        const uint64_t k0 = in0 ? minKey(v0) : ~0ull, k1 = in1 ? minKey(v1) : ~0ull;
        uint64_t key = k1 < k0 ? k1 : k0;
        int jo = 2 * lane + (k1 < k0 ? 1 : 0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ok = __shfl_down_sync(0xffffffffu, key, o);
            const int oj = __shfl_down_sync(0xffffffffu, jo, o);
            if (ok < key || (ok == key && oj < jo)) {
                key = ok;
                jo = oj;
            }
        }
        jo = __shfl_sync(0xffffffffu, jo, 0);
        const double mine = (jo & 1) ? v1 : v0;
        const double val = __shfl_sync(0xffffffffu, mine, jo >> 1);
        if (lane == 0) {
            const long item = r * d.nck + ch;
            d.sumItems[item] = s;
            d.minItems[item] = key == ~0ull ? __builtin_huge_val() : val;
            d.locItems[2 * item] = (int)i;
            d.locItems[2 * item + 1] = (int)(base + jo);
        }
        up = mid;
        mid = dn;
        dn = dn2;
        emid = edn;
        edn = edn2;
    }
}

__global__ void __launch_bounds__(HT) kHeatOne(dvmhgb_heat_desc d) {
    for (long s = (blockIdx.x * (long)HT + threadIdx.x) >> 5; s < d.strips; s += (long)gridDim.x * (HT / 32))
        heatStrip(d, s);
}

// strips of array k are [d[k].stripBase, d[k].stripBase + d[k].strips)
__global__ void __launch_bounds__(HT) kHeatMany(const dvmhgb_heat_desc *__restrict__ ds, int n, long total) {
    __shared__ long sb[MAX_CACHED];
    const bool cached = n <= MAX_CACHED;
    if (cached)
        for (int q = threadIdx.x; q < n; q += HT) sb[q] = ds[q].stripBase;
    __syncthreads();
    for (long s = (blockIdx.x * (long)HT + threadIdx.x) >> 5; s < total; s += (long)gridDim.x * (HT / 32)) {
        int lo = 0, hi = n - 1;  // last array whose stripBase <= s
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((cached ? sb[mid] : ds[mid].stripBase) <= s) lo = mid;
            else hi = mid - 1;
        }
        heatStrip(ds[lo], s - (cached ? sb[lo] : ds[lo].stripBase));
    }
}

int smCount() { return gbdev::smCount(); }

}  // namespace

extern "C" {

int dvmhgb_heat_desc_fill(dvmhgb_heat_desc *d, const double *src, double *dst, long rowStride, const long lo[2],
                          const long hi[2], const double *coefDev) {
    // 128-bit accesses: even row stride and 16-byte aligned bases
    if (!d || hi[0] < lo[0] || hi[1] < lo[1] || lo[0] < 1 || lo[1] < 1 || (rowStride & 1) ||
        ((uintptr_t)src & 15) || ((uintptr_t)dst & 15))
        return -1;
    d->src = src;
    d->dst = dst;
    d->s0 = rowStride;
    d->lo0 = lo[0];
    d->hi0 = hi[0];
    d->lo1 = lo[1];
    d->hi1 = hi[1];
    d->coef = coefDev;
    d->c0 = lo[1] / 64;
    d->nck = hi[1] / 64 - d->c0 + 1;
    d->units = (hi[0] - lo[0] + 1) * d->nck;
    d->unitBase = 0;
    d->sr = DVMHGB_HEAT_STRIP;
    d->strips = d->nck * ((hi[0] - lo[0] + d->sr) / d->sr);
    d->stripBase = 0;
    if (d->units >= (1L << 31) || d->strips >= (1L << 31)) return -1;
    d->sumItems = d->minItems = nullptr;
    d->locItems = nullptr;
    return 0;
}

int dvmhgb_heat(const dvmhgb_heat_desc *d, void *stream) {
    if (!d || !d->sumItems || !d->minItems || !d->locItems) return -1;
    // one loop alone: strips short enough that there is one for every warp the GPU holds
    dvmhgb_heat_desc e = *d;
    const long nrows = e.hi0 - e.lo0 + 1, warps = (long)smCount() * 8 * (HT / 32);
    long sr = (nrows * e.nck + warps - 1) / warps;
    e.sr = sr < 1 ? 1 : (sr > DVMHGB_HEAT_STRIP ? DVMHGB_HEAT_STRIP : sr);
    e.strips = e.nck * ((nrows + e.sr - 1) / e.sr);
    long blocks = (e.strips + HT / 32 - 1) / (HT / 32);
    if (blocks > (long)smCount() * 8) blocks = (long)smCount() * 8;
    kHeatOne<<<(unsigned)blocks, HT, 0, (cudaStream_t)stream>>>(e);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_heat_desc_rows(dvmhgb_heat_desc *d, long sr) {
    if (!d || sr < 1) return -1;
    d->sr = sr;
    d->strips = d->nck * ((d->hi0 - d->lo0 + sr) / sr);
    return d->strips < (1L << 31) ? 0 : -1;
}

int dvmhgb_heat_many_grid(const dvmhgb_heat_desc *dDev, int n, long totalStrips, int ctasPerSm, void *stream) {
    if (!dDev || n < 1 || totalStrips < 1 || ctasPerSm < 1 || ctasPerSm > 8) return -1;
    long blocks = (totalStrips + HT / 32 - 1) / (HT / 32);
    if (blocks > (long)smCount() * ctasPerSm) blocks = (long)smCount() * ctasPerSm;
    kHeatMany<<<(unsigned)blocks, HT, 0, (cudaStream_t)stream>>>(dDev, n, totalStrips);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_heat_many(const dvmhgb_heat_desc *dDev, int n, long totalStrips, void *stream) {
    return dvmhgb_heat_many_grid(dDev, n, totalStrips, 8, stream);
}

}  // extern "C"
