// Explicit 2-D heat step with SUM and MINLOC reductions, FP64, for sm_103a:
// the loop of dvm-snapshot-r6603-fork_gb300/workloads/heat.c
//   dst[i][j] = src[i][j] + c * (src[i-1][j] + src[i+1][j] + src[i][j-1] + src[i][j+1] - 4.0 * src[i][j])
//   sum += dst[i][j];  if (dst[i][j] < mn) { mn = dst[i][j]; loc = {i, j}; }
//
// A warp handles one unit: a row i and a 64-wide chunk of j aligned to a
// multiple of 64 of the array index (lane l holds j = base+2l, base+2l+1 as one
// 128-bit access).  Per unit it writes one SUM item -- the pairwise tree over
// the chunk's 64 positions (pair sum, then xor-butterfly 1..16), the canonical
// order the reduction engine folds -- and one MINLOC item: the smallest value,
// ties to the smallest j, i.e. the first in loop order, as the strict '<' of
// the source gives.  Items are in row-major (row, chunk) order.
//
// The same unit code serves one array (plain per-loop launches) and a table
// of arrays of uneven sizes (batched mode): there units of all arrays form one
// index space that a persistent grid strides over, so small and large arrays
// share the GPU in a single launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"

namespace {

constexpr int HT = 256;  // threads per CTA (8 warps)

struct Unit {
    long i, ch;
};

__device__ __forceinline__ uint64_t minKey(double v) {
    // IEEE order as unsigned order; -0 keyed as +0 (they compare equal); NaN last
    uint64_t b = (uint64_t)__double_as_longlong(v);
    if ((b & 0x7FFFFFFFFFFFFFFFull) == 0) b = 0;
    if ((b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return ~0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ void heatUnit(const dvmhgb_heat_desc &d, long u) {
    const int lane = threadIdx.x & 31;
    const long r = u / d.nck, ch = u - r * d.nck;
    const long i = d.lo0 + r;
    const long base = (d.c0 + ch) * 64;
    const long j = base + 2 * lane;
    const double c = *d.coef;
    const double *row = d.src + i * d.s0;
    // element pairs of rows i-1, i, i+1; only pairs that hold a cell of the loop or
    // its right neighbour are read (j <= hi1+1 keeps j+1 inside the 16-byte padded row)
    const bool need = j <= d.hi1 + 1;
    const double2 z = make_double2(0.0, 0.0);
    double2 up = need ? *reinterpret_cast<const double2 *>(row - d.s0 + j) : z;
    double2 mid = need ? *reinterpret_cast<const double2 *>(row + j) : z;
    double2 dn = need ? *reinterpret_cast<const double2 *>(row + d.s0 + j) : z;
    double left = __shfl_up_sync(0xffffffffu, mid.y, 1), right = __shfl_down_sync(0xffffffffu, mid.x, 1);
    if (lane == 0) left = j >= 1 ? row[j - 1] : 0.0;
    if (lane == 31) right = (j + 2 <= d.hi1 + 1) ? row[j + 2] : 0.0;
    const bool in0 = j >= d.lo1 && j <= d.hi1, in1 = j + 1 >= d.lo1 && j + 1 <= d.hi1;
    double v0 = mid.x + c * ((((up.x + dn.x) + left) + mid.y) - 4.0 * mid.x);
    double v1 = mid.y + c * ((((up.y + dn.y) + mid.x) + right) - 4.0 * mid.y);
    double *out = d.dst + i * d.s0 + j;
    if (in0 && in1) *reinterpret_cast<double2 *>(out) = make_double2(v0, v1);
    else if (in0) out[0] = v0;
    else if (in1) out[1] = v1;
    // SUM: pairwise tree over the chunk's positions, -0.0 outside the loop
    double s = (in0 ? v0 : -0.0) + (in1 ? v1 : -0.0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
    // MINLOC: smallest key, then smallest j
    uint64_t k0 = in0 ? minKey(v0) : ~0ull, k1 = in1 ? minKey(v1) : ~0ull;
    uint64_t key = k0;
    double val = v0;
    long jj = j;
    if (k1 < k0) {
        key = k1;
        val = v1;
        jj = j + 1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t ok = __shfl_down_sync(0xffffffffu, key, o);
        double ov = __shfl_down_sync(0xffffffffu, val, o);
        long oj = __shfl_down_sync(0xffffffffu, jj, o);
        if (ok < key || (ok == key && oj < jj)) {
            key = ok;
            val = ov;
            jj = oj;
        }
    }
    if (lane == 0) {
        long item = r * d.nck + ch;
        d.sumItems[item] = s;
        d.minItems[item] = key == ~0ull ? __builtin_huge_val() : val;
        d.locItems[2 * item] = (int)i;
        d.locItems[2 * item + 1] = (int)jj;
    }
}

__global__ void __launch_bounds__(HT) kHeatOne(dvmhgb_heat_desc d) {
    const long units = d.units;
    for (long u = (blockIdx.x * (long)HT + threadIdx.x) >> 5; u < units; u += (long)gridDim.x * (HT / 32))
        heatUnit(d, u);
}

// units of array k are [d[k].unitBase, d[k].unitBase + d[k].units)
__global__ void __launch_bounds__(HT) kHeatMany(const dvmhgb_heat_desc *__restrict__ ds, int n, long total) {
    for (long u = (blockIdx.x * (long)HT + threadIdx.x) >> 5; u < total; u += (long)gridDim.x * (HT / 32)) {
        int lo = 0, hi = n - 1;  // last array whose unitBase <= u
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (ds[mid].unitBase <= u) lo = mid;
            else hi = mid - 1;
        }
        heatUnit(ds[lo], u - ds[lo].unitBase);
    }
}

int smCount() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 152;
    }
    return n;
}

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
    d->sumItems = d->minItems = nullptr;
    d->locItems = nullptr;
    return 0;
}

int dvmhgb_heat(const dvmhgb_heat_desc *d, void *stream) {
    if (!d || !d->sumItems || !d->minItems || !d->locItems) return -1;
    long blocks = (d->units + HT / 32 - 1) / (HT / 32);
    if (blocks > (long)smCount() * 8) blocks = (long)smCount() * 8;
    kHeatOne<<<(unsigned)blocks, HT, 0, (cudaStream_t)stream>>>(*d);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_heat_many(const dvmhgb_heat_desc *dDev, int n, long totalUnits, void *stream) {
    if (!dDev || n < 1 || totalUnits < 1) return -1;
    long blocks = (totalUnits + HT / 32 - 1) / (HT / 32);
    if (blocks > (long)smCount() * 8) blocks = (long)smCount() * 8;
    kHeatMany<<<(unsigned)blocks, HT, 0, (cudaStream_t)stream>>>(dDev, n, totalUnits);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // extern "C"
