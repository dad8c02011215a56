// Synthetic parallel loops for the CUDA-block tuner: the shape of loop the
// tuner sees in DVMH programs, with the launch configuration as a parameter.
//
//   for x in box (rank 1..4):  v = in[x] + sum over axes a, offsets o = 1..R of
//                              (in[x - o e_a] + in[x + o e_a]);   out[x] = v
//   optional reduction of v: SUM / MAX / MINLOC (one partial per CTA)
//   optional ACROSS on the outermost loop axis: that axis runs in order inside
//   each thread (a dependence the launch cannot spread across threads)
// Element types: float, double, int.  The launch configuration is
// (bx, by, bz) threads, the loop axis mapped to threadIdx.x (the innermost --
// contiguous -- one or the outermost), and elements per thread along x.
// Arrays are padded by R on every side, innermost axis contiguous.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"

namespace {

struct Shape {
    int rank, radius, across;
    long ext[4];     // loop extents (innermost last)
    long st[4];      // array strides (elements), innermost 1
    long base;       // offset of loop point 0 inside the padded array
    int xaxis;       // loop axis on threadIdx.x
    int yaxis;       // loop axis on threadIdx.y (-1: none)
    int zaxes[4];    // loop axes folded into threadIdx.z / blockIdx.z
    int nz;
    int ept;         // elements per thread along x
};

template <typename T>
__device__ __forceinline__ T lowest() { return (T)-1e30; }
template <>
__device__ __forceinline__ int lowest<int>() { return (int)0x80000000; }
template <typename T>
__device__ __forceinline__ T highest() { return (T)1e30; }
template <>
__device__ __forceinline__ int highest<int>() { return 0x7fffffff; }

// RED: 0 none, 1 sum, 2 max, 3 minloc
template <typename T, int RED>
__global__ void kSynth(const T *__restrict__ in, T *__restrict__ out, Shape s, T *items, long *locs) {
    const long X = s.ext[s.xaxis], Y = s.yaxis >= 0 ? s.ext[s.yaxis] : 1;
    long Z = 1;
    for (int q = 0; q < s.nz; q++) Z *= s.ext[s.zaxes[q]];
    const long x0 = ((long)blockIdx.x * blockDim.x + threadIdx.x) * s.ept;
    const long y = (long)blockIdx.y * blockDim.y + threadIdx.y;
    T acc = RED == 1 ? (T)0 : (RED == 2 ? lowest<T>() : highest<T>());
    long accLoc = -1;
    auto body = [&](long z) {
        long zoff = 0, zr = z;
        for (int q = s.nz - 1; q >= 0; q--) {
            int a = s.zaxes[q];
            zoff += (zr % s.ext[a]) * s.st[a];
            zr /= s.ext[a];
        }
        for (int e = 0; e < s.ept; e++) {
            long x = x0 + e;
            if (x >= X) break;
            long off = s.base + zoff + x * s.st[s.xaxis] + (s.yaxis >= 0 ? y * s.st[s.yaxis] : 0);
            T v = in[off];
            for (int a = 0; a < s.rank; a++)
                for (int o = 1; o <= s.radius; o++) v = v + in[off - o * s.st[a]] + in[off + o * s.st[a]];
            out[off] = v;
            if (RED == 1) acc = acc + v;
            if (RED == 2) acc = v > acc ? v : acc;
            if (RED == 3 && v < acc) {
                acc = v;
                accLoc = off;
            }
        }
    };
    if (s.across) {
        // the dependent axis is walked in order, blockDim.z planes at a time, with a
        // barrier between steps; the trip count is the same for every thread of
        // the CTA (grid.z is 1 for ACROSS launches)
        for (long zz = 0; zz < Z; zz += blockDim.z) {
            long z = zz + threadIdx.z;
            if (y < Y && z < Z) body(z);
            __syncthreads();
        }
    } else if (y < Y) {
        for (long z = (long)blockIdx.z * blockDim.z + threadIdx.z; z < Z; z += (long)gridDim.z * blockDim.z) body(z);
    }
    if (RED) {
        // CTA reduction through shared memory (thread 0 combines in thread order)
        __shared__ T sv[1024];
        __shared__ long sl[1024];
        const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
        const int nt = blockDim.x * blockDim.y * blockDim.z;
        sv[t] = acc;
        sl[t] = accLoc;
        __syncthreads();
        if (t == 0) {
            T r = sv[0];
            long rl = sl[0];
            for (int q = 1; q < nt; q++) {
                if (RED == 1) r = r + sv[q];
                if (RED == 2) r = sv[q] > r ? sv[q] : r;
                if (RED == 3 && sv[q] < r) {
                    r = sv[q];
                    rl = sl[q];
                }
            }
            long b = blockIdx.x + (long)gridDim.x * (blockIdx.y + (long)gridDim.y * blockIdx.z);
            items[b] = r;
            if (RED == 3) locs[b] = rl;
        }
    }
}

template <typename T>
void launchT(int red, dim3 grid, dim3 blk, const void *in, void *out, const Shape &s, void *items, long *locs,
             cudaStream_t st) {
    switch (red) {
        case 0: kSynth<T, 0><<<grid, blk, 0, st>>>((const T *)in, (T *)out, s, (T *)items, locs); break;
        case 1: kSynth<T, 1><<<grid, blk, 0, st>>>((const T *)in, (T *)out, s, (T *)items, locs); break;
        case 2: kSynth<T, 2><<<grid, blk, 0, st>>>((const T *)in, (T *)out, s, (T *)items, locs); break;
        default: kSynth<T, 3><<<grid, blk, 0, st>>>((const T *)in, (T *)out, s, (T *)items, locs); break;
    }
}

bool shapeOf(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, Shape &s, dim3 &grid, dim3 &blk) {
    if (L->rank < 1 || L->rank > 4 || L->radius < 0 || L->radius > 3) return false;
    s.rank = L->rank;
    s.radius = L->radius;
    s.across = L->across ? 1 : 0;
    long c = 1;
    for (int a = L->rank - 1; a >= 0; a--) {
        s.ext[a] = L->ext[a];
        if (s.ext[a] < 1) return false;
        s.st[a] = c;
        c *= L->ext[a] + 2 * L->radius;
    }
    s.base = 0;
    for (int a = 0; a < L->rank; a++) s.base += L->radius * s.st[a];
    int inner = L->rank - 1;
    s.xaxis = C->xinner ? inner : 0;
    if (L->rank == 1) s.xaxis = 0;
    s.yaxis = -1;
    s.nz = 0;
    // y: the innermost axis not on x (if the block has y threads or rank >= 2)
    for (int a = L->rank - 1; a >= 0; a--) {
        if (a == s.xaxis) continue;
        if (s.yaxis < 0 && !(L->across && a == 0)) s.yaxis = a;
        else s.zaxes[s.nz++] = a;
    }
    // ACROSS: the dependent (outermost) axis must be a z axis, walked in order
    if (L->across && L->rank >= 2 && s.xaxis == 0) return false;
    s.ept = C->ept < 1 ? 1 : C->ept;
    blk = dim3((unsigned)C->bx, (unsigned)C->by, (unsigned)C->bz);
    if (C->bx * C->by * C->bz > 1024 || C->bx < 1 || C->by < 1 || C->bz < 1) return false;
    long X = s.ext[s.xaxis], Y = s.yaxis >= 0 ? s.ext[s.yaxis] : 1, Z = 1;
    for (int q = 0; q < s.nz; q++) Z *= s.ext[s.zaxes[q]];
    long gx = (X + (long)C->bx * s.ept - 1) / ((long)C->bx * s.ept);
    long gy = (Y + C->by - 1) / C->by;
    long gz = s.across ? 1 : (Z + C->bz - 1) / C->bz;
    if (gz > 65535) gz = 65535;  // z is grid-strided
    if (gx >= (1L << 31) || gy > 65535) return false;
    grid = dim3((unsigned)gx, (unsigned)gy, (unsigned)gz);
    return true;
}

}  // namespace

extern "C" {

long dvmhgb_synth_elems(const dvmhgb_synth_loop *L) {
    long c = 1;
    for (int a = 0; a < L->rank; a++) c *= L->ext[a] + 2 * L->radius;
    return c;
}

long dvmhgb_synth_items(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C) {
    Shape s;
    dim3 g, b;
    if (!shapeOf(L, C, s, g, b)) return -1;
    return (long)g.x * g.y * g.z;
}

int dvmhgb_synth_run(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, const void *in, void *out, void *items,
                     long *locs, void *stream) {
    Shape s;
    dim3 g, b;
    if (!L || !C || !in || !out || !shapeOf(L, C, s, g, b)) return -1;
    if (L->red && (!items || (L->red == 3 && !locs))) return -1;
    cudaStream_t st = (cudaStream_t)stream;
    if (L->esize == 4 && L->isint) launchT<int>(L->red, g, b, in, out, s, items, locs, st);
    else if (L->esize == 4) launchT<float>(L->red, g, b, in, out, s, items, locs, st);
    else if (L->esize == 8) launchT<double>(L->red, g, b, in, out, s, items, locs, st);
    else return -1;
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // extern "C"
