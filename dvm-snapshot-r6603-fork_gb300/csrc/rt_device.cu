// libdvmh_gb device layer: the GPU, its stream, a caching allocator, pinned
// host memory, host<->device copies of arrays and variables, and the
// reduction fold.
//
// The fold replaces the reference's two-stage finish (cuda_reduction.cu:168-312:
// grid-stride kernel, per-warp partials copied to the host and folded there,
// one more copy for the MINLOC record).  Here the items a loop kernel wrote are
// folded on the device by a fixed pairwise tree over item indices (padded with
// the identity to a power of two), the initial value of the reduction
// variable is combined last as the reference does it
// (initGlobalValues + postValues + addInitialValues, rts/dvmh/dvmh2.cpp:3848-3851,
// 3950-3953: result = (identity (+) loop value) (+) initial), and the result is
// written to the variable's device copy.  MINLOC/MAXLOC keep the strict
// comparison of RED_MIN/RED_MAX (rts/dvmh/loop.cpp:117-118): of equal values the
// lower item index -- the earlier one in loop order -- wins.
#include <algorithm>
#include <cstring>
#include <map>

#include "rt.h"
#include "rt_layout.h"

namespace dvmhgb {

Device gpu;

// ---------------------------------------------------------------- allocator

namespace {
std::multimap<size_t, void *> freeDev;  // size class -> block
std::map<void *, size_t> usedDev;
size_t sizeClass(size_t b) {
    if (b <= 4096) {
        size_t c = 256;
        while (c < b) c <<= 1;
        return c;
    }
    return (b + 65535) / 65536 * 65536;
}
}  // namespace

void *devAlloc(size_t bytes) {
    size_t c = sizeClass(bytes);
    auto it = freeDev.find(c);
    void *p;
    if (it != freeDev.end()) {
        p = it->second;
        freeDev.erase(it);
    } else {
        cudaError_t e = cudaMalloc(&p, c);
        if (e != cudaSuccess) {
            // give cached blocks back and retry once
            cudaGetLastError();
            for (auto &f : freeDev) cudaFree(f.second);
            freeDev.clear();
            GB_CUDA(cudaMalloc(&p, c));
        }
    }
    usedDev[p] = c;
    return p;
}

void devFree(void *p) {
    if (!p) return;
    auto it = usedDev.find(p);
    GB_INTERNAL(it != usedDev.end(), "freeing unknown device block %p", p);
    freeDev.emplace(it->second, p);
    usedDev.erase(it);
}

void *hostAlloc(size_t bytes) {
    void *p = nullptr;
    GB_CUDA(cudaHostAlloc(&p, bytes, cudaHostAllocPortable));
    return p;
}

void hostFree(void *p) {
    if (p) cudaFreeHost(p);
}

// ---------------------------------------------------------------- device

void deviceInit() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    GB_CHECK(e == cudaSuccess && n > 0, "no CUDA device: this runtime executes parallel loops on the GPU only (%s)",
             cudaGetErrorString(e));
    int dev = 0;
    if (const char *d = getenv("DVMH_GB_DEVICE")) dev = atoi(d);
    GB_CHECK(dev >= 0 && dev < n, "DVMH_GB_DEVICE=%d out of range", dev);
    GB_CUDA(cudaSetDevice(dev));
    GB_CUDA(cudaGetDeviceProperties(&gpu.prop, dev));
    GB_CHECK(gpu.prop.major >= 10, "device %s (sm_%d%d) is not a Blackwell GPU; this library is built for sm_103a",
             gpu.prop.name, gpu.prop.major, gpu.prop.minor);
    gpu.ordinal = dev;
    gpu.smCount = gpu.prop.multiProcessorCount;
    GB_CUDA(cudaStreamCreateWithFlags(&gpu.stream, cudaStreamNonBlocking));
    // status word written by kernels whose bounded waits ran out; read at every sync
    GB_CUDA(cudaHostAlloc((void **)&gpu.statusHost, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable));
    *gpu.statusHost = 0;
    GB_CUDA(cudaHostGetDevicePointer((void **)&gpu.statusDev, (void *)gpu.statusHost, 0));
    gpu.ready = true;
}

void deviceFinish() {
    if (!gpu.ready) return;
    cudaStreamSynchronize(gpu.stream);
}

void collectTimings();
void streamSync() {
    GB_PROF("streamSync");
    GB_CUDA(cudaStreamSynchronize(gpu.stream));
    collectTimings();
    int code = *(volatile int *)gpu.statusHost;
    GB_CHECK(code == 0, "a kernel gave up waiting for a dependency (status 0x%08x): results of the last loops are invalid",
             (unsigned)code);
}

extern dvmhgb_stats_t stats;

// ---------------------------------------------------------------- copies

// Dense host layout <-> device layout whose innermost rows are padded: one 2-D
// copy (rows = product of the outer extents).
// Uploads read the program's own (pinned) host array: they complete before
// returning, so that the program may write the host data again right after.
void copyH2D(Array *a) {
    // the whole device copy is replaced: it is natural afterwards, whatever it was
    for (int i = 0; i < MAXR; i++) a->tperm[i] = 0;
    a->tdiag = 0;
    long rows = (long)(a->helems / a->ext[a->rank - 1]);
    size_t w = a->ext[a->rank - 1] * a->esize;
    size_t dp = (a->rank == 1 ? a->ext[0] : a->dstride[a->rank - 2]) * a->esize;
    if (dp == w)  // unpadded rows: one linear copy
        GB_CUDA(cudaMemcpyAsync(a->dev, a->host, w * rows, cudaMemcpyHostToDevice, gpu.stream));
    else
        GB_CUDA(cudaMemcpy2DAsync(a->dev, dp, a->host, w, w, rows, cudaMemcpyHostToDevice, gpu.stream));
    stats.h2d_bytes += (long)(w * rows);
    streamSync();
}

void copyD2H(Array *a) {
    makeNatural(a);
    long rows = (long)(a->helems / a->ext[a->rank - 1]);
    size_t w = a->ext[a->rank - 1] * a->esize;
    size_t dp = (a->rank == 1 ? a->ext[0] : a->dstride[a->rank - 2]) * a->esize;
    if (dp == w)
        GB_CUDA(cudaMemcpyAsync(a->host, a->dev, w * rows, cudaMemcpyDeviceToHost, gpu.stream));
    else
        GB_CUDA(cudaMemcpy2DAsync(a->host, w, a->dev, dp, w, rows, cudaMemcpyDeviceToHost, gpu.stream));
    stats.d2h_bytes += (long)(w * rows);
    streamSync();
}

// Box copies: the innermost axis is the row; rows are enumerated over the
// outer axes (one 2-D copy per index of the second-innermost axis group).
static void copyBox(Array *a, const long lo[], const long hi[], bool toDev) {
    makeNatural(a);
    int r = a->rank;
    size_t w = (hi[r - 1] - lo[r - 1] + 1) * a->esize;
    if (r == 1) {
        char *h = a->host + lo[0] * a->esize, *d = a->dev + lo[0] * a->esize;
        GB_CUDA(cudaMemcpyAsync(toDev ? (void *)d : (void *)h, toDev ? (void *)h : (void *)d, w,
                                toDev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, gpu.stream));
    } else {
        long idx[MAXR];
        for (int i = 0; i < r - 1; i++) idx[i] = lo[i];
        long nrows = hi[r - 2] - lo[r - 2] + 1;
        while (true) {
            long ho = 0, dof = 0;
            for (int i = 0; i < r - 2; i++) {
                ho += idx[i] * a->hstride[i];
                dof += idx[i] * a->dstride[i];
            }
            ho += lo[r - 2] * a->hstride[r - 2] + lo[r - 1];
            dof += lo[r - 2] * a->dstride[r - 2] + lo[r - 1];
            size_t hp = a->hstride[r - 2] * a->esize, dp = a->dstride[r - 2] * a->esize;
            if (toDev)
                GB_CUDA(cudaMemcpy2DAsync(a->dev + dof * a->esize, dp, a->host + ho * a->esize, hp, w, nrows,
                                          cudaMemcpyHostToDevice, gpu.stream));
            else
                GB_CUDA(cudaMemcpy2DAsync(a->host + ho * a->esize, hp, a->dev + dof * a->esize, dp, w, nrows,
                                          cudaMemcpyDeviceToHost, gpu.stream));
            int ax = r - 3;
            while (ax >= 0 && ++idx[ax] > hi[ax]) {
                idx[ax] = lo[ax];
                ax--;
            }
            if (ax < 0) break;
        }
    }
    long cells = 1;
    for (int i = 0; i < r; i++) cells *= hi[i] - lo[i] + 1;
    if (toDev) stats.h2d_bytes += cells * (long)a->esize;
    else stats.d2h_bytes += cells * (long)a->esize;
}

void copyBoxH2D(Array *a, const long lo[], const long hi[]) {
    copyBox(a, lo, hi, true);
    streamSync();  // the box is read from the program's host array: done before the program may change it
}
void copyBoxD2H(Array *a, const long lo[], const long hi[]) {
    copyBox(a, lo, hi, false);
    streamSync();
}

// ---------------------------------------------------------------- relayout

// One pass over every element in natural index order (last axis fastest):
// read it where layout `from` keeps it, write it where `to` keeps it.  A
// permutation or a diagonal renumbering is a bijection of the index space, so
// every destination element is written exactly once.  One side of the copy
// is strided; the pass runs once per layout change, not per loop.
template <typename T>
__global__ void kRelayout(const T *__restrict__ src, LayoutDesc from, T *__restrict__ dst, LayoutDesc to, long n) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        long idx[LAYOUT_MAXR], r = t;
        for (int a = from.rank - 1; a >= 0; a--) {
            idx[a] = r % from.ext[a];
            r /= from.ext[a];
        }
        dst[layoutOffset(to, idx)] = src[layoutOffset(from, idx)];
    }
}

struct Bytes16 {
    uint4 v;
};

void launchRelayout(const char *src, const LayoutDesc &from, char *dst, const LayoutDesc &to, size_t esize,
                    cudaStream_t s) {
    long n = 1;
    for (int a = 0; a < from.rank; a++) n *= from.ext[a];
    if (n == 0) return;
    long blocks = std::min<long>((n + 255) / 256, (long)gpu.smCount * 8);
    switch (esize) {
        case 1: kRelayout<uint8_t><<<(unsigned)blocks, 256, 0, s>>>((const uint8_t *)src, from, (uint8_t *)dst, to, n); break;
        case 2: kRelayout<uint16_t><<<(unsigned)blocks, 256, 0, s>>>((const uint16_t *)src, from, (uint16_t *)dst, to, n); break;
        case 4: kRelayout<uint32_t><<<(unsigned)blocks, 256, 0, s>>>((const uint32_t *)src, from, (uint32_t *)dst, to, n); break;
        case 8: kRelayout<uint64_t><<<(unsigned)blocks, 256, 0, s>>>((const uint64_t *)src, from, (uint64_t *)dst, to, n); break;
        case 16: kRelayout<Bytes16><<<(unsigned)blocks, 256, 0, s>>>((const Bytes16 *)src, from, (Bytes16 *)dst, to, n); break;
        default: {
            // other element sizes: the same pass over bytes, the element as the innermost axis
            LayoutDesc f = from, g = to;
            GB_CHECK(from.rank < LAYOUT_MAXR, "relayout of a rank-%d array of %zu-byte elements", from.rank, esize);
            f.ext[f.rank] = g.ext[g.rank] = (long)esize;
            for (int a = 0; a < f.rank; a++) {
                f.coef[a] *= (long)esize;
                g.coef[a] *= (long)esize;
            }
            f.coef[f.rank] = g.coef[g.rank] = 1;
            f.diagUnit *= (long)esize;
            g.diagUnit *= (long)esize;
            f.rank++;
            g.rank++;
            kRelayout<uint8_t><<<(unsigned)std::min<long>((n * (long)esize + 255) / 256, (long)gpu.smCount * 8), 256,
                                 0, s>>>((const uint8_t *)src, f, (uint8_t *)dst, g, n * (long)esize);
        }
    }
    GB_CUDA(cudaGetLastError());
    dvmhgb_count_launches(1);
}

// Variables: through a pinned staging copy so the transfer is asynchronous
// and capturable; the staging buffer is reused only after the copy ran.
namespace {
struct Staging {
    char *buf = nullptr;
    size_t size = 0;
    cudaEvent_t done = nullptr;
};
std::map<const Var *, Staging> staging;
Staging &stageFor(const Var *v) {
    Staging &s = staging[v];
    if (s.size < v->size) {
        if (s.buf) {
            if (s.done) cudaEventSynchronize(s.done);
            hostFree(s.buf);
        }
        s.buf = (char *)hostAlloc(std::max<size_t>(v->size, 16));
        s.size = v->size;
    }
    if (!s.done) GB_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    return s;
}
}  // namespace

void varH2D(Var *v) {
    GB_PROF("varH2D");
    ensureVarDev(v);
    queueFlushVar(v);  // the queued loops that name v run first; the others do not see the copy
    Staging &s = stageFor(v);
    GB_CUDA(cudaEventSynchronize(s.done));
    memcpy(s.buf, v->addr, v->size);
    GB_CUDA(cudaMemcpyAsync(v->dev, s.buf, v->size, cudaMemcpyHostToDevice, gpu.stream));
    GB_CUDA(cudaEventRecord(s.done, gpu.stream));
    stats.h2d_bytes += (long)v->size;
}

void varForgetStaging(const Var *v) {
    auto it = staging.find(v);
    if (it == staging.end()) return;
    if (it->second.done) {
        cudaEventSynchronize(it->second.done);
        cudaEventDestroy(it->second.done);
    }
    if (it->second.buf) hostFree(it->second.buf);
    staging.erase(it);
}

void varD2H(Var *v) {
    GB_PROF("varD2H");
    GB_INTERNAL(v->dev, "variable without a device copy");
    queueFlushVar(v);
    Staging &s = stageFor(v);
    GB_CUDA(cudaEventSynchronize(s.done));
    GB_CUDA(cudaMemcpyAsync(s.buf, v->dev, v->size, cudaMemcpyDeviceToHost, gpu.stream));
    streamSync();
    memcpy((void *)v->addr, s.buf, v->size);
    stats.d2h_bytes += (long)v->size;
}

// ---------------------------------------------------------------- reduction identities

template <typename T>
struct Lim;
#define LIM(T, LO, HI)                                             \
    template <>                                                    \
    struct Lim<T> {                                                \
        __host__ __device__ static T lo() { return LO; }           \
        __host__ __device__ static T hi() { return HI; }           \
    };
LIM(char, -128, 127)
LIM(signed char, -128, 127)
LIM(unsigned char, 0, 255)
LIM(short, -32768, 32767)
LIM(unsigned short, 0, 65535)
LIM(int, (-2147483647 - 1), 2147483647)
LIM(unsigned, 0u, 4294967295u)
LIM(long, (-9223372036854775807L - 1), 9223372036854775807L)
LIM(unsigned long, 0ul, 18446744073709551615ul)
LIM(long long, (-9223372036854775807LL - 1), 9223372036854775807LL)
LIM(unsigned long long, 0ull, 18446744073709551615ull)
LIM(float, -__builtin_huge_valf(), __builtin_huge_valf())
LIM(double, -__builtin_huge_val(), __builtin_huge_val())
#undef LIM

// identity of each operation; -0.0 is the exact additive identity of IEEE sums
template <typename T>
__host__ __device__ T identityOf(int op) {
    switch (op) {
        case rf_SUM: return (T)0 * (T)-1 == (T)0 ? (T)-0.0 : (T)0;
        case rf_PROD: return (T)1;
        case rf_MAX: case rf_MAXLOC: return Lim<T>::lo();
        case rf_MIN: case rf_MINLOC: return Lim<T>::hi();
        case rf_AND: return (T)~(T)0;
        case rf_OR: case rf_XOR: case rf_NE: return (T)0;
        case rf_EQU: case rf_EQ: return (T)1;
        default: return (T)0;
    }
}
template <>
__host__ __device__ float identityOf<float>(int op) {
    switch (op) {
        case rf_SUM: return -0.0f;
        case rf_PROD: return 1.0f;
        case rf_MAX: case rf_MAXLOC: return Lim<float>::lo();
        case rf_MIN: case rf_MINLOC: return Lim<float>::hi();
        default: return 0.0f;
    }
}
template <>
__host__ __device__ double identityOf<double>(int op) {
    switch (op) {
        case rf_SUM: return -0.0;
        case rf_PROD: return 1.0;
        case rf_MAX: case rf_MAXLOC: return Lim<double>::lo();
        case rf_MIN: case rf_MINLOC: return Lim<double>::hi();
        default: return 0.0;
    }
}

// dest (+)= src following loop.cpp:116-238; returns true when MIN/MAX replaced dest
template <typename T>
__host__ __device__ __forceinline__ bool combine(int op, T &d, T s) {
    switch (op) {
        case rf_SUM: d = d + s; return false;
        case rf_PROD: d = d * s; return false;
        case rf_MAX: case rf_MAXLOC: if (d < s) { d = s; return true; } return false;
        case rf_MIN: case rf_MINLOC: if (d > s) { d = s; return true; } return false;
        default: return false;
    }
}
template <typename T>
__host__ __device__ __forceinline__ bool combineInt(int op, T &d, T s) {
    switch (op) {
        case rf_AND: d &= s; return false;
        case rf_OR: d |= s; return false;
        case rf_XOR: d ^= s; return false;
        case rf_EQU: case rf_EQ: d = (d == s); return false;
        case rf_NE: d = (d != s); return false;
        default: return combine<T>(op, d, s);
    }
}
template <typename T, bool INT>
struct Comb {
    __host__ __device__ static bool f(int op, T &d, T s) { return combine<T>(op, d, s); }
};
template <typename T>
struct Comb<T, true> {
    __host__ __device__ static bool f(int op, T &d, T s) { return combineInt<T>(op, d, s); }
};

template <typename T>
__global__ void kFill(T *p, long n, T v) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) p[i] = v;
}

// ---------------------------------------------------------------- fold kernels

constexpr int FOLD_THREADS = 512;
constexpr int FOLD_SPAN = 2 * FOLD_THREADS;  // items per block per pass (a pairwise subtree)

// One pass: block b folds items [b*SPAN, (b+1)*SPAN) of every element e by the
// pairwise tree (item i pairs with i^1, then i^2, ...), padding with the
// identity, and writes out[b] (and the winning loc index for LOC ops).
// Items are laid out [item][elem]; locs [item][locSize bytes].
// `final` > 0: a single block, whose result is combined with the initial value
// read from dst and written to dst (+ loc bytes to dstLoc).
template <typename T, bool INT>
__global__ void __launch_bounds__(FOLD_THREADS) kFold(int op, long count, long elemCount, const T *items,
                                                      const long *itemIdx, T *out, long *outIdx, int final,
                                                      T *dst, const char *locItems, long locSize, char *dstLoc) {
    __shared__ T sv[FOLD_SPAN];
    __shared__ long si[FOLD_SPAN];
    const bool loc = (op == rf_MINLOC || op == rf_MAXLOC);
    const T ident = identityOf<T>(op);
    for (long e = 0; e < elemCount; e++) {
        for (int h = 0; h < 2; h++) {
            long i = blockIdx.x * (long)FOLD_SPAN + h * FOLD_THREADS + threadIdx.x;
            bool in = i < count;
            sv[h * FOLD_THREADS + threadIdx.x] = in ? items[i * elemCount + e] : ident;
            si[h * FOLD_THREADS + threadIdx.x] = in ? (itemIdx ? itemIdx[i * elemCount + e] : i) : -1;
        }
        __syncthreads();
        for (int w = 1; w < FOLD_SPAN; w <<= 1) {
            // node pairs (a, a + w) with a a multiple of 2w: pairwise by index
            int pairs = FOLD_SPAN / (2 * w);
            for (int p = threadIdx.x; p < pairs; p += FOLD_THREADS) {
                int a = p * 2 * w, b = a + w;
                T d = sv[a];
                if (loc) {
                    // of equal values the lower index wins; identity slots (index -1) never win
                    T s = sv[b];
                    long ia = si[a], ib = si[b];
                    bool take = (ia < 0 && ib >= 0) || (ib >= 0 && Comb<T, INT>::f(op, d, s));
                    if (take) {
                        sv[a] = s;
                        si[a] = ib;
                    }
                } else {
                    Comb<T, INT>::f(op, d, sv[b]);
                    sv[a] = d;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (!final) {
                out[blockIdx.x * elemCount + e] = sv[0];
                if (outIdx) outIdx[blockIdx.x * elemCount + e] = si[0];
            } else {
                // result = (global start (+) loop value) (+) initial value, where the
                // global start is what DvmhReduction::initValues (loop.cpp:37-100) puts
                // there: +0 for SUM/XOR/NE, 1 for PROD/EQU/EQ, the initial value otherwise
                T init = dst[e];
                T r;
                switch (op) {
                    case rf_SUM: case rf_XOR: case rf_NE: r = (T)0; break;
                    case rf_PROD: case rf_EQU: case rf_EQ: r = (T)1; break;
                    default: r = init;
                }
                long ri = si[0];
                bool fromLoop = false;
                if (loc) {
                    if (ri >= 0) fromLoop = Comb<T, INT>::f(op, r, sv[0]);
                } else {
                    Comb<T, INT>::f(op, r, sv[0]);
                    Comb<T, INT>::f(op, r, init);
                }
                dst[e] = r;
                if (loc && fromLoop && dstLoc && locItems)
                    for (long b = 0; b < locSize; b++) dstLoc[e * locSize + b] = locItems[(ri * elemCount + e) * locSize + b];
            }
        }
        __syncthreads();
    }
}

// ---- the same tree, bandwidth-bound (one value per item: elemCount == 1)
//
// A block folds an aligned span of FOLD2_SPAN = 2048 items: each thread loads 8
// consecutive items with vector loads and folds them as the three lowest tree
// levels in registers, the warp folds its 32 threads' nodes by shuffles (lane
// a takes lane a + w, a a multiple of 2w), and warp 0 folds the 8 warps' nodes.
// Every node is the pairwise tree over an aligned power-of-two index range with
// the identity beyond the last item, exactly as in kFold; spans of 2048 instead
// of 1024 only add levels that combine a node with the identity.  That is why
// this path is taken only for the operations where x (+) identity = x for every
// non-NaN x (SUM, PROD, MAX, MIN, AND, OR, XOR and the LOC pair), not for the
// logical EQU / EQ / NE.
constexpr int FOLD2_THREADS = 256;
constexpr int FOLD2_PER = 8;
constexpr int FOLD2_SPAN = FOLD2_THREADS * FOLD2_PER;

template <typename T>
__device__ __forceinline__ T shflDown(T v, int w) {
    if constexpr (sizeof(T) < 4)
        return (T)__shfl_down_sync(0xffffffffu, (int)v, w);
    else
        return __shfl_down_sync(0xffffffffu, v, w);
}

// 8 consecutive values of a 16-byte aligned (8-byte for 1-byte types) address,
// read once: streaming loads
template <typename T>
__device__ __forceinline__ void load8(const T *p, T v[8]) {
    constexpr int B = (int)sizeof(T) * 8;
    if constexpr (B % 16 == 0) {
        uint4 r[B / 16];
#pragma unroll
        for (int i = 0; i < B / 16; i++) r[i] = __ldcs(reinterpret_cast<const uint4 *>(p) + i);
        memcpy(v, r, B);
    } else {
        uint2 r = __ldcs(reinterpret_cast<const uint2 *>(p));
        memcpy(v, &r, 8);
    }
}

// d (+)= s, d the lower-index node; with LOC the lower index wins ties and an
// identity node (index -1) never wins, as in kFold
template <typename T, bool INT, bool LOC>
__device__ __forceinline__ void step2(int op, T &d, long &di, T s, long si) {
    if (LOC) {
        T x = d;
        const bool take = (di < 0 && si >= 0) || (si >= 0 && Comb<T, INT>::f(op, x, s));
        if (take) {
            d = s;
            di = si;
        }
    } else {
        Comb<T, INT>::f(op, d, s);
    }
}

// The node of aligned span `span` (items [span * FOLD2_SPAN, +FOLD2_SPAN), the
// identity beyond `count`), computed by the whole CTA; true on thread 0, which
// holds it in x (and its item index in xi for LOC ops).  itemIdx: the items'
// indices (a previous pass's winners), null = their positions.  Vector loads
// where the 8 items lie inside `count` on a 16-byte boundary.
template <typename T, bool INT, bool LOC>
__device__ __forceinline__ bool span2(int op, long count, const T *items, const long *itemIdx, long span, T &x,
                                      long &xi) {
    __shared__ T sw[FOLD2_THREADS / 32];
    __shared__ long swi[FOLD2_THREADS / 32];
    const T ident = identityOf<T>(op);
    const long base = span * FOLD2_SPAN + threadIdx.x * (long)FOLD2_PER;
    T v[FOLD2_PER];
    long vi[FOLD2_PER];
    const bool whole = base + FOLD2_PER <= count && ((uintptr_t)(items + base) & 15) == 0 &&
                       (!LOC || !itemIdx || ((uintptr_t)(itemIdx + base) & 15) == 0);
    if (whole) {
        load8(items + base, v);
        if (LOC) {
            if (itemIdx)
                load8(itemIdx + base, vi);
            else
#pragma unroll
                for (int j = 0; j < FOLD2_PER; j++) vi[j] = base + j;
        }
    } else {
#pragma unroll
        for (int j = 0; j < FOLD2_PER; j++) {
            const long i = base + j;
            const bool in = i < count;
            v[j] = in ? items[i] : ident;
            vi[j] = in ? (itemIdx ? itemIdx[i] : i) : -1;
        }
    }
#pragma unroll
    for (int w = 1; w < FOLD2_PER; w <<= 1)
#pragma unroll
        for (int a = 0; a < FOLD2_PER; a += 2 * w) step2<T, INT, LOC>(op, v[a], vi[a], v[a + w], vi[a + w]);
    x = v[0];
    xi = LOC ? vi[0] : 0;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int w = 1; w < 32; w <<= 1) {
        const T sv = shflDown(x, w);
        const long si = LOC ? __shfl_down_sync(0xffffffffu, xi, w) : 0;
        if ((lane & (2 * w - 1)) == 0) step2<T, INT, LOC>(op, x, xi, sv, si);
    }
    if (lane == 0) {
        sw[threadIdx.x >> 5] = x;
        swi[threadIdx.x >> 5] = xi;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return false;
    constexpr int NW = FOLD2_THREADS / 32;
    x = lane < NW ? sw[lane] : ident;
    xi = lane < NW ? swi[lane] : -1;
#pragma unroll
    for (int w = 1; w < NW; w <<= 1) {
        const T sv = shflDown(x, w);
        const long si = LOC ? __shfl_down_sync(0xffffffffu, xi, w) : 0;
        if ((lane & (2 * w - 1)) == 0) step2<T, INT, LOC>(op, x, xi, sv, si);
    }
    return lane == 0;
}

// (global start (+) loop value) (+) initial value into dst[0] (and the winner's
// loc bytes into dstLoc), the combination kFold's final pass makes
template <typename T, bool INT, bool LOC>
__device__ __forceinline__ void finish2(int op, T x, long xi, T *dst, const char *locItems, long locSize,
                                        char *dstLoc) {
    const T init = dst[0];
    T r;
    switch (op) {
        case rf_SUM: case rf_XOR: r = (T)0; break;
        case rf_PROD: r = (T)1; break;
        default: r = init;
    }
    bool fromLoop = false;
    if (LOC) {
        if (xi >= 0) fromLoop = Comb<T, INT>::f(op, r, x);
    } else {
        Comb<T, INT>::f(op, r, x);
        Comb<T, INT>::f(op, r, init);
    }
    dst[0] = r;
    if (LOC && fromLoop && dstLoc && locItems)
        for (long b = 0; b < locSize; b++) dstLoc[b] = locItems[xi * locSize + b];
}

template <typename T, bool INT, bool LOC>
__global__ void __launch_bounds__(FOLD2_THREADS) kFold2(int op, long count, const T *items, const long *itemIdx,
                                                        T *out, long *outIdx, int final, T *dst, const char *locItems,
                                                        long locSize, char *dstLoc) {
    T x;
    long xi;
    if (!span2<T, INT, LOC>(op, count, items, itemIdx, blockIdx.x, x, xi)) return;
    if (final) {
        finish2<T, INT, LOC>(op, x, xi, dst, locItems, locSize, dstLoc);
    } else {
        out[blockIdx.x] = x;
        if (LOC) outIdx[blockIdx.x] = xi;
    }
}

template <typename T, bool INT, bool LOC>
static void fold2T(int op, long count, const void *items, const void *locItems, long locSize, void *dst, void *dstLoc,
                   cudaStream_t s, std::vector<void *> &scratch) {
    const T *cur = (const T *)items;
    const long *curIdx = nullptr;
    long n = count;
    while (n > FOLD2_SPAN) {
        const long blocks = (n + FOLD2_SPAN - 1) / FOLD2_SPAN;
        T *out = (T *)devAlloc(sizeof(T) * blocks);
        long *outIdx = LOC ? (long *)devAlloc(sizeof(long) * blocks) : nullptr;
        scratch.push_back(out);
        if (outIdx) scratch.push_back(outIdx);
        kFold2<T, INT, LOC><<<(unsigned)blocks, FOLD2_THREADS, 0, s>>>(op, n, cur, curIdx, out, outIdx, 0, nullptr,
                                                                      nullptr, 0, nullptr);
        dvmhgb_count_launches(1);
        cur = out;
        curIdx = outIdx;
        n = blocks;
    }
    kFold2<T, INT, LOC><<<1, FOLD2_THREADS, 0, s>>>(op, n, cur, curIdx, nullptr, nullptr, 1, (T *)dst,
                                                   (const char *)locItems, locSize, (char *)dstLoc);
    dvmhgb_count_launches(1);
    GB_CUDA(cudaGetLastError());
}

template <typename T, bool INT>
static void foldT(int op, long count, long elemCount, const void *items, const void *locItems, long locSize, void *dst,
                  void *dstLoc, cudaStream_t s, std::vector<void *> &scratch) {
    const bool loc = op == rf_MINLOC || op == rf_MAXLOC;
    const bool neutralPad = op == rf_SUM || op == rf_PROD || op == rf_MAX || op == rf_MIN || op == rf_AND ||
                            op == rf_OR || op == rf_XOR || loc;
    if (elemCount == 1 && neutralPad && ((uintptr_t)items & 15) == 0) {
        if (loc)
            fold2T<T, INT, true>(op, count, items, locItems, locSize, dst, dstLoc, s, scratch);
        else
            fold2T<T, INT, false>(op, count, items, locItems, locSize, dst, dstLoc, s, scratch);
        return;
    }
    const T *cur = (const T *)items;
    const long *curIdx = nullptr;
    long n = count;
    while (n > FOLD_SPAN) {
        long blocks = (n + FOLD_SPAN - 1) / FOLD_SPAN;
        T *out = (T *)devAlloc(sizeof(T) * blocks * elemCount);
        long *outIdx = (op == rf_MINLOC || op == rf_MAXLOC) ? (long *)devAlloc(sizeof(long) * blocks * elemCount) : nullptr;
        scratch.push_back(out);
        if (outIdx) scratch.push_back(outIdx);
        kFold<T, INT><<<(unsigned)blocks, FOLD_THREADS, 0, s>>>(op, n, elemCount, cur, curIdx, out, outIdx, 0, nullptr,
                                                               nullptr, 0, nullptr);
        dvmhgb_count_launches(1);
        cur = out;
        curIdx = outIdx;
        n = blocks;
    }
    kFold<T, INT><<<1, FOLD_THREADS, 0, s>>>(op, n, elemCount, cur, curIdx, nullptr, nullptr, 1, (T *)dst,
                                            (const char *)locItems, locSize, (char *)dstLoc);
    dvmhgb_count_launches(1);
    GB_CUDA(cudaGetLastError());
}

#define DISPATCH_TYPES(vtype, FN, ...)                                                           \
    switch (vtype) {                                                                             \
        case rt_CHAR: FN<signed char, true>(__VA_ARGS__); break;                                 \
        case rt_UCHAR: FN<unsigned char, true>(__VA_ARGS__); break;                              \
        case rt_SHORT: FN<short, true>(__VA_ARGS__); break;                                      \
        case rt_USHORT: FN<unsigned short, true>(__VA_ARGS__); break;                            \
        case rt_INT: case rt_LOGICAL: FN<int, true>(__VA_ARGS__); break;                         \
        case rt_UINT: FN<unsigned, true>(__VA_ARGS__); break;                                    \
        case rt_LONG: FN<long, true>(__VA_ARGS__); break;                                        \
        case rt_ULONG: FN<unsigned long, true>(__VA_ARGS__); break;                              \
        case rt_LLONG: FN<long long, true>(__VA_ARGS__); break;                                  \
        case rt_ULLONG: FN<unsigned long long, true>(__VA_ARGS__); break;                        \
        case rt_FLOAT: FN<float, false>(__VA_ARGS__); break;                                     \
        case rt_DOUBLE: FN<double, false>(__VA_ARGS__); break;                                   \
        default: GB_CHECK(false, "reduction over type %d is not supported", vtype);              \
    }

void launchRedFold(int op, int vtype, long count, long elemCount, const void *items, const void *locItems,
                   long locSize, void *dst, void *dstLoc, cudaStream_t s, std::vector<void *> &scratch) {
    GB_CHECK(count > 0, "empty reduction buffer");
    bool isFloat = vtype == rt_FLOAT || vtype == rt_DOUBLE;
    GB_CHECK(!isFloat || (op >= rf_SUM && op <= rf_MIN) || op == rf_MINLOC || op == rf_MAXLOC,
             "reduction %d is not defined for floating types", op);
    DISPATCH_TYPES(vtype, foldT, op, count, elemCount, items, locItems, locSize, dst, dstLoc, s, scratch);
}

// ---------------------------------------------------------------- segmented fold (batches)

// Every reduction of a batch at once, by the tree of the single fold (kFold2):
// pass 1 gives every aligned 2048-item span of every job its own CTA, pass 2
// one CTA per job folds that job's span nodes (at most 2048: the spans are the
// next level's items) and combines the result with the initial value.
__device__ __forceinline__ int jobOf(const FoldJob *jobs, int njobs, long gb) {
    int lo = 0, hi = njobs - 1;  // the last job with blockBase <= gb
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blockBase <= gb) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(FOLD2_THREADS) kFoldSegBlocks(const FoldJob *jobs, int njobs, double *bv, long *bi) {
    const long gb = blockIdx.x;
    const FoldJob &J = jobs[jobOf(jobs, njobs, gb)];
    const double *items = (const double *)J.items;
    double x;
    long xi;
    bool lead;
    if (J.op == rf_MINLOC || J.op == rf_MAXLOC)
        lead = span2<double, false, true>(J.op, J.count, items, nullptr, gb - J.blockBase, x, xi);
    else
        lead = span2<double, false, false>(J.op, J.count, items, nullptr, gb - J.blockBase, x, xi);
    if (lead) {
        bv[gb] = x;
        bi[gb] = xi;
    }
}

__global__ void __launch_bounds__(FOLD2_THREADS) kFoldSegFinal(const FoldJob *jobs, const double *bv, const long *bi) {
    const FoldJob &J = jobs[blockIdx.x];
    const long nblk = (J.count + FOLD2_SPAN - 1) / FOLD2_SPAN;
    double x;
    long xi;
    if (J.op == rf_MINLOC || J.op == rf_MAXLOC) {
        if (span2<double, false, true>(J.op, nblk, bv + J.blockBase, bi + J.blockBase, 0, x, xi))
            finish2<double, false, true>(J.op, x, xi, (double *)J.dst, (const char *)J.locItems, J.locSize,
                                         (char *)J.dstLoc);
    } else {
        if (span2<double, false, false>(J.op, nblk, bv + J.blockBase, nullptr, 0, x, xi))
            finish2<double, false, false>(J.op, x, xi, (double *)J.dst, nullptr, 0, nullptr);
    }
}

bool foldBatchable(int op, int vtype, long count, long elemCount) {
    return vtype == rt_DOUBLE && elemCount == 1 && count <= (long)FOLD2_SPAN * FOLD2_SPAN &&
           (op == rf_SUM || op == rf_PROD || op == rf_MAX || op == rf_MIN || op == rf_MINLOC || op == rf_MAXLOC);
}

void launchRedFoldBatch(const std::vector<FoldJob> &jobs, cudaStream_t s, std::vector<void *> &devScratch,
                        std::vector<void *> &hostScratch) {
    if (jobs.empty()) return;
    size_t bytes = sizeof(FoldJob) * jobs.size();
    FoldJob *h = (FoldJob *)hostAlloc(bytes);
    hostScratch.push_back(h);
    memcpy(h, jobs.data(), bytes);
    long blocks = 0;  // 2048-item spans of all jobs
    for (size_t q = 0; q < jobs.size(); q++) {
        h[q].blockBase = blocks;
        blocks += (h[q].count + FOLD2_SPAN - 1) / FOLD2_SPAN;
    }
    GB_INTERNAL(blocks < (1L << 31), "reduction batch too large");
    FoldJob *d = (FoldJob *)devAlloc(bytes);
    devScratch.push_back(d);
    double *bv = (double *)devAlloc(sizeof(double) * (blocks > 0 ? blocks : 1));
    long *bi = (long *)devAlloc(sizeof(long) * (blocks > 0 ? blocks : 1));
    devScratch.push_back(bv);
    devScratch.push_back(bi);
    GB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
    if (blocks > 0) kFoldSegBlocks<<<(unsigned)blocks, FOLD2_THREADS, 0, s>>>(d, (int)jobs.size(), bv, bi);
    kFoldSegFinal<<<(unsigned)jobs.size(), FOLD2_THREADS, 0, s>>>(d, bv, bi);
    dvmhgb_count_launches(2);
    GB_CUDA(cudaGetLastError());
}

template <typename T, bool INT>
static void fillT(int op, void *items, long n, cudaStream_t s) {
    long blocks = std::min<long>((n + 255) / 256, 4 * 152);
    kFill<T><<<(unsigned)std::max<long>(blocks, 1), 256, 0, s>>>((T *)items, n, identityOf<T>(op));
    dvmhgb_count_launches(1);
}

void fillIdentity(int op, int vtype, void *items, long n, cudaStream_t s) {
    DISPATCH_TYPES(vtype, fillT, op, items, n, s);
}

template <typename T, bool INT>
static void identT(int op, void *out) {
    T v = identityOf<T>(op);
    memcpy(out, &v, sizeof(T));
}

void identityValue(int op, int vtype, void *out) { DISPATCH_TYPES(vtype, identT, op, out); }

}  // namespace dvmhgb
