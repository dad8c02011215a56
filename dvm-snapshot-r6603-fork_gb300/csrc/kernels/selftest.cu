// Device self-test of softfp64.cuh: the integer-pipe FP64 operations against
// the FP64 unit on random operands drawn to stress alignment, cancellation,
// carries, rounding ties and the normal-range edges.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/dvmh_gb.h"
#include "softfp64.cuh"

namespace {

__device__ __forceinline__ uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// an operand pair: a class picked from the stream, then bits shaped by it
__device__ void pair(uint64_t seed, uint64_t i, double &a, double &b) {
    uint64_t r0 = mix(seed + 4 * i + 1), r1 = mix(seed + 4 * i + 2), r2 = mix(seed + 4 * i + 3);
    uint64_t A = r0, B = r1;
    switch (r2 & 7) {
        case 0: break;  // any bits (includes NaN, inf, subnormal)
        case 1:         // close exponents, random signs
            B = (A & 0xFFF0000000000000ull) ^ ((r2 >> 8) & 0x0030000000000000ull) | (r1 & sf::MANT);
            break;
        case 2:  // cancellation: b = -a with low bits changed
            B = (A ^ sf::SIGN) ^ (r1 & ((1ull << ((r2 >> 8) % 53)) - 1));
            break;
        case 3:  // values in [0, 1) and small integers, as the stencils see
            A = sf::bits((double)(r0 >> 11) * (1.0 / 9007199254740992.0));
            B = sf::bits((double)(r1 >> 11) * (1.0 / 9007199254740992.0) * (double)((r2 >> 8) & 15));
            break;
        case 4:  // exponent differences around the alignment limits
            B = (A & 0x800FFFFFFFFFFFFFull) | ((((A >> 52) & 0x7FF) - ((r2 >> 8) % 70)) & 0x7FF) << 52;
            break;
        case 5:  // mantissas with long runs of ones (rounding carries)
            A |= 0x000FFFFFFFFFFF00ull;
            B = (A & 0xFFF0000000000000ull) | (r1 & 0xFFull);
            break;
        case 6:  // near the normal-range edges
            A = (A & 0x800FFFFFFFFFFFFFull) | ((r2 >> 8) % 4 + 1) << 52;
            B = (B & 0x800FFFFFFFFFFFFFull) | (0x7FEull - (r2 >> 16) % 3) << 52;
            break;
        default:  // halfway cases: b is a power of two below a's last bit
            B = (A & 0x8000000000000000ull) | ((((A >> 52) & 0x7FF) - 53) & 0x7FF) << 52;
            break;
    }
    a = sf::from(A);
    b = sf::from(B);
}

__device__ __forceinline__ bool same(double x, double y) {
    uint64_t X = sf::bits(x), Y = sf::bits(y);
    return X == Y || ((X & ~sf::SIGN) > sf::EXPINF && (Y & ~sf::SIGN) > sf::EXPINF);  // any NaN = any NaN
}

__global__ void kSelftest(long n, uint64_t seed, unsigned long long *bad) {
    unsigned long long c[4] = {0, 0, 0, 0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double a, b;
        pair(seed, (uint64_t)i, a, b);
        c[0] += !same(sf::add(a, b), __dadd_rn(a, b));
        c[1] += !same(sf::sub(a, b), __dsub_rn(a, b));
        c[2] += !same(sf::mul(a, b), __dmul_rn(a, b));
        c[3] += !same(sf::div3p2(a, 1), a / 6.0);
    }
    for (int k = 0; k < 4; k++)
        if (c[k]) atomicAdd(bad + k, c[k]);
}

// FP64 addition throughput: every thread runs 8 independent chains of native
// additions (enough independent work to keep the FP64 unit busy on every SM)
__global__ void __launch_bounds__(256) kFp64Rate(double *out, int iters) {
    double x[8], c[8];
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        x[q] = 0.25 + 1e-3 * ((t * 7 + q * 13) % 97);
        c[q] = 1e-4 * (1 + (t + q) % 31);
    }
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = sf::nadd(x[q], c[q]);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += x[q];
    out[t] = s;
}

}  // namespace

// Measured FP64 addition rate of this GPU (additions per second): 8 CTAs of
// 256 threads per SM, 8 independent chains per thread, timed with CUDA events
// after a warm-up launch.  The denominator of the FP64 roofline of the stencils.
extern "C" int dvmhgb_fp64_add_rate(double *addsPerSecond) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0 || !addsPerSecond) return -1;
    const int grid = sms * 8, iters = 4000;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * grid * 256) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    kFp64Rate<<<grid, 256>>>(out, 100);
    cudaEventRecord(e0);
    kFp64Rate<<<grid, 256>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t err = cudaGetLastError();
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return -1;
    *addsPerSecond = (double)grid * 256 * 8 * iters / (ms * 1e-3);
    return 0;
}

extern "C" int dvmhgb_selftest_softfp64(long n, unsigned long long seed, long mismatches[4]) {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return -1;
    cudaMemset(d, 0, 4 * sizeof(unsigned long long));
    kSelftest<<<152 * 8, 256>>>(n, seed, d);
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    for (int k = 0; k < 4; k++) mismatches[k] = (long)h[k];
    return e == cudaSuccess ? 0 : -1;
}
