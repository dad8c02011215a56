/*
 * Shared pieces of the workload programs: seeded input generation and the
 * run-parameter structs passed across the workloads' C entry points.
 *
 * Seeding: array stream s of a run seeded with `seed` is the splitmix64
 * sequence (Steele, Lea, Flood 2014; Vigna's reference constants) started at
 * state0 = seed ^ (0xD1B54A32D192ED03 * (s + 1)); element n takes the n-th
 * output, so any element is computable in O(1) on host or device.  A 64-bit
 * output x becomes the double (x >> 11) * 2^-53 in [0, 1), which is exact.
 */
#ifndef WL_COMMON_H
#define WL_COMMON_H

#include <stdint.h>

#ifdef __CUDACC__
#define WL_HD __host__ __device__ __forceinline__
#else
#define WL_HD static inline
#endif

WL_HD uint64_t wl_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

WL_HD double wl_u01(uint64_t seed, uint64_t stream, uint64_t n) {
    uint64_t s0 = seed ^ (0xD1B54A32D192ED03ULL * (stream + 1));
    return (double)(wl_mix64(s0 + (n + 1) * 0x9E3779B97F4A7C15ULL) >> 11) * (1.0 / 9007199254740992.0);
}

/*
 * Host-side element strides of a distributed array from its descriptor: the
 * runtime writes the outer axes' strides (in elements) into desc[1..rank-1];
 * the innermost stride is 1.  Runtimes may pad rows, so programs never assume
 * a dense layout (the reference pads even extents).
 */
#ifndef __CUDACC__
static inline void wl_strides(const long *desc, int rank, long *st) {
    int r;
    st[rank - 1] = 1;
    for (r = 0; r < rank - 1; r++)
        st[r] = desc[r + 1];
}
#endif

/* execution modes understood by the GB300 runtime (ignored by the reference) */
#define WL_MODE_DEFAULT 0

/* Jacobi 2-D / 3-D: n^rank grid, shadow 1, `iters` iterations */
typedef struct {
    long n;
    long iters;
    uint64_t seed;
} wl_jacobi_params;

/* SOR 3-D ACROSS: n^3 grid, omega, `sweeps` sweeps */
typedef struct {
    long n;
    long sweeps;
    double omega;
    uint64_t seed;
} wl_sor_params;

/* batched heat: `count` 2-D arrays, sides log-uniform in [side_lo, side_hi] */
typedef struct {
    long count;
    long side_lo;
    long side_hi;
    long steps;
    double coef;
    uint64_t seed;
} wl_heat_params;

#endif
