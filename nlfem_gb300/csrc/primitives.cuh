// Device primitives: warp scans, a multi-block exclusive scan, and 128-bit fixed-point
// accumulation (order-independent, hence deterministic, summation of FP64 values).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nlg {

constexpr unsigned FULL = 0xffffffffu;

// ceil(log2(x)) for x > 0, exact: frexp splits x = m 2^e with m in [1/2, 1), and only m = 1/2
// (x a power of two) gives e - 1. A rounded log2 can land on the integer below when x is a few
// ulp above a power of two, so the fixed-point scales of the host and the device use this rule.
__host__ __device__ inline int exact_ceil_log2(double x) {
    int e;
    const double m = frexp(x, &e);
    return m == 0.5 ? e - 1 : e;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// ---------------------------------------------------------------- exclusive scan (int64 out)
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename TIn>
__global__ void k_scan_reduce(const TIn *__restrict__ in, long long n, long long *__restrict__ bsum) {
    __shared__ long long ws[SCAN_THREADS / 32];
    const long long base = (long long)blockIdx.x * SCAN_TILE;
    long long s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        long long idx = base + (long long)threadIdx.x * SCAN_ITEMS + i;
        if (idx < n) s += (long long)in[idx];
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < SCAN_THREADS / 32; w++) t += ws[w];
        bsum[blockIdx.x] = t;
    }
}

// Exclusive scan of one tile per block, offset by the scanned block sums: items idx < n_in are
// read (later ones count as 0) and outputs idx < n_out written. in may alias out.
template <typename TIn>
__global__ void k_scan_down(const TIn *in, long long n_in, long long n_out,
                            const long long *__restrict__ boff, long long *out) {
    __shared__ long long ws[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    long long v[SCAN_ITEMS];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        long long idx = base + i;
        v[i] = idx < n_in ? (long long)in[idx] : 0;
        s += v[i];
    }
    long long incl = warp_incl_scan(s, lane);
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    long long woff = 0;
    for (int j = 0; j < w; j++) woff += ws[j];
    long long run = boff[blockIdx.x] + woff + incl - s;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        long long idx = base + i;
        long long t = v[i];
        if (idx < n_out) out[idx] = run;
        run += t;
    }
}

// ---------------------------------------------------------------- double-float accumulation
// An unevaluated sum hi + lo of two floats, updated with error-free transforms (Knuth two-sum):
// about 48 significant bits from FP32 adds only. Used where GB300's FP64 rate would otherwise
// bound the accumulation of per-element blocks and CSR values.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_zero() { return DF{0.f, 0.f}; }
__device__ __forceinline__ DF df_add(DF a, float b) {
    const float s = a.hi + b;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b - bb);
    e += a.lo;
    const float hi = s + e;
    return DF{hi, e - (hi - s)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const float hi = s + e;
    return DF{hi, e - (hi - s)};
}
__device__ __forceinline__ DF df_from_double(double x) {
    const float hi = (float)x;
    return DF{hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }

// ---------------------------------------------------------------- 128-bit fixed point
// A value x of problem scale 2^e is stored as round-toward-zero(x * 2^(FX_FRAC - e)) in a
// two's-complement 128-bit integer split over two uint64 words (lo, hi). Integer addition is
// associative, so the sum is independent of the order atomics land in: run-to-run identical.
constexpr int FX_FRAC = 80;

__device__ __forceinline__ void fx_from_double(double x, int scale_exp, unsigned long long &lo,
                                               long long &hi) {
    lo = 0; hi = 0;
    if (x == 0.0 || !isfinite(x)) return;
    long long bits = __double_as_longlong(x);
    const bool neg = bits < 0;
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffULL);
    int e2;
    if (ex == 0) { e2 = -1074; }            // subnormal
    else { m |= (1ULL << 52); e2 = ex - 1075; }
    const int sh = e2 + FX_FRAC - scale_exp;  // value = m * 2^sh in fixed units
    unsigned long long ulo, uhi;
    if (sh >= 0) {
        if (sh >= 75) { ulo = 0; uhi = 0x7fffffffffffffffULL; }   // saturate (never expected)
        else if (sh >= 64) { ulo = 0; uhi = m << (sh - 64); }
        else if (sh == 0) { ulo = m; uhi = 0; }
        else { ulo = m << sh; uhi = m >> (64 - sh); }
    } else {
        const int r = -sh;
        if (r >= 64) { ulo = 0; uhi = 0; }
        else { ulo = m >> r; uhi = 0; }
    }
    if (neg) {  // two's complement negate
        ulo = ~ulo + 1ULL;
        uhi = ~uhi + (ulo == 0 ? 1ULL : 0ULL);
    }
    lo = ulo;
    hi = (long long)uhi;
}

__device__ __forceinline__ void fx_atomic_add(unsigned long long *acc, double x, int scale_exp,
                                              unsigned *tiny_flag) {
    unsigned long long lo; long long hi;
    fx_from_double(x, scale_exp, lo, hi);
    if (lo == 0 && hi == 0) {
        if (x != 0.0 && tiny_flag) atomicOr(tiny_flag, 1u);
        return;
    }
    unsigned long long old = atomicAdd(&acc[0], lo);
    unsigned long long carry = (old + lo < old) ? 1ULL : 0ULL;
    unsigned long long h = (unsigned long long)hi + carry;
    if (h) atomicAdd(&acc[1], h);
}

__device__ __forceinline__ double fx_to_double(unsigned long long lo, unsigned long long hi,
                                               int scale_exp) {
    const bool neg = (long long)hi < 0;
    if (neg) {
        lo = ~lo + 1ULL;
        hi = ~hi + (lo == 0 ? 1ULL : 0ULL);
    }
    double d = (double)hi * 18446744073709551616.0 + (double)lo;
    d = ldexp(d, scale_exp - FX_FRAC);
    return neg ? -d : d;
}

// Index of (a, b), a <= b, in the row-major upper triangle of a dV x dV symmetric matrix.
template <int dV>
__host__ __device__ __forceinline__ int sym_idx(int a, int b) {
    return a * dV - (a * (a - 1)) / 2 + (b - a);
}

}  // namespace nlg
