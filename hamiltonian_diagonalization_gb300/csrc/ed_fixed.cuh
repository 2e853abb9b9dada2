// Exact fixed-point arithmetic on the integer pipes, for the stored-CRS
// products (ed_spmv.cu, ed_complex.cu).
//
// A value v is held as A = round(v 2^(1080 - E)), |A| < 2^58 when
// |v| < 2^(E - 1022) (E a bound on the biased exponent field), split into
// the limb pair (A mod 2^30, floor(A / 2^30)) of 32-bit integers in one
// 64-bit word.  Products of two such values are formed exactly from four
// 32x32->64-bit multiply-adds, sums are kept exactly in 128 bits, and a sum
// is rounded once to FP64 by integer operations.
#pragma once

#include <cstdint>

namespace edgb {
namespace {

// Biased exponent field, 1 for zeros and subnormals (their scale).
__device__ __forceinline__ int fix_exp(double v)
{
    const int e = (int)(((uint64_t)__double_as_longlong(v) >> 52) & 0x7FF);
    return e ? e : 1;
}

// The limb pair (A mod 2^30, floor(A / 2^30)) of A = round(v 2^(1080 - E)),
// rounded to nearest with ties away from zero, as one 64-bit word (limb
// A mod 2^30 in the low half).  |v| < 2^(E - 1022) gives |A| < 2^58.
__device__ __forceinline__ int64_t fix_pair(double v, int E)
{
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    const uint64_t m = (b & ((1ull << 52) - 1)) | (e ? (1ull << 52) : 0ull);
    const int sh = (e ? e : 1) - E + 5;   // <= 5: m 2^sh < 2^58
    uint64_t q = 0;
    if (sh >= 0) q = m << sh;
    else if (sh > -64) q = (m + (1ull << (-sh - 1))) >> -sh;
    const int64_t A = (b >> 63) ? -(int64_t)q : (int64_t)q;
    const uint32_t lo = (uint32_t)(A & ((1 << 30) - 1));
    const uint32_t hi = (uint32_t)(int32_t)(A >> 30);
    return (int64_t)(((uint64_t)hi << 32) | lo);
}

__device__ __forceinline__ long long mul_wide(int a, int b)
{
    long long d;
    asm("mul.wide.s32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
    return d;
}

__device__ __forceinline__ long long mad_wide(int a, int b, long long c)
{
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// +-(w1 2^64 + w0) 2^sc rounded to the nearest double (ties to even), by
// integer operations only; subnormal and infinite results included.
__device__ __forceinline__ double round_u128(unsigned long long w1, unsigned long long w0, bool neg, int sc)
{
    int nb;                  // bit length of the magnitude
    unsigned long long t;    // its 64 leading bits, the first at bit 63
    bool st;                 // a set bit below them
    if (w1) {
        const int z = __clzll((long long)w1);
        nb = 128 - z;
        t = z ? (w1 << z) | (w0 >> (64 - z)) : w1;
        st = (z ? (w0 << z) : w0) != 0;
    } else if (w0) {
        const int z = __clzll((long long)w0);
        nb = 64 - z;
        t = w0 << z;
        st = false;
    } else {
        return 0.0;
    }
    const unsigned long long sign = neg ? (1ull << 63) : 0ull;
    const int eb = nb + sc + 1022;   // biased exponent of a normal result
    if (eb >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    const int drop = eb >= 1 ? 11 : 12 - eb;   // bits of t below the last place kept
    unsigned long long mant, rnd, stk;
    if (drop <= 63) {
        mant = t >> drop;
        rnd = (t >> (drop - 1)) & 1ull;
        stk = ((t & ((1ull << (drop - 1)) - 1ull)) != 0 || st) ? 1ull : 0ull;
    } else if (drop == 64) {
        mant = 0;
        rnd = t >> 63;
        stk = ((t << 1) != 0 || st) ? 1ull : 0ull;
    } else {
        mant = 0;
        rnd = 0;
        stk = 1;
    }
    mant += rnd & (stk | (mant & 1ull));
    // a carry out of the 53 bits moves into the exponent field by itself
    const unsigned long long bits = eb >= 1 ? ((unsigned long long)(eb - 1) << 52) + mant : mant;
    return __longlong_as_double((long long)(sign | bits));
}

// round(S 2^sc) for a two's complement S.
__device__ __forceinline__ double round_i128(__int128 S, int sc)
{
    const bool neg = S < 0;
    const unsigned __int128 M = neg ? (unsigned __int128)(-S) : (unsigned __int128)S;
    return round_u128((unsigned long long)(M >> 64), (unsigned long long)M, neg, sc);
}

// Per-block maxima of fix_exp over v[0, n) into part[blockIdx.x].
__global__ void __launch_bounds__(256) k_fix_exp(const double* __restrict__ v, int64_t n, int* __restrict__ part)
{
    __shared__ int sm[8];
    int m = 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, fix_exp(v[i]));
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = max(r, sm[w]);
        part[blockIdx.x] = r;
    }
}

// q[i] = fix_pair(v[i], E) with E the maximum of part[0, nparts); block 0
// also stores E in part[nparts] for the product.
__global__ void __launch_bounds__(256) k_fix_conv(const double* __restrict__ v, int64_t n, int* __restrict__ part,
                                                  int nparts, int64_t* __restrict__ q)
{
    __shared__ int sE;
    if (threadIdx.x < 32) {
        int m = 1;
        for (int i = threadIdx.x; i < nparts; i += 32) m = max(m, part[i]);
        m = __reduce_max_sync(0xffffffffu, m);
        if (threadIdx.x == 0) {
            sE = m;
            if (blockIdx.x == 0) part[nparts] = m;
        }
    }
    __syncthreads();
    const int E = sE;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        q[i] = fix_pair(v[i], E);
}

// p2, p1, p0 += the three limb products of a b (weights 2^60, 2^30, 1).
__device__ __forceinline__ void fix_mac(int2 a, int2 b, long long& p2, long long& p1, long long& p0)
{
    p2 = mad_wide(a.y, b.y, p2);
    p1 = mad_wide(a.y, b.x, p1);
    p1 = mad_wide(a.x, b.y, p1);
    p0 = mad_wide(a.x, b.x, p0);
}

__device__ __forceinline__ __int128 fix_combine(long long p2, long long p1, long long p0)
{
    return ((__int128)p2 << 60) + ((__int128)p1 << 30) + (__int128)p0;
}

// The sum of an int128 over the 32 lanes of a warp (exact).
__device__ __forceinline__ __int128 warp_sum_i128(__int128 v)
{
    long long hi = (long long)(v >> 64);
    unsigned long long lo = (unsigned long long)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long ohi = __shfl_xor_sync(0xffffffffu, hi, o);
        const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, o);
        const unsigned long long t = lo + olo;
        hi += ohi + (t < lo ? 1 : 0);
        lo = t;
    }
    return ((__int128)hi << 64) | (__int128)lo;
}

}  // namespace
}  // namespace edgb
