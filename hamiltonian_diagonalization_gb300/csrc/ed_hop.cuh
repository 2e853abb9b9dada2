// Device helpers shared by the Hamiltonian build (K3) and the matrix-free
// product (K5): per-hop table in shared memory, the fermionic sign of a pair
// hop, the diagonal sum, and the rank of a sector word.
#pragma once

#include "ed_internal.h"

namespace edgb {

// Shared-memory image of the hop tables: [w (nw doubles)][diag_a K*K][diag_b K*K][hop_off 2K ints]
struct HopView {
    const double* w;
    const double* da;
    const double* db;
    const int* off;
    int K;
};

__host__ __device__ inline size_t hop_smem_bytes(int K, int nw)
{
    return (size_t)nw * 8 + (size_t)2 * K * K * 8 + (size_t)2 * K * 4;
}

__device__ __forceinline__ HopView load_hop_smem(unsigned char* smem, const double* w, int nw, const double* da,
                                                 const double* db, const int* off, int K)
{
    double* sw = reinterpret_cast<double*>(smem);
    double* sda = sw + nw;
    double* sdb = sda + K * K;
    int* soff = reinterpret_cast<int*>(sdb + K * K);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = w[i];
    for (int i = threadIdx.x; i < K * K; i += blockDim.x) { sda[i] = da[i]; sdb[i] = db[i]; }
    for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) soff[i] = off[i];
    __syncthreads();
    return HopView{sw, sda, sdb, soff, K};
}

// Parity of the operator c+_d c+_c c_b c_a (Evaluate_CdCdCC with k4=a, k3=b,
// k2=c, k1=d; fermions.hpp:87-133) on state st, a<b occupied, c<d empty in
// st without a and b.  Returns 1 for a minus sign.  The reference counts the
// occupied orbitals each operator passes, one operator at a time; mod 2 that
// is 1 + |st in (a,b)| + |rest in (c,d)| (rest = st without a and b, open
// intervals), one popcount.  The reverse hop c+_b c+_a c_d c_c on the result
// has the same parity (the two terms are Hermitian conjugates).
__device__ __forceinline__ uint64_t bits_between(int x, int y)   // x < y <= 63: bits x+1 .. y-1
{
    return ((1ull << y) - 1ull) & ~((2ull << x) - 1ull);
}

__device__ __forceinline__ int hop_parity(uint64_t st, int a, int b, int c, int d)
{
    const uint64_t rest = st ^ (1ull << a) ^ (1ull << b);
    return (1 + __popcll((st & bits_between(a, b)) ^ (rest & bits_between(c, d)))) & 1;
}

// Admissible created pairs (c, d = a+b-c) of the pair hop that removes a<b
// from `in`, as a mask over c: c < d <= K-1, c and d empty once a and b are
// removed, (c,d) != (a,b); with upper, also out > in, i.e. d > b, i.e. c < a.
// Bit c of `mirror` is bit a+b-c of `empty` (a bit reverse and a shift).
__device__ __forceinline__ uint64_t hop_targets(uint64_t in, int a, int b, int K, bool upper)
{
    const int s = a + b;
    const int lo = pair_lo(s, K), hi = (s - 1) >> 1;
    if (hi < lo) return 0ull;
    const uint64_t kmask = K >= 64 ? ~0ull : ((1ull << K) - 1ull);
    const uint64_t empty = ~(in ^ (1ull << a) ^ (1ull << b)) & kmask;
    const uint64_t r = __brevll(empty);
    const uint64_t mirror = s <= 63 ? (r >> (63 - s)) : (r << (s - 63));
    uint64_t range = ((2ull << hi) - 1ull) & ~((1ull << lo) - 1ull);   // hi <= K-2 <= 62
    if (upper) range &= (1ull << a) - 1ull;
    return empty & mirror & range & ~(1ull << a);
}

// Bits of the element <out|H|in> for the pair hop (a,b) -> (c,d) of `in`
// (a<b, c<d), computed from the lower-word side as the reference's upper
// triangle stores it: the table weight with its sign bit flipped for an odd
// parity (negation is exact, so these are the bits of +-w).  The element is
// dropped, as the reference drops it, when hop_zero() holds; testing the bits
// keeps the comparison off the FP64 pipe.
__device__ __forceinline__ uint64_t hop_bits(const HopView& hv, uint64_t in, uint64_t out, int a, int b, int c,
                                             int d)
{
    const int s = a + b;
    const int lo = pair_lo(s, hv.K), cnt = pair_cnt(s, hv.K);
    const uint64_t* wb = reinterpret_cast<const uint64_t*>(hv.w);
    const int idx = out > in ? (a - lo) * cnt + (c - lo) : (c - lo) * cnt + (a - lo);
    const uint64_t w = wb[hv.off[s] + idx];
    return w ^ ((uint64_t)hop_parity(in, a, b, c, d) << 63);
}

// x == 0.0 on the bits of x (true for +0 and -0, false for NaN).
__device__ __forceinline__ bool hop_zero(uint64_t bits) { return (bits << 1) == 0; }

__device__ __forceinline__ double bits_to_double(uint64_t bits) { return __longlong_as_double((long long)bits); }

// Diagonal element in the reference's term order (k4 ascending over the
// occupied bits, k3 ascending over the others, k2 in {k3,k4} ascending),
// added term by term to acc (0 for a one-level Hamiltonian; the running sum of
// the earlier term groups for the two-level one).
__device__ __forceinline__ double diag_element(const HopView& hv, uint64_t in, double acc = 0.0)
{
    for (uint64_t t4 = in; t4; t4 &= t4 - 1) {
        const int k4 = __ffsll((long long)t4) - 1;
        const uint64_t others = in & ~(1ull << k4);
        for (uint64_t t3 = others; t3; t3 &= t3 - 1) {
            const int k3 = __ffsll((long long)t3) - 1;
            acc = acc + hv.da[k4 * hv.K + k3];
            acc = acc + hv.db[k4 * hv.K + k3];
        }
    }
    return acc;
}

__device__ __forceinline__ uint64_t rank_in_sector(uint64_t w, const uint64_t* __restrict__ hi,
                                                   const uint64_t* __restrict__ lo, int L)
{
    const uint64_t eh = __ldg(hi + (w >> L));
    const uint64_t el = __ldg(lo + (w & ((1ull << L) - 1ull)));
    if ((eh >> 48) != ((el >> 32) & 0xFFFFull)) return kMiss;
    return (eh & 0xFFFFFFFFFFFFull) + (el & 0xFFFFFFFFull);
}

}  // namespace edgb
