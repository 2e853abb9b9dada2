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
// st without a and b.  Returns 1 for a minus sign.
__device__ __forceinline__ int hop_parity(uint64_t st, int a, int b, int c, int d)
{
    const uint64_t ba = 1ull << a, bb = 1ull << b, bc = 1ull << c, bd = 1ull << d;
    int n = __popcll(st & (ba - 1));
    uint64_t o = st ^ ba;
    n += __popcll(o & (bb - 1));
    o ^= bb;
    n += __popcll(o & (bc - 1));
    o |= bc;
    n += __popcll(o & (bd - 1));
    return n & 1;
}

// Element <out|H|in> for the pair hop (a,b) -> (c,d) of `in` (a<b, c<d),
// computed from the lower-word side as the reference's upper triangle
// stores it.  Returns 0.0 when the reference drops the element.
__device__ __forceinline__ double hop_element(const HopView& hv, uint64_t in, uint64_t out, int a, int b, int c,
                                              int d)
{
    const int s = a + b;
    const int lo = pair_lo(s, hv.K), cnt = pair_cnt(s, hv.K);
    double w;
    int par;
    if (out > in) {
        w = hv.w[hv.off[s] + (a - lo) * cnt + (c - lo)];
        par = hop_parity(in, a, b, c, d);
    } else {
        w = hv.w[hv.off[s] + (c - lo) * cnt + (a - lo)];
        par = hop_parity(out, c, d, a, b);
    }
    return par ? -w : w;
}

// Diagonal element in the reference's term order (k4 ascending over the
// occupied bits, k3 ascending over the others, k2 in {k3,k4} ascending).
__device__ __forceinline__ double diag_element(const HopView& hv, uint64_t in)
{
    double acc = 0.0;
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
