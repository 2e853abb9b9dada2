// Batched sweep (K6): many Hamiltonians of one Lz sector that differ only in
// their pseudopotentials, solved together in lockstep.
//
// All of them share the sparsity pattern: an element of H(V) is
// sign(state) * W_V[hop] for the pair hop it belongs to, and only the per-hop
// table W_V depends on the pseudopotentials.  The pattern is built once per
// sector as CRS with an int32 column and a uint16 code per element (bit 15 =
// fermionic sign, bits 0..14 = hop index; diagonal elements live in a
// separate n x B array).  The block product Y[:,b] = H_b X[:,b] stages the
// per-Hamiltonian hop tables of a tile of TB Hamiltonians in shared memory and
// gives each lane one (row, Hamiltonian) pair, so every element costs one FP64
// FMA and no cross-lane reduction; the column and code of an element are
// loaded once for the TB lanes that share the row.
//
// Vectors are stored [row][problem] (problem index fastest) so the gathers of
// a tile of Hamiltonians read one contiguous segment.  The thick-restart
// Lanczos of ed_lanczos.cu runs here for B problems at once: the same
// recurrences, full FP64 reorthogonalisation and restarts, with every scalar
// per problem and every kernel covering all problems.
#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "ed_hop.cuh"
#include "ed_lanczos.h"
#include "ed_batch.h"

namespace edgb {

namespace {

constexpr uint16_t kCodeSign = 0x8000;

int sms_b() { return batch_sms(); }

// Element code for the pair hop (a,b)->(c,d) of `in` (canonical direction
// as in hop_bits); keep = the hop exists in at least one Hamiltonian.
__device__ __forceinline__ uint16_t hop_code(const HopView& hv, uint64_t in, uint64_t out, int a, int b, int c, int d,
                                             bool& keep)
{
    const int s = a + b;
    const int lo = pair_lo(s, hv.K), cnt = pair_cnt(s, hv.K);
    int h, par;
    if (out > in) {
        h = hv.off[s] + (a - lo) * cnt + (c - lo);
        par = hop_parity(in, a, b, c, d);
    } else {
        h = hv.off[s] + (c - lo) * cnt + (a - lo);
        par = hop_parity(out, c, d, a, b);
    }
    keep = hv.w[h] != 0.0;
    return (uint16_t)((par ? kCodeSign : 0) | h);
}

// off-diagonal entries per row of the union pattern
__global__ void k_pat_count(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ wu, int nw,
                            const int* __restrict__ off, int K, int64_t* __restrict__ rowlen)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double* sw = reinterpret_cast<double*>(smem);
    int* soff = reinterpret_cast<int*>(sw + nw);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = wu[i];
    for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) soff[i] = off[i];
    __syncthreads();
    const HopView hv{sw, nullptr, nullptr, soff, K};
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        int64_t cnt = 0;
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const int s = a + b;
                const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                const int lo = pair_lo(s, K), pc = pair_cnt(s, K);
                for (int ic = 0; ic < pc; ++ic) {
                    const int c = lo + ic, d = s - c;
                    if (c == a || ((rest >> c) & 1ull) || ((rest >> d) & 1ull)) continue;
                    bool keep;
                    hop_code(hv, in, rest | (1ull << c) | (1ull << d), a, b, c, d, keep);
                    cnt += keep ? 1 : 0;
                }
            }
        }
        rowlen[r] = cnt;
    }
}

// One warp per row: (out word, code) pairs, sorted by word, ranked, stored.
__global__ void k_pat_fill(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ wu, int nw,
                           const int* __restrict__ off, int K, int N, const int64_t* __restrict__ rowptr,
                           const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo_tab, int L, int cap,
                           int32_t* __restrict__ col, uint16_t* __restrict__ code, int* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double* sw = reinterpret_cast<double*>(smem);
    int* soff = reinterpret_cast<int*>(sw + nw);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = wu[i];
    for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) soff[i] = off[i];
    __syncthreads();
    const HopView hv{sw, nullptr, nullptr, soff, K};
    const size_t tbytes = ((size_t)nw * 8 + (size_t)2 * K * 4 + 15) & ~(size_t)15;
    const int wic = threadIdx.x >> 5, lane = threadIdx.x & 31, wpc = blockDim.x >> 5;
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem + tbytes) + (size_t)wic * cap;
    uint32_t* pay = reinterpret_cast<uint32_t*>(smem + tbytes + (size_t)wpc * cap * 8) + (size_t)wic * cap;
    int* counter = reinterpret_cast<int*>(smem + tbytes + (size_t)wpc * cap * 12) + wic;
    unsigned char* occ = reinterpret_cast<unsigned char*>(smem + tbytes + (size_t)wpc * cap * 12 + wpc * 4) +
                         (size_t)wic * 64;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int npairs = N * (N - 1) / 2;
    for (int64_t r = gw; r < n; r += nwarps) {
        const uint64_t in = words[r];
        const int64_t base = rowptr[r];
        const int64_t want = rowptr[r + 1] - base;
        for (int pos0 = 0; pos0 < K; pos0 += 32) {
            const int pos = pos0 + lane;
            const bool set = pos < K && ((in >> pos) & 1ull);
            const unsigned m = __ballot_sync(0xffffffffu, set);
            if (set) occ[__popc(m & ((1u << lane) - 1u)) + __popcll(in & ((1ull << pos0) - 1ull))] = (unsigned char)pos;
        }
        if (lane == 0) *counter = 0;
        __syncwarp();
        for (int p = lane; p < npairs; p += 32) {
            int j = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
            while (j * (j - 1) / 2 > p) --j;
            while ((j + 1) * j / 2 <= p) ++j;
            const int i = p - j * (j - 1) / 2;
            const int a = occ[i], b = occ[j];
            const int s = a + b;
            const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
            const int lo = pair_lo(s, K), pc = pair_cnt(s, K);
            for (int ic = 0; ic < pc; ++ic) {
                const int c = lo + ic, d = s - c;
                if (c == a || ((rest >> c) & 1ull) || ((rest >> d) & 1ull)) continue;
                const uint64_t out = rest | (1ull << c) | (1ull << d);
                bool keep;
                const uint16_t cd = hop_code(hv, in, out, a, b, c, d, keep);
                if (!keep) continue;
                const int slot = atomicAdd(counter, 1);
                if (slot < cap) { keys[slot] = out; pay[slot] = cd; }
            }
        }
        __syncwarp();
        const int cnt = *counter;
        if (cnt != want || cnt > cap) {
            if (lane == 0) atomicOr(err, 1);
            __syncwarp();
            continue;
        }
        int P = 1;
        while (P < cnt) P <<= 1;
        for (int t = cnt + lane; t < P; t += 32) keys[t] = ~0ull;
        __syncwarp();
        for (int k = 2; k <= P; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int t = lane; t < (P >> 1); t += 32) {
                    const int i0 = ((t & ~(jj - 1)) << 1) | (t & (jj - 1));
                    const int i1 = i0 + jj;
                    const bool up = (i0 & k) == 0;
                    const uint64_t k0 = keys[i0], k1 = keys[i1];
                    if ((k0 > k1) == up) {
                        keys[i0] = k1;
                        keys[i1] = k0;
                        const uint32_t p0 = pay[i0];
                        pay[i0] = pay[i1];
                        pay[i1] = p0;
                    }
                }
                __syncwarp();
            }
        }
        for (int t = lane; t < cnt; t += 32) {
            const uint64_t c = rank_in_sector(keys[t], hi, lo_tab, L);
            if (c == kMiss) atomicOr(err, 2);
            col[base + t] = (int32_t)c;
            code[base + t] = (uint16_t)pay[t];
        }
        __syncwarp();
    }
}

// diag[r*B + b] for every Hamiltonian: the reference's term order, per-b tables
__global__ void k_bdiag(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ da,
                        const double* __restrict__ db, int K, int B, double* __restrict__ diag)
{
    const int64_t total = n * (int64_t)B;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / B;
        const int b = (int)(t - r * B);
        const uint64_t in = words[r];
        const double* ta = da + (size_t)b * K * K;
        const double* tb = db + (size_t)b * K * K;
        double acc = 0.0;
        for (uint64_t t4 = in; t4; t4 &= t4 - 1) {
            const int k4 = __ffsll((long long)t4) - 1;
            for (uint64_t t3 = in & ~(1ull << k4); t3; t3 &= t3 - 1) {
                const int k3 = __ffsll((long long)t3) - 1;
                acc = acc + ta[k4 * K + k3];
                acc = acc + tb[k4 * K + k3];
            }
        }
        diag[t] = acc;
    }
}

// W with the element's fermionic sign applied: bit 15 of the code moved to the
// sign bit of the high word, an integer XOR that leaves the FP64 pipe to the FMAs.
__device__ __forceinline__ double signed_w(double w, uint16_t code)
{
    return __hiloint2double(__double2hiint(w) ^ (int)((unsigned)(code & kCodeSign) << 16), __double2loint(w));
}

// Y[r][b] = diag[r][b] X[r][b] + sum_k sign_k W_b[h_k] X[col_k][b] for b in
// this CTA's tile [b0, b0+TB) (NT threads).  The tile's hop values
// W[nhop][TB] sit in shared memory; lane = (row slot, b); U loads in flight.
template <int TB, int U, int NT>
__global__ void __launch_bounds__(NT) k_bspmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                              const uint16_t* __restrict__ code, const double* __restrict__ w,
                                              int nhop, const double* __restrict__ diag, const double* __restrict__ X,
                                              double* __restrict__ Y, int64_t n, int B)
{
    extern __shared__ double sw[];   // [nhop][TB]
    const int b0 = blockIdx.y * TB;
    for (int i = threadIdx.x; i < nhop * TB; i += NT) {
        const int h = i / TB, t = i - h * TB;
        sw[i] = (b0 + t < B) ? w[(size_t)h * B + b0 + t] : 0.0;
    }
    __syncthreads();
    constexpr int RPW = 32 / TB;
    const int lane = threadIdx.x & 31, bl = lane % TB, grp = lane / TB;
    const int b = b0 + bl;
    const bool bvalid = b < B;
    const int64_t warp = (blockIdx.x * (int64_t)NT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * NT) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + grp;
        if (r >= n || !bvalid) continue;
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        double acc0 = diag[r * B + b] * X[r * B + b], acc1 = 0.0;
        for (int64_t k = s; k < e; k += U) {
            int c[U];
            uint16_t cd[U];
            double xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) { c[u] = __ldg(col + k + u); cd[u] = __ldg(code + k + u); }
#pragma unroll
            for (int u = 0; u < U; ++u) xv[u] = __ldg(X + (int64_t)c[u] * B + b);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k + u < e) {
                    const double wv = signed_w(sw[(cd[u] & 0x7FFF) * TB + bl], cd[u]);
                    if (u & 1) acc1 = fma(wv, xv[u], acc1);
                    else acc0 = fma(wv, xv[u], acc0);
                }
            }
        }
        Y[r * B + b] = acc0 + acc1;
    }
}

// TB lanes per row (TB = 16 or 32), lanes = TB consecutive Hamiltonians:
// the row's column and code are loaded once (broadcast), the hop values
// W[h][b0..b0+TB) and the gathered X[c][b0..b0+TB) are each one contiguous
// read, and every lane does one FMA per element with no reduction.  The
// [nhop][B] hop table is read through L1 instead of being staged in shared
// memory, so the tile fits whatever the table size.
template <int U, int TB>
__global__ void __launch_bounds__(256) k_bspmm_warp(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                    const uint16_t* __restrict__ code, const double* __restrict__ w,
                                                    const double* __restrict__ diag, const double* __restrict__ X,
                                                    double* __restrict__ Y, int64_t n, int B)
{
    constexpr int RPW = 32 / TB;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.y * TB + (lane % TB);
    const bool bv = b < B;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + lane / TB;
        if (r >= n) continue;
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        double acc0 = bv ? diag[r * B + b] * X[r * B + b] : 0.0, acc1 = 0.0;
        for (int64_t k = s; k < e; k += U) {
            int c[U];
            uint16_t cd[U];
            double xv[U], wv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) { c[u] = __ldg(col + k + u); cd[u] = __ldg(code + k + u); }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                xv[u] = bv ? __ldg(X + (int64_t)c[u] * B + b) : 0.0;
                wv[u] = bv ? __ldg(w + (int64_t)(cd[u] & 0x7FFF) * B + b) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k + u < e) {
                    if (u & 1) acc1 = fma(signed_w(wv[u], cd[u]), xv[u], acc1);
                    else acc0 = fma(signed_w(wv[u], cd[u]), xv[u], acc0);
                }
            }
        }
        if (bv) Y[r * B + b] = acc0 + acc1;
    }
}

// ------------------------------------------------------ batched Lanczos kernels
// Vectors [n][B]; a block owns a row chunk, thread t handles problem t % BP
// (BP = B rounded up to a power of two) on rows t / BP, t / BP + 256/BP, ...

constexpr int kBT = 256;

__device__ __forceinline__ void chunk_rows(int64_t n, int nb, int b, int64_t& r0, int64_t& r1)
{
    r0 = n * (int64_t)b / nb;
    r1 = n * (int64_t)(b + 1) / nb;
}

// sum over the 256/BP threads of each problem, partial to part[(q*nb + blk)*B + p]
__device__ __forceinline__ void reduce_per_problem(double v, double* red, int BP, int B, double* out_slot_base,
                                                   int64_t stride_q, int q)
{
    red[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < BP) {
        double s = 0.0;
        for (int t = threadIdx.x; t < kBT; t += BP) s += red[t];
        if (threadIdx.x < B) out_slot_base[stride_q * q + threadIdx.x] = s;
    }
    __syncthreads();
}

// part[0][blk][p] = v_p . w_p, part[1][blk][p] = w_p . w_p
__global__ void __launch_bounds__(kBT) k_bdot2(const double* __restrict__ v, const double* __restrict__ w, int64_t n,
                                               int B, int BP, double* __restrict__ part)
{
    __shared__ double red[kBT];
    int64_t r0, r1;
    chunk_rows(n, gridDim.x, blockIdx.x, r0, r1);
    const int p = threadIdx.x % BP, rl = threadIdx.x / BP, nrl = kBT / BP;
    double a = 0.0, c = 0.0;
    if (p < B)
        for (int64_t r = r0 + rl; r < r1; r += nrl) {
            const double wv = w[r * B + p];
            a = fma(v[r * B + p], wv, a);
            c = fma(wv, wv, c);
        }
    const int64_t sq = (int64_t)gridDim.x * B;
    reduce_per_problem(a, red, BP, B, part + (int64_t)blockIdx.x * B, sq, 0);
    reduce_per_problem(c, red, BP, B, part + (int64_t)blockIdx.x * B, sq, 1);
}

// out[q][p] = sum over blocks of part[q][blk][p] for q < Q (t = q*B + p):
// 32 consecutive t per CTA, its 8 warps split the block range, and the
// partial sums are combined in a fixed order.  With mask given, out[t] is
// written only where mask[p] != 0.
__global__ void __launch_bounds__(256) k_bsum(const double* __restrict__ part, int nb, int B, int Q,
                                              double* __restrict__ out, const int* __restrict__ mask)
{
    __shared__ double red[8][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    double s = 0.0;
    if (t < Q * B) {
        const int q = t / B, p = t - q * B;
        const double* src = part + (int64_t)q * nb * B + p;
        for (int blk = warp; blk < nb; blk += 8) s += src[(int64_t)blk * B];
    }
    red[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && t < Q * B) {
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) tot += red[w][lane];
        if (!mask || mask[t % B]) out[t] = tot;
    }
}

// w_p -= alpha_p v_p + beta_p u_p
__global__ void k_baxpy2(double* __restrict__ w, const double* __restrict__ v, const double* __restrict__ u, int64_t n,
                         int B, const double* __restrict__ alpha, const double* __restrict__ beta)
{
    const int64_t total = n * (int64_t)B;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(t % B);
        w[t] = fma(-beta[p], u[t], fma(-alpha[p], v[t], w[t]));
    }
}

// Eight per-problem sums at once: acc[t] of every thread to
// part[(q0+t)*stride_q + p] summed over the block's row lanes, for t < cnt.
__device__ __forceinline__ void reduce8_per_problem(const double (&acc)[8], int cnt, double* red, int BP, int B,
                                                    double* out_slot_base, int64_t stride_q, int q0)
{
#pragma unroll
    for (int t = 0; t < 8; ++t) red[t * kBT + threadIdx.x] = acc[t];
    __syncthreads();
    const int nrl = kBT / BP;
    for (int q = threadIdx.x; q < cnt * BP; q += kBT) {
        const int t = q / BP, pp = q - t * BP;
        double s = 0.0;
        for (int l = 0; l < nrl; ++l) s += red[t * kBT + l * BP + pp];
        if (pp < B) out_slot_base[stride_q * (q0 + t) + pp] = s;
    }
    __syncthreads();
}

// part[i][blk][p] = V_i,p . w_p for i < J; part[J][blk][p] = w_p . w_p.
// Columns in groups of eight: one w load and eight independent V loads per
// row in flight.  Problems with need[p] == 0 (when need is given) contribute
// zeros.
__global__ void __launch_bounds__(kBT, 4) k_bmdot(const double* __restrict__ V, int64_t n, int B, int BP, int J,
                                               const double* __restrict__ w, double* __restrict__ part,
                                               const int* __restrict__ need)
{
    __shared__ double red[8 * kBT];
    int64_t r0, r1;
    chunk_rows(n, gridDim.x, blockIdx.x, r0, r1);
    const int p = threadIdx.x % BP, rl = threadIdx.x / BP, nrl = kBT / BP;
    const int64_t vs = n * (int64_t)B;
    const int64_t sq = (int64_t)gridDim.x * B;
    const bool act = p < B && (!need || need[p]);
    for (int i0 = 0; i0 <= J; i0 += 8) {
        double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (act)
#pragma unroll 2
            for (int64_t r = r0 + rl; r < r1; r += nrl) {
                const double wv = w[r * B + p];
                double v[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int i = i0 + t;
                    v[t] = i < J ? V[i * vs + r * B + p] : (i == J ? wv : 0.0);
                }
#pragma unroll
                for (int t = 0; t < 8; ++t) acc[t] = fma(v[t], wv, acc[t]);
            }
        reduce8_per_problem(acc, min(8, J + 1 - i0), red, BP, B, part + (int64_t)blockIdx.x * B, sq, i0);
    }
}

// w_p -= sum_i c[i][p] V_i,p ; npart[blk][p] = |w_p|^2.  Problems with
// need[p] == 0 (when need is given) are left alone and contribute zeros.
// Eight column loads in flight, two FMA chains (even / odd columns), two rows
// per loop trip; with SC the coefficients are staged in shared memory once
// per block instead of re-read for every row.  Both this kernel and the
// multi-dot are held to 64 registers so that four blocks fit per SM (one
// wave of 4 x SMs blocks); measured on a 64-Hamiltonian sweep sector
// 1.94 -> 1.83 s, unrolling by four spills and is slower.
template <bool SC>
__global__ void __launch_bounds__(kBT, 4) k_bupdate(const double* __restrict__ V, int64_t n, int B, int BP, int J,
                                                 const double* __restrict__ c, double* __restrict__ w,
                                                 double* __restrict__ npart, const int* __restrict__ need)
{
    __shared__ double red[kBT];
    extern __shared__ double sc[];   // SC: -c[i][p], J * B values staged once per block
    if (SC) {
        for (int t = threadIdx.x; t < J * B; t += kBT) sc[t] = -c[t];
        __syncthreads();
    }
    int64_t r0, r1;
    chunk_rows(n, gridDim.x, blockIdx.x, r0, r1);
    const int p = threadIdx.x % BP, rl = threadIdx.x / BP, nrl = kBT / BP;
    auto coef = [&](int i) { return SC ? sc[i * B + p] : -__ldg(c + i * B + p); };
    const int64_t vs = n * (int64_t)B;
    double nn = 0.0;
    if (p < B && (!need || need[p])) {
#pragma unroll 2
        for (int64_t r = r0 + rl; r < r1; r += nrl) {
            double acc = w[r * B + p], acc2 = 0.0;
            int i = 0;
            for (; i + 8 <= J; i += 8) {
                double v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = V[(i + u) * vs + r * B + p];
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    acc = fma(coef(i + u), v[u], acc);
                    acc2 = fma(coef((i + u + 1)), v[u + 1], acc2);
                }
            }
            for (; i < J; ++i) acc = fma(coef(i), V[i * vs + r * B + p], acc);
            acc += acc2;
            w[r * B + p] = acc;
            nn = fma(acc, acc, nn);
        }
    }
    reduce_per_problem(nn, red, BP, B, npart + (int64_t)blockIdx.x * B, 0, 0);
}

// Local step bookkeeping: column j gets alpha at row j and beta_{j-1} at row j-1.
__global__ void k_blocal(double* __restrict__ cj, const double* __restrict__ alpha, const double* __restrict__ beta_prev,
                         int j, int B)
{
    for (int p = threadIdx.x; p < B; p += blockDim.x) {
        cj[(size_t)j * B + p] = alpha[p];
        cj[(size_t)(j - 1) * B + p] = beta_prev[p];
    }
}

// cj[i][p] += c[i][p] for i < J where the pass ran for p
__global__ void k_bacc(double* __restrict__ cj, const double* __restrict__ c, int J, int B,
                       const int* __restrict__ need)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < J * B; t += gridDim.x * blockDim.x) {
        const int p = t % B;
        if (!need || need[p]) cj[t] += c[t];
    }
}

// after pass 1: need2[p] = forced or ||w_after||^2 < eta^2 ||w_before||^2 (DGKS)
__global__ void k_bneed(const double* __restrict__ after, const double* __restrict__ before, int B, int force,
                        int* __restrict__ need2)
{
    for (int p = threadIdx.x; p < B; p += blockDim.x)
        need2[p] = (force || after[p] < 0.5 * before[p]) ? 1 : 0;
}

// beta_j = ||w||; breakdown when it vanishes relative to ||H v_j||
__global__ void k_bfinal(const double* __restrict__ norm2, const double* __restrict__ ref2, double* __restrict__ beta,
                         int* __restrict__ brk, int B, int j)
{
    for (int p = threadIdx.x; p < B; p += blockDim.x) {
        const double b = sqrt(norm2[p]);
        const double ref = sqrt(fmax(ref2[p], 0.0));
        if (!(b > 1e-12 * ref)) {
            if (brk[p] == 0) brk[p] = j + 1;
            beta[p] = 1.0;          // keeps the (abandoned) vector finite
        } else {
            beta[p] = b;
        }
    }
}

__global__ void k_bscale(double* __restrict__ w, int64_t n, int B, const double* __restrict__ beta)
{
    const int64_t total = n * (int64_t)B;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(t % B);
        w[t] = w[t] / beta[p];
    }
}

// Ritz vectors of selected problems: for q < Bq, s = keep[q] (a column of the
// Bs-wide basis V) and d = dst ? dst[q] : q (a column of the Bo-wide output),
// out[i][r][d] = sum_j V[j][r][s] Y[i][j][s] for i < k.  With keep = identity
// and dst = null this is the restart rotation; with keep = the surviving
// problems it also compacts them; with dst = original indices it writes
// finished problems' eigenvectors into the caller's layout.
__global__ void k_bgemm_sel(const double* __restrict__ V, int64_t n, int Bs, int m, const double* __restrict__ Y,
                            int k, double* __restrict__ out, int Bo, int Bq, const int* __restrict__ keep,
                            const int* __restrict__ dst)
{
    const int64_t vs = n * (int64_t)Bs, os = n * (int64_t)Bo;
    const int64_t total = n * (int64_t)Bq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / Bq;
        const int q = (int)(t - r * Bq);
        const int s = keep[q];
        const int d = dst ? dst[q] : q;
        const double* v = V + r * Bs + s;
        for (int i0 = 0; i0 < k; i0 += 8) {
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = 0; j < m; ++j) {
                const double x = v[j * vs];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (i0 + u < k) acc[u] = fma(x, __ldg(Y + ((size_t)(i0 + u) * m + j) * Bs + s), acc[u]);
            }
            for (int u = 0; u < 8 && i0 + u < k; ++u) out[(i0 + u) * os + r * Bo + d] = acc[u];
        }
    }
}

// out[r][q] = in[r][keep[q]] for r < rows, q < Bq (in has Bs columns)
__global__ void k_bgather(const double* __restrict__ in, int64_t rows, int Bs, const int* __restrict__ keep, int Bq,
                          double* __restrict__ out)
{
    const int64_t total = rows * (int64_t)Bq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / Bq;
        const int q = (int)(t - r * Bq);
        out[t] = in[r * Bs + keep[q]];
    }
}

__global__ void k_brandom(double* __restrict__ v, int64_t total, uint64_t seed)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(t + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v[t] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    }
}

// residual part: sum over rows of (y - lambda x)^2 per problem
__global__ void __launch_bounds__(kBT) k_bresid(const double* __restrict__ y, const double* __restrict__ x, int64_t n,
                                                int B, int BP, const double* __restrict__ lam, double* __restrict__ part)
{
    __shared__ double red[kBT];
    int64_t r0, r1;
    chunk_rows(n, gridDim.x, blockIdx.x, r0, r1);
    const int p = threadIdx.x % BP, rl = threadIdx.x / BP, nrl = kBT / BP;
    double s = 0.0;
    if (p < B)
        for (int64_t r = r0 + rl; r < r1; r += nrl) {
            const double d = fma(-lam[p], x[r * B + p], y[r * B + p]);
            s = fma(d, d, s);
        }
    reduce_per_problem(s, red, BP, B, part + (int64_t)blockIdx.x * B, 0, 0);
}

}  // namespace

// ------------------------------------------------------------------ host

void batch_create(ed_batch& bt, const ed_basis& basis, int K, int B, const uint16_t* ktab, const double* vtabs,
                  cudaStream_t st)
{
    ED_REQUIRE(B >= 1 && B <= 256, ED_ERR_ARG, "1..256 Hamiltonians per batch");
    ED_REQUIRE(basis.norb == K, ED_ERR_ARG, "tables and basis have different orbital counts");
    ED_REQUIRE(basis.dim > 0, ED_ERR_EMPTY, "empty sector");
    const size_t K3 = (size_t)K * K * K;
    std::vector<HopTables> hops;
    hops.reserve(B);
    for (int b = 0; b < B; ++b) hops.push_back(derive_hop_tables(K, ktab, vtabs + (size_t)b * K3));
    const int nhop = (int)hops[0].w.size();
    ED_REQUIRE(nhop <= 0x7FFF, ED_ERR_RANGE, "too many hop types for 15-bit codes");
    bt.B = B;
    bt.K = K;
    bt.N = basis.N;
    bt.n = (int64_t)basis.dim;
    bt.nhop = nhop;
    std::vector<double> wu(nhop, 0.0), wall((size_t)nhop * B), da((size_t)B * K * K), db((size_t)B * K * K);
    for (int b = 0; b < B; ++b) {
        for (int h = 0; h < nhop; ++h) {
            wall[(size_t)h * B + b] = hops[b].w[h];
            if (hops[b].w[h] != 0.0) wu[h] = 1.0;
        }
        std::memcpy(&da[(size_t)b * K * K], hops[b].diag_a.data(), (size_t)K * K * 8);
        std::memcpy(&db[(size_t)b * K * K], hops[b].diag_b.data(), (size_t)K * K * 8);
    }
    bt.ncoef = nhop + 2 * K * K;
    bt.coef.assign((size_t)B * bt.ncoef, 0.0);
    for (int b = 0; b < B; ++b) {
        double* c = &bt.coef[(size_t)b * bt.ncoef];
        std::memcpy(c, hops[b].w.data(), (size_t)nhop * 8);
        std::memcpy(c + nhop, hops[b].diag_a.data(), (size_t)K * K * 8);
        std::memcpy(c + nhop + K * K, hops[b].diag_b.data(), (size_t)K * K * 8);
    }
    DevBuf<double> dwu(nhop), dda(da.size()), ddb(db.size());
    DevBuf<int> doff(2 * K);
    bt.w.alloc(wall.size());
    ED_CUDA(cudaMemcpyAsync(dwu.p, wu.data(), wu.size() * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(doff.p, hops[0].hop_off.data(), 2 * K * 4, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(bt.w.p, wall.data(), wall.size() * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(dda.p, da.data(), da.size() * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(ddb.p, db.data(), db.size() * 8, cudaMemcpyHostToDevice, st));
    const int64_t n = bt.n;
    bt.diag.alloc((size_t)n * B);
    k_bdiag<<<sms_b() * 8, 256, 0, st>>>(basis.words.p, n, dda.p, ddb.p, K, B, bt.diag.p); count_launch();
    ED_CUDA(cudaGetLastError());
    // union pattern
    const size_t tsm = (size_t)nhop * 8 + (size_t)2 * K * 4;
    DevBuf<int64_t> rowlen(n);
    bt.rowptr.alloc(n + 1);
    ED_CUDA(cudaFuncSetAttribute(k_pat_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    k_pat_count<<<sms_b() * 4, 256, tsm, st>>>(basis.words.p, n, dwu.p, nhop, doff.p, K, rowlen.p); count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(rowlen.p, bt.rowptr.p, n, st);
    ED_CUDA(cudaMemcpyAsync(&bt.nnz, bt.rowptr.p + n, 8, cudaMemcpyDeviceToHost, st));
    const int64_t maxrow = reduce_max_i64_host(rowlen.p, n, st);
    ED_CUDA(cudaStreamSynchronize(st));
    bt.col.alloc((size_t)bt.nnz + kCrsPad);
    bt.code.alloc((size_t)bt.nnz + kCrsPad);
    ED_CUDA(cudaMemsetAsync(bt.col.p + bt.nnz, 0, kCrsPad * 4, st));
    ED_CUDA(cudaMemsetAsync(bt.code.p + bt.nnz, 0, kCrsPad * 2, st));
    int cap = 32;
    while (cap < maxrow) cap <<= 1;
    const size_t tbytes = (tsm + 15) & ~(size_t)15;
    const size_t per_warp = (size_t)cap * 12 + 4 + 64;
    const size_t budget = 200 * 1024;
    ED_REQUIRE(tbytes + per_warp <= budget, ED_ERR_RANGE, "rows too long for the shared-memory sort");
    int wpc = (int)std::min<size_t>(16, (budget - tbytes) / per_warp);
    const size_t smem = tbytes + (size_t)wpc * per_warp;
    ED_CUDA(cudaFuncSetAttribute(k_pat_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DevBuf<int> err(1);
    ED_CUDA(cudaMemsetAsync(err.p, 0, 4, st));
    k_pat_fill<<<sms_b(), wpc * 32, smem, st>>>(basis.words.p, n, dwu.p, nhop, doff.p, K, basis.N, bt.rowptr.p,
                                                basis.hi.p, basis.lo.p, basis.low_bits, cap, bt.col.p, bt.code.p,
                                                err.p); count_launch();
    ED_CUDA(cudaGetLastError());
    int herr = 0;
    ED_CUDA(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_REQUIRE(herr == 0, ED_ERR_INTERNAL, "batched pattern fill: row count or rank check failed on the device");
}

namespace {

constexpr size_t kSmemOptIn = 227 * 1024;   // dynamic shared memory per CTA on sm_103a

template <int TB, int U, int NT>
void launch_bspmm(const ed_batch& bt, const BlockOperands& o, const double* X, double* Y, int64_t rows,
                  cudaStream_t st)
{
    const size_t smem = (size_t)bt.nhop * TB * 8;
    static_assert(U <= kCrsPad, "batch overruns the padding");
    ED_REQUIRE(smem <= kSmemOptIn, ED_ERR_RANGE, "hop table tile exceeds shared memory");
    if (smem > 48 * 1024)
        ED_CUDA(cudaFuncSetAttribute(k_bspmm<TB, U, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bspmm<TB, U, NT>, NT, smem));
    dim3 grid((unsigned)(sms_b() * std::max(1, per_sm)), (unsigned)((o.B + TB - 1) / TB));
    k_bspmm<TB, U, NT><<<grid, NT, smem, st>>>(bt.rowptr.p, bt.col.p, bt.code.p, o.w, bt.nhop, o.diag, X, Y, rows,
                                                 o.B);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

template <int U, int TB>
void launch_bspmm_warp(const ed_batch& bt, const BlockOperands& o, const double* X, double* Y, int64_t rows,
                       cudaStream_t st)
{
    static_assert(U <= kCrsPad, "batch overruns the padding");
    dim3 grid((unsigned)(sms_b() * 8), (unsigned)((o.B + TB - 1) / TB));
    k_bspmm_warp<U, TB><<<grid, 256, 0, st>>>(bt.rowptr.p, bt.col.p, bt.code.p, o.w, o.diag, X, Y, rows, o.B);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

// One block-product variant on rows [0, rows): l1 = 1 reads the hop values
// through L1 (TB 16 or 32 lanes per row); l1 = 0 stages the tile's hop table
// in shared memory (TB 4, 8 or 16 Hamiltonians, 256 or 1024 threads).
void bspmm_variant(const ed_batch& bt, const BlockOperands& o, int tb, int u, int nt, int l1, const double* X,
                   double* Y, int64_t rows, cudaStream_t st)
{
    if (l1) {
        if (tb == 32)
            u == 4 ? launch_bspmm_warp<4, 32>(bt, o, X, Y, rows, st) : launch_bspmm_warp<8, 32>(bt, o, X, Y, rows, st);
        else
            u == 4 ? launch_bspmm_warp<4, 16>(bt, o, X, Y, rows, st) : launch_bspmm_warp<8, 16>(bt, o, X, Y, rows, st);
        return;
    }
#define ED_BSPMM_CASE(TB_, U_, NT_)                                                   \
    if (tb == TB_ && u == U_ && nt == NT_) {                                          \
        launch_bspmm<TB_, U_, NT_>(bt, o, X, Y, rows, st);                            \
        return;                                                                       \
    }
    ED_BSPMM_CASE(4, 4, 256) ED_BSPMM_CASE(4, 8, 256) ED_BSPMM_CASE(8, 4, 256) ED_BSPMM_CASE(8, 8, 256)
    ED_BSPMM_CASE(16, 4, 256) ED_BSPMM_CASE(16, 8, 256)
    ED_BSPMM_CASE(4, 4, 1024) ED_BSPMM_CASE(4, 8, 1024) ED_BSPMM_CASE(8, 4, 1024) ED_BSPMM_CASE(8, 8, 1024)
    ED_BSPMM_CASE(16, 4, 1024) ED_BSPMM_CASE(16, 8, 1024)
#undef ED_BSPMM_CASE
    throw Error(ED_ERR_INTERNAL, "unknown block-product tile");
}

}  // namespace

int batch_sms()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

BlockOperands full_operands(const ed_batch& bt) { return {bt.w.p, bt.diag.p, bt.B}; }

BlockOperands gather_operands(const ed_batch& bt, const int* sel_host, int nsel, DevBuf<double>& w,
                              DevBuf<double>& diag, cudaStream_t st)
{
    ED_REQUIRE(nsel >= 1 && nsel <= bt.B, ED_ERR_ARG, "selection of 1..B problems");
    for (int q = 0; q < nsel; ++q)
        ED_REQUIRE(sel_host[q] >= 0 && sel_host[q] < bt.B, ED_ERR_ARG, "selected problem out of range");
    DevBuf<int> sel(nsel);
    ED_CUDA(cudaMemcpyAsync(sel.p, sel_host, (size_t)nsel * 4, cudaMemcpyHostToDevice, st));
    w.alloc((size_t)bt.nhop * nsel);
    diag.alloc((size_t)bt.n * nsel);
    const auto grid = [&](int64_t work) {
        return (int)std::max<int64_t>(1, std::min<int64_t>(sms_b() * 8, (work + 255) / 256));
    };
    k_bgather<<<grid((int64_t)bt.nhop * nsel), 256, 0, st>>>(bt.w.p, bt.nhop, bt.B, sel.p, nsel, w.p); count_launch();
    k_bgather<<<grid(bt.n * nsel), 256, 0, st>>>(bt.diag.p, bt.n, bt.B, sel.p, nsel, diag.p); count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));   // sel is freed on return
    return {w.p, diag.p, nsel};
}

void batch_block_product(const ed_batch& bt, const BlockOperands& o, const double* X, double* Y, cudaStream_t st)
{
    const std::array<int, 4> t = batch_tile(bt, o, st);
    bspmm_variant(bt, o, t[0], t[1], t[2], t[3], X, Y, bt.n, st);
}

void batch_spmm(const ed_batch& bt, const double* X, double* Y, cudaStream_t st)
{
    batch_block_product(bt, full_operands(bt), X, Y, st);
}

void batch_residuals(const ed_batch& bt, const BlockOperands& o, const double* X, const double* lam, int k,
                     double* res, cudaStream_t st)
{
    const int B = o.B;
    int BP = 1;
    while (BP < B) BP <<= 1;
    const int64_t n = bt.n;
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(sms_b() * 4, n / 128));
    DevBuf<double> y((size_t)n * B), part((size_t)nb * B), s(B), dl(B);
    std::vector<double> l(B), r(B);
    for (int i = 0; i < k; ++i) {
        for (int b = 0; b < B; ++b) l[b] = lam[(size_t)b * k + i];
        ED_CUDA(cudaMemcpyAsync(dl.p, l.data(), (size_t)B * 8, cudaMemcpyHostToDevice, st));
        const double* x = X + (int64_t)i * n * B;
        batch_block_product(bt, o, x, y.p, st);
        k_bresid<<<nb, kBT, 0, st>>>(y.p, x, n, B, BP, dl.p, part.p); count_launch();
        k_bsum<<<(unsigned)((B + 31) / 32), 256, 0, st>>>(part.p, nb, B, 1, s.p, nullptr); count_launch();
        ED_CUDA(cudaMemcpyAsync(r.data(), s.p, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int b = 0; b < B; ++b) res[(size_t)b * k + i] = std::sqrt(r[b]);
    }
}

// Pick the block-product tile that runs fastest on this data, timed on the
// first rows of the pattern (the rows of a sector are alike, and tuning stays
// a small fraction of a solve); tiles whose hop tables do not fit in shared
// memory are skipped.  Choices are remembered per (device, Hamiltonians, hop
// types, mean row length) so that the sectors of one sweep are tuned once.
// ED_TUNE_VERBOSE=1 prints every candidate's time to stderr.
namespace {
std::mutex g_tune_mu;
std::map<std::vector<int64_t>, std::array<int, 4>> g_tune;
}  // namespace

namespace {

// Problem counts share a tile choice within a power-of-two bucket (at least 4).
int tile_bucket(int B)
{
    int b = 4;
    while (b < B) b <<= 1;
    return b;
}

// The fastest block-product tile for operands like o (o.B problems), timed
// on the first rows of the pattern and remembered per (device, bucket of
// o.B, hop types, mean row length).  Never call it during stream capture.
std::array<int, 4> tune_tile(const ed_batch& bt, const BlockOperands& o, cudaStream_t st)
{
    int dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    const int64_t mean_len = bt.n ? (bt.nnz + bt.n / 2) / bt.n : 0;
    const std::vector<int64_t> key{dev, tile_bucket(o.B), bt.nhop, mean_len / 8};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) return it->second;
    }
    const char* verbose_env = std::getenv("ED_TUNE_VERBOSE");
    const bool verbose = verbose_env && verbose_env[0] == '1';
    const int64_t rows = std::min<int64_t>(bt.n, 65536);
    DevBuf<double> X((size_t)bt.n * o.B), Y((size_t)bt.n * o.B);
    k_brandom<<<sms_b() * 4, 256, 0, st>>>(X.p, bt.n * o.B, 7); count_launch();
    cudaEvent_t a, b;
    ED_CUDA(cudaEventCreate(&a));
    ED_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    std::array<int, 4> pick{32, 4, 256, 1};
    std::vector<std::array<int, 4>> cands;
    for (int tb : {4, 8, 16}) {
        const size_t smem = (size_t)bt.nhop * tb * 8;
        if (smem > kSmemOptIn || (tb > 4 && o.B <= tb / 2)) continue;
        for (int u : {4, 8}) {
            if (smem <= 110 * 1024) cands.push_back({tb, u, 256, 0});   // two or more CTAs per SM
            if (smem > 56 * 1024) cands.push_back({tb, u, 1024, 0});    // one large CTA per SM
        }
    }
    for (int tb : {16, 32}) {
        if (o.B <= tb / 2) continue;
        for (int u : {4, 8}) cands.push_back({tb, u, 256, 1});
    }
    for (const auto& c : cands) {
        bspmm_variant(bt, o, c[0], c[1], c[2], c[3], X.p, Y.p, rows, st);
        ED_CUDA(cudaEventRecord(a, st));
        for (int r = 0; r < 3; ++r) bspmm_variant(bt, o, c[0], c[1], c[2], c[3], X.p, Y.p, rows, st);
        ED_CUDA(cudaEventRecord(b, st));
        ED_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        ED_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (verbose)
            std::fprintf(stderr, "ed_batch tune: B=%d tb=%d unroll=%d threads=%d l1=%d rows=%lld  %.4f ms\n", o.B, c[0],
                         c[1], c[2], c[3], (long long)rows, ms / 3);
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[key] = pick;
    return pick;
}

}  // namespace

void batch_autotune(ed_batch& bt, cudaStream_t st)
{
    const std::array<int, 4> pick = tune_tile(bt, full_operands(bt), st);
    bt.tb = pick[0];
    bt.unroll = pick[1];
    bt.nt = pick[2];
    bt.l1 = pick[3];
    bt.tuned = 1;
}

std::array<int, 4> batch_tile(const ed_batch& bt, const BlockOperands& o, cudaStream_t st)
{
    if (o.B == bt.B || !bt.tuned) return {bt.tb, bt.unroll, bt.nt, bt.l1};
    return tune_tile(bt, o, st);
}

// Lockstep thick-restart Lanczos for the B problems of a batch: the
// recurrences of lanczos_solve (local three-term step, full Gram-Schmidt pass
// with a DGKS second pass, forced on the first step of a cycle), every scalar
// per problem.  All active problems restart together.  At a restart the
// problems whose nev pairs have converged retire: their Ritz vectors go to the
// output at their own column, and the survivors' Krylov basis, hop values and
// diagonals are compacted so that later cycles spend no FP64 work on them.  A
// Krylov breakdown, which needs an exactly invariant subspace, is reported as
// ED_ERR_BREAKDOWN for the batch; such a problem is solved with ed_lanczos.
// A restart cycle runs without host round trips and is replayed as a CUDA
// graph on the solver's own stream.
void batch_solve(const ed_batch& bt, const int* sel, int nsel, const ed_lanczos_params& p, const double* V0,
                 double* evals, double* evecs, ed_batch_info* info, cudaStream_t caller_stream)
{
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t n = bt.n;
    const int B0 = sel ? nsel : bt.B;
    const int nev = p.nev;
    ED_REQUIRE(nev >= 1 && nev + 2 < n, ED_ERR_ARG, "need 1 <= nev < n - 2");
    const double tol = p.tol > 0 ? p.tol : 1e-10;
    const int max_restarts = p.max_restarts > 0 ? p.max_restarts : 2000;
    int64_t m64 = p.ncv > 0 ? p.ncv : std::min<int64_t>(n - 1, 2 * (int64_t)nev + 21);
    m64 = std::max<int64_t>(m64, nev + 2);
    m64 = std::min<int64_t>(m64, std::min<int64_t>(n - 1, 200));
    const int m = (int)m64;
    ED_REQUIRE(B0 <= kBT, ED_ERR_ARG, "at most 256 problems per batch");
    SolveStream ss(caller_stream);
    cudaStream_t st = ss.s;
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(sms_b() * 4, n / 128));
    const int64_t vs0 = n * (int64_t)B0;
    // the Gram-Schmidt update stages its coefficients in shared memory when
    // (m + 1) * B0 doubles fit
    const size_t upd_smem = (size_t)(m + 1) * B0 * 8;
    const bool upd_stage = upd_smem <= 200 * 1024;
    if (upd_stage && upd_smem > 48 * 1024)
        ED_CUDA(cudaFuncSetAttribute(k_bupdate<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem));
    DevBuf<double> V((size_t)vs0 * (m + 1)), V2((size_t)vs0 * (m + 1));
    DevBuf<double> part((size_t)(m + 2) * nb * B0), npart((size_t)nb * B0);
    DevBuf<double> sc((size_t)(m + 2) * B0);
    DevBuf<double> s2((size_t)6 * B0);   // [0] alpha [1] |Hv|^2 [2] scratch [3] |w|^2 after a pass
    DevBuf<int> need2(B0), brk(B0), iota(B0), keep(B0), dst(B0);
    DevBuf<double> coef((size_t)m * (m + 1) * B0);
    DevBuf<double> betas((size_t)(m + 1) * B0);
    DevBuf<double> Yd((size_t)B0 * m * m);
    DevBuf<double> wc[2], dc[2];          // compacted operands (allocated at the first retirement)
    ED_CUDA(cudaMemsetAsync(betas.p, 0, betas.bytes(), st));
    std::vector<int> ident(B0);
    for (int b = 0; b < B0; ++b) ident[b] = b;
    ED_CUDA(cudaMemcpyAsync(iota.p, ident.data(), (size_t)B0 * 4, cudaMemcpyHostToDevice, st));

    // the active problems: count, column -> original index, operands, layout
    int B = B0, BP = 1;
    auto set_bp = [&]() { BP = 1; while (BP < B) BP <<= 1; };
    set_bp();
    std::vector<int> orig = ident;
    // the selected problems' operands (gathered once), or the whole batch's
    DevBuf<double> wsel, dsel;
    const BlockOperands ops0 = sel ? gather_operands(bt, sel, nsel, wsel, dsel, st) : full_operands(bt);
    BlockOperands ops = ops0;
    std::array<int, 4> tile = batch_tile(bt, ops, st);
    int64_t vs = vs0;

    auto grid_for = [&](int64_t work) { return (int)std::max<int64_t>(1, std::min<int64_t>(sms_b() * 8, (work + 255) / 256)); };
    auto bsum = [&](const double* src, int Q, double* out, const int* mask) {
        k_bsum<<<(unsigned)((Q * B + 31) / 32), 256, 0, st>>>(src, nb, B, Q, out, mask); count_launch();
    };
    if (V0) ED_CUDA(cudaMemcpyAsync(V.p, V0, (size_t)vs * 8, cudaMemcpyDeviceToDevice, st));
    else { k_brandom<<<grid_for(vs), 256, 0, st>>>(V.p, vs, p.seed); count_launch(); }
    {   // normalise every start vector, rejecting zero or non-finite ones
        k_bdot2<<<nb, kBT, 0, st>>>(V.p, V.p, n, B, BP, part.p); count_launch();
        bsum(part.p, 1, s2.p, nullptr);
        std::vector<double> nn(B);
        ED_CUDA(cudaMemcpyAsync(nn.data(), s2.p, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int b = 0; b < B; ++b) {
            ED_REQUIRE(nn[b] > 0 && std::isfinite(nn[b]), ED_ERR_ARG, "a start vector is zero or not finite");
            nn[b] = std::sqrt(nn[b]);
        }
        ED_CUDA(cudaMemcpyAsync(s2.p + 2 * B, nn.data(), (size_t)B * 8, cudaMemcpyHostToDevice, st));
        k_bscale<<<grid_for(vs), 256, 0, st>>>(V.p, n, B, s2.p + 2 * B); count_launch();
    }
    ed_batch_info inf;
    std::memset(&inf, 0, sizeof(inf));
    inf.tile_hamiltonians = tile[0];
    inf.tile_l1 = tile[3];
    inf.tile_unroll = tile[1];
    inf.tile_threads = tile[3] ? 256 : tile[2];
    std::vector<std::vector<double>> T(B0, std::vector<double>((size_t)m * m, 0.0)), theta(B0), Y(B0);
    std::vector<double> coef_h((size_t)m * (m + 1) * B0), beta_h((size_t)(m + 1) * B0), Yall((size_t)B0 * m * m);
    std::vector<int> brk_h(B0);
    std::vector<cudaEvent_t> ev(2 * (size_t)(m + 1), nullptr);
    for (auto& e : ev) ED_CUDA(cudaEventCreate(&e));
    struct EvG {
        std::vector<cudaEvent_t>& v;
        ~EvG() { for (auto e : v) if (e) cudaEventDestroy(e); }
    } evg{ev};
    // Ritz coefficients of the active problems, [i][j][column] (column fastest)
    auto pack_Y = [&]() {
        for (int q = 0; q < B; ++q) {
            const std::vector<double>& Yb = Y[orig[q]];
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < m; ++j) Yall[((size_t)i * m + j) * B + q] = Yb[(size_t)j + (size_t)m * i];
        }
        ED_CUDA(cudaMemcpyAsync(Yd.p, Yall.data(), (size_t)m * m * B * 8, cudaMemcpyHostToDevice, st));
    };
    // output eigenvectors: [i][r][original index], i < nev
    DevBuf<double> xtmp;
    double* X = evecs;
    if (!X && p.verify) {
        xtmp.alloc((size_t)vs0 * nev);
        X = xtmp.p;
    }
    auto write_ritz = [&](const std::vector<int>& cols) {   // cols: active columns whose pairs are final
        if (!X || cols.empty()) return;
        std::vector<int> d(cols.size());
        for (size_t i = 0; i < cols.size(); ++i) d[i] = orig[cols[i]];
        ED_CUDA(cudaMemcpyAsync(keep.p, cols.data(), cols.size() * 4, cudaMemcpyHostToDevice, st));
        ED_CUDA(cudaMemcpyAsync(dst.p, d.data(), d.size() * 4, cudaMemcpyHostToDevice, st));
        k_bgemm_sel<<<grid_for(n * (int64_t)cols.size()), 256, 0, st>>>(V.p, n, B, m, Yd.p, nev, X, B0,
                                                                        (int)cols.size(), keep.p, dst.p);
        count_launch();
        ED_CUDA(cudaStreamSynchronize(st));   // keep/dst are reused right away
    };

    auto enqueue_cycle = [&](int k, bool capturing) {
        ED_CUDA(cudaMemsetAsync(coef.p, 0, (size_t)m * (m + 1) * B * 8, st));
        ED_CUDA(cudaMemsetAsync(brk.p, 0, (size_t)B * 4, st));
        for (int j = k; j < m; ++j) {
            double* vj = V.p + (int64_t)j * vs;
            double* w = V.p + (int64_t)(j + 1) * vs;
            double* cj = coef.p + (size_t)j * (m + 1) * B;
            const bool first = (j == k);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j], st));
            bspmm_variant(bt, ops, tile[0], tile[1], tile[2], tile[3], vj, w, n, st);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j + 1], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j + 1], st));
            if (!first) {
                k_bdot2<<<nb, kBT, 0, st>>>(vj, w, n, B, BP, part.p); count_launch();
                bsum(part.p, 2, s2.p, nullptr);
                k_blocal<<<1, 256, 0, st>>>(cj, s2.p, betas.p + (size_t)(j - 1) * B, j, B); count_launch();
                k_baxpy2<<<grid_for(vs), 256, 0, st>>>(w, vj, V.p + (int64_t)(j - 1) * vs, n, B, s2.p,
                                                       betas.p + (size_t)(j - 1) * B); count_launch();
            }
            const int J = j + 1;
            for (int pass = 0; pass < 2; ++pass) {
                const int* mask = pass == 0 ? nullptr : need2.p;
                k_bmdot<<<nb, kBT, 0, st>>>(V.p, n, B, BP, J, w, part.p, mask); count_launch();
                bsum(part.p, J + 1, sc.p, nullptr);
                if (upd_stage)
                    k_bupdate<true><<<nb, kBT, (size_t)J * B * 8, st>>>(V.p, n, B, BP, J, sc.p, w, npart.p, mask);
                else
                    k_bupdate<false><<<nb, kBT, 0, st>>>(V.p, n, B, BP, J, sc.p, w, npart.p, mask);
                count_launch();
                k_bacc<<<grid_for((int64_t)J * B), 256, 0, st>>>(cj, sc.p, J, B, mask); count_launch();
                // the norm after the pass, kept from pass 1 for problems that skip pass 2
                bsum(npart.p, 1, s2.p + 3 * B, mask);
                if (pass == 0) {
                    k_bneed<<<1, 256, 0, st>>>(s2.p + 3 * B, sc.p + (size_t)J * B, B, first ? 1 : 0, need2.p);
                    count_launch();
                    if (first)   // ||H v_j||^2 is the norm before the first pass
                        ED_CUDA(cudaMemcpyAsync(s2.p + B, sc.p + (size_t)J * B, (size_t)B * 8, cudaMemcpyDeviceToDevice,
                                                st));
                }
            }
            k_bfinal<<<1, 256, 0, st>>>(s2.p + 3 * B, s2.p + B, betas.p + (size_t)j * B, brk.p, B, j); count_launch();
            k_bscale<<<grid_for(vs), 256, 0, st>>>(w, n, B, betas.p + (size_t)j * B); count_launch();
            ED_CUDA(cudaGetLastError());
        }
    };
    CycleGraphs cache;
    auto run_cycle = [&](int k) {
        CycleGraphs::Entry* g = cache.find(k, V.p);
        if (!g) {
            const uint64_t c0 = launch_count();
            ED_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            try {
                enqueue_cycle(k, true);
            } catch (...) {
                cudaGraph_t broken = nullptr;
                cudaStreamEndCapture(st, &broken);
                if (broken) cudaGraphDestroy(broken);
                throw;
            }
            cudaGraph_t graph = nullptr;
            ED_CUDA(cudaStreamEndCapture(st, &graph));
            const int64_t kernels = (int64_t)(launch_count() - c0);
            count_launches(-kernels);
            cudaGraphExec_t exec = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            ED_CUDA(e);
            cache.e.push_back({k, V.p, exec, kernels});
            g = &cache.e.back();
        }
        ED_CUDA(cudaGraphLaunch(g->exec, st));
        count_launches(g->kernels);
    };

    double spmm_ms = 0.0;
    bool converged = false;
    int finished = 0;
    double retired_res = 0.0;
    int k = 0;
    for (;;) {
        run_cycle(k);
        inf.block_products += m - k;
        inf.problem_products += (int64_t)(m - k) * B;
        ED_CUDA(cudaMemcpyAsync(coef_h.data(), coef.p, (size_t)m * (m + 1) * B * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(beta_h.data(), betas.p, (size_t)(m + 1) * B * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(brk_h.data(), brk.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int j = k; j < m; ++j) {
            float ms = 0.f;
            ED_CUDA(cudaEventElapsedTime(&ms, ev[2 * j], ev[2 * j + 1]));
            spmm_ms += ms;
        }
        std::vector<int> done, live, solved;
        double maxres = 0.0;
        for (int q = 0; q < B; ++q) {
            if (brk_h[q]) {
                inf.breakdowns++;
                continue;
            }
            const int b = orig[q];
            std::vector<double>& Tb = T[b];
            for (int j = k; j < m; ++j)
                for (int i = 0; i <= j; ++i) {
                    const double v = coef_h[((size_t)j * (m + 1) + i) * B + q];
                    Tb[(size_t)i * m + j] = v;
                    Tb[(size_t)j * m + i] = v;
                }
            solved.push_back(q);
        }
        // the active problems' projected matrices in one device launch (a
        // batch large enough to beat the host)
        if (m <= kDeviceEigenMax && (int)solved.size() >= kDeviceEigenMinBatch) {
            const size_t mm = (size_t)m * m;
            std::vector<double> Ts(solved.size() * mm), Es(solved.size() * m), Zs(solved.size() * mm);
            for (size_t t = 0; t < solved.size(); ++t)
                std::copy(T[orig[solved[t]]].begin(), T[orig[solved[t]]].end(), Ts.begin() + t * mm);
            if (!solved.empty()) sym_eigen_batched(m, (int)solved.size(), Ts.data(), Es.data(), Zs.data(), st);
            for (size_t t = 0; t < solved.size(); ++t) {
                const int b = orig[solved[t]];
                theta[b].assign(Es.begin() + t * m, Es.begin() + (t + 1) * m);
                Y[b].assign(Zs.begin() + t * mm, Zs.begin() + (t + 1) * mm);
            }
        } else {
            for (int q : solved) sym_eigen(m, T[orig[q]], theta[orig[q]], Y[orig[q]]);
        }
        for (int q : solved) {
            const int b = orig[q];
            const double bl = beta_h[(size_t)(m - 1) * B + q];
            bool ok = true;
            double rq = 0.0;
            for (int i = 0; i < nev; ++i) {
                const double r = std::fabs(bl * Y[b][(size_t)(m - 1) + (size_t)m * i]);
                rq = std::max(rq, r);
                if (!(r <= tol)) ok = false;
            }
            maxres = std::max(maxres, rq);
            if (ok) retired_res = std::max(retired_res, rq);
            (ok ? done : live).push_back(q);
        }
        ED_REQUIRE(inf.breakdowns == 0, ED_ERR_BREAKDOWN,
                   "Krylov breakdown in a batched problem: solve it with ed_lanczos");
        // worst estimate: problems still iterating and every retired one
        inf.max_residual = std::max(maxres, retired_res);
        pack_Y();
        if (live.empty()) {
            write_ritz(done);
            finished += (int)done.size();
            converged = true;
            break;
        }
        if (inf.restarts >= max_restarts) {
            std::vector<int> all(B);
            for (int q = 0; q < B; ++q) all[q] = q;
            write_ritz(all);
            finished += (int)done.size();
            break;
        }
        ++inf.restarts;
        // the same keep rule as lanczos_solve (nev 4, m 29: 10 kept; 2.06 s
        // for the 64-point sweep sector against 2.15 s keeping 16)
        int kk = std::min(m - 2, nev + std::max(1, (m - nev) / 4));
        kk = std::max(kk, std::min(nev, m - 1));
        if (!done.empty()) {
            // retire the converged problems and compact the survivors
            write_ritz(done);
            finished += (int)done.size();
            const int Bn = (int)live.size();
            const int64_t vsn = n * (int64_t)Bn;
            ED_CUDA(cudaMemcpyAsync(keep.p, live.data(), (size_t)Bn * 4, cudaMemcpyHostToDevice, st));
            k_bgemm_sel<<<grid_for(vsn), 256, 0, st>>>(V.p, n, B, m, Yd.p, kk, V2.p, Bn, Bn, keep.p, nullptr);
            count_launch();
            k_bgather<<<grid_for(vsn), 256, 0, st>>>(V.p + (int64_t)m * vs, n, B, keep.p, Bn, V2.p + (int64_t)kk * vsn);
            count_launch();
            const int nxt = (ops.w == wc[0].p) ? 1 : 0;
            if (!wc[nxt].p) {
                wc[nxt].alloc((size_t)bt.nhop * B0);
                dc[nxt].alloc((size_t)vs0);
            }
            k_bgather<<<grid_for((int64_t)bt.nhop * Bn), 256, 0, st>>>(ops.w, bt.nhop, B, keep.p, Bn, wc[nxt].p);
            count_launch();
            k_bgather<<<grid_for(vsn), 256, 0, st>>>(ops.diag, n, B, keep.p, Bn, dc[nxt].p);
            count_launch();
            ED_CUDA(cudaGetLastError());
            ops = {wc[nxt].p, dc[nxt].p, Bn};
            tile = batch_tile(bt, ops, st);
            std::vector<int> no(Bn);
            for (int q = 0; q < Bn; ++q) no[q] = orig[live[q]];
            orig = no;
            B = Bn;
            vs = vsn;
            set_bp();
            for (auto& x : cache.e) cudaGraphExecDestroy(x.exec);
            cache.e.clear();
        } else {
            k_bgemm_sel<<<grid_for(vs), 256, 0, st>>>(V.p, n, B, m, Yd.p, kk, V2.p, B, B, iota.p, nullptr);
            count_launch();
            ED_CUDA(cudaMemcpyAsync(V2.p + (int64_t)kk * vs, V.p + (int64_t)m * vs, (size_t)vs * 8,
                                    cudaMemcpyDeviceToDevice, st));
        }
        std::swap(V, V2);
        for (int q = 0; q < B; ++q) {
            const int b = orig[q];
            std::vector<double>& Tb = T[b];
            std::fill(Tb.begin(), Tb.end(), 0.0);
            const double bl = beta_h[(size_t)(m - 1) * (B + (int)done.size()) + (size_t)live[q]];
            for (int i = 0; i < kk; ++i) {
                Tb[(size_t)i * m + i] = theta[b][i];
                const double sv = bl * Y[b][(size_t)(m - 1) + (size_t)m * i];
                Tb[(size_t)i * m + kk] = sv;
                Tb[(size_t)kk * m + i] = sv;
            }
        }
        k = kk;
        ED_CUDA(cudaStreamSynchronize(st));
    }
    inf.converged = finished;
    for (int b = 0; b < B0; ++b)
        for (int i = 0; i < nev; ++i) evals[(size_t)b * nev + i] = theta[b][i];
    if (p.verify && X) {
        // true residuals of every problem, through its own operator
        std::vector<double> res((size_t)B0 * nev);
        batch_residuals(bt, ops0, X, evals, nev, res.data(), st);
        inf.block_products += nev;
        inf.problem_products += (int64_t)nev * B0;
        double worst = 0.0;
        int ok_all = 0;
        for (int b = 0; b < B0; ++b) {
            bool ok = true;
            for (int i = 0; i < nev; ++i) {
                const double r = res[(size_t)b * nev + i];
                worst = std::max(worst, r);
                if (!(r <= tol)) ok = false;
            }
            ok_all += ok ? 1 : 0;
        }
        inf.max_residual = worst;
        inf.converged = ok_all;
    }
    ED_CUDA(cudaStreamSynchronize(st));
    inf.spmm_seconds = spmm_ms * 1e-3;
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = inf;
    ED_REQUIRE(converged, ED_ERR_NOCONV, "batched Lanczos did not converge within the restart cap");
}

}  // namespace edgb

using namespace edgb;

extern "C" {

ed_status ed_batch_create(const ed_basis* b, int nham, const uint16_t* ktable, const double* vtables, int autotune,
                          ed_batch** out)
{
    return guard([&] {
        ED_REQUIRE(b && ktable && vtables && out, ED_ERR_ARG, "NULL argument");
        *out = nullptr;
        ed_batch* bt = new ed_batch();
        try {
            batch_create(*bt, *b, b->norb, nham, ktable, vtables, nullptr);
            if (autotune) batch_autotune(*bt, nullptr);
        } catch (...) {
            delete bt;
            throw;
        }
        *out = bt;
    });
}

ed_status ed_batch_free(ed_batch* bt)
{
    return guard([&] { delete bt; });
}

ed_status ed_batch_dims(const ed_batch* bt, int64_t* n, int64_t* nnz, int* nham)
{
    return guard([&] {
        ED_REQUIRE(bt, ED_ERR_ARG, "NULL batch");
        if (n) *n = bt->n;
        if (nnz) *nnz = bt->nnz;
        if (nham) *nham = bt->B;
    });
}

ed_status ed_batch_spmm(const ed_batch* bt, const double* X, double* Y, ed_stream stream)
{
    return guard([&] {
        ED_REQUIRE(bt && X && Y, ED_ERR_ARG, "NULL argument");
        ED_REQUIRE(X != Y, ED_ERR_ARG, "X and Y must be distinct");
        batch_spmm(*bt, X, Y, (cudaStream_t)stream);
    });
}

ed_status ed_batch_solve(const ed_batch* bt, const ed_lanczos_params* p, const double* V0, double* evals,
                         double* evecs, ed_batch_info* info)
{
    return guard([&] {
        ED_REQUIRE(bt && p && evals, ED_ERR_ARG, "NULL argument");
        if (info) std::memset(info, 0, sizeof(*info));
        batch_solve(*bt, nullptr, 0, *p, V0, evals, evecs, info, nullptr);
    });
}

}  // extern "C"

namespace edgb {
}  // namespace edgb

