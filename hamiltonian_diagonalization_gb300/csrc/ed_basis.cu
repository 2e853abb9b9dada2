// Fock basis of a fixed-Lz sector on the device (K1) and the rank of a
// Fock word in it (K2), plus the int64 scan / max helpers the build uses.
//
// The reference scans every N-bit word of C(norb,N) with Gosper's successor
// and keeps those whose sum of (2k - maxLz) equals 2Lz
// (basis/fermion_fock_basis.cpp:241-354, angular_momentum_constraint.hpp:41-62),
// then ranks with a binary search over the sorted list
// (fermion_fock_basis.cpp:134-161).  Here a word is split into a high half h
// and a low half l.  A sector word fixes, for each h, the popcount and the
// position sum the low half must have: its "class".  The basis in ascending
// order is, for h ascending, h followed by every low word of the needed
// class in ascending order.  Two tables give both the enumeration and the
// rank (H.Q. Lin's two-table indexing):
//   lo[l] = (class(l) << 32) | rank of l among low words of its class
//   hi[h] = (needed class << 48) | number of sector words with high half < h
//   rank(w) = offset(hi[w>>L]) + rank(lo[w & mask]),  miss if classes differ.
// Same words, same order, same indices as the reference: each word of the
// sector has exactly one (h,l) split and both orders are the numeric order.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "ed_internal.h"

namespace edgb {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Per-tile exclusive scan; tile totals to sums[blockIdx.x].
__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                             int64_t* __restrict__ sums)
{
    __shared__ int64_t warp_tot[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t local = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i;
        v[i] = idx < n ? in[idx] : 0;
        local += v[i];
    }
    const int64_t incl = warp_incl_scan(local);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
        t = warp_incl_scan(t);
        if (lane < kScanThreads / 32) warp_tot[lane] = t;
    }
    __syncthreads();
    int64_t run = incl - local + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ offs)
{
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    const int64_t add = offs[blockIdx.x];
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        const int64_t idx = base + i;
        if (idx < n) out[idx] += add;
    }
}

__global__ void k_max_i64(const int64_t* __restrict__ in, int64_t n, unsigned long long* __restrict__ out)
{
    int64_t m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = in[i] > m ? in[i] : m;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        int64_t t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)m);
}

// counts[h] = size of the low class sector words with high half h need.
// wh[i] is the Lz weight of bit L + i.
__global__ void k_basis_count(int H, int L, int N, int64_t S, int max_sum_low,
                              const uint32_t* __restrict__ class_count, const int* __restrict__ wh,
                              int64_t* __restrict__ counts, uint16_t* __restrict__ need_class)
{
    const int64_t nh = 1ll << H;
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
        const int pop_h = __popcll((unsigned long long)h);
        int64_t sum_h = 0;
        uint64_t t = (uint64_t)h;
        while (t) {
            sum_h += wh[__ffsll((long long)t) - 1];
            t &= t - 1;
        }
        const int pl = N - pop_h;
        const int64_t sl = S - sum_h;
        int64_t c = 0;
        uint16_t cls = 0xFFFF;
        if (pl >= 0 && pl <= L && sl >= 0 && sl <= max_sum_low) {
            cls = (uint16_t)(pl * (max_sum_low + 1) + (int)sl);
            c = class_count[cls];
        }
        counts[h] = c;
        need_class[h] = cls;
    }
}

// Momentum sectors: the class of a low word is (popcount, sum kx mod X,
// sum ky mod Y) with bit p at kx = p / Y, ky = p % Y; counts[h] as above.
__global__ void k_basis_count_mom(int H, int L, int N, int X, int Y, int kx_tot, int ky_tot,
                                  const uint32_t* __restrict__ class_count, int64_t* __restrict__ counts,
                                  uint16_t* __restrict__ need_class)
{
    const int64_t nh = 1ll << H;
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
        int sx = 0, sy = 0;
        for (uint64_t t = (uint64_t)h; t; t &= t - 1) {
            const int p = L + __ffsll((long long)t) - 1;
            sx += p / Y;
            sy += p % Y;
        }
        const int pl = N - __popcll((unsigned long long)h);
        int64_t c = 0;
        uint16_t cls = 0xFFFF;
        if (pl >= 0 && pl <= L) {
            const int cx = ((kx_tot - sx) % X + X) % X, cy = ((ky_tot - sy) % Y + Y) % Y;
            cls = (uint16_t)((pl * X + cx) * Y + cy);
            c = class_count[cls];
        }
        counts[h] = c;
        need_class[h] = cls;
    }
}

// One warp per high half: write its block of words and its hi-table entry.
__global__ void k_basis_fill(int H, int L, const int64_t* __restrict__ offs, const int64_t* __restrict__ counts,
                             const uint16_t* __restrict__ need_class, const uint32_t* __restrict__ class_start,
                             const uint32_t* __restrict__ class_list, uint64_t* __restrict__ words,
                             uint64_t* __restrict__ hi)
{
    const int64_t nh = 1ll << H;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t h = warp; h < nh; h += nwarps) {
        const int64_t off = offs[h];
        const int64_t cnt = counts[h];
        const uint16_t cls = need_class[h];
        if (lane == 0) hi[h] = ((uint64_t)cls << 48) | (uint64_t)off;
        if (cnt == 0 || !words) continue;
        const uint32_t start = class_start[cls];
        const uint64_t hw = (uint64_t)h << L;
        for (int64_t t = lane; t < cnt; t += 32) words[off + t] = hw | (uint64_t)class_list[start + t];
    }
}

__global__ void k_basis_rank(const uint64_t* __restrict__ words, uint64_t* __restrict__ idx, uint64_t m,
                             const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo, int L, int norb)
{
    const uint64_t lmask = (1ull << L) - 1ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t w = words[i];
        uint64_t r = kMiss;
        if ((norb >= 64) || (w >> norb) == 0) {
            const uint64_t eh = __ldg(hi + (w >> L));
            const uint64_t el = __ldg(lo + (w & lmask));
            if ((eh >> 48) == ((el >> 32) & 0xFFFFull) && (eh >> 48) != 0xFFFFull)
                r = (eh & 0xFFFFFFFFFFFFull) + (el & 0xFFFFFFFFull);
        }
        idx[i] = r;
    }
}

int grid_for(int64_t work, int threads)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st)
{
    // out has n+1 entries; out[n] = total
    if (n <= 0) {
        ED_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), st));
        return;
    }
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    DevBuf<int64_t> sums(tiles + 1);
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    if (tiles == 1) {
        ED_CUDA(cudaMemcpyAsync(out + n, sums.p, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    } else {
        DevBuf<int64_t> offs(tiles + 1);
        exclusive_scan_i64(sums.p, offs.p, tiles, st);
        k_scan_add<<<(unsigned)tiles, 256, 0, st>>>(out, n, offs.p); ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        ED_CUDA(cudaMemcpyAsync(out + n, offs.p + tiles, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    }
    // the temporaries are freed when they go out of scope; make sure the
    // kernels that read them are done first
    ED_CUDA(cudaStreamSynchronize(st));
}

int64_t reduce_max_i64_host(const int64_t* in, int64_t n, cudaStream_t st)
{
    if (n <= 0) return 0;
    DevBuf<unsigned long long> r(1);
    ED_CUDA(cudaMemsetAsync(r.p, 0, sizeof(unsigned long long), st));
    k_max_i64<<<grid_for(n, 256), 256, 0, st>>>(in, n, r.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    ED_CUDA(cudaMemcpyAsync(&h, r.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    return (int64_t)h;
}

std::vector<int> basis_weights(const ed_basis& b)
{
    std::vector<int> w(b.norb);
    for (int k = 0; k < b.norb; ++k) w[k] = (b.levels == 2 && k >= b.norb1) ? k - b.norb1 + 1 : k;
    return w;
}

namespace {
// Momentum-sector basis (the optical-flux-lattice FermionFockBasis with
// TestLinearMomentumSector2, linear_momentum_constraints_2D.cpp:38-79).
void basis_build_momentum(ed_basis& b, cudaStream_t st)
{
    const int N = b.N, norb = b.norb, X = b.dimX, Y = b.dimY;
    ED_REQUIRE(X >= 1 && Y >= 1 && norb == X * Y && norb <= kMaxOrbitals, ED_ERR_RANGE,
               "momentum basis: need dimX * dimY <= 40 orbitals");
    ED_REQUIRE(N >= 1 && N <= norb && N < 64, ED_ERR_ARG, "need 1 <= N <= norb");
    ED_REQUIRE(b.kx_tot >= 0 && b.kx_tot < X && b.ky_tot >= 0 && b.ky_tot < Y, ED_ERR_ARG,
               "need 0 <= kxTot < dimX and 0 <= kyTot < dimY");
    const int L = norb / 2, H = norb - L;
    b.low_bits = L;
    b.high_bits = H;
    b.dim = 0;
    b.sector_sum = 0;
    const int nclass = (L + 1) * X * Y;
    ED_REQUIRE(nclass < 0xFFFF, ED_ERR_RANGE, "too many low-word classes");
    const uint64_t nl = 1ull << L;
    std::vector<uint32_t> ccount(nclass, 0), cstart(nclass, 0), clist(nl), rank_in_class(nl);
    std::vector<uint64_t> lo(nl);
    for (uint64_t l = 0; l < nl; ++l) {
        int sx = 0, sy = 0;
        for (uint64_t x = l; x; x &= x - 1) {
            const int p = __builtin_ctzll(x);
            sx += p / Y;
            sy += p % Y;
        }
        const int cls = (__builtin_popcountll(l) * X + sx % X) * Y + sy % Y;
        rank_in_class[l] = ccount[cls]++;
        lo[l] = ((uint64_t)cls << 32) | rank_in_class[l];
    }
    uint32_t acc = 0;
    for (int c = 0; c < nclass; ++c) { cstart[c] = acc; acc += ccount[c]; }
    for (uint64_t l = 0; l < nl; ++l) clist[cstart[lo[l] >> 32] + rank_in_class[l]] = (uint32_t)l;
    b.lo.alloc(nl);
    b.hi.alloc(1ull << H);
    DevBuf<uint32_t> d_ccount(nclass), d_cstart(nclass), d_clist(nl);
    ED_CUDA(cudaMemcpyAsync(b.lo.p, lo.data(), nl * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_ccount.p, ccount.data(), nclass * 4, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_cstart.p, cstart.data(), nclass * 4, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_clist.p, clist.data(), nl * 4, cudaMemcpyHostToDevice, st));
    const int64_t nh = 1ll << H;
    DevBuf<int64_t> counts(nh), offs(nh + 1);
    DevBuf<uint16_t> need(nh);
    k_basis_count_mom<<<grid_for(nh, 256), 256, 0, st>>>(H, L, N, X, Y, b.kx_tot, b.ky_tot, d_ccount.p, counts.p,
                                                         need.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(counts.p, offs.p, nh, st);
    int64_t dim = 0;
    ED_CUDA(cudaMemcpyAsync(&dim, offs.p + nh, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    b.dim = (uint64_t)dim;
    b.words.alloc(dim > 0 ? (size_t)dim : 1);
    k_basis_fill<<<grid_for(nh * 32, 256), 256, 0, st>>>(H, L, offs.p, counts.p, need.p, d_cstart.p, d_clist.p,
                                                         b.words.p, b.hi.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));
    if (dim == 0) b.sector_sum = -1;
}
}  // namespace

void basis_build(ed_basis& b, cudaStream_t st)
{
    if (b.dimX > 0) {
        basis_build_momentum(b, st);
        return;
    }
    const int N = b.N, norb = b.norb;
    const int maxbits = b.levels == 2 ? kMaxTwoLevelBits : kMaxOrbitals;
    ED_REQUIRE(norb >= 1 && norb <= maxbits, ED_ERR_RANGE,
               b.levels == 2 ? "two-level words limited to 48 bits (norb0 <= 23)" : "norb must be in 1..40 on the device path");
    ED_REQUIRE(N >= 1 && N <= norb && N < 64, ED_ERR_ARG, "need 1 <= N <= norb");
    // Lz = sum over occupied bits of (2 w - (norbLz - 1)), norbLz the weight span
    const int norb_lz = b.levels == 2 ? b.norb1 : norb;
    const int64_t t = (int64_t)b.two_lz + (int64_t)N * (norb_lz - 1);
    b.dim = 0;
    b.sector_sum = -1;
    const int L = norb / 2, H = norb - L;
    b.low_bits = L;
    b.high_bits = H;
    if (t % 2 != 0) return;
    const int64_t S = t / 2;
    std::vector<int> w = basis_weights(b), ws = w;
    std::sort(ws.begin(), ws.end());
    int64_t smin = 0, smax = 0;
    for (int i = 0; i < N; ++i) smin += ws[i], smax += ws[norb - 1 - i];
    if (S < smin || S > smax) return;
    b.sector_sum = S;

    // low tables on the host (2^L <= 2^24 words)
    int max_sum_low = 0;
    for (int k = 0; k < L; ++k) max_sum_low += w[k];
    const int nclass = (L + 1) * (max_sum_low + 1);
    ED_REQUIRE(nclass < 0xFFFF, ED_ERR_RANGE, "too many low-word classes");
    const uint64_t nl = 1ull << L;
    std::vector<uint32_t> ccount(nclass, 0), cstart(nclass, 0), clist(nl);
    std::vector<uint64_t> lo(nl);
    std::vector<uint32_t> rank_in_class(nl);
    for (uint64_t l = 0; l < nl; ++l) {
        int pop = __builtin_popcountll(l), sum = 0;
        for (uint64_t x = l; x; x &= x - 1) sum += w[__builtin_ctzll(x)];
        const int cls = pop * (max_sum_low + 1) + sum;
        rank_in_class[l] = ccount[cls]++;
        lo[l] = ((uint64_t)cls << 32) | rank_in_class[l];
    }
    uint32_t acc = 0;
    for (int c = 0; c < nclass; ++c) { cstart[c] = acc; acc += ccount[c]; }
    for (uint64_t l = 0; l < nl; ++l) clist[cstart[lo[l] >> 32] + rank_in_class[l]] = (uint32_t)l;

    b.lo.alloc(nl);
    b.hi.alloc(1ull << H);
    DevBuf<uint32_t> d_ccount(nclass), d_cstart(nclass), d_clist(nl);
    ED_CUDA(cudaMemcpyAsync(b.lo.p, lo.data(), nl * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_ccount.p, ccount.data(), nclass * 4, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_cstart.p, cstart.data(), nclass * 4, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(d_clist.p, clist.data(), nl * 4, cudaMemcpyHostToDevice, st));

    const int64_t nh = 1ll << H;
    DevBuf<int64_t> counts(nh), offs(nh + 1);
    DevBuf<uint16_t> need(nh);
    DevBuf<int> d_wh(H);
    ED_CUDA(cudaMemcpyAsync(d_wh.p, w.data() + L, (size_t)H * sizeof(int), cudaMemcpyHostToDevice, st));
    k_basis_count<<<grid_for(nh, 256), 256, 0, st>>>(H, L, N, S, max_sum_low, d_ccount.p, d_wh.p, counts.p, need.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(counts.p, offs.p, nh, st);
    int64_t dim = 0;
    ED_CUDA(cudaMemcpyAsync(&dim, offs.p + nh, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    b.dim = (uint64_t)dim;
    b.words.alloc(dim > 0 ? (size_t)dim : 1);
    k_basis_fill<<<grid_for(nh * 32, 256), 256, 0, st>>>(H, L, offs.p, counts.p, need.p, d_cstart.p, d_clist.p,
                                                         b.words.p, b.hi.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));
}

void basis_compact_tables(const ed_basis& b, cudaStream_t st)
{
    if (b.mf_lo.p || b.dim == 0 || b.levels != 1 || b.dimX > 0) return;
    const int norb = b.norb, L = std::min(13, norb), H = norb - L;
    if (H > 23) return;   // high table over 64 MB: the matrix-free product keeps the main tables
    const int max_sum_low = L * (L - 1) / 2;
    const int nclass = (L + 1) * (max_sum_low + 1);
    const uint64_t nl = 1ull << L;
    std::vector<uint32_t> ccount(nclass, 0);
    std::vector<uint32_t> lo(nl);
    for (uint64_t l = 0; l < nl; ++l) {
        int pop = __builtin_popcountll(l), sum = 0;
        for (uint64_t x = l; x; x &= x - 1) sum += __builtin_ctzll(x);
        const int cls = pop * (max_sum_low + 1) + sum;
        lo[l] = ((uint32_t)cls << 16) | ccount[cls]++;   // classes < 2^16, ranks < C(13,6) < 2^16
    }
    DevBuf<uint32_t> d_ccount(nclass);
    ED_CUDA(cudaMemcpyAsync(d_ccount.p, ccount.data(), nclass * 4, cudaMemcpyHostToDevice, st));
    const int64_t nh = 1ll << H;
    DevBuf<int64_t> counts(nh), offs(nh + 1);
    DevBuf<uint16_t> need(nh);
    DevBuf<uint64_t> hi(nh);
    std::vector<int> wh(H);
    for (int i = 0; i < H; ++i) wh[i] = L + i;   // one level: weights are positions
    DevBuf<int> d_wh(H);
    ED_CUDA(cudaMemcpyAsync(d_wh.p, wh.data(), (size_t)H * sizeof(int), cudaMemcpyHostToDevice, st));
    k_basis_count<<<grid_for(nh, 256), 256, 0, st>>>(H, L, b.N, b.sector_sum, max_sum_low, d_ccount.p, d_wh.p,
                                                     counts.p, need.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(counts.p, offs.p, nh, st);
    k_basis_fill<<<grid_for(nh * 32, 256), 256, 0, st>>>(H, L, offs.p, counts.p, need.p, nullptr, nullptr, nullptr,
                                                         hi.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    DevBuf<uint32_t> dlo(nl);
    ED_CUDA(cudaMemcpyAsync(dlo.p, lo.data(), nl * 4, cudaMemcpyHostToDevice, st));
    int64_t total = 0;
    ED_CUDA(cudaMemcpyAsync(&total, offs.p + nh, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_REQUIRE(total == (int64_t)b.dim, ED_ERR_INTERNAL, "compact rank tables disagree with the basis size");
    b.mf_hi = std::move(hi);
    b.mf_lo = std::move(dlo);
    b.mf_low_bits = L;
}

void basis_rank(const ed_basis& b, const uint64_t* words, uint64_t* idx, uint64_t m, cudaStream_t st)
{
    if (m == 0) return;
    if (b.dim == 0) {
        ED_CUDA(cudaMemsetAsync(idx, 0xFF, m * sizeof(uint64_t), st));
        return;
    }
    k_basis_rank<<<grid_for((int64_t)m, 256), 256, 0, st>>>(words, idx, m, b.hi.p, b.lo.p, b.low_bits, b.norb); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace edgb
