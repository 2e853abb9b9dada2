// Hamiltonian-vector products: stored CRS (K4) and matrix-free (K5).
//
// Reference: MatrixVectorFunction::Simple (hamiltonians/matrix_vector_routines.hpp:94-104)
// -> SymmetricMatrixVectorMultiply (utilities/mathematics/sparse_linear_algebra.hpp:143-164):
//   y[i] += a*x[c]; if (i != c) y[c] += a*x[i]   over the stored upper triangle.
//
// On GB300 FP64 FMA issues at about 0.6e12/s, which is what streaming the CRS
// at HBM rate (12 bytes per nonzero) demands, so the kernels spend FP64
// instructions only on the products: a row is owned by G lanes (G = 4 or 8
// for the model's 200-350 nonzeros per row), each lane accumulates its share
// serially into one FMA chain, and only log2(G) shuffle additions per lane
// remain.  Column and value streams are read once with evict-first loads so
// that x stays resident in L2.
#include <algorithm>
#include <map>

#include "ed_hop.cuh"

namespace edgb {

namespace {

__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int32_t* p) { return __ldcs(p); }

// Byte offset of the low-word table in k_hv_matfree_c's shared memory (after
// nw weights and 2K pair offsets, 16-byte aligned).
__host__ __device__ inline size_t matfree_c_table_offset(int nw, int K)
{
    return ((size_t)nw * 8 + (size_t)2 * K * 4 + 15) & ~(size_t)15;
}

// G lanes per row, each lane summing every G-th element of the row in one
// FMA chain, with the loads of U of its elements issued ahead of their FMAs
// (same element order, so U does not change y).  Measured on GB300 (N=11,
// 2S=30, 30 products): G=8 U=4 0.835-0.841 ms, U=2 0.841, U=1 0.862, U=8
// 0.869; G=4 U=2/4 0.90/0.93 ms, G=16 0.91 ms; two or four FMA chains per
// lane 0.89-1.04 ms.  The extra chains cost registers and FP64 additions
// without adding useful memory parallelism: the warps of a full SM already
// keep the DRAM queue busy.
template <int G, int U = 1>
__global__ void __launch_bounds__(256) k_spmv_full(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                   const double* __restrict__ val, const double* __restrict__ x,
                                                   double* __restrict__ y, int64_t n)
{
    constexpr int RPW = 32 / G;   // rows per warp per step
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {   // warp-uniform loop
        const int64_t r = rb + grp;
        const bool valid = r < n;
        const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
        double acc = 0.0;
        if (U == 1) {
            for (int64_t k = s + sub; k < e; k += G) acc = fma(ld_stream(val + k), __ldg(x + ld_stream(col + k)), acc);
        } else {
            for (int64_t k0 = s + sub; k0 < e; k0 += (int64_t)G * U) {
                double v[U];
                int c[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int64_t k = k0 + (int64_t)u * G;
                    v[u] = k < e ? ld_stream(val + k) : 0.0;
                    c[u] = k < e ? ld_stream(col + k) : 0;
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (k0 + (int64_t)u * G < e) acc = fma(v[u], __ldg(x + c[u]), acc);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (valid && sub == 0) y[r] = acc;
    }
}

// Upper-triangle storage, the reference's layout: gather for the stored
// part, scatter (atomic) for the transposed part.  y must be zero on entry.
template <int G>
__global__ void __launch_bounds__(256) k_spmv_upper(const int64_t* __restrict__ rowptr,
                                                    const int32_t* __restrict__ col, const double* __restrict__ val,
                                                    const double* __restrict__ x, double* __restrict__ y, int64_t n)
{
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + grp;
        const bool valid = r < n;
        const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
        const double xr = valid ? __ldg(x + r) : 0.0;
        double acc = 0.0;
        for (int64_t k = s + sub; k < e; k += G) {
            const int c = ld_stream(col + k);
            const double v = ld_stream(val + k);
            acc = fma(v, __ldg(x + c), acc);
            if (c != r) atomicAdd(y + c, v * xr);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (valid && sub == 0) atomicAdd(y + r, acc);
    }
}

// Matrix-free product: one thread per row regenerates the row's elements
// (pair hops, parity sign, per-hop value from shared memory, two-table rank)
// and accumulates them; the stored diagonal supplies y_i's own term.
__global__ void __launch_bounds__(256) k_hv_matfree(const uint64_t* __restrict__ words, int64_t n,
                                                    const double* __restrict__ diag, const double* __restrict__ w,
                                                    int nw, const double* __restrict__ da,
                                                    const double* __restrict__ db, const int* __restrict__ off, int K,
                                                    const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo_tab,
                                                    int L, const double* __restrict__ x, double* __restrict__ y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const HopView hv = load_hop_smem(smem, w, nw, da, db, off, K);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        double acc = diag[r] * __ldg(x + r);
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const int s = a + b;
                const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                // admissible c ascending, the order of the reference's k2 loop
                for (uint64_t m = hop_targets(in, a, b, K, false); m; m &= m - 1) {
                    const int c = __ffsll((long long)m) - 1, d = s - c;
                    const uint64_t out = rest | (1ull << c) | (1ull << d);
                    const uint64_t vb = hop_bits(hv, in, out, a, b, c, d);
                    if (hop_zero(vb)) continue;
                    const uint64_t j = rank_in_sector(out, hi, lo_tab, L);
                    if (j >= (uint64_t)n) continue;   // cannot happen for a sector word; never read out of range
                    acc = fma(bits_to_double(vb), __ldg(x + j), acc);
                }
            }
        }
        y[r] = acc;
    }
}

// The same product with the compact rank tables: the per-hop weights, the
// pair offsets and the 2^L-entry low-word table in shared memory, the
// high-word table read through L1 (neighbouring rows mostly share its entry).
// Same loops and FMA order as k_hv_matfree, so the same y.
__global__ void __launch_bounds__(1024) k_hv_matfree_c(const uint64_t* __restrict__ words, int64_t n,
                                                     const double* __restrict__ diag, const double* __restrict__ w,
                                                     int nw, const int* __restrict__ off, int K,
                                                     const uint64_t* __restrict__ mhi, const uint32_t* __restrict__ mlo,
                                                     int L, const double* __restrict__ x, double* __restrict__ y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double* sw = reinterpret_cast<double*>(smem);
    int* soff = reinterpret_cast<int*>(sw + nw);
    uint32_t* slo = reinterpret_cast<uint32_t*>(smem + matfree_c_table_offset(nw, K));
    for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = w[i];
    for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) soff[i] = off[i];
    for (int i = threadIdx.x; i < (1 << L); i += blockDim.x) slo[i] = mlo[i];
    __syncthreads();
    const uint64_t* wb = reinterpret_cast<const uint64_t*>(sw);
    const uint64_t lmask = (1ull << L) - 1ull;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        double acc = diag[r] * __ldg(x + r);
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const int s = a + b;
                const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                // per pair: the parity's (a,b) part and the hop-table bases of
                // the two directions (hop_parity, hop_index)
                const int lo = pair_lo(s, K), cnt = pair_cnt(s, K);
                const uint32_t par_ab = (uint32_t)(1 + __popcll(in & bits_between(a, b))) & 1u;
                const int ifwd = soff[s] + (a - lo) * cnt - lo;   // out > in: + c        (>= soff[s], c >= lo)
                const int irev = soff[s] + (a - lo) - lo * cnt;   // out < in: + c * cnt
                for (uint64_t m = hop_targets(in, a, b, K, false); m; m &= m - 1) {
                    const int c = __ffsll((long long)m) - 1, d = s - c;
                    const uint64_t bc = 1ull << c, bd = 1ull << d;
                    const uint64_t out = rest | bc | bd;
                    const uint32_t par = par_ab ^ ((uint32_t)__popcll(rest & (bd - 1ull) & ~(bc + bc - 1ull)) & 1u);
                    const uint64_t vb = wb[c < a ? ifwd + c : irev + c * cnt] ^ ((uint64_t)par << 63);   // c < a: out > in
                    if (hop_zero(vb)) continue;
                    const uint64_t eh = __ldg(mhi + (out >> L));
                    const uint32_t el = slo[out & lmask];
                    if ((eh >> 48) != (uint64_t)(el >> 16)) continue;   // cannot happen for a sector word
                    const uint64_t j = (eh & 0xFFFFFFFFFFFFull) + (el & 0xFFFFu);
                    if (j >= (uint64_t)n) continue;                      // never read out of range
                    acc = fma(bits_to_double(vb), __ldg(x + j), acc);
                }
            }
        }
        y[r] = acc;
    }
}

int sms()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

}  // namespace

void spmv(const ed_crs& a, const double* x, double* y, cudaStream_t st)
{
    if (a.n == 0) return;
    const double avg = a.n ? (double)a.nnz / (double)a.n : 0.0;
    const int threads = 256;
    const int grid = sms() * 8;
    if (!a.upper && avg >= 96) {
        k_spmv_full<8, 4><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
    } else if (!a.upper) {
        // rows of 24-96 elements (two-level sectors, small one-level ones):
        // four lanes per row with four loads ahead, or eight lanes per row
        // with three ahead once x passes about 20 MB (measured on GB300:
        // two-level N=7 sectors of 1.3-2.0M rows 4.3-4.6 TB/s with four lanes,
        // 3.5-3.7 with eight; N=8 sectors of 4.2-5.9M rows 4.3-4.4 TB/s with
        // eight and three ahead, 4.1 with four ahead, 2.9-3.0 with four lanes)
        if (avg >= 24 && a.n >= 2500000)
            k_spmv_full<8, 3><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
        else if (avg >= 24) k_spmv_full<4, 4><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
        else k_spmv_full<2><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
    } else {
        ED_CUDA(cudaMemsetAsync(y, 0, (size_t)a.n * sizeof(double), st));
        if (avg >= 48) k_spmv_upper<8><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
        else k_spmv_upper<4><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
    }
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void hv_matfree(const ed_basis& b, const ed_terms& t, const double* diag, const double* x, double* y, cudaStream_t st)
{
    ED_REQUIRE(b.levels == 1 && b.dimX == 0, ED_ERR_ARG, "the matrix-free product takes a one-level Lz basis");
    if (b.dim == 0) return;
    const int K = t.norb;
    const int nw = (int)t.hop.w.size();
    if (b.mf_lo.p) {
        const int L = b.mf_low_bits;
        const size_t smem = matfree_c_table_offset(nw, K) + ((size_t)4 << L);
        if (smem <= 200 * 1024) {
            // the limit is set on every call: a sector with a smaller table
            // may have lowered it since the last launch of this size
            ED_CUDA(cudaFuncSetAttribute(k_hv_matfree_c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int dev = 0;
            ED_CUDA(cudaGetDevice(&dev));
            // CTAs per SM per (device, shared-memory size)
            static thread_local std::map<std::pair<int, size_t>, int> occ;
            auto it = occ.find({dev, smem});
            if (it == occ.end()) {
                int ob = 0;
                ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, k_hv_matfree_c, 1024, smem));
                it = occ.emplace(std::make_pair(dev, smem), std::max(1, ob)).first;
            }
            k_hv_matfree_c<<<sms() * it->second, 1024, smem, st>>>(b.words.p, (int64_t)b.dim, diag, t.w_dev.p, nw,
                                                                   t.hop_off_dev.p, K, b.mf_hi.p, b.mf_lo.p, L, x, y);
            count_launch();
            ED_CUDA(cudaGetLastError());
            return;
        }
    }
    const size_t smem = hop_smem_bytes(K, nw);
    ED_CUDA(cudaFuncSetAttribute(k_hv_matfree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_hv_matfree<<<sms() * 4, 256, smem, st>>>(b.words.p, (int64_t)b.dim, diag, t.w_dev.p, nw, t.diag_a_dev.p,
                                                t.diag_b_dev.p, t.hop_off_dev.p, K, b.hi.p, b.lo.p, b.low_bits, x, y);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace edgb
