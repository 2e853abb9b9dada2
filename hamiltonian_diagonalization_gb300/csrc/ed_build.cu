// Quartic Hamiltonian build into CRS on the device (K3).
//
// The reference (hamiltonians/spinless_fermion_hamiltonian.hpp:282-436)
// visits, per row, every ordered (k4,k3) pair of occupied orbitals and every
// admissible (k2,k1), adds sign*V into a hash map keyed by (row, column)
// found by binary search, trims |x| < 1e-14, sorts into CRS.  Every
// off-diagonal element is a pair hop (a,b) -> (c,d) with a+b = c+d and
// receives exactly four ordered terms whose relative signs are fixed; the
// host folds them, in the reference's visiting order and with its filters,
// into one value per hop (derive_hop_tables), so the element is
// sign(state) * W[hop] bit for bit.  The diagonal is summed term by term in
// the reference order.  Rows are generated one warp per row, sorted by
// column in shared memory and written coalesced; a count pass sizes the
// rows first.
#include "ed_hop.cuh"

namespace edgb {

namespace {

__global__ void k_diag(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ da,
                       const double* __restrict__ db, int K, double* __restrict__ diag)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double* sda = reinterpret_cast<double*>(smem);
    double* sdb = sda + K * K;
    for (int i = threadIdx.x; i < K * K; i += blockDim.x) { sda[i] = da[i]; sdb[i] = db[i]; }
    __syncthreads();
    HopView hv{nullptr, sda, sdb, nullptr, K};
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        diag[r] = diag_element(hv, words[r]);
}

// Number of stored entries of each row (upper: col >= row; full: all).
__global__ void k_count(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag,
                        const double* __restrict__ w, int nw, const double* __restrict__ da,
                        const double* __restrict__ db, const int* __restrict__ off, int K, int upper,
                        int64_t* __restrict__ rowlen)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const HopView hv = load_hop_smem(smem, w, nw, da, db, off, K);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        int64_t cnt = (fabs(diag[r]) < kSparseZeroTol) ? 0 : 1;
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const int s = a + b;
                const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                const int lo = pair_lo(s, K), pc = pair_cnt(s, K);
                for (int ic = 0; ic < pc; ++ic) {
                    const int c = lo + ic, d = s - c;
                    if (c == a) continue;
                    if ((rest >> c) & 1ull) continue;
                    if ((rest >> d) & 1ull) continue;
                    const uint64_t out = rest | (1ull << c) | (1ull << d);
                    if (upper && out < in) continue;
                    if (hop_element(hv, in, out, a, b, c, d) != 0.0) ++cnt;
                }
            }
        }
        rowlen[r] = cnt;
    }
}

// One warp per row: generate (out word, value), sort by word, rank, store.
__global__ void k_fill(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag,
                       const double* __restrict__ w, int nw, const double* __restrict__ da,
                       const double* __restrict__ db, const int* __restrict__ off, int K, int N, int upper,
                       const int64_t* __restrict__ rowptr, const uint64_t* __restrict__ hi,
                       const uint64_t* __restrict__ lo_tab, int L, int cap, int32_t* __restrict__ col,
                       double* __restrict__ val, int* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const HopView hv = load_hop_smem(smem, w, nw, da, db, off, K);
    const size_t tbytes = (hop_smem_bytes(K, nw) + 15) & ~(size_t)15;
    const int warp_in_cta = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpc = blockDim.x >> 5;
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem + tbytes) + (size_t)warp_in_cta * cap;
    double* vals = reinterpret_cast<double*>(smem + tbytes + (size_t)wpc * cap * 8) + (size_t)warp_in_cta * cap;
    int* counter = reinterpret_cast<int*>(smem + tbytes + (size_t)wpc * cap * 16) + warp_in_cta;
    unsigned char* occ = reinterpret_cast<unsigned char*>(smem + tbytes + (size_t)wpc * cap * 16 + wpc * 4) +
                         (size_t)warp_in_cta * 64;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int npairs = N * (N - 1) / 2;
    for (int64_t r = gw; r < n; r += nwarps) {
        const uint64_t in = words[r];
        const int64_t base = rowptr[r];
        const int64_t want = rowptr[r + 1] - base;
        // positions of the occupied orbitals, ascending
        for (int pos0 = 0; pos0 < K; pos0 += 32) {
            const int pos = pos0 + lane;
            const bool set = pos < K && ((in >> pos) & 1ull);
            const unsigned m = __ballot_sync(0xffffffffu, set);
            if (set) {
                const int rk = __popc(m & ((1u << lane) - 1u)) + __popcll(in & ((1ull << pos0) - 1ull));
                occ[rk] = (unsigned char)pos;
            }
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
                if (c == a) continue;
                if ((rest >> c) & 1ull) continue;
                if ((rest >> d) & 1ull) continue;
                const uint64_t out = rest | (1ull << c) | (1ull << d);
                if (upper && out < in) continue;
                const double v = hop_element(hv, in, out, a, b, c, d);
                if (v == 0.0) continue;
                const int slot = atomicAdd(counter, 1);
                if (slot < cap) { keys[slot] = out; vals[slot] = v; }
            }
        }
        __syncwarp();
        if (lane == 0) {
            const double dv = diag[r];
            if (!(fabs(dv) < kSparseZeroTol)) {
                const int slot = atomicAdd(counter, 1);
                if (slot < cap) { keys[slot] = in; vals[slot] = dv; }
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
                        const double v0 = vals[i0];
                        vals[i0] = vals[i1];
                        vals[i1] = v0;
                    }
                }
                __syncwarp();
            }
        }
        for (int t = lane; t < cnt; t += 32) {
            const uint64_t c = rank_in_sector(keys[t], hi, lo_tab, L);
            if (c == kMiss) atomicOr(err, 2);
            col[base + t] = (int32_t)c;
            val[base + t] = vals[t];
        }
        __syncwarp();
    }
}

int sm_count()
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace

void ham_diagonal(const ed_basis& b, const ed_terms& t, double* diag, cudaStream_t st)
{
    if (b.dim == 0) return;
    const int K = t.norb;
    const size_t smem = (size_t)2 * K * K * 8;
    k_diag<<<sm_count() * 8, 256, smem, st>>>(b.words.p, (int64_t)b.dim, t.diag_a_dev.p, t.diag_b_dev.p, K, diag); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
}

void ham_build_crs(const ed_basis& b, const ed_terms& t, int upper, ed_crs& a, cudaStream_t st)
{
    ED_REQUIRE(t.norb == b.norb, ED_ERR_ARG, "terms and basis have different orbital counts");
    const int64_t n = (int64_t)b.dim;
    ED_REQUIRE(n < (int64_t)0x7fffffff, ED_ERR_RANGE, "sector dimension exceeds int32 column indices");
    a.n = n;
    a.upper = upper ? 1 : 0;
    a.rowptr.alloc(n + 1);
    if (n == 0) {
        ED_CUDA(cudaMemsetAsync(a.rowptr.p, 0, sizeof(int64_t), st));
        a.nnz = 0;
        return;
    }
    const int K = t.norb;
    const int nw = (int)t.hop.w.size();
    const size_t tsm = hop_smem_bytes(K, nw);
    DevBuf<double> diag(n);
    ham_diagonal(b, t, diag.p, st);
    DevBuf<int64_t> rowlen(n);
    ED_CUDA(cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    k_count<<<sm_count() * 4, 256, tsm, st>>>(b.words.p, n, diag.p, t.w_dev.p, nw, t.diag_a_dev.p, t.diag_b_dev.p,
                                              t.hop_off_dev.p, K, a.upper, rowlen.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(rowlen.p, a.rowptr.p, n, st);
    ED_CUDA(cudaMemcpyAsync(&a.nnz, a.rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    const int64_t maxrow = reduce_max_i64_host(rowlen.p, n, st);
    ED_CUDA(cudaStreamSynchronize(st));
    a.max_row = (int)maxrow;
    // kCrsPad zeroed elements past the end let the SpMV batches load
    // without bounds tests (column 0, value 0)
    a.col.alloc((size_t)a.nnz + kCrsPad);
    a.val.alloc((size_t)a.nnz + kCrsPad);
    ED_CUDA(cudaMemsetAsync(a.col.p + a.nnz, 0, kCrsPad * sizeof(int32_t), st));
    ED_CUDA(cudaMemsetAsync(a.val.p + a.nnz, 0, kCrsPad * sizeof(double), st));
    int cap = 32;
    while (cap < maxrow) cap <<= 1;
    const size_t tbytes = (tsm + 15) & ~(size_t)15;
    const size_t per_warp = (size_t)cap * 16 + 4 + 64;
    const size_t budget = 200 * 1024;
    ED_REQUIRE(tbytes + per_warp <= budget, ED_ERR_RANGE, "Hamiltonian rows too long for the shared-memory sort");
    int wpc = (int)((budget - tbytes) / per_warp);
    if (wpc > 16) wpc = 16;
    const size_t smem = tbytes + (size_t)wpc * per_warp;
    ED_CUDA(cudaFuncSetAttribute(k_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ_blocks = 0;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_blocks, k_fill, wpc * 32, smem));
    if (occ_blocks < 1) occ_blocks = 1;
    DevBuf<int> err(1);
    ED_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    k_fill<<<sm_count() * occ_blocks, wpc * 32, smem, st>>>(b.words.p, n, diag.p, t.w_dev.p, nw, t.diag_a_dev.p,
                                                             t.diag_b_dev.p, t.hop_off_dev.p, K, b.N, a.upper,
                                                             a.rowptr.p, b.hi.p, b.lo.p, b.low_bits, cap, a.col.p,
                                                             a.val.p, err.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    int herr = 0;
    ED_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_REQUIRE(herr == 0, ED_ERR_INTERNAL, "Hamiltonian fill: row count or rank check failed on the device");
}

}  // namespace edgb
