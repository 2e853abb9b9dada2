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
// column (in registers, k_fill_reg; in shared memory for rows or sectors too
// large for 32-bit keys, k_fill) and written coalesced; a count pass sizes
// the rows first.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

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

// Number of stored entries of each row (upper: col >= row; full: all), and
// the largest number of admissible hops of a row plus one (the diagonal
// slot), which sizes the register-sort fill's per-warp task list.  With
// nozero (no off-diagonal hop weight is zero) a row's count is the popcount
// of its pairs' target masks.
__global__ void k_count(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag,
                        const double* __restrict__ w, int nw, const double* __restrict__ da,
                        const double* __restrict__ db, const int* __restrict__ off, int K, int upper, int nozero,
                        int64_t* __restrict__ rowlen, int* __restrict__ maxtasks)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const HopView hv = load_hop_smem(smem, w, nw, da, db, off, K);
    unsigned tmax = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        int64_t cnt = (fabs(diag[r]) < kSparseZeroTol) ? 0 : 1;
        unsigned tasks = 1;
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const uint64_t m0 = hop_targets(in, a, b, K, upper != 0);
                const int pc = __popcll(m0);
                tasks += pc;
                if (nozero) {
                    cnt += pc;
                    continue;
                }
                const int s = a + b;
                const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                for (uint64_t m = m0; m; m &= m - 1) {
                    const int c = __ffsll((long long)m) - 1, d = s - c;
                    const uint64_t out = rest | (1ull << c) | (1ull << d);
                    if (!hop_zero(hop_bits(hv, in, out, a, b, c, d))) ++cnt;
                }
            }
        }
        rowlen[r] = cnt;
        tmax = tasks > tmax ? tasks : tmax;
    }
    tmax = __reduce_max_sync(0xffffffffu, tmax);
    if ((threadIdx.x & 31) == 0) atomicMax(maxtasks, (int)tmax);
}

// One warp per row: generate (out word, value), sort by word in shared
// memory, rank, store.  Any row length the shared memory holds, any sector.
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
                const uint64_t vb = hop_bits(hv, in, out, a, b, c, d);
                if (hop_zero(vb)) continue;
                const int slot = atomicAdd(counter, 1);
                if (slot < cap) { keys[slot] = out; vals[slot] = bits_to_double(vb); }
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

// ---------------------------------------------------------------------------
// k_fill_reg: the same rows, sorted in registers.  The admissible hops of
// each occupied pair (hop_targets) are expanded into a task list (a, b, c)
// in shared memory, so that every task yields an element unless its weight
// is zero, and the tasks are spread evenly over the lanes.  Each element is
// ranked as it is generated and stored as a 32-bit key (column << sb | slot),
// sb = log2(cap), with its value at vals[slot]; the host takes this kernel
// only when every key fits below 0xFFFFFFFF.  Slots follow the task order
// (one ballot per 32 tasks) and reuse the task list's storage: a slot never
// passes the task that fills it.  The keys, padded to 32*E with 0xFFFFFFFF,
// are sorted by a bitonic network over the element index lane*E + e:
// exchanges whose partner is nearer than E stay in one lane's registers, the
// rest take one shuffle.  The sorted keys go back through a swizzled
// shared-memory image (index i ^ ((i >> 5) & 31), conflict-free both ways)
// and are written coalesced.

constexpr int kFillMaxE = 32;   // 32 * 32 = 1024 elements per row at most

__host__ __device__ inline size_t fill_reg_warp_bytes(int cap)
{
    return ((size_t)cap * 12 + 64 + 15) & ~(size_t)15;
}

__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 5) & 31); }

template <int E>
__device__ __forceinline__ void sort_row_keys(uint32_t* keys, int cnt, int lane)
{
    uint32_t k[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int t = e * 32 + lane;
        k[e] = t < cnt ? keys[t] : 0xFFFFFFFFu;
    }
    __syncwarp();
#pragma unroll
    for (int kk = 2; kk <= 32 * E; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
            if (j >= E) {
                const int lj = j / E;
                const bool lower = (lane & lj) == 0;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const bool up = (((lane * E + e) & kk) == 0);
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, k[e], lj);
                    k[e] = (up == lower) ? min(k[e], o) : max(k[e], o);
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    if ((e & j) == 0) {
                        const bool up = (((lane * E + e) & kk) == 0);
                        const uint32_t x = k[e], y = k[e ^ j];
                        const uint32_t lo = min(x, y), hi = max(x, y);
                        k[e] = up ? lo : hi;
                        k[e ^ j] = up ? hi : lo;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) keys[swz(lane * E + e)] = k[e];
    __syncwarp();
}

// Sort with the smallest E (a power of two, at most EM) with 32*E >= cnt.
template <int E, int EM>
__device__ __forceinline__ void sort_row_dispatch(uint32_t* keys, int cnt, int lane)
{
    if constexpr (E < EM) {
        if (cnt > 32 * E) {
            sort_row_dispatch<E * 2, EM>(keys, cnt, lane);
            return;
        }
    }
    sort_row_keys<E>(keys, cnt, lane);
}

template <int EM>
__global__ void __launch_bounds__(256) k_fill_reg(
    const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag, const double* __restrict__ w,
    int nw, const double* __restrict__ da, const double* __restrict__ db, const int* __restrict__ off, int K, int N,
    int upper, const int64_t* __restrict__ rowptr, const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo_tab,
    int L, int cap, int sb, int32_t* __restrict__ col, double* __restrict__ val, int* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const HopView hv = load_hop_smem(smem, w, nw, da, db, off, K);
    const size_t tbytes = (hop_smem_bytes(K, nw) + 15) & ~(size_t)15;
    const int warp_in_cta = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int npairs = N * (N - 1) / 2;
    unsigned char* wbase = smem + tbytes + (size_t)warp_in_cta * fill_reg_warp_bytes(cap);
    double* vals = reinterpret_cast<double*>(wbase);
    uint32_t* keys = reinterpret_cast<uint32_t*>(wbase + (size_t)cap * 8);
    unsigned char* occ = wbase + (size_t)cap * 12;
    const uint32_t smask = (uint32_t)cap - 1u;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = gw; r < n; r += nwarps) {
        const uint64_t in = words[r];
        const int64_t base = rowptr[r];
        const int64_t want = rowptr[r + 1] - base;
        for (int pos0 = 0; pos0 < K; pos0 += 32) {
            const int pos = pos0 + lane;
            const bool set = pos < K && ((in >> pos) & 1ull);
            const unsigned m = __ballot_sync(0xffffffffu, set);
            if (set) occ[__popc(m & lt) + __popcll(in & ((1ull << pos0) - 1ull))] = (unsigned char)pos;
        }
        __syncwarp();
        // task list: the admissible (a, b, c) of every occupied pair
        int total = 0;
        for (int p0 = 0; p0 < npairs; p0 += 32) {
            const int p = p0 + lane;
            uint64_t m = 0;
            int a = 0, b = 0;
            if (p < npairs) {
                int j = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
                while (j * (j - 1) / 2 > p) --j;
                while ((j + 1) * j / 2 <= p) ++j;
                a = occ[p - j * (j - 1) / 2];
                b = occ[j];
                m = hop_targets(in, a, b, K, upper != 0);
            }
            const int pc = __popcll(m);
            int x = pc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            int pos = total + x - pc;
            for (; m; m &= m - 1, ++pos)
                if (pos < cap) keys[pos] = (uint32_t)(a | (b << 6) | ((__ffsll((long long)m) - 1) << 12));
            total += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        if (total >= cap) {   // the count pass sized cap above every row's tasks
            if (lane == 0) atomicOr(err, 4);
            __syncwarp();
            continue;
        }
        int cnt = 0;
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            const uint32_t task = t < total ? keys[t] : 0u;
            __syncwarp();
            uint32_t key = 0;
            uint64_t vb = 0;
            bool ok = false;
            if (t < total) {
                const int a = task & 63, b = (task >> 6) & 63, c = (task >> 12) & 63, d = a + b - c;
                const uint64_t out = in ^ (1ull << a) ^ (1ull << b) ^ (1ull << c) ^ (1ull << d);
                vb = hop_bits(hv, in, out, a, b, c, d);
                if (!hop_zero(vb)) {
                    const uint64_t rk = rank_in_sector(out, hi, lo_tab, L);
                    if (rk == kMiss) atomicOr(err, 2);
                    key = (uint32_t)rk << sb;
                    ok = true;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const int slot = cnt + __popc(m & lt);
                keys[slot] = key | (uint32_t)slot;
                vals[slot] = bits_to_double(vb);
            }
            cnt += __popc(m);
        }
        const double dv = diag[r];
        if (!(fabs(dv) < kSparseZeroTol)) {
            if (lane == 0 && cnt < cap) {
                keys[cnt] = ((uint32_t)r << sb) | (uint32_t)cnt;
                vals[cnt] = dv;
            }
            ++cnt;
        }
        __syncwarp();
        if (cnt != want || cnt > cap) {
            if (lane == 0) atomicOr(err, 1);
            __syncwarp();
            continue;
        }
        if (cnt > 0) sort_row_dispatch<1, EM>(keys, cnt, lane);
        for (int t = lane; t < cnt; t += 32) {
            const uint32_t kk = keys[swz(t)];
            col[base + t] = (int32_t)(kk >> sb);
            val[base + t] = vals[kk & smask];
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Two Landau levels: TwoLevelSpinlessFermionHamiltonian
// (two_level_spinless_fermion_hamiltonian.hpp:143-470) as
// SphereTwoLevelPseudopotentialModel::BuildHamiltonian calls it
// (two_level_pseudopotential_model.cpp:190-215).  A state is one word
// (first << n1) | second.  Every term acts within one level's word with the
// other as a spectator, so an off-diagonal element is a one-level pair hop on
// that word with that level's hop table; no cross-level sign arises (each of
// the four operators passes the other level's particles, an even total).  The
// diagonal is one running sum in the reference's call order: level-0
// energies, level-1 energies (occupied k ascending), then the level-0 and
// level-1 quartic diagonal terms.

// Shared-memory image of both levels' hop tables (level 0 first, 16-byte aligned).
__device__ __forceinline__ void load_two_level(unsigned char* smem, const double* w0, int nw0, const double* da0,
                                               const double* db0, const int* off0, int K0, const double* w1, int nw1,
                                               const double* da1, const double* db1, const int* off1, int K1,
                                               HopView& h0, HopView& h1)
{
    h0 = load_hop_smem(smem, w0, nw0, da0, db0, off0, K0);
    const size_t t0 = (hop_smem_bytes(K0, nw0) + 15) & ~(size_t)15;
    h1 = load_hop_smem(smem + t0, w1, nw1, da1, db1, off1, K1);
}

__host__ __device__ inline size_t two_level_table_bytes(int K0, int nw0, int K1, int nw1)
{
    return ((hop_smem_bytes(K0, nw0) + 15) & ~(size_t)15) + ((hop_smem_bytes(K1, nw1) + 15) & ~(size_t)15);
}

__global__ void k_diag2(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ e0,
                        const double* __restrict__ e1, const double* __restrict__ da0, const double* __restrict__ db0,
                        int K0, const double* __restrict__ da1, const double* __restrict__ db1, int K1,
                        double* __restrict__ diag)
{
    extern __shared__ __align__(16) unsigned char smem[];
    double* sda0 = reinterpret_cast<double*>(smem);
    double* sdb0 = sda0 + K0 * K0;
    double* sda1 = sdb0 + K0 * K0;
    double* sdb1 = sda1 + K1 * K1;
    double* se0 = sdb1 + K1 * K1;
    double* se1 = se0 + K0;
    for (int i = threadIdx.x; i < K0 * K0; i += blockDim.x) { sda0[i] = da0[i]; sdb0[i] = db0[i]; }
    for (int i = threadIdx.x; i < K1 * K1; i += blockDim.x) { sda1[i] = da1[i]; sdb1[i] = db1[i]; }
    for (int i = threadIdx.x; i < K0; i += blockDim.x) se0[i] = e0[i];
    for (int i = threadIdx.x; i < K1; i += blockDim.x) se1[i] = e1[i];
    __syncthreads();
    const HopView h0{nullptr, sda0, sdb0, nullptr, K0}, h1{nullptr, sda1, sdb1, nullptr, K1};
    const uint64_t m1 = (1ull << K1) - 1ull;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t w = words[r], first = w >> K1, second = w & m1;
        double acc = 0.0;
        for (uint64_t t = first; t; t &= t - 1) acc = acc + se0[__ffsll((long long)t) - 1];
        for (uint64_t t = second; t; t &= t - 1) acc = acc + se1[__ffsll((long long)t) - 1];
        acc = diag_element(h0, first, acc);
        diag[r] = diag_element(h1, second, acc);
    }
}

__global__ void k_count2(const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag,
                         const double* __restrict__ w0, int nw0, const double* __restrict__ da0,
                         const double* __restrict__ db0, const int* __restrict__ off0, int K0, int nozero0,
                         const double* __restrict__ w1, int nw1, const double* __restrict__ da1,
                         const double* __restrict__ db1, const int* __restrict__ off1, int K1, int nozero1, int upper,
                         int64_t* __restrict__ rowlen, int* __restrict__ maxtasks)
{
    extern __shared__ __align__(16) unsigned char smem[];
    HopView h0, h1;
    load_two_level(smem, w0, nw0, da0, db0, off0, K0, w1, nw1, da1, db1, off1, K1, h0, h1);
    const uint64_t m1 = (1ull << K1) - 1ull;
    unsigned tmax = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t w = words[r];
        int64_t cnt = (fabs(diag[r]) < kSparseZeroTol) ? 0 : 1;
        unsigned tasks = 1;
        for (int lvl = 0; lvl < 2; ++lvl) {
            const uint64_t in = lvl ? (w & m1) : (w >> K1);
            const HopView& hv = lvl ? h1 : h0;
            const int K = lvl ? K1 : K0;
            const bool nz = (lvl ? nozero1 : nozero0) != 0;
            for (uint64_t ta = in; ta; ta &= ta - 1) {
                const int a = __ffsll((long long)ta) - 1;
                for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                    const int b = __ffsll((long long)tb) - 1;
                    const uint64_t m0 = hop_targets(in, a, b, K, upper != 0);
                    const int pc = __popcll(m0);
                    tasks += pc;
                    if (nz) {
                        cnt += pc;
                        continue;
                    }
                    const int s = a + b;
                    const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
                    for (uint64_t m = m0; m; m &= m - 1) {
                        const int c = __ffsll((long long)m) - 1, d = s - c;
                        if (!hop_zero(hop_bits(hv, in, rest | (1ull << c) | (1ull << d), a, b, c, d))) ++cnt;
                    }
                }
            }
        }
        rowlen[r] = cnt;
        tmax = tasks > tmax ? tasks : tmax;
    }
    tmax = __reduce_max_sync(0xffffffffu, tmax);
    if ((threadIdx.x & 31) == 0) atomicMax(maxtasks, (int)tmax);
}

// One warp per row of the two-level Hamiltonian: the admissible hops of every
// same-level occupied pair as tasks (level << 18 | a | b << 6 | c << 12, level
// positions), ranked as generated, register-sorted and stored as k_fill_reg does.
template <int EM>
__global__ void __launch_bounds__(256) k_fill2(
    const uint64_t* __restrict__ words, int64_t n, const double* __restrict__ diag, const double* __restrict__ w0,
    int nw0, const double* __restrict__ da0, const double* __restrict__ db0, const int* __restrict__ off0, int K0,
    const double* __restrict__ w1, int nw1, const double* __restrict__ da1, const double* __restrict__ db1,
    const int* __restrict__ off1, int K1, int N, int upper, const int64_t* __restrict__ rowptr,
    const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo_tab, int L, int cap, int sb,
    int32_t* __restrict__ col, double* __restrict__ val, int* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    HopView h0, h1;
    load_two_level(smem, w0, nw0, da0, db0, off0, K0, w1, nw1, da1, db1, off1, K1, h0, h1);
    const size_t tbytes = two_level_table_bytes(K0, nw0, K1, nw1);
    const int warp_in_cta = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int npairs = N * (N - 1) / 2;
    const int K = K0 + K1;
    unsigned char* wbase = smem + tbytes + (size_t)warp_in_cta * fill_reg_warp_bytes(cap);
    double* vals = reinterpret_cast<double*>(wbase);
    uint32_t* keys = reinterpret_cast<uint32_t*>(wbase + (size_t)cap * 8);
    unsigned char* occ = wbase + (size_t)cap * 12;
    const uint32_t smask = (uint32_t)cap - 1u;
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t m1 = (1ull << K1) - 1ull;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = gw; r < n; r += nwarps) {
        const uint64_t in = words[r], first = in >> K1, second = in & m1;
        const int64_t base = rowptr[r];
        const int64_t want = rowptr[r + 1] - base;
        for (int pos0 = 0; pos0 < K; pos0 += 32) {
            const int pos = pos0 + lane;
            const bool set = pos < K && ((in >> pos) & 1ull);
            const unsigned m = __ballot_sync(0xffffffffu, set);
            if (set) occ[__popc(m & lt) + __popcll(in & ((1ull << pos0) - 1ull))] = (unsigned char)pos;
        }
        __syncwarp();
        int total = 0;
        for (int p0 = 0; p0 < npairs; p0 += 32) {
            const int p = p0 + lane;
            uint64_t m = 0;
            uint32_t tag = 0;
            if (p < npairs) {
                int j = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
                while (j * (j - 1) / 2 > p) --j;
                while ((j + 1) * j / 2 <= p) ++j;
                const int a = occ[p - j * (j - 1) / 2], b = occ[j];
                if (b < K1) {                           // both in level 1 (the low word)
                    m = hop_targets(second, a, b, K1, upper != 0);
                    tag = (1u << 18) | (uint32_t)a | ((uint32_t)b << 6);
                } else if (a >= K1) {                   // both in level 0
                    m = hop_targets(first, a - K1, b - K1, K0, upper != 0);
                    tag = (uint32_t)(a - K1) | ((uint32_t)(b - K1) << 6);
                }
            }
            const int pc = __popcll(m);
            int x = pc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            int pos = total + x - pc;
            for (; m; m &= m - 1, ++pos)
                if (pos < cap) keys[pos] = tag | ((uint32_t)(__ffsll((long long)m) - 1) << 12);
            total += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        if (total >= cap) {
            if (lane == 0) atomicOr(err, 4);
            __syncwarp();
            continue;
        }
        int cnt = 0;
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            const uint32_t task = t < total ? keys[t] : 0u;
            __syncwarp();
            uint32_t key = 0;
            uint64_t vb = 0;
            bool ok = false;
            if (t < total) {
                const int lvl1 = (task >> 18) & 1;
                const int a = task & 63, b = (task >> 6) & 63, c = (task >> 12) & 63, d = a + b - c;
                const uint64_t sub = lvl1 ? second : first;
                const uint64_t out_sub = sub ^ (1ull << a) ^ (1ull << b) ^ (1ull << c) ^ (1ull << d);
                vb = hop_bits(lvl1 ? h1 : h0, sub, out_sub, a, b, c, d);
                if (!hop_zero(vb)) {
                    const uint64_t out = lvl1 ? ((first << K1) | out_sub) : ((out_sub << K1) | second);
                    const uint64_t rk = rank_in_sector(out, hi, lo_tab, L);
                    if (rk == kMiss) atomicOr(err, 2);
                    key = (uint32_t)rk << sb;
                    ok = true;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const int slot = cnt + __popc(m & lt);
                keys[slot] = key | (uint32_t)slot;
                vals[slot] = bits_to_double(vb);
            }
            cnt += __popc(m);
        }
        const double dv = diag[r];
        if (!(fabs(dv) < kSparseZeroTol)) {
            if (lane == 0 && cnt < cap) {
                keys[cnt] = ((uint32_t)r << sb) | (uint32_t)cnt;
                vals[cnt] = dv;
            }
            ++cnt;
        }
        __syncwarp();
        if (cnt != want || cnt > cap) {
            if (lane == 0) atomicOr(err, 1);
            __syncwarp();
            continue;
        }
        if (cnt > 0) sort_row_dispatch<1, EM>(keys, cnt, lane);
        for (int t = lane; t < cnt; t += 32) {
            const uint32_t kk = keys[swz(t)];
            col[base + t] = (int32_t)(kk >> sb);
            val[base + t] = vals[kk & smask];
        }
        __syncwarp();
    }
}

// Level-exchange ladder of the two-level basis: y += T x with T = L0- L1+
// (dir > 0: one level-0 particle one orbital down, one level-1 particle one
// up, total Lz unchanged) or its adjoint T^+ = L0+ L1- (dir < 0), the
// angular-momentum ladder coefficients sqrt((S+m)(S-m+1)) of each level; a
// particle moving to a neighbouring empty orbital passes nobody, so no sign.
// The levels do not mix, so T commutes with the two-level Hamiltonian.
__global__ void k_ladder2(const uint64_t* __restrict__ words, int64_t n, int K0, int K1, int dir,
                          const uint64_t* __restrict__ hi, const uint64_t* __restrict__ lo_tab, int L,
                          const double* __restrict__ x, double* __restrict__ y)
{
    const uint64_t m1 = (1ull << K1) - 1ull;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const double xr = x[r];
        if (xr == 0.0) continue;
        const uint64_t w = words[r], first = w >> K1, second = w & m1;
        for (uint64_t ti = first; ti; ti &= ti - 1) {
            const int i = __ffsll((long long)ti) - 1, i2 = dir > 0 ? i - 1 : i + 1;
            if (i2 < 0 || i2 >= K0 || ((first >> i2) & 1ull)) continue;
            const double c0 = dir > 0 ? sqrt((double)i * (double)(K0 - i)) : sqrt((double)(i + 1) * (double)(K0 - 1 - i));
            const uint64_t f2 = first ^ (1ull << i) ^ (1ull << i2);
            for (uint64_t tj = second; tj; tj &= tj - 1) {
                const int j = __ffsll((long long)tj) - 1, j2 = dir > 0 ? j + 1 : j - 1;
                if (j2 < 0 || j2 >= K1 || ((second >> j2) & 1ull)) continue;
                const double c1 =
                    dir > 0 ? sqrt((double)(K1 - 1 - j) * (double)(j + 1)) : sqrt((double)j * (double)(K1 - j));
                const uint64_t out = (f2 << K1) | (second ^ (1ull << j) ^ (1ull << j2));
                const uint64_t rk = rank_in_sector(out, hi, lo_tab, L);
                if (rk != kMiss) atomicAdd(y + rk, c0 * c1 * xr);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Complex momentum-conserving build: SpinlessFermionHamiltonian<dcmplx>
// Add_CdC_Terms / Add_CdCdCC_Terms (spinless_fermion_hamiltonian.hpp:150-436)
// as InteractingOflModel::BuildHamiltonian calls them with array-format
// tables (interacting_ofl_model.cpp:1034-1052).  As in the one-level build,
// an off-diagonal element is a pair hop (a,b) -> (c,d), here within one
// momentum class, worth sign(state) * W[hop] with the same parity rule; the
// stored (upper) element of row `in` is <out|H|in>, and a lower element of the
// full storage is the conjugate of the upper element it mirrors,
// sign * conj(W[reverse hop]).  The diagonal sums the occupation energies,
// then the quartic diagonal terms, in the reference's order.

struct CView {
    const int* cls_off;
    const uint16_t* pairs;
    const int* pidx;
    const int* w_off;
    const double2* w;
    const double2* da;
    const double2* db;
    const double2* e;
    int K, X, Y;
};

__device__ __forceinline__ int pair_class(int a, int b, int X, int Y)
{
    return ((a / Y + b / Y) % X) * Y + (a % Y + b % Y) % Y;
}

__device__ __forceinline__ bool czero(double2 v)
{
    return ((__double_as_longlong(v.x) << 1) | (__double_as_longlong(v.y) << 1)) == 0;
}

__device__ __forceinline__ double2 cdiag_element(const CView& v, uint64_t in)
{
    double2 acc = make_double2(0.0, 0.0);
    for (uint64_t t = in; t; t &= t - 1) {
        const double2 e = __ldg(v.e + (__ffsll((long long)t) - 1));
        acc.x = acc.x + e.x;
        acc.y = acc.y + e.y;
    }
    for (uint64_t t4 = in; t4; t4 &= t4 - 1) {
        const int k4 = __ffsll((long long)t4) - 1;
        for (uint64_t t3 = in & ~(1ull << k4); t3; t3 &= t3 - 1) {
            const int k3 = __ffsll((long long)t3) - 1;
            const double2 p = __ldg(v.da + k4 * v.K + k3), q = __ldg(v.db + k4 * v.K + k3);
            acc.x = acc.x + p.x;
            acc.y = acc.y + p.y;
            acc.x = acc.x + q.x;
            acc.y = acc.y + q.y;
        }
    }
    return acc;
}

// Weight of the hop (a,b) -> (c,d) of class P as stored in row `in`: the
// upper element (d > b) or the conjugate of the mirrored upper one.
// Negation as a sign-bit flip on the integer pipe (the FP64 pipe is the
// scarce one on this part); identical to IEEE negation for every input.
__device__ __forceinline__ double flip_sign(double x)
{
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

__device__ __forceinline__ double2 chop_weight(const CView& v, int P, int ia, int ic, int cnt, bool upper_el)
{
    const int o = __ldg(v.w_off + P);
    if (upper_el) return __ldg(v.w + o + ia * cnt + ic);
    const double2 r = __ldg(v.w + o + ic * cnt + ia);
    return make_double2(r.x, flip_sign(r.y));
}

__global__ void k_cdiag(const uint64_t* __restrict__ words, int64_t n, CView v, double2* __restrict__ diag)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        diag[r] = cdiag_element(v, words[r]);
}

__global__ void k_ccount(const uint64_t* __restrict__ words, int64_t n, const double2* __restrict__ diag, CView v,
                         int upper, int64_t* __restrict__ rowlen, int* __restrict__ maxtasks)
{
    unsigned tmax = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t in = words[r];
        const double2 dg = diag[r];
        int64_t cnt = hypot(dg.x, dg.y) < kSparseZeroTol ? 0 : 1;
        unsigned tasks = 1;
        for (uint64_t ta = in; ta; ta &= ta - 1) {
            const int a = __ffsll((long long)ta) - 1;
            for (uint64_t tb = ta & (ta - 1); tb; tb &= tb - 1) {
                const int b = __ffsll((long long)tb) - 1;
                const int P = pair_class(a, b, v.X, v.Y);
                const int base = __ldg(v.cls_off + P), m = __ldg(v.cls_off + P + 1) - base;
                const int ia = __ldg(v.pidx + a * v.K + b);
                for (int ic = 0; ic < m; ++ic) {
                    const int pr = __ldg(v.pairs + base + ic), c = pr & 255, d = pr >> 8;
                    if (((in >> c) | (in >> d)) & 1ull) continue;
                    if (upper && d < b) continue;
                    ++tasks;
                    if (!czero(chop_weight(v, P, ia, ic, m, d > b))) ++cnt;
                }
            }
        }
        rowlen[r] = cnt;
        tmax = tasks > tmax ? tasks : tmax;
    }
    tmax = __reduce_max_sync(0xffffffffu, tmax);
    if ((threadIdx.x & 31) == 0) atomicMax(maxtasks, (int)tmax);
}

__host__ __device__ inline size_t cfill_warp_bytes(int cap)
{
    return ((size_t)cap * 20 + 16 + 15) & ~(size_t)15;
}

// One warp per row: the lanes take the occupied pairs, append every nonzero
// hop as (rank << sb | slot) with its complex value, the register sort orders
// the row by column, and the row is written coalesced.
template <int EM>
__global__ void __launch_bounds__(256) k_cfill(const uint64_t* __restrict__ words, int64_t n,
                                               const double2* __restrict__ diag, CView v, int N, int upper,
                                               const int64_t* __restrict__ rowptr, const uint64_t* __restrict__ hi,
                                               const uint64_t* __restrict__ lo_tab, int L, int cap, int sb,
                                               int32_t* __restrict__ col, double2* __restrict__ val,
                                               int* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp_in_cta = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + (size_t)warp_in_cta * cfill_warp_bytes(cap);
    double2* vals = reinterpret_cast<double2*>(wbase);
    uint32_t* keys = reinterpret_cast<uint32_t*>(wbase + (size_t)cap * 16);
    int* counter = reinterpret_cast<int*>(wbase + (size_t)cap * 20);
    const uint32_t smask = (uint32_t)cap - 1u;
    const int npairs = N * (N - 1) / 2;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = gw; r < n; r += nwarps) {
        const uint64_t in = words[r];
        const int64_t base = rowptr[r];
        const int64_t want = rowptr[r + 1] - base;
        if (lane == 0) *counter = 0;
        __syncwarp();
        for (int p = lane; p < npairs; p += 32) {
            // the p-th occupied pair (i < j in occupied order)
            int j = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
            while (j * (j - 1) / 2 > p) --j;
            while ((j + 1) * j / 2 <= p) ++j;
            const int i = p - j * (j - 1) / 2;
            uint64_t t = in;
            for (int q = 0; q < i; ++q) t &= t - 1;
            const int a = __ffsll((long long)t) - 1;
            for (int q = i; q < j; ++q) t &= t - 1;
            const int b = __ffsll((long long)t) - 1;
            const int P = pair_class(a, b, v.X, v.Y);
            const int cb = __ldg(v.cls_off + P), m = __ldg(v.cls_off + P + 1) - cb;
            const int ia = __ldg(v.pidx + a * v.K + b);
            const uint64_t rest = in ^ (1ull << a) ^ (1ull << b);
            for (int ic = 0; ic < m; ++ic) {
                const int pr = __ldg(v.pairs + cb + ic), c = pr & 255, d = pr >> 8;
                if (((in >> c) | (in >> d)) & 1ull) continue;
                if (upper && d < b) continue;
                double2 w = chop_weight(v, P, ia, ic, m, d > b);
                if (czero(w)) continue;
                if (hop_parity(in, a, b, c, d)) w = make_double2(flip_sign(w.x), flip_sign(w.y));
                const uint64_t out = rest | (1ull << c) | (1ull << d);
                const uint64_t rk = rank_in_sector(out, hi, lo_tab, L);
                if (rk == kMiss) atomicOr(err, 2);
                const int slot = atomicAdd(counter, 1);
                if (slot < cap) {
                    keys[slot] = ((uint32_t)rk << sb) | (uint32_t)slot;
                    vals[slot] = w;
                }
            }
        }
        __syncwarp();
        int cnt = *counter;
        const double2 dv = diag[r];
        if (!(hypot(dv.x, dv.y) < kSparseZeroTol)) {
            if (lane == 0 && cnt < cap) {
                keys[cnt] = ((uint32_t)r << sb) | (uint32_t)cnt;
                vals[cnt] = dv;
            }
            ++cnt;
        }
        __syncwarp();
        if (cnt != want || cnt > cap) {
            if (lane == 0) atomicOr(err, 1);
            __syncwarp();
            continue;
        }
        if (cnt > 0) sort_row_dispatch<1, EM>(keys, cnt, lane);
        for (int t2 = lane; t2 < cnt; t2 += 32) {
            const uint32_t kk = keys[swz(t2)];
            col[base + t2] = (int32_t)(kk >> sb);
            val[base + t2] = vals[kk & smask];
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
    ED_REQUIRE(b.levels == 1, ED_ERR_ARG, "a two-level basis takes the two-level Hamiltonian build");
    ED_REQUIRE(b.dimX == 0, ED_ERR_ARG, "a momentum basis takes the complex momentum-conserving build");
    if (b.dim == 0) return;
    const int K = t.norb;
    const size_t smem = (size_t)2 * K * K * 8;
    k_diag<<<sm_count() * 8, 256, smem, st>>>(b.words.p, (int64_t)b.dim, t.diag_a_dev.p, t.diag_b_dev.p, K, diag); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
}

void ham_build_crs(const ed_basis& b, const ed_terms& t, int upper, ed_crs& a, cudaStream_t st)
{
    ED_REQUIRE(b.levels == 1, ED_ERR_ARG, "a two-level basis takes the two-level Hamiltonian build");
    ED_REQUIRE(b.dimX == 0, ED_ERR_ARG, "a momentum basis takes the complex momentum-conserving build");
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
    // with no zero off-diagonal weight every admissible hop is stored
    int nozero = 1;
    for (int s = 1; s <= 2 * K - 3 && nozero; ++s) {
        const int cnt = pair_cnt(s, K);
        for (int ia = 0; ia < cnt && nozero; ++ia)
            for (int ic = 0; ic < cnt; ++ic)
                if (ic != ia && t.hop.w[t.hop.hop_off[s] + ia * cnt + ic] == 0.0) { nozero = 0; break; }
    }
    DevBuf<int> maxtasks_dev(1);
    ED_CUDA(cudaMemsetAsync(maxtasks_dev.p, 0, sizeof(int), st));
    ED_CUDA(cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    k_count<<<sm_count() * 4, 256, tsm, st>>>(b.words.p, n, diag.p, t.w_dev.p, nw, t.diag_a_dev.p, t.diag_b_dev.p,
                                              t.hop_off_dev.p, K, a.upper, nozero, rowlen.p, maxtasks_dev.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(rowlen.p, a.rowptr.p, n, st);
    ED_CUDA(cudaMemcpyAsync(&a.nnz, a.rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    int maxtasks = 0;
    ED_CUDA(cudaMemcpyAsync(&maxtasks, maxtasks_dev.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    const int64_t maxrow = reduce_max_i64_host(rowlen.p, n, st);
    ED_CUDA(cudaStreamSynchronize(st));
    a.max_row = (int)maxrow;
    // kCrsPad zeroed elements past the end let the SpMV batches load
    // without bounds tests (column 0, value 0)
    a.col.alloc((size_t)a.nnz + kCrsPad);
    a.val.alloc((size_t)a.nnz + kCrsPad);
    ED_CUDA(cudaMemsetAsync(a.col.p + a.nnz, 0, kCrsPad * sizeof(int32_t), st));
    ED_CUDA(cudaMemsetAsync(a.val.p + a.nnz, 0, kCrsPad * sizeof(double), st));
    int cap = 32, sb = 5;
    while (cap < maxrow) { cap <<= 1; ++sb; }
    const size_t tbytes = (tsm + 15) & ~(size_t)15;
    const size_t budget = 200 * 1024;
    DevBuf<int> err(1);
    ED_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    // register sort when a row's tasks and elements fit 32*kFillMaxE keys of
    // (column << rsb | slot) below 0xFFFFFFFF; ED_FILL_SORT=smem selects the
    // shared-memory sort for every sector
    int rcap = 32, rsb = 5;
    while (rcap < std::max<int64_t>(maxrow, maxtasks + 1)) { rcap <<= 1; ++rsb; }
    const size_t reg_warp = fill_reg_warp_bytes(rcap);
    const char* sort_env = std::getenv("ED_FILL_SORT");
    const bool force_smem = sort_env && std::strcmp(sort_env, "smem") == 0;
    if (!force_smem && rcap <= 32 * kFillMaxE &&
        ((((uint64_t)(n - 1)) << rsb) | (uint64_t)(rcap - 1)) < 0xFFFFFFFFull && tbytes + reg_warp <= budget) {
        const int smax = std::min<int>(8, (int)((budget - tbytes) / reg_warp));
        auto launch = [&](auto kern) {
            // warps per CTA: the most resident warps per SM, then the larger CTA
            int wpc = smax, best = 0, occ_best = 1;
            for (int c = smax; c >= 1; --c) {
                const size_t sm_c = tbytes + (size_t)c * reg_warp;
                ED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_c));
                int ob = 0;
                ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, kern, c * 32, sm_c));
                if (ob * c > best) { best = ob * c; wpc = c; occ_best = ob < 1 ? 1 : ob; }
            }
            const size_t smem = tbytes + (size_t)wpc * reg_warp;
            ED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<sm_count() * occ_best, wpc * 32, smem, st>>>(
                b.words.p, n, diag.p, t.w_dev.p, nw, t.diag_a_dev.p, t.diag_b_dev.p, t.hop_off_dev.p, K, b.N,
                a.upper, a.rowptr.p, b.hi.p, b.lo.p, b.low_bits, rcap, rsb, a.col.p, a.val.p, err.p);
            ::edgb::count_launch();
        };
        if (rcap <= 128) launch(k_fill_reg<4>);
        else if (rcap <= 512) launch(k_fill_reg<16>);
        else launch(k_fill_reg<32>);
        ED_CUDA(cudaGetLastError());
        int herr = 0;
        ED_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        ED_REQUIRE(herr == 0, ED_ERR_INTERNAL, "Hamiltonian fill: row count or rank check failed on the device");
        return;
    }
    const size_t per_warp = (size_t)cap * 16 + 4 + 64;
    ED_REQUIRE(tbytes + per_warp <= budget, ED_ERR_RANGE, "Hamiltonian rows too long for the shared-memory sort");
    int wpc = (int)((budget - tbytes) / per_warp);
    if (wpc > 16) wpc = 16;
    const size_t smem = tbytes + (size_t)wpc * per_warp;
    ED_CUDA(cudaFuncSetAttribute(k_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ_blocks = 0;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_blocks, k_fill, wpc * 32, smem));
    if (occ_blocks < 1) occ_blocks = 1;
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

namespace {
bool all_hops_nonzero(const ed_terms& t)
{
    const int K = t.norb;
    for (int s = 1; s <= 2 * K - 3; ++s) {
        const int cnt = pair_cnt(s, K);
        for (int ia = 0; ia < cnt; ++ia)
            for (int ic = 0; ic < cnt; ++ic)
                if (ic != ia && t.hop.w[t.hop.hop_off[s] + ia * cnt + ic] == 0.0) return false;
    }
    return true;
}
}  // namespace

void ham2_build_crs(const ed_basis& b, const ed_terms& t0, const ed_terms& t1, const double* e0_host,
                    const double* e1_host, int upper, ed_crs& a, cudaStream_t st)
{
    ED_REQUIRE(b.levels == 2, ED_ERR_ARG, "the two-level build takes a two-level basis");
    ED_REQUIRE(t0.norb == b.norb0 && t1.norb == b.norb1, ED_ERR_ARG,
               "term tables must have norb0 (level 0) and norb0 + 2 (level 1) orbitals");
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
    const int K0 = t0.norb, K1 = t1.norb;
    const int nw0 = (int)t0.hop.w.size(), nw1 = (int)t1.hop.w.size();
    // occupation energies with the reference's per-term filter (|E| > 1e-14)
    std::vector<double> e0(K0, 0.0), e1(K1, 0.0);
    for (int k = 0; k < K0; ++k)
        if (e0_host && std::fabs(e0_host[k]) > kSparseZeroTol) e0[k] = e0_host[k];
    for (int k = 0; k < K1; ++k)
        if (e1_host && std::fabs(e1_host[k]) > kSparseZeroTol) e1[k] = e1_host[k];
    DevBuf<double> de0(K0), de1(K1);
    ED_CUDA(cudaMemcpyAsync(de0.p, e0.data(), K0 * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(de1.p, e1.data(), K1 * 8, cudaMemcpyHostToDevice, st));
    DevBuf<double> diag(n);
    const size_t dsm = ((size_t)2 * K0 * K0 + (size_t)2 * K1 * K1 + K0 + K1) * 8;
    k_diag2<<<sm_count() * 8, 256, dsm, st>>>(b.words.p, n, de0.p, de1.p, t0.diag_a_dev.p, t0.diag_b_dev.p, K0,
                                             t1.diag_a_dev.p, t1.diag_b_dev.p, K1, diag.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    const size_t tsm = two_level_table_bytes(K0, nw0, K1, nw1);
    DevBuf<int64_t> rowlen(n);
    DevBuf<int> maxtasks_dev(1);
    ED_CUDA(cudaMemsetAsync(maxtasks_dev.p, 0, sizeof(int), st));
    ED_CUDA(cudaFuncSetAttribute(k_count2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    k_count2<<<sm_count() * 4, 256, tsm, st>>>(b.words.p, n, diag.p, t0.w_dev.p, nw0, t0.diag_a_dev.p,
                                               t0.diag_b_dev.p, t0.hop_off_dev.p, K0, all_hops_nonzero(t0) ? 1 : 0,
                                               t1.w_dev.p, nw1, t1.diag_a_dev.p, t1.diag_b_dev.p, t1.hop_off_dev.p, K1,
                                               all_hops_nonzero(t1) ? 1 : 0, a.upper, rowlen.p, maxtasks_dev.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(rowlen.p, a.rowptr.p, n, st);
    ED_CUDA(cudaMemcpyAsync(&a.nnz, a.rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    int maxtasks = 0;
    ED_CUDA(cudaMemcpyAsync(&maxtasks, maxtasks_dev.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    const int64_t maxrow = reduce_max_i64_host(rowlen.p, n, st);
    ED_CUDA(cudaStreamSynchronize(st));
    a.max_row = (int)maxrow;
    a.col.alloc((size_t)a.nnz + kCrsPad);
    a.val.alloc((size_t)a.nnz + kCrsPad);
    ED_CUDA(cudaMemsetAsync(a.col.p + a.nnz, 0, kCrsPad * sizeof(int32_t), st));
    ED_CUDA(cudaMemsetAsync(a.val.p + a.nnz, 0, kCrsPad * sizeof(double), st));
    int cap = 32, sb = 5;
    while (cap < std::max<int64_t>(maxrow, maxtasks + 1)) { cap <<= 1; ++sb; }
    const size_t tbytes = tsm;
    const size_t warp_b = fill_reg_warp_bytes(cap);
    const size_t budget = 200 * 1024;
    ED_REQUIRE(cap <= 32 * kFillMaxE && ((((uint64_t)(n - 1)) << sb) | (uint64_t)(cap - 1)) < 0xFFFFFFFFull &&
                   tbytes + warp_b <= budget,
               ED_ERR_RANGE, "two-level sector too large for the register-sort fill");
    DevBuf<int> err(1);
    ED_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    const int wpc = std::min<int>(8, (int)((budget - tbytes) / warp_b));
    const size_t smem = tbytes + (size_t)wpc * warp_b;
    auto launch = [&](auto kern) {
        ED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int ob = 0;
        ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, kern, wpc * 32, smem));
        kern<<<sm_count() * std::max(1, ob), wpc * 32, smem, st>>>(
            b.words.p, n, diag.p, t0.w_dev.p, nw0, t0.diag_a_dev.p, t0.diag_b_dev.p, t0.hop_off_dev.p, K0, t1.w_dev.p,
            nw1, t1.diag_a_dev.p, t1.diag_b_dev.p, t1.hop_off_dev.p, K1, b.N, a.upper, a.rowptr.p, b.hi.p, b.lo.p,
            b.low_bits, cap, sb, a.col.p, a.val.p, err.p);
        ::edgb::count_launch();
    };
    if (cap <= 128) launch(k_fill2<4>);
    else if (cap <= 512) launch(k_fill2<16>);
    else launch(k_fill2<32>);
    ED_CUDA(cudaGetLastError());
    int herr = 0;
    ED_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_REQUIRE(herr == 0, ED_ERR_INTERNAL, "two-level fill: row count or rank check failed on the device");
}

void cham_build_crs(const ed_basis& b, const ed_cterms& t, int upper, ed_ccrs& a, cudaStream_t st)
{
    ED_REQUIRE(b.dimX > 0, ED_ERR_ARG, "the complex build takes a momentum basis");
    ED_REQUIRE(t.norb == b.norb && t.dimX == b.dimX && t.dimY == b.dimY, ED_ERR_ARG,
               "terms and basis have different momentum grids");
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
    CView v{t.cls_off_dev.p, t.pairs_dev.p, t.pair_index_dev.p, t.w_off_dev.p,
            reinterpret_cast<const double2*>(t.w_dev.p), reinterpret_cast<const double2*>(t.da_dev.p),
            reinterpret_cast<const double2*>(t.db_dev.p), reinterpret_cast<const double2*>(t.e_dev.p), t.norb,
            t.dimX, t.dimY};
    DevBuf<double2> diag(n);
    k_cdiag<<<sm_count() * 8, 256, 0, st>>>(b.words.p, n, v, diag.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    DevBuf<int64_t> rowlen(n);
    DevBuf<int> maxtasks_dev(1);
    ED_CUDA(cudaMemsetAsync(maxtasks_dev.p, 0, sizeof(int), st));
    k_ccount<<<sm_count() * 4, 256, 0, st>>>(b.words.p, n, diag.p, v, a.upper, rowlen.p, maxtasks_dev.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    exclusive_scan_i64(rowlen.p, a.rowptr.p, n, st);
    ED_CUDA(cudaMemcpyAsync(&a.nnz, a.rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    int maxtasks = 0;
    ED_CUDA(cudaMemcpyAsync(&maxtasks, maxtasks_dev.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    const int64_t maxrow = reduce_max_i64_host(rowlen.p, n, st);
    ED_CUDA(cudaStreamSynchronize(st));
    a.max_row = (int)maxrow;
    a.col.alloc((size_t)a.nnz + kCrsPad);
    a.val.alloc(2 * ((size_t)a.nnz + kCrsPad));
    ED_CUDA(cudaMemsetAsync(a.col.p + a.nnz, 0, kCrsPad * sizeof(int32_t), st));
    ED_CUDA(cudaMemsetAsync(a.val.p + 2 * a.nnz, 0, 2 * kCrsPad * sizeof(double), st));
    int cap = 32, sb = 5;
    while (cap < std::max<int64_t>(maxrow, maxtasks + 1)) { cap <<= 1; ++sb; }
    const size_t warp_b = cfill_warp_bytes(cap);
    const size_t budget = 200 * 1024;
    ED_REQUIRE(cap <= 32 * kFillMaxE && ((((uint64_t)(n - 1)) << sb) | (uint64_t)(cap - 1)) < 0xFFFFFFFFull &&
                   warp_b <= budget,
               ED_ERR_RANGE, "momentum sector too large for the register-sort fill");
    DevBuf<int> err(1);
    ED_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    const int wpc = std::min<int>(8, (int)(budget / warp_b));
    const size_t smem = (size_t)wpc * warp_b;
    auto launch = [&](auto kern) {
        ED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int ob = 0;
        ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, kern, wpc * 32, smem));
        kern<<<sm_count() * std::max(1, ob), wpc * 32, smem, st>>>(
            b.words.p, n, diag.p, v, b.N, a.upper, a.rowptr.p, b.hi.p, b.lo.p, b.low_bits, cap, sb, a.col.p,
            reinterpret_cast<double2*>(a.val.p), err.p);
        ::edgb::count_launch();
    };
    if (cap <= 128) launch(k_cfill<4>);
    else if (cap <= 512) launch(k_cfill<16>);
    else launch(k_cfill<32>);
    ED_CUDA(cudaGetLastError());
    int herr = 0;
    ED_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_REQUIRE(herr == 0, ED_ERR_INTERNAL, "complex fill: row count or rank check failed on the device");
}

void two_level_ladder(const ed_basis& b, const double* x, double* y, int dir, cudaStream_t st)
{
    ED_REQUIRE(b.levels == 2, ED_ERR_ARG, "the level-exchange ladder takes a two-level basis");
    const int64_t n = (int64_t)b.dim;
    if (n == 0) return;
    ED_CUDA(cudaMemsetAsync(y, 0, (size_t)n * 8, st));
    k_ladder2<<<sm_count() * 8, 256, 0, st>>>(b.words.p, n, b.norb0, b.norb1, dir, b.hi.p, b.lo.p, b.low_bits, x, y);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace edgb
