// Hamiltonian-vector products: stored CRS (K4) and matrix-free (K5).
//
// Reference: MatrixVectorFunction::Simple (hamiltonians/matrix_vector_routines.hpp:94-104)
// -> SymmetricMatrixVectorMultiply (utilities/mathematics/sparse_linear_algebra.hpp:143-164):
//   y[i] += a*x[c]; if (i != c) y[c] += a*x[i]   over the stored upper triangle.
//
// On GB300 the FP64 pipe issues about 0.53e12 FMA/s (ed_fp64_fma_rate), less
// than streaming the CRS at HBM rate (12 bytes per element) demands, so an
// FP64 product is FP64-bound before it is HBM-bound.  The default products of
// full storage therefore run on the integer pipes in exact fixed-point
// arithmetic (ed_fixed.cuh: values and x in 58-bit fixed point, exact 128-bit
// row sums, one rounding to FP64), in one of two layouts:
//  - rows of 96 and more elements (the one-level sectors): k_spmv_fix, 8
//    lanes a row, each lane's exact sum over its share of the row, the lanes'
//    sums added exactly;
//  - shorter rows (two-level sectors): k_spmv_sell_fix over a sliced-ELL copy
//    (rows sorted by length within windows, chunks of 32 rows transposed), one
//    lane a row, no reduction, and the lanes of a chunk finish together.
// Both give the same bits.  The FP64 kernels (k_spmv_full, k_spmv_rows,
// k_spmv_sell) remain as selectable alternatives, spending FP64 instructions
// only where they must: one FMA per element, as few additions as the
// reduction allows, none for lanes with no element.  Column and value streams
// are read once with evict-first loads so that x stays resident in L2.
#include <algorithm>
#include <cmath>
#include <string>
#include <map>
#include <memory>

#include "ed_fixed.cuh"
#include "ed_hop.cuh"

namespace edgb {

namespace {

__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int32_t* p) { return __ldcs(p); }
__device__ __forceinline__ int2 ld_stream(const int2* p) { return __ldcs(p); }

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

// Reduce-scatter of R row sums held by each of the G lanes of a group: while
// a lane holds more than one row it keeps half of them (the upper half when
// the partner bit is set) and adds the partner's copy of that half; once it
// holds one row the remaining steps are plain butterfly additions.  Returns
// the row's total and sets `row` to its index in the group; lanes whose
// butterfly bits are zero own the result.  log2(G) - log2(R) + R - 1
// additions a lane for R rows, against R log2(G) for R separate butterflies.
template <int G, int R>
__device__ __forceinline__ double reduce_scatter_rows(const double (&acc)[R], int sub, int& row)
{
    double v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = acc[t];
    int base = 0;
#pragma unroll
    for (int o = G / 2, c = R; o >= 1; o >>= 1) {
        if (c > 1) {
            const bool hi = (sub & o) != 0;
#pragma unroll
            for (int t = 0; t < R / 2; ++t) {
                if (t < c / 2) {
                    const double send = hi ? v[t] : v[t + c / 2];
                    const double keep = hi ? v[t + c / 2] : v[t];
                    v[t] = keep + __shfl_xor_sync(0xffffffffu, send, o, G);
                }
            }
            if (hi) base += c / 2;
            c /= 2;
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], o, G);
        }
    }
    row = base;
    return v[0];
}

// Row lanes with a shared reduction: a group of G lanes takes R consecutive
// rows one after another (the same lane-strided FMA chain per row as
// k_spmv_full, U loads ahead), keeping one sum per row in registers, and
// reduce-scatters the R sums (reduce_scatter_rows).  Rows of 50-70 elements
// (the two-level sectors) waste fewer lanes with G = 4 and two loads ahead,
// and their reduction is a large share of the FP64 work: a row costs
// G log2 G additions in k_spmv_full, G (log2 G - log2 R + R - 1) / R here.
// Same element order within each lane; the row sum is added in another
// order, so y can differ from k_spmv_full's in the last bits.
template <int G, int U, int R>
__global__ void __launch_bounds__(256) k_spmv_rows(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                   const double* __restrict__ val, const double* __restrict__ x,
                                                   double* __restrict__ y, int64_t n)
{
    static_assert(R >= 1 && R <= G && (R & (R - 1)) == 0, "R a power of two up to G");
    constexpr int RPW = (32 / G) * R;   // rows per warp step
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {   // warp-uniform loop
        const int64_t g0 = rb + (int64_t)grp * R;
        double acc[R];
#pragma unroll
        for (int t = 0; t < R; ++t) {
            const int64_t r = g0 + t;
            const bool valid = r < n;
            const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
            double a = 0.0;
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
                    if (k0 + (int64_t)u * G < e) a = fma(v[u], __ldg(x + c[u]), a);
            }
            acc[t] = a;
        }
        int t = 0;
        const double w = reduce_scatter_rows<G, R>(acc, sub, t);
        constexpr int kButterflyMask = G / R - 1;
        const int64_t r = g0 + t;
        if ((sub & kButterflyMask) == 0 && r < n) y[r] = w;
    }
}

// ------------------------------------------------------------ fixed point
//
// The integer-pipe product.  GB300 issues about 0.53e12 FP64 FMA/s but far
// more 32-bit integer multiply-adds, so the one-level product runs in exact
// fixed-point integer arithmetic and leaves the FP64 pipe alone:
//  - the values and x are rounded to 58-bit fixed point relative to the
//    largest binary exponent of each (a = A 2^(ea-1080), x = X 2^(ex-1080),
//    |A|, |X| < 2^58) and split into 30-bit limbs, A = ah 2^30 + al with
//    0 <= al < 2^30;
//  - each element's A X = ah xh 2^60 + (ah xl + al xh) 2^30 + al xl takes
//    four 32x32->64-bit multiply-adds (mad.wide.s32) into int64 partial sums
//    of eight elements, which are added into the lane's int128 row sum;
//  - the lanes' sums are added (exact: a row of at most 2048 elements sums
//    to less than 2^127) and rounded once to FP64, to nearest:
//    y = round(S 2^(ea+ex-2160)).
// y therefore does not depend on the element order or the lane split, and
// it differs from the exact product of the FP64 inputs only by the
// fixed-point rounding of the inputs (half a unit of 2^-58 of the largest |a|
// and |x|) and the final rounding.  A non-finite entry of x makes every
// entry of y NaN; matrices with a non-finite value or a row longer than 2048
// elements keep the FP64 kernels.

constexpr int kFixPartPerSm = 2;     // blocks of the exponent pass per SM
constexpr int kFixMaxRow = 2048;     // |S| < 2048 * 2^116 = 2^127

// The one-level row kernel on the fixed-point values: G lanes per row, each
// lane one element in G, U elements' loads issued ahead of their
// multiply-adds, the lanes' int128 sums added and rounded by the first lane.
// xexp points at the exponent bound of x (k_fix_conv).
template <int G, int U, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_spmv_fix(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                  const int2* __restrict__ aq, const int2* __restrict__ xq,
                                                  const int* __restrict__ xexp, int ea, double* __restrict__ y,
                                                  int64_t n)
{
    // per element |ah xh| <= 2^56, |ah xl + al xh| < 2^59, 0 <= al xl < 2^60
    static_assert(U >= 1 && U <= 8, "eight elements' products fit the int64 partial sums");
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int ex = __ldg(xexp);
    const bool finite = ex < 2047;
    const int sc = ea + ex - 2160;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {   // warp-uniform loop
        const int64_t r = rb + grp;
        const bool valid = r < n;
        const int64_t s = valid ? rowptr[r] : 0;
        const int len = valid ? (int)(rowptr[r + 1] - s) : 0;
        const int2* ap = aq + s;
        const int32_t* cp = col + s;
        __int128 acc = 0;
        for (int j0 = sub; j0 < len; j0 += G * U) {
            int2 av[U];
            int cc[U];
            if (j0 + (U - 1) * G < len) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    av[u] = ld_stream(ap + j0 + u * G);
                    cc[u] = ld_stream(cp + j0 + u * G);
                }
            } else {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const bool in = j0 + u * G < len;
                    av[u] = in ? ld_stream(ap + j0 + u * G) : make_int2(0, 0);
                    cc[u] = in ? ld_stream(cp + j0 + u * G) : 0;
                }
            }
            int2 xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) xv[u] = __ldg(xq + cc[u]);
            long long p2 = mul_wide(av[0].y, xv[0].y);
            long long p1 = mad_wide(av[0].x, xv[0].y, mul_wide(av[0].y, xv[0].x));
            long long p0 = mul_wide(av[0].x, xv[0].x);
#pragma unroll
            for (int u = 1; u < U; ++u) fix_mac(av[u], xv[u], p2, p1, p0);
            acc += fix_combine(p2, p1, p0);
        }
        long long hi = (long long)(acc >> 64);
        unsigned long long lo = (unsigned long long)acc;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            const long long ohi = __shfl_xor_sync(0xffffffffu, hi, o, G);
            const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, o, G);
            const unsigned long long t = lo + olo;
            hi += ohi + (t < lo ? 1 : 0);
            lo = t;
        }
        if (valid && sub == 0)
            y[r] = finite ? round_i128(((__int128)hi << 64) | (__int128)lo, sc)
                          : __longlong_as_double(0x7FF8000000000000ll);
    }
}

// ------------------------------------------------ staged fixed-point product
//
// k_spmv_fix's arithmetic with the rows' values and columns streamed into
// shared memory by bulk copies (cp.async.bulk, completion counted on an
// mbarrier), so that a warp waits only for its gathers of x, not for the
// DRAM stream in front of them.  Measured on GB300 it is the slower kernel
// (N=11 2S=30: 1.71 ms against 0.77): shared memory holds three stages of
// 16 rows, and with one warp a row the per-row reduction and rounding take
// four times k_spmv_fix's instructions (8 lanes a row, four rows a warp),
// which makes it issue-bound; it is kept as the bulk-copy path, selected by
// ed_spmv_kernel 7.  One producer warp keeps a ring of stages
// filled, each stage the 16 consecutive rows of one row block (row blocks
// round-robin over the CTAs, one CTA per SM); 16 consumer warps take one row
// of each stage, 32 lanes on it, and release the slot on a second mbarrier.
// A stage larger than a slot is read from global memory instead.  Every
// wait is bounded (kFixWaitCycles): when one runs out, the CTA stops, the
// row of each waiting warp is set to NaN, the error word is incremented and
// the producer waits (bounded again) for the copies it issued.

constexpr int kStageRows = 16;
constexpr int kStageConsumers = 16;                          // warps: one row of a stage each
constexpr int kStageThreads = (kStageConsumers + 1) * 32;    // and the producer warp
constexpr int kStageMaxSlots = 4;
constexpr int kStageMetaStride = 20;                         // [17], [18]: the A and C copy origins
constexpr int kStageHeader = 128 + kStageMaxSlots * kStageMetaStride * 8;   // barriers, abort word, meta
constexpr long long kFixWaitCycles = 1ll << 31;             // about a second

__host__ __device__ constexpr int fix_acap(int se) { return (se + 2 + 15) / 16 * 16; }
__host__ __device__ constexpr int fix_ccap(int se) { return (se + 8 + 31) / 32 * 32; }
__host__ __device__ constexpr size_t fix_slot_bytes(int se) { return (size_t)fix_acap(se) * 8 + (size_t)fix_ccap(se) * 4; }

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t a)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

// Whether the barrier's phase of the given parity has completed; a thread
// whose phase is pending is suspended until it completes or about
// kFixSuspendNs pass, so that waiting warps leave the issue slots to the
// working ones.
constexpr uint32_t kFixSuspendNs = 20000;

__device__ __forceinline__ bool mbar_test(uint32_t a, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(kFixSuspendNs)
        : "memory");
    return ok != 0;
}

// Waits for the completion of the barrier's phase of the given parity, for
// at most limit clock cycles.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, long long limit)
{
    if (mbar_test(a, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_test(a, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

__device__ __forceinline__ uint64_t evict_first_policy()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// bytes (a multiple of 16) from global src to shared dst, both 16-byte
// aligned, counted on mbarrier mb; evict-first in L2 so that x stays.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mb, uint64_t pol)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mb), "l"(pol)
        : "memory");
}

// One row's exact sum, this lane's share: elements lane, lane + 32, ... of
// the row's len (A pairs at ap, columns at cp), U gathers of x ahead.
template <int U, bool GLOBAL>
__device__ __forceinline__ __int128 fix_row(const int2* ap, const int32_t* cp, int len, int lane,
                                            const int2* __restrict__ xq)
{
    __int128 acc = 0;
    for (int j0 = lane; j0 < len; j0 += 32 * U) {
        int2 av[U];
        int cc[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = j0 + 32 * u;
            const bool in = j < len;
            if (GLOBAL) {
                av[u] = in ? ld_stream(ap + j) : make_int2(0, 0);
                cc[u] = in ? ld_stream(cp + j) : 0;
            } else {
                av[u] = in ? ap[j] : make_int2(0, 0);
                cc[u] = in ? cp[j] : 0;
            }
        }
        int2 xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = __ldg(xq + cc[u]);
        long long p2 = mul_wide(av[0].y, xv[0].y);
        long long p1 = mad_wide(av[0].x, xv[0].y, mul_wide(av[0].y, xv[0].x));
        long long p0 = mul_wide(av[0].x, xv[0].x);
#pragma unroll
        for (int u = 1; u < U; ++u) fix_mac(av[u], xv[u], p2, p1, p0);
        acc += fix_combine(p2, p1, p0);
    }
    return acc;
}

// stall > 0 is the bounded-wait test: stage 0 is never filled and every wait
// gives up after stall cycles.
template <int U>
__global__ void __launch_bounds__(kStageThreads, 1)
    k_spmv_fix_staged(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                      const int2* __restrict__ aq, const int2* __restrict__ xq, const int* __restrict__ xexp, int ea,
                      double* __restrict__ y, int64_t n, int se, int ns, int* __restrict__ err, long long stall)
{
    static_assert(U >= 1 && U <= 8, "eight elements' products fit the int64 partial sums");
    extern __shared__ __align__(128) unsigned char fsm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(fsm);
    uint64_t* empty = full + kStageMaxSlots;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(fsm + 64);
    int64_t* meta = reinterpret_cast<int64_t*>(fsm + 128);
    const int acap = fix_acap(se), ccap = fix_ccap(se);
    int2* abuf = reinterpret_cast<int2*>(fsm + kStageHeader);
    int32_t* cbuf = reinterpret_cast<int32_t*>(fsm + kStageHeader + (size_t)ns * acap * 8);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < ns; ++i) {
            mbar_init(smem_addr(full + i), 1);
            mbar_init(smem_addr(empty + i), kStageConsumers);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long long limit = stall > 0 ? stall : kFixWaitCycles;
    const int64_t nblocks = (n + kStageRows - 1) / kStageRows;
    if (warp == kStageConsumers) {
        // producer.  The element bounds of 32 stages come in one load (lane l
        // holds stage sb + l's), the next 32 stages' loaded while these are
        // issued; the two batches alternate registers, so that no register
        // move waits for a load in flight.
        const uint64_t pol = evict_first_policy();
        int last[kStageMaxSlots];   // the latest stage issued with copies into each slot, -1 none
#pragma unroll
        for (int i = 0; i < kStageMaxSlots; ++i) last[i] = -1;
        auto load_batch = [&](int sb, int64_t& b0, int64_t& b1) {
            const int64_t gl = blockIdx.x + (int64_t)(sb + lane) * gridDim.x;
            b0 = gl < nblocks ? rowptr[gl * kStageRows] : 0;
            b1 = gl < nblocks ? rowptr[min(gl * kStageRows + kStageRows, n)] : 0;
        };
        // issues stages sb .. sb + 31 from the bounds c0, c1 (loading the next
        // batch into n0, n1); false at the last stage or when stopped
        auto run = [&](int sb, const int64_t& c0, const int64_t& c1, int64_t& n0, int64_t& n1) -> bool {
            load_batch(sb + 32, n0, n1);
            for (int i = 0; i < 32; ++i) {
                const int s = sb + i;
                if (blockIdx.x + (int64_t)s * gridDim.x >= nblocks) return false;
                const int slot = s % ns;
                bool ok = s < ns || mbar_wait(smem_addr(empty + slot), (uint32_t)((s / ns - 1) & 1), limit);
                ok = __all_sync(0xffffffffu, ok) && !*abort_flag;
                if (!ok) {
                    if (lane == 0) {
                        atomicAdd(err, 1);
                        *abort_flag = 1;
                    }
                    return false;
                }
                const int64_t k0 = __shfl_sync(0xffffffffu, c0, i), k1 = __shfl_sync(0xffffffffu, c1, i);
                if (lane == 0) {
                    int64_t* mt = meta + slot * kStageMetaStride;
                    const int64_t k0a = k0 & ~1ll, k1a = (k1 + 1) & ~1ll, k0c = k0 & ~3ll, k1c = (k1 + 3) & ~3ll;
                    const bool fits = k1a - k0a <= acap && k1c - k0c <= ccap;
                    mt[17] = fits ? k0a : -1;
                    mt[18] = k0c;
                    const uint32_t fb = smem_addr(full + slot);
                    // the slot's previous copies have landed: its stage was consumed
                    last[slot] = -1;
                    if (stall > 0 && s == 0) {
                        // never filled: the consumers' waits run out
                    } else if (fits && k1 > k0) {
                        const uint32_t ba = (uint32_t)((k1a - k0a) * 8), bc = (uint32_t)((k1c - k0c) * 4);
                        mbar_expect_tx(fb, ba + bc);
                        bulk_load(smem_addr(abuf + (size_t)slot * acap), aq + k0a, ba, fb, pol);
                        bulk_load(smem_addr(cbuf + (size_t)slot * ccap), col + k0c, bc, fb, pol);
                        last[slot] = s;
                    } else {
                        mbar_arrive(fb);
                    }
                }
                __syncwarp();
            }
            return true;
        };
        int64_t a0, a1, b0, b1;
        load_batch(0, a0, a1);
        for (int sb = 0;; sb += 64) {
            if (!run(sb, a0, a1, b0, b1)) break;
            if (!run(sb + 32, b0, b1, a0, a1)) break;
        }
        // no copy of this CTA outlives it
        if (lane == 0)
            for (int i = 0; i < ns; ++i)
                if (last[i] >= 0 && !mbar_wait(smem_addr(full + i), (uint32_t)((last[i] / ns) & 1), limit))
                    atomicAdd(err, 1);
        return;
    }
    // consumers: lanes 0 and 1 hold the bounds of this warp's row in the
    // coming stage, loaded one stage ahead
    const int ex = __ldg(xexp);
    const bool finite = ex < 2047;
    const int sc = ea + ex - 2160;
    int64_t rp = 0;
    if (lane < 2 && blockIdx.x < nblocks) rp = rowptr[min((int64_t)blockIdx.x * kStageRows + warp + lane, n)];
    int s = 0;
    for (int64_t g = blockIdx.x; g < nblocks; g += gridDim.x, ++s) {
        const int slot = s % ns;
        const int64_t r = g * kStageRows + warp;
        bool ok = mbar_wait(smem_addr(full + slot), (uint32_t)((s / ns) & 1), limit);
        ok = __all_sync(0xffffffffu, ok) && !*abort_flag;
        if (!ok) {
            if (lane == 0) {
                atomicAdd(err, 1);
                *abort_flag = 1;
                if (r < n) y[r] = __longlong_as_double(0x7FF8000000000000ll);
            }
            break;
        }
        const int64_t ks = __shfl_sync(0xffffffffu, rp, 0), ke = __shfl_sync(0xffffffffu, rp, 1);
        const int64_t gn = g + gridDim.x;
        if (lane < 2 && gn < nblocks) rp = rowptr[min(gn * kStageRows + warp + lane, n)];
        const int64_t* mt = meta + slot * kStageMetaStride;
        const int64_t k0a = mt[17], k0c = mt[18];
        const int len = (int)(ke - ks);
        __int128 acc;
        if (k0a >= 0)
            acc = fix_row<U, false>(abuf + (size_t)slot * acap + (ks - k0a), cbuf + (size_t)slot * ccap + (ks - k0c),
                                    len, lane, xq);
        else
            acc = fix_row<U, true>(aq + ks, col + ks, len, lane, xq);
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(empty + slot));
        acc = warp_sum_i128(acc);
        if (lane == 0 && r < n) y[r] = finite ? round_i128(acc, sc) : __longlong_as_double(0x7FF8000000000000ll);
    }
}

// ------------------------------------------------------------ sliced ELL

constexpr int kSellC = 32;          // rows per chunk (one warp)
constexpr int kSellWindow = 1024;   // rows per sorting window (32 chunks)

// Order of each window's rows by length, longest first (ties by row): the
// window's slots row[w0 + i] (-1 past the last row) and its chunks' padded
// lengths clen (the first, longest, row of each chunk).  A bitonic sort of
// (complemented length, slot) keys in shared memory, one CTA per window.
__global__ void __launch_bounds__(1024) k_sell_order(const int64_t* __restrict__ rowptr, int64_t n,
                                                     int32_t* __restrict__ row, int32_t* __restrict__ clen)
{
    __shared__ uint64_t key[kSellWindow];
    const int64_t w0 = (int64_t)blockIdx.x * kSellWindow;
    const int cnt = (int)min((int64_t)kSellWindow, n - w0);
    for (int i = threadIdx.x; i < kSellWindow; i += blockDim.x) {
        uint64_t k = ~0ull;   // empty slots sort last
        if (i < cnt) {
            const int64_t len = rowptr[w0 + i + 1] - rowptr[w0 + i];
            k = ((uint64_t)(0x7FFFFFFFu - (uint32_t)min(len, (int64_t)0x7FFFFFFF)) << 32) | (uint32_t)i;
        }
        key[i] = k;
    }
    __syncthreads();
    for (int size = 2; size <= kSellWindow; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < kSellWindow; i += blockDim.x) {
                const int j = i ^ stride;
                if (j > i) {
                    const uint64_t a = key[i], b = key[j];
                    if ((a > b) == ((i & size) == 0)) {
                        key[i] = b;
                        key[j] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < kSellWindow; i += blockDim.x) {
        const uint64_t k = key[i];
        row[w0 + i] = k == ~0ull ? -1 : (int32_t)(w0 + (int64_t)(uint32_t)k);
    }
    for (int c = threadIdx.x; c < kSellWindow / kSellC; c += blockDim.x) {
        const uint64_t k = key[c * kSellC];
        clen[w0 / kSellC + c] = k == ~0ull ? 0 : (int32_t)(0x7FFFFFFFu - (uint32_t)(k >> 32));
    }
}

__global__ void k_sell_sizes(const int32_t* __restrict__ clen, int64_t nchunks, int64_t* __restrict__ sizes)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nchunks; c += (int64_t)gridDim.x * blockDim.x)
        sizes[c] = (int64_t)clen[c] * kSellC;
}

// One warp per chunk: lane l copies its row's elements into the chunk,
// element j at off[c] + 32 j + l, and pads to the chunk's length with zero
// values at the row's own column (any valid index would do).
__global__ void __launch_bounds__(256) k_sell_fill(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                   const double* __restrict__ val, const int32_t* __restrict__ row,
                                                   const int32_t* __restrict__ clen, const int64_t* __restrict__ off,
                                                   int64_t nchunks, int32_t* __restrict__ scol,
                                                   double* __restrict__ sval)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nwarps) {
        const int L = clen[c];
        if (L == 0) continue;
        const int r = row[c * kSellC + lane];
        const int64_t s = r >= 0 ? rowptr[r] : 0;
        const int len = r >= 0 ? (int)(rowptr[r + 1] - s) : 0;
        const int pad = r >= 0 ? r : 0;
        const int64_t o = off[c] + lane;
        for (int j = 0; j < L; ++j) {
            const bool in = j < len;
            scol[o + (int64_t)j * kSellC] = in ? col[s + j] : pad;
            sval[o + (int64_t)j * kSellC] = in ? val[s + j] : 0.0;
        }
    }
}

// y = A x from the sliced-ELL copy: one warp per chunk, lane l accumulates
// its row in one FMA chain in CRS element order (then the padding's exact
// zeros), U elements' loads issued ahead of their FMAs.  All 32 lanes of a
// chunk run the same number of steps, and each load instruction reads 32
// consecutive values and columns.
template <int U, int CH = 1>
__global__ void __launch_bounds__(256) k_spmv_sell(const int64_t* __restrict__ off, const int32_t* __restrict__ clen,
                                                   const int32_t* __restrict__ row, const int32_t* __restrict__ scol,
                                                   const double* __restrict__ sval, const double* __restrict__ x,
                                                   double* __restrict__ y, int64_t nchunks)
{
    static_assert(CH == 1 || (CH == 2 && U % 2 == 0), "one chain, or two over an even unroll");
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nwarps) {
        const int L = clen[c];
        const int r = row[c * kSellC + lane];
        const double* vp = sval + off[c] + lane;
        const int32_t* cp = scol + off[c] + lane;
        double acc[CH];
#pragma unroll
        for (int h = 0; h < CH; ++h) acc[h] = 0.0;
        int j = 0;
        for (; j + U <= L; j += U) {
            double v[U];
            int cc[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                v[u] = ld_stream(vp + (int64_t)(j + u) * kSellC);
                cc[u] = ld_stream(cp + (int64_t)(j + u) * kSellC);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc[u % CH] = fma(v[u], __ldg(x + cc[u]), acc[u % CH]);
        }
        for (; j < L; ++j)
            acc[0] = fma(ld_stream(vp + (int64_t)j * kSellC), __ldg(x + ld_stream(cp + (int64_t)j * kSellC)), acc[0]);
        double t = acc[0];
#pragma unroll
        for (int h = 1; h < CH; ++h) t += acc[h];
        if (r >= 0) y[r] = t;
    }
}

// The sliced-ELL product on the fixed-point values (k_spmv_fix's exact
// arithmetic, one lane a row): U elements' loads ahead, their products'
// int64 partial sums flushed into the lane's 128-bit row sum every eight,
// one rounding per row.  The row's sum is exact, so y is k_spmv_fix's to the
// bit.
template <int U, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) k_spmv_sell_fix(const int64_t* __restrict__ off,
                                                            const int32_t* __restrict__ clen,
                                                            const int32_t* __restrict__ row,
                                                            const int32_t* __restrict__ scol,
                                                            const int2* __restrict__ sq, const int2* __restrict__ xq,
                                                            const int* __restrict__ xexp, int ea,
                                                            double* __restrict__ y, int64_t nchunks)
{
    static_assert(U % 8 == 0, "whole groups of eight");
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int ex = __ldg(xexp);
    const bool finite = ex < 2047;
    const int sc = ea + ex - 2160;
    for (int64_t c = warp; c < nchunks; c += nwarps) {
        const int L = clen[c];
        const int r = row[c * kSellC + lane];
        const int2* vp = sq + off[c] + lane;
        const int32_t* cp = scol + off[c] + lane;
        __int128 acc = 0;
        int j = 0;
        for (; j + U <= L; j += U) {
            int2 av[U];
            int cc[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                av[u] = ld_stream(vp + (int64_t)(j + u) * kSellC);
                cc[u] = ld_stream(cp + (int64_t)(j + u) * kSellC);
            }
            int2 xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) xv[u] = __ldg(xq + cc[u]);
#pragma unroll
            for (int h = 0; h < U; h += 8) {
                long long p2 = 0, p1 = 0, p0 = 0;
#pragma unroll
                for (int u = h; u < h + 8; ++u) fix_mac(av[u], xv[u], p2, p1, p0);
                acc += fix_combine(p2, p1, p0);
            }
        }
        for (; j < L; ++j) {
            long long p2 = 0, p1 = 0, p0 = 0;
            fix_mac(ld_stream(vp + (int64_t)j * kSellC), __ldg(xq + ld_stream(cp + (int64_t)j * kSellC)), p2, p1, p0);
            acc += fix_combine(p2, p1, p0);
        }
        if (r >= 0) y[r] = finite ? round_i128(acc, sc) : __longlong_as_double(0x7FF8000000000000ll);
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

// FP64 FMA issue rate (a measurement aid for the products' FP64 ceiling):
// eight independent chains r = r * a + b per thread, iters steps each.
__global__ void __launch_bounds__(256) k_dfma_rate(int iters, double a, double b, double* __restrict__ sink)
{
    double r[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = 1e-3 * threadIdx.x + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) r[i] = fma(r[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += r[i];
    if (s == -1.0) sink[0] = s;   // keeps the chains; never true for these inputs
}

int sms()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

}  // namespace

namespace {

void sell_build(const ed_crs& a, cudaStream_t st)
{
    const int64_t n = a.n;
    const int64_t nwin = (n + kSellWindow - 1) / kSellWindow;
    auto sl = std::make_unique<ed_sell>();
    sl->nchunks = nwin * (kSellWindow / kSellC);
    sl->row.alloc((size_t)nwin * kSellWindow);
    sl->len.alloc((size_t)sl->nchunks);
    sl->off.alloc((size_t)sl->nchunks + 1);
    k_sell_order<<<(unsigned)nwin, 1024, 0, st>>>(a.rowptr.p, n, sl->row.p, sl->len.p);
    count_launch();
    {
        DevBuf<int64_t> sizes((size_t)sl->nchunks);
        k_sell_sizes<<<sms() * 4, 256, 0, st>>>(sl->len.p, sl->nchunks, sizes.p);
        count_launch();
        exclusive_scan_i64(sizes.p, sl->off.p, sl->nchunks, st);
        ED_CUDA(cudaMemcpyAsync(&sl->nnz_pad, sl->off.p + sl->nchunks, 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
    }
    // the copy must leave room: decline when it would take more than half
    // of the free device memory
    size_t free_b = 0, total_b = 0;
    ED_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t need = (size_t)sl->nnz_pad * 12 + (size_t)kCrsPad * 12;
    if (need > free_b / 2) {
        a.sell_state = -1;
        return;
    }
    sl->col.alloc((size_t)sl->nnz_pad + kCrsPad);
    sl->val.alloc((size_t)sl->nnz_pad + kCrsPad);
    ED_CUDA(cudaMemsetAsync(sl->col.p + sl->nnz_pad, 0, kCrsPad * 4, st));
    ED_CUDA(cudaMemsetAsync(sl->val.p + sl->nnz_pad, 0, kCrsPad * 8, st));
    k_sell_fill<<<sms() * 8, 256, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, sl->row.p, sl->len.p, sl->off.p,
                                           sl->nchunks, sl->col.p, sl->val.p);
    count_launch();
    ED_CUDA(cudaGetLastError());
    a.sell = std::move(sl);
    a.sell_state = 1;
}

bool stream_capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ED_CUDA(cudaStreamIsCapturing(st, &cs));
    return cs != cudaStreamCaptureStatusNone;
}

template <int U, int CH = 1>
void sell_launch(const ed_crs& a, const double* x, double* y, cudaStream_t st)
{
    const ed_sell& sl = *a.sell;
    k_spmv_sell<U, CH><<<sms() * 8, 256, 0, st>>>(sl.off.p, sl.len.p, sl.row.p, sl.col.p, sl.val.p, x, y,
                                                  sl.nchunks);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace

// Full-storage matrices of at least kSellMinRows rows and fewer than
// kSellMaxAvg elements a row on average get the sliced-ELL copy; the others
// of full storage (the one-level sectors) the fixed-point copy.
constexpr int64_t kSellMinRows = 4096;
constexpr double kSellMaxAvg = 96.0;

namespace {

int fix_parts() { return sms() * kFixPartPerSm; }

// The fixed-point state of a matrix: the values' exponent bound (declined
// for a non-finite value or a row longer than kFixMaxRow); the copies of the
// values are made by fix_copy.
void fix_build(const ed_crs& a, cudaStream_t st)
{
    if (a.max_row > kFixMaxRow) {
        a.fix_state = -1;
        return;
    }
    auto fq = std::make_unique<ed_fixq>();
    const int P = fix_parts();
    DevBuf<int> part((size_t)P + 1);
    k_fix_exp<<<P, 256, 0, st>>>(a.val.p, a.nnz, part.p);
    count_launch();
    k_fix_conv<<<1, 256, 0, st>>>(a.val.p, 0, part.p, P, nullptr);   // the bound into part[P]
    count_launch();
    ED_CUDA(cudaGetLastError());
    int ea = 1;
    ED_CUDA(cudaMemcpyAsync(&ea, part.p + P, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    if (ea >= 2047) {
        a.fix_state = -1;
        return;
    }
    fq->ea = ea;
    // the staged kernel's ring: slots of 1.5 average stages (at least two
    // slots; up to four while the shared memory lasts)
    int smem_max = 0, dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    ED_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t room = (size_t)std::max(0, smem_max - kStageHeader);
    const double avg = (double)a.nnz / (double)std::max<int64_t>(1, a.n);
    int se = (int)std::min(65536.0, std::max(2048.0, std::ceil(1.5 * kStageRows * avg / 32.0) * 32.0));
    if (2 * fix_slot_bytes(se) > room) se = (int)((room / 2 - 512) / 12) / 32 * 32;
    const int ns = se >= 1024 ? (int)std::min<size_t>(kStageMaxSlots, room / fix_slot_bytes(se)) : 0;
    fq->stage_elems = ns >= 2 ? se : 0;
    fq->stages = ns >= 2 ? ns : 0;
    fq->err.alloc(1);
    ED_CUDA(cudaMemsetAsync(fq->err.p, 0, sizeof(int), st));
    ED_CUDA(cudaStreamSynchronize(st));
    a.fixq = std::move(fq);
    a.fix_state = 1;
}

// The stream's scratch for x's fixed-point copy, made on first use outside a
// capture; nullptr while capturing without one.
ed_fixq::Scratch* fix_scratch(const ed_crs& a, cudaStream_t st)
{
    ed_fixq& f = *a.fixq;
    int dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    // the legacy and per-thread streams have the same handle on every device
    const std::pair<int, cudaStream_t> key(dev, st);
    std::lock_guard<std::mutex> lk(f.mu);
    auto it = f.scratch.find(key);
    if (it != f.scratch.end()) return it->second.get();
    if (stream_capturing(st)) return nullptr;
    auto sc = std::make_unique<ed_fixq::Scratch>();
    sc->xq.alloc((size_t)a.n);
    sc->part.alloc((size_t)fix_parts() + 1);
    return f.scratch.emplace(key, std::move(sc)).first->second.get();
}

// The values' limb pairs in the CRS order (sell false) or the sliced-ELL
// order (sell true, after sell_build), made once outside a capture; false
// when the copy is not there (declined when it would take more than half of
// the free device memory).
bool fix_copy(const ed_crs& a, bool sell, cudaStream_t st)
{
    ed_fixq& f = *a.fixq;
    int& state = sell ? f.sval_state : f.val_state;
    if (state != 0) return state == 1;
    if (sell && a.sell_state != 1) return false;
    if (stream_capturing(st)) return false;
    const int64_t cnt = sell ? a.sell->nnz_pad : a.nnz;
    size_t free_b = 0, total_b = 0;
    ED_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if ((size_t)(cnt + kCrsPad) * 8 > free_b / 2) {
        state = -1;
        return false;
    }
    DevBuf<int64_t>& dst = sell ? f.sval : f.val;
    dst.alloc((size_t)(cnt + kCrsPad));
    ED_CUDA(cudaMemsetAsync(dst.p + cnt, 0, (size_t)kCrsPad * 8, st));
    DevBuf<int> part(2);
    ED_CUDA(cudaMemcpyAsync(part.p, &f.ea, sizeof(int), cudaMemcpyHostToDevice, st));
    k_fix_conv<<<sms() * 8, 256, 0, st>>>(sell ? a.sell->val.p : a.val.p, cnt, part.p, 1, dst.p);
    count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));
    state = 1;
    return true;
}

bool fix_shape(const ed_crs& a)
{
    return !a.upper && a.n > 0 && (double)a.nnz >= kSellMaxAvg * (double)a.n;
}

// The fixed-point state, the copy of the values in the wanted order and
// this stream's scratch, made when missing and not capturing; false when one
// of them is not there.
bool fix_ready(const ed_crs& a, cudaStream_t st, bool sell = false)
{
    if (a.fix_state == 0 && !stream_capturing(st)) fix_build(a, st);
    return a.fix_state == 1 && fix_copy(a, sell, st) && fix_scratch(a, st) != nullptr;
}

// x's fixed-point copy into the stream's scratch; returns the scratch.
ed_fixq::Scratch& fix_convert_x(const ed_crs& a, const double* x, cudaStream_t st)
{
    ed_fixq::Scratch& sc = *fix_scratch(a, st);
    const int P = fix_parts();
    k_fix_exp<<<P, 256, 0, st>>>(x, a.n, sc.part.p);
    count_launch();
    k_fix_conv<<<sms() * 4, 256, 0, st>>>(x, a.n, sc.part.p, P, sc.xq.p);
    count_launch();
    return sc;
}

void fix_launch_staged(const ed_crs& a, const double* x, double* y, long long stall, cudaStream_t st)
{
    const ed_fixq& f = *a.fixq;
    ED_REQUIRE(f.stages >= 2, ED_ERR_RANGE, "the staged product's ring does not fit in shared memory");
    ed_fixq::Scratch& sc = fix_convert_x(a, x, st);
    const size_t smem = kStageHeader + (size_t)f.stages * fix_slot_bytes(f.stage_elems);
    ED_CUDA(cudaFuncSetAttribute(k_spmv_fix_staged<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_spmv_fix_staged<8><<<sms(), kStageThreads, smem, st>>>(
        a.rowptr.p, a.col.p, reinterpret_cast<const int2*>(f.val.p), reinterpret_cast<const int2*>(sc.xq.p),
        sc.part.p + fix_parts(), f.ea, y, a.n, f.stage_elems, f.stages, f.err.p, stall);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void fix_launch(const ed_crs& a, const double* x, double* y, cudaStream_t st)
{
    const ed_fixq& f = *a.fixq;
    ed_fixq::Scratch& sc = fix_convert_x(a, x, st);
    const int P = fix_parts();
    // 8 lanes a row, 8 loads ahead, at most 64 registers: four CTAs per SM
    // (GB300, N=11 2S=30 with the two conversion passes: 0.772 ms; 71
    // registers and three CTAs 0.877; 4 loads ahead 0.862; 48 or 40
    // registers with spills 0.88-1.03; each warp's next row tile prefetched
    // into L2 by cp.async.bulk.prefetch 0.99; the rows staged in shared
    // memory by bulk copies, k_spmv_fix_staged, 1.71)
    k_spmv_fix<8, 8, 4><<<sms() * 8, 256, 0, st>>>(a.rowptr.p, a.col.p, reinterpret_cast<const int2*>(f.val.p),
                                                   reinterpret_cast<const int2*>(sc.xq.p), sc.part.p + P, f.ea, y,
                                                   a.n);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void fix_launch_sell(const ed_crs& a, const double* x, double* y, cudaStream_t st)
{
    const ed_fixq& f = *a.fixq;
    const ed_sell& sl = *a.sell;
    ed_fixq::Scratch& sc = fix_convert_x(a, x, st);
    k_spmv_sell_fix<8, 4><<<sms() * 8, 256, 0, st>>>(sl.off.p, sl.len.p, sl.row.p, sl.col.p,
                                                     reinterpret_cast<const int2*>(f.sval.p),
                                                     reinterpret_cast<const int2*>(sc.xq.p), sc.part.p + fix_parts(),
                                                     f.ea, y, sl.nchunks);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace

void spmv_prepare(const ed_crs& a, cudaStream_t st)
{
    if (a.n == 0 || stream_capturing(st)) return;
    const int k = a.product_kernel;
    if (k == 6 || k == 7 || (k == 0 && fix_shape(a))) fix_ready(a, st);
    if ((k == 4 || k == 5 || k == 8) && a.sell_state == 0) sell_build(a, st);
    if (k == 0 && a.sell_state == 0) {
        // one-level sectors (96 and more elements a row) stay with the row lanes
        if (a.upper || a.n < kSellMinRows || (double)a.nnz >= kSellMaxAvg * (double)a.n) a.sell_state = -1;
        else sell_build(a, st);
    }
    if ((k == 0 || k == 8) && a.sell_state == 1) fix_ready(a, st, true);
}

void spmv_kernel(const ed_crs& a, int kernel, const double* x, double* y, cudaStream_t st)
{
    if (a.n == 0) return;
    ED_REQUIRE(kernel >= 0 && kernel <= 8, ED_ERR_ARG,
               "kernel: 0 (chosen by shape), 1 (row lanes 8x4), 2 / 3 (shared reduction 8x4x2 / 8x2x2), "
               "4 / 5 (sliced ELL, 16 / 8 loads ahead), 6 (fixed-point integer rows 8x8), 7 (the same, rows "
               "staged in shared memory by bulk copies), 8 (fixed-point sliced ELL)");
    if (kernel == 0) {
        spmv(a, x, y, st);
        return;
    }
    ED_REQUIRE(!a.upper, ED_ERR_ARG, "the row, sliced-ELL and fixed-point kernels take full storage");
    if (kernel == 8) {
        if (a.sell_state == 0 && !stream_capturing(st)) sell_build(a, st);   // any size here
        ED_REQUIRE(a.sell_state == 1 && fix_ready(a, st, true), ED_ERR_RANGE,
                   "no fixed-point sliced-ELL copy (a non-finite value, a row of more than 2048 elements, not "
                   "enough free device memory, or a first product on this stream inside a capture)");
        fix_launch_sell(a, x, y, st);
        return;
    }
    if (kernel == 6 || kernel == 7) {
        ED_REQUIRE(fix_ready(a, st), ED_ERR_RANGE,
                   "no fixed-point copy (a non-finite value, a row of more than 2048 elements, not enough free "
                   "device memory, or a first product on this stream inside a capture)");
        if (kernel == 6) fix_launch(a, x, y, st);
        else fix_launch_staged(a, x, y, 0, st);
        return;
    }
    const int threads = 256;
    const int grid = sms() * 8;
    const int64_t* rp = a.rowptr.p;
    switch (kernel) {
    case 1: k_spmv_full<8, 4><<<grid, threads, 0, st>>>(rp, a.col.p, a.val.p, x, y, a.n); break;
    case 2: k_spmv_rows<8, 4, 2><<<grid, threads, 0, st>>>(rp, a.col.p, a.val.p, x, y, a.n); break;
    case 3: k_spmv_rows<8, 2, 2><<<grid, threads, 0, st>>>(rp, a.col.p, a.val.p, x, y, a.n); break;
    default:
        if (a.sell_state == 0 && !stream_capturing(st)) sell_build(a, st);   // any size here
        ED_REQUIRE(a.sell_state == 1, ED_ERR_RANGE, "no sliced-ELL copy (not enough free device memory)");
        if (kernel == 4) sell_launch<16>(a, x, y, st);
        else sell_launch<8>(a, x, y, st);
        return;
    }
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void spmv_check(const ed_crs& a, cudaStream_t st)
{
    if (a.fix_state != 1 || !a.fixq->err.p) return;
    int e = 0;
    ED_CUDA(cudaMemcpyAsync(&e, a.fixq->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    if (e == 0) return;
    ED_CUDA(cudaMemsetAsync(a.fixq->err.p, 0, sizeof(int), st));
    ED_CUDA(cudaStreamSynchronize(st));
    throw Error(ED_ERR_CUDA, "a staged product's copy wait ran out (" + std::to_string(e) + " waits)");
}

int spmv_staged_wait_test(const ed_crs& a, const double* x, double* y, long long cycles, cudaStream_t st)
{
    ED_REQUIRE(!a.upper && cycles > 0, ED_ERR_ARG, "full storage and a positive wait limit");
    ED_REQUIRE(fix_ready(a, st), ED_ERR_RANGE, "no fixed-point copy");
    fix_launch_staged(a, x, y, cycles, st);
    int e = 0;
    ED_CUDA(cudaMemcpyAsync(&e, a.fixq->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    ED_CUDA(cudaMemsetAsync(a.fixq->err.p, 0, sizeof(int), st));
    ED_CUDA(cudaStreamSynchronize(st));
    return e;
}

void spmv(const ed_crs& a, const double* x, double* y, cudaStream_t st)
{
    if (a.n == 0) return;
    if (a.product_kernel > 0) {
        spmv_kernel(a, a.product_kernel, x, y, st);
        return;
    }
    if (a.sell_state == 0) spmv_prepare(a, st);   // waits for a solver's explicit call while capturing
    if (a.sell_state == 1) {
        if (fix_ready(a, st, true)) {
            // the fixed-point sliced ELL (two-level N=8, 2S=21: see
            // k_spmv_sell_fix), else the FP64 kernel below
            fix_launch_sell(a, x, y, st);
            return;
        }
        // rows of fewer than 96 elements (two-level sectors, small one-level
        // ones), measured on GB300 at two-level N=8, 2S=18 (2.03M rows of 59
        // on average) / 2S=21 (5.90M rows of 73): sliced ELL with 16 loads
        // ahead 0.305 / 1.052 ms (8 ahead 0.326 / 1.110, 24 0.303 / 1.045,
        // 32 0.310 / 1.055) against the best row kernels 0.333 / 1.197
        sell_launch<16>(a, x, y, st);
        return;
    }
    const double avg = (double)a.nnz / (double)a.n;
    const int threads = 256;
    const int grid = sms() * 8;
    if (!a.upper && avg >= 24) {
        // one-level sectors (190-260 elements a row): 8 lanes, 4 loads ahead,
        // two rows a group (GB300, N=11 2S=30: 0.826-0.838 ms against
        // 0.828-0.841 for k_spmv_full<8,4> and 0.90 for sliced ELL with 16
        // loads ahead; N=10 2S=27: 0.1219-0.1226 against 0.1219-0.1232 and
        // 0.14); also the short-row sectors below kSellMinRows rows
        if (avg >= kSellMaxAvg) {
            if (fix_ready(a, st)) {
                fix_launch(a, x, y, st);
                return;
            }
            k_spmv_rows<8, 4, 2><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
        } else {
            k_spmv_rows<8, 2, 2><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
        }
    } else if (!a.upper) {
        k_spmv_full<2><<<grid, threads, 0, st>>>(a.rowptr.p, a.col.p, a.val.p, x, y, a.n);
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

// DFMA per second of the whole device: blocks_per_sm * SMs blocks of 256
// threads, 8 chains of iters FMAs each; the second of two launches timed.
double measure_dfma_rate(int iters, int blocks_per_sm)
{
    const int grid = sms() * blocks_per_sm;
    DevBuf<double> sink(1);
    cudaEvent_t e0, e1;
    ED_CUDA(cudaEventCreate(&e0));
    ED_CUDA(cudaEventCreate(&e1));
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
        ED_CUDA(cudaEventRecord(e0, nullptr));
        k_dfma_rate<<<grid, 256>>>(iters, 1.0 - 1e-12, 1e-12, sink.p);
        count_launch();
        ED_CUDA(cudaEventRecord(e1, nullptr));
        ED_CUDA(cudaEventSynchronize(e1));
        ED_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ED_CUDA(cudaGetLastError());
    return (double)grid * 256 * 8 * (double)iters / (ms * 1e-3);
}

}  // namespace edgb
