// Thick-restart basis rotation out[:, c] = sum_j V[:, j] Y[j, c] (K7): the
// n x m by m x k product that turns the Krylov basis into Ritz vectors at
// every restart (n*m*k FP64 multiply-adds, 1.4e9 at the headline size).
//
// Two kernels:
//  - k_gemm_vy: plain FP64 (one thread per row, Y staged in shared memory);
//  - k_rotate_oz: the same product on the BF16 tensor cores with FP64
//    accuracy, by error-free splitting (the Ozaki scheme: Ozaki, Ogita,
//    Oishi & Rump, Numer. Algorithms 59 (2012)).  Every row r of V is written
//    as 2^e_r * sum_t a_t 2^(-7(t+1)) with eight signed 7-bit digits a_t, every
//    column c of Y as 2^f_c * sum_u b_u 2^(-7(u+1)); digits are extracted from
//    the FP64 bit patterns with integer operations.  A digit (|a| <= 127) is
//    exact in bfloat16, a digit product (< 2^14) exact in the FP32
//    accumulator, and the group C_d = sum_{t+u=d} sum_j a_t[j] b_u[j] of one
//    anti-diagonal d stays an integer below 8 * 64 * 127^2 < 2^23 for
//    m <= 64, so mma.sync accumulates it exactly.  The groups d = 0..9 are
//    combined exactly in integers and rounded once to FP64,
//    out = 2^(e_r+f_c) sum_d 2^(-7(d+2)) C_d; the dropped
//    groups d >= 10 weigh below 1e-18 of 2^(e_r+f_c), so the result is at
//    least as accurate as an FP64 dot product (whose rounding is ~m * 1e-16).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ed_lanczos.h"

namespace edgb {

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kThreads = 256;
constexpr int kGT = 16;
constexpr int kOzRows = 64;      // rows of V per CTA
constexpr int kOzCols = 32;      // columns of the output per CTA
constexpr int kOzPlanes = 8;     // 7-bit digits per operand (56 bits)
constexpr int kOzGroups = 10;    // anti-diagonals d = t + u kept: 0..9 (49 digit pairs)

int rot_sms()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

// out[:, t] = sum_{i<m} V[:, i] Y[i, t] for t < k (Y column-major, ld m), FP64.
__global__ void __launch_bounds__(kThreads) k_gemm_vy(const double* __restrict__ V, int64_t n, int m,
                                                      const double* __restrict__ Y, int ldy, int k,
                                                      double* __restrict__ out)
{
    extern __shared__ double sy[];   // m * kGT
    for (int t0 = 0; t0 < k; t0 += kGT) {
        const int tn = min(kGT, k - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < m * kGT; q += kThreads) {
            const int i = q / kGT, t = q % kGT;
            sy[q] = (t < tn) ? Y[(int64_t)(t0 + t) * ldy + i] : 0.0;
        }
        __syncthreads();
        for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kThreads) {
            double acc[kGT];
#pragma unroll
            for (int t = 0; t < kGT; ++t) acc[t] = 0.0;
            for (int i = 0; i < m; ++i) {
                const double v = V[(int64_t)i * n + r];
#pragma unroll
                for (int t = 0; t < kGT; ++t) acc[t] = fma(v, sy[i * kGT + t], acc[t]);
            }
            for (int t = 0; t < tn; ++t) out[(int64_t)(t0 + t) * n + r] = acc[t];
        }
    }
}

// Biased exponent field of an FP64 value, 0 for zero and subnormals.
__host__ __device__ __forceinline__ int exp_field(double v)
{
    uint64_t b;
    memcpy(&b, &v, 8);
    return (int)((b >> 52) & 0x7FF);
}

// Eight signed 7-bit digits of v / 2^e with |v| < 2^e: the 56-bit fixed-point
// magnitude F = |v| 2^(56-e) (truncated) split into 7-bit groups, most
// significant first.  Subnormals read as zero.
__host__ __device__ __forceinline__ void digits7(double v, int e, int* d)
{
    uint64_t b;
    memcpy(&b, &v, 8);
    const int E = (int)((b >> 52) & 0x7FF);
    if (E == 0) {
        for (int t = 0; t < kOzPlanes; ++t) d[t] = 0;
        return;
    }
    const uint64_t M = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int s = E - 1075 - e + 56;          // <= 3 because |v| < 2^e
    const uint64_t F = s >= 0 ? (M << s) : (s > -64 ? (M >> -s) : 0ull);
    const bool neg = (b >> 63) != 0;
    for (int t = 0; t < kOzPlanes; ++t) {
        const int x = (int)((F >> (49 - 7 * t)) & 127u);
        d[t] = neg ? -x : x;
    }
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Four 8x8 b16 matrices from shared memory: thread i supplies the address of
// row i%8 of matrix i/8 (16-byte aligned) and receives, from matrix k, the
// elements (row i/4, columns 2(i%4), 2(i%4)+1) in r[k] — the m16n8k16
// fragment layout.
__device__ __forceinline__ void ldsm_x4(uint32_t* r, const bf16* p)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// Two integers of magnitude below 2^7 as a bf16 pair (x = a in the low
// half): float(x) is 1.5 * 2^23 + x read back minus 1.5 * 2^23 (exact for
// |x| < 2^22, on the FP32 pipe), and its top 16 bits are exactly the bf16 of
// x because x has at most 7 significant bits.
__device__ __forceinline__ uint32_t bf16x2_of_small_ints(int a, int b)
{
    const float fa = __int_as_float(0x4B400000 + a) - 12582912.0f;
    const float fb = __int_as_float(0x4B400000 + b) - 12582912.0f;
    return __byte_perm((uint32_t)__float_as_int(fa), (uint32_t)__float_as_int(fb), 0x7632);
}

// Exact conversion of an integer with |x| < 2^53 to double, by integer
// operations only (GB300's FP64 pipe is the scarce unit here).
__device__ __forceinline__ double i53_to_double(long long x)
{
    if (x == 0) return 0.0;
    const unsigned long long sgn = x < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long mag = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
    const int msb = 63 - __clzll((long long)mag);      // <= 52
    const unsigned long long mant = (mag << (52 - msb)) & ((1ull << 52) - 1);
    return __longlong_as_double((long long)(sgn | ((unsigned long long)(msb + 1023) << 52) | mant));
}

// 2^e for a normal exponent, else ldexp.
__device__ __forceinline__ double pow2(int e)
{
    if (e >= -1022 && e <= 1023) return __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(1.0, e);
}

// One CTA (8 warps): rows [r0, r0+64) of V against columns [c0, c0+32) of Y;
// warp w owns rows 16*(w%4).. and columns 16*(w/4)...
// ydig: digit planes of Y for this column block, [plane][column][MP] bf16;
// yexp: f_c per column.  Dynamic shared memory: the V digit planes
// [8][64][MP+8], the Y planes [8][32][MP+8] and the 64 row exponents.
// The ten anti-diagonal groups are combined exactly in two int64 sums,
// hi = sum_{d<5} C_d 2^(7(4-d)) and lo = sum_{d>=5} C_d 2^(7(9-d)) (each
// below 2^52), and out = 2^(e_r+f_c-77) (hi 2^35 + lo) with one FP64 FMA.
template <int MP>
__global__ void __launch_bounds__(256) k_rotate_oz(const double* __restrict__ V, int64_t n, int m,
                                                   const bf16* __restrict__ ydig, const int* __restrict__ yexp,
                                                   int k, double* __restrict__ out)
{
    constexpr int LD = MP + 8;   // row stride in bf16: conflict-free fragment loads
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sA = reinterpret_cast<bf16*>(smem);                       // [8][64][LD]
    bf16* sB = sA + kOzPlanes * kOzRows * LD;                       // [8][32][LD]
    int* se = reinterpret_cast<int*>(sB + kOzPlanes * kOzCols * LD);  // [64]
    const int64_t r0 = (int64_t)blockIdx.x * kOzRows;
    const int cb = blockIdx.y;
    const int c0 = cb * kOzCols;
    const bf16* yblk = ydig + (size_t)cb * kOzPlanes * kOzCols * MP;
    constexpr int NT = 256;

    for (int i = threadIdx.x; i < kOzRows; i += NT) se[i] = 0;
    // Y planes: plain copy of this column block (MP is a multiple of 16)
    for (int i = threadIdx.x; i < kOzPlanes * kOzCols * MP / 8; i += NT) {
        const int e0 = i * 8;
        const int pc = e0 / MP, j = e0 - pc * MP;                    // pc = plane*32 + column
        *reinterpret_cast<uint4*>(sB + (size_t)pc * LD + j) = *reinterpret_cast<const uint4*>(yblk + e0);
    }
    __syncthreads();
    // row exponents e_r = max over the row of (E - 1022), so |V[r][j]| < 2^e_r
    for (int i = threadIdx.x; i < kOzRows * m; i += NT) {
        const int rl = i % kOzRows, j = i / kOzRows;
        const int64_t r = r0 + rl;
        if (r < n) {
            const int E = exp_field(V[(int64_t)j * n + r]);
            if (E) atomicMax(&se[rl], E);
        }
    }
    __syncthreads();
    // V digit planes (zero beyond m and beyond n), two adjacent columns per
    // thread so that each plane gets one 32-bit store
    for (int i = threadIdx.x; i < kOzRows * MP / 2; i += NT) {
        const int rl = i % kOzRows, j = 2 * (i / kOzRows);
        const int64_t r = r0 + rl;
        int d0[kOzPlanes], d1[kOzPlanes];
        const bool live = r < n && se[rl];
        if (live && j < m) digits7(V[(int64_t)j * n + r], se[rl] - 1022, d0);
        else
#pragma unroll
            for (int t = 0; t < kOzPlanes; ++t) d0[t] = 0;
        if (live && j + 1 < m) digits7(V[(int64_t)(j + 1) * n + r], se[rl] - 1022, d1);
        else
#pragma unroll
            for (int t = 0; t < kOzPlanes; ++t) d1[t] = 0;
#pragma unroll
        for (int t = 0; t < kOzPlanes; ++t) {
            __nv_bfloat162 pr;
            pr.x = __int2bfloat16_rn(d0[t]);
            pr.y = __int2bfloat16_rn(d1[t]);
            *reinterpret_cast<__nv_bfloat162*>(sA + ((size_t)t * kOzRows + rl) * LD + j) = pr;
        }
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, tq = lane & 3;
    const int wr = (warp & 3) * 16;            // the warp's 16 rows
    const int wc = (warp >> 2) * 16;           // and 16 columns
    long long hi[2][4], lo[2][4];
#pragma unroll
    for (int ni = 0; ni < 2; ++ni)
#pragma unroll
        for (int e = 0; e < 4; ++e) hi[ni][e] = lo[ni][e] = 0;
#pragma unroll 1
    for (int dg = 0; dg < kOzGroups; ++dg) {
        float acc[2][4];
#pragma unroll
        for (int ni = 0; ni < 2; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[ni][e] = 0.f;
        for (int t = max(0, dg - (kOzPlanes - 1)); t <= min(dg, kOzPlanes - 1); ++t) {
            const int u = dg - t;
            const bf16* A = sA + (size_t)t * kOzRows * LD;
            const bf16* Bp = sB + (size_t)u * kOzCols * LD;
            // ldmatrix row addresses: A matrices (rows +0/+8, k +0/+8) in
            // fragment order; B matrices (n tile 0/1, k +0/+8)
            const int mi = lane >> 3, ri = lane & 7;
            const bf16* pa = A + (wr + (mi & 1) * 8 + ri) * LD + (mi >> 1) * 8;
            const bf16* pb = Bp + (wc + (mi >> 1) * 8 + ri) * LD + (mi & 1) * 8;
#pragma unroll
            for (int kk = 0; kk < MP; kk += 16) {
                uint32_t af[4], bq[4];
                ldsm_x4(af, pa + kk);
                ldsm_x4(bq, pb + kk);
                const uint32_t b0[2] = {bq[0], bq[1]}, b1[2] = {bq[2], bq[3]};
                mma_bf16(acc[0], af, b0);
                mma_bf16(acc[1], af, b1);
            }
        }
        // exact integer group sums into the two int64 accumulators
        const bool upper = dg < 5;
        const long long wgt = 1ll << (7 * (upper ? 4 - dg : 9 - dg));
#pragma unroll
        for (int ni = 0; ni < 2; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const long long c = (long long)__float2int_rz(acc[ni][e]);
                if (upper) hi[ni][e] += c * wgt;
                else lo[ni][e] += c * wgt;
            }
    }
    // scale by 2^(e_r + f_c - 77) and store (column-major output)
#pragma unroll
    for (int ni = 0; ni < 2; ++ni)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int rl = wr + g + ((e >= 2) ? 8 : 0);
            const int cl = wc + ni * 8 + tq * 2 + (e & 1);
            const int64_t r = r0 + rl;
            const int c = c0 + cl;
            if (r < n && c < k) {
                const int er = se[rl], fc = yexp[c];
                double v = 0.0;
                if (er && fc) {
                    v = fma(i53_to_double(hi[ni][e]), 34359738368.0 /* 2^35 */, i53_to_double(lo[ni][e]));
                    v *= pow2((er - 1022) + (fc - 1022) - 77);
                }
                out[(int64_t)c * n + r] = v;
            }
        }
}

// The same product with V's digits in registers.  One warp takes 16 rows
// (tiles over the rows, grid-strided) and all k <= 8 NT8 output columns: each
// lane loads the MP/2 values of its mma.m16n8k16 A-fragment positions (rows
// g and g + 8 of the tile, columns 16 s + 2 tq + {0, 1, 8, 9} for k-step s,
// g = lane / 4, tq = lane % 4), takes the row exponents by shuffles among the
// four lanes of a row, splits every value into its eight 7-bit digits and
// packs them straight into the fragments of the eight planes (each digit's
// bf16 bits from a float add on the FP32 pipe, not a conversion).  Y's digit
// planes sit in shared memory, padded to an even number of 8-column tiles, and
// one ldmatrix.x4 gives the B fragments of two output tiles.  The
// anti-diagonal groups and their exact int64 combination are k_rotate_oz's,
// so the results are the same bits.  No shared memory per row tile.
template <int MP, int NT8>
__global__ void __launch_bounds__(256, 1) k_rotate_ozr(const double* __restrict__ V, int64_t n, int m,
                                                       const bf16* __restrict__ ydig, const int* __restrict__ yexp,
                                                       int k, double* __restrict__ out)
{
    constexpr int KS = MP / 16;           // k-steps
    constexpr int NC = NT8 * 8;           // output columns computed
    constexpr int NCP = (NT8 + 1) / 2 * 16;   // columns held: an even number of 8-column tiles (zeros beyond NC)
    constexpr int LDB = MP + 8;           // bf16 row stride of the Y planes: conflict-free ldmatrix rows
    __shared__ __align__(16) bf16 sB[kOzPlanes * NCP * LDB];
    __shared__ int sfe[NC];
    // Y planes of the first NC columns (host layout [plane][32 columns][MP]),
    // zero columns up to NCP
    for (int i = threadIdx.x; i < kOzPlanes * NCP * MP; i += blockDim.x) {
        const int t = i / (NCP * MP), rem = i - t * NCP * MP, c = rem / MP, j = rem - c * MP;
        sB[(t * NCP + c) * LDB + j] = c < NC ? ydig[((size_t)t * kOzCols + c) * MP + j] : __float2bfloat16(0.f);
    }
    for (int c = threadIdx.x; c < NC; c += blockDim.x) sfe[c] = c < k ? yexp[c] : 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t ntiles = (n + 15) / 16;
    for (int64_t tile = warp; tile < ntiles; tile += nwarps) {
        const int64_t ra = tile * 16 + g, rb = ra + 8;
        // the lane's values at k-step s: q = 0,1 (row ra, columns 16s+2tq+{0,1}),
        // 2,3 (row rb, same), 4,5 (row ra, +8), 6,7 (row rb, +8); read once for
        // the row exponents and once more (from L1) for the digits, so that
        // the values of one k-step at a time are live
        auto value = [&](int s, int q) -> double {
            const int j = 16 * s + 2 * tq + (q & 1) + ((q & 4) ? 8 : 0);
            const int64_t r = (q & 2) ? rb : ra;
            return (j < m && r < n) ? V[(int64_t)j * n + r] : 0.0;
        };
        int emax_a = 0, emax_b = 0;
#pragma unroll
        for (int s = 0; s < KS; ++s)
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int E = exp_field(value(s, q));
                if (q & 2) emax_b = max(emax_b, E);
                else emax_a = max(emax_a, E);
            }
        // row exponents over the four lanes of a row
        emax_a = max(emax_a, __shfl_xor_sync(0xffffffffu, emax_a, 1));
        emax_a = max(emax_a, __shfl_xor_sync(0xffffffffu, emax_a, 2));
        emax_b = max(emax_b, __shfl_xor_sync(0xffffffffu, emax_b, 1));
        emax_b = max(emax_b, __shfl_xor_sync(0xffffffffu, emax_b, 2));
        // A fragments of the eight planes: af[t][s][i], i = 0 (row ra, k 2tq..),
        // 1 (row rb), 2 (row ra, k 2tq+8..), 3 (row rb, k +8)
        uint32_t af[kOzPlanes][KS][4];
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            double vs[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) vs[q] = value(s, q);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int e = (i & 1) ? emax_b : emax_a;
                int d0[kOzPlanes], d1[kOzPlanes];
                if (e) {
                    digits7(vs[2 * i], e - 1022, d0);
                    digits7(vs[2 * i + 1], e - 1022, d1);
                } else {
#pragma unroll
                    for (int t = 0; t < kOzPlanes; ++t) d0[t] = d1[t] = 0;
                }
#pragma unroll
                for (int t = 0; t < kOzPlanes; ++t) af[t][s][i] = bf16x2_of_small_ints(d0[t], d1[t]);
            }
        }
        // two output tiles of 8 columns at a time, so that only their int64
        // sums are live beside the fragments
#pragma unroll 1
        for (int nt0 = 0; nt0 < NT8; nt0 += 2) {
            long long hi[2][4], lo[2][4];
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) hi[nt][e] = lo[nt][e] = 0;
            const int ntn = min(2, NT8 - nt0);
#pragma unroll
            for (int dg = 0; dg < kOzGroups; ++dg) {
                float acc[2][4];
#pragma unroll
                for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
#pragma unroll
                for (int t = 0; t < kOzPlanes; ++t) {
                    const int u = dg - t;
                    if (u < 0 || u >= kOzPlanes) continue;
#pragma unroll
                    for (int ks = 0; ks < KS; ++ks) {
                        // matrices (tile nt0, k 0-7), (nt0, k 8-15), (nt0+1, k 0-7), (nt0+1, k 8-15)
                        const int mi = lane >> 3, ri = lane & 7;
                        uint32_t bq[4];
                        ldsm_x4(bq, sB + (u * NCP + (nt0 + (mi >> 1)) * 8 + ri) * LDB + 16 * ks + (mi & 1) * 8);
                        const uint32_t b0[2] = {bq[0], bq[1]}, b1[2] = {bq[2], bq[3]};
                        mma_bf16(acc[0], af[t][ks], b0);
                        if (ntn > 1) mma_bf16(acc[1], af[t][ks], b1);
                    }
                }
                const bool upper = dg < 5;
                const long long wgt = 1ll << (7 * (upper ? 4 - dg : 9 - dg));
#pragma unroll
                for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const long long c = (long long)__float2int_rz(acc[nt][e]);
                        if (upper) hi[nt][e] += c * wgt;
                        else lo[nt][e] += c * wgt;
                    }
            }
            // scale by 2^(e_r + f_c - 77) and store (column-major output)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int64_t r = (e >= 2) ? rb : ra;
                    const int c = (nt0 + nt) * 8 + tq * 2 + (e & 1);
                    if (nt < ntn && r < n && c < k) {
                        const int er = (e >= 2) ? emax_b : emax_a, fc = sfe[c];
                        double x = 0.0;
                        if (er && fc) {
                            x = fma(i53_to_double(hi[nt][e]), 34359738368.0 /* 2^35 */, i53_to_double(lo[nt][e]));
                            x *= pow2((er - 1022) + (fc - 1022) - 77);
                        }
                        out[(int64_t)c * n + r] = x;
                    }
                }
        }
    }
}

template <int MP, int NT8>
void launch_rotate_ozr(const double* V, int64_t n, int m, const bf16* ydig, const int* yexp, int k, double* out,
                       cudaStream_t st)
{
    // one resident CTA of 8 warps per SM (about 250 registers a thread),
    // the warps striding over the 16-row tiles
    const int64_t tiles = (n + 15) / 16;
    const int64_t grid = std::min<int64_t>((int64_t)rot_sms(), (tiles + 7) / 8);
    k_rotate_ozr<MP, NT8><<<(unsigned)std::max<int64_t>(1, grid), 256, 0, st>>>(V, n, m, ydig, yexp, k, out);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

template <int MP>
void launch_rotate_ozr_k(const double* V, int64_t n, int m, const bf16* ydig, const int* yexp, int k, double* out,
                         cudaStream_t st)
{
    switch ((k + 7) / 8) {
    case 1: launch_rotate_ozr<MP, 1>(V, n, m, ydig, yexp, k, out, st); break;
    case 2: launch_rotate_ozr<MP, 2>(V, n, m, ydig, yexp, k, out, st); break;
    case 3: launch_rotate_ozr<MP, 3>(V, n, m, ydig, yexp, k, out, st); break;
    default: launch_rotate_ozr<MP, 4>(V, n, m, ydig, yexp, k, out, st); break;
    }
}

template <int MP>
void launch_rotate_oz(const double* V, int64_t n, int m, const bf16* ydig, const int* yexp, int k, double* out,
                      cudaStream_t st)
{
    constexpr int LD = MP + 8;
    const size_t smem = (size_t)kOzPlanes * (kOzRows + kOzCols) * LD * 2 + kOzRows * 4;
    ED_CUDA(cudaFuncSetAttribute(k_rotate_oz<MP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((n + kOzRows - 1) / kOzRows), (unsigned)((k + kOzCols - 1) / kOzCols));
    k_rotate_oz<MP><<<grid, 256, smem, st>>>(V, n, m, ydig, yexp, k, out);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace

void rotate_basis(const double* V, int64_t n, int m, const double* Y_host, int ldy, int k, double* out,
                  RotateScratch& sc, int method, cudaStream_t st)
{
    if (k <= 0 || n <= 0) return;
    const bool tensor = method >= 2 || (method == 0 && m <= kRotateTensorMaxM);
    ED_REQUIRE(!tensor || m <= kRotateTensorMaxM, ED_ERR_ARG, "tensor-core rotation takes m <= 64");
    if (!tensor) {
        sc.y.alloc_at_least((size_t)ldy * k);
        ED_CUDA(cudaMemcpyAsync(sc.y.p, Y_host, (size_t)ldy * k * 8, cudaMemcpyHostToDevice, st));
        const size_t smem = (size_t)m * kGT * 8;
        if (smem > 48 * 1024)
            ED_CUDA(cudaFuncSetAttribute(k_gemm_vy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gemm_vy<<<rot_sms() * 4, kThreads, smem, st>>>(V, n, m, sc.y.p, ldy, k, out);
        count_launch();
        ED_CUDA(cudaGetLastError());
        return;
    }
    const int MP = (m + 15) / 16 * 16;
    const int nblk = (k + kOzCols - 1) / kOzCols;
    // digit planes of Y on the host: [block][plane][column][MP], exponents per column
    sc.ydig_h.assign((size_t)nblk * kOzPlanes * kOzCols * MP, 0);
    sc.yexp_h.assign((size_t)nblk * kOzCols, 0);
    for (int c = 0; c < k; ++c) {
        int E = 0;
        for (int j = 0; j < m; ++j) E = std::max(E, exp_field(Y_host[(size_t)c * ldy + j]));
        sc.yexp_h[c] = E;
        if (!E) continue;
        const int blk = c / kOzCols, cl = c % kOzCols;
        for (int j = 0; j < m; ++j) {
            int d[kOzPlanes];
            digits7(Y_host[(size_t)c * ldy + j], E - 1022, d);
            for (int t = 0; t < kOzPlanes; ++t) {
                const bf16 h = __float2bfloat16((float)d[t]);   // exact: |d| <= 127
                uint16_t bits;
                memcpy(&bits, &h, 2);
                sc.ydig_h[(((size_t)blk * kOzPlanes + t) * kOzCols + cl) * MP + j] = bits;
            }
        }
    }
    sc.ydig.alloc_at_least(sc.ydig_h.size());
    sc.yexp.alloc_at_least(sc.yexp_h.size());
    ED_CUDA(cudaMemcpyAsync(sc.ydig.p, sc.ydig_h.data(), sc.ydig_h.size() * 2, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaMemcpyAsync(sc.yexp.p, sc.yexp_h.data(), sc.yexp_h.size() * 4, cudaMemcpyHostToDevice, st));
    const bf16* yd = reinterpret_cast<const bf16*>(sc.ydig.p);
    // digits of V in registers (k_rotate_ozr) up to 32 output columns and
    // m <= 48 (at m = 64 its fragments no longer fit beside the sums)
    if (method != 3 && k <= kOzCols && MP <= 48) {
        switch (MP) {
        case 16: launch_rotate_ozr_k<16>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        case 32: launch_rotate_ozr_k<32>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        default: launch_rotate_ozr_k<48>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        }
    } else {
        switch (MP) {
        case 16: launch_rotate_oz<16>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        case 32: launch_rotate_oz<32>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        case 48: launch_rotate_oz<48>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        default: launch_rotate_oz<64>(V, n, m, yd, sc.yexp.p, k, out, st); break;
        }
    }
    // the host staging is reused by the next call: wait until the copies have read it
    ED_CUDA(cudaStreamSynchronize(st));
}

}  // namespace edgb

using namespace edgb;

extern "C" ed_status ed_basis_rotate(const double* V_dev, int64_t n, int m, const double* Y_host, int ldy, int k,
                                     double* out_dev, int method)
{
    return guard([&] {
        ED_REQUIRE(V_dev && Y_host && out_dev && n >= 1 && m >= 1 && k >= 1 && ldy >= m, ED_ERR_ARG, "bad argument");
        ED_REQUIRE(method >= 0 && method <= 3, ED_ERR_ARG,
                   "method: 0 auto, 1 FP64, 2 tensor cores, 3 tensor cores with V's digits staged in shared memory");
        // scratch kept per host thread, so repeated calls do not allocate
        static thread_local RotateScratch sc;
        rotate_basis(V_dev, n, m, Y_host, ldy, k, out_dev, sc, method, nullptr);
        ED_CUDA(cudaStreamSynchronize(nullptr));
    });
}
