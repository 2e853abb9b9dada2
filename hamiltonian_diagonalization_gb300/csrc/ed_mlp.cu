// Learned warm start (K10/K11): a small MLP maps (occupation bitstring, V1)
// to (log|psi|, sign logit) of the sector's ground state.  It is trained on
// ground states the solver itself produced, with BF16 weights and
// activations and FP32 accumulation on the tensor cores (warp-level
// mma.sync m16n8k16), FP32 master weights and Adam.  Its prediction,
// evaluated on every basis word of a held-out V1, normalised, seeds the
// Lanczos solve.  No reference counterpart: the reference always starts ARPACK
// from its own random vector or a file (arpack_wrapper.hpp:753-774).
//
// Layout: features x = (2*bit_k - 1 for k < norb, (V1 - 1.75)/1.25, zeros)
// padded to 32; hidden width H (multiple of 64) for three SiLU layers; the
// output layer is padded to 8 columns of which 0 = log|psi|, 1 = sign logit.
// Weights are [in][out] row-major.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ed_internal.h"
#include "ed_lanczos.h"

namespace edgb {

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kIn = 64;   // orbital bits, V1, zero padding (up to 63 orbitals)
constexpr int kOut = 8;
constexpr int kLayers = 4;

// ------------------------------------------------------------- GEMM core
// C[M,N] = sum_k A(m,k) B(k,n) with A(m,k) = A[m*sam + k*sak] and
// B(k,n) = Bm[k*sbk + n*sbn] (bf16), FP32 accumulation in mma.sync
// m16n8k16; 64x64 block tile, 128 columns of K per stage, four warps of
// 32x32.  Tiles are staged
// through shared memory with bounds checks, so any strides (transposes)
// and any M, N, K work; the epilogue functor receives (row, col, value).

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// K extent staged per synchronisation, and the shared-memory row stride
// (BK + 8 bf16 = 272 bytes: 16-byte aligned rows, conflict-free fragments).
constexpr int kBK = 128;
constexpr int kLDS = kBK + 8;

// Stage a 64 x kBK tile of an operand into s[row][k] (row = m or n index).
// The operand is P(mn, k) = P[mn*s_mn + k*s_k]; the tile is read in 16-byte
// pieces along whichever index is contiguous (k when kfast, else mn), with
// element-wise bounds checks where a piece crosses an edge or is not 16-byte
// aligned.
__device__ __forceinline__ void stage_tile(bf16 (*s)[kLDS], const bf16* __restrict__ P, int64_t s_mn, int64_t s_k,
                                           bool kfast, int mn0, int MN, int k0, int kend)
{
    const bf16 zero = __float2bfloat16(0.f);
    if (kfast) {
        for (int c = threadIdx.x; c < 64 * kBK / 8; c += 128) {     // 64 rows x kBK/8 pieces of 8 k
            const int r = c / (kBK / 8), kc = (c % (kBK / 8)) * 8;
            const int gmn = mn0 + r, gk = k0 + kc;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gmn < MN && gk < kend) {
                const bf16* src = P + (int64_t)gmn * s_mn + gk;
                if (gk + 8 <= kend && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    v = *reinterpret_cast<const uint4*>(src);
                } else {
                    __align__(16) bf16 t[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) t[e] = (gk + e < kend) ? src[e] : zero;
                    v = *reinterpret_cast<const uint4*>(t);
                }
            }
            *reinterpret_cast<uint4*>(&s[r][kc]) = v;
        }
    } else {
        for (int c = threadIdx.x; c < kBK * 8; c += 128) {          // kBK k x 8 pieces of 8 rows
            const int kk = c >> 3, mc = (c & 7) * 8;
            const int gk = k0 + kk, gmn = mn0 + mc;
            __align__(16) bf16 t[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) t[e] = zero;
            if (gk < kend && gmn < MN) {
                const bf16* src = P + (int64_t)gk * s_k + gmn;
                if (gmn + 8 <= MN && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(src);
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (gmn + e < MN) t[e] = src[e];
                }
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) s[mc + e][kk] = t[e];
        }
    }
}

template <class Epi>
__global__ void __launch_bounds__(128) k_gemm(const bf16* __restrict__ A, int64_t sam, int64_t sak,
                                              const bf16* __restrict__ Bm, int64_t sbk, int64_t sbn, int M, int N, int K,
                                              int kchunk, Epi epi)
{
    __shared__ __align__(16) bf16 sA[64][kLDS];   // [m][k]
    __shared__ __align__(16) bf16 sB[64][kLDS];   // [n][k]
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int g = lane >> 2, tq = lane & 3;
    const bool a_kfast = sak == 1, b_kfast = sbk == 1;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    for (int k0 = kbeg; k0 < kend; k0 += kBK) {
        stage_tile(sA, A, sam, sak, a_kfast, m0, M, k0, kend);
        stage_tile(sB, Bm, sbn, sbk, b_kfast, n0, N, k0, kend);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < min(kBK, kend - k0); kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) {
                const int r = wm + mi * 16 + g;
                af[mi][0] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + tq * 2]);
                af[mi][1] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + tq * 2]);
                af[mi][2] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + tq * 2 + 8]);
                af[mi][3] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + tq * 2 + 8]);
            }
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                const int nn = wn + ni * 8 + g;
                bfr[ni][0] = *reinterpret_cast<const uint32_t*>(&sB[nn][kk + tq * 2]);
                bfr[ni][1] = *reinterpret_cast<const uint32_t*>(&sB[nn][kk + tq * 2 + 8]);
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], af[mi], bfr[ni]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = m0 + wm + mi * 16 + g + ((e >= 2) ? 8 : 0);
                const int col = n0 + wn + ni * 8 + tq * 2 + (e & 1);
                if (row < M && col < N) epi(row, col, acc[mi][ni][e]);
            }
}

template <class Epi>
void gemm(const bf16* A, int64_t sam, int64_t sak, const bf16* B, int64_t sbk, int64_t sbn, int M, int N, int K,
          Epi epi, cudaStream_t st, int splits = 1)
{
    const int kchunk = ((K + splits - 1) / splits + kBK - 1) / kBK * kBK;
    dim3 grid((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64), (unsigned)splits);
    k_gemm<Epi><<<grid, 128, 0, st>>>(A, sam, sak, B, sbk, sbn, M, N, K, kchunk, epi);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// Forward epilogue: Z = acc + bias (FP32, kept for the backward pass) and,
// for hidden layers, H = bf16(SiLU(Z)).
struct EpiForward {
    const float* bias;
    float* Z;
    bf16* Hout;   // nullptr for the output layer
    int ld;
    __device__ void operator()(int r, int c, float v) const
    {
        const float z = v + bias[c];
        Z[(int64_t)r * ld + c] = z;
        if (Hout) Hout[(int64_t)r * ld + c] = __float2bfloat16(silu(z));
    }
};

// Backward-data epilogue: dZ = acc * SiLU'(Z) in bf16 (input of the next GEMMs)
// and FP32 (for the bias gradient).
struct EpiBackData {
    const float* Z;
    bf16* dZ;
    float* dZf;
    int ld;
    __device__ void operator()(int r, int c, float v) const
    {
        const float d = v * dsilu(Z[(int64_t)r * ld + c]);
        dZ[(int64_t)r * ld + c] = __float2bfloat16(d);
        dZf[(int64_t)r * ld + c] = d;
    }
};

// Weight-gradient epilogue of a split-K GEMM: split blockIdx.z stores its
// partial sum to out[z*zstride + r*ld + c]; k_sum_splits adds the splits.
struct EpiSplit {
    float* out;
    int ld;
    int64_t zstride;
    __device__ void operator()(int r, int c, float v) const
    {
        out[(int64_t)blockIdx.z * zstride + (int64_t)r * ld + c] = v;
    }
};

// out[i] = sum_z part[z*count + i], splits added in order
__global__ void k_sum_splits(const float* __restrict__ part, int S, int64_t count, float* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < S; ++z) s += part[(int64_t)z * count + i];
        out[i] = s;
    }
}

// features of sample i: word bits as +-1, scaled V1, zero padding
__global__ void k_features(const uint64_t* __restrict__ words, const float* __restrict__ v1, int64_t m, int norb,
                           bf16* __restrict__ X)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * kIn; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / kIn;
        const int f = (int)(t - i * kIn);
        float x = 0.f;
        if (f < norb) x = ((words[i] >> f) & 1ull) ? 1.f : -1.f;
        else if (f == norb) x = (v1[i] - 1.75f) / 1.25f;
        X[t] = __float2bfloat16(x);
    }
}

// loss and output gradient: L = mean[(y0-t0)^2 + softplus(y1) - t1*y1]
__global__ void k_loss_grad(const float* __restrict__ Z4, const float* __restrict__ target, int64_t m,
                            bf16* __restrict__ dZ4, float* __restrict__ dZ4f, double* __restrict__ loss)
{
    __shared__ double red[256];
    double l = 0.0;
    const float inv = 1.f / (float)m;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const float y0 = Z4[i * kOut], y1 = Z4[i * kOut + 1];
        const float t0 = target[2 * i], t1 = target[2 * i + 1];
        const float d0 = y0 - t0;
        const float sp = y1 > 0 ? y1 + log1pf(__expf(-y1)) : log1pf(__expf(y1));
        l += (double)(d0 * d0 + sp - t1 * y1);
        const float g0 = 2.f * d0 * inv;
        const float g1 = (1.f / (1.f + __expf(-y1)) - t1) * inv;
        for (int c = 0; c < kOut; ++c) {
            const float g = c == 0 ? g0 : (c == 1 ? g1 : 0.f);
            dZ4[i * kOut + c] = __float2bfloat16(g);
            dZ4f[i * kOut + c] = g;
        }
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = 128; s; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// Column sums of dZ (m x n, FP32) in row chunks: block (x, y) covers columns
// [32x, 32x+32) of row chunk y with 8 row lanes of 32 consecutive columns
// (coalesced); part[y*n + c] = the chunk's sum, added up by k_sum_splits.
__global__ void __launch_bounds__(256) k_colsum_part(const float* __restrict__ dZ, int64_t m, int n,
                                                     float* __restrict__ part)
{
    __shared__ float red[8][33];
    const int c = blockIdx.x * 32 + (threadIdx.x & 31), rl = threadIdx.x >> 5;
    const int64_t r0 = m * blockIdx.y / gridDim.y, r1 = m * (blockIdx.y + 1) / gridDim.y;
    float s = 0.f;
    if (c < n)
        for (int64_t i = r0 + rl; i < r1; i += 8) s += dZ[i * n + c];
    red[rl][threadIdx.x & 31] = s;
    __syncthreads();
    if (rl == 0 && c < n) {
        float t = 0.f;
        for (int l = 0; l < 8; ++l) t += red[l][threadIdx.x];
        part[(int64_t)blockIdx.y * n + c] = t;
    }
}

// Training counters on the device, so that a captured training step replays
// with the right values: ctr[0] = Adam step t, ctr[1] = fit step s (both
// advanced at the start of a step, so 1-based inside it).
__global__ void k_advance(int64_t* __restrict__ ctr)
{
    ctr[0] += 1;
    ctr[1] += 1;
}

// Adam on the FP32 masters, refreshing the bf16 copies of the weights.  With
// fit_total > 0 the rate decays linearly from lr0 to lr0/10 over the fit.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, bf16* __restrict__ pb, int64_t n, float lr0,
                       const int64_t* __restrict__ ctr, int64_t fit_total, float b1, float b2, float eps)
{
    const float t = (float)ctr[0];
    const float lr = fit_total > 0 ? lr0 * (1.f - 0.9f * (float)(ctr[1] - 1) / (float)fit_total) : lr0;
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        const float v = p[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        p[i] = v;
        if (pb) pb[i] = __float2bfloat16(v);
    }
}

__global__ void k_to_bf16(const float* __restrict__ x, bf16* __restrict__ y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

// training batch: sample s -> (state r, V1 index b) from a seeded hash; the
// target is (log|psi_b(r)|, sign), log clipped at -40.  Even samples draw r
// uniformly (the network must also learn where the state is small), odd
// samples draw r with probability |psi_b(r)|^2 from the per-column
// cumulative table cdf[b][r] (the configurations that carry the overlap).
__global__ void k_make_batch(const uint64_t* __restrict__ basis, int64_t n, const double* __restrict__ psi, int nv,
                             const float* __restrict__ v1s, const double* __restrict__ cdf, int64_t m, uint64_t seed0,
                             const int64_t* __restrict__ ctr, uint64_t* __restrict__ words, float* __restrict__ v1,
                             float* __restrict__ target)
{
    const uint64_t seed = seed0 + 0x632BE59BD9B4E019ull * (uint64_t)ctr[1];
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < m; s += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(s + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        int64_t r = (int64_t)((z >> 20) % (uint64_t)n);
        const int b = (int)((z & 0xFFFFF) % (uint64_t)nv);
        if ((s & 1) && cdf) {
            const double* c = cdf + (int64_t)b * n;
            const double u = (double)(r + 0.5) / (double)n * c[n - 1];
            int64_t lo = 0, hi = n - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (c[mid] > u) hi = mid;
                else lo = mid + 1;
            }
            r = lo;
        }
        const double a = psi[r * nv + b];
        words[s] = basis[r];
        v1[s] = v1s[b];
        target[2 * s] = (float)fmax(log(fabs(a) + 1e-300), -40.0);
        target[2 * s + 1] = a >= 0.0 ? 1.f : 0.f;
    }
}

// warm start: V0[r][b] = sign * exp(logamp - shift_b); shift per problem
// keeps exp in range, normalisation follows in the solver
__global__ void k_psi_from_out(const float* __restrict__ out, int64_t n, int B, int b, const float* __restrict__ shift,
                               double* __restrict__ V0)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const float y0 = out[r * kOut], y1 = out[r * kOut + 1];
        const double a = exp((double)y0 - (double)shift[0]);
        V0[r * B + b] = y1 >= 0.f ? a : -a;
    }
}

__global__ void k_max_col0(const float* __restrict__ out, int64_t n, float* __restrict__ mx)
{
    __shared__ float red[256];
    float m = -3.0e38f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, out[r * kOut]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = 128; s; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // float atomic max through the ordered-int trick (values may be negative)
        int* addr = reinterpret_cast<int*>(mx);
        float v = red[0];
        int old = *addr;
        while (true) {
            const float cur = __int_as_float(old);
            if (cur >= v) break;
            const int prev = atomicCAS(addr, old, __float_as_int(v));
            if (prev == old) break;
            old = prev;
        }
    }
}

int grid_sz(int64_t work)
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)s * 8, (work + 255) / 256));
}

}  // namespace

}  // namespace edgb

struct ed_mlp {
    int norb = 0, H = 0;
    int dims[edgb::kLayers + 1];          // 32, H, H, H, 8
    int64_t woff[edgb::kLayers], boff[edgb::kLayers], nparam = 0;
    edgb::DevBuf<float> p, g, m1, m2;    // all parameters (weights then bias per layer)
    edgb::DevBuf<__nv_bfloat16> pb;      // bf16 copies (weights only used)
    edgb::DevBuf<int64_t> ctr;           // [0] Adam step, [1] fit step (device-side)
    edgb::DevBuf<float> ws, ws2;         // split-K and column-sum partials
    // activations sized for the largest batch seen
    int64_t cap = 0;
    edgb::DevBuf<__nv_bfloat16> X, Hb[3], dZb[4];
    edgb::DevBuf<float> Z[4], dZf[4];
    edgb::DevBuf<uint64_t> words;
    edgb::DevBuf<float> v1, target;
    edgb::DevBuf<double> loss;
};

namespace edgb {

namespace {

void mlp_reserve(ed_mlp& net, int64_t m)
{
    if (m <= net.cap) return;
    net.X.alloc((size_t)m * kIn);
    for (int l = 0; l < 3; ++l) net.Hb[l].alloc((size_t)m * net.H);
    for (int l = 0; l < 4; ++l) {
        const int w = net.dims[l + 1];
        net.Z[l].alloc((size_t)m * w);
        net.dZf[l].alloc((size_t)m * w);
        net.dZb[l].alloc((size_t)m * w);
    }
    net.words.alloc(m);
    net.v1.alloc(m);
    net.target.alloc((size_t)2 * m);
    net.loss.alloc(1);
    net.cap = m;
}

// forward for m samples whose features are already in net.X; Z[3] holds the outputs
void mlp_forward(ed_mlp& net, int64_t m, cudaStream_t st)
{
    const bf16* in = net.X.p;
    int ldin = kIn;
    for (int l = 0; l < kLayers; ++l) {
        const int K = net.dims[l], N = net.dims[l + 1];
        EpiForward e{net.p.p + net.boff[l], net.Z[l].p, l < 3 ? net.Hb[l].p : nullptr, N};
        gemm(in, ldin, 1, net.pb.p + net.woff[l], N, 1, (int)m, N, K, e, st);
        if (l < 3) {
            in = net.Hb[l].p;
            ldin = N;
        }
    }
}

constexpr int kMaxSplits = 16;

// backward from dZ[3] (set by the loss) into net.g.  The weight gradients
// reduce over the m samples: split-K GEMMs (up to 16 splits of >= 512
// samples) whose partials k_sum_splits adds in order; the bias gradients are
// coalesced column sums over up to 16 row chunks.
void mlp_backward(ed_mlp& net, int64_t m, cudaStream_t st)
{
    const int S = (int)std::max<int64_t>(1, std::min<int64_t>(kMaxSplits, m / 512));
    const int R = (int)std::max<int64_t>(1, std::min<int64_t>(kMaxSplits, m / 256));
    for (int l = kLayers - 1; l >= 0; --l) {
        const int K = net.dims[l], N = net.dims[l + 1];
        // dW_l = in^T dZ_l  (K x N), reduction over the m samples
        const bf16* in = l == 0 ? net.X.p : net.Hb[l - 1].p;
        const int ldin = l == 0 ? kIn : net.dims[l];
        EpiSplit es{net.ws.p, N, (int64_t)K * N};
        gemm(in, 1, ldin, net.dZb[l].p, N, 1, K, N, (int)m, es, st, S);
        k_sum_splits<<<grid_sz((int64_t)K * N), 256, 0, st>>>(net.ws.p, S, (int64_t)K * N, net.g.p + net.woff[l]);
        count_launch();
        k_colsum_part<<<dim3((unsigned)((N + 31) / 32), (unsigned)R), 256, 0, st>>>(net.dZf[l].p, m, N, net.ws2.p);
        count_launch();
        k_sum_splits<<<grid_sz(N), 256, 0, st>>>(net.ws2.p, R, N, net.g.p + net.boff[l]);
        count_launch();
        if (l > 0) {
            // dZ_{l-1} = (dZ_l W_l^T) * SiLU'(Z_{l-1})
            EpiBackData eb{net.Z[l - 1].p, net.dZb[l - 1].p, net.dZf[l - 1].p, K};
            gemm(net.dZb[l].p, N, 1, net.pb.p + net.woff[l], 1, N, (int)m, K, N, eb, st);
        }
    }
}

void mlp_features(ed_mlp& net, const uint64_t* words, const float* v1, int64_t m, cudaStream_t st)
{
    k_features<<<grid_sz(m * kIn), 256, 0, st>>>(words, v1, m, net.norb, net.X.p);
    count_launch();
}

double mlp_loss(ed_mlp& net, const float* target, int64_t m, cudaStream_t st)
{
    ED_CUDA(cudaMemsetAsync(net.loss.p, 0, 8, st));
    k_loss_grad<<<grid_sz(m), 256, 0, st>>>(net.Z[3].p, target, m, net.dZb[3].p, net.dZf[3].p, net.loss.p);
    count_launch();
    double l = 0.0;
    ED_CUDA(cudaMemcpyAsync(&l, net.loss.p, 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    return l / (double)m;
}

void mlp_adam(ed_mlp& net, float lr, int64_t fit_total, cudaStream_t st)
{
    k_advance<<<1, 1, 0, st>>>(net.ctr.p);
    count_launch();
    k_adam<<<grid_sz(net.nparam), 256, 0, st>>>(net.p.p, net.g.p, net.m1.p, net.m2.p, net.pb.p, net.nparam, lr,
                                                net.ctr.p, fit_total, 0.9f, 0.999f, 1e-8f);
    count_launch();
}

}  // namespace

}  // namespace edgb

using namespace edgb;

extern "C" {

ed_status ed_mlp_create(int norb, int hidden, uint64_t seed, ed_mlp** out)
{
    return guard([&] {
        ED_REQUIRE(out, ED_ERR_ARG, "NULL output");
        ED_REQUIRE(norb >= 2 && norb < kIn && norb <= kMaxOrbitals, ED_ERR_RANGE, "orbital count out of range");
        ED_REQUIRE(hidden >= 64 && hidden % 64 == 0 && hidden <= 1024, ED_ERR_ARG, "hidden width: multiple of 64");
        ed_mlp* net = new ed_mlp();
        try {
            net->norb = norb;
            net->H = hidden;
            const int d[kLayers + 1] = {kIn, hidden, hidden, hidden, kOut};
            int64_t off = 0;
            for (int l = 0; l <= kLayers; ++l) net->dims[l] = d[l];
            for (int l = 0; l < kLayers; ++l) {
                net->woff[l] = off;
                off += (int64_t)d[l] * d[l + 1];
                net->boff[l] = off;
                off += d[l + 1];
            }
            net->nparam = off;
            std::vector<float> h(off, 0.f);
            std::mt19937_64 rng(seed);
            for (int l = 0; l < kLayers; ++l) {
                // He-style uniform initialisation for SiLU layers, small output layer
                const float a = (l < 3 ? std::sqrt(6.f / d[l]) : 0.1f * std::sqrt(3.f / d[l]));
                std::uniform_real_distribution<float> U(-a, a);
                for (int64_t i = 0; i < (int64_t)d[l] * d[l + 1]; ++i) h[net->woff[l] + i] = U(rng);
            }
            net->p.alloc(off);
            net->g.alloc(off);
            net->m1.alloc(off);
            net->m2.alloc(off);
            net->pb.alloc(off);
            ED_CUDA(cudaMemcpy(net->p.p, h.data(), off * 4, cudaMemcpyHostToDevice));
            ED_CUDA(cudaMemset(net->m1.p, 0, off * 4));
            ED_CUDA(cudaMemset(net->m2.p, 0, off * 4));
            net->ctr.alloc(2);
            ED_CUDA(cudaMemset(net->ctr.p, 0, 2 * sizeof(int64_t)));
            net->ws.alloc((size_t)kMaxSplits * hidden * std::max(hidden, kIn));
            net->ws2.alloc((size_t)kMaxSplits * hidden);
            k_to_bf16<<<grid_sz(off), 256>>>(net->p.p, net->pb.p, off);
            count_launch();
            ED_CUDA(cudaDeviceSynchronize());
        } catch (...) {
            delete net;
            throw;
        }
        *out = net;
    });
}

ed_status ed_mlp_free(ed_mlp* net)
{
    return guard([&] { delete net; });
}

ed_status ed_mlp_num_params(const ed_mlp* net, int64_t* count)
{
    return guard([&] {
        ED_REQUIRE(net && count, ED_ERR_ARG, "NULL argument");
        *count = net->nparam;
    });
}

ed_status ed_mlp_get_params(const ed_mlp* net, float* host, int64_t count)
{
    return guard([&] {
        ED_REQUIRE(net && host && count == net->nparam, ED_ERR_ARG, "bad buffer");
        ED_CUDA(cudaMemcpy(host, net->p.p, count * 4, cudaMemcpyDeviceToHost));
    });
}

ed_status ed_mlp_set_params(ed_mlp* net, const float* host, int64_t count)
{
    return guard([&] {
        ED_REQUIRE(net && host && count == net->nparam, ED_ERR_ARG, "bad buffer");
        ED_CUDA(cudaMemcpy(net->p.p, host, count * 4, cudaMemcpyHostToDevice));
        k_to_bf16<<<grid_sz(count), 256>>>(net->p.p, net->pb.p, count);
        count_launch();
        ED_CUDA(cudaDeviceSynchronize());
    });
}

ed_status ed_mlp_forward(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, int64_t m, float* out_dev)
{
    return guard([&] {
        ED_REQUIRE(net && words_dev && v1_dev && out_dev && m >= 1, ED_ERR_ARG, "bad argument");
        mlp_reserve(*net, m);
        mlp_features(*net, words_dev, v1_dev, m, nullptr);
        mlp_forward(*net, m, nullptr);
        ED_CUDA(cudaMemcpyAsync(out_dev, net->Z[3].p, (size_t)m * kOut * 4, cudaMemcpyDeviceToDevice, nullptr));
        ED_CUDA(cudaStreamSynchronize(nullptr));
    });
}

ed_status ed_mlp_gradients(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, const float* target_dev,
                           int64_t m, float* grads_host, double* loss_host)
{
    return guard([&] {
        ED_REQUIRE(net && words_dev && v1_dev && target_dev && m >= 1, ED_ERR_ARG, "bad argument");
        mlp_reserve(*net, m);
        mlp_features(*net, words_dev, v1_dev, m, nullptr);
        mlp_forward(*net, m, nullptr);
        const double l = mlp_loss(*net, target_dev, m, nullptr);
        mlp_backward(*net, m, nullptr);
        if (grads_host) ED_CUDA(cudaMemcpy(grads_host, net->g.p, net->nparam * 4, cudaMemcpyDeviceToHost));
        if (loss_host) *loss_host = l;
        ED_CUDA(cudaStreamSynchronize(nullptr));
    });
}

ed_status ed_mlp_train_step(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, const float* target_dev,
                            int64_t m, float lr, double* loss_host)
{
    return guard([&] {
        ED_REQUIRE(net && words_dev && v1_dev && target_dev && m >= 1, ED_ERR_ARG, "bad argument");
        mlp_reserve(*net, m);
        mlp_features(*net, words_dev, v1_dev, m, nullptr);
        mlp_forward(*net, m, nullptr);
        const double l = mlp_loss(*net, target_dev, m, nullptr);
        mlp_backward(*net, m, nullptr);
        mlp_adam(*net, lr, 0, nullptr);
        if (loss_host) *loss_host = l;
    });
}

ed_status ed_mlp_fit(ed_mlp* net, const ed_basis* basis, const double* v1_host, int nv, const double* psi_dev,
                     int steps, int batch, float lr, uint64_t seed, double* final_loss)
{
    return guard([&] {
        ED_REQUIRE(net && basis && v1_host && psi_dev && nv >= 1 && steps >= 1 && batch >= 64, ED_ERR_ARG,
                   "bad argument");
        ED_REQUIRE(basis->norb == net->norb, ED_ERR_ARG, "basis and network have different orbital counts");
        mlp_reserve(*net, batch);
        std::vector<float> v1f(nv);
        for (int i = 0; i < nv; ++i) v1f[i] = (float)v1_host[i];
        DevBuf<float> dv1(nv);
        ED_CUDA(cudaMemcpy(dv1.p, v1f.data(), nv * 4, cudaMemcpyHostToDevice));
        // per-column cumulative |psi|^2 for the importance-sampled half
        const int64_t n = (int64_t)basis->dim;
        std::vector<double> hp((size_t)n * nv), hc((size_t)n * nv);
        ED_CUDA(cudaMemcpy(hp.data(), psi_dev, hp.size() * 8, cudaMemcpyDeviceToHost));
        // Sign gauge: an eigensolver returns each ground state with an arbitrary
        // overall sign, which would hand the sign output contradictory targets.
        // Taking the columns in V1 order, the first gets its largest component
        // positive and each later one the sign that overlaps its predecessor
        // positively (neighbouring V1 points have strongly overlapping ground
        // states away from level crossings).
        std::vector<int> order(nv);
        for (int b = 0; b < nv; ++b) order[b] = b;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return v1_host[x] < v1_host[y]; });
        std::vector<double> flip(nv, 1.0);
        for (int t = 0; t < nv; ++t) {
            const int b = order[t];
            double s = 0.0;
            if (t == 0) {
                int64_t arg = 0;
                for (int64_t r = 1; r < n; ++r)
                    if (std::fabs(hp[(size_t)r * nv + b]) > std::fabs(hp[(size_t)arg * nv + b])) arg = r;
                s = hp[(size_t)arg * nv + b];
            } else {
                const int a = order[t - 1];
                for (int64_t r = 0; r < n; ++r) s += flip[a] * hp[(size_t)r * nv + a] * hp[(size_t)r * nv + b];
            }
            flip[b] = s < 0.0 ? -1.0 : 1.0;
        }
        for (int64_t r = 0; r < n; ++r)
            for (int b = 0; b < nv; ++b) hp[(size_t)r * nv + b] *= flip[b];
        DevBuf<double> psi_g(hp.size());
        ED_CUDA(cudaMemcpy(psi_g.p, hp.data(), hp.size() * 8, cudaMemcpyHostToDevice));
        for (int b = 0; b < nv; ++b) {
            double acc = 0.0;
            for (int64_t r = 0; r < n; ++r) {
                const double a = hp[(size_t)r * nv + b];
                acc += a * a;
                hc[(size_t)b * n + r] = acc;
            }
        }
        DevBuf<double> cdf(hc.size());
        ED_CUDA(cudaMemcpy(cdf.p, hc.data(), hc.size() * 8, cudaMemcpyHostToDevice));
        // One training step (batch draw, forward, loss, backward, Adam with
        // the rate decaying linearly to a tenth over the fit) reads its seed
        // and rates from the device counters, so it is captured once as a
        // CUDA graph on a private stream and replayed `steps` times.
        SolveStream ss(nullptr);
        cudaStream_t st = ss.s;
        ED_CUDA(cudaMemsetAsync(net->ctr.p + 1, 0, sizeof(int64_t), st));
        auto step = [&]() {
            k_make_batch<<<grid_sz(batch), 256, 0, st>>>(basis->words.p, n, psi_g.p, nv, dv1.p, cdf.p, batch, seed,
                                                         net->ctr.p, net->words.p, net->v1.p, net->target.p);
            count_launch();
            mlp_features(*net, net->words.p, net->v1.p, batch, st);
            mlp_forward(*net, batch, st);
            ED_CUDA(cudaMemsetAsync(net->loss.p, 0, 8, st));
            k_loss_grad<<<grid_sz(batch), 256, 0, st>>>(net->Z[3].p, net->target.p, batch, net->dZb[3].p,
                                                        net->dZf[3].p, net->loss.p);
            count_launch();
            mlp_backward(*net, batch, st);
            mlp_adam(*net, lr, steps, st);
        };
        const uint64_t c0 = launch_count();
        ED_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
        try {
            step();
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
        const cudaError_t ge = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ED_CUDA(ge);
        struct ExecGuard {
            cudaGraphExec_t e;
            ~ExecGuard() { cudaGraphExecDestroy(e); }
        } eg{exec};
        for (int s = 0; s < steps; ++s) {
            ED_CUDA(cudaGraphLaunch(exec, st));
            count_launches(kernels);
        }
        double l = 0.0;
        ED_CUDA(cudaMemcpyAsync(&l, net->loss.p, 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        l /= (double)batch;
        if (final_loss) *final_loss = l;
    });
}

ed_status ed_warm_start(ed_mlp* net, const ed_basis* basis, const double* v1_host, int nham, double* V0_dev)
{
    return guard([&] {
        ED_REQUIRE(net && basis && v1_host && V0_dev && nham >= 1, ED_ERR_ARG, "bad argument");
        ED_REQUIRE(basis->norb == net->norb, ED_ERR_ARG, "basis and network have different orbital counts");
        const int64_t n = (int64_t)basis->dim;
        ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "empty sector");
        const int64_t chunk = std::min<int64_t>(n, 1 << 20);
        mlp_reserve(*net, chunk);
        DevBuf<float> v1c(chunk), out((size_t)n * kOut), mx(1);
        for (int b = 0; b < nham; ++b) {
            const float vf = (float)v1_host[b];
            std::vector<float> fill(chunk, vf);
            ED_CUDA(cudaMemcpy(v1c.p, fill.data(), chunk * 4, cudaMemcpyHostToDevice));
            for (int64_t r0 = 0; r0 < n; r0 += chunk) {
                const int64_t m = std::min(chunk, n - r0);
                mlp_features(*net, basis->words.p + r0, v1c.p, m, nullptr);
                mlp_forward(*net, m, nullptr);
                ED_CUDA(cudaMemcpyAsync(out.p + r0 * kOut, net->Z[3].p, (size_t)m * kOut * 4, cudaMemcpyDeviceToDevice,
                                        nullptr));
            }
            const float neg = -3.0e38f;
            ED_CUDA(cudaMemcpy(mx.p, &neg, 4, cudaMemcpyHostToDevice));
            k_max_col0<<<grid_sz(n), 256>>>(out.p, n, mx.p);
            count_launch();
            k_psi_from_out<<<grid_sz(n), 256>>>(out.p, n, nham, b, mx.p, V0_dev);
            count_launch();
        }
        ED_CUDA(cudaDeviceSynchronize());
    });
}

}  // extern "C"
