// Complex Hermitian path of the interacting optical-flux-lattice model
// (optical_flux_lattice/interacting_ofl_model): SpinlessFermionHamiltonian
// <dcmplx> built from momentum-conserving array-format term tables over a
// momentum-sector basis, its product and its eigensolve.
//
// The tables come in the reference's own layout
// (interacting_ofl_model/term_tables.cpp:95-200): for the quartic terms, the
// unordered pair (k3, k4) is one triangular index t = t1*K + t2 - t1(t1+1)/2
// (t1 = min, t2 = max), k1 = kTable[t*K + k2], and V(k1,k2,k3,k4) =
// vTable[t*K + (k4 > k3 ? k1 : k2)]; the quadratic terms are diagonal energies
// E_k (QuadraticTermTables::GetEkk = vTable[k1], :59-65).  The host folds the
// four ordered terms of each pair hop into one complex weight
// (cterms_derive); the device build and product are in ed_build.cu and here.
//
// The eigensolver is a thick-restart Lanczos on complex vectors stored as
// (re, im) pairs, run like the real solver: each restart cycle is one CUDA
// graph in which every step (product, local three-term step, complex
// classical Gram-Schmidt against the whole basis with a DGKS-gated second
// pass, normalisation) keeps its scalars in device memory; the host reads the
// real projected matrix (alpha and beta of a Hermitian operator are real)
// once per cycle, solves it, and restarts by rotating the complex basis with
// the real Ritz coefficients.  It replaces ArpackWrapper's complex driver
// (the T = dcmplx branches of arpack_wrapper.hpp:255-937, znaupd_/zneupd_
// with WHICH "SR").
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "ed_fixed.cuh"
#include "ed_lanczos.h"

namespace edgb {

namespace {

typedef std::complex<double> cplx;

constexpr int kCThreads = 256;

int ofl_tri(int k3, int k4, int K)
{
    const int t1 = k4 > k3 ? k3 : k4, t2 = k4 > k3 ? k4 : k3;
    return t1 * K + t2 - t1 * (t1 + 1) / 2;
}

int csms()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

// y = M x for the full storage (both triangles): one FMA chain per lane and
// component, G lanes per row.
template <int G>
__global__ void __launch_bounds__(kCThreads) k_cspmv_full(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const double2* __restrict__ val,
                                                          const double2* __restrict__ x, double2* __restrict__ y,
                                                          int64_t n)
{
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + grp;
        const bool valid = r < n;
        const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
        double re = 0.0, im = 0.0;
        for (int64_t k = s + sub; k < e; k += G) {
            const double2 v = __ldcs(val + k);
            const double2 xc = __ldg(x + __ldcs(col + k));
            re = fma(v.x, xc.x, re);
            re = fma(-v.y, xc.y, re);
            im = fma(v.x, xc.y, im);
            im = fma(v.y, xc.x, im);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o, G);
            im += __shfl_xor_sync(0xffffffffu, im, o, G);
        }
        if (valid && sub == 0) y[r] = make_double2(re, im);
    }
}

// The same product on the integer pipes in exact fixed-point arithmetic (the
// real kernel's scheme, ed_fixed.cuh): the values' real and imaginary parts
// share one 58-bit exponent bound ea, x's parts another ex, each element is
// two limb pairs (16 bytes, as the FP64 value), and per element
//   re += ar xr - ai xi,  im += ar xi + ai xr
// takes 16 mad.wide.s32 into six int64 partial sums of U <= 4 elements,
// flushed into the lane's two 128-bit sums; the G lanes' sums are added
// exactly and rounded once to FP64 (rows of at most 1024 elements keep
// |S| < 2^127).  4 DFMA an element made the FP64 kernel FP64-bound at 2.6 TB/s.
template <int G, int U, int MINB = 1>
__global__ void __launch_bounds__(kCThreads, MINB) k_cspmv_fix(const int64_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ col,
                                                         const int4* __restrict__ aq, const int4* __restrict__ xq,
                                                         const int* __restrict__ xexp, int ea,
                                                         double2* __restrict__ y, int64_t n)
{
    // per element |r2| <= 2^57, |r1| < 2^60, |r0| < 2^61 (the same for im)
    static_assert(U >= 1 && U <= 4, "four elements' products fit the int64 partial sums");
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
        const int4* ap = aq + s;
        const int32_t* cp = col + s;
        __int128 sre = 0, sim = 0;
        for (int j0 = sub; j0 < len; j0 += G * U) {
            int4 av[U];
            int cc[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = j0 + u * G < len;
                av[u] = in ? __ldcs(ap + j0 + u * G) : make_int4(0, 0, 0, 0);
                cc[u] = in ? __ldcs(cp + j0 + u * G) : 0;
            }
            int4 xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) xv[u] = __ldg(xq + cc[u]);
            long long r2 = 0, r1 = 0, r0 = 0, i2 = 0, i1 = 0, i0 = 0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int2 ar = make_int2(av[u].x, av[u].y), ai = make_int2(av[u].z, av[u].w);
                const int2 nai = make_int2(-av[u].z, -av[u].w);
                const int2 xr = make_int2(xv[u].x, xv[u].y), xi = make_int2(xv[u].z, xv[u].w);
                fix_mac(ar, xr, r2, r1, r0);
                fix_mac(nai, xi, r2, r1, r0);
                fix_mac(ar, xi, i2, i1, i0);
                fix_mac(ai, xr, i2, i1, i0);
            }
            sre += fix_combine(r2, r1, r0);
            sim += fix_combine(i2, i1, i0);
        }
        long long rh = (long long)(sre >> 64), ih = (long long)(sim >> 64);
        unsigned long long rl = (unsigned long long)sre, il = (unsigned long long)sim;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            const long long orh = __shfl_xor_sync(0xffffffffu, rh, o, G), oih = __shfl_xor_sync(0xffffffffu, ih, o, G);
            const unsigned long long orl = __shfl_xor_sync(0xffffffffu, rl, o, G);
            const unsigned long long oil = __shfl_xor_sync(0xffffffffu, il, o, G);
            const unsigned long long tr = rl + orl, ti = il + oil;
            rh += orh + (tr < rl ? 1 : 0);
            ih += oih + (ti < il ? 1 : 0);
            rl = tr;
            il = ti;
        }
        if (valid && sub == 0) {
            const double nan = __longlong_as_double(0x7FF8000000000000ll);
            y[r] = finite ? make_double2(round_i128(((__int128)rh << 64) | (__int128)rl, sc),
                                         round_i128(((__int128)ih << 64) | (__int128)il, sc))
                          : make_double2(nan, nan);
        }
    }
}

// The reference's upper storage: y_i += A_ij x_j for the stored part and
// y_j += conj(A_ij) x_i for its mirror (sparse_linear_algebra.hpp:148-164).
// y must be zero on entry.
template <int G>
__global__ void __launch_bounds__(kCThreads) k_cspmv_upper(const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ col,
                                                           const double2* __restrict__ val,
                                                           const double2* __restrict__ x, double2* __restrict__ y,
                                                           int64_t n)
{
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + grp;
        const bool valid = r < n;
        const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
        const double2 xr = valid ? __ldg(x + r) : make_double2(0.0, 0.0);
        double re = 0.0, im = 0.0;
        for (int64_t k = s + sub; k < e; k += G) {
            const int c = __ldcs(col + k);
            const double2 v = __ldcs(val + k);
            const double2 xc = __ldg(x + c);
            re = fma(v.x, xc.x, re);
            re = fma(-v.y, xc.y, re);
            im = fma(v.x, xc.y, im);
            im = fma(v.y, xc.x, im);
            if (c != r) {
                atomicAdd(&y[c].x, v.x * xr.x + v.y * xr.y);
                atomicAdd(&y[c].y, v.x * xr.y - v.y * xr.x);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o, G);
            im += __shfl_xor_sync(0xffffffffu, im, o, G);
        }
        if (valid && sub == 0) {
            atomicAdd(&y[r].x, re);
            atomicAdd(&y[r].y, im);
        }
    }
}

__device__ __forceinline__ double cblock_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kCThreads / 32; ++i) s += red[i];
    return s;
}

__device__ __forceinline__ void cchunk(int64_t n, int nb, int b, int64_t& r0, int64_t& r1)
{
    const int64_t per = (n + nb - 1) / nb;
    r0 = (int64_t)b * per;
    r1 = r0 + per < n ? r0 + per : n;
    if (r0 > n) r0 = n;
}

constexpr double kCDgksEta = 0.7071067811865476;

__device__ __forceinline__ double cwarp_sum(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Completion of a reduction launch without a second kernel: every block calls
// this after writing its partials; it returns true in exactly one block, the
// last to arrive, which then sees every block's partials and resets the
// counter for the next launch.  Nothing waits on another block.
__device__ __forceinline__ bool clast_block(unsigned int* counter)
{
    __shared__ unsigned int ticket;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
    __syncthreads();
    const bool last = ticket == gridDim.x - 1;
    if (last) {
        __threadfence();
        if (threadIdx.x == 0) *counter = 0u;
    }
    return last;
}

// Sum of nb partials (stride st) in a fixed order, whichever block runs it; in
// thread 0.
__device__ __forceinline__ double csum_parts(const double* p, int nb, int stride, double* red)
{
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kCThreads) s += __ldcg(p + (int64_t)i * stride);
    return cblock_sum(s, red);
}

// Local step scalars of step j (w = H v_j): alpha = Re v_j^H w into
// coefcol[j] (a Hermitian operator's alpha is real), beta_{j-1} into
// coefcol[j-1], ||w||^2 into *hv2; the last block writes them.
__global__ void __launch_bounds__(kCThreads) k_clocal(const double2* __restrict__ vj, const double2* __restrict__ w,
                                                      int64_t n, double* __restrict__ part,
                                                      unsigned int* __restrict__ counter, double* __restrict__ coefcol,
                                                      int j, const double* __restrict__ beta_prev,
                                                      double* __restrict__ hv2, const int* __restrict__ stop)
{
    if (*stop) return;
    __shared__ double red[kCThreads / 32];
    int64_t r0, r1;
    cchunk(n, gridDim.x, blockIdx.x, r0, r1);
    double a = 0.0, b = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
        const double2 v = vj[r], x = w[r];
        a = fma(v.x, x.x, a);
        a = fma(v.y, x.y, a);
        b = fma(x.x, x.x, b);
        b = fma(x.y, x.y, b);
    }
    a = cblock_sum(a, red);
    b = cblock_sum(b, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
    if (!clast_block(counter)) return;
    a = csum_parts(part, gridDim.x, 1, red);
    b = csum_parts(part + gridDim.x, gridDim.x, 1, red);
    if (threadIdx.x == 0) {
        coefcol[j] = a;
        coefcol[j - 1] = *beta_prev;
        *hv2 = b;
    }
}

// Complex multi-dot against the Krylov basis, R rows per block (R double2 of
// dynamic shared memory hold the block's slice of w): the block's shares of
// V_i^H w (i < J) and of ||w||^2 go to part[(i*nb + b)*2 + {re, im}].  With
// local != 0 the three-term step w -= alpha v_{J-1} + beta v_{J-2} (real
// alpha, beta) is applied to the slice while it is staged and written back.
// Warps take the columns in turn, eight loads per lane in flight.  The last
// block sums the partials column by column in a fixed order: c[i] (i < J;
// Re c[i] also added to coefcol[i] when coefcol is given) and *before =
// ||w||^2.  Runs when run is null or *run != 0, and stop is clear.
__global__ void __launch_bounds__(kCThreads) k_cmdot(const double2* __restrict__ V, int64_t n, int R, int J,
                                                     double2* __restrict__ w, int local,
                                                     const double* __restrict__ alpha,
                                                     const double* __restrict__ beta_prev, double* __restrict__ part,
                                                     unsigned int* __restrict__ counter, double2* __restrict__ c,
                                                     double* __restrict__ coefcol, double* __restrict__ before,
                                                     const int* __restrict__ run, const int* __restrict__ stop)
{
    if ((run && !*run) || (stop && *stop)) return;
    extern __shared__ double2 csw[];
    const int64_t r0 = (int64_t)blockIdx.x * R;
    const int len = (int)min((int64_t)R, n - r0);
    if (local) {
        const double a = *alpha, b = *beta_prev;
        const double2* vj = V + (int64_t)(J - 1) * n + r0;
        const double2* vjm1 = V + (int64_t)(J - 2) * n + r0;
        for (int i = threadIdx.x; i < len; i += kCThreads) {
            const double2 p = vj[i], q = vjm1[i];
            double2 x = w[r0 + i];
            x.x = fma(-b, q.x, fma(-a, p.x, x.x));
            x.y = fma(-b, q.y, fma(-a, p.y, x.y));
            w[r0 + i] = x;
            csw[i] = x;
        }
    } else {
        for (int i = threadIdx.x; i < len; i += kCThreads) csw[i] = w[r0 + i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nb = gridDim.x;
    for (int i = warp; i <= J; i += kCThreads / 32) {
        double re0 = 0.0, re1 = 0.0, im0 = 0.0, im1 = 0.0;
        int r = lane;
        if (i < J) {
            const double2* col = V + (int64_t)i * n + r0;
            for (; r + 224 < len; r += 256) {
                double2 x[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) x[u] = col[r + 32 * u];
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    const double2 s0 = csw[r + 32 * u], s1 = csw[r + 32 * (u + 1)];
                    re0 = fma(x[u].x, s0.x, re0);
                    re0 = fma(x[u].y, s0.y, re0);
                    im0 = fma(x[u].x, s0.y, im0);
                    im0 = fma(-x[u].y, s0.x, im0);
                    re1 = fma(x[u + 1].x, s1.x, re1);
                    re1 = fma(x[u + 1].y, s1.y, re1);
                    im1 = fma(x[u + 1].x, s1.y, im1);
                    im1 = fma(-x[u + 1].y, s1.x, im1);
                }
            }
            for (; r < len; r += 32) {
                const double2 x = col[r], s0 = csw[r];
                re0 = fma(x.x, s0.x, re0);
                re0 = fma(x.y, s0.y, re0);
                im0 = fma(x.x, s0.y, im0);
                im0 = fma(-x.y, s0.x, im0);
            }
        } else {
            for (; r < len; r += 32) {
                const double2 s0 = csw[r];
                re0 = fma(s0.x, s0.x, re0);
                re0 = fma(s0.y, s0.y, re0);
            }
        }
        const double re = cwarp_sum(re0 + re1), im = cwarp_sum(im0 + im1);
        if (lane == 0) {
            part[((int64_t)i * nb + blockIdx.x) * 2] = re;
            part[((int64_t)i * nb + blockIdx.x) * 2 + 1] = im;
        }
    }
    if (!clast_block(counter)) return;
    for (int i = warp; i <= J; i += kCThreads / 32) {
        double re = 0.0, im = 0.0;
        for (int b = lane; b < nb; b += 32) {
            re += __ldcg(part + ((int64_t)i * nb + b) * 2);
            im += __ldcg(part + ((int64_t)i * nb + b) * 2 + 1);
        }
        re = cwarp_sum(re);
        im = cwarp_sum(im);
        if (lane == 0) {
            if (i < J) {
                c[i] = make_double2(re, im);
                if (coefcol) coefcol[i] += re;
            } else {
                *before = re;
            }
        }
    }
}

// w -= V[:, 0..J) c (complex c) and a per-block partial of ||w||^2.  The last
// block then finishes the pass:
//   mode 1 (first pass): *need2 = force2 or ||w||^2 < eta^2 *before (the
//          DGKS test); without a second pass also beta and the breakdown test;
//   mode 2 (second pass): beta and the breakdown test;
//   mode 0: nothing (the counter is not touched).
// beta = ||w||; breakdown (stop = j + 1) when beta <= 1e-12 sqrt(*ref2).
__global__ void __launch_bounds__(kCThreads) k_cupd(const double2* __restrict__ V, int64_t n, int J,
                                                    const double2* __restrict__ c, double2* __restrict__ w,
                                                    double* __restrict__ npart, unsigned int* __restrict__ counter,
                                                    int mode, int force2, const double* __restrict__ before,
                                                    int* __restrict__ need2, double* __restrict__ beta,
                                                    const double* __restrict__ ref2, int j,
                                                    const int* __restrict__ run, int* __restrict__ stop)
{
    if ((run && !*run) || (stop && *stop)) return;
    extern __shared__ double2 cc[];
    __shared__ double red[kCThreads / 32];
    for (int i = threadIdx.x; i < J; i += kCThreads) cc[i] = c[i];
    __syncthreads();
    int64_t r0, r1;
    cchunk(n, gridDim.x, blockIdx.x, r0, r1);
    double nn = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
        double2 a = w[r], b = make_double2(0.0, 0.0);
        int i = 0;
        for (; i + 4 <= J; i += 4) {
            double2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = V[(int64_t)(i + u) * n + r];
#pragma unroll
            for (int u = 0; u < 4; u += 2) {
                const double2 c0 = cc[i + u], c1 = cc[i + u + 1];
                a.x = fma(-c0.x, v[u].x, a.x);
                a.x = fma(c0.y, v[u].y, a.x);
                a.y = fma(-c0.x, v[u].y, a.y);
                a.y = fma(-c0.y, v[u].x, a.y);
                b.x = fma(-c1.x, v[u + 1].x, b.x);
                b.x = fma(c1.y, v[u + 1].y, b.x);
                b.y = fma(-c1.x, v[u + 1].y, b.y);
                b.y = fma(-c1.y, v[u + 1].x, b.y);
            }
        }
        for (; i < J; ++i) {
            const double2 v = V[(int64_t)i * n + r], c0 = cc[i];
            a.x = fma(-c0.x, v.x, a.x);
            a.x = fma(c0.y, v.y, a.x);
            a.y = fma(-c0.x, v.y, a.y);
            a.y = fma(-c0.y, v.x, a.y);
        }
        a.x += b.x;
        a.y += b.y;
        w[r] = a;
        nn = fma(a.x, a.x, nn);
        nn = fma(a.y, a.y, nn);
    }
    nn = cblock_sum(nn, red);
    if (threadIdx.x == 0) npart[blockIdx.x] = nn;
    if (mode == 0 || !clast_block(counter)) return;
    const double s = csum_parts(npart, gridDim.x, 1, red);
    if (threadIdx.x == 0) {
        bool finish = true;
        if (mode == 1) {
            const int again = (force2 || s < kCDgksEta * kCDgksEta * (*before)) ? 1 : 0;
            *need2 = again;
            finish = !again;
        }
        if (finish) {
            const double b = sqrt(s);
            *beta = b;
            if (!(b > 1e-12 * sqrt(fmax(*ref2, 0.0)))) *stop = j + 1;
        }
    }
}

// w /= *beta unless the cycle stopped.
__global__ void __launch_bounds__(kCThreads) k_cscale_dev(double2* __restrict__ w, int64_t n,
                                                          const double* __restrict__ beta, const int* __restrict__ stop)
{
    if (*stop) return;
    const double inv = 1.0 / *beta;
    for (int64_t r = blockIdx.x * (int64_t)kCThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kCThreads) {
        double2 a = w[r];
        a.x *= inv;
        a.y *= inv;
        w[r] = a;
    }
}

__global__ void __launch_bounds__(kCThreads) k_cnorm2(const double2* __restrict__ w, int64_t n, double* __restrict__ part)
{
    __shared__ double red[kCThreads / 32];
    int64_t r0, r1;
    cchunk(n, gridDim.x, blockIdx.x, r0, r1);
    double s = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
        const double2 a = w[r];
        s = fma(a.x, a.x, s);
        s = fma(a.y, a.y, s);
    }
    s = cblock_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kCThreads) k_cscale(double2* __restrict__ w, int64_t n, double s)
{
    for (int64_t r = blockIdx.x * (int64_t)kCThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kCThreads) {
        double2 a = w[r];
        a.x *= s;
        a.y *= s;
        w[r] = a;
    }
}

// Seeded uniform(-1,1) real and imaginary parts (splitmix64 of seed and index).
__global__ void k_crandom(double* __restrict__ v, int64_t m, uint64_t seed)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(r + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v[r] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    }
}

// ||y - lambda x||^2 partials.
__global__ void __launch_bounds__(kCThreads) k_cresid(const double2* __restrict__ y, const double2* __restrict__ x,
                                                      double lambda, int64_t n, double* __restrict__ part)
{
    __shared__ double red[kCThreads / 32];
    int64_t r0, r1;
    cchunk(n, gridDim.x, blockIdx.x, r0, r1);
    double s = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
        const double2 a = y[r], b = x[r];
        const double dx = fma(-lambda, b.x, a.x), dy = fma(-lambda, b.y, a.y);
        s = fma(dx, dx, s);
        s = fma(dy, dy, s);
    }
    s = cblock_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

std::vector<double> host_parts(const DevBuf<double>& part, size_t count, cudaStream_t st)
{
    std::vector<double> h(count);
    ED_CUDA(cudaMemcpyAsync(h.data(), part.p, count * 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    return h;
}

// Working state of one complex solve: reduction partials, the projected
// matrix's columns as the device accumulates them (coef, (m+1) per step),
// beta, the current pass's coefficients, the step scalars (scal: 0 ||w||^2
// before the first pass, 1 ||H v_j||^2, 2 before the second pass, 3 scratch)
// and the flags (need2, stop) and completion counters of the cycle's kernels.
struct CWork {
    int64_t n = 0;
    int m = 0;
    int nb = 1;            // blocks of the row-chunked kernels
    int R = 512, nbm = 1;  // multi-dot: rows per block, blocks
    DevBuf<double> part, npart, coef, beta, c, scal;
    DevBuf<int> flags;
    DevBuf<unsigned int> counters;

    void mdot(const double2* V, int J, double2* w, int local, const double* alpha, const double* beta_prev,
              double* coefcol, double* before, const int* run, const int* stop, cudaStream_t st)
    {
        k_cmdot<<<nbm, kCThreads, (size_t)R * 16, st>>>(V, n, R, J, w, local, alpha, beta_prev, part.p,
                                                        counters.p + 1, reinterpret_cast<double2*>(c.p), coefcol,
                                                        before, run, stop);
        count_launch();
    }
    void update(const double2* V, int J, double2* w, int mode, int force2, const double* before, int* need2,
                double* b, const double* ref2, int j, const int* run, int* stop, cudaStream_t st)
    {
        k_cupd<<<nb, kCThreads, (size_t)J * 16, st>>>(V, n, J, reinterpret_cast<const double2*>(c.p), w, npart.p,
                                                      counters.p + 2, mode, force2, before, need2, b, ref2, j, run,
                                                      stop);
        count_launch();
    }
};

double cnorm(CWork& cw, const double2* w, cudaStream_t st)
{
    k_cnorm2<<<cw.nb, kCThreads, 0, st>>>(w, cw.n, cw.part.p);
    count_launch();
    ED_CUDA(cudaGetLastError());
    const std::vector<double> h = host_parts(cw.part, cw.nb, st);
    double s = 0.0;
    for (double v : h) s += v;
    return std::sqrt(s);
}

void cscale(double2* w, int64_t n, double s, cudaStream_t st)
{
    k_cscale<<<csms() * 4, kCThreads, 0, st>>>(w, n, s);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

// Orthogonalise column col of V against columns [0, col) twice, then
// normalise it; fails on a zero or non-finite result.
void corthonormalise(CWork& cw, double2* V, int col, cudaStream_t st)
{
    double2* x = V + (int64_t)col * cw.n;
    for (int pass = 0; col > 0 && pass < 2; ++pass) {
        cw.mdot(V, col, x, 0, nullptr, nullptr, nullptr, cw.scal.p + 3, nullptr, nullptr, st);
        cw.update(V, col, x, 0, 0, nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr, st);
        ED_CUDA(cudaGetLastError());
    }
    const double nrm = cnorm(cw, x, st);
    ED_REQUIRE(nrm > 0.0 && std::isfinite(nrm), ED_ERR_ARG, "start vector is zero or not finite");
    cscale(x, cw.n, 1.0 / nrm, st);
}

// Dense path (dimension below 60, as the real solver): M applied to the unit
// vectors, the real symmetric embedding [[Re M, -Im M], [Im M, Re M]] solved on
// the host, whose eigenvalues come in pairs; one complex vector per pair is
// kept, complex-orthogonalised against those already kept.
void cdense_solve(const ed_ccrs& a, int nev, double* evals, double* evecs_dev, ed_solve_info* info, cudaStream_t st)
{
    const int64_t n = a.n;
    DevBuf<double> X(2 * (size_t)n), Y(2 * (size_t)n);
    std::vector<cplx> M((size_t)n * n);
    std::vector<double> e(2 * (size_t)n, 0.0), y(2 * (size_t)n);
    for (int64_t j = 0; j < n; ++j) {
        std::fill(e.begin(), e.end(), 0.0);
        e[2 * j] = 1.0;
        ED_CUDA(cudaMemcpyAsync(X.p, e.data(), e.size() * 8, cudaMemcpyHostToDevice, st));
        cspmv(a, X.p, Y.p, st);
        ED_CUDA(cudaMemcpyAsync(y.data(), Y.p, y.size() * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int64_t i = 0; i < n; ++i) M[(size_t)i * n + j] = cplx(y[2 * i], y[2 * i + 1]);
    }
    const int m = (int)(2 * n);
    std::vector<double> R((size_t)m * m);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < n; ++j) {
            // Hermitian part, against round-off
            const cplx h = 0.5 * (M[(size_t)i * n + j] + std::conj(M[(size_t)j * n + i]));
            R[(size_t)i * m + j] = h.real();
            R[(size_t)(i + n) * m + (j + n)] = h.real();
            R[(size_t)i * m + (j + n)] = -h.imag();
            R[(size_t)(i + n) * m + j] = h.imag();
        }
    std::vector<double> ev, vec;
    sym_eigen(m, R, ev, vec);
    std::vector<std::vector<cplx>> kept;
    std::vector<double> vals;
    for (int k = 0; k < m && (int)kept.size() < nev; ++k) {
        std::vector<cplx> u(n);
        for (int64_t i = 0; i < n; ++i) u[i] = cplx(vec[(size_t)m * k + i], vec[(size_t)m * k + n + i]);
        for (int pass = 0; pass < 2; ++pass)
            for (const auto& q : kept) {
                cplx d(0.0, 0.0);
                for (int64_t i = 0; i < n; ++i) d += std::conj(q[i]) * u[i];
                for (int64_t i = 0; i < n; ++i) u[i] -= d * q[i];
            }
        double nn = 0.0;
        for (const auto& z : u) nn += std::norm(z);
        if (nn < 0.25) continue;   // the partner (i times a kept vector) of an earlier pair
        const double s = 1.0 / std::sqrt(nn);
        for (auto& z : u) z *= s;
        kept.push_back(u);
        vals.push_back(ev[k]);
    }
    ED_REQUIRE((int)kept.size() == nev, ED_ERR_INTERNAL, "complex dense path lost eigenvectors");
    for (int i = 0; i < nev; ++i) evals[i] = vals[i];
    if (evecs_dev) {
        std::vector<double> h(2 * (size_t)n * nev);
        for (int i = 0; i < nev; ++i)
            for (int64_t r = 0; r < n; ++r) {
                h[2 * ((size_t)i * n + r)] = kept[i][r].real();
                h[2 * ((size_t)i * n + r) + 1] = kept[i][r].imag();
            }
        ED_CUDA(cudaMemcpyAsync(evecs_dev, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st));
        ED_CUDA(cudaStreamSynchronize(st));
    }
    if (info) {
        info->converged = nev;
        info->matvecs = n;
        info->max_residual = 0.0;
    }
}

}  // namespace

// ------------------------------------------------------------ terms

void cterms_derive(ed_cterms& t)
{
    const int K = t.norb, X = t.dimX, Y = t.dimY;
    ED_REQUIRE(K >= 2 && K <= kMaxOrbitals && X >= 1 && Y >= 1 && X * Y == K, ED_ERR_RANGE,
               "momentum grid: need dimX * dimY = norb in 2..40");
    const size_t tdim = (size_t)(K + 1) * K * K / 2;
    ED_REQUIRE(t.ktab.size() == tdim && t.vtab.size() == 2 * tdim, ED_ERR_ARG, "term tables of the wrong size");
    auto cls = [&](int a, int b) { return ((a / Y + b / Y) % X) * Y + (a % Y + b % Y) % Y; };
    auto K1 = [&](int k2, int k3, int k4) { return (int)t.ktab[(size_t)ofl_tri(k3, k4, K) * K + k2]; };
    auto V = [&](int k1, int k2, int k3, int k4) {
        const size_t i = (size_t)ofl_tri(k3, k4, K) * K + (k4 > k3 ? k1 : k2);
        return cplx(t.vtab[2 * i], t.vtab[2 * i + 1]);
    };
    // the device enumerates hops within momentum classes: accept only tables
    // whose k1 conserves the pair momentum (FindK1, interacting_ofl_model.cpp:366-410)
    for (int k4 = 0; k4 < K; ++k4)
        for (int k3 = 0; k3 < K; ++k3) {
            if (k3 == k4) continue;
            for (int k2 = 0; k2 < K; ++k2) {
                const int k1 = K1(k2, k3, k4);
                ED_REQUIRE(k1 < K && cls(k1, k2) == cls(k3, k4), ED_ERR_ARG,
                           "k-table does not conserve the 2D momentum (k1 + k2 = k3 + k4 modulo the grid)");
            }
        }
    const int C = X * Y;
    std::vector<std::vector<int>> lists(C);
    t.pair_index.assign((size_t)K * K, -1);
    for (int a = 0; a < K; ++a)
        for (int b = a + 1; b < K; ++b) {
            const int P = cls(a, b);
            t.pair_index[(size_t)a * K + b] = (int)lists[P].size();
            lists[P].push_back(a | (b << 8));
        }
    t.cls_off.assign(C + 1, 0);
    t.w_off.assign(C + 1, 0);
    t.pairs.clear();
    for (int P = 0; P < C; ++P) {
        t.cls_off[P + 1] = t.cls_off[P] + (int)lists[P].size();
        t.w_off[P + 1] = t.w_off[P] + (int)(lists[P].size() * lists[P].size());
        for (int pr : lists[P]) t.pairs.push_back((uint16_t)pr);
    }
    t.w.assign(2 * (size_t)t.w_off[C], 0.0);
    auto keep = [](const cplx& z) { return std::abs(z) > kSparseZeroTol; };
    for (int P = 0; P < C; ++P) {
        const int m = (int)lists[P].size();
        for (int ia = 0; ia < m; ++ia) {
            const int a = lists[P][ia] & 255, b = lists[P][ia] >> 8;
            for (int ic = 0; ic < m; ++ic) {
                const int c = lists[P][ic] & 255, d = lists[P][ic] >> 8;
                if (c == a || c == b || d == a || d == b) continue;
                // visiting order: k4=a,k3=b (k2=c then k2=d), then k4=b,k3=a;
                // relative signs +,-,-,+
                cplx acc(0.0, 0.0);
                const struct { int k1, k2, k3, k4; double s; } terms[4] = {
                    {d, c, b, a, 1.0}, {c, d, b, a, -1.0}, {d, c, a, b, -1.0}, {c, d, a, b, 1.0}};
                for (const auto& q : terms) {
                    if (K1(q.k2, q.k3, q.k4) != q.k1) continue;
                    const cplx term = q.s * V(q.k1, q.k2, q.k3, q.k4);
                    if (keep(term)) acc = acc + term;
                }
                if (std::abs(acc) < kSparseZeroTol) acc = cplx(0.0, 0.0);   // the trim
                const size_t o = (size_t)t.w_off[P] + (size_t)ia * m + ic;
                t.w[2 * o] = acc.real();
                t.w[2 * o + 1] = acc.imag();
            }
        }
    }
    t.da.assign(2 * (size_t)K * K, 0.0);
    t.db.assign(2 * (size_t)K * K, 0.0);
    for (int k4 = 0; k4 < K; ++k4)
        for (int k3 = 0; k3 < K; ++k3) {
            if (k3 == k4) continue;
            cplx tA(0.0, 0.0), tB(0.0, 0.0);
            if (K1(k3, k3, k4) == k4) tA = V(k4, k3, k3, k4);          // k2 = k3, k1 = k4: sign +1
            if (K1(k4, k3, k4) == k3) tB = -V(k3, k4, k3, k4);         // k2 = k4, k1 = k3: sign -1
            if (!keep(tA)) tA = cplx(0.0, 0.0);
            if (!keep(tB)) tB = cplx(0.0, 0.0);
            const bool k3_first = k3 < k4;                             // k2 runs upward
            const cplx first = k3_first ? tA : tB, second = k3_first ? tB : tA;
            const size_t o = (size_t)k4 * K + k3;
            t.da[2 * o] = first.real();
            t.da[2 * o + 1] = first.imag();
            t.db[2 * o] = second.real();
            t.db[2 * o + 1] = second.imag();
        }
    if (t.e.size() != 2 * (size_t)K) t.e.assign(2 * (size_t)K, 0.0);
    for (int k = 0; k < K; ++k)
        if (!keep(cplx(t.e[2 * k], t.e[2 * k + 1]))) t.e[2 * k] = t.e[2 * k + 1] = 0.0;
    t.cls_off_dev.alloc(t.cls_off.size());
    t.w_off_dev.alloc(t.w_off.size());
    t.pair_index_dev.alloc(t.pair_index.size());
    t.pairs_dev.alloc(std::max<size_t>(1, t.pairs.size()));
    t.w_dev.alloc(std::max<size_t>(2, t.w.size()));
    t.da_dev.alloc(t.da.size());
    t.db_dev.alloc(t.db.size());
    t.e_dev.alloc(t.e.size());
    ED_CUDA(cudaMemcpy(t.cls_off_dev.p, t.cls_off.data(), t.cls_off.size() * sizeof(int), cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.w_off_dev.p, t.w_off.data(), t.w_off.size() * sizeof(int), cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.pair_index_dev.p, t.pair_index.data(), t.pair_index.size() * sizeof(int),
                       cudaMemcpyHostToDevice));
    if (!t.pairs.empty())
        ED_CUDA(cudaMemcpy(t.pairs_dev.p, t.pairs.data(), t.pairs.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    if (!t.w.empty()) ED_CUDA(cudaMemcpy(t.w_dev.p, t.w.data(), t.w.size() * 8, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.da_dev.p, t.da.data(), t.da.size() * 8, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.db_dev.p, t.db.data(), t.db.size() * 8, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.e_dev.p, t.e.data(), t.e.size() * 8, cudaMemcpyHostToDevice));
}

// ------------------------------------------------------------ product

namespace {

constexpr int kCFixMaxRow = 1024;   // |S| < 1024 * 2^117 = 2^127

int cfix_parts() { return csms() * 2; }

bool capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ED_CUDA(cudaStreamIsCapturing(st, &cs));
    return cs != cudaStreamCaptureStatusNone;
}

// The fixed-point copy of the values (declined when it would take more than
// half of the free device memory, for long rows or a non-finite value).
void cfix_build(const ed_ccrs& a, cudaStream_t st)
{
    size_t free_b = 0, total_b = 0;
    ED_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t need = (size_t)(a.nnz + kCrsPad) * 16 + (size_t)a.n * 16;
    if (a.upper || need > free_b / 2 || a.max_row > kCFixMaxRow) {
        a.fix_state = -1;
        return;
    }
    auto fq = std::make_unique<ed_fixq>();
    const int P = cfix_parts();
    DevBuf<int> part((size_t)P + 1);
    fq->val.alloc(2 * (size_t)(a.nnz + kCrsPad));
    ED_CUDA(cudaMemsetAsync(fq->val.p + 2 * a.nnz, 0, (size_t)kCrsPad * 16, st));
    k_fix_exp<<<P, 256, 0, st>>>(a.val.p, 2 * a.nnz, part.p);
    count_launch();
    k_fix_conv<<<csms() * 8, 256, 0, st>>>(a.val.p, 2 * a.nnz, part.p, P, fq->val.p);
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
    a.fixq = std::move(fq);
    a.fix_state = 1;
}

// This stream's scratch (x's 2n fixed-point words), made outside a capture.
ed_fixq::Scratch* cfix_scratch(const ed_ccrs& a, cudaStream_t st)
{
    ed_fixq& f = *a.fixq;
    int dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    const std::pair<int, cudaStream_t> key(dev, st);
    std::lock_guard<std::mutex> lk(f.mu);
    auto it = f.scratch.find(key);
    if (it != f.scratch.end()) return it->second.get();
    if (capturing(st)) return nullptr;
    auto sc = std::make_unique<ed_fixq::Scratch>();
    sc->xq.alloc(2 * (size_t)a.n);
    sc->part.alloc((size_t)cfix_parts() + 1);
    return f.scratch.emplace(key, std::move(sc)).first->second.get();
}

bool cfix_ready(const ed_ccrs& a, cudaStream_t st)
{
    if (a.fix_state == 0 && !capturing(st)) cfix_build(a, st);
    return a.fix_state == 1 && cfix_scratch(a, st) != nullptr;
}

void cfix_launch(const ed_ccrs& a, const double* x, double* y, cudaStream_t st)
{
    const ed_fixq& f = *a.fixq;
    ed_fixq::Scratch& sc = *cfix_scratch(a, st);
    const int P = cfix_parts();
    k_fix_exp<<<P, 256, 0, st>>>(x, 2 * a.n, sc.part.p);
    count_launch();
    k_fix_conv<<<csms() * 4, 256, 0, st>>>(x, 2 * a.n, sc.part.p, P, sc.xq.p);
    count_launch();
    const double avg = (double)a.nnz / (double)a.n;
    const int4* A = reinterpret_cast<const int4*>(f.val.p);
    const int4* X = reinterpret_cast<const int4*>(sc.xq.p);
    double2* yy = reinterpret_cast<double2*>(y);
    // 8 lanes a row, 4 elements ahead, at most 64 registers: four CTAs per SM
    // (GB300, N=10 on 5x6: 1.363 ms; 92 registers and two CTAs 1.77, 2
    // ahead 2.69, 16 lanes 2.72, 48 registers with spills 1.62; the FP64
    // kernel 2.31)
    if (avg >= 48) k_cspmv_fix<8, 4, 4><<<csms() * 8, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, A, X, sc.part.p + P, f.ea, yy, a.n);
    else k_cspmv_fix<4, 4, 4><<<csms() * 8, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, A, X, sc.part.p + P, f.ea, yy, a.n);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void cspmv_fp64(const ed_ccrs& a, const double* x, double* y, cudaStream_t st)
{
    const double avg = (double)a.nnz / (double)a.n;
    const int grid = csms() * 8;
    const double2* v = reinterpret_cast<const double2*>(a.val.p);
    const double2* xx = reinterpret_cast<const double2*>(x);
    double2* yy = reinterpret_cast<double2*>(y);
    if (!a.upper) {
        if (avg >= 48) k_cspmv_full<8><<<grid, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, v, xx, yy, a.n);
        else k_cspmv_full<4><<<grid, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, v, xx, yy, a.n);
    } else {
        ED_CUDA(cudaMemsetAsync(y, 0, (size_t)a.n * 16, st));
        if (avg >= 24) k_cspmv_upper<8><<<grid, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, v, xx, yy, a.n);
        else k_cspmv_upper<4><<<grid, kCThreads, 0, st>>>(a.rowptr.p, a.col.p, v, xx, yy, a.n);
    }
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace

void cspmv_prepare(const ed_ccrs& a, cudaStream_t st)
{
    if (a.n > 0 && !a.upper && !capturing(st)) cfix_ready(a, st);
}

// Full storage takes the integer-pipe kernel (made on first use outside a
// capture); the reference's upper storage and declined matrices the FP64 one.
void cspmv(const ed_ccrs& a, const double* x, double* y, cudaStream_t st)
{
    if (a.n == 0) return;
    if (!a.upper && cfix_ready(a, st)) {
        cfix_launch(a, x, y, st);
        return;
    }
    cspmv_fp64(a, x, y, st);
}

void cspmv_kernel(const ed_ccrs& a, int kernel, const double* x, double* y, cudaStream_t st)
{
    ED_REQUIRE(kernel >= 0 && kernel <= 2, ED_ERR_ARG,
               "kernel: 0 (chosen by storage), 1 (FP64 rows), 2 (fixed-point integer rows)");
    if (a.n == 0) return;
    if (kernel == 0) {
        cspmv(a, x, y, st);
        return;
    }
    if (kernel == 1) {
        cspmv_fp64(a, x, y, st);
        return;
    }
    ED_REQUIRE(!a.upper, ED_ERR_ARG, "the fixed-point kernel takes full storage");
    ED_REQUIRE(cfix_ready(a, st), ED_ERR_RANGE,
               "no fixed-point copy (a non-finite value, a row of more than 1024 elements, not enough free device "
               "memory, or a first product on this stream inside a capture)");
    cfix_launch(a, x, y, st);
}

// ------------------------------------------------------------ eigensolver

// Lowest p.nev eigenpairs of the Hermitian operator of `a` (complex vectors
// as (re, im) pairs; v0_dev 2n doubles or null; evecs_dev nev x 2n or null).
void clanczos_solve(const ed_ccrs& a, const ed_lanczos_params& p, const double* v0_dev, double* evals,
                    double* evecs_dev, ed_solve_info* info, cudaStream_t caller)
{
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t n = a.n;
    const int nev = p.nev;
    ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
    ED_REQUIRE(nev >= 1 && nev <= n, ED_ERR_ARG, "need 1 <= nev <= n");
    const double tol = p.tol > 0 ? p.tol : 1e-10;
    const int max_restarts = p.max_restarts > 0 ? p.max_restarts : 2000;
    ed_solve_info inf;
    std::memset(&inf, 0, sizeof(inf));
    SolveStream ss(caller);
    cudaStream_t st = ss.s;
    if (p.diagonal_check &&
        diagonal_spectrum(a.rowptr.p, a.col.p, a.val.p, 1, n, nev, evals, evecs_dev, info, st))
        return;
    cspmv_prepare(a, st);   // before the cycles are captured
    if (n < 60 || n <= (int64_t)nev + 2) {
        cdense_solve(a, nev, evals, evecs_dev, &inf, st);
        inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (info) *info = inf;
        return;
    }
    int64_t m64 = p.ncv > 0 ? p.ncv : std::min<int64_t>(n, 2 * (int64_t)nev + 21);
    m64 = std::max<int64_t>(m64, nev + 2);
    m64 = std::min<int64_t>(m64, n - 1);
    m64 = std::min<int64_t>(m64, 1000);
    const int m = (int)m64;
    const int nsm = csms();
    CWork cw;
    cw.n = n;
    cw.m = m;
    cw.nb = (int)std::max<int64_t>(1, std::min<int64_t>(nsm * 4, n / 1024));
    // multi-dot slices: three blocks per SM, 512 to 6144 rows (96 KB of
    // shared memory) a block, a multiple of 128
    {
        int64_t nbt = (int64_t)nsm * 3, R = 0;
        for (;;) {
            R = std::max<int64_t>(512, ((n + nbt - 1) / nbt + 127) / 128 * 128);
            if (R <= 6144) break;
            nbt += nsm;
        }
        cw.R = (int)R;
        cw.nbm = (int)((n + R - 1) / R);
        if ((size_t)R * 16 > 48 * 1024)
            ED_CUDA(cudaFuncSetAttribute(k_cmdot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(R * 16)));
    }
    cw.part.alloc((size_t)(m + 2) * std::max(cw.nb, cw.nbm) * 2);
    cw.npart.alloc(cw.nb);
    cw.coef.alloc((size_t)(m + 1) * (m + 1));
    cw.beta.alloc(m + 2);
    cw.c.alloc(2 * (size_t)(m + 2));
    cw.scal.alloc(4);
    cw.flags.alloc(2);
    cw.counters.alloc(4);
    ED_CUDA(cudaMemsetAsync(cw.beta.p, 0, (m + 2) * 8, st));
    ED_CUDA(cudaMemsetAsync(cw.counters.p, 0, 4 * sizeof(unsigned int), st));
    DevBuf<double> Vb(2 * (size_t)n * (m + 1)), V2b(2 * (size_t)n * (m + 1));
    auto col = [&](DevBuf<double>& B, int j) { return reinterpret_cast<double2*>(B.p + 2 * (size_t)n * j); };
    RotateScratch rot;
    if (v0_dev) ED_CUDA(cudaMemcpyAsync(Vb.p, v0_dev, 2 * (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    else {
        k_crandom<<<nsm * 4, kCThreads, 0, st>>>(Vb.p, 2 * n, p.seed);
        count_launch();
        ED_CUDA(cudaGetLastError());
    }
    corthonormalise(cw, col(Vb, 0), 0, st);

    std::vector<cudaEvent_t> ev(2 * (m + 1), nullptr);
    for (auto& e : ev) ED_CUDA(cudaEventCreate(&e));
    struct EvGuard {
        std::vector<cudaEvent_t>& v;
        ~EvGuard() { for (auto e : v) if (e) cudaEventDestroy(e); }
    } evguard{ev};

    // One restart cycle, steps k..m-1, all on the device (the real solver's
    // scheme): the step scalars stay in device memory, the second
    // Gram-Schmidt pass and a breakdown are flags that later kernels read, and
    // the cycle is replayed as one CUDA graph.
    int* need2 = cw.flags.p;
    int* stop = cw.flags.p + 1;
    auto enqueue_cycle = [&](double2* V, int k, bool capturing) {
        ED_CUDA(cudaMemsetAsync(cw.flags.p, 0, 2 * sizeof(int), st));
        ED_CUDA(cudaMemsetAsync(cw.coef.p + (size_t)k * (m + 1), 0, (size_t)(m - k) * (m + 1) * 8, st));
        for (int j = k; j < m; ++j) {
            double2* vj = V + (int64_t)j * n;
            double2* w = V + (int64_t)(j + 1) * n;
            double* coefcol = cw.coef.p + (size_t)j * (m + 1);
            const bool first = (j == k);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j], st));
            cspmv(a, reinterpret_cast<const double*>(vj), reinterpret_cast<double*>(w), st);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j + 1], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j + 1], st));
            if (!first) {
                k_clocal<<<cw.nb, kCThreads, 0, st>>>(vj, w, n, cw.part.p, cw.counters.p, coefcol, j,
                                                      cw.beta.p + (j - 1), cw.scal.p + 1, stop);
                count_launch();
            }
            const int J = j + 1;
            const double* ref2 = first ? cw.scal.p : cw.scal.p + 1;
            cw.mdot(V, J, w, first ? 0 : 1, first ? nullptr : coefcol + j, first ? nullptr : cw.beta.p + (j - 1),
                    coefcol, cw.scal.p, nullptr, stop, st);
            cw.update(V, J, w, 1, first ? 1 : 0, cw.scal.p, need2, cw.beta.p + j, ref2, j, nullptr, stop, st);
            cw.mdot(V, J, w, 0, nullptr, nullptr, coefcol, cw.scal.p + 2, need2, stop, st);
            cw.update(V, J, w, 2, 0, nullptr, nullptr, cw.beta.p + j, ref2, j, need2, stop, st);
            k_cscale_dev<<<cw.nb, kCThreads, 0, st>>>(w, n, cw.beta.p + j, stop);
            count_launch();
            ED_CUDA(cudaGetLastError());
        }
    };
    CycleGraphs cache;
    auto run_cycle = [&](int k) {
        double2* V = col(Vb, 0);
        CycleGraphs::Entry* g = cache.find(k, Vb.p);
        if (!g) {
            const uint64_t c0 = launch_count();
            ED_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            try {
                enqueue_cycle(V, k, true);
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
            cache.e.push_back({k, Vb.p, exec, kernels});
            g = &cache.e.back();
        }
        ED_CUDA(cudaGraphLaunch(g->exec, st));
        count_launches(g->kernels);
    };

    std::vector<double> T((size_t)m * m, 0.0), coef_h((size_t)(m + 1) * (m + 1)), beta_h(m + 1);
    std::vector<double> theta, Y, prev_theta;
    int k = 0, m_eff = m;
    bool converged = false;
    double spmv_ms = 0.0;
    for (;;) {
        run_cycle(k);
        inf.matvecs += m - k;
        int hstop = 0;
        ED_CUDA(cudaMemcpyAsync(&hstop, stop, sizeof(int), cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(coef_h.data(), cw.coef.p, coef_h.size() * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(beta_h.data(), cw.beta.p, (size_t)(m + 1) * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int j = k; j < m; ++j) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev[2 * j], ev[2 * j + 1]) == cudaSuccess) spmv_ms += ms;
        }
        (void)cudaGetLastError();
        m_eff = hstop ? hstop : m;
        if (hstop) {
            ++inf.breakdowns;
            inf.matvecs -= m - hstop;   // the steps after the breakdown launched no product work
        }
        for (int j = k; j < m_eff; ++j)
            for (int i = 0; i <= j; ++i) {
                const double v = coef_h[(size_t)j * (m + 1) + i];
                T[(size_t)i * m + j] = v;
                T[(size_t)j * m + i] = v;
            }
        std::vector<double> Tm((size_t)m_eff * m_eff);
        for (int i = 0; i < m_eff; ++i)
            for (int j = 0; j < m_eff; ++j) Tm[(size_t)i * m_eff + j] = T[(size_t)i * m + j];
        sym_eigen(m_eff, Tm, theta, Y);
        const double bl = hstop ? 0.0 : beta_h[m - 1];
        int nconv = 0;
        double maxres = 0.0;
        const int want = std::min(nev, m_eff);
        for (int i = 0; i < want; ++i) {
            const double r = std::fabs(bl * Y[(size_t)(m_eff - 1) + (size_t)m_eff * i]);
            maxres = std::max(maxres, r);
            if (r <= tol) ++nconv;
        }
        inf.converged = nconv;
        inf.max_residual = maxres;
        // after a breakdown accept only once a cycle leaves the nev lowest
        // values unchanged (a fresh direction may uncover more copies of a
        // degenerate eigenvalue), or when the whole space is spanned
        bool stable = !hstop || (int64_t)m_eff >= n;
        if (hstop && !stable && (int)prev_theta.size() >= nev && m_eff >= nev) {
            stable = true;
            for (int i = 0; i < nev; ++i)
                if (std::fabs(theta[i] - prev_theta[i]) > tol * std::max(1.0, std::fabs(theta[i]))) stable = false;
        }
        prev_theta.assign(theta.begin(), theta.begin() + std::min<int>(nev, (int)theta.size()));
        if (m_eff >= nev && nconv == nev && stable) {
            converged = true;
            break;
        }
        if (inf.restarts >= max_restarts) break;
        ++inf.restarts;
        int kk = std::min(m - 2, nev + std::max(1, (m - nev) / 4));
        kk = std::max(kk, std::min(nev, m - 1));
        if (hstop) kk = std::min(kk, m_eff);
        rotate_basis(Vb.p, 2 * n, m_eff, Y.data(), m_eff, kk, V2b.p, rot, 0, st);
        if (!hstop) {
            ED_CUDA(cudaMemcpyAsync(col(V2b, kk), col(Vb, m), 2 * (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        } else {
            k_crandom<<<nsm * 4, kCThreads, 0, st>>>(reinterpret_cast<double*>(col(V2b, kk)), 2 * n,
                                                     p.seed + 0x51ED2701ull * (uint64_t)inf.restarts);
            count_launch();
            ED_CUDA(cudaGetLastError());
            corthonormalise(cw, col(V2b, 0), kk, st);
        }
        std::swap(Vb.p, V2b.p);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < kk; ++i) {
            T[(size_t)i * m + i] = theta[i];
            if (!hstop) {
                const double s = bl * Y[(size_t)(m_eff - 1) + (size_t)m_eff * i];
                T[(size_t)i * m + kk] = s;
                T[(size_t)kk * m + i] = s;
            }
        }
        k = kk;
        ED_CUDA(cudaStreamSynchronize(st));
    }
    // an unconverged run can end inside a breakdown cycle with fewer Ritz
    // pairs than requested: report the ones there are, NaN for the rest
    const int nfound = std::min(nev, m_eff);
    for (int i = 0; i < nev; ++i) evals[i] = i < nfound ? theta[i] : std::nan("");
    DevBuf<double> xtmp;
    double* Xo = evecs_dev;
    if (!Xo && p.verify) {
        xtmp.alloc(2 * (size_t)n * nev);
        Xo = xtmp.p;
    }
    if (Xo) {
        if (nfound < nev) ED_CUDA(cudaMemsetAsync(Xo, 0, 2 * (size_t)n * nev * 8, st));
        rotate_basis(Vb.p, 2 * n, m_eff, Y.data(), m_eff, nfound, Xo, rot, 0, st);
    }
    if (p.verify && Xo && nfound == nev) {
        DevBuf<double> yv(2 * (size_t)n);
        double worst = 0.0;
        int nc = 0;
        for (int i = 0; i < nev; ++i) {
            const double* xi = Xo + 2 * (size_t)n * i;
            cspmv(a, xi, yv.p, st);
            ++inf.matvecs;
            k_cresid<<<cw.nb, kCThreads, 0, st>>>(reinterpret_cast<const double2*>(yv.p),
                                                 reinterpret_cast<const double2*>(xi), evals[i], n, cw.part.p);
            count_launch();
            ED_CUDA(cudaGetLastError());
            const std::vector<double> h = host_parts(cw.part, cw.nb, st);
            double s = 0.0;
            for (double v : h) s += v;
            const double r = std::sqrt(s);
            worst = std::max(worst, r);
            nc += r <= tol ? 1 : 0;
        }
        inf.max_residual = worst;
        inf.converged = nc;
    }
    ED_CUDA(cudaStreamSynchronize(st));
    inf.spmv_seconds = spmv_ms * 1e-3;
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = inf;
    ED_REQUIRE(converged, ED_ERR_NOCONV, "Lanczos did not converge within the restart cap");
}

}  // namespace edgb

using namespace edgb;

// ------------------------------------------------------------ C ABI

extern "C" ed_status ed_cterms_create(int norb, int dimX, int dimY, const uint16_t* ktable, const double* vtable,
                                      const double* energies, ed_cterms** out)
{
    return guard([&] {
        ED_REQUIRE(out && ktable && vtable, ED_ERR_ARG, "ktable, vtable and out must not be NULL");
        *out = nullptr;
        ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals && dimX >= 1 && dimY >= 1 && dimX * dimY == norb, ED_ERR_RANGE,
                   "momentum grid: need dimX * dimY = norb in 2..40");
        const size_t tdim = (size_t)(norb + 1) * norb * norb / 2;
        ed_cterms* t = new ed_cterms();
        try {
            t->norb = norb;
            t->dimX = dimX;
            t->dimY = dimY;
            t->ktab.assign(ktable, ktable + tdim);
            t->vtab.assign(vtable, vtable + 2 * tdim);
            if (energies) t->e.assign(energies, energies + 2 * (size_t)norb);
            cterms_derive(*t);
        } catch (...) {
            delete t;
            throw;
        }
        *out = t;
    });
}

extern "C" ed_status ed_cterms_free(ed_cterms* t)
{
    return guard([&] { delete t; });
}

extern "C" ed_status ed_basis_momentum_build(int N, int dimX, int dimY, int kx_tot, int ky_tot, ed_stream stream,
                                             ed_basis** out)
{
    return guard([&] {
        ED_REQUIRE(out != nullptr, ED_ERR_ARG, "out must not be NULL");
        *out = nullptr;
        ED_REQUIRE(dimX >= 1 && dimY >= 1 && dimX * dimY <= kMaxOrbitals, ED_ERR_RANGE,
                   "momentum basis: need dimX * dimY <= 40 orbitals");
        ed_basis* b = new ed_basis();
        b->N = N;
        b->norb = dimX * dimY;
        b->dimX = dimX;
        b->dimY = dimY;
        b->kx_tot = kx_tot;
        b->ky_tot = ky_tot;
        try {
            basis_build(*b, (cudaStream_t)stream);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

extern "C" ed_status ed_cham_build_crs(const ed_basis* b, const ed_cterms* t, int store_upper, ed_stream stream,
                                       ed_ccrs** out)
{
    return guard([&] {
        ED_REQUIRE(b && t && out, ED_ERR_ARG, "basis, terms and out must not be NULL");
        *out = nullptr;
        ed_ccrs* a = new ed_ccrs();
        try {
            cham_build_crs(*b, *t, store_upper, *a, (cudaStream_t)stream);
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

extern "C" ed_status ed_ccrs_free(ed_ccrs* a)
{
    return guard([&] { delete a; });
}

extern "C" ed_status ed_ccrs_info(const ed_ccrs* a, int64_t* n, int64_t* nnz, int* upper)
{
    return guard([&] {
        ED_REQUIRE(a != nullptr, ED_ERR_ARG, "matrix must not be NULL");
        if (n) *n = a->n;
        if (nnz) *nnz = a->nnz;
        if (upper) *upper = a->upper;
    });
}

extern "C" ed_status ed_ccrs_get(const ed_ccrs* a, int64_t* rowptr, int32_t* col, double* val)
{
    return guard([&] {
        ED_REQUIRE(a && rowptr && (a->nnz == 0 || (col && val)), ED_ERR_ARG, "NULL argument");
        ED_CUDA(cudaMemcpy(rowptr, a->rowptr.p, (size_t)(a->n + 1) * 8, cudaMemcpyDeviceToHost));
        if (a->nnz) {
            ED_CUDA(cudaMemcpy(col, a->col.p, (size_t)a->nnz * 4, cudaMemcpyDeviceToHost));
            ED_CUDA(cudaMemcpy(val, a->val.p, (size_t)a->nnz * 16, cudaMemcpyDeviceToHost));
        }
    });
}

extern "C" ed_status ed_cspmv_kernel(const ed_ccrs* a, int kernel, const double* x_dev, double* y_dev,
                                     ed_stream stream)
{
    return guard([&] {
        ED_REQUIRE(a && x_dev && y_dev, ED_ERR_ARG, "null argument");
        ED_REQUIRE(x_dev != y_dev, ED_ERR_ARG, "x and y must be distinct");
        cspmv_kernel(*a, kernel, x_dev, y_dev, (cudaStream_t)stream);
    });
}

extern "C" ed_status ed_cspmv(const ed_ccrs* a, const double* x_dev, double* y_dev, ed_stream stream)
{
    return guard([&] {
        ED_REQUIRE(a != nullptr, ED_ERR_ARG, "matrix must not be NULL");
        if (a->n == 0) return;
        ED_REQUIRE(x_dev && y_dev && x_dev != y_dev, ED_ERR_ARG, "x and y must be distinct device vectors");
        cspmv(*a, x_dev, y_dev, (cudaStream_t)stream);
        ED_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    });
}

extern "C" ed_status ed_clanczos(const ed_ccrs* a, const ed_lanczos_params* p, const double* v0_host,
                                 double* evals_host, double* evecs_host, ed_solve_info* info)
{
    return guard([&] {
        ED_REQUIRE(a && p && evals_host, ED_ERR_ARG, "matrix, params and evals must not be NULL");
        if (info) std::memset(info, 0, sizeof(*info));
        const int64_t n = a->n;
        ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
        ED_REQUIRE(p->nev >= 1 && p->nev <= n, ED_ERR_ARG, "need 1 <= nev <= n");
        DevBuf<double> v0, ev;
        if (v0_host) {
            v0.alloc(2 * (size_t)n);
            ED_CUDA(cudaMemcpy(v0.p, v0_host, 2 * (size_t)n * 8, cudaMemcpyHostToDevice));
        }
        if (evecs_host) ev.alloc(2 * (size_t)n * p->nev);
        ed_status deferred = ED_OK;
        std::string msg;
        try {
            clanczos_solve(*a, *p, v0.p, evals_host, ev.p, info, nullptr);
        } catch (const Error& e) {
            if (e.code != ED_ERR_NOCONV) throw;
            deferred = e.code;
            msg = e.what();
        }
        if (evecs_host)
            ED_CUDA(cudaMemcpy(evecs_host, ev.p, 2 * (size_t)n * p->nev * 8, cudaMemcpyDeviceToHost));
        if (deferred != ED_OK) throw Error(deferred, msg);
    });
}
