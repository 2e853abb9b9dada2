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
// (re, im) pairs: full complex Gram-Schmidt (two passes) against the Krylov
// basis, the real projected matrix (alpha and beta of a Hermitian operator
// are real) solved on the host, restart rotations of the complex basis by the
// real Ritz coefficients.  It replaces ArpackWrapper's complex driver
// (the T = dcmplx branches of arpack_wrapper.hpp:255-937, znaupd_/zneupd_
// with WHICH "SR").
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

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

// part[(i*nb + b)*2 + {0,1}] = block b's share of V_i^H w (complex), i < J,
// and part[(J*nb + b)*2] its share of ||w||^2.
__global__ void __launch_bounds__(kCThreads) k_cdots(const double2* __restrict__ V, int J, const double2* __restrict__ w,
                                                     int64_t n, double* __restrict__ part)
{
    __shared__ double red[kCThreads / 32];
    int64_t r0, r1;
    cchunk(n, gridDim.x, blockIdx.x, r0, r1);
    {
        double s = 0.0;
        for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
            const double2 b = w[r];
            s = fma(b.x, b.x, s);
            s = fma(b.y, b.y, s);
        }
        s = cblock_sum(s, red);
        if (threadIdx.x == 0) {
            part[((int64_t)J * gridDim.x + blockIdx.x) * 2] = s;
            part[((int64_t)J * gridDim.x + blockIdx.x) * 2 + 1] = 0.0;
        }
    }
    for (int i = 0; i < J; ++i) {
        const double2* vi = V + (int64_t)i * n;
        double re = 0.0, im = 0.0;
        for (int64_t r = r0 + threadIdx.x; r < r1; r += kCThreads) {
            const double2 a = vi[r], b = w[r];
            re = fma(a.x, b.x, re);
            re = fma(a.y, b.y, re);
            im = fma(a.x, b.y, im);
            im = fma(-a.y, b.x, im);
        }
        re = cblock_sum(re, red);
        im = cblock_sum(im, red);
        if (threadIdx.x == 0) {
            part[((int64_t)i * gridDim.x + blockIdx.x) * 2] = re;
            part[((int64_t)i * gridDim.x + blockIdx.x) * 2 + 1] = im;
        }
    }
}

// w -= sum_i c_i V_i (c complex, device).
__global__ void __launch_bounds__(kCThreads) k_cupdate(const double2* __restrict__ V, int J,
                                                       const double2* __restrict__ c, double2* __restrict__ w,
                                                       int64_t n)
{
    for (int64_t r = blockIdx.x * (int64_t)kCThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kCThreads) {
        double2 a = w[r];
        for (int i = 0; i < J; ++i) {
            const double2 v = V[(int64_t)i * n + r], ci = c[i];
            a.x = fma(-ci.x, v.x, a.x);
            a.x = fma(ci.y, v.y, a.x);
            a.y = fma(-ci.x, v.y, a.y);
            a.y = fma(-ci.y, v.x, a.y);
        }
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

// Working state of one complex solve.
struct CWork {
    int64_t n = 0;
    int nb = 1;
    DevBuf<double> part, c;
};

// Orthogonalise w against V[0..J) twice (complex); returns the summed
// coefficients V_i^H w of both passes.  norm_in: ||w|| before the passes;
// norm_out: ||w|| after them, from the second pass's dots (Pythagoras: w
// loses exactly V c of norm |c| to an orthonormal V), so a step needs two
// host round trips.
std::vector<cplx> cgram_schmidt(CWork& cw, const double2* V, int J, double2* w, cudaStream_t st,
                                double* norm_in = nullptr, double* norm_out = nullptr)
{
    std::vector<cplx> acc(J, cplx(0.0, 0.0));
    for (int pass = 0; pass < 2; ++pass) {
        k_cdots<<<cw.nb, kCThreads, 0, st>>>(V, J, w, cw.n, cw.part.p);
        count_launch();
        ED_CUDA(cudaGetLastError());
        const std::vector<double> h = host_parts(cw.part, (size_t)(J + 1) * cw.nb * 2, st);
        double nn = 0.0;
        for (int b = 0; b < cw.nb; ++b) nn += h[((size_t)J * cw.nb + b) * 2];
        std::vector<double> c(2 * (size_t)J);
        for (int i = 0; i < J; ++i) {
            double re = 0.0, im = 0.0;
            for (int b = 0; b < cw.nb; ++b) {
                re += h[((size_t)i * cw.nb + b) * 2];
                im += h[((size_t)i * cw.nb + b) * 2 + 1];
            }
            c[2 * i] = re;
            c[2 * i + 1] = im;
            acc[i] += cplx(re, im);
        }
        if (pass == 0 && norm_in) *norm_in = std::sqrt(nn);
        if (pass == 1 && norm_out) {
            double removed = 0.0;
            for (int i = 0; i < J; ++i) removed += c[2 * i] * c[2 * i] + c[2 * i + 1] * c[2 * i + 1];
            *norm_out = std::sqrt(std::max(0.0, nn - removed));
        }
        if (J == 0) break;
        ED_CUDA(cudaMemcpyAsync(cw.c.p, c.data(), c.size() * 8, cudaMemcpyHostToDevice, st));
        k_cupdate<<<csms() * 4, kCThreads, 0, st>>>(V, J, reinterpret_cast<const double2*>(cw.c.p), w, cw.n);
        count_launch();
        ED_CUDA(cudaGetLastError());
    }
    return acc;
}

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

void cspmv(const ed_ccrs& a, const double* x, double* y, cudaStream_t st)
{
    if (a.n == 0) return;
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
    CWork cw;
    cw.n = n;
    cw.nb = (int)std::max<int64_t>(1, std::min<int64_t>(csms() * 4, n / 1024));
    cw.part.alloc((size_t)(m + 2) * cw.nb * 2);
    cw.c.alloc(2 * (size_t)(m + 2));
    DevBuf<double> Vb(2 * (size_t)n * (m + 1)), V2b(2 * (size_t)n * (m + 1));
    auto col = [&](DevBuf<double>& B, int j) { return reinterpret_cast<double2*>(B.p + 2 * (size_t)n * j); };
    RotateScratch rot;
    if (v0_dev) ED_CUDA(cudaMemcpyAsync(Vb.p, v0_dev, 2 * (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    else {
        k_crandom<<<csms() * 4, kCThreads, 0, st>>>(Vb.p, 2 * n, p.seed);
        count_launch();
        ED_CUDA(cudaGetLastError());
    }
    {
        const double nrm = cnorm(cw, col(Vb, 0), st);
        ED_REQUIRE(nrm > 0.0 && std::isfinite(nrm), ED_ERR_ARG, "start vector is zero or not finite");
        cscale(col(Vb, 0), n, 1.0 / nrm, st);
    }
    std::vector<double> T((size_t)m * m, 0.0), theta, Y;
    std::vector<double> beta(m + 1, 0.0);
    int k = 0;
    bool converged = false;
    float spmv_ms = 0.f;
    cudaEvent_t e0, e1;
    ED_CUDA(cudaEventCreate(&e0));
    ED_CUDA(cudaEventCreate(&e1));
    struct EvG {
        cudaEvent_t a, b;
        ~EvG() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } evg{e0, e1};
    for (;;) {
        for (int j = k; j < m; ++j) {
            double2* vj = col(Vb, j);
            double2* w = col(Vb, j + 1);
            ED_CUDA(cudaEventRecord(e0, st));
            cspmv(a, reinterpret_cast<const double*>(vj), reinterpret_cast<double*>(w), st);
            ED_CUDA(cudaEventRecord(e1, st));
            ++inf.matvecs;
            double hnorm = 0.0, b = 0.0;
            const std::vector<cplx> c = cgram_schmidt(cw, col(Vb, 0), j + 1, w, st, &hnorm, &b);
            float ms = 0.f;
            ED_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            spmv_ms += ms;
            for (int i = 0; i <= j; ++i) {
                T[(size_t)i * m + j] = c[i].real();
                T[(size_t)j * m + i] = c[i].real();
            }
            // below 1e-6 of ||H v|| the Pythagorean norm loses digits: measure it
            if (b < 1e-6 * hnorm) b = cnorm(cw, w, st);
            if (!(b > 1e-13 * std::max(1.0, hnorm))) {
                // invariant subspace: continue from a fresh direction
                ++inf.breakdowns;
                k_crandom<<<csms() * 4, kCThreads, 0, st>>>(reinterpret_cast<double*>(w), 2 * n,
                                                           p.seed + 0x51ED2701ull * (uint64_t)(inf.matvecs + 1));
                count_launch();
                ED_CUDA(cudaGetLastError());
                cgram_schmidt(cw, col(Vb, 0), j + 1, w, st);
                const double nr = cnorm(cw, w, st);
                ED_REQUIRE(nr > 0.0, ED_ERR_INTERNAL, "no direction left after a Krylov breakdown");
                cscale(w, n, 1.0 / nr, st);
                b = 0.0;
            } else {
                cscale(w, n, 1.0 / b, st);
            }
            beta[j] = b;
            if (j + 1 < m) {
                T[(size_t)j * m + j + 1] = b;
                T[(size_t)(j + 1) * m + j] = b;
            }
        }
        sym_eigen(m, T, theta, Y);
        const double bl = beta[m - 1];
        int nconv = 0;
        double maxres = 0.0;
        for (int i = 0; i < nev; ++i) {
            const double r = std::fabs(bl * Y[(size_t)(m - 1) + (size_t)m * i]);
            maxres = std::max(maxres, r);
            if (r <= tol) ++nconv;
        }
        inf.converged = nconv;
        inf.max_residual = maxres;
        if (nconv == nev) {
            converged = true;
            break;
        }
        if (inf.restarts >= max_restarts) break;
        ++inf.restarts;
        int kk = std::min(m - 2, nev + std::max(1, (m - nev) / 4));
        kk = std::max(kk, std::min(nev, m - 1));
        rotate_basis(Vb.p, 2 * n, m, Y.data(), m, kk, V2b.p, rot, 0, st);
        ED_CUDA(cudaMemcpyAsync(col(V2b, kk), col(Vb, m), 2 * (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        std::swap(Vb.p, V2b.p);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < kk; ++i) {
            T[(size_t)i * m + i] = theta[i];
            const double s = bl * Y[(size_t)(m - 1) + (size_t)m * i];
            T[(size_t)i * m + kk] = s;
            T[(size_t)kk * m + i] = s;
        }
        k = kk;
        ED_CUDA(cudaStreamSynchronize(st));
    }
    for (int i = 0; i < nev; ++i) evals[i] = theta[i];
    DevBuf<double> xtmp;
    double* Xo = evecs_dev;
    if (!Xo && p.verify) {
        xtmp.alloc(2 * (size_t)n * nev);
        Xo = xtmp.p;
    }
    if (Xo) rotate_basis(Vb.p, 2 * n, m, Y.data(), m, nev, Xo, rot, 0, st);
    if (p.verify && Xo) {
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
