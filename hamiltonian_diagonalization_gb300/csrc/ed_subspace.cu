// Shared-subspace Rayleigh-Ritz for the Hamiltonians of a batch (eigenvector
// continuation).  No reference counterpart: the reference solves each
// Hamiltonian of a sweep from scratch.
//
// The Hamiltonians of a pseudopotential sweep lie in a low-dimensional linear
// family (H(V1) = V1 P_1 + R), and their low eigenvectors change smoothly
// along it, so the eigenvectors of a few solved members (anchors) span a
// subspace in which the other members' low eigenpairs are found by a
// Rayleigh-Ritz step.  The subspace Q (n x d, orthonormal) is kept row-major
// on the device.  For the Ritz step the batch's coefficient vectors (hop
// values and diagonal-term tables, which a Hamiltonian is linear in) are
// reduced to a basis of r members H_k; Q^T H_k Q is formed once per basis
// member (r multi-vector products and r d x d Gram matrices), and every
// Hamiltonian's projected matrix is the combination of those.  The Ritz
// vectors of all Hamiltonians are then formed in the batch layout and their
// true residuals computed with the batch's own block product, so a Ritz pair
// is accepted only on the operator's residual, never on the projection.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ed_batch.h"
#include "ed_lanczos.h"

struct ed_subspace {
    int64_t n = 0;
    int max_dim = 0, dim = 0;
    edgb::DevBuf<double> Q;        // [n][max_dim], columns 0..dim orthonormal
    edgb::DevBuf<double> u, part, h;
};

namespace edgb {

namespace {

constexpr int kMaxSubspace = 256;   // columns: eight per lane in the warp-per-row kernels
constexpr int kST = 256;

int sub_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(batch_sms() * 4, (n + 255) / 256)); }

__device__ __forceinline__ void chunk(int64_t n, int nb, int b, int64_t& r0, int64_t& r1)
{
    r0 = n * (int64_t)b / nb;
    r1 = n * (int64_t)(b + 1) / nb;
}

// u[r] = U[g][r][a] (column a of group g of a [groups][n][width] array)
__global__ void k_sub_col(const double* __restrict__ U, int64_t n, int width, int g, int a, double* __restrict__ u)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        u[r] = U[((int64_t)g * n + r) * width + a];
}

// part[blk][i] = sum over the block's rows of Q[r][i] u[r] (i < c) and
// part[blk][c] = sum of u[r]^2: one warp per row, lanes over the columns.
__global__ void __launch_bounds__(kST) k_sub_mdot(const double* __restrict__ Q, int ldq, int c,
                                                  const double* __restrict__ u, int64_t n, double* __restrict__ part)
{
    __shared__ double red[kST / 32][kMaxSubspace + 1];
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double acc[kMaxSubspace / 32];
#pragma unroll
    for (int t = 0; t < kMaxSubspace / 32; ++t) acc[t] = 0.0;
    double uu = 0.0;
    for (int64_t r = r0 + wid; r < r1; r += kST / 32) {
        const double ur = u[r];
        uu = fma(ur, ur, uu);
        const double* q = Q + r * ldq;
#pragma unroll
        for (int t = 0; t < kMaxSubspace / 32; ++t) {
            const int i = lane + 32 * t;
            if (i < c) acc[t] = fma(q[i], ur, acc[t]);
        }
    }
#pragma unroll
    for (int t = 0; t < kMaxSubspace / 32; ++t) {
        const int i = lane + 32 * t;
        if (i < c) red[wid][i] = acc[t];
    }
    if (lane == 0) red[wid][c] = uu;
    __syncthreads();
    for (int i = threadIdx.x; i <= c; i += kST) {
        double s = 0.0;
        for (int w = 0; w < kST / 32; ++w) s += red[w][i];
        part[(int64_t)blockIdx.x * (c + 1) + i] = s;
    }
}

// out[i] = sum over blocks of part[blk][i], i < cnt, in block order
__global__ void k_sub_sum(const double* __restrict__ part, int nb, int cnt, double* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[(int64_t)b * cnt + i];
        out[i] = s;
    }
}

// u[r] -= sum_i Q[r][i] h[i], i < c: one warp per row, shuffle reduction
__global__ void __launch_bounds__(kST) k_sub_update(const double* __restrict__ Q, int ldq, int c,
                                                    const double* __restrict__ h, double* __restrict__ u, int64_t n)
{
    __shared__ double hs[kMaxSubspace];
    for (int i = threadIdx.x; i < c; i += kST) hs[i] = h[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)kST + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * kST) >> 5;
    for (int64_t r = w0; r < n; r += nw) {
        const double* q = Q + r * ldq;
        double s = 0.0;
        for (int i = lane; i < c; i += 32) s = fma(q[i], hs[i], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) u[r] -= s;
    }
}

// Q[r][c] = u[r] * s
__global__ void k_sub_store(const double* __restrict__ u, int64_t n, double s, double* __restrict__ Q, int ldq, int c)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        Q[r * ldq + c] = u[r] * s;
}

__device__ __forceinline__ double signed_hop(double w, uint16_t code)
{
    return __longlong_as_double(__double_as_longlong(w) ^ ((long long)(code & 0x8000u) << 48));
}

// Y[r][j] = H_b X[r][j] for j < ncols (X, Y row-major with leading dimensions
// ldx, ldy): one row per warp, lanes over 32 consecutive columns, the element's
// column and code loaded once for the row and its hop value broadcast.
template <int U>
__global__ void __launch_bounds__(256) k_sub_apply(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                   const uint16_t* __restrict__ code, const double* __restrict__ w,
                                                   const double* __restrict__ diag, int B, int b,
                                                   const double* __restrict__ X, int ldx, double* __restrict__ Y,
                                                   int ldy, int64_t n, int ncols)
{
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.y * 32 + lane;
    const bool jv = j < ncols;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < n; r += nwarps) {
        const int64_t s = rowptr[r], e = rowptr[r + 1];
        double acc0 = jv ? diag[r * B + b] * X[r * ldx + j] : 0.0, acc1 = 0.0;
        for (int64_t k = s; k < e; k += U) {
            int c[U];
            double wv[U], xv[U];
#pragma unroll
            for (int t = 0; t < U; ++t) {
                c[t] = __ldg(col + k + t);
                const uint16_t cd = __ldg(code + k + t);
                wv[t] = signed_hop(__ldg(w + (int64_t)(cd & 0x7FFF) * B + b), cd);
            }
#pragma unroll
            for (int t = 0; t < U; ++t) xv[t] = jv ? __ldg(X + (int64_t)c[t] * ldx + j) : 0.0;
#pragma unroll
            for (int t = 0; t < U; ++t)
                if (k + t < e) {
                    if (t & 1) acc1 = fma(wv[t], xv[t], acc1);
                    else acc0 = fma(wv[t], xv[t], acc0);
                }
        }
        if (jv) Y[r * ldy + j] = acc0 + acc1;
    }
}

// Tall-skinny products with 64 x 64 output tiles, 4 x 4 per thread.
constexpr int kTile = 64, kRows = 16;

// part[blk][tile] = A[rows of blk]^T B[rows of blk] restricted to output tile
// (ti, tj) = (blockIdx.y / ntj, blockIdx.y % ntj); A is n x p (lda), B n x q (ldb).
__global__ void __launch_bounds__(256) k_ts_gram(const double* __restrict__ A, int lda, int p,
                                                 const double* __restrict__ Bm, int ldb, int q, int64_t n,
                                                 double* __restrict__ part)
{
    __shared__ double As[kRows][kTile], Bs[kRows][kTile];
    const int ntj = (q + kTile - 1) / kTile;
    const int ti = blockIdx.y / ntj, tj = blockIdx.y % ntj;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    double acc[4][4] = {};
    for (int64_t rb = r0; rb < r1; rb += kRows) {
        for (int t = threadIdx.x; t < kRows * kTile; t += 256) {
            const int rr = t / kTile, cc = t % kTile;
            const int64_t r = rb + rr;
            const int ia = ti * kTile + cc, ib = tj * kTile + cc;
            As[rr][cc] = (r < r1 && ia < p) ? A[r * lda + ia] : 0.0;
            Bs[rr][cc] = (r < r1 && ib < q) ? Bm[r * ldb + ib] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < kRows; ++rr) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { a[u] = As[rr][tx * 4 + u]; b[u] = Bs[rr][ty * 4 + u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
    double* out = part + ((int64_t)blockIdx.x * gridDim.y + blockIdx.y) * (kTile * kTile);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) out[(tx * 4 + u) * kTile + ty * 4 + v] = acc[u][v];
}

// C[i][j] (p x q, row-major) = sum over blocks of the tile partials, in block order
__global__ void k_ts_gram_sum(const double* __restrict__ part, int nb, int ntiles, int p, int q,
                              double* __restrict__ C)
{
    const int ntj = (q + kTile - 1) / kTile;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < p * q; t += gridDim.x * blockDim.x) {
        const int i = t / q, j = t % q;
        const int tile = (i / kTile) * ntj + (j / kTile);
        const int e = (i % kTile) * kTile + (j % kTile);
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[((int64_t)b * ntiles + tile) * (kTile * kTile) + e];
        C[t] = s;
    }
}

// Y[r][j] = A[r][:] M[:][j] for a 64-row x 64-column output tile per block
// (A n x p with lda, M p x q row-major, Y with ldy); M and A staged in
// chunks of 16 of the inner dimension.
__global__ void __launch_bounds__(256) k_ts_combine(const double* __restrict__ A, int lda, int p,
                                                    const double* __restrict__ M, int q, double* __restrict__ Y,
                                                    int ldy, int64_t n)
{
    __shared__ double As[kTile][kRows + 1], Ms[kRows][kTile];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t rbase = (int64_t)blockIdx.x * kTile;
    const int cbase = blockIdx.y * kTile;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < p; k0 += kRows) {
        for (int t = threadIdx.x; t < kTile * kRows; t += 256) {
            const int rr = t / kRows, kk = t % kRows;
            const int64_t r = rbase + rr;
            As[rr][kk] = (r < n && k0 + kk < p) ? A[r * lda + k0 + kk] : 0.0;
            const int mk = t / kTile, mc = t % kTile;
            Ms[mk][mc] = (k0 + mk < p && cbase + mc < q) ? M[(int64_t)(k0 + mk) * q + cbase + mc] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kRows; ++kk) {
            double a[4], m[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { a[u] = As[ty * 4 + u][kk]; m[u] = Ms[kk][tx * 4 + u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], m[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t r = rbase + ty * 4 + u;
        if (r >= n) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int c = cbase + tx * 4 + v;
            if (c < q) Y[r * ldy + c] = acc[u][v];
        }
    }
}

int grid1(int64_t work) { return (int)std::max<int64_t>(1, std::min<int64_t>(batch_sms() * 8, (work + 255) / 256)); }

// C_dev (p x q row-major) = A^T B over n rows
void ts_gram_dev(const double* A, int lda, int p, const double* Bm, int ldb, int q, int64_t n, double* C_dev,
                 cudaStream_t st)
{
    const int ntiles = ((p + kTile - 1) / kTile) * ((q + kTile - 1) / kTile);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(std::max(1, batch_sms() * 2 / ntiles), n / kRows));
    DevBuf<double> part((size_t)nb * ntiles * kTile * kTile);
    k_ts_gram<<<dim3((unsigned)nb, (unsigned)ntiles), 256, 0, st>>>(A, lda, p, Bm, ldb, q, n, part.p); count_launch();
    k_ts_gram_sum<<<grid1((int64_t)p * q), 256, 0, st>>>(part.p, nb, ntiles, p, q, C_dev); count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));   // part is freed on return
}

// M[b] = sum_k alpha[b][k] (A_k + A_k^T) / 2 for the B Hamiltonians (d x d each)
__global__ void k_sub_assemble(const double* __restrict__ Ak, int r, int d, const double* __restrict__ alpha, int B,
                               double* __restrict__ M)
{
    const int64_t dd = (int64_t)d * d, total = dd * B;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / dd);
        const int64_t e = t - (int64_t)b * dd;
        const int i = (int)(e / d), j = (int)(e % d);
        double s = 0.0;
        for (int k = 0; k < r; ++k)
            s = fma(alpha[b * r + k], 0.5 * (Ak[k * dd + (int64_t)i * d + j] + Ak[k * dd + (int64_t)j * d + i]), s);
        M[t] = s;
    }
}

// Mi[i][c][b] = Z_b[c + d i] (the Ritz coefficients of the nev lowest pairs
// in the combine layout), evals_out[b][i] = E[b][i]
__global__ void k_sub_ritz_coef(const double* __restrict__ Z, const double* __restrict__ E, int d, int B, int nev,
                                double* __restrict__ Mi, double* __restrict__ evals_out)
{
    const int64_t total = (int64_t)nev * d * B;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t % B);
        const int64_t ic = t / B;
        const int c = (int)(ic % d), i = (int)(ic / d);
        Mi[t] = Z[(int64_t)b * d * d + c + (int64_t)d * i];
        if (c == 0) evals_out[(int64_t)b * nev + i] = E[(int64_t)b * d + i];
    }
}

void ts_combine(const double* A, int lda, int p, const double* M_dev, int q, double* Y, int ldy, int64_t n,
                cudaStream_t st)
{
    dim3 grid((unsigned)((n + kTile - 1) / kTile), (unsigned)((q + kTile - 1) / kTile));
    k_ts_combine<<<grid, 256, 0, st>>>(A, lda, p, M_dev, q, Y, ldy, n); count_launch();
    ED_CUDA(cudaGetLastError());
}

// Y = H_b X for ncols row-major columns on the batch's pattern
void batch_apply(const ed_batch& bt, int b, const double* X, int ldx, double* Y, int ldy, int ncols, cudaStream_t st)
{
    static_assert(4 <= kCrsPad, "apply overruns the padding");
    dim3 grid((unsigned)(batch_sms() * 8), (unsigned)((ncols + 31) / 32));
    k_sub_apply<4><<<grid, 256, 0, st>>>(bt.rowptr.p, bt.col.p, bt.code.p, bt.w.p, bt.diag.p, bt.B, b, X, ldx, Y, ldy,
                                         bt.n, ncols);
    count_launch();
    ED_CUDA(cudaGetLastError());
}

}  // namespace

// The batch's Hamiltonians as combinations of r of its members: basis[k] is a
// member index and alpha[b * r + k] the weight of basis[k] in Hamiltonian b.
// Pivoted modified Gram-Schmidt on the coefficient vectors; every vector must
// be reproduced to 1e-12 of its norm by at most max_rank members.
void batch_linear_family(const ed_batch& bt, int max_rank, std::vector<int>& basis, std::vector<double>& alpha)
{
    const int B = bt.B, L = bt.ncoef;
    ED_REQUIRE(L > 0 && (int64_t)bt.coef.size() == (int64_t)B * L, ED_ERR_INTERNAL, "batch coefficients missing");
    std::vector<double> nrm(B);
    for (int b = 0; b < B; ++b) {
        double s = 0.0;
        for (int t = 0; t < L; ++t) s += bt.coef[(size_t)b * L + t] * bt.coef[(size_t)b * L + t];
        nrm[b] = std::sqrt(s);
    }
    std::vector<std::vector<double>> E;   // orthonormal directions
    std::vector<std::vector<double>> Rm;  // Rm[k][j]: coefficient of E[j] in member basis[k]
    basis.clear();
    std::vector<double> res((size_t)B * L);
    std::copy(bt.coef.begin(), bt.coef.end(), res.begin());
    for (;;) {
        // the member with the largest remainder relative to its norm
        int best = -1;
        double bestv = 0.0;
        for (int b = 0; b < B; ++b) {
            if (!(nrm[b] > 0)) continue;
            double s = 0.0;
            for (int t = 0; t < L; ++t) s += res[(size_t)b * L + t] * res[(size_t)b * L + t];
            const double rel = std::sqrt(s) / nrm[b];
            if (rel > bestv) { bestv = rel; best = b; }
        }
        if (best < 0 || bestv <= 1e-12) break;
        ED_REQUIRE((int)basis.size() < max_rank, ED_ERR_ARG,
                   "the batch's Hamiltonians are not a low-rank linear family");
        // new direction from the member's remainder (a second pass for orthogonality)
        std::vector<double> e(res.begin() + (size_t)best * L, res.begin() + (size_t)(best + 1) * L);
        for (const auto& f : E) {
            double d = 0.0;
            for (int t = 0; t < L; ++t) d += f[t] * e[t];
            for (int t = 0; t < L; ++t) e[t] -= d * f[t];
        }
        double en = 0.0;
        for (int t = 0; t < L; ++t) en += e[t] * e[t];
        en = std::sqrt(en);
        for (int t = 0; t < L; ++t) e[t] /= en;
        E.push_back(e);
        basis.push_back(best);
        for (int b = 0; b < B; ++b) {
            double d = 0.0;
            for (int t = 0; t < L; ++t) d += e[t] * res[(size_t)b * L + t];
            for (int t = 0; t < L; ++t) res[(size_t)b * L + t] -= d * e[t];
        }
    }
    const int r = (int)basis.size();
    ED_REQUIRE(r >= 1, ED_ERR_ARG, "all Hamiltonians of the batch are zero");
    // G[j][k] = E_j . coef_{basis[k]} (upper triangular), z_b[j] = E_j . coef_b; alpha_b = G^-1 z_b
    std::vector<double> G((size_t)r * r), z(r);
    for (int j = 0; j < r; ++j)
        for (int k = 0; k < r; ++k) {
            double d = 0.0;
            for (int t = 0; t < L; ++t) d += E[j][t] * bt.coef[(size_t)basis[k] * L + t];
            G[(size_t)j * r + k] = d;
        }
    alpha.assign((size_t)B * r, 0.0);
    for (int b = 0; b < B; ++b) {
        for (int j = 0; j < r; ++j) {
            double d = 0.0;
            for (int t = 0; t < L; ++t) d += E[j][t] * bt.coef[(size_t)b * L + t];
            z[j] = d;
        }
        for (int j = r - 1; j >= 0; --j) {   // back substitution (G[j][k] ~ 0 below the diagonal)
            double s = z[j];
            for (int k = j + 1; k < r; ++k) s -= G[(size_t)j * r + k] * alpha[(size_t)b * r + k];
            alpha[(size_t)b * r + j] = s / G[(size_t)j * r + j];
        }
    }
}

// Orthonormalise the columns of U [groups][n][width] against the subspace and
// each other (classical Gram-Schmidt, two passes per column), appending every
// column whose remainder keeps more than drop_tol of its norm.
int subspace_add(ed_subspace& sp, const double* U, int groups, int width, double drop_tol, cudaStream_t st)
{
    const int64_t n = sp.n;
    const int nb = sub_blocks(n);
    sp.u.alloc_at_least((size_t)n);
    sp.part.alloc_at_least((size_t)nb * (kMaxSubspace + 1));
    sp.h.alloc_at_least((size_t)kMaxSubspace + 1);
    int kept = 0;
    double nn[2];
    for (int g = 0; g < groups; ++g)
        for (int a = 0; a < width; ++a) {
            ED_REQUIRE(sp.dim < sp.max_dim, ED_ERR_RANGE, "subspace is full");
            const int c = sp.dim;
            k_sub_col<<<grid1(n), 256, 0, st>>>(U, n, width, g, a, sp.u.p); count_launch();
            for (int pass = 0; pass < 3; ++pass) {
                // pass 0, 1: project out Q[:, :c] (and record |u|^2 before); pass 2: final |u|^2
                const int cc = pass < 2 ? c : 0;
                k_sub_mdot<<<nb, kST, 0, st>>>(sp.Q.p, sp.max_dim, cc, sp.u.p, n, sp.part.p); count_launch();
                k_sub_sum<<<1, 256, 0, st>>>(sp.part.p, nb, cc + 1, sp.h.p); count_launch();
                if (pass == 0 || pass == 2)
                    ED_CUDA(cudaMemcpyAsync(&nn[pass / 2], sp.h.p + cc, 8, cudaMemcpyDeviceToHost, st));
                if (pass < 2 && c > 0) {
                    k_sub_update<<<nb, kST, 0, st>>>(sp.Q.p, sp.max_dim, c, sp.h.p, sp.u.p, n); count_launch();
                }
            }
            ED_CUDA(cudaGetLastError());
            ED_CUDA(cudaStreamSynchronize(st));
            ED_REQUIRE(std::isfinite(nn[0]) && std::isfinite(nn[1]), ED_ERR_ARG, "a subspace vector is not finite");
            if (!(nn[0] > 0) || !(nn[1] > drop_tol * drop_tol * nn[0])) continue;
            k_sub_store<<<grid1(n), 256, 0, st>>>(sp.u.p, n, 1.0 / std::sqrt(nn[1]), sp.Q.p, sp.max_dim, c);
            count_launch();
            ED_CUDA(cudaGetLastError());
            ++sp.dim;
            ++kept;
        }
    ED_CUDA(cudaStreamSynchronize(st));
    return kept;
}

// Ritz pairs of every Hamiltonian of the batch in the subspace: evals
// [B][nev] ascending, X [nev][n][B] (device), res [B][nchk] the true residual
// norms of the first nchk pairs through the batch's block product.
void batch_subspace_ritz(const ed_batch& bt, const ed_subspace& sp, int nev, int nchk, double* evals, double* X,
                         double* res, cudaStream_t caller)
{
    const int d = sp.dim, B = bt.B;
    const int64_t n = bt.n;
    ED_REQUIRE(sp.n == n, ED_ERR_ARG, "subspace and batch have different dimensions");
    ED_REQUIRE(nev >= 1 && nev <= d, ED_ERR_ARG, "need 1 <= nev <= subspace dimension");
    ED_REQUIRE(nchk >= 0 && nchk <= nev, ED_ERR_ARG, "need 0 <= nchk <= nev");
    std::vector<int> basis;
    std::vector<double> alpha;
    batch_linear_family(bt, 8, basis, alpha);
    const int r = (int)basis.size();
    SolveStream ss(caller);
    cudaStream_t st = ss.s;
    // projected matrices of the basis members
    DevBuf<double> HQ((size_t)n * d), Akd((size_t)r * d * d);
    for (int k = 0; k < r; ++k) {
        batch_apply(bt, basis[k], sp.Q.p, sp.max_dim, HQ.p, d, d, st);
        ts_gram_dev(sp.Q.p, sp.max_dim, d, HQ.p, d, d, n, Akd.p + (size_t)k * d * d, st);
    }
    HQ.release();
    // every Hamiltonian's projected matrix and its lowest nev Ritz pairs
    DevBuf<double> Md((size_t)nev * d * B);
    if (d <= kDeviceEigenMax && B >= kDeviceEigenMinBatch) {
        // assembled, solved (one CTA per Hamiltonian) and laid out on the device
        DevBuf<double> al((size_t)B * r), Mall((size_t)B * d * d), E((size_t)B * d), Z((size_t)B * d * d),
            ev((size_t)B * nev);
        ED_CUDA(cudaMemcpyAsync(al.p, alpha.data(), alpha.size() * 8, cudaMemcpyHostToDevice, st));
        k_sub_assemble<<<grid1((int64_t)B * d * d), 256, 0, st>>>(Akd.p, r, d, al.p, B, Mall.p); count_launch();
        ED_CUDA(cudaGetLastError());
        sym_eigen_device(d, B, Mall.p, E.p, Z.p, st);
        k_sub_ritz_coef<<<grid1((int64_t)nev * d * B), 256, 0, st>>>(Z.p, E.p, d, B, nev, Md.p, ev.p); count_launch();
        ED_CUDA(cudaGetLastError());
        ED_CUDA(cudaMemcpyAsync(evals, ev.p, (size_t)B * nev * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
    } else {
        // subspaces above the device eigensolver's size, or too few
        // Hamiltonians to beat the host: the same on the host
        std::vector<std::vector<double>> A(r, std::vector<double>((size_t)d * d));
        for (int k = 0; k < r; ++k)
            ED_CUDA(cudaMemcpyAsync(A[k].data(), Akd.p + (size_t)k * d * d, (size_t)d * d * 8, cudaMemcpyDeviceToHost,
                                    st));
        ED_CUDA(cudaStreamSynchronize(st));
        std::vector<double> Mi((size_t)nev * d * B), M((size_t)d * d), th, Yv;
        for (int b = 0; b < B; ++b) {
            for (int i = 0; i < d; ++i)
                for (int j = 0; j <= i; ++j) {
                    double s = 0.0;
                    for (int k = 0; k < r; ++k) {
                        const double* Ak = A[k].data();
                        s += alpha[(size_t)b * r + k] * 0.5 * (Ak[(size_t)i * d + j] + Ak[(size_t)j * d + i]);
                    }
                    M[(size_t)i * d + j] = s;
                    M[(size_t)j * d + i] = s;
                }
            sym_eigen(d, M, th, Yv);
            for (int i = 0; i < nev; ++i) {
                evals[(size_t)b * nev + i] = th[i];
                for (int c = 0; c < d; ++c) Mi[((size_t)i * d + c) * B + b] = Yv[(size_t)c + (size_t)d * i];
            }
        }
        ED_CUDA(cudaMemcpyAsync(Md.p, Mi.data(), Mi.size() * 8, cudaMemcpyHostToDevice, st));
    }
    // Ritz vectors in the batch layout, then their true residuals
    for (int i = 0; i < nev; ++i)
        ts_combine(sp.Q.p, sp.max_dim, d, Md.p + (size_t)i * d * B, B, X + (int64_t)i * n * B, B, n, st);
    if (nchk > 0) {
        std::vector<double> lam((size_t)B * nchk);
        for (int b = 0; b < B; ++b)
            for (int i = 0; i < nchk; ++i) lam[(size_t)b * nchk + i] = evals[(size_t)b * nev + i];
        batch_residuals(bt, full_operands(bt), X, lam.data(), nchk, res, st);
    }
    ED_CUDA(cudaStreamSynchronize(st));
}

}  // namespace edgb

using namespace edgb;

extern "C" {

ed_status ed_subspace_create(int64_t n, int max_dim, ed_subspace** out)
{
    return guard([&] {
        ED_REQUIRE(out, ED_ERR_ARG, "NULL argument");
        *out = nullptr;
        ED_REQUIRE(n >= 1, ED_ERR_ARG, "n must be positive");
        ED_REQUIRE(max_dim >= 1 && max_dim <= kMaxSubspace, ED_ERR_RANGE, "subspace dimension must be 1..256");
        ed_subspace* sp = new ed_subspace();
        try {
            sp->n = n;
            sp->max_dim = max_dim;
            sp->Q.alloc((size_t)n * max_dim);
        } catch (...) {
            delete sp;
            throw;
        }
        *out = sp;
    });
}

ed_status ed_subspace_free(ed_subspace* sp)
{
    return guard([&] { delete sp; });
}

ed_status ed_subspace_dim(const ed_subspace* sp, int* dim)
{
    return guard([&] {
        ED_REQUIRE(sp && dim, ED_ERR_ARG, "NULL argument");
        *dim = sp->dim;
    });
}

ed_status ed_subspace_add(ed_subspace* sp, const double* U, int groups, int width, double drop_tol, int* kept)
{
    return guard([&] {
        ED_REQUIRE(sp && U, ED_ERR_ARG, "NULL argument");
        ED_REQUIRE(groups >= 0 && width >= 1, ED_ERR_ARG, "need groups >= 0 and width >= 1");
        ED_REQUIRE(drop_tol >= 0 && drop_tol < 1, ED_ERR_ARG, "need 0 <= drop_tol < 1");
        ED_REQUIRE(sp->dim + (int64_t)groups * width <= sp->max_dim, ED_ERR_RANGE, "subspace would overflow");
        SolveStream ss(nullptr);
        const int k = subspace_add(*sp, U, groups, width, drop_tol, ss.s);
        if (kept) *kept = k;
    });
}

ed_status ed_batch_subspace_ritz(const ed_batch* bt, const ed_subspace* sp, int nev, int nchk, double* evals,
                                 double* X, double* res)
{
    return guard([&] {
        ED_REQUIRE(bt && sp && evals && X && (nchk == 0 || res), ED_ERR_ARG, "NULL argument");
        batch_subspace_ritz(*bt, *sp, nev, nchk, evals, X, res, nullptr);
    });
}

ed_status ed_batch_solve_subset(const ed_batch* bt, const int* sel, int nsel, const ed_lanczos_params* p,
                                const double* V0, double* evals, double* evecs, ed_batch_info* info)
{
    return guard([&] {
        ED_REQUIRE(bt && sel && p && evals, ED_ERR_ARG, "NULL argument");
        if (info) std::memset(info, 0, sizeof(*info));
        batch_solve(*bt, sel, nsel, *p, V0, evals, evecs, info, nullptr);
    });
}

}  // extern "C"
