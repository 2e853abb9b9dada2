// Dense symmetric eigen-decompositions of the small projected matrices on the
// device, in FP64: the Rayleigh-Ritz problems of the thick-restart Lanczos
// (one matrix per restart), of the batched solver (one per problem) and of the
// shared-subspace Ritz step (one per Hamiltonian).  They stand in for the
// Hessenberg/Schur work ARPACK performs on the host inside pdneupd_
// (utilities/wrappers/arpack_wrapper.hpp:880).
//
// Method: cyclic two-sided Jacobi with the parallel round-robin ordering
// (Golub & Van Loan, "Matrix Computations", sections 8.5.2-8.5.4; the
// rotation from Rutishauser's stable formulas), one CTA per matrix.  A sweep
// is m_pad - 1 steps (m_pad = m rounded up to even, with a dummy index for odd
// m); each step rotates m_pad / 2 disjoint pairs (p, q) at once: rows, then
// columns of A in shared memory, then the columns of the accumulated
// eigenvector matrix V in global memory; the rotated 2 x 2 block is then set
// from Rutishauser's formulas (a_pq = 0 exactly, a_pp - t a_pq, a_qq + t a_pq).
// A pair is rotated only when |a_pq| > 1e-16 sqrt(|a_pp a_qq|) (or when
// a_pp a_qq = 0 and a_pq != 0), and the iteration ends after a sweep that
// rotates no pair.  Jacobi is at least as accurate as the Householder + QR
// route (relatively accurate eigenvalues).  Eigenvalues come out ascending
// with their columns.
#include <algorithm>
#include <cmath>

#include "ed_internal.h"

namespace edgb {

namespace {

constexpr int kEigMax = kDeviceEigenMax;   // largest matrix; A in shared memory (129 KB)
constexpr int kEigThreads = 256;

// player at position x of round r of the round-robin schedule over mp players
__device__ __forceinline__ int rr_player(int x, int r, int mp)
{
    return x == 0 ? 0 : ((x - 1 + r) % (mp - 1)) + 1;
}

// A: count matrices, m x m row-major; evals count x m; Vw: count x m x m
// column-major (V[i + m j] = component i of eigenvector j), the accumulator,
// then sorted into evecs (same layout).
__global__ void __launch_bounds__(kEigThreads) k_sym_jacobi(const double* __restrict__ Ain, int m,
                                                            double* __restrict__ evals, double* __restrict__ Vw,
                                                            double* __restrict__ evecs, int max_sweeps)
{
    extern __shared__ double smem[];
    const int ld = m + 1;                            // padded row stride
    double* a = smem;                                // m x ld
    double* cs = a + (size_t)m * ld;                 // cos per pair
    double* sn = cs + kEigMax / 2;                   // sin per pair
    double* tn = sn + kEigMax / 2;                   // tan per pair
    double* apq0 = tn + kEigMax / 2;                 // the pair's a_pq, a_pp, a_qq before the rotation
    double* app0 = apq0 + kEigMax / 2;
    double* aqq0 = app0 + kEigMax / 2;
    int* pp = (int*)(aqq0 + kEigMax / 2);            // p per pair (-1: skip)
    int* qq = pp + kEigMax / 2;
    __shared__ int rotated;
    __shared__ int rank[kEigMax];
    const int mat = blockIdx.x;
    const double* A = Ain + (size_t)mat * m * m;
    double* V = Vw + (size_t)mat * m * m;
    for (int t = threadIdx.x; t < m * m; t += kEigThreads) {
        const int i = t / m, j = t % m;
        a[i * ld + j] = A[t];
        V[t] = (t % (m + 1) == 0) ? 1.0 : 0.0;      // identity
    }
    __syncthreads();
    const int mp = m + (m & 1);
    const int npairs = mp / 2;
    for (int sweep = 0; sweep < max_sweeps && m > 1; ++sweep) {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < mp - 1; ++r) {
            // the rotation of each pair
            for (int k = threadIdx.x; k < npairs; k += kEigThreads) {
                int p = rr_player(k, r, mp), q = rr_player(mp - 1 - k, r, mp);
                if (p > q) { const int x = p; p = q; q = x; }
                double c = 1.0, s = 0.0, t = 0.0;
                int use = 0;
                if (q < m) {
                    const double apq = a[p * ld + q];
                    const double app = a[p * ld + p], aqq = a[q * ld + q];
                    const double scale = sqrt(fabs(app) * fabs(aqq));
                    if (apq != 0.0 && (scale == 0.0 || fabs(apq) > 1e-16 * scale)) {
                        const double theta = (aqq - app) / (2.0 * apq);
                        if (fabs(theta) > 1e150) t = 0.5 / theta;
                        else t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
                        c = 1.0 / sqrt(fma(t, t, 1.0));
                        s = t * c;
                        use = 1;
                    }
                    apq0[k] = apq;
                    app0[k] = app;
                    aqq0[k] = aqq;
                }
                cs[k] = c;
                sn[k] = s;
                tn[k] = t;
                pp[k] = use ? p : -1;
                qq[k] = q;
                if (use) rotated = 1;
            }
            __syncthreads();
            // rows p, q of A
            for (int t = threadIdx.x; t < npairs * m; t += kEigThreads) {
                const int k = t / m, j = t % m;
                const int p = pp[k];
                if (p < 0) continue;
                const int q = qq[k];
                const double c = cs[k], s = sn[k];
                const double x = a[p * ld + j], y = a[q * ld + j];
                a[p * ld + j] = c * x - s * y;
                a[q * ld + j] = fma(s, x, c * y);
            }
            __syncthreads();
            // columns p, q of A and of V
            for (int t = threadIdx.x; t < npairs * m; t += kEigThreads) {
                const int k = t / m, i = t % m;
                const int p = pp[k];
                if (p < 0) continue;
                const int q = qq[k];
                const double c = cs[k], s = sn[k];
                const double x = a[i * ld + p], y = a[i * ld + q];
                a[i * ld + p] = c * x - s * y;
                a[i * ld + q] = fma(s, x, c * y);
                const double vx = V[i + (size_t)m * p], vy = V[i + (size_t)m * q];
                V[i + (size_t)m * p] = c * vx - s * vy;
                V[i + (size_t)m * q] = fma(s, vx, c * vy);
            }
            __syncthreads();
            // the rotated 2 x 2 blocks from the exact formulas
            for (int k = threadIdx.x; k < npairs; k += kEigThreads) {
                const int p = pp[k];
                if (p < 0) continue;
                const int q = qq[k];
                a[p * ld + p] = fma(-tn[k], apq0[k], app0[k]);
                a[q * ld + q] = fma(tn[k], apq0[k], aqq0[k]);
                a[p * ld + q] = 0.0;
                a[q * ld + p] = 0.0;
            }
            __syncthreads();
        }
        if (!rotated) break;
        __syncthreads();
    }
    // ascending order: the rank of each eigenvalue (ties by index)
    for (int i = threadIdx.x; i < m; i += kEigThreads) {
        const double e = a[i * ld + i];
        int rk = 0;
        for (int j = 0; j < m; ++j) {
            const double f = a[j * ld + j];
            rk += (f < e || (f == e && j < i)) ? 1 : 0;
        }
        rank[i] = rk;
        evals[(size_t)mat * m + rk] = e;
    }
    __syncthreads();
    double* out = evecs + (size_t)mat * m * m;
    for (int t = threadIdx.x; t < m * m; t += kEigThreads) {
        const int j = t / m, i = t % m;              // column j, row i
        out[i + (size_t)m * rank[j]] = V[i + (size_t)m * j];
    }
}

size_t jacobi_smem(int m) { return (size_t)m * (m + 1) * 8 + (size_t)3 * kEigMax * 8 + (size_t)kEigMax * 4; }

}  // namespace

void sym_eigen_device(int m, int count, const double* A_dev, double* evals_dev, double* evecs_dev, cudaStream_t st)
{
    ED_REQUIRE(m >= 1 && m <= kEigMax, ED_ERR_RANGE, "device eigensolver: 1 <= m <= 128");
    if (count <= 0) return;
    DevBuf<double> V((size_t)count * m * m);
    const size_t smem = jacobi_smem(m);
    ED_CUDA(cudaFuncSetAttribute(k_sym_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_sym_jacobi<<<count, kEigThreads, smem, st>>>(A_dev, m, evals_dev, V.p, evecs_dev, 60);
    count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));   // V is freed on return
}

// Host matrices in and out (the restart bookkeeping of the solvers keeps the
// projected matrices and Ritz coefficients on the host): uploads, solves on
// the device, downloads.  Same layouts as sym_eigen.
void sym_eigen_batched(int m, int count, const double* a_host, double* evals_host, double* evecs_host,
                       cudaStream_t st)
{
    DevBuf<double> A((size_t)count * m * m), E((size_t)count * m), Z((size_t)count * m * m);
    ED_CUDA(cudaMemcpyAsync(A.p, a_host, A.bytes(), cudaMemcpyHostToDevice, st));
    sym_eigen_device(m, count, A.p, E.p, Z.p, st);
    ED_CUDA(cudaMemcpyAsync(evals_host, E.p, E.bytes(), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaMemcpyAsync(evecs_host, Z.p, Z.bytes(), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
}

void sym_eigen_small(int m, const std::vector<double>& a, std::vector<double>& evals, std::vector<double>& evecs,
                     cudaStream_t st)
{
    ED_REQUIRE(m >= 1 && (int64_t)a.size() >= (int64_t)m * m, ED_ERR_ARG, "sym_eigen_small: bad size");
    if (m > kDeviceEigenMax) {
        sym_eigen(m, a, evals, evecs);
        return;
    }
    evals.resize(m);
    evecs.resize((size_t)m * m);
    sym_eigen_batched(m, 1, a.data(), evals.data(), evecs.data(), st);
}

}  // namespace edgb
