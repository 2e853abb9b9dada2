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
// eigenvector matrix V (in shared memory too up to m = 118, else in global
// memory), with the rotated 2 x 2 block set from
// Rutishauser's formulas (a_pq = 0 exactly, a_pp - t a_pq, a_qq + t a_pq).
// A pair is rotated only when |a_pq| > 1e-16 sqrt(|a_pp a_qq|) (or when
// a_pp a_qq = 0 and a_pq != 0), and the iteration ends after a sweep that
// rotates no pair.  Jacobi is at least as accurate as the Householder + QR
// route (relatively accurate eigenvalues).  Eigenvalues come out ascending
// with their columns.
#include <algorithm>
#include <cmath>
#include <map>

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

// A: count matrices, m x m row-major; evals count x m; the accumulated
// eigenvectors V (V[i + vld j] = component i of eigenvector j) in shared
// memory after A when VS (m up to 118), else in Vw (count x m x m, global),
// then sorted into evecs (count x m x m, column-major).
template <bool VS>
__global__ void __launch_bounds__(kEigThreads) k_sym_jacobi(const double* __restrict__ Ain, int m,
                                                            double* __restrict__ evals, double* __restrict__ Vw,
                                                            double* __restrict__ evecs, int max_sweeps)
{
    extern __shared__ double smem[];
    const int ld = m + 1;                            // padded row stride
    double* a = smem;                                // m x ld
    double* cs = a + (size_t)(VS ? 2 : 1) * m * ld;  // cos per pair (after A, and V when VS)
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
    const int vld = VS ? ld : m;                     // column stride of V
    double* V = VS ? a + (size_t)m * ld : Vw + (size_t)mat * m * m;
    for (int t = threadIdx.x; t < m * m; t += kEigThreads) {
        const int i = t / m, j = t % m;
        a[i * ld + j] = A[t];
        V[i + (size_t)vld * j] = (i == j) ? 1.0 : 0.0;   // identity
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
            // columns p, q of A and of V; the rotated 2 x 2 block (rows p, q
            // of columns p, q, written only by this pair's threads) from the
            // exact formulas
            for (int t = threadIdx.x; t < npairs * m; t += kEigThreads) {
                const int k = t / m, i = t % m;
                const int p = pp[k];
                if (p < 0) continue;
                const int q = qq[k];
                const double c = cs[k], s = sn[k];
                if (i == p) {
                    a[p * ld + p] = fma(-tn[k], apq0[k], app0[k]);
                    a[p * ld + q] = 0.0;
                } else if (i == q) {
                    a[q * ld + q] = fma(tn[k], apq0[k], aqq0[k]);
                    a[q * ld + p] = 0.0;
                } else {
                    const double x = a[i * ld + p], y = a[i * ld + q];
                    a[i * ld + p] = c * x - s * y;
                    a[i * ld + q] = fma(s, x, c * y);
                }
                const double vx = V[i + (size_t)vld * p], vy = V[i + (size_t)vld * q];
                V[i + (size_t)vld * p] = c * vx - s * vy;
                V[i + (size_t)vld * q] = fma(s, vx, c * vy);
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
        out[i + (size_t)m * rank[j]] = V[i + (size_t)vld * j];
    }
}

size_t jacobi_smem(int m, bool vs)
{
    return (size_t)(vs ? 2 : 1) * m * (m + 1) * 8 + (size_t)3 * kEigMax * 8 + (size_t)kEigMax * 4;
}
constexpr size_t kSmemLimit = 227 * 1024 - 2048;   // dynamic shared memory per CTA, less the static arrays

}  // namespace

// Device scratch of the eigensolver, kept per host thread and device and
// grown on demand, so that a solver restart costs no allocation.
struct EigWork {
    DevBuf<double> V, A, E, Z;
    int smem_set[2] = {0, 0};
};
EigWork& eig_work()
{
    thread_local std::map<int, EigWork> work;
    int dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    return work[dev];
}

void jacobi_launch(int m, int count, const double* A_dev, double* evals_dev, double* evecs_dev, EigWork& w,
                   cudaStream_t st)
{
    ED_REQUIRE(m >= 1 && m <= kEigMax, ED_ERR_RANGE, "device eigensolver: 1 <= m <= 128");
    const bool vs = jacobi_smem(m, true) <= kSmemLimit;
    const size_t smem = jacobi_smem(m, vs);
    if ((int)smem > w.smem_set[vs]) {
        ED_CUDA(cudaFuncSetAttribute(vs ? k_sym_jacobi<true> : k_sym_jacobi<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        w.smem_set[vs] = (int)smem;
    }
    if (vs) {
        k_sym_jacobi<true><<<count, kEigThreads, smem, st>>>(A_dev, m, evals_dev, nullptr, evecs_dev, 60);
    } else {
        w.V.alloc_at_least((size_t)count * m * m);
        k_sym_jacobi<false><<<count, kEigThreads, smem, st>>>(A_dev, m, evals_dev, w.V.p, evecs_dev, 60);
    }
    count_launch();
    ED_CUDA(cudaGetLastError());
}

void sym_eigen_device(int m, int count, const double* A_dev, double* evals_dev, double* evecs_dev, cudaStream_t st)
{
    if (count <= 0) return;
    jacobi_launch(m, count, A_dev, evals_dev, evecs_dev, eig_work(), st);
}

// Host matrices in and out (the restart bookkeeping of the solvers keeps the
// projected matrices and Ritz coefficients on the host): uploads, solves on
// the device, downloads.  Same layouts as sym_eigen.
void sym_eigen_batched(int m, int count, const double* a_host, double* evals_host, double* evecs_host,
                       cudaStream_t st)
{
    if (count <= 0) return;
    EigWork& w = eig_work();
    const size_t mm = (size_t)count * m * m;
    w.A.alloc_at_least(mm);
    w.E.alloc_at_least((size_t)count * m);
    w.Z.alloc_at_least(mm);
    ED_CUDA(cudaMemcpyAsync(w.A.p, a_host, mm * 8, cudaMemcpyHostToDevice, st));
    jacobi_launch(m, count, w.A.p, w.E.p, w.Z.p, w, st);
    ED_CUDA(cudaMemcpyAsync(evals_host, w.E.p, (size_t)count * m * 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaMemcpyAsync(evecs_host, w.Z.p, mm * 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
}

}  // namespace edgb
