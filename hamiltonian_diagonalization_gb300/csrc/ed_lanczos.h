// Operator handle and eigensolver entry shared by ed_lanczos.cu and the C ABI.
#pragma once

#include <vector>

#include "ed_internal.h"

struct ed_op {
    enum Kind { CRS = 0, MATFREE = 1, HOST = 2, DEFLATED = 3 };
    Kind kind = CRS;
    int64_t n = 0;
    const ed_crs* crs = nullptr;
    const ed_basis* basis = nullptr;
    const ed_terms* terms = nullptr;
    edgb::DevBuf<double> diag;          // matrix-free: stored diagonal
    ed_host_matvec fn = nullptr;
    void* user = nullptr;
    mutable std::vector<double> hx, hy; // host staging for HOST operators
    // DEFLATED: inner + shift * X X^T for nlock orthonormal device columns X
    // (Wielandt deflation of converged eigenvectors); scratch for the dots
    const ed_op* inner = nullptr;
    const double* lock = nullptr;
    int nlock = 0;
    double shift = 0.0;
    int lock_blocks = 0;
    edgb::DevBuf<double> lock_part;     // nlock * lock_blocks partials, then nlock coefficients
    edgb::DevBuf<unsigned int> lock_counter;
};

namespace edgb {

// Instantiated restart cycles, one per (first step, Krylov buffer), with the
// number of kernels each launches.
struct CycleGraphs {
    struct Entry {
        int k;
        const double* V;
        cudaGraphExec_t exec;
        int64_t kernels;
    };
    std::vector<Entry> e;
    ~CycleGraphs() { for (auto& x : e) cudaGraphExecDestroy(x.exec); }
    Entry* find(int k, const double* V)
    {
        for (auto& x : e)
            if (x.k == k && x.V == V) return &x;
        return nullptr;
    }
};

// The solver's own stream: stream capture is not available on the legacy
// default stream, so the solve runs on a private non-blocking stream that
// is ordered after the caller's stream on entry and before it on exit.
struct SolveStream {
    cudaStream_t s = nullptr;
    cudaStream_t caller = nullptr;
    cudaEvent_t e = nullptr;
    explicit SolveStream(cudaStream_t c) : caller(c)
    {
        ED_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        ED_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ED_CUDA(cudaEventRecord(e, caller));
        ED_CUDA(cudaStreamWaitEvent(s, e, 0));
    }
    ~SolveStream()
    {
        if (cudaEventRecord(e, s) == cudaSuccess) cudaStreamWaitEvent(caller, e, 0);
        cudaEventDestroy(e);
        cudaStreamDestroy(s);
    }
};

// Thick-restart basis rotation out[:, c] = sum_j V[:, j] Y[j, c], c < k
// (V n x m and out n x k column-major on the device, Y host, column-major with
// leading dimension ldy).  method 0: tensor cores (FP64-accurate digit
// splitting) when m <= kRotateTensorMaxM, else FP64; 1: FP64; 2: tensor cores.
constexpr int kRotateTensorMaxM = 64;
struct RotateScratch {
    DevBuf<double> y;
    DevBuf<uint16_t> ydig;
    DevBuf<int> yexp;
    std::vector<uint16_t> ydig_h;
    std::vector<int> yexp_h;
};
void rotate_basis(const double* V, int64_t n, int m, const double* Y_host, int ldy, int k, double* out,
                  RotateScratch& sc, int method, cudaStream_t st);

void op_apply(const ed_op& op, const double* x, double* y, cudaStream_t st);
// once-per-operator work of the product, before a solver captures its cycles
void op_prepare(const ed_op& op, cudaStream_t st);
// throws when one of the operator's products ran out of a bounded wait
void op_check(const ed_op& op, cudaStream_t st);
// Lowest p.nev eigenpairs; v0_dev may be null; evecs_dev (n*nev) may be null.
void lanczos_solve(const ed_op& op, const ed_lanczos_params& p, const double* v0_dev, double* evals_host,
                   double* evecs_dev, ed_solve_info* info, cudaStream_t st);
void residual_norms(const ed_op& op, const double* x, const double* lambda, int k, double* res, cudaStream_t st);
// The nev lowest eigenpairs of a stored matrix (n rows, values double or,
// with complex_values, (re, im) pairs) when no off-diagonal element exceeds
// 1e-14 in modulus: its nev smallest diagonal entries ascending (ties by
// index), each with its unit vector in evecs_dev (n * nev, real or complex
// layout; may be null).  Returns false, doing nothing more, otherwise.
bool diagonal_spectrum(const int64_t* rowptr, const int32_t* col, const double* val, int complex_values, int64_t n,
                       int nev, double* evals_host, double* evecs_dev, ed_solve_info* info, cudaStream_t st);
// Lowest p.nev eigenpairs of a two-level Hamiltonian, every copy of a
// degenerate eigenvalue from the level-exchange ladder of basis b.
void lanczos_solve_two_level(const ed_basis& b, const ed_op& op, const ed_lanczos_params& p, const double* v0_dev,
                             double* evals_host, double* evecs_dev, ed_solve_info* info, cudaStream_t caller);
}  // namespace edgb
