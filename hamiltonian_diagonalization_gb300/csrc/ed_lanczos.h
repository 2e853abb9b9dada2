// Operator handle and eigensolver entry shared by ed_lanczos.cu and the C ABI.
#pragma once

#include <vector>

#include "ed_internal.h"

struct ed_op {
    enum Kind { CRS = 0, MATFREE = 1, HOST = 2 };
    Kind kind = CRS;
    int64_t n = 0;
    const ed_crs* crs = nullptr;
    const ed_basis* basis = nullptr;
    const ed_terms* terms = nullptr;
    edgb::DevBuf<double> diag;          // matrix-free: stored diagonal
    ed_host_matvec fn = nullptr;
    void* user = nullptr;
    mutable std::vector<double> hx, hy; // host staging for HOST operators
};

namespace edgb {
void op_apply(const ed_op& op, const double* x, double* y, cudaStream_t st);
// Lowest p.nev eigenpairs; v0_dev may be null; evecs_dev (n*nev) may be null.
void lanczos_solve(const ed_op& op, const ed_lanczos_params& p, const double* v0_dev, double* evals_host,
                   double* evecs_dev, ed_solve_info* info, cudaStream_t st);
void residual_norms(const ed_op& op, const double* x, const double* lambda, int k, double* res, cudaStream_t st);
}  // namespace edgb
