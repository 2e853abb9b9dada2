// C ABI of libedgb300: argument checks, handle management, error capture.
// No C++ exception crosses this boundary; every entry returns ed_status and
// leaves a message for ed_last_error() on failure.
#include <atomic>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "ed_lanczos.h"

namespace edgb {

namespace {
thread_local std::string g_last_error;

template <class F>
ed_status guarded(F&& f)
{
    try {
        f();
        return ED_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return ED_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return ED_ERR_INTERNAL;
    } catch (...) {
        g_last_error = "unknown error";
        return ED_ERR_INTERNAL;
    }
}
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {
std::atomic<uint64_t> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(int64_t d) { g_launches.fetch_add((uint64_t)d, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

void terms_upload(ed_terms& t)
{
    t.w_dev.alloc(t.hop.w.size());
    t.hop_off_dev.alloc(t.hop.hop_off.size());
    t.diag_a_dev.alloc(t.hop.diag_a.size());
    t.diag_b_dev.alloc(t.hop.diag_b.size());
    ED_CUDA(cudaMemcpy(t.w_dev.p, t.hop.w.data(), t.hop.w.size() * 8, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.hop_off_dev.p, t.hop.hop_off.data(), t.hop.hop_off.size() * 4, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.diag_a_dev.p, t.hop.diag_a.data(), t.hop.diag_a.size() * 8, cudaMemcpyHostToDevice));
    ED_CUDA(cudaMemcpy(t.diag_b_dev.p, t.hop.diag_b.data(), t.hop.diag_b.size() * 8, cudaMemcpyHostToDevice));
}

}  // namespace edgb

using namespace edgb;

#define ED_NONNULL(p) ED_REQUIRE((p) != nullptr, ED_ERR_ARG, #p " must not be NULL")

extern "C" {

int ed_version(void) { return 1; }

uint64_t ed_kernel_launches(void) { return launch_count(); }

const char* ed_status_string(ed_status s)
{
    switch (s) {
    case ED_OK: return "ok";
    case ED_ERR_ARG: return "invalid argument";
    case ED_ERR_OOM: return "out of memory";
    case ED_ERR_CUDA: return "CUDA error";
    case ED_ERR_NOCONV: return "eigensolver did not converge";
    case ED_ERR_BREAKDOWN: return "Krylov breakdown";
    case ED_ERR_RANGE: return "problem size outside the supported range";
    case ED_ERR_INTERNAL: return "internal consistency check failed";
    case ED_ERR_EMPTY: return "empty sector";
    }
    return "unknown status";
}

const char* ed_last_error(void) { return g_last_error.c_str(); }

int ed_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// ------------------------------------------------------------ term tables

ed_status ed_coulomb_pseudopotentials(int norb, double* out)
{
    return guarded([&] {
        ED_NONNULL(out);
        coulomb_pseudopotentials(norb, out);
    });
}

ed_status ed_quartic_tables(int norb, const double* pp, int npp, uint16_t* ktable, double* vtable)
{
    return guarded([&] {
        ED_NONNULL(ktable);
        ED_NONNULL(vtable);
        ED_REQUIRE(npp == 0 || pp != nullptr, ED_ERR_ARG, "pseudopotentials must not be NULL");
        quartic_tables(norb, pp, npp, ktable, vtable);
    });
}

double ed_clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM)
{
    try {
        return clebsch_gordan(tj1, tm1, tj2, tm2, tJ, tM);
    } catch (...) {
        return 0.0;
    }
}

// ------------------------------------------------------------------ basis

ed_status ed_basis_build(int N, int norb, int two_lz, ed_stream stream, ed_basis** out)
{
    return guarded([&] {
        ED_NONNULL(out);
        *out = nullptr;
        ed_basis* b = new ed_basis();
        b->N = N;
        b->norb = norb;
        b->two_lz = two_lz;
        try {
            basis_build(*b, (cudaStream_t)stream);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

ed_status ed_basis2_build(int N, int norb0, int two_lz, ed_stream stream, ed_basis** out)
{
    return guarded([&] {
        ED_NONNULL(out);
        ED_REQUIRE(norb0 >= 1 && 2 * norb0 + 2 <= kMaxTwoLevelBits, ED_ERR_RANGE,
                   "two-level basis: need 1 <= norb0 and 2*norb0 + 2 <= 48 bits");
        *out = nullptr;
        ed_basis* b = new ed_basis();
        b->N = N;
        b->levels = 2;
        b->norb0 = norb0;
        b->norb1 = norb0 + 2;
        b->norb = 2 * norb0 + 2;
        b->two_lz = two_lz;
        try {
            basis_build(*b, (cudaStream_t)stream);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

ed_status ed_basis_levels(const ed_basis* b, int* levels, int* norb0, int* norb1)
{
    return guarded([&] {
        ED_NONNULL(b);
        if (levels) *levels = b->levels;
        if (norb0) *norb0 = b->levels == 2 ? b->norb0 : b->norb;
        if (norb1) *norb1 = b->levels == 2 ? b->norb1 : 0;
    });
}

ed_status ed_basis_free(ed_basis* b)
{
    return guarded([&] { delete b; });
}

ed_status ed_basis_dim(const ed_basis* b, uint64_t* dim)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(dim);
        *dim = b->dim;
    });
}

ed_status ed_basis_words(const ed_basis* b, const uint64_t** words_dev)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(words_dev);
        *words_dev = b->dim ? b->words.p : nullptr;
    });
}

ed_status ed_basis_get(const ed_basis* b, uint64_t* host_words, uint64_t n)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_REQUIRE(n <= b->dim, ED_ERR_ARG, "copy length exceeds the basis dimension");
        if (n == 0) return;
        ED_NONNULL(host_words);
        ED_CUDA(cudaMemcpy(host_words, b->words.p, n * 8, cudaMemcpyDeviceToHost));
    });
}

ed_status ed_basis_rank(const ed_basis* b, const uint64_t* words_dev, uint64_t* idx_dev, uint64_t m,
                        ed_stream stream)
{
    return guarded([&] {
        ED_NONNULL(b);
        if (m == 0) return;
        ED_NONNULL(words_dev);
        ED_NONNULL(idx_dev);
        basis_rank(*b, words_dev, idx_dev, m, (cudaStream_t)stream);
    });
}

ed_status ed_basis_rank_host(const ed_basis* b, const uint64_t* words, uint64_t* idx, uint64_t m)
{
    return guarded([&] {
        ED_NONNULL(b);
        if (m == 0) return;
        ED_NONNULL(words);
        ED_NONNULL(idx);
        DevBuf<uint64_t> dw(m), di(m);
        ED_CUDA(cudaMemcpy(dw.p, words, m * 8, cudaMemcpyHostToDevice));
        basis_rank(*b, dw.p, di.p, m, nullptr);
        ED_CUDA(cudaMemcpy(idx, di.p, m * 8, cudaMemcpyDeviceToHost));
    });
}

// ------------------------------------------------------------------ terms

ed_status ed_terms_set(int norb, const uint16_t* ktable, const double* vtable, ed_terms** out)
{
    return guarded([&] {
        ED_NONNULL(out);
        *out = nullptr;
        ED_NONNULL(ktable);
        ED_NONNULL(vtable);
        ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals, ED_ERR_RANGE, "norb must be in 2..40 on the device path");
        ed_terms* t = new ed_terms();
        try {
            const size_t K3 = (size_t)norb * norb * norb;
            t->norb = norb;
            t->ktab.assign(ktable, ktable + K3);
            t->vtab.assign(vtable, vtable + K3);
            t->hop = derive_hop_tables(norb, ktable, vtable);
            terms_upload(*t);
        } catch (...) {
            delete t;
            throw;
        }
        *out = t;
    });
}

ed_status ed_terms_free(ed_terms* t)
{
    return guarded([&] { delete t; });
}

// ------------------------------------------------------------ Hamiltonian

ed_status ed_ham_build_crs(const ed_basis* b, const ed_terms* t, int store_upper, ed_stream stream, ed_crs** out)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(t);
        ED_NONNULL(out);
        *out = nullptr;
        ed_crs* a = new ed_crs();
        try {
            ham_build_crs(*b, *t, store_upper, *a, (cudaStream_t)stream);
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

ed_status ed_ham2_build_crs(const ed_basis* b, const ed_terms* t0, const ed_terms* t1, const double* energies0,
                            const double* energies1, int store_upper, ed_stream stream, ed_crs** out)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(t0);
        ED_NONNULL(t1);
        ED_NONNULL(out);
        *out = nullptr;
        ed_crs* a = new ed_crs();
        try {
            ham2_build_crs(*b, *t0, *t1, energies0, energies1, store_upper, *a, (cudaStream_t)stream);
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

ed_status ed_crs_free(ed_crs* a)
{
    return guarded([&] { delete a; });
}

ed_status ed_crs_info(const ed_crs* a, int64_t* n, int64_t* nnz, int* upper)
{
    return guarded([&] {
        ED_NONNULL(a);
        if (n) *n = a->n;
        if (nnz) *nnz = a->nnz;
        if (upper) *upper = a->upper;
    });
}

ed_status ed_crs_arrays(const ed_crs* a, const int64_t** rowptr_dev, const int32_t** col_dev, const double** val_dev)
{
    return guarded([&] {
        ED_NONNULL(a);
        if (rowptr_dev) *rowptr_dev = a->rowptr.p;
        if (col_dev) *col_dev = a->col.p;
        if (val_dev) *val_dev = a->val.p;
    });
}

ed_status ed_crs_get(const ed_crs* a, int64_t* rowptr, int32_t* col, double* val)
{
    return guarded([&] {
        ED_NONNULL(a);
        if (rowptr) ED_CUDA(cudaMemcpy(rowptr, a->rowptr.p, (size_t)(a->n + 1) * 8, cudaMemcpyDeviceToHost));
        if (a->nnz > 0) {
            if (col) ED_CUDA(cudaMemcpy(col, a->col.p, (size_t)a->nnz * 4, cudaMemcpyDeviceToHost));
            if (val) ED_CUDA(cudaMemcpy(val, a->val.p, (size_t)a->nnz * 8, cudaMemcpyDeviceToHost));
        }
    });
}

ed_status ed_ham_diagonal(const ed_basis* b, const ed_terms* t, double* diag_dev, ed_stream stream)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(t);
        ED_REQUIRE(t->norb == b->norb, ED_ERR_ARG, "terms and basis have different orbital counts");
        if (b->dim == 0) return;
        ED_NONNULL(diag_dev);
        ham_diagonal(*b, *t, diag_dev, (cudaStream_t)stream);
    });
}

// ------------------------------------------------------------------- H*v

ed_status ed_spmv(const ed_crs* a, const double* x_dev, double* y_dev, ed_stream stream)
{
    return guarded([&] {
        ED_NONNULL(a);
        if (a->n == 0) return;
        ED_NONNULL(x_dev);
        ED_NONNULL(y_dev);
        ED_REQUIRE(x_dev != y_dev, ED_ERR_ARG, "x and y must be distinct");
        spmv(*a, x_dev, y_dev, (cudaStream_t)stream);
    });
}

ed_status ed_spmv_kernel(const ed_crs* a, int kernel, const double* x_dev, double* y_dev, ed_stream stream)
{
    return guarded([&] {
        ED_NONNULL(a);
        if (a->n == 0) return;
        ED_NONNULL(x_dev);
        ED_NONNULL(y_dev);
        ED_REQUIRE(x_dev != y_dev, ED_ERR_ARG, "x and y must be distinct");
        spmv_kernel(*a, kernel, x_dev, y_dev, (cudaStream_t)stream);
    });
}

ed_status ed_spmv_staged_wait_test(const ed_crs* a, const double* x_dev, double* y_dev, long long wait_cycles,
                                   int* timeouts)
{
    return guarded([&] {
        ED_NONNULL(a);
        ED_NONNULL(x_dev);
        ED_NONNULL(y_dev);
        ED_NONNULL(timeouts);
        *timeouts = spmv_staged_wait_test(*a, x_dev, y_dev, wait_cycles, nullptr);
    });
}

ed_status ed_crs_set_product_kernel(ed_crs* a, int kernel)
{
    return guarded([&] {
        ED_NONNULL(a);
        ED_REQUIRE(kernel >= 0 && kernel <= 8, ED_ERR_ARG, "kernel: 0 (chosen by shape) or 1-8 (ed_spmv_kernel)");
        ED_REQUIRE(kernel == 0 || !a->upper, ED_ERR_ARG, "kernels 1-8 take full storage");
        a->product_kernel = kernel;
    });
}

ed_status ed_fp64_fma_rate(int iters, int blocks_per_sm, double* fma_per_second)
{
    return guarded([&] {
        ED_NONNULL(fma_per_second);
        ED_REQUIRE(iters >= 1 && iters <= (1 << 24) && blocks_per_sm >= 1 && blocks_per_sm <= 32, ED_ERR_ARG,
                   "1 <= iters <= 2^24, 1 <= blocks_per_sm <= 32");
        *fma_per_second = measure_dfma_rate(iters, blocks_per_sm);
    });
}

ed_status ed_hv_matfree(const ed_basis* b, const ed_terms* t, const double* x_dev, double* y_dev, ed_stream stream)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(t);
        ED_REQUIRE(t->norb == b->norb, ED_ERR_ARG, "terms and basis have different orbital counts");
        if (b->dim == 0) return;
        ED_NONNULL(x_dev);
        ED_NONNULL(y_dev);
        ED_REQUIRE(x_dev != y_dev, ED_ERR_ARG, "x and y must be distinct");
        cudaStream_t st = (cudaStream_t)stream;
        basis_compact_tables(*b, st);
        DevBuf<double> diag(b->dim);
        ham_diagonal(*b, *t, diag.p, st);
        hv_matfree(*b, *t, diag.p, x_dev, y_dev, st);
        ED_CUDA(cudaStreamSynchronize(st));
    });
}

// ----------------------------------------------------------------- solver

ed_status ed_op_from_crs(const ed_crs* a, ed_op** out)
{
    return guarded([&] {
        ED_NONNULL(a);
        ED_NONNULL(out);
        ed_op* op = new ed_op();
        op->kind = ed_op::CRS;
        op->n = a->n;
        op->crs = a;
        *out = op;
    });
}

ed_status ed_op_matfree(const ed_basis* b, const ed_terms* t, ed_op** out)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(t);
        ED_NONNULL(out);
        ED_REQUIRE(t->norb == b->norb, ED_ERR_ARG, "terms and basis have different orbital counts");
        ed_op* op = new ed_op();
        try {
            op->kind = ed_op::MATFREE;
            op->n = (int64_t)b->dim;
            op->basis = b;
            op->terms = t;
            op->diag.alloc(b->dim ? b->dim : 1);
            if (b->dim) ham_diagonal(*b, *t, op->diag.p, nullptr);
            basis_compact_tables(*b, nullptr);   // before any product is captured into a graph
            ED_CUDA(cudaStreamSynchronize(nullptr));
        } catch (...) {
            delete op;
            throw;
        }
        *out = op;
    });
}

ed_status ed_op_host_callback(int64_t n, ed_host_matvec fn, void* user, ed_op** out)
{
    return guarded([&] {
        ED_NONNULL(fn);
        ED_NONNULL(out);
        ED_REQUIRE(n >= 1, ED_ERR_ARG, "n must be positive");
        ed_op* op = new ed_op();
        op->kind = ed_op::HOST;
        op->n = n;
        op->fn = fn;
        op->user = user;
        op->hx.resize(n);
        op->hy.resize(n);
        *out = op;
    });
}

ed_status ed_op_free(ed_op* op)
{
    return guarded([&] { delete op; });
}

ed_status ed_op_dim(const ed_op* op, int64_t* n)
{
    return guarded([&] {
        ED_NONNULL(op);
        ED_NONNULL(n);
        *n = op->n;
    });
}

ed_status ed_lanczos_device(const ed_op* op, const ed_lanczos_params* p, const double* v0_dev, double* evals_host,
                            double* evecs_dev, ed_solve_info* info)
{
    return guarded([&] {
        ED_NONNULL(op);
        ED_NONNULL(p);
        ED_NONNULL(evals_host);
        if (info) std::memset(info, 0, sizeof(*info));
        lanczos_solve(*op, *p, v0_dev, evals_host, evecs_dev, info, nullptr);
    });
}

ed_status ed_lanczos_two_level(const ed_basis* b, const ed_op* op, const ed_lanczos_params* p, const double* v0_host,
                               double* evals_host, double* evecs_host, ed_solve_info* info)
{
    return guarded([&] {
        ED_NONNULL(b);
        ED_NONNULL(op);
        ED_NONNULL(p);
        ED_NONNULL(evals_host);
        if (info) std::memset(info, 0, sizeof(*info));
        const int64_t n = op->n;
        ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
        ED_REQUIRE(p->nev >= 1 && p->nev <= n, ED_ERR_ARG, "need 1 <= nev <= n");
        DevBuf<double> v0, ev;
        if (v0_host) {
            v0.alloc(n);
            ED_CUDA(cudaMemcpy(v0.p, v0_host, (size_t)n * 8, cudaMemcpyHostToDevice));
        }
        if (evecs_host) ev.alloc((size_t)n * p->nev);
        lanczos_solve_two_level(*b, *op, *p, v0.p, evals_host, ev.p, info, nullptr);
        if (evecs_host)
            ED_CUDA(cudaMemcpy(evecs_host, ev.p, (size_t)n * p->nev * 8, cudaMemcpyDeviceToHost));
    });
}

ed_status ed_lanczos(const ed_op* op, const ed_lanczos_params* p, const double* v0_host, double* evals_host,
                     double* evecs_host, ed_solve_info* info)
{
    return guarded([&] {
        ED_NONNULL(op);
        ED_NONNULL(p);
        ED_NONNULL(evals_host);
        if (info) std::memset(info, 0, sizeof(*info));
        const int64_t n = op->n;
        ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
        ED_REQUIRE(p->nev >= 1 && p->nev <= n, ED_ERR_ARG, "need 1 <= nev <= n");
        DevBuf<double> v0, ev;
        if (v0_host) {
            v0.alloc(n);
            ED_CUDA(cudaMemcpy(v0.p, v0_host, (size_t)n * 8, cudaMemcpyHostToDevice));
        }
        if (evecs_host) ev.alloc((size_t)n * p->nev);
        ed_status deferred = ED_OK;
        std::string msg;
        try {
            lanczos_solve(*op, *p, v0.p, evals_host, ev.p, info, nullptr);
        } catch (const Error& e) {
            if (e.code != ED_ERR_NOCONV) throw;
            deferred = e.code;   // still hand back the best Ritz pairs
            msg = e.what();
        }
        if (evecs_host)
            ED_CUDA(cudaMemcpy(evecs_host, ev.p, (size_t)n * p->nev * 8, cudaMemcpyDeviceToHost));
        if (deferred != ED_OK) throw Error(deferred, msg);
    });
}

ed_status ed_dense_sym_eigen(int m, const double* a, double* evals, double* evecs)
{
    return guarded([&] {
        ED_NONNULL(a);
        ED_NONNULL(evals);
        ED_REQUIRE(m >= 1 && m <= 20000, ED_ERR_ARG, "m out of range");
        std::vector<double> A(a, a + (size_t)m * m), ev, vec;
        sym_eigen(m, A, ev, vec);
        std::memcpy(evals, ev.data(), (size_t)m * 8);
        if (evecs) std::memcpy(evecs, vec.data(), (size_t)m * m * 8);
    });
}

ed_status ed_sym_eigen_batched(int m, int count, const double* a, double* evals, double* evecs)
{
    return guarded([&] {
        ED_NONNULL(a);
        ED_NONNULL(evals);
        ED_NONNULL(evecs);
        ED_REQUIRE(m >= 1 && m <= kDeviceEigenMax, ED_ERR_RANGE, "m must be 1..128");
        ED_REQUIRE(count >= 1, ED_ERR_ARG, "count must be positive");
        sym_eigen_batched(m, count, a, evals, evecs, nullptr);
    });
}

ed_status ed_residuals(const ed_op* op, const double* x_dev, const double* lambda_host, int k, double* res_host)
{
    return guarded([&] {
        ED_NONNULL(op);
        ED_NONNULL(x_dev);
        ED_NONNULL(lambda_host);
        ED_NONNULL(res_host);
        ED_REQUIRE(k >= 1, ED_ERR_ARG, "k must be positive");
        residual_norms(*op, x_dev, lambda_host, k, res_host, nullptr);
    });
}

ed_status ed_solve_sector(int N, int norb, int two_lz, const double* pp, int npp, int matfree,
                          const ed_lanczos_params* p, const double* v0_host, double* evals_host, double* evecs_host,
                          ed_solve_info* info)
{
    return guarded([&] {
        ED_NONNULL(p);
        ED_NONNULL(evals_host);
        ED_REQUIRE(npp == 0 || pp != nullptr, ED_ERR_ARG, "pseudopotentials must not be NULL");
        if (info) std::memset(info, 0, sizeof(*info));
        ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals, ED_ERR_RANGE, "norb must be in 2..40 on the device path");
        ed_basis b;
        b.N = N;
        b.norb = norb;
        b.two_lz = two_lz;
        basis_build(b, nullptr);
        ED_REQUIRE(b.dim > 0, ED_ERR_EMPTY, "the requested sector has dimension 0");
        const size_t K3 = (size_t)norb * norb * norb;
        ed_terms t;
        t.norb = norb;
        t.ktab.resize(K3);
        t.vtab.resize(K3);
        quartic_tables(norb, pp, npp, t.ktab.data(), t.vtab.data());
        t.hop = derive_hop_tables(norb, t.ktab.data(), t.vtab.data());
        terms_upload(t);
        ed_crs a;
        ed_op op;
        op.n = (int64_t)b.dim;
        if (matfree) {
            op.kind = ed_op::MATFREE;
            op.basis = &b;
            op.terms = &t;
            op.diag.alloc(b.dim);
            ham_diagonal(b, t, op.diag.p, nullptr);
            basis_compact_tables(b, nullptr);
        } else {
            ham_build_crs(b, t, 0, a, nullptr);
            op.kind = ed_op::CRS;
            op.crs = &a;
        }
        const int64_t n = (int64_t)b.dim;
        ED_REQUIRE(p->nev >= 1 && p->nev <= n, ED_ERR_ARG, "need 1 <= nev <= sector dimension");
        DevBuf<double> v0, ev;
        if (v0_host) {
            v0.alloc(n);
            ED_CUDA(cudaMemcpy(v0.p, v0_host, (size_t)n * 8, cudaMemcpyHostToDevice));
        }
        if (evecs_host) ev.alloc((size_t)n * p->nev);
        lanczos_solve(op, *p, v0.p, evals_host, ev.p, info, nullptr);
        if (evecs_host)
            ED_CUDA(cudaMemcpy(evecs_host, ev.p, (size_t)n * p->nev * 8, cudaMemcpyDeviceToHost));
    });
}

}  // extern "C"
