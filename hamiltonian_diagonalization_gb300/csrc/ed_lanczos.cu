// Thick-restart Lanczos with full FP64 reorthogonalisation on the device
// (K7 vector kernels, K8 projected eigenproblem on the host, K9 residuals).
//
// Stands in for ArpackWrapper::DiagonalizeSymmetricMatrix<double>
// (utilities/wrappers/arpack_wrapper.hpp:595-937), which runs ARPACK's
// implicitly restarted Arnoldi (pdnaupd_/pdneupd_, WHICH="SR",
// NCV = min(N, 2*NEV+21), 2000 iterations) with MatrixVectorFunction::Simple
// as the reverse-communication product.  Here the Krylov basis lives in HBM,
// every vector operation is a device kernel, and the host only sees the
// small projected matrix once per restart cycle.
//
// One Lanczos step j (v_j = V[:,j], w written into V[:,j+1]):
//   w = H v_j
//   local three-term step  alpha = v_j.w ; w -= alpha v_j + beta_{j-1} v_{j-1}
//   full Gram-Schmidt pass c = V[:,0..j]^T w ; w -= V c  (the projections are
//   added to column j of the projected matrix), second pass when the norm
//   dropped below 1/sqrt(2) of its value before the pass (DGKS test), and
//   always on the first step of a cycle, where the thick-restart arrow makes
//   the local step inapplicable;
//   beta_j = ||w|| ; v_{j+1} = w / beta_j.
// Kernels per step: the product, k_local_dot (alpha, ||H v_j||), k_mdot with
// the three-term step folded into its staging, k_update, the gated second
// k_mdot/k_update pair (an early return when the DGKS test passed) and
// k_scale.  Each reduction is finished by the last block of its own launch.
// Every decision (second pass, breakdown) is a device flag, so a whole cycle
// is enqueued without host round trips and replayed as a CUDA graph.
// After m steps the m x m projected matrix is diagonalised on the host, the
// residual of Ritz pair i is |beta_{m-1} y_{m-1,i}|, and the cycle restarts
// from the k lowest Ritz vectors plus v_m (Wu & Simon's thick restart).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "ed_lanczos.h"

namespace edgb {

namespace {

constexpr int kThreads = 256;
constexpr double kDgksEta = 0.7071067811865476;

int sm_count()
{
    int dev = 0, s = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s;
}

// Block-wide sum of kThreads doubles held one per thread; result in thread 0.
__device__ __forceinline__ double block_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = lane < (kThreads / 32) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 4; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

// Row range of block b when n rows are cut into nb contiguous chunks.
__device__ __forceinline__ void chunk(int64_t n, int nb, int b, int64_t& r0, int64_t& r1)
{
    r0 = n * (int64_t)b / nb;
    r1 = n * (int64_t)(b + 1) / nb;
}

// Completion of a reduction launch without a second kernel: every block calls
// this after writing its partials; it returns true in exactly one block, the
// last one to arrive, which then sees every block's partials.  That block
// resets the counter for the next launch.  Nothing waits, so no block can
// stall on another.
__device__ __forceinline__ bool last_block(unsigned int* counter)
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

// Sum of nb partials in a fixed order (thread-strided, then block_sum), so
// the result does not depend on which block finished last; in thread 0.
__device__ __forceinline__ double sum_parts(const double* p, int nb, double* red)
{
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) s += __ldcg(p + i);
    return block_sum(s, red);
}

// part[0*nb+b] = sum x.y, part[1*nb+b] = sum y.y over block b's rows.
__global__ void __launch_bounds__(kThreads) k_dot2(const double* __restrict__ x, const double* __restrict__ y,
                                                   int64_t n, double* __restrict__ part)
{
    __shared__ double red[kThreads / 32];
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    double a = 0.0, b = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
        const double yr = y[r];
        a = fma(x[r], yr, a);
        b = fma(yr, yr, b);
    }
    a = block_sum(a, red);
    b = block_sum(b, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
}

// Local step scalars of step j (w = H v_j): alpha = v_j.w goes to column j's
// diagonal, beta_{j-1} to row j-1 of column j, and ||H v_j||^2 to *hvnorm2,
// all written by the last block from the per-block partials.
__global__ void __launch_bounds__(kThreads) k_local_dot(const double* __restrict__ vj, const double* __restrict__ w,
                                                        int64_t n, double* __restrict__ part,
                                                        unsigned int* __restrict__ counter, double* __restrict__ coefcol,
                                                        int j, const double* __restrict__ beta_prev,
                                                        double* __restrict__ hvnorm2, const int* __restrict__ stop)
{
    if (*stop) return;
    __shared__ double red[kThreads / 32];
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    double a = 0.0, b = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
        const double wr = w[r];
        a = fma(vj[r], wr, a);
        b = fma(wr, wr, b);
    }
    a = block_sum(a, red);
    b = block_sum(b, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
    if (!last_block(counter)) return;
    a = sum_parts(part, gridDim.x, red);
    b = sum_parts(part + gridDim.x, gridDim.x, red);
    if (threadIdx.x == 0) {
        coefcol[j] = a;
        coefcol[j - 1] = *beta_prev;
        *hvnorm2 = b;
    }
}

// Multi-dot against the Krylov basis, R rows per block (R doubles of dynamic
// shared memory hold the block's slice of w): part[i*nb + b] = V[:,i].w for
// i < J and part[J*nb + b] = w.w.  With local != 0 the three-term step
// w -= alpha v_{J-1} + beta v_{J-2} is applied to the slice while it is staged
// and written back, so the pass sees the locally orthogonalised w.  Warps take
// the columns in turn, each streaming its column slice coalesced with four
// independent FMA chains.  The last block sums the partials column by column:
// c[i] for i < J (also added to coefcol[i] when coefcol is given) and
// *before = w.w.  Runs when run is null or *run != 0, and stop is clear.
__global__ void __launch_bounds__(kThreads) k_mdot(const double* __restrict__ V, int64_t n, int R, int J,
                                                   double* __restrict__ w, int local, const double* __restrict__ alpha,
                                                   const double* __restrict__ beta_prev, double* __restrict__ part,
                                                   unsigned int* __restrict__ counter, double* __restrict__ c,
                                                   double* __restrict__ coefcol, double* __restrict__ before,
                                                   const int* __restrict__ run, const int* __restrict__ stop)
{
    if ((run && !*run) || (stop && *stop)) return;
    extern __shared__ double sw[];
    const int64_t r0 = (int64_t)blockIdx.x * R;
    const int len = (int)min((int64_t)R, n - r0);
    if (local) {
        const double a = *alpha, b = *beta_prev;
        const double* vj = V + (int64_t)(J - 1) * n + r0;
        const double* vjm1 = V + (int64_t)(J - 2) * n + r0;
        for (int i = threadIdx.x; i < len; i += kThreads) {
            const double x = fma(-b, vjm1[i], fma(-a, vj[i], w[r0 + i]));
            w[r0 + i] = x;
            sw[i] = x;
        }
    } else {
        for (int i = threadIdx.x; i < len; i += kThreads) sw[i] = w[r0 + i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nb = gridDim.x;
    for (int i = warp; i <= J; i += kThreads / 32) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int r = lane;
        if (i < J) {
            const double* col = V + (int64_t)i * n + r0;
            // 16 independent loads per lane in flight, four FMA chains
            for (; r + 480 < len; r += 512) {
                double x[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) x[u] = col[r + 32 * u];
#pragma unroll
                for (int u = 0; u < 16; u += 4) {
                    a0 = fma(x[u], sw[r + 32 * u], a0);
                    a1 = fma(x[u + 1], sw[r + 32 * (u + 1)], a1);
                    a2 = fma(x[u + 2], sw[r + 32 * (u + 2)], a2);
                    a3 = fma(x[u + 3], sw[r + 32 * (u + 3)], a3);
                }
            }
            for (; r < len; r += 32) a0 = fma(col[r], sw[r], a0);
        } else {
            for (; r < len; r += 32) a0 = fma(sw[r], sw[r], a0);
        }
        double s = (a0 + a1) + (a2 + a3);
#pragma unroll
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) part[(int64_t)i * nb + blockIdx.x] = s;
    }
    if (!last_block(counter)) return;
    for (int i = warp; i <= J; i += kThreads / 32) {
        double s = 0.0;
        for (int b = lane; b < nb; b += 32) s += __ldcg(part + (int64_t)i * nb + b);
#pragma unroll
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            if (i < J) {
                c[i] = s;
                if (coefcol) coefcol[i] += s;
            } else {
                *before = s;
            }
        }
    }
}

// w -= V[:,0..J) c and a per-block partial of ||w||^2.  The last block then
// finishes the pass:
//   mode 1 (first pass): *need2 = force2 or ||w||^2 < eta^2 *before (the
//          DGKS test); without a second pass also beta and the breakdown test;
//   mode 2 (second pass): beta and the breakdown test;
//   mode 0: nothing (the counter is not touched).
// beta = ||w||; breakdown (stop = j + 1) when beta <= 1e-12 sqrt(*ref2), the
// new direction having vanished relative to ||H v_j||.
__global__ void __launch_bounds__(kThreads) k_update(const double* __restrict__ V, int64_t n, int J,
                                                     const double* __restrict__ c, double* __restrict__ w,
                                                     double* __restrict__ npart, unsigned int* __restrict__ counter,
                                                     int mode, int force2, const double* __restrict__ before,
                                                     int* __restrict__ need2, double* __restrict__ beta,
                                                     const double* __restrict__ ref2, int j,
                                                     const int* __restrict__ run, int* __restrict__ stop)
{
    if ((run && !*run) || (stop && *stop)) return;
    extern __shared__ double sc[];
    __shared__ double red[kThreads / 32];
    for (int i = threadIdx.x; i < J; i += kThreads) sc[i] = -c[i];
    __syncthreads();
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    double nn = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
        // eight column loads in flight, two FMA chains (even / odd columns)
        double acc = w[r], acc2 = 0.0;
        int i = 0;
        for (; i + 8 <= J; i += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = V[(int64_t)(i + u) * n + r];
#pragma unroll
            for (int u = 0; u < 8; u += 2) {
                acc = fma(sc[i + u], v[u], acc);
                acc2 = fma(sc[i + u + 1], v[u + 1], acc2);
            }
        }
        for (; i < J; ++i) acc = fma(sc[i], V[(int64_t)i * n + r], acc);
        acc += acc2;
        w[r] = acc;
        nn = fma(acc, acc, nn);
    }
    nn = block_sum(nn, red);
    if (threadIdx.x == 0) npart[blockIdx.x] = nn;
    if (mode == 0 || !last_block(counter)) return;
    const double s = sum_parts(npart, gridDim.x, red);
    if (threadIdx.x == 0) {
        bool finish = true;
        if (mode == 1) {
            const int again = (force2 || s < kDgksEta * kDgksEta * (*before)) ? 1 : 0;
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

__global__ void __launch_bounds__(kThreads) k_scale(double* __restrict__ w, int64_t n,
                                                    const double* __restrict__ beta, const int* __restrict__ stop)
{
    if (stop && *stop) return;
    const double inv = 1.0 / *beta;
    for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kThreads)
        w[r] *= inv;
}

// Seeded uniform(-1,1) vector (splitmix64 of seed and index).
__global__ void k_random(double* __restrict__ v, int64_t n, uint64_t seed)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(r + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v[r] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    }
}

// res[i] = || y_i - lambda_i x_i ||^2 partials -> host sums
__global__ void __launch_bounds__(kThreads) k_resid_part(const double* __restrict__ y, const double* __restrict__ x,
                                                         double lambda, int64_t n, double* __restrict__ part)
{
    __shared__ double red[kThreads / 32];
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    double s = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
        const double d = fma(-lambda, x[r], y[r]);
        s = fma(d, d, s);
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Deflated operator, part 1: c_i = shift * X_i . x for the nlock locked
// columns; per-block partials, summed in block order by the last block.
__global__ void __launch_bounds__(kThreads) k_lock_dots(const double* __restrict__ X, int nlock,
                                                        const double* __restrict__ x, int64_t n, double shift,
                                                        double* __restrict__ part, unsigned int* __restrict__ counter)
{
    __shared__ double red[kThreads / 32];
    int64_t r0, r1;
    chunk(n, gridDim.x, blockIdx.x, r0, r1);
    for (int i = 0; i < nlock; ++i) {
        const double* xi = X + (int64_t)i * n;
        double s = 0.0;
        for (int64_t r = r0 + threadIdx.x; r < r1; r += kThreads) s = fma(xi[r], x[r], s);
        s = block_sum(s, red);
        if (threadIdx.x == 0) part[(int64_t)i * gridDim.x + blockIdx.x] = s;
        __syncthreads();
    }
    if (!last_block(counter)) return;
    double* coef = part + (int64_t)nlock * gridDim.x;
    for (int i = 0; i < nlock; ++i) {
        const double s = sum_parts(part + (int64_t)i * gridDim.x, gridDim.x, red);
        if (threadIdx.x == 0) coef[i] = shift * s;
        __syncthreads();
    }
}

// Deflated operator, part 2: y += sum_i c_i X_i.
__global__ void __launch_bounds__(kThreads) k_lock_axpy(double* __restrict__ y, const double* __restrict__ X,
                                                        int nlock, const double* __restrict__ coef, int64_t n)
{
    for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kThreads) {
        double acc = y[r];
        for (int i = 0; i < nlock; ++i) acc = fma(coef[i], X[(int64_t)i * n + r], acc);
        y[r] = acc;
    }
}

__global__ void __launch_bounds__(kThreads) k_mul(double* __restrict__ v, int64_t n, double s)
{
    for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kThreads)
        v[r] *= s;
}

}  // namespace

// -------------------------------------------------------------- operator

namespace {
bool op_on_host(const ed_op& op)
{
    return op.kind == ed_op::HOST || (op.kind == ed_op::DEFLATED && op.inner && op.inner->kind == ed_op::HOST);
}
}  // namespace

// Work a product does once per operator (the stored CRS's sliced-ELL copy),
// done before a solver captures its cycles.
void op_prepare(const ed_op& op, cudaStream_t st)
{
    if (op.kind == ed_op::CRS) spmv_prepare(*op.crs, st);
    else if (op.kind == ed_op::DEFLATED && op.inner) op_prepare(*op.inner, st);
}

// Throws when one of the operator's products ran out of a bounded wait.
void op_check(const ed_op& op, cudaStream_t st)
{
    if (op.kind == ed_op::CRS) spmv_check(*op.crs, st);
    else if (op.kind == ed_op::DEFLATED && op.inner) op_check(*op.inner, st);
}

void op_apply(const ed_op& op, const double* x, double* y, cudaStream_t st)
{
    switch (op.kind) {
    case ed_op::CRS:
        spmv(*op.crs, x, y, st);
        break;
    case ed_op::MATFREE:
        hv_matfree(*op.basis, *op.terms, op.diag.p, x, y, st);
        break;
    case ed_op::HOST: {
        std::vector<double>& hx = const_cast<std::vector<double>&>(op.hx);
        std::vector<double>& hy = const_cast<std::vector<double>&>(op.hy);
        ED_CUDA(cudaMemcpyAsync(hx.data(), x, (size_t)op.n * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        op.fn(hx.data(), hy.data(), op.user);
        ED_CUDA(cudaMemcpyAsync(y, hy.data(), (size_t)op.n * 8, cudaMemcpyHostToDevice, st));
        break;
    }
    case ed_op::DEFLATED: {
        op_apply(*op.inner, x, y, st);
        double* part = const_cast<double*>(op.lock_part.p);
        k_lock_dots<<<op.lock_blocks, kThreads, 0, st>>>(op.lock, op.nlock, x, op.n, op.shift, part,
                                                         const_cast<unsigned int*>(op.lock_counter.p));
        ::edgb::count_launch();
        k_lock_axpy<<<op.lock_blocks, kThreads, 0, st>>>(y, op.lock, op.nlock,
                                                         part + (int64_t)op.nlock * op.lock_blocks, op.n);
        ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        break;
    }
    }
}

// --------------------------------------------------------------- solver

namespace {

struct Work {
    int64_t n = 0;
    int m = 0;
    int nb = 0;                      // blocks of the row-chunked reductions
    int R = 0;                       // rows per multi-dot block
    int nbm = 0;                     // blocks of the multi-dot
    DevBuf<double> V, V2;            // n x (m+1), column-major
    DevBuf<double> part;             // (m+2) * max(nb, nbm)
    DevBuf<double> npart;            // nb
    DevBuf<double> coef;             // (m+1) x (m+1); column j holds step j's projections
    DevBuf<double> beta;             // m+2
    DevBuf<double> c;                // m+2
    DevBuf<double> junk;             // m+2, coefficient sink for host-side orthonormalisation
    DevBuf<double> scal;             // [0] ||w||^2 before pass 1, [1] ||H v_j||^2, [2] before pass 2
    DevBuf<int> flags;               // [0] second pass wanted, [1] breakdown step + 1
    DevBuf<unsigned int> counters;   // last-block counters: [0] local dot, [1] multi-dot, [2] update
    DevBuf<double> Y;                // m x m Ritz coefficients
    RotateScratch rot;               // restart rotation scratch

    void mdot(const double* Vb, int J, double* x, int local, const double* alpha, const double* beta_prev,
              double* coefcol, double* before, const int* run, const int* stop, cudaStream_t st)
    {
        k_mdot<<<nbm, kThreads, (size_t)R * 8, st>>>(Vb, n, R, J, x, local, alpha, beta_prev, part.p,
                                                      counters.p + 1, c.p, coefcol, before, run, stop);
        ::edgb::count_launch();
    }
    void update(const double* Vb, int J, double* x, int mode, int force2, const double* before, int* need2,
                double* b, const double* ref2, int j, const int* run, int* stop, cudaStream_t st)
    {
        k_update<<<nb, kThreads, (size_t)J * 8, st>>>(Vb, n, J, c.p, x, npart.p, counters.p + 2, mode, force2,
                                                       before, need2, b, ref2, j, run, stop);
        ::edgb::count_launch();
    }
};

double host_sum_parts(const double* dev, int count, cudaStream_t st)
{
    std::vector<double> h(count);
    ED_CUDA(cudaMemcpyAsync(h.data(), dev, (size_t)count * 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (int i = 0; i < count; ++i) s += h[i];
    return s;
}

// Orthogonalise column `col` of V against columns [0, col) twice, then
// normalise it.  Returns the norm before normalisation.
double orthonormalise_column(Work& w, double* Vbase, int col, cudaStream_t st)
{
    double* x = Vbase + (int64_t)col * w.n;
    if (col > 0) {
        for (int pass = 0; pass < 2; ++pass) {
            w.mdot(Vbase, col, x, 0, nullptr, nullptr, w.junk.p, w.scal.p + 3, nullptr, nullptr, st);
            w.update(Vbase, col, x, 0, 0, nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr, st);
            ED_CUDA(cudaGetLastError());
        }
    }
    k_dot2<<<w.nb, kThreads, 0, st>>>(x, x, w.n, w.part.p); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    const double nrm = std::sqrt(host_sum_parts(w.part.p, w.nb, st));
    ED_REQUIRE(nrm > 0.0 && std::isfinite(nrm), ED_ERR_ARG, "start vector is zero or not finite");
    ED_CUDA(cudaMemcpyAsync(w.beta.p + w.m + 1, &nrm, 8, cudaMemcpyHostToDevice, st));
    k_scale<<<w.nb, kThreads, 0, st>>>(x, w.n, w.beta.p + w.m + 1, nullptr); ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaStreamSynchronize(st));
    return nrm;
}

void dense_solve(const ed_op& op, int nev, double* evals_host, double* evecs_dev, ed_solve_info* info,
                 cudaStream_t st)
{
    const int64_t n = op.n;
    DevBuf<double> X((size_t)n * n), HX((size_t)n * n);
    std::vector<double> id((size_t)n * n, 0.0);
    for (int64_t i = 0; i < n; ++i) id[(size_t)i * n + i] = 1.0;
    ED_CUDA(cudaMemcpyAsync(X.p, id.data(), id.size() * 8, cudaMemcpyHostToDevice, st));
    for (int64_t i = 0; i < n; ++i) op_apply(op, X.p + i * n, HX.p + i * n, st);
    std::vector<double> hx((size_t)n * n);
    ED_CUDA(cudaMemcpyAsync(hx.data(), HX.p, hx.size() * 8, cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    // column i of HX is H e_i; symmetrise against round-off
    std::vector<double> A((size_t)n * n);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < n; ++j) A[(size_t)i * n + j] = 0.5 * (hx[(size_t)j * n + i] + hx[(size_t)i * n + j]);
    std::vector<double> ev, vec;
    sym_eigen((int)n, A, ev, vec);
    for (int i = 0; i < nev; ++i) evals_host[i] = ev[i];
    if (evecs_dev)
        ED_CUDA(cudaMemcpyAsync(evecs_dev, vec.data(), (size_t)n * nev * 8, cudaMemcpyHostToDevice, st));
    ED_CUDA(cudaStreamSynchronize(st));
    if (info) {
        info->converged = nev;
        info->matvecs = n;
        info->max_residual = 0.0;
    }
}

}  // namespace

void residual_norms(const ed_op& op, const double* x, const double* lambda, int k, double* res, cudaStream_t st)
{
    const int64_t n = op.n;
    DevBuf<double> y(n);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count() * 2, n / 2048));
    DevBuf<double> part(nb);
    for (int i = 0; i < k; ++i) {
        op_apply(op, x + (int64_t)i * n, y.p, st);
        k_resid_part<<<nb, kThreads, 0, st>>>(y.p, x + (int64_t)i * n, lambda[i], n, part.p); ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        std::vector<double> h(nb);
        ED_CUDA(cudaMemcpyAsync(h.data(), part.p, (size_t)nb * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        double s = 0.0;
        for (double v : h) s += v;
        res[i] = std::sqrt(s);
    }
}

namespace {
void lanczos_once(const ed_op& op, const ed_lanczos_params& p, const double* v0_dev, double* evals_host,
                  double* evecs_dev, ed_solve_info* info, cudaStream_t caller_stream)
{
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t n = op.n;
    const int nev = p.nev;
    ED_REQUIRE(n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
    ED_REQUIRE(nev >= 1 && nev <= n, ED_ERR_ARG, "need 1 <= nev <= n");
    const double tol = p.tol > 0 ? p.tol : 1e-10;
    const int max_restarts = p.max_restarts > 0 ? p.max_restarts : 2000;
    ed_solve_info inf;
    std::memset(&inf, 0, sizeof(inf));
    SolveStream ss(caller_stream);
    cudaStream_t st = ss.s;
    const int nsm = sm_count();
    op_prepare(op, st);

    if (v0_dev) {
        // a start vector must be finite and nonzero on every path
        const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(nsm * 2, n / 2048));
        DevBuf<double> part(2 * (size_t)nb);
        k_dot2<<<nb, kThreads, 0, st>>>(v0_dev, v0_dev, n, part.p); ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        std::vector<double> h(2 * (size_t)nb);
        ED_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        double nn = 0.0;
        for (int i = 0; i < nb; ++i) nn += h[i];
        ED_REQUIRE(nn > 0.0 && std::isfinite(nn), ED_ERR_ARG, "start vector is zero or not finite");
    }
    // The reference switches to dense LAPACK below dimension 60
    // (pseudopotential_model_base.hpp:244-251); so do we.
    if (n < 60 || n <= (int64_t)nev + 2) {
        dense_solve(op, nev, evals_host, evecs_dev, &inf, st);
        inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (info) *info = inf;
        return;
    }
    int64_t m64 = p.ncv > 0 ? p.ncv : std::min<int64_t>(n, 2 * (int64_t)nev + 21);
    m64 = std::max<int64_t>(m64, nev + 2);
    m64 = std::min<int64_t>(m64, n - 1);
    m64 = std::min<int64_t>(m64, 1000);
    const int m = (int)m64;
    ED_REQUIRE(m > nev, ED_ERR_ARG, "Krylov subspace must exceed nev");

    Work w;
    w.n = n;
    w.m = m;
    w.nb = (int)std::max<int64_t>(1, std::min<int64_t>(nsm * 4, n / 1024));
    // multi-dot slices: three blocks per SM, a whole wave (a cap of 4096 rows
    // gave 335 blocks at the headline size, 2 or 3 per SM, and a Lanczos phase
    // 2 % longer; 2 or 4 blocks per SM measured 0.3 / 0.6 % longer than 3),
    // at least 512 and at most 12288 rows (a multiple of 128)
    {
        int64_t nbt = (int64_t)nsm * 3, R = 0;
        for (;;) {
            R = std::max<int64_t>(512, ((n + nbt - 1) / nbt + 127) / 128 * 128);
            if (R <= 12288) break;
            nbt += nsm;
        }
        w.R = (int)R;
        w.nbm = (int)((n + R - 1) / R);
        if ((size_t)R * 8 > 48 * 1024)
            ED_CUDA(cudaFuncSetAttribute(k_mdot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(R * 8)));
    }
    w.V.alloc((size_t)n * (m + 1));
    w.V2.alloc((size_t)n * (m + 1));
    w.part.alloc((size_t)(m + 2) * std::max(w.nb, w.nbm));
    w.npart.alloc(w.nb);
    w.coef.alloc((size_t)(m + 1) * (m + 1));
    w.beta.alloc(m + 2);
    w.c.alloc(m + 2);
    w.junk.alloc(m + 2);
    w.scal.alloc(4);
    w.flags.alloc(2);
    w.counters.alloc(4);
    w.Y.alloc((size_t)m * m);
    ED_CUDA(cudaMemsetAsync(w.beta.p, 0, (m + 2) * 8, st));
    ED_CUDA(cudaMemsetAsync(w.junk.p, 0, (m + 2) * 8, st));
    ED_CUDA(cudaMemsetAsync(w.counters.p, 0, 4 * sizeof(unsigned int), st));

    if (v0_dev) ED_CUDA(cudaMemcpyAsync(w.V.p, v0_dev, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    else {
        k_random<<<nsm * 4, kThreads, 0, st>>>(w.V.p, n, p.seed); ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
    }
    orthonormalise_column(w, w.V.p, 0, st);

    std::vector<cudaEvent_t> ev(2 * (m + 1), nullptr);
    for (auto& e : ev) ED_CUDA(cudaEventCreate(&e));
    struct EvGuard {
        std::vector<cudaEvent_t>& v;
        ~EvGuard() { for (auto e : v) if (e) cudaEventDestroy(e); }
    } evguard{ev};

    // One restart cycle, steps k..m-1, all on the device: breakdown and the
    // second Gram-Schmidt pass are flags that later kernels read, so the host
    // enqueues a whole cycle without waiting, and (for device operators)
    // replays it as one CUDA graph.
    int* need2 = w.flags.p;
    int* stop = w.flags.p + 1;
    auto enqueue_cycle = [&](int k, bool capturing) {
        ED_CUDA(cudaMemsetAsync(w.flags.p, 0, 2 * sizeof(int), st));
        ED_CUDA(cudaMemsetAsync(w.coef.p + (size_t)k * (m + 1), 0, (size_t)(m - k) * (m + 1) * 8, st));
        for (int j = k; j < m; ++j) {
            double* vj = w.V.p + (int64_t)j * n;
            double* wv = w.V.p + (int64_t)(j + 1) * n;
            double* coefcol = w.coef.p + (size_t)j * (m + 1);
            const bool first = (j == k);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j], st));
            op_apply(op, vj, wv, st);
            if (capturing) ED_CUDA(cudaEventRecordWithFlags(ev[2 * j + 1], st, cudaEventRecordExternal));
            else ED_CUDA(cudaEventRecord(ev[2 * j + 1], st));
            if (!first) {
                k_local_dot<<<w.nb, kThreads, 0, st>>>(vj, wv, n, w.part.p, w.counters.p, coefcol, j,
                                                       w.beta.p + (j - 1), w.scal.p + 1, stop); ::edgb::count_launch();
            }
            const int J = j + 1;
            // pass 1 (with the three-term step on non-first steps), then the
            // DGKS-gated pass 2; breakdown is judged against ||H v_j||
            w.mdot(w.V.p, J, wv, first ? 0 : 1, coefcol + j, w.beta.p + (j - 1), coefcol, w.scal.p, nullptr, stop, st);
            w.update(w.V.p, J, wv, 1, first ? 1 : 0, w.scal.p, need2, w.beta.p + j,
                     first ? w.scal.p : w.scal.p + 1, j, nullptr, stop, st);
            w.mdot(w.V.p, J, wv, 0, nullptr, nullptr, coefcol, w.scal.p + 2, need2, stop, st);
            w.update(w.V.p, J, wv, 2, 0, nullptr, nullptr, w.beta.p + j, first ? w.scal.p : w.scal.p + 1, j, need2,
                     stop, st);
            k_scale<<<w.nb, kThreads, 0, st>>>(wv, n, w.beta.p + j, stop); ::edgb::count_launch();
            ED_CUDA(cudaGetLastError());
        }
    };
    const bool graphs = !op_on_host(op);
    CycleGraphs cache;
    auto run_cycle = [&](int k) {
        if (!graphs) {
            enqueue_cycle(k, false);
            return;
        }
        CycleGraphs::Entry* g = cache.find(k, w.V.p);
        if (!g) {
            const uint64_t c0 = launch_count();
            ED_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            try {
                enqueue_cycle(k, true);
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
            cache.e.push_back({k, w.V.p, exec, kernels});
            g = &cache.e.back();
        }
        ED_CUDA(cudaGraphLaunch(g->exec, st));
        count_launches(g->kernels);
    };

    std::vector<double> T((size_t)m * m, 0.0), coef_h((size_t)(m + 1) * (m + 1)), beta_h(m + 1);
    std::vector<double> theta, Y, prev_theta;
    int k = 0, m_eff = m;
    double beta_last = 0.0;
    bool converged = false;
    double spmv_ms = 0.0;
    for (;;) {
        run_cycle(k);
        inf.matvecs += m - k;
        int hstop = 0;
        ED_CUDA(cudaMemcpyAsync(&hstop, stop, sizeof(int), cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(coef_h.data(), w.coef.p, coef_h.size() * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaMemcpyAsync(beta_h.data(), w.beta.p, (size_t)(m + 1) * 8, cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        for (int j = k; j < m; ++j) {
            float ms = 0.f;
            ED_CUDA(cudaEventElapsedTime(&ms, ev[2 * j], ev[2 * j + 1]));
            spmv_ms += ms;
        }
        m_eff = hstop ? hstop : m;
        if (hstop) ++inf.breakdowns;
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
        beta_last = hstop ? 0.0 : beta_h[m - 1];
        int nconv = 0;
        double maxres = 0.0;
        const int want = std::min(nev, m_eff);
        for (int i = 0; i < want; ++i) {
            const double r = std::fabs(beta_last * Y[(size_t)(m_eff - 1) + (size_t)m_eff * i]);
            maxres = std::max(maxres, r);
            if (r <= tol) ++nconv;
        }
        inf.converged = nconv;
        inf.max_residual = maxres;
        // After a breakdown the Ritz pairs are exact but a fresh direction may
        // still uncover more copies of a degenerate eigenvalue: accept only
        // once a cycle leaves the nev lowest values unchanged, or when the
        // whole space has been spanned.
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
        // thick restart from the kk lowest Ritz vectors: the nev wanted ones
        // plus a quarter of the rest.  Measured on GB300 against Wu & Simon's
        // half: about the same number of products (nev 10, m 41: 337-348 vs
        // 339) with 11 instead of 18 restarts, and each restart's rotation
        // and the Gram-Schmidt passes shrink with kk (0.44-0.45 s vs 0.46 s);
        // below about nev + 4 convergence degrades sharply.
        int kk = std::min(m - 2, nev + std::max(1, (m - nev) / 4));
        kk = std::max(kk, std::min(nev, m - 1));
        if (hstop) kk = std::min(kk, m_eff);
        rotate_basis(w.V.p, n, m_eff, Y.data(), m_eff, kk, w.V2.p, w.rot, 0, st);
        if (!hstop) {
            ED_CUDA(cudaMemcpyAsync(w.V2.p + (int64_t)kk * n, w.V.p + (int64_t)m * n, (size_t)n * 8,
                                    cudaMemcpyDeviceToDevice, st));
        } else {
            k_random<<<sm_count() * 4, kThreads, 0, st>>>(w.V2.p + (int64_t)kk * n, n,
                                                         p.seed + 0x51ED2701ull * (uint64_t)inf.restarts); ::edgb::count_launch();
            ED_CUDA(cudaGetLastError());
            orthonormalise_column(w, w.V2.p, kk, st);
        }
        std::swap(w.V, w.V2);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < kk; ++i) {
            T[(size_t)i * m + i] = theta[i];
            if (!hstop) {
                const double s = beta_last * Y[(size_t)(m_eff - 1) + (size_t)m_eff * i];
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
    for (int i = 0; i < nev; ++i) evals_host[i] = i < nfound ? theta[i] : std::nan("");
    DevBuf<double> xtmp;
    double* X = evecs_dev;
    if (!X && p.verify) {
        xtmp.alloc((size_t)n * nev);
        X = xtmp.p;
    }
    if (X) {
        if (nfound < nev) ED_CUDA(cudaMemsetAsync(X, 0, (size_t)n * nev * 8, st));
        rotate_basis(w.V.p, n, m_eff, Y.data(), m_eff, nfound, X, w.rot, 0, st);
    }
    if (p.verify && X && nfound == nev) {
        std::vector<double> res(nev);
        residual_norms(op, X, evals_host, nev, res.data(), st);
        inf.matvecs += nev;
        inf.max_residual = *std::max_element(res.begin(), res.end());
        int nc = 0;
        for (double r : res) nc += (r <= tol) ? 1 : 0;
        inf.converged = nc;
    }
    ED_CUDA(cudaStreamSynchronize(st));
    op_check(op, st);
    inf.spmv_seconds = spmv_ms * 1e-3;
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = inf;
    ED_REQUIRE(converged, ED_ERR_NOCONV, "Lanczos did not converge within the restart cap");
}

// ------------------------------------------------------------ two-level start

// Keep the entries of the block 2 M0 in {0, 1} (M0 = the lowest level's Lz,
// from its norb0 high bits: orbital i has 2 m = 2 i - (norb0 - 1)) and zero
// the rest; *kept counts the block.  No term mixes the levels, so H keeps M0:
// a Krylov space started inside the block stays there.
__global__ void __launch_bounds__(kThreads) k_keep_m0_block(const uint64_t* __restrict__ words, int64_t n, int K0,
                                                            int K1, double* __restrict__ v,
                                                            unsigned long long* __restrict__ kept)
{
    unsigned long long c = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int two_m0 = 0;
        for (uint64_t f = words[r] >> K1; f; f &= f - 1) two_m0 += 2 * (__ffsll((long long)f) - 1) - (K0 - 1);
        if (two_m0 == 0 || two_m0 == 1) ++c;
        else v[r] = 0.0;
    }
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(kept, c);
}

// ------------------------------------------------------------ diagonal matrices

// A stored matrix with no off-diagonal element above the reference's
// 1e-14 (HamiltonianBase::MatrixDiagonalCheck, hamiltonian_base.hpp:378-449)
// has its spectrum on the diagonal.  Values are double or complex (double2).
__device__ __forceinline__ double dmod(double v) { return fabs(v); }
__device__ __forceinline__ double dmod(double2 v) { return hypot(v.x, v.y); }
__device__ __forceinline__ double dreal(double v) { return v; }
__device__ __forceinline__ double dreal(double2 v) { return v.x; }

template <class T>
__global__ void __launch_bounds__(kThreads) k_crs_offdiag(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col, const T* __restrict__ val,
                                                          int64_t n, int* __restrict__ flag)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (col[k] != r && dmod(val[k]) > kSparseZeroTol) {
                atomicOr(flag, 1);
                break;
            }
    }
}

// d[r] = the real part of the stored diagonal of row r (0 when none)
template <class T>
__global__ void __launch_bounds__(kThreads) k_crs_diag(const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ col, const T* __restrict__ val,
                                                       int64_t n, double* __restrict__ d)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (col[k] == r) s += dreal(val[k]);
        d[r] = s;
    }
}

__device__ __forceinline__ bool pair_less(double av, int64_t ai, double bv, int64_t bi)
{
    return av < bv || (av == bv && ai < bi);
}

// Selection step t: the smallest (d[j], j) above (selv[t-1], seli[t-1]) in the
// lexicographic order (values, then index), so that t = 0..nev-1 give the nev
// smallest entries in ascending order, each copy of a repeated value at its
// own index.  Block partials, finished by the last block.
__global__ void __launch_bounds__(kThreads) k_select_next(const double* __restrict__ d, int64_t n, int t,
                                                          double* __restrict__ selv, int64_t* __restrict__ seli,
                                                          double* __restrict__ pv, int64_t* __restrict__ pi,
                                                          unsigned int* __restrict__ counter)
{
    __shared__ double sv[kThreads];
    __shared__ int64_t si[kThreads];
    const double lv = t > 0 ? selv[t - 1] : -INFINITY;
    const int64_t li = t > 0 ? seli[t - 1] : -1;
    double bv = INFINITY;
    int64_t bi = n;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double v = d[j];
        if (pair_less(lv, li, v, j) && pair_less(v, j, bv, bi)) {
            bv = v;
            bi = j;
        }
    }
    sv[threadIdx.x] = bv;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int o = kThreads / 2; o; o >>= 1) {
        if (threadIdx.x < o && pair_less(sv[threadIdx.x + o], si[threadIdx.x + o], sv[threadIdx.x], si[threadIdx.x])) {
            sv[threadIdx.x] = sv[threadIdx.x + o];
            si[threadIdx.x] = si[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pv[blockIdx.x] = sv[0];
        pi[blockIdx.x] = si[0];
    }
    if (!last_block(counter)) return;
    if (threadIdx.x == 0) {
        double v = INFINITY;
        int64_t i = n;
        for (unsigned b = 0; b < gridDim.x; ++b) {
            const double x = __ldcg(pv + b);
            const int64_t y = __ldcg(pi + b);
            if (pair_less(x, y, v, i)) {
                v = x;
                i = y;
            }
        }
        selv[t] = v;
        seli[t] = i;
    }
}

// column t of the eigenvectors = the unit vector at seli[t] (stride values
// per entry: 1 real, 2 complex)
__global__ void k_unit_columns(const int64_t* __restrict__ seli, int nev, int64_t n, int stride, double* __restrict__ X)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nev; t += gridDim.x * blockDim.x)
        X[((int64_t)t * n + seli[t]) * stride] = 1.0;
}

template <class T>
bool diagonal_spectrum_impl(const int64_t* rowptr, const int32_t* col, const T* val, int64_t n, int nev,
                            double* evals_host, double* evecs_dev, int stride, ed_solve_info* info, cudaStream_t st)
{
    const auto t0 = std::chrono::steady_clock::now();
    const int grid = sm_count() * 4;
    DevBuf<int> flag(1);
    ED_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
    k_crs_offdiag<T><<<grid, kThreads, 0, st>>>(rowptr, col, val, n, flag.p);
    ::edgb::count_launch();
    ED_CUDA(cudaGetLastError());
    int h = 0;
    ED_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ED_CUDA(cudaStreamSynchronize(st));
    if (h) return false;
    DevBuf<double> d(n), selv(nev), pv(grid);
    DevBuf<int64_t> seli(nev), pi(grid);
    DevBuf<unsigned int> counter(1);
    ED_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
    k_crs_diag<T><<<grid, kThreads, 0, st>>>(rowptr, col, val, n, d.p);
    ::edgb::count_launch();
    for (int t = 0; t < nev; ++t) {
        k_select_next<<<grid, kThreads, 0, st>>>(d.p, n, t, selv.p, seli.p, pv.p, pi.p, counter.p);
        ::edgb::count_launch();
    }
    ED_CUDA(cudaGetLastError());
    ED_CUDA(cudaMemcpyAsync(evals_host, selv.p, (size_t)nev * 8, cudaMemcpyDeviceToHost, st));
    if (evecs_dev) {
        ED_CUDA(cudaMemsetAsync(evecs_dev, 0, (size_t)n * nev * stride * 8, st));
        k_unit_columns<<<1, 256, 0, st>>>(seli.p, nev, n, stride, evecs_dev);
        ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
    }
    ED_CUDA(cudaStreamSynchronize(st));
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->converged = nev;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return true;
}

}  // namespace

bool diagonal_spectrum(const int64_t* rowptr, const int32_t* col, const double* val, int complex_values, int64_t n,
                       int nev, double* evals_host, double* evecs_dev, ed_solve_info* info, cudaStream_t st)
{
    if (complex_values)
        return diagonal_spectrum_impl(rowptr, col, reinterpret_cast<const double2*>(val), n, nev, evals_host,
                                      evecs_dev, 2, info, st);
    return diagonal_spectrum_impl(rowptr, col, val, n, nev, evals_host, evecs_dev, 1, info, st);
}

namespace {

void add_info(ed_solve_info& a, const ed_solve_info& b)
{
    a.restarts += b.restarts;
    a.matvecs += b.matvecs;
    a.spmv_seconds += b.spmv_seconds;
    a.breakdowns += b.breakdowns;
}
}  // namespace

// One Krylov sequence sees one vector of each eigenspace, so a degenerate
// eigenvalue comes out once (only rounding could add copies).  With
// p.degeneracy_passes > 0, each further pass solves for the nev lowest pairs
// of H + shift * X X^T, X the pairs found so far and shift above their spread:
// the found eigenvalues move up, the complement keeps its spectrum, and any
// value below the nev-th found (a further copy) is merged in.  The passes end
// when one adds nothing.
void lanczos_solve(const ed_op& op, const ed_lanczos_params& p, const double* v0_dev, double* evals_host,
                   double* evecs_dev, ed_solve_info* info, cudaStream_t caller_stream)
{
    const int64_t n = op.n;
    const int nev = p.nev;
    if (p.diagonal_check && op.kind == ed_op::CRS && n >= 1 && nev >= 1 && nev <= n) {
        SolveStream ss(caller_stream);
        const ed_crs& a = *op.crs;
        if (diagonal_spectrum(a.rowptr.p, a.col.p, a.val.p, 0, n, nev, evals_host, evecs_dev, info, ss.s)) return;
    }
    if (p.degeneracy_passes <= 0 || n < 60 || n <= (int64_t)nev + 2) {
        lanczos_once(op, p, v0_dev, evals_host, evecs_dev, info, caller_stream);
        return;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const double tol = p.tol > 0 ? p.tol : 1e-10;
    ed_lanczos_params q = p;
    q.verify = 0;
    q.degeneracy_passes = 0;
    DevBuf<double> X((size_t)n * nev), Y((size_t)n * nev), Xn((size_t)n * nev);
    std::vector<double> theta(nev), mu(nev);
    ed_solve_info total, part;
    std::memset(&total, 0, sizeof(total));
    std::memset(&part, 0, sizeof(part));
    lanczos_once(op, q, v0_dev, theta.data(), X.p, &part, caller_stream);
    add_info(total, part);
    SolveStream ss(caller_stream);
    cudaStream_t st = ss.s;
    ed_op D;
    D.kind = ed_op::DEFLATED;
    D.n = n;
    D.inner = &op;
    D.nlock = nev;
    D.lock_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count() * 2, n / 2048));
    D.lock_part.alloc((size_t)nev * (D.lock_blocks + 1));
    D.lock_counter.alloc(1);
    ED_CUDA(cudaMemsetAsync(D.lock_counter.p, 0, sizeof(unsigned int), st));
    for (int pass = 1; pass <= p.degeneracy_passes; ++pass) {
        D.lock = X.p;
        D.shift = (theta[nev - 1] - theta[0]) + std::max(1.0, std::fabs(theta[nev - 1]));
        ed_lanczos_params r = q;
        r.seed = p.seed + 0x2545F4914F6CDD1Dull * (uint64_t)pass;
        ED_CUDA(cudaStreamSynchronize(st));
        lanczos_once(D, r, nullptr, mu.data(), Y.p, &part, caller_stream);
        add_info(total, part);
        const double thr = theta[nev - 1] - tol * std::max(1.0, std::fabs(theta[nev - 1]));
        std::vector<std::pair<double, int>> all;
        for (int i = 0; i < nev; ++i) all.push_back({theta[i], i});
        int added = 0;
        for (int i = 0; i < nev; ++i)
            if (mu[i] < thr) {
                all.push_back({mu[i], nev + i});
                ++added;
            }
        if (!added) break;
        std::stable_sort(all.begin(), all.end(),
                         [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first; });
        for (int i = 0; i < nev; ++i) {
            const int src = all[i].second;
            const double* from = src < nev ? X.p + (int64_t)src * n : Y.p + (int64_t)(src - nev) * n;
            ED_CUDA(cudaMemcpyAsync(Xn.p + (int64_t)i * n, from, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
            theta[i] = all[i].first;
        }
        std::swap(X.p, Xn.p);
    }
    for (int i = 0; i < nev; ++i) evals_host[i] = theta[i];
    if (evecs_dev) ED_CUDA(cudaMemcpyAsync(evecs_dev, X.p, (size_t)n * nev * 8, cudaMemcpyDeviceToDevice, st));
    ED_CUDA(cudaStreamSynchronize(st));
    total.converged = nev;
    total.max_residual = part.max_residual;
    if (p.verify) {
        std::vector<double> res(nev);
        residual_norms(op, X.p, theta.data(), nev, res.data(), st);
        total.matvecs += nev;
        total.max_residual = *std::max_element(res.begin(), res.end());
        int nc = 0;
        for (double rr : res) nc += (rr <= tol) ? 1 : 0;
        total.converged = nc;
    }
    ED_CUDA(cudaStreamSynchronize(st));
    total.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = total;
}

// Two-level solve: one Krylov sequence, then the copies of each degenerate
// eigenvalue from the level-exchange ladder T = L0- L1+ and its adjoint,
// which commute with the Hamiltonian (the levels do not mix) and map a
// multiplet state |L0 m0>|L1 m1> to its neighbours in m0 at fixed total Lz.
// For the found vectors in ascending order, each chain T^k x (both
// directions) is orthogonalised against the vectors kept so far and kept when
// something of it is left, until nev vectors are kept; those are then checked
// by their true residuals (after a Rayleigh-Ritz step on their span if
// needed).  The chain divides by ||T x||, which magnifies the Ritz vectors'
// error components, so a failed check repeats the sequence two digits past
// the target from the found vectors; should that fail too (a degeneracy the
// ladder does not generate), the deflated passes take over.
// Rayleigh-Ritz rounds that refine the ladder's copies before a sequence is
// repeated (round 0 on the kept span, then widened by the residuals).
constexpr int kLadderRefineRounds = 5;

void lanczos_solve_two_level(const ed_basis& b, const ed_op& op, const ed_lanczos_params& p, const double* v0_dev,
                             double* evals_host, double* evecs_dev, ed_solve_info* info, cudaStream_t caller)
{
    ED_REQUIRE(b.levels == 2 && (int64_t)b.dim == op.n, ED_ERR_ARG, "the ladder solve takes the operator's two-level basis");
    const int64_t n = op.n;
    const int nev = p.nev;
    if (p.diagonal_check && op.kind == ed_op::CRS && n >= 1 && nev >= 1 && nev <= n) {
        SolveStream ds(caller);
        const ed_crs& a = *op.crs;
        if (diagonal_spectrum(a.rowptr.p, a.col.p, a.val.p, 0, n, nev, evals_host, evecs_dev, info, ds.s)) return;
    }
    if (n < 60 || n <= (int64_t)nev + 2) {   // the dense path sees every copy
        lanczos_once(op, p, v0_dev, evals_host, evecs_dev, info, caller);
        return;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const double tol = p.tol > 0 ? p.tol : 1e-10;
    ed_lanczos_params q = p;
    q.verify = 0;
    q.degeneracy_passes = 0;
    DevBuf<double> X((size_t)n * nev);
    std::vector<double> theta(nev);
    ed_solve_info total, part;
    std::memset(&total, 0, sizeof(total));
    std::memset(&part, 0, sizeof(part));
    SolveStream ss(caller);
    cudaStream_t st = ss.s;
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count() * 2, n / 2048));
    DevBuf<double> A((size_t)n * nev), cur(n), u(n), v0w(n), lpart((size_t)nev * (nb + 1)), dpart(2 * (size_t)nb);
    DevBuf<unsigned int> counter(1);
    ED_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
    std::vector<double> lam;
    int acc = 0;
    auto norm = [&](const double* v) {
        k_dot2<<<nb, kThreads, 0, st>>>(v, v, n, dpart.p);
        ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        return std::sqrt(host_sum_parts(dpart.p, nb, st));
    };
    auto mul = [&](double* v, double sc) {
        k_mul<<<sm_count() * 4, kThreads, 0, st>>>(v, n, sc);
        ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
    };
    auto orth = [&](double* v) {
        for (int pass = 0; pass < 2 && acc > 0; ++pass) {
            k_lock_dots<<<nb, kThreads, 0, st>>>(A.p, acc, v, n, -1.0, lpart.p, counter.p);
            ::edgb::count_launch();
            k_lock_axpy<<<nb, kThreads, 0, st>>>(v, A.p, acc, lpart.p + (int64_t)acc * nb, n);
            ::edgb::count_launch();
            ED_CUDA(cudaGetLastError());
        }
    };
    auto try_keep = [&](const double* v, double value) {
        ED_CUDA(cudaMemcpyAsync(u.p, v, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        const double n0 = norm(u.p);
        if (!(n0 > 0.0)) return;
        orth(u.p);
        const double n1 = norm(u.p);
        if (!(n1 > 1e-6 * n0)) return;
        mul(u.p, 1.0 / n1);
        ED_CUDA(cudaMemcpyAsync(A.p + (int64_t)acc * n, u.p, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
        lam.push_back(value);
        ++acc;
    };
    const double lscale = (double)b.norb0 * b.norb1;   // the ladder's norm is below K0*K1/4
    std::vector<double> res(nev, 0.0);
    // At Lz = 0 every multiplet (L0, L1) has exactly one member in the block
    // 2 M0 in {0, 1} (its members span M0 = -min(L0, L1) .. min(L0, L1)), so
    // a sequence started there meets each multiplet once, with no copy for
    // rounding to grow, and the ladder supplies the copies.  Elsewhere, or
    // with a caller's start, the start covers the whole sector.
    DevBuf<double> vblock;
    const double* v0_seq = v0_dev;
    if (!v0_dev && b.two_lz == 0) {
        vblock.alloc(n);
        DevBuf<unsigned long long> kept(1);
        ED_CUDA(cudaMemsetAsync(kept.p, 0, sizeof(unsigned long long), st));
        k_random<<<sm_count() * 4, kThreads, 0, st>>>(vblock.p, n, p.seed);
        ::edgb::count_launch();
        k_keep_m0_block<<<sm_count() * 4, kThreads, 0, st>>>(b.words.p, n, b.norb0, b.norb1, vblock.p, kept.p);
        ::edgb::count_launch();
        ED_CUDA(cudaGetLastError());
        unsigned long long hk = 0;
        ED_CUDA(cudaMemcpyAsync(&hk, kept.p, sizeof(hk), cudaMemcpyDeviceToHost, st));
        ED_CUDA(cudaStreamSynchronize(st));
        if (hk >= (unsigned long long)nev + 2) v0_seq = vblock.p;
    }
    bool ok = false;
    for (int attempt = 0; attempt < 2 && !ok; ++attempt) {
        const double* v0a = v0_seq;
        q.tol = attempt == 0 ? tol : tol * 1e-2;
        if (attempt == 1) {
            // start from the sum of the first attempt's vectors
            std::vector<double> ones(nev, 1.0);
            ED_CUDA(cudaMemsetAsync(v0w.p, 0, (size_t)n * 8, st));
            ED_CUDA(cudaMemcpyAsync(lpart.p, ones.data(), (size_t)nev * 8, cudaMemcpyHostToDevice, st));
            k_lock_axpy<<<nb, kThreads, 0, st>>>(v0w.p, X.p, nev, lpart.p, n);
            ::edgb::count_launch();
            ED_CUDA(cudaGetLastError());
            v0a = v0w.p;
        }
        ED_CUDA(cudaStreamSynchronize(st));
        lanczos_once(op, q, v0a, theta.data(), X.p, &part, caller);
        add_info(total, part);
        acc = 0;
        lam.clear();
        for (int k = 0; k < nev && acc < nev; ++k) {
            const double* xk = X.p + (int64_t)k * n;
            try_keep(xk, theta[k]);
            for (int dir = 1; dir >= -1 && acc < nev; dir -= 2) {
                ED_CUDA(cudaMemcpyAsync(cur.p, xk, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
                for (int step = 0; step < b.norb0 + b.norb1 && acc < nev; ++step) {
                    two_level_ladder(b, cur.p, u.p, dir, st);
                    const double nt = norm(u.p);
                    if (!(nt > 1e-8 * lscale)) break;               // the end of the multiplet
                    std::swap(cur.p, u.p);
                    mul(cur.p, 1.0 / nt);
                    try_keep(cur.p, theta[k]);
                }
            }
        }
        if (acc != nev) continue;
        residual_norms(op, A.p, lam.data(), nev, res.data(), st);
        total.matvecs += nev;
        ok = *std::max_element(res.begin(), res.end()) <= tol;
        if (ok) break;
        // The ladder multiplies a Ritz vector's error by up to its norm, so the
        // copies can miss the bar that the sequence met.  Refine them in
        // place: Rayleigh-Ritz on the kept span, then on the span widened by
        // the residuals R = H A - A diag(lam) (one step of a block Krylov
        // space), a few times, 2 nev products and a residual check a round.
        DevBuf<double> W((size_t)n * 2 * nev), HW((size_t)n * 2 * nev), Ar((size_t)n * nev);
        ED_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
        DevBuf<double> wpart((size_t)2 * nev * (nb + 1));
        RotateScratch rot;
        auto dots = [&](const double* B, int m, const double* v, double scale) {
            k_lock_dots<<<nb, kThreads, 0, st>>>(B, m, v, n, scale, wpart.p, counter.p);
            ::edgb::count_launch();
            ED_CUDA(cudaGetLastError());
        };
        for (int round = 0; round < kLadderRefineRounds && !ok; ++round) {
            // W = [A, Q], Q orthonormal residual directions (none in round 0)
            ED_CUDA(cudaMemcpyAsync(W.p, A.p, (size_t)n * nev * 8, cudaMemcpyDeviceToDevice, st));
            for (int i = 0; i < nev; ++i) op_apply(op, A.p + (int64_t)i * n, HW.p + (int64_t)i * n, st);
            total.matvecs += nev;
            int m = nev;
            if (round > 0) {
                for (int i = 0; i < nev; ++i) {
                    double* w = W.p + (int64_t)m * n;
                    // w = H a_i - lam_i a_i, against the columns so far (twice)
                    ED_CUDA(cudaMemcpyAsync(w, HW.p + (int64_t)i * n, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
                    for (int pass = 0; pass < 2; ++pass) {
                        dots(W.p, m, w, -1.0);
                        k_lock_axpy<<<nb, kThreads, 0, st>>>(w, W.p, m, wpart.p + (int64_t)m * nb, n);
                        ::edgb::count_launch();
                        ED_CUDA(cudaGetLastError());
                    }
                    const double nw = norm(w);
                    if (!(nw > 1e-14 * std::max(1.0, std::fabs(lam[i])))) continue;   // nothing new
                    mul(w, 1.0 / nw);
                    op_apply(op, w, HW.p + (int64_t)m * n, st);
                    ++total.matvecs;
                    ++m;
                }
            }
            // P = W^T H W (symmetrised), lowest nev Ritz pairs
            std::vector<double> P((size_t)m * m), c(m);
            for (int j = 0; j < m; ++j) {
                dots(W.p, m, HW.p + (int64_t)j * n, 1.0);
                ED_CUDA(cudaMemcpyAsync(c.data(), wpart.p + (int64_t)m * nb, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
                ED_CUDA(cudaStreamSynchronize(st));
                for (int i = 0; i < m; ++i) P[(size_t)i * m + j] = c[i];
            }
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < i; ++j) {
                    const double a = 0.5 * (P[(size_t)i * m + j] + P[(size_t)j * m + i]);
                    P[(size_t)i * m + j] = P[(size_t)j * m + i] = a;
                }
            std::vector<double> ev, Y;
            sym_eigen(m, P, ev, Y);
            rotate_basis(W.p, n, m, Y.data(), m, nev, Ar.p, rot, 0, st);
            std::swap(A.p, Ar.p);
            lam.assign(ev.begin(), ev.begin() + nev);
            residual_norms(op, A.p, lam.data(), nev, res.data(), st);
            total.matvecs += nev;
            ok = *std::max_element(res.begin(), res.end()) <= tol;
        }
    }
    if (!ok) {
        // a degeneracy the ladder does not generate: the deflated passes
        ed_lanczos_params r = p;
        if (r.degeneracy_passes <= 0) r.degeneracy_passes = nev;
        ed_solve_info pi;
        ED_CUDA(cudaStreamSynchronize(st));
        lanczos_solve(op, r, v0_dev, evals_host, evecs_dev, &pi, caller);
        add_info(total, pi);
        total.converged = pi.converged;
        total.max_residual = pi.max_residual;
        total.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (info) *info = total;
        return;
    }
    for (int i = 0; i < nev; ++i) evals_host[i] = lam[i];
    if (evecs_dev) ED_CUDA(cudaMemcpyAsync(evecs_dev, A.p, (size_t)n * nev * 8, cudaMemcpyDeviceToDevice, st));
    ED_CUDA(cudaStreamSynchronize(st));
    total.converged = nev;
    total.max_residual = *std::max_element(res.begin(), res.end());
    total.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = total;
}

}  // namespace edgb
