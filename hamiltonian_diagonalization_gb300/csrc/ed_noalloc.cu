// Allocation-free residual norms: ed_residuals_noalloc.
//
// ed_residuals allocates a product vector and a partial-sum buffer with
// cudaMalloc on every call.  Some callers cannot allow that: applications
// that hand the whole device memory to their own pool allocator, and solver
// loops that must not call cudaMalloc/cudaFree because those synchronise the
// device and stall other streams.  This variant fuses the product into the
// residual (each row's (Hx)_r - lambda x_r is formed and squared in
// registers) and keeps its only scratch, the per-block partial sums and the
// per-vector totals, in one file-scope device array of fixed size.
//
// Limits and sharing rules (also in include/ed_capi.h):
//  - at most kNoallocMaxVectors vectors per call and kNoallocMaxBlocks row
//    blocks (the scratch is 513 KiB per device, held until the process exits);
//  - only a stored CRS with both triangles (ed_ham_build_crs store_upper = 0);
//  - every call on a device shares the one array: calls that overlap on the
//    GPU (from several host threads or streams) race and must be serialised
//    by the caller;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and keeps it, so make
//    the first call before any stream capture; a cudaDeviceReset unloads the
//    module and leaves that address stale, so the entry point must not be
//    used after one;
//  - it runs on the legacy default stream, which does not wait for work on
//    non-blocking streams: x_dev must be complete before the call.
#include <mutex>
#include <string>

#include "ed_lanczos.h"

namespace edgb {

namespace {

constexpr int kNoallocMaxVectors = 64;
constexpr int kNoallocMaxBlocks = 1024;
constexpr int kNoallocThreads = 256;
constexpr int kNoallocMaxDevices = 64;

// [vector][block] partial sums, then kNoallocMaxVectors totals
__device__ __align__(256) double g_noalloc_scratch[kNoallocMaxVectors * kNoallocMaxBlocks + kNoallocMaxVectors];

double* g_scratch_addr[kNoallocMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (set-up once
// per device).  The host-side symbol is only a stand-in and must not be
// handed to a kernel.
double* scratch_for_current_device()
{
    int dev = 0;
    ED_CUDA(cudaGetDevice(&dev));
    ED_REQUIRE(dev >= 0 && dev < kNoallocMaxDevices, ED_ERR_RANGE, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        ED_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    return g_scratch_addr[dev];
}

// Block b of vector blockIdx.y: sum over its rows of ((Hx)_r - lambda x_r)^2,
// four lanes per row as in the stored-CRS product.
__global__ void __launch_bounds__(kNoallocThreads) k_resid_fused(const int64_t* __restrict__ rowptr,
                                                               const int32_t* __restrict__ col,
                                                               const double* __restrict__ val,
                                                               const double* __restrict__ X, int64_t n,
                                                               const double* __restrict__ lambdas,
                                                               double* __restrict__ scratch)
{
    constexpr int G = 4;
    __shared__ double red[kNoallocThreads / 32];
    const int v = blockIdx.y;
    const double* x = X + (int64_t)v * n;
    const double lam = lambdas[v];
    const int lane = threadIdx.x & 31, sub = lane & (G - 1);
    const int64_t r0 = n * (int64_t)blockIdx.x / gridDim.x, r1 = n * (int64_t)(blockIdx.x + 1) / gridDim.x;
    double s2 = 0.0;
    // rows of this block, G lanes each, warp-uniform loop
    const int64_t first = r0 + (threadIdx.x >> 5) * (32 / G);
    for (int64_t rb = first; rb < r1; rb += (kNoallocThreads / 32) * (32 / G)) {
        const int64_t r = rb + lane / G;
        const bool valid = r < r1;
        const int64_t s = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
        double acc = 0.0;
        for (int64_t k = s + sub; k < e; k += G) acc = fma(val[k], __ldg(x + col[k]), acc);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (valid && sub == 0) {
            const double d = fma(-lam, x[r], acc);
            s2 = fma(d, d, s2);
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    if (lane == 0) red[threadIdx.x >> 5] = s2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kNoallocThreads / 32; ++w) t += red[w];
        scratch[(int64_t)v * kNoallocMaxBlocks + blockIdx.x] = t;
    }
}

// totals[v] = sqrt(sum over blocks); warps take vectors in turn.
__global__ void k_resid_total(double* __restrict__ scratch, int nb, int k)
{
    const int lane = threadIdx.x & 31;
    for (int v = threadIdx.x >> 5; v < k; v += blockDim.x >> 5) {
        double s = 0.0;
        for (int b = lane; b < nb; b += 32) s += scratch[(int64_t)v * kNoallocMaxBlocks + b];
#pragma unroll
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) scratch[(int64_t)kNoallocMaxVectors * kNoallocMaxBlocks + v] = sqrt(s);
    }
}

}  // namespace

namespace {

// The device on which ptr lives must be the current one: the scratch address
// and the launch belong to the current device.
void require_on_device(const void* ptr, int dev, const char* what)
{
    cudaPointerAttributes at{};
    ED_CUDA(cudaPointerGetAttributes(&at, ptr));
    ED_REQUIRE((at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev, ED_ERR_ARG,
               std::string("ed_residuals_noalloc: ") + what + " is not memory of the current device");
}

}  // namespace

}  // namespace edgb

using namespace edgb;

extern "C" ed_status ed_residuals_noalloc(const ed_op* op, const double* x_dev, const double* lambda_host, int k,
                                          double* res_host)
{
    return guard([&] {
        ED_REQUIRE(op && x_dev && lambda_host && res_host, ED_ERR_ARG, "NULL argument");
        ED_REQUIRE(k >= 1 && k <= kNoallocMaxVectors, ED_ERR_ARG,
                   "ed_residuals_noalloc takes 1..64 vectors per call");
        ED_REQUIRE(op->kind == ed_op::CRS && op->crs && !op->crs->upper, ED_ERR_ARG,
                   "ed_residuals_noalloc needs a stored full-storage CRS operator");
        const ed_crs& a = *op->crs;
        ED_REQUIRE(a.n >= 1, ED_ERR_EMPTY, "operator has dimension 0");
        int dev = 0, sms = 148;
        ED_CUDA(cudaGetDevice(&dev));
        require_on_device(a.val.p, dev, "the operator's CRS");
        require_on_device(x_dev, dev, "x_dev");
        double* scratch = scratch_for_current_device();
        // eigenvalues go through the tail of the scratch array (no buffer of our own)
        double* lam_dev = scratch + (int64_t)kNoallocMaxVectors * kNoallocMaxBlocks;
        ED_CUDA(cudaMemcpyAsync(lam_dev, lambda_host, (size_t)k * 8, cudaMemcpyHostToDevice, nullptr));
        ED_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int64_t nb = a.n / 2048;
        if (nb > (int64_t)sms * 4) nb = (int64_t)sms * 4;
        if (nb > kNoallocMaxBlocks) nb = kNoallocMaxBlocks;
        if (nb < 1) nb = 1;
        // the lambdas occupy the totals slots until k_resid_fused has read
        // them; it copies them to registers at entry, and k_resid_total
        // runs after it on the same stream
        dim3 grid((unsigned)nb, (unsigned)k);
        k_resid_fused<<<grid, kNoallocThreads, 0, nullptr>>>(a.rowptr.p, a.col.p, a.val.p, x_dev, a.n, lam_dev,
                                                             scratch);
        count_launch();
        ED_CUDA(cudaGetLastError());
        k_resid_total<<<1, 256, 0, nullptr>>>(scratch, (int)nb, k);
        count_launch();
        ED_CUDA(cudaGetLastError());
        ED_CUDA(cudaMemcpyAsync(res_host, lam_dev, (size_t)k * 8, cudaMemcpyDeviceToHost, nullptr));
        ED_CUDA(cudaStreamSynchronize(nullptr));
    });
}
