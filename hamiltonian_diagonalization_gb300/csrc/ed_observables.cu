// Observables of a sector eigenvector: the reference's Observables
// (observables/fermion_observables.hpp) for a real eigenvector of the basis's
// sector, as device reductions over the basis.
//
//   DensityFunction          (fermion_observables.hpp:48-104)   rho[k] = sum_s psi_s^2 n_k(s)
//   DensityDensityFunction   (fermion_observables.hpp:117-200)  D[k][q] = sum_s psi_s^2 n_k(s) n_q(s)
//   GetParticipationRatio    (fermion_observables.hpp:528-562)  1 / sum_s |psi_s|^4
//   GetMostProbable          (fermion_observables.hpp:437-517)  the k largest |psi_s| with their words
//
// Every reduction is deterministic: each block sums its rows in a fixed
// order, writes one partial per output, and the host adds the partials in
// block order, so repeated calls return the same bits.  The most-probable
// selection finds the exact k-th largest |psi| by a radix select on its bits
// (four 16-bit levels; the bits of a non-negative double order like the
// values), gathers every candidate at or above it and sorts them on the host
// by |psi| descending, then row ascending (the reference's partial quicksort
// leaves the order of ties unspecified).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ed_internal.h"

namespace edgb {

namespace {

constexpr int kObsThreads = 256;
constexpr int kObsWarps = kObsThreads / 32;

int obs_blocks(int64_t n)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + kObsThreads - 1) / kObsThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * 4, want));
}

// Sums T per-thread values over the block in a fixed order (lanes by
// shuffle, then warps in order); the totals land in out[0..T) of thread 0's
// block slot.
template <int T>
__device__ __forceinline__ void block_sums(const double (&acc)[T], double* red, double* out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < T; ++t) {
        double v = acc[t];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[t * kObsWarps + warp] = v;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < T; t += kObsThreads) {
        double s = 0.0;
        for (int w = 0; w < kObsWarps; ++w) s += red[t * kObsWarps + w];
        out[t] = s;
    }
}

// part[blk][t] = sum over the block's rows of psi^2 * n_{k0+t}, t < 8.
__global__ void __launch_bounds__(kObsThreads) k_obs_density(const uint64_t* __restrict__ words,
                                                             const double* __restrict__ psi, int64_t n, int k0,
                                                             double* __restrict__ part)
{
    __shared__ double red[8 * kObsWarps];
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t s = blockIdx.x * (int64_t)kObsThreads + threadIdx.x; s < n; s += (int64_t)gridDim.x * kObsThreads) {
        const double p = psi[s] * psi[s];
        const uint64_t w = words[s] >> k0;
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if ((w >> t) & 1ull) acc[t] += p;
    }
    block_sums<8>(acc, red, part + (int64_t)blockIdx.x * 8);
}

// part[blk][a*8+b] = sum over the block's rows of psi^2 * n_{k0+a} n_{q0+b}.
__global__ void __launch_bounds__(kObsThreads) k_obs_density2(const uint64_t* __restrict__ words,
                                                              const double* __restrict__ psi, int64_t n, int k0,
                                                              int q0, double* __restrict__ part)
{
    __shared__ double red[64 * kObsWarps];
    double acc[64];
#pragma unroll
    for (int t = 0; t < 64; ++t) acc[t] = 0.0;
    for (int64_t s = blockIdx.x * (int64_t)kObsThreads + threadIdx.x; s < n; s += (int64_t)gridDim.x * kObsThreads) {
        const double p = psi[s] * psi[s];
        const uint64_t wk = words[s] >> k0, wq = words[s] >> q0;
#pragma unroll
        for (int a = 0; a < 8; ++a)
            if ((wk >> a) & 1ull) {
#pragma unroll
                for (int b = 0; b < 8; ++b)
                    if ((wq >> b) & 1ull) acc[a * 8 + b] += p;
            }
    }
    block_sums<64>(acc, red, part + (int64_t)blockIdx.x * 64);
}

// part[blk] = sum over the block's rows of |psi|^4.
__global__ void __launch_bounds__(kObsThreads) k_obs_psi4(const double* __restrict__ psi, int64_t n,
                                                          double* __restrict__ part)
{
    __shared__ double red[kObsWarps];
    double acc[1] = {0.0};
    for (int64_t s = blockIdx.x * (int64_t)kObsThreads + threadIdx.x; s < n; s += (int64_t)gridDim.x * kObsThreads) {
        const double p = psi[s] * psi[s];
        acc[0] += p * p;
    }
    block_sums<1>(acc, red, part + blockIdx.x);
}

__device__ __forceinline__ uint64_t abs_bits(double x) { return (uint64_t)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull; }

// Histogram of bits [shift, shift+16) of |psi|'s bit pattern over the rows
// whose bits above shift+16 equal prefix (all rows when shift == 48).
__global__ void __launch_bounds__(kObsThreads) k_obs_hist(const double* __restrict__ psi, int64_t n, int shift,
                                                          uint64_t prefix, unsigned int* __restrict__ hist)
{
    for (int64_t s = blockIdx.x * (int64_t)kObsThreads + threadIdx.x; s < n; s += (int64_t)gridDim.x * kObsThreads) {
        const uint64_t u = abs_bits(psi[s]);
        if (shift < 48 && (u >> (shift + 16)) != prefix) continue;
        atomicAdd(hist + ((u >> shift) & 0xFFFFull), 1u);
    }
}

// Rows with |psi| bits >= thr, appended as (row, psi) in any order; at most
// cap of them are stored (the host sized cap to the exact count).
__global__ void __launch_bounds__(kObsThreads) k_obs_collect(const double* __restrict__ psi, int64_t n, uint64_t thr,
                                                             unsigned long long* __restrict__ count, int64_t cap,
                                                             int64_t* __restrict__ rows, double* __restrict__ vals)
{
    for (int64_t s = blockIdx.x * (int64_t)kObsThreads + threadIdx.x; s < n; s += (int64_t)gridDim.x * kObsThreads) {
        const double v = psi[s];
        if (abs_bits(v) < thr) continue;
        const unsigned long long slot = atomicAdd(count, 1ull);
        if ((int64_t)slot < cap) {
            rows[slot] = s;
            vals[slot] = v;
        }
    }
}

// out[i] = words[rows[i]] for i < m.
__global__ void k_obs_words(const uint64_t* __restrict__ words, const int64_t* __restrict__ rows, int64_t m,
                            uint64_t* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = words[rows[i]];
}

// The block partials of one launch summed in block order.
std::vector<double> sum_partials(const DevBuf<double>& part, int nb, int width)
{
    std::vector<double> h((size_t)nb * width), out(width, 0.0);
    ED_CUDA(cudaMemcpy(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost));
    for (int b = 0; b < nb; ++b)
        for (int t = 0; t < width; ++t) out[t] += h[(size_t)b * width + t];
    return out;
}

struct DevPsi {
    DevBuf<double> buf;
    DevPsi(const double* host, int64_t n) : buf((size_t)std::max<int64_t>(n, 1))
    {
        if (n > 0) ED_CUDA(cudaMemcpy(buf.p, host, (size_t)n * 8, cudaMemcpyHostToDevice));
    }
};

}  // namespace

}  // namespace edgb

using namespace edgb;

extern "C" ed_status ed_obs_density(const ed_basis* b, const double* psi_host, double* rho_host)
{
    return guard([&] {
        ED_REQUIRE(b && psi_host && rho_host, ED_ERR_ARG, "basis, psi and rho must not be NULL");
        const int K = b->norb;
        const int64_t n = (int64_t)b->dim;
        std::fill(rho_host, rho_host + K, 0.0);
        if (n == 0) return;
        DevPsi psi(psi_host, n);
        const int nb = obs_blocks(n);
        DevBuf<double> part((size_t)nb * 8);
        for (int k0 = 0; k0 < K; k0 += 8) {
            k_obs_density<<<nb, kObsThreads>>>(b->words.p, psi.buf.p, n, k0, part.p);
            count_launch();
            ED_CUDA(cudaGetLastError());
            const std::vector<double> s = sum_partials(part, nb, 8);
            for (int t = 0; t < 8 && k0 + t < K; ++t) rho_host[k0 + t] = s[t];
        }
    });
}

extern "C" ed_status ed_obs_density_density(const ed_basis* b, const double* psi_host, double* table_host)
{
    return guard([&] {
        ED_REQUIRE(b && psi_host && table_host, ED_ERR_ARG, "basis, psi and table must not be NULL");
        const int K = b->norb;
        const int64_t n = (int64_t)b->dim;
        std::fill(table_host, table_host + (size_t)K * K, 0.0);
        if (n == 0) return;
        DevPsi psi(psi_host, n);
        const int nb = obs_blocks(n);
        DevBuf<double> part((size_t)nb * 64);
        // tiles on and above the diagonal; the table is symmetric
        for (int k0 = 0; k0 < K; k0 += 8)
            for (int q0 = k0; q0 < K; q0 += 8) {
                k_obs_density2<<<nb, kObsThreads>>>(b->words.p, psi.buf.p, n, k0, q0, part.p);
                count_launch();
                ED_CUDA(cudaGetLastError());
                const std::vector<double> s = sum_partials(part, nb, 64);
                for (int a = 0; a < 8 && k0 + a < K; ++a)
                    for (int c = 0; c < 8 && q0 + c < K; ++c) {
                        table_host[(size_t)(k0 + a) * K + (q0 + c)] = s[a * 8 + c];
                        table_host[(size_t)(q0 + c) * K + (k0 + a)] = s[a * 8 + c];
                    }
            }
    });
}

extern "C" ed_status ed_obs_participation_ratio(const ed_basis* b, const double* psi_host, double* ratio)
{
    return guard([&] {
        ED_REQUIRE(b && psi_host && ratio, ED_ERR_ARG, "basis, psi and ratio must not be NULL");
        const int64_t n = (int64_t)b->dim;
        ED_REQUIRE(n > 0, ED_ERR_ARG, "empty sector");
        DevPsi psi(psi_host, n);
        const int nb = obs_blocks(n);
        DevBuf<double> part(nb);
        k_obs_psi4<<<nb, kObsThreads>>>(psi.buf.p, n, part.p);
        count_launch();
        ED_CUDA(cudaGetLastError());
        const double s = sum_partials(part, nb, 1)[0];
        ED_REQUIRE(s > 0.0, ED_ERR_ARG, "zero eigenvector");
        *ratio = 1.0 / s;
    });
}

extern "C" ed_status ed_obs_most_probable(const ed_basis* b, const double* psi_host, int64_t k, uint64_t* states_host,
                                          double* amps_host, int64_t* count_out)
{
    return guard([&] {
        ED_REQUIRE(b && psi_host && states_host && amps_host && count_out && k >= 0, ED_ERR_ARG, "bad argument");
        const int64_t n = (int64_t)b->dim;
        const int64_t kk = std::min<int64_t>(k, n);
        *count_out = kk;
        if (kk == 0) return;
        DevPsi psi(psi_host, n);
        const int nb = obs_blocks(n);
        // radix select of the kk-th largest |psi| bit pattern, 16 bits a level
        DevBuf<unsigned int> hist(65536);
        std::vector<unsigned int> h(65536);
        uint64_t prefix = 0;
        int64_t need = kk, above = 0;
        for (int shift = 48; shift >= 0; shift -= 16) {
            ED_CUDA(cudaMemset(hist.p, 0, 65536 * 4));
            k_obs_hist<<<nb, kObsThreads>>>(psi.buf.p, n, shift, prefix, hist.p);
            count_launch();
            ED_CUDA(cudaGetLastError());
            ED_CUDA(cudaMemcpy(h.data(), hist.p, 65536 * 4, cudaMemcpyDeviceToHost));
            int bin = 65535;
            for (; bin > 0; --bin) {
                if ((int64_t)h[bin] >= need) break;
                need -= h[bin];
                above += h[bin];
            }
            prefix = (prefix << 16) | (uint64_t)bin;
        }
        const uint64_t thr = prefix;   // the kk-th largest pattern: `above` rows lie strictly above it
        // every row at or above the threshold (ties included), sorted on the host
        DevBuf<unsigned long long> cnt(1);
        ED_CUDA(cudaMemset(cnt.p, 0, 8));
        unsigned long long total = 0;
        // first pass counts (cap 0), second stores
        k_obs_collect<<<nb, kObsThreads>>>(psi.buf.p, n, thr, cnt.p, 0, nullptr, nullptr);
        count_launch();
        ED_CUDA(cudaGetLastError());
        ED_CUDA(cudaMemcpy(&total, cnt.p, 8, cudaMemcpyDeviceToHost));
        ED_REQUIRE((int64_t)total >= kk && (int64_t)total >= above, ED_ERR_INTERNAL, "radix select miscounted");
        DevBuf<int64_t> rows(total);
        DevBuf<double> vals(total);
        ED_CUDA(cudaMemset(cnt.p, 0, 8));
        k_obs_collect<<<nb, kObsThreads>>>(psi.buf.p, n, thr, cnt.p, (int64_t)total, rows.p, vals.p);
        count_launch();
        ED_CUDA(cudaGetLastError());
        std::vector<int64_t> hr(total);
        std::vector<double> hv(total);
        ED_CUDA(cudaMemcpy(hr.data(), rows.p, total * 8, cudaMemcpyDeviceToHost));
        ED_CUDA(cudaMemcpy(hv.data(), vals.p, total * 8, cudaMemcpyDeviceToHost));
        std::vector<size_t> order(total);
        for (size_t i = 0; i < total; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
            const double ax = std::fabs(hv[x]), ay = std::fabs(hv[y]);
            return ax != ay ? ax > ay : hr[x] < hr[y];
        });
        std::vector<int64_t> pick(kk);
        for (int64_t i = 0; i < kk; ++i) {
            const size_t o = order[(size_t)i];
            amps_host[i] = hv[o];
            pick[(size_t)i] = hr[o];
        }
        DevBuf<int64_t> dpick(kk);
        DevBuf<uint64_t> dwords(kk);
        ED_CUDA(cudaMemcpy(dpick.p, pick.data(), (size_t)kk * 8, cudaMemcpyHostToDevice));
        k_obs_words<<<obs_blocks(kk), kObsThreads>>>(b->words.p, dpick.p, kk, dwords.p);
        count_launch();
        ED_CUDA(cudaGetLastError());
        ED_CUDA(cudaMemcpy(states_host, dwords.p, (size_t)kk * 8, cudaMemcpyDeviceToHost));
    });
}
