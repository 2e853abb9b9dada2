// Internal declarations shared by the translation units of libedgb300.
#pragma once

#include <cstdint>
#include <cstddef>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ed_capi.h"

namespace edgb {

// Largest orbital count of the device path: the two-table rank splits a word
// into a low and a high half of at most 20 bits each, and the per-hop tables
// must fit in shared memory.
constexpr int kMaxOrbitals = 40;
constexpr int kMaxTwoLevelBits = 48;          // two-level words: norb0 + norb1 bits
constexpr uint64_t kMiss = ~0ull;             // FindFockStateIndex miss code
constexpr double kSparseZeroTol = 1e-14;      // hamiltonian_data.hpp:53
constexpr double kCgEps = 1e-12;              // clebsch_gordan_coefficients.hpp:53
constexpr int64_t kCrsPad = 256;              // zeroed CRS elements after the last row

struct Error : std::runtime_error {
    ed_status code;
    Error(ed_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);
// Number of kernels this library has launched (all devices, all threads).
void count_launch();
// Adds d (may be negative): kernels recorded into a CUDA graph are counted
// when the graph is launched, not when they are captured.
void count_launches(int64_t d);
uint64_t launch_count();

#define ED_CUDA(x)                                                                            \
    do {                                                                                      \
        cudaError_t _e = (x);                                                                 \
        if (_e != cudaSuccess) {                                                              \
            throw ::edgb::Error(_e == cudaErrorMemoryAllocation ? ED_ERR_OOM : ED_ERR_CUDA,     \
                                std::string(#x) + ": " + cudaGetErrorString(_e));             \
        }                                                                                     \
    } while (0)

#define ED_REQUIRE(cond, code, msg)                                                           \
    do {                                                                                      \
        if (!(cond)) throw ::edgb::Error((code), (msg));                                      \
    } while (0)

// Run f, turning any exception into a status code and a last-error message
// (no exception crosses the C ABI).
template <class F>
ed_status guard(F&& f)
{
    try {
        f();
        return ED_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return ED_ERR_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return ED_ERR_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return ED_ERR_INTERNAL;
    }
}

// Owning device buffer.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count) ED_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
    // grow (without keeping the contents) when fewer than count elements are held
    void alloc_at_least(size_t count) {
        if (count > n) alloc(count);
    }
};

// ------------------------------------------------------------ host tables

// Quartic term tables as the reference keeps them (QuarticTermTables) plus
// the derived per-hop table the device kernels read.
struct HopTables {
    int K = 0;
    // pair sums s = a+b (a<b) run over 1..2K-3; pairs of sum s are
    // (a, s-a) for a = lo(s) .. lo(s)+cnt(s)-1 with lo(s) = max(0, s-K+1).
    std::vector<int> hop_off;     // size 2K: offset of the cnt(s)^2 block of sum s
    std::vector<double> w;        // per (pair_in, pair_out) element value, 0 if dropped
    std::vector<double> diag_a;   // K*K: first  diagonal term of ordered pair (k4,k3)
    std::vector<double> diag_b;   // K*K: second diagonal term of ordered pair (k4,k3)
};

uint64_t binomial_u64(int n, int k);
void coulomb_pseudopotentials(int norb, double* out);
double clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM);
void quartic_tables(int norb, const double* pp, int npp, uint16_t* ktab, double* vtab);
HopTables derive_hop_tables(int norb, const uint16_t* ktab, const double* vtab);

// Symmetric eigen-decomposition of a dense m x m matrix (row-major, both
// triangles filled).  evals ascending; evecs column-major (evecs[i + m*j] =
// component i of eigenvector j).
void sym_eigen(int m, const std::vector<double>& a, std::vector<double>& evals, std::vector<double>& evecs);

// The same decompositions on the device (ed_eigen_dev.cu, FP64 Jacobi, one CTA
// per matrix) for m <= kDeviceEigenMax.  sym_eigen_device: count matrices
// already on the device (row-major) to device eigenvalues (count x m,
// ascending) and eigenvectors (count x m x m, column-major).
// sym_eigen_batched: the same from and to host arrays.
// One SM issues about two FP64 FMAs per clock, so one small matrix solves
// faster on a host core (m = 41: 1.63 ms on the device, 0.13 ms on the host,
// measured on GB300); a batch solves in the time of one matrix (64 of m = 41:
// 1.87 ms against 8.2 ms).  The solvers therefore use the device for batches
// of at least kDeviceEigenMinBatch matrices and the host otherwise.
constexpr int kDeviceEigenMax = 128;
constexpr int kDeviceEigenMinBatch = 16;
void sym_eigen_device(int m, int count, const double* A_dev, double* evals_dev, double* evecs_dev, cudaStream_t st);
void sym_eigen_batched(int m, int count, const double* a_host, double* evals_host, double* evecs_host, cudaStream_t st);

// ------------------------------------------------------------- pair indexing

// Helpers shared by host and device code for the per-hop table layout.
#if defined(__CUDACC__)
#define ED_HD __host__ __device__ __forceinline__
#else
#define ED_HD inline
#endif

ED_HD int pair_lo(int s, int K) { return s - (K - 1) > 0 ? s - (K - 1) : 0; }
ED_HD int pair_cnt(int s, int K) {
    int hi = (s - 1) / 2;                 // largest a with a < s-a
    int lo = pair_lo(s, K);
    return hi >= lo ? hi - lo + 1 : 0;
}

}  // namespace edgb

// ------------------------------------------------------------ handle types

struct ed_basis {
    // norb bits per word.  One level: bit k is orbital k (Lz weight k).  Two
    // levels (TwoLevelFermionFockBasis): the low norb1 = norb0 + 2 bits are
    // the second level's orbitals (weight j), the high norb0 bits the lowest
    // level's (weight i + 1), so ascending words follow the reference's
    // (first, second) order and the sector is a fixed sum of weights.
    // Momentum sectors (dimX > 0, the optical-flux-lattice basis): bit
    // p = kx * dimY + ky, the sector fixes (sum kx mod dimX, sum ky mod dimY).
    int N = 0, norb = 0, two_lz = 0;
    int levels = 1, norb0 = 0, norb1 = 0;
    int dimX = 0, dimY = 0, kx_tot = 0, ky_tot = 0;
    int64_t sector_sum = -1;     // sum of occupied positions in the sector (-1: empty)
    uint64_t dim = 0;
    int low_bits = 0, high_bits = 0;
    edgb::DevBuf<uint64_t> words;   // dim ascending words
    edgb::DevBuf<uint64_t> hi;      // 2^high_bits: (class << 48) | offset
    edgb::DevBuf<uint64_t> lo;      // 2^low_bits : (class << 32) | rank in class
    // Compact rank tables for the matrix-free product (basis_compact_tables):
    // the same scheme with mf_low_bits (<= 13) low bits, whose 4-byte
    // (class << 16) | rank entries fit in shared memory.  Built on first use.
    mutable int mf_low_bits = 0;
    mutable edgb::DevBuf<uint64_t> mf_hi;   // 2^(norb - mf_low_bits): (class << 48) | offset
    mutable edgb::DevBuf<uint32_t> mf_lo;   // 2^mf_low_bits: (class << 16) | rank in class
};

struct ed_terms {
    int norb = 0;
    std::vector<uint16_t> ktab;
    std::vector<double> vtab;
    edgb::HopTables hop;
    edgb::DevBuf<double> w_dev;       // hop.w
    edgb::DevBuf<int> hop_off_dev;    // hop.hop_off
    edgb::DevBuf<double> diag_a_dev;  // hop.diag_a
    edgb::DevBuf<double> diag_b_dev;  // hop.diag_b
};

// Sliced-ELL copy of a full-storage CRS (SELL-C-sigma with C = 32): within
// windows of kSellWindow rows the rows are ordered by length (longest first)
// and cut into chunks of 32; chunk c holds its rows column-major, element j
// of its lane l at off[c] + 32 j + l, padded with zeros to the chunk's
// longest row len[c].  row[32 c + l] is the CRS row of lane l (-1: none).
// The product reads it with one lane per row: coalesced loads, no cross-lane
// reduction, and lanes of a chunk that finish together.
struct ed_sell {
    int64_t nchunks = 0, nnz_pad = 0;
    edgb::DevBuf<int64_t> off;
    edgb::DevBuf<int32_t> len;
    edgb::DevBuf<int32_t> row;
    edgb::DevBuf<int32_t> col;
    edgb::DevBuf<double> val;
};

// Fixed-point copy of a full-storage CRS's values for the integer-pipe
// product: value a = A 2^(ea - 1080) with A = round(a 2^(1080 - ea)),
// |A| < 2^58 (ea the largest biased exponent field of the values, at least
// 1), held as the pair (A mod 2^30, floor(A / 2^30)) of 32-bit integers in
// one 64-bit word.  x is converted the same way into a per-stream scratch
// before each product; part holds the per-block exponent maxima of x and,
// after them, the vector's exponent bound.
struct ed_fixq {
    int ea = 1;
    // the values as limb pairs, each copy made when a kernel first needs it
    // (state 0 not yet tried, 1 made, -1 declined for memory): val in the
    // CRS order (nnz + kCrsPad pairs, zero pairs after the last row), sval in
    // the sliced-ELL order (nnz_pad + kCrsPad)
    edgb::DevBuf<int64_t> val, sval;
    int val_state = 0, sval_state = 0;
    // the staged kernel's ring: stage capacity (elements) and stage count,
    // 0 when it does not fit; err counts its waits that ran out
    int stage_elems = 0, stages = 0;
    edgb::DevBuf<int> err;
    struct Scratch {
        edgb::DevBuf<int64_t> xq;
        edgb::DevBuf<int> part;
    };
    std::mutex mu;
    std::map<std::pair<int, cudaStream_t>, std::unique_ptr<Scratch>> scratch;   // by (device, stream)
};

struct ed_crs {
    int64_t n = 0, nnz = 0;
    int upper = 0;
    int max_row = 0;
    edgb::DevBuf<int64_t> rowptr;
    edgb::DevBuf<int32_t> col;
    edgb::DevBuf<double> val;
    // the product's sliced-ELL copy (full storage), made on the first
    // product outside a stream capture; state 0 not yet tried, 1 made,
    // -1 not made (upper storage, short rows, or not enough free memory)
    mutable std::unique_ptr<ed_sell> sell;
    mutable int sell_state = 0;
    // the integer-pipe product's fixed-point values (full storage, rows of
    // 96 and more elements on average), same states
    mutable std::unique_ptr<ed_fixq> fixq;
    mutable int fix_state = 0;
    int product_kernel = 0;   // 0: chosen by shape; else an ed_spmv_kernel id for every product
};

// Complex momentum-conserving terms (the optical-flux-lattice QuarticTermTables
// and QuadraticTermTables in the array format): orbital p = kx * dimY + ky, a
// pair's class is ((kx_a + kx_b) mod dimX, (ky_a + ky_b) mod dimY), and every
// off-diagonal element is a pair hop within one class.  w holds, per class,
// cnt x cnt complex hop weights [removed pair][created pair] with the four
// ordered terms folded in the reference's visiting order and relative signs
// +,-,-,+ (exact zero where no term survives the 1e-14 filters), da/db the
// two diagonal terms of each ordered (k4, k3), and e the occupation energies.
struct ed_cterms {
    int norb = 0, dimX = 0, dimY = 0;
    std::vector<uint16_t> ktab;     // reference layout, (K+1) K^2 / 2 entries
    std::vector<double> vtab;       // same, complex as (re, im) pairs
    std::vector<double> e;          // K complex energies (zero without Add_CdC_Terms)
    std::vector<int> cls_off;       // dimX*dimY + 1: start of each class's pair list
    std::vector<uint16_t> pairs;    // created/removed pairs c | d << 8, c < d, by class
    std::vector<int> pair_index;    // K*K: (a, b), a < b -> index within its class
    std::vector<int> w_off;         // dimX*dimY + 1: start of each class's weights
    std::vector<double> w;          // complex hop weights
    std::vector<double> da, db;     // K*K complex diagonal terms
    edgb::DevBuf<int> cls_off_dev, pair_index_dev, w_off_dev;
    edgb::DevBuf<uint16_t> pairs_dev;
    edgb::DevBuf<double> w_dev, da_dev, db_dev, e_dev;
};

// Complex CRS (std::complex<double> values as (re, im) pairs).  upper = 1 is
// the reference's storage: row = in-state, column = out-state >= in-state,
// value <out|H|in>, applied as y_i += A_ij x_j, y_j += conj(A_ij) x_i.
struct ed_ccrs {
    int64_t n = 0, nnz = 0;
    int upper = 0;
    int max_row = 0;
    edgb::DevBuf<int64_t> rowptr;
    edgb::DevBuf<int32_t> col;
    edgb::DevBuf<double> val;       // 2 * (nnz + kCrsPad)
    // the integer-pipe product's fixed-point values (full storage): the real
    // and imaginary parts as two limb pairs an element, 2 * (nnz + kCrsPad)
    // words, one exponent bound; state 0 not yet tried, 1 made, -1 declined
    mutable std::unique_ptr<ed_fixq> fixq;
    mutable int fix_state = 0;
};

// ----------------------------------------------------- device-side entry points
namespace edgb {
void two_level_ladder(const ed_basis& b, const double* x, double* y, int dir, cudaStream_t st);
void cterms_derive(ed_cterms& t);
void cham_build_crs(const ed_basis& b, const ed_cterms& t, int upper, ed_ccrs& a, cudaStream_t st);
void cspmv(const ed_ccrs& a, const double* x, double* y, cudaStream_t st);
// kernel 0: as cspmv; 1: the FP64 row kernel; 2: the fixed-point integer kernel (full storage)
void cspmv_kernel(const ed_ccrs& a, int kernel, const double* x, double* y, cudaStream_t st);
// the complex product's fixed-point copy, made before a solver captures its cycles
void cspmv_prepare(const ed_ccrs& a, cudaStream_t st);
void basis_build(ed_basis& b, cudaStream_t st);
std::vector<int> basis_weights(const ed_basis& b);
void basis_rank(const ed_basis& b, const uint64_t* words, uint64_t* idx, uint64_t m, cudaStream_t st);
void basis_compact_tables(const ed_basis& b, cudaStream_t st);
void ham2_build_crs(const ed_basis& b, const ed_terms& t0, const ed_terms& t1, const double* e0_host,
                    const double* e1_host, int upper, ed_crs& a, cudaStream_t st);
void terms_upload(ed_terms& t);
void ham_diagonal(const ed_basis& b, const ed_terms& t, double* diag, cudaStream_t st);
void ham_build_crs(const ed_basis& b, const ed_terms& t, int upper, ed_crs& a, cudaStream_t st);
void spmv(const ed_crs& a, const double* x, double* y, cudaStream_t st);
// Make the product's sliced-ELL copy of a full-storage CRS now (a no-op when
// made, declined, or the stream is capturing); solvers call it before they
// capture their cycles.
void spmv_prepare(const ed_crs& a, cudaStream_t st);
// kernel 0: as spmv; 1: row lanes k_spmv_full<8,4>; 2, 3: shared reduction k_spmv_rows<8,4,2>,
// <8,2,2>; 4, 5: sliced ELL k_spmv_sell<16>, <8>; 6: fixed-point integer rows k_spmv_fix<8,8>;
// 7: the same with the rows staged in shared memory by bulk copies, k_spmv_fix_staged; 8: fixed-point
// sliced ELL k_spmv_sell_fix (full storage)
void spmv_kernel(const ed_crs& a, int kernel, const double* x, double* y, cudaStream_t st);
// Throws when a staged product's wait ran out since the last call (reads a
// device word: synchronises the stream).
void spmv_check(const ed_crs& a, cudaStream_t st);
// The staged kernel with stage 0 never filled and every wait limited to
// cycles: returns the number of waits that ran out (reset afterwards).
int spmv_staged_wait_test(const ed_crs& a, const double* x, double* y, long long cycles, cudaStream_t st);
double measure_dfma_rate(int iters, int blocks_per_sm);
void hv_matfree(const ed_basis& b, const ed_terms& t, const double* diag, const double* x, double* y,
                cudaStream_t st);
void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st);
int64_t reduce_max_i64_host(const int64_t* in, int64_t n, cudaStream_t st);
}  // namespace edgb
