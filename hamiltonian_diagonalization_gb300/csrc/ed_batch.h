// The batch handle (many Hamiltonians of one sector on one shared pattern)
// and the batched helpers shared by ed_batched.cu and ed_subspace.cu.
#pragma once

#include <array>
#include <vector>

#include "ed_internal.h"

struct ed_batch {
    int B = 0;                    // Hamiltonians
    int K = 0, N = 0;
    int64_t n = 0, nnz = 0;       // sector dimension, off-diagonal pattern entries
    int nhop = 0;
    edgb::DevBuf<int64_t> rowptr;
    edgb::DevBuf<int32_t> col;    // nnz + pad
    edgb::DevBuf<uint16_t> code;  // nnz + pad
    edgb::DevBuf<double> w;       // [nhop][B] per-Hamiltonian hop values
    edgb::DevBuf<double> diag;    // [n][B]
    // Per-Hamiltonian coefficient vectors [B][nhop + 2 K^2]: the hop values
    // and the two diagonal-term tables, everything a Hamiltonian of the batch
    // depends on.  A Hamiltonian is linear in this vector, so linear relations
    // between the vectors are relations between the Hamiltonians.
    std::vector<double> coef;
    int ncoef = 0;
    // tuned block-product tile: Hamiltonians per tile, loads in flight, threads
    // per CTA, hop values through L1 (1) or staged in shared memory (0)
    int tb = 32, unroll = 4, nt = 256, l1 = 1;
    int tuned = 0;                // 1 after batch_autotune: subsets get their own tuned tiles
};

namespace edgb {

int batch_sms();

// The per-Hamiltonian operands of a block product: hop values [nhop][B] and
// diagonals [n][B] for the B problems being multiplied (all of a batch, or
// a compacted subset of it).
struct BlockOperands {
    const double* w;
    const double* diag;
    int B;
};

BlockOperands full_operands(const ed_batch& bt);

// Operands of the problems sel[0..nsel) gathered into w [nhop][nsel] and
// diag [n][nsel] (device buffers sized by the call).
BlockOperands gather_operands(const ed_batch& bt, const int* sel_host, int nsel, DevBuf<double>& w,
                              DevBuf<double>& diag, cudaStream_t st);

// Block-product tile (Hamiltonians per tile, loads in flight, threads, L1)
// for operands like o: the batch's own for the whole batch, else one tuned
// for o's problem count (when the batch was autotuned).  Not during capture.
std::array<int, 4> batch_tile(const ed_batch& bt, const BlockOperands& o, cudaStream_t st);

// Y[r][b] = H_b X[r][b] for the o.B problems of o, with the tile for o.
void batch_block_product(const ed_batch& bt, const BlockOperands& o, const double* X, double* Y, cudaStream_t st);

// res[b * k + i] = || H_b x_{i,b} - lam[b * k + i] x_{i,b} || for the o.B
// problems of o, X [k][n][o.B] on the device, lam and res on the host.
void batch_residuals(const ed_batch& bt, const BlockOperands& o, const double* X, const double* lam, int k,
                     double* res, cudaStream_t st);

// Lockstep thick-restart Lanczos for the problems sel[0..nsel) of the batch
// (all of them when sel is null); V0 [n][nsel], evals [nsel][nev], evecs
// [nev][n][nsel] follow the selection's order.
void batch_solve(const ed_batch& bt, const int* sel, int nsel, const ed_lanczos_params& p, const double* V0,
                 double* evals, double* evecs, ed_batch_info* info, cudaStream_t caller_stream);

}  // namespace edgb
