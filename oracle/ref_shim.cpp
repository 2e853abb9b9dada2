// C-ABI shim over the reference's own bit-level primitives, so the oracle's
// restatement can be pinned against the reference compiled from its sources.
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile (target `ref`) into
// oracle/_ref/libref.so, and only when the reference source tree is present.
// The reference headers are included from that tree at build time; none of
// their code is copied here.
#include <cstdint>
#include <cmath>
#include <functional>
#include "utilities/general/orbital_and_state_defs.hpp"
#include "utilities/mathematics/binary_number_tools.hpp"
#include "utilities/mathematics/binomials.hpp"
#include "utilities/mathematics/fermions.hpp"
#include "utilities/algorithms/binary_search.hpp"
#include "fqhe_sphere/pseudopotential_model/angular_momentum_constraint.hpp"

extern "C" {

// fermions.hpp:52 Evaluate_CdCdCC
uint64_t ref_evaluate_cdcdcc(int* sign, uint64_t k1o, uint64_t k2o, uint64_t k3o, uint64_t k4o,
                             uint64_t state, uint64_t highest)
{
    int s = 0;
    uint64_t out = utilities::Evaluate_CdCdCC(s, k1o, k2o, k3o, k4o, state, highest);
    *sign = s;
    return out;
}

// binary_number_tools.cpp:255 NextHammingNumber64
uint64_t ref_next_hamming(uint64_t x) { return utilities::binary::NextHammingNumber64(x); }

// binary_number_tools.cpp:297 GenerateHammingNumber
uint64_t ref_generate_hamming(unsigned int w, uint64_t index)
{
    return utilities::binary::GenerateHammingNumber(w, index);
}

// binary_number_tools.cpp:137 HammingWeight64Iterative
int ref_hamming_weight(uint64_t x) { return utilities::binary::HammingWeight64Iterative(x); }

// binary_number_tools.cpp:190 Base2Log
unsigned int ref_base2log(uint64_t x) { return utilities::binary::Base2Log(x); }

// binomials.cpp:34 BinomialFromTable
long int ref_binomial(int n, int k) { return utilities::BinomialFromTable(n, k); }

// binary_search.hpp:50 BinarySearch<uint64_t, uint64_t>
uint64_t ref_binary_search(uint64_t value, const uint64_t* array, uint64_t dim)
{
    return utilities::BinarySearch<uint64_t, uint64_t>(value, array, dim);
}

// angular_momentum_constraint.hpp:41 TestAngularMomentumSector
int ref_lz_ok(uint64_t state, int twoLz, int maxLz)
{
    return diagonalization::TestAngularMomentumSector(state, (diagonalization::mState_t)twoLz, (diagonalization::mState_t)maxLz) ? 1 : 0;
}

}  // extern "C"

extern "C" {
// Sector scan driven by the reference's own primitives, in the order of
// fermion_fock_basis.cpp:266-307: unrank the first word, then step with
// NextHammingNumber64 over all C(norb,N) words, keeping those that pass
// TestAngularMomentumSector.  With out == nullptr only counts.
uint64_t ref_basis_scan(int N, int norb, int twoLz, uint64_t* out)
{
    uint64_t full = 1;
    for (int i = 1; i <= N; ++i) full = full * (uint64_t)(norb - N + i) / (uint64_t)i;
    uint64_t w = utilities::binary::GenerateHammingNumber((unsigned)N, 0);
    uint64_t c = 0;
    for (uint64_t i = 0; i < full; ++i) {
        if (diagonalization::TestAngularMomentumSector(w, (diagonalization::mState_t)twoLz,
                                                       (diagonalization::mState_t)(norb - 1))) {
            if (out) out[c] = w;
            ++c;
        }
        w = utilities::binary::NextHammingNumber64(w);
    }
    return c;
}
}  // extern "C"
