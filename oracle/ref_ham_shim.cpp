// C-ABI shim over the reference's own sector basis, quartic Hamiltonian build
// and observables, so the oracle's restatement of them can be pinned against
// the reference compiled from its sources.
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile (target `ref`) into
// oracle/_ref/libref_ham.so when the reference source tree is present.  The
// reference's files are included from that tree at build time; none of their
// code is copied here.  They reach MPI only through the reference's
// MpiWrapper, compiled here against the one-rank stand-in oracle/ref_stubs/mpi.h,
// and include option-description helpers compiled against the compile-only
// oracle/ref_stubs/boost/program_options.hpp (never called).
//
// Calls follow the reference's model driver
// (fqhe_sphere/pseudopotential_model/pseudopotential_model.cpp:160-189,233-249):
// FermionFockBasis::GenerateFockSpace with std::bind(TestAngularMomentumSector,
// _1, 2Lz, 2S), SetFockBasis, Initialize with mapped storage,
// Add_CdCdCC_Terms over all rows, then the mapped -> CRS conversion of
// hamiltonian_base.hpp:183-251 (ResetMatrixStorageMethod) and the CRS
// writer of crs_sparse_matrix.hpp:662-705 in its binary format.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

// headers the reference's own translation units see before these (its
// templates name their symbols at definition)
#include "utilities/general/serialize.hpp"
#include "utilities/general/i_const_def.hpp"
#include "utilities/general/pi_const_def.hpp"
#include "basis/fermion_fock_basis.hpp"
#include "hamiltonians/spinless_fermion_hamiltonian.hpp"
#include "observables/fermion_observables.hpp"
#include "fqhe_sphere/pseudopotential_model/angular_momentum_constraint.hpp"
#include "fqhe_sphere/pseudopotential_model/term_tables.hpp"
#include "basis/two_level_fermion_fock_basis.hpp"
#include "hamiltonians/two_level_spinless_fermion_hamiltonian.hpp"
#include "fqhe_sphere/pseudopotential_model/two_level_angular_momentum_constraint.hpp"

// The reference defines its output-verbosity object in each program's main
// file; this shim is such a program.
namespace utilities {
Cout cout;
}

namespace {

utilities::MpiWrapper& session()
{
    static utilities::MpiWrapper* mpi = nullptr;
    if (!mpi) {
        mpi = new utilities::MpiWrapper();
        // its constructor leaves the exit flag unset (the reference's programs
        // create the wrapper with static storage, which starts zeroed)
        mpi->m_exitFlag = false;
        char* argv[] = {nullptr};
        mpi->Init(0, argv, true);
        const char* v = std::getenv("ORACLE_REF_VERBOSE");   // the reference's own messages, 0..3
        utilities::cout.SetVerbosity(v ? std::atoi(v) : 0);
    }
    return *mpi;
}

// The reference's Hamiltonian with its protected storage conversion
// (mapped -> CRS, the step its LanczosDiagonalize takes first) reachable.
struct RefHamiltonian : diagonalization::SpinlessFermionHamiltonian<double> {
    void ToCrs(utilities::MpiWrapper& mpi)
    {
        this->ResetMatrixStorageMethod(utilities::_SPARSE_CRS_, diagonalization::_PARALLEL_, mpi);
    }
};

struct RefTwoLevelHamiltonian : diagonalization::TwoLevelSpinlessFermionHamiltonian<double> {
    void ToCrs(utilities::MpiWrapper& mpi)
    {
        this->ResetMatrixStorageMethod(utilities::_SPARSE_CRS_, diagonalization::_PARALLEL_, mpi);
    }
};

// The reference's two-level sector basis
// (two_level_pseudopotential_model.cpp:114-145): norb0 lowest-level orbitals
// and norb0 + 2 in the second level, maxLz2 = norb0 + 1.
bool make_basis2(int N, int norb0, int twoLz, diagonalization::TwoLevelFermionFockBasis& basis)
{
    utilities::MpiWrapper& mpi = session();
    const diagonalization::mState_t lz = (diagonalization::mState_t)twoLz;
    const diagonalization::mState_t maxLz2 = (diagonalization::mState_t)(norb0 + 1);
    return basis.GenerateFockSpace(N, norb0, norb0 + 2, std::bind(&diagonalization::TestAngularMomentumSector2LL,
                                                                  std::placeholders::_1, lz, maxLz2), mpi);
}

// The reference's sector basis: 2Lz in twice units, maxLz = 2S = norb - 1.
bool make_basis(int N, int norb, int twoLz, diagonalization::FermionFockBasis& basis)
{
    utilities::MpiWrapper& mpi = session();
    const diagonalization::mState_t lz = (diagonalization::mState_t)twoLz;
    const diagonalization::mState_t maxLz = (diagonalization::mState_t)(norb - 1);
    return basis.GenerateFockSpace(N, norb, std::bind(&diagonalization::TestAngularMomentumSector,
                                                      std::placeholders::_1, lz, maxLz), mpi);
}

}  // namespace

extern "C" {

// Sector basis words in the reference's order (fermion_fock_basis.cpp:241-354);
// returns the dimension, copies the words when out is given.
uint64_t refh_basis(int N, int norb, int twoLz, uint64_t* out)
{
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, norb, twoLz, basis)) return 0;
    const uint64_t dim = basis.GetStoredDimension();
    if (out) {
        std::vector<diagonalization::fock_t>::const_iterator it;
        diagonalization::fock_t s = basis.GetFirstState(0, N, it);
        for (uint64_t i = 0; i < dim; ++i) {
            out[i] = s;
            s = basis.GetNextState(s, it);
        }
    }
    return dim;
}

// Upper-triangle CRS of the quartic Hamiltonian built by the reference from
// the given tables (ktab/vtab in QuarticTermTables layout, K^3 entries),
// written to path in the reference's binary CRS format.  Returns the number
// of stored elements, or -1 for an empty sector.
int64_t refh_build_crs_file(int N, int norb, int twoLz, const uint16_t* ktab, const double* vtab, const char* path)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, norb, twoLz, basis)) return -1;
    diagonalization::QuarticTermTables tables;
    tables.Initialize(norb, mpi);
    std::memcpy(tables.GetKTable()->data(), ktab, tables.GetKTable()->size() * sizeof(diagonalization::kState_t));
    std::memcpy(tables.GetVTable()->data(), vtab, tables.GetVTable()->size() * sizeof(double));
    RefHamiltonian H;
    H.SetFockBasis(basis);
    H.Initialize(N, norb, utilities::_SPARSE_MAPPED_, mpi);
    H.Add_CdCdCC_Terms(&tables, 0, H.m_data.m_fockSpaceDim, mpi);
    H.ToCrs(mpi);
    H.m_crsSparseMatrix.ToFile(std::string(path), io::_BINARY_, mpi);
    return (int64_t)H.m_crsSparseMatrix.GetNbrNonZeros();
}

// The reference's two-level basis (two_level_fermion_fock_basis.cpp:289-506):
// dimension, and the (first, second) words when the buffers are given.
uint64_t refh2_basis(int N, int norb0, int twoLz, uint64_t* first, uint64_t* second)
{
    diagonalization::TwoLevelFermionFockBasis basis;
    if (make_basis2(N, norb0, twoLz, basis)) return 0;
    const uint64_t dim = basis.GetStoredDimension();
    if (first && second) {
        std::vector<diagonalization::TwoLevelFockState>::const_iterator it;
        basis.GetFirstState(0, it);
        for (uint64_t i = 0; i < dim; ++i, basis.GetNextState(it)) {
            first[i] = it->m_first;
            second[i] = it->m_second;
        }
    }
    return dim;
}

// The two-level model's Hamiltonian (two_level_pseudopotential_model.cpp:190-215):
// occupation energies of each level (e0: norb0 values, e1: norb0 + 2; either
// may be NULL), then the quartic terms of level 0 and of level 1 from their
// tables, mapped storage, trim, CRS; written to path in the reference's binary
// CRS format.  Returns the stored elements, or -1 for an empty sector.
int64_t refh2_build_crs_file(int N, int norb0, int twoLz, const uint16_t* kt0, const double* vt0, const uint16_t* kt1,
                             const double* vt1, const double* e0, const double* e1, const char* path)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::TwoLevelFermionFockBasis basis;
    if (make_basis2(N, norb0, twoLz, basis)) return -1;
    diagonalization::QuarticTermTables q0, q1;
    q0.Initialize(norb0, mpi);
    q1.Initialize(norb0 + 2, mpi);
    std::memcpy(q0.GetKTable()->data(), kt0, q0.GetKTable()->size() * sizeof(diagonalization::kState_t));
    std::memcpy(q0.GetVTable()->data(), vt0, q0.GetVTable()->size() * sizeof(double));
    std::memcpy(q1.GetKTable()->data(), kt1, q1.GetKTable()->size() * sizeof(diagonalization::kState_t));
    std::memcpy(q1.GetVTable()->data(), vt1, q1.GetVTable()->size() * sizeof(double));
    diagonalization::QuadraticTermTables c0, c1;
    RefTwoLevelHamiltonian H;
    H.SetFockBasis(basis);
    H.Initialize(N, 2 * norb0 + 2, utilities::_SPARSE_MAPPED_, mpi);
    const uint64_t dim = H.m_data.m_fockSpaceDim;
    if (e0) {
        c0.Initialize(norb0, mpi);
        std::memcpy(c0.GetVTable()->data(), e0, sizeof(double) * norb0);
        H.Add_CdC_Terms(&c0, 0, 0, 0, dim, mpi);
    }
    if (e1) {
        c1.Initialize(norb0 + 2, mpi);
        std::memcpy(c1.GetVTable()->data(), e1, sizeof(double) * (norb0 + 2));
        H.Add_CdC_Terms(&c1, 1, 1, 0, dim, mpi);
    }
    H.Add_CdCdCC_Terms(&q0, 0, 0, 0, 0, 0, dim, mpi);
    H.Add_CdCdCC_Terms(&q1, 1, 1, 1, 1, 0, dim, mpi);
    H.ToCrs(mpi);
    H.m_crsSparseMatrix.ToFile(std::string(path), io::_BINARY_, mpi);
    return (int64_t)H.m_crsSparseMatrix.GetNbrNonZeros();
}

// The reference's observables of eigenvector e out of nev given real vectors
// (evecs[i * dim + r], the reference's storage) on the sector basis: density
// (norb), density-density (norb^2) and participation ratio.
int refh_observables(int N, int norb, int twoLz, const double* evecs, int nev, int e, double* density,
                     double* dd, double* pr)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, norb, twoLz, basis)) return -1;
    diagonalization::SpinlessFermionHamiltonian<double> H;
    H.SetFockBasis(basis);
    H.Initialize(N, norb, utilities::_SPARSE_MAPPED_, mpi);
    const uint64_t dim = H.m_data.m_fockSpaceDim;
    H.m_data.m_nbrEigenvalues = nev;
    H.m_eigenvectors.assign(evecs, evecs + dim * (uint64_t)nev);
    H.m_eigenvalues.assign(nev, 0.0);
    H.m_data.m_eigenvectorsCalculated = true;
    diagonalization::Observables obs;
    if (density) obs.DensityFunction(H, e, density, mpi);
    if (dd) obs.DensityDensityFunction(H, e, dd, mpi);
    if (pr) *pr = obs.GetParticipationRatio(H, e, mpi);
    return 0;
}

// The reference's nmost most probable states of each of nev complex vectors
// (evecs_c: (re, im) pairs, [i * dim + r]) with their complex amplitudes
// (states [nev][nmost], amps_c [nev][nmost] as (re, im)).  Only complex
// vectors: for a real Hamiltonian the reference's routine copies
// dcmplx-sized blocks out of its double eigenvector array.
int refh_most_probable_complex(int N, int norb, int twoLz, const double* evecs_c, int nev, int nmost,
                               uint64_t* states, double* amps_c)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, norb, twoLz, basis)) return -1;
    diagonalization::SpinlessFermionHamiltonian<dcmplx> H;
    H.SetFockBasis(basis);
    H.Initialize(N, norb, utilities::_SPARSE_MAPPED_, mpi);
    const uint64_t dim = H.m_data.m_fockSpaceDim;
    H.m_data.m_nbrEigenvalues = nev;
    H.m_eigenvectors.resize(dim * (uint64_t)nev);
    for (uint64_t i = 0; i < dim * (uint64_t)nev; ++i) H.m_eigenvectors[i] = dcmplx(evecs_c[2 * i], evecs_c[2 * i + 1]);
    H.m_eigenvalues.assign(nev, 0.0);
    H.m_data.m_eigenvectorsCalculated = true;
    diagonalization::Observables obs;
    std::vector<dcmplx> a((size_t)nmost * nev);
    obs.GetMostProbable(H, nmost, states, a.data(), mpi);
    for (size_t i = 0; i < a.size(); ++i) {
        amps_c[2 * i] = std::real(a[i]);
        amps_c[2 * i + 1] = std::imag(a[i]);
    }
    return 0;
}

}  // extern "C"
