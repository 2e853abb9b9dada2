// C-ABI shim over the reference's own momentum-sector basis and complex
// Hamiltonian build of the interacting optical-flux-lattice model, so the
// oracle's restatement of them can be pinned against the reference compiled
// from its sources.
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile (target `ref`) into
// oracle/_ref/libref_ofl.so when the reference source tree is present (a
// library of its own: the model's term-table classes share their names with
// the sphere model's).  The reference's files are included from that tree at
// build time; none of their code is copied here.  MPI and Boost come from the
// stand-ins in oracle/ref_stubs/.
//
// Calls follow the model driver
// (optical_flux_lattice/interacting_ofl_model/interacting_ofl_model.cpp:990-1000,
// 1034-1052): FermionFockBasis::GenerateFockSpace with
// std::bind(TestLinearMomentumSector2, _1, kx, ky, dimX, dimY), SetFockBasis,
// Initialize with mapped storage over dimX * dimY orbitals, Add_CdC_Terms and
// Add_CdCdCC_Terms from the array-format tables, then the mapped -> CRS
// conversion and the binary CRS writer.  The hash-table entries follow
// InteractingOflModel::ConvertTableFormat and TermsToFile / TermsFromFile
// (interacting_ofl_model.cpp:597-691) and its hash-format BuildHamiltonian
// branch (:1046-1049).
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include "utilities/general/serialize.hpp"
#include "utilities/general/i_const_def.hpp"
#include "utilities/general/pi_const_def.hpp"
#include "basis/fermion_fock_basis.hpp"
#include "hamiltonians/spinless_fermion_hamiltonian.hpp"
#include "optical_flux_lattice/interacting_ofl_model/linear_momentum_constraints_2D.hpp"
#include "optical_flux_lattice/interacting_ofl_model/term_tables.hpp"
#include "optical_flux_lattice/interacting_ofl_model/term_hash_tables.hpp"

namespace utilities {
Cout cout;
}

namespace {

utilities::MpiWrapper& session()
{
    static utilities::MpiWrapper* mpi = nullptr;
    if (!mpi) {
        mpi = new utilities::MpiWrapper();
        mpi->m_exitFlag = false;   // left unset by its constructor (see ref_ham_shim.cpp)
        char* argv[] = {nullptr};
        mpi->Init(0, argv, true);
        const char* v = std::getenv("ORACLE_REF_VERBOSE");
        utilities::cout.SetVerbosity(v ? std::atoi(v) : 0);
    }
    return *mpi;
}

struct RefComplexHamiltonian : diagonalization::SpinlessFermionHamiltonian<dcmplx> {
    void ToCrs(utilities::MpiWrapper& mpi)
    {
        this->ResetMatrixStorageMethod(utilities::_SPARSE_CRS_, diagonalization::_PARALLEL_, mpi);
    }
};

bool make_basis(int N, int X, int Y, int kx, int ky, diagonalization::FermionFockBasis& basis)
{
    utilities::MpiWrapper& mpi = session();
    return basis.GenerateFockSpace(N, X * Y, std::bind(diagonalization::TestLinearMomentumSector2, std::placeholders::_1,
                                                       (diagonalization::kState_t)kx, (diagonalization::kState_t)ky,
                                                       (diagonalization::kState_t)X, (diagonalization::kState_t)Y),
                                   mpi);
}

// Array tables as the shim's callers pass them (ktab, vtab as (re, im) pairs,
// energies as (re, im) pairs or NULL).
void load_tables(int K, const uint16_t* ktab, const double* vtab, const double* energies,
                 diagonalization::QuarticTermTables& quartic, diagonalization::QuadraticTermTables& quadratic)
{
    utilities::MpiWrapper& mpi = session();
    quartic.Initialize(K, mpi);
    std::memcpy(quartic.GetKTable()->data(), ktab, quartic.GetKTable()->size() * sizeof(diagonalization::kState_t));
    for (size_t i = 0; i < quartic.GetVTable()->size(); ++i)
        (*quartic.GetVTable())[i] = dcmplx(vtab[2 * i], vtab[2 * i + 1]);
    quadratic.Initialize(K, mpi);
    for (int k = 0; k < K; ++k)
        (*quadratic.GetVTable())[k] = energies ? dcmplx(energies[2 * k], energies[2 * k + 1]) : dcmplx(0.0, 0.0);
}

}  // namespace

extern "C" {

// The momentum sector's basis words (fermion_fock_basis.cpp:241-354 with
// linear_momentum_constraints_2D.cpp:38-79); returns the dimension.
uint64_t refo_basis(int N, int X, int Y, int kx, int ky, uint64_t* out)
{
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, X, Y, kx, ky, basis)) return 0;
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

// The reference's hash tables filled from array tables (SetQuarticFromArray,
// SetQuadraticFromArray) and written by its ToFile (binary or text).
int refo_hash_files(int X, int Y, const uint16_t* ktab, const double* vtab, const double* energies,
                    const char* quartic_path, const char* quadratic_path, int binary)
{
    utilities::MpiWrapper& mpi = session();
    const int K = X * Y;
    diagonalization::QuarticTermTables quartic;
    diagonalization::QuadraticTermTables quadratic;
    load_tables(K, ktab, vtab, energies, quartic, quadratic);
    diagonalization::QuarticTermHashTables qh;
    diagonalization::QuadraticTermHashTables dh;
    qh.Initialize(K);
    dh.Initialize(K);
    dh.SetQuadraticFromArray(&quadratic);
    qh.SetQuarticFromArray(&quartic);
    const io::fileFormat_t f = binary ? io::_BINARY_ : io::_TEXT_;
    qh.ToFile(std::string(quartic_path), f, mpi);
    dh.ToFile(std::string(quadratic_path), f, mpi);
    return mpi.m_exitFlag ? 1 : 0;
}

// V(k1, k2, k3, k4) and the k1 count of every (k2, k3, k4) as the reference
// reads them back from its hash-table file (FromFile, GetK1, GetVkkkk):
// k1out[K^3] (the first k1, 65535 where none), nk1[K^3], v[2 K^4] at
// ((k1 K + k2) K + k3) K + k4.  Returns 0 on success.
int refo_hash_read(int K, const char* quartic_path, int binary, uint16_t* k1out, uint32_t* nk1, double* v)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::QuarticTermHashTables qh;
    qh.Initialize(K);
    qh.FromFile(std::string(quartic_path), binary ? io::_BINARY_ : io::_TEXT_, mpi);
    if (mpi.m_exitFlag) return 1;
    std::vector<diagonalization::kState_t> buf(std::max<size_t>(1, qh.GetMaxKCount()) + 8);
    for (int k2 = 0; k2 < K; ++k2)
        for (int k3 = 0; k3 < K; ++k3)
            for (int k4 = 0; k4 < K; ++k4) {
                diagonalization::iSize_t n = 0;
                qh.GetK1(buf.data(), n, k2, k3, k4);
                const size_t i = ((size_t)k2 * K + k3) * K + k4;
                nk1[i] = n;
                k1out[i] = n ? buf[0] : 65535;
            }
    for (int k1 = 0; k1 < K; ++k1)
        for (int k2 = 0; k2 < K; ++k2)
            for (int k3 = 0; k3 < K; ++k3)
                for (int k4 = 0; k4 < K; ++k4) {
                    const dcmplx z = qh.GetVkkkk(k1, k2, k3, k4);
                    const size_t i = (((size_t)k1 * K + k2) * K + k3) * K + k4;
                    v[2 * i] = std::real(z);
                    v[2 * i + 1] = std::imag(z);
                }
    return 0;
}

// The complex Hamiltonian of a momentum sector built from hash-table files
// (FromFile, then the hash-format BuildHamiltonian branch: Add_CdC_Terms and
// Add_CdCdCC_Terms on the hash tables), written to path in the binary CRS
// format.  Returns the stored elements, or -1 for an empty sector.
int64_t refo_build_crs_file_hash(int N, int X, int Y, int kx, int ky, const char* quartic_path,
                                 const char* quadratic_path, int binary, const char* path)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, X, Y, kx, ky, basis)) return -1;
    const int K = X * Y;
    const io::fileFormat_t f = binary ? io::_BINARY_ : io::_TEXT_;
    diagonalization::QuarticTermHashTables qh;
    diagonalization::QuadraticTermHashTables dh;
    qh.Initialize(K);
    dh.Initialize(K);
    qh.FromFile(std::string(quartic_path), f, mpi);
    dh.FromFile(std::string(quadratic_path), f, mpi);
    RefComplexHamiltonian H;
    H.SetFockBasis(basis);
    H.Initialize(N, K, utilities::_SPARSE_MAPPED_, mpi);
    H.Add_CdC_Terms(&dh, 0, H.m_data.m_fockSpaceDim, mpi);
    H.Add_CdCdCC_Terms(&qh, 0, H.m_data.m_fockSpaceDim, mpi);
    H.ToCrs(mpi);
    H.m_crsSparseMatrix.ToFile(std::string(path), io::_BINARY_, mpi);
    return (int64_t)H.m_crsSparseMatrix.GetNbrNonZeros();
}

// The complex Hamiltonian from array-format tables (ktab: (K+1) K^2 / 2 k1
// labels; vtab the same count of (re, im) pairs; energies K (re, im) pairs
// or NULL), K = X * Y orbitals, written to path in the reference's binary CRS
// format.  Returns the stored elements, or -1 for an empty sector.
int64_t refo_build_crs_file(int N, int X, int Y, int kx, int ky, const uint16_t* ktab, const double* vtab,
                            const double* energies, const char* path)
{
    utilities::MpiWrapper& mpi = session();
    diagonalization::FermionFockBasis basis;
    if (make_basis(N, X, Y, kx, ky, basis)) return -1;
    const int K = X * Y;
    diagonalization::QuarticTermTables quartic;
    quartic.Initialize(K, mpi);
    std::memcpy(quartic.GetKTable()->data(), ktab, quartic.GetKTable()->size() * sizeof(diagonalization::kState_t));
    for (size_t i = 0; i < quartic.GetVTable()->size(); ++i)
        (*quartic.GetVTable())[i] = dcmplx(vtab[2 * i], vtab[2 * i + 1]);
    RefComplexHamiltonian H;
    H.SetFockBasis(basis);
    H.Initialize(N, K, utilities::_SPARSE_MAPPED_, mpi);
    diagonalization::QuadraticTermTables quadratic;
    if (energies) {
        quadratic.Initialize(K, mpi);
        for (int k = 0; k < K; ++k) (*quadratic.GetVTable())[k] = dcmplx(energies[2 * k], energies[2 * k + 1]);
        H.Add_CdC_Terms(&quadratic, 0, H.m_data.m_fockSpaceDim, mpi);
    }
    H.Add_CdCdCC_Terms(&quartic, 0, H.m_data.m_fockSpaceDim, mpi);
    H.ToCrs(mpi);
    H.m_crsSparseMatrix.ToFile(std::string(path), io::_BINARY_, mpi);
    return (int64_t)H.m_crsSparseMatrix.GetNbrNonZeros();
}

}  // extern "C"
