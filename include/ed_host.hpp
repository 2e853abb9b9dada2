// ed_host.hpp - C++ host classes with the reference's call surface for the
// exact-diagonalization hot path, implemented over the C ABI (ed_capi.h).
//
// Drop-in names and argument meaning of SimonDavenport/hamiltonian_diagonalization:
//   diagonalization::FermionFockBasis            basis/fermion_fock_basis.hpp:45
//   diagonalization::QuarticTermTables           fqhe_sphere/pseudopotential_model/term_tables.hpp
//   diagonalization::SpinlessFermionHamiltonian  hamiltonians/spinless_fermion_hamiltonian.hpp:52
//   diagonalization::MatrixVectorFunction        hamiltonians/matrix_vector_routines.hpp:41
//   utilities::linearAlgebra::ArpackWrapper      utilities/wrappers/arpack_wrapper.hpp:187
//   utilities::MpiWrapper                        a single-rank stand-in; accepted and ignored
// Differences, all deliberate:
//   - GenerateFockSpace accepts the reference's predicate (e.g.
//     std::bind(&TestAngularMomentumSector, _1, twoLz, maxLz)) but the device
//     enumerates one whole Lz sector: the predicate must select exactly one
//     (found by evaluating it on a few words of every sector, and checked on
//     the words built); a predicate that selects several sectors (the
//     always-true one of a run without block diagonalisation) or splits one
//     is refused.  The overload taking twice Lz directly is kept.
//   - MatrixVectorFunction::Simple takes DEVICE vectors (the Krylov basis
//     lives in HBM).  ArpackWrapper still accepts a host std::function
//     product, called once per product with host vectors.
//   - Failures set mpi.m_exitFlag and print to std::cerr like the reference,
//     and also raise utilities::EdError from the call that failed.
//   - Eigenvalues come back sorted ascending.
// Link with -ledgb300 (hamiltonian_diagonalization_gb300/libedgb300.so).
#pragma once

#include <algorithm>
#include <array>
#include <cstdio>
#include <complex>
#include <cstdint>
#include <functional>
#include <utility>
#include <iostream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "ed_capi.h"

namespace utilities {

typedef uint64_t fock_t;

enum storageMethod_t { _DENSE_ = 0, _SPARSE_MAPPED_ = 1, _SPARSE_CRS_ = 2 };

struct MpiWrapper {
    int m_id = 0;
    int m_nbrProcs = 1;
    bool m_exitFlag = false;
    void ExitFlagTest() const
    {
        if (m_exitFlag) throw std::runtime_error("exit flag set");
    }
};

struct EdError : std::runtime_error {
    ed_status status;
    EdError(ed_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void EdCheck(ed_status s, MpiWrapper* mpi = nullptr)
{
    if (s != ED_OK) {
        std::string msg = std::string(ed_status_string(s)) + ": " + ed_last_error();
        std::cerr << "\n\tERROR: " << msg << std::endl;
        if (mpi) mpi->m_exitFlag = true;
        throw EdError(s, msg);
    }
}

}  // namespace utilities

// utilities/wrappers/io_wrapper.hpp:24
namespace io {
enum fileFormat_t { _TEXT_ = 0, _BINARY_ = 1 };
}

namespace diagonalization {

using utilities::fock_t;
typedef uint32_t iSize_t;
typedef uint16_t kState_t;
typedef int16_t mState_t;

// Quartic term tables: kTable[(k4*K+k3)*K+k2] = k1, vTable[...] = V_{k1k2k3k4}.
class QuarticTermTables {
  public:
    QuarticTermTables() = default;
    QuarticTermTables(const QuarticTermTables&) = delete;
    QuarticTermTables& operator=(const QuarticTermTables&) = delete;
    ~QuarticTermTables() { if (m_h) ed_terms_free(m_h); }

    // BaseGenerate4KTable + BaseTermsFromPseudopotentials for one Landau level
    void Initialize(iSize_t nbrOrbitals, const std::vector<double>& pseudopotentials)
    {
        m_kMax = nbrOrbitals;
        const size_t K3 = (size_t)m_kMax * m_kMax * m_kMax;
        m_kTable.assign(K3, 0);
        m_vTable.assign(K3, 0.0);
        utilities::EdCheck(ed_quartic_tables((int)m_kMax, pseudopotentials.data(), (int)pseudopotentials.size(),
                                             m_kTable.data(), m_vTable.data()));
        Reset();
    }
    // Tables supplied by the caller (e.g. read from a file)
    void SetTables(iSize_t nbrOrbitals, const std::vector<kState_t>& kTable, const std::vector<double>& vTable)
    {
        m_kMax = nbrOrbitals;
        m_kTable = kTable;
        m_vTable = vTable;
        Reset();
    }
    iSize_t GetMaxKCount() const { return 1; }
    void GetK1(kState_t* buf, iSize_t& nbrK1, kState_t k2, kState_t k3, kState_t k4) const
    {
        nbrK1 = 1;
        buf[0] = m_kTable[((size_t)k4 * m_kMax + k3) * m_kMax + k2];
        if (buf[0] >= m_kMax) nbrK1 = 0;
    }
    double GetVkkkk(kState_t, kState_t k2, kState_t k3, kState_t k4) const
    {
        return m_vTable[((size_t)k4 * m_kMax + k3) * m_kMax + k2];
    }
    iSize_t GetKMax() const { return m_kMax; }
    ed_terms* handle()
    {
        if (!m_h) utilities::EdCheck(ed_terms_set((int)m_kMax, m_kTable.data(), m_vTable.data(), &m_h));
        return m_h;
    }

  private:
    void Reset()
    {
        if (m_h) ed_terms_free(m_h);
        m_h = nullptr;
    }
    iSize_t m_kMax = 0;
    std::vector<kState_t> m_kTable;
    std::vector<double> m_vTable;
    ed_terms* m_h = nullptr;
};

// angular_momentum_constraint.hpp:41-62: the Lz of a word (twice units, orbital
// k at 2k - max) equals lzTot.  The predicate the reference binds into
// GenerateFockSpace; GenerateFockSpace below recognises the sector it selects.
inline bool TestAngularMomentumSector(const fock_t state, const mState_t lzTot, const mState_t max)
{
    int lz = 0;
    for (fock_t t = state; t; t &= t - 1) {
        int k = 0;
        while (!((t >> k) & 1u)) ++k;
        lz += 2 * k - max;
    }
    return lz == lzTot;
}

class FermionFockBasis {
  public:
    FermionFockBasis() = default;
    // A copy is the same sector built again on the device (the reference's
    // SetFockBasis takes the basis by const reference and copies it).
    FermionFockBasis(const FermionFockBasis& o) { CopyFrom(o); }
    FermionFockBasis& operator=(const FermionFockBasis& o)
    {
        if (this != &o) CopyFrom(o);
        return *this;
    }
    FermionFockBasis(FermionFockBasis&& o) noexcept
        : m_basisStored(o.m_basisStored), m_h(o.m_h), m_kind(o.m_kind), m_par(o.m_par)
    {
        o.m_h = nullptr;
    }
    FermionFockBasis& operator=(FermionFockBasis&& o) noexcept
    {
        if (this != &o) {
            if (m_h) ed_basis_free(m_h);
            m_h = o.m_h;
            m_basisStored = o.m_basisStored;
            m_kind = o.m_kind;
            m_par = o.m_par;
            o.m_h = nullptr;
        }
        return *this;
    }
    ~FermionFockBasis() { if (m_h) ed_basis_free(m_h); }

    // fermion_fock_basis.cpp:241 with the reference's predicate argument: the
    // Lz sector the predicate selects (see the header notes); true when empty
    bool GenerateFockSpace(iSize_t nbrParticles, iSize_t nbrOrbitals, const std::function<bool(const fock_t)>& inSector,
                           utilities::MpiWrapper& mpi)
    {
        const int N = (int)nbrParticles, K = (int)nbrOrbitals;
        if (N < 1 || K < N || K > 64) {
            std::cerr << "\n\tERROR in GenerateFockSpace: bad particle/orbital numbers" << std::endl;
            mpi.m_exitFlag = true;
            throw utilities::EdError(ED_ERR_ARG, "bad particle/orbital numbers");
        }
        // position sums S of the N-particle words; 2Lz = 2S - N (K - 1)
        const int smin = N * (N - 1) / 2, smax = N * (2 * K - N - 1) / 2;
        std::vector<int> chosen;
        for (int S = smin; S <= smax; ++S) {
            int yes = 0, tried = 0;
            for (fock_t w : SectorWords(N, K, S)) {
                ++tried;
                yes += inSector(w) ? 1 : 0;
            }
            if (yes != 0 && yes != tried) Refuse(mpi, "the predicate splits an Lz sector; the device builds whole sectors");
            if (yes) chosen.push_back(S);
        }
        if (chosen.size() > 1)
            Refuse(mpi, "the predicate selects several Lz sectors; the device basis holds one (pass one sector)");
        if (chosen.empty()) {
            if (m_h) ed_basis_free(m_h);
            m_h = nullptr;
            m_basisStored = true;
            return true;
        }
        const bool empty = GenerateFockSpace(nbrParticles, nbrOrbitals, 2 * chosen[0] - N * (K - 1), mpi);
        // the words built satisfy the predicate (every word, or an even sample of 100,000)
        const fock_t n = GetStoredDimension();
        std::vector<fock_t> w(n);
        if (n) GetFockBasis(w.data(), n, mpi);
        const fock_t step = n > 100000 ? n / 100000 : 1;
        for (fock_t i = 0; i < n; i += step)
            if (!inSector(w[i])) Refuse(mpi, "a word of the selected sector fails the predicate");
        return empty;
    }

    // the optical-flux-lattice momentum sector: GenerateFockSpace with
    // TestLinearMomentumSector2 (interacting_ofl_model.cpp:994-1001); true when empty
    bool GenerateFockSpaceMomentum(iSize_t nbrParticles, iSize_t dimX, iSize_t dimY, iSize_t kxTot, iSize_t kyTot,
                                   utilities::MpiWrapper& mpi)
    {
        if (m_h) ed_basis_free(m_h);
        m_h = nullptr;
        utilities::EdCheck(ed_basis_momentum_build((int)nbrParticles, (int)dimX, (int)dimY, (int)kxTot, (int)kyTot,
                                                   nullptr, &m_h),
                           &mpi);
        m_basisStored = true;
        m_kind = 2;
        m_par = {(int)nbrParticles, (int)dimX, (int)dimY, (int)kxTot, (int)kyTot};
        return GetStoredDimension() == 0;
    }

    // fermion_fock_basis.cpp:241: returns true when the sector is empty
    bool GenerateFockSpace(iSize_t nbrParticles, iSize_t nbrOrbitals, int twoLz, utilities::MpiWrapper& mpi)
    {
        if (m_h) ed_basis_free(m_h);
        m_h = nullptr;
        utilities::EdCheck(ed_basis_build((int)nbrParticles, (int)nbrOrbitals, twoLz, nullptr, &m_h), &mpi);
        m_basisStored = true;
        m_kind = 1;
        m_par = {(int)nbrParticles, (int)nbrOrbitals, twoLz, 0, 0};
        return GetStoredDimension() == 0;
    }
    iSize_t NbrParticles() const { return m_kind ? (iSize_t)m_par[0] : 0; }
    // the momentum grid of a momentum sector (0 for other bases)
    iSize_t DimX() const { return m_kind == 2 ? (iSize_t)m_par[1] : 0; }
    iSize_t DimY() const { return m_kind == 2 ? (iSize_t)m_par[2] : 0; }
    iSize_t NbrOrbitals() const { return m_kind == 1 ? (iSize_t)m_par[1] : m_kind == 2 ? (iSize_t)(m_par[1] * m_par[2]) : 0; }
    fock_t GetStoredDimension() const
    {
        uint64_t d = 0;
        if (m_h) utilities::EdCheck(ed_basis_dim(m_h, &d));
        return d;
    }
    // fermion_fock_basis.cpp:134: UINT64_MAX when absent
    fock_t FindFockStateIndex(fock_t offset, fock_t state) const
    {
        uint64_t idx = 0;
        utilities::EdCheck(ed_basis_rank_host(m_h, &state, &idx, 1));
        return idx == ~0ull ? idx : idx + offset;
    }
    void FindFockStateIndices(const fock_t* states, fock_t* idx, fock_t m) const
    {
        utilities::EdCheck(ed_basis_rank_host(m_h, states, idx, m));
    }
    // fermion_fock_basis.cpp:359
    void GetFockBasis(fock_t* buffer, fock_t dim, utilities::MpiWrapper& mpi) const
    {
        utilities::EdCheck(ed_basis_get(m_h, buffer, dim), &mpi);
    }
    ed_basis* handle() const { return m_h; }
    bool m_basisStored = false;

  private:
    // Up to three words of N particles among K orbitals whose positions sum to
    // S: the lowest positions with the excess taken by the highest particles,
    // the highest positions with the deficit taken by the lowest, and a
    // seeded walk of sum-preserving moves from the first.
    static std::vector<fock_t> SectorWords(int N, int K, int S)
    {
        std::vector<fock_t> out;
        std::vector<int> lo(N), hi(N);
        for (int i = 0; i < N; ++i) { lo[i] = i; hi[i] = K - N + i; }
        int excess = S - N * (N - 1) / 2;
        for (int i = N - 1; i >= 0 && excess > 0; --i) {
            const int room = (K - N + i) - lo[i];
            const int d = room < excess ? room : excess;
            lo[i] += d;
            excess -= d;
        }
        int deficit = N * (2 * K - N - 1) / 2 - S;
        for (int i = 0; i < N && deficit > 0; ++i) {
            const int room = hi[i] - i;
            const int d = room < deficit ? room : deficit;
            hi[i] -= d;
            deficit -= d;
        }
        auto word = [](const std::vector<int>& p) {
            fock_t w = 0;
            for (int q : p) w |= (fock_t)1 << q;
            return w;
        };
        out.push_back(word(lo));
        if (word(hi) != out[0]) out.push_back(word(hi));
        std::vector<int> p = lo;
        uint64_t r = 0x9E3779B97F4A7C15ull ^ (uint64_t)S;
        for (int t = 0; t < 64 * N; ++t) {   // move one particle up and another down by one
            r ^= r << 13; r ^= r >> 7; r ^= r << 17;
            const int a = (int)(r % (uint64_t)N), b = (int)((r >> 20) % (uint64_t)N);
            if (a == b) continue;
            const int up = p[a] + 1, down = p[b] - 1;
            if (up >= K || down < 0 || up == down) continue;
            bool clash = false;
            for (int i = 0; i < N; ++i)
                if (i != a && i != b && (p[i] == up || p[i] == down)) clash = true;
            if (clash || up == p[b] || down == p[a]) continue;
            p[a] = up;
            p[b] = down;
        }
        const fock_t wm = word(p);
        if (wm != out[0] && (out.size() < 2 || wm != out[1])) out.push_back(wm);
        return out;
    }
    void Refuse(utilities::MpiWrapper& mpi, const char* why)
    {
        std::cerr << "\n\tERROR in GenerateFockSpace: " << why << std::endl;
        mpi.m_exitFlag = true;
        throw utilities::EdError(ED_ERR_ARG, why);
    }
    void CopyFrom(const FermionFockBasis& o)
    {
        utilities::MpiWrapper mpi;
        if (m_h) ed_basis_free(m_h);
        m_h = nullptr;
        m_kind = 0;
        m_basisStored = o.m_basisStored;
        if (o.m_kind == 1 && o.m_h) GenerateFockSpace(o.m_par[0], o.m_par[1], o.m_par[2], mpi);
        else if (o.m_kind == 2 && o.m_h) GenerateFockSpaceMomentum(o.m_par[0], o.m_par[1], o.m_par[2], o.m_par[3], o.m_par[4], mpi);
        m_basisStored = o.m_basisStored;
    }
    ed_basis* m_h = nullptr;
    int m_kind = 0;                           // 0 none, 1 Lz sector, 2 momentum sector
    std::array<int, 5> m_par{};               // the generation parameters
};

template <typename T>
class SpinlessFermionHamiltonian;

template <typename T, class L1 = QuarticTermTables, class L2 = QuarticTermTables>
class MatrixVectorFunction {
  public:
    MatrixVectorFunction(SpinlessFermionHamiltonian<T>& hamiltonian, const utilities::MpiWrapper&)
        : hamiltonian(&hamiltonian) {}
    // matrix_vector_routines.hpp:94: y = H x on device vectors of the sector dimension
    void Simple(T* x, T* y, const utilities::MpiWrapper&) { hamiltonian->Apply(x, y); }
    SpinlessFermionHamiltonian<T>* hamiltonian;
};

namespace detail {
inline void host_trampoline(const double* x, double* y, void* user)
{
    auto* fn = static_cast<std::function<void(double*, double*, utilities::MpiWrapper&)>*>(user);
    utilities::MpiWrapper mpi;
    (*fn)(const_cast<double*>(x), y, mpi);
}
}  // namespace detail

}  // namespace diagonalization

namespace utilities {
namespace linearAlgebra {

class ArpackWrapper {
  public:
    ArpackWrapper() = default;
    void SetMaxIterations(int maxIterations) { m_maxIterations = maxIterations; }
    void SetTolerance(double tol) { m_tol = tol; }
    void SetNcv(int ncv) { m_ncv = ncv; }
    void SetSeed(uint64_t seed) { m_seed = seed; }
    // further deflated solves that recover copies of degenerate eigenvalues
    void SetDegeneracyPasses(int passes) { m_degeneracyPasses = passes; }
    // a stored matrix with no off-diagonal element is solved from its
    // diagonal (HamiltonianBase::MatrixDiagonalCheck and its shortcut,
    // hamiltonian_base.hpp:378-449, 803-850); the Hamiltonian classes turn
    // it on, as the reference's LanczosDiagonalize does the check
    void SetDiagonalCheck(bool check) { m_diagonalCheck = check; }
    // start vector (host, nodeDim doubles) in place of --use-initial's file
    void SetInitialVector(const std::vector<double>& v) { m_initial = v; }
    // arpack_wrapper.hpp: --use-initial reads the start vector (raw FP64,
    // nodeDim values) from the initial-vector file; --store-final writes the
    // final vector there (here the lowest eigenvector, a restart vector)
    void SetUseInitial(bool use) { m_useInitial = use; }
    void SetStoreFinal(bool store) { m_storeFinal = store; }
    void SetInitialVectorFile(const std::string& name) { m_initialFile = name; }
    void SetFinalVectorFile(const std::string& name) { m_finalFile = name; }
    const ed_solve_info& LastInfo() const { return m_info; }

    // arpack_wrapper.hpp:595: generic host product (std::function form)
    template <typename T>
    bool DiagonalizeSymmetricMatrix(const std::function<void(T*, T*, MpiWrapper&)>& MatrixVectorMultiply,
                                    T* eigenvectors, double* eigenvalues, int nodeDim, int fullDim, int nbrEigenvalues,
                                    MpiWrapper& mpi)
    {
        static_assert(sizeof(T) == sizeof(double), "real FP64 only");
        if (nodeDim != fullDim) return Fail(ED_ERR_ARG, "one device holds the whole vector", mpi);
        std::function<void(double*, double*, MpiWrapper&)> fn = MatrixVectorMultiply;
        ed_op* op = nullptr;
        ed_status s = ed_op_host_callback(fullDim, &diagonalization::detail::host_trampoline, &fn, &op);
        if (s != ED_OK) return Fail(s, ed_last_error(), mpi);
        const bool ok = Run(op, eigenvectors, eigenvalues, fullDim, nbrEigenvalues, mpi);
        ed_op_free(op);
        return ok;
    }

    // the device product of a built Hamiltonian (the fast path)
    template <typename T, class L1, class L2>
    bool DiagonalizeSymmetricMatrix(diagonalization::MatrixVectorFunction<T, L1, L2>& mv, T* eigenvectors,
                                    double* eigenvalues, int nodeDim, int fullDim, int nbrEigenvalues, MpiWrapper& mpi)
    {
        if (nodeDim != fullDim) return Fail(ED_ERR_ARG, "one device holds the whole vector", mpi);
        ed_op* op = mv.hamiltonian->MakeOperator();
        const bool ok = Run(op, eigenvectors, eigenvalues, fullDim, nbrEigenvalues, mpi);
        ed_op_free(op);
        return ok;
    }

    // any engine operator (a two-level Hamiltonian's, for one)
    bool DiagonalizeOperator(ed_op* op, double* eigenvectors, double* eigenvalues, int fullDim, int nbrEigenvalues,
                             MpiWrapper& mpi)
    {
        return Run(op, eigenvectors, eigenvalues, fullDim, nbrEigenvalues, mpi);
    }

  private:
    bool Fail(ed_status s, const std::string& msg, MpiWrapper& mpi)
    {
        std::cerr << "\n\tERROR in DiagonalizeSymmetricMatrix: " << ed_status_string(s) << ": " << msg << std::endl;
        mpi.m_exitFlag = true;
        m_status = s;
        return false;
    }
    bool Run(ed_op* op, double* eigenvectors, double* eigenvalues, int n, int nev, MpiWrapper& mpi)
    {
        ed_lanczos_params p{};
        p.nev = nev;
        p.ncv = m_ncv;
        p.max_restarts = m_maxIterations;
        p.tol = m_tol;
        p.seed = m_seed;
        p.want_vectors = eigenvectors != nullptr;
        p.verify = 1;
        p.degeneracy_passes = m_degeneracyPasses;
        p.diagonal_check = m_diagonalCheck ? 1 : 0;
        if (m_useInitial && !m_initialFile.empty()) {
            std::vector<double> v(n);
            FILE* f = std::fopen(m_initialFile.c_str(), "rb");
            const bool read = f && std::fread(v.data(), sizeof(double), (size_t)n, f) == (size_t)n;
            if (f) std::fclose(f);
            if (!read) return Fail(ED_ERR_ARG, "cannot read " + std::to_string(n) + " values from " + m_initialFile, mpi);
            m_initial = v;
        }
        const double* v0 = ((int)m_initial.size() == n) ? m_initial.data() : nullptr;
        ed_status s = ed_lanczos(op, &p, v0, eigenvalues, eigenvectors, &m_info);
        m_status = s;
        if (s != ED_OK) return Fail(s, ed_last_error(), mpi);
        if (m_storeFinal && !m_finalFile.empty() && eigenvectors) {
            FILE* f = std::fopen(m_finalFile.c_str(), "wb");
            const bool wrote = f && std::fwrite(eigenvectors, sizeof(double), (size_t)n, f) == (size_t)n;
            if (f) std::fclose(f);
            if (!wrote) return Fail(ED_ERR_ARG, "cannot write " + m_finalFile, mpi);
        }
        return true;
    }
    int m_maxIterations = 2000;
    int m_degeneracyPasses = 0;
    bool m_diagonalCheck = false;
    int m_ncv = 0;
    double m_tol = 1e-10;
    uint64_t m_seed = 0;
    std::vector<double> m_initial;
    bool m_useInitial = false, m_storeFinal = false;
    std::string m_initialFile, m_finalFile;
    ed_solve_info m_info{};
    ed_status m_status = ED_OK;
};

}  // namespace linearAlgebra
}  // namespace utilities

namespace diagonalization {

template <typename T>
class SpinlessFermionHamiltonian {
    static_assert(sizeof(T) == sizeof(double), "the device path is real FP64");

  public:
    SpinlessFermionHamiltonian() = default;
    SpinlessFermionHamiltonian(const SpinlessFermionHamiltonian&) = delete;
    SpinlessFermionHamiltonian& operator=(const SpinlessFermionHamiltonian&) = delete;
    ~SpinlessFermionHamiltonian() { Clear(); }

    // hamiltonian_base.hpp:597
    void SetFockBasis(const FermionFockBasis& fockBasis) { m_fockBasis = fockBasis; }
    void SetFockBasis(FermionFockBasis&& fockBasis) { m_fockBasis = std::move(fockBasis); }

    // spinless_fermion_hamiltonian.hpp:59, after SetFockBasis (the reference's
    // model sequence): the basis set must hold nbrParticles in nbrOrbitals
    void Initialize(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::storageMethod_t storageMethod,
                    utilities::MpiWrapper& mpi)
    {
        CheckNumbers(nbrParticles, nbrOrbitals, mpi);
        if (!m_fockBasis.handle() || m_fockBasis.NbrParticles() != nbrParticles ||
            m_fockBasis.NbrOrbitals() != nbrOrbitals) {
            std::cerr << "\n\tERROR: set a Fock basis of these particle/orbital numbers first" << std::endl;
            mpi.m_exitFlag = true;
            throw utilities::EdError(ED_ERR_ARG, "SetFockBasis before Initialize (or pass the sector)");
        }
        SetData(nbrParticles, nbrOrbitals, storageMethod);
    }
    // the same with the sector given (twice Lz): the basis is built here
    void Initialize(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::storageMethod_t storageMethod,
                    utilities::MpiWrapper& mpi, int twoLz)
    {
        CheckNumbers(nbrParticles, nbrOrbitals, mpi);
        m_fockBasis.GenerateFockSpace(nbrParticles, nbrOrbitals, twoLz, mpi);
        SetData(nbrParticles, nbrOrbitals, storageMethod);
    }
    // spinless_fermion_hamiltonian.hpp:282.  The whole sector is built in one
    // device call; minRow/maxRow are accepted for signature compatibility.
    template <class L>
    void Add_CdCdCC_Terms(L* termTables, fock_t /*minRow*/, fock_t /*maxRow*/, utilities::MpiWrapper& mpi,
                          bool storeUpper = false)
    {
        if (m_crs) ed_crs_free(m_crs);
        m_crs = nullptr;
        m_terms = termTables;
        utilities::EdCheck(ed_ham_build_crs(m_fockBasis.handle(), termTables->handle(), storeUpper ? 1 : 0, nullptr,
                                            &m_crs),
                           &mpi);
    }
    // regenerate elements on the fly instead of storing them
    template <class L>
    void SetMatrixFree(L* termTables)
    {
        if (m_crs) ed_crs_free(m_crs);
        m_crs = nullptr;
        m_terms = termTables;
    }
    fock_t GetFockSpaceDimension() const { return m_fockBasis.GetStoredDimension(); }
    int64_t GetNbrNonZeros() const
    {
        int64_t nnz = 0;
        if (m_crs) utilities::EdCheck(ed_crs_info(m_crs, nullptr, &nnz, nullptr));
        return nnz;
    }
    void GetCrs(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& data) const
    {
        int64_t n = 0, nnz = 0;
        utilities::EdCheck(ed_crs_info(m_crs, &n, &nnz, nullptr));
        rowStarts.resize(n + 1);
        cols.resize(nnz);
        data.resize(nnz);
        utilities::EdCheck(ed_crs_get(m_crs, rowStarts.data(), cols.data(), data.data()));
    }
    void Apply(const double* x_dev, double* y_dev)
    {
        if (m_crs) utilities::EdCheck(ed_spmv(m_crs, x_dev, y_dev, nullptr));
        else utilities::EdCheck(ed_hv_matfree(m_fockBasis.handle(), m_terms->handle(), x_dev, y_dev, nullptr));
    }
    ed_op* MakeOperator()
    {
        ed_op* op = nullptr;
        if (m_crs) utilities::EdCheck(ed_op_from_crs(m_crs, &op));
        else utilities::EdCheck(ed_op_matfree(m_fockBasis.handle(), m_terms->handle(), &op));
        return op;
    }
    // hamiltonian_base.hpp:770, the reference's call shape: the product of mv
    // (this Hamiltonian's), the table arguments accepted as the reference
    // passes them; eigenvalues ascending, eigenvectors n x nev column-major
    template <class L1, class L2>
    bool LanczosDiagonalize(L1* /*quadraticLookUpTables*/, L2* /*quarticLookUpTables*/,
                            MatrixVectorFunction<T, L1, L2>& mv, iSize_t& nbrEigenvalues, utilities::MpiWrapper& mpi)
    {
        SetNbrEigenvalues(nbrEigenvalues, mpi);
        nbrEigenvalues = m_data.m_nbrEigenvalues;
        const fock_t n = GetFockSpaceDimension();
        m_eigenvalues.assign(nbrEigenvalues, 0.0);
        m_eigenvectors.assign((size_t)n * nbrEigenvalues, 0.0);
        m_arpackWrapper.SetDiagonalCheck(true);
        const bool ok = m_arpackWrapper.DiagonalizeSymmetricMatrix(mv, m_eigenvectors.data(), m_eigenvalues.data(),
                                                                   (int)n, (int)n, (int)nbrEigenvalues, mpi);
        m_data.m_eigenvectorsCalculated = ok;
        return ok;
    }
    // the same with the tolerance and vectors as arguments
    bool LanczosDiagonalize(iSize_t nbrEigenvalues, utilities::MpiWrapper& mpi, double tol = 1e-10,
                            bool wantVectors = true)
    {
        const fock_t n = GetFockSpaceDimension();
        m_eigenvalues.assign(nbrEigenvalues, 0.0);
        m_eigenvectors.assign(wantVectors ? (size_t)n * nbrEigenvalues : 0, 0.0);
        MatrixVectorFunction<T> mv(*this, mpi);
        m_arpackWrapper.SetTolerance(tol);
        m_arpackWrapper.SetDiagonalCheck(true);
        const bool ok = m_arpackWrapper.DiagonalizeSymmetricMatrix(mv, wantVectors ? m_eigenvectors.data() : nullptr,
                                                                   m_eigenvalues.data(), (int)n, (int)n,
                                                                   (int)nbrEigenvalues, mpi);
        m_data.m_nbrEigenvalues = nbrEigenvalues;
        m_data.m_eigenvectorsCalculated = ok && wantVectors;
        return ok;
    }
    // hamiltonian_base.hpp:634-758: every eigenpair of the dense matrix (the
    // reference's choice below dimension 60), the lowest nbrEigenvalues kept
    bool FullDiagonalize(iSize_t& nbrEigenvalues, utilities::MpiWrapper& mpi)
    {
        SetNbrEigenvalues(nbrEigenvalues, mpi);
        nbrEigenvalues = m_data.m_nbrEigenvalues;
        const fock_t n = GetFockSpaceDimension();
        if (n > 20000) {
            std::cerr << "\n\tERROR in FullDiagonalize: dimension too large for a dense solve" << std::endl;
            mpi.m_exitFlag = true;
            return false;
        }
        std::vector<int64_t> rs;
        std::vector<int32_t> cs;
        std::vector<double> vs;
        GetCrs(rs, cs, vs);
        int upper = 0;
        utilities::EdCheck(ed_crs_info(m_crs, nullptr, nullptr, &upper), &mpi);
        std::vector<double> dense((size_t)n * n, 0.0), w(n), z((size_t)n * n);
        for (fock_t i = 0; i < n; ++i)
            for (int64_t k = rs[i]; k < rs[i + 1]; ++k) {
                dense[(size_t)i * n + cs[k]] = vs[k];
                if (upper) dense[(size_t)cs[k] * n + i] = vs[k];
            }
        utilities::EdCheck(ed_dense_sym_eigen((int)n, dense.data(), w.data(), z.data()), &mpi);
        m_eigenvalues.assign(w.begin(), w.begin() + nbrEigenvalues);
        m_eigenvectors.assign(z.begin(), z.begin() + (size_t)n * nbrEigenvalues);
        m_data.m_eigenvectorsCalculated = true;
        return true;
    }
    // hamiltonian_base.hpp:568-594 (the ARPACK vector files of one run)
    void UpdateArpackFileNames(const std::string& inFileName, const std::string& outFileName,
                               utilities::MpiWrapper&)
    {
        m_arpackWrapper.SetInitialVectorFile(inFileName);
        m_arpackWrapper.SetFinalVectorFile(outFileName);
    }
    // hamiltonian_base.hpp:603
    void SetNbrEigenvalues(iSize_t nbrEigenvalues, const utilities::MpiWrapper&)
    {
        const fock_t n = GetFockSpaceDimension();
        m_data.m_nbrEigenvalues = nbrEigenvalues > n ? (iSize_t)n : nbrEigenvalues;
    }
    void Clear()
    {
        if (m_crs) ed_crs_free(m_crs);
        m_crs = nullptr;
    }

    // hamiltonian_data.hpp: the fields the reference's callers read
    struct HamiltonianData {
        iSize_t m_nbrParticles = 0, m_nbrOrbitals = 0, m_nbrEigenvalues = 0;
        fock_t m_fockSpaceDim = 0;
        utilities::storageMethod_t m_storageMethod = utilities::_SPARSE_CRS_;
        bool m_eigenvectorsCalculated = false;
    } m_data;
    FermionFockBasis m_fockBasis;
    utilities::linearAlgebra::ArpackWrapper m_arpackWrapper;
    std::vector<double> m_eigenvalues;
    std::vector<double> m_eigenvectors;   // column-major n x nev

  private:
    void CheckNumbers(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::MpiWrapper& mpi)
    {
        if (nbrParticles == 0 || nbrOrbitals == 0 || nbrParticles >= 64 || nbrParticles > nbrOrbitals) {
            std::cerr << "\n\tERROR: bad particle/orbital numbers" << std::endl;
            mpi.m_exitFlag = true;
            throw utilities::EdError(ED_ERR_ARG, "bad particle/orbital numbers");
        }
    }
    void SetData(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::storageMethod_t storageMethod)
    {
        m_data.m_nbrParticles = nbrParticles;
        m_data.m_nbrOrbitals = nbrOrbitals;
        m_data.m_storageMethod = storageMethod;
        m_data.m_fockSpaceDim = m_fockBasis.GetStoredDimension();
        m_data.m_eigenvectorsCalculated = false;
    }
    ed_crs* m_crs = nullptr;
    QuarticTermTables* m_terms = nullptr;
};

// term_tables.hpp QuadraticTermTables as the two-level model fills it: one
// occupation energy per orbital of a level (GetVTable()->data(), length
// GetDimension()).
class QuadraticTermTables {
  public:
    void Initialize(iSize_t nbrOrbitals, const utilities::MpiWrapper&) { m_vTable.assign(nbrOrbitals, 0.0); }
    std::vector<double>* GetVTable() { return &m_vTable; }
    const std::vector<double>* GetVTable() const { return &m_vTable; }
    iSize_t GetDimension() const { return (iSize_t)m_vTable.size(); }

  private:
    std::vector<double> m_vTable;
};

// two_level_fermion_fock_basis.hpp:62.  A state (first, second) is stored on
// the device as one word (first << nbrOrbitals2) | second; the ascending order
// of those words is the reference's (first, second) sort.
class TwoLevelFermionFockBasis {
  public:
    TwoLevelFermionFockBasis() = default;
    TwoLevelFermionFockBasis(const TwoLevelFermionFockBasis&) = delete;
    TwoLevelFermionFockBasis& operator=(const TwoLevelFermionFockBasis&) = delete;
    ~TwoLevelFermionFockBasis() { if (m_h) ed_basis_free(m_h); }

    // two_level_fermion_fock_basis.cpp:289 with TestAngularMomentumSector2LL
    // for the sector twoLz; returns true when the sector is empty
    bool GenerateFockSpace(iSize_t nbrParticles, iSize_t nbrOrbitals1, iSize_t nbrOrbitals2, int twoLz,
                           utilities::MpiWrapper& mpi)
    {
        if (nbrOrbitals2 != nbrOrbitals1 + 2)
            throw utilities::EdError(ED_ERR_ARG, "the second level has nbrOrbitals1 + 2 orbitals on the sphere");
        if (m_h) ed_basis_free(m_h);
        m_h = nullptr;
        utilities::EdCheck(ed_basis2_build((int)nbrParticles, (int)nbrOrbitals1, twoLz, nullptr, &m_h), &mpi);
        m_nbrOrbitals2 = nbrOrbitals2;
        m_basisStored = true;
        return GetStoredDimension() == 0;
    }
    fock_t GetStoredDimension() const
    {
        uint64_t d = 0;
        if (m_h) utilities::EdCheck(ed_basis_dim(m_h, &d));
        return d;
    }
    // two_level_fermion_fock_basis.cpp:211: UINT64_MAX when absent
    void FindFockStateIndex(fock_t offset, fock_t first, fock_t second, fock_t& index) const
    {
        const uint64_t word = (first << m_nbrOrbitals2) | second;
        uint64_t idx = 0;
        utilities::EdCheck(ed_basis_rank_host(m_h, &word, &idx, 1));
        index = idx == ~0ull ? idx : idx + offset;
    }
    // two_level_fermion_fock_basis.cpp:477
    void GetFockBasis(fock_t* buffer1, fock_t* buffer2, fock_t dim, utilities::MpiWrapper& mpi) const
    {
        std::vector<uint64_t> w(dim);
        utilities::EdCheck(ed_basis_get(m_h, w.data(), dim), &mpi);
        const uint64_t mask = (1ull << m_nbrOrbitals2) - 1ull;
        for (fock_t i = 0; i < dim; ++i) {
            buffer1[i] = w[i] >> m_nbrOrbitals2;
            buffer2[i] = w[i] & mask;
        }
    }
    ed_basis* handle() const { return m_h; }
    bool m_basisStored = false;

  private:
    ed_basis* m_h = nullptr;
    iSize_t m_nbrOrbitals2 = 0;
};

// two_level_spinless_fermion_hamiltonian.hpp:52 for T = double, driven as
// SphereTwoLevelPseudopotentialModel::BuildHamiltonian does
// (two_level_pseudopotential_model.cpp:190-215).  Add_CdC_Terms and
// Add_CdCdCC_Terms record each level's tables (terms within one level only,
// as in the reference); the device build runs once, at the first product or
// solve, and sums each entry in that call order.
template <typename T>
class TwoLevelSpinlessFermionHamiltonian {
    static_assert(sizeof(T) == sizeof(double), "the device path is real FP64");

  public:
    TwoLevelSpinlessFermionHamiltonian() = default;
    TwoLevelSpinlessFermionHamiltonian(const TwoLevelSpinlessFermionHamiltonian&) = delete;
    TwoLevelSpinlessFermionHamiltonian& operator=(const TwoLevelSpinlessFermionHamiltonian&) = delete;
    ~TwoLevelSpinlessFermionHamiltonian() { Clear(); }

    // nbrOrbitals = 2 (2S+1) + 2, both levels (two_level_pseudopotential_model.cpp:73)
    void Initialize(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::storageMethod_t storageMethod,
                    utilities::MpiWrapper& mpi, int twoLz = 0)
    {
        if (nbrParticles == 0 || nbrOrbitals < 4 || nbrOrbitals % 2) {
            mpi.m_exitFlag = true;
            throw utilities::EdError(ED_ERR_ARG, "need nbrParticles > 0 and nbrOrbitals = 2 * norb0 + 2");
        }
        m_norb0 = (nbrOrbitals - 2) / 2;
        m_storageMethod = storageMethod;
        m_fockBasis.GenerateFockSpace(nbrParticles, m_norb0, m_norb0 + 2, twoLz, mpi);
    }
    // two_level_spinless_fermion_hamiltonian.hpp:147
    void Add_CdC_Terms(QuadraticTermTables* tables, iSize_t level1, iSize_t level2, fock_t /*minRow*/,
                       fock_t /*maxRow*/, utilities::MpiWrapper& mpi)
    {
        const iSize_t lvl = Level(level1, level2, level2, level2, mpi);
        if (tables->GetDimension() != m_norb0 + 2 * lvl) Refuse("occupation energies of the wrong length", mpi);
        m_energies[lvl] = *tables->GetVTable();
        Clear();
    }
    // two_level_spinless_fermion_hamiltonian.hpp:306
    void Add_CdCdCC_Terms(QuarticTermTables* tables, iSize_t level1, iSize_t level2, iSize_t level3,
                          iSize_t level4, fock_t /*minRow*/, fock_t /*maxRow*/, utilities::MpiWrapper& mpi,
                          bool storeUpper = false)
    {
        const iSize_t lvl = Level(level1, level2, level3, level4, mpi);
        m_quartic[lvl] = tables;
        m_storeUpper = storeUpper;
        Clear();
    }
    void Build(utilities::MpiWrapper& mpi)
    {
        Clear();
        QuarticTermTables* q[2] = {m_quartic[0], m_quartic[1]};
        for (int l = 0; l < 2; ++l)
            if (!q[l]) {
                m_zero[l].Initialize(m_norb0 + 2 * l, std::vector<double>{0.0});
                q[l] = &m_zero[l];
            }
        utilities::EdCheck(ed_ham2_build_crs(m_fockBasis.handle(), q[0]->handle(), q[1]->handle(),
                                             m_energies[0].empty() ? nullptr : m_energies[0].data(),
                                             m_energies[1].empty() ? nullptr : m_energies[1].data(),
                                             m_storeUpper ? 1 : 0, nullptr, &m_crs),
                           &mpi);
    }
    fock_t GetFockSpaceDimension() const { return m_fockBasis.GetStoredDimension(); }
    int64_t GetNbrNonZeros() const
    {
        int64_t nnz = 0;
        if (m_crs) utilities::EdCheck(ed_crs_info(m_crs, nullptr, &nnz, nullptr));
        return nnz;
    }
    void GetCrs(std::vector<int64_t>& rowStarts, std::vector<int32_t>& cols, std::vector<double>& data) const
    {
        int64_t n = 0, nnz = 0;
        utilities::EdCheck(ed_crs_info(m_crs, &n, &nnz, nullptr));
        rowStarts.resize(n + 1);
        cols.resize(nnz);
        data.resize(nnz);
        utilities::EdCheck(ed_crs_get(m_crs, rowStarts.data(), cols.data(), data.data()));
    }
    void Apply(const double* x_dev, double* y_dev)
    {
        utilities::MpiWrapper mpi;
        if (!m_crs) Build(mpi);
        utilities::EdCheck(ed_spmv(m_crs, x_dev, y_dev, nullptr));
    }
    // hamiltonian_base.hpp:770.  The levels do not mix, so a sector's
    // eigenvalues E0(L0) + E1(L1) repeat 2 min(L0, L1) + 1 times: every copy
    // comes from the level-exchange ladder (ed_lanczos_two_level), or from
    // deflated passes after SetDegeneracyPasses(k) (k = 0: one sequence).
    bool LanczosDiagonalize(iSize_t nbrEigenvalues, utilities::MpiWrapper& mpi, double tol = 1e-10,
                            bool wantVectors = true)
    {
        if (!m_crs) Build(mpi);
        const fock_t n = GetFockSpaceDimension();
        m_eigenvalues.assign(nbrEigenvalues, 0.0);
        m_eigenvectors.assign(wantVectors ? (size_t)n * nbrEigenvalues : 0, 0.0);
        m_arpackWrapper.SetTolerance(tol);
        ed_op* op = nullptr;
        utilities::EdCheck(ed_op_from_crs(m_crs, &op), &mpi);
        bool ok = true;
        if (m_passesSet) {
            m_arpackWrapper.SetDiagonalCheck(true);
            ok = m_arpackWrapper.DiagonalizeOperator(op, wantVectors ? m_eigenvectors.data() : nullptr,
                                                     m_eigenvalues.data(), (int)n, (int)nbrEigenvalues, mpi);
        } else {
            ed_lanczos_params p{};
            p.nev = (int)nbrEigenvalues;
            p.tol = tol;
            p.verify = 1;
            p.want_vectors = wantVectors;
            p.diagonal_check = 1;
            const ed_status s = ed_lanczos_two_level(m_fockBasis.handle(), op, &p, nullptr, m_eigenvalues.data(),
                                                     wantVectors ? m_eigenvectors.data() : nullptr, &m_info);
            if (s != ED_OK) {
                std::cerr << "\n\tERROR in LanczosDiagonalize: " << ed_status_string(s) << ": " << ed_last_error()
                          << std::endl;
                mpi.m_exitFlag = true;
                ok = false;
            }
        }
        ed_op_free(op);
        return ok;
    }
    void SetDegeneracyPasses(int passes)
    {
        m_arpackWrapper.SetDegeneracyPasses(passes);
        m_passesSet = true;
    }
    void Clear()
    {
        if (m_crs) ed_crs_free(m_crs);
        m_crs = nullptr;
    }

    TwoLevelFermionFockBasis m_fockBasis;
    utilities::linearAlgebra::ArpackWrapper m_arpackWrapper;
    std::vector<double> m_eigenvalues;
    std::vector<double> m_eigenvectors;   // column-major n x nev

  private:
    iSize_t Level(iSize_t l1, iSize_t l2, iSize_t l3, iSize_t l4, utilities::MpiWrapper& mpi)
    {
        if (l1 > 1 || l2 > 1 || l3 > 1 || l4 > 1) Refuse("level specification incorrect (set to 0,1 only)", mpi);
        if (l1 != l2 || l2 != l3 || l3 != l4) Refuse("only coded for terms in the same level so far", mpi);
        return l1;
    }
    [[noreturn]] void Refuse(const char* msg, utilities::MpiWrapper& mpi)
    {
        std::cerr << "\n\tERROR in TwoLevelSpinlessFermionHamiltonian: " << msg << std::endl;
        mpi.m_exitFlag = true;
        throw utilities::EdError(ED_ERR_ARG, msg);
    }
    iSize_t m_norb0 = 0;
    utilities::storageMethod_t m_storageMethod = utilities::_SPARSE_CRS_;
    std::vector<double> m_energies[2];
    QuarticTermTables* m_quartic[2] = {nullptr, nullptr};
    QuarticTermTables m_zero[2];
    bool m_storeUpper = false;
    bool m_passesSet = false;
    ed_crs* m_crs = nullptr;
    ed_solve_info m_info{};
};

// interacting_ofl_model/term_tables.hpp QuarticTermTables (array format):
// (K+1) K^2 / 2 k1 values and complex V values at (t1*K + t2 - t1(t1+1)/2)*K
// + k, t1 = min(k3,k4), t2 = max(k3,k4) (term_tables.cpp:95-200).
class OflQuarticTermTables {
  public:
    void Initialize(iSize_t dimX, iSize_t dimY, const utilities::MpiWrapper&)
    {
        m_dimX = dimX;
        m_dimY = dimY;
        m_kMax = dimX * dimY;
        const size_t dim = (size_t)(m_kMax + 1) * m_kMax * m_kMax / 2;
        m_kTable.assign(dim, 0);
        m_vTable.assign(dim, std::complex<double>(0.0, 0.0));
    }
    std::vector<kState_t>* GetKTable() { return &m_kTable; }
    std::vector<std::complex<double>>* GetVTable() { return &m_vTable; }
    void GetK1(kState_t* buf, iSize_t& nbrK1, kState_t k2, kState_t k3, kState_t k4) const
    {
        nbrK1 = 1;
        buf[0] = m_kTable[(size_t)Tri(k3, k4) * m_kMax + k2];
    }
    std::complex<double> GetVkkkk(kState_t k1, kState_t k2, kState_t k3, kState_t k4) const
    {
        return m_vTable[(size_t)Tri(k3, k4) * m_kMax + (k4 > k3 ? k1 : k2)];
    }
    iSize_t m_dimX = 0, m_dimY = 0, m_kMax = 0;

  private:
    size_t Tri(kState_t k3, kState_t k4) const
    {
        const size_t t1 = k4 > k3 ? k3 : k4, t2 = k4 > k3 ? k4 : k3;
        return t1 * m_kMax + t2 - t1 * (t1 + 1) / 2;
    }
    std::vector<kState_t> m_kTable;
    std::vector<std::complex<double>> m_vTable;
};

// interacting_ofl_model/term_tables.hpp QuadraticTermTables: one complex
// occupation energy per orbital (GetEkk, term_tables.cpp:59-65).
class OflQuadraticTermTables {
  public:
    void Initialize(iSize_t nbrOrbitals, const utilities::MpiWrapper&)
    {
        m_vTable.assign(nbrOrbitals, std::complex<double>(0.0, 0.0));
    }
    std::vector<std::complex<double>>* GetVTable() { return &m_vTable; }
    const std::vector<std::complex<double>>* GetVTable() const { return &m_vTable; }
    iSize_t GetDimension() const { return (iSize_t)m_vTable.size(); }

  private:
    std::vector<std::complex<double>> m_vTable;
};

// hamiltonians/term_hash_tables_base.hpp:44-276 TermHashTables<dcmplx>: the
// k-table (keys of nlabels - 1 labels, each with one k1; a key may repeat)
// and the value table, kept as the flat key and value lists of its files;
// keys packed as utilities::Key does (two labels (k1 << 32) | k2, three
// (k2 << 48) | (k3 << 32) | (k4 << 16), four (k1 << 48) | (k2 << 32) |
// (k3 << 16) | k4).  Files through ed_term_hash_write / ed_term_hash_read.
class OflTermHashTablesBase {
  public:
    explicit OflTermHashTablesBase(int nbrLabels) : m_nbrLabels(nbrLabels) {}
    void Initialize(kState_t kMax) { m_kMax = kMax; }
    void Clear()
    {
        m_kKeys.clear();
        m_kValues.clear();
        m_vKeys.clear();
        m_vValues.clear();
        m_kLookup.clear();
        m_vLookup.clear();
    }
    iSize_t GetMaxKCount() const
    {
        std::unordered_map<uint64_t, iSize_t> c;
        iSize_t m = 1;
        for (uint64_t k : m_kKeys) m = std::max(m, ++c[k]);
        return m;
    }
    void ToFile(const std::string& fileName, io::fileFormat_t format, utilities::MpiWrapper& mpi) const
    {
        utilities::EdCheck(ed_term_hash_write(fileName.c_str(), format == io::_BINARY_ ? 1 : 0, m_nbrLabels,
                                              (uint32_t)m_kKeys.size(), m_kKeys.data(), m_kValues.data(),
                                              (uint32_t)m_vKeys.size(), m_vKeys.data(),
                                              reinterpret_cast<const double*>(m_vValues.data())),
                           &mpi);
    }
    void FromFile(const std::string& fileName, io::fileFormat_t format, utilities::MpiWrapper& mpi)
    {
        uint32_t nk = 0, nv = 0;
        const int b = format == io::_BINARY_ ? 1 : 0;
        utilities::EdCheck(ed_term_hash_read(fileName.c_str(), b, &nk, nullptr, nullptr, &nv, nullptr, nullptr), &mpi);
        Clear();
        m_kKeys.resize(nk);
        m_kValues.resize(nk);
        m_vKeys.resize(nv);
        m_vValues.resize(nv);
        utilities::EdCheck(ed_term_hash_read(fileName.c_str(), b, &nk, m_kKeys.data(), m_kValues.data(), &nv,
                                             m_vKeys.data(), reinterpret_cast<double*>(m_vValues.data())),
                           &mpi);
        Index();
    }
    static uint64_t Key(uint32_t k1, uint32_t k2) { return ((uint64_t)k1 << 32) | k2; }
    static uint64_t Key(uint16_t k2, uint16_t k3, uint16_t k4)
    {
        return ((uint64_t)k2 << 48) | ((uint64_t)k3 << 32) | ((uint64_t)k4 << 16);
    }
    static uint64_t Key(uint16_t k1, uint16_t k2, uint16_t k3, uint16_t k4)
    {
        return ((uint64_t)k1 << 48) | ((uint64_t)k2 << 32) | ((uint64_t)k3 << 16) | k4;
    }

    kState_t m_kMax = 0;
    std::vector<uint64_t> m_kKeys, m_vKeys;
    std::vector<kState_t> m_kValues;
    std::vector<std::complex<double>> m_vValues;

  protected:
    void Insert(uint64_t kkey, kState_t k1, uint64_t vkey, std::complex<double> v)
    {
        m_kKeys.push_back(kkey);
        m_kValues.push_back(k1);
        m_vKeys.push_back(vkey);
        m_vValues.push_back(v);
    }
    void Index()
    {
        m_kLookup.clear();
        m_vLookup.clear();
        for (size_t i = 0; i < m_kKeys.size(); ++i) m_kLookup[m_kKeys[i]].push_back(m_kValues[i]);
        for (size_t i = 0; i < m_vKeys.size(); ++i) m_vLookup.emplace(m_vKeys[i], m_vValues[i]);
    }
    void K1(kState_t* buf, iSize_t& nbr, uint64_t key) const
    {
        nbr = 0;   // a missing key has no k1 (the reference leaves the count unset)
        auto it = m_kLookup.find(key);
        if (it == m_kLookup.end()) return;
        for (kState_t k : it->second) buf[nbr++] = k;
    }
    std::complex<double> V(uint64_t key) const
    {
        auto it = m_vLookup.find(key);
        return it == m_vLookup.end() ? std::complex<double>(0.0, 0.0) : it->second;
    }

  private:
    int m_nbrLabels;
    std::unordered_map<uint64_t, std::vector<kState_t>> m_kLookup;
    std::unordered_map<uint64_t, std::complex<double>> m_vLookup;
};

// interacting_ofl_model/term_hash_tables.hpp QuarticTermHashTables
class OflQuarticTermHashTables : public OflTermHashTablesBase {
  public:
    OflQuarticTermHashTables() : OflTermHashTablesBase(4) {}
    // term_hash_tables_base.hpp:229-247: every (k2, k3, k4)
    void SetQuarticFromArray(OflQuarticTermTables* a)
    {
        Clear();
        m_kMax = (kState_t)a->m_kMax;
        kState_t k1 = 0;
        iSize_t n = 0;
        for (kState_t k2 = 0; k2 < m_kMax; ++k2)
            for (kState_t k3 = 0; k3 < m_kMax; ++k3)
                for (kState_t k4 = 0; k4 < m_kMax; ++k4) {
                    a->GetK1(&k1, n, k2, k3, k4);
                    Insert(Key(k2, k3, k4), k1, Key(k1, k2, k3, k4), a->GetVkkkk(k1, k2, k3, k4));
                }
        Index();
    }
    void GetK1(kState_t* buf, iSize_t& nbrK1, kState_t k2, kState_t k3, kState_t k4) const
    {
        K1(buf, nbrK1, Key(k2, k3, k4));
    }
    std::complex<double> GetVkkkk(kState_t k1, kState_t k2, kState_t k3, kState_t k4) const
    {
        return V(Key(k1, k2, k3, k4));
    }
};

// interacting_ofl_model/term_hash_tables.hpp QuadraticTermHashTables
class OflQuadraticTermHashTables : public OflTermHashTablesBase {
  public:
    OflQuadraticTermHashTables() : OflTermHashTablesBase(2) {}
    // term_hash_tables_base.hpp:262-275 (the array tables: k1 = k2)
    void SetQuadraticFromArray(OflQuadraticTermTables* a)
    {
        Clear();
        m_kMax = (kState_t)a->GetDimension();
        for (kState_t k = 0; k < m_kMax; ++k) Insert(k, k, Key((uint32_t)k, (uint32_t)k), (*a->GetVTable())[k]);
        Index();
    }
    void GetK1(kState_t* buf, iSize_t& nbrK1, kState_t k2) const { K1(buf, nbrK1, k2); }
    std::complex<double> GetEkk(kState_t k1, kState_t k2) const { return V(Key((uint32_t)k1, (uint32_t)k2)); }
};

// spinless_fermion_hamiltonian.hpp:52 for T = dcmplx, as InteractingOflModel
// drives it (interacting_ofl_model.cpp:952-1135): SetFockBasis (a momentum
// sector), Add_CdC_Terms, Add_CdCdCC_Terms, LanczosDiagonalize.  The device
// build runs at the first solve; vectors are std::complex<double>.
template <>
class SpinlessFermionHamiltonian<std::complex<double>> {
  public:
    SpinlessFermionHamiltonian() = default;
    SpinlessFermionHamiltonian(const SpinlessFermionHamiltonian&) = delete;
    SpinlessFermionHamiltonian& operator=(const SpinlessFermionHamiltonian&) = delete;
    ~SpinlessFermionHamiltonian() { Clear(); }

    void Initialize(iSize_t nbrParticles, iSize_t nbrOrbitals, utilities::storageMethod_t storageMethod,
                    utilities::MpiWrapper&)
    {
        m_nbrParticles = nbrParticles;
        m_nbrOrbitals = nbrOrbitals;
        m_storageMethod = storageMethod;
    }
    void SetFockBasis(FermionFockBasis&& basis)
    {
        m_fockBasis = std::move(basis);
        Clear();
    }
    void Add_CdC_Terms(OflQuadraticTermTables* tables, fock_t /*minRow*/, fock_t /*maxRow*/, utilities::MpiWrapper&)
    {
        m_energies = *tables->GetVTable();
        Clear();
    }
    void Add_CdCdCC_Terms(OflQuarticTermTables* tables, fock_t /*minRow*/, fock_t /*maxRow*/, utilities::MpiWrapper&,
                          bool storeUpper = false)
    {
        m_tables = tables;
        m_hashTables = nullptr;
        m_storeUpper = storeUpper;
        Clear();
    }
    // the hash-format branch of InteractingOflModel::BuildHamiltonian
    // (interacting_ofl_model.cpp:1046-1049); momentum-conserving tables only
    void Add_CdC_Terms(OflQuadraticTermHashTables* tables, fock_t /*minRow*/, fock_t /*maxRow*/,
                       utilities::MpiWrapper&)
    {
        m_hashEnergies = tables;
        Clear();
    }
    void Add_CdCdCC_Terms(OflQuarticTermHashTables* tables, fock_t /*minRow*/, fock_t /*maxRow*/,
                          utilities::MpiWrapper&, bool storeUpper = false)
    {
        m_hashTables = tables;
        m_tables = nullptr;
        m_storeUpper = storeUpper;
        Clear();
    }
    void Build(utilities::MpiWrapper& mpi)
    {
        Clear();
        if (m_hashTables) {
            const OflQuarticTermHashTables& q = *m_hashTables;
            static const OflQuadraticTermHashTables none;
            const OflQuadraticTermHashTables& d = m_hashEnergies ? *m_hashEnergies : none;
            ed_cterms* t = nullptr;
            utilities::EdCheck(
                ed_cterms_create_hash((int)m_nbrOrbitals, (int)m_fockBasis.DimX(), (int)m_fockBasis.DimY(),
                                      (uint32_t)q.m_kKeys.size(), q.m_kKeys.data(), q.m_kValues.data(),
                                      (uint32_t)q.m_vKeys.size(), q.m_vKeys.data(),
                                      reinterpret_cast<const double*>(q.m_vValues.data()), (uint32_t)d.m_kKeys.size(),
                                      d.m_kKeys.data(), d.m_kValues.data(), (uint32_t)d.m_vKeys.size(),
                                      d.m_vKeys.data(), reinterpret_cast<const double*>(d.m_vValues.data()), &t),
                &mpi);
            const ed_status s = ed_cham_build_crs(m_fockBasis.handle(), t, m_storeUpper ? 1 : 0, nullptr, &m_crs);
            ed_cterms_free(t);
            utilities::EdCheck(s, &mpi);
            return;
        }
        if (!m_tables) throw utilities::EdError(ED_ERR_ARG, "Add_CdCdCC_Terms first");
        ed_cterms* t = nullptr;
        const double* e = m_energies.empty() ? nullptr : reinterpret_cast<const double*>(m_energies.data());
        utilities::EdCheck(ed_cterms_create((int)m_tables->m_kMax, (int)m_tables->m_dimX, (int)m_tables->m_dimY,
                                            m_tables->GetKTable()->data(),
                                            reinterpret_cast<const double*>(m_tables->GetVTable()->data()), e, &t),
                           &mpi);
        const ed_status s = ed_cham_build_crs(m_fockBasis.handle(), t, m_storeUpper ? 1 : 0, nullptr, &m_crs);
        ed_cterms_free(t);
        utilities::EdCheck(s, &mpi);
    }
    fock_t GetFockSpaceDimension() const { return m_fockBasis.GetStoredDimension(); }
    int64_t GetNbrNonZeros() const
    {
        int64_t nnz = 0;
        if (m_crs) utilities::EdCheck(ed_ccrs_info(m_crs, nullptr, &nnz, nullptr));
        return nnz;
    }
    // hamiltonian_base.hpp:770 with the complex driver; eigenvalues ascending
    bool LanczosDiagonalize(iSize_t nbrEigenvalues, utilities::MpiWrapper& mpi, double tol = 1e-10,
                            bool wantVectors = true)
    {
        if (!m_crs) Build(mpi);
        const fock_t n = GetFockSpaceDimension();
        m_eigenvalues.assign(nbrEigenvalues, 0.0);
        m_eigenvectors.assign(wantVectors ? (size_t)n * nbrEigenvalues : 0, std::complex<double>(0.0, 0.0));
        ed_lanczos_params p{};
        p.nev = (int)nbrEigenvalues;
        p.tol = tol;
        p.verify = 1;
        p.want_vectors = wantVectors;
        p.diagonal_check = 1;
        const ed_status s = ed_clanczos(m_crs, &p, nullptr, m_eigenvalues.data(),
                                        wantVectors ? reinterpret_cast<double*>(m_eigenvectors.data()) : nullptr,
                                        &m_info);
        if (s != ED_OK) {
            std::cerr << "\n\tERROR in LanczosDiagonalize: " << ed_status_string(s) << ": " << ed_last_error()
                      << std::endl;
            mpi.m_exitFlag = true;
            return false;
        }
        return true;
    }
    void Clear()
    {
        if (m_crs) ed_ccrs_free(m_crs);
        m_crs = nullptr;
    }
    const ed_solve_info& LastInfo() const { return m_info; }

    FermionFockBasis m_fockBasis;
    std::vector<double> m_eigenvalues;
    std::vector<std::complex<double>> m_eigenvectors;   // nev vectors of n entries

  private:
    iSize_t m_nbrParticles = 0, m_nbrOrbitals = 0;
    utilities::storageMethod_t m_storageMethod = utilities::_SPARSE_CRS_;
    std::vector<std::complex<double>> m_energies;
    OflQuarticTermTables* m_tables = nullptr;
    OflQuarticTermHashTables* m_hashTables = nullptr;
    OflQuadraticTermHashTables* m_hashEnergies = nullptr;
    bool m_storeUpper = false;
    ed_ccrs* m_crs = nullptr;
    ed_solve_info m_info{};
};

// observables/fermion_observables.hpp:39, for the eigenvectors of a real
// Hamiltonian built here (H provides m_fockBasis and a column-major n x nev
// m_eigenvectors, as SpinlessFermionHamiltonian<double> does).  Out-of-range
// indices and missing eigenvectors throw EdError.
struct Observables {
    template <class H>
    static const double* Vector(const H& hamiltonian, iSize_t eigenvectorIndex)
    {
        const size_t n = (size_t)hamiltonian.m_fockBasis.GetStoredDimension();
        if (n == 0 || hamiltonian.m_eigenvectors.size() < n * ((size_t)eigenvectorIndex + 1))
            throw utilities::EdError(ED_ERR_ARG, "eigenvector not calculated or eigenvectorIndex out of range");
        return hamiltonian.m_eigenvectors.data() + n * eigenvectorIndex;
    }
    // fermion_observables.hpp:48: probabilityList[k] = <c+_k c_k>, k < norb
    template <class H>
    void DensityFunction(const H& hamiltonian, iSize_t eigenvectorIndex, double* probabilityList,
                         utilities::MpiWrapper& mpi)
    {
        utilities::EdCheck(ed_obs_density(hamiltonian.m_fockBasis.handle(), Vector(hamiltonian, eigenvectorIndex),
                                          probabilityList),
                           &mpi);
    }
    // fermion_observables.hpp:117: probabilityList[k*norb + q] = <c+_k c_k c+_q c_q>
    template <class H>
    void DensityDensityFunction(const H& hamiltonian, iSize_t eigenvectorIndex, double* probabilityList,
                                utilities::MpiWrapper& mpi)
    {
        utilities::EdCheck(ed_obs_density_density(hamiltonian.m_fockBasis.handle(),
                                                  Vector(hamiltonian, eigenvectorIndex), probabilityList),
                           &mpi);
    }
    // fermion_observables.hpp:528: 1 / sum |psi|^4
    template <class H>
    double GetParticipationRatio(const H& hamiltonian, iSize_t eigenvectorIndex, utilities::MpiWrapper& mpi)
    {
        double r = 0.0;
        utilities::EdCheck(ed_obs_participation_ratio(hamiltonian.m_fockBasis.handle(),
                                                      Vector(hamiltonian, eigenvectorIndex), &r),
                           &mpi);
        return r;
    }
    // fermion_observables.hpp:437: for every eigenvector e, the nbrStates
    // largest |psi| in descending order at states/amplitudes + e*nbrStates
    // (fewer, min(nbrStates, n), when the sector is smaller)
    template <class H>
    void GetMostProbable(const H& hamiltonian, iSize_t nbrStates, fock_t* states, double* amplitudes,
                         utilities::MpiWrapper& mpi)
    {
        const size_t n = (size_t)hamiltonian.m_fockBasis.GetStoredDimension();
        const size_t nev = n ? hamiltonian.m_eigenvectors.size() / n : 0;
        const size_t k = std::min<size_t>(nbrStates, n);
        for (size_t e = 0; e < nev; ++e) {
            int64_t cnt = 0;
            utilities::EdCheck(ed_obs_most_probable(hamiltonian.m_fockBasis.handle(),
                                                    hamiltonian.m_eigenvectors.data() + n * e, (int64_t)k,
                                                    states + e * k, amplitudes + e * k, &cnt),
                               &mpi);
        }
    }
    template <class H>
    void GetMostProbable(const H& hamiltonian, iSize_t nbrStates, fock_t* states, std::complex<double>* amplitudes,
                         utilities::MpiWrapper& mpi)
    {
        const size_t n = (size_t)hamiltonian.m_fockBasis.GetStoredDimension();
        const size_t nev = n ? hamiltonian.m_eigenvectors.size() / n : 0;
        std::vector<double> re(std::min<size_t>(nbrStates, n) * nev);
        GetMostProbable(hamiltonian, nbrStates, states, re.data(), mpi);
        for (size_t i = 0; i < re.size(); ++i) amplitudes[i] = re[i];
    }
};

}  // namespace diagonalization
