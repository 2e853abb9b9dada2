// Exercises the reference-shaped C++ host classes (include/ed_host.hpp) the
// way the reference's model layer drives them for one sector:
// tables -> basis -> Add_CdCdCC_Terms -> LanczosDiagonalize, plus the
// std::function product path of ArpackWrapper, the ground state's
// observables, a two-level sector (N=4, norb0=6, Lz=0) as
// SphereTwoLevelPseudopotentialModel builds it, and a complex momentum sector
// (N=4 on a 3x4 grid, momentum (1,2)) as InteractingOflModel builds it, and
// the reference's own model sequence written as it reads there (a predicate
// basis, SetFockBasis, Initialize, Add_CdCdCC_Terms, FullDiagonalize or
// LanczosDiagonalize).  Prints one JSON line.
#include <cmath>
#include <complex>
#include <cstdio>
#include <functional>
#include <vector>

#include "ed_host.hpp"

int main(int argc, char** argv)
{
    const int N = argc > 1 ? std::atoi(argv[1]) : 6;
    const int norb = argc > 2 ? std::atoi(argv[2]) : 16;
    const int twoLz = argc > 3 ? std::atoi(argv[3]) : 0;
    const int nev = 3;
    utilities::MpiWrapper mpi;
    std::vector<double> coul(norb);
    utilities::EdCheck(ed_coulomb_pseudopotentials(norb, coul.data()));
    std::vector<double> pp(coul.begin(), coul.begin() + (norb - 1));
    for (size_t m = 0; m < pp.size(); m += 2) pp[m] = 0.0;

    diagonalization::QuarticTermTables tables;
    tables.Initialize(norb, pp);
    diagonalization::SpinlessFermionHamiltonian<double> H;
    H.Initialize(N, norb, utilities::_SPARSE_CRS_, mpi, twoLz);
    const diagonalization::fock_t dim = H.GetFockSpaceDimension();
    H.Add_CdCdCC_Terms(&tables, 0, dim, mpi);
    bool ok = H.LanczosDiagonalize(nev, mpi, 1e-10);

    // the generic std::function product: a host upper-triangle loop over the CRS
    std::vector<int64_t> rs;
    std::vector<int32_t> cs;
    std::vector<double> vs;
    H.GetCrs(rs, cs, vs);
    std::function<void(double*, double*, utilities::MpiWrapper&)> mv = [&](double* x, double* y, utilities::MpiWrapper&) {
        for (diagonalization::fock_t i = 0; i < dim; ++i) {
            double s = 0.0;
            for (int64_t k = rs[i]; k < rs[i + 1]; ++k) s += vs[k] * x[cs[k]];
            y[i] = s;
        }
    };
    utilities::linearAlgebra::ArpackWrapper arp;
    std::vector<double> ev2(nev), vec2((size_t)dim * nev);
    bool ok2 = arp.DiagonalizeSymmetricMatrix<double>(mv, vec2.data(), ev2.data(), (int)dim, (int)dim, nev, mpi);

    // basis round trip through FindFockStateIndex
    std::vector<diagonalization::fock_t> words(dim);
    H.m_fockBasis.GetFockBasis(words.data(), dim, mpi);
    bool rank_ok = true;
    for (diagonalization::fock_t i = 0; i < dim; i += 97)
        rank_ok = rank_ok && H.m_fockBasis.FindFockStateIndex(0, words[i]) == i;

    // observables of the ground state (fermion_observables.hpp)
    diagonalization::Observables obs;
    std::vector<double> rho(norb), dd((size_t)norb * norb);
    obs.DensityFunction(H, 0, rho.data(), mpi);
    obs.DensityDensityFunction(H, 0, dd.data(), mpi);
    const double pr = obs.GetParticipationRatio(H, 0, mpi);
    std::vector<diagonalization::fock_t> top(3 * nev);
    std::vector<std::complex<double>> amp(3 * nev);
    obs.GetMostProbable(H, 3, top.data(), amp.data(), mpi);
    double nsum = 0.0;
    for (double r : rho) nsum += r;

    std::printf("{\"ok\": %s, \"ok_host_product\": %s, \"rank_ok\": %s, \"dim\": %llu, \"nnz\": %lld, \"eigenvalues\": [",
                ok ? "true" : "false", ok2 ? "true" : "false", rank_ok ? "true" : "false",
                (unsigned long long)dim, (long long)H.GetNbrNonZeros());
    for (int i = 0; i < nev; ++i) std::printf("%s%.17g", i ? ", " : "", H.m_eigenvalues[i]);
    std::printf("], \"eigenvalues_host_product\": [");
    for (int i = 0; i < nev; ++i) std::printf("%s%.17g", i ? ", " : "", ev2[i]);
    std::printf("], \"density\": [");
    for (int k = 0; k < norb; ++k) std::printf("%s%.17g", k ? ", " : "", rho[k]);
    std::printf("], \"density_sum\": %.17g, \"dd00\": %.17g, \"participation\": %.17g, \"top_state\": %llu, "
                "\"top_amp\": %.17g", nsum, dd[0], pr, (unsigned long long)top[0], amp[0].real());
    // two levels: LLL tables of norb0 orbitals, second-level tables of norb0 + 2
    // (odd-m Coulomb lists of those sizes), second-level occupation energy 0.4
    const int n0 = 6;
    std::vector<double> pp0(n0 - 1, 0.0), pp1(n0 + 1, 0.0), c0(n0), c1(n0 + 2);
    utilities::EdCheck(ed_coulomb_pseudopotentials(n0, c0.data()));
    utilities::EdCheck(ed_coulomb_pseudopotentials(n0 + 2, c1.data()));
    for (int m = 1; m < n0 - 1; m += 2) pp0[m] = c0[m];
    for (int m = 1; m < n0 + 1; m += 2) pp1[m] = c1[m];
    diagonalization::QuarticTermTables q0, q1;
    q0.Initialize(n0, pp0);
    q1.Initialize(n0 + 2, pp1);
    diagonalization::QuadraticTermTables e1;
    e1.Initialize(n0 + 2, mpi);
    for (double& e : *e1.GetVTable()) e = 0.4;
    diagonalization::TwoLevelSpinlessFermionHamiltonian<double> H2;
    H2.Initialize(4, 2 * n0 + 2, utilities::_SPARSE_CRS_, mpi, 0);
    const diagonalization::fock_t dim2 = H2.GetFockSpaceDimension();
    H2.Add_CdC_Terms(&e1, 1, 1, 0, dim2, mpi);
    H2.Add_CdCdCC_Terms(&q0, 0, 0, 0, 0, 0, dim2, mpi);
    H2.Add_CdCdCC_Terms(&q1, 1, 1, 1, 1, 0, dim2, mpi);
    const bool ok3 = H2.LanczosDiagonalize(4, mpi, 1e-10);
    std::vector<diagonalization::fock_t> f2(dim2), s2(dim2);
    H2.m_fockBasis.GetFockBasis(f2.data(), s2.data(), dim2, mpi);
    bool rank2_ok = true;
    for (diagonalization::fock_t i = 0; i < dim2; i += 7) {
        diagonalization::fock_t idx = 0;
        H2.m_fockBasis.FindFockStateIndex(0, f2[i], s2[i], idx);
        rank2_ok = rank2_ok && idx == i;
    }
    std::printf(", \"residual\": %.3e, \"two_level\": {\"ok\": %s, \"rank_ok\": %s, \"dim\": %llu, \"nnz\": %lld, "
                "\"eigenvalues\": [",
                H.m_arpackWrapper.LastInfo().max_residual, ok3 ? "true" : "false", rank2_ok ? "true" : "false",
                (unsigned long long)dim2, (long long)H2.GetNbrNonZeros());
    for (int i = 0; i < 4; ++i) std::printf("%s%.17g", i ? ", " : "", H2.m_eigenvalues[i]);
    std::printf("]}");

    // complex momentum sector: tables with FindK1's momentum rule and
    // exactly representable values, real where the diagonal terms read them
    const int X = 3, Y = 4, K = X * Y;
    diagonalization::OflQuarticTermTables oq;
    oq.Initialize(X, Y, mpi);
    for (int t1 = 0; t1 < K; ++t1)
        for (int t2 = t1; t2 < K; ++t2) {
            const size_t base = (size_t)(t1 * K + t2 - t1 * (t1 + 1) / 2) * K;
            for (int k2 = 0; k2 < K; ++k2) {
                const int kx = ((t1 / Y + t2 / Y - k2 / Y) % X + X) % X;
                const int ky = ((t1 % Y + t2 % Y - k2 % Y) % Y + Y) % Y;
                (*oq.GetKTable())[base + k2] = (diagonalization::kState_t)(kx * Y + ky);
                const size_t i = base + k2;
                const double re = (double)((i * 7919) % 1000) / 500.0 - 1.0;
                const double im = (k2 == t1 || k2 == t2) ? 0.0 : (double)((i * 104729) % 1000) / 500.0 - 1.0;
                (*oq.GetVTable())[i] = std::complex<double>(re, im);
            }
        }
    diagonalization::OflQuadraticTermTables oe;
    oe.Initialize(K, mpi);
    for (int k = 0; k < K; ++k) (*oe.GetVTable())[k] = std::complex<double>(0.125 * k, 0.0);
    diagonalization::FermionFockBasis mb;
    mb.GenerateFockSpaceMomentum(4, X, Y, 1, 2, mpi);
    diagonalization::SpinlessFermionHamiltonian<std::complex<double>> Hc;
    Hc.Initialize(4, K, utilities::_SPARSE_MAPPED_, mpi);
    Hc.SetFockBasis(std::move(mb));
    const diagonalization::fock_t dimc = Hc.GetFockSpaceDimension();
    Hc.Add_CdC_Terms(&oe, 0, dimc, mpi);
    Hc.Add_CdCdCC_Terms(&oq, 0, dimc, mpi);
    const bool ok4 = Hc.LanczosDiagonalize(3, mpi, 1e-10);
    std::printf(", \"ofl\": {\"ok\": %s, \"dim\": %llu, \"nnz\": %lld, \"eigenvalues\": [", ok4 ? "true" : "false",
                (unsigned long long)dimc, (long long)Hc.GetNbrNonZeros());
    for (int i = 0; i < 3; ++i) std::printf("%s%.17g", i ? ", " : "", Hc.m_eigenvalues[i]);
    std::printf("]}");

    // the same terms in the hash-table format, as InteractingOflModel's
    // ConvertTableFormat, TermsToFile / TermsFromFile and hash-format
    // BuildHamiltonian use them (interacting_ofl_model.cpp:597-691, 1046-1049)
    diagonalization::OflQuarticTermHashTables qh;
    diagonalization::OflQuadraticTermHashTables dh;
    qh.Initialize(K);
    dh.Initialize(K);
    dh.SetQuadraticFromArray(&oe);
    qh.SetQuarticFromArray(&oq);
    qh.ToFile("quartic_coefficient_table_kx_3_ky_4.dat", io::_BINARY_, mpi);
    dh.ToFile("quadratic_coefficient_table_kx_3_ky_4.dat", io::_BINARY_, mpi);
    diagonalization::OflQuarticTermHashTables qh2;
    diagonalization::OflQuadraticTermHashTables dh2;
    qh2.Initialize(K);
    dh2.Initialize(K);
    qh2.FromFile("quartic_coefficient_table_kx_3_ky_4.dat", io::_BINARY_, mpi);
    dh2.FromFile("quadratic_coefficient_table_kx_3_ky_4.dat", io::_BINARY_, mpi);
    diagonalization::kState_t k1buf[4];
    diagonalization::iSize_t nk1 = 0;
    qh2.GetK1(k1buf, nk1, 2, 5, 7);
    diagonalization::kState_t k1arr = 0;
    diagonalization::iSize_t na = 0;
    oq.GetK1(&k1arr, na, 2, 5, 7);
    const bool lookups_ok = nk1 == 1 && k1buf[0] == k1arr && qh2.GetVkkkk(k1arr, 2, 5, 7) == oq.GetVkkkk(k1arr, 2, 5, 7) &&
                            qh2.GetMaxKCount() == 1;
    diagonalization::FermionFockBasis mb2;
    mb2.GenerateFockSpaceMomentum(4, X, Y, 1, 2, mpi);
    diagonalization::SpinlessFermionHamiltonian<std::complex<double>> Hh;
    Hh.Initialize(4, K, utilities::_SPARSE_MAPPED_, mpi);
    Hh.SetFockBasis(std::move(mb2));
    Hh.Add_CdC_Terms(&dh2, 0, dimc, mpi);
    Hh.Add_CdCdCC_Terms(&qh2, 0, dimc, mpi);
    const bool ok6 = Hh.LanczosDiagonalize(3, mpi, 1e-10);
    bool same = ok6 && Hh.GetNbrNonZeros() == Hc.GetNbrNonZeros();
    for (int i = 0; i < 3 && same; ++i) same = Hh.m_eigenvalues[i] == Hc.m_eigenvalues[i];
    std::printf(", \"ofl_hash\": {\"ok\": %s, \"lookups_ok\": %s, \"same_as_array\": %s}", ok6 ? "true" : "false",
                lookups_ok ? "true" : "false", same ? "true" : "false");

    // The reference's model sequence as it is written there
    // (pseudopotential_model.cpp:160-189 BuildFockBasis, :233-249
    // BuildHamiltonian, pseudopotential_model_base.hpp:235-275 BaseDiagonalize):
    // the sector of a std::bind predicate, SetFockBasis, Initialize with
    // mapped storage, Add_CdCdCC_Terms over all rows, then FullDiagonalize
    // below dimension 60 and LanczosDiagonalize with a MatrixVectorFunction
    // above it.  Run for the sector above and for a small one.
    bool ok5 = true;
    std::printf(", \"reference_sequence\": [");
    const int seqN[2] = {N, 4}, seqOrb[2] = {norb, 10};
    for (int c = 0; c < 2; ++c) {
        const int n5 = seqN[c], k5 = seqOrb[c];
        std::vector<double> pc(k5);
        utilities::EdCheck(ed_coulomb_pseudopotentials(k5, pc.data()));
        std::vector<double> p5(pc.begin(), pc.begin() + (k5 - 1));
        for (size_t m = 0; m < p5.size(); m += 2) p5[m] = 0.0;
        diagonalization::QuadraticTermTables m_quadraticTables;
        diagonalization::QuarticTermTables m_quarticTables;
        m_quarticTables.Initialize(k5, p5);
        diagonalization::SpinlessFermionHamiltonian<double> m_hamiltonian;
        const diagonalization::mState_t totalLz = (diagonalization::mState_t)(c == 0 ? twoLz : 0);
        const diagonalization::mState_t maxLz = (diagonalization::mState_t)(k5 - 1);
        diagonalization::FermionFockBasis basis;
        const bool isZeroDimensional = basis.GenerateFockSpace(
            n5, k5, std::bind(&diagonalization::TestAngularMomentumSector, std::placeholders::_1, totalLz, maxLz), mpi);
        m_hamiltonian.SetFockBasis(basis);
        m_hamiltonian.Initialize(n5, k5, utilities::_SPARSE_MAPPED_, mpi);
        m_hamiltonian.Add_CdCdCC_Terms(&m_quarticTables, 0, m_hamiltonian.m_data.m_fockSpaceDim, mpi);
        diagonalization::iSize_t nbrEigenvaluesToFind = nev;
        bool done = false;
        const bool full = m_hamiltonian.m_data.m_fockSpaceDim < 60;
        if (full) {
            done = m_hamiltonian.FullDiagonalize(nbrEigenvaluesToFind, mpi);
        } else {
            diagonalization::MatrixVectorFunction<double, diagonalization::QuadraticTermTables,
                                                  diagonalization::QuarticTermTables>
                mv(m_hamiltonian, mpi);
            done = m_hamiltonian.LanczosDiagonalize(&m_quadraticTables, &m_quarticTables, mv, nbrEigenvaluesToFind, mpi);
        }
        ok5 = ok5 && done && !isZeroDimensional;
        std::printf("%s{\"N\": %d, \"norb\": %d, \"two_lz\": %d, \"ok\": %s, \"full\": %s, \"dim\": %llu, \"eigenvalues\": [",
                    c ? ", " : "", n5, k5, (int)totalLz, done ? "true" : "false", full ? "true" : "false",
                    (unsigned long long)m_hamiltonian.m_data.m_fockSpaceDim);
        for (diagonalization::iSize_t i = 0; i < nbrEigenvaluesToFind; ++i)
            std::printf("%s%.17g", i ? ", " : "", m_hamiltonian.m_eigenvalues[i]);
        std::printf("]}");
    }
    // a predicate that selects every sector (the reference's run without
    // block diagonalisation) is refused: the device builds one sector
    bool refused = false;
    try {
        diagonalization::FermionFockBasis all;
        utilities::MpiWrapper mpi2;
        all.GenerateFockSpace(4, 10, [](const diagonalization::fock_t) { return true; }, mpi2);
    } catch (const utilities::EdError&) {
        refused = true;
    }
    std::printf("], \"all_sectors_refused\": %s}\n", refused ? "true" : "false");
    return (ok && ok2 && rank_ok && ok3 && rank2_ok && ok4 && ok5 && refused) ? 0 : 1;
}
