// Exercises the reference-shaped C++ host classes (include/ed_host.hpp) the
// way the reference's model layer drives them for one sector:
// tables -> basis -> Add_CdCdCC_Terms -> LanczosDiagonalize, plus the
// std::function product path of ArpackWrapper, and the ground state's
// observables.  Prints one JSON line.
#include <cmath>
#include <complex>
#include <cstdio>
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
    std::printf(", \"residual\": %.3e}\n", H.m_arpackWrapper.LastInfo().max_residual);
    return (ok && ok2 && rank_ok) ? 0 : 1;
}
