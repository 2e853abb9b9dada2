// Host-side term tables of the LLL pseudopotential Hamiltonian.
//
//  - Clebsch-Gordan coefficients from the Racah closed form rewritten as an
//    alternating sum of products of binomials, summed EXACTLY in multiword
//    integers, then one square root in double.  The reference obtains the same
//    numbers from an SU(N) code that solves for them with LAPACK dgesvd_
//    (utilities/mathematics/clebsch_gordan_coefficients.cpp:534,554); any
//    per-multiplet phase cancels in the CG*CG products of the V table.
//  - k-table and V-table in the reference's layout and summation order
//    (fqhe_sphere/pseudopotential_model/pseudopotential_model_base.hpp:62-229).
//  - The per-hop element table the device kernels use: for every pair hop
//    (a,b) -> (c,d) with a+b = c+d, the sum of the four ordered terms in the
//    order spinless_fermion_hamiltonian.hpp:316-391 visits them, with the
//    1e-14 per-term filter (:371) and the trim (mapped_sparse_matrix.hpp:447).
//
// Built with -ffp-contract=off so x86-64 and aarch64 hosts produce identical
// tables.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "ed_internal.h"

namespace edgb {

typedef unsigned __int128 u128;

uint64_t binomial_u64(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    u128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (u128)(n - k + i) / (u128)i;
    return (uint64_t)r;
}

namespace {

u128 binomial_u128(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    u128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (u128)(n - k + i) / (u128)i;
    return r;
}

// Unsigned multiword integer, little-endian 32-bit limbs.
struct Big {
    static constexpr int L = 20;
    uint32_t w[L];
    Big() { std::memset(w, 0, sizeof(w)); }
    static Big from_u128(u128 x)
    {
        Big b;
        for (int i = 0; i < 4; ++i) { b.w[i] = (uint32_t)(x & 0xffffffffu); x >>= 32; }
        return b;
    }
    int top() const
    {
        for (int i = L - 1; i >= 0; --i)
            if (w[i]) return i;
        return -1;
    }
    Big mul(const Big& o) const
    {
        Big r;
        int ta = top(), tb = o.top();
        if (ta < 0 || tb < 0) return r;
        ED_REQUIRE(ta + tb + 2 <= L, ED_ERR_INTERNAL, "multiword product overflow");
        for (int i = 0; i <= ta; ++i) {
            uint64_t carry = 0;
            for (int j = 0; j <= tb; ++j) {
                uint64_t t = (uint64_t)w[i] * o.w[j] + r.w[i + j] + carry;
                r.w[i + j] = (uint32_t)t;
                carry = t >> 32;
            }
            int p = i + tb + 1;
            while (carry) {
                uint64_t t = (uint64_t)r.w[p] + carry;
                r.w[p] = (uint32_t)t;
                carry = t >> 32;
                ++p;
            }
        }
        return r;
    }
    void add(const Big& o)
    {
        uint64_t c = 0;
        for (int i = 0; i < L; ++i) {
            uint64_t t = (uint64_t)w[i] + o.w[i] + c;
            w[i] = (uint32_t)t;
            c = t >> 32;
        }
        ED_REQUIRE(c == 0, ED_ERR_INTERNAL, "multiword sum overflow");
    }
    // this -= o, requires this >= o
    void sub(const Big& o)
    {
        int64_t b = 0;
        for (int i = 0; i < L; ++i) {
            int64_t t = (int64_t)w[i] - (int64_t)o.w[i] - b;
            b = t < 0;
            w[i] = (uint32_t)(t + (b ? ((int64_t)1 << 32) : 0));
        }
    }
    int cmp(const Big& o) const
    {
        for (int i = L - 1; i >= 0; --i) {
            if (w[i] != o.w[i]) return w[i] < o.w[i] ? -1 : 1;
        }
        return 0;
    }
    double to_double() const
    {
        int t = top();
        if (t < 0) return 0.0;
        double r = 0.0;
        for (int i = t; i >= 0 && i >= t - 3; --i) r += std::ldexp((double)w[i], 32 * i);
        return r;
    }
};

}  // namespace

// <j1 m1; j2 m2 | J M>, twice-unit arguments.
//   CG^2 = S^2 (2J+1) C(2j1,a) C(2j2,c)
//          / [ (T+1) C(T,a) C(2J,J+M) C(2j1,j1-m1) C(2j2,j2-m2) ]
//   S    = sum_k (-1)^k C(a,k) C(b,j1-m1-k) C(c,j2+m2-k)
// with a = j1+j2-J, b = j1-j2+J, c = -j1+j2+J, T = j1+j2+J (the Racah
// formula with every pair of factorials in the sum grouped into a binomial);
// the sign of CG is the sign of S.
double clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM)
{
    if (tm1 + tm2 != tM) return 0.0;
    if (std::abs(tm1) > tj1 || std::abs(tm2) > tj2 || std::abs(tM) > tJ) return 0.0;
    if (tJ > tj1 + tj2 || tJ < std::abs(tj1 - tj2) || ((tj1 + tj2 + tJ) & 1)) return 0.0;
    if (((tj1 + tm1) & 1) || ((tj2 + tm2) & 1) || ((tJ + tM) & 1)) return 0.0;
    // binomials up to C(120, 60) stay inside 128 bits
    ED_REQUIRE(tj1 + tj2 + tJ <= 240, ED_ERR_RANGE, "angular momentum too large (j1+j2+J <= 120)");
    const int a = (tj1 + tj2 - tJ) / 2;
    const int b = (tj1 - tj2 + tJ) / 2;
    const int c = (-tj1 + tj2 + tJ) / 2;
    const int T = (tj1 + tj2 + tJ) / 2;
    const int j1m = (tj1 - tm1) / 2;   // j1 - m1
    const int j2p = (tj2 + tm2) / 2;   // j2 + m2
    const int j2m = (tj2 - tm2) / 2;   // j2 - m2
    const int Jp = (tJ + tM) / 2;      // J + M
    Big pos, neg;
    const int kmin = std::max(0, std::max(j1m - b, j2p - c));
    const int kmax = std::min(a, std::min(j1m, j2p));
    for (int k = kmin; k <= kmax; ++k) {
        Big t = Big::from_u128(binomial_u128(a, k))
                    .mul(Big::from_u128(binomial_u128(b, j1m - k)))
                    .mul(Big::from_u128(binomial_u128(c, j2p - k)));
        if (k & 1) neg.add(t);
        else pos.add(t);
    }
    int sgn = pos.cmp(neg);
    if (sgn == 0) return 0.0;
    Big s = pos;
    if (sgn > 0) s.sub(neg);
    else { s = neg; s.sub(pos); }
    const double sd = s.to_double();
    const double num = (double)(tJ + 1) * (double)binomial_u128(tj1, a) * (double)binomial_u128(tj2, c);
    const double den = (double)(T + 1) * (double)binomial_u128(T, a) * (double)binomial_u128(tJ, Jp) *
                       (double)binomial_u128(tj1, j1m) * (double)binomial_u128(tj2, j2m);
    double v = sd * std::sqrt(num / den);
    if (sgn < 0) v = -v;
    if (std::fabs(v) <= kCgEps) return 0.0;
    return v;
}

// V_m = 2/sqrt(S) C(4S-2L, 2S-L) C(4S+2L+2, 2S+L+1) / C(4S+2, 2S+1)^2 at
// index 2S-L (coulomb_pseudopotentials.cpp:60-67), with the binomials held
// exactly in multiword integers and one division in double.
void coulomb_pseudopotentials(int norb, double* out)
{
    ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals, ED_ERR_RANGE, "norb out of range");
    const int maxLz = norb - 1;
    auto bigbin = [](int n, int k) {
        // C(n,k) by the product formula in multiword integers
        Big r = Big::from_u128(1);
        if (k > n - k) k = n - k;
        for (int i = 1; i <= k; ++i) {
            r = r.mul(Big::from_u128((u128)(n - k + i)));
            // exact division by i
            uint64_t rem = 0;
            for (int l = Big::L - 1; l >= 0; --l) {
                uint64_t cur = (rem << 32) | r.w[l];
                r.w[l] = (uint32_t)(cur / (uint64_t)i);
                rem = cur % (uint64_t)i;
            }
        }
        return r;
    };
    Big den = bigbin(2 * maxLz + 2, maxLz + 1);
    den = den.mul(den);
    const double dd = den.to_double();
    for (int L = 0; L <= maxLz; ++L) {
        Big num = bigbin(2 * maxLz - 2 * L, maxLz - L).mul(bigbin(2 * maxLz + 2 * L + 2, maxLz + L + 1));
        out[maxLz - L] = 2.0 / std::sqrt((double)maxLz / 2.0) * (num.to_double() / dd);
    }
}

namespace {

// CG(maxLz/2, m1; maxLz/2, m2 | Lact, m1+m2) for every (k1, k2) and every
// l = 0..norb-2 (Lact = 2 maxLz - 2 l), indexed ((k1*K + k2)*(K-1) + l).  The
// values depend only on the orbital count, so each table is computed once per
// process and shared by every later call (sweeps build many V tables per K).
const std::vector<double>& cg_table(int norb)
{
    static std::mutex mu;
    static std::map<int, std::vector<double>> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(norb);
    if (it != cache.end()) return it->second;
    const int maxLz = norb - 1, K = norb, NL = std::max(norb - 1, 1);
    std::vector<double> cg((size_t)K * K * NL, 0.0);
    for (int k1 = 0; k1 < K; ++k1)
        for (int k2 = 0; k2 < K; ++k2)
            for (int l = 0; l < norb - 1; ++l) {
                const int m1 = maxLz - 2 * k1, m2 = maxLz - 2 * k2;
                const int lact = 2 * maxLz - 2 * l;
                const int M = m1 + m2;
                double v = 0.0;
                if (-lact <= M && M <= lact) v = clebsch_gordan(maxLz, m1, maxLz, m2, lact, M);
                cg[((size_t)k1 * K + k2) * NL + l] = v;
            }
    return cache.emplace(norb, std::move(cg)).first->second;
}

}  // namespace

// pseudopotential_model_base.hpp:62-229 for one Landau level (maxLz2 =
// maxLz, so FindM1's error code maxLz+2 converts to k = 65535).
void quartic_tables(int norb, const double* pp, int npp, uint16_t* ktab, double* vtab)
{
    ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals, ED_ERR_RANGE, "norb out of range");
    ED_REQUIRE(npp >= 0 && npp <= norb - 1, ED_ERR_ARG,
               "too many two-body pseudopotential coefficients (at most 2S = norb-1)");
    const int maxLz = norb - 1;
    const int K = norb;
    const std::vector<double>& cg = cg_table(norb);
    const int NL = std::max(norb - 1, 1);
    size_t it = 0;
    for (int m4 = maxLz; m4 >= -maxLz; m4 -= 2) {
        for (int m3 = maxLz; m3 >= -maxLz; m3 -= 2) {
            for (int m2 = maxLz; m2 >= -maxLz; m2 -= 2, ++it) {
                int m1 = m3 + m4 - m2;
                const bool ok = (m1 <= maxLz && m1 >= -maxLz);
                const int m1e = ok ? m1 : maxLz + 2;
                ktab[it] = (uint16_t)((-m1e + maxLz) / 2);
                double total = 0.0;
                if (ok) {
                    const int k1 = (maxLz - m1) / 2, k2 = (maxLz - m2) / 2;
                    const int k3 = (maxLz - m3) / 2, k4 = (maxLz - m4) / 2;
                    const int M = m1 + m2;
                    for (int l = 0; l < npp; ++l) {
                        double temp = 0.0;
                        const int lact = 2 * maxLz - 2 * l;
                        if (-lact <= M && M <= lact) {
                            temp += cg[((size_t)k1 * K + k2) * NL + l] * cg[((size_t)k3 * K + k4) * NL + l];
                        }
                        total -= pp[l] * temp;
                    }
                }
                vtab[it] = total;
            }
        }
    }
}

HopTables derive_hop_tables(int norb, const uint16_t* ktab, const double* vtab)
{
    const int K = norb;
    ED_REQUIRE(K >= 2 && K <= kMaxOrbitals, ED_ERR_RANGE, "norb out of range for the device path");
    // The device build enumerates pair hops with a+b = c+d; accept only the
    // momentum-conserving k-table that the sphere model produces.
    for (int k4 = 0; k4 < K; ++k4)
        for (int k3 = 0; k3 < K; ++k3)
            for (int k2 = 0; k2 < K; ++k2) {
                const int k1 = k3 + k4 - k2;
                const uint16_t want = (k1 >= 0 && k1 < K) ? (uint16_t)k1 : (uint16_t)0;
                const uint16_t got = ktab[((size_t)k4 * K + k3) * K + k2];
                const bool in_range = k1 >= 0 && k1 < K;
                ED_REQUIRE(in_range ? got == want : got >= K, ED_ERR_ARG,
                           "k-table is not the momentum-conserving table k1 = k3 + k4 - k2");
            }
    HopTables h;
    h.K = K;
    h.hop_off.assign(2 * K, 0);
    int off = 0;
    for (int s = 0; s < 2 * K; ++s) {
        h.hop_off[s] = off;
        const int c = pair_cnt(s, K);
        off += c * c;
    }
    h.w.assign(off, 0.0);
    auto V = [&](int k4, int k3, int k2) { return vtab[((size_t)k4 * K + k3) * K + k2]; };
    auto filt = [](double x) { return std::fabs(x) > kSparseZeroTol ? x : 0.0; };
    for (int s = 1; s <= 2 * K - 3; ++s) {
        const int lo = pair_lo(s, K), cnt = pair_cnt(s, K);
        for (int ia = 0; ia < cnt; ++ia) {
            const int a = lo + ia, b = s - a;      // removed pair, a < b
            for (int ic = 0; ic < cnt; ++ic) {
                if (ic == ia) continue;
                const int c = lo + ic, d = s - c;  // created pair, c < d
                // terms in visiting order: k4=a,k3=b (k2=c then k2=d), then
                // k4=b,k3=a (k2=c then k2=d); relative signs +,-,-,+ (swapping
                // k1<->k2 or k3<->k4 flips the fermionic sign)
                double acc = 0.0;
                acc = acc + filt(V(a, b, c));
                acc = acc + (-filt(V(a, b, d)));
                acc = acc + (-filt(V(b, a, c)));
                acc = acc + filt(V(b, a, d));
                h.w[h.hop_off[s] + ia * cnt + ic] = (std::fabs(acc) < kSparseZeroTol) ? 0.0 : acc;
            }
        }
    }
    h.diag_a.assign((size_t)K * K, 0.0);
    h.diag_b.assign((size_t)K * K, 0.0);
    for (int k4 = 0; k4 < K; ++k4)
        for (int k3 = 0; k3 < K; ++k3) {
            if (k3 == k4) continue;
            const double tA = filt(V(k4, k3, k3));      // k2 = k3, k1 = k4: sign +1
            const double tB = -filt(V(k4, k3, k4));     // k2 = k4, k1 = k3: sign -1
            const bool k3_first = k3 < k4;              // k2 runs upward
            h.diag_a[(size_t)k4 * K + k3] = k3_first ? tA : tB;
            h.diag_b[(size_t)k4 * K + k3] = k3_first ? tB : tA;
        }
    return h;
}

}  // namespace edgb
