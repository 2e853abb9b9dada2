// Term tables of the optical-flux-lattice model in the reference's hash-table
// format (host code): the file layout, and the conversion of
// momentum-conserving hash tables into the array tables the device build
// reads.
//
// Reference: TermHashTables<dcmplx> (hamiltonians/term_hash_tables_base.hpp:
// 44-276) over MultiHashMap / MultiHashMultiMap
// (utilities/data_structures/multi_key_hash.hpp:480-682), with
// QuarticTermHashTables (4 labels) and QuadraticTermHashTables (2 labels)
// (optical_flux_lattice/interacting_ofl_model/term_hash_tables.cpp).
//  - Keys pack the labels as the reference's utilities::Key does
//    (multi_key_hash.hpp:59-92, general/serialize.hpp:96-130): two labels
//    (k1 << 32) | k2, three labels (k2 << 48) | (k3 << 32) | (k4 << 16), four
//    labels (k1 << 48) | (k2 << 32) | (k3 << 16) | k4.
//  - A file is the header line "# File contains term table data in hash
//    table format", then the k-table (keys of nlabels - 1 labels, each with
//    one k1 value; a key may repeat) and the value table (keys of nlabels
//    labels, complex values).  Binary: uint32 header length and the header
//    bytes, then per table uint32 count, count uint64 keys and count values
//    (uint16 k1 values, then (re, im) double pairs).  Text: the header line,
//    then per table the count and the label count on lines of their own and
//    one line per entry, its labels and value tab-separated, numbers at
//    std::setprecision(15) (utilities/wrappers/io_wrapper.hpp:77-92), so a
//    text file keeps 15 significant digits of each value.
//  - The reference fills hash tables from its arrays by SetQuarticFromArray /
//    SetQuadraticFromArray (term_hash_tables_base.hpp:229-275): every
//    (k2, k3, k4) gets the one k1 the momentum rule gives and V(k1, k2, k3, k4),
//    every k2 gets k1 = k2 and E(k2, k2).  ed_cterms_create_hash reverses that:
//    one k1 per (k2, k3, k4), a diagonal quadratic table (an off-diagonal
//    one-body term, as in the reference's Wannier basis, conserves no
//    momentum), and values that the array layout can hold (one slot serves
//    V(k1, k2, k3 < k4) at index k1 and V(k1', k2', k4, k3) at index k2').
#include <algorithm>
#include <complex>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "ed_internal.h"

namespace edgb {

namespace {

const char* kHashHeader = "# File contains term table data in hash table format";

uint64_t pack2x32(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | (uint64_t)b; }
uint64_t pack4x16(uint16_t a, uint16_t b, uint16_t c, uint16_t d)
{
    return ((uint64_t)a << 48) | ((uint64_t)b << 32) | ((uint64_t)c << 16) | (uint64_t)d;
}

std::string num15(double v)
{
    std::stringstream ss;
    ss << std::setprecision(15) << v;
    return ss.str();
}

// the key's labels, written as the reference's ToFileBase does for nbrLabels
void write_labels(std::ofstream& f, uint64_t key, int labels)
{
    switch (labels) {
    case 1: f << key; break;
    case 2: f << (uint32_t)(key >> 32) << "\t" << (uint32_t)(key & 0xFFFFFFFFu); break;
    case 3: f << ((key >> 48) & 0xFFFF) << "\t" << ((key >> 32) & 0xFFFF) << "\t" << ((key >> 16) & 0xFFFF); break;
    default:
        f << ((key >> 48) & 0xFFFF) << "\t" << ((key >> 32) & 0xFFFF) << "\t" << ((key >> 16) & 0xFFFF) << "\t"
          << (key & 0xFFFF);
        break;
    }
}

uint64_t read_labels(std::ifstream& f, uint64_t labels)
{
    switch (labels) {
    case 1: {
        uint64_t k = 0;
        f >> k;
        return k;
    }
    case 2: {
        uint32_t a = 0, b = 0;
        f >> a >> b;
        return pack2x32(a, b);
    }
    case 3: {
        uint32_t a = 0, b = 0, c = 0;
        f >> a >> b >> c;
        ED_REQUIRE(a <= 0xFFFF && b <= 0xFFFF && c <= 0xFFFF, ED_ERR_ARG, "hash-table file: label beyond 16 bits");
        return pack4x16((uint16_t)a, (uint16_t)b, (uint16_t)c, 0);
    }
    case 4: {
        uint32_t a = 0, b = 0, c = 0, d = 0;
        f >> a >> b >> c >> d;
        ED_REQUIRE(a <= 0xFFFF && b <= 0xFFFF && c <= 0xFFFF && d <= 0xFFFF, ED_ERR_ARG,
                   "hash-table file: label beyond 16 bits");
        return pack4x16((uint16_t)a, (uint16_t)b, (uint16_t)c, (uint16_t)d);
    }
    default: throw Error(ED_ERR_ARG, "hash-table file: label count not 1, 2, 3 or 4");
    }
}

template <class T>
void read_raw(std::ifstream& f, T* p, size_t count)
{
    if (count == 0) return;
    f.read(reinterpret_cast<char*>(p), (std::streamsize)(count * sizeof(T)));
    ED_REQUIRE((size_t)f.gcount() == count * sizeof(T), ED_ERR_ARG, "hash-table file is truncated");
}

struct HashContent {
    std::vector<uint64_t> kkeys, vkeys;
    std::vector<uint16_t> kvals;
    std::vector<double> vvals;   // (re, im) pairs
};

HashContent read_hash_file(const char* path, int binary)
{
    std::ifstream f(path, binary ? (std::ios::in | std::ios::binary) : std::ios::in);
    ED_REQUIRE(f.is_open(), ED_ERR_ARG, std::string("could not open file ") + path);
    HashContent h;
    std::string header;
    if (binary) {
        uint32_t len = 0;
        read_raw(f, &len, 1);
        ED_REQUIRE(len < (1u << 20), ED_ERR_ARG, "hash-table file: bad header length");
        header.resize(len);
        read_raw(f, &header[0], len);
    } else {
        std::getline(f, header);
    }
    ED_REQUIRE(header == kHashHeader, ED_ERR_ARG, "hash-table file: wrong file header " + header);
    if (binary) {
        uint32_t nk = 0;
        read_raw(f, &nk, 1);
        h.kkeys.resize(nk);
        h.kvals.resize(nk);
        read_raw(f, h.kkeys.data(), nk);
        read_raw(f, h.kvals.data(), nk);
        uint32_t nv = 0;
        read_raw(f, &nv, 1);
        h.vkeys.resize(nv);
        h.vvals.resize(2 * (size_t)nv);
        read_raw(f, h.vkeys.data(), nv);
        read_raw(f, h.vvals.data(), 2 * (size_t)nv);
    } else {
        uint64_t nk = 0, kl = 0;
        f >> nk >> kl;
        ED_REQUIRE(!f.fail() && nk < (1ull << 32), ED_ERR_ARG, "hash-table file: bad k-table size");
        h.kkeys.resize(nk);
        h.kvals.resize(nk);
        for (uint64_t i = 0; i < nk; ++i) {
            h.kkeys[i] = read_labels(f, kl);
            uint32_t v = 0;
            f >> v;
            ED_REQUIRE(v <= 0xFFFF, ED_ERR_ARG, "hash-table file: k value beyond 16 bits");
            h.kvals[i] = (uint16_t)v;
        }
        uint64_t nv = 0, vl = 0;
        f >> nv >> vl;
        ED_REQUIRE(!f.fail() && nv < (1ull << 32), ED_ERR_ARG, "hash-table file: bad value-table size");
        h.vkeys.resize(nv);
        h.vvals.resize(2 * nv);
        for (uint64_t i = 0; i < nv; ++i) {
            h.vkeys[i] = read_labels(f, vl);
            f >> h.vvals[2 * i] >> h.vvals[2 * i + 1];
        }
        ED_REQUIRE(!f.fail(), ED_ERR_ARG, "hash-table file: bad entry list");
    }
    return h;
}

}  // namespace

}  // namespace edgb

using namespace edgb;

extern "C" {

ed_status ed_term_hash_write(const char* path, int binary, int nlabels, uint32_t nk, const uint64_t* kkeys,
                             const uint16_t* kvals, uint32_t nv, const uint64_t* vkeys, const double* vvals)
{
    return guard([&] {
        ED_REQUIRE(path, ED_ERR_ARG, "path must not be NULL");
        ED_REQUIRE(nlabels == 2 || nlabels == 4, ED_ERR_ARG, "nlabels: 2 (quadratic) or 4 (quartic)");
        ED_REQUIRE((nk == 0 || (kkeys && kvals)) && (nv == 0 || (vkeys && vvals)), ED_ERR_ARG, "NULL table");
        std::ofstream f(path, binary ? (std::ios::out | std::ios::binary) : std::ios::out);
        ED_REQUIRE(f.is_open(), ED_ERR_ARG, std::string("could not open file ") + path);
        const std::string header = kHashHeader;
        if (binary) {
            const uint32_t len = (uint32_t)header.size();
            f.write(reinterpret_cast<const char*>(&len), 4);
            f.write(header.data(), len);
            f.write(reinterpret_cast<const char*>(&nk), 4);
            f.write(reinterpret_cast<const char*>(kkeys), (std::streamsize)nk * 8);
            f.write(reinterpret_cast<const char*>(kvals), (std::streamsize)nk * 2);
            f.write(reinterpret_cast<const char*>(&nv), 4);
            f.write(reinterpret_cast<const char*>(vkeys), (std::streamsize)nv * 8);
            f.write(reinterpret_cast<const char*>(vvals), (std::streamsize)nv * 16);
        } else {
            f << header << "\n";
            f << nk << "\n" << nlabels - 1 << "\n";
            for (uint32_t i = 0; i < nk; ++i) {
                write_labels(f, kkeys[i], nlabels - 1);
                f << "\t" << kvals[i] << "\n";
            }
            f << nv << "\n" << nlabels << "\n";
            for (uint32_t i = 0; i < nv; ++i) {
                write_labels(f, vkeys[i], nlabels);
                f << "\t" << num15(vvals[2 * i]) << "\t" << num15(vvals[2 * i + 1]) << "\n";
            }
        }
        ED_REQUIRE(f.good(), ED_ERR_ARG, std::string("error writing ") + path);
    });
}

ed_status ed_term_hash_read(const char* path, int binary, uint32_t* nk, uint64_t* kkeys, uint16_t* kvals,
                            uint32_t* nv, uint64_t* vkeys, double* vvals)
{
    return guard([&] {
        ED_REQUIRE(path && nk && nv, ED_ERR_ARG, "path, nk and nv must not be NULL");
        const HashContent h = read_hash_file(path, binary);
        const bool fill = kkeys || kvals || vkeys || vvals;
        if (fill) {
            ED_REQUIRE(*nk >= h.kkeys.size() && *nv >= h.vkeys.size(), ED_ERR_RANGE,
                       "hash-table file holds more entries than the buffers");
            ED_REQUIRE((h.kkeys.empty() || (kkeys && kvals)) && (h.vkeys.empty() || (vkeys && vvals)), ED_ERR_ARG,
                       "NULL buffer");
            std::copy(h.kkeys.begin(), h.kkeys.end(), kkeys);
            std::copy(h.kvals.begin(), h.kvals.end(), kvals);
            std::copy(h.vkeys.begin(), h.vkeys.end(), vkeys);
            std::copy(h.vvals.begin(), h.vvals.end(), vvals);
        }
        *nk = (uint32_t)h.kkeys.size();
        *nv = (uint32_t)h.vkeys.size();
    });
}

ed_status ed_cterms_create_hash(int norb, int dimX, int dimY, uint32_t nk, const uint64_t* kkeys,
                                const uint16_t* kvals, uint32_t nv, const uint64_t* vkeys, const double* vvals,
                                uint32_t nqk, const uint64_t* qkkeys, const uint16_t* qkvals, uint32_t nqv,
                                const uint64_t* qvkeys, const double* qvvals, ed_cterms** out)
{
    return guard([&] {
        ED_REQUIRE(out, ED_ERR_ARG, "out must not be NULL");
        *out = nullptr;
        ED_REQUIRE(norb >= 2 && norb <= kMaxOrbitals && dimX >= 1 && dimY >= 1 && dimX * dimY == norb, ED_ERR_RANGE,
                   "momentum grid: need dimX * dimY = norb in 2..40");
        ED_REQUIRE((nk == 0 || (kkeys && kvals)) && (nv == 0 || (vkeys && vvals)) &&
                       (nqk == 0 || (qkkeys && qkvals)) && (nqv == 0 || (qvkeys && qvvals)),
                   ED_ERR_ARG, "NULL table");
        const int K = norb;
        // the k-table as a multimap, the values as a map (a repeated value key
        // keeps its first entry, as std::unordered_map::insert does)
        std::unordered_map<uint64_t, std::vector<uint16_t>> kmap;
        kmap.reserve(nk);
        for (uint32_t i = 0; i < nk; ++i) kmap[kkeys[i]].push_back(kvals[i]);
        std::unordered_map<uint64_t, std::complex<double>> vmap;
        vmap.reserve(nv);
        for (uint32_t i = 0; i < nv; ++i) vmap.emplace(vkeys[i], std::complex<double>(vvals[2 * i], vvals[2 * i + 1]));
        auto k1_of = [&](int k2, int k3, int k4) -> int {
            auto it = kmap.find(pack4x16((uint16_t)k2, (uint16_t)k3, (uint16_t)k4, 0));
            ED_REQUIRE(it != kmap.end(), ED_ERR_ARG,
                       "hash tables lack the k1 of (k2, k3, k4) = (" + std::to_string(k2) + ", " + std::to_string(k3) +
                           ", " + std::to_string(k4) + ")");
            ED_REQUIRE(it->second.size() == 1, ED_ERR_ARG,
                       "more than one k1 for one (k2, k3, k4): not a momentum-conserving table");
            ED_REQUIRE(it->second[0] < K, ED_ERR_ARG, "k1 beyond the orbital count");
            return it->second[0];
        };
        auto v_of = [&](int k1, int k2, int k3, int k4, bool& found) {
            auto it = vmap.find(pack4x16((uint16_t)k1, (uint16_t)k2, (uint16_t)k3, (uint16_t)k4));
            found = it != vmap.end();
            return found ? it->second : std::complex<double>(0.0, 0.0);
        };
        const size_t tdim = (size_t)(K + 1) * K * K / 2;
        std::vector<uint16_t> ktab(tdim, 0);
        std::vector<double> vtab(2 * tdim, 0.0);
        std::vector<char> set(tdim, 0);
        for (int t1 = 0; t1 < K; ++t1)
            for (int t2 = t1; t2 < K; ++t2) {
                const size_t t = (size_t)t1 * K + t2 - (size_t)t1 * (t1 + 1) / 2;
                for (int k2 = 0; k2 < K; ++k2) {
                    // the ordering (k3, k4) = (t2, t1) reads slot k2
                    const int k1 = k1_of(k2, t2, t1);
                    if (t1 != t2)
                        ED_REQUIRE(k1_of(k2, t1, t2) == k1, ED_ERR_ARG,
                                   "k1 of (k2, k3, k4) and (k2, k4, k3) differ: not a momentum-conserving table");
                    ktab[t * K + k2] = (uint16_t)k1;
                    bool found = false;
                    const std::complex<double> v = v_of(k1, k2, t2, t1, found);
                    vtab[2 * (t * K + k2)] = v.real();
                    vtab[2 * (t * K + k2) + 1] = v.imag();
                    set[t * K + k2] = found ? 1 : 0;
                }
                if (t1 == t2) continue;
                // the ordering (k3, k4) = (t1, t2) reads slot k1: the same slot
                // must hold the same value
                for (int k2 = 0; k2 < K; ++k2) {
                    const int k1 = ktab[t * K + k2];
                    bool found = false;
                    const std::complex<double> v = v_of(k1, k2, t1, t2, found);
                    if (!found) continue;
                    const size_t s = t * K + k1;
                    if (!set[s]) {
                        vtab[2 * s] = v.real();
                        vtab[2 * s + 1] = v.imag();
                        set[s] = 1;
                    } else {
                        ED_REQUIRE(vtab[2 * s] == v.real() && vtab[2 * s + 1] == v.imag(), ED_ERR_ARG,
                                   "V(k1, k2, k3, k4) and V(k1', k2', k4, k3) share an array slot with different "
                                   "values: the tables do not have the array format's symmetry");
                    }
                }
            }
        // occupation energies from the quadratic tables
        std::vector<double> e;
        if (nqk || nqv) {
            e.assign(2 * (size_t)K, 0.0);
            for (uint32_t i = 0; i < nqk; ++i) {
                ED_REQUIRE(qkkeys[i] < (uint64_t)K, ED_ERR_ARG, "quadratic k2 beyond the orbital count");
                ED_REQUIRE(qkvals[i] == qkkeys[i], ED_ERR_ARG,
                           "an off-diagonal one-body term (k1 != k2) conserves no momentum");
            }
            for (uint32_t i = 0; i < nqv; ++i) {
                const uint32_t k1 = (uint32_t)(qvkeys[i] >> 32), k2 = (uint32_t)(qvkeys[i] & 0xFFFFFFFFu);
                ED_REQUIRE(k1 < (uint32_t)K && k2 < (uint32_t)K, ED_ERR_ARG, "quadratic label beyond the orbital count");
                if (k1 != k2) {
                    ED_REQUIRE(qvvals[2 * i] == 0.0 && qvvals[2 * i + 1] == 0.0, ED_ERR_ARG,
                               "an off-diagonal one-body term (k1 != k2) conserves no momentum");
                    continue;
                }
                e[2 * k1] = qvvals[2 * i];
                e[2 * k1 + 1] = qvvals[2 * i + 1];
            }
        }
        const ed_status s = ed_cterms_create(norb, dimX, dimY, ktab.data(), vtab.data(), e.empty() ? nullptr : e.data(),
                                             out);
        if (s != ED_OK) throw Error(s, ed_last_error());
    });
}

}  // extern "C"
