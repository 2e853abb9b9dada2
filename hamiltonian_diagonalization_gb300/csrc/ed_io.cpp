// File formats of the reference, so that results and inputs move between a
// reference run and this engine (host code).
//
//  - Eigensystem files: HamiltonianBase::EigensystemToFile / EigensystemFromFile
//    (hamiltonians/hamiltonian_base.hpp:1204-1304, 1309-1400).  Text:
//      "##  NBR EIGENVALUES", nev, "##  EIGENVALUES", nev values, then
//      optionally "##  FOCK SPACE DIMENSION", dim, "##  EIGENVECTORS" and the
//      nev*dim vector entries, one per line, every number at
//      std::setprecision(15) (utilities/wrappers/io_wrapper.hpp:77-92).
//    Binary: uint32 nev, nev doubles, then optionally uint32 dim and the
//    nev*dim entries.
//  - CRS files: CrsSparseMatrix::ToFile / FromFile
//    (utilities/data_structures/crs_sparse_matrix.hpp:662-740).  Text: nnz,
//    n, the n row starts (without the final one), then "row col value" per
//    element.  Binary: uint32 nnz, uint32 n, n+1 int32 row starts, nnz int32
//    columns, nnz doubles.  The reference's text reader takes the missing
//    final row start as 0 and so drops the last row; the reader here takes it
//    as nnz.
//  - Quartic term-table files: TermTablesBase::ToFileBase / FromFileBase
//    (hamiltonians/term_tables_base.hpp:179-335) with 4 labels.  Binary:
//    uint32 header length, the header text, uint32 label count (4), kMax in a
//    4-byte field (the reference writes its uint16 kMax with sizeof(iSize_t);
//    here the upper two bytes are zero), the K^3 uint16 k-table and the K^3
//    double V-table.  Text: the header line, 4, kMax, then "k1 k2 k3 k4 V"
//    tab-separated in k4, k3, k2 order, k1 = the table entry (65535 where no
//    k1 exists) and V the table value.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "ed_internal.h"

namespace edgb {

namespace {

const char* kTableHeader = "# File contains term table data in array format";

std::ofstream open_out(const char* path, int binary)
{
    std::ofstream f(path, binary ? (std::ios::out | std::ios::binary) : std::ios::out);
    ED_REQUIRE(f.is_open(), ED_ERR_ARG, std::string("could not open file ") + path);
    return f;
}

std::ifstream open_in(const char* path, int binary)
{
    std::ifstream f(path, binary ? (std::ios::in | std::ios::binary) : std::ios::in);
    ED_REQUIRE(f.is_open(), ED_ERR_ARG, std::string("could not open file ") + path);
    return f;
}

std::string num15(double v)
{
    std::stringstream ss;
    ss << std::setprecision(15) << v;
    return ss.str();
}

void skip_to(std::ifstream& f, const char* marker)
{
    std::string line;
    while (std::getline(f, line))
        if (line == marker) return;
    throw Error(ED_ERR_ARG, std::string("marker not found in file: ") + marker);
}

template <class T>
void read_raw(std::ifstream& f, T* p, size_t count)
{
    f.read(reinterpret_cast<char*>(p), (std::streamsize)(count * sizeof(T)));
    ED_REQUIRE(f.good() || (f.eof() && (size_t)f.gcount() == count * sizeof(T)), ED_ERR_ARG, "file is truncated");
}

}  // namespace

}  // namespace edgb

using namespace edgb;

extern "C" {

ed_status ed_eigensystem_write(const char* path, int binary, int nev, const double* evals, uint64_t dim,
                               const double* evecs)
{
    return guard([&] {
        ED_REQUIRE(path && evals && nev >= 1, ED_ERR_ARG, "bad argument");
        ED_REQUIRE(!evecs || (dim >= 1 && dim <= std::numeric_limits<uint32_t>::max()), ED_ERR_RANGE,
                   "the file format stores the dimension in 32 bits");
        std::ofstream f = open_out(path, binary);
        if (binary) {
            const uint32_t k = (uint32_t)nev;
            f.write(reinterpret_cast<const char*>(&k), 4);
            f.write(reinterpret_cast<const char*>(evals), (std::streamsize)nev * 8);
            if (evecs) {
                const uint32_t d = (uint32_t)dim;
                f.write(reinterpret_cast<const char*>(&d), 4);
                f.write(reinterpret_cast<const char*>(evecs), (std::streamsize)(dim * (uint64_t)nev * 8));
            }
        } else {
            f << "##  NBR EIGENVALUES\n" << nev << "\n" << "##  EIGENVALUES\n";
            for (int i = 0; i < nev; ++i) f << std::setprecision(15) << evals[i] << "\n";
            if (evecs) {
                f << "##  FOCK SPACE DIMENSION\n" << dim << "\n" << "##  EIGENVECTORS\n";
                for (uint64_t j = 0; j < dim * (uint64_t)nev; ++j) f << num15(evecs[j]) << "\n";
            }
        }
        ED_REQUIRE(f.good(), ED_ERR_ARG, "write failed");
    });
}

ed_status ed_eigensystem_read(const char* path, int binary, int* nev, double* evals, uint64_t* dim, double* evecs)
{
    return guard([&] {
        ED_REQUIRE(path && nev && dim, ED_ERR_ARG, "bad argument");
        std::ifstream f = open_in(path, binary);
        uint32_t k = 0, d = 0;
        std::vector<double> ev;
        if (binary) {
            read_raw(f, &k, 1);
            ev.resize(k);
            read_raw(f, ev.data(), k);
            if (f.read(reinterpret_cast<char*>(&d), 4)) {
                if (evecs) read_raw(f, evecs, (size_t)d * k);
            } else {
                d = 0;
            }
        } else {
            skip_to(f, "##  NBR EIGENVALUES");
            f >> k;
            skip_to(f, "##  EIGENVALUES");
            ev.resize(k);
            for (uint32_t i = 0; i < k; ++i) f >> ev[i];
            ED_REQUIRE(!f.fail(), ED_ERR_ARG, "bad eigenvalue list");
            std::string line;
            d = 0;
            while (std::getline(f, line))
                if (line == "##  FOCK SPACE DIMENSION") {
                    f >> d;
                    skip_to(f, "##  EIGENVECTORS");
                    if (evecs)
                        for (uint64_t j = 0; j < (uint64_t)d * k; ++j) f >> evecs[j];
                    ED_REQUIRE(!f.fail(), ED_ERR_ARG, "bad eigenvector list");
                    break;
                }
        }
        *nev = (int)k;
        *dim = d;
        if (evals) std::memcpy(evals, ev.data(), (size_t)k * 8);
    });
}

ed_status ed_crs_write(const ed_crs* a, const char* path, int binary)
{
    return guard([&] {
        ED_REQUIRE(a && path, ED_ERR_ARG, "bad argument");
        ED_REQUIRE(a->nnz <= (int64_t)std::numeric_limits<int32_t>::max() &&
                       a->n <= (int64_t)std::numeric_limits<int32_t>::max(),
                   ED_ERR_RANGE, "the reference's CRS file format indexes with int32");
        std::vector<int64_t> rp(a->n + 1);
        std::vector<int32_t> col(a->nnz);
        std::vector<double> val(a->nnz);
        ED_CUDA(cudaMemcpy(rp.data(), a->rowptr.p, rp.size() * 8, cudaMemcpyDeviceToHost));
        ED_CUDA(cudaMemcpy(col.data(), a->col.p, col.size() * 4, cudaMemcpyDeviceToHost));
        ED_CUDA(cudaMemcpy(val.data(), a->val.p, val.size() * 8, cudaMemcpyDeviceToHost));
        std::ofstream f = open_out(path, binary);
        if (binary) {
            const uint32_t nnz = (uint32_t)a->nnz, n = (uint32_t)a->n;
            std::vector<int32_t> rs(rp.begin(), rp.end());
            f.write(reinterpret_cast<const char*>(&nnz), 4);
            f.write(reinterpret_cast<const char*>(&n), 4);
            f.write(reinterpret_cast<const char*>(rs.data()), (std::streamsize)rs.size() * 4);
            f.write(reinterpret_cast<const char*>(col.data()), (std::streamsize)col.size() * 4);
            f.write(reinterpret_cast<const char*>(val.data()), (std::streamsize)val.size() * 8);
        } else {
            f << a->nnz << "\n" << a->n << "\n";
            for (int64_t i = 0; i < a->n; ++i) f << rp[i] << "\n";
            for (int64_t i = 0; i < a->n; ++i)
                for (int64_t j = rp[i]; j < rp[i + 1]; ++j) f << i << " " << col[j] << " " << num15(val[j]) << "\n";
        }
        ED_REQUIRE(f.good(), ED_ERR_ARG, "write failed");
    });
}

ed_status ed_crs_read(const char* path, int binary, int upper, ed_crs** out)
{
    return guard([&] {
        ED_REQUIRE(path && out, ED_ERR_ARG, "bad argument");
        *out = nullptr;
        std::ifstream f = open_in(path, binary);
        uint32_t nnz = 0, n = 0;
        std::vector<int64_t> rp;
        std::vector<int32_t> col;
        std::vector<double> val;
        if (binary) {
            read_raw(f, &nnz, 1);
            read_raw(f, &n, 1);
            std::vector<int32_t> rs(n + 1);
            read_raw(f, rs.data(), rs.size());
            rp.assign(rs.begin(), rs.end());
            col.resize(nnz);
            val.resize(nnz);
            read_raw(f, col.data(), nnz);
            read_raw(f, val.data(), nnz);
        } else {
            f >> nnz >> n;
            rp.resize(n + 1);
            for (uint32_t i = 0; i < n; ++i) f >> rp[i];
            rp[n] = nnz;   // not in the text format
            col.resize(nnz);
            val.resize(nnz);
            for (uint32_t i = 0; i < n; ++i)
                for (int64_t j = rp[i]; j < rp[i + 1]; ++j) {
                    int64_t row = 0;
                    f >> row >> col[j] >> val[j];
                    ED_REQUIRE(row == (int64_t)i, ED_ERR_ARG, "CRS file: element listed under the wrong row");
                }
            ED_REQUIRE(!f.fail(), ED_ERR_ARG, "CRS file: bad element list");
        }
        for (uint32_t i = 0; i < n; ++i)
            ED_REQUIRE(rp[i] <= rp[i + 1] && rp[i + 1] <= (int64_t)nnz, ED_ERR_ARG, "CRS file: bad row starts");
        for (uint32_t j = 0; j < nnz; ++j)
            ED_REQUIRE(col[j] >= 0 && (uint32_t)col[j] < n, ED_ERR_ARG, "CRS file: column out of range");
        ed_crs* a = new ed_crs();
        try {
            a->n = n;
            a->nnz = nnz;
            a->upper = upper ? 1 : 0;
            int64_t mr = 0;
            for (uint32_t i = 0; i < n; ++i) mr = std::max<int64_t>(mr, rp[i + 1] - rp[i]);
            a->max_row = (int)mr;
            a->rowptr.alloc(n + 1);
            a->col.alloc((size_t)nnz + kCrsPad);
            a->val.alloc((size_t)nnz + kCrsPad);
            ED_CUDA(cudaMemcpy(a->rowptr.p, rp.data(), rp.size() * 8, cudaMemcpyHostToDevice));
            ED_CUDA(cudaMemcpy(a->col.p, col.data(), (size_t)nnz * 4, cudaMemcpyHostToDevice));
            ED_CUDA(cudaMemcpy(a->val.p, val.data(), (size_t)nnz * 8, cudaMemcpyHostToDevice));
            ED_CUDA(cudaMemset(a->col.p + nnz, 0, kCrsPad * 4));
            ED_CUDA(cudaMemset(a->val.p + nnz, 0, kCrsPad * 8));
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

ed_status ed_quartic_tables_write(const char* path, int binary, int norb, const uint16_t* ktable,
                                  const double* vtable)
{
    return guard([&] {
        ED_REQUIRE(path && ktable && vtable && norb >= 1 && norb < 65535, ED_ERR_ARG, "bad argument");
        const size_t K3 = (size_t)norb * norb * norb;
        std::ofstream f = open_out(path, binary);
        const std::string header = kTableHeader;
        if (binary) {
            const uint32_t len = (uint32_t)header.size(), labels = 4, kmax = (uint32_t)norb;
            f.write(reinterpret_cast<const char*>(&len), 4);
            f.write(header.data(), len);
            f.write(reinterpret_cast<const char*>(&labels), 4);
            f.write(reinterpret_cast<const char*>(&kmax), 4);
            f.write(reinterpret_cast<const char*>(ktable), (std::streamsize)(K3 * 2));
            f.write(reinterpret_cast<const char*>(vtable), (std::streamsize)(K3 * 8));
        } else {
            f << header << "\n" << 4 << "\n" << norb << "\n";
            for (int k4 = 0; k4 < norb; ++k4)
                for (int k3 = 0; k3 < norb; ++k3)
                    for (int k2 = 0; k2 < norb; ++k2) {
                        const size_t i = ((size_t)k4 * norb + k3) * norb + k2;
                        f << ktable[i] << "\t" << k2 << "\t" << k3 << "\t" << k4 << "\t" << num15(vtable[i]) << "\n";
                    }
        }
        ED_REQUIRE(f.good(), ED_ERR_ARG, "write failed");
    });
}

ed_status ed_quartic_tables_read(const char* path, int binary, int* norb, uint16_t* ktable, double* vtable)
{
    return guard([&] {
        ED_REQUIRE(path && norb, ED_ERR_ARG, "bad argument");
        std::ifstream f = open_in(path, binary);
        uint32_t labels = 0, kmax = 0;
        std::string header;
        if (binary) {
            uint32_t len = 0;
            read_raw(f, &len, 1);
            ED_REQUIRE(len < (1u << 20), ED_ERR_ARG, "term-table file: bad header length");
            header.resize(len);
            if (len) read_raw(f, &header[0], len);
            ED_REQUIRE(header == kTableHeader, ED_ERR_ARG, "term-table file: wrong file header");
            read_raw(f, &labels, 1);
            read_raw(f, &kmax, 1);
            kmax &= 0xFFFFu;   // a 16-bit value in a 4-byte field
            ED_REQUIRE(labels == 4, ED_ERR_ARG, "not a quartic term table (label count != 4)");
            const size_t K3 = (size_t)kmax * kmax * kmax;
            if (ktable && vtable) {
                read_raw(f, ktable, K3);
                read_raw(f, vtable, K3);
            }
        } else {
            std::getline(f, header);
            ED_REQUIRE(header == kTableHeader, ED_ERR_ARG, "term-table file: wrong file header");
            f >> labels >> kmax;
            ED_REQUIRE(labels == 4, ED_ERR_ARG, "not a quartic term table (label count != 4)");
            if (ktable && vtable) {
                for (uint32_t k4 = 0; k4 < kmax; ++k4)
                    for (uint32_t k3 = 0; k3 < kmax; ++k3)
                        for (uint32_t k2 = 0; k2 < kmax; ++k2) {
                            const size_t i = ((size_t)k4 * kmax + k3) * kmax + k2;
                            unsigned k1 = 0, a = 0, b = 0, c = 0;
                            f >> k1 >> a >> b >> c >> vtable[i];
                            ktable[i] = (uint16_t)k1;
                        }
                ED_REQUIRE(!f.fail(), ED_ERR_ARG, "term-table file: bad entry list");
            }
        }
        *norb = (int)kmax;
    });
}

}  // extern "C"
