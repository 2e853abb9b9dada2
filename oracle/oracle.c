/*
 * CPU oracle for the LLL spinless-fermion exact-diagonalization hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference algorithm (SimonDavenport/hamiltonian_diagonalization) that the
 * tests compare the CUDA library against, and the timed CPU baseline.  Nothing
 * in the shipped library links, loads or calls it.
 *
 * Every function names the reference file:line it restates.  The loops keep
 * the reference's order on purpose (enumeration order of the Fock basis, the
 * k4/k3/k2 loop order of the quartic build, per-element accumulation order),
 * so that the integer outputs and the floating-point sums match the
 * reference's step for step.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MISS UINT64_MAX            /* _SEARCH_ERROR_CODE_ (binary_search.hpp) */
#define OR_SPARSE_ZERO_TOL 1e-14      /* _SPARSE_ZERO_TOL_ (hamiltonian_data.hpp:53) */

/* ---------------------------------------------------------------- bit tools */

/* popcount by repeated x &= x-1: binary_number_tools.cpp:137-144
 * (HammingWeight64Iterative, the variant the reference is built with). */
static inline int or_popcount(uint64_t x)
{
    int c = 0;
    while (x) { x &= x - 1; ++c; }
    return c;
}

/* position of a single set bit: binary_number_tools.cpp:190-195 (Base2Log). */
static inline int or_bitpos(uint64_t onehot)
{
    int p = 0;
    while (onehot > 1) { onehot >>= 1; ++p; }
    return p;
}

/* Binomial coefficient C(n,k) as uint64 (binomials.cpp:34-64 BinomialFromTable
 * returns the same integers for the sizes used here). */
uint64_t or_binomial(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned __int128)(n - k + i) / (unsigned __int128)i;
    return (uint64_t)r;
}

/* Next larger word with the same popcount (Gosper's successor):
 * binary_number_tools.cpp:255-261 (NextHammingNumber64). */
uint64_t or_next_hamming(uint64_t x)
{
    if (x == 0) return 0;
    uint64_t low = x & (~x + 1);
    uint64_t ripple = x + low;
    return (((x ^ ripple) / low) >> 2) | ripple;
}

/* Colex unrank: the index-th word of popcount w in ascending order.
 * binary_number_tools.cpp:297-331 (GenerateHammingNumber). */
uint64_t or_unrank_hamming(int w, uint64_t index)
{
    if (index == 0) return (w >= 64) ? ~0ull : ((1ull << w) - 1ull);
    uint64_t out = 0, acc = 0;
    for (int p = w - 1; p >= 0; --p) {
        int m = p;
        uint64_t inc;
        do { inc = or_binomial(m, p); acc += inc; ++m; } while (index >= acc);
        acc -= inc;
        out |= 1ull << (m - 1);
    }
    return out;
}

/* Lz-sector predicate: sum over occupied bits of (2*bit - maxLz) == twoLz.
 * angular_momentum_constraint.hpp:41-62 (TestAngularMomentumSector). */
int or_lz_ok(uint64_t state, int twoLz, int maxLz)
{
    int acc = 0;
    uint64_t t = state;
    while (t) {
        uint64_t r = t & (~t + 1);
        acc += 2 * or_bitpos(r) - maxLz;
        t ^= r;
    }
    return acc == twoLz;
}

/* -------------------------------------------------------------- Fock basis */

/* Sector basis by a serial scan of all C(norb,N) words in ascending order,
 * keeping those that pass the Lz predicate.  fermion_fock_basis.cpp:241-354
 * (GenerateFockSpace: GenerateHammingNumber for the first word, then
 * NextHammingNumber64).  With out==NULL only counts.  Multi-threaded: the
 * full space is cut into contiguous chunks (the reference's DivideTasks over
 * MPI ranks), each chunk starts from its own unranked first word, and the
 * per-chunk lists are concatenated in chunk order, which is ascending order. */
uint64_t or_basis_build(int N, int norb, int twoLz, uint64_t *out, int nthreads)
{
    const int maxLz = norb - 1;
    const uint64_t full = or_binomial(norb, N);
    if (nthreads < 1) nthreads = 1;
    uint64_t *counts = (uint64_t *)calloc((size_t)nthreads + 1, sizeof(uint64_t));
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
#endif
    for (int t = 0; t < nthreads; ++t) {
        uint64_t first = full * (uint64_t)t / (uint64_t)nthreads;
        uint64_t last = full * (uint64_t)(t + 1) / (uint64_t)nthreads;
        uint64_t w = or_unrank_hamming(N, first), c = 0;
        for (uint64_t i = first; i < last; ++i) {
            if (or_lz_ok(w, twoLz, maxLz)) ++c;
            w = or_next_hamming(w);
        }
        counts[t + 1] = c;
    }
    for (int t = 0; t < nthreads; ++t) counts[t + 1] += counts[t];
    uint64_t total = counts[nthreads];
    if (out) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
#endif
        for (int t = 0; t < nthreads; ++t) {
            uint64_t first = full * (uint64_t)t / (uint64_t)nthreads;
            uint64_t last = full * (uint64_t)(t + 1) / (uint64_t)nthreads;
            uint64_t w = or_unrank_hamming(N, first), pos = counts[t];
            for (uint64_t i = first; i < last; ++i) {
                if (or_lz_ok(w, twoLz, maxLz)) out[pos++] = w;
                w = or_next_hamming(w);
            }
        }
    }
    free(counts);
    return total;
}

/* Ascending-array binary search; OR_MISS when absent.
 * binary_search.hpp:50-81 (BinarySearch) as called by
 * fermion_fock_basis.cpp:134-161 (FindFockStateIndex with offset 0). */
uint64_t or_find_index(const uint64_t *basis, uint64_t n, uint64_t state)
{
    if (n == 0) return OR_MISS;
    uint64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        uint64_t mid = lo + ((hi - lo) >> 1);
        uint64_t v = basis[mid];
        if (v == state) return mid;
        if (v < state) lo = mid + 1;
        else { if (mid == 0) break; hi = mid - 1; }
    }
    return OR_MISS;
}

void or_find_indices(const uint64_t *basis, uint64_t n, const uint64_t *words, uint64_t *idx, uint64_t m)
{
    for (uint64_t i = 0; i < m; ++i) idx[i] = or_find_index(basis, n, words[i]);
}

/* --------------------------------------------------------- operator action */

/* c+_{k1} c+_{k2} c_{k3} c_{k4} on a state: returns the out word and writes
 * the sign (0 when the action vanishes).  fermions.hpp:52-144
 * (Evaluate_CdCdCC): k4 annihilated first, then k3, then k2 and k1 created;
 * the sign is the parity of the occupied bits below each operator at the
 * moment it acts. */
uint64_t or_evaluate_cdcdcc(int *sign, uint64_t k1o, uint64_t k2o, uint64_t k3o, uint64_t k4o,
                            uint64_t state, uint64_t highest)
{
    if (k3o > highest || k4o > highest || (state & k3o) == 0 || (state & k4o) == 0 ||
        (k1o & k2o) || (k3o & k4o) ||
        (!(k1o & k3o) && !(k1o & k4o) && (state & k1o) != 0) ||
        (!(k2o & k3o) && !(k2o & k4o) && (state & k2o) != 0)) {
        *sign = 0;
        return 0;
    }
    int c = or_popcount(state & (k4o - 1));
    uint64_t out = state ^ k4o;
    c += or_popcount(out & (k3o - 1));
    out ^= k3o;
    c += or_popcount(out & (k2o - 1));
    out |= k2o;
    c += or_popcount(out & (k1o - 1));
    out |= k1o;
    *sign = (c & 1) ? -1 : 1;
    return out;
}

/* ------------------------------------------------------------ quartic build */

typedef struct { int64_t col; double val; } or_entry;

/* Per-row accumulator standing in for the reference's hash map for one row:
 * key = column, value summed term by term in arrival order, which is how
 * m_sparseMap.Insert(i,j) += x forms every element.  Open addressing over a
 * power-of-two table; e[] keeps the entries in first-insertion order. */
typedef struct { or_entry *e; int64_t n, cap; int32_t *slot; int64_t tcap; int64_t *pos; } or_rowacc;

static void or_acc_reset(or_rowacc *a)
{
    for (int64_t t = 0; t < a->n; ++t) a->slot[a->pos[t]] = -1;
    a->n = 0;
}

static void or_acc_grow(or_rowacc *a)
{
    int64_t ncap = a->cap ? 2 * a->cap : 1024;
    a->e = (or_entry *)realloc(a->e, (size_t)ncap * sizeof(or_entry));
    a->pos = (int64_t *)realloc(a->pos, (size_t)ncap * sizeof(int64_t));
    a->cap = ncap;
    free(a->slot);
    a->tcap = 4 * ncap;
    a->slot = (int32_t *)malloc((size_t)a->tcap * sizeof(int32_t));
    for (int64_t i = 0; i < a->tcap; ++i) a->slot[i] = -1;
    for (int64_t t = 0; t < a->n; ++t) {
        uint64_t h = ((uint64_t)a->e[t].col * 0x9E3779B97F4A7C15ull) & (uint64_t)(a->tcap - 1);
        while (a->slot[h] != -1) h = (h + 1) & (uint64_t)(a->tcap - 1);
        a->slot[h] = (int32_t)t;
        a->pos[t] = (int64_t)h;
    }
}

static void or_acc_add(or_rowacc *a, int64_t col, double v)
{
    if (a->n == a->cap) or_acc_grow(a);
    uint64_t h = ((uint64_t)col * 0x9E3779B97F4A7C15ull) & (uint64_t)(a->tcap - 1);
    while (a->slot[h] != -1) {
        or_entry *x = &a->e[a->slot[h]];
        if (x->col == col) { x->val += v; return; }
        h = (h + 1) & (uint64_t)(a->tcap - 1);
    }
    a->slot[h] = (int32_t)a->n;
    a->pos[a->n] = (int64_t)h;
    a->e[a->n].col = col;
    a->e[a->n].val = 0.0 + v;
    a->n++;
}

static void or_acc_free(or_rowacc *a)
{
    free(a->e);
    free(a->slot);
    free(a->pos);
}

static int or_cmp_entry(const void *x, const void *y)
{
    int64_t a = ((const or_entry *)x)->col, b = ((const or_entry *)y)->col;
    return (a > b) - (a < b);
}

/* One row of the quartic Hamiltonian, upper triangle (col >= row).
 * spinless_fermion_hamiltonian.hpp:310-403 (Add_CdCdCC_Terms row loop):
 *   k4 over occupied bits ascending; k3 over the other occupied bits
 *   ascending (stripped as it goes); k2 over  mask ^ (occupied bits above k3
 *   other than k4)  ascending; k1 = kTable[(k4*K+k3)*K+k2] (skip if >= K,
 *   term_tables.cpp:109-124); the filter of :351-355; Evaluate_CdCdCC; keep
 *   out >= in; binary-search the column; add sign*V when |sign*V| > 1e-14.
 * or_row_finish then applies the per-row part of Trim
 * (mapped_sparse_matrix.hpp:423-460: drop |sum| < 1e-14) and the column sort
 * of CrsSparseMatrix::Initialize (crs_sparse_matrix.hpp:193-254). */
static void or_build_row(const uint64_t *basis, uint64_t n, int norb, int64_t row,
                         const uint16_t *ktab, const double *vtab, int K, or_rowacc *acc)
{
    const uint64_t in = basis[row];
    const uint64_t mask = (norb >= 64) ? ~0ull : ((1ull << norb) - 1ull);
    const uint64_t highest = 1ull << (norb - 1);
    if (acc->cap == 0) or_acc_grow(acc);
    or_acc_reset(acc);
    uint64_t t4 = in;
    while (t4) {
        uint64_t k4o = t4 & (~t4 + 1);
        int k4 = or_popcount(k4o - 1);
        uint64_t t3 = in ^ k4o;
        while (t3) {
            uint64_t k3o = t3 & (~t3 + 1);
            int k3 = or_popcount(k3o - 1);
            if (k3 != k4) {
                uint64_t t2 = mask ^ (t3 ^ k3o);
                while (t2) {
                    uint64_t k2o = t2 & (~t2 + 1);
                    int k2 = or_popcount(k2o - 1);
                    size_t ti = ((size_t)k4 * K + k3) * K + k2;
                    int k1 = ktab[ti];
                    if (k1 < K) {
                        uint64_t k1o = 1ull << k1;
                        if ((!(k1o & in) || ((k1o & k3o) || (k1o & k4o))) &&
                            (!(k2o & in) || ((k2o & k3o) || (k2o & k4o))) &&
                            !(k1o & k2o)) {
                            int s;
                            uint64_t out = or_evaluate_cdcdcc(&s, k1o, k2o, k3o, k4o, in, highest);
                            if (s != 0 && out >= in) {
                                uint64_t j = or_find_index(basis, n, out);
                                if (j < n) {
                                    double el = (double)s * vtab[ti];
                                    if (fabs(el) > OR_SPARSE_ZERO_TOL) or_acc_add(acc, (int64_t)j, el);
                                }
                            }
                        }
                    }
                    t2 ^= k2o;
                }
            }
            t3 ^= k3o;
        }
        t4 ^= k4o;
    }
}

/* Trim (|x| < 1e-14 dropped) and sort by column into out[]; returns count. */
static int64_t or_row_finish(or_rowacc *acc, or_entry **out, int64_t *outcap)
{
    if (*outcap < acc->n) {
        *outcap = acc->cap;
        *out = (or_entry *)realloc(*out, (size_t)(*outcap) * sizeof(or_entry));
    }
    int64_t w = 0;
    for (int64_t t = 0; t < acc->n; ++t)
        if (!(fabs(acc->e[t].val) < OR_SPARSE_ZERO_TOL)) (*out)[w++] = acc->e[t];
    qsort(*out, (size_t)w, sizeof(or_entry), or_cmp_entry);
    return w;
}

/* Count pass: stored entries per row of the upper triangle for rows
 * [r0, r1).  Returns the total. */
int64_t or_build_upper_count(const uint64_t *basis, uint64_t n, int norb, const uint16_t *ktab,
                             const double *vtab, int K, int64_t r0, int64_t r1, int64_t *rowlen,
                             int nthreads)
{
    int64_t total = 0;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
#endif
    {
        or_rowacc acc = {0, 0, 0, 0, 0, 0};
        or_entry *fin = 0;
        int64_t fcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = r0; r < r1; ++r) {
            or_build_row(basis, n, norb, r, ktab, vtab, K, &acc);
            int64_t m = or_row_finish(&acc, &fin, &fcap);
            rowlen[r - r0] = m;
            total += m;
        }
        or_acc_free(&acc);
        free(fin);
    }
    return total;
}

/* Fill pass for rows [r0, r1): rowptr (size r1-r0+1) must hold the
 * exclusive prefix of the count pass; writes col/val. */
void or_build_upper_fill(const uint64_t *basis, uint64_t n, int norb, const uint16_t *ktab,
                         const double *vtab, int K, int64_t r0, int64_t r1, const int64_t *rowptr,
                         int32_t *col, double *val, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        or_rowacc acc = {0, 0, 0, 0, 0, 0};
        or_entry *fin = 0;
        int64_t fcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = r0; r < r1; ++r) {
            or_build_row(basis, n, norb, r, ktab, vtab, K, &acc);
            int64_t m = or_row_finish(&acc, &fin, &fcap);
            int64_t p = rowptr[r - r0];
            for (int64_t t = 0; t < m; ++t) {
                col[p + t] = (int32_t)fin[t].col;
                val[p + t] = fin[t].val;
            }
        }
        or_acc_free(&acc);
        free(fin);
    }
}

/* --------------------------------------------------------- two Landau levels */

static int or_cmp_u64(const void *x, const void *y)
{
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return (a > b) - (a < b);
}

/* TwoLevelFermionFockBasis::GenerateFockSpace with TestAngularMomentumSector2LL
 * (two_level_fermion_fock_basis.cpp:289-470, two_level_angular_momentum_constraint.hpp:41-70)
 * as combined words (first << K1) | second, K1 = K0 + 2, ascending (the
 * reference's (first, second) order): for every split n0 + n1 = N, every
 * lowest-level word (weight of bit i: i + 1) paired with every second-level
 * word (weight of bit j: j) whose weights sum to S = (2Lz + N(K1 - 1)) / 2.
 * With out == NULL only counts. */
uint64_t or_basis2_build(int N, int K0, int twoLz, uint64_t *out)
{
    const int K1 = K0 + 2;
    const int64_t t = (int64_t)twoLz + (int64_t)N * (K1 - 1);
    if (t % 2) return 0;
    const int64_t S = t / 2;
    uint64_t total = 0;
    for (int n0 = 0; n0 <= N; ++n0) {
        const int n1 = N - n0;
        if (n0 > K0 || n1 > K1) continue;
        const uint64_t c1 = or_binomial(K1, n1), c0 = or_binomial(K0, n0);
        /* second-level words bucketed by weight */
        const int wmax1 = K1 * K1;
        uint64_t *cnt = (uint64_t *)calloc((size_t)wmax1 + 2, sizeof(uint64_t));
        uint64_t *w1 = (uint64_t *)malloc((size_t)(c1 ? c1 : 1) * sizeof(uint64_t));
        int *wt1 = (int *)malloc((size_t)(c1 ? c1 : 1) * sizeof(int));
        uint64_t w = n1 ? ((1ull << n1) - 1ull) : 0ull;
        for (uint64_t i = 0; i < c1; ++i) {
            int s = 0;
            for (uint64_t x = w; x; x &= x - 1) s += or_bitpos(x & (~x + 1));
            w1[i] = w;
            wt1[i] = s;
            cnt[s + 1]++;
            if (n1) w = or_next_hamming(w);
        }
        for (int k = 0; k <= wmax1; ++k) cnt[k + 1] += cnt[k];
        uint64_t *sorted = (uint64_t *)malloc((size_t)(c1 ? c1 : 1) * sizeof(uint64_t));
        uint64_t *fillp = (uint64_t *)malloc(((size_t)wmax1 + 1) * sizeof(uint64_t));
        memcpy(fillp, cnt, ((size_t)wmax1 + 1) * sizeof(uint64_t));
        for (uint64_t i = 0; i < c1; ++i) sorted[fillp[wt1[i]]++] = w1[i];
        uint64_t a = n0 ? ((1ull << n0) - 1ull) : 0ull;
        for (uint64_t i = 0; i < c0; ++i) {
            int s0 = 0;
            for (uint64_t x = a; x; x &= x - 1) s0 += or_bitpos(x & (~x + 1)) + 1;
            const int64_t need = S - s0;
            if (need >= 0 && need <= wmax1) {
                for (uint64_t q = cnt[need]; q < cnt[need + 1]; ++q) {
                    if (out) out[total] = (a << K1) | sorted[q];
                    ++total;
                }
            }
            if (n0) a = or_next_hamming(a);
        }
        free(cnt);
        free(w1);
        free(wt1);
        free(sorted);
        free(fillp);
    }
    if (out) qsort(out, (size_t)total, sizeof(uint64_t), or_cmp_u64);
    return total;
}

/* The single-level quartic loop of or_build_row on one level's word `lw`
 * (K orbitals, tables kt/vt) with the other level's bits `other` fixed at
 * shift `osh`; the level's word sits at shift `lsh` of the combined word. */
static void or_level_quartic(const uint64_t *basis, uint64_t n, uint64_t lw, int K, int lsh, uint64_t other,
                             const uint16_t *kt, const double *vt, or_rowacc *acc)
{
    const uint64_t mask = (1ull << K) - 1ull;
    const uint64_t highest = 1ull << (K - 1);
    uint64_t t4 = lw;
    while (t4) {
        uint64_t k4o = t4 & (~t4 + 1);
        int k4 = or_popcount(k4o - 1);
        uint64_t t3 = lw ^ k4o;
        while (t3) {
            uint64_t k3o = t3 & (~t3 + 1);
            int k3 = or_popcount(k3o - 1);
            if (k3 != k4) {
                uint64_t t2 = mask ^ (t3 ^ k3o);
                while (t2) {
                    uint64_t k2o = t2 & (~t2 + 1);
                    int k2 = or_popcount(k2o - 1);
                    size_t ti = ((size_t)k4 * K + k3) * K + k2;
                    int k1 = kt[ti];
                    if (k1 < K) {
                        uint64_t k1o = 1ull << k1;
                        if ((!(k1o & lw) || ((k1o & k3o) || (k1o & k4o))) &&
                            (!(k2o & lw) || ((k2o & k3o) || (k2o & k4o))) && !(k1o & k2o)) {
                            int sgn;
                            uint64_t out = or_evaluate_cdcdcc(&sgn, k1o, k2o, k3o, k4o, lw, highest);
                            if (sgn != 0 && out >= lw) {
                                uint64_t j = or_find_index(basis, n, (out << lsh) | other);
                                if (j < n) {
                                    double el = (double)sgn * vt[ti];
                                    if (fabs(el) > OR_SPARSE_ZERO_TOL) or_acc_add(acc, (int64_t)j, el);
                                }
                            }
                        }
                    }
                    t2 ^= k2o;
                }
            }
            t3 ^= k3o;
        }
        t4 ^= k4o;
    }
}

/* One upper-triangle row of the two-level Hamiltonian in the model's call
 * order (two_level_pseudopotential_model.cpp:190-215): level-0 then level-1
 * occupation energies (Add_CdC_Terms, two_level_spinless_fermion_hamiltonian.hpp:
 * 143-270), then the level-0 and level-1 quartic terms (Add_CdCdCC_Terms,
 * :306-470), each on its level's word with the other fixed. */
static void or_build2_row(const uint64_t *basis, uint64_t n, int K0, int64_t row, const uint16_t *kt0,
                          const double *vt0, const uint16_t *kt1, const double *vt1, const double *e0,
                          const double *e1, or_rowacc *acc)
{
    const int K1 = K0 + 2;
    const uint64_t w = basis[row], first = w >> K1, second = w & ((1ull << K1) - 1ull);
    if (acc->cap == 0) or_acc_grow(acc);
    or_acc_reset(acc);
    if (e0)
        for (uint64_t x = first; x; x &= x - 1) {
            double v = e0[or_bitpos(x & (~x + 1))];
            if (fabs(v) > OR_SPARSE_ZERO_TOL) or_acc_add(acc, row, v);
        }
    if (e1)
        for (uint64_t x = second; x; x &= x - 1) {
            double v = e1[or_bitpos(x & (~x + 1))];
            if (fabs(v) > OR_SPARSE_ZERO_TOL) or_acc_add(acc, row, v);
        }
    or_level_quartic(basis, n, first, K0, K1, second, kt0, vt0, acc);
    or_level_quartic(basis, n, second, K1, 0, first << K1, kt1, vt1, acc);
}

int64_t or_build2_upper_count(const uint64_t *basis, uint64_t n, int K0, const uint16_t *kt0, const double *vt0,
                              const uint16_t *kt1, const double *vt1, const double *e0, const double *e1,
                              int64_t *rowlen, int nthreads)
{
    int64_t total = 0;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
#endif
    {
        or_rowacc acc = {0, 0, 0, 0, 0, 0};
        or_entry *fin = 0;
        int64_t fcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = 0; r < (int64_t)n; ++r) {
            or_build2_row(basis, n, K0, r, kt0, vt0, kt1, vt1, e0, e1, &acc);
            int64_t m = or_row_finish(&acc, &fin, &fcap);
            rowlen[r] = m;
            total += m;
        }
        or_acc_free(&acc);
        free(fin);
    }
    return total;
}

void or_build2_upper_fill(const uint64_t *basis, uint64_t n, int K0, const uint16_t *kt0, const double *vt0,
                          const uint16_t *kt1, const double *vt1, const double *e0, const double *e1,
                          const int64_t *rowptr, int32_t *col, double *val, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        or_rowacc acc = {0, 0, 0, 0, 0, 0};
        or_entry *fin = 0;
        int64_t fcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = 0; r < (int64_t)n; ++r) {
            or_build2_row(basis, n, K0, r, kt0, vt0, kt1, vt1, e0, e1, &acc);
            int64_t m = or_row_finish(&acc, &fin, &fcap);
            for (int64_t t = 0; t < m; ++t) {
                col[rowptr[r] + t] = (int32_t)fin[t].col;
                val[rowptr[r] + t] = fin[t].val;
            }
        }
        or_acc_free(&acc);
        free(fin);
    }
}

/* ----------------------------------------- complex momentum path (OFL model) */

/* FermionFockBasis::GenerateFockSpace with TestLinearMomentumSector2
 * (interacting_ofl_model.cpp:994-1001, linear_momentum_constraints_2D.cpp:38-79):
 * Gosper's successor over the N-bit words of X*Y orbitals (bit p at kx = p/Y,
 * ky = p%Y), kept when (sum kx mod X, sum ky mod Y) = (kx, ky); ascending.
 * With out == NULL only counts. */
uint64_t or_basis_momentum(int N, int X, int Y, int kx, int ky, uint64_t *out)
{
    const int K = X * Y;
    const uint64_t full = or_binomial(K, N);
    uint64_t w = (1ull << N) - 1ull, c = 0;
    for (uint64_t i = 0; i < full; ++i) {
        int sx = 0, sy = 0;
        for (uint64_t x = w; x; x &= x - 1) {
            int p = or_bitpos(x & (~x + 1));
            sx += p / Y;
            sy += p % Y;
        }
        if (sx % X == kx && sy % Y == ky) {
            if (out) out[c] = w;
            ++c;
        }
        if (i + 1 < full) w = or_next_hamming(w);
    }
    return c;
}

typedef struct { int64_t col; double re, im; } or_centry;
typedef struct { or_centry *e; int64_t n, cap; int32_t *slot; int64_t tcap; int64_t *pos; } or_crowacc;

static void or_cacc_reset(or_crowacc *a)
{
    for (int64_t t = 0; t < a->n; ++t) a->slot[a->pos[t]] = -1;
    a->n = 0;
}

static void or_cacc_grow(or_crowacc *a)
{
    int64_t ncap = a->cap ? 2 * a->cap : 1024;
    a->e = (or_centry *)realloc(a->e, (size_t)ncap * sizeof(or_centry));
    a->pos = (int64_t *)realloc(a->pos, (size_t)ncap * sizeof(int64_t));
    a->cap = ncap;
    free(a->slot);
    a->tcap = 4 * ncap;
    a->slot = (int32_t *)malloc((size_t)a->tcap * sizeof(int32_t));
    for (int64_t i = 0; i < a->tcap; ++i) a->slot[i] = -1;
    for (int64_t t = 0; t < a->n; ++t) {
        uint64_t h = ((uint64_t)a->e[t].col * 0x9E3779B97F4A7C15ull) & (uint64_t)(a->tcap - 1);
        while (a->slot[h] != -1) h = (h + 1) & (uint64_t)(a->tcap - 1);
        a->slot[h] = (int32_t)t;
        a->pos[t] = (int64_t)h;
    }
}

/* entry(col) += (re, im), first insertion from (0, 0): Insert(i,j) += x with T = dcmplx */
static void or_cacc_add(or_crowacc *a, int64_t col, double re, double im)
{
    if (a->n == a->cap) or_cacc_grow(a);
    uint64_t h = ((uint64_t)col * 0x9E3779B97F4A7C15ull) & (uint64_t)(a->tcap - 1);
    while (a->slot[h] != -1) {
        or_centry *x = &a->e[a->slot[h]];
        if (x->col == col) { x->re += re; x->im += im; return; }
        h = (h + 1) & (uint64_t)(a->tcap - 1);
    }
    a->slot[h] = (int32_t)a->n;
    a->pos[a->n] = (int64_t)h;
    a->e[a->n].col = col;
    a->e[a->n].re = 0.0 + re;
    a->e[a->n].im = 0.0 + im;
    a->n++;
}

static int or_cmp_centry(const void *x, const void *y)
{
    int64_t a = ((const or_centry *)x)->col, b = ((const or_centry *)y)->col;
    return (a > b) - (a < b);
}

static int or_ofl_index(int k3, int k4, int K)
{
    const int t1 = k4 > k3 ? k3 : k4, t2 = k4 > k3 ? k4 : k3;
    return t1 * K + t2 - t1 * (t1 + 1) / 2;
}

/* One upper-triangle row of SpinlessFermionHamiltonian<dcmplx> from the
 * array-format OFL tables (spinless_fermion_hamiltonian.hpp:150-436 with
 * interacting_ofl_model/term_tables.cpp:59-200): occupation energies, then the
 * quartic loop of or_build_row with k1 = kTable[t*K + k2] and V =
 * vTable[t*K + (k4 > k3 ? k1 : k2)], t the (k3, k4) triangle index; each
 * term kept when abs > 1e-14 (hypot, the std::abs of std::complex). */
static void or_cbuild_row(const uint64_t *basis, uint64_t n, int K, int64_t row, const uint16_t *kt,
                          const double *vt, const double *e, or_crowacc *acc)
{
    const uint64_t in = basis[row];
    const uint64_t mask = (1ull << K) - 1ull;
    const uint64_t highest = 1ull << (K - 1);
    if (acc->cap == 0) or_cacc_grow(acc);
    or_cacc_reset(acc);
    if (e)
        for (uint64_t x = in; x; x &= x - 1) {
            int k = or_bitpos(x & (~x + 1));
            if (hypot(e[2 * k], e[2 * k + 1]) > OR_SPARSE_ZERO_TOL) or_cacc_add(acc, row, e[2 * k], e[2 * k + 1]);
        }
    uint64_t t4 = in;
    while (t4) {
        uint64_t k4o = t4 & (~t4 + 1);
        int k4 = or_popcount(k4o - 1);
        uint64_t t3 = in ^ k4o;
        while (t3) {
            uint64_t k3o = t3 & (~t3 + 1);
            int k3 = or_popcount(k3o - 1);
            if (k3 != k4) {
                const size_t base = (size_t)or_ofl_index(k3, k4, K) * K;
                uint64_t t2 = mask ^ (t3 ^ k3o);
                while (t2) {
                    uint64_t k2o = t2 & (~t2 + 1);
                    int k2 = or_popcount(k2o - 1);
                    int k1 = kt[base + k2];
                    uint64_t k1o = 1ull << k1;
                    if ((!(k1o & in) || ((k1o & k3o) || (k1o & k4o))) &&
                        (!(k2o & in) || ((k2o & k3o) || (k2o & k4o))) && !(k1o & k2o)) {
                        int sgn;
                        uint64_t out = or_evaluate_cdcdcc(&sgn, k1o, k2o, k3o, k4o, in, highest);
                        if (sgn != 0 && out >= in) {
                            uint64_t j = or_find_index(basis, n, out);
                            if (j < n) {
                                const size_t vi = base + (size_t)(k4 > k3 ? k1 : k2);
                                const double re = (double)sgn * vt[2 * vi], im = (double)sgn * vt[2 * vi + 1];
                                if (hypot(re, im) > OR_SPARSE_ZERO_TOL) or_cacc_add(acc, (int64_t)j, re, im);
                            }
                        }
                    }
                    t2 ^= k2o;
                }
            }
            t3 ^= k3o;
        }
        t4 ^= k4o;
    }
}

static int64_t or_crow_finish(or_crowacc *acc, or_centry **out, int64_t *outcap)
{
    if (*outcap < acc->n) {
        *outcap = acc->cap;
        *out = (or_centry *)realloc(*out, (size_t)(*outcap) * sizeof(or_centry));
    }
    int64_t w = 0;
    for (int64_t t = 0; t < acc->n; ++t)
        if (!(hypot(acc->e[t].re, acc->e[t].im) < OR_SPARSE_ZERO_TOL)) (*out)[w++] = acc->e[t];
    qsort(*out, (size_t)w, sizeof(or_centry), or_cmp_centry);
    return w;
}

/* Count (col == NULL) or fill pass of the complex upper-triangle CRS. */
int64_t or_cbuild_upper(const uint64_t *basis, uint64_t n, int K, const uint16_t *kt, const double *vt,
                        const double *e, int64_t *rowlen, const int64_t *rowptr, int32_t *col, double *val,
                        int nthreads)
{
    int64_t total = 0;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
#endif
    {
        or_crowacc acc = {0, 0, 0, 0, 0, 0};
        or_centry *fin = 0;
        int64_t fcap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = 0; r < (int64_t)n; ++r) {
            or_cbuild_row(basis, n, K, r, kt, vt, e, &acc);
            int64_t m = or_crow_finish(&acc, &fin, &fcap);
            if (rowlen) rowlen[r] = m;
            if (col)
                for (int64_t t = 0; t < m; ++t) {
                    col[rowptr[r] + t] = (int32_t)fin[t].col;
                    val[2 * (rowptr[r] + t)] = fin[t].re;
                    val[2 * (rowptr[r] + t) + 1] = fin[t].im;
                }
            total += m;
        }
        free(acc.e);
        free(acc.slot);
        free(acc.pos);
        free(fin);
    }
    return total;
}

/* y = M x with the reference's Hermitian completion of the upper storage
 * (sparse_linear_algebra.hpp:148-164 for T = dcmplx): y_i += A_ij x_j and,
 * for j != i, y_j += conj(A_ij) x_i; complex as (re, im) pairs, rows split
 * over threads with private y. */
void or_cspmv_upper_mt(const int64_t *rowptr, const int32_t *col, const double *val, int64_t n, const double *x,
                       double *y, double *scratch, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        double *yt = scratch + (size_t)t * 2 * n;
        for (int64_t i = 0; i < 2 * n; ++i) yt[i] = 0.0;
        const int64_t r0 = n * t / nthreads, r1 = n * (t + 1) / nthreads;
        for (int64_t i = r0; i < r1; ++i) {
            const double xr = x[2 * i], xi = x[2 * i + 1];
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const int64_t c = col[k];
                const double ar = val[2 * k], ai = val[2 * k + 1];
                yt[2 * i] += ar * x[2 * c] - ai * x[2 * c + 1];
                yt[2 * i + 1] += ar * x[2 * c + 1] + ai * x[2 * c];
                if (c != i) {
                    yt[2 * c] += ar * xr + ai * xi;
                    yt[2 * c + 1] += ar * xi - ai * xr;
                }
            }
        }
    }
    for (int64_t i = 0; i < 2 * n; ++i) {
        double s = 0.0;
        for (int t = 0; t < nthreads; ++t) s += scratch[(size_t)t * 2 * n + i];
        y[i] = s;
    }
}

/* ------------------------------------------------------------------- SpMV */

/* y = A x for A symmetric stored as its upper triangle in CRS:
 * sparse_linear_algebra.hpp:143-164 (the non-MKL loop of
 * SymmetricMatrixVectorMultiply with ALPHA=1, BETA=0):
 *   y[i] += a*x[c];  if (i != c) y[c] += a*x[i]. */
void or_spmv_sym_upper(const int64_t *rowptr, const int32_t *col, const double *val, int64_t n,
                       const double *x, double *y)
{
    for (int64_t i = 0; i < n; ++i) y[i] = 0.0 * x[i];
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = rowptr[i]; j < rowptr[i + 1]; ++j) {
            int64_t c = col[j];
            double a = val[j];
            y[i] += a * x[c];
            if (i != c) y[c] += a * x[i];
        }
    }
}

/* Threaded form of the same product laid out like the reference's MPI
 * scheme (sparse_linear_algebra.hpp:218-312, ParallelSymmetricMatrixVectorMultiply):
 * rows are cut into contiguous blocks, each worker runs the serial loop over
 * its block into a private y, and the private vectors are then reduced.
 * work must hold nthreads*n doubles. */
void or_spmv_sym_upper_mt(const int64_t *rowptr, const int32_t *col, const double *val, int64_t n,
                          const double *x, double *y, double *work, int nthreads)
{
    if (nthreads <= 1) { or_spmv_sym_upper(rowptr, col, val, n, x, y); return; }
    int64_t nnz = rowptr[n];
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        double *yy = work + (size_t)t * (size_t)n;
        memset(yy, 0, (size_t)n * sizeof(double));
        /* balance by nonzeros, like DivideTasks balances by rows */
        int64_t lo_nz = nnz * t / nthreads, hi_nz = nnz * (t + 1) / nthreads;
        int64_t r0 = 0, r1 = 0;
        { int64_t a = 0, b = n; while (a < b) { int64_t m = (a + b) / 2; if (rowptr[m] < lo_nz) a = m + 1; else b = m; } r0 = a; }
        { int64_t a = 0, b = n; while (a < b) { int64_t m = (a + b) / 2; if (rowptr[m] < hi_nz) a = m + 1; else b = m; } r1 = a; }
        if (t == nthreads - 1) r1 = n;
        for (int64_t i = r0; i < r1; ++i) {
            double xi = x[i], acc = 0.0;
            for (int64_t j = rowptr[i]; j < rowptr[i + 1]; ++j) {
                int64_t c = col[j];
                double a = val[j];
                acc += a * x[c];
                if (i != c) yy[c] += a * xi;
            }
            yy[i] += acc;
        }
#ifdef _OPENMP
#pragma omp barrier
#pragma omp for schedule(static)
#endif
        for (int64_t i = 0; i < n; ++i) {
            double s = 0.0;
            for (int u = 0; u < nthreads; ++u) s += work[(size_t)u * (size_t)n + i];
            y[i] = s;
        }
    }
}

/* y = A x for a full (both triangles) CRS matrix. */
void or_spmv_full(const int64_t *rowptr, const int32_t *col, const double *val, int64_t n,
                  const double *x, double *y, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static, 1024)
#endif
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int64_t j = rowptr[i]; j < rowptr[i + 1]; ++j) s += val[j] * x[col[j]];
        y[i] = s;
    }
}

int or_num_procs(void)
{
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}
