"""CPU oracle for the LLL spinless-fermion exact-diagonalization hot path.

TEST INFRASTRUCTURE ONLY.  Only the tests, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` import this module, and only as the reference the
tests compare against or as the timed CPU baseline.  The shipped library never calls into it.

It restates the reference (SimonDavenport/hamiltonian_diagonalization):

* ``oracle.c`` (loaded through ctypes): Fock-basis scan, binary-search rank,
  ``Evaluate_CdCdCC``, the quartic build in the reference's loop order, and
  the symmetric upper-triangle SpMV;
* this file: the term tables (``BaseGenerate4KTable`` /
  ``BaseTermsFromPseudopotentials``, pseudopotential_model_base.hpp:62-229)
  with Clebsch-Gordan coefficients evaluated EXACTLY (rational Racah
  formula), the LLL Coulomb pseudopotentials
  (coulomb_pseudopotentials.cpp:40-69, exact integers), and the eigenvalue
  oracle: SciPy's ARPACK, the same library family the reference drives
  through ``pdnaupd_/pdneupd_`` (arpack_wrapper.hpp:595-937).

``pin_against_reference()`` checks the bit-level restatement against the
reference's own primitives compiled from its sources (oracle/_ref).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from fractions import Fraction
from functools import lru_cache

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_HAM_PATH = os.path.join(HERE, "_ref", "libref_ham.so")
REF_OFL_PATH = os.path.join(HERE, "_ref", "libref_ofl.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
MISS = np.uint64(0xFFFFFFFFFFFFFFFF)
SPARSE_ZERO_TOL = 1e-14          # hamiltonian_data.hpp:53
CG_EPS = 1e-12                   # clebsch_gordan_coefficients.hpp:53 (values at or below are not stored)

_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile oracle/liboracle.so (and oracle/_ref when the reference tree is present)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
        os.path.join(HERE, "oracle.c")
    ):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB_PATH


def build_ref(src: str | None = None) -> str | None:
    """Compile oracle/_ref/libref.so from the reference's source directory
    (src, else the REFSRC environment variable); None when neither names an
    existing directory."""
    src = src or os.environ.get("REFSRC")
    if not src or not os.path.isdir(src):
        return None
    subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFSRC={src}"])
    return REF_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.or_binomial.restype = ctypes.c_uint64
        L.or_binomial.argtypes = [ctypes.c_int, ctypes.c_int]
        L.or_next_hamming.restype = ctypes.c_uint64
        L.or_next_hamming.argtypes = [ctypes.c_uint64]
        L.or_unrank_hamming.restype = ctypes.c_uint64
        L.or_unrank_hamming.argtypes = [ctypes.c_int, ctypes.c_uint64]
        L.or_lz_ok.restype = ctypes.c_int
        L.or_lz_ok.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        L.or_basis_build.restype = ctypes.c_uint64
        L.or_basis_build.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_int]
        L.or_find_index.restype = ctypes.c_uint64
        L.or_find_index.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        L.or_find_indices.restype = None
        L.or_find_indices.argtypes = [_u64p, ctypes.c_uint64, _u64p, _u64p, ctypes.c_uint64]
        L.or_evaluate_cdcdcc.restype = ctypes.c_uint64
        L.or_evaluate_cdcdcc.argtypes = [ctypes.POINTER(ctypes.c_int)] + [ctypes.c_uint64] * 6
        L.or_build_upper_count.restype = ctypes.c_int64
        L.or_build_upper_count.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_int, _u16p, _f64p, ctypes.c_int,
                                           ctypes.c_int64, ctypes.c_int64, _i64p, ctypes.c_int]
        L.or_build_upper_fill.restype = None
        L.or_build_upper_fill.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_int, _u16p, _f64p, ctypes.c_int,
                                          ctypes.c_int64, ctypes.c_int64, _i64p, _i32p, _f64p, ctypes.c_int]
        L.or_spmv_sym_upper.restype = None
        L.or_spmv_sym_upper.argtypes = [_i64p, _i32p, _f64p, ctypes.c_int64, _f64p, _f64p]
        L.or_spmv_sym_upper_mt.restype = None
        L.or_spmv_sym_upper_mt.argtypes = [_i64p, _i32p, _f64p, ctypes.c_int64, _f64p, _f64p, _f64p, ctypes.c_int]
        L.or_spmv_full.restype = None
        L.or_spmv_full.argtypes = [_i64p, _i32p, _f64p, ctypes.c_int64, _f64p, _f64p, ctypes.c_int]
        L.or_basis2_build.restype = ctypes.c_uint64
        L.or_basis2_build.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _u64p]
        L.or_build2_upper_count.restype = ctypes.c_int64
        L.or_build2_upper_count.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_int, _u16p, _f64p, _u16p, _f64p,
                                            _f64p, _f64p, _i64p, ctypes.c_int]
        L.or_build2_upper_fill.restype = None
        L.or_build2_upper_fill.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_int, _u16p, _f64p, _u16p, _f64p,
                                           _f64p, _f64p, _i64p, _i32p, _f64p, ctypes.c_int]
        L.or_basis_momentum.restype = ctypes.c_uint64
        L.or_basis_momentum.argtypes = [ctypes.c_int] * 5 + [_u64p]
        L.or_cbuild_upper.restype = ctypes.c_int64
        L.or_cbuild_upper.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_int, _u16p, _f64p, _f64p, _i64p, _i64p,
                                      _i32p, _f64p, ctypes.c_int]
        L.or_cspmv_upper_mt.restype = None
        L.or_cspmv_upper_mt.argtypes = [_i64p, _i32p, _f64p, ctypes.c_int64, _f64p, _f64p, _f64p, ctypes.c_int]
        L.or_num_procs.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


def num_procs() -> int:
    return int(lib().or_num_procs())


# ------------------------------------------------------------------ bit tools

def binomial(n: int, k: int) -> int:
    return int(lib().or_binomial(n, k))


def next_hamming(x: int) -> int:
    return int(lib().or_next_hamming(x))


def unrank_hamming(w: int, index: int) -> int:
    return int(lib().or_unrank_hamming(w, index))


def lz_ok(state: int, two_lz: int, max_lz: int) -> bool:
    return bool(lib().or_lz_ok(state, two_lz, max_lz))


def evaluate_cdcdcc(k1: int, k2: int, k3: int, k4: int, state: int, norb: int):
    """(out_word, sign) of c+_k1 c+_k2 c_k3 c_k4 |state>  (fermions.hpp:52-144)."""
    s = ctypes.c_int(0)
    out = lib().or_evaluate_cdcdcc(ctypes.byref(s), 1 << k1, 1 << k2, 1 << k3, 1 << k4, state,
                                   1 << (norb - 1))
    return int(out), int(s.value)


# ---------------------------------------------------------------- Fock basis

def sector_sum(N: int, norb: int, two_lz: int):
    """Sum of occupied bit positions of every state in the sector, or None if empty
    (angular_momentum_constraint.hpp:41-62: sum(2k - maxLz) == 2Lz)."""
    t = two_lz + N * (norb - 1)
    if t % 2:
        return None
    return t // 2


def basis(N: int, norb: int, two_lz: int, nthreads: int | None = None) -> np.ndarray:
    """Ascending sector basis (fermion_fock_basis.cpp:241-354)."""
    nt = nthreads or num_procs()
    n = int(lib().or_basis_build(N, norb, two_lz, None, nt))
    out = np.empty(n, dtype=np.uint64)
    if n:
        lib().or_basis_build(N, norb, two_lz, _p(out, _u64p), nt)
    return out


def find_indices(b: np.ndarray, words: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(b, dtype=np.uint64)
    w = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.empty(len(w), dtype=np.uint64)
    lib().or_find_indices(_p(b, _u64p), len(b), _p(w, _u64p), _p(out, _u64p), len(w))
    return out


# --------------------------------------------------------------- term tables

def k_table(norb: int) -> np.ndarray:
    """kTable[(k4*K+k3)*K+k2] = k1 with m1+m2 = m3+m4, 65535 when out of range.

    pseudopotential_model_base.hpp:62-139 (ConvertStateLabel k=(maxLz-m)/2,
    FindM1 with error code maxLz2+2 = maxLz+2 for one Landau level,
    BaseGenerate4KTable loop order m4, m3, m2 from +maxLz down in steps of 2).
    """
    max_lz = norb - 1
    K = norb
    out = np.empty(K ** 3, dtype=np.uint16)
    it = 0
    for m4 in range(max_lz, -max_lz - 1, -2):
        for m3 in range(max_lz, -max_lz - 1, -2):
            for m2 in range(max_lz, -max_lz - 1, -2):
                m1 = m3 + m4 - m2
                if not (-max_lz <= m1 <= max_lz):
                    m1 = max_lz + 2
                out[it] = ((-m1 + max_lz) // 2) & 0xFFFF
                it += 1
    return out


_FACT = [1]
for _i in range(1, 400):
    _FACT.append(_FACT[-1] * _i)


@lru_cache(maxsize=None)
def cg_exact(tj1: int, tm1: int, tj2: int, tm2: int, tJ: int, tM: int) -> float:
    """<j1 m1; j2 m2 | J M> from the Racah closed form in exact rational
    arithmetic; all arguments are twice the physical quantum numbers.
    Magnitudes at or below 1e-12 are returned as 0, as the reference's table
    does not store them (clebsch_gordan_wrapper.hpp:116-124)."""
    if tm1 + tm2 != tM or abs(tm1) > tj1 or abs(tm2) > tj2 or abs(tM) > tJ:
        return 0.0
    if tJ > tj1 + tj2 or tJ < abs(tj1 - tj2) or (tj1 + tj2 + tJ) % 2:
        return 0.0
    if (tj1 + tm1) % 2 or (tj2 + tm2) % 2 or (tJ + tM) % 2:
        return 0.0
    j1p, j1m = (tj1 + tm1) // 2, (tj1 - tm1) // 2
    j2p, j2m = (tj2 + tm2) // 2, (tj2 - tm2) // 2
    Jp, Jm = (tJ + tM) // 2, (tJ - tM) // 2
    a = (tj1 + tj2 - tJ) // 2
    b = (tj1 - tj2 + tJ) // 2
    c = (-tj1 + tj2 + tJ) // 2
    s = (tj1 + tj2 + tJ) // 2
    F = _FACT
    pref2 = Fraction((tJ + 1) * F[a] * F[b] * F[c], F[s + 1]) * (F[j1p] * F[j1m] * F[j2p] * F[j2m] * F[Jp] * F[Jm])
    e1 = (tJ - tj2 + tm1) // 2      # J - j2 + m1
    e2 = (tJ - tj1 - tm2) // 2      # J - j1 - m2
    kmin = max(0, -e1, -e2)
    kmax = min(a, j1m, j2p)
    tot = Fraction(0)
    for k in range(kmin, kmax + 1):
        d = F[k] * F[a - k] * F[j1m - k] * F[j2p - k] * F[e1 + k] * F[e2 + k]
        tot += Fraction(-1 if k & 1 else 1, d)
    if tot == 0:
        return 0.0
    val = math.sqrt(float(pref2 * tot * tot))
    if tot < 0:
        val = -val
    if abs(val) <= CG_EPS:
        return 0.0
    return val


def v_table(norb: int, pseudopotentials) -> np.ndarray:
    """vTable[(k4*K+k3)*K+k2] = -sum_L V_L <S m1,S m2|Lact M><S m3,S m4|Lact M>.

    pseudopotential_model_base.hpp:150-229 (BaseTermsFromPseudopotentials):
    loop over m4,m3,m2 from +maxLz down; m1 = FindM1; for L = 0,2,..
    < 2*len(V): Lact = 2*maxLz - L, M = m1+m2, the product of the two
    coefficients when |M| <= Lact, subtracted with weight V[L/2]."""
    max_lz = norb - 1
    K = norb
    pp = [float(v) for v in pseudopotentials]
    out = np.zeros(K ** 3, dtype=np.float64)
    it = 0
    for m4 in range(max_lz, -max_lz - 1, -2):
        for m3 in range(max_lz, -max_lz - 1, -2):
            for m2 in range(max_lz, -max_lz - 1, -2):
                total = 0.0
                m1 = m3 + m4 - m2
                if -max_lz <= m1 <= max_lz:
                    M = m1 + m2
                    for L in range(0, 2 * len(pp), 2):
                        temp = 0.0
                        lact = 2 * max_lz - L
                        if -lact <= M <= lact:
                            temp += cg_exact(max_lz, m1, max_lz, m2, lact, M) * cg_exact(max_lz, m3, max_lz, m4, lact, M)
                        total -= pp[L // 2] * temp
                out[it] = total
                it += 1
    return out


def quartic_tables(norb: int, pseudopotentials):
    return k_table(norb), v_table(norb, pseudopotentials)


def coulomb_pseudopotentials(norb: int) -> np.ndarray:
    """LLL Coulomb pseudopotentials on the sphere, V_m for m = 0..2S with
    mulFactor 1 (coulomb_pseudopotentials.cpp:40-69):
    p[2S-L] = 2/sqrt(S) C(4S-2L,2S-L) C(4S+2L+2,2S+L+1) / C(4S+2,2S+1)^2,
    here with exact integer binomials."""
    max_lz = norb - 1
    p = np.zeros(max_lz + 1)
    den = math.comb(2 * max_lz + 2, max_lz + 1) ** 2
    for L in range(max_lz + 1):
        r = Fraction(math.comb(2 * max_lz - 2 * L, max_lz - L) * math.comb(2 * max_lz + 2 * L + 2, max_lz + L + 1), den)
        p[max_lz - L] = 2.0 / math.sqrt(max_lz / 2.0) * float(r)
    return p


def odd_coulomb_list(norb: int) -> np.ndarray:
    """The pseudopotential list the measured configurations use: Coulomb V_m
    for odd m with 1 <= m <= 2S-1, even m set to 0, length 2S (the longest
    list the reference accepts, pseudopotential_model_data.cpp:285-290)."""
    v = coulomb_pseudopotentials(norb)[: norb - 1].copy()
    v[0::2] = 0.0
    return v


def sweep_list(norb: int, v1: float) -> np.ndarray:
    """H(V1) = V1*P_1 + sum_{odd m>=3} V_m^Coulomb P_m as a pseudopotential list."""
    v = odd_coulomb_list(norb)
    v[1] = v1
    return v


# ------------------------------------------------------------- quartic build

def build_upper(b: np.ndarray, norb: int, ktab: np.ndarray, vtab: np.ndarray,
                nthreads: int | None = None, rows: tuple[int, int] | None = None):
    """Upper-triangle CRS (int64 rowptr, int32 col, f64 val) in the
    reference's loop and summation order (spinless_fermion_hamiltonian.hpp:282-436,
    mapped_sparse_matrix.hpp:423-460, crs_sparse_matrix.hpp:193-254).
    ``rows`` restricts the build to a row range [r0, r1)."""
    nt = nthreads or num_procs()
    b = np.ascontiguousarray(b, dtype=np.uint64)
    kt = np.ascontiguousarray(ktab, dtype=np.uint16)
    vt = np.ascontiguousarray(vtab, dtype=np.float64)
    K = norb
    r0, r1 = rows if rows is not None else (0, len(b))
    rowlen = np.zeros(r1 - r0, dtype=np.int64)
    L = lib()
    L.or_build_upper_count(_p(b, _u64p), len(b), norb, _p(kt, _u16p), _p(vt, _f64p), K, r0, r1,
                           _p(rowlen, _i64p), nt)
    rowptr = np.zeros(r1 - r0 + 1, dtype=np.int64)
    np.cumsum(rowlen, out=rowptr[1:])
    nnz = int(rowptr[-1])
    col = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=np.float64)
    L.or_build_upper_fill(_p(b, _u64p), len(b), norb, _p(kt, _u16p), _p(vt, _f64p), K, r0, r1,
                          _p(rowptr, _i64p), _p(col, _i32p), _p(val, _f64p), nt)
    return rowptr, col, val


def upper_to_full(rowptr, col, val, n):
    """Both triangles of the symmetric matrix as CRS with ascending columns;
    the lower entries are the exact transposes of the stored upper ones."""
    import scipy.sparse as sp
    U = sp.csr_matrix((val, col, rowptr), shape=(n, n))
    D = sp.diags(U.diagonal())
    A = (U + U.T - D).tocsr()
    A.sort_indices()
    # drop structural zeros that the sum above cannot create (kept explicit)
    return A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.astype(np.float64)


def spmv_sym_upper(rowptr, col, val, x, nthreads: int = 1):
    """y = H x from the stored upper triangle (sparse_linear_algebra.hpp:143-164)."""
    n = len(rowptr) - 1
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(n, dtype=np.float64)
    L = lib()
    if nthreads <= 1:
        L.or_spmv_sym_upper(_p(rowptr, _i64p), _p(col, _i32p), _p(val, _f64p), n, _p(x, _f64p), _p(y, _f64p))
    else:
        work = np.empty(n * nthreads, dtype=np.float64)
        L.or_spmv_sym_upper_mt(_p(rowptr, _i64p), _p(col, _i32p), _p(val, _f64p), n, _p(x, _f64p),
                               _p(y, _f64p), _p(work, _f64p), nthreads)
    return y


# -------------------------------------------------------------- eigen oracle

def start_vector(n: int, seed: int) -> np.ndarray:
    """Seeded uniform(-1,1) start vector, normalised."""
    v = np.random.default_rng(seed).uniform(-1.0, 1.0, n)
    return v / np.linalg.norm(v)


def lowest_eigenpairs(rowptr, col, val, nev: int, tol: float = 1e-12, v0=None, upper: bool = True,
                      nthreads: int = 1, driver: str = "eigs"):
    """Lowest ``nev`` eigenpairs with SciPy's ARPACK.  ``driver='eigs'`` uses the
    non-symmetric driver with which='SR', ncv = min(n, 2*nev+21) and maxiter
    2000, the reference's settings (arpack_wrapper.hpp:702-708); ``'eigsh'``
    uses the symmetric driver.  The matrix-vector product is the upper-
    triangle loop of the reference when ``upper`` is set."""
    import scipy.sparse.linalg as sla
    n = len(rowptr) - 1
    if upper:
        op = sla.LinearOperator((n, n), matvec=lambda x: spmv_sym_upper(rowptr, col, val, x, nthreads),
                                dtype=np.float64)
    else:
        import scipy.sparse as sp
        op = sp.csr_matrix((val, col, rowptr), shape=(n, n))
    ncv = min(n, 2 * nev + 21)
    if driver == "eigs":
        w, v = sla.eigs(op, k=nev, which="SR", tol=tol, v0=v0, ncv=ncv, maxiter=2000)
        w, v = w.real, v.real
    else:
        w, v = sla.eigsh(op, k=nev, which="SA", tol=tol, v0=v0, ncv=ncv, maxiter=2000)
    order = np.argsort(w)
    w, v = w[order], v[:, order]
    v = v / np.linalg.norm(v, axis=0)
    return w, v


# ------------------------------------------------------------ two Landau levels

def basis2(N: int, norb0: int, two_lz: int):
    """TwoLevelFermionFockBasis::GenerateFockSpace (two_level_fermion_fock_basis.cpp:289-470)
    with TestAngularMomentumSector2LL (two_level_angular_momentum_constraint.hpp:41-70):
    for n0 = 0..N every lowest-level word of n0 bits and every second-level word
    of N - n0 bits (norb0 + 2 orbitals) whose Lz sum, 2i - (max-2) per
    lowest-level bit and 2j - max per second-level bit with max = norb0 + 1,
    equals two_lz; sorted by (first, second).  Returns (first, second)."""
    from itertools import combinations
    norb1 = norb0 + 2
    mx = norb1 - 1
    firsts, seconds = [], []
    for n0 in range(N + 1):
        n1 = N - n0
        if n0 > norb0 or n1 > norb1:
            continue
        w0 = [sum(1 << i for i in c) for c in combinations(range(norb0), n0)]
        l0 = [sum(2 * i - (mx - 2) for i in c) for c in combinations(range(norb0), n0)]
        by_lz = {}
        for c in combinations(range(norb1), n1):
            by_lz.setdefault(sum(2 * j - mx for j in c), []).append(sum(1 << j for j in c))
        for a, lz in zip(w0, l0):
            for b in by_lz.get(two_lz - lz, ()):
                firsts.append(a)
                seconds.append(b)
    order = sorted(range(len(firsts)), key=lambda i: (firsts[i], seconds[i]))
    return (np.array([firsts[i] for i in order], dtype=np.uint64),
            np.array([seconds[i] for i in order], dtype=np.uint64))


def build_upper2(first: np.ndarray, second: np.ndarray, norb0: int, kt0, vt0, kt1, vt1, e0=None, e1=None):
    """Upper-triangle CRS of the two-level Hamiltonian in the reference's call,
    loop and summation order: SphereTwoLevelPseudopotentialModel::BuildHamiltonian
    (two_level_pseudopotential_model.cpp:190-215) adds the quadratic
    occupation energies of level 0 then level 1 (Add_CdC_Terms,
    two_level_spinless_fermion_hamiltonian.hpp:143-270: diagonal E_k for every
    occupied k, ascending), then the quartic terms of level 0 then level 1
    (Add_CdCdCC_Terms, :306-470: the single-level loop on the level's word with
    the other word fixed).  Every term is kept when |term| > 1e-14 and added to
    its (row, column) entry in that order; entries below 1e-14 are trimmed
    (mapped_sparse_matrix.hpp:423-460) and columns sorted.  Python loops:
    small sectors only."""
    norb1 = norb0 + 2
    tol = 1e-14
    n = len(first)
    f_ = [int(x) for x in first]
    s_ = [int(x) for x in second]
    index = {(a, b): i for i, (a, b) in enumerate(zip(f_, s_))}
    rows = [dict() for _ in range(n)]

    def bits(w):
        while w:
            lo = w & -w
            yield lo.bit_length() - 1, lo
            w ^= lo

    for lvl, E in ((0, e0), (1, e1)):
        if E is None:
            continue
        for i in range(n):
            for k, _ in bits(f_[i] if lvl == 0 else s_[i]):
                v = float(E[k])
                if abs(v) > tol:
                    rows[i][i] = rows[i].get(i, 0.0) + v
    for lvl, kt, vt, K in ((0, kt0, vt0, norb0), (1, kt1, vt1, norb1)):
        mask = (1 << K) - 1
        for i in range(n):
            inw = f_[i] if lvl == 0 else s_[i]
            t4 = inw
            while t4:
                k4o = t4 & -t4
                k4 = k4o.bit_length() - 1
                t3 = inw ^ k4o
                while t3:
                    k3o = t3 & -t3
                    k3 = k3o.bit_length() - 1
                    if k3 != k4:
                        t2 = mask ^ (t3 ^ k3o)
                        while t2:
                            k2o = t2 & -t2
                            k2 = k2o.bit_length() - 1
                            idx = (k4 * K + k3) * K + k2
                            k1 = int(kt[idx])
                            if k1 < K:
                                k1o = 1 << k1
                                if ((not (k1o & inw) or (k1o & k3o) or (k1o & k4o)) and
                                        (not (k2o & inw) or (k2o & k3o) or (k2o & k4o)) and not (k1o & k2o)):
                                    out, sign = evaluate_cdcdcc(k1, k2, k3, k4, inw, K)
                                    if sign != 0 and out >= inw:
                                        j = index.get((out, s_[i]) if lvl == 0 else (f_[i], out))
                                        if j is not None:
                                            v = float(sign) * float(vt[idx])
                                            if abs(v) > tol:
                                                rows[i][j] = rows[i].get(j, 0.0) + v
                            t2 ^= k2o
                    t3 ^= k3o
                t4 ^= k4o
    rowptr = np.zeros(n + 1, dtype=np.int64)
    cols, vals = [], []
    for i in range(n):
        kept = sorted((j, v) for j, v in rows[i].items() if not abs(v) < tol)
        cols.extend(j for j, _ in kept)
        vals.extend(v for _, v in kept)
        rowptr[i + 1] = len(cols)
    return rowptr, np.array(cols, dtype=np.int32), np.array(vals, dtype=np.float64)


# ------------------------------------------- complex momentum path (OFL)

def basis_momentum(N: int, X: int, Y: int, kx: int, ky: int) -> np.ndarray:
    """FermionFockBasis::GenerateFockSpace with TestLinearMomentumSector2
    (interacting_ofl_model.cpp:994-1001, linear_momentum_constraints_2D.cpp:38-79):
    every N-bit word over X*Y orbitals (bit p at kx = p // Y, ky = p % Y) with
    (sum kx mod X, sum ky mod Y) == (kx, ky), ascending."""
    from itertools import combinations
    K = X * Y
    out = []
    for c in combinations(range(K), N):
        if sum(p // Y for p in c) % X == kx and sum(p % Y for p in c) % Y == ky:
            out.append(sum(1 << p for p in c))
    return np.array(sorted(out), dtype=np.uint64)


def ofl_index(k3: int, k4: int, K: int) -> int:
    """Triangular (k3, k4) index of the reference's OFL term tables
    (interacting_ofl_model/term_tables.cpp:108-126)."""
    t1, t2 = (k3, k4) if k4 > k3 else (k4, k3)
    return t1 * K + t2 - t1 * (t1 + 1) // 2


def ofl_k1(ktab, K: int, k2: int, k3: int, k4: int) -> int:
    """QuarticTermTables::GetK1 (term_tables.cpp:108-126)."""
    return int(ktab[ofl_index(k3, k4, K) * K + k2])


def ofl_v(vtab, K: int, k1: int, k2: int, k3: int, k4: int) -> complex:
    """QuarticTermTables::GetVkkkk (term_tables.cpp:157-175): the entry of
    (min, max)(k3, k4) at k2, or at k1 when k4 > k3."""
    return complex(vtab[ofl_index(k3, k4, K) * K + (k1 if k4 > k3 else k2)])


def ofl_tables(X: int, Y: int, seed: int, scale: float = 1.0):
    """Seeded momentum-conserving complex tables in the reference's layout:
    k1 from FindK1's rule (interacting_ofl_model.cpp:366-410: kx1 = kx3 + kx4 -
    kx2 and ky1 likewise, modulo the grid) and V uniform in the unit square
    (the Bloch-overlap integrals of BuildTermTables are not restated).  Returns
    (ktab uint16, vtab complex128), (K+1) K^2 / 2 entries each."""
    K = X * Y
    dim = (K + 1) * K * K // 2
    ktab = np.zeros(dim, dtype=np.uint16)
    for t1 in range(K):
        for t2 in range(t1, K):
            base = ofl_index(t1, t2, K) * K
            for k2 in range(K):
                kx = (t1 // Y + t2 // Y - k2 // Y) % X
                ky = (t1 % Y + t2 % Y - k2 % Y) % Y
                ktab[base + k2] = kx * Y + ky
    rng = np.random.default_rng(seed)
    vtab = scale * (rng.uniform(-1, 1, dim) + 1j * rng.uniform(-1, 1, dim))
    # the diagonal terms V(k4,k3,k3,k4) and V(k3,k4,k3,k4) read the entries at
    # k = min(k3,k4) and max(k3,k4): real there, as Hermitian tables have them,
    # so that the completed operator is Hermitian
    for t1 in range(K):
        for t2 in range(t1, K):
            base = ofl_index(t1, t2, K) * K
            vtab[base + t1] = vtab[base + t1].real
            vtab[base + t2] = vtab[base + t2].real
    return ktab, vtab


def build_upper_complex(words: np.ndarray, K: int, ktab, vtab, energies=None):
    """Upper-triangle complex CRS of SpinlessFermionHamiltonian<dcmplx> in the
    reference's loop and summation order (spinless_fermion_hamiltonian.hpp:150-436,
    as InteractingOflModel::BuildHamiltonian calls it, interacting_ofl_model.cpp:
    1047-1050): Add_CdC_Terms (E_k for every occupied k, ascending) then
    Add_CdCdCC_Terms (k4 over occupied bits ascending, k3 over the others, k2 over
    the complement of the higher occupied bits, k1 from the k-table, the occupancy
    filters, Evaluate_CdCdCC, out >= in); each term kept when abs > 1e-14 and
    added to entry (row = in, column = out) in arrival order; entries with abs <
    1e-14 trimmed; columns ascending.  Python loops: small sectors only."""
    tol = 1e-14
    n = len(words)
    ws = [int(w) for w in words]
    index = {w: i for i, w in enumerate(ws)}
    mask = (1 << K) - 1
    rows = [dict() for _ in range(n)]
    if energies is not None:
        for i, w in enumerate(ws):
            t = w
            while t:
                lo = t & -t
                k = lo.bit_length() - 1
                v = complex(energies[k])
                if abs(v) > tol:
                    rows[i][i] = rows[i].get(i, 0j) + v
                t ^= lo
    for i, inw in enumerate(ws):
        t4 = inw
        while t4:
            k4o = t4 & -t4
            k4 = k4o.bit_length() - 1
            t3 = inw ^ k4o
            while t3:
                k3o = t3 & -t3
                k3 = k3o.bit_length() - 1
                if k3 != k4:
                    t2 = mask ^ (t3 ^ k3o)
                    while t2:
                        k2o = t2 & -t2
                        k2 = k2o.bit_length() - 1
                        k1 = ofl_k1(ktab, K, k2, k3, k4)
                        k1o = 1 << k1
                        if ((not (k1o & inw) or (k1o & k3o) or (k1o & k4o)) and
                                (not (k2o & inw) or (k2o & k3o) or (k2o & k4o)) and not (k1o & k2o)):
                            out, sign = evaluate_cdcdcc(k1, k2, k3, k4, inw, K)
                            if sign != 0 and out >= inw:
                                j = index.get(out)
                                if j is not None:
                                    v = float(sign) * ofl_v(vtab, K, k1, k2, k3, k4)
                                    if abs(v) > tol:
                                        rows[i][j] = rows[i].get(j, 0j) + v
                        t2 ^= k2o
                t3 ^= k3o
            t4 ^= k4o
    rowptr = np.zeros(n + 1, dtype=np.int64)
    cols, vals = [], []
    for i in range(n):
        kept = sorted((j, v) for j, v in rows[i].items() if not abs(v) < tol)
        cols.extend(j for j, _ in kept)
        vals.extend(v for _, v in kept)
        rowptr[i + 1] = len(cols)
    return rowptr, np.array(cols, dtype=np.int32), np.array(vals, dtype=np.complex128)


def basis_momentum_c(N: int, X: int, Y: int, kx: int, ky: int) -> np.ndarray:
    """C restatement of basis_momentum (oracle.c or_basis_momentum)."""
    n = int(lib().or_basis_momentum(N, X, Y, kx, ky, None))
    out = np.empty(n, dtype=np.uint64)
    if n:
        lib().or_basis_momentum(N, X, Y, kx, ky, _p(out, _u64p))
    return out


def build_upper_complex_c(words: np.ndarray, K: int, ktab, vtab, energies=None, nthreads: int | None = None):
    """C restatement of build_upper_complex (oracle.c or_cbuild_row, same
    loops and arrival-order accumulation), multi-threaded over rows: the CPU
    baseline of the complex build."""
    nt = nthreads or num_procs()
    w = np.ascontiguousarray(words, dtype=np.uint64)
    kt = np.ascontiguousarray(ktab, dtype=np.uint16)
    vt = np.ascontiguousarray(np.asarray(vtab, dtype=np.complex128).view(np.float64))
    e = None if energies is None else np.ascontiguousarray(np.asarray(energies, dtype=np.complex128).view(np.float64))
    n = len(w)
    rowlen = np.zeros(n, dtype=np.int64)
    L = lib()
    L.or_cbuild_upper(_p(w, _u64p), n, K, _p(kt, _u16p), _p(vt, _f64p), None if e is None else _p(e, _f64p),
                      _p(rowlen, _i64p), None, None, None, nt)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(rowlen, out=rowptr[1:])
    col = np.empty(int(rowptr[-1]), dtype=np.int32)
    val = np.empty(int(rowptr[-1]), dtype=np.complex128)
    L.or_cbuild_upper(_p(w, _u64p), n, K, _p(kt, _u16p), _p(vt, _f64p), None if e is None else _p(e, _f64p),
                      None, _p(rowptr, _i64p), _p(col, _i32p), _p(val.view(np.float64), _f64p), nt)
    return rowptr, col, val


def cspmv_upper(rowptr, col, val, x, nthreads: int | None = None) -> np.ndarray:
    """The reference's complex upper-triangle product (or_cspmv_upper_mt)."""
    nt = nthreads or num_procs()
    n = len(rowptr) - 1
    xv = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).view(np.float64))
    y = np.empty(2 * n)
    scratch = np.empty(2 * n * nt)
    v = np.ascontiguousarray(np.asarray(val, dtype=np.complex128).view(np.float64))
    lib().or_cspmv_upper_mt(_p(np.ascontiguousarray(rowptr, dtype=np.int64), _i64p),
                            _p(np.ascontiguousarray(col, dtype=np.int32), _i32p), _p(v, _f64p), n, _p(xv, _f64p),
                            _p(y, _f64p), _p(scratch, _f64p), nt)
    return y.view(np.complex128)


def complex_upper_to_full(rowptr, col, val, n):
    """The reference's Hermitian completion of the upper storage
    (sparse_linear_algebra.hpp:148-164): M = U + conj(strictly upper U)^T,
    as CRS with ascending columns."""
    import scipy.sparse as sp
    U = sp.csr_matrix((val, col, rowptr), shape=(n, n))
    S = sp.triu(U, 1)
    M = (U + S.conj().T).tocsr()
    M.sort_indices()
    return M.indptr.astype(np.int64), M.indices.astype(np.int32), M.data.astype(np.complex128)


def basis2_c(N: int, norb0: int, two_lz: int) -> np.ndarray:
    """The two-level basis as combined words (first << (norb0+2)) | second,
    ascending: the C restatement of basis2 (oracle.c or_basis2_build)."""
    n = int(lib().or_basis2_build(N, norb0, two_lz, None))
    out = np.empty(n, dtype=np.uint64)
    if n:
        lib().or_basis2_build(N, norb0, two_lz, _p(out, _u64p))
    return out


def build_upper2_c(words: np.ndarray, norb0: int, kt0, vt0, kt1, vt1, e0=None, e1=None,
                   nthreads: int | None = None):
    """The C restatement of build_upper2 (oracle.c or_build2_row: same loops,
    same arrival-order accumulation) over combined words, multi-threaded over
    rows: the CPU baseline of the two-level build."""
    nt = nthreads or num_procs()
    w = np.ascontiguousarray(words, dtype=np.uint64)
    a0 = [np.ascontiguousarray(kt0, dtype=np.uint16), np.ascontiguousarray(vt0, dtype=np.float64)]
    a1 = [np.ascontiguousarray(kt1, dtype=np.uint16), np.ascontiguousarray(vt1, dtype=np.float64)]
    ee = [None if e is None else np.ascontiguousarray(e, dtype=np.float64) for e in (e0, e1)]
    ep = [None if e is None else _p(e, _f64p) for e in ee]
    n = len(w)
    rowlen = np.zeros(n, dtype=np.int64)
    L = lib()
    L.or_build2_upper_count(_p(w, _u64p), n, norb0, _p(a0[0], _u16p), _p(a0[1], _f64p), _p(a1[0], _u16p),
                            _p(a1[1], _f64p), ep[0], ep[1], _p(rowlen, _i64p), nt)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(rowlen, out=rowptr[1:])
    col = np.empty(int(rowptr[-1]), dtype=np.int32)
    val = np.empty(int(rowptr[-1]), dtype=np.float64)
    L.or_build2_upper_fill(_p(w, _u64p), n, norb0, _p(a0[0], _u16p), _p(a0[1], _f64p), _p(a1[0], _u16p),
                           _p(a1[1], _f64p), ep[0], ep[1], _p(rowptr, _i64p), _p(col, _i32p), _p(val, _f64p), nt)
    return rowptr, col, val


# ------------------------------------------------------------ observables

def density(words: np.ndarray, psi: np.ndarray, norb: int) -> np.ndarray:
    """rho[k] = sum_s |psi_s|^2 n_k(s) (psi real or complex): Observables::DensityFunction
    (fermion_observables.hpp:48-104), the state loop binning each occupied
    orbital (bit k of the word) with the state's probability."""
    p = np.abs(np.asarray(psi)) ** 2
    w = np.asarray(words, dtype=np.uint64)
    return np.array([p[((w >> np.uint64(k)) & np.uint64(1)) == 1].sum() for k in range(norb)])


def density_density(words: np.ndarray, psi: np.ndarray, norb: int) -> np.ndarray:
    """D[k, q] = sum_s |psi_s|^2 n_k(s) n_q(s): Observables::DensityDensityFunction
    (fermion_observables.hpp:117-200) -- the k = q bin gets n_k^2 = n_k and
    every ordered pair of distinct occupied orbitals its (k, q) bin."""
    p = np.abs(np.asarray(psi)) ** 2
    w = np.asarray(words, dtype=np.uint64)
    occ = np.stack([((w >> np.uint64(k)) & np.uint64(1)).astype(np.float64) for k in range(norb)], axis=1)
    return (occ * p[:, None]).T @ occ


def participation_ratio(psi: np.ndarray) -> float:
    """1 / sum_s |psi_s|^4: Observables::GetParticipationRatio
    (fermion_observables.hpp:528-562; the code returns 1/sum, its 1/D factor
    is commented out)."""
    return 1.0 / float(np.sum(np.abs(np.asarray(psi)) ** 4))


def most_probable(words: np.ndarray, psi: np.ndarray, k: int):
    """The min(k, n) largest |psi_s| in descending order with their words:
    Observables::GetMostProbable (fermion_observables.hpp:437-517) for one
    eigenvector (real or complex; ranked by modulus); ties (unordered in the
    reference's partial quicksort) by row."""
    psi = np.asarray(psi)
    m = min(int(k), len(psi))
    order = np.lexsort((np.arange(len(psi)), -np.abs(psi)))[:m]
    return np.asarray(words, dtype=np.uint64)[order], psi[order]


# ----------------------------------------------- pin against the reference

def ref_lib():
    """The reference's own primitives (oracle/_ref/libref.so), or None."""
    if not os.path.exists(REF_PATH):
        try:
            if build_ref() is None:
                return None
        except Exception:
            return None
    L = ctypes.CDLL(REF_PATH)
    L.ref_evaluate_cdcdcc.restype = ctypes.c_uint64
    L.ref_evaluate_cdcdcc.argtypes = [ctypes.POINTER(ctypes.c_int)] + [ctypes.c_uint64] * 6
    L.ref_next_hamming.restype = ctypes.c_uint64
    L.ref_next_hamming.argtypes = [ctypes.c_uint64]
    L.ref_generate_hamming.restype = ctypes.c_uint64
    L.ref_generate_hamming.argtypes = [ctypes.c_uint, ctypes.c_uint64]
    L.ref_hamming_weight.restype = ctypes.c_int
    L.ref_hamming_weight.argtypes = [ctypes.c_uint64]
    L.ref_base2log.restype = ctypes.c_uint
    L.ref_base2log.argtypes = [ctypes.c_uint64]
    L.ref_binomial.restype = ctypes.c_long
    L.ref_binomial.argtypes = [ctypes.c_int, ctypes.c_int]
    L.ref_binary_search.restype = ctypes.c_uint64
    L.ref_binary_search.argtypes = [ctypes.c_uint64, _u64p, ctypes.c_uint64]
    L.ref_lz_ok.restype = ctypes.c_int
    L.ref_lz_ok.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
    return L


# ------------------------- pin against the reference's basis, build, observables

def ref_ham_lib():
    """The reference's own sector basis, quartic build and observables
    (oracle/_ref/libref_ham.so, built by `make ref` with the reference tree
    present), or None."""
    if not os.path.exists(REF_HAM_PATH):
        try:
            if build_ref() is None or not os.path.exists(REF_HAM_PATH):
                return None
        except Exception:
            return None
    L = ctypes.CDLL(REF_HAM_PATH)
    L.refh_basis.restype = ctypes.c_uint64
    L.refh_basis.argtypes = [ctypes.c_int] * 3 + [_u64p]
    L.refh_build_crs_file.restype = ctypes.c_int64
    L.refh_build_crs_file.argtypes = [ctypes.c_int] * 3 + [_u16p, _f64p, ctypes.c_char_p]
    L.refh_observables.restype = ctypes.c_int
    L.refh_observables.argtypes = [ctypes.c_int] * 3 + [_f64p, ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p]
    L.refh2_basis.restype = ctypes.c_uint64
    L.refh2_basis.argtypes = [ctypes.c_int] * 3 + [_u64p, _u64p]
    L.refh2_build_crs_file.restype = ctypes.c_int64
    L.refh2_build_crs_file.argtypes = [ctypes.c_int] * 3 + [_u16p, _f64p, _u16p, _f64p, _f64p, _f64p, ctypes.c_char_p]
    L.refh_most_probable_complex.restype = ctypes.c_int
    L.refh_most_probable_complex.argtypes = [ctypes.c_int] * 3 + [_f64p, ctypes.c_int, ctypes.c_int, _u64p, _f64p]
    return L


def ref_basis(R, N: int, norb: int, two_lz: int) -> np.ndarray:
    """FermionFockBasis::GenerateFockSpace of the reference (fermion_fock_basis.cpp:241-354)."""
    n = R.refh_basis(N, norb, two_lz, None)
    w = np.empty(n, dtype=np.uint64)
    if n:
        R.refh_basis(N, norb, two_lz, _p(w, _u64p))
    return w


def read_reference_crs(path: str):
    """A CRS file in the reference's binary format (crs_sparse_matrix.hpp:662-705:
    uint32 nnz, uint32 rows, int32 row starts, int32 columns, values)."""
    raw = open(path, "rb").read()
    nnz, rows = (int(x) for x in np.frombuffer(raw[:8], dtype=np.uint32))
    o = 8
    rp = np.frombuffer(raw[o:o + 4 * (rows + 1)], dtype=np.int32).astype(np.int64)
    o += 4 * (rows + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32).copy()
    o += 4 * nnz
    val = np.frombuffer(raw[o:o + 8 * nnz], dtype=np.float64).copy()
    return rp, col, val


def ref_build_upper(R, N: int, norb: int, two_lz: int, ktab, vtab):
    """The reference's own SpinlessFermionHamiltonian<double>::Add_CdCdCC_Terms
    (spinless_fermion_hamiltonian.hpp:282-436) into its mapped storage, trim and
    CRS conversion, from the given term tables; (rowptr int64, col, val)."""
    import tempfile
    kt = np.ascontiguousarray(ktab, dtype=np.uint16)
    vt = np.ascontiguousarray(vtab, dtype=np.float64)
    fd, path = tempfile.mkstemp(suffix=".bin")
    os.close(fd)
    try:
        nnz = R.refh_build_crs_file(N, norb, two_lz, _p(kt, _u16p), _p(vt, _f64p), path.encode())
        if nnz < 0:
            return None
        return read_reference_crs(path)
    finally:
        os.unlink(path)


def crs_digest(rowptr, col, val) -> str:
    """SHA-256 of a CRS: row pointers as little-endian int64, columns as int32,
    values as their FP64 bits."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rowptr, dtype="<i8").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(val, dtype="<f8").tobytes())
    return h.hexdigest()


def ref_basis2(R, N: int, norb0: int, two_lz: int):
    """TwoLevelFermionFockBasis::GenerateFockSpace of the reference
    (two_level_fermion_fock_basis.cpp:289-506); (first, second) words."""
    n = R.refh2_basis(N, norb0, two_lz, None, None)
    f = np.empty(n, dtype=np.uint64)
    s = np.empty(n, dtype=np.uint64)
    if n:
        R.refh2_basis(N, norb0, two_lz, _p(f, _u64p), _p(s, _u64p))
    return f, s


def ref_build_upper2(R, N: int, norb0: int, two_lz: int, kt0, vt0, kt1, vt1, e0=None, e1=None):
    """The reference's own two-level model build (two_level_pseudopotential_model.cpp:190-215:
    Add_CdC_Terms of each level, then Add_CdCdCC_Terms of level 0 and level 1,
    two_level_spinless_fermion_hamiltonian.hpp:143-470), trim and CRS conversion."""
    import tempfile
    a = [np.ascontiguousarray(x, dtype=t) for x, t in ((kt0, np.uint16), (vt0, np.float64), (kt1, np.uint16),
                                                         (vt1, np.float64))]
    e = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (e0, e1)]
    fd, path = tempfile.mkstemp(suffix=".bin")
    os.close(fd)
    try:
        nnz = R.refh2_build_crs_file(N, norb0, two_lz, _p(a[0], _u16p), _p(a[1], _f64p), _p(a[2], _u16p),
                                     _p(a[3], _f64p), None if e[0] is None else _p(e[0], _f64p),
                                     None if e[1] is None else _p(e[1], _f64p), path.encode())
        if nnz < 0:
            return None
        return read_reference_crs(path)
    finally:
        os.unlink(path)


def ref_ofl_lib():
    """The reference's own momentum-sector basis and complex optical-flux-lattice
    build (oracle/_ref/libref_ofl.so), or None."""
    if not os.path.exists(REF_OFL_PATH):
        try:
            if build_ref() is None or not os.path.exists(REF_OFL_PATH):
                return None
        except Exception:
            return None
    L = ctypes.CDLL(REF_OFL_PATH)
    L.refo_basis.restype = ctypes.c_uint64
    L.refo_basis.argtypes = [ctypes.c_int] * 5 + [_u64p]
    L.refo_build_crs_file.restype = ctypes.c_int64
    L.refo_build_crs_file.argtypes = [ctypes.c_int] * 5 + [_u16p, _f64p, _f64p, ctypes.c_char_p]
    if hasattr(L, "refo_hash_files"):
        L.refo_hash_files.restype = ctypes.c_int
        L.refo_hash_files.argtypes = [ctypes.c_int] * 2 + [_u16p, _f64p, _f64p, ctypes.c_char_p, ctypes.c_char_p,
                                                           ctypes.c_int]
        L.refo_hash_read.restype = ctypes.c_int
        L.refo_hash_read.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _u16p,
                                     ctypes.POINTER(ctypes.c_uint32), _f64p]
        L.refo_build_crs_file_hash.restype = ctypes.c_int64
        L.refo_build_crs_file_hash.argtypes = [ctypes.c_int] * 5 + [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                                                    ctypes.c_char_p]
    return L


def _read_reference_ccrs(path: str):
    """A complex CRS file of the reference's binary format: (rowptr int64,
    col, complex values)."""
    raw = open(path, "rb").read()
    nnz, rows = (int(x) for x in np.frombuffer(raw[:8], dtype=np.uint32))
    o = 8
    rp = np.frombuffer(raw[o:o + 4 * (rows + 1)], dtype=np.int32).astype(np.int64)
    o += 4 * (rows + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32).copy()
    o += 4 * nnz
    val = np.frombuffer(raw[o:o + 16 * nnz], dtype=np.complex128).copy()
    return rp, col, val


def ref_hash_files(R, X: int, Y: int, ktab, vtab, energies, quartic_path: str, quadratic_path: str,
                   binary: bool = True):
    """The reference's hash tables filled from array tables
    (term_hash_tables_base.hpp:229-275 SetQuarticFromArray /
    SetQuadraticFromArray) and written by its ToFile (:139-170)."""
    kt = np.ascontiguousarray(ktab, dtype=np.uint16)
    vt = np.ascontiguousarray(vtab, dtype=np.complex128).view(np.float64)
    e = None if energies is None else np.ascontiguousarray(energies, dtype=np.complex128).view(np.float64)
    rc = R.refo_hash_files(X, Y, _p(kt, _u16p), _p(vt, _f64p), None if e is None else _p(e, _f64p),
                           quartic_path.encode(), quadratic_path.encode(), int(binary))
    if rc != 0:
        raise RuntimeError("reference hash-table writer failed")


def ref_hash_read(R, K: int, quartic_path: str, binary: bool = True):
    """What the reference reads back from a quartic hash-table file (FromFile,
    GetK1, GetVkkkk): (first k1 [K,K,K] with 65535 where none, k1 counts
    [K,K,K], V [K,K,K,K] complex), indexed [k2,k3,k4] and [k1,k2,k3,k4]."""
    k1 = np.empty(K ** 3, dtype=np.uint16)
    nk = np.empty(K ** 3, dtype=np.uint32)
    v = np.empty(2 * K ** 4, dtype=np.float64)
    if R.refo_hash_read(K, quartic_path.encode(), int(binary), _p(k1, _u16p),
                        nk.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _p(v, _f64p)) != 0:
        raise RuntimeError("reference hash-table reader failed")
    return k1.reshape(K, K, K), nk.reshape(K, K, K), v.view(np.complex128).reshape(K, K, K, K)


def ref_build_upper_complex_hash(R, N: int, X: int, Y: int, kx: int, ky: int, quartic_path: str,
                                 quadratic_path: str, binary: bool = True):
    """The reference's own complex build from hash-table files (the
    hash-format branch of interacting_ofl_model.cpp:1046-1049); (rowptr
    int64, col, complex values), or None for an empty sector."""
    import tempfile
    fd, path = tempfile.mkstemp(suffix=".bin")
    os.close(fd)
    try:
        nnz = R.refo_build_crs_file_hash(N, X, Y, kx, ky, quartic_path.encode(), quadratic_path.encode(),
                                         int(binary), path.encode())
        if nnz < 0:
            return None
        return _read_reference_ccrs(path)
    finally:
        os.unlink(path)


def ref_basis_momentum(R, N: int, X: int, Y: int, kx: int, ky: int) -> np.ndarray:
    """The reference's momentum-sector basis (interacting_ofl_model.cpp:990-1000)."""
    n = R.refo_basis(N, X, Y, kx, ky, None)
    w = np.empty(n, dtype=np.uint64)
    if n:
        R.refo_basis(N, X, Y, kx, ky, _p(w, _u64p))
    return w


def ref_build_upper_complex(R, N: int, X: int, Y: int, kx: int, ky: int, ktab, vtab, energies=None):
    """The reference's own complex build from array-format tables
    (interacting_ofl_model.cpp:1034-1052: Add_CdC_Terms, Add_CdCdCC_Terms of
    SpinlessFermionHamiltonian<dcmplx>), trim and CRS conversion;
    (rowptr int64, col, complex values)."""
    import tempfile
    kt = np.ascontiguousarray(ktab, dtype=np.uint16)
    vt = np.ascontiguousarray(vtab, dtype=np.complex128).view(np.float64)
    e = None if energies is None else np.ascontiguousarray(energies, dtype=np.complex128).view(np.float64)
    fd, path = tempfile.mkstemp(suffix=".bin")
    os.close(fd)
    try:
        nnz = R.refo_build_crs_file(N, X, Y, kx, ky, _p(kt, _u16p), _p(vt, _f64p),
                                    None if e is None else _p(e, _f64p), path.encode())
        if nnz < 0:
            return None
        raw = open(path, "rb").read()
    finally:
        os.unlink(path)
    nnz, rows = (int(x) for x in np.frombuffer(raw[:8], dtype=np.uint32))
    o = 8
    rp = np.frombuffer(raw[o:o + 4 * (rows + 1)], dtype=np.int32).astype(np.int64)
    o += 4 * (rows + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32).copy()
    o += 4 * nnz
    val = np.frombuffer(raw[o:o + 16 * nnz], dtype=np.complex128).copy()
    return rp, col, val
