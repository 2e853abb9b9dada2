"""Host-side mirror of the reference's C++ call surface for the hot path,
over the C ABI of libedgb300.

Classes keep the reference's names, method names and argument meaning so a
caller of the reference finds the same entry points; the `mpi` arguments are
accepted and ignored (one GPU, no ranks):

  FermionFockBasis            basis/fermion_fock_basis.hpp:45
  QuarticTermTables           fqhe_sphere/pseudopotential_model/term_tables.hpp
  SpinlessFermionHamiltonian  hamiltonians/spinless_fermion_hamiltonian.hpp:52
  MatrixVectorFunction        hamiltonians/matrix_vector_routines.hpp:41
  ArpackWrapper               utilities/wrappers/arpack_wrapper.hpp:187
  SpherePseudopotentialModel  fqhe_sphere/pseudopotential_model/pseudopotential_model.hpp
Errors surface as EDError (status code + message), the counterpart of the
reference's exit flag.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C
from ._capi import EDError, LanczosParams, SolveInfo, check, lib

SPARSE_MAPPED = 1   # utilities::_SPARSE_MAPPED_ (build-time storage of the reference)
SPARSE_CRS = 2      # utilities::_SPARSE_CRS_


class MpiWrapper:
    """Stand-in for utilities::MpiWrapper: a single rank."""
    m_id = 0
    m_nbrProcs = 1
    m_exitFlag = False

    def ExitFlagTest(self):
        if self.m_exitFlag:
            raise EDError(C.ED_ERR_ARG, "exit flag set")


def _dptr(t) -> int:
    """Device pointer of a CUDA tensor-like object (torch.Tensor)."""
    if hasattr(t, "data_ptr"):
        if hasattr(t, "is_cuda") and not t.is_cuda:
            raise EDError(C.ED_ERR_ARG, "expected a device (CUDA) tensor")
        return int(t.data_ptr())
    return int(t)


def _f64p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def coulomb_pseudopotentials(norb: int) -> np.ndarray:
    """LLL Coulomb V_m, m = 0..norb-1 (coulomb_pseudopotentials.cpp:40-69)."""
    out = np.zeros(norb)
    check(lib().ed_coulomb_pseudopotentials(norb, _f64p(out)))
    return out


def odd_coulomb_list(norb: int) -> np.ndarray:
    """Coulomb V_m for odd m <= 2S-1, even m zero, length 2S: the list the
    measured configurations pass as --two-body-pseudopotentials."""
    v = coulomb_pseudopotentials(norb)[: norb - 1].copy()
    v[0::2] = 0.0
    return v


def clebsch_gordan(tj1, tm1, tj2, tm2, tJ, tM) -> float:
    return float(lib().ed_clebsch_gordan(tj1, tm1, tj2, tm2, tJ, tM))


def dense_sym_eigen(a: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.float64)
    m = a.shape[0]
    ev = np.empty(m)
    vec = np.empty(m * m)
    check(lib().ed_dense_sym_eigen(m, _f64p(a), _f64p(ev), _f64p(vec)))
    return ev, vec.reshape(m, m).T.copy()


class QuarticTermTables:
    """k-table / V-table container (QuarticTermTables) plus its device image."""

    def __init__(self, nbrOrbitals: int, pseudopotentials=None, ktable=None, vtable=None):
        self.m_kMax = int(nbrOrbitals)
        K = self.m_kMax
        if ktable is None or vtable is None:
            pp = np.ascontiguousarray(pseudopotentials if pseudopotentials is not None else [0.0, 1.0],
                                      dtype=np.float64)
            ktable = np.empty(K ** 3, dtype=np.uint16)
            vtable = np.empty(K ** 3, dtype=np.float64)
            check(lib().ed_quartic_tables(K, _f64p(pp), len(pp), ktable.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                          _f64p(vtable)))
        self.m_kTable = np.ascontiguousarray(ktable, dtype=np.uint16)
        self.m_vTable = np.ascontiguousarray(vtable, dtype=np.float64)
        self._h = None

    # term_tables.cpp:109-124
    def GetMaxKCount(self) -> int:
        return 1

    def GetK1(self, k2: int, k3: int, k4: int) -> list:
        k1 = int(self.m_kTable[(k4 * self.m_kMax + k3) * self.m_kMax + k2])
        return [k1] if k1 < self.m_kMax else []

    # term_tables.cpp:144-156
    def GetVkkkk(self, k1: int, k2: int, k3: int, k4: int) -> float:
        return float(self.m_vTable[(k4 * self.m_kMax + k3) * self.m_kMax + k2])

    # term_tables_base.hpp:179-245 (4 labels); fmt "text" or "binary"
    def ToFile(self, fileName: str, fmt: str = "text", mpi=None):
        check(lib().ed_quartic_tables_write(fileName.encode(), int(fmt == "binary"), self.m_kMax,
                                            self.m_kTable.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                            _f64p(self.m_vTable)))

    # term_tables_base.hpp:250-335
    @classmethod
    def FromFile(cls, fileName: str, fmt: str = "text", mpi=None) -> "QuarticTermTables":
        K = ctypes.c_int()
        b = int(fmt == "binary")
        check(lib().ed_quartic_tables_read(fileName.encode(), b, ctypes.byref(K), None, None))
        kt = np.empty(K.value ** 3, dtype=np.uint16)
        vt = np.empty(K.value ** 3, dtype=np.float64)
        check(lib().ed_quartic_tables_read(fileName.encode(), b, ctypes.byref(K),
                                           kt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), _f64p(vt)))
        return cls(K.value, ktable=kt, vtable=vt)

    def handle(self):
        if self._h is None:
            h = ctypes.c_void_p()
            check(lib().ed_terms_set(self.m_kMax, self.m_kTable.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                     _f64p(self.m_vTable), ctypes.byref(h)))
            self._h = h
        return self._h

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_terms_free(self._h)
            self._h = None


class FermionFockBasis:
    """Sector basis on the device (fermion_fock_basis.hpp:45)."""

    def __init__(self):
        self._h = None
        self.m_basisStored = False

    def GenerateFockSpace(self, nbrParticles: int, nbrOrbitals: int, twoLz: int, mpi=None, stream=None) -> bool:
        """Build the fixed-Lz sector; returns True when its dimension is 0
        (fermion_fock_basis.cpp:241-354).  The reference takes the Lz
        predicate as a std::function; here the sector is named directly."""
        self.free()
        h = ctypes.c_void_p()
        check(lib().ed_basis_build(int(nbrParticles), int(nbrOrbitals), int(twoLz), stream, ctypes.byref(h)))
        self._h = h
        self.m_basisStored = True
        self.nbrParticles, self.nbrOrbitals, self.twoLz = int(nbrParticles), int(nbrOrbitals), int(twoLz)
        return self.GetStoredDimension() == 0

    def GenerateFockSpaceMomentum(self, nbrParticles: int, dimX: int, dimY: int, kxTot: int, kyTot: int, mpi=None,
                                  stream=None) -> bool:
        """The momentum sector (kxTot, kyTot) of dimX*dimY orbitals p = kx*dimY + ky:
        GenerateFockSpace with TestLinearMomentumSector2 (interacting_ofl_model.cpp:
        994-1001, linear_momentum_constraints_2D.cpp:38-79); True when empty."""
        self.free()
        h = ctypes.c_void_p()
        check(lib().ed_basis_momentum_build(int(nbrParticles), int(dimX), int(dimY), int(kxTot), int(kyTot), stream,
                                            ctypes.byref(h)))
        self._h = h
        self.m_basisStored = True
        self.nbrParticles, self.nbrOrbitals = int(nbrParticles), int(dimX) * int(dimY)
        self.dimX, self.dimY, self.kxTot, self.kyTot = int(dimX), int(dimY), int(kxTot), int(kyTot)
        return self.GetStoredDimension() == 0

    def handle(self):
        if self._h is None:
            raise EDError(C.ED_ERR_ARG, "basis not generated")
        return self._h

    def GetStoredDimension(self) -> int:
        d = ctypes.c_uint64()
        check(lib().ed_basis_dim(self.handle(), ctypes.byref(d)))
        return int(d.value)

    def GetFockBasis(self, dim: int | None = None, mpi=None) -> np.ndarray:
        n = self.GetStoredDimension() if dim is None else int(dim)
        out = np.empty(n, dtype=np.uint64)
        check(lib().ed_basis_get(self.handle(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n))
        return out

    def FindFockStateIndices(self, states) -> np.ndarray:
        w = np.ascontiguousarray(states, dtype=np.uint64)
        out = np.empty(len(w), dtype=np.uint64)
        check(lib().ed_basis_rank_host(self.handle(), w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(w)))
        return out

    def FindFockStateIndex(self, offset: int, state: int) -> int:
        """Index of `state` (+offset), UINT64_MAX when absent (fermion_fock_basis.cpp:134-161)."""
        i = int(self.FindFockStateIndices(np.array([state], dtype=np.uint64))[0])
        return i if i == C.MISS else i + int(offset)

    def words_device_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(lib().ed_basis_words(self.handle(), ctypes.byref(p)))
        return int(p.value or 0)

    def free(self):
        if self._h is not None and C._LIB is not None:
            C._LIB.ed_basis_free(self._h)
        self._h = None

    def __del__(self):
        self.free()


class TwoLevelFermionFockBasis(FermionFockBasis):
    """Two-Landau-level basis (two_level_fermion_fock_basis.hpp:62): states
    are (first, second) pairs of lowest- and second-level words, stored on the
    device as one word (first << nbrOrbitals2) | second, whose ascending
    order is the reference's sort (two_level_fermion_fock_basis.cpp:34-46)."""

    def GenerateFockSpace(self, nbrParticles: int, nbrOrbitals1: int, nbrOrbitals2: int, twoLz: int, mpi=None,
                          stream=None) -> bool:
        """TwoLevelFermionFockBasis::GenerateFockSpace with
        TestAngularMomentumSector2LL for the sector twoLz
        (two_level_fermion_fock_basis.cpp:289-470); True when empty."""
        if int(nbrOrbitals2) != int(nbrOrbitals1) + 2:
            raise EDError(C.ED_ERR_ARG, "the second level has nbrOrbitals1 + 2 orbitals on the sphere")
        self.free()
        h = ctypes.c_void_p()
        check(lib().ed_basis2_build(int(nbrParticles), int(nbrOrbitals1), int(twoLz), stream, ctypes.byref(h)))
        self._h = h
        self.m_basisStored = True
        self.nbrParticles, self.twoLz = int(nbrParticles), int(twoLz)
        self.nbrOrbitals1, self.nbrOrbitals2 = int(nbrOrbitals1), int(nbrOrbitals2)
        self.nbrOrbitals = self.nbrOrbitals1 + self.nbrOrbitals2
        return self.GetStoredDimension() == 0

    def GetWords(self) -> np.ndarray:
        """The combined words, ascending."""
        return FermionFockBasis.GetFockBasis(self)

    def GetFockBasis(self, dim: int | None = None, mpi=None):
        """(first, second) arrays (two_level_fermion_fock_basis.cpp:477-506)."""
        w = FermionFockBasis.GetFockBasis(self, dim)
        return w >> np.uint64(self.nbrOrbitals2), w & np.uint64((1 << self.nbrOrbitals2) - 1)

    def FindFockStateIndex(self, offset: int, first: int, second: int) -> int:
        """Index of the state (first, second) (+offset), UINT64_MAX when absent
        (two_level_fermion_fock_basis.cpp:211-241)."""
        word = (int(first) << self.nbrOrbitals2) | int(second)
        return FermionFockBasis.FindFockStateIndex(self, offset, word)


class CrsSparseMatrix:
    """Device CRS handle (crs_sparse_matrix.hpp:123) with int64 row pointers."""

    def __init__(self, h):
        self._h = h

    def info(self):
        n, nnz, up = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        check(lib().ed_crs_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(up)))
        return int(n.value), int(nnz.value), bool(up.value)

    def GetNbrRows(self) -> int:
        return self.info()[0]

    def GetNbrNonZeros(self) -> int:
        return self.info()[1]

    def to_host(self):
        n, nnz, _ = self.info()
        rp = np.empty(n + 1, dtype=np.int64)
        col = np.empty(max(nnz, 0), dtype=np.int32)
        val = np.empty(max(nnz, 0), dtype=np.float64)
        check(lib().ed_crs_get(self._h, rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                               col.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _f64p(val)))
        return rp, col, val

    # crs_sparse_matrix.hpp:662-705
    def ToFile(self, fileName: str, fmt: str = "text", mpi=None):
        check(lib().ed_crs_write(self._h, fileName.encode(), int(fmt == "binary")))

    # crs_sparse_matrix.hpp:710-740 (the final row start, absent from text files, is nnz)
    @classmethod
    def FromFile(cls, fileName: str, fmt: str = "text", upper: bool = True, mpi=None) -> "CrsSparseMatrix":
        h = ctypes.c_void_p()
        check(lib().ed_crs_read(fileName.encode(), int(fmt == "binary"), int(upper), ctypes.byref(h)))
        return cls(h)

    def set_product_kernel(self, kernel: int):
        """Kernel of every later product, eigensolvers included
        (ed_crs_set_product_kernel; 0 restores the choice by shape)."""
        check(lib().ed_crs_set_product_kernel(self._h, int(kernel)))

    def multiply(self, x, y, kernel: int = 0, stream=None):
        """y = A x on device vectors with a chosen product kernel (ed_spmv_kernel:
        0 by shape, 1 row lanes, 2-3 shared-reduction rows, 4-5 sliced ELL,
        6 fixed-point integer rows, 7 the same with bulk-copy staging, 8
        fixed-point sliced ELL)."""
        check(lib().ed_spmv_kernel(self._h, int(kernel), _dptr(x), _dptr(y), stream))

    def device_arrays(self):
        a, b, c = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().ed_crs_arrays(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return int(a.value or 0), int(b.value or 0), int(c.value or 0)

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_crs_free(self._h)
            self._h = None


class SpinlessFermionHamiltonian:
    """spinless_fermion_hamiltonian.hpp:52 for T = double."""

    def __init__(self):
        self.m_fockBasis = FermionFockBasis()
        self.m_crsSparseMatrix = None
        self.m_matrixFree = False
        self.m_terms = None
        self.m_eigenvalues = None
        self.m_eigenvectors = None
        self.last_info = None

    def Initialize(self, nbrParticles: int, nbrOrbitals: int, storageMethod=SPARSE_CRS, mpi=None,
                   twoLz: int | None = None):
        if nbrParticles <= 0 or nbrOrbitals <= 0:
            raise EDError(C.ED_ERR_ARG, "MUST SPECIFY nbr particles > 0 and nbr orbitals > 0")
        if nbrParticles >= 64:
            raise EDError(C.ED_ERR_ARG, "CANNOT ADDRESS 64 PARTICLES OR MORE")
        if nbrParticles > nbrOrbitals:
            raise EDError(C.ED_ERR_ARG, "NBR PARTICLES > NBR ORBITALS - NOT ALLOWED")
        self.m_nbrParticles, self.m_nbrOrbitals = int(nbrParticles), int(nbrOrbitals)
        self.m_storageMethod = storageMethod
        if twoLz is not None:
            self.m_fockBasis.GenerateFockSpace(nbrParticles, nbrOrbitals, twoLz)

    def Add_CdCdCC_Terms(self, termTables: QuarticTermTables, minRow: int = 0, maxRow: int | None = None, mpi=None,
                         store_upper: bool = False, matrix_free: bool = False):
        """Quartic terms into CRS on the device (spinless_fermion_hamiltonian.hpp:282-436).
        The whole sector is built (row slicing was the reference's MPI split)."""
        self.m_terms = termTables
        if matrix_free:
            self.m_matrixFree = True
            self.m_crsSparseMatrix = None
            return
        h = ctypes.c_void_p()
        check(lib().ed_ham_build_crs(self.m_fockBasis.handle(), termTables.handle(), int(bool(store_upper)), None,
                                     ctypes.byref(h)))
        self.m_crsSparseMatrix = CrsSparseMatrix(h)
        self.m_matrixFree = False

    def GetDimension(self) -> int:
        return self.m_fockBasis.GetStoredDimension()

    def operator_handle(self):
        op = ctypes.c_void_p()
        if self.m_matrixFree:
            check(lib().ed_op_matfree(self.m_fockBasis.handle(), self.m_terms.handle(), ctypes.byref(op)))
        else:
            if self.m_crsSparseMatrix is None:
                raise EDError(C.ED_ERR_ARG, "Hamiltonian not built")
            check(lib().ed_op_from_crs(self.m_crsSparseMatrix._h, ctypes.byref(op)))
        return op

    def LanczosDiagonalize(self, nbrEigenvalues: int, tol: float = 1e-10, v0=None, seed: int = 0, ncv: int = 0,
                           want_vectors: bool = True, verify: bool = True, max_restarts: int = 0,
                           degeneracy_passes: int = 0, diagonal_check: bool = True):
        """hamiltonian_base.hpp:770-931 with the device Lanczos; eigenvalues
        ascending.  diagonal_check: a stored matrix without off-diagonal
        elements is solved from its diagonal (MatrixDiagonalCheck, :378-449 and
        :803-850), each copy of a repeated value with its own unit vector."""
        mv = MatrixVectorFunction(self)
        arp = ArpackWrapper()
        n = self.GetDimension()
        evals = np.empty(nbrEigenvalues)
        evecs = np.empty((nbrEigenvalues, n)) if want_vectors else None
        ok = arp.DiagonalizeSymmetricMatrix(mv, evecs, evals, n, n, nbrEigenvalues, tol=tol, v0=v0, seed=seed,
                                            ncv=ncv, verify=verify, max_restarts=max_restarts,
                                            degeneracy_passes=degeneracy_passes, diagonal_check=diagonal_check)
        self.m_eigenvalues = evals
        self.m_eigenvectors = evecs
        self.last_info = arp.last_info
        return ok

    # hamiltonian_base.hpp:1204-1304
    def EigensystemToFile(self, fileName: str, writeValues: bool = True, writeVectors: bool = False,
                          fmt: str = "text", mpi=None):
        eigensystem_to_file(fileName, self.m_eigenvalues, self.m_eigenvectors if writeVectors else None, fmt)

    # hamiltonian_base.hpp:1309-1400
    def EigensystemFromFile(self, fileName: str, readValues: bool = True, readVectors: bool = False,
                            fmt: str = "text", mpi=None):
        ev, vec = eigensystem_from_file(fileName, fmt, vectors=readVectors)
        self.m_eigenvalues = ev
        if readVectors:
            self.m_eigenvectors = vec


class ComplexQuarticTermTables:
    """Complex momentum-conserving quartic terms of the optical-flux-lattice
    model in the reference's array layout (interacting_ofl_model/term_tables.cpp:
    95-200): (K+1) K^2 / 2 entries at (t1*K + t2 - t1(t1+1)/2)*K + k with
    t1 = min(k3,k4), t2 = max(k3,k4); k1 = m_kTable[.. + k2] and
    V(k1,k2,k3,k4) = m_vTable[.. + (k4 > k3 ? k1 : k2)].  The tables are the
    input (the reference computes them from Bloch functions in BuildTermTables)."""

    def __init__(self, dimX: int, dimY: int, ktable, vtable):
        self.dimX, self.dimY = int(dimX), int(dimY)
        K = self.m_kMax = self.dimX * self.dimY
        dim = (K + 1) * K * K // 2
        self.m_kTable = np.ascontiguousarray(ktable, dtype=np.uint16)
        self.m_vTable = np.ascontiguousarray(vtable, dtype=np.complex128)
        if self.m_kTable.shape != (dim,) or self.m_vTable.shape != (dim,):
            raise EDError(C.ED_ERR_ARG, f"tables of {dim} entries expected for a {dimX} x {dimY} grid")

    def _index(self, k3: int, k4: int) -> int:
        t1, t2 = (k3, k4) if k4 > k3 else (k4, k3)
        return t1 * self.m_kMax + t2 - t1 * (t1 + 1) // 2

    # term_tables.cpp:108-126
    def GetK1(self, k2: int, k3: int, k4: int) -> list:
        return [int(self.m_kTable[self._index(k3, k4) * self.m_kMax + k2])]

    # term_tables.cpp:157-175
    def GetVkkkk(self, k1: int, k2: int, k3: int, k4: int) -> complex:
        return complex(self.m_vTable[self._index(k3, k4) * self.m_kMax + (k1 if k4 > k3 else k2)])


def hash_key(*labels) -> int:
    """utilities::Key of the reference's multi-key hash tables
    (utilities/data_structures/multi_key_hash.hpp:59-92,
    general/serialize.hpp:96-130): two labels (k1 << 32) | k2, three
    (k2 << 48) | (k3 << 32) | (k4 << 16), four (k1 << 48) | (k2 << 32) |
    (k3 << 16) | k4."""
    if len(labels) == 2:
        return (int(labels[0]) << 32) | int(labels[1])
    if len(labels) in (3, 4):
        a = list(labels) + [0] * (4 - len(labels))
        return (int(a[0]) << 48) | (int(a[1]) << 32) | (int(a[2]) << 16) | int(a[3])
    raise EDError(C.ED_ERR_ARG, "two, three or four labels")


class _TermHashTables:
    """TermHashTables<dcmplx> (hamiltonians/term_hash_tables_base.hpp:44-276):
    a k-table (keys of nlabels - 1 labels, each with one k1; a key may repeat)
    and a value table (keys of nlabels labels, complex values), kept as flat
    key/value arrays in the order of the reference's file, with dictionaries
    for the look-ups.  Files in its binary or text layout (ed_term_hash_write /
    ed_term_hash_read)."""

    NLABELS = 4

    def __init__(self):
        self.m_kMax = 0
        self.Clear()

    def Initialize(self, kMax: int):
        self.m_kMax = int(kMax)

    def Clear(self):
        self.kkeys = np.zeros(0, dtype=np.uint64)
        self.kvals = np.zeros(0, dtype=np.uint16)
        self.vkeys = np.zeros(0, dtype=np.uint64)
        self.vvals = np.zeros(0, dtype=np.complex128)
        self._kd = self._vd = None

    def _set(self, kkeys, kvals, vkeys, vvals):
        self.kkeys = np.ascontiguousarray(kkeys, dtype=np.uint64)
        self.kvals = np.ascontiguousarray(kvals, dtype=np.uint16)
        self.vkeys = np.ascontiguousarray(vkeys, dtype=np.uint64)
        self.vvals = np.ascontiguousarray(vvals, dtype=np.complex128)
        self._kd = self._vd = None

    def _klookup(self, key: int) -> list:
        if self._kd is None:
            d = {}
            for k, v in zip(self.kkeys.tolist(), self.kvals.tolist()):
                d.setdefault(k, []).append(v)
            self._kd = d
        return list(self._kd.get(int(key), []))

    def _vlookup(self, key: int) -> complex:
        if self._vd is None:
            d = {}
            for k, v in zip(self.vkeys.tolist(), self.vvals.tolist()):
                d.setdefault(k, v)
            self._vd = d
        return complex(self._vd.get(int(key), 0.0))

    def GetMaxKCount(self) -> int:
        if self.kkeys.size == 0:
            return 1
        _, counts = np.unique(self.kkeys, return_counts=True)
        return int(counts.max())

    def ToFile(self, fileName: str, fmt: str = "binary", mpi=None):
        vv = np.ascontiguousarray(self.vvals.view(np.float64))
        check(lib().ed_term_hash_write(fileName.encode(), int(fmt == "binary"), self.NLABELS, len(self.kkeys),
                                       self.kkeys.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                       self.kvals.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), len(self.vkeys),
                                       self.vkeys.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _f64p(vv)))

    def FromFile(self, fileName: str, fmt: str = "binary", mpi=None):
        nk, nv = ctypes.c_uint32(), ctypes.c_uint32()
        b = int(fmt == "binary")
        check(lib().ed_term_hash_read(fileName.encode(), b, ctypes.byref(nk), None, None, ctypes.byref(nv), None,
                                      None))
        kk = np.empty(nk.value, dtype=np.uint64)
        kv = np.empty(nk.value, dtype=np.uint16)
        vk = np.empty(nv.value, dtype=np.uint64)
        vv = np.empty(2 * nv.value, dtype=np.float64)
        check(lib().ed_term_hash_read(fileName.encode(), b, ctypes.byref(nk),
                                      kk.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                      kv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), ctypes.byref(nv),
                                      vk.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _f64p(vv)))
        self._set(kk, kv, vk, vv.view(np.complex128))


class QuarticTermHashTables(_TermHashTables):
    """interacting_ofl_model/term_hash_tables.hpp QuarticTermHashTables
    (term_hash_tables.cpp): k1 for (k2, k3, k4) and V(k1, k2, k3, k4)."""

    NLABELS = 4

    # term_hash_tables_base.hpp:229-247: every (k2, k3, k4), k3 == k4 included
    def SetQuarticFromArray(self, quarticArray: ComplexQuarticTermTables):
        K = self.m_kMax = quarticArray.m_kMax
        k2, k3, k4 = (a.ravel() for a in np.meshgrid(np.arange(K), np.arange(K), np.arange(K), indexing="ij"))
        t1, t2 = np.minimum(k3, k4), np.maximum(k3, k4)
        t = t1 * K + t2 - t1 * (t1 + 1) // 2
        k1 = quarticArray.m_kTable[t * K + k2].astype(np.int64)
        v = quarticArray.m_vTable[t * K + np.where(k4 > k3, k1, k2)]
        u = np.uint64
        kk = (k2.astype(u) << u(48)) | (k3.astype(u) << u(32)) | (k4.astype(u) << u(16))
        vk = (k1.astype(u) << u(48)) | (k2.astype(u) << u(32)) | (k3.astype(u) << u(16)) | k4.astype(u)
        self._set(kk, k1, vk, v)

    # term_hash_tables.cpp: GetK1 (k-table look-up), GetVkkkk (0 when absent)
    def GetK1(self, k2: int, k3: int, k4: int) -> list:
        return self._klookup(hash_key(k2, k3, k4))

    def GetVkkkk(self, k1: int, k2: int, k3: int, k4: int) -> complex:
        return self._vlookup(hash_key(k1, k2, k3, k4))


class QuadraticTermHashTables(_TermHashTables):
    """interacting_ofl_model/term_hash_tables.hpp QuadraticTermHashTables:
    k1 for k2 and E(k1, k2)."""

    NLABELS = 2

    # term_hash_tables_base.hpp:262-275, from occupation energies (the array
    # QuadraticTermTables: GetK1(k2) = k2, GetEkk(k1, k2) = E[k1])
    def SetQuadraticFromArray(self, quadraticArray):
        e = np.ascontiguousarray(getattr(quadraticArray, "m_vTable", quadraticArray), dtype=np.complex128)
        K = self.m_kMax = len(e)
        k = np.arange(K, dtype=np.uint64)
        self._set(k, k.astype(np.uint16), (k << np.uint64(32)) | k, e)

    def GetK1(self, k2: int) -> list:
        return self._klookup(int(k2))

    def GetEkk(self, k1: int, k2: int) -> complex:
        return self._vlookup(hash_key(k1, k2))


def synthetic_ofl_tables(dimX: int, dimY: int, seed: int = 0):
    """Seeded complex quartic tables with the reference's momentum rule
    (FindK1, interacting_ofl_model.cpp:366-410: kx1 = kx3 + kx4 - kx2 and ky1
    likewise, modulo the grid) and values uniform in the unit square, real at
    the entries the diagonal terms read (Hermitian tables have them real): a
    stand-in input for benchmarks, since the reference derives the values from
    its non-interacting band structure."""
    X, Y = int(dimX), int(dimY)
    K = X * Y
    t1 = np.repeat(np.arange(K), K)
    t2 = np.tile(np.arange(K), K)
    keep = t2 >= t1
    t1, t2 = t1[keep], t2[keep]
    tri = t1 * K + t2 - t1 * (t1 + 1) // 2
    order = np.argsort(tri)
    t1, t2 = t1[order], t2[order]
    k2 = np.arange(K)
    kx = (t1[:, None] // Y + t2[:, None] // Y - k2[None, :] // Y) % X
    ky = (t1[:, None] % Y + t2[:, None] % Y - k2[None, :] % Y) % Y
    ktab = (kx * Y + ky).astype(np.uint16).ravel()
    rng = np.random.default_rng(seed)
    dim = len(ktab)
    vtab = rng.uniform(-1, 1, dim) + 1j * rng.uniform(-1, 1, dim)
    rows = np.arange(len(t1)) * K
    vtab[rows + t1] = vtab[rows + t1].real
    vtab[rows + t2] = vtab[rows + t2].real
    return ComplexQuarticTermTables(X, Y, ktab, vtab)


class ComplexCrsSparseMatrix:
    """Device CRS of complex values (CrsSparseMatrix<dcmplx>)."""

    def __init__(self, h):
        self._h = h

    def info(self):
        n, nnz, up = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        check(lib().ed_ccrs_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(up)))
        return int(n.value), int(nnz.value), bool(up.value)

    def GetNbrRows(self) -> int:
        return self.info()[0]

    def GetNbrNonZeros(self) -> int:
        return self.info()[1]

    def multiply(self, x, y, kernel: int = 0, stream=None):
        """y = A x on device complex vectors (float64 (re, im) pairs) with a
        chosen kernel (ed_cspmv_kernel: 0 by storage, 1 FP64 rows, 2
        fixed-point integer rows)."""
        check(lib().ed_cspmv_kernel(self._h, int(kernel), _dptr(x), _dptr(y), stream))

    def to_host(self):
        n, nnz, _ = self.info()
        rp = np.empty(n + 1, dtype=np.int64)
        col = np.empty(max(nnz, 0), dtype=np.int32)
        val = np.empty(max(nnz, 0), dtype=np.complex128)
        check(lib().ed_ccrs_get(self._h, rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                col.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _f64p(val.view(np.float64))))
        return rp, col, val

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_ccrs_free(self._h)
            self._h = None


class ComplexSpinlessFermionHamiltonian:
    """spinless_fermion_hamiltonian.hpp:52 for T = dcmplx over a momentum
    sector, as InteractingOflModel drives it (interacting_ofl_model.cpp:
    952-1135): SetFockBasis, Add_CdC_Terms (diagonal occupation energies),
    Add_CdCdCC_Terms, LanczosDiagonalize.  The device build runs at the first
    product or solve; upper storage is the reference's (row in, column out >=
    in, value <out|H|in>, Hermitian completion in the product), full storage
    holds the completion explicitly.  Vectors are complex128."""

    def __init__(self):
        self.m_fockBasis = FermionFockBasis()
        self.m_crsSparseMatrix = None
        self._energies = None
        self._tables = None
        self._store_upper = False
        self.m_eigenvalues = None
        self.m_eigenvectors = None
        self.last_info = None

    def Initialize(self, nbrParticles: int, nbrOrbitals: int, storageMethod=SPARSE_CRS, mpi=None):
        self.m_nbrParticles, self.m_nbrOrbitals = int(nbrParticles), int(nbrOrbitals)

    def SetFockBasis(self, basis: FermionFockBasis):
        self.m_fockBasis = basis
        self.m_crsSparseMatrix = None

    def Add_CdC_Terms(self, energies, minRow: int = 0, maxRow: int | None = None, mpi=None):
        """Occupation energies E_k (QuadraticTermTables::GetEkk with k1 = k2,
        spinless_fermion_hamiltonian.hpp:150-262): an array of K values, an
        object with m_vTable, or QuadraticTermHashTables (diagonal)."""
        if isinstance(energies, QuadraticTermHashTables):
            self._energies = energies
        else:
            self._energies = np.ascontiguousarray(getattr(energies, "m_vTable", energies), dtype=np.complex128)
        self.m_crsSparseMatrix = None

    def Add_CdCdCC_Terms(self, termTables, minRow: int = 0, maxRow: int | None = None, mpi=None,
                         store_upper: bool = False):
        """termTables: ComplexQuarticTermTables (array format) or
        QuarticTermHashTables (hash format, momentum-conserving)."""
        self._tables = termTables
        self._store_upper = bool(store_upper)
        self.m_crsSparseMatrix = None

    def _terms_from_hash(self, t: QuarticTermHashTables):
        K = t.m_kMax
        q = self._energies
        if q is not None and not isinstance(q, QuadraticTermHashTables):
            if q.shape != (K,):
                raise EDError(C.ED_ERR_ARG, f"{K} occupation energies expected")
            qq = QuadraticTermHashTables()
            qq.SetQuadraticFromArray(q)
            q = qq
        if q is None:
            q = QuadraticTermHashTables()
        u64p, u16p = ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint16)
        vv = np.ascontiguousarray(t.vvals.view(np.float64))
        qv = np.ascontiguousarray(q.vvals.view(np.float64))
        dimX = getattr(self, "dimX", None) or self.m_fockBasis.dimX
        dimY = getattr(self, "dimY", None) or self.m_fockBasis.dimY
        th = ctypes.c_void_p()
        check(lib().ed_cterms_create_hash(K, dimX, dimY, len(t.kkeys), t.kkeys.ctypes.data_as(u64p),
                                          t.kvals.ctypes.data_as(u16p), len(t.vkeys), t.vkeys.ctypes.data_as(u64p),
                                          _f64p(vv), len(q.kkeys), q.kkeys.ctypes.data_as(u64p),
                                          q.kvals.ctypes.data_as(u16p), len(q.vkeys), q.vkeys.ctypes.data_as(u64p),
                                          _f64p(qv), ctypes.byref(th)))
        return th

    def Build(self):
        t = self._tables
        if t is None:
            raise EDError(C.ED_ERR_ARG, "Add_CdCdCC_Terms first")
        if isinstance(t, QuarticTermHashTables):
            th = self._terms_from_hash(t)
            try:
                h = ctypes.c_void_p()
                check(lib().ed_cham_build_crs(self.m_fockBasis.handle(), th, int(self._store_upper), None,
                                              ctypes.byref(h)))
            finally:
                lib().ed_cterms_free(th)
            self.m_crsSparseMatrix = ComplexCrsSparseMatrix(h)
            return
        if isinstance(self._energies, QuadraticTermHashTables):
            raise EDError(C.ED_ERR_ARG, "hash-format quadratic terms go with hash-format quartic terms")
        e = None
        if self._energies is not None:
            if self._energies.shape != (t.m_kMax,):
                raise EDError(C.ED_ERR_ARG, f"{t.m_kMax} occupation energies expected")
            e = np.ascontiguousarray(self._energies.view(np.float64))
        vt = np.ascontiguousarray(t.m_vTable.view(np.float64))
        th = ctypes.c_void_p()
        check(lib().ed_cterms_create(t.m_kMax, t.dimX, t.dimY, t.m_kTable.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                     _f64p(vt), None if e is None else _f64p(e), ctypes.byref(th)))
        try:
            h = ctypes.c_void_p()
            check(lib().ed_cham_build_crs(self.m_fockBasis.handle(), th, int(self._store_upper), None,
                                          ctypes.byref(h)))
        finally:
            lib().ed_cterms_free(th)
        self.m_crsSparseMatrix = ComplexCrsSparseMatrix(h)

    def GetDimension(self) -> int:
        return self.m_fockBasis.GetStoredDimension()

    def apply(self, x, y, stream=None):
        """y = H x on device complex128 vectors (torch tensors or pointers)."""
        if self.m_crsSparseMatrix is None:
            self.Build()
        check(lib().ed_cspmv(self.m_crsSparseMatrix._h, _dptr(x), _dptr(y), stream))

    def LanczosDiagonalize(self, nbrEigenvalues: int, tol: float = 1e-10, v0=None, seed: int = 0, ncv: int = 0,
                           want_vectors: bool = True, verify: bool = True, max_restarts: int = 0,
                           diagonal_check: bool = True) -> bool:
        """Lowest eigenpairs (hamiltonian_base.hpp:770-931 with the complex
        driver); eigenvalues ascending, eigenvectors complex128 (nev, n).
        diagonal_check as the real class's."""
        if self.m_crsSparseMatrix is None:
            self.Build()
        n = self.GetDimension()
        p = LanczosParams(nev=int(nbrEigenvalues), ncv=int(ncv), max_restarts=int(max_restarts or 0), tol=float(tol),
                          seed=int(seed), want_vectors=int(bool(want_vectors)), verify=int(bool(verify)),
                          diagonal_check=int(bool(diagonal_check)))
        info = SolveInfo()
        ev = np.empty(nbrEigenvalues)
        vec = np.empty((nbrEigenvalues, n), dtype=np.complex128) if want_vectors else None
        v0a = None if v0 is None else np.ascontiguousarray(np.asarray(v0, dtype=np.complex128).view(np.float64))
        st = lib().ed_clanczos(self.m_crsSparseMatrix._h, ctypes.byref(p), None if v0a is None else _f64p(v0a),
                               _f64p(ev), None if vec is None else _f64p(vec.view(np.float64)), ctypes.byref(info))
        self.last_info = info.as_dict()
        self.m_eigenvalues = ev
        self.m_eigenvectors = vec
        if st != C.ED_OK:
            self.last_error = lib().ed_last_error().decode(errors="replace")
            return False
        return True


class InteractingOflModel:
    """Sector driver of the interacting optical-flux-lattice model
    (interacting_ofl_model.cpp:97-105 SetSector, :952-1027 BuildFockBasis,
    :1034-1060 BuildHamiltonian, :1067-1135 Diagonalize), with the term tables
    and occupation energies given (the reference computes them from the
    non-interacting band structure).  The tables are in the array format until
    ConvertTableFormat (:597-618) turns them into hash tables; TermsToFile and
    TermsFromFile (:623-691) store and read hash tables under the reference's
    file names."""

    def __init__(self, nbrParticles: int, dimX: int, dimY: int, quarticTables: ComplexQuarticTermTables | None,
                 energies=None, nbrEigenvalues: int = 1):
        self.N, self.dimX, self.dimY = int(nbrParticles), int(dimX), int(dimY)
        self.tables = quarticTables
        self.energies = None if energies is None else np.asarray(energies, dtype=np.complex128)
        self.nev = int(nbrEigenvalues)
        self.kxTot = self.kyTot = 0
        self.hamiltonian = None
        self.m_tableFormat = "array"
        self.m_quarticHashTables = QuarticTermHashTables()
        self.m_quadraticHashTables = QuadraticTermHashTables()

    def ConvertTableFormat(self):
        """Array tables to hash tables (interacting_ofl_model.cpp:597-618);
        the arrays are dropped, as the reference clears them."""
        if self.m_tableFormat != "array":
            return
        K = self.dimX * self.dimY
        self.m_quarticHashTables.Clear()
        self.m_quadraticHashTables.Clear()
        self.m_quarticHashTables.Initialize(K)
        self.m_quadraticHashTables.Initialize(K)
        self.m_quadraticHashTables.SetQuadraticFromArray(
            self.energies if self.energies is not None else np.zeros(K, dtype=np.complex128))
        self.m_quarticHashTables.SetQuarticFromArray(self.tables)
        self.tables = None
        self.energies = None
        self.m_tableFormat = "hash"

    def _term_file_names(self, outPath: str):
        import os
        tail = f"_table_kx_{self.dimX}_ky_{self.dimY}.dat"
        return (os.path.join(outPath, "quadratic_coefficient" + tail), os.path.join(outPath, "quartic_coefficient" + tail))

    def TermsToFile(self, outPath: str, fmt: str = "binary"):
        """The hash tables to quadratic_/quartic_coefficient_table_kx_X_ky_Y.dat
        in outPath (interacting_ofl_model.cpp:623-651); the array format's own
        complex table files are not written here."""
        if self.m_tableFormat != "hash":
            raise EDError(C.ED_ERR_ARG, "ConvertTableFormat first: only hash-format term files are written")
        fq, f4 = self._term_file_names(outPath)
        self.m_quadraticHashTables.ToFile(fq, fmt)
        self.m_quarticHashTables.ToFile(f4, fmt)

    def TermsFromFile(self, outPath: str, fmt: str = "binary"):
        """Hash tables from the files TermsToFile writes
        (interacting_ofl_model.cpp:656-691); the model then builds from them."""
        K = self.dimX * self.dimY
        fq, f4 = self._term_file_names(outPath)
        self.m_quarticHashTables.Initialize(K)
        self.m_quadraticHashTables.Initialize(K)
        self.m_quarticHashTables.FromFile(f4, fmt)
        self.m_quadraticHashTables.FromFile(fq, fmt)
        self.tables = None
        self.energies = None
        self.m_tableFormat = "hash"

    def SetSector(self, kxSector: int, kySector: int):
        self.kxTot, self.kyTot = int(kxSector), int(kySector)

    def BuildFockBasis(self) -> bool:
        basis = FermionFockBasis()
        empty = basis.GenerateFockSpaceMomentum(self.N, self.dimX, self.dimY, self.kxTot, self.kyTot)
        self.hamiltonian = ComplexSpinlessFermionHamiltonian()
        self.hamiltonian.Initialize(self.N, self.dimX * self.dimY)
        self.hamiltonian.SetFockBasis(basis)
        return empty

    def BuildHamiltonian(self, store_upper: bool = False):
        if self.m_tableFormat == "hash":
            self.hamiltonian.Add_CdC_Terms(self.m_quadraticHashTables)
            self.hamiltonian.Add_CdCdCC_Terms(self.m_quarticHashTables, store_upper=store_upper)
        else:
            if self.energies is not None:
                self.hamiltonian.Add_CdC_Terms(self.energies)
            self.hamiltonian.Add_CdCdCC_Terms(self.tables, store_upper=store_upper)
        self.hamiltonian.Build()

    def Diagonalize(self, **kw) -> bool:
        return self.hamiltonian.LanczosDiagonalize(self.nev, **kw)


class Observables:
    """Observables of an eigenvector of a real sector Hamiltonian
    (observables/fermion_observables.hpp:39), computed on the device.  The
    methods take the Hamiltonian and an eigenvector index, as the reference
    does (its eigenvectors after LanczosDiagonalize), or a basis and a host
    vector (``*_of_vector``)."""

    @staticmethod
    def _vector(hamiltonian, eigenvectorIndex):
        vecs = hamiltonian.m_eigenvectors
        if vecs is None:
            raise EDError(C.ED_ERR_ARG, "eigenvectors not calculated")
        if not 0 <= eigenvectorIndex < len(vecs):
            raise EDError(C.ED_ERR_ARG, "eigenvectorIndex out of range")
        v = np.asarray(vecs[eigenvectorIndex])
        return hamiltonian.m_fockBasis, v if np.iscomplexobj(v) else np.ascontiguousarray(v, dtype=np.float64)

    @staticmethod
    def _magnitude(psi) -> np.ndarray:
        """The observables depend on |psi| only: complex eigenvectors (the
        optical-flux-lattice model's) enter through their moduli."""
        psi = np.asarray(psi)
        return np.ascontiguousarray(np.abs(psi) if np.iscomplexobj(psi) else psi, dtype=np.float64)

    @staticmethod
    def density_of_vector(basis, psi) -> np.ndarray:
        """rho[k] = sum_s |psi_s|^2 n_k(s) (fermion_observables.hpp:48-104)."""
        psi = Observables._magnitude(psi)
        rho = np.empty(basis.nbrOrbitals)
        check(lib().ed_obs_density(basis.handle(), _f64p(psi), _f64p(rho)))
        return rho

    @staticmethod
    def density_density_of_vector(basis, psi) -> np.ndarray:
        """D[k, q] = sum_s |psi_s|^2 n_k(s) n_q(s) (fermion_observables.hpp:117-200)."""
        psi = Observables._magnitude(psi)
        K = basis.nbrOrbitals
        t = np.empty(K * K)
        check(lib().ed_obs_density_density(basis.handle(), _f64p(psi), _f64p(t)))
        return t.reshape(K, K)

    @staticmethod
    def participation_ratio_of_vector(basis, psi) -> float:
        """1 / sum_s |psi_s|^4 (fermion_observables.hpp:528-562)."""
        psi = Observables._magnitude(psi)
        r = ctypes.c_double()
        check(lib().ed_obs_participation_ratio(basis.handle(), _f64p(psi), ctypes.byref(r)))
        return float(r.value)

    @staticmethod
    def most_probable_of_vector(basis, psi, nbrStates: int):
        """The nbrStates largest |psi_s| with their Fock words, descending
        (fermion_observables.hpp:437-517); complex psi gives its complex
        amplitudes."""
        original = np.asarray(psi)
        psi = Observables._magnitude(original)
        k = max(int(nbrStates), 0)
        states = np.empty(max(k, 1), dtype=np.uint64)
        amps = np.empty(max(k, 1))
        cnt = ctypes.c_int64()
        check(lib().ed_obs_most_probable(basis.handle(), _f64p(psi), k,
                                         states.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _f64p(amps),
                                         ctypes.byref(cnt)))
        m = int(cnt.value)
        if np.iscomplexobj(original) and m:
            idx = basis.FindFockStateIndices(states[:m]).astype(np.int64)
            return states[:m].copy(), original[idx].astype(np.complex128)
        return states[:m].copy(), amps[:m].copy()

    # the reference's call shapes (the MpiWrapper argument is accepted and ignored)
    def DensityFunction(self, hamiltonian, eigenvectorIndex: int, mpi=None) -> np.ndarray:
        return self.density_of_vector(*self._vector(hamiltonian, eigenvectorIndex))

    def DensityDensityFunction(self, hamiltonian, eigenvectorIndex: int, mpi=None) -> np.ndarray:
        return self.density_density_of_vector(*self._vector(hamiltonian, eigenvectorIndex))

    def GetParticipationRatio(self, hamiltonian, eigenvectorIndex: int, mpi=None) -> float:
        return self.participation_ratio_of_vector(*self._vector(hamiltonian, eigenvectorIndex))

    def GetMostProbable(self, hamiltonian, nbrStates: int, mpi=None):
        """Per eigenvector e: (states[e], amplitudes[e]) of the nbrStates largest |psi|."""
        vecs = hamiltonian.m_eigenvectors
        if vecs is None:
            raise EDError(C.ED_ERR_ARG, "eigenvectors not calculated")
        return [self.most_probable_of_vector(hamiltonian.m_fockBasis, v, nbrStates) for v in vecs]


class MatrixVectorFunction:
    """H*v callback bound into the eigensolver (matrix_vector_routines.hpp:41)."""

    def __init__(self, hamiltonian: SpinlessFermionHamiltonian, mpi=None):
        self.hamiltonian = hamiltonian

    def Simple(self, x, y, mpi=None, stream=None):
        """y = H x on device vectors (torch CUDA tensors or raw pointers),
        matrix_vector_routines.hpp:94-104."""
        h = self.hamiltonian
        if h.m_matrixFree:
            check(lib().ed_hv_matfree(h.m_fockBasis.handle(), h.m_terms.handle(), _dptr(x), _dptr(y), stream))
        else:
            check(lib().ed_spmv(h.m_crsSparseMatrix._h, _dptr(x), _dptr(y), stream))


class ArpackWrapper:
    """Eigensolver front end (arpack_wrapper.hpp:187) over the device Lanczos."""

    def __init__(self):
        self.m_eigenvalueMagnitude = "S"
        self.m_whatMagnitude = "R"
        self.m_maxIterations = 2000
        self.last_info = None
        self.last_status = C.ED_OK

    def DiagonalizeSymmetricMatrix(self, MatrixVectorMultiply, eigenvectors, eigenvalues, nodeDim: int, fullDim: int,
                                   nbrEigenvalues: int, mpi=None, tol: float = 1e-10, v0=None, seed: int = 0,
                                   ncv: int = 0, verify: bool = True, max_restarts: int = 0,
                                   degeneracy_passes: int = 0, diagonal_check: bool = False) -> bool:
        """Lowest `nbrEigenvalues` eigenpairs.  MatrixVectorMultiply is either
        a MatrixVectorFunction (device product) or a Python callable
        f(x_host, y_host) on numpy arrays (the reference's std::function form).
        eigenvalues: float64 array (filled ascending); eigenvectors: array of
        shape (nbrEigenvalues, n) or None.  degeneracy_passes > 0 adds deflated
        solves that recover further copies of degenerate eigenvalues.  Returns
        False on failure, like the reference, with the status in last_status."""
        if nodeDim != fullDim:
            raise EDError(C.ED_ERR_ARG, "one device holds the whole vector: nodeDim must equal fullDim")
        n = int(fullDim)
        cb = None
        op = ctypes.c_void_p()
        if isinstance(MatrixVectorMultiply, MatrixVectorFunction):
            op = MatrixVectorMultiply.hamiltonian.operator_handle()
        else:
            fn = MatrixVectorMultiply

            def _tramp(xp, yp, _user):
                x = np.ctypeslib.as_array(xp, shape=(n,))
                y = np.ctypeslib.as_array(yp, shape=(n,))
                fn(x, y)

            cb = C.HOST_MATVEC(_tramp)
            check(lib().ed_op_host_callback(n, cb, None, ctypes.byref(op)))
        try:
            p = LanczosParams(nev=int(nbrEigenvalues), ncv=int(ncv), max_restarts=int(max_restarts or 0), tol=float(tol),
                              seed=int(seed), want_vectors=int(eigenvectors is not None), verify=int(bool(verify)),
                              degeneracy_passes=int(degeneracy_passes), diagonal_check=int(bool(diagonal_check)))
            info = SolveInfo()
            ev = np.empty(nbrEigenvalues)
            vec = np.empty(n * nbrEigenvalues) if eigenvectors is not None else None
            v0a = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64)
            st = lib().ed_lanczos(op, ctypes.byref(p), _f64p(v0a) if v0a is not None else None, _f64p(ev),
                                  _f64p(vec) if vec is not None else None, ctypes.byref(info))
            self.last_info = info.as_dict()
            self.last_status = st
            eigenvalues[:nbrEigenvalues] = ev
            if eigenvectors is not None:
                eigenvectors[...] = vec.reshape(nbrEigenvalues, n)
            if st != C.ED_OK:
                self.last_error = lib().ed_last_error().decode(errors="replace")
                return False
            return True
        finally:
            lib().ed_op_free(op)
            del cb


class SpherePseudopotentialModel:
    """One-sector driver: BuildTermTables / BuildFockBasis / BuildHamiltonian /
    Diagonalize (pseudopotential_model.cpp:64-95, 160, 233, 264)."""

    def __init__(self, nbrParticles: int, nbrOrbitals: int, pseudopotentials, nbrEigenvalues: int = 1):
        self.N, self.norb = int(nbrParticles), int(nbrOrbitals)
        self.pseudopotentials = np.ascontiguousarray(pseudopotentials, dtype=np.float64)
        if len(self.pseudopotentials) > self.norb - 1:
            raise EDError(C.ED_ERR_ARG, "TOO MANY 2-BODY PSEUDOPOTENTIAL COEFFICIENTS SPECIFIED")
        self.nev = int(nbrEigenvalues)
        self.twoLz = 0
        self.tables = None
        self.hamiltonian = None

    def SetSector(self, twoLz: int):
        self.twoLz = int(twoLz)

    def BuildTermTables(self):
        self.tables = QuarticTermTables(self.norb, self.pseudopotentials)

    def BuildFockBasis(self) -> bool:
        self.hamiltonian = SpinlessFermionHamiltonian()
        self.hamiltonian.Initialize(self.N, self.norb, SPARSE_CRS)
        return self.hamiltonian.m_fockBasis.GenerateFockSpace(self.N, self.norb, self.twoLz)

    def BuildHamiltonian(self, matrix_free: bool = False, store_upper: bool = False):
        self.hamiltonian.Add_CdCdCC_Terms(self.tables, store_upper=store_upper, matrix_free=matrix_free)

    def Diagonalize(self, **kw):
        return self.hamiltonian.LanczosDiagonalize(self.nev, **kw)


class TwoLevelSpinlessFermionHamiltonian(SpinlessFermionHamiltonian):
    """two_level_spinless_fermion_hamiltonian.hpp:52 for T = double: spinless
    fermions in the two lowest Landau levels, terms within one level only (as
    the reference codes them).  Add_CdC_Terms / Add_CdCdCC_Terms record each
    level's tables; the device build (ed_ham2_build_crs) runs once when the
    matrix is first needed and sums each entry in the reference model's call
    order: level-0 and level-1 occupation energies, then the level-0 and level-1
    quartic terms (two_level_pseudopotential_model.cpp:203-212)."""

    def __init__(self):
        super().__init__()
        self.m_fockBasis = TwoLevelFermionFockBasis()
        self._quartic = [None, None]
        self._energies = [None, None]
        self._store_upper = False

    def Initialize(self, nbrParticles: int, nbrOrbitals: int, storageMethod=SPARSE_CRS, mpi=None,
                   twoLz: int | None = None):
        """nbrOrbitals = total over both levels, 2*(2S+1) + 2 (two_level_pseudopotential_model.cpp:73)."""
        if nbrParticles <= 0 or nbrOrbitals < 4 or nbrOrbitals % 2:
            raise EDError(C.ED_ERR_ARG, "need nbrParticles > 0 and nbrOrbitals = 2 * norb0 + 2")
        self.m_nbrParticles, self.m_nbrOrbitals = int(nbrParticles), int(nbrOrbitals)
        self.m_storageMethod = storageMethod
        self.norb0 = (int(nbrOrbitals) - 2) // 2
        if twoLz is not None:
            self.m_fockBasis.GenerateFockSpace(nbrParticles, self.norb0, self.norb0 + 2, twoLz)

    @staticmethod
    def _same_level(*levels) -> int:
        if any(lv not in (0, 1) for lv in levels):
            raise EDError(C.ED_ERR_ARG, "level specification incorrect (set to 0,1 only)")
        if len(set(levels)) != 1:
            raise EDError(C.ED_ERR_ARG, "only coded for terms in the same level so far")
        return int(levels[0])

    def Add_CdC_Terms(self, energies, level1: int, level2: int, minRow: int = 0, maxRow: int | None = None,
                      mpi=None):
        """Occupation energies of one level (two_level_spinless_fermion_hamiltonian.hpp:143-270):
        an array of that level's orbital count, or an object with m_vTable."""
        lvl = self._same_level(level1, level2)
        e = np.ascontiguousarray(getattr(energies, "m_vTable", energies), dtype=np.float64)
        need = self.norb0 + 2 * lvl
        if e.shape != (need,):
            raise EDError(C.ED_ERR_ARG, f"level {lvl} energies need {need} values")
        self._energies[lvl] = e
        self.m_crsSparseMatrix = None

    def Add_CdCdCC_Terms(self, termTables: QuarticTermTables, level1: int = 0, level2: int = 0, level3: int = 0,
                         level4: int = 0, minRow: int = 0, maxRow: int | None = None, mpi=None,
                         store_upper: bool = False, matrix_free: bool = False):
        """Quartic terms of one level (two_level_spinless_fermion_hamiltonian.hpp:306-470)."""
        if matrix_free:
            raise EDError(C.ED_ERR_ARG, "the two-level Hamiltonian is built into CRS")
        lvl = self._same_level(level1, level2, level3, level4)
        if termTables.m_kMax != self.norb0 + 2 * lvl:
            raise EDError(C.ED_ERR_ARG, f"level {lvl} tables need {self.norb0 + 2 * lvl} orbitals")
        self._quartic[lvl] = termTables
        self._store_upper = bool(store_upper)
        self.m_crsSparseMatrix = None

    def Build(self):
        q = [t if t is not None else QuarticTermTables(self.norb0 + 2 * lv, [0.0])
             for lv, t in enumerate(self._quartic)]
        e0, e1 = self._energies
        h = ctypes.c_void_p()
        check(lib().ed_ham2_build_crs(self.m_fockBasis.handle(), q[0].handle(), q[1].handle(),
                                      None if e0 is None else _f64p(e0), None if e1 is None else _f64p(e1),
                                      int(self._store_upper), None, ctypes.byref(h)))
        self.m_crsSparseMatrix = CrsSparseMatrix(h)
        self.m_matrixFree = False
        self._keep = q

    def operator_handle(self):
        if self.m_crsSparseMatrix is None:
            self.Build()
        return super().operator_handle()

    def LanczosDiagonalize(self, nbrEigenvalues: int, tol: float = 1e-10, v0=None, seed: int = 0, ncv: int = 0,
                           want_vectors: bool = True, verify: bool = True, max_restarts: int = 0,
                           degeneracy_passes: int | None = None, diagonal_check: bool = True):
        """Lowest eigenpairs with every copy of a degenerate eigenvalue: the
        levels do not mix, so every pair of level-0 and level-1 multiplets
        (L0, L1) gives 2 min(L0, L1) + 1 states of one energy in a sector.  By
        default the copies come from the level-exchange ladder
        (ed_lanczos_two_level); degeneracy_passes = k uses k deflated passes
        instead, 0 the plain single-sequence solve.  diagonal_check as the
        one-level class's."""
        if self.m_crsSparseMatrix is None:
            self.Build()
        if degeneracy_passes is not None:
            return super().LanczosDiagonalize(nbrEigenvalues, tol=tol, v0=v0, seed=seed, ncv=ncv,
                                              want_vectors=want_vectors, verify=verify, max_restarts=max_restarts,
                                              degeneracy_passes=degeneracy_passes, diagonal_check=diagonal_check)
        n = self.GetDimension()
        op = self.operator_handle()
        try:
            p = LanczosParams(nev=int(nbrEigenvalues), ncv=int(ncv), max_restarts=int(max_restarts or 0),
                              tol=float(tol), seed=int(seed), want_vectors=int(bool(want_vectors)),
                              verify=int(bool(verify)), diagonal_check=int(bool(diagonal_check)))
            info = SolveInfo()
            ev = np.empty(nbrEigenvalues)
            vec = np.empty((nbrEigenvalues, n)) if want_vectors else None
            v0a = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64)
            st = lib().ed_lanczos_two_level(self.m_fockBasis.handle(), op, ctypes.byref(p),
                                            None if v0a is None else _f64p(v0a), _f64p(ev),
                                            None if vec is None else _f64p(vec), ctypes.byref(info))
        finally:
            lib().ed_op_free(op)
        self.last_info = info.as_dict()
        self.m_eigenvalues = ev
        self.m_eigenvectors = vec
        if st != C.ED_OK:
            self.last_error = lib().ed_last_error().decode(errors="replace")
            return False
        return True


class SphereTwoLevelPseudopotentialModel:
    """Two-Landau-level sector driver (two_level_pseudopotential_model.cpp:61-215):
    BuildTermTables (LLL tables of norb0 = 2S+1 orbitals, second-level tables
    of norb0 + 2 from its own pseudopotentials), SetOccupationEnergies,
    BuildFockBasis, BuildHamiltonian, Diagonalize."""

    def __init__(self, nbrParticles: int, norb0: int, pseudopotentials, pseudopotentials2LL,
                 nbrEigenvalues: int = 1):
        self.N, self.norb0 = int(nbrParticles), int(norb0)
        self.pp0 = np.ascontiguousarray(pseudopotentials, dtype=np.float64)
        self.pp1 = np.ascontiguousarray(pseudopotentials2LL, dtype=np.float64)
        self.nev = int(nbrEigenvalues)
        self.twoLz = 0
        self.energies = None
        self.hamiltonian = None

    def SetSector(self, twoLz: int):
        self.twoLz = int(twoLz)

    def BuildTermTables(self):
        self.tables = (QuarticTermTables(self.norb0, self.pp0), QuarticTermTables(self.norb0 + 2, self.pp1))

    def SetOccupationEnergies(self, energyLevels):
        """energyLevels: norb0 lowest-level values followed by norb0 + 2 second-level ones
        (two_level_pseudopotential_model.cpp:92-108)."""
        e = np.ascontiguousarray(energyLevels, dtype=np.float64)
        if len(e) != 2 * self.norb0 + 2:
            raise EDError(C.ED_ERR_ARG, "Must specify same number of energy levels as orbitals")
        self.energies = (e[:self.norb0].copy(), e[self.norb0:].copy())

    def BuildFockBasis(self) -> bool:
        self.hamiltonian = TwoLevelSpinlessFermionHamiltonian()
        self.hamiltonian.Initialize(self.N, 2 * self.norb0 + 2, SPARSE_CRS)
        return self.hamiltonian.m_fockBasis.GenerateFockSpace(self.N, self.norb0, self.norb0 + 2, self.twoLz)

    def BuildHamiltonian(self, store_upper: bool = False):
        H = self.hamiltonian
        if self.energies is not None:
            H.Add_CdC_Terms(self.energies[0], 0, 0)
            H.Add_CdC_Terms(self.energies[1], 1, 1)
        H.Add_CdCdCC_Terms(self.tables[0], 0, 0, 0, 0, store_upper=store_upper)
        H.Add_CdCdCC_Terms(self.tables[1], 1, 1, 1, 1, store_upper=store_upper)
        H.Build()

    def Diagonalize(self, **kw):
        return self.hamiltonian.LanczosDiagonalize(self.nev, **kw)


def eigensystem_to_file(fileName: str, eigenvalues, eigenvectors=None, fmt: str = "text"):
    """The reference's eigensystem file (text or binary); eigenvectors [nev, dim] or None."""
    ev = np.ascontiguousarray(eigenvalues, dtype=np.float64)
    vec = None if eigenvectors is None else np.ascontiguousarray(eigenvectors, dtype=np.float64)
    dim = 0 if vec is None else int(vec.shape[-1])
    check(lib().ed_eigensystem_write(fileName.encode(), int(fmt == "binary"), len(ev), _f64p(ev), dim,
                                     None if vec is None else _f64p(vec)))


def eigensystem_from_file(fileName: str, fmt: str = "text", vectors: bool = True):
    """Read an eigensystem file: (eigenvalues, eigenvectors [nev, dim] or None)."""
    b = int(fmt == "binary")
    nev, dim = ctypes.c_int(), ctypes.c_uint64()
    check(lib().ed_eigensystem_read(fileName.encode(), b, ctypes.byref(nev), None, ctypes.byref(dim), None))
    ev = np.empty(nev.value)
    vec = np.empty(nev.value * dim.value) if (vectors and dim.value) else None
    check(lib().ed_eigensystem_read(fileName.encode(), b, ctypes.byref(nev), _f64p(ev), ctypes.byref(dim),
                                    None if vec is None else _f64p(vec)))
    return ev, (None if vec is None else vec.reshape(nev.value, dim.value))


def solve_sector(N: int, norb: int, twoLz: int, pseudopotentials, nev: int, tol: float = 1e-10, v0=None,
                 seed: int = 0, ncv: int = 0, matrix_free: bool = False, want_vectors: bool = False,
                 verify: bool = True):
    """Whole-sector solve in one C-ABI call from host inputs (ed_solve_sector)."""
    pp = np.ascontiguousarray(pseudopotentials, dtype=np.float64)
    p = LanczosParams(nev=nev, ncv=ncv, max_restarts=0, tol=tol, seed=seed, want_vectors=int(want_vectors),
                      verify=int(verify))
    info = SolveInfo()
    ev = np.empty(nev)
    v0a = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64)
    vec = None
    if want_vectors:
        n = int(np.asarray(v0a).shape[0]) if v0a is not None else None
        if n is None:
            b = FermionFockBasis()
            b.GenerateFockSpace(N, norb, twoLz)
            n = b.GetStoredDimension()
        vec = np.empty(n * nev)
    check(lib().ed_solve_sector(N, norb, twoLz, _f64p(pp), len(pp), int(matrix_free), ctypes.byref(p),
                                _f64p(v0a) if v0a is not None else None, _f64p(ev),
                                _f64p(vec) if vec is not None else None, ctypes.byref(info)))
    out = {"eigenvalues": ev, "info": info.as_dict()}
    if vec is not None:
        out["eigenvectors"] = vec.reshape(nev, -1)
    return out


class HamiltonianBatch:
    """Many Hamiltonians of one sector differing only in their pseudopotential
    lists, sharing one device pattern (ed_batch_create).  No reference
    counterpart: the reference solves one Hamiltonian per run."""

    def __init__(self, basis: FermionFockBasis, pseudopotential_lists, autotune: bool = True):
        lists = [np.ascontiguousarray(v, dtype=np.float64) for v in pseudopotential_lists]
        self.nham = len(lists)
        K = basis.nbrOrbitals
        self.K = K
        tabs = [QuarticTermTables(K, v) for v in lists]
        kt = tabs[0].m_kTable
        vts = np.ascontiguousarray(np.concatenate([t.m_vTable for t in tabs]))
        self.basis = basis
        h = ctypes.c_void_p()
        check(lib().ed_batch_create(basis.handle(), self.nham, kt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                    _f64p(vts), int(autotune), ctypes.byref(h)))
        self._h = h
        n, nnz, nh = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        check(lib().ed_batch_dims(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nh)))
        self.n, self.nnz = int(n.value), int(nnz.value)

    def spmm(self, X, Y, stream=None):
        """Y[:, b] = H_b X[:, b] on device [n][nham] arrays (torch CUDA tensors)."""
        check(lib().ed_batch_spmm(self._h, _dptr(X), _dptr(Y), stream))

    def solve(self, nev: int, tol: float = 1e-10, V0=None, seed: int = 0, ncv: int = 0, want_vectors: bool = False,
              verify: bool = True, max_restarts: int = 0, select=None):
        """Lowest nev eigenpairs of every Hamiltonian (or of the Hamiltonians
        listed in select, in that order).  V0: device [n][count] start vectors
        (torch tensor) or None.  Returns (evals [count, nev], evecs device
        tensor [nev, n, count] or None, info dict)."""
        p = C.LanczosParams(nev=nev, ncv=ncv, max_restarts=max_restarts, tol=tol, seed=seed,
                            want_vectors=int(want_vectors), verify=int(verify))
        info = C.BatchInfo()
        cnt = self.nham if select is None else len(select)
        ev = np.empty(cnt * nev)
        vec = None
        if want_vectors:
            import torch
            vec = torch.empty((nev, self.n, cnt), dtype=torch.float64, device="cuda")
        v0p = None if V0 is None else _dptr(V0)
        vp = None if vec is None else _dptr(vec)
        if select is None:
            check(lib().ed_batch_solve(self._h, ctypes.byref(p), v0p, _f64p(ev), vp, ctypes.byref(info)))
        else:
            sel = np.ascontiguousarray(select, dtype=np.int32)
            check(lib().ed_batch_solve_subset(self._h, sel.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(sel),
                                              ctypes.byref(p), v0p, _f64p(ev), vp, ctypes.byref(info)))
        return ev.reshape(cnt, nev), vec, info.as_dict()

    def subspace_ritz(self, subspace: "Subspace", nev: int, nchk: int | None = None):
        """Lowest nev Ritz pairs of every Hamiltonian in the subspace, with the
        true residual norms of the first nchk (default nev) through the batch's
        operator.  Returns (evals [nham, nev], X device tensor [nev, n, nham],
        res [nham, nchk])."""
        import torch
        nchk = nev if nchk is None else nchk
        ev = np.empty(self.nham * nev)
        res = np.empty(max(1, self.nham * nchk))
        X = torch.empty((nev, self.n, self.nham), dtype=torch.float64, device="cuda")
        check(lib().ed_batch_subspace_ritz(self._h, subspace._h, nev, nchk, _f64p(ev), _dptr(X), _f64p(res)))
        return ev.reshape(self.nham, nev), X, res[:self.nham * nchk].reshape(self.nham, nchk)

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_batch_free(self._h)
            self._h = None


class Subspace:
    """Orthonormal device vectors of one sector shared by the Ritz step of a
    batch (ed_subspace_*).  No reference counterpart."""

    def __init__(self, n: int, max_dim: int):
        h = ctypes.c_void_p()
        check(lib().ed_subspace_create(int(n), int(max_dim), ctypes.byref(h)))
        self._h = h
        self.n, self.max_dim = int(n), int(max_dim)

    @property
    def dim(self) -> int:
        d = ctypes.c_int()
        check(lib().ed_subspace_dim(self._h, ctypes.byref(d)))
        return int(d.value)

    def add(self, U, drop_tol: float = 1e-14) -> int:
        """Append the columns of a device tensor U [groups, n, width] (the
        layout of a batch solve's eigenvectors) after Gram-Schmidt; returns how
        many were kept."""
        if U.dim() == 2:
            U = U[None]
        kept = ctypes.c_int()
        check(lib().ed_subspace_add(self._h, _dptr(U.contiguous()), int(U.shape[0]), int(U.shape[2]), float(drop_tol),
                                    ctypes.byref(kept)))
        return int(kept.value)

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_subspace_free(self._h)
            self._h = None


class WarmStartMLP:
    """Learned warm start (ed_mlp_*): an MLP from (occupation bits, V1) to
    (log|psi|, sign logit), trained on ground states the solver produced and
    evaluated on a sector to seed Lanczos."""

    def __init__(self, norb: int, hidden: int = 256, seed: int = 0):
        h = ctypes.c_void_p()
        check(lib().ed_mlp_create(norb, hidden, seed, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int64()
        check(lib().ed_mlp_num_params(h, ctypes.byref(n)))
        self.nparam = int(n.value)
        self.norb, self.hidden = norb, hidden

    def params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        check(lib().ed_mlp_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.nparam))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().ed_mlp_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.nparam))

    def forward(self, words_dev, v1_dev, out_dev):
        check(lib().ed_mlp_forward(self._h, _dptr(words_dev), _dptr(v1_dev), int(words_dev.numel()), _dptr(out_dev)))

    def gradients(self, words_dev, v1_dev, target_dev):
        g = np.empty(self.nparam, dtype=np.float32)
        loss = ctypes.c_double()
        check(lib().ed_mlp_gradients(self._h, _dptr(words_dev), _dptr(v1_dev), _dptr(target_dev),
                                     int(words_dev.numel()), g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                     ctypes.byref(loss)))
        return g, loss.value

    def fit(self, basis: FermionFockBasis, v1s, psi_dev, steps: int = 2000, batch: int = 4096, lr: float = 1e-3,
            seed: int = 0) -> float:
        """psi_dev: device [n][len(v1s)] ground states (torch tensor)."""
        v = np.ascontiguousarray(v1s, dtype=np.float64)
        loss = ctypes.c_double()
        check(lib().ed_mlp_fit(self._h, basis.handle(), _f64p(v), len(v), _dptr(psi_dev), steps, batch, lr, seed,
                               ctypes.byref(loss)))
        return loss.value

    def warm_start(self, basis: FermionFockBasis, v1s, V0_dev):
        v = np.ascontiguousarray(v1s, dtype=np.float64)
        check(lib().ed_warm_start(self._h, basis.handle(), _f64p(v), len(v), _dptr(V0_dev)))

    def __del__(self):
        if getattr(self, "_h", None) is not None and C._LIB is not None:
            C._LIB.ed_mlp_free(self._h)
            self._h = None
