"""GB300-native exact diagonalization of the lowest-Landau-level spinless-fermion
pseudopotential model on the sphere: device Fock basis, quartic Hamiltonian
build into CRS, H*v products and a thick-restart Lanczos in FP64, behind the C
ABI of libedgb300 (include/ed_capi.h)."""
from ._capi import EDError, LanczosParams, SolveInfo, lib  # noqa: F401
from .host import (  # noqa: F401
    ArpackWrapper,
    ComplexCrsSparseMatrix,
    ComplexQuarticTermTables,
    ComplexSpinlessFermionHamiltonian,
    CrsSparseMatrix,
    FermionFockBasis,
    HamiltonianBatch,
    Subspace,
    InteractingOflModel,
    MatrixVectorFunction,
    MpiWrapper,
    Observables,
    QuadraticTermHashTables,
    QuarticTermHashTables,
    QuarticTermTables,
    SpherePseudopotentialModel,
    SphereTwoLevelPseudopotentialModel,
    SpinlessFermionHamiltonian,
    TwoLevelFermionFockBasis,
    TwoLevelSpinlessFermionHamiltonian,
    WarmStartMLP,
    clebsch_gordan,
    coulomb_pseudopotentials,
    dense_sym_eigen,
    eigensystem_from_file,
    eigensystem_to_file,
    hash_key,
    odd_coulomb_list,
    solve_sector,
    synthetic_ofl_tables,
)

