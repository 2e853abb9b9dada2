/*
 * ed_capi.h - C ABI of the GB300-native exact-diagonalization engine for the
 * lowest-Landau-level spinless-fermion model on the sphere.
 *
 * The engine replaces, on one GPU, the hot path of the reference
 * (SimonDavenport/hamiltonian_diagonalization):
 *   Fock basis of a fixed-Lz sector  -> quartic Hamiltonian build into CRS
 *   -> Hamiltonian-vector product   -> Lanczos/ARPACK eigensolve.
 * Each entry point below names the reference interface it stands in for.
 *
 * Conventions
 *  - Every function returns ed_status (0 = ED_OK).  No C++ exception crosses
 *    this boundary.  ed_last_error() gives the message of the last failure on
 *    the calling thread.
 *  - Handles are opaque, library-owned, released with the matching *_free.
 *    A handle must not be used by two host threads at once.
 *  - Pointers named *_dev are device pointers owned by the caller; pointers
 *    named *_host (or plain arrays in host-side calls) are host memory.
 *  - Streams are CUDA runtime streams (cudaStream_t is `struct CUstream_st*`);
 *    NULL means the legacy default stream.
 *  - Fock states are uint64 words, bit k = orbital k occupied, orbital k
 *    carrying twice-angular-momentum m = 2k - (norb-1) in the Lz predicate
 *    (angular_momentum_constraint.hpp:56).  The term tables use the
 *    reference's k = (maxLz - m)/2 labels (pseudopotential_model_base.hpp:67).
 *  - Indices and dimensions are uint64/int64; CRS column indices are int32
 *    and row pointers int64 (the reference uses int32 for both; int64 row
 *    pointers lift its 2^31-1 nonzero cap).
 */
#ifndef ED_CAPI_H
#define ED_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ed_stream;

typedef enum {
    ED_OK = 0,
    ED_ERR_ARG = 1,          /* bad argument (null pointer, size, range)            */
    ED_ERR_OOM = 2,          /* device or host allocation failed                    */
    ED_ERR_CUDA = 3,         /* CUDA runtime error                                  */
    ED_ERR_NOCONV = 4,       /* eigensolver hit its iteration cap                   */
    ED_ERR_BREAKDOWN = 5,    /* Krylov breakdown that could not be recovered        */
    ED_ERR_RANGE = 6,        /* problem outside the supported sizes                 */
    ED_ERR_INTERNAL = 7,     /* a device-side consistency check failed              */
    ED_ERR_EMPTY = 8         /* the requested sector has dimension 0                */
} ed_status;

typedef struct ed_basis ed_basis;   /* FermionFockBasis (basis/fermion_fock_basis.hpp:45)        */
typedef struct ed_terms ed_terms;   /* QuarticTermTables (fqhe_sphere/.../term_tables.hpp)      */
typedef struct ed_crs ed_crs;       /* CrsSparseMatrix<double> (utilities/data_structures/crs_sparse_matrix.hpp:123) */
typedef struct ed_op ed_op;         /* the H*v operator bound into the eigensolver               */
typedef struct ed_cterms ed_cterms; /* complex QuarticTermTables + QuadraticTermTables of the
                                       optical-flux-lattice model (interacting_ofl_model/term_tables.hpp) */
typedef struct ed_ccrs ed_ccrs;     /* CrsSparseMatrix<dcmplx>                                    */

/* ------------------------------------------------------------------ misc */
int ed_version(void);
const char* ed_status_string(ed_status s);
const char* ed_last_error(void);
/* Kernels launched by this library since it was loaded (a counter kept on
 * the host at every launch site). */
uint64_t ed_kernel_launches(void);
/* Number of visible CUDA devices (0 without a GPU); never fails. */
int ed_device_count(void);

/* ----------------------------------------------------- term tables (host) */

/* LLL Coulomb pseudopotentials on the sphere, out[m] = V_m, m = 0..norb-1.
 * Replaces GenCoulombPseudopotentials (fqhe_sphere/interaction_pseudopotentials/
 * coulomb_pseudopotentials.cpp:40-69) with mulFactor 1. */
ed_status ed_coulomb_pseudopotentials(int norb, double* out);

/* Quartic term tables of the pseudopotential Hamiltonian, K = norb:
 *   ktable[(k4*K+k3)*K+k2] = k1 with m1+m2 = m3+m4, 65535 if out of range
 *   vtable[(k4*K+k3)*K+k2] = -sum_L V_L <S m1,S m2|J M><S m3,S m4|J M>,
 *                            J = 2S - L (twice-units Lact = 2*maxLz - L)
 * Host arrays of K^3 entries.  Replaces BaseGenerate4KTable and
 * BaseTermsFromPseudopotentials (fqhe_sphere/pseudopotential_model/
 * pseudopotential_model_base.hpp:97-139, 150-229).  npp may not exceed
 * norb-1 (the reference's check, pseudopotential_model_data.cpp:285). */
ed_status ed_quartic_tables(int norb, const double* pseudopotentials, int npp,
                            uint16_t* ktable, double* vtable);

/* Clebsch-Gordan coefficient <j1 m1; j2 m2 | J M>, all arguments twice the
 * physical values; magnitudes at or below 1e-12 read as 0 like the
 * reference's stored table (utilities/wrappers/clebsch_gordan_wrapper.hpp:160). */
double ed_clebsch_gordan(int tj1, int tm1, int tj2, int tm2, int tJ, int tM);

/* --------------------------------------------------------------- basis K1/K2 */

/* Fock basis of the sector (N particles, norb orbitals, twice total Lz),
 * ascending uint64 words, built on the device.  A sector of dimension 0 gives
 * a valid handle with dim 0 (the reference's isZeroDim == true).
 * Replaces FermionFockBasis::GenerateFockSpace (fermion_fock_basis.cpp:241-354)
 * with the TestAngularMomentumSector constraint. */
ed_status ed_basis_build(int N, int norb, int two_lz, ed_stream stream, ed_basis** out);
/* Two-Landau-level sector basis: N particles in norb0 = 2S+1 lowest-level
 * orbitals and norb0 + 2 second-level orbitals with total 2Lz = two_lz,
 * ordered as TwoLevelFermionFockBasis::GenerateFockSpace sorts it
 * (two_level_fermion_fock_basis.cpp:289-470; TestAngularMomentumSector2LL,
 * two_level_angular_momentum_constraint.hpp:41-70).  Each state is one word,
 * (first << (norb0 + 2)) | second, so ascending words are the reference's
 * (first, second) order; words of up to 48 bits (norb0 <= 23). */
ed_status ed_basis2_build(int N, int norb0, int two_lz, ed_stream stream, ed_basis** out);
/* levels (1 or 2) and the orbital counts of each level (norb1 = 0 for one level). */
ed_status ed_basis_levels(const ed_basis* b, int* levels, int* norb0, int* norb1);
ed_status ed_basis_free(ed_basis* b);
ed_status ed_basis_dim(const ed_basis* b, uint64_t* dim);
/* Device pointer to the n basis words (valid while the handle lives). */
ed_status ed_basis_words(const ed_basis* b, const uint64_t** words_dev);
/* Copy the first n words to host (GetFockBasis, fermion_fock_basis.cpp:359). */
ed_status ed_basis_get(const ed_basis* b, uint64_t* host_words, uint64_t n);
/* Index of each word in the basis, UINT64_MAX when absent.  Device arrays.
 * Replaces FindFockStateIndex (fermion_fock_basis.cpp:134-161) with offset 0. */
ed_status ed_basis_rank(const ed_basis* b, const uint64_t* words_dev, uint64_t* idx_dev,
                        uint64_t m, ed_stream stream);
/* Host-array convenience form of ed_basis_rank. */
ed_status ed_basis_rank_host(const ed_basis* b, const uint64_t* words, uint64_t* idx, uint64_t m);

/* ------------------------------------------------------------------- terms */

/* Upload the quartic tables (host, K^3 entries each) and derive the per-hop
 * matrix-element table used by the device build.  Stands in for the
 * QuarticTermTables object handed to Add_CdCdCC_Terms
 * (spinless_fermion_hamiltonian.hpp:263-282: GetK1/GetVkkkk). */
ed_status ed_terms_set(int norb, const uint16_t* ktable, const double* vtable, ed_terms** out);
ed_status ed_terms_free(ed_terms* t);

/* -------------------------------------------------------- Hamiltonian K3 */

/* Build H into CRS on the device: int64 row pointers, int32 columns
 * ascending within each row, FP64 values.  store_upper = 1 keeps the upper
 * triangle (col >= row) exactly as the reference stores it; 0 stores both
 * triangles, the lower part being the bit-exact transpose of the upper.
 * Same element set, signs, summation order and 1e-14 trims as
 * SpinlessFermionHamiltonian::Add_CdCdCC_Terms + MappedSparseMatrix::Trim +
 * CrsSparseMatrix::Initialize (spinless_fermion_hamiltonian.hpp:282-436,
 * mapped_sparse_matrix.hpp:423-460, crs_sparse_matrix.hpp:193-254). */
ed_status ed_ham_build_crs(const ed_basis* b, const ed_terms* t, int store_upper,
                           ed_stream stream, ed_crs** out);
/* Two-Landau-level Hamiltonian into CRS for a basis from ed_basis2_build:
 * level-0 quartic terms t0 (norb0 orbitals) and level-1 terms t1 (norb0 + 2
 * orbitals, from the second level's pseudopotentials), plus optional
 * occupation energies energies0[norb0] / energies1[norb0 + 2] (host, NULL for
 * none).  Replaces SphereTwoLevelPseudopotentialModel::BuildHamiltonian
 * (two_level_pseudopotential_model.cpp:190-215) over
 * TwoLevelSpinlessFermionHamiltonian::Add_CdC_Terms / Add_CdCdCC_Terms
 * (two_level_spinless_fermion_hamiltonian.hpp:143-470): same elements, signs,
 * call-order summation of the diagonal and 1e-14 trims; columns ascending. */
ed_status ed_ham2_build_crs(const ed_basis* b, const ed_terms* t0, const ed_terms* t1, const double* energies0,
                            const double* energies1, int store_upper, ed_stream stream, ed_crs** out);
ed_status ed_crs_free(ed_crs* a);
ed_status ed_crs_info(const ed_crs* a, int64_t* n, int64_t* nnz, int* upper);
ed_status ed_crs_arrays(const ed_crs* a, const int64_t** rowptr_dev, const int32_t** col_dev,
                        const double** val_dev);
/* Copy CRS to host arrays of n+1 / nnz / nnz entries. */
ed_status ed_crs_get(const ed_crs* a, int64_t* rowptr, int32_t* col, double* val);
/* Diagonal of H (n doubles, device), computed in the reference's term order. */
ed_status ed_ham_diagonal(const ed_basis* b, const ed_terms* t, double* diag_dev, ed_stream stream);

/* ------------------------------------------------------------ H*v K4 / K5 */

/* y = H x from a stored CRS (either storage).  Device vectors of n doubles.
 * Replaces MatrixVectorFunction::Simple (hamiltonians/matrix_vector_routines.hpp:94-104)
 * -> SymmetricMatrixVectorMultiply (utilities/mathematics/sparse_linear_algebra.hpp:78-168).
 * Full storage uses the fixed-point integer kernels (kernel 6 below for 96
 * and more elements a row on average, the one-level sectors; kernel 8 on
 * the sliced-ELL copy for shorter rows from 4096 rows up, the two-level
 * sectors): the first product makes a fixed-point copy of the values (8
 * bytes an element) and, per stream, an n-element scratch for x; products of
 * one matrix on one stream must not overlap (they share that stream's
 * scratch). */
ed_status ed_spmv(const ed_crs* a, const double* x_dev, double* y_dev, ed_stream stream);

/* The same product with a chosen kernel of the full storage, for measuring
 * and testing them side by side: 0 as ed_spmv (chosen by shape), 1 the
 * row-lane kernel (8 lanes a row, 4 loads ahead), 2 / 3 the shared-reduction
 * kernel (8 lanes take two consecutive rows and reduce-scatter their sums; 4 /
 * 2 loads ahead), 4 / 5 the sliced-ELL kernel (one lane a row over a
 * length-sorted, chunk-transposed copy made on first use; 16 / 8 loads
 * ahead), 6 the fixed-point integer kernel (8 lanes a row, 8 loads ahead):
 * values and x rounded to 58-bit fixed point relative to their largest
 * binary exponents, each row's sum formed exactly in integers and rounded
 * once to FP64, so y does not depend on the element order; a non-finite
 * entry of x gives NaN in every entry of y; 7 the same arithmetic with the
 * rows' values and columns streamed into shared memory by bulk copies (a
 * producer warp and a ring of stages of 16 rows, one consumer warp a row;
 * the same bits as 6); 8 the same arithmetic over the sliced-ELL copy (one
 * lane a row; the same bits as 6; the default for rows shorter than 96
 * elements on average).  ED_ERR_ARG for 1-8 on upper-triangle storage;
 * ED_ERR_RANGE for 4-8 when the copy does not fit in half the free device
 * memory, for 6-8 also when a value is not finite, a row has more than 2048
 * elements, or the stream's first product is inside a capture.  The values
 * must not change after the first product (the copies are made once). */
ed_status ed_spmv_kernel(const ed_crs* a, int kernel, const double* x_dev, double* y_dev, ed_stream stream);

/* Use kernel (an ed_spmv_kernel id; 0 restores the choice by shape) for every
 * later product of a, including those inside the eigensolvers. */
ed_status ed_crs_set_product_kernel(ed_crs* a, int kernel);

/* A test of the staged kernel's (ed_spmv_kernel 7) bounded waits on the
 * legacy stream: the kernel runs with its first stage never filled and every
 * wait limited to wait_cycles SM clock cycles, so that the waits run out; it
 * returns, leaves NaN in the rows of the waiting warps, and *timeouts is the
 * number of waits that ran out (their error word is then reset).  The device
 * stays usable. */
ed_status ed_spmv_staged_wait_test(const ed_crs* a, const double* x_dev, double* y_dev, long long wait_cycles,
                                   int* timeouts);

/* Measured FP64 FMA issue rate of the current device (FMA per second): a
 * kernel of blocks_per_sm blocks per SM, 256 threads, eight independent FMA
 * chains of iters steps per thread; the ceiling of the FP64 products. */
ed_status ed_fp64_fma_rate(int iters, int blocks_per_sm, double* fma_per_second);

/* y = H x with the matrix elements regenerated on the fly from the basis and
 * the term tables (no stored matrix).  Stands in for the reference's
 * unfinished MatrixVectorFunction::Recalculate (matrix_vector_routines.hpp:112-143). */
ed_status ed_hv_matfree(const ed_basis* b, const ed_terms* t, const double* x_dev, double* y_dev,
                        ed_stream stream);

/* ------------------------------------------------------------ eigensolver */

typedef void (*ed_host_matvec)(const double* x_host, double* y_host, void* user);

/* Operators the eigensolver can drive. */
ed_status ed_op_from_crs(const ed_crs* a, ed_op** out);
ed_status ed_op_matfree(const ed_basis* b, const ed_terms* t, ed_op** out);
/* A host callback y = A x on host arrays of n doubles: the generic
 * std::function form of ArpackWrapper::DiagonalizeSymmetricMatrix
 * (arpack_wrapper.hpp:595-606).  Vectors cross PCIe/NVLink-C2C per product. */
ed_status ed_op_host_callback(int64_t n, ed_host_matvec fn, void* user, ed_op** out);
ed_status ed_op_free(ed_op* op);
ed_status ed_op_dim(const ed_op* op, int64_t* n);

typedef struct {
    int nev;            /* eigenpairs wanted (lowest algebraic)                      */
    int ncv;            /* Krylov subspace size; 0 -> min(n, 2*nev+21) like ARPACK     */
    int max_restarts;   /* 0 -> 2000 (the reference's ARPACK iteration cap)           */
    double tol;         /* residual ||H x - theta x||_2 (x unit) required per pair     */
    uint64_t seed;      /* start vector uniform(-1,1) from this seed if none is given  */
    int want_vectors;   /* caller's note only: eigenvectors are written whenever the
                           eigenvector pointer of the call is non-NULL              */
    int verify;         /* 1 -> recompute true residuals with extra products            */
    int degeneracy_passes;  /* 0 -> one Krylov sequence.  k > 0 -> up to k further solves
                           of H + s X X^T (X the pairs found, s above their spread),
                           each merging eigenvalues below the nev-th found: the extra
                           copies of degenerate eigenvalues one start vector cannot
                           see.  Ends early when a pass adds nothing.  The batched
                           solver ignores it.                                         */
    int diagonal_check;  /* 1 -> a stored matrix (CRS operator, complex CRS) with no
                           off-diagonal element above 1e-14 in modulus is solved
                           directly: its nev lowest diagonal entries, each with its
                           own unit vector (HamiltonianBase::MatrixDiagonalCheck and
                           the shortcut after it, hamiltonian_base.hpp:378-449,
                           660-700, 803-850; the reference gives every copy of a
                           repeated value the same normalised indicator vector).    */
} ed_lanczos_params;

typedef struct {
    int converged;      /* number of converged pairs among the nev returned           */
    int restarts;
    int64_t matvecs;
    double max_residual;    /* max over returned pairs of the residual (true one if verify) */
    double seconds;         /* wall time of the solve                                  */
    double spmv_seconds;    /* device time inside the H*v products                     */
    int breakdowns;
} ed_solve_info;

/* Lowest nev eigenpairs of a real symmetric operator by thick-restart Lanczos
 * with full FP64 reorthogonalisation on the device.  v0_host (n doubles) may
 * be NULL (seeded random start).  evals_host receives nev values ascending;
 * evecs_host (n*nev, column-major, may be NULL) the unit eigenvectors.
 * Replaces ArpackWrapper::DiagonalizeSymmetricMatrix<double> (MPI form,
 * arpack_wrapper.hpp:595-937) as driven by LanczosDiagonalize
 * (hamiltonian_base.hpp:770-931); unlike the reference, which returns
 * ARPACK's Ritz order, the values come sorted ascending. */
ed_status ed_lanczos(const ed_op* op, const ed_lanczos_params* p, const double* v0_host,
                     double* evals_host, double* evecs_host, ed_solve_info* info);

/* Two-level Hamiltonian (ed_ham2_build_crs on basis b): one Krylov sequence,
 * then every copy of each degenerate eigenvalue from the level-exchange
 * ladder L0- L1+ and its adjoint, which commute with H (the levels do not
 * mix: eigenvalues E0(L0) + E1(L1) repeat 2 min(L0, L1) + 1 times); the kept
 * vectors are checked by their residuals (a Rayleigh-Ritz step if needed, the
 * degeneracy passes as the last resort).  Same arguments as ed_lanczos;
 * replaces LanczosDiagonalize for TwoLevelSpinlessFermionHamiltonian
 * (hamiltonian_base.hpp:770-931), whose ARPACK call returns copies only as
 * rounding lets it. */
ed_status ed_lanczos_two_level(const ed_basis* b, const ed_op* op, const ed_lanczos_params* p,
                               const double* v0_host, double* evals_host, double* evecs_host, ed_solve_info* info);

/* Same solve with device-resident start vector and outputs (n doubles /
 * n*nev doubles, column-major).  Either output may be NULL. */
ed_status ed_lanczos_device(const ed_op* op, const ed_lanczos_params* p, const double* v0_dev,
                            double* evals_host, double* evecs_dev, ed_solve_info* info);

/* Dense symmetric eigen-decomposition on the host (FP64; Householder
 * tridiagonalisation + implicit QR with Wilkinson shifts): a is m*m row-major,
 * evals ascending, evecs column-major (may be NULL).  The projected-matrix
 * solver of ed_lanczos (one small matrix per restart solves faster on a host
 * core than on one SM's FP64 pipe), exposed for reuse; replaces the small
 * dense problems the reference hands to LAPACK dsyevr_
 * (utilities/wrappers/lapack_wrapper.hpp:479-540, FullDiagonalize,
 * hamiltonians/hamiltonian_base.hpp:634-758). */
ed_status ed_dense_sym_eigen(int m, const double* a, double* evals, double* evecs);
/* count such m x m matrices (1 <= m <= 128) at once on the device (FP64
 * cyclic Jacobi, one CTA each): a count*m*m, evals count*m, evecs count*m*m
 * (host arrays).  The projected problems of the batched solver and of the
 * subspace Ritz step, where a batch solves in the time of one matrix; the
 * batched counterpart of the dsyevr_ calls above. */
ed_status ed_sym_eigen_batched(int m, int count, const double* a, double* evals, double* evecs);

/* ||H x_i - lambda_i x_i||_2 for k device vectors (column-major n*k). */
ed_status ed_residuals(const ed_op* op, const double* x_dev, const double* lambda_host, int k,
                       double* res_host);

/* Allocation-free form of ed_residuals, for callers that cannot let the
 * library call cudaMalloc (programs that give all device memory to their own
 * pool allocator, and loops where cudaMalloc/cudaFree would synchronise the
 * device).  Same inputs and outputs; no reference counterpart (the reference
 * computes no residuals on a device).  The product is fused into the residual
 * and the only scratch is one file-scope device array of 513 KiB per device,
 * held until the process exits.  Limits: 1..64 vectors per call; a stored CRS
 * with both triangles only; the CRS and x_dev on the current device
 * (ED_ERR_ARG otherwise).  All calls on a device share that array, so calls
 * that overlap on the GPU race: serialise them.  The first call on a device
 * looks up the array's address with that device current and keeps it; make
 * that call before any stream capture, and do not use the entry point after
 * a cudaDeviceReset (the kept address is then stale).  It runs on the legacy
 * default stream, which does not wait for non-blocking streams: x_dev must be
 * complete before the call (synchronise the stream that wrote it).  Returns
 * when res_host is filled. */
ed_status ed_residuals_noalloc(const ed_op* op, const double* x_dev, const double* lambda_host, int k,
                               double* res_host);

/* Thick-restart basis rotation out = V Y[:, 0..k): V_dev n x m and out_dev
 * n x k column-major device arrays, Y_host column-major with leading
 * dimension ldy >= m.  method 1: FP64 FMAs; 2: BF16 tensor cores with
 * FP64-accurate digit splitting (m <= 64; V's digits in registers for
 * m <= 48 and k <= 32, else staged in shared memory); 3: the same with V's
 * digits always staged in shared memory (same bits as 2); 0: the solver's
 * choice (2 when m <= 64).  The step of ARPACK's dneupd/dnaupd that forms Ritz vectors from
 * the Arnoldi basis (arpack_wrapper.hpp:873-883 call site); exported so the
 * two methods can be compared.  Returns when out_dev is written. */
ed_status ed_basis_rotate(const double* V_dev, int64_t n, int m, const double* Y_host, int ldy, int k,
                          double* out_dev, int method);

/* ------------------------------------------------------------- file formats */

/* The reference's file formats (text = 0 or binary = 1), so that data moves
 * between reference runs and this engine.  Host arrays.
 * Eigensystem files: HamiltonianBase::EigensystemToFile / EigensystemFromFile
 * (hamiltonians/hamiltonian_base.hpp:1204-1304, 1309-1400); evecs (nev x dim,
 * vector after vector) may be NULL to write eigenvalues only.  Reading: call
 * with evals = evecs = NULL to learn nev and dim (dim 0: no vectors stored). */
ed_status ed_eigensystem_write(const char* path, int binary, int nev, const double* evals, uint64_t dim,
                               const double* evecs);
ed_status ed_eigensystem_read(const char* path, int binary, int* nev, double* evals, uint64_t* dim,
                              double* evecs);
/* CRS files: CrsSparseMatrix::ToFile / FromFile
 * (utilities/data_structures/crs_sparse_matrix.hpp:662-740); int32 indices,
 * so ED_ERR_RANGE above 2^31-1 nonzeros.  `upper` tells the reader whether
 * the file holds the upper triangle (the reference's storage) or both. */
ed_status ed_crs_write(const ed_crs* a, const char* path, int binary);
ed_status ed_crs_read(const char* path, int binary, int upper, ed_crs** out);
/* Quartic term-table files: TermTablesBase::ToFileBase / FromFileBase with 4
 * labels (hamiltonians/term_tables_base.hpp:179-335).  Reading: call with
 * ktable = vtable = NULL to learn norb, then with K^3-entry arrays. */
ed_status ed_quartic_tables_write(const char* path, int binary, int norb, const uint16_t* ktable,
                                  const double* vtable);
ed_status ed_quartic_tables_read(const char* path, int binary, int* norb, uint16_t* ktable, double* vtable);

/* ------------------------------------------------------ batched sweep K6 */

/* Many Hamiltonians of one sector that differ only in their pseudopotentials
 * (e.g. a V1 sweep), solved together.  No reference counterpart: the
 * reference solves one Hamiltonian per run (pseudopotential_model.cpp:264).
 * Vectors of a batch are [row][problem] arrays: element (r, b) at r*nham + b. */
typedef struct ed_batch ed_batch;

typedef struct {
    int converged;            /* problems whose nev pairs all converged             */
    int restarts;
    int64_t block_products;   /* each applies every Hamiltonian of the batch once   */
    double max_residual;
    double seconds;
    double spmm_seconds;      /* device time inside the block products               */
    int breakdowns;
    int tile_hamiltonians;    /* autotuned Hamiltonians per row tile of the block product */
    int tile_unroll;          /* autotuned loads in flight per lane                  */
    int tile_l1;              /* 1: hop values read through L1, 0: staged in shared memory */
    int tile_threads;         /* threads per CTA of the block product                */
    int64_t problem_products; /* sum over block products of the Hamiltonians still
                                 iterating (converged ones retire at restarts)        */
} ed_batch_info;

/* Shared pattern (int32 column + uint16 hop code per element) built once on
 * the device, per-Hamiltonian hop tables and diagonals.  vtables holds nham
 * V tables of K^3 entries each (ed_quartic_tables), all with the one
 * momentum-conserving ktable.  autotune != 0 times the block-product
 * variants on this data and keeps the fastest. */
ed_status ed_batch_create(const ed_basis* b, int nham, const uint16_t* ktable, const double* vtables, int autotune,
                          ed_batch** out);
ed_status ed_batch_free(ed_batch* bt);
ed_status ed_batch_dims(const ed_batch* bt, int64_t* n, int64_t* nnz_offdiag, int* nham);
/* Y[:, b] = H_b X[:, b] for every Hamiltonian b (device [n][nham] arrays). */
ed_status ed_batch_spmm(const ed_batch* bt, const double* X_dev, double* Y_dev, ed_stream stream);
/* Lowest p->nev eigenpairs of every Hamiltonian, all in lockstep (the
 * thick-restart Lanczos of ed_lanczos, batched).  V0_dev: [n][nham] start
 * vectors or NULL (seeded random); evals_host: nham*nev values, ascending per
 * Hamiltonian; evecs_dev (may be NULL): nev consecutive [n][nham] arrays. */
ed_status ed_batch_solve(const ed_batch* bt, const ed_lanczos_params* p, const double* V0_dev, double* evals_host,
                         double* evecs_dev, ed_batch_info* info);
/* The same solve for the Hamiltonians sel[0..nsel) of the batch only (no
 * reference counterpart: the sweep's anchor and fallback solves).  V0_dev:
 * [n][nsel] or NULL; evals_host: nsel*nev; evecs_dev: nev consecutive
 * [n][nsel] arrays; both in the selection's order. */
ed_status ed_batch_solve_subset(const ed_batch* bt, const int* sel, int nsel, const ed_lanczos_params* p,
                                const double* V0_dev, double* evals_host, double* evecs_dev, ed_batch_info* info);

/* -------------------------- shared-subspace Rayleigh-Ritz (eigenvector continuation)
 * No reference counterpart: the reference solves every Hamiltonian of a
 * pseudopotential sweep from scratch.  A subspace is an orthonormal set of up
 * to 256 device vectors of one sector; ed_batch_subspace_ritz finds every
 * batch Hamiltonian's lowest Ritz pairs in it and checks them with the
 * batch's own operator. */
typedef struct ed_subspace ed_subspace;
ed_status ed_subspace_create(int64_t n, int max_dim, ed_subspace** out);
ed_status ed_subspace_free(ed_subspace* sp);
ed_status ed_subspace_dim(const ed_subspace* sp, int* dim);
/* Append the columns of U_dev ([groups][n][width], e.g. the eigenvectors of
 * ed_batch_solve) after two classical Gram-Schmidt passes against the
 * subspace; a column keeping no more than drop_tol of its norm is dropped.
 * *kept (may be NULL) = columns appended. */
ed_status ed_subspace_add(ed_subspace* sp, const double* U_dev, int groups, int width, double drop_tol, int* kept);
/* Lowest nev Ritz pairs of every Hamiltonian of the batch in the subspace:
 * evals_host [nham][nev] ascending, X_dev nev consecutive [n][nham] arrays,
 * res_host [nham][nchk] = ||H_b x - theta x|| of the first nchk pairs through
 * the batch's block product.  The Hamiltonians must form a linear family of
 * rank <= 8 (a pseudopotential sweep has rank 2), else ED_ERR_ARG. */
ed_status ed_batch_subspace_ritz(const ed_batch* bt, const ed_subspace* sp, int nev, int nchk, double* evals_host,
                                 double* X_dev, double* res_host);

/* ------------------------------------- complex path (optical-flux-lattice model) */

/* Momentum-sector basis: N particles on dimX*dimY orbitals p = kx*dimY + ky
 * whose total (kx mod dimX, ky mod dimY) is (kxTot, kyTot), words ascending.
 * Replaces FermionFockBasis::GenerateFockSpace with TestLinearMomentumSector2
 * (interacting_ofl_model.cpp:994-1001, linear_momentum_constraints_2D.cpp:38-79).
 * The rank, word and observable entries above accept the handle. */
ed_status ed_basis_momentum_build(int N, int dimX, int dimY, int kxTot, int kyTot, ed_stream stream,
                                  ed_basis** out);
/* Complex term tables in the reference's array layout (QuarticTermTables,
 * interacting_ofl_model/term_tables.cpp:95-200): ktable and vtable (complex as
 * re, im pairs) of (norb+1)*norb*norb/2 entries at (t1*norb + t2 -
 * t1(t1+1)/2)*norb + k, t1 = min(k3,k4), t2 = max(k3,k4); k1 = ktable[.. + k2]
 * and V(k1,k2,k3,k4) = vtable[.. + (k4 > k3 ? k1 : k2)].  energies: norb
 * complex occupation energies (QuadraticTermTables::GetEkk, :59-65) or NULL.
 * The k-table must conserve the 2D momentum (FindK1, interacting_ofl_model.cpp:366-410). */
ed_status ed_cterms_create(int norb, int dimX, int dimY, const uint16_t* ktable, const double* vtable,
                           const double* energies, ed_cterms** out);
ed_status ed_cterms_free(ed_cterms* t);
/* The same terms from the reference's hash-table format (TermHashTables,
 * hamiltonians/term_hash_tables_base.hpp:44-276, as InteractingOflModel::
 * ConvertTableFormat fills it, interacting_ofl_model.cpp:597-618): the quartic
 * k-table (nk keys of (k2, k3, k4) packed as (k2 << 48) | (k3 << 32) | (k4 <<
 * 16), each with one k1) and value table (nv keys of (k1, k2, k3, k4) packed
 * as (k1 << 48) | (k2 << 32) | (k3 << 16) | k4, complex values as re, im
 * pairs), and optionally the quadratic ones (k-table keys k2 with k1 values,
 * value keys (k1 << 32) | k2).  The tables must be momentum-conserving: one
 * k1 for every (k2, k3, k4), k1 = k2 in the quadratic tables, and values that
 * the array layout holds (ED_ERR_ARG otherwise).  Same result as
 * ed_cterms_create on the arrays they were filled from. */
ed_status ed_cterms_create_hash(int norb, int dimX, int dimY, uint32_t nk, const uint64_t* kkeys,
                                const uint16_t* kvals, uint32_t nv, const uint64_t* vkeys, const double* vvals,
                                uint32_t nqk, const uint64_t* qkkeys, const uint16_t* qkvals, uint32_t nqv,
                                const uint64_t* qvkeys, const double* qvvals, ed_cterms** out);
/* The hash-table files of TermHashTables::ToFileBase / FromFileBase
 * (term_hash_tables_base.hpp:139-205 with multi_key_hash.hpp:480-682): the
 * header line, then the k-table (nlabels - 1 labels) and the value table
 * (nlabels labels: 4 quartic, 2 quadratic), binary (uint32 count, uint64 keys,
 * then uint16 k1 values or (re, im) doubles) or text (count and label count,
 * then one tab-separated entry a line at 15 significant digits).
 * ed_term_hash_read: with NULL arrays it sets nk and nv to the entry counts;
 * with arrays of at least *nk and *nv entries it fills them. */
ed_status ed_term_hash_write(const char* path, int binary, int nlabels, uint32_t nk, const uint64_t* kkeys,
                             const uint16_t* kvals, uint32_t nv, const uint64_t* vkeys, const double* vvals);
ed_status ed_term_hash_read(const char* path, int binary, uint32_t* nk, uint64_t* kkeys, uint16_t* kvals,
                            uint32_t* nv, uint64_t* vkeys, double* vvals);
/* SpinlessFermionHamiltonian<dcmplx>::Add_CdC_Terms + Add_CdCdCC_Terms
 * (spinless_fermion_hamiltonian.hpp:150-436) as InteractingOflModel::
 * BuildHamiltonian calls them (interacting_ofl_model.cpp:1034-1052).  Upper
 * storage is the reference's: row = in-state, column = out-state >= in-state,
 * value <out|H|in>; full storage adds each element's conjugate at the mirrored
 * position.  Bit-exact against the reference's loops. */
ed_status ed_cham_build_crs(const ed_basis* b, const ed_cterms* t, int store_upper, ed_stream stream,
                            ed_ccrs** out);
ed_status ed_ccrs_free(ed_ccrs* a);
ed_status ed_ccrs_info(const ed_ccrs* a, int64_t* n, int64_t* nnz, int* upper);
/* Host copies: n+1 row pointers, nnz columns, 2*nnz doubles (re, im). */
ed_status ed_ccrs_get(const ed_ccrs* a, int64_t* rowptr, int32_t* col, double* val);
/* y = H x on device complex vectors (re, im pairs) with the reference's
 * Hermitian completion (SymmetricMatrixVectorMultiply<dcmplx>,
 * sparse_linear_algebra.hpp:143-164).  Full storage uses the fixed-point
 * integer kernel (ed_cspmv_kernel 2): the first product makes a fixed-point
 * copy of the values (16 bytes an element) and, per stream, a 2n-word scratch
 * for x; products of one matrix on one stream must not overlap. */
ed_status ed_cspmv(const ed_ccrs* a, const double* x_dev, double* y_dev, ed_stream stream);
/* The same product with a chosen kernel, for measuring and testing them side
 * by side: 0 as ed_cspmv, 1 the FP64 row kernel (4 FMA an element), 2 the
 * fixed-point integer kernel for full storage: the values' and x's real and
 * imaginary parts rounded to 58-bit fixed point relative to the largest
 * binary exponent of each, each row's real and imaginary sums formed exactly
 * in integers and rounded once to FP64 (y does not depend on element order; a
 * non-finite entry of x gives NaN in every entry of y).  ED_ERR_ARG for 2 on
 * upper-triangle storage; ED_ERR_RANGE for 2 when the copy does not fit in
 * half the free device memory, a value is not finite, a row has more than
 * 1024 elements, or the stream's first product is inside a capture.  Returns
 * after enqueueing on stream. */
ed_status ed_cspmv_kernel(const ed_ccrs* a, int kernel, const double* x_dev, double* y_dev, ed_stream stream);
/* Lowest nev eigenpairs of the complex Hermitian matrix by thick-restart
 * Lanczos with complex Gram-Schmidt; v0_host (2n doubles) may be NULL,
 * evecs_host receives nev vectors of n complex entries (re, im pairs).
 * Replaces ArpackWrapper::DiagonalizeSymmetricMatrix<dcmplx> (znaupd_/
 * zneupd_ branches, arpack_wrapper.hpp:255-937); values ascending. */
ed_status ed_clanczos(const ed_ccrs* a, const ed_lanczos_params* p, const double* v0_host, double* evals_host,
                      double* evecs_host, ed_solve_info* info);

/* ------------------------------------------------- learned warm start K10/K11 */

/* A small MLP (features: occupation bits as +-1 and the scaled V1, padded to
 * 32; three SiLU hidden layers of `hidden` units; outputs log|psi| and a sign
 * logit) trained with BF16 weights/activations and FP32 accumulation on the
 * tensor cores, FP32 master weights and Adam.  No reference counterpart: the
 * reference starts ARPACK from a random or file vector
 * (arpack_wrapper.hpp:753-774).  Parameters are laid out layer by layer,
 * weights [in][out] row-major then biases. */
typedef struct ed_mlp ed_mlp;
ed_status ed_mlp_create(int norb, int hidden, uint64_t seed, ed_mlp** out);
ed_status ed_mlp_free(ed_mlp* net);
ed_status ed_mlp_num_params(const ed_mlp* net, int64_t* count);
ed_status ed_mlp_get_params(const ed_mlp* net, float* host, int64_t count);
ed_status ed_mlp_set_params(ed_mlp* net, const float* host, int64_t count);
/* out_dev: m x 8 floats, columns 0 (log|psi|) and 1 (sign logit) used. */
ed_status ed_mlp_forward(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, int64_t m, float* out_dev);
/* Loss (mean squared log-amplitude error + sign cross-entropy) and its
 * gradient for one batch; target_dev: m x 2 (log|psi|, sign as 0/1). */
ed_status ed_mlp_gradients(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, const float* target_dev,
                           int64_t m, float* grads_host, double* loss_host);
ed_status ed_mlp_train_step(ed_mlp* net, const uint64_t* words_dev, const float* v1_dev, const float* target_dev,
                            int64_t m, float lr, double* loss_host);
/* Train on ground states psi_dev ([n][nv], one column per V1 value) of the
 * basis: `steps` Adam steps on seeded random batches of (state, V1).  The
 * columns' overall signs are first made consistent (V1 order, each overlapping
 * its predecessor positively); psi_dev itself is not changed. */
ed_status ed_mlp_fit(ed_mlp* net, const ed_basis* b, const double* v1_host, int nv, const double* psi_dev, int steps,
                     int batch, float lr, uint64_t seed, double* final_loss);
/* Start vectors for nham Hamiltonians: V0_dev[r*nham + j] = predicted psi of
 * basis word r at v1_host[j] (unnormalised; the solvers normalise). */
ed_status ed_warm_start(ed_mlp* net, const ed_basis* b, const double* v1_host, int nham, double* V0_dev);

/* ------------------------------------------------------------- observables */

/* Observables of a real eigenvector psi_host (n doubles on the host) of the
 * basis's sector: the reference's Observables (observables/fermion_observables.hpp)
 * for a real Hamiltonian, as device reductions over the basis.  Deterministic:
 * repeated calls return the same bits.  Orbital k is bit k of a Fock word. */
/* rho_host[k] = sum_s psi_s^2 n_k(s), k < norb.  Replaces
 * Observables::DensityFunction (fermion_observables.hpp:48-104). */
ed_status ed_obs_density(const ed_basis* b, const double* psi_host, double* rho_host);
/* table_host[k*norb + q] = sum_s psi_s^2 n_k(s) n_q(s) (symmetric; the diagonal
 * is rho).  Replaces Observables::DensityDensityFunction (fermion_observables.hpp:117-200). */
ed_status ed_obs_density_density(const ed_basis* b, const double* psi_host, double* table_host);
/* *ratio = 1 / sum_s |psi_s|^4.  Replaces Observables::GetParticipationRatio
 * (fermion_observables.hpp:528-562). */
ed_status ed_obs_participation_ratio(const ed_basis* b, const double* psi_host, double* ratio);
/* The min(k, n) entries of largest |psi_s| in descending order (ties: row
 * ascending) with their Fock words; *count_out = min(k, n).  Replaces
 * Observables::GetMostProbable (fermion_observables.hpp:437-517) for one
 * eigenvector (the reference loops over all of them). */
ed_status ed_obs_most_probable(const ed_basis* b, const double* psi_host, int64_t k, uint64_t* states_host,
                               double* amps_host, int64_t* count_out);

/* ------------------------------------------------------- one-call driver */

/* Whole sector solve from host inputs: basis -> tables -> CRS (or matrix-free
 * when matfree != 0) -> Lanczos; eigenvalues and optional eigenvectors to host.
 * The sequence SpherePseudopotentialModel::BuildTermTables / BuildFockBasis /
 * BuildHamiltonian / Diagonalize performs (pseudopotential_model.cpp:64-95,
 * 160, 233, 264) for one sector. */
ed_status ed_solve_sector(int N, int norb, int two_lz, const double* pseudopotentials, int npp,
                          int matfree, const ed_lanczos_params* p, const double* v0_host,
                          double* evals_host, double* evecs_host, ed_solve_info* info);

#ifdef __cplusplus
}
#endif
#endif /* ED_CAPI_H */
