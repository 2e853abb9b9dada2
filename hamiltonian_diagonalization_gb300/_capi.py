"""ctypes binding of libedgb300.so (the C ABI declared in include/ed_capi.h).

The library is the only compute path: if it is not built, loading fails with
an error instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libedgb300.so")

ED_OK = 0
ED_ERR_ARG = 1
ED_ERR_OOM = 2
ED_ERR_CUDA = 3
ED_ERR_NOCONV = 4
ED_ERR_BREAKDOWN = 5
ED_ERR_RANGE = 6
ED_ERR_INTERNAL = 7
ED_ERR_EMPTY = 8
MISS = 0xFFFFFFFFFFFFFFFF

c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_u64 = ctypes.c_uint64
c_double = ctypes.c_double
P = ctypes.POINTER


class EDError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


class LanczosParams(ctypes.Structure):
    _fields_ = [("nev", c_int), ("ncv", c_int), ("max_restarts", c_int), ("tol", c_double), ("seed", c_u64),
                ("want_vectors", c_int), ("verify", c_int), ("degeneracy_passes", c_int), ("diagonal_check", c_int)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("converged", c_int), ("restarts", c_int), ("matvecs", c_i64), ("max_residual", c_double),
                ("seconds", c_double), ("spmv_seconds", c_double), ("breakdowns", c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchInfo(ctypes.Structure):
    _fields_ = [("converged", c_int), ("restarts", c_int), ("block_products", c_i64), ("max_residual", c_double),
                ("seconds", c_double), ("spmm_seconds", c_double), ("breakdowns", c_int),
                ("tile_hamiltonians", c_int), ("tile_unroll", c_int), ("tile_l1", c_int),
                ("tile_threads", c_int), ("problem_products", c_i64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


HOST_MATVEC = ctypes.CFUNCTYPE(None, P(c_double), P(c_double), c_void_p)

_SIGS = {
    "ed_version": (c_int, []),
    "ed_status_string": (ctypes.c_char_p, [c_int]),
    "ed_last_error": (ctypes.c_char_p, []),
    "ed_device_count": (c_int, []),
    "ed_coulomb_pseudopotentials": (c_int, [c_int, P(c_double)]),
    "ed_quartic_tables": (c_int, [c_int, P(c_double), c_int, P(ctypes.c_uint16), P(c_double)]),
    "ed_clebsch_gordan": (c_double, [c_int] * 6),
    "ed_basis_build": (c_int, [c_int, c_int, c_int, c_void_p, P(c_void_p)]),
    "ed_basis_free": (c_int, [c_void_p]),
    "ed_basis_dim": (c_int, [c_void_p, P(c_u64)]),
    "ed_basis_words": (c_int, [c_void_p, P(c_void_p)]),
    "ed_basis_get": (c_int, [c_void_p, P(c_u64), c_u64]),
    "ed_basis_rank": (c_int, [c_void_p, c_void_p, c_void_p, c_u64, c_void_p]),
    "ed_basis_rank_host": (c_int, [c_void_p, P(c_u64), P(c_u64), c_u64]),
    "ed_terms_set": (c_int, [c_int, P(ctypes.c_uint16), P(c_double), P(c_void_p)]),
    "ed_terms_free": (c_int, [c_void_p]),
    "ed_ham_build_crs": (c_int, [c_void_p, c_void_p, c_int, c_void_p, P(c_void_p)]),
    "ed_crs_free": (c_int, [c_void_p]),
    "ed_crs_info": (c_int, [c_void_p, P(c_i64), P(c_i64), P(c_int)]),
    "ed_basis2_build": (c_int, [c_int, c_int, c_int, c_void_p, P(c_void_p)]),
    "ed_basis_momentum_build": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, P(c_void_p)]),
    "ed_cterms_create": (c_int, [c_int, c_int, c_int, P(ctypes.c_uint16), P(c_double), P(c_double), P(c_void_p)]),
    "ed_cterms_create_hash": (c_int, [c_int, c_int, c_int, ctypes.c_uint32, P(c_u64), P(ctypes.c_uint16), ctypes.c_uint32,
                                      P(c_u64), P(c_double), ctypes.c_uint32, P(c_u64), P(ctypes.c_uint16),
                                      ctypes.c_uint32, P(c_u64), P(c_double), P(c_void_p)]),
    "ed_term_hash_write": (c_int, [ctypes.c_char_p, c_int, c_int, ctypes.c_uint32, P(c_u64), P(ctypes.c_uint16),
                                   ctypes.c_uint32, P(c_u64), P(c_double)]),
    "ed_term_hash_read": (c_int, [ctypes.c_char_p, c_int, P(ctypes.c_uint32), P(c_u64), P(ctypes.c_uint16),
                                  P(ctypes.c_uint32), P(c_u64), P(c_double)]),
    "ed_cterms_free": (c_int, [c_void_p]),
    "ed_cham_build_crs": (c_int, [c_void_p, c_void_p, c_int, c_void_p, P(c_void_p)]),
    "ed_ccrs_free": (c_int, [c_void_p]),
    "ed_ccrs_info": (c_int, [c_void_p, P(c_i64), P(c_i64), P(c_int)]),
    "ed_ccrs_get": (c_int, [c_void_p, P(c_i64), P(ctypes.c_int32), P(c_double)]),
    "ed_cspmv": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ed_cspmv_kernel": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "ed_clanczos": (c_int, [c_void_p, P(LanczosParams), P(c_double), P(c_double), P(c_double), P(SolveInfo)]),
    "ed_ham2_build_crs": (c_int, [c_void_p, c_void_p, c_void_p, P(c_double), P(c_double), c_int, c_void_p,
                                  P(c_void_p)]),
    "ed_basis_levels": (c_int, [c_void_p, P(c_int), P(c_int), P(c_int)]),
    "ed_obs_density": (c_int, [c_void_p, P(c_double), P(c_double)]),
    "ed_obs_density_density": (c_int, [c_void_p, P(c_double), P(c_double)]),
    "ed_obs_participation_ratio": (c_int, [c_void_p, P(c_double), P(c_double)]),
    "ed_obs_most_probable": (c_int, [c_void_p, P(c_double), c_i64, P(c_u64), P(c_double), P(c_i64)]),
    "ed_crs_arrays": (c_int, [c_void_p, P(c_void_p), P(c_void_p), P(c_void_p)]),
    "ed_crs_get": (c_int, [c_void_p, P(c_i64), P(ctypes.c_int32), P(c_double)]),
    "ed_ham_diagonal": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ed_spmv": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ed_spmv_kernel": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "ed_fp64_fma_rate": (c_int, [c_int, c_int, P(c_double)]),
    "ed_crs_set_product_kernel": (c_int, [c_void_p, c_int]),
    "ed_spmv_staged_wait_test": (c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_longlong, ctypes.POINTER(c_int)]),
    "ed_hv_matfree": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "ed_op_from_crs": (c_int, [c_void_p, P(c_void_p)]),
    "ed_op_matfree": (c_int, [c_void_p, c_void_p, P(c_void_p)]),
    "ed_op_host_callback": (c_int, [c_i64, HOST_MATVEC, c_void_p, P(c_void_p)]),
    "ed_op_free": (c_int, [c_void_p]),
    "ed_op_dim": (c_int, [c_void_p, P(c_i64)]),
    "ed_lanczos": (c_int, [c_void_p, P(LanczosParams), P(c_double), P(c_double), P(c_double), P(SolveInfo)]),
    "ed_lanczos_two_level": (c_int, [c_void_p, c_void_p, P(LanczosParams), P(c_double), P(c_double), P(c_double),
                                     P(SolveInfo)]),
    "ed_lanczos_device": (c_int, [c_void_p, P(LanczosParams), c_void_p, P(c_double), c_void_p, P(SolveInfo)]),
    "ed_residuals": (c_int, [c_void_p, c_void_p, P(c_double), c_int, P(c_double)]),
    "ed_residuals_noalloc": (c_int, [c_void_p, c_void_p, P(c_double), c_int, P(c_double)]),
    "ed_basis_rotate": (c_int, [c_void_p, c_i64, c_int, P(c_double), c_int, c_int, c_void_p, c_int]),
    "ed_eigensystem_write": (c_int, [ctypes.c_char_p, c_int, c_int, P(c_double), ctypes.c_uint64, P(c_double)]),
    "ed_eigensystem_read": (c_int, [ctypes.c_char_p, c_int, P(c_int), P(c_double), P(ctypes.c_uint64),
                                    P(c_double)]),
    "ed_crs_write": (c_int, [c_void_p, ctypes.c_char_p, c_int]),
    "ed_crs_read": (c_int, [ctypes.c_char_p, c_int, c_int, P(c_void_p)]),
    "ed_quartic_tables_write": (c_int, [ctypes.c_char_p, c_int, c_int, P(ctypes.c_uint16), P(c_double)]),
    "ed_quartic_tables_read": (c_int, [ctypes.c_char_p, c_int, P(c_int), P(ctypes.c_uint16), P(c_double)]),
    "ed_kernel_launches": (c_u64, []),
    "ed_dense_sym_eigen": (c_int, [c_int, P(c_double), P(c_double), P(c_double)]),
    "ed_solve_sector": (c_int, [c_int, c_int, c_int, P(c_double), c_int, c_int, P(LanczosParams), P(c_double),
                                P(c_double), P(c_double), P(SolveInfo)]),
    "ed_batch_create": (c_int, [c_void_p, c_int, P(ctypes.c_uint16), P(c_double), c_int, P(c_void_p)]),
    "ed_batch_free": (c_int, [c_void_p]),
    "ed_batch_dims": (c_int, [c_void_p, P(c_i64), P(c_i64), P(c_int)]),
    "ed_batch_spmm": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ed_batch_solve": (c_int, [c_void_p, P(LanczosParams), c_void_p, P(c_double), c_void_p, P(BatchInfo)]),
    "ed_batch_solve_subset": (c_int, [c_void_p, P(c_int), c_int, P(LanczosParams), c_void_p, P(c_double), c_void_p,
                                      P(BatchInfo)]),
    "ed_sym_eigen_batched": (c_int, [c_int, c_int, P(c_double), P(c_double), P(c_double)]),
    "ed_subspace_create": (c_int, [c_i64, c_int, P(c_void_p)]),
    "ed_subspace_free": (c_int, [c_void_p]),
    "ed_subspace_dim": (c_int, [c_void_p, P(c_int)]),
    "ed_subspace_add": (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, P(c_int)]),
    "ed_batch_subspace_ritz": (c_int, [c_void_p, c_void_p, c_int, c_int, P(c_double), c_void_p, P(c_double)]),
    "ed_mlp_create": (c_int, [c_int, c_int, c_u64, P(c_void_p)]),
    "ed_mlp_free": (c_int, [c_void_p]),
    "ed_mlp_num_params": (c_int, [c_void_p, P(c_i64)]),
    "ed_mlp_get_params": (c_int, [c_void_p, P(ctypes.c_float), c_i64]),
    "ed_mlp_set_params": (c_int, [c_void_p, P(ctypes.c_float), c_i64]),
    "ed_mlp_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
    "ed_mlp_gradients": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_i64, P(ctypes.c_float), P(c_double)]),
    "ed_mlp_train_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_i64, ctypes.c_float, P(c_double)]),
    "ed_mlp_fit": (c_int, [c_void_p, c_void_p, P(c_double), c_int, c_void_p, c_int, c_int, ctypes.c_float, c_u64,
                           P(c_double)]),
    "ed_warm_start": (c_int, [c_void_p, c_void_p, P(c_double), c_int, c_void_p]),
}

_LIB = None


def lib():
    """Load libedgb300.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run `python -m hamiltonian_diagonalization_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(status: int):
    if status != ED_OK:
        msg = lib().ed_last_error().decode(errors="replace")
        raise EDError(status, msg)


def declared_symbols(header: str) -> list[str]:
    """Function names declared in an ed_capi.h-style header."""
    import re
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ed_[a-z0-9_]+)\s*\(", text)) - {"ed_host_matvec"})
