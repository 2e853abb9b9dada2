"""The C ABI library loads without a GPU, exports every symbol the header
declares, and rejects bad arguments on the host before any device work."""
import ctypes
import os

import pytest

from hamiltonian_diagonalization_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def test_exports_every_declared_symbol(edlib):
    declared = []
    for h in HEADERS:
        declared += _capi.declared_symbols(h)
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(edlib, s)]
    assert missing == []


def test_status_strings(edlib):
    for code in range(0, 9):
        assert edlib.ed_status_string(code)
    assert edlib.ed_version() >= 1
    assert edlib.ed_device_count() >= 0


def test_bad_arguments_rejected_on_host(edlib):
    h = ctypes.c_void_p()
    assert edlib.ed_basis_build(5, 4, 0, None, ctypes.byref(h)) == _capi.ED_ERR_ARG       # N > norb
    assert b"N <= norb" in edlib.ed_last_error()
    assert edlib.ed_basis_build(3, 41, 0, None, ctypes.byref(h)) == _capi.ED_ERR_RANGE    # beyond 40 orbitals
    assert edlib.ed_basis_build(3, 8, 0, None, None) == _capi.ED_ERR_ARG
    assert edlib.ed_spmv(None, None, None, None) == _capi.ED_ERR_ARG
    assert edlib.ed_terms_set(1, None, None, ctypes.byref(h)) == _capi.ED_ERR_ARG
    assert edlib.ed_lanczos(None, None, None, None, None, None) == _capi.ED_ERR_ARG
    assert edlib.ed_coulomb_pseudopotentials(1, None) == _capi.ED_ERR_ARG
    # free functions accept NULL like free()
    assert edlib.ed_basis_free(None) == 0 and edlib.ed_crs_free(None) == 0 and edlib.ed_op_free(None) == 0


def test_no_device_path_fails_loudly_without_gpu(edlib):
    if edlib.ed_device_count() > 0:
        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    st = edlib.ed_basis_build(4, 10, 0, None, ctypes.byref(h))
    assert st in (_capi.ED_ERR_CUDA, _capi.ED_ERR_OOM)
    assert h.value is None
