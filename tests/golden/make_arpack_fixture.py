"""Reference-family eigenpairs of the stored-CRS configuration, on the CPU.

Builds the N=11, 2S=30, Lz=0 Hamiltonian (1,371,535 states, LLL Coulomb odd
m) with the CPU oracle (the restated Add_CdCdCC_Terms), then runs ARPACK's
non-symmetric driver (SciPy's bundled ARPACK, the library the reference calls
as pdnaupd_/pdneupd_) with the reference's settings: which='SR', ncv =
2*nev+21, maxiter 2000, from the seed-42 uniform(-1,1) start vector, with the
reference's upper-triangle product loop as the operator.  Writes
tests/golden/arpack_n11_2s30_lz0.json: the 10 lowest eigenvalues, the number
of products ARPACK needed and the wall times of each phase on this host.

    python tests/golden/make_arpack_fixture.py        # ~2-4 minutes on 16 cores
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

N, NORB, TWO_LZ, NEV, SEED, TOL = 11, 31, 0, 10, 42, 1e-12


def main():
    import scipy.sparse.linalg as sla
    threads = O.num_procs()
    t0 = time.perf_counter()
    b = O.basis(N, NORB, TWO_LZ, threads)
    t_basis = time.perf_counter() - t0
    pp = O.odd_coulomb_list(NORB)
    kt, vt = O.quartic_tables(NORB, pp)
    t0 = time.perf_counter()
    rp, col, val = O.build_upper(b, NORB, kt, vt, threads)
    t_build = time.perf_counter() - t0
    n = len(b)
    count = [0]

    def mv(x):
        count[0] += 1
        return O.spmv_sym_upper(rp, col, val, np.ascontiguousarray(x, dtype=np.float64), threads)

    op = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    v0 = O.start_vector(n, SEED)
    t0 = time.perf_counter()
    w, v = sla.eigs(op, k=NEV, which="SR", tol=TOL, v0=v0, ncv=2 * NEV + 21, maxiter=2000)
    t_arpack = time.perf_counter() - t0
    # true residuals of the returned pairs (Rayleigh quotient of each vector)
    res = []
    for i in range(NEV):
        x = v[:, i].real
        x = x / np.linalg.norm(x)
        hx = O.spmv_sym_upper(rp, col, val, x, threads)
        res.append(float(np.linalg.norm(hx - (x @ hx) * x)))
    w = np.sort(w.real)
    out = {"N": N, "norb": NORB, "two_lz": TWO_LZ, "n": n, "nnz_upper": int(rp[-1]), "nev": NEV,
           "ncv": 2 * NEV + 21, "tol": TOL, "seed": SEED, "which": "SR", "driver": "scipy ARPACK eigs (dnaupd/dneupd)",
           "eigenvalues": [float(x) for x in w], "matvecs": count[0], "threads": threads,
           "seconds": {"basis": t_basis, "build": t_build, "arpack": t_arpack}, "max_residual": max(res)}
    with open(os.path.join(HERE, "arpack_n11_2s30_lz0.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
