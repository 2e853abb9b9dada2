"""Micro-benchmark of the Hamiltonian-vector products on one GPU.

    python -m hamiltonian_diagonalization_gb300.microbench --sector 11,31,0 --reps 20 [--upper] [--matfree]
    python -m hamiltonian_diagonalization_gb300.microbench --sector 10,28,0 --batch 32 --reps 20
    python -m hamiltonian_diagonalization_gb300.microbench --rotate 1371535,41,25 --reps 20
    python -m hamiltonian_diagonalization_gb300.microbench --sector 11,31,0 --build --reps 3 [--upper]
    python -m hamiltonian_diagonalization_gb300.microbench --sector 11,31,0 --observables --reps 5

Builds the sector's Hamiltonian (LLL Coulomb pseudopotentials, odd m) on the
device, then times `reps` products with CUDA events on the launching stream
and prints one JSON line: dimension, stored nonzeros, ms per product,
algorithmic bytes per product (nnz*(8+4) + (n+1)*8 + 2*n*8 for stored CRS)
and the implied GB/s.  Used for the SpMV roofline and its ncu profiles.
With --batch B it times the block product of B Hamiltonians of the sector
(the V1 sweep's shared pattern, ed_batch_spmm) instead and reports FP64 FMAs
per second (one FMA per stored element per Hamiltonian, diagonal included).
With --rotate n,m,k it times the thick-restart rotation of an n x m basis
into k Ritz vectors (ed_basis_rotate) in FP64 and on the tensor cores.
With --build it times the whole CRS build (diagonal, count, scan, fill;
host clock around a synchronised call, best of reps) with the register-sort
fill and with the shared-memory fill (ED_FILL_SORT=smem).  With
--observables it times the eigenvector observables (density, density-density,
participation ratio, 100 most probable states) end to end from a host vector.
With --two-level the sector is N,norb0,twoLz of the two-Landau-level model
(norb0 lowest-level orbitals, norb0 + 2 in the second level, odd-m Coulomb
pseudopotential lists of those sizes for the two levels' tables, second-level
occupation energy 1.0): it times the basis, the CRS build, the product and
the --nev lowest eigenpairs from one Krylov sequence, with the degeneracy
passes and with the level-exchange ladder (with
--build, the basis and the CRS build only).  With --ofl N,dimX,dimY,kxTot,kyTot
it does the same for a complex optical-flux-lattice momentum sector built from
seeded synthetic tables (synthetic_ofl_tables) and occupation energies
linspace(-0.5, 0.5).
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sector", default="11,31,0", help="N,norb,twoLz")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--upper", action="store_true", help="store the upper triangle (the reference's layout)")
    ap.add_argument("--matfree", action="store_true", help="regenerate elements on the fly")
    ap.add_argument("--batch", type=int, default=0, help="time the block product of this many Hamiltonians")
    ap.add_argument("--no-autotune", action="store_true", help="batch: keep the default tile (32 per row, L1)")
    ap.add_argument("--rotate", default="", help="n,m,k: time the restart rotation instead")
    ap.add_argument("--build", action="store_true",
                    help="time the CRS build instead (register sort, then ED_FILL_SORT=smem)")
    ap.add_argument("--observables", action="store_true",
                    help="time the eigenvector observables on a seeded unit vector of the sector")
    ap.add_argument("--two-level", action="store_true", help="two-Landau-level sector N,norb0,twoLz")
    ap.add_argument("--ofl", default="", help="N,dimX,dimY,kxTot,kyTot: complex optical-flux-lattice sector")
    ap.add_argument("--nev", type=int, default=4, help="two-level: eigenpairs to solve for")
    ap.add_argument("--products-only", action="store_true", help="two-level / complex: stop after the products")
    ap.add_argument("--kernel", type=int, default=0,
                    help="full-storage product kernel (ed_spmv_kernel): 0 by shape, 1 row lanes, "
                         "2-3 shared-reduction rows, 4-5 sliced ELL, 6 fixed-point integer rows, 7 the same "
                         "with bulk-copy staging, 8 fixed-point sliced ELL")
    ap.add_argument("--fp64-rate", action="store_true", help="measure the FP64 FMA issue rate instead")
    args = ap.parse_args()
    import torch

    import hamiltonian_diagonalization_gb300 as ed
    from hamiltonian_diagonalization_gb300 import _capi as C

    if args.fp64_rate:
        out = {"mode": "fp64_fma_rate"}
        for bps in (2, 4, 8):
            r = ctypes.c_double()
            C.check(C.lib().ed_fp64_fma_rate(20000, bps, ctypes.byref(r)))
            out[f"fma_per_s_{bps}_blocks_per_sm"] = r.value
        print(json.dumps(out))
        return
    if args.rotate:
        return rotate_main(C, torch, args)
    if args.ofl:
        return ofl_main(ed, torch, args)
    N, norb, tlz = (int(x) for x in args.sector.split(","))
    if args.batch:
        return batch_main(ed, C, torch, N, norb, tlz, args)
    if args.two_level:
        return two_level_main(ed, C, torch, N, norb, tlz, args)
    if args.build:
        return build_main(ed, torch, N, norb, tlz, args)
    if args.observables:
        return observables_main(ed, N, norb, tlz, args)
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=tlz)
    T = ed.QuarticTermTables(norb, ed.odd_coulomb_list(norb))
    H.Add_CdCdCC_Terms(T, store_upper=args.upper, matrix_free=args.matfree)
    n = H.GetDimension()
    mv = ed.MatrixVectorFunction(H)
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, n)).cuda()
    y = torch.empty_like(x)
    if args.kernel:
        crs = H.m_crsSparseMatrix
        product = lambda: crs.multiply(x, y, args.kernel)   # noqa: E731
    else:
        product = lambda: mv.Simple(x, y)   # noqa: E731
    import time
    torch.cuda.synchronize()
    t_first = time.perf_counter()
    product()                      # the first product also makes the sliced-ELL copy
    torch.cuda.synchronize()
    ms_first = 1e3 * (time.perf_counter() - t_first)
    for _ in range(args.warmup):
        product()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = C.lib().ed_kernel_launches()
    a.record()
    for _ in range(args.reps):
        product()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.reps
    out = {"sector": [N, norb, tlz], "n": n, "mode": "matfree" if args.matfree else ("upper" if args.upper else "full"),
           "kernel": args.kernel, "ms_per_product": ms, "ms_first_product": ms_first,
           "launches": int(C.lib().ed_kernel_launches() - launches0)}
    if not args.matfree:
        nnz = H.m_crsSparseMatrix.GetNbrNonZeros()
        by = nnz * 12 + (n + 1) * 8 + 2 * n * 8
        out.update({"nnz": nnz, "bytes_per_product": by, "GBps": by / ms / 1e6})
    print(json.dumps(out))


def build_main(ed, torch, N, norb, tlz, args):
    import os
    import time
    T = ed.QuarticTermTables(norb, ed.odd_coulomb_list(norb))
    res = {"sector": [N, norb, tlz], "mode": "build", "layout": "upper" if args.upper else "full"}
    for name, env in (("register", None), ("smem", "smem")):
        if env:
            os.environ["ED_FILL_SORT"] = env
        else:
            os.environ.pop("ED_FILL_SORT", None)
        times = []
        for i in range(args.warmup + args.reps):
            H = ed.SpinlessFermionHamiltonian()
            H.Initialize(N, norb, twoLz=tlz)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            H.Add_CdCdCC_Terms(T, store_upper=args.upper)
            torch.cuda.synchronize()
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
            res["n"], res["nnz"] = H.GetDimension(), H.m_crsSparseMatrix.GetNbrNonZeros()
            del H
        res[f"ms_build_{name}"] = 1e3 * min(times)
    os.environ.pop("ED_FILL_SORT", None)
    print(json.dumps(res))


def two_level_main(ed, C, torch, N, norb0, tlz, args):
    import time
    res = {"sector": [N, norb0, tlz], "mode": "two-level", "layout": "upper" if args.upper else "full"}
    t0 = ed.QuarticTermTables(norb0, ed.odd_coulomb_list(norb0))
    t1 = ed.QuarticTermTables(norb0 + 2, ed.odd_coulomb_list(norb0 + 2))
    e1 = np.ones(norb0 + 2)

    def make():
        H = ed.TwoLevelSpinlessFermionHamiltonian()
        H.Initialize(N, 2 * norb0 + 2)
        torch.cuda.synchronize()
        a = time.perf_counter()
        H.m_fockBasis.GenerateFockSpace(N, norb0, norb0 + 2, tlz)
        torch.cuda.synchronize()
        b = time.perf_counter()
        H.Add_CdC_Terms(e1, 1, 1)
        H.Add_CdCdCC_Terms(t0, 0, 0, 0, 0, store_upper=args.upper)
        H.Add_CdCdCC_Terms(t1, 1, 1, 1, 1, store_upper=args.upper)
        H.Build()
        torch.cuda.synchronize()
        return H, b - a, time.perf_counter() - b

    tb, tc = [], []
    for i in range(args.warmup + args.reps):
        H, x, y = make()
        if i >= args.warmup:
            tb.append(x)
            tc.append(y)
    n, nnz = H.GetDimension(), H.m_crsSparseMatrix.GetNbrNonZeros()
    res.update({"n": n, "nnz": nnz, "ms_basis": 1e3 * min(tb), "ms_build": 1e3 * min(tc)})
    if args.build:                      # basis and CRS build only
        print(json.dumps(res))
        return
    mv = ed.MatrixVectorFunction(H)
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, n)).cuda()
    y = torch.empty_like(x)
    if args.kernel:
        crs = H.m_crsSparseMatrix
        crs.set_product_kernel(args.kernel)      # the solves below use it too
        product = lambda: crs.multiply(x, y, args.kernel)   # noqa: E731
    else:
        product = lambda: mv.Simple(x, y)   # noqa: E731
    for _ in range(3):
        product()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(20):
        product()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / 20
    by = nnz * 12 + (n + 1) * 8 + 2 * n * 8
    res.update({"kernel": args.kernel, "ms_per_product": ms, "GBps": by / ms / 1e6})
    if args.products_only:
        print(json.dumps(res))
        return
    for name, passes in (("single", 0), ("passes", args.nev), ("ladder", None)):
        H.LanczosDiagonalize(args.nev, tol=1e-10, seed=1, degeneracy_passes=passes, want_vectors=False)
        t = time.perf_counter()
        ok = H.LanczosDiagonalize(args.nev, tol=1e-10, seed=1, degeneracy_passes=passes, want_vectors=False)
        res[f"solve_{name}"] = {"ok": bool(ok), "s": time.perf_counter() - t,
                                "eigenvalues": [float(v) for v in H.m_eigenvalues],
                                "matvecs": H.last_info["matvecs"], "max_residual": H.last_info["max_residual"]}
    print(json.dumps(res))


def ofl_main(ed, torch, args):
    import time
    N, X, Y, kx, ky = (int(v) for v in args.ofl.split(","))
    T = ed.synthetic_ofl_tables(X, Y, 1)
    e = np.linspace(-0.5, 0.5, X * Y)
    res = {"ofl": [N, X, Y, kx, ky], "mode": "complex", "layout": "upper" if args.upper else "full"}
    tb, tc = [], []
    for i in range(args.warmup + args.reps):
        model = ed.InteractingOflModel(N, X, Y, T, e, nbrEigenvalues=args.nev)
        model.SetSector(kx, ky)
        torch.cuda.synchronize()
        a = time.perf_counter()
        model.BuildFockBasis()
        torch.cuda.synchronize()
        b = time.perf_counter()
        model.BuildHamiltonian(store_upper=args.upper)
        torch.cuda.synchronize()
        if i >= args.warmup:
            tb.append(b - a)
            tc.append(time.perf_counter() - b)
    H = model.hamiltonian
    n, nnz = H.GetDimension(), H.m_crsSparseMatrix.GetNbrNonZeros()
    res.update({"n": n, "nnz": nnz, "ms_basis": 1e3 * min(tb), "ms_build": 1e3 * min(tc)})
    if args.build:
        print(json.dumps(res))
        return
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, 2 * n)).cuda()
    y = torch.empty_like(x)
    for _ in range(3):
        H.apply(x, y)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(20):
        H.apply(x, y)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / 20
    by = nnz * 20 + (n + 1) * 8 + 2 * n * 16
    res.update({"ms_per_product": ms, "GBps": by / ms / 1e6})
    if args.products_only:
        print(json.dumps(res))
        return
    model.Diagonalize(tol=1e-10, seed=1, want_vectors=False)
    t = time.perf_counter()
    ok = model.Diagonalize(tol=1e-10, seed=1, want_vectors=False)
    res["solve"] = {"ok": bool(ok), "s": time.perf_counter() - t, "eigenvalues": [float(v) for v in H.m_eigenvalues],
                    "matvecs": H.last_info["matvecs"], "restarts": H.last_info["restarts"],
                    "spmv_s": H.last_info["spmv_seconds"], "max_residual": H.last_info["max_residual"]}
    # what a step costs beyond its product (Gram-Schmidt, restarts, the host)
    res["solve"]["overhead_ms_per_step"] = 1e3 * (res["solve"]["s"] - H.last_info["spmv_seconds"]) / max(
        1, H.last_info["matvecs"])
    print(json.dumps(res))


def observables_main(ed, N, norb, tlz, args):
    import time
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    n = b.GetStoredDimension()
    psi = np.random.default_rng(3).standard_normal(n)
    psi /= np.linalg.norm(psi)
    O = ed.Observables
    calls = {"density": lambda: O.density_of_vector(b, psi),
             "density_density": lambda: O.density_density_of_vector(b, psi),
             "participation_ratio": lambda: O.participation_ratio_of_vector(b, psi),
             "most_probable_100": lambda: O.most_probable_of_vector(b, psi, 100)}
    res = {"sector": [N, norb, tlz], "n": n, "mode": "observables",
           "note": "host vector in, host results out (the H2D copy of psi included)"}
    for name, f in calls.items():
        for _ in range(args.warmup):
            f()
        t0 = time.perf_counter()
        for _ in range(args.reps):
            f()
        res[f"ms_{name}"] = 1e3 * (time.perf_counter() - t0) / args.reps
    print(json.dumps(res))


def batch_main(ed, C, torch, N, norb, tlz, args):
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    base = ed.odd_coulomb_list(norb)
    lists = []
    for v1 in np.linspace(0.5, 3.0, args.batch):
        v = base.copy()
        v[1] = v1
        lists.append(v)
    bt = ed.HamiltonianBatch(b, lists, autotune=not args.no_autotune)
    n, B = bt.n, bt.nham
    X = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, (n, B))).cuda()
    Y = torch.empty_like(X)
    for _ in range(args.warmup):
        bt.spmm(X, Y)
    torch.cuda.synchronize()
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.reps):
        bt.spmm(X, Y)
    e.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(e) / args.reps
    fma = (bt.nnz + n) * B
    print(json.dumps({"sector": [N, norb, tlz], "n": n, "mode": "batch", "hamiltonians": B, "nnz_offdiag": bt.nnz,
                      "ms_per_block_product": ms, "ms_per_hamiltonian_product": ms / B,
                      "fp64_fma_per_s": fma / ms * 1e3, "fp64_tflops": 2 * fma / ms / 1e9}))


def rotate_main(C, torch, args):
    n, m, k = (int(x) for x in args.rotate.split(","))
    V = torch.from_numpy(np.random.default_rng(1).standard_normal(n * m)).cuda()
    out = torch.empty(n * k, dtype=torch.float64, device="cuda")
    Y = np.asfortranarray(np.random.default_rng(2).standard_normal((m, m)))
    yp = Y.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    res = {"rotate": [n, m, k]}
    for method, name in ((1, "fp64"), (2, "tensor"), (3, "tensor_shared_digits")):
        def call():
            st = C.lib().ed_basis_rotate(ctypes.c_void_p(V.data_ptr()), n, m, yp, m, k,
                                         ctypes.c_void_p(out.data_ptr()), method)
            assert st == 0, C.lib().ed_last_error()
        for _ in range(args.warmup):
            call()
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.reps):
            call()
        e.record()
        torch.cuda.synchronize()
        res[f"ms_{name}"] = a.elapsed_time(e) / args.reps
    res["fp64_multiply_adds"] = n * m * k
    print(json.dumps(res))


if __name__ == "__main__":
    main()
