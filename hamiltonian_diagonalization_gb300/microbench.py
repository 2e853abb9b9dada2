"""Micro-benchmark of the Hamiltonian-vector products on one GPU.

    python -m hamiltonian_diagonalization_gb300.microbench --sector 11,31,0 --reps 20 [--upper] [--matfree]

Builds the sector's Hamiltonian (LLL Coulomb pseudopotentials, odd m) on the
device, then times `reps` products with CUDA events on the launching stream
and prints one JSON line: dimension, stored nonzeros, ms per product,
algorithmic bytes per product (nnz*(8+4) + (n+1)*8 + 2*n*8 for stored CRS)
and the implied GB/s.  Used for the SpMV roofline and its ncu profiles.
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
    args = ap.parse_args()
    import torch

    import hamiltonian_diagonalization_gb300 as ed
    from hamiltonian_diagonalization_gb300 import _capi as C

    N, norb, tlz = (int(x) for x in args.sector.split(","))
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=tlz)
    T = ed.QuarticTermTables(norb, ed.odd_coulomb_list(norb))
    H.Add_CdCdCC_Terms(T, store_upper=args.upper, matrix_free=args.matfree)
    n = H.GetDimension()
    mv = ed.MatrixVectorFunction(H)
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, n)).cuda()
    y = torch.empty_like(x)
    for _ in range(args.warmup):
        mv.Simple(x, y)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = C.lib().ed_kernel_launches()
    a.record()
    for _ in range(args.reps):
        mv.Simple(x, y)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.reps
    out = {"sector": [N, norb, tlz], "n": n, "mode": "matfree" if args.matfree else ("upper" if args.upper else "full"),
           "ms_per_product": ms, "launches": int(C.lib().ed_kernel_launches() - launches0)}
    if not args.matfree:
        nnz = H.m_crsSparseMatrix.GetNbrNonZeros()
        by = nnz * 12 + (n + 1) * 8 + 2 * n * 8
        out.update({"nnz": nnz, "bytes_per_product": by, "GBps": by / ms / 1e6})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
