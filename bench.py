"""Time-to-eigenpairs benchmark on one GB300 (or N independent replicas).

Workload: the stored-CRS configuration, N=11 electrons at flux 2S=30 (31
orbitals) in the Lz=0 sector (1,371,535 states), LLL Coulomb pseudopotentials
(odd m <= 2S-1), lowest 10 eigenpairs to residual ||Hx - lambda x|| <= 1e-10
from the seed-42 uniform(-1,1) start vector.  One step = one whole solve:
device basis -> term tables -> CRS build -> Lanczos with full FP64
reorthogonalisation -> verified residuals.

  value  device-resident solve (start vector already in HBM, eigenvectors
         left in HBM), seconds per solve, CUDA events on the launching stream
  e2e    the one-call public API ed_solve_sector from host buffers: start
         vector in, eigenvalues and eigenvectors out, copies inside the timing
  roofline  the stored-CRS SpMV, algorithmic bytes per product
         nnz*(8+4) + (n+1)*8 + 2*n*8 over its average in-solve duration
  cpu_baseline  the CPU oracle (a restatement of the reference's algorithm)
         on the host cores, measured on bounded samples and scaled

`--impl reference` times the same CPU restatement as the reference arm.
The inputs (4.2 GB of CRS per product) are larger than the 129 MB L2.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PART, NORB, TWO_LZ, NEV, TOL, SEED = 11, 31, 0, 10, 1e-10, 42
METRIC = "time-to-eigenpairs @1e-10 residual (N=11, 2S=30, Lz=0, 10 lowest)"
WORKLOAD = "stored-CRS LLL Coulomb sphere N=11 2S=30 Lz=0 (1,371,535 states), 10 lowest eigenpairs"


def start_vector(n: int, seed: int) -> np.ndarray:
    v = np.random.default_rng(seed).uniform(-1.0, 1.0, n)
    return v / np.linalg.norm(v)


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """The slowest replica's value (the step time the job is charged)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, path: str):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self, device_index: int = 0):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9 or p[0] != str(device_index):
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU oracle leg

class CpuLeg:
    """The CPU restatement of the reference path (oracle port) on all host
    threads, measured on bounded samples of the solve.

    Set-up (untimed): the full upper-triangle CRS built once by the oracle.
    Each sample measures the full sector scan (basis), the quartic build of
    one eighth of the rows (scaled by rows), and two products of the
    reference's upper-triangle SpMV loop over the whole matrix (rows split
    over threads like its MPI ranks).  Estimate = basis + build + products x
    the product count ARPACK needed for this problem with the reference's
    settings (recorded in tests/golden/arpack_n11_2s30_lz0.json).  ARPACK's
    own dense work is not counted, so the estimate favours the CPU."""

    def __init__(self):
        from oracle import oracle as O
        self.O = O
        self.threads = O.num_procs()
        self.kt, self.vt = O.quartic_tables(NORB, O.odd_coulomb_list(NORB))
        self.b = O.basis(N_PART, NORB, TWO_LZ, self.threads)
        t0 = time.perf_counter()
        self.rp, self.col, self.val = O.build_upper(self.b, NORB, self.kt, self.vt, self.threads)
        self.t_build_full = time.perf_counter() - t0
        self.n = len(self.b)
        self.x = np.random.default_rng(1).uniform(-1, 1, self.n)
        fx = os.path.join(ROOT, "tests", "golden", "arpack_n11_2s30_lz0.json")
        self.matvecs = json.load(open(fx))["matvecs"] if os.path.exists(fx) else None
        self.arpack_fixture = json.load(open(fx)) if os.path.exists(fx) else None

    def sample(self):
        O = self.O
        t0 = time.perf_counter()
        O.basis(N_PART, NORB, TWO_LZ, self.threads)
        t_basis = time.perf_counter() - t0
        rows = self.n // 8
        r0 = (self.n - rows) // 2
        t0 = time.perf_counter()
        O.build_upper(self.b, NORB, self.kt, self.vt, self.threads, rows=(r0, r0 + rows))
        t_build = (time.perf_counter() - t0) * self.n / rows
        O.spmv_sym_upper(self.rp, self.col, self.val, self.x, self.threads)
        t0 = time.perf_counter()
        for _ in range(2):
            O.spmv_sym_upper(self.rp, self.col, self.val, self.x, self.threads)
        t_prod = (time.perf_counter() - t0) / 2
        return {"t_basis": t_basis, "t_build": t_build, "t_prod": t_prod}

    def estimate(self, s, matvecs):
        return s["t_basis"] + s["t_build"] + matvecs * s["t_prod"]

    def describe(self, s, matvecs):
        return (f"oracle port on {self.threads} threads: full basis scan {s['t_basis']:.2f}s; quartic build of "
                f"n/8 rows scaled to {s['t_build']:.1f}s (full build measured once: {self.t_build_full:.1f}s); "
                f"reference upper-triangle SpMV {s['t_prod']:.3f}s/product over the whole matrix x {matvecs} "
                f"products (ARPACK's count for this problem); ARPACK dense work not counted")


# ------------------------------------------------------------- device leg

def run_gpu(args, ws, rank):
    import torch
    import hamiltonian_diagonalization_gb300 as ed
    from hamiltonian_diagonalization_gb300 import _capi as C

    L = ed.lib()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    pp = ed.odd_coulomb_list(NORB)
    # term tables on the host once (inputs); the device build consumes them
    K = NORB
    kt = np.empty(K ** 3, dtype=np.uint16)
    vt = np.empty(K ** 3)
    C.check(L.ed_quartic_tables(K, pp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(pp),
                                kt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                vt.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    probe = ed.FermionFockBasis()
    probe.GenerateFockSpace(N_PART, NORB, TWO_LZ)
    n = probe.GetStoredDimension()
    probe.free()
    v0h = start_vector(n, SEED)
    v0d = torch.from_numpy(v0h).cuda()
    evecs_d = torch.empty(n * NEV, dtype=torch.float64, device="cuda")
    params = C.LanczosParams(nev=NEV, ncv=args.ncv, max_restarts=0, tol=TOL, seed=SEED, want_vectors=1, verify=1)

    phases = []

    def solve_device():
        t0 = time.perf_counter()
        bh = ctypes.c_void_p()
        C.check(L.ed_basis_build(N_PART, NORB, TWO_LZ, None, ctypes.byref(bh)))
        t1 = time.perf_counter()
        th = ctypes.c_void_p()
        C.check(L.ed_terms_set(K, kt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                               vt.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(th)))
        t2 = time.perf_counter()
        ah = ctypes.c_void_p()
        C.check(L.ed_ham_build_crs(bh, th, 0, None, ctypes.byref(ah)))
        t3 = time.perf_counter()
        oh = ctypes.c_void_p()
        C.check(L.ed_op_from_crs(ah, ctypes.byref(oh)))
        ev = np.empty(NEV)
        info = C.SolveInfo()
        st = L.ed_lanczos_device(oh, ctypes.byref(params), ctypes.c_void_p(v0d.data_ptr()),
                                 ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 ctypes.c_void_p(evecs_d.data_ptr()), ctypes.byref(info))
        t4 = time.perf_counter()
        nnz = ctypes.c_int64()
        L.ed_crs_info(ah, None, ctypes.byref(nnz), None)
        for f, h in ((L.ed_op_free, oh), (L.ed_crs_free, ah), (L.ed_terms_free, th), (L.ed_basis_free, bh)):
            f(h)
        t5 = time.perf_counter()
        phases.append({"basis": t1 - t0, "terms": t2 - t1, "crs_build": t3 - t2, "lanczos": t4 - t3, "free": t5 - t4})
        C.check(st)
        return ev, info, int(nnz.value)

    def solve_e2e():
        ev = np.empty(NEV)
        vec = np.empty(n * NEV)
        info = C.SolveInfo()
        C.check(L.ed_solve_sector(N_PART, NORB, TWO_LZ, pp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(pp),
                                  0, ctypes.byref(params), v0h.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(info)))
        return ev, info

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        solve_device()
    torch.cuda.synchronize()
    launches0 = L.ed_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    infos = []
    with ClockSampler(os.path.join(args.clock_log_dir, f"clocks_rank{rank}.csv")) as clk:
        barrier()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            ev, info, nnz = solve_device()
            infos.append(info.as_dict())
        e1.record()
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = L.ed_kernel_launches() - launches0
    clocks = clk.summary(dev)
    # end-to-end through the one-call API from host buffers
    solve_e2e()
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(max(1, min(args.steps, 3))):
        a, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ev_e2e, info_e2e = solve_e2e()
        b2.record()
        torch.cuda.synchronize()
        e2e_times.append(a.elapsed_time(b2) / 1000.0)
    # standalone SpMV timing on the same CRS for the roofline cross-check
    spmv_ms_alone = spmv_alone(L, C, kt, vt, n, torch)
    if ws > 1:
        ms = max_over_ranks(ms, "cuda")
    return {"ms": ms, "infos": infos, "ev": ev, "nnz": nnz, "n": n, "launches": launches, "clocks": clocks,
            "e2e_s": statistics.median(e2e_times), "ev_e2e": ev_e2e, "spmv_ms_alone": spmv_ms_alone,
            "phases": phases[-args.steps:]}


def spmv_alone(L, C, kt, vt, n, torch, reps: int = 20):
    bh, th, ah = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    C.check(L.ed_basis_build(N_PART, NORB, TWO_LZ, None, ctypes.byref(bh)))
    C.check(L.ed_terms_set(NORB, kt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                           vt.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(th)))
    C.check(L.ed_ham_build_crs(bh, th, 0, None, ctypes.byref(ah)))
    x = torch.rand(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    for _ in range(3):
        C.check(L.ed_spmv(ah, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), None))
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        C.check(L.ed_spmv(ah, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), None))
    b.record()
    torch.cuda.synchronize()
    for f, h in ((L.ed_crs_free, ah), (L.ed_terms_free, th), (L.ed_basis_free, bh)):
        f(h)
    return a.elapsed_time(b) / reps


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "spmv_traffic.txt")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncv", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--clock-log-dir", default="/tmp",
                    help="directory for the raw nvidia-smi clock samples of the timed region")
    args = ap.parse_args()
    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend)

    config = {"workload": WORKLOAD, "n_states": 1371535, "nev": NEV, "tol": TOL, "start": "seed-42 uniform(-1,1)",
              "storage": "full CRS (int64 rowptr, int32 col, f64 val)",
              "l2": "inputs larger than L2 (4.2 GB CRS streamed per product)", "replicas": ws}

    if args.impl == "reference":
        if rank != 0:
            return
        leg = CpuLeg()
        matvecs = leg.matvecs or 334
        samples = []
        for i in range(args.warmup + args.steps):
            s = leg.sample()
            if i >= args.warmup:
                samples.append(s)
        ests = [leg.estimate(s, matvecs) for s in samples]
        v = statistics.median(ests)
        line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": v * 1000.0, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (parameters only)", "config": config,
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "s", "cores": leg.threads, "kind": "port",
                                 "sample": leg.describe(samples[-1], matvecs)},
                "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if leg.arpack_fixture:
            fx = leg.arpack_fixture
            line["arpack_recorded"] = {"seconds": fx["seconds"], "matvecs": fx["matvecs"], "threads": fx["threads"],
                                       "note": "one full CPU solve (oracle build + SciPy ARPACK), "
                                               "tests/golden/make_arpack_fixture.py"}
        print(json.dumps(line))
        return

    r = run_gpu(args, ws, rank)
    if rank != 0:
        return
    infos = r["infos"]
    n, nnz = r["n"], r["nnz"]
    timed_products = [i["matvecs"] - NEV for i in infos]      # verify products are outside spmv_seconds
    spmv_s = statistics.median([i["spmv_seconds"] / max(1, tp) for i, tp in zip(infos, timed_products)])
    bytes_per = nnz * 12 + (n + 1) * 8 + 2 * n * 8
    peak, peak_kind = load_peaks()
    achieved = bytes_per / spmv_s / 1e9
    traffic = load_traffic()
    line = {"metric": METRIC, "value": r["ms"] / 1000.0 / ws, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (parameters only)", "config": config,
            "eigenvalues": [float(x) for x in r["ev"]],
            "solve": {"matvecs": infos[-1]["matvecs"], "restarts": infos[-1]["restarts"],
                      "max_residual": infos[-1]["max_residual"], "converged": infos[-1]["converged"],
                      "spmv_share": statistics.median(i["spmv_seconds"] for i in infos) / (r["ms"] / 1000.0),
                      "nnz_full": nnz},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": (traffic or {}).get("bytes_per_launch"),
                         "kernel": "k_spmv_full<8,4>", "bytes_per_launch": bytes_per,
                         "avg_launch_ms": spmv_s * 1000.0, "standalone_launch_ms": r["spmv_ms_alone"],
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "e2e": {"value": r["e2e_s"], "unit": "s", "h2d_bytes_per_step": n * 8 + NORB * 8,
                    "d2h_bytes_per_step": n * NEV * 8 + NEV * 8},
            "gpu_launches": int(r["launches"]),
            "phases_s": {k: statistics.median(p[k] for p in r["phases"]) for k in r["phases"][0]},
            "clocks": r["clocks"]}
    if not args.no_cpu and ws == 1:
        try:
            leg = CpuLeg()
            matvecs = leg.matvecs or int(infos[-1]["matvecs"])
            s = leg.sample()
            v = leg.estimate(s, matvecs)
            line["cpu_baseline"] = {"value": v, "unit": "s", "cores": leg.threads, "kind": "port",
                                    "sample": leg.describe(s, matvecs)}
        except Exception as e:  # the CPU leg must not hide the device result
            line["cpu_baseline"] = {"value": None, "unit": "s", "cores": None, "kind": "port",
                                    "sample": f"failed: {e}"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
