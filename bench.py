"""Benchmark: seconds to 10 interior eigenpairs of the 3-D Anderson model.

Workload: Anderson model on an m^3 periodic lattice (hopping -1, diagonal
i.i.d. uniform in [-8.25, 8.25] from a seeded splitmix64 stream; the named
configuration is m = 100, n = 1e6; ``--size`` sets m and the default is the
largest lattice whose whole run finishes within minutes),
10 eigenpairs closest to sigma = 0, residual tolerance 1e-10, float64
Jacobi-Davidson with the multilevel ILDL preconditioner stored and applied in
float32 (ICNTL(5)=1).  Synthetic data generated in-process.

A step is one complete solve (DPJD with NINIT=0) to 10 converged eigenpairs.
The preconditioner is factored once on the host before the timed region
(reported as ``factor_s``) and reused with ICNTL(2) = -1, the reference's
static-reuse mode; every timed step runs the whole eigensolve.

``value``: seconds per solve with the matrix resident in HBM (CUDA events on
the solver stream).  ``e2e``: the same through the Fortran-style C ABI
(dpjd_) with host arrays: matrix upload, solve and eigenvector download.
``roofline``: the preconditioner application (the dominant kernels).
``cpu_baseline``: the CPU oracle (a restatement of the reference's algorithm)
solving the same matrix with the same factor on one host core: a complete
solve when it fits the sample budget, else a capped number of MATVECs scaled
by the GPU solve's MATVEC count.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                       [--workload anderson|laplace|tightbinding|fem|batch]
Multi-GPU runs of the single-matrix workloads are independent replicas (the
path does not shard); the batch workload splits its problems over the ranks.
Rank 0 prints the line.  ``--impl reference`` runs the CPU oracle on the same
workload (the batch: a sampled subset in a process pool, scaled).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s to 10 eigpairs at resid 1e-10 (3D Anderson, sigma=0, FP32 factor / FP64 outer)"
DEFAULT_SIZE = 100


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=64, help="batch workload: number of problems (512 is the named case)")
    ap.add_argument("--workers", type=int, default=16, help="batch workload: host worker threads / CUDA streams")
    ap.add_argument("--workload", default="anderson", choices=["anderson", "laplace", "tightbinding", "fem", "batch"],
                    help="anderson: the headline 3-D Anderson model (default); laplace: 20^3 Dirichlet Laplacian, "
                         "plain float64; tightbinding: complex Hermitian 64^3 Peierls model, complex64 factor; "
                         "fem: P1-FEM K x = lambda M x, 512^2 nodes, float64; batch: --batch Anderson problems, "
                         "edges uniform in 16..40, 5 eigpairs closest to 0 each, float32 factor")
    ap.add_argument("--size", type=int, default=None,
                    help="lattice edge m (anderson: n = m^3, default %d, 100 is the named 1e6 case; laplace 20; "
                         "tightbinding 64; fem: nodes per side, 512)" % DEFAULT_SIZE)
    ap.add_argument("--droptol", type=float, default=1e-3,
                    help="ILDLC drop tolerance (1e-3 as the reference's Anderson sample)")
    ap.add_argument("--mem", type=float, default=20.0,
                    help="fill limit over nnz(A) (the sample's 15 fits ILUPACK's factor; this one needs 18.1 at 100^3)")
    ap.add_argument("--precision", type=int, default=None,
                    help="ICNTL(5): 0 fp64, 1 fp32, 2 bf16 factor (default: 1 for anderson and tightbinding, 0 else)")
    ap.add_argument("--neig", type=int, default=None, help="default: 10 (anderson, laplace), 8, 6")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-precision-check", action="store_true",
                    help="skip the float64 / bfloat16 comparison solves after the timed region")
    ap.add_argument("--ref-seconds", type=float, default=180.0,
                    help="reference arm: budget of all its steps (capped samples when complete solves do not fit)")
    args = ap.parse_args()
    defaults = {"anderson": (DEFAULT_SIZE, 1, 10), "laplace": (20, 0, 10), "tightbinding": (64, 1, 8),
                "fem": (512, 0, 6), "batch": (40, 1, 5)}[args.workload]
    if args.size is None:
        args.size = defaults[0]
    if args.precision is None:
        args.precision = defaults[1]
    if args.neig is None:
        args.neig = defaults[2]
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """Samples SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value, world, device="cpu"):
    """The largest of `value` over the ranks of the default process group
    (replicas report the slowest rank); the value itself for one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_problems(weights, world):
    """Independent problems over ranks: heaviest first, each to the least
    loaded rank (ties to the lower rank).  One index list per rank."""
    order = sorted(range(len(weights)), key=lambda q: (-weights[q], q))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for q in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(q)
        load[r] += weights[q]
    return parts


def gather_to_root(obj, world):
    """Host-side gather of one object per rank to rank 0 (None elsewhere)."""
    if world <= 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def merge_shards(parts, results):
    """Per-problem results in the original order from the ranks' shards."""
    merged = [None] * sum(len(p) for p in parts)
    for part, res in zip(parts, results):
        for q, r in zip(part, res):
            merged[q] = r
    return merged


def _finite(v):
    """JSON-safe copy: NaN (a figure not measured for this workload) becomes null."""
    if isinstance(v, dict):
        return {k: _finite(x) for k, x in v.items()}
    if isinstance(v, (list, tuple)):
        return [_finite(x) for x in v]
    if isinstance(v, (float, np.floating)) and not np.isfinite(v):
        return None
    if isinstance(v, np.floating):
        return float(v)
    return v


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_workload(args):
    """Matrix and solver settings of the chosen workload (synthetic, seeded)."""
    from jadamilu_gb300 import matrices as M
    w = {"name": args.workload, "B": None, "kind": "d", "resident": True}
    if args.workload == "anderson":
        w["A"] = M.anderson3d(args.size, disorder=16.5, seed=0)
        w["kw"] = dict(isearch=2, sigma=0.0, madspace=25, droptol=args.droptol, mem=args.mem)
        w["desc"] = (f"anderson3d {args.size}^3 periodic, W=16.5, seed 0, n={args.size ** 3}, {args.neig} eigpairs "
                     f"closest to 0, TOL 1e-10")
    elif args.workload == "laplace":
        w["A"] = M.laplace3d(args.size)
        w["kw"] = dict(isearch=0, sigma=0.0, madspace=20, droptol=1e-3, mem=20.0)
        w["desc"] = f"7-point Dirichlet Laplacian {args.size}^3, n={args.size ** 3}, {args.neig} smallest, TOL 1e-10"
    elif args.workload == "tightbinding":
        w["A"] = M.tight_binding3d(args.size, phi=1.0 / 17.0, disorder=4.0, seed=1)
        w["kw"] = dict(isearch=0, sigma=0.0, madspace=20, droptol=1e-3, mem=20.0)
        w["kind"], w["resident"] = "z", False
        w["desc"] = (f"complex Hermitian tight-binding {args.size}^3, Peierls phi=1/17, on-site U[-2,2], seed 1, "
                     f"n={args.size ** 3}, {args.neig} lowest, TOL 1e-10 (matrix uploaded by every solve)")
    else:
        K, Mm = M.fem_p1(args.size, sigma=0.5, seed=3)
        w["A"], w["B"] = K, Mm
        w["kw"] = dict(isearch=0, sigma=0.0, madspace=20, droptol=1e-3, mem=20.0)
        w["kind"], w["resident"] = "gep", False
        w["desc"] = (f"P1-FEM K x = lambda M x, {args.size}x{args.size} nodes, lognormal sigma 0.5, seed 3, "
                     f"n={(args.size - 2) ** 2}, {args.neig} smallest, TOL 1e-10 (matrices uploaded by every solve)")
    return w


def solve_kwargs(args, icntl2, w=None):
    kw = dict(w["kw"]) if w is not None else dict(isearch=2, sigma=0.0, madspace=25, droptol=args.droptol,
                                                   mem=args.mem)
    kw.update(maxit=100000, tol=1e-10, icntl=(0, icntl2, 0, 0, args.precision))
    return kw


def workload(size):
    from jadamilu_gb300 import matrices as M
    return M.anderson3d(size, disorder=16.5, seed=0)


def run_solve(J, w, args, icntl2):
    a, ja, ia = w["A"][2], w["A"][1], w["A"][0]
    kw = solve_kwargs(args, icntl2, w)
    if w["kind"] == "z":
        return J.zpjd((a, ja, ia), args.neig, **kw)
    if w["kind"] == "gep":
        B = w["B"]
        return J.dpjd_gep((a, ja, ia), (B[2], B[1], B[0]), args.neig, **kw)
    return J.dpjd((a, ja, ia), args.neig, **kw)


def cpu_baseline_sample(J, ia, ja, a, args, gpu_iter, w=None):
    """Oracle iterations on the same matrix with the GPU run's factor."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    L = J.load()
    n_out = np.zeros(1, np.int32)
    nnz = np.zeros(1, np.int64)
    sh = np.zeros(1)
    p = lambda v: v.ctypes.data_as(C.c_void_p)
    L.jdgpu_dfactor_export.argtypes = [C.c_void_p] * 12
    L.jdgpu_dfactor_export(p(n_out), p(nnz), p(sh), *([None] * 9))
    n, nz = int(n_out[0]), int(nnz[0])
    perm = np.zeros(n, np.int32)
    lp = np.zeros(n + 1, np.int64)
    li = np.zeros(nz, np.int32)
    lx = np.zeros(nz)
    blk = np.zeros(n, np.int8)
    dinv, doff, ainv, aoff = (np.zeros(n) for _ in range(4))
    L.jdgpu_dfactor_export(p(n_out), p(nnz), p(sh), p(perm), p(lp), p(li), p(lx), p(blk), p(dinv), p(doff),
                           p(ainv), p(aoff))
    cpl, nlev, nnzf = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1, np.int64)
    L.jdgpu_dfactor_export_levels.argtypes = [C.c_void_p] * 7
    L.jdgpu_dfactor_export_levels(p(cpl), p(nlev), p(nnzf), None, None, None, None)
    ls = np.zeros(int(nlev[0]) + 1, np.int32)
    fp = np.zeros(n + 1, np.int64)
    fi = np.zeros(max(1, int(nnzf[0])), np.int32)
    fx = np.zeros(max(1, int(nnzf[0])))
    L.jdgpu_dfactor_export_levels(p(cpl), p(nlev), p(nnzf), p(ls), p(fp), p(fi), p(fx))
    O = oracle_lib.lib()
    O.orc_dimport_factor.argtypes = [C.c_int] + [C.c_void_p] * 9 + [C.c_double]
    O.orc_dimport_factor(n, p(perm), p(lp), p(li), p(lx), p(blk), p(dinv), p(doff), p(ainv), p(aoff), float(sh[0]))
    O.orc_dimport_levels.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 4
    O.orc_dimport_levels(int(cpl[0]), int(nlev[0]), p(ls), p(fp), p(fi), p(fx))
    # a short capped run gives the cost per MATVEC; a complete solve follows when it fits the budget
    kw = solve_kwargs(args, -1, w)
    kw["maxit"] = 16
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw)
    per_mv = (time.perf_counter() - t0) / max(r["iter"], 1)
    if per_mv * gpu_iter * 1.3 <= args.cpu_seconds:
        t0 = time.perf_counter()
        r = oracle_lib.dpjd(ia, ja, a, args.neig, **solve_kwargs(args, -1, w))
        dt = time.perf_counter() - t0
        return {"value": dt, "unit": "s", "cores": 1, "kind": "port",
                "sample": f"CPU oracle, same matrix and factor, one complete solve: {r['iter']} MATVECs, "
                          f"INFO {r['info']}, {dt:.1f} s"}
    cap = max(16, int(args.cpu_seconds / per_mv))
    kw["maxit"] = cap
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw)
    dt = time.perf_counter() - t0
    it = r["iter"]
    per_mv = dt / max(it, 1)
    return {"value": per_mv * gpu_iter, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"CPU oracle, same matrix and factor, {it} MATVECs in {dt:.1f} s "
                      f"({per_mv * 1e3:.1f} ms/MATVEC) scaled to the GPU solve's {gpu_iter} MATVECs"}


def cpu_baseline_own_factor(args, w, gpu_iter):
    """Oracle iterations for the complex and generalized workloads, whose
    factors are not exported: the oracle factors the same matrix with its
    own code on all host threads (untimed, as the reference arm does), then
    runs the MATVECs that fit --cpu-seconds on one core, scaled to the GPU
    solve's MATVEC count."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    ia, ja, a = w["A"]
    extra = {"complex_": True} if w["kind"] == "z" else {"b": w["B"]}
    O = oracle_lib.lib()
    O.orc_set_threads.argtypes = [C.c_int]
    threads = os.cpu_count() or 1
    O.orc_set_threads(threads)
    kw = solve_kwargs(args, 1, w)
    kw["maxit"] = 4
    t0 = time.perf_counter()
    oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
    factor_s = time.perf_counter() - t0
    kw = solve_kwargs(args, -1, w)
    kw["maxit"] = 16
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
    per_mv = (time.perf_counter() - t0) / max(r["iter"], 1)
    kw["maxit"] = max(16, int(args.cpu_seconds / per_mv))
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
    dt = time.perf_counter() - t0
    it = r["iter"]
    per_mv = dt / max(it, 1)
    return {"value": per_mv * gpu_iter, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"CPU oracle, same matrix, its own factor ({factor_s:.1f} s on {threads} threads, untimed); "
                      f"{it} MATVECs in {dt:.1f} s on one core ({per_mv * 1e3:.1f} ms/MATVEC) scaled to the GPU "
                      f"solve's {gpu_iter} MATVECs"}


def precision_check(J, w, args, timed, stream, torch):
    """One solve with the factor in float64 (the plain FP64 GPU method) and
    one in bfloat16, reusing the host factor (ICNTL(2) = -1, ICNTL(5) 0 / 2):
    seconds per solve (CUDA events), MATVECs, and per eigenvalue the error of
    the timed run's eigenvalues against the float64 run's."""
    out = {}
    ref = None
    for name, prec in (("fp64", 0), ("bf16", 2)):
        a2 = argparse.Namespace(**vars(args))
        a2.precision = prec
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = run_solve(J, w, a2, -1)
        e1.record(stream)
        torch.cuda.synchronize()
        ok = r["info"] == 0 and r["neig"] == args.neig
        ev = np.sort(r["eigs"])
        out[name] = {"s_per_solve": e0.elapsed_time(e1) / 1e3, "matvec": r["iter"], "converged": ok,
                     "max_res": float(np.max(r["res"])) if len(r["res"]) else None}
        if prec == 0:
            ref = ev if ok else None
        elif ref is not None and ok:
            out[name]["eig_rel_err_vs_fp64"] = (np.abs(ev - ref) / np.abs(ref)).tolist()
    mixed = np.sort(timed["eigs"])
    if ref is not None and len(mixed) == len(ref):
        err = np.abs(mixed - ref)
        # the tests' bound: 1e-10 relative, or 64 eps ||A|| for eigenvalues near 0
        a, ja, ia = w["A"][2], w["A"][1], w["A"][0]
        rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
        rs = np.zeros(len(ia) - 1)
        np.add.at(rs, rows, np.abs(a))
        np.add.at(rs, np.asarray(ja) - 1, np.where(rows == np.asarray(ja) - 1, 0.0, np.abs(a)))
        bound = np.maximum(1e-10 * np.abs(ref), 64 * np.finfo(float).eps * float(rs.max()))
        out["mixed_eig_abs_err_vs_fp64"] = err.tolist()
        out["mixed_eig_rel_err_vs_fp64"] = (err / np.abs(ref)).tolist()
        out["mixed_max_rel_err_vs_fp64"] = float(np.max(err / np.abs(ref)))
        out["mixed_within_tolerance"] = bool(np.all(err <= bound))
        out["tolerance"] = "max(1e-10 |lambda|, 64 eps ||A||_inf)"
    # restore the timed run's factor precision for the legs that follow
    run_solve(J, w, args, -1)
    return out


def profile_traffic(w, args):
    """DRAM bytes (read + write) per preconditioner application from the
    committed ncu summary of the same workload, when there is one."""
    path = os.path.join(ROOT, "profiles", "ildl_apply_anderson%d.md" % args.size)
    if w["name"] != "anderson" or not os.path.exists(path):
        return None
    key = "traffic_bytes_per_application_%s:" % {0: "fp64", 1: "fp32", 2: "bf16"}[args.precision]
    for line in open(path):
        if line.strip().startswith(key):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def run_gb300(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    import jadamilu_gb300 as J
    from jadamilu_gb300 import build
    build.build_all()
    L = J.load()
    w = make_workload(args)
    ia, ja, a = w["A"]
    n = len(ia) - 1
    nnz_upper = len(a)
    stream = torch.cuda.Stream()
    J.set_stream(stream.cuda_stream)
    if w["resident"]:
        J.prepare_matrix((a, ja, ia))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # factorisation (host) + first solve; then warm-up solves reusing the factor
    J.reset_stats()
    t0 = time.perf_counter()
    r = run_solve(J, w, args, 1)
    first_s = time.perf_counter() - t0
    st = J.stats(complex_=w["kind"] == "z")
    if r["info"] != 0:
        raise SystemExit(f"first solve failed: INFO={r['info']}")
    for _ in range(max(0, args.warmup - 1)):
        r = run_solve(J, w, args, -1)
    # timed region: device-resident solves
    clocks = Clocks(local)
    barrier()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = L.jdgpu_launch_count()
    iters, results = [], []
    J.reset_stats()
    e0.record(stream)
    for _ in range(args.steps):
        r = run_solve(J, w, args, -1)
        iters.append(r["iter"])
        results.append(r)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = L.jdgpu_launch_count() - l0
    timed_st = J.stats(complex_=w["kind"] == "z")
    clk = clocks.stop()
    ms = max_over_ranks(ms, world, device="cuda")
    # the solver's own test (INFO = 0, all pairs returned); the final Rayleigh-Ritz
    # refinement of a converged cluster recomputes RES, which can end slightly
    # above TOL, as in the reference (JDaux.F:2270-2300); max_res reports it
    ok = all(rr["info"] == 0 and rr["neig"] == args.neig for rr in results)
    eigs = np.sort(results[-1]["eigs"])
    # roofline of the dominant kernels (preconditioner application) and of SpMV,
    # with the last solve's factor and matrix (real or complex state)
    pb = np.full(6, np.nan)
    sb = np.full(4, np.nan)
    pre = "z" if w["kind"] == "z" else "d"
    for name, reps, buf in (("jdgpu_%sprecond_bench" % pre, 20, pb), ("jdgpu_%sspmv_bench" % pre, 50, sb)):
        fn = getattr(L, name)
        fn.argtypes = [C.c_int, C.c_void_p]
        if fn(reps, buf.ctypes.data_as(C.c_void_p)) != 0:
            buf[:] = np.nan
    peak, peak_kind = measured_peaks()
    # achieved bandwidth on the algorithmic bytes of one application (pb[5]:
    # every L entry once per sweep, F and F^H, D, vectors); pb[1] adds what the
    # dense blocks' explicit-inverse tiles stream instead of their L entries
    prec_gbs = pb[5] / (pb[0] * 1e-3) / 1e9
    prec_streamed_gbs = pb[1] / (pb[0] * 1e-3) / 1e9
    spmv_gbs = sb[1] / (sb[0] * 1e-3) / 1e9
    # the same factor in float64 (the plain FP64 method) and in bfloat16, one
    # build: seconds per solve and the error of each eigenvalue of the timed
    # (mixed) run against the float64 run
    prec_check = None
    if w["resident"] and w["kind"] == "d" and not args.no_precision_check:
        prec_check = precision_check(J, w, args, results[-1], stream, torch)
    # e2e: through the C ABI with host buffers (matrix upload + eigenvector download)
    if w["resident"]:
        J.release_matrix()
    torch.cuda.synchronize()
    vb = 16 if w["kind"] == "z" else 8
    h2d = (n + 1) * 4 + nnz_upper * 4 + nnz_upper * vb
    if w["B"] is not None:
        h2d += (n + 1) * 4 + len(w["B"][2]) * 12
    d2h = args.neig * n * vb + 2 * args.neig * 8
    e2e_s = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run_solve(J, w, args, -1)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            if w["kind"] == "d":
                cpu = cpu_baseline_sample(J, ia, ja, a, args, int(np.median(iters)), w)
            else:
                cpu = cpu_baseline_own_factor(args, w, int(np.median(iters)))
        except Exception as ex:  # reported, not fatal
            cpu = {"value": None, "unit": "s", "cores": 1, "kind": "port", "sample": f"failed: {ex}"}
    if rank == 0:
        metric = METRIC if w["name"] == "anderson" else f"s to {args.neig} eigpairs at resid 1e-10 ({w['name']})"
        outer = "c128" if w["kind"] == "z" else "f64"
        inner = {0: outer, 1: "c64" if w["kind"] == "z" else "f32", 2: "bf16"}[args.precision]
        line = {
            "metric": metric,
            "value": ms / 1e3,
            "unit": "s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": False,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": outer if args.precision == 0 else f"{outer} outer / {inner} factor",
            "data": "synthetic (seeded splitmix64 generators)",
            "config": {"workload": w["desc"],
                       "n": n, "nnz_upper": nnz_upper, "droptol": w["kw"]["droptol"], "condest": 5.0,
                       "madspace": w["kw"]["madspace"], "icntl": [0, -1, 0, 0, args.precision],
                       "factor_s": st["factor_s"], "first_solve_with_factor_s": first_s,
                       "fill": st["fill"], "nnz_l": st["nnz_l"], "levels": st["levels"],
                       "fwd_depth": st["fwd_depth"], "dense_rows": st["dense_rows"],
                       "dense_blocks": st["dense_blocks"], "matvec_per_solve": int(np.median(iters)),
                       "precond_per_solve": timed_st["n_precond"] / args.steps,
                       "precond_share_of_solve": timed_st["n_precond"] / args.steps * pb[0] / ms,
                       "parallelism": f"replicas x{world}", "l2": "working set > L2 (no flush needed)",
                       "eigs_min_max": [float(eigs[0]), float(eigs[-1])], "converged": ok,
                       "eigs": [float(v) for v in eigs],
                       "info": [rr["info"] for rr in results], "neig": [rr["neig"] for rr in results],
                       "max_res": max(float(np.max(rr["res"])) if len(rr["res"]) else 0.0 for rr in results)},
            "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"kernel": f"ildl_apply graph (level sweeps, coupling blocks, dense-block tiles; {inner})",
                         "bound": "hbm",
                         "achieved": prec_gbs, "peak": peak, "unit": "GB/s", "frac": prec_gbs / peak,
                         "traffic": profile_traffic(w, args), "bytes_per_launch": pb[5], "ms_per_launch": pb[0],
                         "kernels_per_launch": pb[4], "peak_kind": peak_kind,
                         "streamed": {"bytes_per_launch": pb[1], "achieved": prec_streamed_gbs,
                                      "frac": prec_streamed_gbs / peak}},
            "roofline_spmv": {"achieved": spmv_gbs, "peak": peak, "unit": "GB/s", "frac": spmv_gbs / peak,
                              "bytes_per_launch": sb[1], "ms_per_launch": sb[0]},
            "precision_check": prec_check,
            "gpu_launches": int(launches),
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        _emit(_finite(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def fixture_matvecs(args):
    """MATVECs of the oracle's complete solve of the Anderson workload of this
    size, from the committed fixture (tests/golden/anderson_eigs.json), when
    the settings match; None otherwise."""
    path = os.path.join(ROOT, "tests", "golden", "anderson_eigs.json")
    try:
        with open(path) as f:
            d = json.load(f)
    except Exception:
        return None
    st = d.get("settings", {})
    if st.get("droptol") != args.droptol or list(st.get("icntl", []))[4:5] != [args.precision] or args.neig != 10:
        return None
    case = d.get("cases", {}).get(str(args.size))
    return int(case["oracle_matvec"]) if case and "oracle_matvec" in case else None


def run_reference(args):
    """The reference path on the host cores: the CPU oracle (the reference's
    algorithm restated; the Fortran library cannot be built on this image).

    The factor is computed once (all host threads) and every step is one
    complete solve reusing it (ICNTL(2) = -1), as in the GPU arm.  When a
    complete solve does not fit the step budget (--ref-seconds over all
    steps), each step runs the MATVECs that fit and is scaled to the MATVEC
    count of the oracle's complete solve of the same workload, recorded in
    tests/golden/anderson_eigs.json."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "batch":
        run_reference_batch(args, world)
        return
    w = make_workload(args)
    extra = {}
    if w["kind"] == "z":
        extra["complex_"] = True
    elif w["kind"] == "gep":
        extra["b"] = w["B"]
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    from jadamilu_gb300 import build
    build.build_oracle()
    ia, ja, a = w["A"]
    n = len(ia) - 1
    O = oracle_lib.lib()
    threads = os.cpu_count() or 1
    O.orc_set_threads.argtypes = [C.c_int]
    O.orc_set_threads(threads)
    t0 = time.perf_counter()
    kw = solve_kwargs(args, 1, w)
    kw["maxit"] = 4
    oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
    factor_s = time.perf_counter() - t0
    # Each step is a complete solve when one fits the step budget; otherwise a
    # solve capped at the MATVECs that fit, scaled to the oracle's own MATVEC
    # count of a complete solve of this workload (the committed fixture), so
    # the whole arm ends within about --ref-seconds.
    budget = args.ref_seconds / max(1, args.warmup + args.steps)
    kw = solve_kwargs(args, -1, w)
    kw["maxit"] = 16
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
    per_mv = (time.perf_counter() - t0) / max(1, r["iter"])
    full = fixture_matvecs(args) if w["name"] == "anderson" else None
    mv = full if (full is not None and per_mv * full > budget) else None
    times, iters, infos = [], [], []
    for step in range(args.warmup + args.steps):
        kw = solve_kwargs(args, -1, w)
        if mv:
            kw["maxit"] = max(16, int(budget / per_mv))
        t0 = time.perf_counter()
        r = oracle_lib.dpjd(ia, ja, a, args.neig, **kw, **extra)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt * (mv / max(1, r["iter"]) if mv else 1.0))
            iters.append(r["iter"])
            infos.append(r["info"])
    v = float(np.median(times))
    sample = (f"CPU oracle, {'capped samples scaled to %d MATVECs (its complete solve)' % mv if mv else 'complete solves'}, "
              f"factor {factor_s:.1f} s on {threads} threads (untimed), solve on 1 core, "
              f"MATVECs {iters}, INFO {infos}")
    metric = METRIC if w["name"] == "anderson" else f"s to {args.neig} eigpairs at resid 1e-10 ({w['name']})"
    outer = "c128" if w["kind"] == "z" else "f64"
    inner = {0: outer, 1: "c64" if w["kind"] == "z" else "f32", 2: "bf16"}[args.precision]
    line = {"impl": "reference", "metric": metric, "value": v, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": outer if args.precision == 0 else f"{outer} outer / {inner} factor",
            "data": "synthetic (seeded splitmix64 generators)",
            "config": {"workload": w["desc"], "factor_s": factor_s, "matvec_per_solve": int(np.median(iters))},
            "cpu_baseline": {"value": v, "unit": "s", "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    _emit(line)


def _oracle_batch_solve(job):
    """One problem of the batch on the CPU oracle, single-threaded (pool worker)."""
    q, m, neig, droptol, mem, precision = job
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, ROOT)
    import oracle_lib
    from jadamilu_gb300 import matrices as M
    oracle_lib.lib().orc_set_threads(1)
    ia, ja, a = M.anderson3d(int(m), disorder=16.5, seed=1000 + q)
    t0 = time.perf_counter()
    r = oracle_lib.dpjd(ia, ja, a, neig, sigma=0.0, isearch=2, madspace=20, maxit=100000, tol=1e-10,
                        droptol=droptol, mem=mem, icntl=(0, 0, 0, 0, precision))
    return q, time.perf_counter() - t0, r["info"], r["iter"]


def oracle_batch_sample(args, edges, stride, rounds=1):
    """The CPU oracle on every stride-th problem of the batch (factor and
    solve on one core each) in a spawn-started process pool over the host
    cores; returns the median over rounds of the sample's wall time scaled by
    the batch's total nnz^1.75 weight over the sample's, the description of
    the sample and the processes used."""
    import multiprocessing as mp
    weight = [float(7 * int(m) ** 3) ** 1.75 for m in edges]
    picked = [q for q in range(len(edges)) if q % stride == 0]
    cores = os.cpu_count() or 1
    jobs = [(q, int(edges[q]), args.neig, args.droptol, args.mem, args.precision) for q in picked]
    ctx = mp.get_context("spawn")
    times, infos, iters = [], [], []
    with ctx.Pool(min(cores, len(jobs))) as pool:
        for _ in range(rounds):
            t0 = time.perf_counter()
            out = pool.map(_oracle_batch_solve, jobs)
            times.append((time.perf_counter() - t0) * sum(weight) / sum(weight[q] for q in picked))
            infos = [o[2] for o in out]
            iters = [o[3] for o in out]
    sample = (f"CPU oracle, problems {picked} of {len(edges)} (every {stride}th), factor and solve on one core "
              f"each, {min(cores, len(jobs))} processes; wall time scaled by nnz^1.75 weight to the whole batch; "
              f"MATVECs {iters}, INFO {infos}")
    return float(np.median(times)), sample, min(cores, len(jobs))


def run_reference_batch(args, world):
    """The batch on the host cores: the CPU oracle solves (factor included,
    one core each) a bounded sample of the batch's problems in a process
    pool over all host cores; the step time is the sample's wall time scaled
    by the batch's total nnz^1.75 weight over the sample's."""
    from jadamilu_gb300 import build
    build.build_oracle()
    edges = np.random.default_rng(2).integers(16, 41, size=args.batch)
    stride = max(1, int(os.environ.get("JDG_BATCH_SAMPLE_STRIDE", "8")))
    oracle_batch_sample(args, edges, stride, rounds=args.warmup) if args.warmup > 0 else None
    v, sample, procs = oracle_batch_sample(args, edges, stride, rounds=args.steps)
    line = {"impl": "reference",
            "metric": f"s to {args.neig} eigpairs per problem at resid 1e-10, batch of {args.batch} Anderson problems",
            "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
            "dtype": "f64 outer / f32 factor" if args.precision == 1 else "f64",
            "data": "synthetic (seeded splitmix64 generators)",
            "config": {"workload": f"{args.batch} Anderson problems, edges 16..40 (seed 2), {args.neig} eigpairs "
                                   f"closest to 0 each, TOL 1e-10, host ILDLC per problem included",
                       "sampled_problems": len(range(0, args.batch, stride))},
            "cpu_baseline": {"value": v, "unit": "s", "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    _emit(_finite(line))


def run_batch(args):
    """Batched workload: --batch independent Anderson problems (edges uniform
    in 16..40 from seed 2, W=16.5, disorder seeds 1000+q), 5 eigenpairs closest
    to 0 each, solved by jdgpu_dpjd_batch with --workers threads / streams.
    A step is one batch call, host ILDLC factorisations included (every
    problem gets its own preconditioner); wall clock around the call.  With N
    ranks the problems are split by greedy balancing of nnz^1.75 (the growth
    of the host factor time with size), no collective on the data path; the
    step time is the slowest rank's and rank 0 gathers the results."""
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    import jadamilu_gb300 as J
    from jadamilu_gb300 import build
    from jadamilu_gb300 import matrices as M
    build.build_all()
    L = J.load()
    edges = np.random.default_rng(2).integers(16, 41, size=args.batch)
    parts = shard_problems([float(7 * int(m) ** 3) ** 1.75 for m in edges], world)
    mine = parts[rank]
    probs = [M.anderson3d(int(edges[q]), disorder=16.5, seed=1000 + q) for q in mine]
    mats = [(a, ja, ia) for ia, ja, a in probs]
    kw = dict(sigma=0.0, isearch=2, madspace=20, maxit=100000, tol=1e-10, droptol=args.droptol, mem=args.mem,
              icntl=(0, 0, 0, 0, args.precision))

    def one():
        fresh = [(a.copy(), ja.copy(), ia.copy()) for a, ja, ia in mats]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = J.dpjd_batch(fresh, args.neig, workers=args.workers, **kw)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, out

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        one()
    clocks = Clocks(local)
    clocks.start()
    l0 = L.jdgpu_launch_count()
    times, outs = [], None
    for _ in range(args.steps):
        barrier()
        dt, outs = one()
        times.append(max_over_ranks(dt, world, device="cuda"))
    launches = int(max_over_ranks(L.jdgpu_launch_count() - l0, world, device="cuda"))
    clk = clocks.stop()
    v = float(np.mean(times))
    summary = [dict(info=r["info"], neig=r["neig"], iter=r["iter"]) for r in outs]
    h2d_local = int(sum((len(ia) + len(ja)) * 4 + len(a) * 8 for a, ja, ia in mats))
    gathered = gather_to_root((summary, h2d_local), world)
    if rank != 0:
        return
    outs = merge_shards(parts, [g[0] for g in gathered])
    ok = all(r["info"] == 0 and r["neig"] == args.neig for r in outs)
    # representative kernels: the largest problem solved alone by the single-
    # problem driver, its preconditioner application and SpMV timed on the GPU
    roof = None
    qbig = int(np.argmax(edges))
    ia, ja, a = M.anderson3d(int(edges[qbig]), disorder=16.5, seed=1000 + qbig)
    rb = J.dpjd((a, ja, ia), args.neig, **dict(kw, icntl=(0, 1, 0, 0, args.precision)))
    if rb["info"] == 0:
        pb = np.full(6, np.nan)
        sb = np.full(4, np.nan)
        L.jdgpu_dprecond_bench.argtypes = [C.c_int, C.c_void_p]
        L.jdgpu_dprecond_bench(20, pb.ctypes.data_as(C.c_void_p))
        L.jdgpu_dspmv_bench.argtypes = [C.c_int, C.c_void_p]
        L.jdgpu_dspmv_bench(50, sb.ctypes.data_as(C.c_void_p))
        peak, peak_kind = measured_peaks()
        gbs = pb[5] / (pb[0] * 1e-3) / 1e9
        roof = {"kernel": f"ildl_apply graph of the largest problem ({int(edges[qbig])}^3)", "bound": "hbm",
                "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "traffic": None,
                "bytes_per_launch": pb[5], "ms_per_launch": pb[0], "peak_kind": peak_kind,
                "spmv": {"achieved": sb[1] / (sb[0] * 1e-3) / 1e9, "ms_per_launch": sb[0]}}
    cpu = None
    if world == 1 and not args.no_cpu:
        v_cpu, sample, procs = oracle_batch_sample(args, edges, max(1, args.batch // 8))
        cpu = {"value": v_cpu, "unit": "s", "cores": procs, "kind": "port", "sample": sample}
    n_tot = int(sum(int(m) ** 3 for m in edges))
    h2d = int(sum(g[1] for g in gathered))
    d2h = int(sum(int(m) ** 3 * args.neig * 8 for m in edges))
    line = {"metric": f"s to {args.neig} eigpairs per problem at resid 1e-10, batch of {args.batch} Anderson problems",
            "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
            "dtype": "f64 outer / f32 factor" if args.precision == 1 else "f64",
            "data": "synthetic (seeded splitmix64 generators)",
            "config": {"workload": f"{args.batch} Anderson problems, edges 16..40 (seed 2), n total {n_tot}, "
                                   f"{args.neig} eigpairs closest to 0 each, TOL 1e-10, host ILDLC per problem "
                                   f"included",
                       "workers": args.workers, "droptol": args.droptol, "converged": ok,
                       "parallelism": f"problems sharded over {world} rank(s), no collective",
                       "matvec_total": int(sum(r["iter"] for r in outs)),
                       "info_nonzero": int(sum(r["info"] != 0 for r in outs))},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roof, "gpu_launches": int(launches), "clocks": clk, "cpu_baseline": cpu}
    _emit(_finite(line))


_RESULT_OUT = None


def _emit(line):
    """Write the one result line to the process's original standard output."""
    out = _RESULT_OUT or sys.stdout
    out.write(json.dumps(line) + "\n")
    out.flush()


def main():
    global _RESULT_OUT
    args = parse()
    # The solver writes its own messages (factor restarts, IPRINT reports) to
    # standard output as the reference does; move them to stderr so that
    # standard output carries the result line alone.
    sys.stdout.flush()
    _RESULT_OUT = os.fdopen(os.dup(1), "w")
    os.dup2(2, 1)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
