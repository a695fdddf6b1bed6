#!/usr/bin/env python
"""Benchmark of the PLR solve path: RHS/s at N = 2^18 with 256 right-hand sides.

Workload (the mixed-precision configuration of the reference's target):
N = 262144 points uniform in the unit square, ordered by kd-tree bisection,
Gaussian kernel exp(-r^2 / (2 * 0.05^2)) + 1e-2 * I, leaf 256 (10 levels),
adaptive off-diagonal ranks (tol 1e-10, clamped to [8, 128]), 256
standard-normal right-hand sides; a step is one solve of all 256 right-hand
sides refined to relative residual <= 1e-12 (max over columns), the
residual computed by the FP64 PLR apply of the matrix.

Arms:
  --impl ours       libdplr_gb300.so: Woodbury factorisation on the GPU
                    (setup, untimed), then timed refined solves.
  --impl reference  the reference algorithm on the host cores: the explicit
                    PLR inverse (dplrgeinv) applied with dplrgepdmm and
                    refined with dplrgepdmm of the matrix, run by the CPU
                    oracle (the reference's C restated, linked to an
                    optimised BLAS, all host threads) on a bounded sample.

Prints one JSON line (rank 0).  Under torchrun each rank solves its own
replica (the path does not shard: replicas only) and the value is the
aggregate over ranks.
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("PLR solve RHS/s @N=2^18,256 RHS: mixed+refined vs FP64 GPU at ≤1e-12 rel resid")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1 << 18)
    ap.add_argument("--leaf", type=int, default=256)
    ap.add_argument("--rhs", type=int, default=256)
    ap.add_argument("--rmax", type=int, default=128)
    ap.add_argument("--tol", type=float, default=1e-12)
    ap.add_argument("--maxiter", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed",
                    help="inner solver of the refinement: sliced tensor-core sweep or FP64 sweep")
    ap.add_argument("--mixed-slices", type=int, default=7,
                    help="bf16 slices of the mixed inner solve (3 to 7)")
    ap.add_argument("--residual", choices=["sliced", "fp64"], default="sliced",
                    help="refinement residual: exact-slice tensor-core products or the FP64 apply")
    ap.add_argument("--workload", choices=["solve", "apply", "batched", "adjoint", "compress", "ppmm", "c2"],
                    default="solve",
                    help="solve: the headline refined solve; the others are secondary workloads "
                         "(dplr_gb300/workloads.py)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-sample", type=int, default=1 << 14,
                    help="size of the diagonal sub-block of the CPU arm's whole-solve detail")
    ap.add_argument("--cpu-rhs", type=int, default=64,
                    help="right-hand sides of the CPU arm's timed solve step (a bounded sample)")
    ap.add_argument("--geinv-cap", type=float, default=300.0,
                    help="wall-time cap (s) of the CPU arm's full-size dplrgeinv")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers

class ClockSampler:
    """nvidia-smi samples of SM clock, power and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # the sampler never outlives the run, even one that raises
            atexit.register(self._end)
        except Exception:
            self.proc = None

    def _end(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._end()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v == "Active"})
        clocks = sorted(r[0] for r in rows)
        return {"sm_mhz": clocks[len(clocks) // 2], "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def workload_config(args, stats=None, extra=None) -> dict:
    cfg = {
        "workload": (f"2D Gaussian kernel PLR solve, N={args.n}, leaf {args.leaf}, "
                     f"{args.rhs} RHS, refined to {args.tol:g}"),
        "n": args.n, "leaf": args.leaf, "levels": 0, "rhs": args.rhs,
        "kernel": "exp(-r^2/(2*0.05^2)) + 1e-2*I on uniform unit-square points, kd-tree order",
        "ranks": "adaptive, tol 1e-10, clamped to [8, %d]" % args.rmax,
        "tol": args.tol, "seed": args.seed,
        "l2": "inputs larger than L2 (factors several GB)",
    }
    if stats is not None:
        cfg["ranks_by_level"] = stats.ranks
    if extra:
        cfg.update(extra)
    return cfg


def build_matrix(args, device="cuda"):
    from dplr_gb300 import gen_gpu
    stats = gen_gpu.GenStats()
    t = gen_gpu.kernel_tree_2d(n=args.n, leaf=args.leaf, rmax=args.rmax, seed=args.seed,
                               device=device, stats=stats)
    return t, stats


# --------------------------------------------------------------- CPU legs
#
# The reference's own algorithm for the path runs on the host cores through
# the oracle (its C restated, linked to an optimised BLAS, all host threads).
# Only these CPU legs touch the oracle; the measured GPU path never does.

class HostMatrix:
    """The benchmark matrix as a DPlrMtx tree in host memory."""

    def __init__(self, t):
        from dplr_gb300 import tree as tr
        self.t, self.m, self.c, self.nnz = t, t.size, tr.to_c(t), tr.nnz(t)

    def close(self):
        from dplr_gb300 import tree as tr
        tr.free_c(self.c)


def cpu_apply(hm: HostMatrix, X, threads: int):
    """One full-size dplrgepdmm Y = A X (src/dplrpdmm.c:454 restated) on
    `threads` host threads; X is (nrhs, m).  Returns (seconds, Y)."""
    import numpy as np

    from oracle import pyoracle
    orc = pyoracle.oracle("best")
    pyoracle.set_threads(orc, threads)
    nrhs, m = X.shape
    xf = np.ascontiguousarray(X).reshape(-1)
    y = np.zeros(nrhs * m)
    t0 = time.perf_counter()
    orc.gepdmm("N", "N", m, nrhs, 1.0, hm.c, xf, m, 0.0, y, m)
    return time.perf_counter() - t0, y.reshape(nrhs, m)


class InverseShape:
    """A host tree shaped like DPLR's explicit inverse of the matrix (own
    rank + every ancestor's correction in each block, leaves unchanged;
    oracle/shape.c), filled with a constant: the reference's solve applies
    inv(A), and dplrgeinv itself does not finish at full size in the time a
    benchmark step allows, so its apply is timed on this stand-in."""

    def __init__(self, hm: HostMatrix):
        from dplr_gb300 import tree as tr
        from oracle import pyoracle
        orc = pyoracle.oracle("best")
        self.m, self.c = hm.m, tr.new_empty()
        if orc.lib.orc_inverse_shape(hm.m, hm.c, self.c, 1e-3) != 0:
            self.close()
            raise MemoryError("cannot build the inverse-shaped tree")
        self.nnz = orc.nz(hm.m, self.c)

    def close(self):
        from dplr_gb300 import tree as tr
        tr.free_c(self.c)


class HostInverse:
    """inv(A) for the reference's solve: DPLR's own dplrgeinv (src/dplrinv.c:93
    restated) of the full matrix on the host cores, given cap_s seconds on a
    daemon thread (the foreign call releases the GIL).  If it has not
    returned by then, the InverseShape stand-in (same rank structure) is
    used for timing and `kind` says so."""

    def __init__(self, hm: HostMatrix, cap_s: float, threads: int):
        import threading

        from dplr_gb300 import tree as tr
        from oracle import pyoracle
        orc = pyoracle.oracle("best")
        pyoracle.set_threads(orc, threads)
        self.m, self.c = hm.m, tr.new_empty()
        box = {}

        def run():
            t0 = time.perf_counter()
            box["info"] = orc.geinv(hm.m, hm.c, self.c, 0.0)
            box["seconds"] = time.perf_counter() - t0

        th = threading.Thread(target=run, daemon=True)
        th.start()
        th.join(cap_s)
        if not th.is_alive() and box.get("info") == 0:
            self.kind, self.seconds, self.owned = "dplrgeinv", box["seconds"], True
            self.nnz = orc.nz(hm.m, self.c)
            return
        # not finished in time (or failed): the tree is the thread's; time the stand-in
        self.owned = False
        self.seconds = None
        self.kind = (f"stand-in with dplrgeinv's rank structure (dplrgeinv not completed in {cap_s:.0f} s)"
                     if th.is_alive() else f"stand-in (dplrgeinv info {box.get('info')})")
        shape = InverseShape(hm)
        self.c, self.nnz = shape.c, shape.nnz

    def close(self):
        from dplr_gb300 import tree as tr
        tr.free_c(self.c)


def cpu_refine_history(hm: HostMatrix, inv, B, steps: int, threads: int) -> list:
    """Relative residuals max_j ||b_j - A x_j|| / ||b_j|| of the reference's
    solve refined with FP64 residuals: x = inv(A) b, then x += inv(A) r."""
    import numpy as np

    from oracle import pyoracle
    orc = pyoracle.oracle("best")
    pyoracle.set_threads(orc, threads)
    nrhs, m = B.shape
    bf = np.ascontiguousarray(B).reshape(-1)
    bn = np.linalg.norm(B, axis=1)
    x, r, d = np.zeros(nrhs * m), np.empty(nrhs * m), np.empty(nrhs * m)
    orc.gepdmm("N", "N", m, nrhs, 1.0, inv.c, bf, m, 0.0, x, m)
    hist = []
    for it in range(steps + 1):
        r[:] = bf
        orc.gepdmm("N", "N", m, nrhs, -1.0, hm.c, x, m, 1.0, r, m)
        hist.append(float(np.max(np.linalg.norm(r.reshape(nrhs, m), axis=1) / bn)))
        if it < steps:
            orc.gepdmm("N", "N", m, nrhs, 1.0, inv.c, r, m, 0.0, d, m)
            x += d
    return hist


def cpu_solve_step(hm: HostMatrix, inv, B, threads: int):
    """One step of the reference's solve on the host cores (the oracle
    restating src/dplrpdmm.c:454): x = inv(A) b with dplrgepdmm, then the
    residual b - A x with dplrgepdmm of A.  B is (nrhs, m).  Returns
    seconds."""
    import numpy as np

    from oracle import pyoracle
    orc = pyoracle.oracle("best")
    pyoracle.set_threads(orc, threads)
    nrhs, m = B.shape
    bf = np.ascontiguousarray(B).reshape(-1)
    x = np.zeros(nrhs * m)
    r = bf.copy()
    t0 = time.perf_counter()
    orc.gepdmm("N", "N", m, nrhs, 1.0, inv.c, bf, m, 0.0, x, m)
    orc.gepdmm("N", "N", m, nrhs, -1.0, hm.c, x, m, 1.0, r, m)
    return time.perf_counter() - t0


def oracle_check(hm: HostMatrix, X, B, AX, dd_cols: int, threads: int) -> dict:
    """Residual of the GPU's solution X of A X = B, computed on the host by
    the oracle: from its FP64 dplrgepdmm AX for every column, and in
    double-double arithmetic (exact for all practical purposes) for
    `dd_cols` columns spread over the block."""
    import numpy as np

    from oracle import pyoracle
    bn = np.linalg.norm(B, axis=1)
    r64 = np.linalg.norm(B - AX, axis=1) / bn
    cols = np.unique(np.linspace(0, X.shape[0] - 1, dd_cols).astype(int))
    t0 = time.perf_counter()
    rn, an = pyoracle.resid_dd(pyoracle.oracle("best"), hm.c, X[cols], B[cols], threads)
    return {"oracle_fp64_rel_resid_max": float(r64.max()),
            "oracle_dd_rel_resid_max": float((rn / bn[cols]).max()),
            "oracle_dd_columns": int(len(cols)),
            "oracle_abs_ax_over_b_max": float((an / bn[cols]).max()),
            "oracle_dd_seconds": time.perf_counter() - t0}


def sub_block_solve(t, args, threads: int, maxiter: int = 20) -> dict:
    """The reference's whole solve (explicit inverse by dplrgeinv, applied by
    dplrgepdmm, refined with dplrgepdmm of A) on the leading diagonal
    sub-block of args.cpu_sample rows: iterates until the FP64 residual
    reaches args.tol, stops growing smaller, or maxiter is hit, and reports
    the residual it reached."""
    import numpy as np

    from dplr_gb300 import tree as tr
    from oracle import pyoracle
    orc = pyoracle.oracle("best")
    pyoracle.set_threads(orc, threads)
    sub = t
    while sub.size > args.cpu_sample and isinstance(sub, tr.HNode):
        sub = sub.nw
    m, nrhs = sub.size, args.rhs
    a, b_inv = tr.to_c(sub), tr.new_empty()
    t0 = time.perf_counter()
    info = orc.geinv(m, a, b_inv, 0.0)
    t_inv = time.perf_counter() - t0
    if info != 0:
        raise RuntimeError(f"oracle geinv failed: {info}")
    rng = np.random.default_rng(args.seed + 7)
    bvec = rng.standard_normal(m * nrhs)
    x, r, d = np.zeros(m * nrhs), np.empty(m * nrhs), np.empty(m * nrhs)
    bn = np.linalg.norm(bvec.reshape(nrhs, m), axis=1)
    t0 = time.perf_counter()
    orc.gepdmm("N", "N", m, nrhs, 1.0, b_inv, bvec, m, 0.0, x, m)
    its, hist = 0, []
    while True:
        r[:] = bvec
        orc.gepdmm("N", "N", m, nrhs, -1.0, a, x, m, 1.0, r, m)
        hist.append(float(np.max(np.linalg.norm(r.reshape(nrhs, m), axis=1) / bn)))
        stalled = len(hist) >= 3 and hist[-1] >= 0.9 * min(hist[:-1])
        if hist[-1] <= args.tol or its >= maxiter or stalled:
            break
        orc.gepdmm("N", "N", m, nrhs, 1.0, b_inv, r, m, 0.0, d, m)
        x += d
        its += 1
    t_solve = time.perf_counter() - t0
    nnz_inv = orc.nz(m, b_inv)
    tr.free_c(a)
    tr.free_c(b_inv)
    return {"n": m, "rhs": nrhs, "geinv_s": t_inv, "solve_s": t_solve, "rhs_per_s": nrhs / t_solve,
            "corrections": its, "rel_resid": hist[-1], "reached_tol": hist[-1] <= args.tol,
            "tol_gap": hist[-1] / args.tol, "resid_history": hist, "nnz_inverse": nnz_inv}


def ppmm_cpu_leg(t, got):
    """One product C := A A + 0.5 C by the restatement of src/dplrppmm.c
    (oracle/ppmm.py, numpy BLAS on all host threads) on the GPU leg's
    input; returns its cpu_baseline entry and the largest difference from
    the GPU's product."""
    import copy

    from dplr_gb300 import workloads
    from oracle import ppmm as oppmm
    c = copy.deepcopy(t)
    t0 = time.perf_counter()
    oppmm.geppmm("N", "N", 1.0, t, t, 0.5, c, workloads.PPMM["eps"])
    sec = time.perf_counter() - t0
    cb = {"value": 1.0 / sec, "unit": "products/s", "cores": os.cpu_count(), "kind": "port",
          "sample": f"one whole product by the restatement of src/dplrppmm.c (oracle/ppmm.py, numpy BLAS "
                    f"on all host threads): {sec:.2f} s"}
    return cb, workloads._max_rel_diff(got, c)


def ppmm_reference_arm(steps: int, warmup: int) -> dict:
    """The reference arm of the product workload, on the host cores only:
    the input is generated on the host, each step is one whole product by
    the restatement of src/dplrppmm.c."""
    import copy

    from dplr_gb300 import workloads
    from oracle import ppmm as oppmm
    t = workloads.ppmm_input("cpu")
    secs = []
    for i in range(warmup + steps):
        c = copy.deepcopy(t)
        t0 = time.perf_counter()
        oppmm.geppmm("N", "N", 1.0, t, t, 0.5, c, workloads.PPMM["eps"])
        if i >= warmup:
            secs.append(time.perf_counter() - t0)
    return workloads.ppmm_reference_record(secs)


def c2_cpu_leg(t, hm=None) -> dict:
    """The reference's dplrgepdmm of the C2 matrix with its 64 RHS on all
    host threads (the oracle restating src/dplrpdmm.c:454): one full-size
    product, timed."""
    from dplr_gb300 import workloads
    threads = os.cpu_count() or 1
    own = hm is None
    hm = HostMatrix(t) if own else hm
    X = workloads.c2_rhs("cpu").numpy()
    cpu_apply(hm, X, threads)                 # warm-up (pages, BLAS threads)
    sec, _ = cpu_apply(hm, X, threads)
    if own:
        hm.close()
    return {"value": X.shape[0] / sec, "unit": "RHS/s", "cores": threads, "kind": "port",
            "sample": f"one whole dplrgepdmm (N={hm.m}, {X.shape[0]} RHS) by the oracle on {threads} host "
                      f"threads: {sec:.3f} s"}


def c2_reference_arm(steps: int, warmup: int) -> dict:
    """The reference arm of the C2 workload: each step one whole dplrgepdmm
    of the C2 matrix with 64 RHS on the host cores."""
    from dplr_gb300 import workloads
    t = workloads.c2_input()
    hm = HostMatrix(t)
    X = workloads.c2_rhs("cpu").numpy()
    threads = os.cpu_count() or 1
    for _ in range(max(0, warmup)):
        cpu_apply(hm, X, threads)
    secs = [cpu_apply(hm, X, threads)[0] for _ in range(max(1, steps))]
    hm.close()
    sec = sorted(secs)[len(secs) // 2]
    nrhs = X.shape[0]
    return {"metric": f"PLR product RHS/s (dplrgepdmm, N={t.size}, rank {workloads.C2['rank']}, {nrhs} RHS, FP64)",
            "value": nrhs / sec, "unit": "RHS/s", "ms_per_step": sec * 1e3, "higher_is_better": True,
            "dtype": "f64", "steps": len(secs), "impl": "reference",
            "cpu_baseline": {"value": nrhs / sec, "unit": "RHS/s", "cores": threads, "kind": "port",
                             "sample": f"one whole dplrgepdmm per step by the oracle on {threads} host threads"},
            "e2e": {"value": nrhs / sec, "unit": "RHS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config": {"workload": "C2 1D exponential-kernel PLR, N=131072, rank 32, 64 RHS",
                       "parallelism": "host cores"}}


def inverse_nnz(t) -> int:
    """dplrnz of DPLR's explicit inverse: every block keeps its own rank and
    gains the rank of each ancestor's correction on its side."""
    from dplr_gb300 import tree as tr

    def walk(node, extra_ne_sw):
        if isinstance(node, tr.Dense):
            return node.size * node.size
        h = node.size // 2
        r1, r2 = node.ne.rank, node.sw.rank
        tot = node.size * (r1 + r2 + 2 * extra_ne_sw)
        return tot + walk(node.nw, extra_ne_sw + r2) + walk(node.se, extra_ne_sw + r1)

    return walk(t, 0)


# --------------------------------------------------------------------- arms

def run_reference(args):
    world, rank, local = dist_init()
    if rank != 0:
        return
    if args.workload in ("compress", "ppmm", "c2"):
        from dplr_gb300 import workloads
        fn = {"compress": workloads.compress_reference, "ppmm": ppmm_reference_arm,
              "c2": c2_reference_arm}[args.workload]
        out = fn(max(1, args.steps), max(0, args.warmup))
        out.update({"n_gpus": 1, "warmup": max(0, args.warmup), "scaling": "weak", "vs_baseline": None,
                    "data": "synthetic"})
        print(json.dumps(out))
        return
    import numpy as np  # noqa: F401
    torch_ok = True
    try:
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
    except Exception:
        torch_ok = False
        dev = "cpu"
    if not torch_ok:
        print(json.dumps({"impl": "reference", "unavailable": "torch missing for input generation"}))
        return
    t, stats = build_matrix(args, device=dev)
    threads = os.cpu_count() or 1
    warm = max(0, args.warmup)
    hm = HostMatrix(t)
    inv = HostInverse(hm, args.geinv_cap, threads)
    nrhs = min(args.cpu_rhs, args.rhs)
    Bs = np.random.default_rng(args.seed + 11).standard_normal((nrhs, args.n))
    for _ in range(warm):                     # untimed (page faults, BLAS thread pool)
        cpu_solve_step(hm, inv, Bs, threads)
    secs = [cpu_solve_step(hm, inv, Bs, threads) for _ in range(max(1, args.steps))]
    sec = sorted(secs)[len(secs) // 2]
    value = nrhs / sec
    sample = (f"one step of the reference's solve per timed step, on {nrhs} of the {args.rhs} RHS at full "
              f"size N={args.n}: x = inv(A) b and the residual b - A x, two dplrgepdmm calls of the "
              f"oracle (src/dplrpdmm.c:454 restated, optimised BLAS, {threads} host threads); inv(A) from "
              f"{inv.kind} (nnz {inv.nnz:.4g}, {inv.nnz / hm.nnz:.1f}x A), formed once before the steps "
              f"as the GPU arm's factorisation is. Median {sec:.2f} s. ")
    detail = {"solve_step_seconds": secs, "solve_step_rhs": nrhs, "nnz_a": hm.nnz, "nnz_inverse": inv.nnz,
              "inverse": inv.kind, "geinv_s": inv.seconds}
    if inv.owned:
        hist = detail["refine_history"] = cpu_refine_history(hm, inv, Bs, 3, threads)
        hit = next((k for k, r in enumerate(hist) if r <= args.tol), None)
        sample += (f"Refined with FP64 residuals it stalls at {min(hist):.2g} > {args.tol:g} (detail.refine_history), "
                   f"so one step per solve is an upper bound of its RHS/s at the tolerance"
                   if hit is None else
                   f"It reaches {args.tol:g} after {hit} corrections: a solve is {hit + 1} such steps")
    else:
        sample += "The value is an upper bound of its RHS/s at the tolerance (one unrefined step)"
    inv.close()
    detail["apply_a_256rhs_s"] = cpu_apply(
        hm, np.random.default_rng(args.seed + 12).standard_normal((args.rhs, args.n)), threads)[0]
    detail["sub_block_solve"] = sub_block_solve(t, args, threads)
    out = {
        "metric": METRIC, "value": value, "unit": "RHS/s", "n_gpus": 1, "steps": len(secs),
        "warmup": warm, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": workload_config(args, stats, {
            "parallelism": "host cores", "levels": tree_levels(t), "nnz": hm.nnz,
            "inverse": inv.kind, "geinv_full_s": inv.seconds,
            "reference_rel_resid": (detail["refine_history"][-1] if "refine_history" in detail else None),
            "sub_block_rel_resid": detail["sub_block_solve"]["rel_resid"]}),
        "cpu_baseline": {"value": value, "unit": "RHS/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "RHS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "detail": detail,
    }
    print(json.dumps(out), flush=True)
    # a dplrgeinv still running past its cap ends with the process
    os._exit(0)


def tree_levels(t) -> int:
    from dplr_gb300 import tree as tr
    return tr.depth(t)


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)

    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan

    t, stats = build_matrix(args, device=str(device))
    t_gen = stats.seconds
    t0 = time.time()
    plan = GpuPlan(t)
    t_upload = time.time() - t0
    torch.cuda.synchronize()
    t0 = time.time()
    plan.factor()
    torch.cuda.synchronize()
    t_factor = time.time() - t0
    precise = args.residual == "sliced"
    t0 = time.time()
    if precise:
        plan.prepare_sliced()
    torch.cuda.synchronize()
    t_slice = time.time() - t0

    g = torch.Generator(device=device)
    g.manual_seed(args.seed + 1000 * rank + 3)
    B = torch.randn(args.rhs, args.n, dtype=torch.float64, device=device, generator=g)
    X = torch.empty_like(B)
    stream = torch.cuda.current_stream(device)
    mixed = args.precision == "mixed"
    t0 = time.time()
    if mixed:
        plan.prepare_mixed(args.mixed_slices)
    torch.cuda.synchronize()
    t_mixed = time.time() - t0

    def run_steps(use_mixed, steps, profile=False):
        """Warm up, then time `steps` refined solves; returns timing and stats."""
        for _ in range(max(3, args.warmup)):
            plan.solve_refined(B, tol=args.tol, maxiter=args.maxiter, out=X, strict=False,
                               precise=precise, mixed=use_mixed)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if profile else None
        if profile:
            sampler.start()
            _native.profile_start()
        l0 = _native.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        resid, iters = [], []
        for _ in range(steps):
            _, res, its = plan.solve_refined(B, tol=args.tol, maxiter=args.maxiter, out=X,
                                             strict=False, precise=precise, mixed=use_mixed)
            resid.append(res)
            iters.append(its)
        e1.record(stream)
        torch.cuda.synchronize()
        out = {"launches": _native.launch_count() - l0, "resid": resid, "iters": iters}
        if profile:
            out["prof"] = _native.profile_stop()
            out["clocks"] = sampler.stop()
        barrier(world)
        ms = e0.elapsed_time(e1)
        out["ms"] = max_over_ranks(ms, world, device)
        return out

    # ---------------- timed region: device-resident inputs (headline path)
    head = run_steps(mixed, args.steps, profile=True)
    X_head = X.clone()                         # the headline solution, checked on the host below
    ms_max = head["ms"]
    value = args.rhs * args.steps * world / (ms_max / 1000.0)
    prof, clocks, launches = head["prof"], head["clocks"], head["launches"]
    resid, iters = head["resid"], head["iters"]
    ms = ms_max
    # ---------------- the same mixed solve with FP64 capacitance arithmetic
    capfp64 = None
    if mixed:
        plan.prepare_mixed(args.mixed_slices, fp64_capacitance=True)
        capfp64 = run_steps(True, args.steps)
        plan.prepare_mixed(args.mixed_slices)
    # ---------------- the plain FP64 GPU solve (FP64 Woodbury sweeps), same residual
    fp64 = run_steps(False, args.steps) if mixed else head
    fp64_value = args.rhs * args.steps * world / (fp64["ms"] / 1000.0)
    # ---------------- one unrefined FP64 Woodbury solve (does not reach the tolerance)
    for _ in range(3):
        plan.solve(B, out=X)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.steps):
        plan.solve(B, out=X)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = max_over_ranks(p0.elapsed_time(p1), world, device)
    R = plan.residual(X, B, precise=precise)
    plain_res = float((R.norm(dim=1) / B.norm(dim=1)).max())
    del R

    # ---------------- end to end: host buffers through the C ABI
    import ctypes
    Bh = B.cpu().pin_memory()
    Xh = torch.empty_like(Bh).pin_memory()
    lib = _native.lib()
    res_c, its_c = ctypes.c_double(), ctypes.c_int()

    def e2e_step():
        rc = lib.dplr_gpu_solve_refined_host(plan.handle, args.rhs, Bh.data_ptr(), args.n,
                                             Xh.data_ptr(), args.n, args.tol, args.maxiter,
                                             (1 if precise else 0) | (2 if mixed else 0),
                                             ctypes.byref(res_c), ctypes.byref(its_c),
                                             stream.cuda_stream)
        if rc != -5:
            _native.check(rc, "dplr_gpu_solve_refined_host")

    e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, device)
    e2e_value = args.rhs * args.steps * world / e2e_s
    nbytes = args.rhs * args.n * 8

    # ---------------- roofline of the dominant kernel
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    name, (kms, kfl, kby, kla) = dom
    tflops = kfl / (kms / 1000.0) / 1e12
    gbs = kby / (kms / 1000.0) / 1e9
    from dplr_gb300 import workloads
    fp64_meas = workloads.fp64_gemm_peak()
    fp64_peak = fp64_meas["tflops"]
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        peaks = json.load(open(peaks_path))
        bf16_peak, peak_src = float(peaks["bf16_tflops_sustained"]), "of measured (sustained bf16)"
    except Exception:
        bf16_peak, peak_src = 1700.0, "of fallback (sustained bf16)"
    # DRAM traffic per launch of the dominant kernel, from the ncu capture summarised
    # in profiles/ (scaled to a full-size launch by the units it processes)
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "traffic_per_launch.json")))
        if name in tr and tr[name].get("n") == args.n and tr[name].get("rhs") == args.rhs:
            traffic = tr[name]["bytes"]
    except Exception:
        traffic = None
    if name.startswith(("sliced_", "mixed_")):
        roofline = {"kernel": name, "bound": "tensor", "achieved": tflops, "peak": bf16_peak,
                    "unit": "TFLOP/s", "frac": tflops / bf16_peak, "traffic": traffic,
                    "algorithmic_gbs": gbs, "share_of_timed": kms / ms, "peak_source": peak_src,
                    "note": "bf16 MMA flops of all slice pairs (tcgen05.mma kind::f16, 128-row tiles)"}
    else:
        roofline = {"kernel": name, "bound": "fp64", "achieved": tflops, "peak": fp64_peak,
                    "unit": "TFLOP/s", "frac": tflops / fp64_peak, "traffic": None,
                    "algorithmic_gbs": gbs, "share_of_timed": kms / ms,
                    "peak_source": "of " + fp64_meas["source"]}
    kernels = {k: {"ms": v[0], "tflops": v[1] / (v[0] / 1e3) / 1e12 if v[0] else 0.0,
                   "gbs": v[2] / (v[0] / 1e3) / 1e9 if v[0] else 0.0, "launches": v[3]}
               for k, v in prof.items()}

    out = {
        "metric": METRIC, "value": value, "unit": "RHS/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+bf16" if mixed else "f64",
        "data": "synthetic",
        "config": workload_config(args, stats, {
            "levels": plan.levels, "nnz": plan.nnz,
            "precision": ((f"mixed: {args.mixed_slices}-slice bf16 Woodbury inner solves on the tensor "
                           "cores, capacitance inverses (FP64) applied from 8 exact slices (rank-128 nodes) or "
                           "in FP64, " if mixed else "fp64 Woodbury inner solves, ") +
                          ("residual from 8 exact bf16 slices with double-double accumulation"
                           if precise else "FP64 residual")),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "setup_s": {"generate": t_gen, "upload": t_upload, "factor": t_factor,
                        "slice": t_slice, "mixed_slices": t_mixed},
            "fp64_gpu_solve": {"value": fp64_value, "unit": "RHS/s",
                               "ms_per_step": fp64["ms"] / args.steps,
                               "refinement_iters": fp64["iters"],
                               "final_rel_resid": fp64["resid"],
                               "converged": all(r <= args.tol for r in fp64["resid"])},
            "mixed_fp64_capacitance": (None if capfp64 is None else {
                "value": args.rhs * args.steps * world / (capfp64["ms"] / 1000.0), "unit": "RHS/s",
                "ms_per_step": capfp64["ms"] / args.steps, "refinement_iters": capfp64["iters"],
                "final_rel_resid": capfp64["resid"],
                "note": "the headline path with every capacitance inverse applied in FP64 arithmetic"}),
            "fp64_plain_solve": {"value": args.rhs * args.steps * world / (plain_ms / 1000.0),
                                 "unit": "RHS/s", "ms_per_step": plain_ms / args.steps,
                                 "rel_resid": plain_res,
                                 "note": "one FP64 Woodbury sweep without refinement"},
            "refinement_iters": iters, "final_rel_resid": resid,
            "converged": all(r <= args.tol for r in resid),
            # flat copies of the comparison the metric names
            "fp64_gpu_solve_rhs_s": fp64_value,
            "fp64_gpu_solve_rel_resid": max(fp64["resid"]),
            "fp64_gpu_solve_converged": all(r <= args.tol for r in fp64["resid"]),
            "mixed_rel_resid": max(resid),
            "mixed_over_fp64": value / fp64_value}),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "RHS/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": launches,
        "roofline": roofline,
        "kernels": kernels,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            threads = os.cpu_count() or 1
            Xh, Bh_np = X_head.cpu().numpy(), B.cpu().numpy()
            hm = HostMatrix(t)
            sec_full, AX = cpu_apply(hm, Xh, threads)
            chk = oracle_check(hm, Xh, Bh_np, AX, 16, threads)
            inv = HostInverse(hm, args.geinv_cap, threads)
            nrhs_cpu = min(args.cpu_rhs, args.rhs)
            cpu_solve_step(hm, inv, Bh_np[:nrhs_cpu], threads)          # warm-up
            sec = cpu_solve_step(hm, inv, Bh_np[:nrhs_cpu], threads)
            inv.close()
            hm.close()
            out["cpu_baseline"] = {
                "value": nrhs_cpu / sec, "unit": "RHS/s", "cores": threads, "kind": "port",
                "sample": (f"one step of the reference's solve on {nrhs_cpu} of the RHS at full size: "
                           f"x = inv(A) b and b - A x by two dplrgepdmm calls of the oracle ({threads} host "
                           f"threads; inv(A) from {inv.kind}, formed before the step), {sec:.2f} s; its FP64 "
                           f"residuals stall above 1e-12 here, so this is an upper bound of the reference's "
                           f"RHS/s at 1e-12"),
                "apply_a_full_s": sec_full, "geinv_full_s": inv.seconds}
            # the same product checks the GPU's solution on the host
            out["config"].update(chk)
        except Exception as exc:  # the baseline must not hide the GPU result
            out.setdefault("cpu_baseline", {"value": None, "unit": "RHS/s"})["error"] = str(exc)
    if rank == 0:
        print(json.dumps(out))
    plan.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_secondary(args):
    """Secondary workloads on one GPU (replicas under torchrun: rank 0 reports)."""
    import torch
    from dplr_gb300 import workloads
    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    try:
        if args.workload == "apply":
            t, stats = build_matrix(args, device=f"cuda:{local}")
            from dplr_gb300.plan import GpuPlan
            plan = GpuPlan(t)
            sampler.start()
            out = workloads.apply_workload(plan, args.n, max(args.steps, 10), args.warmup, ROOT)
        elif args.workload == "batched":
            sampler.start()
            out = workloads.batched_workload(max(args.steps, 10), args.warmup)
        elif args.workload == "ppmm":
            t = workloads.ppmm_input(f"cuda:{local}")
            sampler.start()
            out, got = workloads.ppmm_workload(t, max(args.steps, 3), args.warmup)
            if not args.no_cpu and rank == 0:
                cb, diff = ppmm_cpu_leg(t, got)
                out["cpu_baseline"] = cb
                out["config"]["max_rel_diff_vs_cpu"] = diff
        elif args.workload == "c2":
            t = workloads.c2_input()
            sampler.start()
            out = workloads.c2_workload(t, max(args.steps, 10), args.warmup, ROOT)
            if not args.no_cpu and rank == 0:
                out["cpu_baseline"] = c2_cpu_leg(t)
        elif args.workload == "compress":
            sampler.start()
            out = workloads.compress_workload(max(args.steps, 3), args.warmup,
                                              cpu=not args.no_cpu and rank == 0)
        else:
            sampler.start()
            out = workloads.adjoint_workload(max(args.steps, 5), args.warmup)
    finally:
        clocks = sampler.stop()
    out["clocks"] = clocks
    out.update({"n_gpus": 1, "steps": out.pop("steps", max(args.steps, 10)), "warmup": max(3, args.warmup),
                "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
    if rank == 0:
        print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "solve":
        run_secondary(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
