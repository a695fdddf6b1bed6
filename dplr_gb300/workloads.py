"""Secondary benchmark workloads (selected by ``bench.py --workload``).

* ``apply``: the product Y = A X (dplrgepmv / dplrgepdmm) on the 2D
  Gaussian-kernel matrix of the solve benchmark.  The FP64 kernels are timed
  for 1, 16 and 256 right-hand sides; the FP64-accurate float-pair kernels
  (dplr_gpu_prepare_pairs) for 1.  The 1-RHS product is HBM-bound, so it is
  reported as algorithmic GB/s (8 nnz + 16 N bytes) against the measured
  copy bandwidth; the record's value is the float-pair apply.
* ``batched``: 512 independent 1D exponential-kernel matrices, N = 64 2^L
  log-uniform in [1024, 16384], length scale uniform in [0.05, 0.5],
  leaf 64, ranks 1 to 4, 1 to 16 right-hand sides each, FP64; one step is
  one replay of a captured CUDA graph that applies all matrices and one of
  a graph that solves all of them, after the autotuner picked the launch
  shapes.
* ``adjoint``: N = 65536 sorted uniform 1D points, exponential kernel
  length 0.1 + 1e-2 I, leaf 128, rank 16, FP64; one step evaluates
  L = ||A^-1 b - t||^2 and its gradient with respect to b and every factor:
  refactorisation (the factors change between steps of an optimisation),
  solve, transposed solve, factor gradient.

* ``compress``: dense -> PLR compression (dplrd2gep) of the 2D Gaussian
  kernel matrix of 4096 points (2-D uniform, cluster-sorted), 4 levels,
  eps = 1e-8; one step is one host-to-host call (A copied in, the tree
  copied out).  The CPU legs restate the same compression with LAPACK on
  the host cores: dgesvd (the reference's SVD) timed on one half-tree and
  one top-level block, and gesdd (numpy) on the whole matrix.

* ``ppmm``: the PLR x PLR product C := A A + 0.5 C (dplrgeppmm) on the 2D
  Gaussian-kernel matrix of the solve benchmark at N = 16384 (leaf 256,
  ranks up to 64), eps = 1e-8; one step is one host-to-host call (A and C
  uploaded, C's grown tree copied back).  bench.py adds the CPU leg (the
  restatement of the reference's recursion on all host threads, on the
  same inputs), whose result is also the parity check.

Each returns the JSON record of its line; the caller adds clocks.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

from . import _native, gen, tree
from .plan import GpuGraph, GpuPlan


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _peaks(root):
    try:
        p = json.load(open(os.path.join(root, "MEASURED_PEAKS.json")))
        return float(p["hbm_gbs"]), "of measured"
    except Exception:
        return 6800.0, "of fallback"


_FP64_PEAK: dict = {}


def fp64_gemm_peak() -> dict:
    """FP64 roofline denominator measured in this process: cuBLAS DGEMM
    (torch.matmul, float64, 4096^3, 2 n^3 flops), best of 5 after one warm-up,
    timed with CUDA events.  Measured once per process."""
    if _FP64_PEAK:
        return _FP64_PEAK
    n = 4096
    g = torch.Generator(device="cuda").manual_seed(1)
    a = torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")
    c = torch.matmul(a, b)
    best = float("inf")
    for _ in range(5):
        e0, e1 = _events()
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    _FP64_PEAK.update({"tflops": 2.0 * n ** 3 / (best / 1e3) / 1e12,
                       "source": "measured cuBLAS DGEMM 4096^3 in this run (best of 5)"})
    del a, b, c
    return _FP64_PEAK


def apply_workload(plan: GpuPlan, n: int, steps: int, warmup: int, root: str) -> dict:
    """FP64 apply bandwidth for 1, 16 and 256 right-hand sides; the record's
    value is the 1-RHS case."""
    stream = torch.cuda.current_stream()
    hbm, src = _peaks(root)
    fp64 = fp64_gemm_peak()["tflops"]
    rows = {}
    for nrhs in (1, 16, 256):
        tune = plan.autotune(nrhs)             # launch shapes for this right-hand-side count
        g = torch.Generator(device="cuda").manual_seed(11)
        X = torch.randn(nrhs, n, generator=g, dtype=torch.float64, device="cuda")
        Y = torch.empty_like(X)
        by = 8.0 * plan.nnz + 16.0 * n * nrhs
        fl = 2.0 * plan.nnz * nrhs
        for mode in ("persistent", "launches"):
            # the default is one persistent launch; DPLR_GB300_APPLY=launches
            # selects the panel / reduce / expand launches
            if mode == "launches":
                os.environ["DPLR_GB300_APPLY"] = "launches"
            try:
                for _ in range(max(3, warmup)):
                    plan.apply(X, out=Y)
                torch.cuda.synchronize()
                l0 = _native.launch_count()
                e0, e1 = _events()
                e0.record(stream)
                for _ in range(steps):
                    plan.apply(X, out=Y)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / steps
                launches = (_native.launch_count() - l0) / steps
            finally:
                os.environ.pop("DPLR_GB300_APPLY", None)
            rec = {"ms": ms, "gbs": by / (ms / 1e3) / 1e9, "tflops": fl / (ms / 1e3) / 1e12,
                   "frac_hbm": by / (ms / 1e3) / 1e9 / hbm, "frac_fp64": fl / (ms / 1e3) / 1e12 / fp64,
                   # roofline of min(HBM, FP64): the slower of moving the bytes and doing the flops
                   "frac_roofline": max(by / (hbm * 1e9), fl / (fp64 * 1e12)) / (ms / 1e3),
                   "launches_per_apply": launches, "autotune": tune}
            if mode == "persistent":
                rows[nrhs] = rec
            else:
                rows[nrhs]["three_launches"] = rec
    one = rows[1]
    # FP64-accurate 1-RHS apply on the FP32 pipes (float-pair copy of the
    # factors); the FP64 kernels' result on the same vector is the reference
    g = torch.Generator(device="cuda").manual_seed(11)
    X = torch.randn(1, n, generator=g, dtype=torch.float64, device="cuda")
    y64 = plan.apply(X)
    plan.prepare_pairs()
    Y = torch.empty_like(X)
    for _ in range(max(3, warmup)):
        plan.apply(X, out=Y)
    torch.cuda.synchronize()
    l0 = _native.launch_count()
    e0, e1 = _events()
    e0.record(stream)
    for _ in range(steps):
        plan.apply(X, out=Y)
    e1.record(stream)
    torch.cuda.synchronize()
    pms = e0.elapsed_time(e1) / steps
    launches = (_native.launch_count() - l0) // max(steps, 1)
    _native.profile_start()                   # per-kernel split of one more batch of applies
    for _ in range(steps):
        plan.apply(X, out=Y)
    torch.cuda.synchronize()
    kern = {k: {"ms": v[0] / steps, "gbs": v[2] / (v[0] / 1e3) / 1e9 if v[0] else 0.0}
            for k, v in _native.profile_stop().items()}
    by = 8.0 * plan.nnz + 16.0 * n
    pgbs = by / (pms / 1e3) / 1e9
    diff = float((Y - y64).norm() / y64.norm())
    pairs = {"ms": pms, "gbs": pgbs, "frac_hbm": pgbs / hbm, "launches_per_apply": launches,
             "rel_diff_vs_fp64_kernels": diff, "kernels": kern}
    return {
        "metric": "FP64-accurate PLR apply GB/s (1 RHS, float-pair kernels) @N=2^18", "value": pgbs,
        "unit": "GB/s", "ms_per_step": pms, "higher_is_better": True, "dtype": "f32 pairs (48-bit operands)",
        "roofline": {"kernel": "pair apply (split x, panel, reduce, split T, expand)", "bound": "hbm",
                     "achieved": pgbs, "peak": hbm, "unit": "GB/s", "frac": pgbs / hbm, "traffic": None,
                     "peak_source": src,
                     "note": "FP32-pair products (exact high part) with compensated sums; the FP64 kernels "
                             "are capped by FP64 issue (fp64_1rhs.fp64_bound_gbs)"},
        "pairs_1rhs": pairs,
        "fp64_by_rhs": rows,
        "fp64_1rhs": {"gbs": one["gbs"], "frac_hbm": one["frac_hbm"],
                      "fp64_bound_gbs": fp64 * 1e12 / 2.0 * 8.0 / 1e9,
                      "fp64_peak_tflops": fp64, "fp64_peak_source": fp64_gemm_peak()["source"]},
        "config": {"workload": f"apply of the 2D Gaussian-kernel PLR, N={n}, nnz={plan.nnz}",
                   "bytes_per_rhs": "8*nnz + 16*N (factors read once, x read and y written once)"},
    }


def batched_trees(count: int = 512, seed: int = 0):
    rng = np.random.default_rng(seed)
    trees, nrhs = [], []
    for i in range(count):
        L = int(rng.integers(4, 9))                   # N = 64 * 2^L in [1024, 16384]
        n = 64 << L
        x = np.sort(rng.uniform(0.0, 1.0, n))
        trees.append(gen.exp1d_tree(x, ell=float(rng.uniform(0.05, 0.5)), shift=1e-2, leaf=64,
                                    rank=int(rng.integers(1, 5)), seed=seed * 100000 + i))
        nrhs.append(int(rng.integers(1, 17)))
    return trees, nrhs


# right-hand-side buckets of the batched workload: measured on the GB300,
# (1, 2, 4, 8, 12, 16) gave 156.9 K RHS/s, (2, 4, 8, 16) 145.2 K and
# (1, 2, 3, 4, 6, 8, 12, 16) 151.8 K (more groups, more replays)
RHS_BUCKETS = (1, 2, 4, 8, 12, 16)


def batched_workload(steps: int, warmup: int, count: int = 512) -> dict:
    """The 512 matrices grouped by their right-hand-side count into batch
    plans of at most 1, 2, 4, 8, 12 and 16 stacked columns (so a matrix with
    one right-hand side does not pay for 16); each plan is autotuned and
    factored, and one step replays every plan's apply graph and
    refined-solve graph."""
    t0 = time.time()
    trees, nrhs = batched_trees(count)
    t_gen = time.time() - t0
    groups = []
    lo = 0
    for hi in RHS_BUCKETS:
        idx = [i for i, k in enumerate(nrhs) if lo < k <= hi]
        lo = hi
        if idx:
            groups.append({"idx": idx, "n": max(nrhs[i] for i in idx)})
    t_up = t_fac = 0.0
    g = torch.Generator(device="cuda").manual_seed(5)
    for grp in groups:
        gt = [trees[i] for i in grp["idx"]]
        t0 = time.time()
        plan = GpuPlan.batch(gt)
        t_up += time.time() - t0
        grp["tune"] = plan.autotune(grp["n"])
        torch.cuda.synchronize()
        t0 = time.time()
        plan.factor()
        torch.cuda.synchronize()
        t_fac += time.time() - t0
        X = torch.zeros(grp["n"], plan.m, dtype=torch.float64, device="cuda")
        for o, i in zip(plan.offsets(), grp["idx"]):       # matrix i uses its first nrhs_i columns
            X[:nrhs[i], o:o + trees[i].size] = torch.randn(nrhs[i], trees[i].size, generator=g,
                                                           dtype=torch.float64, device="cuda")
        grp.update(plan=plan, X=X, Y=torch.empty_like(X), Z=torch.empty_like(X))
        grp["ga"] = GpuGraph(plan, "A", X, grp["Y"])
        grp["gs"] = GpuGraph(plan, "C", X, grp["Z"])       # solve + one FP64-residual correction

    def step():
        for grp in groups:
            grp["ga"].launch()
            grp["gs"].launch()

    stream = torch.cuda.current_stream()
    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize()
    l0 = _native.launch_count()
    e0, e1 = _events()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = _native.launch_count() - l0
    ms = e0.elapsed_time(e1) / steps
    # algorithmic FP64 flops of one step, launch by launch (graph replays
    # carry no events), counted on the right-hand sides the matrices have:
    # each group's stacked count scaled by its real columns
    flops, kern = 0.0, {}
    for grp in groups:
        plan = grp["plan"]
        _native.profile_start()
        plan.apply(grp["X"], out=grp["Y"])
        _refined_once(plan, grp["X"], grp["Z"])
        prof = _native.profile_stop()
        real = sum(nrhs[i] for i in grp["idx"]) / (grp["n"] * len(grp["idx"]))
        flops += real * sum(v[1] for v in prof.values())
        for k, v in prof.items():
            kern[k] = kern.get(k, 0.0) + v[0]
    fp64 = fp64_gemm_peak()
    tflops = flops / (ms / 1e3) / 1e12
    # accuracy of every matrix's own right-hand sides, from the exact-slice
    # residual of the replayed refined solve (FP64 residuals cannot resolve
    # below ~1e-12 on the longer length scales); and the same graph with
    # exact-slice residuals in its corrections
    worst, exact_worst, exact_ms, exact_kernels = 0.0, 0.0, 0.0, 0
    for grp in groups:
        plan = grp["plan"]
        plan.prepare_sliced()

        def worst_resid(Zs):
            R = plan.residual(Zs, grp["X"], precise=True)
            w = 0.0
            for o, i in zip(plan.offsets(), grp["idx"]):
                k, n_i = nrhs[i], trees[i].size
                w = max(w, float((R[:k, o:o + n_i].norm(dim=1) / grp["X"][:k, o:o + n_i].norm(dim=1)).max()))
            return w

        worst = max(worst, worst_resid(grp["Z"]))
        Z2 = torch.empty_like(grp["X"])
        gx = GpuGraph(plan, "R", grp["X"], Z2)
        gx.launch()
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record(stream)
        gx.launch()
        e1.record(stream)
        torch.cuda.synchronize()
        exact_ms += e0.elapsed_time(e1)
        exact_kernels += gx.kernels
        exact_worst = max(exact_worst, worst_resid(Z2))
        gx.close()
    total_rhs = sum(nrhs)
    out = {
        "metric": "batched PLR apply+refined solve RHS/s (512 matrices, uneven N/rank/RHS, graph replay)",
        "value": 2.0 * total_rhs / (ms / 1e3), "unit": "RHS/s", "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f64", "gpu_launches": launches,
        "roofline": {"kernel": "whole step (apply graphs + refined-solve graphs)", "bound": "fp64",
                     "achieved": tflops, "peak": fp64["tflops"], "unit": "TFLOP/s",
                     "frac": tflops / fp64["tflops"], "traffic": None, "peak_source": "of " + fp64["source"],
                     "algorithmic": f"{flops:.4g} flop per step (the launches' algorithmic counts, scaled to "
                                    f"the right-hand sides each matrix has)"},
        "config": {"workload": "512 1D exponential-kernel PLR matrices, N in [1024, 16384], leaf 64, "
                               "ranks 1-4, 1-16 RHS each, grouped by RHS count into batch plans of <= 1, 2, 4, 8, "
                               "12, 16 columns; per step every plan's apply graph and refined-solve graph "
                               "(one correction with FP64 residuals: further ones stay at the rounding floor)",
                   "matrices": count, "rows_total": sum(t.size for t in trees), "rhs_total": total_rhs,
                   "groups": [{"matrices": len(grp["idx"]), "rhs_stacked": grp["n"],
                               "graph_kernels": {"apply": grp["ga"].kernels, "refined_solve": grp["gs"].kernels},
                               "autotune": grp["tune"]} for grp in groups],
                   "refined_solve_max_rel_resid": worst,
                   "refined_solve_exact_residual": {
                       "ms": exact_ms, "rhs_per_s": total_rhs / (exact_ms / 1e3) if exact_ms > 0 else None,
                       "max_rel_resid": exact_worst, "kernels": exact_kernels,
                       "note": "refined-solve graphs with two exact-slice-residual corrections "
                               "(tcgen05 kernels; the 64-row leaves and blocks are stored as half-empty "
                               "128-row tiles)"},
                   "kernels_ms": kern,
                   "setup_s": {"generate": t_gen, "upload": t_up, "factor": t_fac}},
    }
    for grp in groups:
        grp["ga"].close()
        grp["gs"].close()
        grp["plan"].close()
    return out


def _refined_once(plan, b, x):
    """Solve + one correction launch by launch (what the 'C' graph
    replays), for profiling."""
    x0 = plan.solve(b, out=x)
    for _ in range(1):
        r = plan.residual(x0, b, precise=False)
        x0 += plan.solve(r)
    return x0


def adjoint_workload(steps: int, warmup: int, n: int = 65536) -> dict:
    from .autograd import plr_solve
    rng = np.random.default_rng(0)
    x = np.sort(rng.uniform(0.0, 1.0, n))
    t = gen.exp1d_tree(x, ell=0.1, shift=1e-2, leaf=128, rank=16, seed=1)
    plan = GpuPlan(t)
    pool = plan.read_pool()
    b = torch.tensor(rng.standard_normal((1, n)), device="cuda")
    tt = torch.tensor(rng.standard_normal((1, n)), device="cuda")

    def step():
        p = pool.clone().requires_grad_()     # new factor values: refactorised inside
        bb = b.clone().requires_grad_()
        xs = plr_solve(plan, p, bb)
        loss = ((xs - tt) ** 2).sum()
        loss.backward()
        return loss, p.grad, bb.grad

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    l0 = _native.launch_count()
    e0, e1 = _events()
    e0.record(stream)
    for _ in range(steps):
        loss, gp, gb = step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    launches = _native.launch_count() - l0
    # algorithmic FP64 work of one step, from the profiled launches
    _native.profile_start()
    step()
    prof = _native.profile_stop()
    flops = sum(v[1] for v in prof.values())
    fp64 = fp64_gemm_peak()
    tflops = flops / (ms / 1e3) / 1e12
    # spot check against central differences (h = 1e-6) on two factor entries
    blocks = plan.pool_blocks()
    idx = [blocks[0]["u"] + 7, blocks[len(blocks) // 2]["d"] if "d" in blocks[len(blocks) // 2]
           else blocks[len(blocks) // 2]["v"] + 3]
    fd = []
    with torch.no_grad():
        for i in idx:
            pp, pm = pool.clone(), pool.clone()
            pp[i] += 1e-6
            pm[i] -= 1e-6
            lp = float(((plr_solve(plan, pp, b) - tt) ** 2).sum())
            lm = float(((plr_solve(plan, pm, b) - tt) ** 2).sum())
            fd.append({"index": i, "fd": (lp - lm) / 2e-6, "grad": float(gp[i])})
    return {
        "metric": "adjoint steps/s: loss=||A^-1 b - t||^2 and gradients (b, U, V, sig, leaves) @N=65536",
        "value": 1000.0 / ms, "unit": "steps/s", "ms_per_step": ms, "higher_is_better": True,
        "dtype": "f64", "gpu_launches": launches,
        "roofline": {"kernel": "whole step (factorisation: leaf and capacitance inverses, truncated sweeps; "
                               "solve, transposed solve)", "bound": "fp64", "achieved": tflops,
                     "peak": fp64["tflops"], "unit": "TFLOP/s", "frac": tflops / fp64["tflops"], "traffic": None,
                     "peak_source": "of " + fp64["source"],
                     "algorithmic": f"{flops:.4g} flop per step (the profiled launches' algorithmic counts; "
                                    f"inverses at 2 n^3)"},
        "config": {"workload": "1D exponential kernel, N=65536, leaf 128, rank 16; factorisation, solve, "
                               "transposed solve and factor gradient per step",
                   "pool_doubles": plan.pool_size(), "loss": float(loss), "fd_check": fd,
                   "kernels_ms": {k: v[0] for k, v in prof.items()}},
    }


def gauss2d_dense(m: int, seed: int = 0, width: float = 0.05, shift: float = 1e-3) -> np.ndarray:
    """exp(-|p_i - p_j|^2 / width) + shift I for m uniform points in the unit
    square, sorted into 16 x 16 cells so that index blocks are clusters."""
    pts = np.random.default_rng(seed).random((m, 2))
    pts = pts[np.argsort(np.floor(pts[:, 0] * 16) * 16 + pts[:, 1])]
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    return np.exp(-d2 / width) + shift * np.eye(m)


def _lapack_compress(a: np.ndarray, eps: float, nlvl: int, driver: str):
    """The compression of src/dplrd2p.c:186 on the host with one LAPACK SVD
    driver; returns the ranks in DPLR's order."""
    import scipy.linalg as sl
    ranks = []

    def rec(blk, e, lv):
        if lv == 0:
            return
        e2 = e / 2.0 if lv == 1 else e / 4.0
        h = blk.shape[0] // 2
        for off in (blk[:h, h:], blk[h:, :h]):
            s = sl.svd(off, full_matrices=False, compute_uv=True, lapack_driver=driver)[1]
            ranks.append(int(np.argmax(s < e2)) if np.any(s < e2) else len(s))
        rec(blk[:h, :h], e2, lv - 1)
        rec(blk[h:, h:], e2, lv - 1)

    rec(a, eps, nlvl)
    return ranks


def compress_workload(steps: int, warmup: int, m: int = 4096, nlvl: int = 4, eps: float = 1e-8,
                      cpu: bool = True) -> dict:
    from .compress import d2gep
    a = np.asfortranarray(gauss2d_dense(m))
    times = {}
    launches = 0
    for workers in (1, 0):
        for _ in range(max(3, warmup) if workers == 0 else 1):
            t = d2gep(a, eps, nlvl, workers)
        torch.cuda.synchronize()
        k = steps if workers == 0 else max(1, steps // 3)
        l0 = _native.launch_count()
        t0 = time.perf_counter()
        for _ in range(k):
            t = d2gep(a, eps, nlvl, workers)
        times[workers] = (time.perf_counter() - t0) / k
        launches = (_native.launch_count() - l0) // k
    ranks = tree.ranks_by_level(t)
    out_bytes = 8 * _stored(t)
    sec = times[0]
    rec = {
        "metric": _compress_metric(m, nlvl, eps),
        "value": 1.0 / sec, "unit": "compressions/s", "ms_per_step": sec * 1e3, "higher_is_better": True,
        "dtype": "f64", "gpu_launches": launches, "steps": steps,
        "e2e": {"value": 1.0 / sec, "unit": "compressions/s", "h2d_bytes_per_step": 8 * m * m,
                "d2h_bytes_per_step": out_bytes},
        "config": {"workload": _compress_workload_name(m, nlvl, eps) + "; "
                               "blocks >= 512: verified sketch (own Gaussian, FP64 GEMM and norm kernels; "
                               "cuSOLVER QR and SVD of the sketch), smaller blocks: cuSOLVER gesvd",
                   "ms_one_worker": times[1] * 1e3, "ms_default_workers": sec * 1e3,
                   "max_rank_by_level": ranks},
    }
    if cpu:
        smp = _compress_cpu_sample(a, eps, nlvl)
        t0 = time.perf_counter()
        dd = _lapack_compress(a, eps, nlvl, "gesdd")
        t_dd = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": 1.0 / smp["seconds"], "unit": "compressions/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": smp["sample"]}
        rec["config"]["cpu_gesdd_s"] = t_dd
        rec["config"]["ranks_match_gesdd"] = dd == _ranks_all(t)
        rec["config"]["half_ranks_match"] = smp["half_ranks"] == _ranks_all(t.nw)
    return rec


def _compress_metric(m: int, nlvl: int, eps: float) -> str:
    return f"dense->PLR compressions/s (dplrd2gep, N={m}, {nlvl} levels, eps={eps:g})"


def _compress_workload_name(m: int, nlvl: int, eps: float) -> str:
    return (f"2D Gaussian kernel, {m} uniform points in the unit square (width 0.05, shift 1e-3), "
            f"{nlvl} levels, eps {eps:g}; host A in, host tree out")


def _compress_cpu_sample(a: np.ndarray, eps: float, nlvl: int) -> dict:
    """The reference's compression on the host cores (LAPACK dgesvd, the SVD
    src/dplrd2p.c calls, scipy/OpenBLAS on all threads), timed on one
    half-tree and one top-level block; the whole compression is two of
    each."""
    import scipy.linalg as sl
    m = a.shape[0]
    h = m // 2
    t0 = time.perf_counter()
    half = _lapack_compress(a[:h, :h], eps / 4.0, nlvl - 1, "gesvd")
    t_half = time.perf_counter() - t0
    t0 = time.perf_counter()
    sl.svd(a[:h, h:], full_matrices=False, lapack_driver="gesvd")
    t_top = time.perf_counter() - t0
    return {"seconds": 2 * t_top + 2 * t_half, "half_ranks": half,
            "sample": (f"LAPACK dgesvd (the reference's SVD, scipy/OpenBLAS, all host threads): one "
                       f"half-tree ({h}, {nlvl - 1} levels) {t_half:.2f} s and one top-level block "
                       f"{t_top:.2f} s timed; whole compression = 2 x both")}


def compress_reference(steps: int, warmup: int, m: int = 4096, nlvl: int = 4, eps: float = 1e-8) -> dict:
    """The reference arm of the compression workload (host cores only)."""
    a = np.asfortranarray(gauss2d_dense(m))
    for _ in range(max(0, warmup)):
        _compress_cpu_sample(a, eps, nlvl)
    runs = [_compress_cpu_sample(a, eps, nlvl) for _ in range(max(1, steps))]
    sec = sorted(r["seconds"] for r in runs)[len(runs) // 2]
    return {
        "metric": _compress_metric(m, nlvl, eps), "value": 1.0 / sec, "unit": "compressions/s",
        "ms_per_step": sec * 1e3, "higher_is_better": True, "dtype": "f64", "steps": len(runs),
        "impl": "reference",
        "cpu_baseline": {"value": 1.0 / sec, "unit": "compressions/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": runs[0]["sample"]},
        "e2e": {"value": 1.0 / sec, "unit": "compressions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "config": {"workload": _compress_workload_name(m, nlvl, eps), "parallelism": "host cores"},
    }


def _stored(t) -> int:
    """Doubles held by the tree: n^2 per leaf, (2 n + 1) r per low-rank block."""
    if isinstance(t, tree.HNode):
        return sum(_stored(c) for c in (t.nw, t.ne, t.se, t.sw))
    if isinstance(t, tree.LowRank):
        return (2 * t.size + 1) * t.rank
    return t.size * t.size


def _ranks_all(t) -> list:
    """Low-rank block ranks in DPLR's depth-first NE, SW, NW, SE order."""
    out = []

    def walk(nd):
        if isinstance(nd, tree.HNode):
            out.extend([nd.ne.rank, nd.sw.rank])
            walk(nd.nw)
            walk(nd.se)

    walk(t)
    return out


def _max_rel_diff(a, b) -> float:
    """Largest difference of two trees of one structure, relative to the
    largest entry of the node it occurs in; inf if structures, ranks or
    capacities differ."""
    if type(a) is not type(b) or a.size != b.size:
        return float("inf")
    if isinstance(a, tree.HNode):
        return max(_max_rel_diff(getattr(a, k), getattr(b, k)) for k in ("nw", "ne", "se", "sw"))
    if isinstance(a, tree.LowRank):
        if a.rank != b.rank or a.capacity != b.capacity:
            return float("inf")
        pairs = [(a.u, b.u), (a.v, b.v), (a.sig, b.sig)]
    else:
        pairs = [(a.d, b.d)]
    out = 0.0
    for x, y in pairs:
        if y.size:
            out = max(out, float(np.abs(x - y).max()) / max(1.0, float(np.abs(y).max())))
    return out


PPMM = {"n": 16384, "leaf": 256, "rmax": 64, "eps": 1e-8}


def ppmm_input(device: str):
    """A of the product workload: the 2D Gaussian-kernel PLR of the solve
    benchmark at N = 16384 (leaf 256, ranks up to 64)."""
    from . import gen_gpu
    return gen_gpu.kernel_tree_2d(n=PPMM["n"], leaf=PPMM["leaf"], rmax=PPMM["rmax"], seed=0, device=device)


def ppmm_workload(t, steps: int, warmup: int):
    """C := A A + 0.5 C (C = A) through dplr_gpu_geppmm, host trees in and
    out; returns the record and the last product."""
    n, eps = t.size, PPMM["eps"]
    lib = _native.lib()
    ca = tree.to_c(t)
    nw = max(3, warmup)
    cs = [tree.to_c(t) for _ in range(nw + steps)]
    try:
        def call(c):
            rc = lib.dplr_gpu_geppmm(b"N", b"N", n, 1.0, ca, ca, 0.5, c, eps, None)
            _native.check(rc, "dplr_gpu_geppmm")

        for i in range(nw):
            call(cs[i])
        torch.cuda.synchronize()
        l0 = _native.launch_count()
        t0 = time.perf_counter()
        for i in range(steps):
            call(cs[nw + i])
        sec = (time.perf_counter() - t0) / steps
        launches = (_native.launch_count() - l0) // steps
        got = tree.from_c(cs[-1])
        # the device kernels of one more product, timed on their stream
        extra = tree.to_c(t)
        try:
            _native.profile_start()
            call(extra)
            prof = _native.profile_stop()
        finally:
            tree.free_c(extra)
    finally:
        tree.free_c(ca)
        for c in cs:
            tree.free_c(c)
    h2d = 8 * (2 * tree.nnz(t) + 2 * n)          # A and C (two copies of the matrix)
    d2h = 8 * _stored(got)
    rec = {
        "metric": _ppmm_metric(n),
        "value": 1.0 / sec, "unit": "products/s", "ms_per_step": sec * 1e3, "higher_is_better": True,
        "dtype": "f64", "gpu_launches": launches, "steps": steps,
        "e2e": {"value": 1.0 / sec, "unit": "products/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "config": {"workload": _ppmm_workload_name(n, PPMM["leaf"], PPMM["rmax"], eps),
                   "ranks_in": tree.ranks_by_level(t), "ranks_out": tree.ranks_by_level(got),
                   "stored_doubles_in": _stored(t), "stored_doubles_out": _stored(got),
                   "kernels_ms": {k: v[0] for k, v in prof.items()}},
    }
    if prof:
        # the dominant FP64 product kernel of one product against the run's DGEMM rate
        name, (kms, kfl, _, _) = max(prof.items(), key=lambda kv: kv[1][0])
        fp64 = fp64_gemm_peak()
        ach = kfl / (kms / 1e3) / 1e12 if kms > 0 else 0.0
        rec["roofline"] = {"kernel": f"{name} (FP64 apply kernels of the product)", "bound": "fp64", "achieved": ach,
                           "peak": fp64["tflops"], "unit": "TFLOP/s", "frac": ach / fp64["tflops"], "traffic": None,
                           "peak_source": "of " + fp64["source"],
                           "note": "device kernels are part of the step; the rest moves the host trees"}
    return rec, got


def _ppmm_metric(n: int) -> str:
    return f"PLR x PLR products/s (dplrgeppmm C := A A + 0.5 C, N={n}, host trees in and out)"


def _ppmm_workload_name(n: int, leaf: int, rmax: int, eps: float) -> str:
    return f"2D Gaussian kernel PLR, N={n}, leaf {leaf}, ranks up to {rmax}; C := A A + 0.5 C with eps {eps:g}"


def ppmm_reference_record(seconds: list) -> dict:
    """The reference arm's line of the product workload from the timed
    products (host cores)."""
    sec = sorted(seconds)[len(seconds) // 2]
    n = PPMM["n"]
    return {
        "metric": _ppmm_metric(n), "value": 1.0 / sec, "unit": "products/s", "ms_per_step": sec * 1e3,
        "higher_is_better": True, "dtype": "f64", "steps": len(seconds), "impl": "reference",
        "cpu_baseline": {"value": 1.0 / sec, "unit": "products/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "whole products by the restatement of src/dplrppmm.c (numpy BLAS on all "
                                   "host threads), median of the timed steps"},
        "e2e": {"value": 1.0 / sec, "unit": "products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "config": {"workload": _ppmm_workload_name(n, PPMM["leaf"], PPMM["rmax"], PPMM["eps"]),
                   "parallelism": "host cores"},
    }


# --------------------------------------------------------------------------
# C2: plain FP64 multi-RHS products at scale
# --------------------------------------------------------------------------

C2 = {"n": 131072, "leaf": 256, "rank": 32, "ell": 0.05, "shift": 1e-2, "rhs": 64, "seed": 0}


def c2_input():
    """The fixed-rank 1D exponential-kernel PLR: N = 131072 sorted uniform
    points on [0, 1], exp(-|x_i - x_j| / 0.05) + 1e-2 I, leaf 256 (9
    levels).  Every off-diagonal block of this kernel is exactly rank one
    (it is semiseparable), so a rank-32 truncated SVD of it is the exact
    rank-one factor plus 31 orthonormal tail columns with round-off-level
    singular values; gen.exp1d_tree builds that without the dense matrix.
    dplrnz = 2 N sum(r) + N b = 109,051,904 stored doubles (872 MB)."""
    x = np.sort(np.random.default_rng(C2["seed"]).uniform(0.0, 1.0, C2["n"]))
    return gen.exp1d_tree(x, ell=C2["ell"], shift=C2["shift"], leaf=C2["leaf"], rank=C2["rank"],
                          seed=C2["seed"] + 1)


def c2_rhs(device: str = "cuda") -> torch.Tensor:
    g = torch.Generator(device="cpu").manual_seed(C2["seed"] + 2)
    return torch.randn(C2["rhs"], C2["n"], generator=g, dtype=torch.float64).to(device)


def _timed(fn, steps: int, warmup: int):
    """Mean device milliseconds of fn() over `steps` calls after warm-up,
    CUDA events on the current stream; factors (> L2) are re-read every call."""
    stream = torch.cuda.current_stream()
    for _ in range(max(3, warmup)):
        fn()
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def c2_workload(t, steps: int, warmup: int, root: str) -> dict:
    """dplrgepdmm (Y = A X, 64 RHS) and the inverse apply on the C2 matrix.

    The record's value is the product (RHS/s); the inverse apply is reported
    twice: DPLR's way (the explicit inverse B = inv(A) made by the drop-in
    dplrgeinv, then B X) and this library's Woodbury solve refined to 1e-12.
    """
    n, nrhs = t.size, C2["rhs"]
    X = c2_rhs()
    plan = GpuPlan(t)
    Y = torch.empty_like(X)
    l0 = _native.launch_count()
    ms_apply = _timed(lambda: plan.apply(X, out=Y), steps, warmup)
    launches = (_native.launch_count() - l0) // (steps + max(3, warmup))
    flops = 2.0 * plan.nnz * nrhs
    fp64 = fp64_gemm_peak()
    tflops = flops / (ms_apply / 1e3) / 1e12
    # explicit inverse (DPLR's dplrgeinv, on the GPU through the drop-in) and its apply
    a = tree.to_c(t)
    b_inv = tree.new_empty()
    t0 = time.perf_counter()
    info = _native.api().geinv(n, a, b_inv, 0.0)
    t_inv = time.perf_counter() - t0
    if info != 0:
        raise RuntimeError(f"dplrgeinv failed: info {info}")
    nnz_inv = _native.api().nz(n, b_inv)
    pinv = GpuPlan(b_inv)
    tree.free_c(b_inv)
    tree.free_c(a)
    Z = torch.empty_like(X)
    ms_inv = _timed(lambda: pinv.apply(X, out=Z), steps, warmup)
    res_inv = plan.residual(Z, X, precise=False)
    rel_inv = float((res_inv.norm(dim=1) / X.norm(dim=1)).max())
    del res_inv
    pinv.close()
    # Woodbury factorisation + refined solve
    t0 = time.perf_counter()
    plan.factor()
    torch.cuda.synchronize()
    t_fac = time.perf_counter() - t0
    plan.prepare_sliced()                    # FP64 residuals stall near 4e-12 on this matrix
    W = torch.empty_like(X)
    info = {}

    def solve():
        _, info["res"], info["its"] = plan.solve_refined(X, tol=1e-12, maxiter=8, out=W, strict=False,
                                                         precise=True)
    ms_solve = _timed(solve, steps, warmup)
    plan.close()
    return {
        "metric": f"PLR product RHS/s (dplrgepdmm, N={n}, rank {C2['rank']}, {nrhs} RHS, FP64)",
        "value": nrhs / (ms_apply / 1e3), "unit": "RHS/s", "ms_per_step": ms_apply,
        "higher_is_better": True, "dtype": "f64", "gpu_launches": launches,
        "roofline": {"kernel": "FP64 apply (panel, reduce, expand)", "bound": "fp64", "achieved": tflops,
                     "peak": fp64["tflops"], "unit": "TFLOP/s", "frac": tflops / fp64["tflops"],
                     "traffic": None, "peak_source": "of " + fp64["source"],
                     "algorithmic": f"2 nnz n = {flops:.4g} flop, 8 nnz + 16 N n = "
                                    f"{8.0 * plan.nnz + 16.0 * n * nrhs:.4g} bytes"},
        "config": {"workload": (f"1D exponential kernel (l={C2['ell']}, +{C2['shift']:g} I) PLR, N={n}, leaf "
                                f"{C2['leaf']}, 9 levels, fixed rank {C2['rank']} (exact rank-1 factor + "
                                f"round-off tail), {nrhs} standard-normal RHS"),
                   "nnz": plan.nnz, "l2": "factors (872 MB) larger than L2",
                   "inverse_apply_explicit": {"ms": ms_inv, "rhs_per_s": nrhs / (ms_inv / 1e3),
                                              "nnz_inverse": nnz_inv, "geinv_s": t_inv,
                                              "max_rel_resid_fp64": rel_inv},
                   "solve_woodbury_refined": {"ms": ms_solve, "rhs_per_s": nrhs / (ms_solve / 1e3),
                                              "factor_s": t_fac, "rel_resid": info.get("res"),
                                              "corrections": info.get("its")}},
    }
