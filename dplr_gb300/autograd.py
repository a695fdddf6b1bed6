"""Differentiable PLR products and solves (torch.autograd over the C ABI).

The factors are one flat float64 CUDA tensor in the plan's pool layout
(``GpuPlan.read_pool``); gradients come back in the same layout, and
``GpuPlan.pool_blocks`` maps it to the blocks of the tree.

* ``plr_apply(plan, pool, x)``: Y = A X.  Backward: dX = A^T dY (the
  transposed apply), d(pool) from ``dplr_gpu_grad_factors`` (dU, dV, dsig,
  d(leaf) of <dY, A X>).
* ``plr_solve(plan, pool, b)``: X = A^-1 B with the FP64 Woodbury sweep
  (refined with exact-slice residuals when ``refine``).  Backward:
  dB = A^-T G (a transposed sweep over the same factorisation, its per-level
  intermediates recomputed rather than stored), d(pool) = -projection of
  dB X^T onto the factors.

Rows of x / b are right-hand sides (shape (n, m)), as everywhere in the
Python API.
"""
from __future__ import annotations

import torch

from .plan import GpuPlan


def _sync_pool(plan: GpuPlan, pool: torch.Tensor, factor: bool) -> None:
    """Load `pool` into the plan if it is not the values the plan holds, and
    (re)build the Woodbury factorisation (both directions) when asked."""
    key = (pool.data_ptr(), pool._version)
    if getattr(plan, "_pool_key", None) != key:
        plan.write_pool(pool.detach())
        plan._pool_key = key
    if factor and not plan.factored:
        plan.factor()


class _PlrApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pool, x, plan):
        _sync_pool(plan, pool, factor=False)
        y = plan.apply(x.contiguous())
        ctx.save_for_backward(pool, x)
        ctx.plan = plan
        return y

    @staticmethod
    def backward(ctx, dy):
        pool, x = ctx.saved_tensors
        plan = ctx.plan
        _sync_pool(plan, pool, factor=False)
        dy = dy.contiguous()
        dx = plan.apply(dy, trans="T") if ctx.needs_input_grad[1] else None
        dpool = plan.grad_factors(x.contiguous(), dy, 1.0) if ctx.needs_input_grad[0] else None
        return dpool, dx, None


class _PlrSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pool, b, plan, refine):
        _sync_pool(plan, pool, factor=True)
        b = b.contiguous()
        if refine:
            x, _, _ = plan.solve_refined(b, tol=1e-13, maxiter=6, strict=False)
        else:
            x = plan.solve(b)
        ctx.save_for_backward(pool, x)
        ctx.plan = plan
        ctx.refine = refine
        return x

    @staticmethod
    def backward(ctx, g):
        pool, x = ctx.saved_tensors
        plan = ctx.plan
        _sync_pool(plan, pool, factor=True)
        lam = plan.solve(g.contiguous(), trans="T")
        dpool = plan.grad_factors(x, lam, -1.0) if ctx.needs_input_grad[0] else None
        return dpool, (lam if ctx.needs_input_grad[1] else None), None, None


def plr_apply(plan: GpuPlan, pool: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    """Y = A X with A's factors given by `pool` (differentiable in both)."""
    return _PlrApply.apply(pool, x, plan)


def plr_solve(plan: GpuPlan, pool: torch.Tensor, b: torch.Tensor, refine: bool = False) -> torch.Tensor:
    """X = A^-1 B with A's factors given by `pool` (differentiable in both)."""
    return _PlrSolve.apply(pool, b, plan, refine)


def pool_views(plan: GpuPlan, pool: torch.Tensor) -> list[dict]:
    """Per-block views of a pool-layout tensor (U, V: (rank, n) views of the
    column-major n x rank factors; sig; leaf D as a (b, b) view of the
    column-major matrix, i.e. D^T)."""
    out = []
    for blk in plan.pool_blocks():
        if blk["kind"] == "lowrank":
            n, r = blk["n"], blk["rank"]
            out.append({**blk,
                        "U": pool[blk["u"]:blk["u"] + n * r].view(r, n),
                        "V": pool[blk["v"]:blk["v"] + n * r].view(r, n),
                        "S": pool[blk["sig"]:blk["sig"] + r]})
        else:
            b = blk["b"]
            out.append({**blk, "D": pool[blk["d"]:blk["d"] + b * b].view(b, b)})
    return out
