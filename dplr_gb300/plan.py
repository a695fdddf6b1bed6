"""Device-resident PLR matrices: the Python face of the plan API.

A ``GpuPlan`` owns one ``dplr_gpu_plan`` (block table + factor pool in
HBM) built from a host tree.  Right-hand sides are torch CUDA tensors of
shape (n, m), float64, contiguous: row j is column j of the column-major
m x n block the C ABI sees (leading dimension m).  All calls go through
libdplr_gb300.so; there is no other code path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native, tree


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream


def _check_block(x: torch.Tensor, m: int, name: str) -> None:
    if not (x.is_cuda and x.dtype == torch.float64 and x.dim() == 2 and x.shape[1] == m
            and x.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous CUDA float64 tensor of shape (n, {m})")


class GpuPlan:
    def __init__(self, node_or_cptr, stream=None, _handle=None):
        lib = _native.lib()
        self._owned_c = None
        if _handle is not None:
            self._h = _handle
            mm = ctypes.c_int()
            lib.dplr_gpu_plan_info(self._h, ctypes.byref(mm), None, None, None)
            self.m = mm.value
        else:
            if isinstance(node_or_cptr, (tree.Dense, tree.HNode)):
                cptr = tree.to_c(node_or_cptr)
                self._owned_c = cptr
            else:
                cptr = node_or_cptr
            self.m = int(cptr.contents.size)
            h = ctypes.c_void_p()
            _native.check(lib.dplr_gpu_plan_create(self.m, cptr, _stream_ptr(stream), ctypes.byref(h)),
                          "dplr_gpu_plan_create")
            self._h = h
            if self._owned_c is not None:
                tree.free_c(self._owned_c)
                self._owned_c = None
        mm, nnz, lev, mr = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
        lib.dplr_gpu_plan_info(self._h, ctypes.byref(mm), ctypes.byref(nnz), ctypes.byref(lev),
                               ctypes.byref(mr))
        self.nnz, self.levels, self.max_rank = nnz.value, lev.value, mr.value
        self.factored = False
        self.factored_transposed = False
        self.sliced = False
        self.mixed = False
        self.pairs = False

    RESIDUAL_SLICED = 1
    SOLVE_MIXED = 2

    @classmethod
    def batch(cls, trees: list, stream=None) -> "GpuPlan":
        """One plan over many independent matrices (block diagonal): matrix i
        occupies rows offsets()[i] : offsets()[i] + trees[i].size."""
        lib = _native.lib()
        cptrs = [tree.to_c(t) for t in trees]
        try:
            arr = (tree.PDPlrMtx * len(cptrs))(*cptrs)
            ms = (ctypes.c_int * len(trees))(*[t.size for t in trees])
            h = ctypes.c_void_p()
            _native.check(lib.dplr_gpu_batch_create(len(trees), ms, arr, _stream_ptr(stream),
                                                    ctypes.byref(h)), "dplr_gpu_batch_create")
        finally:
            for c in cptrs:
                tree.free_c(c)
        return cls(None, _handle=h)

    def offsets(self) -> list[int]:
        """First row of every matrix of a batch ([0] for a single matrix)."""
        lib = _native.lib()
        cnt = ctypes.c_int()
        _native.check(lib.dplr_gpu_batch_offsets(self._h, ctypes.byref(cnt), None), "dplr_gpu_batch_offsets")
        rows = (ctypes.c_int * cnt.value)()
        _native.check(lib.dplr_gpu_batch_offsets(self._h, None, rows), "dplr_gpu_batch_offsets")
        return list(rows)

    def autotune(self, n: int, stream=None) -> dict:
        """Pick the fastest panel chunk length and right-hand-side tile of the
        FP64 apply for n right-hand sides (call before factor())."""
        c, nb, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _native.check(_native.lib().dplr_gpu_autotune(self._h, int(n), _stream_ptr(stream), ctypes.byref(c),
                                                      ctypes.byref(nb), ctypes.byref(ms)), "dplr_gpu_autotune")
        form = _native.lib().dplr_gpu_apply_form(self._h)
        return {"chunk_rows": c.value, "nb_cap": nb.value, "apply_ms": ms.value,
                "apply_form": "three launches" if form == 1 else "persistent"}

    def prepare_mixed(self, slices: int = 7, fp64_capacitance: bool = False, stream=None) -> None:
        """Sliced factor copies (3 to 7 bf16 slices) for the low-precision inner
        solve; the capacitance inverses apply from 8 exact slices on the tensor
        cores (rank-128 nodes) unless fp64_capacitance."""
        _native.check(_native.lib().dplr_gpu_prepare_mixed_caps(self._h, int(slices), int(bool(fp64_capacitance)),
                                                               _stream_ptr(stream)), "dplr_gpu_prepare_mixed")
        self.mixed = True
        self.mixed_slices = int(slices)

    def scal(self, alpha: float, stream=None) -> None:
        """A := alpha A on the device (dplrscal's sign convention); the
        factorisation and sliced copies must be rebuilt afterwards."""
        _native.check(_native.lib().dplr_gpu_scal(self._h, float(alpha), _stream_ptr(stream)), "dplr_gpu_scal")
        self.factored = self.factored_transposed = self.sliced = self.mixed = False

    def adpy(self, alpha: float, d: torch.Tensor, stream=None) -> None:
        """A := alpha diag(d) + A on the device (d: CUDA float64, m entries)."""
        if not (d.is_cuda and d.dtype == torch.float64 and d.is_contiguous() and d.numel() == self.m):
            raise ValueError(f"d must be a contiguous CUDA float64 tensor of {self.m} entries")
        _native.check(_native.lib().dplr_gpu_adpy(self._h, float(alpha), d.data_ptr(), _stream_ptr(stream)),
                      "dplr_gpu_adpy")
        self.factored = self.factored_transposed = self.sliced = self.mixed = False

    def copy(self, stream=None) -> "GpuPlan":
        """A new plan equal to this one, made on the device (dplrcpy)."""
        h = ctypes.c_void_p()
        _native.check(_native.lib().dplr_gpu_plan_copy(self._h, _stream_ptr(stream), ctypes.byref(h)),
                      "dplr_gpu_plan_copy")
        return GpuPlan(None, _handle=h)

    def axpy(self, alpha: float, other: "GpuPlan", stream=None) -> "GpuPlan":
        """A new plan alpha * self + other, made on the device with dplraxpy's
        layout (other's columns, then self's; ranks add)."""
        h = ctypes.c_void_p()
        _native.check(_native.lib().dplr_gpu_axpy(float(alpha), self._h, other._h, _stream_ptr(stream),
                                                  ctypes.byref(h)), "dplr_gpu_axpy")
        return GpuPlan(None, _handle=h)

    def reduce_svd(self, eps: float, workers: int = 0, stream=None) -> "GpuPlan":
        """A new plan with every low-rank block replaced by its truncated SVD
        (dplrreduce's thresholds, eps / 4 per level), made on the device."""
        h = ctypes.c_void_p()
        rc = _native.lib().dplr_gpu_plan_reduce_svd(self._h, float(eps), int(workers), _stream_ptr(stream),
                                                     ctypes.byref(h))
        if not h.value:
            _native.check(rc, "dplr_gpu_plan_reduce_svd")
        return GpuPlan(None, _handle=h)

    def to_dense(self, stream=None) -> torch.Tensor:
        """The dense m x m matrix on the device (dplrgep2d), as a (m, m)
        tensor whose row j is column j of the matrix."""
        d = torch.empty(self.m, self.m, dtype=torch.float64, device="cuda")
        _native.check(_native.lib().dplr_gpu_gep2d(self._h, d.data_ptr(), self.m, _stream_ptr(stream)),
                      "dplr_gpu_gep2d")
        return d

    def prepare_pairs(self, stream=None) -> None:
        """Float-pair copy of the factors: 1-RHS op-N applies then run on the
        FP32 pipes (FP64-accurate, compensated sums) at HBM speed."""
        _native.check(_native.lib().dplr_gpu_prepare_pairs(self._h, _stream_ptr(stream)), "dplr_gpu_prepare_pairs")
        self.pairs = True

    def prepare_sliced(self, stream=None) -> None:
        """Exact-slice factor copies for the precise (tensor-core) residual."""
        _native.check(_native.lib().dplr_gpu_prepare_sliced(self._h, _stream_ptr(stream)),
                      "dplr_gpu_prepare_sliced")
        self.sliced = True

    def residual(self, x: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None,
                 precise: bool = True, stream=None) -> torch.Tensor:
        """out := b - A x (exact-slice products when precise)."""
        _check_block(x, self.m, "x")
        _check_block(b, self.m, "b")
        out = torch.empty_like(b) if out is None else out
        _check_block(out, self.m, "out")
        _native.check(_native.lib().dplr_gpu_residual(
            self._h, x.shape[0], x.data_ptr(), self.m, b.data_ptr(), self.m, out.data_ptr(),
            self.m, self.RESIDUAL_SLICED if precise else 0, _stream_ptr(stream)), "dplr_gpu_residual")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().dplr_gpu_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def device_bytes(self) -> int:
        lib = _native.lib()
        return int(lib.dplr_gpu_plan_device_bytes(self._h)) + int(
            lib.dplr_gpu_factor_device_bytes(self._h))

    # -------------------------------------------------------------- apply
    def apply(self, x: torch.Tensor, trans: str = "N", alpha: float = 1.0, beta: float = 0.0,
              out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """out := alpha*op(A) x + beta*out for x of shape (n, m)."""
        _check_block(x, self.m, "x")
        if out is None:
            out = torch.empty_like(x)
            beta = 0.0
        _check_block(out, self.m, "out")
        n = x.shape[0]
        _native.check(_native.lib().dplr_gpu_apply(self._h, trans.encode(), n, alpha, x.data_ptr(),
                                                   self.m, beta, out.data_ptr(), self.m,
                                                   _stream_ptr(stream)), "dplr_gpu_apply")
        return out

    # -------------------------------------------------------------- factor pool
    def pool_size(self) -> int:
        return int(_native.lib().dplr_gpu_pool_size(self._h))

    def read_pool(self, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """Device copy of every factor value (pool layout, float64)."""
        n = self.pool_size()
        out = torch.empty(n, dtype=torch.float64, device="cuda") if out is None else out
        if not (out.is_cuda and out.dtype == torch.float64 and out.is_contiguous() and out.numel() == n):
            raise ValueError(f"pool tensor must be a contiguous CUDA float64 tensor of {n} elements")
        _native.check(_native.lib().dplr_gpu_pool_read(self._h, out.data_ptr(), _stream_ptr(stream)),
                      "dplr_gpu_pool_read")
        return out

    def write_pool(self, values: torch.Tensor, stream=None) -> None:
        """Replace the factor values (same structure); the factorisation and
        sliced copies must be rebuilt afterwards."""
        n = self.pool_size()
        if not (values.is_cuda and values.dtype == torch.float64 and values.is_contiguous()
                and values.numel() == n):
            raise ValueError(f"pool tensor must be a contiguous CUDA float64 tensor of {n} elements")
        _native.check(_native.lib().dplr_gpu_pool_write(self._h, values.data_ptr(), _stream_ptr(stream)),
                      "dplr_gpu_pool_write")
        self.factored = self.factored_transposed = self.sliced = self.mixed = False

    def pool_blocks(self) -> list[dict]:
        """Layout of the pool: low-rank blocks (pre-order, ne before sw), then
        leaves; offsets in doubles."""
        lib = _native.lib()
        nlr, nlf = ctypes.c_int(), ctypes.c_int()
        _native.check(lib.dplr_gpu_pool_blocks(self._h, ctypes.byref(nlr), ctypes.byref(nlf)),
                      "dplr_gpu_pool_blocks")
        out = []
        u, v, sg = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        n, r, r0, c0 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        for i in range(nlr.value + nlf.value):
            _native.check(lib.dplr_gpu_pool_block(self._h, i, ctypes.byref(u), ctypes.byref(v),
                                                  ctypes.byref(sg), ctypes.byref(n), ctypes.byref(r),
                                                  ctypes.byref(r0), ctypes.byref(c0)),
                          "dplr_gpu_pool_block")
            if i < nlr.value:
                out.append({"kind": "lowrank", "u": u.value, "v": v.value, "sig": sg.value,
                            "n": n.value, "rank": r.value, "row0": r0.value, "col0": c0.value})
            else:
                out.append({"kind": "leaf", "d": u.value, "b": n.value, "row0": r0.value})
        return out

    def grad_factors(self, x: torch.Tensor, dy: torch.Tensor, alpha: float = 1.0,
                     out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """out (pool layout) += alpha * d<dy, A x>/d(factors)."""
        _check_block(x, self.m, "x")
        _check_block(dy, self.m, "dy")
        if x.shape[0] != dy.shape[0]:
            raise ValueError("x and dy must have the same number of columns")
        out = torch.zeros(self.pool_size(), dtype=torch.float64, device="cuda") if out is None else out
        _native.check(_native.lib().dplr_gpu_grad_factors(self._h, x.shape[0], x.data_ptr(), self.m,
                                                          dy.data_ptr(), self.m, alpha, out.data_ptr(),
                                                          _stream_ptr(stream)), "dplr_gpu_grad_factors")
        return out

    # -------------------------------------------------------------- solve
    def factor(self, transposed: bool = False, stream=None) -> None:
        _native.check(_native.lib().dplr_gpu_factor(self._h, 1 if transposed else 0,
                                                    _stream_ptr(stream)), "dplr_gpu_factor")
        self.factored = True
        self.factored_transposed = bool(transposed)

    def solve(self, b: torch.Tensor, trans: str = "N", out: torch.Tensor | None = None,
              stream=None) -> torch.Tensor:
        _check_block(b, self.m, "b")
        out = torch.empty_like(b) if out is None else out
        _check_block(out, self.m, "out")
        _native.check(_native.lib().dplr_gpu_solve(self._h, trans.encode(), b.shape[0],
                                                   b.data_ptr(), self.m, out.data_ptr(), self.m,
                                                   _stream_ptr(stream)), "dplr_gpu_solve")
        return out

    def solve_refined(self, b: torch.Tensor, tol: float = 1e-12, maxiter: int = 10,
                      out: torch.Tensor | None = None, stream=None, strict: bool = True,
                      precise: bool | None = None, mixed: bool = False):
        """Refined solve; returns (x, relative residual, corrections).  The
        residual uses exact-slice products when `precise` (default: when
        the plan has them).  With strict=False a solve that stops above
        `tol` is returned too."""
        if precise is None:
            precise = self.sliced
        _check_block(b, self.m, "b")
        out = torch.empty_like(b) if out is None else out
        _check_block(out, self.m, "out")
        res, its = ctypes.c_double(), ctypes.c_int()
        rc = _native.lib().dplr_gpu_solve_refined(self._h, b.shape[0], b.data_ptr(), self.m,
                                                  out.data_ptr(), self.m, tol, maxiter,
                                                  (self.RESIDUAL_SLICED if precise else 0)
                                                  | (self.SOLVE_MIXED if mixed else 0),
                                                  ctypes.byref(res), ctypes.byref(its),
                                                  _stream_ptr(stream))
        if rc != -5 or strict:
            _native.check(rc, "dplr_gpu_solve_refined")
        return out, res.value, its.value


class GpuGraph:
    """A captured CUDA graph of one apply ('A'), solve ('S'), or solve
    refined by one ('C') or two ('R') correction steps of a plan, with fixed
    tensors x (input) and y (output); launch() replays it."""

    def __init__(self, plan: GpuPlan, op: str, x: torch.Tensor, y: torch.Tensor, trans: str = "N",
                 stream=None):
        _check_block(x, plan.m, "x")
        _check_block(y, plan.m, "y")
        if x.shape != y.shape:
            raise ValueError("x and y must have the same shape")
        self.plan, self.x, self.y = plan, x, y
        h = ctypes.c_void_p()
        _native.check(_native.lib().dplr_gpu_graph_create(plan.handle, op.encode(), trans.encode(), x.shape[0],
                                                          x.data_ptr(), plan.m, y.data_ptr(), plan.m,
                                                          _stream_ptr(stream), ctypes.byref(h)),
                      "dplr_gpu_graph_create")
        self._h = h

    @property
    def kernels(self) -> int:
        return int(_native.lib().dplr_gpu_graph_kernels(self._h))

    def launch(self, stream=None) -> None:
        _native.check(_native.lib().dplr_gpu_graph_launch(self._h, _stream_ptr(stream)), "dplr_gpu_graph_launch")

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().dplr_gpu_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
