"""Batched conjugate gradient on the ADRT normal equations.

Solves A^T A x = A^T b for every image of a batch, A = adrt (n x n image ->
(4, 2n-1, n)), A^T = its exact transpose (the adjoint kernel).  This is the
reconstruction recipe the reference documents with SciPy
(docs/examples.cginverse.md:40-67, operator truncate(bdrt(adrt(x))).mean(0));
the mean there is 1/4 of A^T, which leaves the solution unchanged.

With ``ridge_param`` = lambda > 0 the operator is the reference's
``ADRTRidgeOperator`` (docs/examples.tomography.md:63-76): its normal
operator is the quadrant *mean* plus lambda I, so the system solved is
(A^T A / 4 + lambda I) x = A^T b / 4, i.e. (A^T A + 4 lambda I) x = A^T b.

Each image stops when its normal-equation residual
||A^T b - (A^T A + 4 lambda I) x|| / ||A^T b|| <= tol (the quantity CG controls); the
batch runs until all images stopped or `max_iters`.  All vector algebra runs
in the library's CG kernels with float64 per-image scalars; with
``graph=True`` one CG iteration is captured in a CUDA graph and replayed.

With ``precond`` (a symmetric positive definite operator with an
``apply(x, out)`` method, e.g. ``adrt_gb300.precond.ConvPreconditioner``)
the iteration is preconditioned CG: z = M r, alpha = <r, z> / <p, A^T A p>,
p = z + beta p with beta = <r_new, z_new> / <r, z>; the stopping rule stays
the unpreconditioned normal-equation residual above.
"""

from __future__ import annotations

from dataclasses import dataclass

import torch

from . import _lib
from ._ops import adrt as _adrt
from .autograd import _adjoint_raw as _adjoint
from ._wrappers import float_code

__all__ = ["normal_op", "cg", "residuals_of", "CGResult"]


def normal_op(x: torch.Tensor, lam: float = 0.0) -> torch.Tensor:
    """(A^T A + lam I) x for a batch of images on the device."""
    y = _adjoint(_adrt(x))
    if lam:
        rc = _lib.load().adrt_gb300_axpy(float(lam), x.data_ptr(), y.data_ptr(), x.numel(), float_code(x),
                                         torch.cuda.current_stream(x.device).cuda_stream)
        _lib.check(rc, "axpy")
    return y


@dataclass
class CGResult:
    x: torch.Tensor            # (B, n, n) solutions
    iterations: torch.Tensor   # (B,) iterations each image ran
    normal_residual: torch.Tensor  # (B,) ||A^T(Ax - b)|| / ||A^T b|| (recomputed)
    data_residual: torch.Tensor    # (B,) ||Ax - b|| / ||b|| (recomputed)
    total_iterations: int


class _State:
    def __init__(self, b, x0, lam=0.0, precond=None):
        self.lam = lam
        self.precond = precond
        self.dev = b.device
        self.B = b.shape[0]
        n = b.shape[-1]
        self.per = n * n
        self.code = float_code(b)
        self.x = torch.zeros((self.B, n, n), dtype=b.dtype, device=b.device) if x0 is None else x0.clone().contiguous()
        self.rhs = _adjoint(b.contiguous())
        self.r = self.rhs - normal_op(self.x, lam) if x0 is not None else self.rhs.clone()
        self.ws = torch.empty(_lib.load().adrt_gb300_cg_workspace_size(self.B), dtype=torch.uint8, device=b.device)
        # rs: numerator of alpha (<r, r>, or <r, z> when preconditioned);
        # rr: <r, r> for the stopping rule.
        self.rr = self.dot(self.r, self.r)
        if precond is not None:
            self.z = precond.apply(self.r)
            self.p = self.z.clone()
            self.rs = self.dot(self.r, self.z)
            self.rz_new = torch.empty_like(self.rs)
            self.fused = hasattr(precond, "apply_dot")
            if self.fused:
                self.pws = precond.dot_workspace(self.B, n, b.device)
        else:
            self.p = self.r.clone()
            self.rs = self.rr.clone()
        self.rhs2 = self.dot(self.rhs, self.rhs)
        self.rs_new = torch.empty_like(self.rs)
        self.pAp = torch.empty_like(self.rs)
        self.active = torch.ones(self.B, dtype=torch.int32, device=b.device)
        self.iters = torch.zeros(self.B, dtype=torch.int32, device=b.device)

    def stream(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def subset(self, sel: torch.Tensor) -> None:
        """Keep only the images at positions `sel` (still-active ones)."""
        names = ["x", "r", "p", "rhs", "rs", "rr", "rhs2", "rs_new", "pAp", "active", "iters"]
        if self.precond is not None:
            names += ["z", "rz_new"]
        for name in names:
            setattr(self, name, getattr(self, name).index_select(0, sel).contiguous())
        self.B = int(sel.numel())
        self.ws = torch.empty(_lib.load().adrt_gb300_cg_workspace_size(self.B), dtype=torch.uint8, device=self.dev)
        if self.precond is not None and self.fused:
            self.pws = self.precond.dot_workspace(self.B, self.x.shape[-1], self.dev)

    def dot(self, a, b):
        out = torch.empty(self.B, dtype=torch.float64, device=self.dev)
        rc = _lib.load().adrt_gb300_batched_dot(a.data_ptr(), b.data_ptr(), out.data_ptr(), self.B,
                                               self.per, self.code, self.ws.data_ptr(), self.stream())
        _lib.check(rc, "batched_dot")
        return out

    def iterate(self, thr2):
        lib = _lib.load()
        Ap = normal_op(self.p, self.lam)
        rc = lib.adrt_gb300_batched_dot(self.p.data_ptr(), Ap.data_ptr(), self.pAp.data_ptr(), self.B,
                                        self.per, self.code, self.ws.data_ptr(), self.stream())
        _lib.check(rc, "batched_dot")
        self.iters += self.active
        rc = lib.adrt_gb300_cg_update(self.x.data_ptr(), self.r.data_ptr(), self.p.data_ptr(), Ap.data_ptr(),
                                      self.rs.data_ptr(), self.pAp.data_ptr(), self.active.data_ptr(),
                                      self.rs_new.data_ptr(), self.B, self.per, self.code,
                                      self.ws.data_ptr(), self.stream())
        _lib.check(rc, "cg_update")
        # Images whose residual reached the tolerance stop here.
        self.active.mul_((self.rs_new > thr2).to(torch.int32))
        if self.precond is not None:
            if self.fused:  # z = M r and <r, z> in one kernel
                self.precond.apply_dot(self.r, self.z, self.rz_new, self.pws)
            else:
                self.precond.apply(self.r, out=self.z)
                rc = lib.adrt_gb300_batched_dot(self.r.data_ptr(), self.z.data_ptr(), self.rz_new.data_ptr(), self.B,
                                                self.per, self.code, self.ws.data_ptr(), self.stream())
                _lib.check(rc, "batched_dot")
            d, num = self.z, self.rz_new
        else:
            d, num = self.r, self.rs_new
        rc = lib.adrt_gb300_cg_direction(self.p.data_ptr(), d.data_ptr(), num.data_ptr(),
                                         self.rs.data_ptr(), self.active.data_ptr(), self.B, self.per,
                                         self.code, self.stream())
        _lib.check(rc, "cg_direction")


def cg(b: torch.Tensor, x0: torch.Tensor | None = None, *, tol: float = 1e-4, max_iters: int = 1000,
       check_every: int = 4, graph: bool = False, ridge_param: float = 0.0, compact: float = 0.5,
       precond=None, residuals: bool = True) -> CGResult:
    """Batched CG for (A^T A + 4 ridge_param I) x = A^T b; b: CUDA tensor
    (B, 4, 2n-1, n).

    Images converge after different numbers of iterations; when at most
    `compact` of the images still iterating are active (checked every
    `check_every` iterations), the finished ones are written out and the
    batch shrinks to the active ones, so the work follows the iterations each
    image needs rather than the slowest image's (0 disables).  `precond`:
    preconditioner for PCG (see the module docstring).  `residuals=False`
    skips recomputing the reported residuals (the fields are then None;
    ``residuals_of`` computes them later)."""
    if not (isinstance(b, torch.Tensor) and b.is_cuda and b.ndim == 4):
        raise TypeError("cg expects a CUDA tensor of shape (B, 4, 2n-1, n)")
    if ridge_param < 0:
        raise ValueError("ridge_param must be non-negative")
    st = _State(b, x0, 4.0 * float(ridge_param), precond)
    thr2 = st.rhs2 * (tol * tol)
    st.active.copy_((st.rr > thr2).to(torch.int32))
    B_full = st.B
    rhs_full = st.rhs
    x_full = st.x
    iters_full = torch.zeros(B_full, dtype=torch.int32, device=st.dev)
    idx = torch.arange(B_full, device=st.dev)
    compacted = False
    k = 0
    g = None
    while k < max_iters:
        if graph and g is None and k >= 1:
            # Capture on a side stream with the graph's own memory pool
            # (capture_begin/end directly: the torch.cuda.graph context
            # manager also runs the Python garbage collector and empties the
            # allocator cache, which costs several iterations' time here).
            s = torch.cuda.Stream(device=st.dev)
            s.wait_stream(torch.cuda.current_stream(st.dev))
            with torch.cuda.stream(s):
                st.iterate(thr2)  # warm the capture stream's allocator
                k += 1
                g = torch.cuda.CUDAGraph()
                g.capture_begin()
                try:
                    st.iterate(thr2)
                finally:
                    g.capture_end()
            torch.cuda.current_stream(st.dev).wait_stream(s)
            # capture does not execute; the first replay below runs it
        steps = min(check_every, max_iters - k)
        for _ in range(steps):
            if g is not None:
                g.replay()
            else:
                st.iterate(thr2)
        k += steps
        n_active = int(st.active.sum().item())
        if n_active == 0:
            break
        if compact > 0 and st.B > 1 and n_active <= compact * st.B:
            # Write every row back, then continue with the active images only
            # (before the first shrink the state's tensors are the full ones).
            if compacted:
                x_full.index_copy_(0, idx, st.x)
                iters_full.index_copy_(0, idx, st.iters)
            else:
                x_full, iters_full = st.x, st.iters
            sel = st.active.nonzero().flatten()
            idx = idx.index_select(0, sel)
            st.subset(sel)
            thr2 = thr2.index_select(0, sel).contiguous()
            g = None
            compacted = True
    if compacted:
        x_full.index_copy_(0, idx, st.x)
        iters_full.index_copy_(0, idx, st.iters)
    else:
        iters_full = st.iters.clone()
    if not residuals:
        return CGResult(x_full, iters_full, None, None, k)
    normal_residual, data_residual = residuals_of(b, x_full, ridge_param, rhs_full)
    return CGResult(x_full, iters_full, normal_residual, data_residual, k)


def residuals_of(b: torch.Tensor, x: torch.Tensor, ridge_param: float = 0.0, rhs: torch.Tensor | None = None):
    """(||A^T b - (A^T A + 4 ridge_param I) x|| / ||A^T b||, ||Ax - b|| / ||b||)
    per image, recomputed from scratch (float64 sums); `rhs`: A^T b if known."""
    B = b.shape[0]
    if rhs is None:
        rhs = _adjoint(b.contiguous())
    res_n = normal_op(x, 4.0 * float(ridge_param)) - rhs
    ws = torch.empty(_lib.load().adrt_gb300_cg_workspace_size(B), dtype=torch.uint8, device=b.device)

    def dot(u, v):
        out = torch.empty(B, dtype=torch.float64, device=b.device)
        rc = _lib.load().adrt_gb300_batched_dot(u.data_ptr(), v.data_ptr(), out.data_ptr(), B, u[0].numel(),
                                               float_code(u), ws.data_ptr(),
                                               torch.cuda.current_stream(b.device).cuda_stream)
        _lib.check(rc, "batched_dot")
        return out

    normal_residual = torch.sqrt(dot(res_n, res_n) / dot(rhs, rhs))
    dr = _adrt(x) - b
    nb = (b.reshape(B, -1).double() ** 2).sum(1)
    data_residual = torch.sqrt((dr.reshape(B, -1).double() ** 2).sum(1) / nb)
    return normal_residual, data_residual
