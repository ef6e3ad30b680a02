"""torch.autograd wrapper around the GB300 solve and its hand-written adjoint.

x = A(vals)^-1 b. The backward pass solves A^T lambda = dL/dx with the
transposed SpMV and U^T/L^T sweeps that reuse the forward ILU0 factors
(gbilu_adjoint), and returns dL/db = lambda and dL/dvals = -lambda_i x_j^T on
the sparsity pattern (one 3x3 block per stored block of A).

The handle keeps one factorization. If another forward with different values
runs on the same handle before this backward, the backward refactors with
the values it saved, so gradients always belong to their own forward.
"""
from __future__ import annotations

import numpy as np
import torch

from .native import GbIlu


class _State:
    def __init__(self):
        self.version = 0


_states = {}


def _state(solver):
    st = _states.get(id(solver))
    if st is None:
        st = _states[id(solver)] = _State()
    return st


class IluBicgstabSolve(torch.autograd.Function):
    """solve(vals[nnzb,3,3], b[3*nb]) -> x with gradients for vals and b."""

    @staticmethod
    def forward(ctx, vals, b, solver: GbIlu, tol: float, maxit: int):
        st = _state(solver)
        v = vals.detach().to("cpu", torch.float64).contiguous().numpy()
        solver.factor(v)
        st.version += 1
        x, res = solver.solve(b.detach().to("cpu", torch.float64).numpy(), tol=tol, maxit=maxit)
        if res.status not in (0,):
            raise RuntimeError(f"forward solve did not converge (status {res.status})")
        xt = torch.from_numpy(x).to(b.device)
        ctx.solver, ctx.tol, ctx.maxit, ctx.version = solver, tol, maxit, st.version
        ctx.vals = v
        ctx.save_for_backward(xt)
        return xt

    @staticmethod
    def backward(ctx, gx):
        (x,) = ctx.saved_tensors
        solver = ctx.solver
        st = _state(solver)
        if st.version != ctx.version:
            solver.factor(ctx.vals)
            st.version += 1
            ctx.version = st.version
        g = gx.detach().to("cpu", torch.float64).numpy()
        lam, dA, res = solver.adjoint(g, x.detach().cpu().numpy(), tol=ctx.tol,
                                      maxit=ctx.maxit, want_dA=ctx.needs_input_grad[0])
        if res.status not in (0, 2):
            raise RuntimeError(f"adjoint solve did not converge (status {res.status})")
        d_vals = torch.from_numpy(dA).to(gx.device) if dA is not None else None
        d_b = torch.from_numpy(lam).to(gx.device)
        return d_vals, d_b, None, None, None


def solve(vals, b, solver: GbIlu, tol: float = 1e-10, maxit: int = 2000):
    """Differentiable x = A^-1 b for a solver whose pattern is analyzed."""
    return IluBicgstabSolve.apply(vals, b, solver, tol, maxit)
