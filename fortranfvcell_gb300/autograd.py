"""Differentiable sparse solves on the GPU.

``LinearSolve`` is a ``torch.autograd.Function`` around the library's
solver: the forward pass solves A x = b with A in the reference's CSRD
layout (diagonal ``ad``, off-diagonals ``au`` as stored, i.e. the matrix
entries themselves, src/Datastruct.f) and the backward pass solves the
adjoint system A^T lambda = dL/dx, giving

    dL/db = lambda,   dL/dad_i = -lambda_i x_i,   dL/dau_k = -lambda_i x_j

for slot k at (row i, column j).  The reference has no adjoint; this is
the building block of sensitivity studies on top of its discretisation.
For the cell-adjacency structures of fortranFVCell the off-diagonal pattern
is symmetric, so A^T has the same structure and its values are a
permutation of au, applied on the device before every adjoint solve.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Context, make_opts


def transpose_permutation(ia, ja, n):
    """perm with au_T = au[perm] for a CSRD structure (1-based ia/ja) whose
    off-diagonal pattern is symmetric; ValueError otherwise."""
    ia = np.asarray(ia, np.int64)
    nad = int(ia[n] - 1)
    ja = np.asarray(ja, np.int64)[:nad]
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(ia[: n + 1]))
    cols = ja - 1
    key = rows * n + cols
    order = np.argsort(key, kind="stable")
    keyt = cols * n + rows
    pos = np.searchsorted(key[order], keyt)
    if np.any(pos >= nad) or np.any(key[order][np.minimum(pos, nad - 1)] != keyt):
        raise ValueError("the off-diagonal pattern is not symmetric")
    return order[pos], rows, cols


class CsrdSystem:
    """One CSRD structure on the GPU with its transpose: two solver contexts
    (A and A^T), the transpose permutation and the slot rows/columns on the
    device.  code 1 (PCG, symmetric A) or 2 (BiCGSTAB) for both solves."""

    def __init__(self, ia, ja, n, code=2, tol=1e-12, maxit=100000, device=0):
        self.n = int(n)
        self.ia = np.ascontiguousarray(ia, np.int32)
        self.nad = int(self.ia[n] - 1)
        self.ja = np.ascontiguousarray(np.asarray(ja)[: max(self.nad, 1)], np.int32)
        perm, rows, cols = transpose_permutation(self.ia, self.ja, n)
        dev = torch.device("cuda", device)
        self.perm = torch.from_numpy(perm).to(dev)
        self.rows = torch.from_numpy(rows).to(dev)
        self.cols = torch.from_numpy(cols).to(dev)
        self.code, self.tol, self.maxit = code, tol, maxit
        self.opts = make_opts("fp64", init=1)
        one = np.ones(n)
        zero = np.zeros(max(self.nad, 1))
        self.A = Context(device=device)
        self.A.set_matrix(1, True, n, self.nad, one, zero, zero, self.ia, self.ja)
        self.AT = Context(device=device)
        self.AT.set_matrix(1, True, n, self.nad, one, zero, zero, self.ia, self.ja)

    def solve(self, ctx, ad, au, rhs):
        if not bool(torch.any(rhs != 0)):
            # x = 0 exactly; Krylov recurrences divide 0 by 0 on a zero
            # right-hand side (the reference's SIMPLE skips such solves)
            return torch.zeros_like(rhs)
        torch.cuda.synchronize()
        ctx.update_values(ad.contiguous(), au.contiguous(), au.contiguous())
        x = torch.zeros_like(rhs)
        ctx.solve(self.code, rhs.contiguous(), x, self.tol, self.maxit, self.opts)
        return x

    def close(self):
        self.A.close()
        self.AT.close()


class LinearSolve(torch.autograd.Function):
    """x = A^{-1} b for A = (ad, au) on ``system``'s structure; all tensors
    float64 on the GPU."""

    @staticmethod
    def forward(ctx, ad, au, b, system):
        x = system.solve(system.A, ad, au, b)
        ctx.save_for_backward(ad, au, x)
        ctx.system = system
        return x

    @staticmethod
    def backward(ctx, gx):
        ad, au, x = ctx.saved_tensors
        s = ctx.system
        lam = s.solve(s.AT, ad, au[s.perm], gx)
        g_ad = -lam * x
        g_au = -lam[s.rows] * x[s.cols]
        return g_ad, g_au, lam, None


def linear_solve(ad, au, b, system):
    return LinearSolve.apply(ad, au, b, system)
