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
is symmetric, so the adjoint BiCGSTAB runs on A's own storage through the
library's transposed SpMV (fvc_solve_transposed: entry (i, j) of A^T is
read at the slot of (j, i)); no transposed copy of the values exists.  PCG
(code 1) serves symmetric A, where A^T = A.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Context, make_opts


def transpose_permutation(ia, ja, n):
    """perm with au_T = au[perm] for a CSRD structure (1-based ia/ja) whose
    off-diagonal pattern is symmetric (the slot of (j, i) for the slot of
    (i, j)), with the slots' rows and columns; ValueError otherwise.  The
    gradient of the matrix values uses the rows and columns."""
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
    """One CSRD structure on the GPU: a solver context for A (whose
    transposed solves use the same storage) and the slots' rows and columns
    on the device.  code 1 (PCG, symmetric A) or 2 (BiCGSTAB)."""

    def __init__(self, ia, ja, n, code=2, tol=1e-12, maxit=100000, device=0):
        self.n = int(n)
        self.ia = np.ascontiguousarray(ia, np.int32)
        self.nad = int(self.ia[n] - 1)
        self.ja = np.ascontiguousarray(np.asarray(ja)[: max(self.nad, 1)], np.int32)
        _, rows, cols = transpose_permutation(self.ia, self.ja, n)   # checks the symmetry
        dev = torch.device("cuda", device)
        self.rows = torch.from_numpy(rows).to(dev)
        self.cols = torch.from_numpy(cols).to(dev)
        self.code, self.tol, self.maxit = code, tol, maxit
        self.opts = make_opts("fp64", init=1)
        one = np.ones(n)
        zero = np.zeros(max(self.nad, 1))
        self.A = Context(device=device)
        self.A.set_matrix(1, True, n, self.nad, one, zero, zero, self.ia, self.ja)

    def solve(self, ad, au, rhs, transposed=False):
        """x with A x = rhs (or A^T x = rhs), A = (ad, au)."""
        if not bool(torch.any(rhs != 0)):
            # x = 0 exactly; Krylov recurrences divide 0 by 0 on a zero
            # right-hand side (the reference's SIMPLE skips such solves)
            return torch.zeros_like(rhs)
        torch.cuda.synchronize()
        self.A.update_values(ad.contiguous(), au.contiguous(), au.contiguous())
        x = torch.zeros_like(rhs)
        if transposed and self.code == 2:
            self.A.solve_transposed(rhs.contiguous(), x, self.tol, self.maxit, self.opts)
        else:
            self.A.solve(self.code, rhs.contiguous(), x, self.tol, self.maxit, self.opts)
        return x

    def close(self):
        self.A.close()


class LinearSolve(torch.autograd.Function):
    """x = A^{-1} b for A = (ad, au) on ``system``'s structure; all tensors
    float64 on the GPU."""

    @staticmethod
    def forward(ctx, ad, au, b, system):
        x = system.solve(ad, au, b)
        ctx.save_for_backward(ad, au, x)
        ctx.system = system
        return x

    @staticmethod
    def backward(ctx, gx):
        ad, au, x = ctx.saved_tensors
        s = ctx.system
        lam = s.solve(ad, au, gx, transposed=True)
        g_ad = -lam * x
        g_au = -lam[s.rows] * x[s.cols]
        return g_ad, g_au, lam, None


def linear_solve(ad, au, b, system):
    return LinearSolve.apply(ad, au, b, system)
