"""Ready-made cases for the SIMPLE outer iteration.

``lid_driven_cavity`` builds the isothermal lid-driven cavity in the
layouts the reference's input decks produce (ix with the material in the
last column, nelcon, RCM equation numbers, per-face boundary codes pedge
and values sedge, materials e(10, nmat)) with this library's own mesh
chain (adjacency, RCM, numeq): walls pedge 0, the lid (y = 1) a moving wall
(pedge 1, sedge = (lid, 0)), one cell's pressure correction pinned
(pedge(nshared+1) = -1), one material e = (nu, rho, 0, 0, 0, cc, limiter).
"""
from __future__ import annotations

import numpy as np

from . import mesh as _mesh


def lid_driven_cavity(nx: int, kind: str = "quad", nu: float = 0.01, rho: float = 1.0,
                      lid: float = 1.0, pin_cell: int = 1, limiter: int = 7, cc: float = 1.0,
                      jitter: float = 0.0, seed: int = 1234) -> dict:
    m = _mesh.square_mesh(nx, kind=kind, jitter=jitter, seed=seed)
    nelcon = _mesh.adjacency(m)
    num = _mesh.rcm(nelcon)
    ident = _mesh.numeq(num, nelcon)
    numel, nsh = m.numel, m.nshared
    ix = np.concatenate([m.ix, np.ones((numel, 1), np.int32)], axis=1)
    pedge = np.zeros((numel, nsh + 1), np.int32)
    sedge = np.zeros((numel, nsh + 1, 3))
    ns = m.nsides
    a = m.coor[m.ix - 1]                                   # (numel, nsh, 2) face start nodes
    nxt = np.take_along_axis(m.ix, (np.arange(nsh)[None, :] + 1) % ns[:, None], axis=1)
    b = m.coor[nxt - 1]                                    # face end nodes
    used = np.arange(nsh)[None, :] < ns[:, None]
    top = used & (nelcon < 0) & (np.abs(a[..., 1] - 1.0) < 1e-12) & (np.abs(b[..., 1] - 1.0) < 1e-12)
    pedge[:, :nsh][top] = 1
    sedge[:, :nsh, 0][top] = lid
    pedge[pin_cell - 1, nsh] = -1
    e = np.zeros((1, 10))
    e[0, 0], e[0, 1], e[0, 5], e[0, 6] = nu, rho, cc, limiter
    return dict(coor=m.coor, ix=ix, nelcon=nelcon, num=num, ident=ident, pedge=pedge,
                sedge=sedge, e=e, nshared=nsh, numel=numel, mesh=m)
