"""Lid-driven cavity set-up on the oracle's graph chain, and the reference's
SIMPLE iteration (oracle/simple_ref.py) the GPU loop is checked against."""
import numpy as np

from _systems import graph
from oracle.simple_ref import SimpleRef  # noqa: F401


def cavity(orc, nx, kind="quad", nu=0.01, rho=1.0, lid=1.0, pin_cell=1, limiter=7, cc=1.0,
           jitter=0.0):
    """Unit-square cavity: walls pedge 0, moving lid (y = 1) pedge 1 with
    sedge = (lid, 0), cell pin_cell's p' pinned (pedge(idCell) = -1), one
    material e = (nu, rho, 0, 0, 0, cc, limiter, ...)."""
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(nx, kind=kind, jitter=jitter, seed=1234)
    nelcon, num, ident = graph(orc, m)
    numel, nsh = m.numel, m.nshared
    ix = np.concatenate([m.ix, np.ones((numel, 1), np.int32)], axis=1)
    pedge = np.zeros((numel, nsh + 1), np.int32)
    sedge = np.zeros((numel, nsh + 1, 3))
    ns = m.nsides
    for c in range(numel):
        for i in range(ns[c]):
            if nelcon[c, i] < 0:
                a = m.coor[m.ix[c, i] - 1]
                bnode = m.coor[m.ix[c, (i + 1) % ns[c]] - 1]
                if abs(a[1] - 1.0) < 1e-12 and abs(bnode[1] - 1.0) < 1e-12:
                    pedge[c, i] = 1
                    sedge[c, i, 0] = lid
    pedge[pin_cell - 1, nsh] = -1
    e = np.zeros((1, 10))
    e[0, 0], e[0, 1], e[0, 5], e[0, 6] = nu, rho, cc, limiter
    return dict(coor=m.coor, ix=ix, nelcon=nelcon, num=num, ident=ident, pedge=pedge,
                sedge=sedge, e=e, nshared=nsh, numel=numel, mesh=m)


def hot_wall_nusselt(case, temp):
    """Mean Nusselt number of the hot (x = 0) wall of a natural_convection_cavity
    on uniform quads: (T_wall - T_P) / (h/2) L / dT averaged over the wall."""
    nx = int(round(np.sqrt(case["numel"])))
    side, dt_wall = case["side"], 1.0
    h = side / nx
    t_wall = case["t0"] + 0.5 * dt_wall
    tp = temp.reshape(nx, nx)[:, 0]
    return float(np.mean((t_wall - tp) / (0.5 * h)) * side / dt_wall)
