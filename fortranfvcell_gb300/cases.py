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


# air at 20 C, the material of the reference's natural-convection deck
# (viscosity, reference density, conductivity, specific heat, reference
# temperature): mu, rho, k, cp, tRef
AIR = (1.72e-5, 1.204, 2.42e-2, 1.012e3, 20.0)


def natural_convection_cavity(nx: int, ra: float = 1.0e6, dt_wall: float = 1.0,
                              t0: float = 20.0, kind: str = "quad", limiter: int = 7,
                              jitter: float = 0.0, seed: int = 1234) -> dict:
    """Differentially heated square cavity for the ideal-gas SIMPLE loop
    (material type 55): walls no-slip (pedge 0), the left wall at
    t0 + dt_wall/2 and the right one at t0 - dt_wall/2 (energy pedge 1),
    top and bottom adiabatic (energy pedge 0, zero flux), gravity (0, -9.81),
    cell 1's pressure correction pinned.  The side L is set so that
    Ra = g beta dt_wall L^3 / (nu alpha) with beta = 1/(t0 + 273.15) K and
    nu, alpha of air; the returned dict adds pedgeE, sedgeE, gravity, t0 and
    side to the keys of lid_driven_cavity."""
    mu, rho, k, cp, tref = AIR
    nu, alpha, g = mu / rho, k / (rho * cp), 9.81
    beta = 1.0 / (t0 + 273.15)
    side = (ra * nu * alpha / (g * beta * dt_wall)) ** (1.0 / 3.0)
    c = lid_driven_cavity(nx, kind=kind, lid=0.0, limiter=limiter, jitter=jitter, seed=seed)
    c["coor"] = c["coor"] * side
    c["mesh"].coor = c["coor"]
    c["pedge"][:, :c["nshared"]] = 0          # no moving lid
    c["sedge"][:] = 0.0
    c["e"] = np.zeros((1, 10))
    c["e"][0, :7] = [mu, rho, k, cp, tref, 1.0, limiter]
    nsh, n = c["nshared"], c["numel"]
    m = c["mesh"]
    a = c["coor"][m.ix - 1]
    nxt = np.take_along_axis(m.ix, (np.arange(nsh)[None, :] + 1) % m.nsides[:, None], axis=1)
    b = c["coor"][nxt - 1]
    used = np.arange(nsh)[None, :] < m.nsides[:, None]
    bnd = used & (c["nelcon"] < 0)
    tol = 1e-9 * side
    left = bnd & (np.abs(a[..., 0]) < tol) & (np.abs(b[..., 0]) < tol)
    right = bnd & (np.abs(a[..., 0] - side) < tol) & (np.abs(b[..., 0] - side) < tol)
    pe = np.zeros((n, nsh + 1), np.int32)
    se = np.zeros((n, nsh + 1))
    pe[:, :nsh][left | right] = 1
    se[:, :nsh][left] = t0 + 0.5 * dt_wall
    se[:, :nsh][right] = t0 - 0.5 * dt_wall
    c.update(pedgeE=pe, sedgeE=se, gravity=np.array([0.0, -g]), t0=t0, side=side, ra=ra,
             dt_wall=dt_wall)
    c["e"][0, 1] = rho
    return c


def heated_lid_cavity(nx: int, re: float = 100.0, side: float = 0.01, dt_wall: float = 1.0,
                      t0: float = 20.0, kind: str = "quad") -> dict:
    """Lid-driven cavity of air for the ideal-gas loop with the energy
    equation: the top wall moves at U = Re nu / side (momentum pedge 1,
    sedge (U, 0)), the other walls are at rest; the left wall is held at
    t0 + dt_wall/2 and the right one at t0 - dt_wall/2, top and bottom are
    adiabatic; no gravity, so the temperature is carried by the flow (forced
    convection) and acts only through the ideal-gas density.  Keys as
    natural_convection_cavity, plus re and lid."""
    mu, rho, k, cp, _ = AIR
    nu, alpha, g = mu / rho, k / (rho * cp), 9.81
    beta = 1.0 / (t0 + 273.15)
    ra = g * beta * dt_wall * side ** 3 / (nu * alpha)   # the side's Ra, for the builder
    c = natural_convection_cavity(nx, ra=ra, dt_wall=dt_wall, t0=t0, kind=kind)
    lid = re * nu / side
    nsh = c["nshared"]
    m = c["mesh"]
    a = c["coor"][m.ix - 1]
    nxt = np.take_along_axis(m.ix, (np.arange(nsh)[None, :] + 1) % m.nsides[:, None], axis=1)
    b = c["coor"][nxt - 1]
    used = np.arange(nsh)[None, :] < m.nsides[:, None]
    tol = 1e-9 * c["side"]
    top = (used & (c["nelcon"] < 0) & (np.abs(a[..., 1] - c["side"]) < tol)
           & (np.abs(b[..., 1] - c["side"]) < tol))
    c["pedge"][:, :nsh][top] = 1
    c["sedge"][:, :nsh, 0][top] = lid
    c.update(gravity=np.array([0.0, 0.0]), re=re, lid=lid)
    return c


def heated_channel(nx: int, re: float = 100.0, side: float = 0.01, dt_wall: float = 1.0,
                   t0: float = 20.0, kind: str = "quad") -> dict:
    """A square section of a heated channel of air for the ideal-gas loop
    with the energy equation: inflow at x = 0 with U = Re nu / side (momentum
    pedge 2, sedge (U, 0)), outflow at x = side at the reference pressure
    (pedge 3, pressure 0), no-slip walls at y = 0 and y = side; no pressure
    pin, because the outflow fixes the pressure level; the air enters at
    t0 - dt_wall/2 (energy pedge 2), the bottom wall is held at t0 + dt_wall/2
    (energy pedge 1), the top wall is adiabatic and the outflow carries the
    enthalpy out (energy pedge 4); no gravity (forced convection).  Keys as
    heated_lid_cavity, plus u_in."""
    c = heated_lid_cavity(nx, re=re, side=side, dt_wall=dt_wall, t0=t0, kind=kind)
    mu, rho, _, _, _ = AIR
    u_in = re * (mu / rho) / side
    nsh, n = c["nshared"], c["numel"]
    m = c["mesh"]
    a = c["coor"][m.ix - 1]
    nxt = np.take_along_axis(m.ix, (np.arange(nsh)[None, :] + 1) % m.nsides[:, None], axis=1)
    b = c["coor"][nxt - 1]
    used = np.arange(nsh)[None, :] < m.nsides[:, None]
    bnd = used & (c["nelcon"] < 0)
    tol = 1e-9 * c["side"]
    on = lambda d, v: bnd & (np.abs(a[..., d] - v) < tol) & (np.abs(b[..., d] - v) < tol)
    left, right = on(0, 0.0), on(0, c["side"])
    bottom = on(1, 0.0)
    pedge = np.zeros((n, nsh + 1), np.int32)          # walls, and no p' pin
    sedge = np.zeros((n, nsh + 1, 3))
    pedge[:, :nsh][left] = 2
    sedge[:, :nsh, 0][left] = u_in
    pedge[:, :nsh][right] = 3                          # pressure 0 on the outflow
    pe = np.zeros((n, nsh + 1), np.int32)
    se = np.zeros((n, nsh + 1))
    pe[:, :nsh][left] = 2
    se[:, :nsh][left] = t0 - 0.5 * dt_wall
    pe[:, :nsh][bottom] = 1
    se[:, :nsh][bottom] = t0 + 0.5 * dt_wall
    pe[:, :nsh][right] = 4
    c.update(pedge=pedge, sedge=sedge, pedgeE=pe, sedgeE=se, lid=0.0, u_in=u_in)
    return c
