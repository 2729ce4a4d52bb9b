"""Wall-temperature sensitivity of the heat transfer of a natural-convection
cavity by the adjoint method (fortranfvcell_gb300.autograd).

At a converged state of the ideal-gas SIMPLE loop (cells.SimpleLoop with
the energy equation) the flow and the densities are frozen and the
enthalpy equation of cell_e_eb_idg_ggl (src/CellibTrans.f:39-349) is the
linear system A h = b(h_w), assembled on the GPU by the same cell kernel
the loop uses.  The prescribed-temperature faces of the hot wall enter b
through ap_f h_f with ap_f = (k/cp) |f| / ca_f.  The reference stores the
boundary enthalpy as an integer (the `enthalpia` declaration), so its b is
piecewise constant in the wall temperature; here the wall enthalpies h_f are
the continuous parameters, and dJ/dT_f = cp dJ/dh_f.

J is the mean hot-wall Nusselt number,
    J = mean_f (T_f - T_P(f)) / ca_f * L / dT,   T = tRef + h / cp,
and its gradient with respect to all wall enthalpies takes one forward and
one adjoint solve (A^T lambda = dJ/dh).
"""
from __future__ import annotations

import numpy as np
import torch

from . import cells as _cells
from . import mesh as _mesh
from .autograd import CsrdSystem, linear_solve


def wall_faces(case, x: float = 0.0):
    """Boundary faces on the line x = const: (cell, face, |f|, ca) arrays
    (0-based cell and face), ca = the distance from the cell centroid to the
    face along its outward normal, as cellGeom2D computes it."""
    m = case["mesh"]
    coor, ix = case["coor"], m.ix
    tol = 1e-9 * float(np.ptp(coor[:, 0]))
    cells, faces, meta, ca = [], [], [], []
    for c in np.nonzero((case["nelcon"] < 0).any(axis=1))[0]:
        ns = int(m.nsides[c])
        xc = coor[ix[c, :ns] - 1].mean(axis=0)
        for i in range(ns):
            if case["nelcon"][c, i] >= 0:
                continue
            a, b = coor[ix[c, i] - 1], coor[ix[c, (i + 1) % ns] - 1]
            if abs(a[0] - x) > tol or abs(b[0] - x) > tol:
                continue
            eta = b - a
            length = float(np.hypot(eta[0], eta[1]))
            n = np.array([eta[1], -eta[0]]) / length
            cells.append(c)
            faces.append(i)
            meta.append(length)
            ca.append(float((0.5 * (a + b) - xc) @ n))
    return (np.array(cells), np.array(faces), np.array(meta), np.array(ca))


def frozen_energy_system(case, loop, dt: float = 1.0e10, grad_sweeps: int = 3):
    """The enthalpy system at the loop's current state, on the GPU: dict with
    ad, au, b (torch, equation order), ia, ja (numpy), the hot-wall faces and
    their rows, ap_f and the wall enthalpies h_f the assembly used."""
    w, _ = loop.fields()
    _, en, ro = loop.energy_fields()
    n, nsh = case["numel"], case["nshared"]
    ident = case["ident"] if "ident" in case else _mesh.numeq(case["num"], case["nelcon"])
    ia, ja, nad = _mesh.datastruc(ident, 1, True)
    m = _cells.CellMesh(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                        case["sedge"], case["e"])
    dev = lambda a, t=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", t)
    pe, se = dev(case["pedgeE"], torch.int32), dev(case["sedgeE"])
    en_d, ro_d, w_d = dev(en), dev(ro), dev(w)
    ge = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    for _ in range(grad_sweeps):                 # lib 3 extrapolates with the last gradient
        _cells.energy_gradient(m, 3, pe, se, en_d, ge)
    ad = torch.zeros(n, dtype=torch.float64, device="cuda")
    au = torch.zeros(max(int(ja.size), 1), dtype=torch.float64, device="cuda")
    b = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc = torch.zeros(n, dtype=torch.float64, device="cuda")
    ia_d, ja_d = dev(ia, torch.int32), dev(ja, torch.int32)
    _cells.energy(m, 3, 1, pe, se, en_d, en_d, ro_d, w_d, ge, dt, ia_d, ja_d, 1, ad, au, b, rc)
    b0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    _cells.energy(m, 3, 4, pe, se, en_d, en_d, ro_d, None, None, dt, ia_d, ja_d, 1, None, None,
                  b0, None)
    torch.cuda.synchronize()
    b = b + b0
    e = case["e"][0]
    kc, cp, tref = e[2], e[3], e[4]
    cells, faces, meta, ca = wall_faces(case, 0.0)
    hot = case["pedgeE"][cells, faces] == 1
    cells, faces, meta, ca = cells[hot], faces[hot], meta[hot], ca[hot]
    rows = case["num"][cells] - 1
    ap = (kc / cp) * meta / ca
    # the enthalpy the cell used: cp (T - tRef) truncated toward zero
    h_int = np.trunc(cp * (case["sedgeE"][cells, faces] - tref))
    return dict(ad=ad, au=au[:nad], b=b, ia=ia, ja=ja, nad=nad, rows=rows, ap=ap, ca=ca,
                h_wall=h_int, cp=cp, tref=tref, en=en)


class NusseltProblem:
    """J(h_w) on the frozen enthalpy system; the wall enthalpies enter b
    through ap_f h_f (the assembled b's own wall terms are taken out)."""

    def __init__(self, case, sysd, tol=1e-12):
        self.s = sysd
        self.solver = CsrdSystem(sysd["ia"], sysd["ja"], case["numel"], code=2, tol=tol)
        d = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
        self.rows = torch.from_numpy(sysd["rows"]).cuda()
        self.ap, self.ca = d(sysd["ap"]), d(sysd["ca"])
        self.b_rest = sysd["b"].index_add(0, self.rows, -self.ap * d(sysd["h_wall"]))
        self.scale = float(case["side"]) / float(case.get("dt_wall", 1.0)) / sysd["cp"]

    def __call__(self, h_wall):
        b = self.b_rest.index_add(0, self.rows, self.ap * h_wall)
        h = linear_solve(self.s["ad"], self.s["au"], b, self.solver)
        return ((h_wall - h[self.rows]) / self.ca).mean() * self.scale

    def close(self):
        self.solver.close()


def nusselt_wall_gradient(prob: NusseltProblem, h_wall):
    """J and dJ/dh_f for every hot-wall face (one forward, one adjoint solve)."""
    hw = torch.tensor(np.asarray(h_wall, np.float64), device="cuda", requires_grad=True)
    j = prob(hw)
    j.backward()
    return float(j.detach()), hw.grad.cpu().numpy()


def nusselt_fd(prob: NusseltProblem, h_wall, idx, step):
    """Central differences of J in the wall enthalpies idx (two solves each)."""
    out = []
    with torch.no_grad():
        base = torch.tensor(np.asarray(h_wall, np.float64), device="cuda")
        for i in idx:
            e = torch.zeros_like(base)
            e[i] = step
            out.append((float(prob(base + e)) - float(prob(base - e))) / (2 * step))
    return np.array(out)
