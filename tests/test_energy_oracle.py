"""CPU checks of the restated energy / transport cells (src/CellibTrans.f in
oracle/fvc_oracle_simple.c).  The reference ships no outputs of these
routines, so they are pinned by exact discrete solutions: on a uniform
quadrilateral mesh the cell-centred scheme reproduces a linear
conduction profile, a constant field under a uniform velocity and a linear
field's Green-Gauss gradient exactly."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from _simple_ref import cavity


def energy_case(orc, nx, kc=0.5, cesp=1.0, tref=0.0, cc=0.0, limiter=7):
    case = cavity(orc, nx)
    case["e"] = np.zeros((1, 10))
    case["e"][0, 1], case["e"][0, 2], case["e"][0, 3] = 1.0, kc, cesp
    case["e"][0, 4], case["e"][0, 5], case["e"][0, 6] = tref, cc, limiter
    n, nsh = case["numel"], case["nshared"]
    case["pe"] = np.zeros((n, nsh + 1), np.int32)
    case["se"] = np.zeros((n, nsh + 1))
    return case


def boundary_faces(case):
    """(cell, face, midpoint x, midpoint y) of every boundary face."""
    coor, ix, nelcon = case["coor"], case["ix"], case["nelcon"]
    nsh = case["nshared"]
    out = []
    for c in range(case["numel"]):
        for f in range(nsh):
            if nelcon[c, f] < 0:
                a = coor[ix[c, f] - 1]
                b = coor[ix[c, (f + 1) % nsh] - 1]
                out.append((c, f, 0.5 * (a[0] + b[0]), 0.5 * (a[1] + b[1])))
    return out


def centroids(case):
    coor, ix, nsh = case["coor"], case["ix"], case["nshared"]
    return coor[ix[:, :nsh] - 1].mean(axis=1)


def assemble_and_solve(orc, case, lib, u, w, ro, dt=1.0):
    n = case["numel"]
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
    orc.pform_energy(case, lib, 1, case["pe"], case["se"], u, u, ro, w, np.zeros((n, 2)), dt,
                     ia, ja, 1, b, rc, ad=ad, au=au)
    rows = np.repeat(np.arange(n), np.diff(ia))
    A = sp.csr_matrix((au, (rows, ja - 1)), shape=(n, n)) + sp.diags(ad)
    x = spla.spsolve(A.tocsc(), b)
    return x[case["num"] - 1], rc      # back to cell order


def conduction_bcs(case, left, right):
    for c, f, xm, ym in boundary_faces(case):
        if abs(xm) < 1e-12:
            case["pe"][c, f], case["se"][c, f] = 1, left
        elif abs(xm - 1.0) < 1e-12:
            case["pe"][c, f], case["se"][c, f] = 1, right
        else:
            case["pe"][c, f], case["se"][c, f] = 0, 0.0     # adiabatic: zero flux


def test_transport_linear_conduction_exact(orc):
    case = energy_case(orc, 12, kc=0.7)
    conduction_bcs(case, 1.0, 0.0)
    n = case["numel"]
    T, _ = assemble_and_solve(orc, case, 4, np.zeros(n), np.zeros((n, 2)), np.ones((n, 3)))
    xc = centroids(case)[:, 0]
    np.testing.assert_allclose(T, 1.0 - xc, rtol=0, atol=1e-12)


def test_enthalpy_linear_conduction_and_integer_enthalpy(orc):
    # lib 3 solves for h = cEsp (T - tRef) with conductivity kc/cEsp; the
    # boundary enthalpy is an integer in the reference (truncated toward 0)
    case = energy_case(orc, 10, kc=2.0, cesp=1000.0, tref=0.5)
    conduction_bcs(case, 1.5, 0.5)                 # h = 1000 and 0
    n = case["numel"]
    args = (np.zeros(n), np.zeros((n, 2)), np.ones((n, 3)))
    h, _ = assemble_and_solve(orc, case, 3, *args)
    xc = centroids(case)[:, 0]
    np.testing.assert_allclose(h, 1000.0 * (1.0 - xc), rtol=0, atol=1e-9)
    # 1.5007 K gives 1000.7 J/kg, truncated to 1000; -0.9993 K gives -999.3 -> -999
    conduction_bcs(case, 1.5007, 0.5 - 0.9993)
    h2, _ = assemble_and_solve(orc, case, 3, *args)
    np.testing.assert_allclose(h2, 1000.0 - 1999.0 * xc, rtol=0, atol=1e-9)


def test_uniform_flow_keeps_constant_field(orc):
    # uniform velocity, inflow at x = 0 (pedge 2, value 0.8), outflow at x = 1
    # (pedge 4), walls with zero flux: the constant field solves the system
    for lib, uin in ((4, 0.8), (3, 800.0)):
        case = energy_case(orc, 10, kc=1e-3, cesp=1000.0 if lib == 3 else 1.0)
        for c, f, xm, ym in boundary_faces(case):
            if abs(xm) < 1e-12:
                case["pe"][c, f], case["se"][c, f] = 2, 0.8
            elif abs(xm - 1.0) < 1e-12:
                case["pe"][c, f] = 4
        n = case["numel"]
        w = np.tile([1.0, 0.0], (n, 1))
        T, _ = assemble_and_solve(orc, case, lib, np.full(n, uin), w, np.ones((n, 3)))
        np.testing.assert_allclose(T, uin, rtol=1e-10)


def test_time_term_and_source(orc):
    case = energy_case(orc, 6, cc=2.0)
    n, nsh = case["numel"], case["nshared"]
    rng = np.random.default_rng(5)
    u, u0 = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    ro = rng.uniform(0.5, 1.5, (n, 3))
    case["pe"][::3, nsh] = 1
    case["se"][:, nsh] = rng.uniform(-1, 1, n)
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    area = 1.0 / 36.0
    src = np.where(case["pe"][:, nsh] != 0, case["se"][:, nsh] * area, 0.0)
    for lib in (3, 4):
        for bs in (False, True):
            b = np.zeros(n)
            orc.pform_energy(case, lib, 4, case["pe"], case["se"], u, u0, ro, np.zeros((n, 2)),
                             np.zeros((n, 2)), 0.1, ia, ja, 1, b, np.zeros(n), bs=bs)
            m2 = ro[:, 1] * 2.0 * area / 0.1
            want = m2 * u
            if bs:
                want = 2 * want - 0.5 * (ro[:, 0] * 2.0 * area / 0.1) * u0
            want = want + src
            np.testing.assert_allclose(b[case["num"] - 1], want, rtol=1e-13, atol=1e-15)


def test_gradient_of_linear_field_is_exact_inside(orc):
    case = energy_case(orc, 8)
    n = case["numel"]
    xc = centroids(case)
    u = 0.3 * xc[:, 0] - 1.7 * xc[:, 1] + 0.25
    interior = (case["nelcon"] > 0).all(axis=1)
    for lib in (3, 4):
        g = np.zeros((n, 2))
        orc.gform_energy(case, lib, case["pe"], case["se"], u, g)
        np.testing.assert_allclose(g[interior], np.tile([0.3, -1.7], (interior.sum(), 1)),
                                   rtol=0, atol=1e-12)
