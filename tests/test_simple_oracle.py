"""CPU checks of the restated SIMPLE cells (oracle/fvc_oracle_simple.c):
the isothermal lid-driven cavity they drive reaches the known Re = 100
centreline extrema, and the pressure-correction coefficients agree with the
coefficient-only restatement the GPU assembly is already pinned to."""
import numpy as np

from _simple_ref import SimpleRef, cavity


def test_cavity_re100_centreline_extrema(orc):
    # Re = 100 lid-driven cavity (Ghia, Ghia & Shin 1982: u_min ~ -0.211 at
    # y ~ 0.45 on the vertical centreline, v_max ~ 0.175 and v_min ~ -0.245
    # on the horizontal one); a 40 x 40 mesh lands within a few percent
    nx = 40
    s = SimpleRef(orc, cavity(orc, nx))
    for _ in range(300):
        r = s.step()
    assert max(r) < 1e-4
    u = s.w[:, 0].reshape(nx, nx)
    v = s.w[:, 1].reshape(nx, nx)
    uc = 0.5 * (u[:, nx // 2 - 1] + u[:, nx // 2])
    vc = 0.5 * (v[nx // 2 - 1, :] + v[nx // 2, :])
    y = (np.arange(nx) + 0.5) / nx
    assert -0.23 < uc.min() < -0.19 and 0.40 < y[uc.argmin()] < 0.52
    assert 0.16 < vc.max() < 0.19
    assert -0.27 < vc.min() < -0.23


def test_residuals_decrease(orc):
    s = SimpleRef(orc, cavity(orc, 12, kind="tri"))
    hist = [s.step() for _ in range(40)]
    assert hist[-1][0] < 0.05 * hist[1][0] and hist[-1][2] < 0.05 * hist[1][2]


def test_pc_coefficients_match_pressure_restatement(orc):
    case = cavity(orc, 10, kind="quad", jitter=0.2)
    n = case["numel"]
    rng = np.random.default_rng(3)
    d = rng.uniform(0.5, 1.5, (n, 2))
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
    w = rng.uniform(-1, 1, (n, 2))
    orc.pform_pc(case, w, d, np.zeros(n), np.zeros((n, 2)), ia, ja, 1, ad, au, b, rc)
    m = case["mesh"]
    ad0, au0 = orc.pform_pressure(m.coor, np.concatenate([m.ix, np.ones((n, 1), np.int32)], 1),
                                  m.nshared, case["nelcon"], case["num"], ia, ja, 1,
                                  kprop=np.ones(n), dsim=d, pin_cell=1)
    assert np.array_equal(ad, ad0) and np.array_equal(au, au0)
    # the right-hand side is minus the face mass fluxes: it sums to zero
    # over the cells (every interior flux appears twice, walls carry none)
    assert abs(b.sum()) < 1e-12 * np.abs(b).sum()


def test_product_cavity_builder_matches_oracle_chain(orc):
    from _simple_ref import cavity
    from fortranfvcell_gb300.cases import lid_driven_cavity
    for kind, nx, jit in (("quad", 16, 0.0), ("tri", 9, 0.1), ("mixed", 10, 0.2)):
        a = cavity(orc, nx, kind=kind, jitter=jit)
        b = lid_driven_cavity(nx, kind=kind, jitter=jit)
        for k in ("coor", "ix", "nelcon", "num", "ident", "pedge", "sedge", "e"):
            assert np.array_equal(a[k], b[k]), (kind, k)


def test_ideal_gas_momentum_hydrostatic_rest(orc):
    # at rest with a uniform density rho != rho_ref and the hydrostatic
    # pressure p = (rho - rho_ref) g . x, buoyancy balances the pressure
    # force in every cell (second-order face pressure is exact for a linear p)
    case = cavity(orc, 10)
    case["sedge"][:] = 0.0                  # fixed walls all round (no lid)
    n = case["numel"]
    m = case["mesh"]
    xc = m.coor[m.ix - 1].mean(axis=1)
    rho_ref = case["e"][0, 1]
    rho = 1.3 * rho_ref
    grav = np.array([0.0, -9.81])
    p = (rho - rho_ref) * (xc @ grav)
    gp = np.tile((rho - rho_ref) * grav, (n, 1))
    ro = np.full((n, 3), rho)
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    z2 = np.zeros((n, 2))
    for comp in (1, 2):
        b, rc = np.zeros(n), np.zeros(n)
        orc.pform_momentum_idg(case, comp, 1, np.zeros(n), p, z2, z2, z2, gp, ro, np.zeros(n),
                               grav, 1e10, ia, ja, 1, b, np.zeros((n, 4)), z2.copy(), rc,
                               ad=np.zeros(n), au=np.zeros(ja.size))
        scale = abs(rho - rho_ref) * 9.81 / n
        assert np.abs(b).max() < 1e-12 * scale * n and np.abs(rc).max() < 1e-12 * scale * n


def test_ideal_gas_momentum_reduces_to_incompressible(orc):
    # constant density equal to e(2), no divergence, no gravity: the ideal-gas
    # cell gives the incompressible cell's system (up to the rounding of the
    # interpolated face density)
    case = cavity(orc, 9, kind="mixed", jitter=0.2)
    n = case["numel"]
    rng = np.random.default_rng(11)
    w, gu, gv, gp = (rng.uniform(-1, 1, (n, 2)) for _ in range(4))
    u, p = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    ro = np.full((n, 3), case["e"][0, 1])
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    out = []
    for idg in (False, True):
        ad, au, b = np.zeros(n), np.zeros(ja.size), np.zeros(n)
        im, d, rc = np.zeros((n, 4)), np.zeros((n, 2)), np.zeros(n)
        if idg:
            orc.pform_momentum_idg(case, 1, 1, u, p, w, gu, gv, gp, ro, np.zeros(n),
                                   np.zeros(2), 0.2, ia, ja, 1, b, im, d, rc, ad=ad, au=au)
        else:
            orc.pform_momentum(case, 1, 1, u, p, w, gu, gv, gp, 0.2, ia, ja, 1, b, im, d, rc,
                               ad=ad, au=au)
        out.append((ad, au, b, im, d, rc))
    for x, y in zip(*out):
        np.testing.assert_allclose(y, x, rtol=1e-12, atol=1e-14 * np.abs(x).max())


def test_ideal_gas_pc_reduces_to_incompressible_and_stores_mass(orc):
    case = cavity(orc, 9, kind="mixed", jitter=0.2)
    n = case["numel"]
    nsh = case["nshared"]
    case["pedge"][:, :nsh] = np.where(case["nelcon"] < 0,
                                      np.random.default_rng(1).integers(0, 3, (n, nsh)), 0)
    rng = np.random.default_rng(4)
    w, d, gp = rng.uniform(-1, 1, (n, 2)), rng.uniform(0.5, 1.5, (n, 2)), rng.uniform(-1, 1, (n, 2))
    p = rng.uniform(-1, 1, n)
    ia, ja, _ = orc.datastruc(case["ident"], 1, True)
    ro = np.full((n, 3), case["e"][0, 1])
    outs = []
    for idg in (False, True):
        ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
        if idg:
            orc.pform_pc_idg(case, w, d, p, gp, ro, 0.1, ia, ja, 1, ad, au, b, rc)
        else:
            orc.pform_pc(case, w, d, p, gp, ia, ja, 1, ad, au, b, rc)
        outs.append((ad, au, b, rc))
    (ad0, au0, b0, rc0), (ad1, au1, b1, rc1) = outs
    assert np.array_equal(ad1, ad0) and np.array_equal(au1, au0) and np.array_equal(b1, b0)
    assert np.array_equal(rc1, np.abs(rc0))
    # at rest the right-hand side is the mass storage -A (rho - rho_n)/dt
    ro = rng.uniform(1.0, 1.3, (n, 3))
    b = np.zeros(n)
    orc.pform_pc_idg(case, np.zeros((n, 2)), d, np.zeros(n), np.zeros((n, 2)), ro, 0.1, ia, ja,
                     1, np.zeros(n), np.zeros(ja.size), b, np.zeros(n))
    m = case["mesh"]
    area = np.zeros(n)
    for c in range(n):
        xy = m.coor[m.ix[c, :m.nsides[c]] - 1]
        area[c] = 0.5 * abs(np.dot(xy[:, 0], np.roll(xy[:, 1], -1))
                            - np.dot(xy[:, 1], np.roll(xy[:, 0], -1)))
    np.testing.assert_allclose(b[case["num"] - 1], -area * (ro[:, 2] - ro[:, 1]) / 0.1,
                               rtol=1e-12)


def test_ideal_gas_density_and_enthalpy(orc):
    t = np.array([20.0, -10.0, 300.0])
    ro = np.zeros((3, 3))
    orc.ideal_gas(ro, t, 3)
    M = 0.21 * 0.032 + 0.78 * 0.028 + 0.01 * 0.03995
    np.testing.assert_allclose(ro[:, 2], 101325.0 * M / (8.31431 * (t + 273.15)), rtol=1e-15)
    assert abs(ro[0, 2] - 1.204) < 1e-3                     # air at 20 C
    e = np.zeros((1, 10))
    e[0, 3], e[0, 4] = 1012.0, 20.0
    h, tt = np.zeros(3), t.copy()
    orc.enthalpy_temp(h, tt, e, False)
    np.testing.assert_allclose(h, 1012.0 * (t - 20.0))
    t2 = np.zeros(3)
    orc.enthalpy_temp(h, t2, e, True)
    np.testing.assert_allclose(t2, t, rtol=1e-15)


def test_natural_convection_nusselt(orc):
    # differentially heated cavity, ideal gas with the energy equation:
    # hot-wall Nusselt numbers near de Vahl Davis (1983), 1.118 at Ra = 1e3
    # and 2.243 at Ra = 1e4 (coarse meshes: within 2% and 3%)
    from oracle.simple_ref import GasSimpleRef
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from _simple_ref import hot_wall_nusselt
    for nx, ra, nit, nu_ref, tol in ((16, 1e3, 300, 1.118, 0.02), (24, 1e4, 400, 2.243, 0.03)):
        c = natural_convection_cavity(nx, ra=ra)
        s = GasSimpleRef(orc, c, dt=1e10)
        for _ in range(nit):
            r = s.step()
        assert max(r[:3]) < 1e-12
        nu = hot_wall_nusselt(c, s.temp)
        assert abs(nu - nu_ref) < tol * nu_ref, (ra, nu)
        # buoyancy turns the flow clockwise: up along the hot wall
        v = s.w[:, 1].reshape(nx, nx)
        assert v[nx // 2, 0] > 0 and v[nx // 2, -1] < 0
