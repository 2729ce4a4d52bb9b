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
