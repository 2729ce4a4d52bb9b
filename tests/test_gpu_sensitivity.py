"""Adjoint wall-temperature sensitivity of the hot-wall Nusselt number
(fortranfvcell_gb300.sensitivity) at a converged natural-convection state:
one adjoint solve against central finite differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_nusselt_wall_gradient_matches_finite_differences(orc):
    from fortranfvcell_gb300 import sensitivity as sv
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    from _simple_ref import hot_wall_nusselt
    c = natural_convection_cavity(16, ra=1e3)
    cells, faces, _, _ = sv.wall_faces(c, 0.0)
    rng = np.random.default_rng(11)
    t_cold = c["t0"] - 0.5
    c["sedgeE"][cells, faces] = t_cold + (1.0 + rng.normal(0.0, 0.05, cells.size))
    loop = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"], c["e"],
                      opts=simple_opts())
    loop.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
    res, _ = loop.iterate_energy(300)
    assert res[-1, :3].max() < 1e-12
    sysd = sv.frozen_energy_system(c, loop)
    t_loop, _, _ = loop.energy_fields()
    loop.close()
    prob = sv.NusseltProblem(c, sysd, tol=1e-13)
    j, g = sv.nusselt_wall_gradient(prob, sysd["h_wall"])
    # the frozen system reproduces the converged heat transfer (the wall
    # temperatures the cells used are the truncated enthalpies) to the
    # loop's enthalpy solver tolerance (1e-8)
    h_t = c["t0"] - 0.5 + (sysd["tref"] + sysd["h_wall"] / sysd["cp"] - t_cold)
    assert abs(j - hot_wall_nusselt_at(c, t_loop, h_t)) < 1e-4 * abs(j)
    idx = rng.choice(g.size, 4, replace=False)
    fd = sv.nusselt_fd(prob, sysd["h_wall"], idx, step=sysd["cp"] * 1e-3)
    # the same differences through the restated reference BiCGSTAB
    # (src/Iterativos.f:140-234) on the frozen system's host arrays
    fd_ref = _oracle_fd(orc, prob, idx, sysd["cp"] * 1e-3, 1e-13)
    prob.close()
    # J is affine in the wall enthalpies: the differences are exact up to the
    # two iterative solves (each to 1e-13 of its own initial residual)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-6)
    np.testing.assert_allclose(g[idx], fd_ref, rtol=1e-6)
    assert (g > 0).all()          # a warmer hot-wall face raises the wall heat flux


def _oracle_fd(orc, prob, idx, step, tol):
    s = prob.s
    n = int(s["ad"].numel())
    ad, au, b_rest = s["ad"].cpu().numpy(), s["au"].cpu().numpy(), prob.b_rest.cpu().numpy()
    hw0 = np.asarray(s["h_wall"], np.float64)

    def jval(hw):
        b = b_rest.copy()
        np.add.at(b, s["rows"], s["ap"] * hw)
        x = np.zeros(n)
        st, _ = orc.solver(ad.copy(), au.copy(), au.copy(), x, b, s["ia"], s["ja"], n, s["nad"],
                           True, tol, 100000, 2, 1)
        assert st == 0
        return float(np.mean((hw - x[s["rows"]]) / s["ca"]) * prob.scale)
    out = []
    for i in idx:
        e = np.zeros_like(hw0)
        e[i] = step
        out.append((jval(hw0 + e) - jval(hw0 - e)) / (2 * step))
    return np.array(out)


def hot_wall_nusselt_at(c, temp, t_wall):
    """Mean over the hot faces of (T_f - T_P)/(h/2) L/dT on uniform quads."""
    nx = int(round(np.sqrt(c["numel"])))
    h = c["side"] / nx
    tp = temp.reshape(nx, nx)[:, 0]
    return float(np.mean((t_wall - tp) / (0.5 * h)) * c["side"] / 1.0)
