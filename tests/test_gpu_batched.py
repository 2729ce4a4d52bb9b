"""Batched solves (fvc_solve_batched, fvc_solve_batched_ex): many
independent systems of different sizes and cell shapes in one persistent
launch -- pressure-correction systems by PCG, and convection-like
unsymmetric systems by BiCGSTAB beside them -- each checked against the
restated reference solver (src/Iterativos.f:29-106, 140-234) run on that
system alone."""
import numpy as np
import pytest

from _systems import pressure, unsymmetric

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
ITS_TOL = 2


def batch(orc):
    from fortranfvcell_gb300 import mesh
    shapes = [("quad", 1), ("tri", 3), ("quad", 17), ("mixed", 9), ("tri", 14), ("quad", 5),
              ("mixed", 23), ("quad", 31), ("tri", 2), ("mixed", 12)]
    systems = []
    for k, (kind, nx) in enumerate(shapes):
        m = mesh.square_mesh(nx, kind=kind, jitter=0.2 if kind != "quad" else 0.0, seed=k)
        s = pressure(orc, m, 1, True)
        s["b"] = np.random.default_rng(100 + k).uniform(-1, 1, s["n"])
        systems.append(s)
    return systems


def solve_batch(systems, tol, maxit, raise_on_error=True, codes=None, tols=None, its_hint=None):
    import torch
    from fortranfvcell_gb300 import Context, make_opts, pack_block_diagonal
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    b = np.zeros(pk["neq"])
    for s, r in zip(systems, pk["rows"]):
        b[r] = s["b"]
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
    rc, st = ctx.solve_batched(pk["row_start"], bd, xd, tol, maxit, make_opts("fp64", init=1),
                               raise_on_error=raise_on_error, codes=codes, tols=tols,
                               its_hint=its_hint)
    x = xd.cpu().numpy()
    ctx.close()
    return rc, st, [x[r] for r in pk["rows"]]


def test_batched_pcg_matches_reference_per_system(orc):
    systems = batch(orc)
    rc, st, xs = solve_batch(systems, 1e-10, 20000)
    assert rc == 0
    for s, t, x in zip(systems, st, xs):
        x_ref = np.zeros(s["n"])
        status, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref,
                                s["b"].copy(), s["ia"], s["ja"], s["n"], s["nad"], True, 1e-10,
                                20000, 1, 1)
        assert status == 0 and t.status == 0
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err <= REL_TOL, (s["n"], err)
        assert abs(t.iterations - so.iterations) <= ITS_TOL, (s["n"], t.iterations, so.iterations)
        assert abs(t.energy - so.energy) <= 1e-9 * abs(so.energy)


def test_batched_systems_stop_independently(orc):
    # a small iteration limit: the one-cell and the 2x2 systems converge,
    # the large ones report non-convergence, each on its own
    from fortranfvcell_gb300 import _lib
    systems = batch(orc)
    rc, st, _ = solve_batch(systems, 1e-10, 12, raise_on_error=False)
    assert rc == _lib.FVC_ERR_NOCONV
    for s, t in zip(systems, st):
        if s["n"] <= 8:
            assert t.status == 0 and t.iterations <= 12, s["n"]
        if s["n"] >= 200:
            assert t.status == _lib.FVC_ERR_NOCONV and t.iterations == 12, s["n"]


def test_batched_rejects_unaligned_layout(orc):
    import torch
    from fortranfvcell_gb300 import Context, FvcError, pack_block_diagonal
    systems = batch(orc)[:3]
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    bd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
    xd = torch.zeros_like(bd)
    bad = pk["row_start"].copy()
    bad[1] += 1                              # not a multiple of 32
    with pytest.raises(FvcError):
        ctx.solve_batched(bad, bd, xd, 1e-8, 100)
    ctx.close()


def test_batched_mixed_solvers_match_reference_per_system(orc):
    # the u, v, T and p' pattern of a SIMPLE iteration: unsymmetric systems
    # by BiCGSTAB beside p' systems by PCG, with a tolerance per system
    systems = batch(orc)
    codes, tols = [], []
    for k, s in enumerate(systems):
        if k % 2:
            u = unsymmetric(s, seed=k)
            s.update(ad=u["ad"], au=u["au"])
            codes.append(2)
            tols.append(1e-11)
        else:
            codes.append(1)
            tols.append(1e-10)
    rc, st, xs = solve_batch(systems, 0.0, 20000, codes=codes, tols=tols)
    assert rc == 0
    for s, t, x, code, tol in zip(systems, st, xs, codes, tols):
        x_ref = np.zeros(s["n"])
        status, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref,
                                s["b"].copy(), s["ia"], s["ja"], s["n"], s["nad"], True, tol,
                                20000, code, 1)
        assert status == 0 and t.status == 0
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err <= (REL_TOL if code == 1 else 1e-9), (code, s["n"], err)
        # BiCGSTAB's exit iteration moves with the summation order (15%)
        bar = ITS_TOL if code == 1 else max(2, int(0.15 * so.iterations))
        assert abs(t.iterations - so.iterations) <= bar, (code, s["n"], t.iterations,
                                                          so.iterations)


def test_batched_iteration_hints_move_only_the_speed(orc):
    # hints change each system's share of blocks, so only the reductions'
    # summation order: the same solutions to rounding, counts within 2
    # (BiCGSTAB not on the one-cell system 0: its first half-step zeroes the
    # residual and the reference's omega = 0/0 breaks down)
    systems = batch(orc)
    codes = [2 if k % 3 == 1 else 1 for k in range(len(systems))]
    for k, s in enumerate(systems):
        if codes[k] == 2:
            u = unsymmetric(s, seed=k)
            s.update(ad=u["ad"], au=u["au"])
    _, st0, x0 = solve_batch(systems, 1e-10, 20000, codes=codes)
    hints = [5.0 if k % 2 else 500.0 for k in range(len(systems))]
    _, st1, x1 = solve_batch(systems, 1e-10, 20000, codes=codes, its_hint=hints)
    for a, b, t0, t1 in zip(x0, x1, st0, st1):
        assert t0.status == 0 and t1.status == 0
        assert np.linalg.norm(a - b) <= 1e-9 * max(np.linalg.norm(a), 1e-300)
        assert abs(t0.iterations - t1.iterations) <= 2


def test_batched_mixed_precision_reaches_tolerance(orc):
    # mixed precision per system (FP32 iterations, FP64 residual
    # replacement / defect correction): every system of a PCG + BiCGSTAB
    # batch reaches ||b - Ax|| / ||b|| <= 1e-8 recomputed in FP64, and its
    # solution agrees with the FP64 one within that residual times the
    # condition number of these systems (at most ~1e4)
    import torch
    from fortranfvcell_gb300 import Context, make_opts, pack_block_diagonal
    systems = batch(orc)[1:]                 # no one-cell system (BiCGSTAB breakdown)
    codes = []
    for k, s in enumerate(systems):
        if k % 2:
            u = unsymmetric(s, seed=k)
            s.update(ad=u["ad"], au=u["au"])
        codes.append(2 if k % 2 else 1)
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    b = np.zeros(pk["neq"])
    for s, r in zip(systems, pk["rows"]):
        b[r] = s["b"]
    bd = torch.from_numpy(b).cuda()
    xs = {}
    for prec in ("mixed", "fp64"):
        xd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
        o = make_opts(prec, init=1, stop_rule=1)
        rc, st = ctx.solve_batched(pk["row_start"], bd, xd, 1e-8 if prec == "mixed" else 1e-12,
                                   50000, o, codes=codes)
        assert rc == 0, prec
        xs[prec] = xd.cpu().numpy()
        if prec == "mixed":
            for t in st:
                assert t.status == 0 and t.rel_residual <= 1e-8 and t.iterations > 0
    ctx.close()
    for s, r in zip(systems, pk["rows"]):
        xm, x64 = xs["mixed"][r], xs["fp64"][r]
        assert np.linalg.norm(xm - x64) <= 1e-4 * np.linalg.norm(x64), s["n"]
