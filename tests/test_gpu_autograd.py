"""Differentiable GPU solves (fortranfvcell_gb300.autograd): the adjoint
gradients of a scalar loss against central finite differences of the
restated reference solver, and torch's gradcheck."""
import numpy as np
import pytest

from _systems import pressure, unsymmetric

pytestmark = pytest.mark.gpu


def system(orc, sym):
    from fortranfvcell_gb300 import mesh
    s = pressure(orc, mesh.square_mesh(6, kind="mixed", jitter=0.2, seed=1), 1, True)
    if not sym:
        s = unsymmetric(s, seed=3)
    else:
        s["ad"] = s["ad"].copy()
        s["ad"][s["ad"] > 1e30] = 4.0     # drop the pin: a plain SPD Laplacian + diagonal
        s["ad"] = s["ad"] + 0.5
    return s


def ref_solve(orc, s, ad, au, b, code):
    x = np.zeros(s["n"])
    st, _ = orc.solver(ad.copy(), au.copy(), au.copy(), x, b.copy(), s["ia"], s["ja"], s["n"],
                       s["nad"], True, 1e-14, 100000, code, 1)
    assert st == 0
    return x


@pytest.mark.parametrize("sym,code", [(False, 2), (True, 1)])
def test_adjoint_gradients_match_finite_differences(orc, sym, code):
    import torch
    from fortranfvcell_gb300.autograd import CsrdSystem, linear_solve
    s = system(orc, sym)
    n, nad = s["n"], s["nad"]
    rng = np.random.default_rng(5)
    b = rng.uniform(-1, 1, n)
    wt = rng.uniform(-1, 1, n)
    sysg = CsrdSystem(s["ia"], s["ja"], n, code=code, tol=1e-13)
    dev = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
    ad_t, au_t, b_t = dev(s["ad"]), dev(s["au"][:nad]), dev(b)
    x = linear_solve(ad_t, au_t, b_t, sysg)
    loss = (x * torch.tensor(wt, device="cuda")).sum()
    loss.backward()
    g_ad, g_au, g_b = (t.grad.cpu().numpy() for t in (ad_t, au_t, b_t))
    sysg.close()
    loss_of = lambda ad, au, bb: float(wt @ ref_solve(orc, s, ad, au, bb, code))
    ad0, au0 = s["ad"].copy(), s["au"][:nad].copy()
    for i in rng.choice(n, 4, replace=False):
        h = 1e-6 * max(1.0, abs(b[i]))
        bp, bm = b.copy(), b.copy()
        bp[i] += h
        bm[i] -= h
        fd = (loss_of(ad0, au0, bp) - loss_of(ad0, au0, bm)) / (2 * h)
        assert abs(g_b[i] - fd) <= 1e-6 * max(1.0, abs(fd)), ("b", i)
        h = 1e-6 * abs(ad0[i])
        ap, am = ad0.copy(), ad0.copy()
        ap[i] += h
        am[i] -= h
        fd = (loss_of(ap, au0, b) - loss_of(am, au0, b)) / (2 * h)
        assert abs(g_ad[i] - fd) <= 1e-6 * max(1.0, abs(fd)), ("ad", i)
    for k in rng.choice(nad, 4, replace=False):
        h = 1e-6 * max(abs(au0[k]), 1e-3)
        up, um = au0.copy(), au0.copy()
        up[k] += h
        um[k] -= h
        fd = (loss_of(ad0, up, b) - loss_of(ad0, um, b)) / (2 * h)
        assert abs(g_au[k] - fd) <= 1e-6 * max(1.0, abs(fd)), ("au", k)


def test_gradcheck_small_system(orc):
    import torch
    from fortranfvcell_gb300 import mesh
    from fortranfvcell_gb300.autograd import CsrdSystem, linear_solve
    s = unsymmetric(pressure(orc, mesh.square_mesh(3, kind="tri", seed=2), 1, True), seed=4)
    n, nad = s["n"], s["nad"]
    # tol 1e-12: on 18 rows a tighter test drives BiCGSTAB to an exactly
    # vanishing s, where omega = t.s / t.t is 0/0 (the reference's recurrence
    # breaks down the same way; the solver reports it as NaN)
    sysg = CsrdSystem(s["ia"], s["ja"], n, code=2, tol=1e-12)
    dev = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
    b = np.random.default_rng(1).uniform(-1, 1, n)
    inputs = (dev(s["ad"]), dev(s["au"][:nad]), dev(b))
    assert torch.autograd.gradcheck(lambda ad, au, bb: linear_solve(ad, au, bb, sysg), inputs,
                                    eps=1e-6, atol=1e-6, rtol=1e-5)
    sysg.close()


@pytest.mark.parametrize("kind,nx", [("mixed", 6), ("tri", 20), ("quad", 40)])
def test_transposed_solve_over_stored_matrix(orc, kind, nx):
    # fvc_solve_transposed: A^T x = b by BiCGSTAB through the mirror slots
    # of A's own storage, against a direct solve of the transposed matrix
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    import torch
    from fortranfvcell_gb300 import Context, make_opts, mesh
    s = unsymmetric(pressure(orc, mesh.square_mesh(nx, kind=kind, jitter=0.2, seed=nx), 1, True),
                    seed=nx)
    n, nad = s["n"], s["nad"]
    rows = np.repeat(np.arange(n), np.diff(s["ia"]))
    A = sp.csr_matrix((s["au"][:nad], (rows, s["ja"][:nad] - 1)), shape=(n, n)) + sp.diags(s["ad"])
    b = np.random.default_rng(nx).uniform(-1, 1, n)
    x_ref = spla.spsolve(A.T.tocsc(), b)
    ctx = Context()
    ctx.set_matrix(1, True, n, nad, s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = ctx.solve_transposed(torch.from_numpy(b).cuda(), x, 1e-12, 10000,
                              make_opts("fp64", init=1))
    assert st.status == 0 and st.iterations > 0
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err < 1e-9, err
    # the same context still solves A x = b
    x2 = torch.zeros_like(x)
    ctx.solve(2, torch.from_numpy(b).cuda(), x2, 1e-12, 10000, make_opts("fp64", init=1))
    x2_ref = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x2.cpu().numpy() - x2_ref) <= 1e-9 * np.linalg.norm(x2_ref)
    ctx.close()


def test_transposed_and_batched_edge_cases(orc):
    # unsupported requests return FVC_ERR_UNSUPPORTED without touching x:
    # a transposed solve on a pattern that is not symmetric, or by PCG or
    # mixed precision; a batched solver code other than PCG / BiCGSTAB.
    # The autotuner runs on a one-row system.
    import torch
    from fortranfvcell_gb300 import Context, FvcError, _lib, make_opts
    # 3 rows, entries (1,2) and (2,3) only: no mirror for either
    ia = np.array([1, 2, 3, 3], np.int32)
    ja = np.array([2, 3], np.int32)
    ad, au = np.array([4.0, 4.0, 4.0]), np.array([-1.0, -1.0])
    ctx = Context()
    ctx.set_matrix(1, True, 3, 2, ad, au, au, ia, ja)
    b = torch.ones(3, dtype=torch.float64, device="cuda")
    x = torch.full((3,), 7.0, dtype=torch.float64, device="cuda")
    for opts in (make_opts("fp64", init=1), make_opts("mixed", init=1)):
        with pytest.raises(FvcError) as e:
            ctx.solve_transposed(b, x, 1e-10, 100, opts)
        assert e.value.status == _lib.FVC_ERR_UNSUPPORTED
    assert bool(torch.all(x == 7.0))
    # the forward solve of the same matrix still works
    st = ctx.solve(2, b, x, 1e-12, 100, make_opts("fp64", init=1))
    assert st.status == 0
    rs = np.array([0, 32], np.int32)     # one system padded to 32 rows is not this matrix
    with pytest.raises(FvcError):
        ctx.solve_batched(np.array([0, 3], np.int32), b, x, 1e-10, 100, codes=[3])
    with pytest.raises(ValueError):
        ctx.solve_batched(rs, b, x, 1e-10, 100, codes=[1, 2])
    ctx.close()
    one = Context()
    one.set_matrix(1, True, 1, 0, np.array([2.0]), np.zeros(1), np.zeros(1),
                   np.array([1, 1], np.int32), np.zeros(1, np.int32))
    o, us = one.autotune(1, "fp64", 5)
    assert us > 0.0
    one.close()
