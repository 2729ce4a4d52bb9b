"""Mixed BiCGSTAB on a system where its FP32-inner defect-correction sweeps
stall: an enthalpy system of the ideal-gas natural-convection cavity
(512 x 512 quads, Ra 1e6).  Those of its FP64 outer iterations from about
the ninth on stall the FP32 sweeps; the fixture takes the first that does.
The kernel stops the sweeps once three in a row each fail to cut the FP64
residual by a tenth, and the synchronous solve finishes in FP64 BiCGSTAB from
that iterate, so precision=mixed reaches the target where FP64 does."""
import numpy as np
import pytest

from _systems import csr_matrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def enthalpy_system():
    import torch
    from fortranfvcell_gb300 import Context, make_opts, mesh
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    c = natural_convection_cavity(512, ra=1e6)
    lp = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"], c["e"],
                    opts=simple_opts(precision="fp64"))
    lp.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
    ia, ja, nad = mesh.datastruc(c["ident"], 1, True)
    try:
        for k in range(1, 25):
            lp.iterate_energy(1)
            if k < 9:
                continue
            ad, au, b = lp.system(4)
            ctx = Context()
            ctx.set_matrix(1, True, ad.size, nad, ad, au, au, ia, ja)
            x = torch.zeros(ad.size, dtype=torch.float64, device="cuda")
            st = ctx.solve(2, torch.from_numpy(b).cuda(), x, 1e-8, 50000,
                           make_opts("mixed", init=1), raise_on_error=False)
            ctx.close()
            if st.status == 0 and 0 < st.inner_iterations < st.iterations:
                return dict(n=ad.size, ia=ia, ja=ja, au=au, ad=ad, nad=nad, k=k), b
    finally:
        lp.close()
    pytest.fail("no enthalpy system of the first 24 outer iterations stalled the FP32 sweeps")


def _solve(s, b, prec, **kw):
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    ctx = Context()
    ctx.set_matrix(1, True, s["n"], s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    x = torch.zeros(s["n"], dtype=torch.float64, device="cuda")
    st = ctx.solve(2, torch.from_numpy(b).cuda(), x, 1e-8, 50000,
                   make_opts(prec, init=1, **kw), raise_on_error=False)
    out = x.cpu().numpy()
    ctx.close()
    return st, out


def test_mixed_bicgstab_stall_finishes_in_fp64(enthalpy_system):
    s, b = enthalpy_system
    A = csr_matrix(s)
    st64, x64 = _solve(s, b, "fp64", stop_rule=1)
    stm, xm = _solve(s, b, "mixed")
    rel = lambda x: np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    print(f"fp64: its {st64.iterations} rel {rel(x64):.2e}; mixed: status {stm.status} "
          f"sweeps {stm.refinements} fp32 its {stm.inner_iterations} its {stm.iterations} "
          f"rel {rel(xm):.2e} ms {stm.solve_ms:.1f}")
    assert st64.status == 0 and stm.status == 0
    assert 0 < stm.inner_iterations < stm.iterations      # the stall and the FP64 finish
    assert rel(xm) <= 2e-8
    # the two answers agree to the conditioning of the solve
    assert np.linalg.norm(xm - x64) <= 1e-4 * np.linalg.norm(x64)


def test_gas_loop_with_every_solve_mixed_runs_through():
    # the same cavity with the FP32-inner solves for momentum and enthalpy
    # too (warm-started from the previous outer iteration): 30 outer
    # iterations run through without a solver error and track the FP64 loop
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    c = natural_convection_cavity(512, ra=1e6)
    hist = {}
    for prec in ("fp64", "mixed"):
        lp = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"],
                        c["e"], opts=simple_opts(precision=prec, precision_u=prec))
        lp.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
        hist[prec] = lp.iterate_energy(30)
        lp.close()
    (rd, itd), (rm, itm) = hist["fp64"], hist["mixed"]
    print("enthalpy its fp64", np.asarray(itd)[-5:].tolist(), "mixed", np.asarray(itm)[-5:].tolist())
    print("last residuals fp64", np.asarray(rd)[-1].tolist(), "mixed", np.asarray(rm)[-1].tolist())
    assert np.all(np.isfinite(rm))
    np.testing.assert_allclose(np.asarray(rm)[-1], np.asarray(rd)[-1], rtol=0.05)


def test_stalled_structure_runs_later_mixed_solves_in_fp64(enthalpy_system):
    # one context: the first mixed BiCGSTAB of the stalling system stalls and
    # is finished in FP64.  The next mixed BiCGSTAB of the same structure
    # (fvc_solve) and an enqueued one (fvc_solve_async, the path graphs
    # capture) then start in FP64 and report no FP32 iterations; a new
    # structure (fvc_matrix_set) clears the route.
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    s, b = enthalpy_system
    A = csr_matrix(s)
    rel = lambda x: np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    ctx = Context()
    ctx.set_matrix(1, True, s["n"], s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    bd = torch.from_numpy(b).cuda()
    om = make_opts("mixed", init=1)
    x1 = torch.zeros(s["n"], dtype=torch.float64, device="cuda")
    st1 = ctx.solve(2, bd, x1, 1e-8, 50000, om, raise_on_error=False)
    x2 = torch.zeros_like(x1)
    st2 = ctx.solve(2, bd, x2, 1e-8, 50000, om, raise_on_error=False)
    print(f"outer iteration {s['k']}: first fp32 its {st1.inner_iterations} sweeps "
          f"{st1.refinements} its {st1.iterations}; second fp32 its {st2.inner_iterations} its "
          f"{st2.iterations}")
    assert st1.status == 0 and 0 < st1.inner_iterations < st1.iterations
    assert st2.status == 0 and st2.inner_iterations == 0 and st2.refinements == 0
    assert st2.iterations > 0 and rel(x2.cpu().numpy()) <= 2e-8
    x3 = torch.zeros_like(x1)
    status = torch.zeros(4, dtype=torch.int32, device="cuda")
    ctx.solve_async(2, bd, x3, 1e-8, 50000, status, om)
    torch.cuda.synchronize()
    stv = status.cpu().numpy()
    assert stv[0] == 0 and stv[1] > 0
    assert rel(x3.cpu().numpy()) <= 2e-8
    # a new structure: the FP32 path again (and the same stall)
    ctx.set_matrix(1, True, s["n"], s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    x4 = torch.zeros_like(x1)
    st4 = ctx.solve(2, bd, x4, 1e-8, 50000, om, raise_on_error=False)
    assert st4.status == 0 and 0 < st4.inner_iterations < st4.iterations
    ctx.close()
