"""BiCGSTAB where the reference's recurrence divides by zero.

pbicgstab (src/Iterativos.f:140-234) forms alpha = (r0.s)/(r0.v),
w = (t.s)/(t.t) and beta = (r0.s_new/rr0)(alpha/w) with no test of the
denominators; an exact zero gives Inf/NaN, the iteration runs on to maxit
and the reference STOPs (the restated reference returns non-convergence
with a NaN solution, checked here).  The GPU solvers guard those branches
only: t = 0 gives w = 0 (the alpha step already solved the system), a zero
denominator in the middle of a solve restarts the recurrence from the
current residual, and one in an iteration that itself started from its
residual ends the solve with FVC_ERR_BREAKDOWN and a finite x.  Solves
without a breakdown are unchanged (the parity tests)."""
import numpy as np
import pytest

from _systems import pressure, unsymmetric

pytestmark = pytest.mark.gpu


def _diag2(n=64):
    # A = 2 I on a one-off-diagonal structure (zero values), Jacobi m = 2:
    # z = p/2 and v = 2 z = p are exact, alpha = 1, s' = s - v = 0 and t = 0
    ia = np.arange(1, n + 2, dtype=np.int32)
    ja = np.array([(i + 1) % n + 1 for i in range(n)], np.int32)
    b = np.random.default_rng(1).uniform(-1.0, 1.0, n)
    return dict(n=n, ia=ia, ja=ja, nad=n, ad=np.full(n, 2.0), au=np.zeros(n), b=b)


def _indefinite2():
    # A = [[1, -1.25], [-1.25, 1]] (symmetric, indefinite, nonsingular),
    # b = (2, 1): r0.(A r0) = 0 exactly, so alpha = (r0.r0)/0 at the start
    return dict(n=2, ia=np.array([1, 2, 3], np.int32), ja=np.array([2, 1], np.int32), nad=2,
                ad=np.ones(2), au=np.array([-1.25, -1.25]), b=np.array([2.0, 1.0]))


def _reference(orc, s, maxit=50):
    x = np.zeros(s["n"])
    rc, st = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x, s["b"].copy(),
                        s["ia"], s["ja"], s["n"], s["nad"], True, 1e-8, maxit, 2, 1)
    return rc, st, x


def test_exact_alpha_step_converges_where_the_reference_gives_nan(fvc, orc):
    s = _diag2()
    rc, _, x_ref = _reference(orc, s)
    assert rc != 0 and not np.isfinite(x_ref).all()
    x = np.zeros(s["n"])
    st = fvc.solver(s["ad"], s["au"], s["au"], x, s["b"], s["ia"], s["ja"], s["n"], s["nad"],
                    True, 1e-8, 50, 2, 1)
    assert st.status == 0 and st.iterations == 1
    np.testing.assert_array_equal(x, s["b"] / 2.0)


def test_breakdown_at_the_start_is_reported(fvc, orc):
    from fortranfvcell_gb300 import FvcError, _lib
    s = _indefinite2()
    rc, _, x_ref = _reference(orc, s)
    assert rc != 0 and not np.isfinite(x_ref).all()
    x = np.zeros(2)
    with pytest.raises(FvcError) as e:
        fvc.solver(s["ad"], s["au"], s["au"], x, s["b"], s["ia"], s["ja"], 2, 2, True, 1e-8, 50,
                   2, 1)
    assert e.value.status == _lib.FVC_ERR_BREAKDOWN
    assert np.isfinite(x).all()


def test_breakdowns_stay_in_their_system_of_a_batch(orc):
    # the two systems above between two ordinary ones in one batched launch:
    # each ends with its own status, the ordinary ones match the reference
    import torch
    from fortranfvcell_gb300 import Context, _lib, make_opts, mesh, pack_block_diagonal
    plain = []
    for k, (kind, nx) in enumerate([("mixed", 9), ("quad", 12)]):
        m = mesh.square_mesh(nx, kind=kind, jitter=0.2 if kind != "quad" else 0.0, seed=k)
        u = unsymmetric(pressure(orc, m, 1, True), seed=k)
        u["b"] = np.random.default_rng(200 + k).uniform(-1, 1, u["n"])
        plain.append(u)
    systems = [plain[0], _diag2(), _indefinite2(), plain[1]]
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    b = np.zeros(pk["neq"])
    for s, r in zip(systems, pk["rows"]):
        b[r] = s["b"]
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
    rc, st = ctx.solve_batched(pk["row_start"], bd, xd, 1e-10, 2000, make_opts("fp64", init=1),
                               raise_on_error=False, codes=[2, 2, 2, 2])
    x = xd.cpu().numpy()
    ctx.close()
    assert rc == _lib.FVC_ERR_BREAKDOWN
    assert [t.status for t in st] == [0, 0, _lib.FVC_ERR_BREAKDOWN, 0]
    assert np.isfinite(x).all()
    np.testing.assert_array_equal(x[pk["rows"][1]], systems[1]["b"] / 2.0)
    for k in (0, 3):
        s = systems[k]
        x_ref = np.zeros(s["n"])
        rc_o, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref,
                              s["b"].copy(), s["ia"], s["ja"], s["n"], s["nad"], True, 1e-10,
                              2000, 2, 1)
        assert rc_o == 0
        err = np.linalg.norm(x[pk["rows"][k]] - x_ref) / np.linalg.norm(x_ref)
        assert err <= 1e-8, (k, err)


def test_dropin_breakdown_stops_like_the_reference(fvc, tmp_path):
    # through solver_ (the drop-in): the reference would run its NaN to
    # maxit, print its BiCGSTAB warning and STOP; so does the drop-in, in a
    # child process so that the test runner survives
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "breakdown.py"
    script.write_text(f"""
import sys, ctypes as C, numpy as np
sys.path.insert(0, {root!r})
import fortranfvcell_gb300 as f
L = f.load()
ad = np.ones(2); au = np.array([-1.25, -1.25]); b = np.array([2.0, 1.0]); x = np.zeros(2)
ia = np.array([1, 2, 3], np.int32); ja = np.array([2, 1], np.int32)
i32 = lambda v: C.byref(C.c_int32(v)); f64 = lambda v: C.byref(C.c_double(v))
p = lambda a: a.ctypes.data_as(C.c_void_p)
L.fvc_solver(p(ad), p(au), p(au), p(x), p(b), C.cast(p(ia), C.POINTER(C.c_int32)),
             C.cast(p(ja), C.POINTER(C.c_int32)), i32(2), i32(2), i32(1), f64(1e-8),
             i32(50), i32(2), i32(1), i32(0))
print("RETURNED", bool(np.isfinite(x).all()))
""")
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, timeout=300)
    assert "BiPCGSTAB no convergence reached after" in r.stdout
    assert "RETURNED" not in r.stdout and r.returncode == 0
    env = dict(os.environ, FVC_STOP_ON_ERROR="0")
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, timeout=300,
                       env=env)
    assert "RETURNED True" in r.stdout
