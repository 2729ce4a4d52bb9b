"""Many SIMPLE cases advanced together (fvc_simple_batch): every stage's
solves of all cases in one persistent launch, one outer iteration of all
cases one CUDA graph.

The batch against each case's own loop (fvc_simple_iterate_energy, whose
outer iteration matches the restated Simple.f iteration, test_gpu_simple):
the two differ only in the summation order of the solvers' reductions, so
at solver tolerances of 1e-13 their residual histories agree to 1e-7, the
bar the single loop meets against the restated iteration.  Cases: heated
lid-driven cavities and heated channel sections (inflow, outflow at a fixed
pressure, a heated wall) of air, the two kinds of the batched benchmark."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _case(kind, nx, re):
    from fortranfvcell_gb300.cases import heated_channel, heated_lid_cavity
    return (heated_channel if kind == "channel" else heated_lid_cavity)(nx, re=re)


def _loop(c, tol=TOL, **kw):
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    lp = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"], c["e"],
                    opts=simple_opts(matriz_u=1, tol_u=tol, tol_pc=tol, **kw))
    lp.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
    return lp


SPECS = [("cavity", 16, 100.0), ("channel", 12, 200.0), ("cavity", 24, 300.0),
         ("channel", 20, 80.0), ("cavity", 10, 50.0)]


def test_channel_loop_matches_reference(orc):
    # the heated channel (inflow pedge 2, outflow pedge 3 at pressure 0,
    # energy pedge 2 / 1 / 4) on the GPU loop against the restated iteration
    from oracle.simple_ref import GasSimpleRef
    c = _case("channel", 10, 150.0)
    ref = GasSimpleRef(orc, c, dt=1e10, tol_pcg=TOL, tol_bcg=TOL, matriz_u=1)
    lp = _loop(c)
    hist = np.array([ref.step() for _ in range(12)])
    res, its = lp.iterate_energy(12)
    w, _ = lp.fields()
    t, _, _ = lp.energy_fields()
    lp.close()
    np.testing.assert_allclose(res, hist, rtol=1e-7, atol=1e-18)
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-9 * np.abs(ref.w).max())
    np.testing.assert_allclose(t, ref.temp, rtol=0, atol=1e-10)
    # every solve ran but the first v-momentum one: the flow starts at rest,
    # so its right-hand side is zero and the reference's test skips it
    assert (its[1:] > 0).all() and its[0, 1] == 0


def test_batch_equals_single_loops():
    from fortranfvcell_gb300.cells import SimpleBatch
    cases = [_case(*sp) for sp in SPECS]
    nit = 10
    single = []
    for c in cases:
        lp = _loop(c)
        r, i = lp.iterate_energy(nit)
        w, p = lp.fields()
        t, _, _ = lp.energy_fields()
        single.append((r, i, w, t))
        lp.close()
    loops = [_loop(c) for c in cases]
    bt = SimpleBatch(loops, "fp64")
    res, its = bt.iterate(nit, 4)
    for k, (c, lp) in enumerate(zip(cases, loops)):
        r, i, w, t = single[k]
        wb, _ = lp.fields()
        tb, _, _ = lp.energy_fields()
        print(f"case {k} {SPECS[k]}: its batch {its[-1, k].tolist()} single {i[-1].tolist()}")
        np.testing.assert_allclose(res[:, k, :], r, rtol=1e-7, atol=1e-18)
        np.testing.assert_allclose(wb, w, rtol=0, atol=1e-9 * np.abs(w).max())
        np.testing.assert_allclose(tb, t, rtol=0, atol=1e-10)
        np.testing.assert_array_equal(its[:, k, :] > 0, i > 0)     # the same skipped solves
    bt.close()
    for lp in loops:
        lp.close()


@pytest.mark.parametrize("precision_u", ["fp64", "mixed"])
def test_batch_mixed_precision_tracks_fp64(precision_u):
    # the batch with FP32-inner p' solves (FP64 refinement to the same
    # tolerances), and u, v, enthalpy solves in FP64 or mixed, against the
    # FP64 batch: the fields after 12 outer iterations at solver tolerance
    # 1e-10
    from fortranfvcell_gb300.cells import SimpleBatch
    cases = [_case(*sp) for sp in SPECS]
    out = {}
    for prec in ("fp64", "mixed"):
        loops = [_loop(c, tol=1e-10) for c in cases]
        bt = SimpleBatch(loops, prec, precision_u if prec == "mixed" else None)
        res, its = bt.iterate(12, 4)
        out[prec] = (res, [lp.fields()[0] for lp in loops],
                     [lp.energy_fields()[0] for lp in loops])
        bt.close()
        for lp in loops:
            lp.close()
    (r64, w64, t64), (rm, wm, tm) = out["fp64"], out["mixed"]
    assert np.all(np.isfinite(rm))
    for k in range(len(cases)):
        dw = np.abs(wm[k] - w64[k]).max() / np.abs(w64[k]).max()
        dt = np.abs(tm[k] - t64[k]).max()
        print(f"case {k}: max rel w diff {dw:.2e}, max T diff {dt:.2e} K")
        assert dw < 1e-5 and dt < 1e-6


def test_batch_skips_the_solves_of_a_case_at_rest():
    # a cavity with the lid at rest and every wall at the initial
    # temperature: every right-hand side is zero, so the reference's tests
    # skip each of its solves (and the p' update); in the batch its systems
    # are masked out of the launches while the other cases run as alone
    from fortranfvcell_gb300.cells import SimpleBatch
    rest = _case("cavity", 12, 100.0)
    rest["sedge"][:] = 0.0
    rest["sedgeE"][rest["pedgeE"] == 1] = rest["t0"]
    others = [_case(*sp) for sp in SPECS[:2]]
    nit = 6
    single = []
    for c in others:
        lp = _loop(c)
        single.append(lp.iterate_energy(nit)[0])
        lp.close()
    loops = [_loop(c) for c in [others[0], rest, others[1]]]
    bt = SimpleBatch(loops, "fp64")
    res, its = bt.iterate(nit, 4)
    w, p = loops[1].fields()
    bt.close()
    assert (its[:, 1, :] == 0).all()
    assert not w.any() and not p.any()
    np.testing.assert_allclose(res[:, 0, :], single[0], rtol=1e-7, atol=1e-18)
    np.testing.assert_allclose(res[:, 2, :], single[1], rtol=1e-7, atol=1e-18)
    for lp in loops:
        lp.close()
