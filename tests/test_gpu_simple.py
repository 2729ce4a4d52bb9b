"""The GPU-resident SIMPLE outer iteration (fvc_simple_*) against the
reference's iteration restated on the CPU (tests/_simple_ref.py): the
same residual history and fields, to the accuracy of the linear solves
(which differ between the two only in rounding)."""
import numpy as np
import pytest

from _simple_ref import SimpleRef, cavity

pytestmark = pytest.mark.gpu


def gpu_loop(case, **kw):
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    return SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                      case["sedge"], case["e"], opts=simple_opts(**kw))


@pytest.mark.parametrize("kind,nx,matriz_u", [("quad", 20, 4), ("tri", 12, 1),
                                              ("mixed", 14, 1)])
def test_simple_loop_matches_reference(orc, kind, nx, matriz_u):
    case = cavity(orc, nx, kind=kind, jitter=0.15 if kind != "quad" else 0.0)
    ref = SimpleRef(orc, case, tol_pcg=1e-13, tol_bcg=1e-13, matriz_u=matriz_u)
    loop = gpu_loop(case, tol_u=1e-13, tol_pc=1e-13, matriz_u=matriz_u)
    nit = 25
    hist = np.array([ref.step() for _ in range(nit)])
    res, its = loop.iterate(nit)
    w, p = loop.fields()
    loop.close()
    np.testing.assert_allclose(res, hist, rtol=1e-7, atol=1e-15)
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-9 * np.abs(ref.w).max())
    np.testing.assert_allclose(p, ref.p, rtol=0, atol=1e-9 * np.abs(ref.p).max())
    if kind == "quad":  # iteration 1 on the uniform mesh: v's right-hand side is zero
        assert its[0, 1] == 0 and its[0, 0] > 0


def test_simple_loop_reaches_steady_cavity(orc):
    # Re = 100 cavity, 200 outer iterations at the reference's default
    # solver tolerances; the GPU and CPU states agree to 1e-6
    case = cavity(orc, 32)
    ref = SimpleRef(orc, case)
    loop = gpu_loop(case)
    hist = np.array([ref.step() for _ in range(200)])
    res, _ = loop.iterate(200)
    w, p = loop.fields()
    assert res[-1].max() < 1e-3 * res[1].max()
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-6)
    np.testing.assert_allclose(res[-1], hist[-1], rtol=1e-3)


def test_simple_loop_mixed_precision_solves(orc):
    case = cavity(orc, 24)
    fp64 = gpu_loop(case)
    mixed = gpu_loop(case, precision="mixed")
    r64, _ = fp64.iterate(60)
    rmx, _ = mixed.iterate(60)
    w64, _ = fp64.fields()
    wmx, _ = mixed.fields()
    np.testing.assert_allclose(rmx[-1], r64[-1], rtol=1e-3)
    np.testing.assert_allclose(wmx, w64, rtol=0, atol=1e-6)


def test_time_steps_and_restart(orc):
    # transient run: two time steps of 10 outer iterations (second-order
    # backward time term), then a restart from downloaded fields
    case = cavity(orc, 12)
    a = gpu_loop(case, dt=0.05, bs=1)
    a.iterate(10)
    a.time_step()
    ra, _ = a.iterate(10)
    w, p = a.fields()
    b = gpu_loop(case, dt=0.05, bs=1)
    b.set_fields(w, p)
    wb, pb = b.fields()
    assert np.array_equal(wb, w) and np.array_equal(pb, p)
    assert np.isfinite(ra).all()


def test_bad_inputs_rejected(orc):
    from fortranfvcell_gb300 import FvcError
    case = cavity(orc, 6)
    with pytest.raises(FvcError):
        gpu_loop(case, int_vel=3)
    with pytest.raises(FvcError):
        gpu_loop(case, matriz_u=2)


def gas_loop(case, **kw):
    loop = gpu_loop(case, **kw)
    loop.enable_energy(case["pedgeE"], case["sedgeE"], case["gravity"], case["t0"])
    return loop


@pytest.mark.parametrize("kind,nx", [("quad", 12), ("tri", 9)])
def test_ideal_gas_loop_matches_reference(orc, kind, nx):
    # transient natural convection (dt 0.5 s, two steps of 8 outer
    # iterations): the GPU loop against the restated iteration, solver
    # tolerances 1e-13 so that the two differ only in rounding
    from oracle.simple_ref import GasSimpleRef
    from fortranfvcell_gb300.cases import natural_convection_cavity
    c = natural_convection_cavity(nx, ra=1e4, kind=kind, jitter=0.15 if kind == "tri" else 0.0)
    ref = GasSimpleRef(orc, c, dt=0.5, tol_pcg=1e-13, tol_bcg=1e-13, matriz_u=1)
    loop = gas_loop(c, dt=0.5, tol_u=1e-13, tol_pc=1e-13, matriz_u=1)
    hist, res = [], []
    for step in range(2):
        if step:
            ref.end_step()
            ref.start_step()
            loop.time_step()
        hist += [ref.step() for _ in range(8)]
        r, _ = loop.iterate_energy(8)
        res.append(r)
    res = np.concatenate(res)
    np.testing.assert_allclose(res, np.array(hist), rtol=1e-7, atol=1e-18)
    w, p = loop.fields()
    t, h, ro = loop.energy_fields()
    loop.close()
    np.testing.assert_allclose(w, ref.w, rtol=0, atol=1e-9 * np.abs(ref.w).max())
    np.testing.assert_allclose(t, ref.temp, rtol=0, atol=1e-10)
    np.testing.assert_allclose(ro, ref.ro, rtol=1e-13)


def test_ideal_gas_loop_reaches_steady_convection(orc):
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from _simple_ref import hot_wall_nusselt
    c = natural_convection_cavity(16, ra=1e3)
    loop = gas_loop(c)
    res, its = loop.iterate_energy(300)
    t, _, _ = loop.energy_fields()
    loop.close()
    assert res[-1, :3].max() < 1e-12 and (its[:, 3] > 0).any()
    assert abs(hot_wall_nusselt(c, t) - 1.118) < 0.02 * 1.118


def test_restart_from_saved_state(orc, tmp_path):
    # a step, then the state saveSimple writes (w, w0, p, en, en0, ro).  As
    # with the reference's load, the restart does not carry the gradients
    # the ghost cells extrapolate with, so it is compared with the restated
    # iteration restarted from the same state (tight solver tolerances), and
    # the restart through the file with the one from the arrays
    from fortranfvcell_gb300 import io
    from oracle.simple_ref import GasSimpleRef
    from fortranfvcell_gb300.cases import natural_convection_cavity
    c = natural_convection_cavity(10, ra=1e4)
    kw = dict(dt=0.5, tol_u=1e-13, tol_pc=1e-13)
    a = gas_loop(c, **kw)
    a.iterate_energy(6)
    a.time_step()
    st = a.get_state(energy=True)
    a.close()
    path = str(tmp_path / "restart.dat")
    io.save_simple(path, 1, 0.5, st["w"], st["w0"], st["p"], st["ro"], en=st["en"],
                   en0=st["en0"])
    b = gas_loop(c, **kw)
    b.set_state(st)
    rb, _ = b.iterate_energy(6)
    b.close()
    ref = GasSimpleRef(orc, c, dt=0.5, tol_pcg=1e-13, tol_bcg=1e-13)
    ref.w, ref.w0, ref.p = st["w"].copy(), st["w0"].copy(), st["p"].copy()
    ref.en, ref.en0, ref.ro = st["en"].copy(), st["en0"].copy(), st["ro"].copy()
    orc.enthalpy_temp(ref.en, ref.temp, c["e"], True)
    ref.start_step()
    hist = np.array([ref.step() for _ in range(6)])
    np.testing.assert_allclose(rb, hist, rtol=1e-7, atol=1e-18)
    f = gas_loop(c, **kw)
    f.set_state(io.load_simple(path, c["numel"], energy=True))
    rf, _ = f.iterate_energy(6)
    f.close()
    np.testing.assert_allclose(rf, rb, rtol=1e-6)


def test_loop_exports_the_systems_it_solves(orc):
    # fvc_simple_system: the u1, u2 and p' systems of the last outer
    # iteration against those the restated iteration assembled; iteration 1
    # starts from the same state, so they agree to the assembly's rounding
    case = cavity(orc, 12)
    ref = SimpleRef(orc, case, tol_pcg=1e-13, tol_bcg=1e-13, matriz_u=1)
    loop = gpu_loop(case, tol_u=1e-13, tol_pc=1e-13, matriz_u=1)
    ref.step()
    loop.iterate(1)
    for which, key in ((1, "u1"), (2, "u2"), (3, "pc")):
        ad, au, b = loop.system(which)
        rad, rau, rb = ref.systems[key]
        np.testing.assert_allclose(ad, rad, rtol=1e-13, atol=0)
        np.testing.assert_allclose(au, rau[:au.size], rtol=1e-13, atol=1e-300)
        np.testing.assert_allclose(b, rb, rtol=1e-13, atol=1e-13 * np.abs(rb).max())
    from fortranfvcell_gb300 import FvcError
    for bad in (4, 0, 5):                  # 4: no energy equation in this loop
        with pytest.raises(FvcError):
            loop.system(bad)
    loop.close()
