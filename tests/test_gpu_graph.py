"""The SIMPLE outer iteration as one CUDA graph per iteration
(fvc_simple_set_graph) and the capturable solve (fvc_solve_async) against
the uncaptured calls: the same kernels in the same order, so residual
histories, iteration counts and fields are compared for equality."""
import numpy as np
import pytest

from _simple_ref import cavity

pytestmark = pytest.mark.gpu


def gpu_loop(case, **kw):
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    return SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                      case["sedge"], case["e"], opts=simple_opts(**kw))


def pair(case, energy=False, **kw):
    loops = [gpu_loop(case, **kw), gpu_loop(case, **kw)]
    if energy:
        for lp in loops:
            lp.enable_energy(case["pedgeE"], case["sedgeE"], case["gravity"], case["t0"])
    loops[1].use_graph(True)
    return loops


def assert_same_state(a, b, energy=False):
    sa, sb = a.get_state(energy=energy), b.get_state(energy=energy)
    for k, v in sa.items():
        if v is not None:
            assert np.array_equal(v, sb[k]), k


@pytest.mark.parametrize("kind,nx,matriz_u", [("quad", 20, 4), ("tri", 12, 1),
                                              ("mixed", 14, 1)])
def test_graph_loop_equals_uncaptured(orc, kind, nx, matriz_u):
    case = cavity(orc, nx, kind=kind, jitter=0.15 if kind != "quad" else 0.0)
    a, b = pair(case, matriz_u=matriz_u)
    for nit in (25, 7):   # a second call replays the same graph
        ra, ia = a.iterate(nit)
        rb, ib = b.iterate(nit)
        assert np.array_equal(ra, rb) and np.array_equal(ia, ib)
    assert_same_state(a, b)
    if kind == "quad":    # iteration 1: v's right-hand side is zero, its solve skipped
        assert ia[0, 1] > 0
    a.close()
    b.close()


def test_graph_batches_and_skipped_solves(orc):
    # 300 iterations: a batch of 256 launches and one of 44; a cavity at rest
    # (lid 0) skips every solve through the conditional nodes
    from fortranfvcell_gb300.solver import kernel_launches
    a, b = pair(cavity(orc, 8))
    l0 = kernel_launches()
    ra, ia = a.iterate(300)
    l1 = kernel_launches()
    rb, ib = b.iterate(300)
    l2 = kernel_launches()
    assert np.array_equal(ra, rb) and np.array_equal(ia, ib)
    assert_same_state(a, b)
    assert l2 - l1 > l1 - l0 > 0     # graph launches are counted per replay
    a, b = pair(cavity(orc, 8, lid=0.0))
    ra, ia = a.iterate(5)
    rb, ib = b.iterate(5)
    assert np.array_equal(ra, rb) and np.array_equal(ia, ib)
    assert not ib.any()
    assert_same_state(a, b)


def test_graph_gas_loop_equals_uncaptured(orc):
    from fortranfvcell_gb300.cases import natural_convection_cavity
    c = natural_convection_cavity(12, ra=1e4)
    a, b = pair(c, energy=True, dt=0.5, matriz_u=1)
    for step in range(2):
        if step:
            a.time_step()
            b.time_step()
        ra, ia = a.iterate_energy(8)
        rb, ib = b.iterate_energy(8)
        assert np.array_equal(ra, rb) and np.array_equal(ia, ib)
        assert (ib[:, 3] > 0).all()
    assert_same_state(a, b, energy=True)
    ta, ha, roa = a.energy_fields()
    tb, hb, rob = b.energy_fields()
    assert np.array_equal(ta, tb) and np.array_equal(roa, rob)


def test_graph_loop_failure_like_uncaptured(orc):
    # maxit 2 at tol 1e-13: the first solve fails in iteration 1; both loops
    # return its status and leave the same fields
    from fortranfvcell_gb300 import FvcError
    a, b = pair(cavity(orc, 16), maxit=2, tol_u=1e-13, tol_pc=1e-13)
    with pytest.raises(FvcError) as ea:
        a.iterate(3)
    with pytest.raises(FvcError) as eb:
        b.iterate(3)
    assert ea.value.status == eb.value.status == 1   # FVC_ERR_NOCONV
    assert_same_state(a, b)


@pytest.mark.parametrize("energy", [False, True])
def test_graph_loop_with_mixed_solves(orc, energy):
    # mixed-precision p' (and, in the gas loop, momentum) solves inside the
    # graph: the FP32 operator is rebuilt from the uploaded values by a
    # captured kernel; the same results as the uncaptured mixed loop
    from fortranfvcell_gb300.cases import natural_convection_cavity
    if energy:
        c = natural_convection_cavity(12, ra=1e4)
        a, b = pair(c, energy=True, dt=0.5, matriz_u=1, precision="mixed", precision_u="mixed")
        ra, ia = a.iterate_energy(6)
        rb, ib = b.iterate_energy(6)
    else:
        a, b = pair(cavity(orc, 20), precision="mixed")
        ra, ia = a.iterate(20)
        rb, ib = b.iterate(20)
    assert np.array_equal(ra, rb) and np.array_equal(ia, ib)
    assert (ib[:, 2] > 0).any()
    assert_same_state(a, b, energy=energy)
    a.close()
    b.close()


@pytest.mark.parametrize("nx,code", [(40, 1), (130, 1), (40, 2), (30, 3)])
def test_solve_async_and_capture(nx, code):
    # fvc_solve_async equals fvc_solve (cluster PCG, grid PCG, BiCGSTAB,
    # GMRES); captured with new values into a torch CUDA graph and replayed
    # with other values and right-hand side, it equals a synchronous solve
    import torch
    from fortranfvcell_gb300 import mesh
    from fortranfvcell_gb300.solver import Context
    s = mesh.pressure_system(mesh.square_mesh(nx, kind="quad", jitter=0.2, seed=nx), matriz=1,
                             unsym=True, pin_cell=1)
    n, tol, maxit = s.neq, 1e-10, 20000
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    ctx = Context()
    ctx.set_matrix(1, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    b = dev(np.random.default_rng(nx).uniform(-1, 1, n))
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    st = ctx.solve(code, b, x1, tol, maxit)
    status = torch.zeros(4, dtype=torch.int32, device="cuda")
    ctx.solve_async(code, b, x2, tol, maxit, status)
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    assert status.tolist() == [0, st.iterations, st.inner_iterations, 0]
    stream = torch.cuda.Stream()
    ctx.set_stream(stream)
    ad, au = dev(s.ad), dev(s.au[:max(s.nad, 1)])
    x3 = torch.zeros_like(b)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream, capture_error_mode="relaxed"):
        x3.zero_()
        ctx.update_values_async(ad, au, au)
        ctx.solve_async(code, b, x3, tol, maxit, status)
    ad.mul_(1.5)
    au.mul_(1.5)
    b.copy_(dev(np.random.default_rng(nx + 1).uniform(-1, 1, n)))
    with torch.cuda.stream(stream):  # the context's stream: one solve at a time per context
        g.replay()
    stream.synchronize()
    assert status.tolist()[0] == 0
    ctx.update_values(ad, au, au)
    x4 = torch.zeros_like(b)
    st4 = ctx.solve(code, b, x4, tol, maxit)
    torch.cuda.synchronize()
    assert torch.equal(x3, x4)
    assert status.tolist()[:2] == [0, st4.iterations]
    ctx.close()


def test_solve_async_mixed_and_tuner_rejections():
    # fvc_solve_async with mixed precision equals fvc_solve (the FP32
    # operator rebuilt by a stream-ordered kernel after a value upload);
    # mixed GMRES is rejected by the async solve and by the tuner
    import torch
    from fortranfvcell_gb300 import FvcError, _lib, mesh
    from fortranfvcell_gb300.solver import Context, make_opts
    s = mesh.pressure_system(mesh.square_mesh(90, kind="mixed", jitter=0.2, seed=3), matriz=1,
                             unsym=True, pin_cell=1)
    n = s.neq
    ctx = Context()
    ctx.set_matrix(1, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    b = torch.from_numpy(np.random.default_rng(2).uniform(-1, 1, n)).cuda()
    o = make_opts("mixed", init=1)
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    st = ctx.solve(1, b, x1, 1e-9, 50000, o)
    status = torch.zeros(4, dtype=torch.int32, device="cuda")
    ad = torch.from_numpy(s.ad).cuda()
    au = torch.from_numpy(s.au[:max(s.nad, 1)]).cuda()
    ctx.update_values_async(ad, au, au)
    ctx.solve_async(1, b, x2, 1e-9, 50000, status, o)
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    assert status.tolist()[:2] == [0, st.iterations]
    with pytest.raises(FvcError) as e:
        ctx.solve_async(3, b, x2, 1e-9, 100, status, o)
    assert e.value.status == _lib.FVC_ERR_UNSUPPORTED
    with pytest.raises(FvcError) as e:
        ctx.autotune(3, "mixed", 5)
    assert e.value.status == _lib.FVC_ERR_UNSUPPORTED
    ctx.close()
