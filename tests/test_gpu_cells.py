"""The GPU cell kernels of the SIMPLE iteration against the restated
reference (oracle/fvc_oracle_simple.c), bit for bit, on random states with
every boundary code the cells handle -- each test twice: with the cell
geometry computed in every kernel, as the reference's cell routines do, and
read from the mesh's geometry cache (fvc_cells_geometry_create), which the
SIMPLE loops use."""
import numpy as np
import pytest

from _simple_ref import cavity

pytestmark = pytest.mark.gpu

CACHE_GEOMETRY = False


@pytest.fixture(autouse=True, params=[False, True], ids=["geometry-per-kernel", "geometry-cached"])
def _geometry(request):
    global CACHE_GEOMETRY
    CACHE_GEOMETRY = request.param
    yield
    CACHE_GEOMETRY = False


def dev(a, dtype=None):
    import torch
    a = np.ascontiguousarray(a if dtype is None else a.astype(dtype))
    return torch.from_numpy(a).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def random_case(orc, kind, nx, seed):
    case = cavity(orc, nx, kind=kind, jitter=0.2 if kind != "quad" else 0.0)
    rng = np.random.default_rng(seed)
    n, nsh = case["numel"], case["nshared"]
    bnd = case["nelcon"] < 0
    codes = rng.integers(0, 5, size=bnd.shape).astype(np.int32)
    case["pedge"][:, :nsh] = np.where(bnd, codes, 0)
    case["sedge"][:, :nsh, :] = rng.uniform(-1, 1, (n, nsh, 3)) * bnd[..., None]
    case["pedge"][:, nsh] = 0
    case["pedge"][0, nsh] = -1          # p' pin
    case["pedge"][n // 2, nsh] = -2     # fixed velocity
    case["e"][0, 6] = 1 + seed % 7      # every TVD limiter across the cases
    return case, rng


def fields(rng, n):
    return dict(w=rng.uniform(-1, 1, (n, 2)), p=rng.uniform(-1, 1, n),
                u1=rng.uniform(-1, 1, n), u2=rng.uniform(-1, 1, n),
                g1=rng.uniform(-2, 2, (n, 2)), g2=rng.uniform(-2, 2, (n, 2)),
                gp=rng.uniform(-2, 2, (n, 2)), d=rng.uniform(0.2, 2.0, (n, 2)))


def mesh_on_gpu(case):
    from fortranfvcell_gb300 import cells
    m = cells.CellMesh(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                       case["sedge"], case["e"])
    if CACHE_GEOMETRY:
        m.cache_geometry()
    return m


@pytest.mark.parametrize("kind,nx,seed", [("quad", 9, 1), ("tri", 7, 2), ("mixed", 8, 3)])
def test_gradient_bit_exact(orc, kind, nx, seed):
    from fortranfvcell_gb300 import cells
    case, rng = random_case(orc, kind, nx, seed)
    f = fields(rng, case["numel"])
    m = mesh_on_gpu(case)
    for gkind, comp, u in ((1, 1, f["u1"]), (1, 2, f["u2"]), (2, 3, f["p"]), (2, 2, f["p"])):
        g_ref = f["gp"].copy()
        orc.gform(case, gkind, comp, u, g_ref)
        g = dev(f["gp"])
        cells.gradient(m, gkind, comp, dev(u), g)
        assert np.array_equal(host(g), g_ref), (gkind, comp)


@pytest.mark.parametrize("kind,nx,seed,matriz", [("quad", 9, 4, 4), ("quad", 9, 5, 1),
                                                 ("tri", 7, 6, 1), ("mixed", 8, 7, 1)])
def test_momentum_bit_exact(orc, kind, nx, seed, matriz):
    from fortranfvcell_gb300 import cells
    case, rng = random_case(orc, kind, nx, seed)
    n = case["numel"]
    f = fields(rng, n)
    ia, ja, _ = orc.datastruc(case["ident"], matriz, True)
    m = mesh_on_gpu(case)
    for comp in (1, 2):
        u = f["u1"] if comp == 1 else f["u2"]
        g_own, g_oth = (f["g1"], f["g2"]) if comp == 1 else (f["g2"], f["g1"])
        for simple_c in (False, True):
            ad, au = np.zeros(n), np.zeros(ja.size)
            b, im, d, rc = np.zeros(n), np.zeros((n, 4)), f["d"].copy(), np.zeros(n)
            orc.pform_momentum(case, comp, 1, u, f["p"], f["w"], g_own, g_oth, f["gp"], 0.37,
                               ia, ja, matriz, b, im, d, rc, ad=ad, au=au, under_u=0.7,
                               simple_c=simple_c)
            t = {k: dev(v) for k, v in dict(ad=np.zeros(n), au=np.zeros(ja.size), b=np.zeros(n),
                                              im=np.zeros((n, 4)), d=f["d"].copy(),
                                              rc=np.zeros(n)).items()}
            cells.momentum(m, comp, 1, dev(u), dev(f["p"]), dev(f["w"]), dev(g_own), dev(g_oth),
                           dev(f["gp"]), 0.37, dev(ia, np.int32), dev(ja.ravel(), np.int32),
                           matriz, t["ad"], t["au"], t["b"], t["im"], t["d"], t["rc"],
                           under_u=0.7, simple_c=simple_c)
            for k, ref in (("ad", ad), ("au", au), ("b", b), ("im", im), ("d", d), ("rc", rc)):
                assert np.array_equal(host(t[k]), ref), (comp, simple_c, k)
        # the time term (iws 3), first and second order
        for bs in (False, True):
            b = np.zeros(n)
            orc.pform_momentum(case, comp, 3, u, f["u2"], f["w"], g_own, g_oth, f["gp"], 0.37,
                               ia, ja, matriz, b, np.zeros((n, 4)), np.zeros((n, 2)),
                               np.zeros(n), bs=bs)
            tb = dev(np.zeros(n))
            cells.momentum(m, comp, 3, dev(u), dev(f["u2"]), None, None, None, None, 0.37,
                           dev(ia, np.int32), dev(ja.ravel(), np.int32), matriz, None, None, tb,
                           None, None, None, bs=bs)
            assert np.array_equal(host(tb), b), (comp, bs)


@pytest.mark.parametrize("kind,nx,seed,matriz", [("quad", 9, 14, 4), ("tri", 7, 15, 1),
                                                 ("mixed", 8, 16, 1), ("mixed", 8, 17, 4)])
def test_momentum_ideal_gas_bit_exact(orc, kind, nx, seed, matriz):
    from fortranfvcell_gb300 import cells
    case, rng = random_case(orc, kind, nx, seed)
    n = case["numel"]
    f = fields(rng, n)
    ro = rng.uniform(0.8, 1.4, (n, 3))
    div = rng.uniform(-0.5, 0.5, n)
    grav = np.array([0.3, -9.81])
    ia, ja, _ = orc.datastruc(case["ident"], matriz, True)
    m = mesh_on_gpu(case)
    ia_d, ja_d = dev(ia, np.int32), dev(ja.ravel(), np.int32)
    for comp in (1, 2):
        u = f["u1"] if comp == 1 else f["u2"]
        g_own, g_oth = (f["g1"], f["g2"]) if comp == 1 else (f["g2"], f["g1"])
        for simple_c, bs in ((False, False), (True, True)):
            ad, au = np.zeros(n), np.zeros(ja.size)
            b, im, d, rc = np.zeros(n), np.zeros((n, 4)), f["d"].copy(), np.zeros(n)
            orc.pform_momentum_idg(case, comp, 1, u, f["p"], f["w"], g_own, g_oth, f["gp"], ro,
                                   div, grav, 0.37, ia, ja, matriz, b, im, d, rc, ad=ad, au=au,
                                   under_u=0.7, simple_c=simple_c, bs=bs)
            t = {k: dev(v) for k, v in dict(ad=np.zeros(n), au=np.zeros(ja.size), b=np.zeros(n),
                                              im=np.zeros((n, 4)), d=f["d"].copy(),
                                              rc=np.zeros(n)).items()}
            cells.momentum_ideal_gas(m, comp, 1, dev(u), dev(f["p"]), dev(f["w"]), dev(g_own),
                                     dev(g_oth), dev(f["gp"]), dev(ro), dev(div), grav, 0.37,
                                     ia_d, ja_d, matriz, t["ad"], t["au"], t["b"], t["im"],
                                     t["d"], t["rc"], under_u=0.7, simple_c=simple_c, bs=bs)
            for k, ref in (("ad", ad), ("au", au), ("b", b), ("im", im), ("d", d), ("rc", rc)):
                assert np.array_equal(host(t[k]), ref), (comp, simple_c, k)
        for bs in (False, True):    # time term from the densities of levels n-1, n
            b = np.zeros(n)
            orc.pform_momentum_idg(case, comp, 3, u, f["u2"], f["w"], g_own, g_oth, f["gp"], ro,
                                   div, grav, 0.37, ia, ja, matriz, b, np.zeros((n, 4)),
                                   np.zeros((n, 2)), np.zeros(n), bs=bs)
            tb = dev(np.zeros(n))
            cells.momentum_ideal_gas(m, comp, 3, dev(u), dev(f["u2"]), None, None, None, None,
                                     dev(ro), None, grav, 0.37, ia_d, ja_d, matriz, None, None,
                                     tb, None, None, None, bs=bs)
            assert np.array_equal(host(tb), b), (comp, bs)


@pytest.mark.parametrize("kind,nx,seed,matriz", [("quad", 9, 8, 1), ("quad", 9, 9, 4),
                                                 ("tri", 7, 10, 1), ("mixed", 8, 11, 1)])
def test_pressure_correction_bit_exact(orc, kind, nx, seed, matriz):
    from fortranfvcell_gb300 import cells
    case, rng = random_case(orc, kind, nx, seed)
    n = case["numel"]
    f = fields(rng, n)
    ia, ja, _ = orc.datastruc(case["ident"], matriz, True)
    m = mesh_on_gpu(case)
    for int_vel in (1, 2, 5):
        ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
        orc.pform_pc(case, f["w"], f["d"], f["p"], f["gp"], ia, ja, matriz, ad, au, b, rc,
                     int_vel=int_vel)
        t = [dev(np.zeros(n)), dev(np.zeros(ja.size)), dev(np.zeros(n)), dev(np.zeros(n))]
        cells.pressure_correction(m, dev(f["w"]), dev(f["d"]), dev(f["p"]), dev(f["gp"]),
                                  dev(ia, np.int32), dev(ja.ravel(), np.int32), matriz, *t,
                                  int_vel=int_vel)
        for k, (got, ref) in enumerate(zip(t, (ad, au, b, rc))):
            assert np.array_equal(host(got), ref), (int_vel, k)


def test_update_sweeps_bit_exact(orc):
    from fortranfvcell_gb300 import cells
    rng = np.random.default_rng(12)
    n = 1000
    f = fields(rng, n)
    pc = rng.uniform(-1, 1, n)
    w, p = f["w"].copy(), f["p"].copy()
    orc.simple_update(w, p, f["u1"], f["u2"], pc, f["gp"], f["d"], 0.3)
    tw, tp = dev(f["w"]), dev(f["p"])
    cells.simple_update(tw, tp, dev(f["u1"]), dev(f["u2"]), dev(pc), dev(f["gp"]), dev(f["d"]),
                        0.3)
    assert np.array_equal(host(tw), w) and np.array_equal(host(tp), p)
    div = dev(np.zeros(n))
    cells.divergence(div, dev(f["g1"]), dev(f["g2"]))
    assert np.array_equal(host(div), orc.divergente(f["g1"], f["g2"]))
    num = (rng.permutation(n) + 1).astype(np.int32)
    x = dev(np.zeros(n))
    cells.getres(dev(num), dev(f["u1"]), x, True)
    xe = np.zeros(n)
    xe[num - 1] = f["u1"]
    assert np.array_equal(host(x), xe)
    u = dev(np.zeros(n))
    cells.getres(dev(num), u, x, False)
    assert np.array_equal(host(u), f["u1"])


@pytest.mark.parametrize("kind,nx,seed,matriz,int_vel", [("quad", 9, 21, 1, 5), ("tri", 7, 22, 4, 2),
                                                         ("mixed", 8, 23, 1, 5),
                                                         ("mixed", 8, 24, 1, 1)])
def test_pressure_correction_ideal_gas_bit_exact(orc, kind, nx, seed, matriz, int_vel):
    from fortranfvcell_gb300 import cells
    case, rng = random_case(orc, kind, nx, seed)
    n = case["numel"]
    f = fields(rng, n)
    ro = rng.uniform(0.9, 1.3, (n, 3))
    ia, ja, _ = orc.datastruc(case["ident"], matriz, True)
    m = mesh_on_gpu(case)
    for bs in (False, True):
        ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
        orc.pform_pc_idg(case, f["w"], f["d"], f["p"], f["gp"], ro, 0.05, ia, ja, matriz, ad, au,
                         b, rc, int_vel=int_vel, bs=bs)
        t = {k: dev(np.zeros(s)) for k, s in (("ad", n), ("au", ja.size), ("b", n), ("rc", n))}
        cells.pressure_correction_ideal_gas(m, dev(f["w"]), dev(f["d"]), dev(f["p"]), dev(f["gp"]),
                                            dev(ro), 0.05, dev(ia, np.int32),
                                            dev(ja.ravel(), np.int32), matriz, t["ad"], t["au"],
                                            t["b"], t["rc"], int_vel=int_vel, bs=bs)
        for k, ref in (("ad", ad), ("au", au), ("b", b), ("rc", rc)):
            assert np.array_equal(host(t[k]), ref), (bs, k)
    for comp in (2, 3):                 # ideal-gas pressure gradient rules (p', p)
        g_ref = f["gp"].copy()
        orc.gform(case, 3, comp, f["p"], g_ref)
        g = dev(f["gp"])
        cells.gradient(m, 3, comp, dev(f["p"]), g)
        assert np.array_equal(host(g), g_ref), comp


def test_ideal_gas_sweeps_bit_exact(orc):
    from fortranfvcell_gb300 import cells
    rng = np.random.default_rng(31)
    n = 1000
    temp = rng.uniform(-20, 80, n)
    ro_ref = rng.uniform(1.0, 1.3, (n, 3))
    ro = dev(ro_ref)
    for row, under in ((3, 1.0), (2, 0.7)):
        orc.ideal_gas(ro_ref, temp, row, pressure_ratio=1.1, under_ro=under)
        cells.ideal_gas_density(ro, dev(temp), row, pressure_ratio=1.1, under_ro=under)
        assert np.array_equal(host(ro), ro_ref), row
    e = np.zeros((1, 10))
    e[0, 3], e[0, 4] = 1012.0, 20.0
    h_ref, t_ref = rng.uniform(-5e3, 5e4, n), np.zeros(n)
    h, t = dev(h_ref), dev(t_ref)
    orc.enthalpy_temp(h_ref, t_ref, e, True)
    cells.enthalpy_temperature(h, t, 1012.0, 20.0, True)
    assert np.array_equal(host(t), t_ref)
    orc.enthalpy_temp(h_ref, t_ref, e, False)
    cells.enthalpy_temperature(h, t, 1012.0, 20.0, False)
    assert np.array_equal(host(h), h_ref)
