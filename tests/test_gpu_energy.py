"""The GPU energy / transport cells (fvc_cells_energy, fvc_cells_energy_
gradient) against the restated reference cells of src/CellibTrans.f
(oracle/fvc_oracle_simple.c), bit for bit: both cell libraries, CSRD and
ELLPACK, quadrilateral, triangle and mixed meshes, two materials, every
boundary code, volume sources and random states; each test with the cell
geometry computed in the kernels and read from the mesh's geometry cache."""
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


def energy_case(orc, kind, nx, seed):
    case = cavity(orc, nx, kind=kind, jitter=0.2 if kind != "quad" else 0.0)
    rng = np.random.default_rng(seed)
    n, nsh = case["numel"], case["nshared"]
    # two materials: rho, conductivity, specific heat, reference temperature,
    # time coefficient, limiter (every limiter code across the seeds)
    e = np.zeros((2, 10))
    e[0, 1:7] = [1.204, 0.0242, 1012.0, 20.0, 1.0, 1 + seed % 7]
    e[1, 1:7] = [2.7, 0.05, 880.0, 20.0, 1.0, 1 + (seed + 3) % 7]
    case["e"] = e
    case["ix"][:, -1] = rng.integers(1, 3, n).astype(np.int32)
    bnd = case["nelcon"] < 0
    pe = np.zeros((n, nsh + 1), np.int32)
    pe[:, :nsh] = np.where(bnd, rng.integers(0, 5, bnd.shape), 0)
    pe[:, nsh] = rng.integers(0, 2, n)               # volume source on about half
    se = rng.uniform(15.0, 30.0, (n, nsh + 1))       # temperatures: fractional enthalpies
    case["pe"], case["se"] = pe, se
    return case, rng


def mesh_on_gpu(case):
    from fortranfvcell_gb300 import cells
    m = cells.CellMesh(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                       case["sedge"], case["e"])
    if CACHE_GEOMETRY:
        m.cache_geometry()
    return m


def state(rng, n, lib):
    scale = 1000.0 if lib == 3 else 1.0
    w = rng.uniform(-1, 1, (n, 2))
    w[::7] = 0.0                                      # zero face velocities too
    return dict(u=scale * rng.uniform(-1, 1, n), u0=scale * rng.uniform(-1, 1, n),
                ro=rng.uniform(0.8, 1.4, (n, 3)), w=w,
                g=scale * rng.uniform(-2, 2, (n, 2)))


@pytest.mark.parametrize("kind,nx,seed,matriz", [("quad", 9, 1, 1), ("quad", 9, 2, 4),
                                                 ("tri", 7, 3, 1), ("mixed", 8, 4, 1),
                                                 ("mixed", 8, 5, 4)])
def test_energy_system_bit_exact(orc, kind, nx, seed, matriz):
    from fortranfvcell_gb300 import cells
    case, rng = energy_case(orc, kind, nx, seed)
    n = case["numel"]
    ia, ja, _ = orc.datastruc(case["ident"], matriz, True)
    m = mesh_on_gpu(case)
    pe_d, se_d = dev(case["pe"]), dev(case["se"])
    ia_d, ja_d = dev(ia, np.int32), dev(ja.ravel(), np.int32)
    for lib in (3, 4):
        f = state(rng, n, lib)
        for bs in (False, True):
            ad, au, b, rc = np.zeros(n), np.zeros(ja.size), np.zeros(n), np.zeros(n)
            orc.pform_energy(case, lib, 1, case["pe"], case["se"], f["u"], f["u0"], f["ro"],
                             f["w"], f["g"], 0.37, ia, ja, matriz, b, rc, ad=ad, au=au, bs=bs)
            t = {k: dev(np.zeros(s)) for k, s in (("ad", n), ("au", ja.size), ("b", n),
                                                   ("rc", n))}
            cells.energy(m, lib, 1, pe_d, se_d, dev(f["u"]), dev(f["u0"]), dev(f["ro"]),
                         dev(f["w"]), dev(f["g"]), 0.37, ia_d, ja_d, matriz, t["ad"], t["au"],
                         t["b"], t["rc"], bs=bs)
            for k, ref in (("ad", ad), ("au", au), ("b", b), ("rc", rc)):
                assert np.array_equal(host(t[k]), ref), (lib, bs, k)
            # time term + volume source (iws 4)
            b4 = np.zeros(n)
            orc.pform_energy(case, lib, 4, case["pe"], case["se"], f["u"], f["u0"], f["ro"],
                             f["w"], f["g"], 0.37, ia, ja, matriz, b4, np.zeros(n), bs=bs)
            tb = dev(np.zeros(n))
            cells.energy(m, lib, 4, pe_d, se_d, dev(f["u"]), dev(f["u0"]), dev(f["ro"]), None,
                         None, 0.37, ia_d, ja_d, matriz, None, None, tb, None, bs=bs)
            assert np.array_equal(host(tb), b4), (lib, bs, "iws 4")


@pytest.mark.parametrize("kind,nx,seed", [("quad", 9, 6), ("tri", 7, 7), ("mixed", 8, 8)])
def test_energy_gradient_bit_exact(orc, kind, nx, seed):
    from fortranfvcell_gb300 import cells
    case, rng = energy_case(orc, kind, nx, seed)
    n = case["numel"]
    m = mesh_on_gpu(case)
    for lib in (3, 4):
        f = state(rng, n, lib)
        g_ref = f["g"].copy()
        orc.gform_energy(case, lib, case["pe"], case["se"], f["u"], g_ref)
        g = dev(f["g"])
        cells.energy_gradient(m, lib, dev(case["pe"]), dev(case["se"]), dev(f["u"]), g)
        assert np.array_equal(host(g), g_ref), lib


def test_energy_bad_arguments(orc):
    from fortranfvcell_gb300 import FvcError, cells
    case, rng = energy_case(orc, "quad", 4, 9)
    n = case["numel"]
    m = mesh_on_gpu(case)
    f = state(rng, n, 4)
    z = dev(np.zeros(n))
    with pytest.raises(FvcError):       # lib 5 does not exist
        cells.energy(m, 5, 4, dev(case["pe"]), dev(case["se"]), dev(f["u"]), None,
                     dev(f["ro"]), None, None, 0.1, None, None, 1, None, None, z, None)
    with pytest.raises(FvcError):       # iws 4 with bs needs u0
        cells.energy(m, 4, 4, dev(case["pe"]), dev(case["se"]), dev(f["u"]), None,
                     dev(f["ro"]), None, None, 0.1, None, None, 1, None, None, z, None, bs=True)
