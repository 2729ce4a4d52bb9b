"""Mixed-precision CG: the kernel that streams its arrays through shared
memory with bulk asynchronous copies (staging 2 here; the default from
524288 rows) against the plain-load kernel of the same arithmetic.  Both
must give the same iterates bit for bit: the staging changes where the
operands come from, not the sums."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def laplace_csrd(nx, ny, shift=1e-3):
    """5-point Laplacian + shift*I on an nx-by-ny grid in row-major order
    (couplings at +-1 and +-nx), as CSRD arrays: ad, then the off-diagonals
    of each row in column order (ia, ja 1-based)."""
    n = nx * ny
    ia = np.zeros(n + 1, np.int32)
    ja, au, ad = [], [], np.zeros(n)
    for r in range(n):
        i, j = r % nx, r // nx
        nb = [r - nx] if j > 0 else []
        nb += [r - 1] if i > 0 else []
        nb += [r + 1] if i < nx - 1 else []
        nb += [r + nx] if j < ny - 1 else []
        ja += [c + 1 for c in nb]
        au += [-1.0] * len(nb)
        ad[r] = len(nb) + shift
        ia[r + 1] = ia[r] + len(nb)
    ia += 1
    return dict(n=n, ia=ia, ja=np.array(ja, np.int32), au=np.array(au), ad=ad, nad=len(au))


def _solve_both(s, b, tol=1e-8):
    from fortranfvcell_gb300 import Context, make_opts
    n = s["n"]
    ctx = Context()
    ctx.set_matrix(1, True, n, s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    out = []
    for staging in (1, 2):
        bd, xd = torch_dev(b), torch_dev(np.zeros(n))
        st = ctx.solve(1, bd, xd, tol, 200000, make_opts("mixed", init=1, staging=staging))
        out.append((st, xd.cpu().numpy()))
    return out


def _relres(s, x, b):
    import scipy.sparse as sp
    n, ia, ja = s["n"], s["ia"], s["ja"]
    r = np.repeat(np.arange(n), np.diff(ia))
    A = sp.csr_matrix((s["au"], (r, ja - 1)), shape=(n, n)) + sp.diags(s["ad"])
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)


def test_staged_matches_plain_on_mesh():
    # 240k cells: every one of the 152 blocks walks several 1024-row chunks
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(400, kind="mixed", jitter=0.2, seed=1234)
    ps = mesh.pressure_system(m, 1, True, pin_cell=1)
    s = dict(n=ps.neq, ia=ps.ia, ja=ps.ja, au=ps.au, ad=ps.ad, nad=ps.nad)
    b = np.random.default_rng(42).uniform(-1, 1, s["n"])
    (st1, x1), (st0, x0) = _solve_both(s, b)
    assert st1.status == 0 and st0.status == 0
    assert st1.iterations == st0.iterations and st1.refinements == st0.refinements
    assert np.array_equal(x1, x0)
    assert _relres(s, x1, b) <= 1e-8


def test_staged_matches_plain_triangles():
    # triangle-only mesh: every slice has width 3 (the uniform-width-3 kernel)
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(300, kind="tri", jitter=0.2, seed=5)
    ps = mesh.pressure_system(m, 1, True, pin_cell=1)
    s = dict(n=ps.neq, ia=ps.ia, ja=ps.ja, au=ps.au, ad=ps.ad, nad=ps.nad)
    b = np.random.default_rng(8).uniform(-1, 1, s["n"])
    (st1, x1), (st0, x0) = _solve_both(s, b)
    assert st1.status == 0 and st0.status == 0
    assert st1.iterations == st0.iterations
    assert np.array_equal(x1, x0)
    assert _relres(s, x1, b) <= 1e-8


def test_staged_matches_plain_beyond_window():
    # couplings 4000 rows apart: beyond the staged kernel's shared-memory
    # window (+-3072 rows), so those neighbours come from global memory;
    # slices of width 3 and 4 mixed (the general staged kernel)
    s = laplace_csrd(4000, 12)
    b = np.random.default_rng(3).uniform(-1, 1, s["n"])
    (st1, x1), (st0, x0) = _solve_both(s, b)
    assert st1.status == 0 and st0.status == 0
    assert st1.iterations == st0.iterations
    assert np.array_equal(x1, x0)
    assert _relres(s, x1, b) <= 1e-8


def test_staged_matches_plain_with_long_blocks():
    # 1.21M cells: every block walks about eight 1024-row chunks, so the
    # copy window wraps within one phase and the prefetched stages of the
    # next phase are drained and issued again after each reliable update
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(1100, kind="quad", jitter=0.1, seed=7)
    ps = mesh.pressure_system(m, 1, True, pin_cell=1)
    s = dict(n=ps.neq, ia=ps.ia, ja=ps.ja, au=ps.au, ad=ps.ad, nad=ps.nad)
    assert s["n"] >= 152 * 7 * 1024
    b = np.random.default_rng(11).uniform(-1, 1, s["n"])
    (st1, x1), (st0, x0) = _solve_both(s, b)
    assert st1.status == 0 and st0.status == 0 and st0.refinements >= 2
    assert st1.iterations == st0.iterations
    assert np.array_equal(x1, x0)


@pytest.mark.parametrize("kind,nx", [("quad", 300), ("tri", 210)])
def test_mixed_on_ellpack_input_with_padding(kind, nx):
    # the reference's ELLPACK (matriz 4) pads boundary rows with column 1 and
    # value 0 (src/EllPack.f:19-42): the FP32 operator points those slots at
    # their own row, so the padded matrix keeps 16-bit offsets and the
    # uniform-width staged kernel; staged and plain loads give the same bits
    # and the solve reaches ||b - Ax|| <= 1e-8 ||b|| (FP64 recomputed)
    import scipy.sparse as sp
    from fortranfvcell_gb300 import Context, make_opts, mesh
    s = mesh.pressure_system(mesh.square_mesh(nx, kind=kind, jitter=0.2, seed=3), matriz=4,
                             unsym=True, pin_cell=1)
    n, w = s.neq, int(s.ia[0])
    jj = s.ja.reshape(n, w) - 1
    pads = int(np.sum((jj == 0) & (s.au.reshape(n, w) == 0.0)))
    assert pads > 0
    b = np.random.default_rng(5).uniform(-1, 1, n)
    ctx = Context()
    ctx.set_matrix(4, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    out = []
    for staging in (1, 2):
        bd, xd = torch_dev(b), torch_dev(np.zeros(n))
        st = ctx.solve(1, bd, xd, 1e-8, 200000, make_opts("mixed", init=1, staging=staging))
        out.append((st, xd.cpu().numpy()))
    (s1, x1), (s2, x2) = out
    assert s1.inner_iterations == s2.inner_iterations
    assert np.array_equal(x1, x2)
    rows = np.repeat(np.arange(n), w)
    A = sp.csr_matrix((s.au, (rows, jj.ravel())), shape=(n, n)) + sp.diags(s.ad)
    rel = np.linalg.norm(b - A @ x2) / np.linalg.norm(b)
    print(f"{kind} ELLPACK {n} rows, {pads} pad slots: its {s2.inner_iterations} rel {rel:.2e}")
    assert rel <= 1e-8


@pytest.mark.parametrize("staging", [1, 2])
def test_fp32_slice_widths_give_the_same_bits(staging):
    # fvc_opts.fp32_layout: every slice padded to the widest row (width 4 on
    # the mixed mesh) or each slice its own width (SELL-32).  The true terms
    # are summed in the same order and the padding slots add exactly 0, so
    # the two layouts give the same iterates; switching lays the operator out
    # anew on the same context
    from fortranfvcell_gb300 import Context, make_opts, mesh
    s = mesh.pressure_system(mesh.square_mesh(300, kind="mixed", jitter=0.2, seed=8), matriz=1,
                             unsym=True, pin_cell=1)
    n = s.neq
    b = np.random.default_rng(2).uniform(-1, 1, n)
    ctx = Context()
    ctx.set_matrix(1, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    out = []
    for layout in (0, 1, 0):
        bd, xd = torch_dev(b), torch_dev(np.zeros(n))
        st = ctx.solve(1, bd, xd, 1e-8, 200000,
                       make_opts("mixed", init=1, staging=staging, fp32_layout=layout))
        out.append((st.inner_iterations, xd.cpu().numpy()))
    assert out[0][0] == out[1][0] == out[2][0]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][1], out[2][1])
