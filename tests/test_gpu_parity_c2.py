"""FP64 GPU solves against the restated reference at the size of the
standalone solver configuration: p' systems of about one million cells.

The systems are those of the benchmark's C2 family (unit square, nodes
jittered by +-20% of the edge, seed 1234, RCM, b ~ U[-1, 1] seed 42,
x0 = 0): the 50/50 triangle/quad mesh in CSRD (matriz 1) and the
quadrilateral mesh in ELLPACK (matriz 4), solved by Jacobi-PCG with the
reference's own stopping test (sqrt|r.z| < 1e-8 sqrt|r0.z0|,
src/Iterativos.f:57,73), and an unsymmetric system of the mixed mesh's
structure by BiCGSTAB.  Bars as for the small systems: solution within
1e-10 relative L2, iteration count within +-2 (BiCGSTAB: within 15%,
compared at its working tolerance), energy norm x.Ax within 1e-9.

For scale: on a 1.57M-cell system of this family the reference's own two
PCG paths, sequential pcg (src/Iterativos.f:29-106) and pcg_omp
(src/Iterativos_omp.f:30-127, another dot-product summation order), stop
after 8471 and 8470 iterations with solutions 1.4e-11 apart.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
ITS_TOL = 2
ENERGY_TOL = 1e-9


def _system(orc, kind, nx, matriz):
    """Product adjacency (equal to the restated Adjacency.f, tested in
    test_mesh_tools), then the restated RCM, numbering, structure and p'
    assembly: the reference's arrays for this mesh."""
    from fortranfvcell_gb300 import mesh
    from _systems import _ptr
    m = mesh.square_mesh(nx, kind=kind, jitter=0.2, seed=1234)
    nelcon = mesh.adjacency(m)
    num = orc.reord(nelcon)
    ident = orc.numeq(num, nelcon)
    ia, ja, nad = orc.datastruc(ident, matriz, True)
    n = m.numel
    ad = np.zeros(n)
    au = np.zeros(ja.size)
    L = orc.lib()
    L.oref_pform_pressure(_ptr(np.ascontiguousarray(m.coor)), m.nnode,
                          _ptr(np.ascontiguousarray(m.ix, np.int32)), m.ix.shape[1], n,
                          m.nshared, _ptr(nelcon), _ptr(num), _ptr(np.ones(n)),
                          _ptr(np.ones((n, 2))), 1, 5, matriz, 1, _ptr(ia), _ptr(ja),
                          _ptr(ad), _ptr(au))
    b = np.random.default_rng(42).uniform(-1.0, 1.0, n)
    return dict(n=n, ia=ia, ja=ja.ravel(), nad=nad, ad=ad, au=au.ravel(), b=b)


def _compare(fvc, orc, s, code, matriz, tol, omp_threads=0, its_tol=ITS_TOL):
    n = s["n"]
    x_ref = np.zeros(n)
    rc, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref, s["b"].copy(),
                        s["ia"], s["ja"], n, s["nad"], True, tol, 200000, code, matriz,
                        omp_threads=omp_threads)
    assert rc == 0, "restated reference did not converge"
    x = np.zeros(n)
    sg = fvc.solver(s["ad"], s["au"], s["au"], x, s["b"], s["ia"], s["ja"], n, s["nad"], True,
                    tol, 200000, code, matriz)
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    de = abs(sg.energy - so.energy) / abs(so.energy)
    print(f"n {n} code {code} matriz {matriz} tol {tol:g}: its ref {so.iterations} gpu "
          f"{sg.iterations}, rel err {err:.2e}, energy rel diff {de:.2e}")
    return so, sg, err, de


def test_pcg_csrd_1m_mixed_mesh(fvc, orc):
    # the sequential pcg of Iterativos.f on the same arrays (matriz 1 zeroes
    # x on both sides, Solver.f:130)
    s = _system(orc, "mixed", 836, 1)
    assert s["n"] >= 1_000_000
    so, sg, err, de = _compare(fvc, orc, s, 1, 1, 1e-8)
    assert err <= REL_TOL
    assert abs(sg.iterations - so.iterations) <= ITS_TOL
    assert de <= ENERGY_TOL


def test_pcg_ellpack_1m_quad_mesh(fvc, orc):
    # ELLPACK on 1024 x 1024 quads; the restated pcg_omp with
    # matvec_ellpack_omp (Matvec_omp.f:1036-1086), warm start from x = 0
    s = _system(orc, "quad", 1024, 4)
    so, sg, err, de = _compare(fvc, orc, s, 1, 4, 1e-8, omp_threads=os.cpu_count() or 1)
    assert err <= REL_TOL
    assert abs(sg.iterations - so.iterations) <= ITS_TOL
    assert de <= ENERGY_TOL


def test_bicgstab_csrd_1m_unsymmetric(fvc, orc):
    # an unsymmetric system on the mixed mesh's structure (off-diagonals
    # scaled by 1 + 0.4 U[-1, 1], diagonally dominant).  Solutions at
    # tol 1e-14, iteration counts at 1e-10 (the spread of BiCGSTAB's exit
    # iteration under another summation order is 15% of the count).  At
    # 1e-12 the two exits can fall one iteration apart (51 and 50 here), and
    # one iteration still moves x by ~1e-9 relative at this size; at 1e-14
    # the last iterations move it by far less than the 1e-10 bar
    s = _system(orc, "mixed", 836, 1)
    rng = np.random.default_rng(5)
    au = s["au"] * (1.0 + 0.4 * rng.uniform(-1.0, 1.0, s["au"].size))
    rows = np.repeat(np.arange(s["n"]), np.diff(s["ia"]))
    s["ad"] = np.bincount(rows, weights=np.abs(au), minlength=s["n"]) * 1.05 + 1e-3
    s["au"] = au
    so, sg, err, de = _compare(fvc, orc, s, 2, 1, 1e-14)
    assert err <= REL_TOL
    assert de <= ENERGY_TOL
    so, sg, _, _ = _compare(fvc, orc, s, 2, 1, 1e-10)
    assert abs(sg.iterations - so.iterations) <= max(ITS_TOL, int(0.15 * so.iterations))


def test_mixed_precision_1m_against_fp64_reference(fvc, orc):
    # the mixed FP32/FP64 PCG reaches ||b - Ax|| <= 1e-8 ||b|| (FP64
    # recomputed) on the 1M mixed mesh; its distance to the restated FP64
    # solution at the same rule is reported and bounded
    import scipy.sparse as sp
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    s = _system(orc, "mixed", 836, 1)
    n = s["n"]
    ctx = Context()
    ctx.set_matrix(1, True, n, s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    bd = torch.from_numpy(s["b"]).cuda()
    xd = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = ctx.solve(1, bd, xd, 1e-8, 200000, make_opts("mixed", init=1))
    x = xd.cpu().numpy()
    rows = np.repeat(np.arange(n), np.diff(s["ia"]))
    A = sp.csr_matrix((s["au"], (rows, s["ja"] - 1)), shape=(n, n)) + sp.diags(s["ad"])
    rel = np.linalg.norm(s["b"] - A @ x) / np.linalg.norm(s["b"])
    x_ref = np.zeros(n)
    rc, so = orc.pcg_omp_sample(s["ad"].copy(), s["au"].copy(), x_ref, s["b"].copy(), s["ia"],
                                s["ja"], n, s["nad"], 1e-8, 200000, 1, os.cpu_count() or 1,
                                stop_rule=1)
    assert rc == 0
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    print(f"mixed 1M: inner its {st.inner_iterations} (FP64 reference {so.iterations}), "
          f"rel res {rel:.2e}, rel err vs FP64 reference {err:.2e}")
    assert rel <= 1e-8
    assert err <= 1e-4
    assert st.inner_iterations <= 1.02 * so.iterations
