"""Pins the CPU restatement (oracle/) to the reference's own known answers
and to hand-derived cases (tests/golden/golden.json)."""
import json
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def test_dot_known_answer(orc):
    # src/BenchMark.f:40-52: |dot(i,2i) - sumSquares(n)| <= 1e-15
    for n, expect in GOLDEN["dot_kat"].items():
        n = int(n)
        x = np.arange(1, n + 1, dtype=np.float64)
        assert abs(orc.dot(x, 2.0 * x) - float(expect)) <= 1e-15 * max(1.0, float(expect))


def test_smachn(orc):
    # Iterativos.f:450-462 halves until 1+s == 1: the unit roundoff 2^-53
    assert orc.smachn() == 2.0 ** -53


@pytest.mark.parametrize("case", ["quad2x2", "strip4"])
def test_adjacency_and_rcm_hand_derived(orc, case):
    g = GOLDEN[case]
    ix = np.array(g["ix"], dtype=np.int32)
    ixm = np.concatenate([ix, np.ones((ix.shape[0], 1), np.int32)], axis=1)
    nelcon = orc.adjacency(ixm, g["nnode"], 4)
    assert nelcon.tolist() == g["nelcon"]
    assert orc.reord(nelcon).tolist() == g["num"]


def test_rcm_identity_when_disabled(orc):
    g = GOLDEN["quad2x2"]
    nelcon = np.array(g["nelcon"], dtype=np.int32)
    assert orc.reord(nelcon, freord=False).tolist() == [1, 2, 3, 4]


def _spd2():
    g = GOLDEN["spd2"]
    return (np.array(g["ad"]), np.array(g["au"]), np.array(g["ia"], np.int32),
            np.array(g["ja"], np.int32), np.array(g["b"]), np.array(g["x"]))


@pytest.mark.parametrize("code", [1, 2, 3])
def test_krylov_2x2_known_solution(orc, code):
    ad, au, ia, ja, b, xs = _spd2()
    x = np.zeros(2)
    st, s = orc.solver(ad.copy(), au.copy(), au.copy(), x, b.copy(), ia, ja, 2, 2, True,
                       1e-12, 50, code, 1)
    assert st == 0
    np.testing.assert_allclose(x, xs, rtol=1e-13)
    if code == 1:
        assert s.iterations == 2


def test_initmatvec_spmv_against_dense(orc):
    # src/BenchMark.f:456-476 initMatVec: ad = 1, off = -0.1, x alternating
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(7, kind="quad")
    ixm = np.concatenate([m.ix, np.ones((m.numel, 1), np.int32)], axis=1)
    nelcon = orc.adjacency(ixm, m.nnode, 4)
    num = orc.reord(nelcon)
    ident = orc.numeq(num, nelcon)
    n = m.numel
    i = np.arange(1, n + 1)
    x = np.where(i % 2 == 0, i / 1000.0, -2.0 * i / 1000.0)
    for matriz, unsym, kind in [(1, True, "csrd"), (1, False, "csrd_sym"), (3, False, "csrc_sym"),
                                (4, True, "ellpack")]:
        ia, ja, nad = orc.datastruc(ident, matriz, unsym)
        ad = np.ones(n)
        off = np.full(ja.size, -0.1)
        dense = np.diag(ad)
        if matriz == 4:
            for r in range(n):
                for j in range(4):
                    if ident[r, j] != -1:
                        dense[r, ident[r, j] - 1] += -0.1
            off = np.where(ident.ravel() != -1, -0.1, 0.0)
        else:
            for r in range(n):
                for k in range(ia[r] - 1, ia[r + 1] - 1):
                    dense[r, ja[k] - 1] += -0.1
                    if not unsym or matriz == 3:
                        dense[ja[k] - 1, r] += -0.1
        y = orc.matvec(kind, ad, off, off, x, ia, ja.ravel(), n)
        np.testing.assert_allclose(y, dense @ x, rtol=1e-14, atol=1e-16)


def test_pcg_sequential_vs_openmp(orc):
    # pcg vs pcg_omp (Iterativos.f vs Iterativos_omp.f) on a p' matrix:
    # same algorithm, different dot summation order
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(24, kind="quad", jitter=0.2, seed=3)
    ixm = np.concatenate([m.ix, np.ones((m.numel, 1), np.int32)], axis=1)
    nelcon = orc.adjacency(ixm, m.nnode, 4)
    num = orc.reord(nelcon)
    ident = orc.numeq(num, nelcon)
    ia, ja, nad = orc.datastruc(ident, 1, True)
    ad = np.zeros(m.numel)
    au = np.zeros(nad)
    orc.lib().oref_pform_pressure(*[orc._p(v) if isinstance(v, np.ndarray) else v for v in (
        np.ascontiguousarray(m.coor), m.nnode, m.ix, 4, m.numel, 4, nelcon, num,
        np.ones(m.numel), np.ones((m.numel, 2)), 1, 5, 1, 1, ia, ja, ad, au)])
    rng = np.random.default_rng(0)
    b = rng.uniform(-1, 1, m.numel)
    x1 = np.zeros(m.numel)
    x2 = np.zeros(m.numel)
    s1, st1 = orc.solver(ad, au, au, x1, b.copy(), ia, ja, m.numel, nad, True, 1e-10, 5000, 1, 1)
    s2, st2 = orc.solver(ad, au, au, x2, b.copy(), ia, ja, m.numel, nad, True, 1e-10, 5000, 1, 1,
                         omp_threads=4)
    assert s1 == 0 and s2 == 0
    assert abs(st1.iterations - st2.iterations) <= 2
    assert np.linalg.norm(x1 - x2) / np.linalg.norm(x1) < 1e-8
