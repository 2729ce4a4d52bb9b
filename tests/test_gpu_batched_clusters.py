"""Batched solves with one thread-block cluster per system
(fvc_opts.cluster_size): each system's blocks reduce through the cluster
barrier and distributed shared memory instead of global-memory waits, in
an ordinary launch whose clusters start as SMs free up.  The same
per-system bars as the grouped form, against the restated reference
solvers (src/Iterativos.f:29-106, 140-234) on each system alone."""
import numpy as np
import pytest

from _systems import unsymmetric
from test_gpu_batched import ITS_TOL, REL_TOL, batch

pytestmark = pytest.mark.gpu


def _solve(systems, tol, maxit, opts, codes=None, tols=None):
    import torch
    from fortranfvcell_gb300 import Context, pack_block_diagonal
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    b = np.zeros(pk["neq"])
    for s, r in zip(systems, pk["rows"]):
        b[r] = s["b"]
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
    rc, st = ctx.solve_batched(pk["row_start"], bd, xd, tol, maxit, opts, raise_on_error=False,
                               codes=codes, tols=tols)
    x = xd.cpu().numpy()
    ctx.close()
    return rc, st, [x[r] for r in pk["rows"]]


def _mixed_codes(systems):
    codes, tols = [], []
    for k, s in enumerate(systems):
        if k % 2:
            u = unsymmetric(s, seed=k)
            s.update(ad=u["ad"], au=u["au"])
            codes.append(2)
            tols.append(1e-11)
        else:
            codes.append(1)
            tols.append(1e-10)
    return codes, tols


@pytest.mark.parametrize("csize", [2, 8, 16, -1])
def test_fp64_clusters_match_reference_per_system(orc, csize):
    # PCG beside BiCGSTAB, systems of 1 to ~2000 rows (some with fewer
    # slices than the cluster has blocks)
    from fortranfvcell_gb300 import make_opts
    systems = batch(orc)
    codes, tols = _mixed_codes(systems)
    rc, st, xs = _solve(systems, 0.0, 20000, make_opts("fp64", init=1, cluster_size=csize),
                        codes, tols)
    assert rc == 0
    for s, t, x, code, tol in zip(systems, st, xs, codes, tols):
        x_ref = np.zeros(s["n"])
        status, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref,
                                s["b"].copy(), s["ia"], s["ja"], s["n"], s["nad"], True, tol,
                                20000, code, 1)
        assert status == 0 and t.status == 0
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err <= (REL_TOL if code == 1 else 1e-9), (code, s["n"], err)
        bar = ITS_TOL if code == 1 else max(2, int(0.15 * so.iterations))
        assert abs(t.iterations - so.iterations) <= bar, (code, s["n"], t.iterations,
                                                          so.iterations)
        assert abs(t.energy - so.energy) <= 1e-9 * abs(so.energy)


@pytest.mark.parametrize("csize", [0, 4, 16])
def test_mixed_clusters_reach_tolerance(orc, csize):
    # mixed precision (0: the automatic choice, one cluster per system sized
    # to it, one launch per size on forked streams): every system
    # to ||b - Ax|| <= 1e-8 ||b|| recomputed in FP64, within 1e-4 of the
    # FP64 solution
    from fortranfvcell_gb300 import make_opts
    systems = batch(orc)[1:]
    codes, _ = _mixed_codes(systems)
    rc, st, xm = _solve(systems, 1e-8, 50000,
                        make_opts("mixed", init=1, stop_rule=1, cluster_size=csize), codes)
    assert rc == 0
    for t in st:
        assert t.status == 0 and t.rel_residual <= 1e-8 and t.iterations > 0
    rc, _, x64 = _solve(systems, 1e-12, 50000, make_opts("fp64", init=1, stop_rule=1), codes)
    assert rc == 0
    for s, a, b in zip(systems, xm, x64):
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), s["n"]


def test_clusters_and_groups_agree_and_repeat(orc):
    # groups (cluster_size 1) and clusters (8, and sized per system: these
    # systems fall into several sizes, so several launches on forked
    # streams) partition a system's rows differently, so only the dot
    # products' summation order differs: the same solutions to rounding;
    # two runs of one form are bit-identical
    from fortranfvcell_gb300 import make_opts
    systems = batch(orc)
    codes, tols = _mixed_codes(systems)
    runs = [_solve(systems, 0.0, 20000, make_opts("fp64", init=1, cluster_size=c), codes, tols)
            for c in (1, 8, 8, -1, -1)]
    for _, _, xc in (runs[1], runs[3]):
        for a, b in zip(runs[0][2], xc):
            assert np.linalg.norm(a - b) <= 1e-9 * max(np.linalg.norm(a), 1e-300)
    for i, j in ((1, 2), (3, 4)):
        for a, b in zip(runs[i][2], runs[j][2]):
            np.testing.assert_array_equal(a, b)


def test_cluster_size_outside_the_range_is_refused(orc):
    from fortranfvcell_gb300 import _lib, make_opts
    systems = batch(orc)[:3]
    for bad in (-2, 17):
        rc, _, _ = _solve(systems, 1e-8, 100, make_opts("fp64", init=1, cluster_size=bad))
        assert rc == _lib.FVC_ERR_ARG
