"""The allocation-free PCG entry point, fvc_pcg_csrd_noalloc.

Some callers of this library cannot allocate device memory when they solve:
a host code that hands the GPU a fixed memory budget at start-up, a process
whose device allocations belong to a pool it does not control, or a time step
that must not stall on a cudaMalloc.  For them the library has one entry
point that takes the matrix and vectors already on the device and solves with
scratch from a static device array.  This file checks, through the C ABI,
two calls in a row against the existing entry point (fvc_solve on a context
with the same CSRD matrix) with the FP64 parity tolerance the other tests
use, and the rejection of systems beyond the array's capacity.  It is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from _systems import pressure

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10   # FP64 parity bar of the other solver tests
ITS_TOL = 2
MAX_ROWS = 131072  # capacity of the static scratch array


def _system(orc):
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(150, kind="mixed", jitter=0.2, seed=21)   # ~33k cells
    s = pressure(orc, m, 1, True)
    assert s["n"] <= MAX_ROWS
    return s


def _noalloc(L, dev, n, b, x, tol, maxit, init=1, stop_rule=0):
    from fortranfvcell_gb300._lib import FvcStats
    st = FvcStats()
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = L.fvc_pcg_csrd_noalloc(p(dev["ad"]), p(dev["au"]), p(dev["ia"]), p(dev["ja"]), n,
                                p(b), p(x), tol, maxit, init, stop_rule, None, C.byref(st))
    return rc, st


def test_noalloc_pcg_matches_context_solve(fvc, orc):
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    L = fvc.load()
    s = _system(orc)
    n = s["n"]
    rng = np.random.default_rng(42)
    b = rng.uniform(-1.0, 1.0, n)
    dev = {k: torch.from_numpy(np.ascontiguousarray(s[k])).cuda()
           for k in ("ad", "au", "ia", "ja")}
    bd = torch.from_numpy(b).cuda()
    # the existing entry point on the same matrix
    ctx = Context()
    ctx.set_matrix(1, True, n, s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    x_ref = torch.zeros(n, dtype=torch.float64, device="cuda")
    st_ref = ctx.solve(1, bd, x_ref, 1e-10, 20000, make_opts("fp64", init=1))
    torch.cuda.synchronize()
    xr = x_ref.cpu().numpy()
    results = []
    for call in range(2):
        x = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")  # init=1 zeroes it
        torch.cuda.synchronize()
        rc, st = _noalloc(L, dev, n, bd, x, 1e-10, 20000)
        assert rc == 0, f"call {call}: status {rc}"
        xn = x.cpu().numpy()
        err = np.linalg.norm(xn - xr) / np.linalg.norm(xr)
        assert err <= REL_TOL, f"call {call}: rel err {err:.3e}"
        assert abs(st.iterations - st_ref.iterations) <= ITS_TOL
        results.append(xn)
    # the static array keeps the previous call's contents; a fresh call must
    # not depend on them
    assert np.array_equal(results[0], results[1])


def test_noalloc_allocates_nothing_and_rejects_oversize(fvc, orc):
    import torch
    L = fvc.load()
    s = _system(orc)
    n = s["n"]
    dev = {k: torch.from_numpy(np.ascontiguousarray(s[k])).cuda()
           for k in ("ad", "au", "ia", "ja")}
    bd = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(L, dev, n, bd, x, 1e-8, 20000)      # first call: symbol look-up
    assert rc == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc, st = _noalloc(L, dev, n, bd, x, 1e-8, 20000)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert rc == 0 and st.iterations > 0
    assert free_after == free_before
    # a system beyond the static capacity is refused before any device work
    rc, _ = _noalloc(L, dev, MAX_ROWS + 1, bd, x, 1e-8, 100)
    assert rc == 6  # FVC_ERR_ARG
