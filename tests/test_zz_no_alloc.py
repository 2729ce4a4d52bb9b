"""The allocation-free PCG entry point, fvc_pcg_csrd_noalloc.

Some callers of this library cannot allocate device memory when they solve:
a host code that hands the GPU a fixed memory budget at start-up, a process
whose device allocations belong to a pool it does not control, or a time step
that must not stall on a cudaMalloc.  For them the library has one entry
point that takes the matrix and vectors already on the device and solves with
scratch from a static device array.  This file checks, through the C ABI:

* two calls in a row against the existing entry point (fvc_solve on a context
  with the same CSRD matrix) and against the restated reference PCG, with
  the FP64 parity bars of the other solver tests (1e-10 relative L2,
  iterations +-2);
* a warm start (init = 0) from a nonzero guess and the ||r|| <= tol ||b||
  stopping rule (stop_rule = 1), each against the restated OpenMP PCG with
  the same start and rule, and against fvc_solve;
* the refusals: a symmetric CSRD (strictly lower part only), a column out of
  range, and a system beyond the array's capacity;
* that no call after the first on a device changes the free device memory,
  and, in a fresh process, what the first call does.

It is collected last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from _systems import pressure

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10   # FP64 parity bar of the other solver tests
ITS_TOL = 2
MAX_ROWS = 131072  # capacity of the static scratch array
FVC_ERR_ARG = 6
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _system(orc, matriz=1, unsym=True):
    from fortranfvcell_gb300 import mesh
    m = mesh.square_mesh(150, kind="mixed", jitter=0.2, seed=21)   # ~33k cells
    s = pressure(orc, m, matriz, unsym)
    assert s["n"] <= MAX_ROWS
    return s


def _dev(s):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(s[k])).cuda()
            for k in ("ad", "au", "ia", "ja")}


def _noalloc(L, dev, n, b, x, tol, maxit, init=1, stop_rule=0):
    from fortranfvcell_gb300._lib import FvcStats
    st = FvcStats()
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = L.fvc_pcg_csrd_noalloc(p(dev["ad"]), p(dev["au"]), p(dev["ia"]), p(dev["ja"]), n,
                                p(b), p(x), tol, maxit, init, stop_rule, None, C.byref(st))
    return rc, st


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_pcg_matches_context_solve_and_reference(fvc, orc):
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    L = fvc.load()
    s = _system(orc)
    n = s["n"]
    b = np.random.default_rng(42).uniform(-1.0, 1.0, n)
    dev = _dev(s)
    bd = torch.from_numpy(b).cuda()
    # the existing entry point on the same matrix
    ctx = Context()
    ctx.set_matrix(1, True, n, s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    x_ctx = torch.zeros(n, dtype=torch.float64, device="cuda")
    st_ctx = ctx.solve(1, bd, x_ctx, 1e-10, 20000, make_opts("fp64", init=1))
    torch.cuda.synchronize()
    xc = x_ctx.cpu().numpy()
    # the restated reference: sequential CSRD PCG zeroes x (Solver.f:130)
    x_ref = np.zeros(n)
    rs, so = orc.solver(s["ad"].copy(), s["au"].copy(), s["au"].copy(), x_ref, b.copy(),
                        s["ia"], s["ja"], n, s["nad"], True, 1e-10, 20000, 1, 1)
    assert rs == 0
    results = []
    for call in range(2):
        x = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")  # init=1 zeroes it
        torch.cuda.synchronize()
        rc, st = _noalloc(L, dev, n, bd, x, 1e-10, 20000)
        assert rc == 0, f"call {call}: status {rc}"
        xn = x.cpu().numpy()
        e_ctx, e_ref = _rel(xn, xc), _rel(xn, x_ref)
        print(f"call {call}: its {st.iterations} (context {st_ctx.iterations}, reference "
              f"{so.iterations}); rel err vs context {e_ctx:.2e}, vs reference {e_ref:.2e}")
        assert e_ctx <= REL_TOL, f"call {call}: rel err vs fvc_solve {e_ctx:.3e}"
        assert e_ref <= REL_TOL, f"call {call}: rel err vs reference {e_ref:.3e}"
        assert abs(st.iterations - st_ctx.iterations) <= ITS_TOL
        assert abs(st.iterations - so.iterations) <= ITS_TOL
        results.append(xn)
    # the static array keeps the previous call's contents; a fresh call must
    # not depend on them
    assert np.array_equal(results[0], results[1])


@pytest.mark.parametrize("init,stop_rule", [(0, 0), (1, 1), (0, 1)])
def test_noalloc_warm_start_and_residual_rule(fvc, orc, init, stop_rule):
    # init = 0 starts from the caller's x (as the OpenMP CSRD path of the
    # reference does, Solver.f:104); stop_rule = 1 stops on ||r|| < tol ||b||.
    # The restated pcg_omp takes the same start and rule.
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    L = fvc.load()
    s = _system(orc)
    n = s["n"]
    rng = np.random.default_rng(7 + 2 * init + stop_rule)
    b = rng.uniform(-1.0, 1.0, n)
    x0 = rng.uniform(-1.0, 1.0, n) if init == 0 else np.zeros(n)
    # the pinned p' row (diagonal 1e60, CellibPressure.f:557) starts at its
    # solution, ~0, as a previous outer iteration's field does: a random
    # entry there puts ~1e60 x0 into its residual, and the cancellation
    # rounding left in that row, not the method, would then decide when
    # ||r|| first drops below tol ||b|| (stop_rule 1)
    x0[s["ad"] > 1e30] = 0.0
    tol = 1e-10 if stop_rule == 0 else 1e-11
    x_ref = x0.copy()
    rs, so = orc.pcg_omp_sample(s["ad"].copy(), s["au"].copy(), x_ref, b.copy(), s["ia"],
                                s["ja"], n, s["nad"], tol, 20000, 1, 4, init=bool(init),
                                stop_rule=stop_rule)
    assert rs == 0
    ctx = Context()
    ctx.set_matrix(1, True, n, s["nad"], s["ad"], s["au"], s["au"], s["ia"], s["ja"])
    bd = torch.from_numpy(b).cuda()
    x_ctx = torch.from_numpy(x0.copy()).cuda()
    st_ctx = ctx.solve(1, bd, x_ctx, tol, 20000,
                       make_opts("fp64", init=init, stop_rule=stop_rule))
    xc = x_ctx.cpu().numpy()
    dev = _dev(s)
    x = torch.from_numpy(x0.copy()).cuda()
    rc, st = _noalloc(L, dev, n, bd, x, tol, 20000, init=init, stop_rule=stop_rule)
    assert rc == 0
    xn = x.cpu().numpy()
    e_ref, e_ctx = _rel(xn, x_ref), _rel(xn, xc)
    print(f"init {init} stop_rule {stop_rule}: its {st.iterations} (reference {so.iterations}, "
          f"context {st_ctx.iterations}); rel err vs reference {e_ref:.2e}, vs context "
          f"{e_ctx:.2e}")
    assert e_ref <= REL_TOL and e_ctx <= REL_TOL
    assert abs(st.iterations - so.iterations) <= ITS_TOL
    assert abs(st.iterations - st_ctx.iterations) <= ITS_TOL


def test_noalloc_refuses_bad_structures_and_allocates_nothing(fvc, orc):
    import torch
    L = fvc.load()
    s = _system(orc)
    n = s["n"]
    dev = _dev(s)
    bd = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(L, dev, n, bd, x, 1e-8, 20000)      # the first call on this device
    assert rc == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc, st = _noalloc(L, dev, n, bd, x, 1e-8, 20000)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert rc == 0 and st.iterations > 0
    assert free_after == free_before
    # symmetric CSRD keeps only the strictly lower triangle: refused, x untouched
    sym = _system(orc, 1, False)
    assert np.all(sym["ja"] - 1 < np.repeat(np.arange(n), np.diff(sym["ia"])))
    xs = torch.full((n,), 3.0, dtype=torch.float64, device="cuda")
    rc, st = _noalloc(L, _dev(sym), n, bd, xs, 1e-8, 100)
    assert rc == FVC_ERR_ARG and st.iterations == 0
    assert torch.all(xs == 3.0)
    # a column outside [1, neq] is found before any gather
    bad = dict(s)
    bad["ja"] = s["ja"].copy()
    bad["ja"][len(bad["ja"]) // 2] = n + 1
    rc, _ = _noalloc(L, _dev(bad), n, bd, x, 1e-8, 100)
    assert rc == FVC_ERR_ARG
    # a solve after the refusals is unaffected
    rc, st2 = _noalloc(L, dev, n, bd, x, 1e-8, 20000)
    assert rc == 0 and st2.iterations > 0
    # a system beyond the static capacity is refused before any device work
    rc, _ = _noalloc(L, dev, MAX_ROWS + 1, bd, x, 1e-8, 100)
    assert rc == FVC_ERR_ARG
    # stop rules other than 0 and 1 are refused
    rc, _ = _noalloc(L, dev, n, bd, x, 1e-8, 100, stop_rule=2)
    assert rc == FVC_ERR_ARG


_FIRST_CALL = r"""
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, ROOT)
import torch
import fortranfvcell_gb300 as f
from fortranfvcell_gb300._lib import FvcStats
L = f.load()
n = 4096
ad = torch.full((n,), 2.0, dtype=torch.float64, device="cuda")
ia = np.zeros(n + 1, np.int32); ja = []
k = 1
for i in range(1, n + 1):
    ia[i - 1] = k
    for j in (i - 1, i + 1):
        if 1 <= j <= n:
            ja.append(j); k += 1
ia[n] = k
au = torch.full((len(ja),), -1.0, dtype=torch.float64, device="cuda")
iad = torch.from_numpy(ia).cuda(); jad = torch.from_numpy(np.array(ja, np.int32)).cuda()
b = torch.ones(n, dtype=torch.float64, device="cuda"); x = torch.zeros_like(b)
p = lambda t: C.c_void_p(t.data_ptr())
def call():
    st = FvcStats()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = L.fvc_pcg_csrd_noalloc(p(ad), p(au), p(iad), p(jad), n, p(b), p(x), 1e-8, 20000, 1, 0,
                                None, C.byref(st))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    return rc, free0 - free1
out = [call() for _ in range(3)]
print(json.dumps({"calls": out}))
""".replace("ROOT", repr(ROOT))


def test_noalloc_first_call_in_a_fresh_process(tmp_path):
    # Under CUDA's lazy module loading (the default) the first call on a
    # device loads this library's module there, and that load places the
    # static array (~5.0 MiB) in device memory.  The calls after it allocate
    # nothing.  A host with a fixed budget therefore makes one call at
    # start-up.
    script = tmp_path / "first_call.py"
    script.write_text(_FIRST_CALL)
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    calls = json.loads(r.stdout.strip().splitlines()[-1])["calls"]
    print(f"free-memory drop per call (bytes): {[d for _, d in calls]}")
    assert all(rc == 0 for rc, _ in calls)
    first, later = calls[0][1], [d for _, d in calls[1:]]
    assert all(d == 0 for d in later)
    # the array and the module's code, rounded up to the driver's pages
    assert 0 <= first <= 64 << 20
