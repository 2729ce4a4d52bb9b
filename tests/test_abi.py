"""libfvcgpu.so loads and exports every function include/fvcgpu.h declares
(no compute calls: runs without a GPU)."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fvcgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:void|int32_t|int64_t)\s+\**\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_dropin_entries():
    names = declared_functions()
    for required in ("fvc_solver", "solver_", "fvc_solver_ex", "fvc_solve", "fvc_spmv"):
        assert required in names


def test_library_exports_every_declared_symbol(fvc):
    from fortranfvcell_gb300 import _lib
    path = _lib.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"not exported: {missing}"
    L = fvc.load()
    for n in declared_functions():
        assert hasattr(L, n)


def test_ctypes_signatures_cover_header(fvc):
    from fortranfvcell_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_no_gpu_context_errors_cleanly(fvc):
    import ctypes as C
    import torch
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    rc = fvc.load().fvc_context_create(C.byref(h), 0)
    assert rc == 5  # FVC_ERR_CUDA: no device, no silent fallback
