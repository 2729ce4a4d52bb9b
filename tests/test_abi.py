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


def _f90():
    src = open(os.path.join(ROOT, "include", "fvcgpu.f90")).read()
    return re.sub(r"!.*", "", src)


def test_fortran_module_binds_exported_symbols(fvc):
    # every bind(C, name=...) of include/fvcgpu.f90 is declared in the C
    # header (no Fortran compiler runs here; this keeps the module honest)
    names = re.findall(r'bind\(C,\s*name="(\w+)"\)', _f90())
    assert names and not set(names) - set(declared_functions())


def test_fortran_derived_types_match_the_c_structs(fvc):
    # field names, order and kinds of the bind(C) types against the ctypes
    # structures that mirror fvcgpu.h
    import ctypes as C
    from fortranfvcell_gb300 import _lib
    kind = {"real(c_double)": C.c_double, "integer(c_int32_t)": C.c_int32}
    src = _f90()
    for ftype, cls in (("fvc_opts", _lib.FvcOpts), ("fvc_stats", _lib.FvcStats),
                       ("fvc_simple_opts", _lib.FvcSimpleOpts)):
        body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % ftype, src, re.S).group(1)
        fields = []
        for line in body.strip().splitlines():
            t, names = line.split("::")
            fields += [(n.strip(), kind[t.strip()]) for n in names.split(",")]
        assert fields == [(n, t) for n, t in cls._fields_], ftype


def test_solver_log_line_matches_fortran_format(fvc):
    # the reference's unit-13 line, format (a,a,i9,a,d20.10,a,d20.10)
    # (src/Iterativos.f:91-93): labels, an i9 count and two D20.10 fields,
    # checked against an independent Fortran E-format writer
    from fortranfvcell_gb300.io import fortran_e
    from fortranfvcell_gb300.solver import format_solver_log
    labels = {1: "PCG:       ", 2: "PBICGSTAB: ", 3: "GMRES: "}
    for code, its, energy, tol in [(1, 123, 1.234567890123, 1e-8), (2, 7, -0.0, 1e-12),
                                   (3, 45, 9.99999999996e99, 1e-10), (1, 0, 0.5, 1.0),
                                   (2, 123456789, -3.0e-200, 5e-324)]:
        d = lambda v: fortran_e(v, 20, 10).replace("E", "D")
        want = f"{labels[code]}it{its:9d} energy norm {d(energy)} tol {d(tol)}"
        assert format_solver_log(code, its, energy, tol) == want
