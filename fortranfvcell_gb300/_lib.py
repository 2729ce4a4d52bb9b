"""ctypes binding of libfvcgpu.so (the C ABI declared in include/fvcgpu.h).

The library is built in-tree by :mod:`fortranfvcell_gb300.build`.  Loading
fails loudly when it is missing: there is no CPU fallback for any entry
point of this package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

I32, I64, F64 = C.c_int32, C.c_int64, C.c_double
P = C.c_void_p
PI32 = C.POINTER(C.c_int32)
PF64 = C.POINTER(C.c_double)

FVC_OK = 0
FVC_ERR_NOCONV = 1
FVC_ERR_BREAKDOWN = 2
FVC_ERR_NAN = 3
FVC_ERR_UNSUPPORTED = 4
FVC_ERR_CUDA = 5
FVC_ERR_ARG = 6
FVC_ERR_TIMEOUT = 7
STATUS_NAMES = {0: "OK", 1: "NOCONV", 2: "BREAKDOWN", 3: "NAN", 4: "UNSUPPORTED",
                5: "CUDA", 6: "ARG", 7: "TIMEOUT"}

FVC_PREC_FP64 = 0
FVC_PREC_MIXED = 1


class FvcOpts(C.Structure):
    _fields_ = [
        ("precision", I32),
        ("init", I32),
        ("refine_tol", F64),
        ("inner_tol", F64),
        ("max_refine", I32),
        ("block_threads", I32),
        ("blocks_per_sm", I32),
        ("stop_rule", I32),
        ("want_residual", I32),
        ("update_beta", I32),
        ("staging", I32),
        ("max_blocks", I32),
        ("fp32_layout", I32),
        ("cluster_size", I32),
    ]


class FvcStats(C.Structure):
    _fields_ = [
        ("status", I32),
        ("iterations", I32),
        ("inner_iterations", I32),
        ("refinements", I32),
        ("energy", F64),
        ("conv", F64),
        ("final_crit", F64),
        ("rel_residual", F64),
        ("solve_ms", F64),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class FvcCellMesh(C.Structure):
    """fvc_cell_mesh: device pointers to a mesh in the reference's layouts."""
    _fields_ = [
        ("numel", I32),
        ("nshared", I32),
        ("nnode", I32),
        ("nmat", I32),
        ("coor", C.c_void_p),
        ("ix", C.c_void_p),
        ("nelcon", C.c_void_p),
        ("num", C.c_void_p),
        ("pedge", C.c_void_p),
        ("sedge", C.c_void_p),
        ("e", C.c_void_p),
        ("geometry", C.c_void_p),
    ]


class FvcSimpleOpts(C.Structure):
    _fields_ = [
        ("dt", F64),
        ("under_u", F64),
        ("under_pc", F64),
        ("simple_c", I32),
        ("bs", I32),
        ("int_vel", I32),
        ("matriz_u", I32),
        ("code_u", I32),
        ("tol_u", F64),
        ("matriz_pc", I32),
        ("code_pc", I32),
        ("tol_pc", F64),
        ("maxit", I32),
        ("precision", I32),
        ("precision_u", I32),
    ]


# name -> (argtypes, restype); mirrors include/fvcgpu.h
SIGNATURES = {
    "fvc_solver": ([P] * 5 + [PI32, PI32, PI32, PI32, PI32, PF64, PI32, PI32, PI32, PI32], None),
    "solver_": ([P] * 5 + [PI32, PI32, PI32, PI32, PI32, PF64, PI32, PI32, PI32, PI32], None),
    "fvc_opts_default": ([C.POINTER(FvcOpts)], None),
    "fvc_solver_ex": ([P] * 7 + [I32, I32, I32, F64, I32, I32, I32, C.POINTER(FvcOpts),
                                 C.POINTER(FvcStats)], I32),
    "fvc_context_create": ([C.POINTER(P), I32], I32),
    "fvc_context_destroy": ([P], I32),
    "fvc_context_set_stream": ([P, P], I32),
    "fvc_matrix_set": ([P, I32, I32, I32, I32, P, P, P, P, P], I32),
    "fvc_matrix_update_values": ([P, P, P, P], I32),
    "fvc_matrix_update_values_async": ([P, P, P, P], I32),
    "fvc_solve_async": ([P, I32, P, P, F64, I32, C.POINTER(FvcOpts), P], I32),
    "fvc_autotune": ([P, I32, I32, I32, C.POINTER(FvcOpts), P], I32),
    "fvc_set_solver_log": ([P, P], None),
    "fvc_format_solver_log": ([I32, I32, F64, F64, P, I32], I32),
    "fvc_solve_transposed": ([P, I32, P, P, F64, I32, C.POINTER(FvcOpts),
                              C.POINTER(FvcStats)], I32),
    "fvc_solve": ([P, I32, P, P, F64, I32, C.POINTER(FvcOpts), C.POINTER(FvcStats)], I32),
    "fvc_solve_batched": ([P, I32, P, P, P, F64, I32, C.POINTER(FvcOpts), P], I32),
    "fvc_solve_batched_ex": ([P, I32, P, P, P, P, P, P, F64, I32, C.POINTER(FvcOpts), P],
                             I32),
    "fvc_spmv": ([P, P, P], I32),
    "fvc_spmv_fast": ([P, P, P], I32),
    "fvc_spmv_f32": ([P, P, P], I32),
    "fvc_matrix_info": ([P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)], I32),
    "fvc_kernel_launches": ([], I64),
    "fvc_solve_trace": ([P, I32, P, P], I32),
    "fvc_solve_history": ([P, I32, P], I32),
    "fvc_pcg_csrd_noalloc": ([P, P, P, P, I32, P, P, F64, I32, I32, I32, P,
                              C.POINTER(FvcStats)], I32),
    "fvc_mesh_adjacency": ([P, I32, I32, I32, I32, P], I32),
    "fvc_mesh_rcm": ([P, I32, I32, I32, P], I32),
    "fvc_mesh_numeq": ([P, P, I32, I32, P], I32),
    "fvc_mesh_datastruc": ([P, I32, I32, I32, I32, P, P, PI32, C.POINTER(I64)], I32),
    "fvc_assemble_pressure": ([P, I32, P, I32, I32, I32, P, P, P, P, I32, I32, I32, I32, P, P,
                               P, P], I32),
    "fvc_cells_gradient": ([C.POINTER(FvcCellMesh), I32, I32, P, P, P], I32),
    "fvc_cells_geometry_create": ([C.POINTER(FvcCellMesh), C.POINTER(C.c_void_p)], I32),
    "fvc_cells_geometry_destroy": ([P], I32),
    "fvc_cells_momentum": ([C.POINTER(FvcCellMesh), I32, I32, P, P, P, P, P, P, F64, I32, F64,
                            I32, I32, P, P, P, P, P, P, P, P, P], I32),
    "fvc_cells_momentum_ideal_gas": ([C.POINTER(FvcCellMesh), I32, I32, P, P, P, P, P, P, P, P,
                                      F64, F64, F64, I32, F64, I32, I32, P, P, P, P, P, P, P, P,
                                      P], I32),
    "fvc_cells_pressure_correction": ([C.POINTER(FvcCellMesh), P, P, P, P, I32, I32, P, P, P, P,
                                       P, P, P], I32),
    "fvc_cells_simple_update": ([I32, P, P, P, P, P, P, P, F64, P], I32),
    "fvc_cells_pressure_correction_ideal_gas": ([C.POINTER(FvcCellMesh), P, P, P, P, P, I32,
                                                 F64, I32, I32, P, P, P, P, P, P, P], I32),
    "fvc_cells_enthalpy_temperature": ([I32, P, P, F64, F64, I32, P], I32),
    "fvc_cells_ideal_gas_density": ([I32, P, P, I32, I32, F64, F64, P], I32),
    "fvc_cells_divergence": ([I32, P, P, P, P], I32),
    "fvc_getres": ([I32, P, P, P, I32, P], I32),
    "fvc_cells_energy": ([C.POINTER(FvcCellMesh), I32, I32, P, P, P, P, P, P, P, F64, I32, I32,
                          P, P, P, P, P, P, P], I32),
    "fvc_cells_energy_gradient": ([C.POINTER(FvcCellMesh), I32, P, P, P, P, P], I32),
    "fvc_simple_opts_default": ([C.POINTER(FvcSimpleOpts)], None),
    "fvc_simple_create": ([C.POINTER(P), I32, I32, I32, I32, I32, P, P, P, P, P, P, P,
                           C.POINTER(FvcSimpleOpts)], I32),
    "fvc_simple_iterate": ([P, I32, P, P], I32),
    "fvc_simple_set_graph": ([P, I32], I32),
    "fvc_simple_system": ([P, I32, P, P, P, P], I32),
    "fvc_simple_iterate_energy": ([P, I32, P, P], I32),
    "fvc_simple_energy": ([P, P, P, F64, F64, F64], I32),
    "fvc_simple_energy_fields": ([P, P, P, P], I32),
    "fvc_simple_get_state": ([P, P, P, P, P, P, P], I32),
    "fvc_simple_set_state": ([P, P, P, P, P, P, P], I32),
    "fvc_simple_time_step": ([P], I32),
    "fvc_simple_fields": ([P, P, P], I32),
    "fvc_simple_set_fields": ([P, P, P], I32),
    "fvc_simple_destroy": ([P], I32),
    "fvc_simple_batch_create": ([P, I32, P, I32, I32], I32),
    "fvc_simple_batch_iterate": ([P, I32, P, P], I32),
    "fvc_simple_batch_destroy": ([P], I32),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libfvcgpu.so, building it first when absent or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and _build.needs_build():
        _build.build()
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libfvcgpu.so not found at {path}; run fortranfvcell_gb300.build")
    L = C.CDLL(path)
    for name, (argt, rest) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = argt
        f.restype = rest
    _lib = L
    return L


def check(rc: int, what: str = "fvcgpu call") -> None:
    if rc != FVC_OK:
        raise FvcError(rc, f"{what} failed: {STATUS_NAMES.get(rc, rc)}")


class FvcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status
