"""GB300 (sm_103a) linear-solver hot path of the fortranFVCell finite-volume
code: sliced-ELLPACK SpMV, persistent PCG / BiCGSTAB / GMRES(15) kernels,
mixed-precision defect correction and the pressure-correction assembly,
behind the reference's ``solver`` call (C ABI in include/fvcgpu.h).
"""
from ._lib import FvcError, FvcOpts, FvcStats, load  # noqa: F401
from .solver import Context, kernel_launches, make_opts, pack_block_diagonal, solver  # noqa: F401

__all__ = ["Context", "FvcError", "FvcOpts", "FvcStats", "kernel_launches", "load",
           "make_opts", "pack_block_diagonal", "solver"]
