"""ctypes front end of the CPU restatement (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
load this module.  It wraps ``oracle/build/liboracle.so`` (built from
``fvc_oracle.c`` by ``oracle/Makefile``).  All index arrays carry Fortran
1-based values, exactly as the reference's Fortran routines see them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class Stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("inner_its", C.c_int32),
        ("energy", C.c_double),
        ("conv", C.c_double),
        ("final_crit", C.c_double),
        ("status", C.c_int32),
    ]


OK, NOCONV, UNSUPPORTED = 0, 1, 2


def build() -> str:
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        srcs = ("fvc_oracle.c", "fvc_oracle_simple.c", "fvc_oracle.h")
        if not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, f)) for f in srcs
        ):
            build()
        L = C.CDLL(LIB_PATH)
        I, D = C.c_int32, C.c_double
        vp = C.c_void_p
        sig = {
            "oref_adjtria3": [vp, vp, vp, I, I, I, vp],
            "oref_adjquad4": [vp, vp, vp, I, I, I, vp],
            "oref_reord": [vp, vp, I, I, I],
            "oref_adjacency_mixed": [vp, I, vp, vp, I, I, I],
            "oref_pform_pressure": [vp, I, vp, I, I, I, vp, vp, vp, vp, I, I, I, I, vp, vp, vp,
                                    vp],
            "oref_numeq": [vp, vp, vp, I, I, vp],
            "oref_datastruc": [vp, vp, vp, I, I, I, I],
            "oref_banda_csr": [vp, vp, I],
            "oref_assbly": [vp, vp, vp, vp, vp, vp, vp, D, vp, I, I, I, I, I],
            "oref_matvec_csrd": [vp] * 7 + [I],
            "oref_matvec_csr": [vp] * 7 + [I],
            "oref_matvec_csrc": [vp] * 7 + [I],
            "oref_matvec_csrc_sym": [vp] * 7 + [I],
            "oref_matvec_csrd_sym": [vp] * 7 + [I],
            "oref_matvec_ellpack": [vp] * 7 + [I],
            "oref_dot": [vp, vp, I],
            "oref_solver": [vp] * 7 + [I, I, I, D, I, I, I, I, C.POINTER(Stats)],
            "oref_pcg_omp_sample": [vp] * 7 + [I, I, D, I, I, I, I, I, C.POINTER(Stats)],
            "oref_smachn": [],
            "oref_getres": [vp, vp, vp, I, I, I],
            "oref_gform": [vp, vp, I, I, I, vp, vp, vp, I, I, vp, vp],
            "oref_pform_momentum": [vp, vp, I, I, I, vp, vp, vp, vp, vp, I, I, vp, vp, vp, vp,
                                    vp, vp, D, I, D, I, I, I, vp, vp, vp, vp, vp, vp, vp, vp],
            "oref_pform_pc": [vp, vp, I, I, I, vp, vp, vp, vp, vp, vp, vp, vp, vp, I, I, I, vp,
                              vp, vp, vp, vp, vp],
            "oref_simple_update": [vp, vp, vp, vp, vp, vp, vp, I, D],
            "oref_divergente": [vp, vp, vp, I],
            "oref_gform_energy": [vp, vp, I, I, I, vp, vp, vp, vp, I, vp, vp],
            "oref_pform_pc_idg": [vp, vp, I, I, I, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, I,
                                  D, I, I, I, vp, vp, vp, vp, vp, vp],
            "oref_enthalpy_temp": [vp, vp, vp, I, I],
            "oref_ideal_gas": [vp, vp, I, I, I, D, D],
            "oref_pform_momentum_idg": [vp, vp, I, I, I, vp, vp, vp, vp, vp, I, I, vp, vp, vp,
                                        vp, vp, vp, vp, vp, vp, D, I, D, I, I, I, vp, vp, vp,
                                        vp, vp, vp, vp, vp],
            "oref_pform_energy": [vp, vp, I, I, I, vp, vp, vp, vp, vp, I, I, vp, vp, vp, vp,
                                  vp, D, I, I, I, vp, vp, vp, vp, vp, vp],
        }
        res = {"oref_dot": D, "oref_smachn": D, "oref_banda_csr": I, "oref_datastruc": I,
               "oref_solver": I, "oref_pcg_omp_sample": I, "oref_gform": I,
               "oref_pform_momentum": I, "oref_pform_pc": I, "oref_gform_energy": I,
               "oref_pform_energy": I, "oref_pform_momentum_idg": I, "oref_pform_pc_idg": I}
        for name, argt in sig.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = res.get(name, None)
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def adjacency(ix: np.ndarray, nnode: int, nen: int) -> np.ndarray:
    """nelcon(nen, numel) from ix(nen+1, numel) (Adjacency.f)."""
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    numel = ix.shape[0]
    nelcon = np.zeros((numel, nen), dtype=np.int32)
    nodcon = np.zeros(nnode, dtype=np.int32)
    nedge = C.c_int32(0)
    f = lib().oref_adjquad4 if nen == 4 else lib().oref_adjtria3
    f(_p(ix), _p(nodcon), _p(nelcon), nnode, numel, nen, C.byref(nedge))
    return nelcon


def adjacency_mixed(ix: np.ndarray, nnode: int, nshared: int) -> np.ndarray:
    """nelcon for meshes mixing triangles and quads (0 = unused node slot)."""
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    numel, ld = ix.shape
    nelcon = np.zeros((numel, nshared), dtype=np.int32)
    nodcon = np.zeros(nnode, dtype=np.int32)
    lib().oref_adjacency_mixed(_p(ix), ld, _p(nodcon), _p(nelcon), nnode, numel, nshared)
    return nelcon


def pform_pressure(coor, ix, nshared, nelcon, num, ia, ja, matriz, unsym=True, kprop=None,
                   dsim=None, pin_cell=1, int_vel=5):
    """(ad, au) of the pressure-correction system (CellibPressure.f)."""
    coor = np.ascontiguousarray(coor, np.float64)
    ix = np.ascontiguousarray(ix, np.int32)
    numel = ix.shape[0]
    kprop = np.ones(numel) if kprop is None else np.ascontiguousarray(kprop, np.float64)
    dsim = np.ones((numel, 2)) if dsim is None else np.ascontiguousarray(dsim, np.float64)
    ja = np.ascontiguousarray(ja, np.int32).ravel()
    ad = np.zeros(numel)
    au = np.zeros(ja.size)
    lib().oref_pform_pressure(_p(coor), coor.shape[0], _p(ix), ix.shape[1], numel, nshared,
                              _p(np.ascontiguousarray(nelcon, np.int32)),
                              _p(np.ascontiguousarray(num, np.int32)), _p(kprop), _p(dsim),
                              pin_cell, int_vel, matriz, int(unsym),
                              _p(np.ascontiguousarray(ia, np.int32)), _p(ja), _p(ad), _p(au))
    return ad, au


def reord(nelcon: np.ndarray, freord: bool = True) -> np.ndarray:
    """num(old cell) = new equation (Reord.f, RCM)."""
    nelcon = np.ascontiguousarray(nelcon, dtype=np.int32)
    numel, nshared = nelcon.shape
    iperm = np.zeros(numel, dtype=np.int32)
    lib().oref_reord(_p(nelcon), _p(iperm), numel, nshared, int(freord))
    return iperm


def numeq(num: np.ndarray, nelcon: np.ndarray) -> np.ndarray:
    nelcon = np.ascontiguousarray(nelcon, dtype=np.int32)
    numel, nshared = nelcon.shape
    ident = np.zeros((numel, nshared), dtype=np.int32)
    neq = C.c_int32(0)
    lib().oref_numeq(_p(ident), _p(np.ascontiguousarray(num, np.int32)), _p(nelcon), numel,
                     nshared, C.byref(neq))
    return ident


def datastruc(ident: np.ndarray, matriz: int, unsym: bool):
    """(ia, ja, nad) for matriz 1..4 (Datastruct.f)."""
    ident = np.ascontiguousarray(ident, dtype=np.int32)
    neq, nshared = ident.shape
    ia = np.zeros(2 if matriz == 4 else neq + 1, dtype=np.int32)
    n = lib().oref_datastruc(_p(ident), _p(ia), None, neq, nshared, matriz, int(unsym))
    ja = np.zeros(max(n, 1), dtype=np.int32)
    nad = lib().oref_datastruc(_p(ident), _p(ia), _p(ja), neq, nshared, matriz, int(unsym))
    if matriz == 4:
        ja = ja.reshape(neq, nshared)
    return ia, ja, nad


def banda_csr(ia, ja, neq):
    return lib().oref_banda_csr(_p(ia), _p(ja), neq)


def dot(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return lib().oref_dot(_p(a), _p(b), a.size)


def smachn():
    return lib().oref_smachn()


_MV = {
    "csrd": "oref_matvec_csrd",
    "csr": "oref_matvec_csr",
    "csrc": "oref_matvec_csrc",
    "csrc_sym": "oref_matvec_csrc_sym",
    "csrd_sym": "oref_matvec_csrd_sym",
    "ellpack": "oref_matvec_ellpack",
}


def matvec(kind, ad, au, al, x, ia, ja, neq, y=None):
    """Call the restated Matvec.f routine with the argument order that
    Solver.f passes (ad, au, al, x, y, ia, ja, neq)."""
    if y is None:
        y = np.zeros(neq, dtype=np.float64)
    args = {
        "csrd": (ad, au, al),
        "csr": (ad, au, al),
        "csrc": (ad, au, al),
        "csrc_sym": (ad, au, al),
        "csrd_sym": (ad, au, al),
        "ellpack": (ad, au, al),
    }[kind]
    getattr(lib(), _MV[kind])(*[_p(a) for a in args], _p(x), _p(y), _p(ia), _p(ja), neq)
    return y


def solver(ad, au, al, x, b, iax, ja, neq, nad, unsym, tol, maxit, code, matriz,
           omp_threads=0):
    """Solver.f:28 restated.  x and b are updated in place (b is clobbered
    as in the reference).  Returns (status, Stats)."""
    st = Stats()
    dummy = np.zeros(1, np.float64)
    au = dummy if au is None else au
    al = dummy if al is None else al
    status = lib().oref_solver(_p(ad), _p(au), _p(al), _p(x), _p(b), _p(iax), _p(ja),
                               neq, nad, int(unsym), tol, maxit, code, matriz,
                               omp_threads, C.byref(st))
    return status, st


def pcg_omp_sample(ad, au, x, b, iax, ja, neq, nad, tol, maxit, matriz, nthreads,
                   init=True, stop_rule=0):
    """pcg_omp (Iterativos_omp.f:30-127) for at most maxit iterations; b is
    clobbered.  stop_rule 0 is the reference's test, 1 stops on
    ||r|| < tol ||b|| (the GPU solves' stop_rule 1)."""
    st = Stats()
    status = lib().oref_pcg_omp_sample(_p(ad), _p(au), _p(au), _p(x), _p(b), _p(iax),
                                       _p(ja), neq, nad, tol, maxit, matriz, nthreads,
                                       int(init), int(stop_rule), C.byref(st))
    return status, st


# ----------------------------------------------------------------------
# SIMPLE outer-loop cells (fvc_oracle_simple.c).  A "cavity" bundle is a
# dict with coor (nnode,2), ix (numel,ld), nelcon (numel,nshared),
# pedge (numel,nshared+1), sedge (numel,nshared+1,3), e (nmat,10), num,
# and nshared; cell fields are cell-ordered numpy arrays, 2-vectors
# shaped (numel, 2), iM (numel, 4).

def _c(a, t):
    return np.ascontiguousarray(a, t)


def gform(m, kind, comp, u, grad):
    """Green-Gauss gradient of u (Pform.f gform): kind 1 = momentum ghost
    rules for component comp, kind 2 = pressure ghost rules.  grad (numel,2)
    is read (the pressure rules extrapolate with it) and overwritten."""
    u = _c(u, np.float64)
    assert grad.flags.c_contiguous and grad.dtype == np.float64
    rc = lib().oref_gform(_p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)),
                          m["ix"].shape[1], m["ix"].shape[0], m["nshared"],
                          _p(_c(m["nelcon"], np.int32)), _p(_c(m["pedge"], np.int32)),
                          _p(_c(m["sedge"], np.float64)), kind, comp, _p(u), _p(grad))
    if rc != 0:
        raise ValueError("boundary code without a defined ghost value")
    return grad


def pform_momentum(m, comp, iws, u, u0, w, g_own, g_oth, gradp, dt, ia, ja, matriz,
                   b, im, d, rescell, ad=None, au=None, bs=False, under_u=0.7,
                   simple_c=False, unsym=True):
    """Momentum system of component comp (cell_si_eb_i_ggl): iws 1 assembles
    (ad, au), adds to b and writes iM, d, the cell residual; iws 3 adds the
    time term rho cc A/dt u to b only."""
    numel = m["ix"].shape[0]
    ad = np.zeros(1) if ad is None else ad
    au = np.zeros(1) if au is None else au
    rc = lib().oref_pform_momentum(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1], numel,
        m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(m["num"], np.int32)),
        _p(_c(m["pedge"], np.int32)), _p(_c(m["sedge"], np.float64)), _p(_c(m["e"], np.float64)),
        comp, iws, _p(_c(u, np.float64)), _p(_c(u0, np.float64)), _p(_c(w, np.float64)),
        _p(_c(g_own, np.float64)), _p(_c(g_oth, np.float64)), _p(_c(gradp, np.float64)),
        dt, int(bs), under_u, int(simple_c), matriz, int(unsym), _p(_c(ia, np.int32)),
        _p(_c(ja, np.int32)), _p(ad), _p(au), _p(b), _p(im), _p(d), _p(rescell))
    if rc != 0:
        raise ValueError("oref_pform_momentum failed")
    return ad, au


def pform_momentum_idg(m, comp, iws, u, u0, w, g_own, g_oth, gradp, ro, div, grav, dt, ia, ja,
                       matriz, b, im, d, rescell, ad=None, au=None, bs=False, under_u=0.7,
                       simple_c=False, unsym=True):
    """Ideal-gas momentum system (cell_si_eb_idg_ggl): as pform_momentum with
    the densities ro (numel,3), the divergence div (numel) and gravity (2,)."""
    numel = m["ix"].shape[0]
    ad = np.zeros(1) if ad is None else ad
    au = np.zeros(1) if au is None else au
    rc = lib().oref_pform_momentum_idg(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1], numel,
        m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(m["num"], np.int32)),
        _p(_c(m["pedge"], np.int32)), _p(_c(m["sedge"], np.float64)), _p(_c(m["e"], np.float64)),
        comp, iws, _p(_c(u, np.float64)), _p(_c(u0, np.float64)), _p(_c(w, np.float64)),
        _p(_c(g_own, np.float64)), _p(_c(g_oth, np.float64)), _p(_c(gradp, np.float64)),
        _p(_c(ro, np.float64)), _p(_c(div, np.float64)), _p(_c(grav, np.float64)), dt, int(bs),
        under_u, int(simple_c), matriz, int(unsym), _p(_c(ia, np.int32)), _p(_c(ja, np.int32)),
        _p(ad), _p(au), _p(b), _p(im), _p(d), _p(rescell))
    if rc != 0:
        raise ValueError("oref_pform_momentum_idg failed")
    return ad, au


def pform_pc(m, w, d, p, gradp, ia, ja, matriz, ad, au, b, rescell, int_vel=5, unsym=True):
    """Pressure-correction system with its right-hand side (cell_si_p_i_ggl
    iws 1 with cellVel)."""
    numel = m["ix"].shape[0]
    rc = lib().oref_pform_pc(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1], numel,
        m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(m["num"], np.int32)),
        _p(_c(m["pedge"], np.int32)), _p(_c(m["sedge"], np.float64)), _p(_c(m["e"], np.float64)),
        _p(_c(w, np.float64)), _p(_c(d, np.float64)), _p(_c(p, np.float64)),
        _p(_c(gradp, np.float64)), int_vel, matriz, int(unsym), _p(_c(ia, np.int32)),
        _p(_c(ja, np.int32)), _p(ad), _p(au), _p(b), _p(rescell))
    if rc != 0:
        raise ValueError("oref_pform_pc: unsupported intVel")
    return ad, au


def simple_update(w, p, u1, u2, pc, gradpc, d, under_pc):
    lib().oref_simple_update(_p(w), _p(p), _p(_c(u1, np.float64)), _p(_c(u2, np.float64)),
                             _p(_c(pc, np.float64)), _p(_c(gradpc, np.float64)),
                             _p(_c(d, np.float64)), w.shape[0], under_pc)


def divergente(gu1, gu2):
    div = np.zeros(gu1.shape[0])
    lib().oref_divergente(_p(div), _p(_c(gu1, np.float64)), _p(_c(gu2, np.float64)),
                          gu1.shape[0])
    return div


def gform_energy(m, lib_, pedge, sedge, u, grad):
    """Green-Gauss gradient of the energy / transported scalar u (gform with
    lib 3: ideal-gas enthalpy ghost rules, lib 4: transport ghost rules).
    pedge, sedge: the scalar's (numel, nshared+1) boundary arrays.  grad
    (numel,2) is read (lib 3 extrapolates with it) and overwritten."""
    assert grad.flags.c_contiguous and grad.dtype == np.float64
    rc = lib().oref_gform_energy(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1],
        m["ix"].shape[0], m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(pedge, np.int32)),
        _p(_c(sedge, np.float64)), _p(_c(m["e"], np.float64)), lib_, _p(_c(u, np.float64)),
        _p(grad))
    if rc != 0:
        raise ValueError("oref_gform_energy: lib must be 3 or 4")
    return grad


def pform_energy(m, lib_, iws, pedge, sedge, u, u0, ro, w, grad, dt, ia, ja, matriz, b,
                 rescell, ad=None, au=None, bs=False, unsym=True):
    """Energy / scalar system (cell_e_eb_idg_ggl for lib 3, cell_t_eb_ggl
    for lib 4): iws 1 assembles (ad, au), b and the cell residual; iws 4
    writes the time term plus the volume source into b only.  ro (numel,3):
    densities at levels n-1, n and the current iterate."""
    numel = m["ix"].shape[0]
    ad = np.zeros(1) if ad is None else ad
    au = np.zeros(1) if au is None else au
    rc = lib().oref_pform_energy(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1], numel,
        m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(m["num"], np.int32)),
        _p(_c(pedge, np.int32)), _p(_c(sedge, np.float64)), _p(_c(m["e"], np.float64)),
        lib_, iws, _p(_c(u, np.float64)), _p(_c(u0, np.float64)), _p(_c(ro, np.float64)),
        _p(_c(w, np.float64)), _p(_c(grad, np.float64)), dt, int(bs), matriz, int(unsym),
        _p(_c(ia, np.int32)), _p(_c(ja, np.int32)), _p(ad), _p(au), _p(b), _p(rescell))
    if rc != 0:
        raise ValueError("oref_pform_energy: lib must be 3 or 4 and iws 1 or 4")
    return ad, au


def pform_pc_idg(m, w, d, p, gradp, ro, dt, ia, ja, matriz, ad, au, b, rescell, int_vel=5,
                 bs=False, unsym=True):
    """Ideal-gas pressure-correction system (cell_si_p_idg_ggl iws 1)."""
    numel = m["ix"].shape[0]
    rc = lib().oref_pform_pc_idg(
        _p(_c(m["coor"], np.float64)), _p(_c(m["ix"], np.int32)), m["ix"].shape[1], numel,
        m["nshared"], _p(_c(m["nelcon"], np.int32)), _p(_c(m["num"], np.int32)),
        _p(_c(m["pedge"], np.int32)), _p(_c(m["sedge"], np.float64)), _p(_c(m["e"], np.float64)),
        _p(_c(w, np.float64)), _p(_c(d, np.float64)), _p(_c(p, np.float64)),
        _p(_c(gradp, np.float64)), _p(_c(ro, np.float64)), int_vel, dt, int(bs), matriz,
        int(unsym), _p(_c(ia, np.int32)), _p(_c(ja, np.int32)), _p(ad), _p(au), _p(b),
        _p(rescell))
    if rc != 0:
        raise ValueError("oref_pform_pc_idg: unsupported intVel")
    return ad, au


def enthalpy_temp(h, t, e, to_temp):
    """EnthalpyForTemp in place: to_temp -> t from h, else h from t."""
    lib().oref_enthalpy_temp(_p(h), _p(t), _p(_c(e, np.float64)), h.shape[0], int(to_temp))


def ideal_gas(ro, temp, row, celsius=True, pressure_ratio=1.0, under_ro=1.0):
    """idealGas: ro[:, row-1] relaxed toward the air density at temp."""
    assert ro.flags.c_contiguous and ro.shape[1] == 3
    lib().oref_ideal_gas(_p(ro), _p(_c(temp, np.float64)), ro.shape[0], int(celsius), row,
                         pressure_ratio, under_ro)
