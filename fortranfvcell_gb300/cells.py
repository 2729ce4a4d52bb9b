"""Device-side cell kernels of the SIMPLE outer iteration (C ABI
``fvc_cells_*`` of include/fvcgpu.h) over torch CUDA tensors.

``CellMesh`` uploads a mesh with its boundary codes and materials in the
reference's layouts (src/Pform.f: ix(nshared+1,numel) with the material
last, nelcon, pedge(nshared+1,numel), sedge(3,nshared+1,numel),
e(10,nmat)); the functions take cell-ordered torch float64 tensors, with
2-vectors shaped (numel, 2) and iM shaped (numel, 4).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _addr(t) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class CellMesh:
    def __init__(self, coor, ix, nelcon, num, pedge, sedge, e):
        import torch
        dev = "cuda"
        ix = np.ascontiguousarray(ix, np.int32)
        self.numel, ld = ix.shape
        self.nshared = ld - 1
        self.t = dict(
            coor=torch.from_numpy(np.ascontiguousarray(coor, np.float64)).to(dev),
            ix=torch.from_numpy(ix).to(dev),
            nelcon=torch.from_numpy(np.ascontiguousarray(nelcon, np.int32)).to(dev),
            num=torch.from_numpy(np.ascontiguousarray(num, np.int32)).to(dev),
            pedge=torch.from_numpy(np.ascontiguousarray(pedge, np.int32)).to(dev),
            sedge=torch.from_numpy(np.ascontiguousarray(sedge, np.float64)).to(dev),
            e=torch.from_numpy(np.ascontiguousarray(e, np.float64)).to(dev),
        )
        self.s = _lib.FvcCellMesh(self.numel, self.nshared, int(np.asarray(coor).shape[0]),
                                  int(np.asarray(e).shape[0]),
                                  *[self.t[k].data_ptr() for k in
                                    ("coor", "ix", "nelcon", "num", "pedge", "sedge", "e")])
        self._geo = None

    def cache_geometry(self, on: bool = True) -> None:
        """Compute every cell's geometry once (fvc_cells_geometry_create) for
        the cell routines to read instead of recomputing it; the same bits
        either way.  on=False drops the cache."""
        import torch
        L = _lib.load()
        if self._geo is not None:
            L.fvc_cells_geometry_destroy(self._geo)
            self._geo = None
            self.s.geometry = None
        if on:
            torch.cuda.synchronize()
            g = C.c_void_p()
            _lib.check(L.fvc_cells_geometry_create(C.byref(self.s), C.byref(g)),
                       "fvc_cells_geometry_create")
            self._geo = g
            self.s.geometry = g.value

    def __del__(self):
        if getattr(self, "_geo", None) is not None:
            try:
                _lib.load().fvc_cells_geometry_destroy(self._geo)
            except Exception:
                pass

    @property
    def num(self):
        return self.t["num"]


def gradient(m: CellMesh, kind: int, comp: int, u, grad) -> None:
    _lib.check(_lib.load().fvc_cells_gradient(C.byref(m.s), kind, comp, _addr(u), _addr(grad),
                                              _stream()), "fvc_cells_gradient")


def momentum(m: CellMesh, comp, iws, u, u0, w, g_own, g_oth, gradp, dt, ia, ja, matriz, ad, au,
             b, im, d, rescell, bs=False, under_u=0.7, simple_c=False) -> None:
    _lib.check(_lib.load().fvc_cells_momentum(
        C.byref(m.s), comp, iws, _addr(u), _addr(u0), _addr(w), _addr(g_own), _addr(g_oth),
        _addr(gradp), dt, int(bs), under_u, int(simple_c), matriz, _addr(ia), _addr(ja),
        _addr(ad), _addr(au), _addr(b), _addr(im), _addr(d), _addr(rescell), _stream()),
        "fvc_cells_momentum")


def momentum_ideal_gas(m: CellMesh, comp, iws, u, u0, w, g_own, g_oth, gradp, ro, div, grav,
                       dt, ia, ja, matriz, ad, au, b, im, d, rescell, bs=False, under_u=0.7,
                       simple_c=False) -> None:
    """Ideal-gas momentum cells (buoyancy): ro (numel, 3) densities, div
    (numel) divergence, grav = (gx, gy)."""
    _lib.check(_lib.load().fvc_cells_momentum_ideal_gas(
        C.byref(m.s), comp, iws, _addr(u), _addr(u0), _addr(w), _addr(g_own), _addr(g_oth),
        _addr(gradp), _addr(ro), _addr(div), float(grav[0]), float(grav[1]), dt, int(bs),
        under_u, int(simple_c), matriz, _addr(ia), _addr(ja), _addr(ad), _addr(au), _addr(b),
        _addr(im), _addr(d), _addr(rescell), _stream()), "fvc_cells_momentum_ideal_gas")


def pressure_correction(m: CellMesh, w, d, p, gradp, ia, ja, matriz, ad, au, b, rescell,
                        int_vel=5) -> None:
    _lib.check(_lib.load().fvc_cells_pressure_correction(
        C.byref(m.s), _addr(w), _addr(d), _addr(p), _addr(gradp), int_vel, matriz, _addr(ia),
        _addr(ja), _addr(ad), _addr(au), _addr(b), _addr(rescell), _stream()),
        "fvc_cells_pressure_correction")


def energy(m: CellMesh, lib: int, iws: int, pedge, sedge, u, u0, ro, w, grad, dt, ia, ja,
           matriz, ad, au, b, rescell, bs=False) -> None:
    """Energy / transported-scalar system (lib 3: ideal-gas enthalpy cell,
    lib 4: transport cell); pedge, sedge: the scalar's (numel, nshared+1)
    device boundary arrays, ro (numel, 3) the densities."""
    _lib.check(_lib.load().fvc_cells_energy(
        C.byref(m.s), lib, iws, _addr(pedge), _addr(sedge), _addr(u), _addr(u0), _addr(ro),
        _addr(w), _addr(grad), dt, int(bs), matriz, _addr(ia), _addr(ja), _addr(ad), _addr(au),
        _addr(b), _addr(rescell), _stream()), "fvc_cells_energy")


def energy_gradient(m: CellMesh, lib: int, pedge, sedge, u, grad) -> None:
    _lib.check(_lib.load().fvc_cells_energy_gradient(
        C.byref(m.s), lib, _addr(pedge), _addr(sedge), _addr(u), _addr(grad), _stream()),
        "fvc_cells_energy_gradient")


def pressure_correction_ideal_gas(m: CellMesh, w, d, p, gradp, ro, dt, ia, ja, matriz, ad, au,
                                  b, rescell, int_vel=5, bs=False) -> None:
    _lib.check(_lib.load().fvc_cells_pressure_correction_ideal_gas(
        C.byref(m.s), _addr(w), _addr(d), _addr(p), _addr(gradp), _addr(ro), int_vel, dt,
        int(bs), matriz, _addr(ia), _addr(ja), _addr(ad), _addr(au), _addr(b), _addr(rescell),
        _stream()), "fvc_cells_pressure_correction_ideal_gas")


def enthalpy_temperature(h, t, cp, tref, to_temperature: bool) -> None:
    _lib.check(_lib.load().fvc_cells_enthalpy_temperature(
        h.shape[0], _addr(h), _addr(t), cp, tref, int(to_temperature), _stream()),
        "fvc_cells_enthalpy_temperature")


def ideal_gas_density(ro, temp, row, celsius=True, pressure_ratio=1.0, under_ro=1.0) -> None:
    _lib.check(_lib.load().fvc_cells_ideal_gas_density(
        ro.shape[0], _addr(ro), _addr(temp), int(celsius), row, pressure_ratio, under_ro,
        _stream()), "fvc_cells_ideal_gas_density")


def simple_update(w, p, u1, u2, pc, gradpc, d, under_pc) -> None:
    _lib.check(_lib.load().fvc_cells_simple_update(
        w.shape[0], _addr(w), _addr(p), _addr(u1), _addr(u2), _addr(pc), _addr(gradpc),
        _addr(d), under_pc, _stream()), "fvc_cells_simple_update")


def divergence(div, gu1, gu2) -> None:
    _lib.check(_lib.load().fvc_cells_divergence(div.shape[0], _addr(div), _addr(gu1),
                                                _addr(gu2), _stream()), "fvc_cells_divergence")


def getres(num, u, x, to_equations: bool) -> None:
    _lib.check(_lib.load().fvc_getres(u.shape[0], _addr(num), _addr(u), _addr(x),
                                      int(to_equations), _stream()), "fvc_getres")


def simple_opts(**kw):
    """fvc_simple_opts with the library defaults, overridden by keyword."""
    o = _lib.FvcSimpleOpts()
    _lib.load().fvc_simple_opts_default(C.byref(o))
    for k, v in kw.items():
        if k in ("precision", "precision_u"):
            v = {"fp64": _lib.FVC_PREC_FP64, "mixed": _lib.FVC_PREC_MIXED}.get(v, v)
        setattr(o, k, v)
    return o


class SimpleLoop:
    """The isothermal SIMPLE outer iteration resident on the GPU
    (fvc_simple_* of include/fvcgpu.h).  Mesh arrays are host numpy arrays
    in the reference layouts (see CellMesh); ``opts`` from simple_opts()."""

    def __init__(self, coor, ix, nelcon, num, pedge, sedge, e, opts=None, device: int = 0):
        self._L = _lib.load()
        ix = np.ascontiguousarray(ix, np.int32)
        self.numel, ld = ix.shape
        self._keep = [np.ascontiguousarray(coor, np.float64), ix,
                      np.ascontiguousarray(nelcon, np.int32), np.ascontiguousarray(num, np.int32),
                      np.ascontiguousarray(pedge, np.int32), np.ascontiguousarray(sedge, np.float64),
                      np.ascontiguousarray(e, np.float64)]
        coor_, ix_, nel_, num_, pe_, se_, e_ = self._keep
        h = C.c_void_p()
        o = simple_opts() if opts is None else opts
        _lib.check(self._L.fvc_simple_create(
            C.byref(h), device, self.numel, coor_.shape[0], ld - 1, e_.reshape(-1, 10).shape[0],
            *[a.ctypes.data_as(C.c_void_p) for a in self._keep], C.byref(o)), "fvc_simple_create")
        self._h = h

    def iterate(self, nit: int):
        """Runs nit outer iterations; returns (residuals (nit,3), solver
        iterations (nit,3)) -- the cell-residual norms of u1, u2 and p'."""
        res = np.zeros((nit, 3))
        its = np.zeros((nit, 3), np.int32)
        _lib.check(self._L.fvc_simple_iterate(self._h, nit, res.ctypes.data_as(C.c_void_p),
                                              its.ctypes.data_as(C.c_void_p)),
                   "fvc_simple_iterate")
        return res, its

    def enable_energy(self, pedge_e, sedge_e, gravity, t0: float) -> None:
        """Ideal-gas iteration with the energy equation (fvc_simple_energy)."""
        pe = np.ascontiguousarray(pedge_e, np.int32)
        se = np.ascontiguousarray(sedge_e, np.float64)
        _lib.check(self._L.fvc_simple_energy(self._h, pe.ctypes.data_as(C.c_void_p),
                                             se.ctypes.data_as(C.c_void_p), float(gravity[0]),
                                             float(gravity[1]), float(t0)), "fvc_simple_energy")

    def iterate_energy(self, nit: int):
        """nit outer iterations of the energy loop: (residuals (nit,4),
        solver iterations (nit,4)) for u1, u2, p' and the enthalpy."""
        res = np.zeros((nit, 4))
        its = np.zeros((nit, 4), np.int32)
        _lib.check(self._L.fvc_simple_iterate_energy(self._h, nit,
                                                     res.ctypes.data_as(C.c_void_p),
                                                     its.ctypes.data_as(C.c_void_p)),
                   "fvc_simple_iterate_energy")
        return res, its

    def energy_fields(self):
        """(temperature, enthalpy, densities (numel,3))."""
        t, h, ro = np.zeros(self.numel), np.zeros(self.numel), np.zeros((self.numel, 3))
        _lib.check(self._L.fvc_simple_energy_fields(self._h, t.ctypes.data_as(C.c_void_p),
                                                    h.ctypes.data_as(C.c_void_p),
                                                    ro.ctypes.data_as(C.c_void_p)),
                   "fvc_simple_energy_fields")
        return t, h, ro

    def get_state(self, energy: bool = False) -> dict:
        """w, w0, p (and en, en0, ro with the energy equation), as saveSimple
        writes them."""
        n = self.numel
        st = dict(w=np.zeros((n, 2)), w0=np.zeros((n, 2)), p=np.zeros(n))
        if energy:
            st.update(en=np.zeros(n), en0=np.zeros(n), ro=np.zeros((n, 3)))
        ptr = lambda k: st[k].ctypes.data_as(C.c_void_p) if k in st else None
        _lib.check(self._L.fvc_simple_get_state(self._h, *[ptr(k) for k in
                                                          ("w", "w0", "p", "en", "en0", "ro")]),
                   "fvc_simple_get_state")
        return st

    def set_state(self, st: dict) -> None:
        """Uploads a saved state and starts a step from it."""
        arrs = {k: np.ascontiguousarray(v, np.float64) for k, v in st.items()
                if k in ("w", "w0", "p", "en", "en0", "ro") and v is not None}
        ptr = lambda k: arrs[k].ctypes.data_as(C.c_void_p) if k in arrs else None
        _lib.check(self._L.fvc_simple_set_state(self._h, *[ptr(k) for k in
                                                          ("w", "w0", "p", "en", "en0", "ro")]),
                   "fvc_simple_set_state")

    def time_step(self) -> None:
        _lib.check(self._L.fvc_simple_time_step(self._h), "fvc_simple_time_step")

    def system(self, which: int):
        """(ad, au, b) of the last outer iteration's system: which = 1 u1,
        2 u2, 3 p', 4 the enthalpy; equation order, the structure of
        mesh.datastruc for the system's matriz."""
        nja = C.c_int64()
        _lib.check(self._L.fvc_simple_system(self._h, int(which), None, None, None,
                                             C.byref(nja)), "fvc_simple_system")
        ad = np.zeros(self.numel)
        au = np.zeros(max(nja.value, 1))
        b = np.zeros(self.numel)
        _lib.check(self._L.fvc_simple_system(self._h, int(which), ad.ctypes.data_as(C.c_void_p),
                                             au.ctypes.data_as(C.c_void_p),
                                             b.ctypes.data_as(C.c_void_p), C.byref(nja)),
                   "fvc_simple_system")
        return ad, au[:nja.value], b

    def use_graph(self, on: bool = True) -> None:
        """Run each outer iteration as one CUDA graph launch (same results)."""
        _lib.check(self._L.fvc_simple_set_graph(self._h, int(bool(on))), "fvc_simple_set_graph")

    def fields(self):
        w = np.zeros((self.numel, 2))
        p = np.zeros(self.numel)
        _lib.check(self._L.fvc_simple_fields(self._h, w.ctypes.data_as(C.c_void_p),
                                             p.ctypes.data_as(C.c_void_p)), "fvc_simple_fields")
        return w, p

    def set_fields(self, w=None, p=None) -> None:
        w = None if w is None else np.ascontiguousarray(w, np.float64)
        p = None if p is None else np.ascontiguousarray(p, np.float64)
        _lib.check(self._L.fvc_simple_set_fields(
            self._h, None if w is None else w.ctypes.data_as(C.c_void_p),
            None if p is None else p.ctypes.data_as(C.c_void_p)), "fvc_simple_set_fields")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.fvc_simple_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SimpleBatch:
    """Many SimpleLoop cases advanced together (fvc_simple_batch_* of
    include/fvcgpu.h): per outer iteration every stage's solves of all
    cases in one persistent launch, the whole iteration one CUDA graph.
    The loops must outlive the batch.  precision ("fp64" or "mixed") for the
    p' solves, precision_u for u, v and the enthalpy (None: as precision)."""

    def __init__(self, loops, precision: str = "fp64", precision_u: str | None = None):
        self._L = _lib.load()
        self.loops = list(loops)
        handles = (C.c_void_p * len(self.loops))(*[lp._h.value for lp in self.loops])
        h = C.c_void_p()
        code = {"fp64": _lib.FVC_PREC_FP64, "mixed": _lib.FVC_PREC_MIXED}
        prec_u = -1 if precision_u is None else code[precision_u]
        _lib.check(self._L.fvc_simple_batch_create(C.byref(h), len(self.loops),
                                                   C.cast(handles, C.c_void_p), code[precision],
                                                   prec_u),
                   "fvc_simple_batch_create")
        self._h = h

    def iterate(self, nit: int, nres: int):
        """nit outer iterations of every case: (residuals (nit, ncases,
        nres), solver iterations (nit, ncases, nres)); nres 3 (isothermal
        loops) or 4 (loops with the energy equation)."""
        nc = len(self.loops)
        res = np.zeros((nit, nc, nres))
        its = np.zeros((nit, nc, nres), np.int32)
        _lib.check(self._L.fvc_simple_batch_iterate(self._h, nit, res.ctypes.data_as(C.c_void_p),
                                                    its.ctypes.data_as(C.c_void_p)),
                   "fvc_simple_batch_iterate")
        return res, its

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.fvc_simple_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
