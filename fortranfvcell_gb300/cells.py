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


def pressure_correction(m: CellMesh, w, d, p, gradp, ia, ja, matriz, ad, au, b, rescell,
                        int_vel=5) -> None:
    _lib.check(_lib.load().fvc_cells_pressure_correction(
        C.byref(m.s), _addr(w), _addr(d), _addr(p), _addr(gradp), int_vel, matriz, _addr(ia),
        _addr(ja), _addr(ad), _addr(au), _addr(b), _addr(rescell), _stream()),
        "fvc_cells_pressure_correction")


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
