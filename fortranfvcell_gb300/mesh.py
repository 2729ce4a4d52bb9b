"""Meshes and the equation graph (host side of libfvcgpu).

``square_mesh`` generates the synthetic 2-D meshes the benchmarks run on
(unit square, uniform or jittered nodes, quads, triangles or a seeded mix),
stored the way the reference stores cells: ``ix`` holds each cell's 1-based
node numbers counter-clockwise, one row per cell (the reference's
``ix(nen+1,numel)`` without the material column; unused slots are 0).

The remaining functions call the C ABI of libfvcgpu for the reference's
setup chain (src/Main.f:588-692): face adjacency (Adjacency.f), RCM
(Reord.f), equation numbering (Numeq.f), sparse structures (Datastruct.f),
and the GPU assembly of the pressure-correction matrix (CellibPressure.f).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class Mesh:
    coor: np.ndarray   # (nnode, 2) float64
    ix: np.ndarray     # (numel, ld) int32, 1-based nodes, 0 = unused slot
    nshared: int       # faces per cell slot (3 tri, 4 quad or mixed)

    @property
    def nnode(self) -> int:
        return self.coor.shape[0]

    @property
    def numel(self) -> int:
        return self.ix.shape[0]

    @property
    def nsides(self) -> np.ndarray:
        return (self.ix > 0).sum(axis=1).astype(np.int32)


def square_mesh(nx: int, ny: int | None = None, kind: str = "quad", jitter: float = 0.0,
                seed: int = 1234, split_seed: int | None = None) -> Mesh:
    """Unit square split into ``nx`` x ``ny`` cells.

    kind: "quad" (nen 4), "tri" (each quad cut along a seeded diagonal, nen 3)
    or "mixed" (each quad kept or cut with probability 1/2, nshared 4).
    jitter: interior nodes move by uniform[-jitter, jitter] * h in x and y.
    Nodes are numbered row by row (node (i, j) -> 1 + i + j*(nx+1)).
    """
    ny = nx if ny is None else ny
    hx, hy = 1.0 / nx, 1.0 / ny
    xs, ys = np.meshgrid(np.arange(nx + 1) * hx, np.arange(ny + 1) * hy)
    coor = np.stack([xs.ravel(), ys.ravel()], axis=1).astype(np.float64)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=coor.shape) * np.array([hx, hy])
        ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1))
        interior = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)).ravel()
        coor[interior] += d[interior]
    i, j = np.meshgrid(np.arange(nx), np.arange(ny))
    i, j = i.ravel(), j.ravel()
    n00 = 1 + i + j * (nx + 1)
    n10 = n00 + 1
    n11 = n10 + (nx + 1)
    n01 = n00 + (nx + 1)
    if kind == "quad":
        ix = np.stack([n00, n10, n11, n01], axis=1).astype(np.int32)
        return Mesh(coor, ix, 4)
    rng = np.random.default_rng(seed + 1 if split_seed is None else split_seed)
    diag = rng.integers(0, 2, size=n00.size).astype(bool)   # which diagonal
    if kind == "tri":
        cut = np.ones(n00.size, dtype=bool)
    elif kind == "mixed":
        cut = rng.integers(0, 2, size=n00.size).astype(bool)
    else:
        raise ValueError(kind)
    # triangles of cut quads, diagonal n00-n11 or n10-n01
    ta = np.where(diag[:, None], np.stack([n00, n10, n11], 1), np.stack([n00, n10, n01], 1))
    tb = np.where(diag[:, None], np.stack([n00, n11, n01], 1), np.stack([n10, n11, n01], 1))
    quads = np.stack([n00, n10, n11, n01], axis=1)
    if kind == "tri":
        cells = np.empty((2 * n00.size, 3), dtype=np.int32)
        cells[0::2] = ta
        cells[1::2] = tb
        return Mesh(coor, cells, 3)
    counts = np.where(cut, 2, 1)
    out = np.zeros((counts.sum(), 4), dtype=np.int32)
    pos = np.concatenate([[0], np.cumsum(counts)[:-1]])
    keep = ~cut
    out[pos[keep]] = quads[keep]
    out[pos[cut], :3] = ta[cut]
    out[pos[cut] + 1, :3] = tb[cut]
    return Mesh(coor, out, 4)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def adjacency(mesh: Mesh) -> np.ndarray:
    """nelcon (numel, nshared): neighbour across each side, -1 boundary."""
    L = _lib.load()
    ix = np.ascontiguousarray(mesh.ix, dtype=np.int32)
    nelcon = np.empty((mesh.numel, mesh.nshared), dtype=np.int32)
    _lib.check(L.fvc_mesh_adjacency(_ptr(ix), ix.shape[1], mesh.nnode, mesh.numel,
                                    mesh.nshared, _ptr(nelcon)), "fvc_mesh_adjacency")
    return nelcon


def rcm(nelcon: np.ndarray, freord: bool = True) -> np.ndarray:
    """num (numel,): 1-based equation of each cell (RCM, src/Reord.f)."""
    L = _lib.load()
    nelcon = np.ascontiguousarray(nelcon, dtype=np.int32)
    num = np.empty(nelcon.shape[0], dtype=np.int32)
    _lib.check(L.fvc_mesh_rcm(_ptr(nelcon), nelcon.shape[0], nelcon.shape[1], int(freord),
                              _ptr(num)), "fvc_mesh_rcm")
    return num


def numeq(num: np.ndarray, nelcon: np.ndarray) -> np.ndarray:
    """id (neq, nshared): equation numbers of each equation's neighbours."""
    L = _lib.load()
    nelcon = np.ascontiguousarray(nelcon, dtype=np.int32)
    num = np.ascontiguousarray(num, dtype=np.int32)
    ident = np.empty_like(nelcon)
    _lib.check(L.fvc_mesh_numeq(_ptr(num), _ptr(nelcon), nelcon.shape[0], nelcon.shape[1],
                                _ptr(ident)), "fvc_mesh_numeq")
    return ident


def datastruc(ident: np.ndarray, matriz: int, unsym: bool):
    """(ia, ja, nad) as src/Datastruct.f builds them (1-based)."""
    L = _lib.load()
    ident = np.ascontiguousarray(ident, dtype=np.int32)
    neq, nshared = ident.shape
    ia = np.zeros(2 if matriz == 4 else neq + 1, dtype=np.int32)
    nad = C.c_int32(0)
    jalen = C.c_int64(0)
    _lib.check(L.fvc_mesh_datastruc(_ptr(ident), neq, nshared, matriz, int(unsym), _ptr(ia),
                                    None, C.byref(nad), C.byref(jalen)), "fvc_mesh_datastruc")
    ja = np.zeros(max(jalen.value, 1), dtype=np.int32)
    _lib.check(L.fvc_mesh_datastruc(_ptr(ident), neq, nshared, matriz, int(unsym), _ptr(ia),
                                    _ptr(ja), C.byref(nad), C.byref(jalen)), "fvc_mesh_datastruc")
    if matriz == 4:
        ja = ja.reshape(neq, nshared)
    return ia, ja, int(nad.value)


def assemble_pressure(mesh: Mesh, nelcon: np.ndarray, num: np.ndarray, ia: np.ndarray,
                      ja: np.ndarray, matriz: int, unsym: bool = True, kprop=None, dsim=None,
                      pin_cell: int = 0, int_vel: int = 5):
    """Pressure-correction coefficients on the GPU (CellibPressure.f:476-572).

    Returns (ad, au): diagonal and the negated off-diagonals in the slots of
    (ia, ja).  kprop: k(2,cell) per cell (default 1); dsim: the SIMPLE d per
    cell, shape (numel, 2) (default 1); pin_cell: 1-based cell with the 1e60
    pressure pin (0 = none).
    """
    L = _lib.load()
    n = mesh.numel
    kprop = np.ones(n) if kprop is None else np.ascontiguousarray(kprop, np.float64)
    dsim = np.ones((n, 2)) if dsim is None else np.ascontiguousarray(dsim, np.float64)
    coor = np.ascontiguousarray(mesh.coor, np.float64)
    ix = np.ascontiguousarray(mesh.ix, np.int32)
    nelcon = np.ascontiguousarray(nelcon, np.int32)
    num = np.ascontiguousarray(num, np.int32)
    ad = np.zeros(n, np.float64)
    nad = int(ia[-1] - 1) if matriz == 1 else n * mesh.nshared
    au = np.zeros(nad, np.float64)
    ia_ = np.ascontiguousarray(ia, np.int32)
    ja_ = np.ascontiguousarray(ja, np.int32).ravel()
    _lib.check(L.fvc_assemble_pressure(_ptr(coor), mesh.nnode, _ptr(ix), ix.shape[1], n,
                                       mesh.nshared, _ptr(nelcon), _ptr(num), _ptr(kprop),
                                       _ptr(dsim), int(pin_cell), int(int_vel), int(matriz),
                                       int(unsym), _ptr(ia_), _ptr(ja_), _ptr(ad), _ptr(au)),
               "fvc_assemble_pressure")
    return ad, au


@dataclass
class PressureSystem:
    mesh: Mesh
    nelcon: np.ndarray
    num: np.ndarray
    ident: np.ndarray
    ia: np.ndarray
    ja: np.ndarray
    nad: int
    ad: np.ndarray
    au: np.ndarray
    matriz: int
    unsym: bool

    @property
    def neq(self) -> int:
        return self.mesh.numel


def pressure_system(mesh: Mesh, matriz: int = 1, unsym: bool = True, freord: bool = True,
                    pin_cell: int | None = None, int_vel: int = 5) -> PressureSystem:
    """Full setup chain for one p' system: adjacency -> RCM -> numbering ->
    structure -> GPU assembly.  pin_cell (1-based, original numbering)
    defaults to cell 1, the cell the reference's cavity decks pin with
    pedge = -1 (input/cavidade/cavidade_quadrada/quad_cav4_b_restricion.dat)."""
    nelcon = adjacency(mesh)
    num = rcm(nelcon, freord)
    ident = numeq(num, nelcon)
    ia, ja, nad = datastruc(ident, matriz, unsym)
    pin = 1 if pin_cell is None else pin_cell
    ad, au = assemble_pressure(mesh, nelcon, num, ia, ja, matriz, unsym, pin_cell=pin,
                               int_vel=int_vel)
    return PressureSystem(mesh, nelcon, num, ident, ia, ja, nad, ad, au, matriz, unsym)
