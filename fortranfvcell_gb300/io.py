"""Host-side file formats of fortranFVCell.

* MatrixMarket export and import of the linear systems, in the layout of the
  reference's ``exportCoo`` / ``csrToCoo`` / ``writeCoo``
  (src/ExportCoo.f:23-62, src/CsrToCoo.f:29-180): ``<prefix>.mtx`` holds the
  matrix in coordinate form, row by row with each row's diagonal first and
  then its off-diagonals in the CSR order of the structure, written as
  ``(2i9,e24.16)``; ``<prefix>_b.mtx`` holds the right-hand side as a dense
  array.  ``read_mtx`` reads any MatrixMarket coordinate or array file and
  ``coo_to_csrd`` turns a coordinate matrix back into the CSRD arrays of
  src/Datastruct.f (diagonal apart, sorted off-diagonals, values negated as
  stored).
* ``read_deck``: the mesh, material, boundary and SIMPLE-parameter sections
  of the reference's ``.dat`` input decks (src/Rdata_mvf.f:20-807 and the
  macro list of src/Main.f), with ``insert`` files.  The deck's output and
  loop macros are recorded, not executed.
"""
from __future__ import annotations

import os

import numpy as np


# ---------------------------------------------------------------- MatrixMarket
def fortran_e(v: float, w: int = 24, d: int = 16) -> str:
    """v in Fortran ``Ew.d`` form (0.ddd...E+xx, right-justified to w); a
    three-digit exponent drops the E as Fortran does."""
    v = float(v)
    if v == 0.0 or not np.isfinite(v):
        body = f"0.{'0' * d}E+00" if v == 0.0 else ("NaN" if v != v else
                                                   ("Infinity" if v > 0 else "-Infinity"))
        if v == 0.0 and np.signbit(v):
            body = "-" + body
        return body.rjust(w)
    s = f"{abs(v):.{d - 1}e}"                  # d significant digits: m.mmme+XX
    mant, ex = s.split("e")
    digits = mant.replace(".", "")
    e = int(ex) + 1                            # 0.ddd x 10^e
    sign = "-" if v < 0 else ""
    if abs(e) <= 99:
        body = f"{sign}0.{digits}E{'+' if e >= 0 else '-'}{abs(e):02d}"
    else:
        body = f"{sign}0.{digits}{'+' if e >= 0 else '-'}{abs(e):03d}"
    return body.rjust(w)


def coo_entries(ia, ja, ad, au, al, neq, matriz=1, unsym=True):
    """(rows, cols, vals), 1-based, in the order of csrToCoo: per row the
    diagonal, then the row's stored off-diagonals.  matriz 1 (CSRD) takes
    every off-diagonal from al (the reference passes al = au when unsym);
    matriz 3 (CSRC) takes the upper ones from au."""
    if matriz not in (1, 3):
        raise ValueError("csrToCoo handles matriz 1 (CSRD) and 3 (CSRC)")
    ia = np.asarray(ia, np.int64)
    ja = np.asarray(ja, np.int64)
    al = np.asarray(au if al is None else al, np.float64)
    au = np.asarray(al if au is None else au, np.float64)
    nad = int(ia[neq] - 1)
    rows = np.empty(neq + nad, np.int64)
    cols = np.empty(neq + nad, np.int64)
    vals = np.empty(neq + nad)
    counts = np.diff(ia[: neq + 1])
    first = np.concatenate([[0], np.cumsum(counts + 1)[:-1]])   # diagonal slot of each row
    rows[first] = np.arange(1, neq + 1)
    cols[first] = np.arange(1, neq + 1)
    vals[first] = np.asarray(ad, np.float64)[:neq]
    off = np.ones(neq + nad, bool)
    off[first] = False
    r = np.repeat(np.arange(1, neq + 1), counts)
    rows[off] = r
    cols[off] = ja[:nad]
    upper = ja[:nad] > r
    v = al[:nad].copy()
    if matriz == 3:
        v[upper] = au[:nad][upper]
    vals[off] = v
    return rows, cols, vals


def write_coo(prefix, ia, ja, ad, au, al, b, neq, unsym=True, matriz=1):
    """Writes <prefix>.mtx and <prefix>_b.mtx as the reference's exportCoo
    does; returns the two file names."""
    rows, cols, vals = coo_entries(ia, ja, ad, au, al, neq, matriz, unsym)
    kind = "general" if unsym else "symmetric"
    name = f"{prefix}.mtx"
    with open(name, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate real {kind}\n")
        f.write(f"{neq:9d}{neq:9d}{rows.size:9d}\n")
        f.writelines(f"{i:9d}{j:9d}{fortran_e(v)}\n" for i, j, v in zip(rows, cols, vals))
    bname = f"{prefix}_b.mtx"
    with open(bname, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{neq:9d}{1:9d}\n")
        f.writelines(f"{fortran_e(v)}\n" for v in np.asarray(b, np.float64)[:neq])
    return name, bname


def _float(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def read_mtx(path):
    """Any MatrixMarket real coordinate or array file: dict(format, field,
    symmetry, shape, rows, cols, vals) with 1-based rows/cols (coordinate)
    or dict(format='array', shape, vals) with vals in column order."""
    with open(path) as f:
        header = f.readline().split()
        if len(header) < 5 or header[0].lower() != "%%matrixmarket":
            raise ValueError(f"{path}: not a MatrixMarket file")
        fmt, field, sym = header[2].lower(), header[3].lower(), header[4].lower()
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        dims = [int(t) for t in line.split()]
        toks = f.read().split()
    if fmt == "array":
        m, n = dims[:2]
        vals = np.array([_float(t) for t in toks[: m * n]])
        return dict(format="array", field=field, symmetry=sym, shape=(m, n), vals=vals)
    m, n, nnz = dims[:3]
    a = np.array(toks[: 3 * nnz], dtype=object).reshape(nnz, 3)
    rows = a[:, 0].astype(np.int64)
    cols = a[:, 1].astype(np.int64)
    vals = np.array([_float(t) for t in a[:, 2]])
    return dict(format="coordinate", field=field, symmetry=sym, shape=(m, n), rows=rows,
                cols=cols, vals=vals)


def coo_to_csrd(rows, cols, vals, n, symmetric=False):
    """CSRD arrays (ad, au, ia, ja, nad) of a coordinate matrix: diagonal in
    ad, the off-diagonals of each row sorted by column (1-based ia/ja).  A
    symmetric file lists one triangle; it is expanded to both (the unsym
    CSRD layout)."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    vals = np.asarray(vals, np.float64)
    if symmetric:
        o = rows != cols
        rows = np.concatenate([rows, cols[o]])
        cols = np.concatenate([cols, rows[: o.size][o]])
        vals = np.concatenate([vals, vals[o]])
    ad = np.zeros(n)
    d = rows == cols
    np.add.at(ad, rows[d] - 1, vals[d])
    r, c, v = rows[~d], cols[~d], vals[~d]
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    ia = np.ones(n + 1, np.int64)
    ia[1:] = 1 + np.cumsum(np.bincount(r - 1, minlength=n))
    return ad, v, ia.astype(np.int32), c.astype(np.int32), int(c.size)


# ---------------------------------------------------------------- .dat decks
# run-section macros of src/Main.f that take one number
_NUMERIC = {"tsimpu1", "tsimpu2", "tsimppc", "tsimpen", "maxitt1", "itsimple", "ttranst1",
            "underpc", "underp", "underu", "dt", "underro", "tolpcg", "tolbipcg", "maxitsol"}
# element sections: name -> nodes per element
_ELEMENTS = {"bar2": 2, "tria3": 3, "quad4": 4, "tetra4": 4, "hexa8": 8}


class _Lines:
    """Token lines of a deck with `insert` expanded in place."""

    def __init__(self, path):
        self.base = os.path.dirname(os.path.abspath(path))
        self.stack = [self._read(path)]

    @staticmethod
    def _read(path):
        with open(path) as f:
            return iter([ln.split() for ln in f.read().splitlines()])

    def next(self):
        while self.stack:
            try:
                toks = next(self.stack[-1])
            except StopIteration:
                self.stack.pop()
                continue
            if not toks or toks[0].startswith("#"):
                continue
            if toks[0] == "insert":
                self.stack.append(self._read(os.path.join(self.base, toks[1])))
                continue
            if toks[0] == "return":
                self.stack.pop()
                continue
            return toks
        return None


def read_deck(path):
    """Parses a fortranFVCell .dat deck.  Returns a dict with
    params (nnode, numel, ndf, ndfF, ndfE, numat, maxno, dim), coor
    (nnode, dim), ix (numel, maxno+1; material last, 0 for absent nodes),
    materials {ma: (type, e(1..))}, e (numat, 10), types (numat),
    pedgeF / sedgeF (numel, maxno+1[, ndfF]) flow boundary codes / values,
    pedgeE / sedgeE (numel, maxno+1) energy ones, gravity, initialE,
    config (key -> value) and run (macro -> value, flags -> True, plus the
    ordered list of run macros)."""
    L = _Lines(path)
    out = dict(params={}, materials={}, gravity=np.zeros(2), config={}, run={},
               run_macros=[], initialE=None)
    toks = L.next()
    while toks is not None:
        key = toks[0]
        if key == "config":
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                for k in range(0, len(t) - 1, 2):
                    out["config"][t[k]] = t[k + 1]
        elif key == "mesh":
            t = L.next()
            p = {t[k]: int(t[k + 1]) for k in range(0, len(t) - 1, 2)}
            out["params"] = p
            nnode, numel, nen = p["nnode"], p["numel"], p["maxno"]
            ndm, ndff = p.get("dim", 2), max(p.get("ndfF", 0), 1)
            out["coor"] = np.zeros((nnode, ndm))
            out["ix"] = np.zeros((numel, nen + 1), np.int32)
            out["pedgeF"] = np.zeros((numel, nen + 1), np.int32)
            out["sedgeF"] = np.zeros((numel, nen + 1, ndff))
            out["pedgeE"] = np.zeros((numel, nen + 1), np.int32)
            out["sedgeE"] = np.zeros((numel, nen + 1))
        elif key == "materials":
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                out["materials"][int(t[0])] = (int(t[1]), [_float(x) for x in t[2:]])
        elif key == "coordinates":
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                out["coor"][int(t[0]) - 1] = [_float(x) for x in t[1:1 + out["coor"].shape[1]]]
        elif key in _ELEMENTS:
            k = _ELEMENTS[key]
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                c = int(t[0]) - 1
                out["ix"][c, :k] = [int(x) for x in t[1:1 + k]]
                out["ix"][c, -1] = int(t[1 + k])
        elif key in ("elconstrainCfd", "elconstrainE"):
            dst = out["pedgeF"] if key == "elconstrainCfd" else out["pedgeE"]
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                v = [int(x) for x in t[1:]]
                dst[int(t[0]) - 1, :len(v)] = v
        elif key in ("edgeCfd", "edgeE"):
            dst = out["sedgeF"] if key == "edgeCfd" else out["sedgeE"]
            while True:
                t = L.next()
                if t is None or t[0] == "end":
                    break
                v = np.array([_float(x) for x in t[1:]])
                row = dst[int(t[0]) - 1]
                if row.ndim == 2:        # values face by face, ndfF per face
                    nf = v.size // row.shape[1]
                    row[:nf] = v[: nf * row.shape[1]].reshape(nf, row.shape[1])
                else:
                    row[: v.size] = v
        elif key == "gravity":
            t = L.next()
            out["gravity"] = np.array([_float(x) for x in t])
            L.next()                     # end gravity
        elif key in ("initialE", "initialT1", "initialtemp"):
            t = L.next()
            out[key if key != "initialtemp" else "initialT1"] = _float(t[0])
            L.next()                     # end
        elif key == "end":
            pass                         # end mesh
        else:
            name = key.lower()
            if name in _NUMERIC and len(toks) > 1:
                out["run"][key] = _float(toks[1])
            elif len(toks) > 1 and toks[1].lstrip("-").isdigit():
                out["run"][key] = int(toks[1])
            else:
                out["run"][key] = True
            out["run_macros"].append(key)
        toks = L.next()
    if out["materials"]:
        numat = max(out["materials"])
        e = np.zeros((numat, 10))
        types = np.zeros(numat, np.int32)
        for ma, (typ, vals) in out["materials"].items():
            types[ma - 1] = typ
            e[ma - 1, : min(10, len(vals))] = vals[:10]
        out["e"], out["types"] = e, types
    return out


def simple_case(deck):
    """The arrays of the SIMPLE loop (cells.SimpleLoop, fvc_simple_create)
    from a parsed deck: coor, ix (material last), nelcon from this library's
    adjacency, num from RCM (or the identity when the deck's config sets
    reord false, as src/Main.f does), pedge / sedge (numel, nshared+1[, 3])
    of the flow and e (numat, 10).  Also the scalar's pedgeE / sedgeE and
    gravity, for the energy cells."""
    from . import mesh as _mesh
    nen = deck["params"]["maxno"]
    m = _mesh.Mesh(np.ascontiguousarray(deck["coor"][:, :2]),
                   np.ascontiguousarray(deck["ix"][:, :nen]), nen)
    nelcon = _mesh.adjacency(m)
    if deck["config"].get("reord", "true").lower() == "false":
        num = np.arange(1, deck["params"]["numel"] + 1, dtype=np.int32)
    else:
        num = _mesh.rcm(nelcon)
    sedge = np.zeros((deck["params"]["numel"], nen + 1, 3))
    k = min(3, deck["sedgeF"].shape[2])
    sedge[:, :, :k] = deck["sedgeF"][:, :, :k]
    return dict(coor=m.coor, ix=np.ascontiguousarray(deck["ix"], np.int32), nelcon=nelcon,
                num=np.ascontiguousarray(num, np.int32), ident=_mesh.numeq(num, nelcon),
                pedge=np.ascontiguousarray(deck["pedgeF"], np.int32), sedge=sedge,
                e=deck["e"], nshared=nen, numel=deck["params"]["numel"], mesh=m,
                pedgeE=deck["pedgeE"], sedgeE=deck["sedgeE"], gravity=deck["gravity"])


# ---------------------------------------------------------------- checkpoints
def save_simple(path, istep, t, w, w0, p, ro, en=None, en0=None):
    """Writes a SIMPLE restart file in the ASCII layout of the reference's
    saveSimple (src/Simple.f:1307-1626): labelled blocks with the step
    (i9), the time (f20.8), w and w0 (3f36.16, two values a line), p
    (f36.16), with the energy equation en and en0 (f36.16), and the three
    density levels (3f36.16)."""
    f36 = lambda v: f"{float(v):36.16f}"
    with open(path, "w") as f:
        f.write("passo de tempo\n")
        f.write(f"{int(istep):9d}\n")
        f.write("tempo \n")
        f.write(f"{float(t):20.8f}\n")
        for label, a in (("Velocidade (n)", w), ("Velocidade (n-1)", w0)):
            f.write(label + "\n")
            f.writelines(f36(u) + f36(v) + "\n" for u, v in np.asarray(a).reshape(-1, 2))
        f.write("pressao (n)\n")
        f.writelines(f36(v) + "\n" for v in np.asarray(p).ravel())
        if en is not None:
            f.write("en (n)\n")
            f.writelines(f36(v) + "\n" for v in np.asarray(en).ravel())
            f.write("en (n-1)\n")
            f.writelines(f36(v) + "\n" for v in np.asarray(en0).ravel())
        f.write("ro      \n")
        f.writelines(f36(a) + f36(b) + f36(c) + "\n" for a, b, c in np.asarray(ro).reshape(-1, 3))


def load_simple(path, numel, energy=False):
    """Reads a saveSimple restart file: dict(istep, t, w, w0, p, ro[, en,
    en0]).  energy says whether the file holds the en blocks (the
    reference's sEnergy at save time)."""
    with open(path) as f:
        lines = f.read().splitlines()
    pos = 0

    def block(ncols):
        nonlocal pos
        pos += 1                                      # label line
        out = np.array([[float(x) for x in ln.split()] for ln in lines[pos:pos + numel]])
        pos += numel
        return out.reshape(numel, ncols) if ncols > 1 else out.ravel()
    st = {"istep": int(lines[1]), "t": float(lines[3])}
    pos = 4
    st["w"] = block(2)
    st["w0"] = block(2)
    st["p"] = block(1)
    if energy:
        st["en"] = block(1)
        st["en0"] = block(1)
    st["ro"] = block(3)
    return st
