"""Test systems built on the CPU: synthetic meshes -> equation graph ->
pressure-correction (p') matrix with the restated assembly, and an
unsymmetric convection-diffusion variant for BiCGSTAB / GMRES."""
import numpy as np


def _ptr(a):
    import ctypes as C
    return a.ctypes.data_as(C.c_void_p)


def graph(orc, m):
    """nelcon, num, id for mesh m (oracle chain; mixed meshes use the
    product adjacency, which has no reference counterpart)."""
    from fortranfvcell_gb300 import mesh
    if m.nshared == m.ix.shape[1] and np.all(m.nsides == m.nshared):
        ixm = np.concatenate([m.ix, np.ones((m.numel, 1), np.int32)], axis=1)
        nelcon = orc.adjacency(ixm, m.nnode, m.ix.shape[1])
    else:
        nelcon = mesh.adjacency(m)
    num = orc.reord(nelcon)
    return nelcon, num, orc.numeq(num, nelcon)


def pressure(orc, m, matriz=1, unsym=True, pin_cell=1, int_vel=5, kprop=None, dsim=None):
    nelcon, num, ident = graph(orc, m)
    ia, ja, nad = orc.datastruc(ident, matriz, unsym)
    n = m.numel
    ad = np.zeros(n)
    au = np.zeros(ja.size)
    kprop = np.ones(n) if kprop is None else kprop
    dsim = np.ones((n, 2)) if dsim is None else dsim
    L = orc.lib()
    L.oref_pform_pressure(_ptr(np.ascontiguousarray(m.coor)), m.nnode,
                          _ptr(np.ascontiguousarray(m.ix, np.int32)), m.ix.shape[1], n,
                          m.nshared, _ptr(nelcon), _ptr(num), _ptr(np.ascontiguousarray(kprop)),
                          _ptr(np.ascontiguousarray(dsim)), pin_cell, int_vel, matriz, int(unsym),
                          _ptr(ia), _ptr(ja), _ptr(ad), _ptr(au))
    return dict(nelcon=nelcon, num=num, ident=ident, ia=ia, ja=ja, nad=nad, ad=ad, au=au, n=n)


def unsymmetric(sys_, seed=0, skew=0.4, lower_only=False):
    """Convection-like unsymmetric M-matrix on the same structure: the
    off-diagonals are scaled by 1 +- skew per entry and the diagonal is the
    row's absolute off-diagonal sum plus 5% (diagonally dominant)."""
    rng = np.random.default_rng(seed)
    au = sys_["au"] * (1.0 + skew * rng.uniform(-1, 1, sys_["au"].size))
    ia, ja = sys_["ia"], sys_["ja"]
    n = sys_["n"]
    ad = np.zeros(n)
    if ia.size == 2:  # ELLPACK
        w = ia[0]
        ad = np.abs(au.reshape(n, w)).sum(axis=1) * 1.05 + 1e-3
    else:
        for r in range(n):
            ad[r] = np.abs(au[ia[r] - 1:ia[r + 1] - 1]).sum()
        if lower_only:
            # symmetric-structure storage (CSRC, CSRD sym): the transposed
            # terms of later rows belong to this row's sum too
            rows = np.repeat(np.arange(n), np.diff(ia))
            np.add.at(ad, ja - 1, np.abs(au))
        ad = ad * 1.05 + 1e-3
    out = dict(sys_)
    out["au"], out["ad"] = au, ad
    return out


def csr_matrix(s, matriz=1, unsym=True):
    """scipy CSR of the system as the reference's matvec applies it."""
    import scipy.sparse as sp
    n, ia, ja = s["n"], s["ia"], s["ja"]
    rows, cols, vals = [], [], []
    if matriz == 4:
        w = ia[0]
        jj = ja.reshape(n, w)
        au = s["au"].reshape(n, w)
        r = np.repeat(np.arange(n), w)
        rows, cols, vals = r, jj.ravel() - 1, au.ravel()
        A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    else:
        r = np.repeat(np.arange(n), np.diff(ia))
        A = sp.csr_matrix((s["au"], (r, ja - 1)), shape=(n, n))
        if matriz in (1, 3) and not unsym:
            A = A + A.T
    return (A + sp.diags(s["ad"])).tocsr()
