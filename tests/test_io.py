"""File formats (fortranfvcell_gb300.io): the MatrixMarket files of the
reference's exportCoo and the .dat deck sections of its Rdata_mvf reader."""
import os

import numpy as np
import pytest

from _systems import pressure
from fortranfvcell_gb300 import io, mesh


def test_fortran_e_format():
    assert io.fortran_e(1.0) == "  0.1000000000000000E+01"
    assert io.fortran_e(-2.5e-7) == " -0.2500000000000000E-06"
    assert io.fortran_e(0.0) == "  0.0000000000000000E+00"
    assert io.fortran_e(123456.789) == "  0.1234567890000000E+06"
    assert io.fortran_e(1e-300) == "  0.1000000000000000-299"      # three-digit exponent
    for v in (np.pi, -1e-12, 6.02214076e23, 0.999999999999999999):
        assert float(io.fortran_e(v).replace("E", "e")) == pytest.approx(v, rel=1e-15)


@pytest.mark.parametrize("unsym", [True, False])
def test_coo_export_round_trip(orc, tmp_path, unsym):
    m = mesh.square_mesh(7, kind="mixed", jitter=0.2, seed=4)
    s = pressure(orc, m, 1, unsym)
    n, nad = s["n"], s["nad"]
    b = np.random.default_rng(2).uniform(-1, 1, n)
    name, bname = io.write_coo(str(tmp_path / "sys"), s["ia"], s["ja"], s["ad"], s["au"],
                               s["au"], b, n, unsym=unsym, matriz=1)
    lines = open(name).read().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate real " + ("general" if unsym else
                                                                   "symmetric")
    assert lines[1] == f"{n:9d}{n:9d}{n + nad:9d}"
    assert all(len(x) == 42 for x in lines[2:])
    mtx = io.read_mtx(name)
    # csrToCoo order: each row starts with its diagonal
    starts = np.concatenate([[0], np.cumsum(np.diff(s["ia"]) + 1)[:-1]])
    assert np.array_equal(mtx["rows"][starts], np.arange(1, n + 1))
    assert np.array_equal(mtx["cols"][starts], np.arange(1, n + 1))
    ad, au, ia, ja, nad2 = io.coo_to_csrd(mtx["rows"], mtx["cols"], mtx["vals"], n)
    # the structure comes back exactly; values to the 16 significant digits of
    # the reference's e24.16 (a double needs 17 to round-trip)
    assert nad2 == nad and np.array_equal(ia, s["ia"]) and np.array_equal(ja, s["ja"][:nad])
    np.testing.assert_allclose(ad, s["ad"], rtol=5e-16, atol=0)
    np.testing.assert_allclose(au, s["au"][:nad], rtol=5e-16, atol=0)
    bb = io.read_mtx(bname)
    assert bb["shape"] == (n, 1)
    np.testing.assert_allclose(bb["vals"], b, rtol=5e-16, atol=0)
    if not unsym:
        # the symmetric file expands to the unsymmetric CSRD layout
        su = pressure(orc, m, 1, True)
        ad, au, ia, ja, _ = io.coo_to_csrd(mtx["rows"], mtx["cols"], mtx["vals"], n,
                                           symmetric=True)
        assert np.array_equal(ia, su["ia"]) and np.array_equal(ja, su["ja"][:su["nad"]])
        np.testing.assert_allclose(au, su["au"][:su["nad"]], rtol=5e-16, atol=0)


DECK = """config
memoria 10 openMpCell false reord false
end config
mesh
nnode 9 numel 4 ndf 0 ndfF 3 ndfE 1 numat 2 maxno 4 dim 2
materials
1 55 1.72d-5 1.204d0 2.42d-2 1.012d3 20.0d0 1.0d0 7
2 65 1.0d-3 1.0d0 0.0 0.0 0.0 1.0 5
end materials
insert part_coor.dat
insert part_elem.dat
elconstrainCfd
1   1 0 0 0 -1
3   0 0 2 4 0
end elconstrainCfd
edgeCfd
1 1.0 0.0 0.0  0 0 0  0 0 0  0 0 0  0 0 0
3 0 0 0  0 0 0  0.5d0 -0.25d0 0  0 0 0  0 0 0
end edgeCfd
elconstrainE
2   0 1 0 0 0
end elconstrainE
edgeE
2   0.0 30.0d0 0.0 0.0 0.0
end edgeE
gravity
0.0d0 -9.81d0
end gravity
initialE
20.0d0
end initialE
end mesh
itSimple 20
simpleC
underU  0.7d0
tSimpPc 1.0d-3
dt 0.02
loop1 5
  simple
next1
stop
"""
COOR = "coordinates\n" + "".join(
    f"{3 * j + i + 1} {0.5 * i} {0.5 * j}\n" for j in range(3) for i in range(3)) + \
    "end coordinates\nreturn\n"
ELEM = "quad4\n1 1 2 5 4 1\n2 2 3 6 5 2\n3 4 5 8 7 1\n4 5 6 9 8 2\nend quad4\nreturn\n"


def test_read_deck_sections(tmp_path):
    (tmp_path / "deck.dat").write_text(DECK)
    (tmp_path / "part_coor.dat").write_text(COOR)
    (tmp_path / "part_elem.dat").write_text(ELEM)
    d = io.read_deck(str(tmp_path / "deck.dat"))
    assert d["params"] == dict(nnode=9, numel=4, ndf=0, ndfF=3, ndfE=1, numat=2, maxno=4, dim=2)
    assert d["config"]["reord"] == "false"
    assert np.array_equal(d["types"], [55, 65])
    assert d["e"][0, 1] == 1.204 and d["e"][0, 3] == 1012.0 and d["e"][1, 6] == 5.0
    assert np.array_equal(d["coor"][4], [0.5, 0.5]) and np.array_equal(d["coor"][8], [1.0, 1.0])
    assert np.array_equal(d["ix"][1], [2, 3, 6, 5, 2])
    assert np.array_equal(d["pedgeF"][0], [1, 0, 0, 0, -1])
    assert np.array_equal(d["pedgeF"][2], [0, 0, 2, 4, 0])
    assert np.array_equal(d["sedgeF"][0, 0], [1.0, 0.0, 0.0])
    assert np.array_equal(d["sedgeF"][2, 2], [0.5, -0.25, 0.0])
    assert np.array_equal(d["pedgeE"][1], [0, 1, 0, 0, 0]) and d["sedgeE"][1, 1] == 30.0
    assert np.array_equal(d["gravity"], [0.0, -9.81]) and d["initialE"] == 20.0
    assert d["run"]["itSimple"] == 20 and d["run"]["simpleC"] is True
    assert d["run"]["underU"] == 0.7 and d["run"]["tSimpPc"] == 1e-3 and d["run"]["dt"] == 0.02
    assert d["run"]["loop1"] == 5 and d["run_macros"][-1] == "stop"


@pytest.mark.skipif("FVC_REF_INPUT" not in os.environ,
                    reason="set FVC_REF_INPUT to the reference's input/ directory")
def test_read_shipped_decks():
    base = os.environ["FVC_REF_INPUT"]
    d = io.read_deck(os.path.join(base, "cavidade", "cavidade_quadrada", "quad_cav4_b.dat"))
    assert d["params"]["numel"] == 10000 and d["types"][0] == 65
    m = mesh.Mesh(d["coor"], d["ix"][:, :4], 4)
    nelcon = mesh.adjacency(m)
    assert (nelcon < 0).sum() == 400                    # 4 x 100 wall faces
    lid = d["pedgeF"][:, :4] == 1
    assert lid.sum() == 100 and (nelcon[lid] < 0).all()  # moving-wall codes on walls only
    assert (d["pedgeF"][:, 4] == -1).sum() == 1
    r = io.read_deck(os.path.join(base, "Ray6", "quad_cav4_b_ray6.dat"))
    assert r["types"][0] == 55 and r["gravity"][1] == -9.81 and r["initialE"] == 20.0
    assert (r["pedgeE"] == 1).sum() == 200


def test_deck_drives_the_restated_simple_loop(orc, tmp_path):
    # a 6 x 6 lid-driven cavity written as a deck, read back and stepped by
    # the restated SIMPLE iteration: the same residual history as the case
    # built directly with the library's cavity builder
    from oracle.simple_ref import SimpleRef
    from fortranfvcell_gb300.cases import lid_driven_cavity
    c = lid_driven_cavity(6)
    n, nsh = c["numel"], c["nshared"]
    coor = "coordinates\n" + "".join(f"{i + 1} {float(x)!r} {float(y)!r}\n" for i, (x, y) in
                                      enumerate(c["coor"])) + "end coordinates\n"
    elem = "quad4\n" + "".join(f"{i + 1} {' '.join(map(str, r[:nsh]))} {r[nsh]}\n"
                               for i, r in enumerate(c["ix"])) + "end quad4\n"
    cons = "elconstrainCfd\n" + "".join(f"{i + 1} {' '.join(map(str, r))}\n"
                                        for i, r in enumerate(c["pedge"])) + "end elconstrainCfd\n"
    edge = "edgeCfd\n" + "".join(f"{i + 1} {' '.join(repr(float(v)) for v in r.ravel())}\n"
                                 for i, r in enumerate(c["sedge"])) + "end edgeCfd\n"
    e = c["e"][0]
    deck = (f"mesh\nnnode {c['coor'].shape[0]} numel {n} ndf 0 ndfF 3 ndfE 0 numat 1 maxno 4 "
            f"dim 2\nmaterials\n1 65 {' '.join(repr(float(v)) for v in e[:7])}\nend materials\n"
            + coor + elem + cons + edge + "end mesh\nitSimple 10\nstop\n")
    (tmp_path / "cav.dat").write_text(deck)
    case = io.simple_case(io.read_deck(str(tmp_path / "cav.dat")))
    for k in ("coor", "ix", "nelcon", "num", "pedge", "sedge", "e"):
        assert np.array_equal(case[k], c[k]), k
    a, b = SimpleRef(orc, case), SimpleRef(orc, c)
    for _ in range(5):
        assert a.step() == b.step()


def test_save_simple_round_trip(tmp_path):
    rng = np.random.default_rng(7)
    n = 13
    st = dict(w=rng.uniform(-1, 1, (n, 2)), w0=rng.uniform(-1, 1, (n, 2)),
              p=rng.uniform(-100, 100, n), en=rng.uniform(-500, 500, n),
              en0=rng.uniform(-500, 500, n), ro=rng.uniform(1.1, 1.3, (n, 3)))
    path = str(tmp_path / "save.dat")
    io.save_simple(path, 42, 0.84, st["w"], st["w0"], st["p"], st["ro"], en=st["en"],
                   en0=st["en0"])
    lines = open(path).read().splitlines()
    assert lines[:4] == ["passo de tempo", f"{42:9d}", "tempo ", f"{0.84:20.8f}"]
    assert lines[4] == "Velocidade (n)" and len(lines[5]) == 72
    assert "pressao (n)" in lines and "en (n)" in lines and "en (n-1)" in lines
    assert lines[-n - 1] == "ro      " and len(lines[-1]) == 108
    back = io.load_simple(path, n, energy=True)
    assert back["istep"] == 42 and back["t"] == 0.84
    for k, v in st.items():     # F36.16: 16 decimals
        np.testing.assert_allclose(back[k], v, rtol=0, atol=5e-17 * 1000)
    # without the energy blocks
    io.save_simple(path, 1, 0.0, st["w"], st["w0"], st["p"], st["ro"])
    back = io.load_simple(path, n)
    assert "en" not in back and np.allclose(back["ro"], st["ro"], atol=1e-15)
