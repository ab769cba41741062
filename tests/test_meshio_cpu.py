"""Mesh files (host code, no GPU): the Gmsh reader and the VTU writer against the reference's own
read_msh_2 and write_mesh_vtk<false> outputs (tests/golden/make_meshio_golden.py)."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from lmtpp_gb300 import abi, make_rect_hexa, make_rect_tetra10, meshio
from lmtpp_gb300.diffusion import make_rect_triangle6

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ELEM = {"hexa": "hexa8", "tetra10": "tetra10", "tri6": "triangle6"}


@pytest.mark.parametrize("name", ["hexa", "tetra10", "tri6"])
def test_read_msh_matches_reference(name):
    """Shuffled node numbers, skipped faces / edges / points, elements listed with the opposite
    orientation: nodes and connectivity bit-exact to LMT++'s read_msh_2."""
    g = np.load(os.path.join(GOLD, "msh_%s.npz" % name))
    pos, conn, tag = meshio.read_msh(os.path.join(GOLD, "msh_%s.msh" % name), ELEM[name])
    assert pos.dtype == np.float64 and np.array_equal(pos, g["pos"])
    assert np.array_equal(conn, g["conn"])
    assert np.array_equal(tag, np.arange(conn.shape[0]) % 3 + 1.0)  # the first of the two tags


def _gold(name):
    with open(os.path.join(GOLD, name)) as f:
        return f.read()


def test_write_vtu_matches_reference_elasticity_mesh(tmp_path):
    """The arrays of LMT++'s elasticity mesh with seeded values: byte-identical file."""
    g = np.load(os.path.join(GOLD, "vtu_elast_fields.npz"))
    pos, conn = make_rect_hexa(3)
    ef = g["fields"]
    point, cell = meshio.elasticity_arrays(pos.shape[0], conn.shape[0], g["dep"], ef[:, :6], ef[:, 6:12],
                                           ef[:, 12], elastic_modulus=float(g["E"]), poisson_ratio=float(g["nu"]))
    out = tmp_path / "e.vtu"
    meshio.write_vtu(out, "hexa8", pos, conn, point, cell)
    assert out.read_text() == _gold("vtu_elast_hexa.vtu")


@pytest.mark.parametrize("elem,mesh,gold", [("tetra10", lambda: make_rect_tetra10(3), "vtu_std_tetra10.vtu"),
                                            ("triangle6", lambda: make_rect_triangle6(4), "vtu_std_tri6.vtu")])
def test_write_vtu_matches_reference_cells(tmp_path, elem, mesh, gold):
    pos, conn = mesh()
    out = tmp_path / "m.vtu"
    meshio.write_vtu(out, elem, pos, conn, [], [("group", np.zeros(conn.shape[0]), meshio.INTEGER)])
    assert out.read_text() == _gold(gold)


def test_write_vtu_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    pos, conn = make_rect_tetra10(3)
    T = rng.standard_normal(pos.shape[0])
    s = rng.standard_normal((conn.shape[0], 6))
    out = tmp_path / "r.vtu"
    meshio.write_vtu(out, "tetra10", pos, conn, [("T", T)], [("s", s, meshio.ELEMENT)])
    piece = ET.parse(out).getroot().find("UnstructuredGrid/Piece")
    arr = {a.get("Name"): a.text for a in piece.iter("DataArray")}
    assert np.allclose(np.array(arr["T"].split(), dtype=float), T, rtol=1e-5, atol=1e-6)
    assert np.allclose(np.array(arr["s"].split(), dtype=float).reshape(-1, 6), s, rtol=1e-5, atol=1e-6)
    assert np.array_equal(np.array(arr["connectivity"].split(), dtype=np.uint32).reshape(-1, 10), conn)
    assert np.array_equal(np.array(arr["types"].split(), dtype=int), np.full(conn.shape[0], 24))
    pts = piece.find("Points/DataArray").text.split()
    assert np.allclose(np.array(pts, dtype=float).reshape(-1, 3), pos, atol=1e-6)


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)


def test_read_msh_errors(tmp_path):
    with pytest.raises(abi.LmtgError) as e:
        meshio.read_msh(tmp_path / "missing.msh", "hexa8")
    assert e.value.status == abi.ERR_ARG
    head = "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n4\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n$EndNodes\n"
    _write(tmp_path / "unknown.msh", head + "$Elements\n1\n1 4 0 1 2 3 9\n$EndElements\n")
    with pytest.raises(abi.LmtgError) as e:  # a volume element (linear tetra) of another type
        meshio.read_msh(tmp_path / "unknown.msh", "tetra10")
    assert e.value.status == abi.ERR_UNSUPPORTED
    _write(tmp_path / "badnode.msh", head + "$Elements\n1\n1 9 0 1 2 3 4 1 99\n$EndElements\n")
    with pytest.raises(abi.LmtgError) as e:  # a Triangle_6 naming a node the file does not list
        meshio.read_msh(tmp_path / "badnode.msh", "triangle6")
    assert e.value.status == abi.ERR_ARG
    _write(tmp_path / "trunc.msh", head + "$Elements\n1\n")
    with pytest.raises(abi.LmtgError) as e:
        meshio.read_msh(tmp_path / "trunc.msh", "hexa8")
    assert e.value.status == abi.ERR_ARG
    # faces only: a valid file with no volume elements
    _write(tmp_path / "faces.msh", head + "$Elements\n1\n1 2 0 1 2 3\n$EndElements\n")
    pos, conn, tag = meshio.read_msh(tmp_path / "faces.msh", "hexa8")
    assert pos.shape == (4, 3) and conn.shape == (0, 8)


REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "ref_meshio")


@pytest.mark.skipif(not os.path.exists(REF), reason="the reference's mesh-file driver is built only where its sources are")
@pytest.mark.parametrize("elem,nb", [("hexa", 17), ("tetra10", 9), ("tri6", 33)])
def test_reader_and_writer_against_the_reference_at_size(tmp_path, elem, nb):
    """A larger generated file and mesh than the fixtures, run through the reference's own code."""
    import subprocess
    import sys
    sys.path.insert(0, GOLD)
    import make_meshio_golden as G
    from lmtpp_gb300 import make_rect_hexa, make_rect_tetra10
    pos, conn = {"hexa": make_rect_hexa, "tetra10": make_rect_tetra10, "tri6": make_rect_triangle6}[elem](nb)
    msh = tmp_path / "m.msh"
    G.write_msh(str(msh), elem, pos, conn, np.random.default_rng(nb))
    subprocess.run([REF, "msh", elem, str(msh), str(tmp_path)], check=True)
    npe, dim = conn.shape[1], pos.shape[1]
    rpos = np.fromfile(tmp_path / "pos.f64").reshape(-1, dim)
    rconn = np.fromfile(tmp_path / "conn.u32", dtype=np.uint32).reshape(-1, npe)
    p2, c2, _ = meshio.read_msh(msh, ELEM[elem])
    assert np.array_equal(p2, rpos) and np.array_equal(c2, rconn)
    subprocess.run([REF, "vtu_std", elem, str(nb), str(tmp_path / "r.vtu")], check=True)
    meshio.write_vtu(tmp_path / "o.vtu", ELEM[elem], pos, conn, [], [("group", np.zeros(conn.shape[0]), meshio.INTEGER)])
    assert (tmp_path / "o.vtu").read_text() == (tmp_path / "r.vtu").read_text()


def test_read_msh_crlf_and_blank_runs(tmp_path):
    """Windows line ends and runs of blanks parse as the stream extraction of the reference does."""
    src = open(os.path.join(GOLD, "msh_tetra10.msh")).read()
    crlf = tmp_path / "crlf.msh"
    with open(crlf, "w", newline="") as f:
        f.write(src.replace("\n", "\r\n").replace(" ", " \t "))
    g = np.load(os.path.join(GOLD, "msh_tetra10.npz"))
    pos, conn, _ = meshio.read_msh(crlf, "tetra10")
    assert np.array_equal(pos, g["pos"]) and np.array_equal(conn, g["conn"])


def test_write_vtu_empty_mesh_and_bad_arguments(tmp_path):
    out = tmp_path / "empty.vtu"
    meshio.write_vtu(out, "hexa8", np.zeros((0, 3)), np.zeros((0, 8), dtype=np.uint32),
                     [("dep", np.zeros((0, 3)))], [("group", np.zeros(0), meshio.INTEGER)])
    text = out.read_text()
    assert "NumberOfPoints='0' NumberOfCells='0'" in text and "Name='dep'" not in text  # as the reference
    ET.parse(out)
    pos, conn = make_rect_hexa(2)
    with pytest.raises(abi.LmtgError) as e:  # a node index past the points
        meshio.write_vtu(tmp_path / "bad.vtu", "hexa8", pos, conn + 100)
    assert e.value.status == abi.ERR_ARG
    with pytest.raises(abi.LmtgError) as e:
        meshio.write_vtu(tmp_path / "no_dir" / "x.vtu", "hexa8", pos, conn)
    assert e.value.status == abi.ERR_ARG


@pytest.mark.skipif(not os.path.exists(REF), reason="the reference's mesh-file driver is built only where its sources are")
@pytest.mark.parametrize("ntags", [0, 1, 3])
@pytest.mark.parametrize("seed", [1, 2])
def test_reader_against_the_reference_tags_and_seeds(tmp_path, ntags, seed):
    import subprocess
    import sys
    sys.path.insert(0, GOLD)
    import make_meshio_golden as G
    for elem, mesh in (("hexa", lambda: make_rect_hexa(4)), ("tetra10", lambda: make_rect_tetra10(3)),
                       ("tri6", lambda: make_rect_triangle6(5))):
        pos, conn = mesh()
        msh = tmp_path / ("%s.msh" % elem)
        G.write_msh(str(msh), elem, pos, conn, np.random.default_rng(seed), ntags=ntags)
        subprocess.run([REF, "msh", elem, str(msh), str(tmp_path)], check=True)
        rpos = np.fromfile(tmp_path / "pos.f64").reshape(-1, pos.shape[1])
        rconn = np.fromfile(tmp_path / "conn.u32", dtype=np.uint32).reshape(-1, conn.shape[1])
        p2, c2, tag = meshio.read_msh(msh, ELEM[elem])
        assert np.array_equal(p2, rpos) and np.array_equal(c2, rconn), (elem, ntags, seed)
        want = np.arange(conn.shape[0]) % 3 + 1.0 if ntags else np.zeros(conn.shape[0])
        assert np.array_equal(tag, want)
