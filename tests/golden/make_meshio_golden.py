"""Generates the mesh-file fixtures of tests/golden from the reference's own reader and writer.

Writes Gmsh ASCII format-2 files (msh_*.msh) from make_rect meshes of this package: node
numbers shuffled and non-contiguous, nodes listed out of order, faces / edges / points mixed in
(the reader skips them), some elements listed with the opposite orientation (the reader
re-orders them) and two tags per element.  Each file is then read by LMT++'s read_msh_2
(oracle/_ref/ref_meshio msh ...), and its nodes and connectivity are stored in msh_*.npz.

For the VTU writer it stores the reference's write_mesh_vtk<false> output (vtu_*.vtu) for the
Hexa unit cube of the generated elasticity mesh carac with seeded fields (vtu_elast_fields.npz;
oracle/_ref/ref_vtu_elast),
and for Tetra_10 / Triangle_6 meshes without fields.

Usage: python tests/golden/make_meshio_golden.py   (needs oracle/_ref/ref_meshio and ref_vtu_elast, built by
oracle/build_ref.sh from the LMTpp sources; run in the build container, the fixtures are
committed).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lmtpp_gb300 import make_rect_hexa, make_rect_tetra10  # noqa: E402
from lmtpp_gb300.diffusion import make_rect_triangle6  # noqa: E402

DRV = os.path.join(ROOT, "oracle", "_ref", "ref_meshio")
DRV_ELAST = os.path.join(ROOT, "oracle", "_ref", "ref_vtu_elast")

# Gmsh element types and the node orders used to write an element with the opposite
# orientation (a reflection of the reference element, in the file's node order)
GMSH = {"hexa": 5, "tetra10": 11, "tri6": 9}
FLIP = {"hexa": [0, 3, 2, 1, 4, 7, 6, 5],
        "tetra10": [0, 2, 1, 3, 6, 5, 4, 7, 9, 8],  # vertices 1 <-> 2 (file order: 8 = (3,2), 9 = (3,1))
        "tri6": [0, 2, 1, 5, 4, 3]}


def mesh(elem):
    if elem == "hexa":
        return make_rect_hexa(4)
    if elem == "tetra10":
        return make_rect_tetra10(3)
    return make_rect_triangle6(4)


def to_file_order(elem, conn):
    """LMT++ node order -> Gmsh's (Tetra_10: the last two edge nodes swapped)."""
    c = conn.copy()
    if elem == "tetra10":
        c[:, [8, 9]] = c[:, [9, 8]]
    return c


def write_msh(path, elem, pos, conn, rng, ntags=2):
    nn = pos.shape[0]
    numbers = rng.permutation(np.arange(1, 3 * nn + 1))[:nn] + 100  # unique, non-contiguous
    order = rng.permutation(nn)
    fc = to_file_order(elem, conn)
    flip = rng.random(conn.shape[0]) < 0.3
    fc[flip] = fc[flip][:, FLIP[elem]]
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(nn)]
    for i in order:
        xyz = list(pos[i]) + [0.0] * (3 - pos.shape[1])
        lines.append("%d %s" % (numbers[i], " ".join(repr(float(v)) for v in xyz)))
    lines += ["$EndNodes", "$Elements"]
    els = []
    k = 1
    for e in range(conn.shape[0]):
        if e % 5 == 0:  # a lower-dimension element before it: a point, an edge or a face
            if elem == "tri6":
                els.append("%d 8 2 7 1 %d %d %d" % (k, numbers[conn[e, 0]], numbers[conn[e, 1]], numbers[conn[e, 3]]))
            elif elem == "hexa":
                els.append("%d 3 2 7 1 %s" % (k, " ".join(str(numbers[j]) for j in conn[e, [0, 1, 2, 3]])))
            else:
                els.append("%d 15 2 7 1 %d" % (k, numbers[conn[e, 0]]))
            k += 1
        tags = [e % 3 + 1, 10 + e, 7][:ntags]
        els.append("%d %d %d %s%s" % (k, GMSH[elem], ntags, "".join("%d " % t for t in tags),
                                      " ".join(str(numbers[j]) for j in fc[e])))
        k += 1
    lines += [str(len(els))] + els + ["$EndElements", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def run(args, drv=DRV):
    subprocess.run([drv] + args, check=True)


def main():
    if not os.path.exists(DRV):
        sys.exit("build oracle/_ref first (sh oracle/build_ref.sh)")
    rng = np.random.default_rng(20251203)
    for elem in ("hexa", "tetra10", "tri6"):
        pos, conn = mesh(elem)
        msh = os.path.join(HERE, "msh_%s.msh" % elem)
        write_msh(msh, elem, pos, conn, rng)
        with tempfile.TemporaryDirectory() as d:
            run(["msh", elem, msh, d])
            nn, ne = map(int, open(os.path.join(d, "info.txt")).read().split())
            dim = 2 if elem == "tri6" else 3
            npe = {"hexa": 8, "tetra10": 10, "tri6": 6}[elem]
            rpos = np.fromfile(os.path.join(d, "pos.f64")).reshape(nn, dim)
            rconn = np.fromfile(os.path.join(d, "conn.u32"), dtype=np.uint32).reshape(ne, npe)
        np.savez_compressed(os.path.join(HERE, "msh_%s.npz" % elem), pos=rpos, conn=rconn)
        print(elem, "msh:", nn, "nodes", ne, "elements")
    # VTU: the Hexa elasticity carac with seeded fields
    pos, conn = make_rect_hexa(3)
    nn, ne = pos.shape[0], conn.shape[0]
    dep = rng.standard_normal((nn, 3)) * 1e-3
    ef = rng.standard_normal((ne, 13)) * np.array([1e-4] * 6 + [1e2] * 6 + [1e-4])
    E, nu = 210000.0, 0.3
    np.savez_compressed(os.path.join(HERE, "vtu_elast_fields.npz"), dep=dep, fields=ef, E=E, nu=nu)
    with tempfile.TemporaryDirectory() as d:
        fin = os.path.join(d, "fields.f64")
        np.concatenate([dep.ravel(), ef.ravel(), [E, nu]]).astype(np.float64).tofile(fin)
        run(["3", fin, os.path.join(HERE, "vtu_elast_hexa.vtu")], DRV_ELAST)
    run(["vtu_std", "tetra10", "3", os.path.join(HERE, "vtu_std_tetra10.vtu")])
    run(["vtu_std", "tri6", "4", os.path.join(HERE, "vtu_std_tri6.vtu")])
    print("vtu fixtures written")


if __name__ == "__main__":
    main()
