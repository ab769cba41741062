"""Mesh files next to the path: the Gmsh reader and the ParaView VTU writer of LMT++.

`read_msh` restates `read_msh_2` (include/mesh/read_msh_2.h:56-235) and `write_vtu` the ASCII
`write_mesh_vtk<false>` (include/mesh/write_mesh_vtk.h:434-655); both run in the library's host
code (lmtg_read_msh, lmtg_write_vtu) and need no GPU.  `write_vtu_elasticity` and
`write_vtu_diffusion` write the arrays of LMT++'s elasticity and heat-diffusion meshes.
"""
import ctypes

import numpy as np

from . import abi

ELEM = {"hexa8": abi.ELEM_HEXA8, "tetra10": abi.ELEM_TETRA10, "triangle6": abi.ELEM_TRIANGLE6}
NPE = {abi.ELEM_HEXA8: 8, abi.ELEM_TETRA10: 10, abi.ELEM_TRIANGLE6: 6}
DIM = {abi.ELEM_HEXA8: 3, abi.ELEM_TETRA10: 3, abi.ELEM_TRIANGLE6: 2}
ELEMENT, GLOBAL, INTEGER = 0, 1, 2  # cell-array kinds


def _elem(e):
    return ELEM[e] if isinstance(e, str) else int(e)


def read_msh(path, elem):
    """Nodes (nn x dim), connectivity (ne x npe, LMT++ node order) and the first tag of each
    element, from a Gmsh ASCII format-2 file.  elem: 'hexa8', 'tetra10' or 'triangle6'."""
    et = _elem(elem)
    lib = abi.load()
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    p = str(path).encode()
    abi.check(lib.lmtg_read_msh(p, et, ctypes.byref(nn), None, ctypes.byref(ne), None, None), None, "read_msh")
    pos = np.zeros((nn.value, DIM[et]))
    conn = np.zeros((ne.value, NPE[et]), dtype=np.uint32)
    tag = np.zeros(ne.value)
    abi.check(lib.lmtg_read_msh(p, et, ctypes.byref(nn), abi.ptr(pos), ctypes.byref(ne), abi.ptr(conn),
                                abi.ptr(tag)), None, "read_msh")
    return pos, conn, tag


def write_vtu(path, elem, pos, conn, point_data=(), cell_data=()):
    """ASCII VTU file in LMT++'s layout.  point_data: (name, array nn x c); cell_data:
    (name, array ne x c, kind) with kind ELEMENT (element field), GLOBAL (a global value written
    for every element) or INTEGER (the element group)."""
    et = _elem(elem)
    lib = abi.load()
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, DIM[et])
    conn = np.ascontiguousarray(conn, dtype=np.uint32).reshape(-1, NPE[et])
    nn, ne = pos.shape[0], conn.shape[0]
    keep = []

    def arrays(items, n, with_kind):
        names, comps, kinds, ptrs = [], [], [], []
        for it in items:
            name, a = it[0], np.ascontiguousarray(it[1], dtype=np.float64)
            a = a.reshape(n, -1) if n else a.reshape(0, max(1, a.size))
            keep.append(a)
            names.append(name.encode())
            comps.append(a.shape[1])
            kinds.append(it[2] if with_kind else 0)
            ptrs.append(a.ctypes.data)
        return names, comps, kinds, ptrs

    pn, pc, _, pp = arrays(point_data, nn, False)
    cn, cc, ck, cp = arrays(cell_data, ne, True)

    def carr(ctype, vals):
        return (ctype * max(1, len(vals)))(*vals)

    abi.check(lib.lmtg_write_vtu(str(path).encode(), et, nn, abi.ptr(pos), ne, abi.ptr(conn),
                                 len(pn), carr(ctypes.c_char_p, pn), carr(ctypes.c_int, pc),
                                 carr(ctypes.c_void_p, pp), len(cn), carr(ctypes.c_char_p, cn),
                                 carr(ctypes.c_int, cc), carr(ctypes.c_int, ck), carr(ctypes.c_void_p, cp)),
              None, "write_vtu")


def elasticity_arrays(nn, ne, dep, epsilon=None, sigma=None, tr_epsilon=None, elastic_modulus=1.0,
                      poisson_ratio=0.33, density=7800.0, f_vol=(0.0, 0.0, 0.0), f_nodal=None, f_surf=None,
                      is_on_skin=None, group=None):
    """The arrays of LMT++'s 3D elasticity mesh (the Mesh_carac_pb_elasticity_dep_static fields,
    include/std_formulations/definition_probleme_elasticity_dep_static.h:72-336), in the order its
    writer lists them: point data dep, f_nodal, is_on_skin, f_surf; cell data epsilon, sigma,
    tr_epsilon (element fields, sorted by name), group, then the global fields elastic_modulus,
    density, poisson_ratio, f_vol.  Values not given take the fields' defaults."""
    z3, z6 = np.zeros((nn, 3)), np.zeros((ne, 6))

    def per_elem(v, c):
        v = np.asarray(v, dtype=np.float64)
        return np.broadcast_to(v.reshape(-1, c) if v.size != c else v.reshape(1, c), (ne, c)).copy()

    point = [("dep", np.asarray(dep, dtype=np.float64).reshape(nn, 3)),
             ("f_nodal", z3 if f_nodal is None else f_nodal),
             ("is_on_skin", np.zeros(nn) if is_on_skin is None else is_on_skin),
             ("f_surf", z3 if f_surf is None else f_surf)]
    cell = [("epsilon", z6 if epsilon is None else epsilon, ELEMENT),
            ("sigma", z6 if sigma is None else sigma, ELEMENT),
            ("tr_epsilon", np.zeros(ne) if tr_epsilon is None else tr_epsilon, ELEMENT),
            ("group", np.zeros(ne) if group is None else group, INTEGER),
            ("elastic_modulus", per_elem(elastic_modulus, 1), GLOBAL),
            ("density", per_elem(density, 1), GLOBAL),
            ("poisson_ratio", per_elem(poisson_ratio, 1), GLOBAL),
            ("f_vol", per_elem(f_vol, 3), GLOBAL)]
    return point, cell


def write_vtu_elasticity(path, formulation, fields=True):
    """The displacement of a solved Formulation (point array dep) and, with fields, its element
    fields epsilon, sigma and tr_epsilon at var_inter = 0.5, in LMT++'s elasticity layout."""
    f = formulation
    u = f.get_result().reshape(-1, 3)
    ef = f.element_fields() if fields else {}
    E = np.asarray(f.elastic_modulus, dtype=np.float64)
    point, cell = elasticity_arrays(f.nn, f.ne, u, ef.get("epsilon"), ef.get("sigma"), ef.get("tr_epsilon"),
                                    elastic_modulus=E if E.size == f.ne else float(E.reshape(-1)[0]),
                                    poisson_ratio=float(np.asarray(f.poisson_ratio).reshape(-1)[0]))
    if E.size == f.ne:  # per-element moduli are an element field, listed with the others by name
        cell = [(n, a, ELEMENT if n == "elastic_modulus" else k) for n, a, k in cell]
        elem_f = sorted([c for c in cell if c[2] == ELEMENT], key=lambda c: c[0])
        cell = elem_f + [c for c in cell if c[2] != ELEMENT]
    elem = "hexa8" if f.conn.shape[1] == 8 else "tetra10"
    write_vtu(path, elem, f.pos, f.conn, point, cell)


def write_vtu_diffusion(path, diffusion, group=None):
    """The temperature of a Diffusion run (point array temperature) on its Triangle_6 mesh."""
    d = diffusion
    T = d.get_state()
    cell = [("group", np.zeros(d.conn.shape[0]) if group is None else group, INTEGER)]
    write_vtu(path, "triangle6", d.pos, d.conn, [("temperature", T)], cell)
