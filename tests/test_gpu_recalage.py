"""GPU parity of the recalage functional against the reference's own runtime.

Fixtures (tests/golden/make_golden.py): the element Hessian and nodal routine that LMT++'s
Codegen engine writes for formulation recalage, scattered into the reference's Sym SparseLine
with 9 unknowns per node, V clamped on x = 0 by a 1e5 max|diag| penalty, solved by LDL.

Tolerances: assembled matrix 1e-12 relative to its largest entry, right-hand side 1e-14
relative; FP64 PCG solutions 1e-9 relative to the LDL solution, mixed precision 1e-7.  On Tetra10
the reference's order-2 rule leaves the quadratic element's mass matrix rank-deficient, so W is
only defined up to that null space: there U and V are compared and the whole solution through
its residual.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from lmtpp_gb300 import abi
from lmtpp_gb300.recalage import Recalage

pytestmark = pytest.mark.gpu


def load(golden_dir, name):
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    d = {k: g[k] for k in g.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def dense_sym(rowptr, col, val, n):
    L = sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(n, n)).toarray()
    return L, L + np.tril(L, -1).T


def make(g, pen=None):
    m = g["meta"]
    pos = g["pos"]
    f = Recalage(pos, g["conn"])
    f.elastic_modulus, f.poisson_ratio, f.density = m["E"], m["nu"], m["rho"]
    f.gamma, f.r, f.omega = m["gamma"], m["r"], m["omega"]
    f.Ud = g["Ud"].reshape(-1, 3)
    f.Ud_valid = np.ones(pos.shape[0])
    x0 = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints([9 * i + 3 + d for i in x0 for d in range(3)], m["penalty"] if pen is None else pen)
    return f


@pytest.mark.parametrize("name", ["recal_hexa_3", "recal_tetra10_2"])
def test_recalage_system_matches_reference(golden_dir, name):
    g = load(golden_dir, name)
    f = make(g)
    f.assemble()
    n = f.n
    rp, col, val = f.get_mat()
    A, _ = dense_sym(g["rowptr"], g["col"], g["val"], n)
    B, S = dense_sym(rp, col, val, n)
    assert np.abs(A - B).max() <= 1e-12 * np.abs(A).max()
    F = f.get_sollicitation()
    assert np.abs(F - g["F"]).max() <= 1e-14 * np.abs(g["F"]).max()
    for mode, tol, crit in (("fp64", 1e-9, 1e-14), ("mixed", 1e-7, 1e-12)):
        st = f.solve_system(crit, mode=mode)
        assert st["status"] == 0
        x = f.get_vector()
        sc = np.abs(g["u_ldl"]).max()
        d = (x - g["u_ldl"]).reshape(-1, 3, 3)
        assert np.abs(d[:, :2]).max() <= tol * sc, mode
        if g["meta"]["elem"] == "hexa":
            assert np.abs(d).max() <= tol * sc, mode
        assert np.abs(S @ x - g["F"]).max() <= 1e3 * crit * np.abs(g["F"]).max(), mode
        U, V, W = f.get_result()
        assert np.array_equal(np.stack([U, V, W], 1).reshape(-1), x)
    f.close()


def test_recalage_hexa_8_solution_matches_reference(golden_dir):
    g = load(golden_dir, "recal_hexa_8")
    f = make(g)
    st = f.solve(1e-14)
    assert st["status"] == 0
    assert np.abs(f.get_sollicitation() - g["F"]).max() <= 1e-14 * np.abs(g["F"]).max()
    x = f.get_vector()
    assert np.abs(x - g["u_ldl"]).max() <= 1e-9 * np.abs(g["u_ldl"]).max()
    f.close()


def test_recalage_refuses_other_formulations_calls(golden_dir):
    g = load(golden_dir, "recal_hexa_3")
    f = make(g)
    f.assemble()
    lib, ctx = f._lib, f._ctx
    # elasticity assembly, allocation and element fields refuse the 9-unknown context
    assert lib.lmtg_assemble(ctx, abi.ASM_MAT64 | abi.ASM_VEC) == abi.ERR_STATE
    assert lib.lmtg_allocate_matrices(ctx, None) == abi.ERR_STATE
    out = np.zeros((f.ne, 13))
    assert lib.lmtg_element_fields(ctx, None, abi.ptr(out)) == abi.ERR_STATE
    # a second setup on the same mesh is refused; mesh_set resets the context
    Ud = np.zeros(3 * f.nn)
    Uv = np.ones(f.nn)
    assert lib.lmtg_recalage_setup(ctx, 1.0, 1.0, 0.5, 0.5, abi.ptr(Ud), abi.ptr(Uv)) == abi.ERR_STATE
    # the wrapper sets the mesh again when a variable changes
    f.gamma = 0.7
    f.assemble()
    st = f.solve_system(1e-12)
    assert st["status"] == 0
    f.close()


def test_recalage_argument_checks(golden_dir):
    g = load(golden_dir, "recal_hexa_3")
    f = Recalage(g["pos"], g["conn"])
    f.elastic_modulus = np.full(f.ne, 2.0)  # one modulus per element: the formulation's E is global
    with pytest.raises(abi.LmtgError):
        f.assemble()
    f.elastic_modulus = 2.0
    f.r = 1.0
    with pytest.raises(abi.LmtgError):
        f.assemble()
    f.r = 0.5
    f.Ud_valid = np.ones(3)
    with pytest.raises(abi.LmtgError):
        f.assemble()
    f.close()
