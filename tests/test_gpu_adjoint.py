"""Adjoint gradients w.r.t. per-element Young's modulus (GPU) against (1) gradients built from the
reference's own LDL solutions (golden fixtures) and (2) central finite differences."""
import json
import os

import numpy as np
import pytest

from lmtpp_gb300 import Formulation, make_rect_hexa, x1_faces_hexa
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def load_golden(golden_dir, name):
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    d = {k: g[k] for k in g.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def build(pos, conn, E, nu, pen):
    f = Formulation(pos, conn)
    f.elastic_modulus = E
    f.poisson_ratio = nu
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), pen)
    f.add_skin_traction(x1_faces_hexa(pos, conn), (1.0, 0.0, 0.0))
    f.allocate_matrices()
    return f


def ldl_gradient(pos, conn, nu, lam, u):
    """-lambda_e^T Khat_e u_e with the oracle's unit-modulus element matrices."""
    g = np.zeros(conn.shape[0])
    for e in range(conn.shape[0]):
        Kh = O.hexa8_ke(pos[conn[e]], 1.0, nu)
        dofs = (3 * conn[e][:, None].astype(np.int64) + np.arange(3)).ravel()
        g[e] = -lam[dofs] @ Kh @ u[dofs]
    return g


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_adjoint_gradients_match_reference_ldl(golden_dir, mode):
    gd = load_golden(golden_dir, "hexa_10x10x10")
    m = gd["meta"]
    pos, conn = make_rect_hexa(m["nb_points"])
    f = build(pos, conn, m["E"], m["nu"], m["penalty"])
    f.solve(1e-13 if mode == "fp64" else 1e-12, mode=mode)
    J, g, _ = f.adjoint_grad("compliance")
    u = gd["u_ldl"]
    assert J == pytest.approx(float(gd["F"] @ u), rel=1e-10)
    g_ref = ldl_gradient(pos, conn, m["nu"], u, u)
    assert np.linalg.norm(g - g_ref) <= 1e-8 * np.linalg.norm(g_ref)
    Jm, gm, st = f.adjoint_grad("misfit", mode=mode, tol=1e-13 if mode == "fp64" else 1e-12)
    assert Jm == pytest.approx(0.5 * float(u @ u), rel=1e-9)
    gm_ref = ldl_gradient(pos, conn, m["nu"], gd["lam_ldl"], u)
    assert np.linalg.norm(gm - gm_ref) <= 1e-8 * np.linalg.norm(gm_ref), st
    f.close()


def test_tetra10_adjoint_matches_oracle_gradient():
    from lmtpp_gb300 import make_rect_tetra10, x1_faces
    pos, conn = make_rect_tetra10(4)
    rng = np.random.default_rng(11)
    E = rng.uniform(1e5, 3e5, conn.shape[0])
    f = Formulation(pos, conn)
    f.elastic_modulus = E
    f.poisson_ratio = 0.3
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), 1e5)
    f.add_skin_traction(x1_faces(pos, conn), (1.0, 0.0, 0.0))
    f.solve(1e-13, mode="fp64")
    u = f.get_result()
    _, g, _ = f.adjoint_grad("compliance")
    g_ref = np.zeros(conn.shape[0])
    for e in range(conn.shape[0]):
        Kh = O.tetra10_ke(pos[conn[e]], 1.0, 0.3)
        dofs = (3 * conn[e][:, None].astype(np.int64) + np.arange(3)).ravel()
        g_ref[e] = -u[dofs] @ Kh @ u[dofs]
    assert np.linalg.norm(g - g_ref) <= 1e-10 * np.linalg.norm(g_ref)
    f.close()


def test_adjoint_gradients_match_central_differences():
    """Central differences with h = 1e-6 E_e on random elements of a lognormal-E mesh.  J(E +- h)
    is evaluated through u+- = u + delta+-, K(E +- h) delta+- = F - K(E +- h) u, which is exact
    and keeps the tiny difference J+ - J- free of the solver's absolute error."""
    pos, conn = make_rect_hexa(11)
    rng = np.random.default_rng(20251204)
    ne = conn.shape[0]
    E = np.exp(np.log(210000.0) + 0.5 * rng.standard_normal(ne))
    f = build(pos, conn, E, 0.3, 1e5)
    f.solve(1e-14, mode="fp64")
    f.set_penalty_scale(f.get_penalty_scale())  # hold the penalty fixed, as the gradient does
    u = f.get_result()
    F = f.get_sollicitation()
    t = rng.standard_normal(u.shape[0]) * np.abs(u).max()
    w = rng.uniform(0.5, 2.0, u.shape[0])
    Jc, gc, _ = f.adjoint_grad("compliance")
    Jm, gm, _ = f.adjoint_grad("misfit", target=t, weights=w, mode="fp64", tol=1e-14)
    r = w * (u - t)
    for e in rng.choice(ne, 6, replace=False):
        h = 1e-6 * E[e]
        d = {}
        for sgn in (1, -1):
            Ep = E.copy()
            Ep[e] += sgn * h
            f.elastic_modulus = Ep
            f.assemble(True, False)
            f.set_nodal_loads(F - f.spmv(u, 0))
            f.assemble(False, True)
            f.set_result(np.zeros_like(u))
            f.solve_system(1e-13, mode="fp64")
            d[sgn] = f.get_result()
        fd_c = (F @ d[1] - F @ d[-1]) / (2 * h)
        fd_m = ((r @ d[1] + 0.5 * d[1] @ (w * d[1])) - (r @ d[-1] + 0.5 * d[-1] @ (w * d[-1]))) / (2 * h)
        assert fd_c == pytest.approx(gc[e], rel=1e-5), (e, fd_c, gc[e])
        assert fd_m == pytest.approx(gm[e], rel=1e-5), (e, fd_m, gm[e])
    f.close()


def test_autograd_wrapper_matches_adjoint_misfit():
    torch = pytest.importorskip("torch")
    from lmtpp_gb300.autograd import elastic_displacement
    pos, conn = make_rect_hexa(9)
    rng = np.random.default_rng(3)
    E0 = np.exp(np.log(210000.0) + 0.3 * rng.standard_normal(conn.shape[0]))
    f = build(pos, conn, E0, 0.3, 1e5)
    E = torch.tensor(E0, dtype=torch.float64, requires_grad=True)
    u = elastic_displacement(E, f, "fp64", 1e-13)
    t = torch.from_numpy(rng.standard_normal(u.shape[0]) * 1e-6)
    loss = 0.5 * ((u - t) ** 2).sum()
    loss.backward()
    Jm, gm, _ = f.adjoint_grad("misfit", target=t.numpy(), mode="fp64", tol=1e-13)
    assert float(loss.detach()) == pytest.approx(Jm, rel=1e-12)
    assert np.linalg.norm(E.grad.numpy() - gm) <= 1e-9 * np.linalg.norm(gm)
    f.close()
