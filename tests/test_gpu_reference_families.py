"""GPU parity against fixtures the reference's own code produced, one per workload family.

The fixtures (tests/golden/make_golden.py) come from LMT++'s runtime around the element routines
that LMT++'s Codegen engine writes for elasticity_iso and difftherm: single distorted elements,
the Hexa8 family with lognormal moduli (16^3), the Tetra10 family (10^3 cubes), the transient
Triangle_6 family (2 x 32^2, Crank-Nicolson and implicit Euler, 10 steps) and the batch family
(three cubes x four load cases), each solved by LMT++'s LDL.

Tolerances: element and assembled matrices 1e-12 relative to their largest entry; loads 1e-13
(single faces) and 1e-14 (assembled, relative to the largest entry);
FP64 solutions 1e-10 and mixed-precision solutions 1e-8 relative to the LDL solution.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from lmtpp_gb300 import Formulation, make_rect_hexa, make_rect_tetra10, x1_faces
from lmtpp_gb300.batch import BatchFormulation
from lmtpp_gb300.diffusion import Diffusion, boundary_nodes, make_rect_triangle6

pytestmark = pytest.mark.gpu

HEXA_FACES = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [3, 7, 6, 2], [0, 4, 7, 3], [1, 2, 6, 5]]
TET_FACES = [[0, 2, 1, 6, 5, 4], [0, 1, 3, 4, 8, 7], [0, 3, 2, 7, 9, 6], [1, 2, 3, 5, 9, 8]]


def load(golden_dir, name):
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    d = {k: g[k] for k in g.files}
    if "meta" in d:
        d["meta"] = json.loads(str(d["meta"]))
    return d


def csr(rowptr, col, val, n):
    return sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(n, n))


def assert_same_lower(rowptr, col, val, g_rowptr, g_col, g_val, n):
    """Assembled lower CSR against the reference's: entries within 1e-12 max|K|; entries the
    reference erased (summed to exactly 0.0 in its floating-point order) are round-off here."""
    A = csr(g_rowptr, g_col, g_val, n)
    B = csr(rowptr, col, val, n)
    kmax = abs(A).max()
    As, Bs = A.copy(), B.copy()
    As.data[:] = 1.0
    Bs.data[:] = 1.0
    extra = As - As.multiply(Bs)
    assert extra.count_nonzero() == 0  # nothing outside the structural pattern
    miss = Bs - As
    miss.eliminate_zeros()
    mi = miss.nonzero()
    assert np.all(np.abs(np.asarray(B[mi]).ravel()) <= 1e-12 * kmax)
    assert abs(A - B).max() <= 1e-12 * kmax


@pytest.mark.parametrize("typ", ["hexa", "tetra10", "tetra10s"])
def test_element_kernel_matches_generated_code(golden_dir, typ):
    """k_elast (FP64 and FP32) and the skin loads against the reference-generated routines on one
    distorted element."""
    g = load(golden_dir, "elem_kernels")
    xyz = g[typ + "_xyz"]
    E, nu = g[typ + "_E_nu"]
    npe = xyz.shape[0]
    conn = np.arange(npe, dtype=np.uint32)[None, :]
    f = Formulation(xyz, conn)
    f.elastic_modulus = E
    f.poisson_ratio = nu
    f.allocate_matrices()
    f.assemble(True, False)
    Ke = f.element_matrices(0, 1)[0]
    Kg = g[typ + "_Ke"]
    up = np.triu(np.ones_like(Kg, dtype=bool))
    kmax = np.abs(Kg).max()
    assert np.abs(Ke[up] - Kg[up]).max() <= 1e-12 * kmax
    assert np.abs(Ke - Ke.T).max() <= 1e-12 * kmax
    f.assemble(True, False, native_fp32=True)
    K32 = f.element_matrices(0, 1, precision=1)[0]
    assert np.abs(K32[up] - Kg[up]).max() <= 2e-6 * kmax
    t, p = g["skin_traction"], float(g["skin_pressure"])
    faces = HEXA_FACES if typ == "hexa" else TET_FACES
    for k, q in enumerate(faces):
        if typ == "tetra10" and k in (1, 2):
            continue  # element_Tetra_10.py:18-19 mirror these children's map on curved faces
        f.set_nodal_loads(np.zeros(3 * npe))
        fa = np.array([q], dtype=np.uint32)
        f.add_skin_traction(fa, t)
        f.add_skin_pressure(fa, p)
        f.assemble(False, True)
        Fg = g[typ + "_skin"][k]
        assert np.abs(f.get_sollicitation() - Fg).max() <= 1e-13 * np.abs(Fg).max(), (typ, k)
    f.close()


@pytest.mark.parametrize("scheme,theta", [("cn", 0.5), ("ie", 1.0)])
def test_diffusion_element_matches_generated_code(golden_dir, scheme, theta):
    """k_tri6_diff's A = M/dt + theta K and B = M/dt - (1 - theta) K on one distorted Triangle_6
    against the reference-generated difftherm routine (Crank-Nicolson: left 0, right 1; implicit
    Euler: the residual at the end of the step)."""
    g = load(golden_dir, "elem_kernels")
    k, rho_c, dt = g["tri6_k_rhoc_dt"]
    d = Diffusion(g["tri6_xy"], np.arange(6, dtype=np.uint32)[None, :])
    d.setup(k, rho_c=rho_c, dt=dt, theta=theta, dirichlet=None, penalty=0.0)
    rowptr, col, A, B = d.get_matrices()
    Ad = csr(rowptr, col, A, 6).toarray()
    Bd = csr(rowptr, col, B, 6).toarray()
    Ag, Bg = g["tri6_A_" + scheme], g["tri6_B_" + scheme]
    low = np.tril(np.ones((6, 6), dtype=bool))
    assert np.abs(Ad[low] - Ag.T[low]).max() <= 1e-12 * np.abs(Ag).max()
    assert np.abs(Bd[low] - Bg[low]).max() <= 1e-12 * np.abs(Bg).max()
    d.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_hexa_lognormal_family_matches_reference_ldl(golden_dir, mode, tol):
    """The Hexa8 benchmark family at 16^3 (lognormal per-element E): the solution of the same
    solver the benchmark uses as its FP64 oracle (PCG to a 1e-14 relative residual) and of the
    mixed solver against LMT++'s LDL; the skin loads against the generated skin routine."""
    g = load(golden_dir, "hexa_16_lognormal")
    m = g["meta"]
    pos, conn = make_rect_hexa(m["nb_points"])
    E = np.exp(m["E_logmean"] + m["E_logstd"] * np.random.default_rng(m["seed"]).standard_normal(conn.shape[0]))
    f = Formulation(pos, conn)
    f.elastic_modulus = E
    f.poisson_ratio = m["nu"]
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), m["penalty"])
    f.add_skin_traction(x1_faces(pos, conn), (1.0, 0.0, 0.0))
    st = f.solve(1e-14 if mode == "fp64" else 1e-12, mode=mode)
    assert f.get_penalty_scale() == pytest.approx(m["max_diag"], rel=1e-13)
    np.testing.assert_allclose(f.get_sollicitation(), g["F"], rtol=0, atol=1e-14 * np.abs(g["F"]).max())
    u, ref = f.get_result(), g["u_ldl"]
    rel = np.linalg.norm(u - ref) / np.linalg.norm(ref)
    assert rel <= tol, (rel, st)
    if mode == "fp64":
        # adjoint of the misfit 1/2 |u|^2: lambda = K^-1 u; the gradient against the one built from
        # the reference's own u and lambda with the reference-pinned element matrices
        J, dJ, _ = f.adjoint_grad("misfit", target=None, mode="fp64", tol=1e-14)
        assert J == pytest.approx(0.5 * float(ref @ ref), rel=1e-9)
        lam = g["lam_ldl"]
        Ke = f.element_matrices(0, conn.shape[0])
        idx = (3 * conn[:, :, None] + np.arange(3)).reshape(conn.shape[0], -1)
        ref_grad = -np.einsum("ei,eij,ej->e", lam[idx], Ke, ref[idx]) / E
        assert np.linalg.norm(dJ - ref_grad) <= 1e-8 * np.linalg.norm(ref_grad)
    f.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_tetra10_family_matches_reference_ldl(golden_dir, mode, tol):
    """The Tetra10 benchmark family at 10^3 cubes x 6 tetrahedra against LMT++'s LDL."""
    g = load(golden_dir, "tetra10_10x10x10")
    m = g["meta"]
    pos, conn = make_rect_tetra10(m["nb_points"])
    f = Formulation(pos, conn)
    f.elastic_modulus = m["E"]
    f.poisson_ratio = m["nu"]
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), m["penalty"])
    f.add_skin_traction(x1_faces(pos, conn), (1.0, 0.0, 0.0))
    st = f.solve(1e-14 if mode == "fp64" else 1e-12, mode=mode)
    np.testing.assert_allclose(f.get_sollicitation(), g["F"], rtol=0, atol=1e-14 * np.abs(g["F"]).max())
    u, ref = f.get_result(), g["u_ldl"]
    rel = np.linalg.norm(u - ref) / np.linalg.norm(ref)
    assert rel <= tol, (rel, st)
    f.close()


@pytest.mark.parametrize("name", ["tri6_32_cn", "tri6_32_ie"])
@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_transient_family_matches_reference_ldl(golden_dir, name, mode, tol):
    """The transient family at 2 x 32^2 (lognormal conductivity, penalty boundary, dt 1e-4):
    A and B against the reference's assembly, and 10 steps against 10 LDL steps."""
    g = load(golden_dir, name)
    m = g["meta"]
    pos, conn = make_rect_triangle6(m["nb_points"])
    assert np.array_equal(pos, g["pos"]) and np.array_equal(conn, g["conn"])
    k = np.exp(m["k_logstd"] * np.random.default_rng(m["seed"]).standard_normal(conn.shape[0]))
    d = Diffusion(pos, conn)
    d.setup(k, rho_c=m["rho_c"], dt=m["dt"], theta=m["theta"], dirichlet=boundary_nodes(pos), penalty=m["penalty"])
    assert d.get_penalty_scale() == pytest.approx(m["max_diag"], rel=1e-13)
    rowptr, col, A, B = d.get_matrices()
    nn = pos.shape[0]
    assert_same_lower(rowptr, col, A, g["rowptr"], g["col"], g["A"], nn)
    assert_same_lower(rowptr, col, B, g["rowptrB"], g["colB"], g["B"], nn)
    d.set_solver(mode)
    states = g["states"]
    kept = list(g["steps_kept"])
    d.set_state(states[0])
    done = 0
    for s, ref in zip(kept[1:], states[1:]):
        d.run(s - done, tol=1e-14 if mode == "fp64" else 1e-12)
        done = s
        T = d.get_state()
        rel = np.linalg.norm(T - ref) / np.linalg.norm(ref)
        assert rel <= tol, (s, rel)
    d.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_batch_family_matches_reference_ldl(golden_dir, mode, tol):
    """Three cubes of different sides, moduli and Poisson ratios, four load cases each, solved in
    one batch against LMT++'s LDL per cube and case; the traction cases' loads against the
    reference's generated skin routines."""
    g = load(golden_dir, "batch_cubes")
    sides = [int(s) for s in g["sides"]]
    meshes = [make_rect_hexa(s + 1) for s in sides]
    bf = BatchFormulation(meshes)
    bf.set_materials(g["E"], g["nu"])
    clamped = np.nonzero(bf.pos[:, 0] < 1e-6)[0]
    bf.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), g["meta"]["penalty"])
    bf.assemble(True, False, mixed=True)
    B = np.zeros((4, bf.n))
    for m in range(len(sides)):
        B[:, bf.dofs(m)] = g["F%d" % m]
    faces = x1_faces(bf.pos, bf.conn)
    for r in range(3):
        bf.set_nodal_loads(np.zeros(bf.n))
        t = np.zeros(3)
        t[r] = 1.0
        bf.add_skin_traction(faces, t)
        bf.assemble(False, True)
        assert np.abs(bf.get_sollicitation() - B[r]).max() <= 1e-14 * np.abs(B[r]).max()
    X, st, its = bf.solve_batch(B, mode=mode, tol=1e-13 if mode == "fp64" else 1e-12)
    for m in range(len(sides)):
        U = g["u%d" % m]
        for r in range(4):
            ref = U[r]
            rel = np.linalg.norm(X[r, bf.dofs(m)] - ref) / np.linalg.norm(ref)
            assert rel <= tol, (m, r, rel)
    bf.close()
