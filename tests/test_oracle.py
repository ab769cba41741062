"""The oracle pinned against the reference's own outputs (CPU only).

Golden fixtures come from LMT++'s own code (tests/golden/make_golden.py): the element routines its
Codegen engine writes for elasticity_iso and difftherm, its Gauss tables, make_rect, the Sym
SparseLine storage with erase-on-exact-zero, max|diag| penalty, LDL and IC(0)-PCG.  The CG known
answers come from the reference's unit tests (conjugate_gradient_test.cpp:15-71).
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O


def err_unit_test(a, b):
    """ERROR_UNIT_TEST of include/util/unit_test.h:17."""
    return np.abs(a - b) / (1e-20 + np.abs(a) + np.abs(b))


def load_golden(golden_dir, name):
    g = np.load(os.path.join(golden_dir, name + ".npz"))
    d = {k: g[k] for k in g.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def csr(rowptr, col, val, n):
    return sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(n, n))


@pytest.mark.parametrize("name", ["hexa_2x2x2", "hexa_10x10x10", "tetra10_3x3x3"])
def test_oracle_matches_reference_runtime(golden_dir, name):
    g = load_golden(golden_dir, name)
    m = g["meta"]
    P = O.elasticity_problem(m["nb_points"], E=m["E"], nu=m["nu"], pen=m["penalty"], elem=m["elem"])
    n = P["F"].shape[0]
    # mesh and connectivity: bit-exact (make_rect node order, accumulated coordinates)
    assert np.array_equal(P["pos"], g["pos"])
    assert np.array_equal(P["conn"], g["conn"])
    # pattern: the reference's is the structural lower pattern minus entries that summed to
    # exactly 0.0 (vecsparse.h:15-40); the oracle keeps the structural pattern.  Which sums are
    # exactly zero depends on the generated code's floating-point order: where the reference
    # erased an entry, the oracle's value is round-off
    A = csr(g["rowptr"], g["col"], g["val"], n)
    B = csr(P["rowptr"], P["col"], P["val"], n)
    Bs, As = B.copy(), A.copy()
    Bs.data[:] = 1.0
    As.data[:] = 1.0
    extra_in_ref = As - As.multiply(Bs)
    assert extra_in_ref.count_nonzero() == 0
    missing = (Bs - As.multiply(Bs))
    missing.eliminate_zeros()
    mi = missing.nonzero()
    kmax = abs(B).max()
    assert np.all(np.abs(B[mi]) <= 1e-12 * kmax)
    # values: the generated integrand and the restatement agree to round-off
    d = abs(A - B)
    assert d.max() <= 1e-12 * kmax
    assert P["max_diag"] == pytest.approx(m["max_diag"], rel=1e-13)
    np.testing.assert_allclose(P["F"], g["F"], rtol=0, atol=1e-15 * max(1.0, np.abs(g["F"]).max()))
    # direct solve: skyline Cholesky vs the reference's LDL
    x = O.skyline_solve(P["rowptr"], P["col"], P["val"], P["F"])
    assert np.linalg.norm(x - g["u_ldl"]) <= 1e-12 * np.linalg.norm(g["u_ldl"])
    # IC(0)-PCG restatement vs the reference's solve_using_incomplete_chol_factorize, on the
    # reference's own matrix (its IC(0) pattern is the value-dependent stored pattern)
    rp, cl, vl = g["rowptr"], g["col"], g["val"]
    fac = O.ic0(rp, cl, vl)
    xi, it = O.ic_pcg(rp, cl, vl, fac, g["F"], 1e-10 * np.abs(g["F"]).max())
    assert it == m["icpcg_iter"]
    assert np.linalg.norm(xi - g["u_icpcg"]) <= 1e-10 * np.linalg.norm(g["u_icpcg"])


def test_oracle_element_routines_match_generated_code(golden_dir):
    """The restated integrands against the element routines that the reference's own Codegen
    engine writes (oracle/ref_codegen.cpp): distorted Hexa8 and Tetra10 (nu != 0.3) summed over the
    reference's Gauss tables, their skin loads on every face, and the Triangle_6 difftherm
    matrices of Crank-Nicolson and implicit Euler."""
    g = np.load(os.path.join(golden_dir, "elem_kernels.npz"))
    t = g["skin_traction"]
    p = float(g["skin_pressure"])
    hexa_faces = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [3, 7, 6, 2], [0, 4, 7, 3], [1, 2, 6, 5]]
    tet_faces = [[0, 2, 1, 6, 5, 4], [0, 1, 3, 4, 8, 7], [0, 3, 2, 7, 9, 6], [1, 2, 3, 5, 9, 8]]
    for typ, ke, faces in (("hexa", O.hexa8_ke, hexa_faces), ("tetra10", O.tetra10_ke, tet_faces),
                           ("tetra10s", O.tetra10_ke, tet_faces)):
        xyz = g[typ + "_xyz"]
        E, nu = g[typ + "_E_nu"]
        Kg = g[typ + "_Ke"]  # upper triangle as the generated code writes it (j >= i)
        Ko = ke(xyz, E, nu)
        up = np.triu(np.ones_like(Kg, dtype=bool))
        assert np.abs(Ko[up] - Kg[up]).max() <= 1e-12 * np.abs(Kg).max()
        assert np.all(Kg[~up] == 0.0)
        for f, q in enumerate(faces):
            if typ == "tetra10" and f in (1, 2):
                # element_Tetra_10.py:18-19 give children 1 and 2 a `var` map that mirrors their
                # node lists, so on a curved face the reference evaluates the test functions at
                # the mirrored point; on straight-edged faces (tetra10s) both integrate alike
                continue
            F = np.zeros(xyz.size)
            q = np.array(q, dtype=np.uint32)[None, :]
            (O.quad4_traction if typ == "hexa" else O.tri6_traction)(q, xyz, t, F)
            F += O.pressure_loads(q, xyz, p)
            Fg = g[typ + "_skin"][f]
            assert np.abs(F - Fg).max() <= 1e-13 * np.abs(Fg).max(), (typ, f)
    k, rho_c, dt = g["tri6_k_rhoc_dt"]
    Kd, Md = O.triangle6_km(g["tri6_xy"], k / rho_c)
    up = np.triu(np.ones((6, 6), dtype=bool))
    for theta, suf in ((0.5, "cn"), (1.0, "ie")):
        A = Md / dt + theta * Kd
        B = Md / dt - (1 - theta) * Kd
        Ag, Bg = g["tri6_A_" + suf], g["tri6_B_" + suf]
        assert np.abs(A[up] - Ag[up]).max() <= 1e-12 * np.abs(Ag).max()
        assert np.abs(B - Bg).max() <= 1e-12 * np.abs(Bg).max()


@pytest.mark.parametrize("case", ["cg0", "cg1"])
def test_oracle_cg_known_answers(golden_dir, case):
    ka = json.load(open(os.path.join(golden_dir, "cg_known_answers.json")))[case]
    A = np.array(ka["A"], dtype=np.float64)
    rowptr, col, val = O.dense_to_lower_csr(A)
    fac = O.ic0(rowptr, col, val)
    x, it = O.cg(rowptr, col, val, np.array(ka["b"], dtype=np.float64), ka["crit_norm_inf_delta"],
                 crit_kind=0, precond=0, fac=fac)
    assert it > 0
    assert np.all(err_unit_test(x, np.array(ka["x"])) < 1e-12)


def test_oracle_patch_test_and_rigid_modes():
    """Element consistency: rigid-body modes are in the kernel of K_e and a linear field gives
    zero interior forces (patch test) on a distorted mesh."""
    pos, conn = O.make_rect_hexa(4)
    rng = np.random.default_rng(0)
    interior = np.all((pos > 1e-9) & (pos < 1 - 1e-9), axis=1)
    pos = pos + interior[:, None] * rng.uniform(-0.05, 0.05, pos.shape)
    Ke = O.hexa8_ke(pos[conn[0]], 210000.0, 0.3)
    assert np.abs(Ke - Ke.T).max() <= 1e-12 * np.abs(Ke).max()
    xyz = pos[conn[0]]
    modes = [np.tile(e, 8) for e in np.eye(3)]
    for ax in range(3):
        w = np.zeros(3)
        w[ax] = 1.0
        modes.append(np.cross(w, xyz).ravel())
    for m in modes:
        assert np.abs(Ke @ m).max() <= 1e-9 * np.abs(Ke).max() * np.abs(m).max()
    rowptr, col = O.pattern_lower(pos.shape[0], 3, conn)
    val = O.assemble_elast(pos, conn, 210000.0, 0.3, rowptr, col)
    G = np.array([[1e-3, 2e-3, -1e-3], [0.5e-3, -2e-3, 1e-3], [3e-3, 1e-3, 2e-3]])
    u = (pos @ G.T).ravel()
    f = O.spmv(rowptr, col, val, u).reshape(-1, 3)
    assert np.abs(f[interior]).max() <= 1e-9 * np.abs(f).max()


def test_oracle_constraint_penalty_semantics():
    """assemble_constraints: K(j,j) += c^2 max|diag| p and F(j) += c max|diag| p res."""
    A = np.array([[4.0, 1.0], [1.0, 3.0]])
    rowptr, col, val = O.dense_to_lower_csr(A)
    F = np.array([1.0, 2.0])
    md = O.penalty(rowptr, col, val, F, [1], [2.0], [0.5], 10.0)
    assert md == 4.0
    assert val[-1] == 3.0 + 2.0 * 2.0 * 4.0 * 10.0
    assert F[1] == 2.0 + 2.0 * 4.0 * 10.0 * 0.5


def test_oracle_adjoint_solve_matches_reference_ldl(golden_dir):
    """K lambda = u (the misfit adjoint) with the oracle's direct solver vs the reference's LDL."""
    g = load_golden(golden_dir, "hexa_10x10x10")
    m = g["meta"]
    P = O.elasticity_problem(m["nb_points"], E=m["E"], nu=m["nu"], pen=m["penalty"])
    lam = O.skyline_solve(P["rowptr"], P["col"], P["val"], g["u_ldl"])
    assert np.linalg.norm(lam - g["lam_ldl"]) <= 1e-12 * np.linalg.norm(g["lam_ldl"])


def test_oracle_diffusion_matches_reference_runtime(golden_dir):
    """Triangle_6 heat diffusion: mesh, Crank-Nicolson matrices (penalty on A) and one LDL step."""
    g = np.load(os.path.join(golden_dir, "tri6_8x8_cn.npz"))
    m = json.loads(str(g["meta"]))
    P = O.diffusion_problem(m["nb_points"], k=m["k"], rho_c=m["rho_c"], dt=m["dt"], theta=m["theta"],
                            pen=m["penalty"])
    assert np.array_equal(P["pos"], g["pos"]) and np.array_equal(P["conn"], g["conn"])
    n = P["pos"].shape[0]
    A = csr(g["rowptr"], g["col"], g["A"], n)
    B = csr(g["rowptrB"], g["colB"], g["B"], n)
    Ao = csr(P["rowptr"], P["col"], P["A"], n)
    Bo = csr(P["rowptr"], P["col"], P["B"], n)
    assert abs(A - Ao).max() <= 1e-12 * abs(Ao).max()
    assert abs(B - Bo).max() <= 1e-12 * abs(Bo).max()
    assert P["max_diag"] == pytest.approx(m["max_diag"], rel=1e-14)
    np.testing.assert_allclose(P["T0"], g["T0"], rtol=1e-15, atol=0)  # exp() of two libms
    T1 = O.diffusion_run(P, 1)[1]
    assert np.linalg.norm(T1 - g["T1"]) <= 1e-12 * np.linalg.norm(g["T1"])


def test_oracle_element_fields_patch_test():
    """A linear displacement gives its exact strain and Hooke stress in every element."""
    G = np.array([[1e-3, 2e-3, -1e-3], [0.5e-3, -2e-3, 1e-3], [3e-3, 1e-3, 2e-3]])
    eps = 0.5 * (G + G.T)
    lam, mu = 2.1e5 * 0.3 / (1.3 * 0.4), 2.1e5 / 2.6
    sig = lam * np.trace(eps) * np.eye(3) + 2 * mu * eps
    idx = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    for make in (O.make_rect_hexa, O.make_rect_tetra10):
        pos, conn = make(3)
        out = O.elem_fields(pos, conn, 2.1e5, 0.3, (pos @ G.T).ravel())
        assert np.abs(out[:, :6] - [eps[i] for i in idx]).max() <= 1e-15
        assert np.abs(out[:, 6:12] - [sig[i] for i in idx]).max() <= 1e-10
        assert np.abs(out[:, 12] - np.trace(G)).max() <= 1e-15


def test_oracle_elimination_equals_lagrange_solution():
    """Exact constraints (penalty 0): the eliminated SPD system gives the solution of the
    reference's Lagrange-multiplier system [[K, C^T], [C, 0]] (formulation.h:1072-1088)."""
    import scipy.sparse.linalg as spla
    pos, conn = O.make_rect_hexa(4)
    rowptr, col = O.pattern_lower(pos.shape[0], 3, conn)
    val = O.assemble_elast(pos, conn, 2.1e5, 0.3, rowptr, col)
    n = 3 * pos.shape[0]
    F = np.zeros(n)
    P = O.elasticity_problem(4)
    O.quad4_traction(P["faces"], pos, (1.0, 0.3, 0.0), F)
    dofs = P["dofs"]
    coef = np.where(dofs % 3 == 1, 2.0, 1.0)
    res = np.where(dofs % 3 == 0, 1e-3, 0.0)
    L = csr(rowptr, col, val, n)
    K = (L + L.T - sp.diags(L.diagonal())).tocsc()
    C = sp.csr_matrix((coef, (np.arange(dofs.size), dofs)), shape=(dofs.size, n))
    S = sp.bmat([[K, C.T], [C, None]]).tocsc()
    x = spla.spsolve(S, np.concatenate([F, res]))[:n]
    val2, F2 = val.copy(), F.copy()
    O.eliminate(rowptr, col, val2, F2, dofs, coef, res)
    u = O.skyline_solve(rowptr, col, val2, F2)
    assert np.linalg.norm(u - x) <= 1e-10 * np.linalg.norm(x)
    assert np.abs(u[dofs] - res / coef).max() <= 1e-18


@pytest.mark.parametrize("name", ["hexa_10x10x10"])
def test_block_ic_pcg_restatement_matches_reference(golden_dir, name):
    """The restated 3x3-block IC(0)-PCG (MatWithTinyBlocks) on the reference's own assembled
    matrix: the factor's diagonal blocks, the iteration count and the solution of the reference's
    solve_using_incomplete_chol_factorize at the same absolute |r|_inf criterion."""
    g = load_golden(golden_dir, name)
    m = g["meta"]
    crit = m["block_crit"] * np.abs(g["F"]).max()
    x, it, dg, tf, ts = O.tiny_block_pcg(g["rowptr"], g["col"], g["val"], g["F"], crit)
    ref_dg = g["block_diag"].reshape(-1, 6)
    assert np.abs(dg - ref_dg).max() <= 1e-15 * np.abs(ref_dg).max()
    assert it == m["block_iter"]
    u = g["u_block"]
    assert np.linalg.norm(x - u) <= 1e-12 * np.linalg.norm(u)
    # and it solves the system: against the LDL solution
    assert np.linalg.norm(x - g["u_ldl"]) <= 1e-9 * np.linalg.norm(g["u_ldl"])


def test_recalage_element_restatement_matches_generated_code(golden_dir):
    """orc_recalage_ke / orc_recalage_nodal against the routines LMT++'s Codegen engine writes for
    formulation recalage (use_test_functions = False, integration_totale, order 2)."""
    g = np.load(os.path.join(golden_dir, "recal_elem.npz"))
    E, nu, rho, omega, gamma, r = g["params"]
    for t in ("hexa", "tetra10"):
        K = O.recalage_ke(g[t + "_xyz"], E, nu, rho, gamma)
        Kr = g[t + "_K"]  # upper triangle
        assert np.allclose(np.triu(K), Kr, rtol=0, atol=1e-14 * np.abs(Kr).max())
        assert np.allclose(K, K.T, rtol=0, atol=1e-15 * np.abs(K).max())
        Kn, Fn = O.recalage_nodal(g["ud"], float(g["valid"]), E, r)
        assert np.allclose(np.triu(Kn), g[t + "_Kn"], rtol=1e-15, atol=0)
        assert np.allclose(Fn, g[t + "_Fn"], rtol=1e-15, atol=0)
        assert np.any(Fn != 0)


@pytest.mark.parametrize("name", ["recal_hexa_3", "recal_tetra10_2"])
def test_recalage_assembly_matches_reference(golden_dir, name):
    """The assembled recalage system (element Hessians + nodal parts + penalty V = 0 on x = 0)
    against the reference's Sym SparseLine, and the LDL solution where it is unique: all of it on
    Hexa8; on Tetra10 the order-2 rule makes the quadratic element's mass matrix rank-deficient,
    so W is defined up to that null space and only U and V are compared."""
    g = load_golden(golden_dir, name)
    m = g["meta"]
    pos, conn = g["pos"], g["conn"]
    nn, n = pos.shape[0], 9 * pos.shape[0]
    rp, col = O.pattern_lower(nn, 9, conn)
    val, F = O.assemble_recalage(pos, conn, m["E"], m["nu"], m["rho"], m["gamma"], m["r"], g["Ud"], np.ones(nn),
                                 rp, col)
    dofs = np.array([9 * i + 3 + d for i in np.nonzero(pos[:, 0] < 1e-6)[0] for d in range(3)])
    md = O.penalty(rp, col, val, F, dofs, np.ones(dofs.size), np.zeros(dofs.size), m["penalty"])
    assert md == pytest.approx(m["max_diag"], rel=1e-15)
    A = csr(g["rowptr"], g["col"], g["val"], n).toarray()
    B = csr(rp, col, val, n).toarray()
    assert np.allclose(A, B, rtol=0, atol=1e-15 * np.abs(A).max())
    assert np.allclose(F, g["F"], rtol=0, atol=1e-15 * np.abs(g["F"]).max())
    S = B + np.tril(B, -1).T
    u = np.linalg.solve(S, F) if m["elem"] == "hexa" else np.linalg.lstsq(S, F, rcond=None)[0]
    assert np.abs(S @ g["u_ldl"] - F).max() <= 1e-12 * np.abs(F).max()
    d = (u - g["u_ldl"]).reshape(nn, 3, 3)
    sc = np.abs(g["u_ldl"]).max()
    assert np.abs(d[:, :2]).max() <= 1e-8 * sc
    if m["elem"] == "hexa":
        assert np.abs(d).max() <= 1e-10 * sc
