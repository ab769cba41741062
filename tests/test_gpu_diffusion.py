"""Transient heat diffusion (Triangle_6, theta scheme) on the GPU against the oracle and the
reference's fixture; the adjoint gradient against central differences and checkpoint-free runs."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from lmtpp_gb300.diffusion import Diffusion, boundary_nodes, make_rect_triangle6
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def csr(rowptr, col, val, n):
    return sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(n, n))


def test_diffusion_matrices_and_step_match_reference(golden_dir):
    g = np.load(os.path.join(golden_dir, "tri6_8x8_cn.npz"))
    m = json.loads(str(g["meta"]))
    pos, conn = make_rect_triangle6(m["nb_points"])
    assert np.array_equal(pos, g["pos"]) and np.array_equal(conn, g["conn"])
    d = Diffusion(pos, conn)
    d.setup(m["k"], rho_c=m["rho_c"], dt=m["dt"], theta=m["theta"], dirichlet=boundary_nodes(pos),
            penalty=m["penalty"])
    rowptr, col, A, B = d.get_matrices()
    n = pos.shape[0]
    Ar = csr(g["rowptr"], g["col"], g["A"], n)
    Br = csr(g["rowptrB"], g["colB"], g["B"], n)
    Ag, Bg = csr(rowptr, col, A, n), csr(rowptr, col, B, n)
    assert abs(Ar - Ag).max() <= 1e-12 * abs(Ar).max()
    assert abs(Br - Bg).max() <= 1e-12 * abs(Br).max()
    assert d.get_penalty_scale() == pytest.approx(m["max_diag"], rel=1e-12)
    d.set_state(g["T0"])
    d.run(1, tol=1e-14)
    T1 = d.get_state()
    assert np.linalg.norm(T1 - g["T1"]) <= 1e-10 * np.linalg.norm(g["T1"])
    d.close()


@pytest.mark.parametrize("theta", [0.5, 1.0])
def test_diffusion_multistep_matches_oracle(theta):
    rng = np.random.default_rng(4)
    P0 = O.diffusion_problem(17, theta=theta)
    k = np.exp(0.3 * rng.standard_normal(P0["conn"].shape[0]))
    P = O.diffusion_problem(17, k=k, theta=theta)
    states = O.diffusion_run(P, 10)
    d = Diffusion(P["pos"], P["conn"])
    d.setup(k, rho_c=1.0, dt=1e-4, theta=theta, dirichlet=boundary_nodes(P["pos"]), penalty=1e5)
    d.set_state(P["T0"])
    st = d.run(10, tol=1e-14)
    T = d.get_state()
    assert np.linalg.norm(T - states[-1]) <= 1e-10 * np.linalg.norm(states[-1]), st
    d.close()


def test_diffusion_adjoint_checkpoints_and_central_differences():
    rng = np.random.default_rng(9)
    pos, conn = make_rect_triangle6(9)
    ne = conn.shape[0]
    k = np.exp(0.3 * rng.standard_normal(ne))
    T0 = O.gaussian_bump(pos)
    target = rng.standard_normal(pos.shape[0]) * 0.05
    d = Diffusion(pos, conn)
    bnd = boundary_nodes(pos)
    d.setup(k, rho_c=1.0, dt=1e-3, theta=1.0, dirichlet=bnd, penalty=1e5)
    d.set_penalty_scale(d.get_penalty_scale())  # held fixed, as the gradient assumes
    nsteps = 12
    J, g = d.adjoint_misfit(T0, target, nsteps, checkpoint_every=5, tol=1e-14)
    J1, g1 = d.adjoint_misfit(T0, target, nsteps, checkpoint_every=1, tol=1e-14)
    assert J == pytest.approx(J1, rel=1e-13)
    assert np.linalg.norm(g - g1) <= 1e-10 * np.linalg.norm(g1)

    def Jof(kk):
        d.setup(kk, rho_c=1.0, dt=1e-3, theta=1.0, dirichlet=bnd, penalty=1e5)
        d.set_state(T0)
        d.run(nsteps, tol=1e-15)
        r = d.get_state() - target
        return 0.5 * r @ r

    for e in rng.choice(ne, 5, replace=False):
        h = 1e-4 * k[e]
        kp, km = k.copy(), k.copy()
        kp[e] += h
        km[e] -= h
        fd = (Jof(kp) - Jof(km)) / (2 * h)
        assert fd == pytest.approx(g[e], rel=1e-5, abs=1e-9 * np.abs(g).max()), (e, fd, g[e])
    d.close()


@pytest.mark.parametrize("theta", [0.5, 1.0])
def test_diffusion_mixed_solver_matches_oracle(theta):
    """FP32-inner steps with FP64 residual replacement reach the FP64 solution: 1e-8 relative."""
    rng = np.random.default_rng(5)
    P0 = O.diffusion_problem(17, theta=theta)
    k = np.exp(0.3 * rng.standard_normal(P0["conn"].shape[0]))
    P = O.diffusion_problem(17, k=k, theta=theta)
    states = O.diffusion_run(P, 10)
    d = Diffusion(P["pos"], P["conn"])
    d.setup(k, rho_c=1.0, dt=1e-4, theta=theta, dirichlet=boundary_nodes(P["pos"]), penalty=1e5)
    d.set_solver("mixed")
    d.set_state(P["T0"])
    st = d.run(10, tol=1e-12)
    T = d.get_state()
    assert np.linalg.norm(T - states[-1]) <= 1e-8 * np.linalg.norm(states[-1]), st
    d.close()


def test_diffusion_bulk_copy_spmv_matches_warp_streamed():
    """The FP32 step solver with the TMA-streamed CSR SpMV (kind 1) and the warp-streamed one
    (kind 0): both reach the oracle's states; kind 1 is deterministic."""
    rng = np.random.default_rng(9)
    P0 = O.diffusion_problem(33)
    k = np.exp(0.3 * rng.standard_normal(P0["conn"].shape[0]))
    P = O.diffusion_problem(33, k=k, theta=1.0)
    states = O.diffusion_run(P, 6)
    out = {}
    for kind in (0, 1, 1):
        d = Diffusion(P["pos"], P["conn"])
        d.setup(k, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=boundary_nodes(P["pos"]), penalty=1e5)
        d.set_solver("mixed")
        d.set_spmv_kind(kind)
        d.set_state(P["T0"])
        d.run(6, tol=1e-12)
        T = d.get_state()
        assert np.linalg.norm(T - states[-1]) <= 1e-8 * np.linalg.norm(states[-1]), kind
        if kind in out:
            assert np.array_equal(T, out[kind])
        out[kind] = T
        d.close()
    assert np.linalg.norm(out[1] - out[0]) <= 1e-9 * np.linalg.norm(out[0])


def test_diffusion_mixed_adjoint_matches_fp64():
    rng = np.random.default_rng(11)
    pos, conn = make_rect_triangle6(13)
    k = np.exp(0.3 * rng.standard_normal(conn.shape[0]))
    T0 = O.gaussian_bump(pos)
    target = rng.standard_normal(pos.shape[0]) * 0.05
    d = Diffusion(pos, conn)
    d.setup(k, rho_c=1.0, dt=1e-3, theta=0.5, dirichlet=boundary_nodes(pos), penalty=1e5)
    J64, g64 = d.adjoint_misfit(T0, target, 8, checkpoint_every=3, tol=1e-13)
    d.set_solver("mixed")
    J32, g32 = d.adjoint_misfit(T0, target, 8, checkpoint_every=3, tol=1e-13)
    assert J32 == pytest.approx(J64, rel=1e-9)
    assert np.linalg.norm(g32 - g64) <= 1e-8 * np.linalg.norm(g64)
    d.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_sources_and_convection_match_oracle(mode, tol):
    """difftherm's other terms: volume source Q (nodal), nodal source Qs, skin convection
    H (T - t0) on the x = 1 edges; T = 0 on x = 0 only."""
    from lmtpp_gb300.diffusion import edges_on
    P = O.diffusion_problem(9, theta=0.5)
    pos = P["pos"]
    left = np.nonzero(pos[:, 0] < 1e-9)[0].astype(np.uint32)
    # the oracle problem with the Dirichlet nodes on x = 0 only
    rowptr, col = P["rowptr"], P["col"]
    A, B = O.assemble_diff(pos, P["conn"], 1.0, 1.0, 1e-4, 0.5, rowptr, col)
    md = O.penalty(rowptr, col, A, None, left, np.ones(left.size), np.zeros(left.size), 1e5)
    P.update(A=A, B=B)
    Q = np.sin(np.pi * pos[:, 0]) * np.cos(np.pi * pos[:, 1])
    Qs = np.zeros(pos.shape[0])
    Qs[[10, 40, 70]] = [3.0, -1.0, 2.0]
    edges = edges_on(pos, P["conn"], 0, 1.0)
    assert edges.shape[0] == 8
    load = O.diffusion_sources(P, Q, Qs) + O.diffusion_convection(P, edges, 2.5, 0.7)
    states = O.diffusion_run(P, 6, load=load)
    d = Diffusion(pos, P["conn"])
    d.setup(1.0, rho_c=1.0, dt=1e-4, theta=0.5, dirichlet=left, penalty=1e5)
    assert d.get_penalty_scale() == pytest.approx(md, rel=1e-12)
    d.set_sources(Q, Qs)
    d.set_convection(edges, 2.5, 0.7)
    rp, cl, Ag, Bg = d.get_matrices()
    n = pos.shape[0]
    assert abs(csr(rp, cl, Ag, n) - csr(rowptr, col, A, n)).max() <= 1e-12 * np.abs(A).max()
    assert abs(csr(rp, cl, Bg, n) - csr(rowptr, col, B, n)).max() <= 1e-12 * np.abs(B).max()
    d.set_solver(mode)
    d.set_state(P["T0"])
    d.run(6, tol=1e-14 if mode == "fp64" else 1e-12)
    T = d.get_state()
    assert np.linalg.norm(T - states[-1]) <= tol * np.linalg.norm(states[-1])
    d.close()


@pytest.mark.parametrize("theta", [0.5, 1.0])
def test_diffusion_multigrid_matches_oracle_and_cuts_iterations(theta):
    """The mixed step solver with the scalar aggregation multigrid (the default from 3000 unknowns)
    and with Jacobi: both reach the oracle's states (1e-8 relative); the multigrid needs under half
    of Jacobi's FP32 iterations at this size (129^2 nodes; the gap grows with the mesh: 49 against
    623 per step at 2049^2) and repeats its results bit for bit."""
    rng = np.random.default_rng(21)
    P0 = O.diffusion_problem(65)
    k = np.exp(0.3 * rng.standard_normal(P0["conn"].shape[0]))
    P = O.diffusion_problem(65, k=k, theta=theta)
    assert P["pos"].shape[0] == 129 * 129
    states = O.diffusion_run(P, 4)
    its, out = {}, {}
    for prec in ("jacobi", "amg", "amg"):
        d = Diffusion(P["pos"], P["conn"])
        d.setup(k, rho_c=1.0, dt=1e-4, theta=theta, dirichlet=boundary_nodes(P["pos"]), penalty=1e5)
        d.set_solver("mixed")
        d.set_preconditioner(prec)
        d.set_state(P["T0"])
        st = d.run(4, tol=1e-12)
        T = d.get_state()
        assert np.linalg.norm(T - states[-1]) <= 1e-8 * np.linalg.norm(states[-1]), (prec, st)
        if prec in out:
            assert np.array_equal(T, out[prec])
        out[prec] = T
        its[prec] = st["iterations"]
        d.close()
    assert its["amg"] * 2 < its["jacobi"], (theta, its)


def test_diffusion_wide_numbering_uses_32bit_columns_and_matches():
    """A node numbering whose column offsets exceed 16 bits (a random relabelling of 257^2
    nodes) keeps the bulk-copy products on 32-bit column indices; the banded numbering uses 16-bit
    deltas. Both reach the oracle's states (1e-8 relative) through the multigrid step solver."""
    rng = np.random.default_rng(33)
    P0 = O.diffusion_problem(129)
    k = np.exp(0.3 * rng.standard_normal(P0["conn"].shape[0]))
    P = O.diffusion_problem(129, k=k, theta=1.0)
    n = P["pos"].shape[0]
    states = O.diffusion_run(P, 3)
    perm = rng.permutation(n)               # new id of old node i: perm[i]
    inv = np.argsort(perm)
    pos_p = P["pos"][inv]                   # node j of the relabelled mesh is old node inv[j]
    conn_p = perm[P["conn"]].astype(np.uint32)
    assert np.abs(conn_p.astype(np.int64)[:, :, None] - conn_p.astype(np.int64)[:, None, :]).max() > 32767
    for pos, conn, back in ((P["pos"], P["conn"], None), (pos_p, conn_p, perm)):
        d = Diffusion(pos, conn)
        d.setup(k, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=boundary_nodes(pos), penalty=1e5)
        d.set_solver("mixed")
        d.set_state(P["T0"] if back is None else P["T0"][inv])
        st = d.run(3, tol=1e-12)
        T = d.get_state()
        if back is not None:
            T = T[back]
        assert np.linalg.norm(T - states[-1]) <= 1e-8 * np.linalg.norm(states[-1]), st
        d.close()


def test_multigrid_is_rebuilt_after_convection_changes_the_matrix():
    """The mixed step solver with the multigrid (65^2 nodes, T = 0 on x = 0 only): three steps,
    then skin convection on the x = 1 edges (A and B change, the multigrid is rebuilt at the next
    solve), three more steps with the convection load; both stretches against the oracle."""
    from lmtpp_gb300.diffusion import edges_on
    P = O.diffusion_problem(33, theta=1.0)
    pos = P["pos"]
    left = np.nonzero(pos[:, 0] < 1e-9)[0].astype(np.uint32)
    rowptr, col = P["rowptr"], P["col"]
    A, B = O.assemble_diff(pos, P["conn"], 1.0, 1.0, 1e-4, 1.0, rowptr, col)
    O.penalty(rowptr, col, A, None, left, np.ones(left.size), np.zeros(left.size), 1e5)
    P.update(A=A, B=B)
    first = O.diffusion_run(P, 3)
    edges = edges_on(pos, P["conn"], 0, 1.0)
    load = O.diffusion_convection(P, edges, 40.0, 0.7)  # adds to P["A"], P["B"]
    second = O.diffusion_run(P, 3, T0=first[-1], load=load)
    d = Diffusion(pos, P["conn"])
    d.setup(1.0, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=left, penalty=1e5)
    d.set_penalty_scale(d.get_penalty_scale())
    d.set_solver("mixed")
    d.set_state(P["T0"])
    d.run(3, tol=1e-12)
    T = d.get_state()
    assert np.linalg.norm(T - first[-1]) <= 1e-8 * np.linalg.norm(first[-1])
    d.set_convection(edges, 40.0, 0.7)
    st = d.run(3, tol=1e-12)
    T = d.get_state()
    assert np.linalg.norm(T - second[-1]) <= 1e-8 * np.linalg.norm(second[-1]), st
    assert np.linalg.norm(second[-1] - first[-1]) > 1e-3 * np.linalg.norm(first[-1])
    d.close()


def test_diffusion_multigrid_adjoint_matches_fp64():
    """The misfit adjoint with the mixed step solver on the multigrid (65^2 nodes) against the
    FP64 Jacobi solver: J to 1e-9, the gradient to 1e-7 (both solved to 1e-13)."""
    rng = np.random.default_rng(13)
    pos, conn = make_rect_triangle6(33)
    assert pos.shape[0] >= 3000
    k = np.exp(0.3 * rng.standard_normal(conn.shape[0]))
    T0 = O.gaussian_bump(pos)
    target = rng.standard_normal(pos.shape[0]) * 0.05
    d = Diffusion(pos, conn)
    d.setup(k, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=boundary_nodes(pos), penalty=1e5)
    J64, g64 = d.adjoint_misfit(T0, target, 6, checkpoint_every=3, tol=1e-13)
    d.set_solver("mixed")
    J32, g32 = d.adjoint_misfit(T0, target, 6, checkpoint_every=3, tol=1e-13)
    assert J32 == pytest.approx(J64, rel=1e-9)
    assert np.linalg.norm(g32 - g64) <= 1e-7 * np.linalg.norm(g64)
    d.close()


def test_diffusion_multigrid_at_full_size_matches_jacobi():
    """At the transient benchmark's size, 2 x 1024^2 elements (4.2 M nodes, a 5-level hierarchy,
    level-0 products on 16-bit column deltas): two steps with the multigrid and with Jacobi
    (both to 1e-12) give the same states to 1e-9 relative, and the multigrid needs under a
    tenth of the iterations."""
    pos, conn = make_rect_triangle6(1025)
    rng = np.random.default_rng(20251203)
    k = np.exp(0.3 * rng.standard_normal(conn.shape[0]))
    d2 = (pos[:, 0] - 0.5) ** 2 + (pos[:, 1] - 0.5) ** 2
    T0 = np.exp(-d2 / (2 * 0.1 * 0.1))
    out, its = {}, {}
    for prec in ("amg", "jacobi"):
        d = Diffusion(pos, conn)
        d.setup(k, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=boundary_nodes(pos), penalty=1e5)
        d.set_solver("mixed")
        d.set_preconditioner(prec)
        d.set_state(T0)
        st = d.run(2, tol=1e-12)
        out[prec], its[prec] = d.get_state(), st["iterations"]
        d.close()
    assert np.linalg.norm(out["amg"] - out["jacobi"]) <= 1e-9 * np.linalg.norm(out["jacobi"])
    assert its["amg"] * 10 < its["jacobi"], its
