"""Batched multi-mesh, multi-RHS solves on the GPU against the oracle's direct solve of every
mesh and right-hand side, and against the single-system solver."""
import numpy as np
import pytest

from lmtpp_gb300.batch import BatchFormulation
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def batch_case(sides, seed):
    """Cubes of side n (elements), E ~ U[5e4, 3e5], nu ~ U[0.2, 0.4], clamped on x = 0 (penalty
    1e5), right-hand sides: unit tractions +x, +y, +z on x = 1 and a N(0, 1) nodal load."""
    rng = np.random.default_rng(seed)
    E = rng.uniform(5e4, 3e5, len(sides))
    nu = rng.uniform(0.2, 0.4, len(sides))
    probs = []
    for m, s in enumerate(sides):
        P = [O.elasticity_problem(s + 1, E=E[m], nu=nu[m], pen=1e5, traction=t) for t in np.eye(3)]
        F = np.stack([p["F"] for p in P] + [rng.standard_normal(P[0]["F"].shape[0])])
        probs.append(dict(P=P[0], F=F))
    return E, nu, probs


def build(sides, seed, mixed):
    E, nu, probs = batch_case(sides, seed)
    bf = BatchFormulation([(p["P"]["pos"], p["P"]["conn"]) for p in probs])
    bf.set_materials(E, nu)
    dofs = np.concatenate([p["P"]["dofs"] + 3 * int(bf.node_off[m]) for m, p in enumerate(probs)])
    bf.add_constraints(dofs, 1e5)
    bf.assemble(True, False, mixed=mixed)
    B = np.zeros((4, bf.n))
    for m, p in enumerate(probs):
        B[:, bf.dofs(m)] = p["F"]
    return bf, probs, B


@pytest.mark.parametrize("mode,tol_sol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_batch_matches_oracle_direct_solves(mode, tol_sol):
    sides = [2, 4, 3, 5, 2]
    bf, probs, B = build(sides, 7, mixed=(mode == "mixed"))
    X, st, its = bf.solve_batch(B, mode=mode, tol=1e-13 if mode == "fp64" else 1e-12)
    assert st["rel_residual"] <= 1e-12, st
    for m, p in enumerate(probs):
        P = p["P"]
        for r in range(4):
            x = O.skyline_solve(P["rowptr"], P["col"], P["val"], p["F"][r])
            rel = np.linalg.norm(X[r, bf.dofs(m)] - x) / np.linalg.norm(x)
            assert rel <= tol_sol, (m, r, rel, its[m, r])
    # larger meshes need more iterations than smaller ones: pairs stop independently
    assert its[3].min() > its[0].max(), its
    bf.close()


def test_batch_matrix_blocks_match_oracle():
    """Each mesh's diagonal block: its own E, nu and penalty scale max|diag| (1e-12)."""
    import scipy.sparse as sp
    bf, probs, B = build([2, 3], 3, mixed=False)
    rowptr, col, val = bf.get_mat()
    K = sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(bf.n, bf.n))
    for m, p in enumerate(probs):
        P, d = p["P"], bf.dofs(m)
        n = P["F"].shape[0]
        Ko = sp.csr_matrix((P["val"], P["col"].astype(np.int64), P["rowptr"].astype(np.int64)), shape=(n, n))
        Km = K[d, d]
        assert abs(Km - Ko).max() <= 1e-12 * abs(Ko).max()
        # nothing couples mesh m to the others
        assert K[d, :].nnz == Km.nnz
    bf.close()


def test_batch_equals_single_system_solves():
    """Every pair of a batch gives the single-mesh solver's answer (both to 1e-12 residual)."""
    from lmtpp_gb300 import Formulation
    sides = [3, 2]
    bf, probs, B = build(sides, 11, mixed=True)
    X, st, _ = bf.solve_batch(B[:3], mode="mixed", tol=1e-12)
    for m, p in enumerate(probs):
        P = p["P"]
        f = Formulation(P["pos"], P["conn"])
        E, nu, _ = batch_case(sides, 11)
        f.elastic_modulus = E[m]
        f.poisson_ratio = nu[m]
        f.add_constraints(P["dofs"], 1e5)
        for r in range(3):
            f.set_nodal_loads(p["F"][r])
            f.solve(1e-12, mode="fp64")
            u = f.get_result()
            assert np.linalg.norm(X[r, bf.dofs(m)] - u) <= 1e-8 * np.linalg.norm(u)
        f.close()
    bf.close()


def test_batch_autotuner_reports_candidates():
    bf, _, B = build([3, 3, 4], 5, mixed=True)
    info = bf.batch_info()
    assert info["tile_rows"] in (16, 32, 64, 128, 256, 512, 1024) and info["variant"] in (0, 1, 2)
    assert all(v > 0 for v in info["tuned_spmv_ms"].values())
    # a fixed choice is honoured and still solves
    bf.set_options(tile_rows=32, variant=0)
    X, st, _ = bf.solve_batch(B, mode="mixed", tol=1e-10)
    assert bf.batch_info()["tile_rows"] == 32 and bf.batch_info()["variant"] == 0
    assert st["rel_residual"] <= 1e-10
    assert info["ntiles"] >= 3
    bf.close()


@pytest.mark.parametrize("tile_rows", [128, 256, 1024])
def test_batch_bulk_copy_spmv_matches_oracle_and_warp_tiles(tile_rows):
    """SpMV variant 2 (matrix streamed by bulk copies, one CTA per tile) solves like the warp
    tiles (variant 1) and matches the oracle's direct solves; uneven meshes, four rhs."""
    sides = [2, 6, 3, 5, 2, 4]
    bf, probs, B = build(sides, 13, mixed=True)
    bf.set_options(tile_rows=min(tile_rows, 128), variant=1)
    X1, _, _ = bf.solve_batch(B, mode="mixed", tol=1e-12)
    bf.set_options(tile_rows=tile_rows, variant=2)
    X2, st, its = bf.solve_batch(B, mode="mixed", tol=1e-12)
    assert bf.batch_info()["variant"] == 2 and bf.batch_info()["tile_rows"] == tile_rows
    assert st["rel_residual"] <= 1e-12, st
    assert np.linalg.norm(X2 - X1) <= 1e-9 * np.linalg.norm(X1)
    for m, p in enumerate(probs):
        P = p["P"]
        for r in range(4):
            x = O.skyline_solve(P["rowptr"], P["col"], P["val"], p["F"][r])
            assert np.linalg.norm(X2[r, bf.dofs(m)] - x) <= 1e-8 * np.linalg.norm(x), (m, r)
    X3, _, _ = bf.solve_batch(B, mode="mixed", tol=1e-12)
    assert np.array_equal(X3, X2)  # deterministic
    bf.close()


def test_batch_of_tetra10_meshes_matches_oracle():
    """Tetra10 rows reach 65 blocks: the batched SpMV's wide-row path."""
    rng = np.random.default_rng(8)
    sides = [2, 3]
    E = rng.uniform(5e4, 3e5, 2)
    nu = rng.uniform(0.2, 0.4, 2)
    probs = [O.elasticity_problem(s + 1, E=E[m], nu=nu[m], pen=1e5, elem="tetra10") for m, s in enumerate(sides)]
    bf = BatchFormulation([(P["pos"], P["conn"]) for P in probs])
    bf.set_materials(E, nu)
    bf.add_constraints(np.concatenate([P["dofs"] + 3 * int(bf.node_off[m]) for m, P in enumerate(probs)]), 1e5)
    bf.assemble(True, False, mixed=True)
    B = rng.standard_normal((4, bf.n))
    for variant in (1, 2):
        bf.set_options(tile_rows=0, variant=variant)
        X, st, its = bf.solve_batch(B, mode="mixed", tol=1e-12)
        for m, P in enumerate(probs):
            d = bf.dofs(m)
            for r in range(4):
                x = O.skyline_solve(P["rowptr"], P["col"], P["val"], B[r, d])
                assert np.linalg.norm(X[r, d] - x) <= 1e-8 * np.linalg.norm(x), (variant, m, r)
    bf.set_options(tile_rows=0, variant=-1)
    for mode, tol in (("mixed", 1e-8), ("fp64", 1e-10)):
        X, st, its = bf.solve_batch(B, mode=mode, tol=1e-13 if mode == "fp64" else 1e-12)
        for m, P in enumerate(probs):
            d = bf.dofs(m)
            for r in range(4):
                x = O.skyline_solve(P["rowptr"], P["col"], P["val"], B[r, d])
                assert np.linalg.norm(X[r, d] - x) <= tol * np.linalg.norm(x), (mode, m, r)
    bf.close()
