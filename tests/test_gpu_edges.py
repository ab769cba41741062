"""Edge cases of the GPU path: single-element meshes, zero loads, an unconstrained (singular)
body, batches with one or three right-hand sides and a one-element mesh, API misuse of batches,
a one-cell diffusion mesh and a one-zone fit."""
import numpy as np
import pytest

from lmtpp_gb300 import Formulation, abi, make_rect_hexa, make_rect_tetra10, x1_faces
from lmtpp_gb300.batch import BatchFormulation
from lmtpp_gb300.diffusion import Diffusion, boundary_nodes, make_rect_triangle6
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def problem(P, **kw):
    f = Formulation(P["pos"], P["conn"])
    f.elastic_modulus = P["E"]
    f.poisson_ratio = P["nu"]
    f.add_constraints(P["dofs"], P["penalty"])
    f.add_skin_traction(P["faces"], (1.0, 0.0, 0.0))
    return f


@pytest.mark.parametrize("elem", ["hexa", "tetra10"])
@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_single_cube_matches_oracle(elem, mode, tol):
    P = O.elasticity_problem(2, elem=elem)  # one cube: 1 Hexa8 or 6 Tetra10
    x = O.skyline_solve(P["rowptr"], P["col"], P["val"], P["F"])
    f = problem(P)
    f.solve(1e-13 if mode == "fp64" else 1e-12, mode=mode)
    u = f.get_result()
    assert np.linalg.norm(u - x) <= tol * np.linalg.norm(x)
    f.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_zero_load_gives_zero_solution_at_once(mode):
    P = O.elasticity_problem(4)
    f = Formulation(P["pos"], P["conn"])
    f.elastic_modulus = P["E"]
    f.add_constraints(P["dofs"], P["penalty"])
    st = f.solve(1e-10, mode=mode)
    assert st["iterations"] == 0 and st["status"] == abi.OK
    assert not np.any(f.get_result())
    f.close()


def test_unconstrained_body_stops_with_a_status():
    """No constraint: K is singular (rigid-body modes) and an unbalanced traction has no
    solution; the solver stops at its iteration cap with a status instead of running on."""
    P = O.elasticity_problem(4)
    f = Formulation(P["pos"], P["conn"])
    f.elastic_modulus = P["E"]
    f.add_skin_traction(P["faces"], (1.0, 0.0, 0.0))
    with pytest.raises(abi.LmtgError) as ei:
        f.solve(1e-10, mode="fp64", maxit=400)
    assert ei.value.status in (abi.ERR_NOT_CONVERGED, abi.ERR_NAN)
    f.close()


@pytest.mark.parametrize("nrhs", [1, 3])
def test_batch_with_one_element_mesh_and_fewer_rhs(nrhs):
    sides = [1, 3, 2]
    rng = np.random.default_rng(nrhs)
    E = rng.uniform(5e4, 3e5, len(sides))
    nu = rng.uniform(0.2, 0.4, len(sides))
    probs = [O.elasticity_problem(s + 1, E=E[m], nu=nu[m], pen=1e5) for m, s in enumerate(sides)]
    bf = BatchFormulation([(P["pos"], P["conn"]) for P in probs])
    bf.set_materials(E, nu)
    bf.add_constraints(np.concatenate([P["dofs"] + 3 * int(bf.node_off[m]) for m, P in enumerate(probs)]), 1e5)
    bf.assemble(True, False, mixed=True)
    B = rng.standard_normal((nrhs, bf.n))
    X, st, its = bf.solve_batch(B, mode="mixed", tol=1e-12)
    assert its.shape == (len(sides), nrhs)
    for m, P in enumerate(probs):
        d = bf.dofs(m)
        for r in range(nrhs):
            x = O.skyline_solve(P["rowptr"], P["col"], P["val"], B[r, d])
            assert np.linalg.norm(X[r, d] - x) <= 1e-8 * np.linalg.norm(x)
    bf.close()


def test_batch_misuse_is_reported():
    pos, conn = make_rect_hexa((3, 3, 3))
    f = Formulation(pos, conn)
    bad = np.array([0, 10, pos.shape[0]], dtype=np.uint64)  # node 10 is shared by elements of both ranges
    assert f._lib.lmtg_batch_set(f._ctx, 2, abi.ptr(bad)) == abi.ERR_ARG
    short = np.array([0, 5], dtype=np.uint64)  # does not end at nn
    assert f._lib.lmtg_batch_set(f._ctx, 1, abi.ptr(short)) == abi.ERR_ARG
    f.close()
    bf = BatchFormulation([make_rect_hexa((3, 3, 3))])
    bf.set_materials([1e5], [0.3])
    with pytest.raises(abi.LmtgError) as ei:
        bf.solve_batch(np.zeros((5, bf.n)))  # more than four right-hand sides
    assert ei.value.status == abi.ERR_ARG
    bf.close()


def test_one_cell_diffusion_matches_oracle():
    P = O.diffusion_problem(2, theta=0.5)
    states = O.diffusion_run(P, 3)
    d = Diffusion(P["pos"], P["conn"])
    d.setup(1.0, rho_c=1.0, dt=1e-4, theta=0.5, dirichlet=boundary_nodes(P["pos"]), penalty=1e5)
    d.set_state(P["T0"])
    d.run(3, tol=1e-14)
    assert np.linalg.norm(d.get_state() - states[-1]) <= 1e-10 * max(np.linalg.norm(states[-1]), 1e-300)
    d.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_exact_constraints_by_elimination_match_oracle(mode, tol):
    """penalty 0 (the reference's Lagrange rows): u_j = res / coef exactly, the rest as the
    oracle's eliminated direct solve; a vector-only reassembly with new loads keeps it."""
    P = O.elasticity_problem(5)
    dofs = P["dofs"]
    coef = np.where(dofs % 3 == 1, 2.0, 1.0)
    res = np.where(dofs % 3 == 0, 1e-3, 0.0)
    f = Formulation(P["pos"], P["conn"])
    f.elastic_modulus = P["E"]
    f.poisson_ratio = P["nu"]
    f.add_constraints(dofs, 0.0, coefs=coef, res=res)
    f.add_skin_traction(P["faces"], (1.0, 0.0, 0.0))
    rowptr, col = O.pattern_lower(P["pos"].shape[0], 3, P["conn"])
    val = O.assemble_elast(P["pos"], P["conn"], P["E"], P["nu"], rowptr, col)
    F = np.zeros(P["F"].shape[0])
    O.quad4_traction(P["faces"], P["pos"], (1.0, 0.0, 0.0), F)
    O.eliminate(rowptr, col, val, F, dofs, coef, res)
    x = O.skyline_solve(rowptr, col, val, F)
    f.solve(1e-13 if mode == "fp64" else 1e-12, mode=mode)
    u = f.get_result()
    assert np.linalg.norm(u - x) <= tol * np.linalg.norm(x)
    assert np.abs(u[dofs] - res / coef).max() <= 1e-12 * np.abs(res).max()
    # the assembled matrix is the oracle's eliminated one
    rp, cl, v = f.get_mat()
    assert np.abs(v - val).max() <= 1e-12 * np.abs(val).max()
    # new loads (set_nodal_loads replaces the whole load vector) through a vector-only assembly
    rng = np.random.default_rng(1)
    G = rng.standard_normal(F.shape[0])
    f.set_nodal_loads(G)
    f.assemble(False, True, mixed=(mode == "mixed"))
    f.solve_system(1e-13 if mode == "fp64" else 1e-12, mode=mode)
    F2 = G.copy()
    val2 = O.assemble_elast(P["pos"], P["conn"], P["E"], P["nu"], rowptr, col)
    O.eliminate(rowptr, col, val2, F2, dofs, coef, res)
    x2 = O.skyline_solve(rowptr, col, val2, F2)
    assert np.linalg.norm(f.get_result() - x2) <= tol * np.linalg.norm(x2)
    f.close()


def test_exact_constraints_refuse_the_adjoint():
    P = O.elasticity_problem(3)
    f = Formulation(P["pos"], P["conn"])
    f.elastic_modulus = P["E"]
    f.add_constraints(P["dofs"], 0.0)
    f.add_skin_traction(P["faces"], (1.0, 0.0, 0.0))
    f.solve(1e-12, mode="fp64")
    with pytest.raises(abi.LmtgError) as ei:
        f.adjoint_grad("compliance")
    assert ei.value.status == abi.ERR_UNSUPPORTED
    f.close()


def test_levenberg_marquadt_term_and_constant_matrix():
    P = O.elasticity_problem(4)
    f = problem(P)
    f.levenberg_marquadt = 1e-3
    f.solve(1e-13, mode="fp64")
    val = P["val"].copy()
    O.add_levenberg_marquadt(P["rowptr"], val, P["max_diag"], 1e-3)
    rp, cl, v = f.get_mat()
    assert np.abs(v - val).max() <= 1e-12 * np.abs(val).max()
    x = O.skyline_solve(P["rowptr"], P["col"], val, P["F"])
    assert np.linalg.norm(f.get_result() - x) <= 1e-10 * np.linalg.norm(x)
    # assume_constant_matrix: a second solve with new loads reassembles only the vector
    f.assume_constant_matrix = True
    n0 = f.launch_count()
    G = np.random.default_rng(2).standard_normal(P["F"].shape[0])
    f.set_nodal_loads(G)
    f.set_result(np.zeros_like(G))
    f.solve(1e-13, mode="fp64")
    Fg = G.copy()
    O.penalty(P["rowptr"], P["col"], val.copy(), Fg, P["dofs"], np.ones(P["dofs"].size), np.zeros(P["dofs"].size),
              P["penalty"])
    x2 = O.skyline_solve(P["rowptr"], P["col"], val, Fg)
    assert np.linalg.norm(f.get_result() - x2) <= 1e-10 * np.linalg.norm(x2)
    f.close()


@pytest.mark.parametrize("elem", ["hexa", "tetra10"])
def test_volume_force_and_nodal_springs_match_oracle(elem):
    """elasticity_iso's density f_vol term and dep_imp_coef_0 springs, on a distorted mesh."""
    P = O.elasticity_problem(4, elem=elem)
    pos = P["pos"].copy()
    rng = np.random.default_rng(4)
    inner = np.all((pos > 1e-9) & (pos < 1 - 1e-9), axis=1)
    pos += inner[:, None] * rng.uniform(-0.04, 0.04, pos.shape)
    nn = pos.shape[0]
    coef = np.where(rng.random(nn) < 0.2, 1e4, 0.0)
    target = rng.standard_normal(3 * nn) * 1e-3
    f = Formulation(pos, P["conn"])
    f.elastic_modulus = P["E"]
    f.poisson_ratio = P["nu"]
    f.add_constraints(P["dofs"], P["penalty"])
    f.set_volume_force((0.0, -9.81, 1.5), density=7800.0)
    f.set_nodal_springs(coef, target)
    f.solve(1e-13, mode="fp64")
    # oracle: element stiffness + springs on the diagonal, then the penalty
    rowptr, col = O.pattern_lower(nn, 3, P["conn"])
    val = O.assemble_elast(pos, P["conn"], P["E"], P["nu"], rowptr, col)
    diag = rowptr[1:].astype(np.int64) - 1
    val[diag] += np.repeat(coef, 3)
    F = O.volume_force(pos, P["conn"], 7800.0, (0.0, -9.81, 1.5)) + np.repeat(coef, 3) * target
    O.penalty(rowptr, col, val, F, P["dofs"], np.ones(P["dofs"].size), np.zeros(P["dofs"].size), P["penalty"])
    np.testing.assert_allclose(f.get_sollicitation(), F, rtol=0, atol=1e-12 * np.abs(F).max())
    rp, cl, v = f.get_mat()
    assert np.abs(v - val).max() <= 1e-12 * np.abs(val).max()
    x = O.skyline_solve(rowptr, col, val, F)
    assert np.linalg.norm(f.get_result() - x) <= 1e-10 * np.linalg.norm(x)
    f.close()


@pytest.mark.parametrize("elem", ["hexa", "tetra10"])
def test_skin_pressure_matches_oracle(elem):
    P = O.elasticity_problem(4, elem=elem)
    pos = P["pos"].copy()
    rng = np.random.default_rng(6)
    inner = np.all((pos > 1e-9) & (pos < 1 - 1e-9), axis=1)
    pos += inner[:, None] * rng.uniform(-0.04, 0.04, pos.shape)
    f = Formulation(pos, P["conn"])
    f.elastic_modulus = P["E"]
    f.add_constraints(P["dofs"], P["penalty"])
    faces = x1_faces(pos, P["conn"])
    f.add_skin_pressure(faces, 2.5)
    f.assemble(True, True)
    F = f.get_sollicitation()
    Fo = O.pressure_loads(faces, pos, 2.5)
    np.testing.assert_allclose(F, Fo, rtol=0, atol=1e-13)
    if elem == "hexa":  # outward normal on x = 1: the same loads as the traction (p, 0, 0)
        Ft = np.zeros_like(Fo)
        O.quad4_traction(faces, pos, (2.5, 0.0, 0.0), Ft)
        np.testing.assert_allclose(Fo, Ft, rtol=0, atol=1e-13)
    f.close()


def test_device_wait_bound_gives_up_and_context_stays_usable():
    """The mbarrier waits of the bulk-copy SpMVs are bounded: a wait that nothing completes
    returns a timeout status after about a second, and the context then solves as before."""
    import ctypes
    P = O.elasticity_problem(4)
    f = problem(P)
    st = ctypes.c_int(-1)
    waited = ctypes.c_double(0.0)
    abi.check(f._lib.lmtg_selftest_bounded_wait(f._ctx, ctypes.byref(st), ctypes.byref(waited)), f._ctx,
              "selftest_bounded_wait")
    assert st.value == abi.ERR_TIMEOUT
    assert 0.5 <= waited.value <= 10.0, waited.value
    f.solve(1e-12, mode="mixed")
    u = f.get_result()
    x = O.skyline_solve(P["rowptr"], P["col"], P["val"], P["F"])
    assert np.linalg.norm(u - x) <= 1e-8 * np.linalg.norm(x)
    f.close()


def fan_tetra10(M=18):
    """Tetra10 fan around a central vertex: 2 M tetrahedra (centre, ring_i, ring_i+1, pole), so
    that the centre's node row holds 5 M + 5 blocks (95 for M = 18; the pattern allows 96)."""
    ang = 2 * np.pi * np.arange(M) / M
    verts = [np.zeros(3)] + [np.array([np.cos(a), np.sin(a), 0.0]) for a in ang] + [np.array([0, 0, 1.0]),
                                                                                       np.array([0, 0, -1.0])]
    pos = list(verts)
    mid = {}

    def m(a, b):
        k = (min(a, b), max(a, b))
        if k not in mid:
            mid[k] = len(pos)
            pos.append(0.5 * (pos[a] + pos[b]))
        return mid[k]
    conn = []
    for i in range(M):
        r0, r1 = 1 + i, 1 + (i + 1) % M
        for pole, sgn in ((M + 1, 1.0), (M + 2, -1.0)):
            v = [0, r0, r1, pole] if sgn > 0 else [0, r1, r0, pole]
            # LMT++ Tetra_10 edge order: (0,1) (1,2) (0,2) (0,3) (1,3) (2,3)
            e = [m(v[0], v[1]), m(v[1], v[2]), m(v[0], v[2]), m(v[0], v[3]), m(v[1], v[3]), m(v[2], v[3])]
            conn.append(v + e)
    return np.array(pos), np.array(conn, dtype=np.uint32)


def test_widest_rows_fan_of_tetra10_matches_oracle():
    """A node row of 95 blocks (next to the pattern's 96): the bulk-copy SpMV's wide-row paths and
    the warp-row kernel give the oracle's direct solution."""
    pos, conn = fan_tetra10(18)
    nn = pos.shape[0]
    # orientation: every element's vertex Jacobian positive
    v = pos[conn[:, :4]]
    assert (np.einsum("ij,ij->i", v[:, 1] - v[:, 0], np.cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 0])) > 0).all()
    rowptr, col = O.pattern_lower(nn, 3, conn)
    val = O.assemble_elast(pos, conn, 2.1e5, 0.3, rowptr, col)
    fixed = np.arange(1, 19 + 2)  # the ring and the poles
    dofs = (3 * fixed[:, None] + np.arange(3)).ravel()
    F = np.random.default_rng(4).standard_normal(3 * nn)
    Fo = F.copy()
    O.penalty(rowptr, col, val, Fo, dofs, np.ones(dofs.shape[0]), np.zeros(dofs.shape[0]), 1e5)
    x = O.skyline_solve(rowptr, col, val, Fo)
    for kind in (0, 1, 2):
        f = Formulation(pos, conn)
        f.elastic_modulus = 2.1e5
        f.poisson_ratio = 0.3
        f.add_constraints(dofs, 1e5)
        f.allocate_matrices()
        f.set_nodal_loads(F)
        f.set_spmv_kind(kind)
        f.solve(1e-12, mode="mixed")
        u = f.get_result()
        assert np.linalg.norm(u - x) <= 1e-8 * np.linalg.norm(x), kind
        f.close()
