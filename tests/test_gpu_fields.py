"""Element fields after the solve (strain, stress, trace) on the GPU against the oracle."""
import numpy as np
import pytest

from lmtpp_gb300 import Formulation, make_rect_hexa, make_rect_tetra10
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def distorted(make, n, seed):
    pos, conn = make((n + 1,) * 3)
    rng = np.random.default_rng(seed)
    interior = np.all((pos > 1e-9) & (pos < 1 - 1e-9), axis=1)
    return pos + interior[:, None] * rng.uniform(-0.2 / n, 0.2 / n, pos.shape), conn


@pytest.mark.parametrize("make", [make_rect_hexa, make_rect_tetra10])
def test_element_fields_match_oracle(make):
    pos, conn = distorted(make, 4, 1)
    rng = np.random.default_rng(2)
    E = np.exp(np.log(2.1e5) + 0.5 * rng.standard_normal(conn.shape[0]))
    u = rng.standard_normal(pos.size) * 1e-3
    f = Formulation(pos, conn)
    f.elastic_modulus = E
    f.poisson_ratio = 0.27
    f.assemble(True, False)
    got = f.element_fields(u)
    ref = O.elem_fields(pos, conn, E, 0.27, u)
    for key, sl in (("epsilon", slice(0, 6)), ("sigma", slice(6, 12)), ("tr_epsilon", 12)):
        r = ref[:, sl]
        assert np.abs(got[key] - r).max() <= 1e-12 * np.abs(r).max(), key
    f.close()


def test_element_fields_of_the_solution_and_patch_test():
    pos, conn = distorted(make_rect_hexa, 5, 3)
    f = Formulation(pos, conn)
    f.elastic_modulus = 2.1e5
    f.poisson_ratio = 0.3
    G = np.array([[1e-3, 2e-3, -1e-3], [0.5e-3, -2e-3, 1e-3], [3e-3, 1e-3, 2e-3]])
    u = (pos @ G.T).ravel()
    f.assemble(True, False)
    out = f.element_fields(u)
    eps = 0.5 * (G + G.T)
    want = np.array([eps[0, 0], eps[1, 1], eps[2, 2], eps[0, 1], eps[0, 2], eps[1, 2]])
    assert np.abs(out["epsilon"] - want).max() <= 1e-12
    assert np.abs(out["tr_epsilon"] - np.trace(G)).max() <= 1e-12
    # default u = the current result
    f.set_result(u)
    again = f.element_fields()
    assert np.array_equal(again["sigma"], out["sigma"])
    f.close()


def test_vtu_of_a_solved_formulation(tmp_path):
    """write_vtu_elasticity: the displacement and the element fields of the solution, in the
    layout of LMT++'s elasticity mesh (the writer itself is pinned byte-for-byte on the CPU)."""
    import xml.etree.ElementTree as ET
    from lmtpp_gb300 import meshio, x1_faces
    pos, conn = make_rect_hexa(4)
    f = Formulation(pos, conn)
    f.elastic_modulus = 2.1e5
    f.poisson_ratio = 0.3
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), 1e5)
    f.add_skin_traction(x1_faces(pos, conn), (1.0, 0.0, 0.0))
    f.solve(1e-12, mode="mixed")
    out = tmp_path / "sol.vtu"
    meshio.write_vtu_elasticity(out, f)
    piece = ET.parse(out).getroot().find("UnstructuredGrid/Piece")
    arr = {a.get("Name"): np.array(a.text.split(), dtype=float) for a in piece.iter("DataArray") if a.get("Name")}
    u = f.get_result()
    assert np.allclose(arr["dep"], u, rtol=1e-5, atol=1e-6 * np.abs(u).max())
    sig = f.element_fields()["sigma"]
    assert np.allclose(arr["sigma"].reshape(-1, 6), sig, rtol=1e-5, atol=1e-6 * np.abs(sig).max())
    assert [a.get("Name") for a in piece.find("CellData")] == [
        "epsilon", "sigma", "tr_epsilon", "group", "elastic_modulus", "density", "poisson_ratio", "f_vol"]
    f.close()
