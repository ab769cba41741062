"""Generates the golden fixtures of tests/golden from the reference's own runtime.

Runs oracle/_ref/ref_driver (LMT++'s make_rect, Sym SparseLine assembly semantics, max|diag|
penalty constraints, LDL and IC(0)-PCG, built by oracle/build_ref.sh from the LMTpp sources)
(and the LDL solution of K lambda = u, the adjoint of the misfit 1/2 |u|^2) on the elasticity
workload of the reference's example -- unit cube of Hexa8 or Tetra_10, penalty clamp
of x = 0, uniform traction (1,0,0) on x = 1 -- and stores its outputs as compressed npz.

For heat diffusion (formulation difftherm) on Triangle_6 it records the mesh, the Crank-Nicolson
matrices A = M/dt + K/2 (with the boundary penalty) and B = M/dt - K/2 in the reference's storage,
and one step A T1 = B T0 solved by the reference's LDL.

Also records the known-answer vectors of the reference's solver unit tests
(tests/include/containers/conjugate_gradient_test.cpp:15-71) as JSON.

Usage: python tests/golden/make_golden.py   (needs the reference sources; run in the build
container, the fixtures are committed).
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

CASES = [  # name, element, nb_points, E, nu, penalty
    ("hexa_2x2x2", "hexa", 3, 210000.0, 0.3, 1e5),
    ("hexa_10x10x10", "hexa", 11, 210000.0, 0.3, 1e5),
    ("tetra10_3x3x3", "tetra10", 4, 210000.0, 0.3, 1e5),
]


def run_case(name, elem, nbp, E, nu, pen):
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    npe = 8 if elem == "hexa" else 10
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([drv, elem, str(nbp), repr(E), repr(nu), repr(pen), d])
        r = lambda f, t: np.fromfile(os.path.join(d, f), dtype=t)
        info = dict(l.split() for l in open(os.path.join(d, "info.txt")))
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            pos=r("pos.f64", np.float64).reshape(-1, 3), conn=r("conn.u32", np.uint32).reshape(-1, npe),
            rowptr=r("rowptr.u64", np.uint64), col=r("col.u32", np.uint32), val=r("val.f64", np.float64),
            F=r("F.f64", np.float64), u_ldl=r("u_ldl.f64", np.float64),
            u_icpcg=r("u_icpcg.f64", np.float64), lam_ldl=r("lam_ldl.f64", np.float64),
            meta=np.array(json.dumps(dict(elem=elem, nb_points=nbp, E=E, nu=nu, penalty=pen,
                                          max_diag=float(info["max_diag"]),
                                          icpcg_iter=int(info["icpcg_iter"]),
                                          nnz=int(info["nnz"])))))


def run_tri6(name, nbp, k, rho_c, dt, theta, pen):
    """Heat diffusion on Triangle_6: mesh, A and B (lower CSR, penalty on A) and one LDL step."""
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([drv, "tri6", str(nbp), repr(k), repr(rho_c), repr(dt), repr(theta),
                               repr(pen), d])
        r = lambda f, t: np.fromfile(os.path.join(d, f), dtype=t)
        info = dict(l.split() for l in open(os.path.join(d, "info.txt")))
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            pos=r("pos.f64", np.float64).reshape(-1, 2), conn=r("conn.u32", np.uint32).reshape(-1, 6),
            rowptr=r("rowptr.u64", np.uint64), col=r("col.u32", np.uint32), A=r("val.f64", np.float64),
            rowptrB=r("rowptrB.u64", np.uint64), colB=r("colB.u32", np.uint32), B=r("valB.f64", np.float64),
            T0=r("T0.f64", np.float64), T1=r("T1.f64", np.float64),
            meta=np.array(json.dumps(dict(nb_points=nbp, k=k, rho_c=rho_c, dt=dt, theta=theta, penalty=pen,
                                          max_diag=float(info["max_diag"])))))


def cg_known_answers():
    # conjugate_gradient_0: 3x3 Sym matrix, b = (3,4,5), x = (11,2,4)
    # conjugate_gradient_1: 10x10 Sym matrix, b given, solution from Maple (s_Maple)
    M10 = [[348, 295, 221, 165, 221, 311, 311, 279, 216, 200],
           [295, 333, 113, 152, 174, 271, 244, 250, 169, 179],
           [221, 113, 277, 125, 166, 215, 272, 159, 207, 134],
           [165, 152, 125, 152, 155, 135, 206, 107, 143, 143],
           [221, 174, 166, 155, 270, 250, 280, 170, 219, 151],
           [311, 271, 215, 135, 250, 412, 389, 287, 247, 167],
           [311, 244, 272, 206, 280, 389, 474, 259, 259, 219],
           [279, 250, 159, 107, 170, 287, 259, 274, 140, 159],
           [216, 169, 207, 143, 219, 247, 259, 140, 297, 141],
           [200, 179, 134, 143, 151, 167, 219, 159, 141, 165]]
    return {
        "source": "tests/include/containers/conjugate_gradient_test.cpp:15-71",
        "tolerance": "ERROR_UNIT_TEST(a,b) = |a-b|/(1e-20+|a|+|b|) < 1e-12",
        "cg0": {"A": [[1, 2, -3], [2, 5, -7], [-3, -7, 13]], "b": [3, 4, 5], "x": [11, 2, 4],
                "crit_norm_inf_delta": 1e-5},
        "cg1": {"A": M10, "b": [0, 8, 1, 4, 6, 6, 0, 9, 0, 6],
                "x": [-1.4176810081375044408, -3.0067729851774937789, 3.5389214608316368121,
                      7.5278767154067853482, -.95330870992906846260, 16.004952790217101221,
                      -11.900092892559983095, -7.5660154416662888416, -6.0846051557343736576,
                      8.5770626957989029109],
                "crit_norm_inf_delta": 1e-5},
    }


if __name__ == "__main__":
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    for c in CASES:
        run_case(*c)
        print("wrote", c[0])
    run_tri6("tri6_8x8_cn", 9, 1.0, 1.0, 1e-3, 0.5, 1e5)
    print("wrote tri6_8x8_cn")
    with open(os.path.join(HERE, "cg_known_answers.json"), "w") as f:
        json.dump(cg_known_answers(), f, indent=1)
    print("wrote cg_known_answers.json")
    sys.exit(0)
