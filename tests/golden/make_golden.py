"""Generates the golden fixtures of tests/golden from the reference's own code.

Runs oracle/_ref/ref_driver, built by oracle/build_ref.sh from the LMTpp sources: LMT++'s
make_rect, the element routines that LMT++'s Codegen engine writes for the weak forms of
elasticity_iso and difftherm (oracle/ref_codegen.cpp), its Gauss tables, the Sym SparseLine
assembly with erase-on-exact-zero, the max|diag| penalty, LDL, IC(0)-PCG and the 3x3-block
IC(0)-PCG.  Fixtures (compressed npz):

  elem_kernels         distorted single elements (Hexa8, Tetra10 with curved and with straight
                       edges, nu != 0.3, Triangle_6):
                       K_e summed over the reference's Gauss table, the skin loads of every face
                       (f_surf = (0.7,-0.2,0.4), p = 2.5), the difftherm A and B for Crank-Nicolson
                       and implicit Euler
  hexa_2x2x2, hexa_10x10x10, tetra10_3x3x3
                       the elasticity workload of the reference's example (unit cube, penalty clamp
                       of x = 0, uniform traction (1,0,0) on x = 1): mesh, lower CSR of K, F, the
                       LDL and IC(0)-PCG solutions, the adjoint LDL solve K lambda = u; for
                       hexa_10x10x10 also the 3x3-block IC(0)-PCG solution and factor diagonal
  hexa_16_lognormal    the Hexa8 benchmark family at 16^3: per-element E lognormal (log-std 0.5,
                       numpy default_rng(20251203), element order), nu 0.3: F, u_ldl, lambda,
                       the block IC(0)-PCG solution
  tetra10_10x10x10     the Tetra10 benchmark family at 10^3 cubes: F, u_ldl
  tri6_8x8_cn          Triangle_6 difftherm, Crank-Nicolson: A, B, one LDL step
  tri6_32_cn, tri6_32_ie
                       the transient family at 2 x 32^2: lognormal conductivity (log-std 0.3,
                       default_rng(20251203)), dt 1e-4, penalty boundary, 10 LDL steps (states 0, 1,
                       5, 10), A and B, for Crank-Nicolson and implicit Euler
  recal_elem           the recalage routines on the distorted Hexa8 and curved Tetra10 of
                       elem_kernels: element Hessian (upper triangle) and one node's nodal part
  recal_hexa_3, recal_tetra10_2, recal_hexa_8
                       the recalage system on the unit cube (3^3 Hexa8, 2^3 Tetra10 cubes, 8^3
                       Hexa8), E 2, nu 0.3, rho 1.5, omega 3, gamma 0.4, r 0.3, Ud a fixed quadratic
                       field, Ud_valid 1, V clamped on x = 0 by penalty 1e5: lower CSR, F, LDL solution
  batch_cubes          the batch family: cubes of side 3, 5 and 7 with E ~ U[5e4, 3e5] and
                       nu ~ U[0.2, 0.4] (default_rng(20251203)), four load cases each (+x, +y, +z
                       unit traction on x = 1, N(0,1) nodal load): F and u_ldl per cube and case

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
DRV = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
SEED = 20251203


def _run(cmd, d, **kw):
    args = [DRV, cmd] + ["%s=%s" % (k, v) for k, v in kw.items()] + ["out=" + d]
    subprocess.check_call(args)
    info = dict(l.split() for l in open(os.path.join(d, "info.txt")))
    r = lambda f, t: np.fromfile(os.path.join(d, f), dtype=t)
    return info, r


def elast_case(name, elem, nbp, E, nu, pen, dumpK=True, icpcg=True, block_crit=None, efile_E=None,
               batch_nodal=None):
    npe = 8 if elem == "hexa" else 10
    with tempfile.TemporaryDirectory() as d:
        kw = dict(elem=elem, nbp=nbp, E=repr(E), nu=repr(nu), penalty=repr(pen), dumpK=int(dumpK),
                  icpcg=int(icpcg))
        if efile_E is not None:
            np.asarray(efile_E, dtype=np.float64).tofile(os.path.join(d, "E.f64"))
            kw["efile"] = os.path.join(d, "E.f64")
        if block_crit is not None:
            kw.update(block=1, crit=repr(block_crit))
        if batch_nodal is not None:
            np.asarray(batch_nodal, dtype=np.float64).tofile(os.path.join(d, "nodal.f64"))
            kw.update(batch4=1, nodal=os.path.join(d, "nodal.f64"))
        info, r = _run("elast", d, **kw)
        n = int(info["n"])
        out = dict(F=r("F.f64", np.float64).reshape(-1, n).squeeze(), u_ldl=r("u_ldl.f64", np.float64).reshape(-1, n).squeeze(),
                   lam_ldl=r("lam_ldl.f64", np.float64))
        if dumpK:
            out.update(pos=r("pos.f64", np.float64).reshape(-1, 3), conn=r("conn.u32", np.uint32).reshape(-1, npe),
                       rowptr=r("rowptr.u64", np.uint64), col=r("col.u32", np.uint32), val=r("val.f64", np.float64))
        if icpcg:
            out["u_icpcg"] = r("u_icpcg.f64", np.float64)
        if block_crit is not None:
            out["u_block"] = r("u_block.f64", np.float64)
            out["block_diag"] = r("block_diag.f64", np.float64)
        meta = dict(elem=elem, nb_points=nbp, E=E, nu=nu, penalty=pen, max_diag=float(info["max_diag"]),
                    icpcg_iter=int(info["icpcg_iter"]), nnz=int(info["nnz"]), block_crit=block_crit,
                    block_iter=int(info["block_iter"]))
        if efile_E is not None:
            meta.update(E="lognormal", E_logmean=float(np.log(210000.0)), E_logstd=0.5, seed=SEED)
        if name is None:
            return out, meta
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), **out)
        return out, meta


def diff_case(name, nbp, k, rho_c, dt, theta, pen, steps, keep, kfield=None):
    with tempfile.TemporaryDirectory() as d:
        kw = dict(nbp=nbp, k=repr(k), rho_c=repr(rho_c), dt=repr(dt), theta=repr(theta), penalty=repr(pen),
                  steps=steps)
        if kfield is not None:
            np.asarray(kfield, dtype=np.float64).tofile(os.path.join(d, "k.f64"))
            kw["kfile"] = os.path.join(d, "k.f64")
        info, r = _run("diff", d, **kw)
        nn = int(info["nn"])
        states = r("states.f64", np.float64).reshape(steps + 1, nn)
        out = dict(pos=r("pos.f64", np.float64).reshape(-1, 2), conn=r("conn.u32", np.uint32).reshape(-1, 6),
                   rowptr=r("rowptr.u64", np.uint64), col=r("col.u32", np.uint32), A=r("val.f64", np.float64),
                   rowptrB=r("rowptrB.u64", np.uint64), colB=r("colB.u32", np.uint32), B=r("valB.f64", np.float64),
                   states=states[list(keep)], steps_kept=np.array(keep))
        if 1 in keep:
            out.update(T0=states[0], T1=states[1])
        meta = dict(nb_points=nbp, k=k if kfield is None else "lognormal", rho_c=rho_c, dt=dt, theta=theta,
                    penalty=pen, steps=steps, max_diag=float(info["max_diag"]))
        if kfield is not None:
            meta.update(k_logstd=0.3, seed=SEED)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), **out)


def elem_kernels():
    """Single distorted elements through the generated routines."""
    rng = np.random.default_rng(7)
    cube = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    hexa = 0.3 * cube + rng.uniform(-0.02, 0.02, cube.shape)
    v4 = np.array([[0, 0, 0], [1, 0.1, 0], [0.05, 1, 0.1], [0.1, 0.05, 1.1]]) * 0.4
    edges = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]  # Tetra_10 nodes 4..9
    tet = np.vstack([v4, [0.5 * (v4[a] + v4[b]) for a, b in edges]])
    tet[4:] += rng.uniform(-0.01, 0.01, (6, 3))  # curved edges
    tri = np.array([[0, 0], [1, 0.1], [0.1, 1], [0.5, 0.06], [0.55, 0.55], [0.04, 0.5]]) * 0.2
    tri[3:] += rng.uniform(-0.005, 0.005, (3, 2))
    tets = np.vstack([v4, [0.5 * (v4[a] + v4[b]) for a, b in edges]])  # straight edges
    res = {"hexa_xyz": hexa, "tetra10_xyz": tet, "tetra10s_xyz": tets, "tri6_xy": tri}
    cases = {"hexa": (hexa, 123456.0, 0.27), "tetra10": (tet, 210000.0, 0.35),
             "tetra10s": (tets, 70000.0, 0.21)}
    with tempfile.TemporaryDirectory() as d:
        for typ, (xyz, E, nu) in cases.items():
            xyz.astype(np.float64).tofile(os.path.join(d, "in.f64"))
            subprocess.check_call([DRV, "elem", "type=" + typ.rstrip("s"), "in=" + os.path.join(d, "in.f64"), "E=" + repr(E),
                                   "nu=" + repr(nu), "out=" + os.path.join(d, "out.f64")])
            o = np.fromfile(os.path.join(d, "out.f64"), dtype=np.float64)
            nd = 3 * xyz.shape[0]
            res[typ + "_Ke"] = o[:nd * nd].reshape(nd, nd)  # upper triangle (the generated tmp_i_j, j >= i)
            res[typ + "_skin"] = o[nd * nd:].reshape(-1, nd)
            res[typ + "_E_nu"] = np.array([E, nu])
        tri.astype(np.float64).tofile(os.path.join(d, "in.f64"))
        k, rho_c, dt = 0.7, 1.3, 1e-3
        subprocess.check_call([DRV, "elem", "type=tri6", "in=" + os.path.join(d, "in.f64"), "k=" + repr(k),
                               "rho_c=" + repr(rho_c), "dt=" + repr(dt), "out=" + os.path.join(d, "out.f64")])
        o = np.fromfile(os.path.join(d, "out.f64"), dtype=np.float64).reshape(4, 6, 6)
        res.update(tri6_A_cn=o[0], tri6_B_cn=o[1], tri6_A_ie=o[2], tri6_B_ie=o[3],
                   tri6_k_rhoc_dt=np.array([k, rho_c, dt]))
    res["skin_traction"] = np.array([0.7, -0.2, 0.4])
    res["skin_pressure"] = np.array(2.5)
    np.savez_compressed(os.path.join(HERE, "elem_kernels.npz"), **res)


RECAL = dict(E=2.0, nu=0.3, rho=1.5, omega=3.0, gamma=0.4, r=0.3)


def recal_case(name, elem, nbp, pen, dumpK=True):
    """The recalage system of the unit cube (V clamped on x = 0 by penalty) and its LDL solution."""
    npe = 8 if elem == "hexa" else 10
    with tempfile.TemporaryDirectory() as d:
        kw = dict(elem=elem, nbp=nbp, penalty=repr(pen), dumpK=int(dumpK), **{k: repr(v) for k, v in RECAL.items()})
        info, r = _run("recalage", d, **kw)
        out = dict(pos=r("pos.f64", np.float64).reshape(-1, 3), conn=r("conn.u32", np.uint32).reshape(-1, npe),
                   F=r("F.f64", np.float64), u_ldl=r("u_ldl.f64", np.float64), Ud=r("Ud.f64", np.float64))
        if dumpK:
            out.update(rowptr=r("rowptr.u64", np.uint64), col=r("col.u32", np.uint32), val=r("val.f64", np.float64))
        meta = dict(elem=elem, nb_points=nbp, penalty=pen, max_diag=float(info["max_diag"]), nnz=int(info["nnz"]),
                    ncons=int(info["ncons"]), **RECAL)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), **out)


def recal_elem():
    """Single distorted elements through the generated recalage routines."""
    ek = np.load(os.path.join(HERE, "elem_kernels.npz"))
    res = dict(params=np.array([RECAL[k] for k in ("E", "nu", "rho", "omega", "gamma", "r")]),
               ud=np.array([0.013, -0.004, 0.021]), valid=np.array(0.8))
    with tempfile.TemporaryDirectory() as d:
        for typ in ("hexa", "tetra10"):
            xyz = ek[typ + "_xyz"]
            xyz.astype(np.float64).tofile(os.path.join(d, "in.f64"))
            args = [DRV, "recal_elem", "type=" + typ, "in=" + os.path.join(d, "in.f64"),
                    "out=" + os.path.join(d, "out.f64"), "valid=0.8"]
            args += ["%s=%r" % (k, v) for k, v in RECAL.items()]
            args += ["ud%d=%r" % (i, float(v)) for i, v in enumerate(res["ud"])]
            subprocess.check_call(args)
            o = np.fromfile(os.path.join(d, "out.f64"), dtype=np.float64)
            nd = 9 * xyz.shape[0]
            res[typ + "_xyz"] = xyz
            res[typ + "_K"] = o[:nd * nd].reshape(nd, nd)  # upper triangle
            res[typ + "_Kn"] = o[nd * nd:nd * nd + 81].reshape(9, 9)
            res[typ + "_Fn"] = o[nd * nd + 81:]
    np.savez_compressed(os.path.join(HERE, "recal_elem.npz"), **res)


def batch_cubes():
    rng = np.random.default_rng(SEED)
    sides = [3, 5, 7]
    E = rng.uniform(5e4, 3e5, len(sides))
    nu = rng.uniform(0.2, 0.4, len(sides))
    res = {"sides": np.array(sides), "E": E, "nu": nu}
    for m, s in enumerate(sides):
        n = 3 * (s + 1) ** 3
        g = rng.standard_normal(n)
        out, meta = elast_case(None, "hexa", s + 1, float(E[m]), float(nu[m]), 1e5, dumpK=False, icpcg=False,
                               batch_nodal=g)
        res["F%d" % m] = out["F"]
        res["u%d" % m] = out["u_ldl"]
    np.savez_compressed(os.path.join(HERE, "batch_cubes.npz"), meta=np.array(json.dumps(
        dict(penalty=1e5, seed=SEED, rhs="+x,+y,+z unit traction on x=1; N(0,1) nodal load"))), **res)


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


def main(which):
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    jobs = {
        "elem_kernels": elem_kernels,
        "hexa_2x2x2": lambda: elast_case("hexa_2x2x2", "hexa", 3, 210000.0, 0.3, 1e5),
        "hexa_10x10x10": lambda: elast_case("hexa_10x10x10", "hexa", 11, 210000.0, 0.3, 1e5, block_crit=1e-10),
        "tetra10_3x3x3": lambda: elast_case("tetra10_3x3x3", "tetra10", 4, 210000.0, 0.3, 1e5),
        "hexa_16_lognormal": lambda: elast_case(
            "hexa_16_lognormal", "hexa", 17, 0.0, 0.3, 1e5, dumpK=False, icpcg=False, block_crit=1e-10,
            efile_E=np.exp(np.log(210000.0) + 0.5 * np.random.default_rng(SEED).standard_normal(16 ** 3))),
        "tetra10_10x10x10": lambda: elast_case("tetra10_10x10x10", "tetra10", 11, 210000.0, 0.3, 1e5,
                                               dumpK=False, icpcg=False),
        "tri6_8x8_cn": lambda: diff_case("tri6_8x8_cn", 9, 1.0, 1.0, 1e-3, 0.5, 1e5, 1, (0, 1)),
        "tri6_32_cn": lambda: diff_case("tri6_32_cn", 33, 1.0, 1.0, 1e-4, 0.5, 1e5, 10, (0, 1, 5, 10),
                                        kfield=np.exp(0.3 * np.random.default_rng(SEED).standard_normal(2 * 32 * 32))),
        "tri6_32_ie": lambda: diff_case("tri6_32_ie", 33, 1.0, 1.0, 1e-4, 1.0, 1e5, 10, (0, 1, 5, 10),
                                        kfield=np.exp(0.3 * np.random.default_rng(SEED).standard_normal(2 * 32 * 32))),
        "batch_cubes": batch_cubes,
        "recal_elem": recal_elem,
        "recal_hexa_3": lambda: recal_case("recal_hexa_3", "hexa", 4, 1e5),
        "recal_tetra10_2": lambda: recal_case("recal_tetra10_2", "tetra10", 3, 1e5),
        "recal_hexa_8": lambda: recal_case("recal_hexa_8", "hexa", 9, 1e5, dumpK=False),
    }
    for name in (which or list(jobs)):
        jobs[name]()
        print("wrote", name, flush=True)
    with open(os.path.join(HERE, "cg_known_answers.json"), "w") as f:
        json.dump(cg_known_answers(), f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
    sys.exit(0)
