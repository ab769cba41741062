"""Python mirror of LMT++'s FormulationAncestor API for the elasticity hot path.

Same method names, argument meaning and error behaviour as the reference's virtual interface
(include/formulation/formulation_ancestor.h:18-262), backed by the C ABI in include/lmtg.h:

    f = Formulation(pos, conn)                  # PB pb(m); f = pb.formulation_nb(0)
    f.elastic_modulus = 210000.0; f.poisson_ratio = 0.3
    f.add_constraint("node[0].dep[0]", 1e5)     # penalty constraint
    f.add_skin_traction(faces, (1, 0, 0))       # f_surf on skin elements
    f.solve(iterative_criterium=1e-10)          # assemble + solve_system
    u = f.get_result()

Failures raise LmtgError (the reference throws SolveException / prints to std::cerr).
"""
import ctypes
import re

import numpy as np

from . import abi

_CONSTRAINT = re.compile(
    r"^\s*(?:(?P<coef>[-+]?[0-9.eE+-]+)\s*\*\s*)?node\[(?P<node>\d+)\]\.dep\[(?P<d>\d)\]"
    r"\s*(?:(?P<sign>[-+])\s*(?P<val>[0-9.eE+-]+))?\s*$")


def parse_constraint(txt):
    """'[c*]node[i].dep[d] [- v]' -> (i, d, c, v): the coefficient and right-hand side the
    reference's Constraint extracts by differentiation (include/formulation/constraint.h:46-93:
    coeff = d(ex)/d(unknown), res = -(ex with the unknown set to 0))."""
    m = _CONSTRAINT.match(txt.replace(" ", ""))
    if not m:
        raise abi.LmtgError(abi.ERR_UNSUPPORTED, "constraint %r is not a linear nodal one" % txt)
    coef = float(m.group("coef")) if m.group("coef") else 1.0
    val = float(m.group("val")) if m.group("val") else 0.0
    if m.group("sign") == "+":
        val = -val
    return int(m.group("node")), int(m.group("d")), coef, val


def make_rect_hexa(nb_points, X0=(0.0, 0.0, 0.0), X1=(1.0, 1.0, 1.0)):
    """make_rect(m, Hexa(), X0, X1, nb_points) (include/mesh/make_rect.h:653-679) -> pos, conn."""
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 3, dtype=np.uint32)
    nn = int(np.prod(nbp.astype(np.int64)))
    ne = int(np.prod(nbp.astype(np.int64) - 1))
    pos = np.zeros((nn, 3))
    conn = np.zeros((ne, 8), dtype=np.uint32)
    x0 = np.ascontiguousarray(X0, dtype=np.float64)
    x1 = np.ascontiguousarray(X1, dtype=np.float64)
    lib = abi.load()
    abi.check(lib.lmtg_make_rect_hexa(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), abi.ptr(pos),
                                      abi.ptr(conn)), None, "make_rect")
    return pos, conn


def make_rect_tetra10(nb_points, X0=(0.0, 0.0, 0.0), X1=(1.0, 1.0, 1.0)):
    """make_rect(m, Tetra_10(), X0, X1, nb_points) (include/mesh/make_rect.h:443-545) -> pos, conn."""
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 3, dtype=np.uint32)
    x0 = np.ascontiguousarray(X0, dtype=np.float64)
    x1 = np.ascontiguousarray(X1, dtype=np.float64)
    lib = abi.load()
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    abi.check(lib.lmtg_make_rect_tetra10(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), ctypes.byref(nn),
                                         ctypes.byref(ne), None, None), None, "make_rect_tetra10")
    pos = np.zeros((nn.value, 3))
    conn = np.zeros((ne.value, 10), dtype=np.uint32)
    abi.check(lib.lmtg_make_rect_tetra10(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), ctypes.byref(nn),
                                         ctypes.byref(ne), abi.ptr(pos), abi.ptr(conn)), None,
              "make_rect_tetra10")
    return pos, conn


# Tetra_10 children faces as Triangle_6 (formulations/element_Tetra_10.py:16-21)
TETRA10_FACES = np.array([[0, 2, 1, 6, 5, 4], [0, 1, 3, 4, 8, 7], [0, 3, 2, 7, 9, 6],
                          [1, 2, 3, 5, 9, 8]])


def x1_faces_tetra10(pos, conn, x1=1.0, eps=1e-6):
    """Triangle_6 skin faces of Tetra10 elements lying on the plane x = x1 (element order, then
    child order)."""
    q = conn[:, TETRA10_FACES]  # ne x 4 x 6
    on = np.all(pos[q, 0] > x1 - eps, axis=2)
    return np.ascontiguousarray(q[on], dtype=np.uint32)


def x1_faces(pos, conn, x1=1.0, eps=1e-6):
    """Skin faces on x = x1 for a Hexa8 (Quad4 faces) or Tetra10 (Triangle_6 faces) mesh."""
    return x1_faces_hexa(pos, conn, x1, eps) if conn.shape[1] == 8 else x1_faces_tetra10(pos, conn, x1, eps)


def x1_faces_hexa(pos, conn, x1=1.0, eps=1e-6):
    """Quad4 skin faces (Hexa child [1,2,6,5], formulations/element_Hexa.py:22-29) on x = x1."""
    cand = np.nonzero(pos[conn[:, 1], 0] > x1 - eps)[0]  # elements whose node 1 lies on the plane
    q = conn[cand][:, [1, 2, 6, 5]]
    on = np.all(pos[q, 0] > x1 - eps, axis=1)
    return np.ascontiguousarray(q[on], dtype=np.uint32)


class Formulation:
    """One elasticity_iso formulation on a Hexa8 or Tetra10 mesh (the element type follows from
    the connectivity width), resident on one GPU."""

    def __init__(self, pos, conn, device=0):
        conn = np.asarray(conn)
        elem = {8: abi.ELEM_HEXA8, 10: abi.ELEM_TETRA10}.get(conn.shape[1])
        if elem is None:
            raise abi.LmtgError(abi.ERR_UNSUPPORTED, "elements with %d nodes are not supported" % conn.shape[1])
        self.npe = conn.shape[1]
        self._lib = abi.load()
        self._ctx = ctypes.c_void_p()
        abi.check(self._lib.lmtg_create(device, ctypes.byref(self._ctx)), None, "lmtg_create")
        self.pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.uint32)
        self.nn, self.ne = self.pos.shape[0], self.conn.shape[0]
        self.n = 3 * self.nn
        abi.check(self._lib.lmtg_mesh_set(self._ctx, elem, self.nn, abi.ptr(self.pos),
                                          self.ne, abi.ptr(self.conn)), self._ctx, "mesh_set")
        # formulation defaults (formulations/formulation_elasticity_iso.py:5-6)
        self._E = np.array([1.0])
        self._nu = 0.33
        self._material_dirty = True
        self._constraints = []  # (dof, coef, res, penalty)
        self._constraints_dirty = False
        self.allocated = False
        self.default_iterative_criterium = 1e-10
        self.levenberg_marquadt = 0.0  # K += levenberg_marquadt * max|diag K| * Id at assembly
        self.assume_constant_matrix = False  # solve() reassembles only the vector once K exists
        self._lm_synced = 0.0
        self._have_matrix = False
        self.nb_threads_assemble_matrix = 1  # accepted for API parity; the GPU grid replaces it
        self.last_stats = None

    # -- material ---------------------------------------------------------------------------
    @property
    def elastic_modulus(self):
        return self._E if self._E.shape[0] > 1 else float(self._E[0])

    @elastic_modulus.setter
    def elastic_modulus(self, E):
        E = np.ascontiguousarray(np.atleast_1d(E), dtype=np.float64)
        if E.shape[0] not in (1, self.ne):
            raise abi.LmtgError(abi.ERR_ARG, "elastic_modulus needs 1 or ne values")
        self._E = E
        self._material_dirty = True

    @property
    def poisson_ratio(self):
        return self._nu

    @poisson_ratio.setter
    def poisson_ratio(self, nu):
        self._nu = float(nu)
        self._material_dirty = True

    def _sync_material(self):
        if self._material_dirty:
            abi.check(self._lib.lmtg_material_set(self._ctx, abi.ptr(self._E), self._E.shape[0],
                                                  self._nu), self._ctx, "material_set")
            self._material_dirty = False

    # -- constraints and loads ----------------------------------------------------------------
    def add_constraint(self, txt, penalty_value):
        """add_constraint("[c*]node[i].dep[d] [- v]", penalty) for linear single-unknown
        constraints (include/formulation/constraint.h:46-93): coefficient c, right side v."""
        node, d, coef, val = parse_constraint(txt)
        if node >= self.nn or d > 2:
            raise abi.LmtgError(abi.ERR_ARG, "constraint on a missing node/component")
        # Constraint::res = -(ex with unknowns set to 0) = v  (constraint.h:86)
        self._constraints.append((np.array([3 * node + d], dtype=np.int64), np.array([coef]), np.array([val]),
                                  float(penalty_value)))
        self._constraints_dirty = True

    def add_constraints(self, dofs, penalty_value, coefs=None, res=None):
        """Vectorised add_constraint for many 'node[i].dep[d]' constraints."""
        dofs = np.asarray(dofs, dtype=np.int64).ravel()
        coefs = np.ones(dofs.shape[0]) if coefs is None else np.asarray(coefs, dtype=np.float64).ravel()
        res = np.zeros(dofs.shape[0]) if res is None else np.asarray(res, dtype=np.float64).ravel()
        if dofs.size and (dofs.min() < 0 or dofs.max() >= self.n):
            raise abi.LmtgError(abi.ERR_ARG, "constraint on a missing DOF")
        self._constraints.append((dofs, coefs, res, float(penalty_value)))
        self._constraints_dirty = True

    def _sync_constraints(self):
        if not self._constraints_dirty:
            return
        pens = {c[3] for c in self._constraints}
        if len(pens) > 1:
            raise abi.LmtgError(abi.ERR_UNSUPPORTED, "one penalty value per formulation")
        cat = (lambda k, t: np.ascontiguousarray(np.concatenate([c[k] for c in self._constraints]), dtype=t)
               if self._constraints else np.zeros(0, dtype=t))
        dof, coef, res = cat(0, np.uint32), cat(1, np.float64), cat(2, np.float64)
        pen = pens.pop() if pens else 0.0
        abi.check(self._lib.lmtg_set_constraints(self._ctx, dof.shape[0], abi.ptr(dof), abi.ptr(coef),
                                                 abi.ptr(res), pen), self._ctx, "set_constraints")
        self._constraints_dirty = False

    def set_nodal_loads(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64).ravel()
        abi.check(self._lib.lmtg_set_nodal_loads(self._ctx, abi.ptr(F)), self._ctx, "nodal loads")

    def add_skin_traction(self, faces, traction):
        faces = np.ascontiguousarray(faces, dtype=np.uint32)
        t = np.ascontiguousarray(traction, dtype=np.float64)
        abi.check(self._lib.lmtg_add_skin_traction(self._ctx, faces.shape[0], abi.ptr(faces), abi.ptr(t)),
                  self._ctx, "skin traction")

    def add_skin_pressure(self, faces, p):
        """p dS_normal on skin faces (the unit normal of the face's node order)."""
        faces = np.ascontiguousarray(faces, dtype=np.uint32)
        abi.check(self._lib.lmtg_add_skin_pressure(self._ctx, faces.shape[0], abi.ptr(faces), float(p)),
                  self._ctx, "skin pressure")

    # -- the hot path -------------------------------------------------------------------------
    def allocate_matrices(self):
        nnz = ctypes.c_uint64(0)
        abi.check(self._lib.lmtg_allocate_matrices(self._ctx, ctypes.byref(nnz)), self._ctx,
                  "allocate_matrices")
        self.nnz_lower = nnz.value
        self.allocated = True
        self._have_matrix = False
        self._material_dirty = True
        self._constraints_dirty = bool(self._constraints)

    def assemble(self, assemble_mat=True, assemble_vec=True, mixed=False, native_fp32=False):
        if not self.allocated:
            self.allocate_matrices()
        self._sync_material()
        self._sync_constraints()
        if self.levenberg_marquadt != self._lm_synced:
            abi.check(self._lib.lmtg_set_levenberg_marquadt(self._ctx, float(self.levenberg_marquadt)), self._ctx,
                      "levenberg_marquadt")
            self._lm_synced = self.levenberg_marquadt
        flags = 0
        if assemble_mat:
            flags |= abi.ASM_MAT32_NATIVE if native_fp32 else (abi.ASM_MAT64 | (abi.ASM_MAT32 if mixed else 0))
        if assemble_vec:
            flags |= abi.ASM_VEC
        abi.check(self._lib.lmtg_assemble(self._ctx, flags), self._ctx, "assemble")
        if assemble_mat:
            self._have_matrix = (mixed or native_fp32, True)

    def solve_system(self, iterative_criterium=None, mode="fp64", criterion="rel_residual",
                     maxit=100000, timeout_s=600.0):
        """solve_system(crit): PCG on the assembled system.  criterion: 'rel_residual'
        (|b-Ku|/|b|), 'norm_inf_delta', 'norm2_delta', 'abs_residual_inf'.  A criterium of 0
        (the reference's direct solve) runs the FP64 PCG to a 1e-14 relative residual."""
        crit = self.default_iterative_criterium if iterative_criterium is None else iterative_criterium
        if crit == 0:
            crit, criterion = 1e-14, "rel_residual"
        kind = {"rel_residual": abi.CRIT_REL_RESIDUAL, "norm_inf_delta": abi.CRIT_NORM_INF_DELTA,
                "norm2_delta": abi.CRIT_NORM2_DELTA, "abs_residual_inf": abi.CRIT_ABS_RESIDUAL_INF}[criterion]
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        st = abi.SolveStats()
        abi.check(self._lib.lmtg_solve_system(self._ctx, m, kind, float(crit), int(maxit),
                                              float(timeout_s), ctypes.byref(st)), self._ctx, "solve_system")
        self.last_stats = st.as_dict()
        return self.last_stats

    def solve(self, iterative_criterium=None, mode="fp64", **kw):
        """solve(): assemble(mat, vec) then solve_system (formulation.h:1517-1568); with
        assume_constant_matrix, a matrix already assembled for this mode is kept."""
        keep = (self.assume_constant_matrix and self._have_matrix
                and (mode != "mixed" or self._have_matrix[0]) and not self._material_dirty
                and not self._constraints_dirty and self.levenberg_marquadt == self._lm_synced)
        self.assemble(not keep, True, mixed=(mode == "mixed"))
        return self.solve_system(iterative_criterium, mode=mode, **kw)

    # -- results ------------------------------------------------------------------------------
    def get_result(self):
        u = np.zeros(self.n)
        abi.check(self._lib.lmtg_get_result(self._ctx, abi.ptr(u)), self._ctx, "get_result")
        return u

    def element_fields(self, u=None):
        """call_after_solve: per element (ne x 13) epsilon[6] (tensor shear, 11 22 33 12 13 23),
        sigma[6] and tr(epsilon) at var_inter = 0.5, from u (default: the current result)."""
        out = np.zeros((self.ne, 13))
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        abi.check(self._lib.lmtg_element_fields(self._ctx, abi.ptr(uu), abi.ptr(out)), self._ctx, "element_fields")
        return {"epsilon": out[:, :6], "sigma": out[:, 6:12], "tr_epsilon": out[:, 12]}

    def set_result(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        abi.check(self._lib.lmtg_set_result(self._ctx, abi.ptr(u)), self._ctx, "set_result")

    def get_sollicitation(self):
        F = np.zeros(self.n)
        abi.check(self._lib.lmtg_get_sollicitation(self._ctx, abi.ptr(F)), self._ctx, "get_sollicitation")
        return F

    def get_mat(self):
        """The assembled matrix as the reference's Sym SparseLine storage: lower CSR
        (rowptr, col, val), each row ascending with the diagonal last."""
        rowptr = np.zeros(self.n + 1, dtype=np.uint64)
        col = np.zeros(self.nnz_lower, dtype=np.uint32)
        val = np.zeros(self.nnz_lower)
        abi.check(self._lib.lmtg_get_matrix_lower(self._ctx, abi.ptr(rowptr), abi.ptr(col), abi.ptr(val)),
                  self._ctx, "get_mat")
        return rowptr, col, val

    def element_matrices(self, e0=0, count=1, precision=0):
        nd = 3 * self.npe
        Ke = np.zeros((count, nd, nd))
        abi.check(self._lib.lmtg_get_element_matrices(self._ctx, precision, e0, count, abi.ptr(Ke)),
                  self._ctx, "element matrices")
        return Ke

    def spmv(self, x, precision=0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        abi.check(self._lib.lmtg_spmv(self._ctx, precision, abi.ptr(x), abi.ptr(y)), self._ctx, "spmv")
        return y

    # -- sensitivities -------------------------------------------------------------------------
    def set_volume_force(self, f_vol, density=7800.0):
        """Volume force density * f_vol (formulation_elasticity_iso.py:4,7; density's default
        7800 as there)."""
        f = np.ascontiguousarray(f_vol, dtype=np.float64)
        abi.check(self._lib.lmtg_set_volume_force(self._ctx, float(density), abi.ptr(f)), self._ctx,
                  "set_volume_force")

    def set_nodal_springs(self, coef, target=None):
        """dep_imp_coef_0 springs: coef per node, target displacement (3 per node) or 0."""
        k = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float64).ravel()
        abi.check(self._lib.lmtg_set_nodal_springs(self._ctx, abi.ptr(k), abi.ptr(t)), self._ctx, "set_nodal_springs")

    def set_inner_reduction(self, inner_reduction):
        """Recursive-residual reduction of each FP32 segment of the mixed solvers (default 0.01)."""
        abi.check(self._lib.lmtg_set_inner_reduction(self._ctx, float(inner_reduction)), self._ctx,
                  "set_inner_reduction")

    def set_preconditioner(self, kind):
        """'amg' (default: aggregation multigrid W-cycle) or 'block_jacobi' for the FP32 inner PCG of
        the mixed solve; the FP64 PCG always uses block Jacobi."""
        k = {"block_jacobi": abi.PREC_BLOCK_JACOBI, "amg": abi.PREC_AMG}[kind]
        abi.check(self._lib.lmtg_set_preconditioner(self._ctx, k), self._ctx, "set_preconditioner")

    def amg_info(self):
        """The multigrid hierarchy of the last mixed solve: per level unknowns, stored blocks,
        smoothing weight and lambda_max(D^-1 K); host setup times (structure, last numeric)."""
        lv = ctypes.c_int()
        nd, nb = (ctypes.c_uint64 * 8)(), (ctypes.c_uint64 * 8)()
        om, la = (ctypes.c_double * 8)(), (ctypes.c_double * 8)()
        sm, nm = ctypes.c_double(), ctypes.c_double()
        ph = (ctypes.c_double * 5)()
        abi.check(self._lib.lmtg_amg_info(self._ctx, ctypes.byref(lv), nd, nb, om, la, ctypes.byref(sm),
                                          ctypes.byref(nm), ph), self._ctx, "amg_info")
        n = lv.value
        return {"levels": n, "ndof": list(nd)[:n], "nnz_blocks": list(nb)[:n], "omega": list(om)[:n],
                "lambda_max": list(la)[:n], "structure_ms": sm.value, "numeric_ms": nm.value,
                "structure_phase_ms": dict(zip(["pattern_modes", "aggregation", "tentative", "coarse_pattern",
                                                "uploads"], list(ph)))}

    def spmv_info(self):
        """FP32 SpMV kind in use, the autotuned kind and the autotuner's per-kind times (ms)."""
        k, t = ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_double * 3)()
        abi.check(self._lib.lmtg_spmv_info(self._ctx, ctypes.byref(k), ctypes.byref(t), ms), self._ctx, "spmv_info")
        return {"kind": k.value, "tuned": t.value, "tune_ms": list(ms)}

    def profile_amg_kernels(self, iters=10):
        """Per-stage device times (ms) of one multigrid-preconditioned FP32 iteration."""
        ms = (ctypes.c_double * 8)()
        abi.check(self._lib.lmtg_profile_amg_kernels(self._ctx, int(iters), ms), self._ctx, "profile_amg_kernels")
        names = ["spmv", "update", "residual0", "restrict0", "coarse", "prolong0", "smooth0", "direction"]
        return dict(zip(names, list(ms)))

    def set_spmv_kind(self, kind):
        """FP32 PCG SpMV: 0 = warp per row pair, 1, 2 = matrix streamed by bulk copies (TMA) with 4 / 5 CTAs per
        SM, -1 (default) = autotuned at the first FP32 solve."""
        abi.check(self._lib.lmtg_set_spmv_kind(self._ctx, int(kind)), self._ctx, "set_spmv_kind")

    def set_penalty_scale(self, max_diag):
        """Hold the penalty scale at max_diag (0 = recompute max|diag K| at each assembly)."""
        abi.check(self._lib.lmtg_set_penalty_scale(self._ctx, float(max_diag)), self._ctx, "penalty scale")

    def get_penalty_scale(self):
        v = ctypes.c_double()
        abi.check(self._lib.lmtg_get_penalty_scale(self._ctx, ctypes.byref(v)), self._ctx, "penalty scale")
        return v.value

    def adjoint_grad(self, objective="compliance", target=None, weights=None, mode="mixed",
                     tol=1e-10, maxit=100000, timeout_s=600.0):
        """Adjoint gradient dJ/dE (one value per element) of the compliance F.u, of the misfit
        1/2 sum w (u - t)^2, or of the linear objective c.u (c passed as target) at the current
        solution; returns (J, dJdE, adjoint solve stats)."""
        obj = {"compliance": abi.OBJ_COMPLIANCE, "misfit": abi.OBJ_MISFIT,
               "linear": abi.OBJ_LINEAR}[objective]
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        g = np.zeros(self.ne)
        J = ctypes.c_double()
        st = abi.SolveStats()
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        abi.check(self._lib.lmtg_adjoint_grad(self._ctx, obj, abi.ptr(t), abi.ptr(w), m, float(tol),
                                              int(maxit), float(timeout_s), ctypes.byref(J), abi.ptr(g),
                                              ctypes.byref(st)), self._ctx, "adjoint_grad")
        return J.value, g, st.as_dict()

    def stream_handle(self):
        """cudaStream_t of this formulation (every kernel and copy is issued on it)."""
        s = ctypes.c_void_p()
        abi.check(self._lib.lmtg_get_stream(self._ctx, ctypes.byref(s)), self._ctx, "get_stream")
        return s.value

    def launch_count(self):
        n = ctypes.c_uint64()
        abi.check(self._lib.lmtg_get_launch_count(self._ctx, ctypes.byref(n)), self._ctx, "launch count")
        return n.value

    def profile_pcg_kernels(self, precision=1, iters=20):
        """Mean device ms of the fused SpMV kernel and of the update kernel (CUDA events)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        abi.check(self._lib.lmtg_profile_pcg_kernels(self._ctx, precision, iters, ctypes.byref(a),
                                                     ctypes.byref(b)), self._ctx, "profile")
        return a.value, b.value

    def close(self):
        if self._ctx:
            self._lib.lmtg_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
