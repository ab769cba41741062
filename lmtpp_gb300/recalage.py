"""Python mirror of formulation recalage (formulations/formulation_recalage.py) on the GPU.

    f = Recalage(pos, conn)                     # a formulation recalage on a Hexa / Tetra_10 mesh
    f.elastic_modulus = 1.0; f.poisson_ratio = 0.3; f.density = 1.0
    f.gamma = 0.5; f.r = 0.5; f.omega = 1.0
    f.Ud = Ud; f.Ud_valid = np.ones(nn)         # measured displacement and its validity per node
    f.add_constraint("node[0].V[1]", 1e5)       # penalty constraint on an unknown of V
    f.solve(iterative_criterium=1e-12)          # assemble + solve_system
    U, V, W = f.get_result()                    # nn x 3 each

The system is the Hessian of the recalage energy with minus its gradient at 0 as right-hand
side (use_test_functions = False), on unknowns ordered per node U, V, W then component
(DOF 9 node + 3 field + component).  Failures raise LmtgError.
"""
import ctypes
import re

import numpy as np

from . import abi

FIELDS = "UVW"

_CONSTRAINT = re.compile(
    r"^\s*(?:(?P<coef>[-+]?[0-9.eE+-]+)\s*\*\s*)?node\[(?P<node>\d+)\]\.(?P<f>[UVW])\[(?P<d>\d)\]"
    r"\s*(?:(?P<sign>[-+])\s*(?P<val>[0-9.eE+-]+))?\s*$")


def parse_constraint(txt):
    """'[c*]node[i].F[d] [- v]' (F one of U, V, W) -> (i, f, d, c, v), the coefficient and right side
    the reference's Constraint extracts (include/formulation/constraint.h:46-93)."""
    m = _CONSTRAINT.match(txt)
    if not m:
        raise abi.LmtgError(abi.ERR_UNSUPPORTED, "only linear single-unknown constraints: %r" % txt)
    coef = float(m.group("coef")) if m.group("coef") else 1.0
    val = 0.0
    if m.group("val"):
        val = float(m.group("val")) * (1.0 if m.group("sign") == "-" else -1.0)
    return int(m.group("node")), FIELDS.index(m.group("f")), int(m.group("d")), coef, val


class Recalage:
    """One recalage formulation on a Hexa8 or Tetra10 mesh, resident on one GPU.  Variable
    defaults are the formulation's (formulation_recalage.py:2-21)."""

    def __init__(self, pos, conn, device=0):
        conn = np.asarray(conn)
        elem = {8: abi.ELEM_HEXA8, 10: abi.ELEM_TETRA10}.get(conn.shape[1])
        if elem is None:
            raise abi.LmtgError(abi.ERR_UNSUPPORTED, "elements with %d nodes are not supported" % conn.shape[1])
        self._elem = elem
        self._lib = abi.load()
        self._ctx = ctypes.c_void_p()
        abi.check(self._lib.lmtg_create(device, ctypes.byref(self._ctx)), None, "lmtg_create")
        self.pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.uint32)
        self.nn, self.ne = self.pos.shape[0], self.conn.shape[0]
        self.n = 9 * self.nn
        self.elastic_modulus = 210e9
        self.poisson_ratio = 0.33
        self.density = 7800.0
        self.gamma = 0.5
        self.r = 0.5
        self.omega = 187.0
        self.Ud = np.zeros((self.nn, 3))
        self.Ud_valid = np.zeros(self.nn)
        self.default_iterative_criterium = 1e-10
        self._constraints = []  # (dof, coef, res, penalty)
        self._state = None  # variables the device system was set up with
        self.last_stats = None

    def add_constraint(self, txt, penalty_value):
        node, f, d, coef, val = parse_constraint(txt)
        if node >= self.nn or d > 2:
            raise abi.LmtgError(abi.ERR_ARG, "constraint on a missing node/component")
        self.add_constraints([9 * node + 3 * f + d], penalty_value, [coef], [val])

    def add_constraints(self, dofs, penalty_value, coefs=None, res=None):
        """Many constraints at once on DOFs 9 node + 3 field + component."""
        dofs = np.asarray(dofs, dtype=np.int64).ravel()
        coefs = np.ones(dofs.shape[0]) if coefs is None else np.asarray(coefs, dtype=np.float64).ravel()
        res = np.zeros(dofs.shape[0]) if res is None else np.asarray(res, dtype=np.float64).ravel()
        if dofs.size and (dofs.min() < 0 or dofs.max() >= self.n):
            raise abi.LmtgError(abi.ERR_ARG, "constraint on a missing DOF")
        self._constraints.append((dofs, coefs, res, float(penalty_value)))
        self._state = None

    def _variables(self):
        if np.size(self.elastic_modulus) != 1 or np.size(self.poisson_ratio) != 1:
            raise abi.LmtgError(abi.ERR_ARG, "elastic_modulus and poisson_ratio of recalage are global variables")
        return (float(np.ravel(self.elastic_modulus)[0]), float(np.ravel(self.poisson_ratio)[0]), float(self.density),
                float(self.gamma), float(self.r), float(self.omega),
                np.ascontiguousarray(self.Ud, dtype=np.float64).reshape(-1),
                np.ascontiguousarray(self.Ud_valid, dtype=np.float64).reshape(-1), len(self._constraints))

    def _setup(self):
        v = self._variables()
        if self._state is not None and all(
                (np.array_equal(a, b) if isinstance(a, np.ndarray) else a == b) for a, b in zip(v, self._state)):
            return
        E, nu, rho, gamma, r, omega, Ud, Uv, _ = v
        if Ud.shape[0] != 3 * self.nn or Uv.shape[0] != self.nn:
            raise abi.LmtgError(abi.ERR_ARG, "Ud needs nn x 3 values, Ud_valid nn")
        lib, ctx = self._lib, self._ctx
        abi.check(lib.lmtg_mesh_set(ctx, self._elem, self.nn, abi.ptr(self.pos), self.ne, abi.ptr(self.conn)), ctx,
                  "mesh_set")
        Ea = np.array([E])
        abi.check(lib.lmtg_material_set(ctx, abi.ptr(Ea), 1, nu), ctx, "material_set")
        abi.check(lib.lmtg_recalage_setup(ctx, rho, omega, gamma, r, abi.ptr(Ud), abi.ptr(Uv)), ctx,
                  "recalage_setup")
        if self._constraints:
            pens = {c[3] for c in self._constraints}
            if len(pens) > 1:
                raise abi.LmtgError(abi.ERR_UNSUPPORTED, "one penalty value per formulation")
            cat = lambda k, t: np.ascontiguousarray(np.concatenate([c[k] for c in self._constraints]), dtype=t)
            dof, coef, res = cat(0, np.uint32), cat(1, np.float64), cat(2, np.float64)
            abi.check(lib.lmtg_set_constraints(ctx, dof.shape[0], abi.ptr(dof), abi.ptr(coef), abi.ptr(res),
                                               pens.pop()), ctx, "set_constraints")
        self._state = v
        sizes = [ctypes.c_uint64() for _ in range(4)]
        abi.check(lib.lmtg_get_sizes(ctx, *[ctypes.byref(s) for s in sizes]), ctx, "get_sizes")
        nblk = sizes[3].value
        self.nnz_lower = 9 * (nblk - 3 * self.nn) // 2 + 6 * 3 * self.nn

    def assemble(self):
        self._setup()
        abi.check(self._lib.lmtg_recalage_assemble(self._ctx), self._ctx, "recalage_assemble")

    def solve_system(self, iterative_criterium=None, mode="fp64", maxit=100000, timeout_s=600.0):
        crit = self.default_iterative_criterium if iterative_criterium is None else iterative_criterium
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        st = abi.SolveStats()
        abi.check(self._lib.lmtg_solve_system(self._ctx, m, abi.CRIT_REL_RESIDUAL, float(crit), int(maxit),
                                              float(timeout_s), ctypes.byref(st)), self._ctx, "solve_system")
        self.last_stats = st.as_dict()
        return self.last_stats

    def solve(self, iterative_criterium=None, mode="fp64", **kw):
        self.assemble()
        return self.solve_system(iterative_criterium, mode=mode, **kw)

    def get_vector(self):
        """The solution as the reference stores it: 9 nn values, per node U, V, W then component."""
        x = np.zeros(self.n)
        abi.check(self._lib.lmtg_get_result(self._ctx, abi.ptr(x)), self._ctx, "get_result")
        return x

    def get_result(self):
        x = self.get_vector().reshape(self.nn, 3, 3)
        return x[:, 0].copy(), x[:, 1].copy(), x[:, 2].copy()

    def get_sollicitation(self):
        F = np.zeros(self.n)
        abi.check(self._lib.lmtg_get_sollicitation(self._ctx, abi.ptr(F)), self._ctx, "get_sollicitation")
        return F

    def get_mat(self):
        """Lower CSR (rowptr, col, val) of the assembled Hessian, rows ascending, diagonal last."""
        rowptr = np.zeros(self.n + 1, dtype=np.uint64)
        col = np.zeros(self.nnz_lower, dtype=np.uint32)
        val = np.zeros(self.nnz_lower)
        abi.check(self._lib.lmtg_get_matrix_lower(self._ctx, abi.ptr(rowptr), abi.ptr(col), abi.ptr(val)),
                  self._ctx, "get_mat")
        return rowptr, col, val

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._lib.lmtg_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
