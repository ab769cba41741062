"""Python mirror of the transient heat-diffusion path (formulation difftherm on Triangle_6).

    pos, conn = make_rect_triangle6(1025)               # make_rect(m, Triangle_6(), 0, 1, 1025)
    d = Diffusion(pos, conn)
    d.setup(k, rho_c=1.0, dt=1e-4, theta=1.0, dirichlet=boundary_nodes(pos))
    d.set_state(T0); d.run(100)                         # ProblemAncestor::iteration x 100
    J, dJdk = d.adjoint_misfit(T0, target, 100, checkpoint_every=10)

The matrices of the theta scheme (A = M/dt + theta K, B = M/dt - (1 - theta) K; theta = 1/2 is the
reference's midpoint-in-time integration) are assembled once, as the reference does with
assume_constant_matrix (include/formulation/problem_ancestor.h:41-126).
"""
import ctypes

import numpy as np

from . import abi


def make_rect_triangle6(nb_points, X0=(0.0, 0.0), X1=(1.0, 1.0)):
    """make_rect(m, Triangle_6(), X0, X1, nb_points) (include/mesh/make_rect.h:141-170)."""
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 2, dtype=np.uint32)
    x0 = np.ascontiguousarray(X0, dtype=np.float64)
    x1 = np.ascontiguousarray(X1, dtype=np.float64)
    lib = abi.load()
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    abi.check(lib.lmtg_make_rect_triangle6(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), ctypes.byref(nn),
                                           ctypes.byref(ne), None, None), None, "make_rect_triangle6")
    pos = np.zeros((nn.value, 2))
    conn = np.zeros((ne.value, 6), dtype=np.uint32)
    abi.check(lib.lmtg_make_rect_triangle6(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), ctypes.byref(nn),
                                           ctypes.byref(ne), abi.ptr(pos), abi.ptr(conn)), None,
              "make_rect_triangle6")
    return pos, conn


def boundary_nodes(pos, eps=1e-9):
    return np.ascontiguousarray(np.nonzero((pos[:, 0] < eps) | (pos[:, 1] < eps) | (pos[:, 0] > 1 - eps)
                                           | (pos[:, 1] > 1 - eps))[0], dtype=np.uint32)


TRIANGLE6_EDGES = [[0, 1, 3], [1, 2, 4], [2, 0, 5]]  # Bar_3 children (formulations/element_Triangle_6.py:9-13)


def edges_on(pos, conn, axis, value, eps=1e-9):
    """Bar_3 skin edges (end, end, middle) of Triangle_6 elements lying on pos[:, axis] = value."""
    q = np.asarray(conn)[:, TRIANGLE6_EDGES]  # ne x 3 x 3
    on = np.all(np.abs(pos[q, axis] - value) < eps, axis=2)
    return np.ascontiguousarray(q[on], dtype=np.uint32)


class Diffusion:
    """Transient heat diffusion on a Triangle_6 mesh, resident on one GPU."""

    def __init__(self, pos, conn, device=0):
        self._lib = abi.load()
        self._ctx = ctypes.c_void_p()
        abi.check(self._lib.lmtg_create(device, ctypes.byref(self._ctx)), None, "lmtg_create")
        self.pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.uint32)
        self.nn, self.ne = self.pos.shape[0], self.conn.shape[0]
        abi.check(self._lib.lmtg_diff_mesh_set(self._ctx, self.nn, abi.ptr(self.pos), self.ne,
                                               abi.ptr(self.conn)), self._ctx, "diff_mesh_set")
        self.last_stats = None

    def setup(self, conductivity, rho_c=1.0, dt=1e-4, theta=0.5, dirichlet=None, penalty=1e5):
        k = np.ascontiguousarray(np.atleast_1d(conductivity), dtype=np.float64)
        bnd = np.ascontiguousarray(dirichlet if dirichlet is not None else [], dtype=np.uint32)
        abi.check(self._lib.lmtg_diff_setup(self._ctx, abi.ptr(k), k.shape[0], float(rho_c), float(dt),
                                            float(theta), bnd.shape[0], abi.ptr(bnd) if bnd.size else None,
                                            float(penalty)), self._ctx, "diff_setup")

    def set_sources(self, Q=None, Qs=None):
        """Constant volume source Q (nodal field) and nodal source Qs of difftherm."""
        q = None if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        qs = None if Qs is None else np.ascontiguousarray(Qs, dtype=np.float64)
        abi.check(self._lib.lmtg_diff_set_sources(self._ctx, abi.ptr(q), abi.ptr(qs)), self._ctx, "set_sources")

    def set_convection(self, edges, H, t0=0.0):
        """Skin convection H (T - t0) on Bar_3 edges (end, end, middle); H: one value or one per
        edge.  Call after setup()."""
        e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 3)
        h = np.ascontiguousarray(np.atleast_1d(H), dtype=np.float64)
        abi.check(self._lib.lmtg_diff_set_convection(self._ctx, e.shape[0], abi.ptr(e), abi.ptr(h), h.shape[0],
                                                     float(t0)), self._ctx, "set_convection")

    def set_solver(self, mode):
        """'fp64' (FP64 Jacobi-PCG) or 'mixed' (FP32 PCG with FP64 residual replacement)."""
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        abi.check(self._lib.lmtg_diff_set_solver(self._ctx, m), self._ctx, "set_solver")

    def set_preconditioner(self, kind):
        """Preconditioner of the mixed step solver's FP32 PCG: 'amg' (default: a W-cycle of the
        scalar aggregation multigrid, from 3000 unknowns) or 'jacobi'."""
        k = {"jacobi": abi.PREC_BLOCK_JACOBI, "amg": abi.PREC_AMG}[kind]
        abi.check(self._lib.lmtg_set_preconditioner(self._ctx, k), self._ctx, "set_preconditioner")

    def set_inner_reduction(self, inner_reduction):
        """Recursive-residual reduction of each FP32 segment of the mixed step solver (default 0.01)."""
        abi.check(self._lib.lmtg_set_inner_reduction(self._ctx, float(inner_reduction)), self._ctx,
                  "set_inner_reduction")

    def set_spmv_kind(self, kind):
        """FP32 SpMV of the mixed step solver: 0 = warp-streamed CSR, any other kind (default -1)
        = the matrix streamed through shared memory by bulk copies (TMA)."""
        abi.check(self._lib.lmtg_set_spmv_kind(self._ctx, int(kind)), self._ctx, "set_spmv_kind")

    def set_penalty_scale(self, max_diag):
        abi.check(self._lib.lmtg_set_penalty_scale(self._ctx, float(max_diag)), self._ctx, "penalty scale")

    def get_penalty_scale(self):
        v = ctypes.c_double()
        abi.check(self._lib.lmtg_get_penalty_scale(self._ctx, ctypes.byref(v)), self._ctx, "penalty scale")
        return v.value

    def set_state(self, T):
        T = np.ascontiguousarray(T, dtype=np.float64)
        abi.check(self._lib.lmtg_diff_set_state(self._ctx, abi.ptr(T)), self._ctx, "set_state")

    def get_state(self):
        T = np.zeros(self.nn)
        abi.check(self._lib.lmtg_diff_get_state(self._ctx, abi.ptr(T)), self._ctx, "get_state")
        return T

    def run(self, nsteps, tol=1e-12, maxit=100000):
        st = abi.SolveStats()
        abi.check(self._lib.lmtg_diff_run(self._ctx, int(nsteps), float(tol), int(maxit), ctypes.byref(st)),
                  self._ctx, "diff_run")
        self.last_stats = st.as_dict()
        return self.last_stats

    def adjoint_misfit(self, T0, target, nsteps, checkpoint_every=10, tol=1e-12, maxit=100000):
        """J = 1/2 |T_N - target|^2 after nsteps from T0 and dJ/dk per element."""
        self.set_state(T0)
        t = np.ascontiguousarray(target, dtype=np.float64)
        g = np.zeros(self.ne)
        J = ctypes.c_double()
        st = abi.SolveStats()
        abi.check(self._lib.lmtg_diff_adjoint_misfit(self._ctx, int(nsteps), int(checkpoint_every), abi.ptr(t),
                                                     float(tol), int(maxit), ctypes.byref(J), abi.ptr(g),
                                                     ctypes.byref(st)), self._ctx, "diff_adjoint")
        self.last_stats = st.as_dict()
        return J.value, g

    def get_matrices(self):
        nnz = ctypes.c_uint64()
        nb = ctypes.c_uint64()
        self._lib.lmtg_get_sizes(self._ctx, None, None, None, ctypes.byref(nb))
        nlow = (nb.value - self.nn) // 2 + self.nn
        rowptr = np.zeros(self.nn + 1, dtype=np.uint64)
        col = np.zeros(nlow, dtype=np.uint32)
        A, B = np.zeros(nlow), np.zeros(nlow)
        abi.check(self._lib.lmtg_diff_get_matrices(self._ctx, abi.ptr(rowptr), abi.ptr(col), abi.ptr(A),
                                                   abi.ptr(B)), self._ctx, "diff_get_matrices")
        return rowptr, col, A, B

    def close(self):
        if self._ctx:
            self._lib.lmtg_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
