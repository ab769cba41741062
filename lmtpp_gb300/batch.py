"""Batches of independent elasticity meshes solved together (lmtg_batch_* of include/lmtg.h).

The reference runs one Formulation per mesh and one solve per right-hand side
(include/formulation/formulation_ancestor.h:64).  BatchFormulation concatenates the meshes into
one context -- one block-diagonal matrix, per-mesh penalty scale max|diag| -- and solves up to
four right-hand sides for every mesh in one batched PCG.
"""
import ctypes

import numpy as np

from . import abi
from .formulation import Formulation


def concat_meshes(meshes):
    """[(pos, conn), ...] -> (pos, conn, node_off, elem_off) with conn renumbered globally."""
    pos = np.concatenate([np.asarray(p, dtype=np.float64) for p, _ in meshes])
    node_off = np.zeros(len(meshes) + 1, dtype=np.uint64)
    elem_off = np.zeros(len(meshes) + 1, dtype=np.uint64)
    conns = []
    for m, (p, c) in enumerate(meshes):
        conns.append(np.asarray(c, dtype=np.uint64) + node_off[m])
        node_off[m + 1] = node_off[m] + p.shape[0]
        elem_off[m + 1] = elem_off[m] + c.shape[0]
    conn = np.concatenate(conns).astype(np.uint32)
    return pos, conn, node_off, elem_off


def shard(costs, rank, world):
    """Contiguous share of a batch for one of `world` replicas: the meshes [a, b) whose
    cumulative cost (e.g. DOF count) falls in this rank's 1/world of the total.  Every mesh is
    in exactly one share; no data crosses ranks (the systems are independent)."""
    c = np.cumsum(np.asarray(costs, dtype=np.float64))
    if c.size == 0:
        return 0, 0
    total = c[-1]
    cuts = [0] + [int(np.searchsorted(c, total * k / world, side="left")) for k in range(1, world)] + [c.size]
    for k in range(1, len(cuts)):  # keep the cuts non-decreasing
        cuts[k] = max(cuts[k], cuts[k - 1])
    return cuts[rank], cuts[rank + 1]


class BatchFormulation(Formulation):
    """Many elasticity_iso formulations (independent meshes of one element type) in one context."""

    def __init__(self, meshes, device=0):
        pos, conn, self.node_off, self.elem_off = concat_meshes(meshes)
        super().__init__(pos, conn, device)
        self.nsys = len(meshes)
        self._nu_elem = None
        abi.check(self._lib.lmtg_batch_set(self._ctx, self.nsys, abi.ptr(self.node_off)), self._ctx, "batch_set")

    def set_materials(self, E, nu):
        """Young's modulus and Poisson ratio per mesh (arrays of nsys)."""
        counts = np.diff(self.elem_off).astype(np.int64)
        self.elastic_modulus = np.repeat(np.asarray(E, dtype=np.float64), counts)
        self._nu_elem = np.ascontiguousarray(np.repeat(np.asarray(nu, dtype=np.float64), counts))
        self._material_dirty = True

    def _sync_material(self):
        dirty = self._material_dirty
        super()._sync_material()
        if dirty and self._nu_elem is not None:
            abi.check(self._lib.lmtg_material_set_nu(self._ctx, abi.ptr(self._nu_elem), self.ne), self._ctx,
                      "material_set_nu")

    def dofs(self, m):
        """Global DOF slice of mesh m."""
        return slice(3 * int(self.node_off[m]), 3 * int(self.node_off[m + 1]))

    def solve_batch(self, B, mode="mixed", tol=1e-10, maxit=100000, timeout_s=600.0):
        """Solves K X[r] = B[r] for every mesh and r < nrhs (B: nrhs x ndof, nrhs <= 4).  Returns
        (X, stats, pair_iters[nsys, nrhs])."""
        B = np.ascontiguousarray(np.atleast_2d(B), dtype=np.float64)
        nrhs = B.shape[0]
        abi.check(self._lib.lmtg_batch_set_rhs(self._ctx, nrhs, abi.ptr(B)), self._ctx, "batch_set_rhs")
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        st = abi.SolveStats()
        its = np.zeros((self.nsys, nrhs), dtype=np.int32)
        abi.check(self._lib.lmtg_batch_solve(self._ctx, m, float(tol), int(maxit), float(timeout_s),
                                             ctypes.byref(st), abi.ptr(its)), self._ctx, "batch_solve")
        self.last_stats = st.as_dict()
        X = np.zeros_like(B)
        abi.check(self._lib.lmtg_batch_get_result(self._ctx, abi.ptr(X)), self._ctx, "batch_get_result")
        return X, self.last_stats, its

    def set_options(self, tile_rows=0, variant=-1):
        """Fixed rows per tile and SpMV variant (0, 1, 2 = bulk copies, FP32); 0 / -1: autotuned."""
        abi.check(self._lib.lmtg_batch_set_options(self._ctx, int(tile_rows), int(variant)), self._ctx,
                  "batch_set_options")

    def batch_info(self):
        rows = ctypes.c_int()
        var = ctypes.c_int()
        nt = ctypes.c_uint64()
        ms = np.zeros(12)
        abi.check(self._lib.lmtg_batch_info(self._ctx, ctypes.byref(rows), ctypes.byref(var), ctypes.byref(nt),
                                            abi.ptr(ms)), self._ctx, "batch_info")
        sizes = ((16, 32, 64, 128), (16, 32, 64, 128), (128, 256, 512, 1024))
        return {"tile_rows": rows.value, "variant": var.value, "ntiles": nt.value,
                "tuned_spmv_ms": {"v%d_r%d" % (v, r): ms[4 * v + i] for v in (0, 1, 2)
                                  for i, r in enumerate(sizes[v])}}
