"""Identification driver: Gauss-Newton on zone moduli (FormulationFit of
include/formulation/FormulationFit.h:7-80) on top of a Formulation, through
lmtg_fit_zone_moduli."""
import ctypes

import numpy as np

from . import abi


class FormulationFit:
    """FormulationFit(f): the reference's attributes levenberg_marq (0), relaxation (1),
    conv (1e-4); exec() identifies E per zone and fills history, residual_history and
    sensitivity_after_fit."""

    def __init__(self, f):
        self.f = f
        self.levenberg_marq = 0.0
        self.relaxation = 1.0
        self.conv = 1e-4
        self.max_iter = 20
        self.history = []
        self.residual_history = []
        self.sensitivity_after_fit = None

    def exec(self, exp_val, zones, p0, exp_weight=None, sens_val=None, mode="mixed", tol=1e-12, maxit=200000):
        """Fit p (one modulus per zone, E_e = p[zones[e]]) to the displacement exp_val with the
        diagonal weight exp_weight (the reference's exp_mat).  Returns p."""
        f = self.f
        if not f.allocated:
            f.allocate_matrices()
        f._sync_material()
        f._sync_constraints()
        zones = np.ascontiguousarray(zones, dtype=np.uint32)
        p = np.ascontiguousarray(p0, dtype=np.float64).copy()
        nz = p.shape[0]
        u = np.ascontiguousarray(exp_val, dtype=np.float64)
        w = None if exp_weight is None else np.ascontiguousarray(exp_weight, dtype=np.float64)
        sv = None if sens_val is None else np.ascontiguousarray(sens_val, dtype=np.float64)
        hist = np.zeros(self.max_iter + 1)
        res = np.zeros(self.max_iter + 1)
        sens = np.zeros(nz)
        n_it = ctypes.c_int()
        m = {"fp64": abi.SOLVE_PCG_F64, "mixed": abi.SOLVE_MIXED_IR}[mode]
        abi.check(f._lib.lmtg_fit_zone_moduli(f._ctx, nz, abi.ptr(zones), abi.ptr(p), abi.ptr(u), abi.ptr(w),
                                              abi.ptr(sv), float(self.relaxation), float(self.levenberg_marq),
                                              float(self.conv), int(self.max_iter), m, float(tol), int(maxit),
                                              abi.ptr(hist), abi.ptr(res), abi.ptr(sens), ctypes.byref(n_it)),
                  f._ctx, "fit_zone_moduli")
        k = n_it.value
        self.history = hist[:k].tolist()
        self.residual_history = res[:k].tolist()
        self.sensitivity_after_fit = sens
        # the context now holds E = p[zones]
        f._E = np.ascontiguousarray(p[zones], dtype=np.float64)
        return p
