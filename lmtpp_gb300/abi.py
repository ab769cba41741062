"""ctypes binding of liblmtg.so (the C ABI declared in include/lmtg.h).

The library is the product: there is no CPU fallback.  load() raises if the shared library is
missing or cannot be built, and every call checks its status code.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "lmtg.h")

OK = 0
ERR_ARG, ERR_CUDA, ERR_STATE, ERR_NOT_CONVERGED, ERR_TIMEOUT, ERR_NAN, ERR_NOMEM, ERR_UNSUPPORTED = range(1, 9)
ELEM_HEXA8, ELEM_TETRA10, ELEM_TRIANGLE6 = 8, 10, 6
ASM_MAT64, ASM_MAT32, ASM_VEC, ASM_MAT32_NATIVE = 1, 2, 4, 8
SOLVE_PCG_F64, SOLVE_MIXED_IR = 0, 1
CRIT_REL_RESIDUAL, CRIT_NORM_INF_DELTA, CRIT_NORM2_DELTA, CRIT_ABS_RESIDUAL_INF = 0, 1, 2, 3
PREC_BLOCK_JACOBI, PREC_AMG = 0, 1
OBJ_COMPLIANCE, OBJ_MISFIT, OBJ_LINEAR = 0, 1, 2

_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_i = ctypes.c_int
_d = ctypes.c_double
_cp = ctypes.c_char_p


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int),
                ("status", ctypes.c_int), ("reserved", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("device_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# name -> (restype, argtypes)
_SIGS = {
    "lmtg_create": (_i, [_i, ctypes.POINTER(_vp)]),
    "lmtg_destroy": (_i, [_vp]),
    "lmtg_last_error": (_cp, [_vp]),
    "lmtg_status_string": (_cp, [_i]),
    "lmtg_make_rect_hexa": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "lmtg_make_rect_tetra10": (_i, [_vp, _vp, _vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64), _vp, _vp]),
    "lmtg_mesh_set": (_i, [_vp, _i, _u64, _vp, _u64, _vp]),
    "lmtg_material_set": (_i, [_vp, _vp, _u64, _d]),
    "lmtg_allocate_matrices": (_i, [_vp, ctypes.POINTER(_u64)]),
    "lmtg_set_nodal_loads": (_i, [_vp, _vp]),
    "lmtg_add_skin_traction": (_i, [_vp, _u64, _vp, _vp]),
    "lmtg_add_skin_pressure": (_i, [_vp, _u64, _vp, _d]),
    "lmtg_set_constraints": (_i, [_vp, _u64, _vp, _vp, _vp, _d]),
    "lmtg_set_levenberg_marquadt": (_i, [_vp, _d]),
    "lmtg_set_volume_force": (_i, [_vp, _d, _vp]),
    "lmtg_set_nodal_springs": (_i, [_vp, _vp, _vp]),
    "lmtg_assemble": (_i, [_vp, _i]),
    "lmtg_get_matrix_lower": (_i, [_vp, _vp, _vp, _vp]),
    "lmtg_get_sollicitation": (_i, [_vp, _vp]),
    "lmtg_get_element_matrices": (_i, [_vp, _i, _u64, _u64, _vp]),
    "lmtg_solve_system": (_i, [_vp, _i, _i, _d, _i, _d, ctypes.POINTER(SolveStats)]),
    "lmtg_solve": (_i, [_vp, _i, _i, _d, _i, _d, ctypes.POINTER(SolveStats)]),
    "lmtg_get_result": (_i, [_vp, _vp]),
    "lmtg_element_fields": (_i, [_vp, _vp, _vp]),
    "lmtg_set_result": (_i, [_vp, _vp]),
    "lmtg_spmv": (_i, [_vp, _i, _vp, _vp]),
    "lmtg_get_sizes": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "lmtg_recalage_setup": (_i, [_vp, _d, _d, _d, _d, _vp, _vp]),
    "lmtg_set_preconditioner": (_i, [_vp, _i]),
    "lmtg_amg_info": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "lmtg_spmv_info": (_i, [_vp, _vp, _vp, _vp]),
    "lmtg_profile_amg_kernels": (_i, [_vp, _i, _vp]),
    "lmtg_recalage_assemble": (_i, [_vp]),
    "lmtg_get_launch_count": (_i, [_vp, ctypes.POINTER(_u64)]),
    "lmtg_make_rect_triangle6": (_i, [_vp, _vp, _vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64), _vp, _vp]),
    "lmtg_diff_mesh_set": (_i, [_vp, _u64, _vp, _u64, _vp]),
    "lmtg_diff_setup": (_i, [_vp, _vp, _u64, _d, _d, _d, _u64, _vp, _d]),
    "lmtg_diff_set_solver": (_i, [_vp, _i]),
    "lmtg_diff_set_sources": (_i, [_vp, _vp, _vp]),
    "lmtg_diff_set_convection": (_i, [_vp, _u64, _vp, _vp, _u64, _d]),
    "lmtg_diff_set_state": (_i, [_vp, _vp]),
    "lmtg_diff_get_state": (_i, [_vp, _vp]),
    "lmtg_diff_run": (_i, [_vp, _i, _d, _i, ctypes.POINTER(SolveStats)]),
    "lmtg_diff_adjoint_misfit": (_i, [_vp, _i, _i, _vp, _d, _i, ctypes.POINTER(_d), _vp,
                                      ctypes.POINTER(SolveStats)]),
    "lmtg_diff_get_matrices": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "lmtg_set_penalty_scale": (_i, [_vp, _d]),
    "lmtg_get_penalty_scale": (_i, [_vp, ctypes.POINTER(_d)]),
    "lmtg_adjoint_grad": (_i, [_vp, _i, _vp, _vp, _i, _d, _i, _d, ctypes.POINTER(_d), _vp,
                               ctypes.POINTER(SolveStats)]),
    "lmtg_get_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "lmtg_batch_set": (_i, [_vp, ctypes.c_uint32, _vp]),
    "lmtg_material_set_nu": (_i, [_vp, _vp, _u64]),
    "lmtg_batch_set_rhs": (_i, [_vp, _i, _vp]),
    "lmtg_batch_solve": (_i, [_vp, _i, _d, _i, _d, ctypes.POINTER(SolveStats), _vp]),
    "lmtg_batch_get_result": (_i, [_vp, _vp]),
    "lmtg_batch_info": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_u64), _vp]),
    "lmtg_batch_set_options": (_i, [_vp, _i, _i]),
    "lmtg_set_inner_reduction": (_i, [_vp, _d]),
    "lmtg_set_spmv_kind": (_i, [_vp, _i]),
    "lmtg_selftest_bounded_wait": (_i, [_vp, _vp, _vp]),
    "lmtg_read_msh": (_i, [ctypes.c_char_p, _i, _vp, _vp, _vp, _vp, _vp]),
    "lmtg_write_vtu": (_i, [ctypes.c_char_p, _i, _u64, _vp, _u64, _vp, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "lmtg_fit_zone_moduli": (_i, [_vp, ctypes.c_uint32, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _i, _i, _d, _i,
                                  _vp, _vp, _vp, ctypes.POINTER(_i)]),
    "lmtg_residual_norm_noalloc": (_i, [_vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_d)]),
    "lmtg_profile_pcg_kernels": (_i, [_vp, _i, _i, ctypes.POINTER(_d), ctypes.POINTER(_d)]),
}

_lib = None


def library_path():
    from . import _build
    return _build.LIB


def load(build=True):
    """Load liblmtg.so, building it in-tree first when asked.  Raises when unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    from . import _build
    if build:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("liblmtg.so is missing: run lmtpp_gb300._build.build() (nvcc)")
    lib = ctypes.CDLL(_build.LIB)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def declared_functions(header=HEADER):
    """Names of the functions declared in include/lmtg.h."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(lmtg_\w+)\s*\(", txt, flags=re.M)))


class LmtgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


def check(status, ctx=None, what=""):
    if status != OK:
        lib = load(build=False)
        msg = lib.lmtg_last_error(ctx).decode() if ctx else lib.lmtg_status_string(status).decode()
        raise LmtgError(status, "%s: %s" % (what, msg or lib.lmtg_status_string(status).decode()))


def ptr(a):
    """Address of a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return ctypes.c_void_p(a.ctypes.data)
