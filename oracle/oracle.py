"""ctypes front-end of the C oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the CPU restatement of LMT++'s finite-element hot path (fe_oracle.c).  Only the
tests, the smoke check and the CPU-baseline leg of bench.py use it, always as the checker or
the timed CPU baseline, never as part of the GPU product path.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force=False):
    """Compile fe_oracle.c into oracle/_build/liboracle.so (plain gcc, portable flags)."""
    src = os.path.join(HERE, "fe_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "fe_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def make_rect_hexa(nb_points, X0=(0.0, 0.0, 0.0), X1=(1.0, 1.0, 1.0)):
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 3, dtype=np.uint32)
    nn = int(np.prod(nbp.astype(np.int64)))
    ne = int(np.prod(nbp.astype(np.int64) - 1))
    pos = np.zeros((nn, 3))
    conn = np.zeros((ne, 8), dtype=np.uint32)
    x0 = np.asarray(X0, dtype=np.float64)
    x1 = np.asarray(X1, dtype=np.float64)
    rc = lib().orc_make_rect_hexa(_p(x0, _f64p), _p(x1, _f64p), _p(nbp, _u32p), _p(pos, _f64p),
                                  _p(conn, _u32p))
    if rc:
        raise RuntimeError("orc_make_rect_hexa failed")
    return pos, conn


def make_rect_tetra10(nb_points, X0=(0.0, 0.0, 0.0), X1=(1.0, 1.0, 1.0)):
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 3, dtype=np.uint32)
    x0 = np.asarray(X0, dtype=np.float64)
    x1 = np.asarray(X1, dtype=np.float64)
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    L = lib()
    L.orc_make_rect_tetra10(_p(x0, _f64p), _p(x1, _f64p), _p(nbp, _u32p), ctypes.byref(nn),
                            ctypes.byref(ne), None, None)
    pos = np.zeros((nn.value, 3))
    conn = np.zeros((ne.value, 10), dtype=np.uint32)
    rc = L.orc_make_rect_tetra10(_p(x0, _f64p), _p(x1, _f64p), _p(nbp, _u32p), ctypes.byref(nn),
                                 ctypes.byref(ne), _p(pos, _f64p), _p(conn, _u32p))
    if rc:
        raise RuntimeError("orc_make_rect_tetra10 failed: %d" % rc)
    return pos, conn


def tetra10_ke(xyz, E, nu):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    Ke = np.zeros((30, 30))
    lib().orc_tetra10_elast_ke(_p(xyz, _f64p), ctypes.c_double(E), ctypes.c_double(nu), _p(Ke, _f64p))
    return Ke


def tri6_traction(faces, pos, t, F):
    faces = np.ascontiguousarray(faces, dtype=np.uint32)
    t = np.asarray(t, dtype=np.float64)
    lib().orc_tri6_traction(ctypes.c_uint64(faces.shape[0]), _p(faces, _u32p), _p(pos, _f64p),
                            _p(t, _f64p), _p(F, _f64p))
    return F


TETRA10_CHILDREN = [[0, 2, 1, 6, 5, 4], [0, 1, 3, 4, 8, 7], [0, 3, 2, 7, 9, 6], [1, 2, 3, 5, 9, 8]]


def x1_faces_tetra10(pos, conn, x1=1.0, eps=1e-6):
    """Triangle_6 skin faces (Tetra_10 children, formulations/element_Tetra_10.py:16-21) on x = x1,
    in element order then child order."""
    out = []
    for e in range(conn.shape[0]):
        for ch in TETRA10_CHILDREN:
            q = conn[e, ch]
            if np.all(pos[q, 0] > x1 - eps):
                out.append(q)
    return np.ascontiguousarray(np.array(out, dtype=np.uint32).reshape(-1, 6))


def hexa8_ke(xyz, E, nu):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    Ke = np.zeros((24, 24))
    lib().orc_hexa8_elast_ke(_p(xyz, _f64p), ctypes.c_double(E), ctypes.c_double(nu), _p(Ke, _f64p))
    return Ke


def pattern_lower(nn, nnu, conn):
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    ne, npe = conn.shape
    n = nn * nnu
    rowptr = np.zeros(n + 1, dtype=np.uint64)
    nnz = ctypes.c_uint64(0)
    L = lib()
    L.orc_pattern_lower(ctypes.c_uint64(nn), ctypes.c_int(nnu), ctypes.c_uint64(ne), ctypes.c_int(npe),
                        _p(conn, _u32p), _p(rowptr, _u64p), None, ctypes.byref(nnz))
    col = np.zeros(nnz.value, dtype=np.uint32)
    L.orc_pattern_lower(ctypes.c_uint64(nn), ctypes.c_int(nnu), ctypes.c_uint64(ne), ctypes.c_int(npe),
                        _p(conn, _u32p), _p(rowptr, _u64p), _p(col, _u32p), ctypes.byref(nnz))
    return rowptr, col


def assemble_elast(pos, conn, E, nu, rowptr, col):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    E = np.ascontiguousarray(np.atleast_1d(E), dtype=np.float64)
    val = np.zeros(col.shape[0])
    rc = lib().orc_assemble_elast(ctypes.c_int(conn.shape[1]), ctypes.c_uint64(pos.shape[0]),
                                  ctypes.c_uint64(conn.shape[0]), _p(pos, _f64p), _p(conn, _u32p),
                                  _p(E, _f64p), ctypes.c_int(1 if E.shape[0] > 1 else 0),
                                  ctypes.c_double(nu), _p(rowptr, _u64p), _p(col, _u32p),
                                  _p(val, _f64p))
    if rc:
        raise RuntimeError("orc_assemble_elast failed: %d" % rc)
    return val


def recalage_ke(xyz, E, nu, rho, gamma):
    """The recalage element Hessian (orc_recalage_ke), 9 npe x 9 npe."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    npe = xyz.shape[0]
    K = np.zeros((9 * npe, 9 * npe))
    lib().orc_recalage_ke(ctypes.c_int(npe), _p(xyz, _f64p), ctypes.c_double(E), ctypes.c_double(nu),
                          ctypes.c_double(rho), ctypes.c_double(gamma), _p(K, _f64p))
    return K


def recalage_nodal(ud, valid, E, r):
    ud = np.ascontiguousarray(ud, dtype=np.float64)
    Kn, Fn = np.zeros((9, 9)), np.zeros(9)
    lib().orc_recalage_nodal(_p(ud, _f64p), ctypes.c_double(valid), ctypes.c_double(E), ctypes.c_double(r),
                             _p(Kn, _f64p), _p(Fn, _f64p))
    return Kn, Fn


def assemble_recalage(pos, conn, E, nu, rho, gamma, r, Ud, Uv, rowptr, col):
    """(val, F) of the recalage system on the lower CSR pattern of pattern_lower(nn, 9, conn)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    Ud = np.ascontiguousarray(Ud, dtype=np.float64).reshape(-1)
    Uv = np.ascontiguousarray(Uv, dtype=np.float64).reshape(-1)
    nn = pos.shape[0]
    val, F = np.zeros(col.shape[0]), np.zeros(9 * nn)
    rc = lib().orc_assemble_recalage(ctypes.c_int(conn.shape[1]), ctypes.c_uint64(nn), ctypes.c_uint64(conn.shape[0]),
                                     _p(pos, _f64p), _p(conn, _u32p), ctypes.c_double(E), ctypes.c_double(nu),
                                     ctypes.c_double(rho), ctypes.c_double(gamma), ctypes.c_double(r), _p(Ud, _f64p),
                                     _p(Uv, _f64p), _p(rowptr, _u64p), _p(col, _u32p), _p(val, _f64p), _p(F, _f64p))
    if rc:
        raise RuntimeError("orc_assemble_recalage failed: %d" % rc)
    return val, F


def elem_fields(pos, conn, E, nu, u):
    """Element fields after the solve (orc_elem_fields): ne x 13 = epsilon[6], sigma[6],
    tr_epsilon at var_inter = 0.5.  E: 1 or ne values; nu: scalar or ne values."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    E = np.ascontiguousarray(np.atleast_1d(E), dtype=np.float64)
    nuv = None if np.ndim(nu) == 0 else np.ascontiguousarray(nu, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros((conn.shape[0], 13))
    rc = lib().orc_elem_fields(ctypes.c_int(conn.shape[1]), ctypes.c_uint64(conn.shape[0]), _p(pos, _f64p),
                               _p(conn, _u32p), _p(E, _f64p), ctypes.c_int(1 if E.shape[0] > 1 else 0),
                               ctypes.c_double(0.0 if nuv is not None else float(nu)),
                               None if nuv is None else _p(nuv, _f64p), _p(u, _f64p), _p(out, _f64p))
    if rc:
        raise RuntimeError("orc_elem_fields failed: %d" % rc)
    return out


def volume_force(pos, conn, density, f_vol):
    """F of the volume force density f_vol . te dV (formulation_elasticity_iso.py:49)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    ne, npe = conn.shape
    w = np.zeros((ne, npe))
    rc = lib().orc_volume_weights(ctypes.c_int(npe), ctypes.c_uint64(ne), _p(pos, _f64p), _p(conn, _u32p),
                                  _p(w, _f64p))
    if rc:
        raise RuntimeError("orc_volume_weights failed: %d" % rc)
    s = np.zeros(pos.shape[0])
    np.add.at(s, conn.ravel().astype(np.int64), w.ravel())
    return (density * s[:, None] * np.asarray(f_vol, dtype=np.float64)[None, :]).ravel()


def quad4_traction(faces, pos, t, F):
    faces = np.ascontiguousarray(faces, dtype=np.uint32)
    t = np.asarray(t, dtype=np.float64)
    lib().orc_quad4_traction(ctypes.c_uint64(faces.shape[0]), _p(faces, _u32p), _p(pos, _f64p),
                             _p(t, _f64p), _p(F, _f64p))
    return F


def penalty(rowptr, col, val, F, dofs, coef, res, pen):
    dofs = np.ascontiguousarray(dofs, dtype=np.uint32)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    res = np.ascontiguousarray(res, dtype=np.float64)
    f = lib().orc_penalty
    f.restype = ctypes.c_double
    return f(ctypes.c_uint64(rowptr.shape[0] - 1), _p(rowptr, _u64p), _p(col, _u32p), _p(val, _f64p),
             _p(F, _f64p), ctypes.c_uint64(dofs.shape[0]), _p(dofs, _u32p), _p(coef, _f64p),
             _p(res, _f64p), ctypes.c_double(pen))


def spmv(rowptr, col, val, x):
    y = np.zeros(rowptr.shape[0] - 1)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_spmv_sym_lower(ctypes.c_uint64(y.shape[0]), _p(rowptr, _u64p), _p(col, _u32p),
                             _p(val, _f64p), _p(x, _f64p), _p(y, _f64p))
    return y


def skyline_solve(rowptr, col, val, b):
    x = np.zeros(rowptr.shape[0] - 1)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rc = lib().orc_skyline_solve(ctypes.c_uint64(x.shape[0]), _p(rowptr, _u64p), _p(col, _u32p),
                                 _p(val, _f64p), _p(b, _f64p), _p(x, _f64p))
    if rc:
        raise RuntimeError("skyline solve failed: %d" % rc)
    return x


def ic0(rowptr, col, val):
    fac = np.array(val, dtype=np.float64, copy=True)
    lib().orc_ic0_factorize(ctypes.c_uint64(rowptr.shape[0] - 1), _p(rowptr, _u64p), _p(col, _u32p),
                            _p(fac, _f64p))
    return fac


def ic_pcg(rowptr, col, val, fac, b, crit, maxit=100000, x0=None):
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    it = lib().orc_ic_pcg(ctypes.c_uint64(n), _p(rowptr, _u64p), _p(col, _u32p), _p(val, _f64p),
                          _p(fac, _f64p), _p(b, _f64p), _p(x, _f64p), ctypes.c_double(crit),
                          ctypes.c_int(maxit))
    return x, it


def tiny_block_pcg(rowptr, col, val, b, crit, maxit=1000000, x0=None):
    """The reference's 3x3-block IC(0)-PCG (MatWithTinyBlocks, orc_tiny_block_pcg): returns
    (x, products of A, factor's diagonal blocks (nn x 6), factor seconds, iteration seconds)."""
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    dg = np.zeros(2 * n)
    tf, ts = ctypes.c_double(), ctypes.c_double()
    it = lib().orc_tiny_block_pcg(ctypes.c_uint64(n), _p(rowptr, _u64p), _p(col, _u32p), _p(val, _f64p),
                                  _p(b, _f64p), _p(x, _f64p), ctypes.c_double(crit), ctypes.c_int(maxit),
                                  _p(dg, _f64p), ctypes.byref(tf), ctypes.byref(ts))
    if it == -2:
        raise ValueError("block PCG: the size is not a multiple of 3")
    return x, it, dg.reshape(-1, 6), tf.value, ts.value


def cg(rowptr, col, val, b, crit, crit_kind=2, precond=0, fac=None, maxit=100000, x0=None):
    n = rowptr.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    it = lib().orc_cg(ctypes.c_uint64(n), _p(rowptr, _u64p), _p(col, _u32p), _p(val, _f64p),
                      _p(fac, _f64p), ctypes.c_int(precond), _p(b, _f64p), _p(x, _f64p),
                      ctypes.c_int(crit_kind), ctypes.c_double(crit), ctypes.c_int(maxit))
    return x, it


def dense_to_lower_csr(A):
    """Lower-CSR (SparseLine Sym) of a dense symmetric matrix, dropping exact zeros."""
    n = A.shape[0]
    rowptr = np.zeros(n + 1, dtype=np.uint64)
    cols, vals = [], []
    for i in range(n):
        for j in range(i + 1):
            if A[i, j] != 0.0:
                cols.append(j)
                vals.append(A[i, j])
        rowptr[i + 1] = len(cols)
    return rowptr, np.array(cols, dtype=np.uint32), np.array(vals, dtype=np.float64)


def x1_faces_hexa(pos, conn, x1=1.0, eps=1e-6):
    """Quad4 skin faces [1,2,6,5] of Hexa elements lying on the plane x = x1."""
    q = conn[:, [1, 2, 6, 5]]
    on = np.all(pos[q, 0] > x1 - eps, axis=1)
    return np.ascontiguousarray(q[on], dtype=np.uint32)


def elasticity_problem(nb_points, E=210000.0, nu=0.3, pen=1e5, traction=(1.0, 0.0, 0.0), elem="hexa"):
    """The elasticity workload of the reference's example: unit cube of Hexa8 (or Tetra10),
    penalty clamp of every node on x = 0, uniform traction on x = 1.  Returns oracle arrays."""
    if elem == "hexa":
        pos, conn = make_rect_hexa(nb_points)
    else:
        pos, conn = make_rect_tetra10(nb_points)
    nn = pos.shape[0]
    rowptr, col = pattern_lower(nn, 3, conn)
    val = assemble_elast(pos, conn, E, nu, rowptr, col)
    F = np.zeros(3 * nn)
    if elem == "hexa":
        faces = x1_faces_hexa(pos, conn)
        quad4_traction(faces, pos, traction, F)
    else:
        faces = x1_faces_tetra10(pos, conn)
        tri6_traction(faces, pos, traction, F)
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    dofs = (3 * clamped[:, None] + np.arange(3)[None, :]).ravel()
    md = penalty(rowptr, col, val, F, dofs, np.ones(dofs.shape[0]), np.zeros(dofs.shape[0]), pen)
    return dict(pos=pos, conn=conn, rowptr=rowptr, col=col, val=val, F=F, faces=faces, dofs=dofs,
                max_diag=md, E=E, nu=nu, penalty=pen)


# ---------------------------------------------------------------------------------------------
# heat diffusion on Triangle_6 (formulations/formulation_difftherm.py)
# ---------------------------------------------------------------------------------------------
def make_rect_triangle6(nb_points, X0=(0.0, 0.0), X1=(1.0, 1.0)):
    nbp = np.asarray(nb_points if np.ndim(nb_points) else [nb_points] * 2, dtype=np.uint32)
    x0 = np.asarray(X0, dtype=np.float64)
    x1 = np.asarray(X1, dtype=np.float64)
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    L = lib()
    L.orc_make_rect_triangle6(_p(x0, _f64p), _p(x1, _f64p), _p(nbp, _u32p), ctypes.byref(nn),
                              ctypes.byref(ne), None, None)
    pos = np.zeros((nn.value, 2))
    conn = np.zeros((ne.value, 6), dtype=np.uint32)
    rc = L.orc_make_rect_triangle6(_p(x0, _f64p), _p(x1, _f64p), _p(nbp, _u32p), ctypes.byref(nn),
                                   ctypes.byref(ne), _p(pos, _f64p), _p(conn, _u32p))
    if rc:
        raise RuntimeError("orc_make_rect_triangle6 failed: %d" % rc)
    return pos, conn


def triangle6_km(xy, a):
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    Ke, Me = np.zeros((6, 6)), np.zeros((6, 6))
    lib().orc_triangle6_diff_km(_p(xy, _f64p), ctypes.c_double(a), _p(Ke, _f64p), _p(Me, _f64p))
    return Ke, Me


def assemble_diff(pos, conn, k, rho_c, dt, theta, rowptr, col):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    k = np.ascontiguousarray(np.atleast_1d(k), dtype=np.float64)
    A, B = np.zeros(col.shape[0]), np.zeros(col.shape[0])
    rc = lib().orc_assemble_diff(ctypes.c_uint64(pos.shape[0]), ctypes.c_uint64(conn.shape[0]),
                                 _p(pos, _f64p), _p(conn, _u32p), _p(k, _f64p),
                                 ctypes.c_int(1 if k.shape[0] > 1 else 0), ctypes.c_double(rho_c),
                                 ctypes.c_double(dt), ctypes.c_double(theta), _p(rowptr, _u64p),
                                 _p(col, _u32p), _p(A, _f64p), _p(B, _f64p))
    if rc:
        raise RuntimeError("orc_assemble_diff failed: %d" % rc)
    return A, B


def boundary_nodes_2d(pos, eps=1e-9):
    return np.nonzero((pos[:, 0] < eps) | (pos[:, 1] < eps) | (pos[:, 0] > 1 - eps) | (pos[:, 1] > 1 - eps))[0]


def gaussian_bump(pos, centre=(0.5, 0.5), sigma=0.1):
    d2 = (pos[:, 0] - centre[0]) ** 2 + (pos[:, 1] - centre[1]) ** 2
    return np.exp(-d2 / (2 * sigma * sigma))


def diffusion_problem(nb_points, k=1.0, rho_c=1.0, dt=1e-4, theta=0.5, pen=1e5):
    """Heat diffusion on the unit square of Triangle_6: theta-scheme matrices (A with the penalty
    T = 0 on the boundary, max|diag A| scale), the Gaussian-bump initial field."""
    pos, conn = make_rect_triangle6(nb_points)
    rowptr, col = pattern_lower(pos.shape[0], 1, conn)
    A, B = assemble_diff(pos, conn, k, rho_c, dt, theta, rowptr, col)
    bnd = boundary_nodes_2d(pos)
    md = penalty(rowptr, col, A, None, bnd, np.ones(bnd.shape[0]), np.zeros(bnd.shape[0]), pen)
    return dict(pos=pos, conn=conn, rowptr=rowptr, col=col, A=A, B=B, bnd=bnd, max_diag=md,
                T0=gaussian_bump(pos), k=k, rho_c=rho_c, dt=dt, theta=theta, penalty=pen)


def diffusion_run(P, nsteps, T0=None, load=None):
    """CPU theta-scheme: A T_{n+1} = B T_n (+ a constant load) with the direct solver; returns
    all states."""
    T = np.array(P["T0"] if T0 is None else T0, dtype=np.float64)
    states = [T.copy()]
    for _ in range(nsteps):
        rhs = spmv(P["rowptr"], P["col"], P["B"], T)
        if load is not None:
            rhs = rhs + load
        T = skyline_solve(P["rowptr"], P["col"], P["A"], rhs)
        states.append(T.copy())
    return states


def diffusion_sources(P, Q=None, Qs=None):
    """The step load M Q + Qs of difftherm's sources (formulations/formulation_difftherm.py:26-29):
    M the consistent Triangle_6 mass matrix (the theta-scheme matrices with k = 0 and dt = 1)."""
    s = np.zeros(P["pos"].shape[0])
    if Q is not None:
        M, _ = assemble_diff(P["pos"], P["conn"], 0.0, 1.0, 1.0, 1.0, P["rowptr"], P["col"])
        s += spmv(P["rowptr"], P["col"], M, np.asarray(Q, dtype=np.float64))
    if Qs is not None:
        s += np.asarray(Qs, dtype=np.float64)
    return s


def diffusion_convection(P, edges, H, t0):
    """Skin convection H (T - t0) te dS on straight Bar_3 edges (end, end, middle) in closed form:
    Ms = L/30 [[4, -1, 2], [-1, 4, 2], [2, 2, 16]], int N ds = L [1/6, 1/6, 2/3].  Adds
    theta H Ms to P["A"] and -(1 - theta) H Ms to P["B"] (lower CSR, in place); returns the load
    H t0 int N ds."""
    pos, rowptr, col, th = P["pos"], P["rowptr"], P["col"], P["theta"]
    H = np.broadcast_to(np.asarray(H, dtype=np.float64), (len(edges),))
    Ms0 = np.array([[4.0, -1.0, 2.0], [-1.0, 4.0, 2.0], [2.0, 2.0, 16.0]]) / 30.0
    Ns0 = np.array([1.0, 1.0, 4.0]) / 6.0
    load = np.zeros(pos.shape[0])
    for e, nd in enumerate(np.asarray(edges, dtype=np.int64)):
        L = np.linalg.norm(pos[nd[1]] - pos[nd[0]])
        load[nd] += H[e] * t0 * L * Ns0
        for a in range(3):
            for b in range(3):
                i, j = nd[a], nd[b]
                if j > i:
                    continue
                q = rowptr[i] + int(np.nonzero(col[rowptr[i]:rowptr[i + 1]] == j)[0][0])
                v = H[e] * L * Ms0[a, b]
                P["A"][q] += th * v
                P["B"][q] -= (1.0 - th) * v
    return load


# ---------------------------------------------------------------------------------------------
# identification driver (include/formulation/FormulationFit.h)
# ---------------------------------------------------------------------------------------------
def fit_zone_moduli(pos, conn, zone, p0, nu, dofs, pen, F, u_exp, w=None, relaxation=1.0, lm=0.0,
                    conv=1e-4, max_iter=20, sens_val=None):
    """Gauss-Newton of FormulationFit::exec (include/formulation/FormulationFit.h:17-80) for the
    zone moduli p (E_e = p[zone[e]]), with W = diag(w) standing for exp_mat:
      assemble (penalty max|diag| recomputed, as assemble() does); u = K^-1 F;
      dU_i = K^-1 (-dK/dp_i u) (the element part; assemble_vector_der_var);
      M_ij = (W dU_i).dU_j, V_i = (W dU_i).(u_exp - u); a zero diagonal becomes 1;
      M_ii += max|diag M| lm; dD = M^-1 V; p += relaxation dD;
      stop when every |dD| < conv or at iteration max_iter (counted from 0);
      sensitivity_i = sum_c |sens_val_c (M^-1 W dU)_ic|.
    Direct solves (skyline Cholesky).  Returns dict(p, history, residual_history, sensitivity,
    iterations)."""
    zone = np.asarray(zone, dtype=np.int64)
    p = np.array(p0, dtype=np.float64)
    nz = p.shape[0]
    nn = pos.shape[0]
    n = 3 * nn
    w = np.ones(n) if w is None else np.asarray(w, dtype=np.float64)
    sv = np.ones(n) if sens_val is None else np.asarray(sens_val, dtype=np.float64)
    rowptr, col = pattern_lower(nn, 3, conn)
    ones = np.ones(dofs.shape[0])
    zeros = np.zeros(dofs.shape[0])
    # unit-modulus zone matrices (no penalty): dK/dp_i = K(1 + mask_i) - K(1), K being linear in E
    # (an E of 0 has no compliance inverse)
    K1 = assemble_elast(pos, conn, np.ones(conn.shape[0]), nu, rowptr, col)
    Kz = [assemble_elast(pos, conn, 1.0 + (zone == i), nu, rowptr, col) - K1 for i in range(nz)]
    hist, res_hist = [], []
    it = 0
    while True:
        val = assemble_elast(pos, conn, p[zone], nu, rowptr, col)
        Fc = np.array(F, dtype=np.float64)
        penalty(rowptr, col, val, Fc, dofs, ones, zeros, pen)
        u = skyline_solve(rowptr, col, val, Fc)
        dU = np.stack([skyline_solve(rowptr, col, val, -spmv(rowptr, col, Kz[i], u)) for i in range(nz)])
        d = u_exp - u
        WdU = dU * w[None, :]
        M = WdU @ dU.T
        V = WdU @ d
        res_hist.append(float(np.sum(w * d * d)))
        if np.max(np.abs(np.diag(M))) == 0:
            M[np.diag_indices(nz)] = 1.0
        if lm:
            M[np.diag_indices(nz)] += np.max(np.abs(np.diag(M))) * lm
        Minv = np.linalg.inv(M)
        dD = Minv @ V
        hist.append(float(np.max(np.abs(dD))))
        p += relaxation * dD
        if np.all(np.abs(dD) < conv) or it == max_iter:
            sens = np.sum(np.abs(sv[None, :] * (Minv @ WdU)), axis=1)
            return dict(p=p, history=hist, residual_history=res_hist, sensitivity=sens, iterations=it + 1)
        it += 1


def eliminate(rowptr, col, val, F, dofs, coef, res):
    """Exact single-unknown constraints coef u_j = res (the reference's Lagrange rows for a zero
    penalty, include/formulation/formulation.h:1072-1088) by elimination on the lower CSR, in
    place: F_k -= (K u_bar)_k, rows and columns j zeroed but the diagonal, F_j = K_jj u_bar_j.
    The solution of the modified SPD system is the Lagrange solution."""
    n = rowptr.shape[0] - 1
    ubar = np.zeros(n)
    dofs = np.asarray(dofs, dtype=np.int64)
    ubar[dofs] = np.asarray(res, dtype=np.float64) / np.asarray(coef, dtype=np.float64)
    F -= spmv(rowptr, col, val, ubar)
    mask = np.zeros(n, bool)
    mask[dofs] = True
    rows = np.repeat(np.arange(n), np.diff(rowptr.astype(np.int64)))
    cols = col.astype(np.int64)
    kill = (mask[rows] | mask[cols]) & (rows != cols)
    val[kill] = 0.0
    diag = rowptr[1:].astype(np.int64) - 1  # the diagonal is last in each lower row
    F[dofs] = val[diag[dofs]] * ubar[dofs]
    return ubar


def add_levenberg_marquadt(rowptr, val, max_diag, lm):
    """K(i,i) += max|diag| * levenberg_marquadt (include/formulation/formulation.h:1033-1034),
    on the lower CSR (the diagonal is last in each row)."""
    diag = rowptr[1:].astype(np.int64) - 1
    val[diag] += max_diag * lm


def pressure_loads(faces, pos, p):
    """Consistent loads of a uniform pressure p dS_normal (formulation_elasticity_iso.py:60) on
    Quad4 (4 nodes) or Triangle_6 (6 nodes) skin faces: n = unit cross(dx/dxi0, dx/dxi1) of the
    face node order (formal_lf/element.py:467-474), integrated with the Python rules of the face
    elements as the generated add_skin_elem_matrix does (formal_lf/formulation.py:400-438):
    element_Quad.py gauss_points[3], element_Triangle_6.py gauss_points[4]."""
    faces = np.asarray(faces, dtype=np.int64)
    F = np.zeros(pos.size)
    if faces.shape[1] == 4:
        a, b = 0.21132486540518711775, 0.78867513459481288225
        pts, w = [(b, b), (a, b), (b, a), (a, a)], [0.25] * 4
        def shape(u, v):
            N = np.array([(1 - u) * (1 - v), u * (1 - v), u * v, (1 - u) * v])
            du = np.array([-(1 - v), 1 - v, v, -v])
            dv = np.array([-(1 - u), -u, u, 1 - u])
            return N, du, dv
    else:
        a, b = 0.445948490915965, 0.091576213509771
        pts = [(a, a), (1.0 - 2.0 * a, a), (a, 1.0 - 2.0 * a), (b, b), (1.0 - 2.0 * b, b), (b, 1.0 - 2.0 * b)]
        w = [0.111690794839005] * 3 + [0.054975871827661] * 3
        def shape(u, v):
            X0 = 1 - u - v
            N = np.array([X0 * (2 * X0 - 1), u * (2 * u - 1), v * (2 * v - 1), 4 * X0 * u, 4 * u * v, 4 * v * X0])
            du = np.array([-(4 * X0 - 1), 4 * u - 1, 0, 4 * (X0 - u), 4 * v, -4 * v])
            dv = np.array([-(4 * X0 - 1), 0, 4 * v - 1, -4 * u, 4 * u, 4 * (X0 - v)])
            return N, du, dv
    for q in faces:
        x = pos[q]
        for (u, v), wg in zip(pts, w):
            N, du, dv = shape(u, v)
            n = np.cross(du @ x, dv @ x)
            area = np.linalg.norm(n)
            for k, node in enumerate(q):
                F[3 * node:3 * node + 3] += N[k] * p * (n / area) * wg * area
    return F
