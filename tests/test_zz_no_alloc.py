"""The allocation-free residual entry point, checked against the regular SpMV entry point.

lmtg_residual_norm_noalloc serves callers that cannot call cudaMalloc -- applications that own
all device memory through their own arena and forbid allocation once they run.  It computes
r = b - K x and |r|^2 for a matrix the caller holds on the device, using a fixed device array
as scratch.  Here the caller's buffers are torch tensors; the expected values come from the
existing lmtg_spmv entry point (FP64) on the same matrix and, independently, from scipy's
b - A x, at the FP64 SpMV tolerance (1e-12 relative).  Two calls in a row check that the shared
scratch is reused correctly.  A block-diagonal matrix of exactly the largest accepted size
fills every one of the scratch's block partials.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from lmtpp_gb300 import Formulation, abi, make_rect_hexa, x1_faces_hexa

pytestmark = pytest.mark.gpu


MAX_ROWS = 524288  # node rows one call accepts (65,536 block partials x 8 rows)


def device_bsr(f):
    """The formulation's assembled FP64 matrix as full 3x3-block CSR (sorted columns), and the
    same matrix for scipy."""
    rowptr, col, val = f.get_mat()
    n = f.n
    L = sp.csr_matrix((val, col.astype(np.int64), rowptr.astype(np.int64)), shape=(n, n))
    A = (L + L.T - sp.diags(L.diagonal())).tocsr()
    B = sp.bsr_matrix(A, blocksize=(3, 3))
    B.sort_indices()
    return (np.ascontiguousarray(B.indptr, dtype=np.uint32),
            np.ascontiguousarray(B.indices, dtype=np.uint32),
            np.ascontiguousarray(B.data.reshape(-1), dtype=np.float64), A)


def call_noalloc(lib, torch, stream, nn, d_bptr, d_bcol, d_K, x, b):
    dev = d_K.device
    d_x = torch.from_numpy(x).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    d_r = torch.empty(3 * nn, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rr = ctypes.c_double(-1.0)
    s = lib.lmtg_residual_norm_noalloc(
        ctypes.c_void_p(stream), nn, ctypes.c_void_p(d_bptr.data_ptr()),
        ctypes.c_void_p(d_bcol.data_ptr()), ctypes.c_void_p(d_K.data_ptr()),
        ctypes.c_void_p(d_x.data_ptr()), ctypes.c_void_p(d_b.data_ptr()),
        ctypes.c_void_p(d_r.data_ptr()), ctypes.byref(rr))
    torch.cuda.synchronize()
    return s, d_r.cpu().numpy(), rr.value


def test_residual_noalloc_matches_spmv_entry_point():
    torch = pytest.importorskip("torch")
    pos, conn = make_rect_hexa(11)
    f = Formulation(pos, conn)
    f.elastic_modulus = 210000.0
    f.poisson_ratio = 0.3
    clamped = np.nonzero(pos[:, 0] < 1e-6)[0]
    f.add_constraints((3 * clamped[:, None] + np.arange(3)).ravel(), 1e5)
    f.add_skin_traction(x1_faces_hexa(pos, conn), (1.0, 0.0, 0.0))
    f.assemble(True, True)
    bptr, bcol, K, A = device_bsr(f)
    dev = torch.device("cuda", 0)
    d_bptr = torch.from_numpy(bptr.view(np.int32)).to(dev)
    d_bcol = torch.from_numpy(bcol.view(np.int32)).to(dev)
    d_K = torch.from_numpy(K).to(dev)
    lib = abi.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(7)
    for call in range(2):
        x = rng.standard_normal(f.n)
        b = rng.standard_normal(f.n) * 1e3
        s, r, rr = call_noalloc(lib, torch, stream, f.nn, d_bptr, d_bcol, d_K, x, b)
        assert s == abi.OK, (call, s)
        scale = np.abs(b).max() + np.abs(A).dot(np.abs(x)).max()
        r_ref = b - f.spmv(x, 0)  # the existing entry point
        assert np.abs(r - r_ref).max() <= 1e-12 * scale, call
        r_sp = b - A @ x  # independent of this library
        assert np.abs(r - r_sp).max() <= 1e-12 * scale, call
        assert rr == pytest.approx(float(r_sp @ r_sp), rel=1e-12), call
    f.close()


def test_residual_noalloc_at_the_size_limit():
    """nn = 524,288 node rows, the largest size accepted: a 65,536-block grid, which uses every
    block partial of the fixed scratch; a block-diagonal matrix of random 3x3 blocks."""
    torch = pytest.importorskip("torch")
    nn = MAX_ROWS
    rng = np.random.default_rng(11)
    blocks = rng.standard_normal((nn, 3, 3))
    bptr = np.arange(nn + 1, dtype=np.uint32)
    bcol = np.arange(nn, dtype=np.uint32)
    dev = torch.device("cuda", 0)
    d_bptr = torch.from_numpy(bptr.view(np.int32)).to(dev)
    d_bcol = torch.from_numpy(bcol.view(np.int32)).to(dev)
    d_K = torch.from_numpy(np.ascontiguousarray(blocks.reshape(-1))).to(dev)
    lib = abi.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        x = rng.standard_normal(3 * nn)
        b = rng.standard_normal(3 * nn)
        s, r, rr = call_noalloc(lib, torch, stream, nn, d_bptr, d_bcol, d_K, x, b)
        assert s == abi.OK, (call, s)
        r_ref = b - np.einsum("nij,nj->ni", blocks, x.reshape(nn, 3)).ravel()
        assert np.abs(r - r_ref).max() <= 1e-12 * (np.abs(b).max() + 9 * np.abs(x).max() * np.abs(blocks).max())
        assert rr == pytest.approx(float(r_ref @ r_ref), rel=1e-12), call


def test_residual_noalloc_rejects_oversize_problems():
    lib = abi.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rr = ctypes.c_double()
    s = lib.lmtg_residual_norm_noalloc(None, 524288 + 1, dummy, dummy, dummy, dummy, dummy, dummy,
                                       ctypes.byref(rr))
    assert s == abi.ERR_ARG
