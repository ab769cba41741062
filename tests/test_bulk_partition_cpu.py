"""Host-side check of the bulk-copy SpMVs' stage partitions (no GPU): the producer warp's rule
restated from lmtpp_gb300/csrc/spmv_bulk.cuh (elasticity), csrc/batch.cu (k_b_rows_bulk, CTA
units of tiles) and csrc/diffusion.cu (k_pcg_spmv_s_bulk, 32-row chunks), run on real and random
patterns.  Every row must land in exactly one stage, every bulk copy must start and end on 16
bytes inside its allocation (the matrix, column and row-pointer buffers carry 16 bytes of
slack) and fit its shared-memory stage, and every shared-memory index a consumer forms must
fall inside the bytes copied."""
import numpy as np
import pytest
import scipy.sparse as sp

from lmtpp_gb300 import make_rect_hexa, make_rect_tetra10
from lmtpp_gb300.diffusion import make_rect_triangle6


def block_pattern(conn, nn):
    ne, npe = conn.shape
    A = sp.csr_matrix((np.ones(conn.size), (np.repeat(np.arange(ne), npe), conn.ravel().astype(np.int64))),
                      shape=(ne, nn))
    return (A.T @ A).tocsr().indptr.astype(np.int64)


def stages_3x3(bptr, row0, row_end, cap, rows_per_stage):
    """The elasticity / batch producer: a warp loads bptr of the next rows_per_stage rows and
    keeps the longest prefix whose blocks fit cap."""
    g0, b0 = row0, (bptr[row0] if row0 < row_end else 0)
    out = []
    while g0 < row_end:
        lanes = np.arange(32)
        gi = g0 + 1 + lanes
        inn = (lanes < rows_per_stage) & (gi <= row_end)
        bi = np.where(inn, bptr[np.minimum(gi, len(bptr) - 1)], 0)
        fits = inn & (bi - b0 <= cap)
        n = int(fits.sum())
        assert n >= 1 and fits[:n].all()  # a prefix of the lanes
        b1 = int(bi[n - 1])
        out.append((g0, g0 + n, b0, b1))
        g0, b0 = g0 + n, b1
    return out


def check_3x3(bptr, chunks, cap, rows_per_stage):
    nn, nnzb = len(bptr) - 1, int(bptr[-1])
    k_alloc, c_alloc = 4 * (9 * nnzb + 4), 4 * (nnzb + 4)
    k_stage, c_stage = 36 * cap + 32, 4 * cap + 32
    seen = np.zeros(nn, np.int64)
    for row0, row_end in chunks:
        for g0, g1, b0, b1 in stages_3x3(bptr, row0, row_end, cap, rows_per_stage):
            kb0, kb1 = (36 * b0) & ~15, (36 * b1 + 15) & ~15
            cb0, cb1 = (4 * b0) & ~15, (4 * b1 + 15) & ~15
            assert kb1 <= k_alloc and cb1 <= c_alloc
            assert kb1 - kb0 <= k_stage and cb1 - cb0 <= c_stage
            assert kb0 % 16 == 0 and (kb1 - kb0) % 16 == 0 and (cb1 - cb0) % 16 == 0
            for r in range(g0, g1):
                rb, d = int(bptr[r]), int(bptr[r + 1] - bptr[r])
                lo, hi = 9 * rb - kb0 // 4, 9 * rb + 8 * d + d - 1 - kb0 // 4  # kidx(rb, d, b, v)
                assert lo >= 0 and 4 * hi < kb1 - kb0
                assert rb - cb0 // 4 >= 0 and 4 * (rb + d - 1 - cb0 // 4) < cb1 - cb0
                seen[r] += 1
    return seen


def patterns():
    rng = np.random.default_rng(1)
    deg = rng.integers(1, 97, 5000)  # the pattern allows 96 blocks per row
    yield "random", np.concatenate([[0], np.cumsum(deg)])
    for name, (pos, conn) in (("hexa8", make_rect_hexa(9)), ("tetra10", make_rect_tetra10(5))):
        yield name, block_pattern(conn, pos.shape[0])


@pytest.mark.parametrize("grid", [1, 7, 608, 5000])
def test_elasticity_stages_cover_rows_and_stay_in_bounds(grid):
    for name, bptr in patterns():
        nn = len(bptr) - 1
        per = -(-nn // grid)
        chunks = [(min(nn, b * per), min(nn, min(nn, b * per) + per)) for b in range(grid)]
        seen = check_3x3(bptr, chunks, cap=512, rows_per_stage=16)
        assert (seen == 1).all(), name


@pytest.mark.parametrize("tile_rows,per_unit", [(128, 1), (128, 8)])
def test_batch_units_cover_rows_and_stay_in_bounds(tile_rows, per_unit):
    """Systems of uneven sizes, 128-row tiles inside each, units of per_unit tiles per CTA."""
    rng = np.random.default_rng(2)
    sizes = rng.integers(1, 900, 12)
    deg = rng.integers(1, 97, int(sizes.sum()))
    bptr = np.concatenate([[0], np.cumsum(deg)])
    off = np.concatenate([[0], np.cumsum(sizes)])
    tiles = [(r0, min(r0 + tile_rows, off[m + 1])) for m in range(len(sizes)) for r0 in range(off[m], off[m + 1], tile_rows)]
    seen = np.zeros(len(bptr) - 1, np.int64)
    for t0 in range(0, len(tiles), per_unit):  # a unit never spans two systems in the product;
        for row0, row_end in tiles[t0:t0 + per_unit]:  # the stage rule is per tile either way
            seen += check_3x3(bptr, [(row0, row_end)], cap=512, rows_per_stage=16)
    assert (seen == 1).all()


@pytest.mark.parametrize("grid", [1, 5, 608, 100000])
def test_diffusion_stages_cover_rows_and_stay_in_bounds(grid):
    pos, conn = make_rect_triangle6(33)
    rp = block_pattern(conn, pos.shape[0])
    n, nnz, cap = len(rp) - 1, int(rp[-1]), 3072
    assert 32 * int(np.diff(rp).max()) <= cap  # the host's condition for this kernel
    k_alloc, r_alloc = 4 * (nnz + 4), 4 * (n + 1 + 4)
    k_stage, r_stage = 4 * cap + 32, 4 * (32 * 8 + 1) + 44
    nch = -(-n // 32)
    per = -(-nch // grid)
    seen = np.zeros(n, np.int64)
    for b in range(grid):
        first, end = min(b * per, nch), min(b * per + per, nch)
        row0, row_end = 32 * first, min(n, 32 * end)
        g0, e0 = row0, (int(rp[row0]) if row0 < row_end else 0)
        while g0 < row_end:
            lanes = np.arange(32)
            inn = (lanes < 8) & (g0 + 32 * lanes < row_end)
            ge = np.minimum(row_end, g0 + 32 * (lanes + 1))
            ei = np.where(inn, rp[ge], 0)
            fits = inn & (ei - e0 <= cap)
            k = int(fits.sum())
            assert k >= 1 and fits[:k].all()
            e1, g1 = int(ei[k - 1]), min(row_end, g0 + 32 * k)
            kb0, kb1 = (4 * e0) & ~15, (4 * e1 + 15) & ~15
            rb0, rb1 = (4 * g0) & ~15, (4 * (g1 + 1) + 15) & ~15
            assert g0 % 32 == 0 and rb0 == 4 * g0
            assert kb1 <= k_alloc and rb1 <= r_alloc and kb1 - kb0 <= k_stage and rb1 - rb0 <= r_stage
            for r in range(g0, g1):
                rs, re = int(rp[r]), int(rp[r + 1])
                assert rs - kb0 // 4 >= 0 and 4 * (re - 1 - kb0 // 4) < kb1 - kb0
                assert 4 * (r + 1 - rb0 // 4) < rb1 - rb0
                seen[r] += 1
            g0, e0 = g1, e1
    assert (seen == 1).all()
