"""CPU checks of the C ABI library: it builds, loads, exports every declared symbol, and its
host-only helpers agree with the oracle.  No GPU compute is launched here."""
import ctypes

import numpy as np
import pytest

from lmtpp_gb300 import abi
from lmtpp_gb300.formulation import parse_constraint
from oracle import oracle as O
from conftest import gpu_available


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    names = abi.declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(abi._SIGS), "ctypes signatures out of sync with include/lmtg.h"


def test_status_strings():
    lib = abi.load()
    assert lib.lmtg_status_string(abi.OK) == b"ok"
    assert lib.lmtg_status_string(abi.ERR_NOT_CONVERGED) == b"not converged"
    assert lib.lmtg_status_string(999) == b"unknown status"


@pytest.mark.parametrize("nbp", [(3, 3, 3), (11, 11, 11), (5, 4, 7), (129, 2, 2)])
def test_make_rect_matches_oracle(nbp):
    from lmtpp_gb300 import make_rect_hexa
    pos, conn = make_rect_hexa(nbp)
    pos_o, conn_o = O.make_rect_hexa(nbp)
    assert np.array_equal(pos, pos_o)
    assert np.array_equal(conn, conn_o)


def test_make_rect_rejects_bad_sizes():
    lib = abi.load()
    pos = np.zeros((8, 3))
    conn = np.zeros((1, 8), dtype=np.uint32)
    x0 = np.zeros(3)
    x1 = np.ones(3)
    nbp = np.array([1, 2, 2], dtype=np.uint32)
    assert lib.lmtg_make_rect_hexa(abi.ptr(x0), abi.ptr(x1), abi.ptr(nbp), abi.ptr(pos),
                                   abi.ptr(conn)) == abi.ERR_ARG


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_returns_cuda_error():
    lib = abi.load()
    ctx = ctypes.c_void_p()
    s = lib.lmtg_create(0, ctypes.byref(ctx))
    assert s == abi.ERR_CUDA
    assert not ctx.value


def test_null_context_is_an_argument_error():
    lib = abi.load()
    assert lib.lmtg_assemble(None, abi.ASM_MAT64) == abi.ERR_ARG
    assert lib.lmtg_destroy(None) == abi.OK


@pytest.mark.parametrize("txt,expect", [
    ("node[12].dep[1]", (12, 1, 1.0, 0.0)),
    ("node[3].dep[0] - 0.25", (3, 0, 1.0, 0.25)),
    ("2*node[7].dep[2]+1.5", (7, 2, 2.0, -1.5)),
    (" node[0].dep[2] ", (0, 2, 1.0, 0.0)),
])
def test_constraint_parser(txt, expect):
    assert parse_constraint(txt) == expect


def test_constraint_parser_rejects_nonlinear():
    with pytest.raises(abi.LmtgError):
        parse_constraint("sin(node[0].dep[0]) - 0.1")


@pytest.mark.parametrize("nbp", [(2, 2, 2), (4, 4, 4), (3, 5, 4)])
def test_make_rect_tetra10_matches_oracle(nbp):
    from lmtpp_gb300 import make_rect_tetra10
    pos, conn = make_rect_tetra10(nbp)
    pos_o, conn_o = O.make_rect_tetra10(nbp)
    assert np.array_equal(pos, pos_o)
    assert np.array_equal(conn, conn_o)


@pytest.mark.parametrize("nbp", [(2, 2), (9, 9), (5, 7)])
def test_make_rect_triangle6_matches_oracle(nbp):
    from lmtpp_gb300.diffusion import make_rect_triangle6
    pos, conn = make_rect_triangle6(nbp)
    pos_o, conn_o = O.make_rect_triangle6(nbp)
    assert np.array_equal(pos, pos_o)
    assert np.array_equal(conn, conn_o)
