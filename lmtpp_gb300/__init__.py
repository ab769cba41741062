"""GB300-native finite-element hot path of LMT++: element matrices -> gather assembly -> PCG.

The compute path is liblmtg.so (hand-written sm_103a CUDA behind a C ABI, include/lmtg.h);
this package holds its in-tree build, the ctypes binding and the Python mirror of LMT++'s
Formulation API.
"""
from . import abi
from .formulation import (Formulation, make_rect_hexa, make_rect_tetra10, x1_faces, x1_faces_hexa,
                          x1_faces_tetra10)

__all__ = ["abi", "Formulation", "make_rect_hexa", "make_rect_tetra10", "x1_faces", "x1_faces_hexa",
           "x1_faces_tetra10"]
