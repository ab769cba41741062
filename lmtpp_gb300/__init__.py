"""GB300-native finite-element hot path of LMT++: element matrices -> gather assembly -> PCG.

The compute path is liblmtg.so (hand-written sm_103a CUDA behind a C ABI, include/lmtg.h);
this package holds its in-tree build, the ctypes binding and the Python mirror of LMT++'s
Formulation API (elasticity on Hexa8 / Tetra10), the difftherm transient solver (Triangle_6),
batches of meshes solved together, the FormulationFit identification driver, and the Gmsh
reader / ParaView VTU writer of LMT++ (meshio).
"""
from . import abi
from .formulation import (Formulation, make_rect_hexa, make_rect_tetra10, x1_faces, x1_faces_hexa,
                          x1_faces_tetra10)
from .batch import BatchFormulation
from .fit import FormulationFit
from .diffusion import Diffusion, make_rect_triangle6
from .recalage import Recalage
from . import meshio

__all__ = ["abi", "Recalage", "Formulation", "make_rect_hexa", "make_rect_tetra10", "x1_faces", "x1_faces_hexa",
           "x1_faces_tetra10", "BatchFormulation", "FormulationFit", "Diffusion", "make_rect_triangle6",
           "meshio"]
