"""Geometry (reference: core/python/spirit/geometry.py)."""
import ctypes

import numpy as np

from .spiritlib import fn

_vp, _i, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
_PF = ctypes.POINTER(ctypes.c_float)
BRAVAIS_LATTICE_IRREGULAR = 0
BRAVAIS_LATTICE_RECTILINEAR = 1
BRAVAIS_LATTICE_SC = 2
BRAVAIS_LATTICE_HEX2D = 3
BRAVAIS_LATTICE_HEX2D_60 = 4
BRAVAIS_LATTICE_HEX2D_120 = 5
BRAVAIS_LATTICE_HCP = 6
BRAVAIS_LATTICE_BCT = 7
BRAVAIS_LATTICE_BCC = 8
BRAVAIS_LATTICE_FCC = 9

_Set_N_Cells = fn("Geometry_Set_N_Cells", [_vp, ctypes.POINTER(ctypes.c_int)])
_Set_mu_s = fn("Geometry_Set_mu_s", [_vp, _f, _i, _i])
_Set_Lattice_Constant = fn("Geometry_Set_Lattice_Constant", [_vp, _f])
_Set_Bravais_Lattice_Type = fn("Geometry_Set_Bravais_Lattice_Type", [_vp, _i])
_Get_Positions = fn("Geometry_Get_Positions", [_vp, _i, _i], ctypes.POINTER(ctypes.c_double))
_Get_N_Cells = fn("Geometry_Get_N_Cells", [_vp, ctypes.POINTER(ctypes.c_int), _i, _i])
_Get_Center = fn("Geometry_Get_Center", [_vp, _PF, _i, _i])
_Get_Bounds = fn("Geometry_Get_Bounds", [_vp, _PF, _PF, _i, _i])
_Get_Dimensionality = fn("Geometry_Get_Dimensionality", [_vp, _i, _i], _i)
_Get_mu_s = fn("Geometry_Get_mu_s", [_vp, _PF, _i, _i])
_Get_N_Cell_Atoms = fn("Geometry_Get_N_Cell_Atoms", [_vp, _i, _i], _i)
_NOS = fn("Geometry_Get_NOS", [_vp], _i)


def set_n_cells(p_state, n_cells=[1, 1, 1], idx_image=-1, idx_chain=-1):
    _Set_N_Cells(_vp(p_state), (ctypes.c_int * 3)(*n_cells))


def set_mu_s(p_state, mu_s, idx_image=-1, idx_chain=-1):
    _Set_mu_s(_vp(p_state), _f(mu_s), _i(idx_image), _i(idx_chain))


def set_lattice_constant(p_state, lattice_constant, idx_image=-1, idx_chain=-1):
    _Set_Lattice_Constant(_vp(p_state), _f(lattice_constant))


def set_bravais_lattice_type(p_state, lattice_type, idx_image=-1, idx_chain=-1):
    _Set_Bravais_Lattice_Type(_vp(p_state), _i(lattice_type))


def get_positions(p_state, idx_image=-1, idx_chain=-1):
    nos = _NOS(_vp(p_state))
    return np.ctypeslib.as_array(_Get_Positions(_vp(p_state), _i(idx_image), _i(idx_chain)), shape=(nos, 3))


def get_n_cells(p_state, idx_image=-1, idx_chain=-1):
    n = (ctypes.c_int * 3)()
    _Get_N_Cells(_vp(p_state), n, _i(idx_image), _i(idx_chain))
    return list(n)


def get_center(p_state, idx_image=-1, idx_chain=-1):
    c = (ctypes.c_float * 3)()
    _Get_Center(_vp(p_state), c, _i(idx_image), _i(idx_chain))
    return list(c)


def get_bounds(p_state, idx_image=-1, idx_chain=-1):
    a, b = (ctypes.c_float * 3)(), (ctypes.c_float * 3)()
    _Get_Bounds(_vp(p_state), a, b, _i(idx_image), _i(idx_chain))
    return list(a), list(b)


def get_dimensionality(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_Dimensionality(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_mu_s(p_state, idx_image=-1, idx_chain=-1):
    nos = _NOS(_vp(p_state))
    a = np.zeros(nos, dtype=np.float32)
    _Get_mu_s(_vp(p_state), a.ctypes.data_as(_PF), _i(idx_image), _i(idx_chain))
    return a


def get_n_cell_atoms(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_N_Cell_Atoms(_vp(p_state), _i(idx_image), _i(idx_chain)))
