"""System getters (reference: core/python/spirit/system.py).  get_spin_directions returns a
numpy view on the image's host spin buffer; writing to it changes the state, as in the reference."""
import ctypes

import numpy as np

from .spiritlib import fn

_vp, _i = ctypes.c_void_p, ctypes.c_int
_Get_Index = fn("System_Get_Index", [_vp], _i)
_Get_NOS = fn("System_Get_NOS", [_vp, _i, _i], _i)
_Get_Spin_Directions = fn("System_Get_Spin_Directions", [_vp, _i, _i], ctypes.POINTER(ctypes.c_double))
_Get_Effective_Field = fn("System_Get_Effective_Field", [_vp, _i, _i], ctypes.POINTER(ctypes.c_double))
_Get_Energy = fn("System_Get_Energy", [_vp, _i, _i], ctypes.c_float)
_Get_Energy_FP64 = fn("System_Get_Energy_FP64", [_vp, _i, _i], ctypes.c_double)
_Get_Rx = fn("System_Get_Rx", [_vp, _i, _i], ctypes.c_float)
_Update_Data = fn("System_Update_Data", [_vp, _i, _i])
_Get_Energy_Array_Names = fn("System_Get_Energy_Array_Names", [_vp, ctypes.c_char_p, _i, _i], _i)
_Get_Energy_Array = fn("System_Get_Energy_Array", [_vp, ctypes.POINTER(ctypes.c_float), ctypes.c_bool, _i, _i], _i)
_Print_Energy_Array = fn("System_Print_Energy_Array", [_vp, _i, _i])


def get_index(p_state):
    return int(_Get_Index(_vp(p_state)))


def get_nos(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_NOS(_vp(p_state), _i(idx_image), _i(idx_chain)))


def _view(ptr, nos):
    return np.ctypeslib.as_array(ptr, shape=(nos, 3))


def get_spin_directions(p_state, idx_image=-1, idx_chain=-1):
    nos = get_nos(p_state, idx_image, idx_chain)
    return _view(_Get_Spin_Directions(_vp(p_state), _i(idx_image), _i(idx_chain)), nos)


def get_effective_field(p_state, idx_image=-1, idx_chain=-1):
    nos = get_nos(p_state, idx_image, idx_chain)
    return _view(_Get_Effective_Field(_vp(p_state), _i(idx_image), _i(idx_chain)), nos)


def get_energy(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Energy(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_energy_fp64(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Energy_FP64(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_rx(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Rx(_vp(p_state), _i(idx_image), _i(idx_chain)))


def update_data(p_state, idx_image=-1, idx_chain=-1):
    _Update_Data(_vp(p_state), _i(idx_image), _i(idx_chain))


def get_energy_contributions(p_state, divide_by_nospins=True, idx_image=-1, idx_chain=-1):
    n = _Get_Energy_Array_Names(_vp(p_state), None, _i(idx_image), _i(idx_chain))
    buf = ctypes.create_string_buffer(n + 1)
    _Get_Energy_Array_Names(_vp(p_state), buf, _i(idx_image), _i(idx_chain))
    names = buf.value.decode().split("|") if n else []
    vals = (ctypes.c_float * 8)()
    _Get_Energy_Array(_vp(p_state), vals, ctypes.c_bool(divide_by_nospins), _i(idx_image), _i(idx_chain))
    return {k: float(vals[t]) for t, k in enumerate(names)}


def print_energy_array(p_state, idx_image=-1, idx_chain=-1):
    _Print_Energy_Array(_vp(p_state), _i(idx_image), _i(idx_chain))
