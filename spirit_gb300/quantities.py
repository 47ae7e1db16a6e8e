"""Quantities (reference: core/python/spirit/quantities.py)."""
import ctypes

from .spiritlib import fn

_Get_Magnetization = fn("Quantity_Get_Magnetization", [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                                       ctypes.c_int, ctypes.c_int])


def get_magnetization(p_state, idx_image=-1, idx_chain=-1):
    m = (ctypes.c_float * 3)()
    _Get_Magnetization(ctypes.c_void_p(p_state), m, ctypes.c_int(idx_image), ctypes.c_int(idx_chain))
    return [float(x) for x in m]
