"""Transitions between images (reference: core/python/spirit/transition.py)."""
import ctypes

from .spiritlib import fn

_Homogeneous = fn("Transition_Homogeneous", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int])


def homogeneous(p_state, idx_1, idx_2, idx_chain=-1):
    _Homogeneous(ctypes.c_void_p(p_state), ctypes.c_int(idx_1), ctypes.c_int(idx_2), ctypes.c_int(idx_chain))
