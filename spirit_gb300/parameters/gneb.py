"""GNEB parameters (reference: core/python/spirit/parameters/gneb.py)."""
import ctypes

from ..spiritlib import fn

_vp, _i, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
IMAGE_NORMAL = 0
IMAGE_CLIMBING = 1
IMAGE_FALLING = 2
IMAGE_STATIONARY = 3
_Set_N_Iterations = fn("Parameters_GNEB_Set_N_Iterations", [_vp, _i, _i, _i])
_Set_Convergence = fn("Parameters_GNEB_Set_Convergence", [_vp, _f, _i, _i])
_Get_Convergence = fn("Parameters_GNEB_Get_Convergence", [_vp, _i, _i], _f)
_Set_Spring_Constant = fn("Parameters_GNEB_Set_Spring_Constant", [_vp, _f, _i, _i])
_Get_Spring_Constant = fn("Parameters_GNEB_Get_Spring_Constant", [_vp, _i, _i], _f)
_Set_Climbing_Falling = fn("Parameters_GNEB_Set_Climbing_Falling", [_vp, _i, _i, _i])
_Get_Climbing_Falling = fn("Parameters_GNEB_Get_Climbing_Falling", [_vp, _i, _i], _i)
_Set_Image_Type_Automatically = fn("Parameters_GNEB_Set_Image_Type_Automatically", [_vp, _i])


def set_iterations(p_state, n_iterations, n_iterations_log, idx_chain=-1):
    _Set_N_Iterations(_vp(p_state), _i(n_iterations), _i(n_iterations_log), _i(idx_chain))


def set_convergence(p_state, convergence, idx_image=-1, idx_chain=-1):
    _Set_Convergence(_vp(p_state), _f(convergence), _i(idx_image), _i(idx_chain))


def get_convergence(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Convergence(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_spring_constant(p_state, spring_constant, idx_image=-1, idx_chain=-1):
    _Set_Spring_Constant(_vp(p_state), _f(spring_constant), _i(idx_image), _i(idx_chain))


def get_spring_constant(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Spring_Constant(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_climbing_falling(p_state, image_type, idx_image=-1, idx_chain=-1):
    _Set_Climbing_Falling(_vp(p_state), _i(image_type), _i(idx_image), _i(idx_chain))


def get_climbing_falling(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_Climbing_Falling(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_image_type_automatically(p_state, idx_chain=-1):
    _Set_Image_Type_Automatically(_vp(p_state), _i(idx_chain))
