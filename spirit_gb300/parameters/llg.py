"""LLG parameters (reference: core/python/spirit/parameters/llg.py)."""
import ctypes

from ..spiritlib import fn

_vp, _i, _f, _b = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_bool
_Set_N_Iterations = fn("Parameters_LLG_Set_N_Iterations", [_vp, _i, _i, _i, _i])
_Get_N_Iterations = fn("Parameters_LLG_Get_N_Iterations", [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), _i, _i])
_Set_Direct_Minimization = fn("Parameters_LLG_Set_Direct_Minimization", [_vp, _b, _i, _i])
_Get_Direct_Minimization = fn("Parameters_LLG_Get_Direct_Minimization", [_vp, _i, _i], _b)
_Set_Convergence = fn("Parameters_LLG_Set_Convergence", [_vp, _f, _i, _i])
_Get_Convergence = fn("Parameters_LLG_Get_Convergence", [_vp, _i, _i], _f)
_Set_Time_Step = fn("Parameters_LLG_Set_Time_Step", [_vp, _f, _i, _i])
_Get_Time_Step = fn("Parameters_LLG_Get_Time_Step", [_vp, _i, _i], _f)
_Set_Damping = fn("Parameters_LLG_Set_Damping", [_vp, _f, _i, _i])
_Get_Damping = fn("Parameters_LLG_Get_Damping", [_vp, _i, _i], _f)
_Set_Temperature = fn("Parameters_LLG_Set_Temperature", [_vp, _f, _i, _i])
_Get_Temperature = fn("Parameters_LLG_Get_Temperature", [_vp, _i, _i], _f)
_Set_Seed = fn("Parameters_LLG_Set_Seed", [_vp, _i, _i, _i])


def set_iterations(p_state, n_iterations, n_iterations_log, idx_image=-1, idx_chain=-1):
    _Set_N_Iterations(_vp(p_state), _i(n_iterations), _i(n_iterations_log), _i(idx_image), _i(idx_chain))


def get_iterations(p_state, idx_image=-1, idx_chain=-1):
    a, b = _i(), _i()
    _Get_N_Iterations(_vp(p_state), ctypes.byref(a), ctypes.byref(b), _i(idx_image), _i(idx_chain))
    return a.value, b.value


def set_direct_minimization(p_state, use_minimization, idx_image=-1, idx_chain=-1):
    _Set_Direct_Minimization(_vp(p_state), _b(use_minimization), _i(idx_image), _i(idx_chain))


def get_direct_minimization(p_state, idx_image=-1, idx_chain=-1):
    return bool(_Get_Direct_Minimization(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_convergence(p_state, convergence, idx_image=-1, idx_chain=-1):
    _Set_Convergence(_vp(p_state), _f(convergence), _i(idx_image), _i(idx_chain))


def get_convergence(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Convergence(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_timestep(p_state, dt, idx_image=-1, idx_chain=-1):
    _Set_Time_Step(_vp(p_state), _f(dt), _i(idx_image), _i(idx_chain))


def get_timestep(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Time_Step(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_damping(p_state, damping, idx_image=-1, idx_chain=-1):
    _Set_Damping(_vp(p_state), _f(damping), _i(idx_image), _i(idx_chain))


def get_damping(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Damping(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_temperature(p_state, temperature, idx_image=-1, idx_chain=-1):
    _Set_Temperature(_vp(p_state), _f(temperature), _i(idx_image), _i(idx_chain))


def get_temperature(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Temperature(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_seed(p_state, seed, idx_image=-1, idx_chain=-1):
    """Thermal-noise seed at run time (extension; the reference takes it from llg_seed only)."""
    _Set_Seed(_vp(p_state), _i(seed), _i(idx_image), _i(idx_chain))
