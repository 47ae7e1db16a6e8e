"""Monte Carlo parameters (reference: core/python/spirit/parameters/mc.py)."""
import ctypes

from ..spiritlib import fn

_vp, _i, _f, _b = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_bool
_Set_N_Iterations = fn("Parameters_MC_Set_N_Iterations", [_vp, _i, _i, _i, _i])
_Get_N_Iterations = fn("Parameters_MC_Get_N_Iterations", [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), _i, _i])
_Set_Temperature = fn("Parameters_MC_Set_Temperature", [_vp, _f, _i, _i])
_Get_Temperature = fn("Parameters_MC_Get_Temperature", [_vp, _i, _i], _f)
_Set_Metropolis_Cone = fn("Parameters_MC_Set_Metropolis_Cone", [_vp, _b, _f, _b, _f, _i, _i])
_Get_Metropolis_Cone = fn("Parameters_MC_Get_Metropolis_Cone",
                          [_vp, ctypes.POINTER(_b), ctypes.POINTER(_f), ctypes.POINTER(_b), ctypes.POINTER(_f), _i, _i])
_Set_Random_Sample = fn("Parameters_MC_Set_Random_Sample", [_vp, _b, _i, _i])
_Get_Random_Sample = fn("Parameters_MC_Get_Random_Sample", [_vp, _i, _i], _b)


def set_iterations(p_state, n_iterations, n_iterations_log, idx_image=-1, idx_chain=-1):
    _Set_N_Iterations(_vp(p_state), _i(n_iterations), _i(n_iterations_log), _i(idx_image), _i(idx_chain))


def get_iterations(p_state, idx_image=-1, idx_chain=-1):
    a, b = _i(), _i()
    _Get_N_Iterations(_vp(p_state), ctypes.byref(a), ctypes.byref(b), _i(idx_image), _i(idx_chain))
    return a.value, b.value


def set_temperature(p_state, temperature, idx_image=-1, idx_chain=-1):
    _Set_Temperature(_vp(p_state), _f(temperature), _i(idx_image), _i(idx_chain))


def get_temperature(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Temperature(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_metropolis_cone(p_state, use_cone=True, cone_angle=30, use_adaptive_cone=True, target_acceptance_ratio=0.5,
                        idx_image=-1, idx_chain=-1):
    _Set_Metropolis_Cone(_vp(p_state), _b(use_cone), _f(cone_angle), _b(use_adaptive_cone),
                         _f(target_acceptance_ratio), _i(idx_image), _i(idx_chain))


def get_metropolis_cone(p_state, idx_image=-1, idx_chain=-1):
    c, a, ad, t = _b(), _f(), _b(), _f()
    _Get_Metropolis_Cone(_vp(p_state), ctypes.byref(c), ctypes.byref(a), ctypes.byref(ad), ctypes.byref(t),
                         _i(idx_image), _i(idx_chain))
    return bool(c.value), float(a.value), bool(ad.value), float(t.value)


def set_random_sample(p_state, random_sample, idx_image=-1, idx_chain=-1):
    _Set_Random_Sample(_vp(p_state), _b(random_sample), _i(idx_image), _i(idx_chain))


def get_random_sample(p_state, idx_image=-1, idx_chain=-1):
    return bool(_Get_Random_Sample(_vp(p_state), _i(idx_image), _i(idx_chain)))
