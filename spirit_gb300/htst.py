"""Harmonic transition-state theory (reference: core/python/spirit/htst.py).

`calculate` runs HTST_Calculate: the geodesic Hessians of the minimum and the saddle point and all
their eigenpairs are computed on the device in FP64.  The getters return the float values of the
C API; `get_result_fp64` returns the FP64 result (extension).
"""
import ctypes

import numpy as np

from . import system
from .spiritlib import fn

_vp, _i, _b, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_bool, ctypes.c_float
_PF = ctypes.POINTER(ctypes.c_float)
_PD = ctypes.POINTER(ctypes.c_double)
_Calculate = fn("HTST_Calculate", [_vp, _i, _i, _i, _b, _i], _f)
_Get_Info = fn("HTST_Get_Info", [_vp, _PF, _PF, _PF, _PF, _PF, _PF, _PF, _PF, ctypes.POINTER(_i), _i])
_Evalues_Min = fn("HTST_Get_Eigenvalues_Min", [_vp, _PF, _i])
_Evectors_Min = fn("HTST_Get_Eigenvectors_Min", [_vp, _PF, _i])
_Evalues_SP = fn("HTST_Get_Eigenvalues_SP", [_vp, _PF, _i])
_Evectors_SP = fn("HTST_Get_Eigenvectors_SP", [_vp, _PF, _i])
_Velocities = fn("HTST_Get_Velocities", [_vp, _PF, _i])
_Result_FP64 = fn("HTST_Get_Result_FP64", [_vp, _PD, _PD, _PD, _PD, _PD, _PD, _i], _i)

INFO_KEYS = ("temperature_exponent", "me", "Omega_0", "s", "volume_min", "volume_sp", "prefactor_dynamical",
             "prefactor")


def calculate(p_state, idx_image_minimum, idx_image_sp, n_eigenmodes_keep=-1, sparse=False, idx_chain=-1):
    """HTST rate prefactor of the transition from a minimum over a saddle point (float)."""
    return float(_Calculate(_vp(p_state), _i(idx_image_minimum), _i(idx_image_sp), _i(n_eigenmodes_keep),
                            _b(sparse), _i(idx_chain)))


def _info(p_state, idx_chain):
    vals = [_f() for _ in INFO_KEYS]
    n = _i()
    _Get_Info(_vp(p_state), *[ctypes.pointer(v) for v in vals], ctypes.pointer(n), _i(idx_chain))
    return tuple(v.value for v in vals), n.value


def get_info(p_state, idx_chain=-1):
    """(temperature_exponent, me, Omega_0, s, volume_min, volume_sp, prefactor_dynamical, prefactor)"""
    return _info(p_state, idx_chain)[0]


def get_info_dict(p_state, idx_chain=-1):
    v, n = _info(p_state, idx_chain)
    d = dict(zip(INFO_KEYS, v))
    d["n_eigenmodes_keep"] = n
    return d


def _nos(p_state):
    return system.get_nos(p_state)


def _vector(getter, p_state, n, idx_chain):
    out = np.zeros(n, dtype=np.float32)
    getter(_vp(p_state), out.ctypes.data_as(_PF), _i(idx_chain))
    return out


def get_eigenvalues_min(p_state, idx_chain=-1):
    return _vector(_Evalues_Min, p_state, 2 * _nos(p_state), idx_chain)


def get_eigenvalues_sp(p_state, idx_chain=-1):
    return _vector(_Evalues_SP, p_state, 2 * _nos(p_state), idx_chain)


def get_eigenvectors_min(p_state, idx_chain=-1):
    """Eigenvectors at the minimum, shape (n_eigenmodes_keep, 2*nos)."""
    n = get_info_dict(p_state, idx_chain)["n_eigenmodes_keep"]
    return _vector(_Evectors_Min, p_state, n * 2 * _nos(p_state), idx_chain).reshape(n, -1)


def get_eigenvectors_sp(p_state, idx_chain=-1):
    """Eigenvectors at the saddle point, shape (n_eigenmodes_keep, 2*nos)."""
    n = get_info_dict(p_state, idx_chain)["n_eigenmodes_keep"]
    return _vector(_Evectors_SP, p_state, n * 2 * _nos(p_state), idx_chain).reshape(n, -1)


def get_velocities(p_state, idx_chain=-1):
    return _vector(_Velocities, p_state, 2 * _nos(p_state), idx_chain)


def get_result_fp64(p_state, idx_chain=-1):
    """FP64 result of the last calculation (extension): dict with the info values, det_min,
    det_sp, status and -- for a dense calculation -- spectra, eigenvectors and velocities."""
    nos = _nos(p_state)
    n2 = 2 * nos
    keep = get_info_dict(p_state, idx_chain)["n_eigenmodes_keep"]
    info = np.zeros(10)
    em, es, vel = np.zeros(n2), np.zeros(n2), np.zeros(n2)
    vm, vs = np.zeros((max(keep, 1), n2)), np.zeros((max(keep, 1), n2))
    p = lambda a: a.ctypes.data_as(_PD)
    status = int(_Result_FP64(_vp(p_state), p(info), p(em), p(es), p(vm), p(vs), p(vel), _i(idx_chain)))
    out = dict(zip(INFO_KEYS + ("det_min", "det_sp"), info.tolist()))
    out.update(status=status, evalues_min=em, evalues_sp=es, evectors_min=vm[:keep], evectors_sp=vs[:keep],
               velocities=vel, n_eigenmodes_keep=keep)
    return out
