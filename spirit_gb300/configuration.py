"""Spin configurations (reference: core/python/spirit/configuration.py)."""
import ctypes

from .spiritlib import fn

_vp, _i, _f, _b = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_bool
_PF = ctypes.POINTER(ctypes.c_float)
_Domain = fn("Configuration_Domain", [_vp, _PF, _PF, _PF, _f, _f, _b, _i, _i])
_PlusZ = fn("Configuration_PlusZ", [_vp, _PF, _PF, _f, _f, _b, _i, _i])
_MinusZ = fn("Configuration_MinusZ", [_vp, _PF, _PF, _f, _f, _b, _i, _i])
_Random = fn("Configuration_Random", [_vp, _PF, _PF, _f, _f, _b, _b, _i, _i])
_Skyrmion = fn("Configuration_Skyrmion", [_vp, _f, _f, _f, _b, _b, _b, _PF, _PF, _f, _f, _b, _i, _i])
_To_Clipboard = fn("Configuration_To_Clipboard", [_vp, _i, _i])
_From_Clipboard = fn("Configuration_From_Clipboard", [_vp, _PF, _PF, _f, _f, _b, _i, _i])


def _v3(x):
    return (ctypes.c_float * 3)(*x)


def domain(p_state, dir, pos=[0, 0, 0], border_rectangular=[-1, -1, -1], border_cylindrical=-1,
           border_spherical=-1, inverted=False, idx_image=-1, idx_chain=-1):
    _Domain(_vp(p_state), _v3(dir), _v3(pos), _v3(border_rectangular), _f(border_cylindrical),
            _f(border_spherical), _b(inverted), _i(idx_image), _i(idx_chain))


def plus_z(p_state, pos=[0, 0, 0], border_rectangular=[-1, -1, -1], border_cylindrical=-1, border_spherical=-1,
           inverted=False, idx_image=-1, idx_chain=-1):
    _PlusZ(_vp(p_state), _v3(pos), _v3(border_rectangular), _f(border_cylindrical), _f(border_spherical),
           _b(inverted), _i(idx_image), _i(idx_chain))


def minus_z(p_state, pos=[0, 0, 0], border_rectangular=[-1, -1, -1], border_cylindrical=-1, border_spherical=-1,
            inverted=False, idx_image=-1, idx_chain=-1):
    _MinusZ(_vp(p_state), _v3(pos), _v3(border_rectangular), _f(border_cylindrical), _f(border_spherical),
            _b(inverted), _i(idx_image), _i(idx_chain))


def random(p_state, pos=[0, 0, 0], border_rectangular=[-1, -1, -1], border_cylindrical=-1, border_spherical=-1,
           inverted=False, idx_image=-1, idx_chain=-1):
    _Random(_vp(p_state), _v3(pos), _v3(border_rectangular), _f(border_cylindrical), _f(border_spherical),
            _b(inverted), _b(False), _i(idx_image), _i(idx_chain))


def skyrmion(p_state, radius, order=1, phase=1, up_down=False, achiral=False, right_left=False, pos=[0, 0, 0],
             border_rectangular=[-1, -1, -1], border_cylindrical=-1, border_spherical=-1, inverted=False,
             idx_image=-1, idx_chain=-1):
    _Skyrmion(_vp(p_state), _f(radius), _f(order), _f(phase), _b(up_down), _b(achiral), _b(right_left), _v3(pos),
              _v3(border_rectangular), _f(border_cylindrical), _f(border_spherical), _b(inverted), _i(idx_image),
              _i(idx_chain))


def to_clipboard(p_state, idx_image=-1, idx_chain=-1):
    _To_Clipboard(_vp(p_state), _i(idx_image), _i(idx_chain))


def from_clipboard(p_state, pos=[0, 0, 0], border_rectangular=[-1, -1, -1], border_cylindrical=-1,
                   border_spherical=-1, inverted=False, idx_image=-1, idx_chain=-1):
    _From_Clipboard(_vp(p_state), _v3(pos), _v3(border_rectangular), _f(border_cylindrical),
                    _f(border_spherical), _b(inverted), _i(idx_image), _i(idx_chain))
