"""Chain of images (reference: core/python/spirit/chain.py)."""
import ctypes

import numpy as np

from .spiritlib import fn

_vp, _i = ctypes.c_void_p, ctypes.c_int
_PF = ctypes.POINTER(ctypes.c_float)
_Get_NOI = fn("Chain_Get_NOI", [_vp, _i], _i)
_next = fn("Chain_next_Image", [_vp, _i], ctypes.c_bool)
_prev = fn("Chain_prev_Image", [_vp, _i], ctypes.c_bool)
_Jump = fn("Chain_Jump_To_Image", [_vp, _i, _i], ctypes.c_bool)
_Set_Length = fn("Chain_Set_Length", [_vp, _i, _i])
_To_Clip = fn("Chain_Image_to_Clipboard", [_vp, _i, _i])
_Replace = fn("Chain_Replace_Image", [_vp, _i, _i])
_Ins_Before = fn("Chain_Insert_Image_Before", [_vp, _i, _i])
_Ins_After = fn("Chain_Insert_Image_After", [_vp, _i, _i])
_Push_Back = fn("Chain_Push_Back", [_vp, _i])
_Delete = fn("Chain_Delete_Image", [_vp, _i, _i], ctypes.c_bool)
_Pop_Back = fn("Chain_Pop_Back", [_vp, _i], ctypes.c_bool)
_Update = fn("Chain_Update_Data", [_vp, _i])
_Setup = fn("Chain_Setup_Data", [_vp, _i])
_Get_Rx = fn("Chain_Get_Rx", [_vp, _PF, _i])
_Get_Energy = fn("Chain_Get_Energy", [_vp, _PF, _i])


def get_noi(p_state, idx_chain=-1):
    return int(_Get_NOI(_vp(p_state), _i(idx_chain)))


def next_image(p_state, idx_chain=-1):
    return bool(_next(_vp(p_state), _i(idx_chain)))


def prev_image(p_state, idx_chain=-1):
    return bool(_prev(_vp(p_state), _i(idx_chain)))


def jump_to_image(p_state, idx_image=-1, idx_chain=-1):
    return bool(_Jump(_vp(p_state), _i(idx_image), _i(idx_chain)))


def set_length(p_state, n_images, idx_chain=-1):
    _Set_Length(_vp(p_state), _i(n_images), _i(idx_chain))


def image_to_clipboard(p_state, idx_image=-1, idx_chain=-1):
    _To_Clip(_vp(p_state), _i(idx_image), _i(idx_chain))


def replace_image(p_state, idx_image=-1, idx_chain=-1):
    _Replace(_vp(p_state), _i(idx_image), _i(idx_chain))


def insert_image_before(p_state, idx_image=-1, idx_chain=-1):
    _Ins_Before(_vp(p_state), _i(idx_image), _i(idx_chain))


def insert_image_after(p_state, idx_image=-1, idx_chain=-1):
    _Ins_After(_vp(p_state), _i(idx_image), _i(idx_chain))


def push_back(p_state, idx_chain=-1):
    _Push_Back(_vp(p_state), _i(idx_chain))


def delete_image(p_state, idx_image=-1, idx_chain=-1):
    return bool(_Delete(_vp(p_state), _i(idx_image), _i(idx_chain)))


def pop_back(p_state, idx_chain=-1):
    return bool(_Pop_Back(_vp(p_state), _i(idx_chain)))


def update_data(p_state, idx_chain=-1):
    _Update(_vp(p_state), _i(idx_chain))


def setup_data(p_state, idx_chain=-1):
    _Setup(_vp(p_state), _i(idx_chain))


def get_reaction_coordinate(p_state, idx_chain=-1):
    n = get_noi(p_state, idx_chain)
    a = np.zeros(n, dtype=np.float32)
    _Get_Rx(_vp(p_state), a.ctypes.data_as(_PF), _i(idx_chain))
    return a


def get_energy(p_state, idx_chain=-1):
    n = get_noi(p_state, idx_chain)
    a = np.zeros(n, dtype=np.float32)
    _Get_Energy(_vp(p_state), a.ctypes.data_as(_PF), _i(idx_chain))
    return a
