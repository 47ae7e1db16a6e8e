"""OVF file input and output (reference: core/python/spirit/io.py).

Segments written by this package carry the image's random-stream positions (LLG noise iterations,
Metropolis sweeps) in a ``# Desc:`` line; ``image_read`` / ``chain_read`` restore them, so a
thermal run resumed from a file continues the same Philox streams.
"""
import ctypes

from .spiritlib import fn

FILEFORMAT_OVF_BIN = 0
FILEFORMAT_OVF_BIN4 = 1
FILEFORMAT_OVF_BIN8 = 2
FILEFORMAT_OVF_TEXT = 3
FILEFORMAT_OVF_CSV = 4

_vp, _i, _s = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p
_N_Images = fn("IO_N_Images_In_File", [_vp, _s, _i, _i], _i)
_Image_Read = fn("IO_Image_Read", [_vp, _s, _i, _i, _i])
_Image_Write = fn("IO_Image_Write", [_vp, _s, _i, _s, _i, _i])
_Image_Append = fn("IO_Image_Append", [_vp, _s, _i, _s, _i, _i])
_Chain_Read = fn("IO_Chain_Read", [_vp, _s, _i, _i, _i, _i])
_Chain_Write = fn("IO_Chain_Write", [_vp, _s, _i, _s, _i])
_Chain_Append = fn("IO_Chain_Append", [_vp, _s, _i, _s, _i])
_Positions_Write = fn("IO_Positions_Write", [_vp, _s, _i, _s, _i, _i])


def _b(text):
    return str(text).encode("utf-8")


def n_images_in_file(p_state, filename, idx_image_inchain=-1, idx_chain=-1):
    return int(_N_Images(_vp(p_state), _b(filename), _i(idx_image_inchain), _i(idx_chain)))


def image_read(p_state, filename, idx_image_infile=0, idx_image_inchain=-1, idx_chain=-1):
    _Image_Read(_vp(p_state), _b(filename), _i(idx_image_infile), _i(idx_image_inchain), _i(idx_chain))


def image_write(p_state, filename, fileformat=FILEFORMAT_OVF_TEXT, comment=" ", idx_image=-1, idx_chain=-1):
    _Image_Write(_vp(p_state), _b(filename), _i(fileformat), _b(comment), _i(idx_image), _i(idx_chain))


def image_append(p_state, filename, fileformat=FILEFORMAT_OVF_TEXT, comment=" ", idx_image=-1, idx_chain=-1):
    _Image_Append(_vp(p_state), _b(filename), _i(fileformat), _b(comment), _i(idx_image), _i(idx_chain))


def chain_read(p_state, filename, starting_image=0, ending_image=-1, insert_idx=-1, idx_chain=-1):
    _Chain_Read(_vp(p_state), _b(filename), _i(starting_image), _i(ending_image), _i(insert_idx), _i(idx_chain))


def chain_write(p_state, filename, fileformat=FILEFORMAT_OVF_TEXT, comment=" ", idx_chain=-1):
    _Chain_Write(_vp(p_state), _b(filename), _i(fileformat), _b(comment), _i(idx_chain))


def chain_append(p_state, filename, fileformat=FILEFORMAT_OVF_TEXT, comment=" ", idx_chain=-1):
    _Chain_Append(_vp(p_state), _b(filename), _i(fileformat), _b(comment), _i(idx_chain))


def positions_write(p_state, filename, fileformat=FILEFORMAT_OVF_TEXT, comment=" ", idx_image=-1, idx_chain=-1):
    _Positions_Write(_vp(p_state), _b(filename), _i(fileformat), _b(comment), _i(idx_image), _i(idx_chain))
