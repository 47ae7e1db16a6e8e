"""State set-up and deletion (reference: core/python/spirit/state.py)."""
import ctypes

from .spiritlib import fn

_Setup = fn("State_Setup", [ctypes.c_char_p, ctypes.c_bool], ctypes.c_void_p)
_Delete = fn("State_Delete", [ctypes.c_void_p])
_To_Config = fn("State_To_Config", [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p])
_DateTime = fn("State_DateTime", [ctypes.c_void_p], ctypes.c_char_p)


class State:
    """Context manager around setup()/delete(), as `with state.State(cfg) as p_state:`."""

    def __init__(self, configfile="", quiet=False):
        self.p_state = setup(configfile, quiet)

    def __enter__(self):
        return self.p_state

    def __exit__(self, exc_type, exc_value, traceback):
        delete(self.p_state)


def setup(configfile="", quiet=False):
    return _Setup(configfile.encode("utf-8"), ctypes.c_bool(quiet))


def delete(p_state):
    _Delete(ctypes.c_void_p(p_state))


def to_config(p_state, filename, comment=""):
    _To_Config(ctypes.c_void_p(p_state), filename.encode("utf-8"), comment.encode("utf-8"))


def date_time(p_state):
    return _DateTime(ctypes.c_void_p(p_state)).decode("utf-8")
