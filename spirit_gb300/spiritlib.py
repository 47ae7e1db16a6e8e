"""Loads libspirit_gb300.so (the C API of this package) -- the counterpart of the reference's
core/python/spirit/spiritlib.py:19-43, which loads libSpirit.so.  There is no fallback: without
the compiled library every call fails loudly."""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.realpath(__file__))
LIB_PATH = os.path.join(_HERE, "libspirit_gb300.so")
_lib = None


def load_spirit_library():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libspirit_gb300.so is not built (run `python -m spirit_gb300.build` or "
                "__graft_entry__.build()); the GB300 engine has no CPU fallback")
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def fn(name, argtypes, restype=None):
    f = getattr(load_spirit_library(), name)
    f.argtypes = argtypes
    f.restype = restype
    return f


def wrap_function(function, arguments):
    """Run a (possibly long) call in a daemon thread so Ctrl-C and Simulation_Stop from the
    caller thread keep working, as the reference bindings do (spiritlib.py:35-43)."""
    t = threading.Thread(target=function, args=arguments)
    t.daemon = True
    t.start()
    while t.is_alive():
        t.join(0.1)
