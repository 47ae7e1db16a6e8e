"""Heisenberg Hamiltonian set-up (reference: core/python/spirit/hamiltonian.py) plus FP64
gradient / energy getters (the reference exposes those only through its C++ internals)."""
import ctypes

import numpy as np

from .spiritlib import fn

_vp, _i, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
_PF, _PD, _PI = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)

DDI_METHOD_NONE = 0
DDI_METHOD_FFT = 1
DDI_METHOD_FMM = 2
DDI_METHOD_CUTOFF = 3
CHIRALITY_BLOCH = 1
CHIRALITY_NEEL = 2
CHIRALITY_BLOCH_INVERSE = -1
CHIRALITY_NEEL_INVERSE = -2

_Set_Boundary_Conditions = fn("Hamiltonian_Set_Boundary_Conditions", [_vp, ctypes.POINTER(ctypes.c_bool), _i, _i])
_Set_Field = fn("Hamiltonian_Set_Field", [_vp, _f, _PF, _i, _i])
_Set_Anisotropy = fn("Hamiltonian_Set_Anisotropy", [_vp, _f, _PF, _i, _i])
_Set_Exchange = fn("Hamiltonian_Set_Exchange", [_vp, _i, _PF, _i, _i])
_Set_DMI = fn("Hamiltonian_Set_DMI", [_vp, _i, _PF, _i, _i, _i])
_Set_DDI = fn("Hamiltonian_Set_DDI", [_vp, _i, _PI, _f, ctypes.c_bool, _i, _i])
_Get_Name = fn("Hamiltonian_Get_Name", [_vp, _i, _i], ctypes.c_char_p)
_Get_Boundary_Conditions = fn("Hamiltonian_Get_Boundary_Conditions", [_vp, ctypes.POINTER(ctypes.c_bool), _i, _i])
_Get_Field = fn("Hamiltonian_Get_Field", [_vp, _PF, _PF, _i, _i])
_Get_Anisotropy = fn("Hamiltonian_Get_Anisotropy", [_vp, _PF, _PF, _i, _i])
_Get_DDI = fn("Hamiltonian_Get_DDI", [_vp, _PI, _PI, _PF, ctypes.POINTER(ctypes.c_bool), _i, _i])
_Get_Exchange_N_Pairs = fn("Hamiltonian_Get_Exchange_N_Pairs", [_vp, _i, _i], _i)
_Get_Exchange_Pairs = fn("Hamiltonian_Get_Exchange_Pairs", [_vp, _PI, _PI, _PF, _i, _i])
_Get_DMI_N_Pairs = fn("Hamiltonian_Get_DMI_N_Pairs", [_vp, _i, _i], _i)
_Get_Gradient = fn("Hamiltonian_Get_Gradient", [_vp, _PD, _i, _i], ctypes.c_double)
_Get_Energy_Contributions = fn("Hamiltonian_Get_Energy_Contributions", [_vp, _PD, _PD, _i, _i], ctypes.c_double)
_Get_DDI_Field = fn("Hamiltonian_Get_DDI_Field", [_vp, _PD, _i, _i])
_NOS = fn("System_Get_NOS", [_vp, _i, _i], _i)
_Get_Gradient_Batched = fn("Hamiltonian_Get_Gradient_Batched", [ctypes.POINTER(_vp), _i, _PD, _PD])

TERMS = ["Zeeman", "Anisotropy", "Exchange", "DMI", "DDI"]


def set_boundary_conditions(p_state, boundaries, idx_image=-1, idx_chain=-1):
    b = (ctypes.c_bool * 3)(*boundaries)
    _Set_Boundary_Conditions(_vp(p_state), b, _i(idx_image), _i(idx_chain))


def set_field(p_state, magnitude, direction, idx_image=-1, idx_chain=-1):
    _Set_Field(_vp(p_state), _f(magnitude), (ctypes.c_float * 3)(*direction), _i(idx_image), _i(idx_chain))


def set_anisotropy(p_state, magnitude, direction, idx_image=-1, idx_chain=-1):
    _Set_Anisotropy(_vp(p_state), _f(magnitude), (ctypes.c_float * 3)(*direction), _i(idx_image), _i(idx_chain))


def set_exchange(p_state, n_shells, J_ij, idx_image=-1, idx_chain=-1):
    _Set_Exchange(_vp(p_state), _i(n_shells), (ctypes.c_float * n_shells)(*J_ij), _i(idx_image), _i(idx_chain))


def set_dmi(p_state, n_shells, D_ij, chirality=CHIRALITY_BLOCH, idx_image=-1, idx_chain=-1):
    _Set_DMI(_vp(p_state), _i(n_shells), (ctypes.c_float * n_shells)(*D_ij), _i(chirality), _i(idx_image),
             _i(idx_chain))


def set_ddi(p_state, ddi_method, n_periodic_images=[4, 4, 4], radius=0.0, pb_zero_padding=True, idx_image=-1,
            idx_chain=-1):
    _Set_DDI(_vp(p_state), _i(ddi_method), (ctypes.c_int * 3)(*n_periodic_images), _f(radius),
             ctypes.c_bool(pb_zero_padding), _i(idx_image), _i(idx_chain))


def get_name(p_state, idx_image=-1, idx_chain=-1):
    return _Get_Name(_vp(p_state), _i(idx_image), _i(idx_chain)).decode()


def get_boundary_conditions(p_state, idx_image=-1, idx_chain=-1):
    b = (ctypes.c_bool * 3)()
    _Get_Boundary_Conditions(_vp(p_state), b, _i(idx_image), _i(idx_chain))
    return [bool(x) for x in b]


def get_field(p_state, idx_image=-1, idx_chain=-1):
    m, n = _f(), (ctypes.c_float * 3)()
    _Get_Field(_vp(p_state), ctypes.byref(m), n, _i(idx_image), _i(idx_chain))
    return float(m.value), [float(x) for x in n]


def get_anisotropy(p_state, idx_image=-1, idx_chain=-1):
    m, n = _f(), (ctypes.c_float * 3)()
    _Get_Anisotropy(_vp(p_state), ctypes.byref(m), n, _i(idx_image), _i(idx_chain))
    return float(m.value), [float(x) for x in n]


def get_ddi(p_state, idx_image=-1, idx_chain=-1):
    method, img, r, pb = _i(), (ctypes.c_int * 3)(), _f(), ctypes.c_bool()
    _Get_DDI(_vp(p_state), ctypes.byref(method), img, ctypes.byref(r), ctypes.byref(pb), _i(idx_image),
             _i(idx_chain))
    return {"ddi_method": method.value, "n_periodic_images": list(img), "radius": r.value,
            "pb_zero_padding": pb.value}


def get_exchange_pairs(p_state, idx_image=-1, idx_chain=-1):
    n = _Get_Exchange_N_Pairs(_vp(p_state), _i(idx_image), _i(idx_chain))
    idx = np.zeros((n, 2), dtype=np.int32)
    tr = np.zeros((n, 3), dtype=np.int32)
    J = np.zeros(n, dtype=np.float32)
    _Get_Exchange_Pairs(_vp(p_state), idx.ctypes.data_as(_PI), tr.ctypes.data_as(_PI), J.ctypes.data_as(_PF),
                        _i(idx_image), _i(idx_chain))
    return idx, tr, J


def get_dmi_n_pairs(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_DMI_N_Pairs(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_gradient(p_state, idx_image=-1, idx_chain=-1):
    """FP64 gradient of the current spins on the GPU; returns (gradient [nos, 3], total energy)."""
    nos = _NOS(_vp(p_state), _i(idx_image), _i(idx_chain))
    g = np.zeros((nos, 3))
    E = _Get_Gradient(_vp(p_state), g.ctypes.data_as(_PD), _i(idx_image), _i(idx_chain))
    return g, float(E)


def get_gradient_batched(p_states):
    """FP64 gradients and energies of the active images of several States evaluated as one batch on
    the GPU (the dipolar term of every system from the batch's shared FFT plan table); returns
    ([gradient [nos_k, 3] per State], energies [n])."""
    n = len(p_states)
    nos = [_NOS(_vp(p), _i(-1), _i(-1)) for p in p_states]
    g = np.zeros((sum(nos), 3))
    e = np.zeros(n)
    arr = (_vp * n)(*p_states)
    _Get_Gradient_Batched(arr, _i(n), g.ctypes.data_as(_PD), e.ctypes.data_as(_PD))
    out, o = [], 0
    for k in nos:
        out.append(g[o:o + k])
        o += k
    return out, e


def get_energy_contributions(p_state, per_spin=False, idx_image=-1, idx_chain=-1):
    """FP64 energy per term {name: value} (and per spin [5, nos] if per_spin) of the current spins."""
    nos = _NOS(_vp(p_state), _i(idx_image), _i(idx_chain))
    t = np.zeros(5)
    ps = np.zeros((5, nos)) if per_spin else None
    E = _Get_Energy_Contributions(_vp(p_state), t.ctypes.data_as(_PD), ps.ctypes.data_as(_PD) if per_spin else None,
                                  _i(idx_image), _i(idx_chain))
    out = {k: float(t[i]) for i, k in enumerate(TERMS)}
    out["total"] = float(E)
    if per_spin:
        return out, ps
    return out


def get_ddi_field(p_state, idx_image=-1, idx_chain=-1):
    nos = _NOS(_vp(p_state), _i(idx_image), _i(idx_chain))
    h = np.zeros((nos, 3))
    _Get_DDI_Field(_vp(p_state), h.ctypes.data_as(_PD), _i(idx_image), _i(idx_chain))
    return h


_Get_Gradient_NoAlloc = fn("Hamiltonian_Get_Gradient_NoAlloc",
                           [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i], _i)


def get_gradient_noalloc(p_state, sx, sy, sz, gx, gy, gz, energy, stream=None, idx_image=-1, idx_chain=-1):
    """Allocation-free FP64 gradient + energy of the stencil terms (no dipolar term) for spins
    already on the device.  All arguments after p_state are device addresses (ints) of FP64
    arrays: sx/sy/sz and gx/gy/gz of length nos, energy of length 1; stream is a cudaStream_t
    address (None: legacy default stream).  Asynchronous on that stream; allocates no device
    memory.  Returns the status code (0 = success)."""
    return int(_Get_Gradient_NoAlloc(_vp(p_state), sx, sy, sz, gx, gy, gz, energy, stream,
                                     _i(idx_image), _i(idx_chain)))
