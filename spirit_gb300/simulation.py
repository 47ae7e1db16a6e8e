"""Simulation control (reference: core/python/spirit/simulation.py) plus the batched extension."""
import ctypes

from . import spiritlib
from .spiritlib import fn

_vp, _i, _b = ctypes.c_void_p, ctypes.c_int, ctypes.c_bool

METHOD_MC = 0
METHOD_LLG = 1
METHOD_GNEB = 2
METHOD_MMF = 3
METHOD_EMA = 4
SOLVER_VP = 0
SOLVER_SIB = 1
SOLVER_DEPONDT = 2
SOLVER_HEUN = 3
SOLVER_RK4 = 4
SOLVER_LBFGS_OSO = 5
SOLVER_VP_OSO = 7


class simulation_run_info(ctypes.Structure):
    _fields_ = [
        ("total_iterations", ctypes.c_int),
        ("total_walltime", ctypes.c_int),
        ("total_ips", ctypes.c_float),
        ("max_torque", ctypes.c_float),
        ("_n_history_iteration", ctypes.c_int),
        ("_history_iteration", ctypes.POINTER(ctypes.c_int)),
        ("_n_history_max_torque", ctypes.c_int),
        ("_history_max_torque", ctypes.POINTER(ctypes.c_float)),
        ("_n_history_energy", ctypes.c_int),
        ("_history_energy", ctypes.POINTER(ctypes.c_float)),
    ]


_P = ctypes.POINTER(simulation_run_info)
_LLG_Start = fn("Simulation_LLG_Start", [_vp, _i, _i, _i, _b, _P, _i, _i])
_GNEB_Start = fn("Simulation_GNEB_Start", [_vp, _i, _i, _i, _b, _P, _i])
_LLG_Start_Batched = fn("Simulation_LLG_Start_Batched", [ctypes.POINTER(_vp), _i, _i, _i, _P])
_SingleShot = fn("Simulation_SingleShot", [_vp, _i, _i])
_N_Shot = fn("Simulation_N_Shot", [_vp, _i, _i, _i])
_Stop = fn("Simulation_Stop", [_vp, _i, _i])
_Stop_All = fn("Simulation_Stop_All", [_vp])
_Running_On_Image = fn("Simulation_Running_On_Image", [_vp, _i, _i], _b)
_Running_On_Chain = fn("Simulation_Running_On_Chain", [_vp, _i], _b)
_Running_Anywhere_On_Chain = fn("Simulation_Running_Anywhere_On_Chain", [_vp, _i], _b)
_Get_IterationsPerSecond = fn("Simulation_Get_IterationsPerSecond", [_vp, _i, _i], ctypes.c_float)
_Get_MaxTorqueNorm = fn("Simulation_Get_MaxTorqueNorm", [_vp, _i, _i], ctypes.c_float)
_Get_Iteration = fn("Simulation_Get_Iteration", [_vp, _i, _i], _i)
_Get_Time = fn("Simulation_Get_Time", [_vp, _i, _i], ctypes.c_float)
_Get_Wall_Time = fn("Simulation_Get_Wall_Time", [_vp, _i, _i], _i)
_Get_Solver_Name = fn("Simulation_Get_Solver_Name", [_vp, _i, _i], ctypes.c_char_p)
_Get_Method_Name = fn("Simulation_Get_Method_Name", [_vp, _i, _i], ctypes.c_char_p)
_Set_Precision = fn("Simulation_Set_Precision", [_vp, _i])
_Get_Precision = fn("Simulation_Get_Precision", [_vp], _i)


_MC_Start = fn("Simulation_MC_Start", [_vp, _i, _i, _b, ctypes.c_void_p, _i, _i])


def start(p_state, method_type, solver_type=None, n_iterations=-1, n_iterations_log=-1, single_shot=False,
          idx_image=-1, idx_chain=-1):
    info = simulation_run_info()
    if method_type == METHOD_MC:
        spiritlib.wrap_function(_MC_Start, [_vp(p_state), _i(n_iterations), _i(n_iterations_log), _b(single_shot),
                                            ctypes.cast(ctypes.pointer(info), ctypes.c_void_p), _i(idx_image),
                                            _i(idx_chain)])
    elif method_type == METHOD_LLG:
        spiritlib.wrap_function(_LLG_Start, [_vp(p_state), _i(solver_type), _i(n_iterations), _i(n_iterations_log),
                                             _b(single_shot), ctypes.pointer(info), _i(idx_image), _i(idx_chain)])
    elif method_type == METHOD_GNEB:
        spiritlib.wrap_function(_GNEB_Start, [_vp(p_state), _i(solver_type), _i(n_iterations), _i(n_iterations_log),
                                              _b(single_shot), ctypes.pointer(info), _i(idx_chain)])
    else:
        raise ValueError("method %s is not part of the GB300 engine (LLG and GNEB are)" % method_type)
    return info


def start_batched(p_states, solver_type, n_iterations=-1):
    """Advance the active image of every state in one batched device run (extension)."""
    arr = (_vp * len(p_states))(*p_states)
    infos = (simulation_run_info * len(p_states))()
    _LLG_Start_Batched(arr, _i(len(p_states)), _i(solver_type), _i(n_iterations), infos)
    return list(infos)


_LLG_Batched_Launch_Steps = fn("Simulation_LLG_Batched_Launch_Steps", [ctypes.POINTER(_vp), _i, _i, _i])
_LLG_Batched_Finish = fn("Simulation_LLG_Batched_Finish", [ctypes.POINTER(_vp), _i])


def batched_launch_steps(p_states, solver_type, n_steps):
    """Enqueue n_steps of an open-ended batched LLG run on the first state's stream, without
    transfers or synchronisation; the first call uploads the spins and starts (extension)."""
    arr = (_vp * len(p_states))(*p_states)
    _LLG_Batched_Launch_Steps(arr, _i(len(p_states)), _i(solver_type), _i(n_steps))


def batched_finish(p_states):
    """End the open batched run: spins back into the host buffers (extension)."""
    arr = (_vp * len(p_states))(*p_states)
    _LLG_Batched_Finish(arr, _i(len(p_states)))


def single_shot(p_state, idx_image=-1, idx_chain=-1):
    _SingleShot(_vp(p_state), _i(idx_image), _i(idx_chain))


def n_shot(p_state, N, idx_image=-1, idx_chain=-1):
    _N_Shot(_vp(p_state), _i(N), _i(idx_image), _i(idx_chain))


def stop(p_state, idx_image=-1, idx_chain=-1):
    _Stop(_vp(p_state), _i(idx_image), _i(idx_chain))


def stop_all(p_state):
    _Stop_All(_vp(p_state))


def running_on_image(p_state, idx_image=-1, idx_chain=-1):
    return bool(_Running_On_Image(_vp(p_state), _i(idx_image), _i(idx_chain)))


def running_on_chain(p_state, idx_chain=-1):
    return bool(_Running_On_Chain(_vp(p_state), _i(idx_chain)))


def running_anywhere_on_chain(p_state, idx_chain=-1):
    return bool(_Running_Anywhere_On_Chain(_vp(p_state), _i(idx_chain)))


def get_iterations_per_second(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_IterationsPerSecond(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_max_torque_norm(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_MaxTorqueNorm(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_iteration(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_Iteration(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_time(p_state, idx_image=-1, idx_chain=-1):
    return float(_Get_Time(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_wall_time(p_state, idx_image=-1, idx_chain=-1):
    return int(_Get_Wall_Time(_vp(p_state), _i(idx_image), _i(idx_chain)))


def get_solver_name(p_state, idx_image=-1, idx_chain=-1):
    return _Get_Solver_Name(_vp(p_state), _i(idx_image), _i(idx_chain)).decode()


def get_method_name(p_state, idx_image=-1, idx_chain=-1):
    return _Get_Method_Name(_vp(p_state), _i(idx_image), _i(idx_chain)).decode()


def set_precision(p_state, bits):
    """Arithmetic of the device step loop: 32 (FP32 bulk, default) or 64 (extension)."""
    _Set_Precision(_vp(p_state), _i(bits))


def get_precision(p_state):
    return int(_Get_Precision(_vp(p_state)))


_Set_Stream = fn("Simulation_Set_Stream", [_vp, _vp])


def set_stream(p_state, stream):
    """Run this State's device work on a caller CUDA stream (a cudaStream_t as int), or on the
    engine's own stream with None (extension)."""
    _Set_Stream(_vp(p_state), _vp(stream) if stream else None)
