"""Adjoint of a T = 0 RK4 LLG trajectory (extension; the reference has no adjoint).

    loss = mean_i |s_i(T) - target_i|^2

with gradients with respect to the initial spins and to params = (J, D, K, B, alpha): J, D, K,
B replace the configured first-shell exchange, first-shell DMI, anisotropy and field magnitudes
(other shells / basis atoms scale with them, the field direction stays), alpha the damping.
The gradients come from hand-written adjoint kernels (Simulation_LLG_Adjoint) with the states
kept every `checkpoint` steps and each segment recomputed once.

LLGTrajectoryLoss wraps it as a torch.autograd.Function.
"""
import ctypes

import numpy as np

from .spiritlib import fn

_vp, _i = ctypes.c_void_p, ctypes.c_int
_PD = ctypes.POINTER(ctypes.c_double)

_Adjoint = fn("Simulation_LLG_Adjoint", [_vp, _PD, _i, _i, _PD, _PD, _PD, _PD, _i, _i], ctypes.c_double)
_Loss = fn("Simulation_LLG_Loss", [_vp, _PD, _i, _PD, _PD, _i, _i], ctypes.c_double)
_NOS = fn("System_Get_NOS", [_vp, _i, _i], _i)

PARAMS = ("J", "D", "K", "B", "alpha")


def _pd(a):
    return None if a is None else a.ctypes.data_as(_PD)


def _params(params):
    return None if params is None else np.ascontiguousarray(params, dtype=np.float64).reshape(5)


def llg_adjoint(p_state, target, n_steps, checkpoint=100, params=None, idx_image=-1, idx_chain=-1):
    """Returns (loss, grad_s0 [nos, 3], grad_params [5], final spins [nos, 3]) for the trajectory
    from the image's current spins."""
    nos = _NOS(_vp(p_state), _i(idx_image), _i(idx_chain))
    t = np.ascontiguousarray(target, dtype=np.float64).reshape(nos, 3)
    g0 = np.zeros((nos, 3))
    gp = np.zeros(5)
    fin = np.zeros((nos, 3))
    pr = _params(params)
    loss = _Adjoint(_vp(p_state), _pd(pr), _i(n_steps), _i(checkpoint), _pd(t), _pd(g0), _pd(gp), _pd(fin),
                    _i(idx_image), _i(idx_chain))
    return float(loss), g0, gp, fin


def llg_loss(p_state, target, n_steps, params=None, idx_image=-1, idx_chain=-1):
    """Returns (loss, final spins [nos, 3]) of the same trajectory, without gradients."""
    nos = _NOS(_vp(p_state), _i(idx_image), _i(idx_chain))
    t = np.ascontiguousarray(target, dtype=np.float64).reshape(nos, 3)
    fin = np.zeros((nos, 3))
    pr = _params(params)
    loss = _Loss(_vp(p_state), _pd(pr), _i(n_steps), _pd(t), _pd(fin), _i(idx_image), _i(idx_chain))
    return float(loss), fin


def _function_class():
    import torch

    class LLGTrajectoryLoss(torch.autograd.Function):
        """loss(s0, params) of the State's image; differentiable in s0 ([nos, 3]) and params ([5])."""

        @staticmethod
        def forward(ctx, s0, params, p_state, target, n_steps, checkpoint=100):
            from . import system

            system.get_spin_directions(p_state)[:] = s0.detach().cpu().double().numpy()
            loss, g0, gp, _ = llg_adjoint(p_state, target, n_steps, checkpoint,
                                          params.detach().cpu().double().numpy())
            ctx.save_for_backward(torch.as_tensor(g0, dtype=s0.dtype, device=s0.device),
                                  torch.as_tensor(gp, dtype=params.dtype, device=params.device))
            return torch.tensor(loss, dtype=torch.float64, device=s0.device)

        @staticmethod
        def backward(ctx, grad_out):
            g0, gp = ctx.saved_tensors
            return grad_out.to(g0.dtype) * g0, grad_out.to(gp.dtype) * gp, None, None, None, None

    return LLGTrajectoryLoss


_FN = None


def trajectory_loss(p_state, s0, params, target, n_steps, checkpoint=100):
    """Differentiable loss (torch) of the RK4 trajectory from s0 with params."""
    global _FN
    if _FN is None:
        _FN = _function_class()
    return _FN.apply(s0, params, p_state, target, n_steps, checkpoint)
