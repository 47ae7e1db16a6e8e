"""Adjoint of the T = 0 RK4 trajectory (Simulation_LLG_Adjoint) -- the reference has no adjoint,
so the checks are (i) its forward pass equals the engine's RK4 bit for bit, (ii) central finite
differences (h = 1e-4) of the FP64 forward, (iii) finite differences of the FP64 CPU oracle, (iv)
checkpoint-interval invariance, (v) FP32 against FP64, (vi) the torch.autograd.Function.

Tolerances: adjoint vs central FD 1e-4 relative (the metric's bar; the FD truncation error is
O(h^2) ~ 1e-8 here), FP32 adjoint vs FP64 adjoint 2e-3 relative to the largest component.
"""
import numpy as np
import pytest

from cases import OPEN2D_DDI, SQ_C1
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu

# open 2D square lattice with padded dipolar FFT, non-square so index transposes show
ADJ = dict(OPEN2D_DDI, n_cells=[10, 9, 1], llg=dict(dt=1e-3, damping=0.3, temperature=0.0))
ADJ_PARAMS = np.array([1.0, 0.3, 0.1, 0.8, 0.3])
N_STEPS = 40


def _setup(spec, seed=3):
    from oracle.oracle import random_spins

    n = spec["n_cells"][0] * spec["n_cells"][1] * spec["n_cells"][2]
    return random_spins(n, seed), random_spins(n, seed + 100)


@pytest.mark.parametrize("precision", [64, 32])
def test_adjoint_forward_equals_engine_rk4(precision, monkeypatch):
    """The adjoint's forward pass is the engine's RK4 operation for operation: FP64, and FP32 with
    the plain FP32 state (SPIRIT_GB300_COMP=0; the engine's default compensated FP32 state differs
    from it by rounding)."""
    from spirit_gb300 import adjoint, simulation

    monkeypatch.setenv("SPIRIT_GB300_COMP", "0")
    s0, tgt = _setup(ADJ)
    with make_state(ADJ, s0, precision=precision) as p:
        loss, fin = adjoint.llg_loss(p, tgt, N_STEPS)
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_RK4, N_STEPS)
        eng = spins_of(p)
    np.testing.assert_array_equal(fin, eng)
    assert abs(loss - np.mean(np.sum((eng - tgt) ** 2, axis=1))) <= 1e-12


def test_adjoint_params_vs_central_fd_fp64():
    from spirit_gb300 import adjoint

    s0, tgt = _setup(ADJ)
    h = 1e-4
    with make_state(ADJ, s0, precision=64) as p:
        loss, g0, gp, _ = adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=7, params=ADJ_PARAMS)
        for q in range(5):
            pp, pm = ADJ_PARAMS.copy(), ADJ_PARAMS.copy()
            pp[q] += h
            pm[q] -= h
            fd = (adjoint.llg_loss(p, tgt, N_STEPS, pp)[0] - adjoint.llg_loss(p, tgt, N_STEPS, pm)[0]) / (2 * h)
            assert abs(gp[q] - fd) <= 1e-4 * abs(fd) + 1e-12, (adjoint.PARAMS[q], gp[q], fd)


def test_adjoint_s0_directional_fd_fp64():
    from spirit_gb300 import adjoint, system

    s0, tgt = _setup(ADJ)
    v = np.random.default_rng(11).normal(size=s0.shape)
    h = 1e-4
    with make_state(ADJ, s0, precision=64) as p:
        _, g0, _, _ = adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=9, params=ADJ_PARAMS)
        system.get_spin_directions(p)[:] = s0 + h * v
        lp = adjoint.llg_loss(p, tgt, N_STEPS, ADJ_PARAMS)[0]
        system.get_spin_directions(p)[:] = s0 - h * v
        lm = adjoint.llg_loss(p, tgt, N_STEPS, ADJ_PARAMS)[0]
    fd = (lp - lm) / (2 * h)
    ad = float(np.sum(g0 * v))
    assert abs(ad - fd) <= 1e-4 * abs(fd), (ad, fd)


def test_adjoint_vs_cpu_oracle_fd_fp64():
    """The FP64 CPU reference gradient: central differences of the oracle's RK4 forward."""
    from oracle.oracle import OracleSystem
    from spirit_gb300 import adjoint

    spec = dict(ADJ, n_cells=[7, 6, 1])
    s0, tgt = _setup(spec, seed=5)
    n = 15
    with make_state(spec, s0, precision=64) as p:
        _, g0, gp, _ = adjoint.llg_adjoint(p, tgt, n, checkpoint=4, params=ADJ_PARAMS)

    def oracle_loss(params):
        sp = dict(spec, jij=[params[0]], dij=[params[1]], anisotropy=(params[2], spec["anisotropy"][1]),
                  field=(params[3], spec["field"][1]))
        s, _ = OracleSystem(sp).llg(s0, "RK4", n, dt=1e-3, damping=params[4], temperature=0.0)
        return float(np.mean(np.sum((s - tgt) ** 2, axis=1)))

    h = 1e-4
    for q in range(5):
        pp, pm = ADJ_PARAMS.copy(), ADJ_PARAMS.copy()
        pp[q] += h
        pm[q] -= h
        fd = (oracle_loss(pp) - oracle_loss(pm)) / (2 * h)
        assert abs(gp[q] - fd) <= 1e-6 * abs(fd) + 1e-12, (adjoint.PARAMS[q], gp[q], fd)


def test_adjoint_checkpoint_interval_invariant():
    from spirit_gb300 import adjoint

    s0, tgt = _setup(ADJ)
    out = []
    with make_state(ADJ, s0, precision=64) as p:
        for k in (1, 6, N_STEPS):
            out.append(adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=k, params=ADJ_PARAMS))
    for o in out[1:]:
        assert o[0] == out[0][0]
        np.testing.assert_array_equal(o[1], out[0][1])
        np.testing.assert_array_equal(o[2], out[0][2])


@pytest.mark.parametrize("precision", [64, 32])
def test_adjoint_pipelined_equals_serial(precision, monkeypatch):
    """Several segments run as a two-stream pipeline (recomputation of segment s - 1 on a second
    stream and dipolar lane beside the adjoint of segment s); SPIRIT_GB300_ADJ_PIPE=0 runs them one
    after another.  Odd K with a ragged last segment (40 = 5 * 7 + 5) flips the ping-pong parity."""
    from spirit_gb300 import adjoint

    s0, tgt = _setup(ADJ, seed=5)
    res = {}
    with make_state(ADJ, s0, precision=precision) as p:
        for pipe in ("1", "0"):
            monkeypatch.setenv("SPIRIT_GB300_ADJ_PIPE", pipe)
            res[pipe] = adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=7, params=ADJ_PARAMS)
    assert res["1"][0] == res["0"][0]
    np.testing.assert_array_equal(res["1"][1], res["0"][1])
    np.testing.assert_array_equal(res["1"][2], res["0"][2])


def test_adjoint_fp32_vs_fp64():
    from spirit_gb300 import adjoint

    s0, tgt = _setup(ADJ)
    res = {}
    for prec in (64, 32):
        with make_state(ADJ, s0, precision=prec) as p:
            res[prec] = adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=10, params=ADJ_PARAMS)
    l64, g64, p64, _ = res[64]
    l32, g32, p32, _ = res[32]
    assert abs(l32 - l64) <= 1e-5 * abs(l64)
    assert np.abs(g32 - g64).max() <= 2e-3 * np.abs(g64).max()
    assert np.all(np.abs(p32 - p64) <= 2e-3 * np.abs(p64) + 1e-9)


def test_adjoint_without_ddi_fd_fp64():
    """Stencil-only system (periodic), parameter gradients against central differences."""
    from spirit_gb300 import adjoint

    spec = dict(SQ_C1, n_cells=[9, 8, 1], llg=dict(dt=1e-3, damping=0.3, temperature=0.0))
    s0, tgt = _setup(spec, seed=8)
    prm = np.array([1.0, 0.3, 0.1, 1.0, 0.3])
    h = 1e-4
    with make_state(spec, s0, precision=64) as p:
        _, _, gp, _ = adjoint.llg_adjoint(p, tgt, 30, checkpoint=8, params=prm)
        for q in range(5):
            pp, pm = prm.copy(), prm.copy()
            pp[q] += h
            pm[q] -= h
            fd = (adjoint.llg_loss(p, tgt, 30, pp)[0] - adjoint.llg_loss(p, tgt, 30, pm)[0]) / (2 * h)
            assert abs(gp[q] - fd) <= 1e-4 * abs(fd) + 1e-12, (adjoint.PARAMS[q], gp[q], fd)


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from spirit_gb300 import adjoint

    s0, tgt = _setup(ADJ)
    with make_state(ADJ, s0, precision=64) as p:
        _, g0, gp, _ = adjoint.llg_adjoint(p, tgt, N_STEPS, checkpoint=10, params=ADJ_PARAMS)
        s = torch.tensor(s0, dtype=torch.float64, requires_grad=True)
        prm = torch.tensor(ADJ_PARAMS, dtype=torch.float64, requires_grad=True)
        loss = adjoint.trajectory_loss(p, s, prm, tgt, N_STEPS, 10)
        (3.0 * loss).backward()
    np.testing.assert_allclose(s.grad.numpy(), 3.0 * g0, rtol=0, atol=1e-15)
    np.testing.assert_allclose(prm.grad.numpy(), 3.0 * gp, rtol=1e-15, atol=0)
