"""GPU parity of the Heisenberg field, energies and LLG integrators against the reference.

Golden fixtures come from the reference itself (tests/golden/make_golden.py); where a case
needs inputs the fixtures do not hold (thermal noise, other sizes) the oracle -- the CPU FP64
restatement pinned by tests/test_oracle_golden.py -- is what the device results are compared with.

Tolerances:
  FP64 device path: gradients 1e-12 relative to max |g|, energies 1e-10 relative,
                    trajectories 1e-10 absolute per spin component.
  FP32 device path: trajectories max|dm| <= 1e-5 after the fixture's iterations (the
                    metric's bar), energies 1e-6 relative.
"""
import numpy as np
import pytest

from cases import GRAD_CASES, LLG_CASES
from conftest import golden
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(n for n in GRAD_CASES if GRAD_CASES[n].get("ddi", {}).get("method", "fft") != "cutoff"))
def test_gradient_energy_fp64(name):
    from spirit_gb300 import hamiltonian

    f = golden("grad_%s.npz" % name)
    with make_state(GRAD_CASES[name], f["spins"]) as p:
        g, E = hamiltonian.get_gradient(p)
        terms = hamiltonian.get_energy_contributions(p)
    scale = np.abs(f["gradient_ge"]).max()
    np.testing.assert_allclose(g, f["gradient_ge"], rtol=0, atol=1e-12 * scale)
    assert abs(E - f["energy_total"]) <= 1e-10 * abs(f["energy_total"])
    for k, v in zip(f["term_names"], f["term_energies"]):
        assert abs(terms[str(k)] - v) <= 1e-10 * abs(f["energy_total"]), (k, terms[str(k)], v)


@pytest.mark.parametrize("case,solver,sid,n_iter", LLG_CASES)
def test_llg_trajectory_fp64(case, solver, sid, n_iter):
    from spirit_gb300 import simulation, system

    f = golden("llg_%s_%s.npz" % (case, solver))
    with make_state(GRAD_CASES[case], f["spins_in"], precision=64) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, n_iter)
        s = spins_of(p)
        assert simulation.get_iteration(p) == int(f["iterations"])
        E = system.get_energy_fp64(p)
        mt = simulation.get_max_torque_norm(p)
    assert np.abs(s - f["spins_out"]).max() <= 1e-10
    assert abs(E - f["energy"]) <= 1e-10 * abs(f["energy"])
    assert abs(mt - f["max_torque"]) <= 1e-5 * abs(f["max_torque"])


@pytest.mark.parametrize("case,solver,sid,n_iter", LLG_CASES)
def test_llg_trajectory_fp32(case, solver, sid, n_iter):
    from spirit_gb300 import simulation, system

    f = golden("llg_%s_%s.npz" % (case, solver))
    with make_state(GRAD_CASES[case], f["spins_in"], precision=32) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, n_iter)
        s = spins_of(p)
        E = system.get_energy_fp64(p)
    # L-BFGS builds its curvature pairs from differences of FP32 gradients, which amplifies the
    # rounding of the trajectory (200 iterations: 1.2e-5 against the FP64 reference run)
    tol = 5e-5 if solver == "LBFGS_OSO" else 1e-5
    assert np.abs(s - f["spins_out"]).max() <= tol
    assert abs(E - f["energy"]) <= 1e-5 * abs(f["energy"])


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("solver", [1, 2, 3, 4])
def test_larmor_precession(solver, precision):
    """core/test/test_physics.cpp:20-88: a single spin in B_z precesses with phi = dtg B t and
    s_z = tanh(alpha dtg B t); 100 single shots.  The reference asserts 1e-6 absolute for its
    FP64 build; the FP32 device path is held to 2e-6 (SIB's own truncation error is ~0.9e-6 here)."""
    from spirit_gb300 import configuration, hamiltonian, parameters, simulation, system
    import spirit_gb300.parameters.llg as llg

    spec = dict(bravais="sc", n_cells=[1, 1, 1], mu_s=[2.0], bc=[1, 1, 0], field=(1.0, (0, 0, 1)),
                anisotropy=(0.0, (0, 0, 1)), jij=[10.0], dij=[6.0], dm_chirality=1,
                llg=dict(dt=0.001, damping=0.0, temperature=0.0, force_convergence=1e-8))
    with make_state(spec, precision=precision) as p:
        damping = 0.3
        llg.set_damping(p, damping)
        tstep = llg.get_timestep(p)
        B, _ = hamiltonian.get_field(p)
        dtg = tstep * 0.1760859644 / (1.0 + damping * damping)
        configuration.domain(p, [1, 0, 0])
        simulation.start(p, simulation.METHOD_LLG, solver, -1, -1, True)
        for i in range(100):
            simulation.single_shot(p)
            d = system.get_spin_directions(p)[0]
            phi = dtg * (i + 1) * B
            sz = np.tanh(damping * dtg * (i + 1) * B)
            sx = np.cos(phi) * np.sqrt(1 - sz * sz)
            tol = 1e-6 if precision == 64 else 2e-6
            assert abs(d[0] - sx) < tol and abs(d[2] - sz) < tol, (i, d, sx, sz)
        simulation.stop(p)


def test_thermal_trajectory_vs_oracle_fp64():
    """T > 0: the device draws the same Philox stream as the oracle, so FP64 trajectories agree
    to rounding (the reference's mt19937 stream cannot be reproduced on a GPU)."""
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation
    import spirit_gb300.parameters.llg as llg

    spec = dict(GRAD_CASES["sc3d_ddi"])
    spec["llg"] = dict(dt=5e-4, damping=0.1, temperature=10.0, seed=4321)
    s0 = random_spins(8 * 8 * 4, 99)
    ref, r = OracleSystem(spec).llg(s0, "Heun", 30, dt=5e-4, damping=0.1, temperature=10.0, seed=4321, stream=0)
    with make_state(spec, s0, precision=64) as p:
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_HEUN, 30)
        s = spins_of(p)
    assert np.abs(s - ref).max() < 1e-9


def test_thermal_trajectory_vs_oracle_fp32():
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation

    spec = dict(GRAD_CASES["sq_c1"])
    spec["llg"] = dict(dt=1e-3, damping=0.2, temperature=20.0, seed=77)
    s0 = random_spins(64, 98)
    ref, _ = OracleSystem(spec).llg(s0, "SIB", 50, dt=1e-3, damping=0.2, temperature=20.0, seed=77, stream=0)
    with make_state(spec, s0, precision=32) as p:
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_SIB, 50)
        s = spins_of(p)
    assert np.abs(s - ref).max() < 1e-4


@pytest.mark.parametrize("solver", ["Heun", "RK4", "SIB"])
def test_row_fused_stages_bitwise(solver, monkeypatch):
    """The row-fused stage kernels (passes along a inside the stage kernel) give the same FP32
    trajectory, bit for bit, as the separate passes A / A' with the same line pairs (thermal noise
    on, dipolar field, 40 steps); SPIRIT_GB300_ROWS=0 selects the separate passes."""
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation

    spec = dict(GRAD_CASES["sc3d_ddi"], n_cells=[32, 24, 4],
                llg=dict(dt=5e-4, damping=0.1, temperature=10.0, seed=3))
    n = 32 * 24 * 4
    s0 = random_spins(n, 21)
    out = []
    for rows in ("1", "0"):
        monkeypatch.setenv("SPIRIT_GB300_ROWS", rows)
        with make_state(spec, s0, precision=32, name="rows%s_%s" % (rows, solver)) as p:
            simulation.start(p, simulation.METHOD_LLG, getattr(simulation, "SOLVER_" + solver.upper()), 40)
            out.append(spins_of(p))
    np.testing.assert_array_equal(out[0], out[1])


def _tuning(p):
    import ctypes

    from spirit_gb300.spiritlib import fn

    get = fn("Simulation_Get_Tuning", [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int], ctypes.c_int)
    v = (ctypes.c_int * 16)()
    n = get(p, v, 16, -1, -1)
    return [int(v[k]) for k in range(n)]


@pytest.mark.parametrize("tma", ["1", "0"])
def test_tma_stage_kernel_selected(tma, monkeypatch):
    """With SPIRIT_GB300_TMA=1 an FP32 2D system runs the TMA-staged stage kernel (tuning value 12);
    otherwise llg_stage; FP32 keeps the compensated state (value 13); FP64 uses neither."""
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation

    monkeypatch.setenv("SPIRIT_GB300_TMA", tma)
    spec = dict(GRAD_CASES["sq_c1"], n_cells=[48, 40, 1], llg=dict(dt=1e-3, damping=0.2, temperature=5.0, seed=1))
    for prec in (32, 64):
        with make_state(spec, random_spins(48 * 40, 5), precision=prec, name="tmasel%s" % tma) as p:
            simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_SIB, 4)
            t = _tuning(p)
        assert len(t) >= 14
        assert t[12] == (1 if (tma == "1" and prec == 32) else 0), (prec, t)
        assert t[13] == (1 if prec == 32 else 0), (prec, t)


@pytest.mark.parametrize("solver", ["SIB", "Heun", "RK4", "Depondt"])
def test_tma_stage_kernel_matches(solver, monkeypatch):
    """The TMA-staged persistent stage kernel (tiles of 1024 spins, configuration window in shared
    memory, SPIRIT_GB300_TMA=1) runs llg_stage's arithmetic: the same FP32 trajectory as llg_stage
    reading neighbours from global memory, to rounding (the compiler may fuse multiplies and adds
    differently in the two kernels): a batch of uneven 2D systems (periodic and open, Neel DMI,
    thermal noise, one with the dipolar interaction), 30 steps, max |dm| <= 1e-6."""
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation
    import contextlib

    specs = [dict(GRAD_CASES["sq_c1"], n_cells=[L, M, 1], bc=bc,
                  llg=dict(dt=1e-3, damping=0.2, temperature=T, seed=11 + k))
             for k, (L, M, bc, T) in enumerate([(45, 37, [1, 1, 0], 15.0), (64, 64, [0, 1, 0], 5.0),
                                                 (33, 70, [1, 0, 0], 0.0), (200, 9, [1, 1, 0], 30.0)])]
    specs.append(dict(GRAD_CASES["open2d_ddi"], n_cells=[40, 24, 1],
                      llg=dict(dt=1e-3, damping=0.3, temperature=4.0, seed=99)))
    s0 = [random_spins(sp["n_cells"][0] * sp["n_cells"][1], 300 + k) for k, sp in enumerate(specs)]
    out = {}
    for tma in ("1", "0"):
        monkeypatch.setenv("SPIRIT_GB300_TMA", tma)
        with contextlib.ExitStack() as st:
            ps = [st.enter_context(make_state(sp, x, precision=32, name="tma%s_%d" % (tma, k)))
                  for k, (sp, x) in enumerate(zip(specs, s0))]
            simulation.start_batched(ps, getattr(simulation, "SOLVER_" + solver.upper()), 30)
            out[tma] = [spins_of(p) for p in ps]
    for a, b in zip(out["1"], out["0"]):
        assert np.abs(a - b).max() <= 1e-6
