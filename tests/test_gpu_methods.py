"""GPU parity of GNEB (VP, climbing image), direct minimisation and batched LLG.

Reference known answers: core/test/test_solvers.cpp (energy -5849.69140625 meV and m_z = 2*0.79977
after direct minimisation of a skyrmion; GNEB skyrmion-collapse saddle -5811.5244140625 meV,
m_z = 2*0.96657), and the golden GNEB fixtures made from the reference's own code.
"""
import numpy as np
import pytest

from cases import GRAD_CASES, SOLVERS
from conftest import golden
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu


def _load_chain(p, chain_in):
    from spirit_gb300 import chain, system

    noi = chain_in.shape[0]
    chain.image_to_clipboard(p)
    for _ in range(1, noi):
        chain.insert_image_after(p)
    for i in range(noi):
        system.get_spin_directions(p, i)[:] = chain_in[i]


@pytest.mark.parametrize("tag", ["gneb_vp", "gneb_vp_ci", "gneb_vp_oso", "gneb_lbfgs_oso", "gneb_lbfgs_oso_ci"])
def test_gneb_short_fp64(tag):
    from spirit_gb300 import chain, simulation, system
    import spirit_gb300.parameters.gneb as gneb

    f = golden("%s.npz" % tag)
    sid = int(f["solver"]) if "solver" in f else simulation.SOLVER_VP
    with make_state(SOLVERS, precision=64) as p:
        _load_chain(p, f["chain_in"])
        simulation.start(p, simulation.METHOD_GNEB, sid, int(f["n_iter"]))
        if int(f["n_iter_ci"]) > 0:
            gneb.set_image_type_automatically(p)
            types = [gneb.get_climbing_falling(p, i) for i in range(9)]
            assert types == list(f["image_type"])
            simulation.start(p, simulation.METHOD_GNEB, sid, int(f["n_iter_ci"]))
        out = np.stack([spins_of(p, i) for i in range(9)])
        E = np.array([system.get_energy_fp64(p, i) for i in range(9)])
        Rx = np.array([system.get_rx(p, i) for i in range(9)])
    assert np.abs(out - f["chain_out"]).max() < 1e-9
    np.testing.assert_allclose(E, f["energies"], rtol=1e-11)
    np.testing.assert_allclose(Rx, f["Rx"], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("solver", [0, 5, 7])
def test_gneb_converged_saddle(solver, precision):
    """Skyrmion collapse on the reference solver-test system (core/test/test_solvers.cpp:73-133,
    solvers VP, LBFGS_OSO, VP_OSO): 20000 iterations, then climbing image until the max torque is
    below the convergence threshold (1e-6 meV FP64, 1e-4 FP32 as the reference's float build
    uses); the saddle energy matches the reference within 1e-5 (FP64) / 5e-3 (FP32)."""
    from spirit_gb300 import simulation, system
    import spirit_gb300.parameters.gneb as gneb

    f = golden("gneb_converged.npz")
    conv, tol = (1e-6, 1e-5) if precision == 64 else (1e-4, 5e-3)
    with make_state(SOLVERS, precision=precision) as p:
        gneb.set_convergence(p, conv)
        _load_chain(p, f["chain_in"])
        simulation.start(p, simulation.METHOD_GNEB, solver, 20000)
        gneb.set_image_type_automatically(p)
        simulation.start(p, simulation.METHOD_GNEB, solver, 200000)
        E = np.array([system.get_energy_fp64(p, i) for i in range(9)])
        mt = simulation.get_max_torque_norm(p)
    assert mt < conv
    assert abs(E.max() - f["energies"].max()) < tol
    # the reference test compares System_Get_Energy (a float) with its float literal
    assert abs(float(np.float32(E.max())) - (-5811.5244140625)) < tol


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("solver", [0, 1, 2, 3, 4, 5, 7])
def test_direct_minimisation_skyrmion(solver, precision):
    """core/test/test_solvers.cpp:18-70: plus-z with a skyrmion of radius 5 (order 1, phase -90),
    direct minimisation to convergence; E = -5849.69140625 meV, m = (0, 0, 2*0.79977)."""
    from spirit_gb300 import configuration, quantities, simulation, system
    import spirit_gb300.parameters.llg as llg

    conv, tol = (1e-8, 1e-5) if precision == 64 else (1e-5, 5e-3)
    with make_state(SOLVERS, precision=precision) as p:
        llg.set_direct_minimization(p, True)
        llg.set_convergence(p, conv)
        configuration.plus_z(p)
        configuration.skyrmion(p, 5, order=1, phase=-90, up_down=False, achiral=False, right_left=False)
        simulation.start(p, simulation.METHOD_LLG, solver, 2000000)
        E = system.get_energy(p)
        m = quantities.get_magnetization(p)
    assert abs(E - (-5849.69140625)) < tol
    assert abs(m[0]) < tol and abs(m[1]) < tol and abs(m[2] - 2.0 * 0.79977) < tol


def test_batched_equals_individual():
    """Batched LLG over uneven systems (different sizes, parameters and lattices) gives the same
    T = 0 trajectories as running each system alone, bit for bit (same kernels, same per-system
    thread decomposition)."""
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation

    specs = []
    for k, L in enumerate([7, 16, 33]):
        s = dict(GRAD_CASES["sq_c1"])
        s["n_cells"] = [L, L + 2, 1]
        s["jij"] = [0.5 + 0.3 * k]
        s["field"] = (0.3 * k, (0, 0, 1))
        s["llg"] = dict(dt=1e-3, damping=0.2, temperature=0.0)
        specs.append(s)
    specs.append(dict(GRAD_CASES["hex2d"], llg=dict(dt=1e-3, damping=0.2, temperature=0.0)))
    inits = [random_spins(s["n_cells"][0] * s["n_cells"][1], 50 + k) for k, s in enumerate(specs)]
    ctxs = [make_state(s, x, precision=32, name="b%d" % k) for k, (s, x) in enumerate(zip(specs, inits))]
    ps = [c.__enter__() for c in ctxs]
    simulation.start_batched(ps, simulation.SOLVER_SIB, 40)
    batched = [spins_of(p) for p in ps]
    for c in ctxs:
        c.__exit__(None, None, None)
    for k, (s, x) in enumerate(zip(specs, inits)):
        with make_state(s, x, precision=32, name="i%d" % k) as p:
            simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_SIB, 40)
            np.testing.assert_array_equal(spins_of(p), batched[k])


def test_batched_uneven_vs_oracle():
    """Each member of an uneven batch against the FP64 oracle with the same Philox stream."""
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation

    specs, inits = [], []
    for k, L in enumerate([9, 20, 31, 12]):
        s = dict(GRAD_CASES["sq_c1"])
        s["n_cells"] = [L, 40 - L, 1]
        s["dij"] = [0.1 * k]
        s["anisotropy"] = (0.05 * k, (0, 0, 1))
        s["llg"] = dict(dt=1e-3, damping=0.2, temperature=10.0 * k, seed=5)
        specs.append(s)
        inits.append(random_spins(L * (40 - L), 70 + k))
    ctxs = [make_state(s, x, precision=64, name="u%d" % k) for k, (s, x) in enumerate(zip(specs, inits))]
    ps = [c.__enter__() for c in ctxs]
    simulation.start_batched(ps, simulation.SOLVER_SIB, 25)
    out = [spins_of(p) for p in ps]
    for c in ctxs:
        c.__exit__(None, None, None)
    for k, (s, x) in enumerate(zip(specs, inits)):
        ref, _ = OracleSystem(s).llg(x, "SIB", 25, dt=1e-3, damping=0.2, temperature=10.0 * k, seed=5, stream=k)
        assert np.abs(out[k] - ref).max() < 1e-9, k


def test_batched_launch_steps_equals_start_batched():
    """The caller-driven batched run (Launch_Steps in pieces, then Finish) gives the same spins,
    bit for bit, as one Simulation_LLG_Start_Batched of the same number of steps (T > 0: the
    Philox counters advance with the device iteration, not with the host calls)."""
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation

    specs = []
    for k, L in enumerate([10, 23, 17]):
        s = dict(GRAD_CASES["sq_c1"])
        s["n_cells"] = [L, 30 - L, 1]
        s["llg"] = dict(dt=1e-3, damping=0.2, temperature=15.0 * (k + 1), seed=9)
        specs.append(s)
    inits = [random_spins(s["n_cells"][0] * s["n_cells"][1], 90 + k) for k, s in enumerate(specs)]
    out = []
    for mode in range(2):
        ctxs = [make_state(s, x, precision=32, name="l%d_%d" % (mode, k)) for k, (s, x) in enumerate(zip(specs, inits))]
        ps = [c.__enter__() for c in ctxs]
        if mode == 0:
            simulation.start_batched(ps, simulation.SOLVER_SIB, 37)
        else:
            for n in (5, 16, 9, 7):
                simulation.batched_launch_steps(ps, simulation.SOLVER_SIB, n)
            simulation.batched_finish(ps)
            assert simulation.get_iteration(ps[0]) == 37
        out.append([spins_of(p) for p in ps])
        for c in ctxs:
            c.__exit__(None, None, None)
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
