"""Monte Carlo on the GPU (Simulation_MC_Start).

The device sweeps colour by colour with one Philox block per spin and sweep; the oracle runs the
same sweep on the CPU in FP64, so FP64 runs agree with it to rounding (tolerance 1e-12, also the
adapted cone angle).  The FP32 path is checked by statistics: free spins in a field against the
Langevin function.  At T = 0 the energy never rises.
"""
import numpy as np
import pytest

from cases import HEX2D, SQ_C1
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu

MU_B = 0.057883817555
K_B = 0.08617330350

SC3D = dict(bravais="sc", n_cells=[6, 5, 4], lattice_constant=1.0, mu_s=[2.0], bc=[1, 0, 1],
            field=(0.7, (0.2, 0.0, 1.0)), anisotropy=(0.1, (0, 0.6, 0.8)), jij=[1.0, 0.3], dij=[0.2], dm_chirality=1,
            llg=dict(dt=1e-3, damping=0.3, temperature=0.0))


@pytest.mark.parametrize("name,spec", [("sq", SQ_C1), ("hex", HEX2D), ("sc3d", SC3D)])
def test_mc_fp64_equals_oracle(name, spec):
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation
    import spirit_gb300.parameters.mc as mc

    n = spec["n_cells"][0] * spec["n_cells"][1] * spec["n_cells"][2]
    s0 = random_spins(n, 17)
    T, sweeps = 5.0, 30
    with make_state(spec, s0, precision=64, name="mc_" + name) as p:
        mc.set_temperature(p, T)
        simulation.start(p, simulation.METHOD_MC, n_iterations=sweeps)
        got = spins_of(p)
        cone = mc.get_metropolis_cone(p)[1]
    ref, st = OracleSystem(spec).mc(s0, sweeps, temperature=T, seed=2006, stream=0)
    assert np.abs(got - ref).max() <= 1e-12
    assert abs(cone - st["cone_angle"]) < 1e-4  # the API returns it as float


def test_mc_single_shot_equals_run_fp64():
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation
    import spirit_gb300.parameters.mc as mc

    s0 = random_spins(64, 4)
    out = []
    for mode in range(2):
        with make_state(SQ_C1, s0, precision=64, name="mcs%d" % mode) as p:
            mc.set_temperature(p, 3.0)
            if mode == 0:
                simulation.start(p, simulation.METHOD_MC, n_iterations=20)
            else:
                simulation.start(p, simulation.METHOD_MC, n_iterations=20, single_shot=True)
                simulation.n_shot(p, 12)
                simulation.n_shot(p, 8)
            out.append(spins_of(p))
    np.testing.assert_array_equal(out[0], out[1])


def test_mc_fp32_langevin_statistics():
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation
    import spirit_gb300.parameters.mc as mc

    spec = dict(bravais="sc", n_cells=[64, 64, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                field=(2.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[], dij=[], dm_chirality=1,
                llg=dict(dt=1e-3, damping=0.3, temperature=0.0))
    T = 20.0
    with make_state(spec, random_spins(64 * 64, 2), precision=32, name="mclang") as p:
        mc.set_temperature(p, T)
        simulation.start(p, simulation.METHOD_MC, n_iterations=200)
        mz = []
        for _ in range(40):
            simulation.start(p, simulation.METHOD_MC, n_iterations=5)
            mz.append(spins_of(p)[:, 2].mean())
    x = 2.0 * MU_B * 2.0 / (K_B * T)
    L = 1.0 / np.tanh(x) - 1.0 / x
    err = np.std(mz) / np.sqrt(len(mz))
    assert abs(np.mean(mz) - L) < 5 * max(err, 1e-3), (np.mean(mz), L, err)


@pytest.mark.parametrize("precision", [64, 32])
def test_mc_zero_temperature_lowers_energy(precision):
    from oracle.oracle import random_spins
    from spirit_gb300 import hamiltonian, simulation

    with make_state(SC3D, random_spins(120, 9), precision=precision, name="mc0") as p:
        e = [hamiltonian.get_gradient(p)[1]]
        for _ in range(5):
            simulation.start(p, simulation.METHOD_MC, n_iterations=4)
            e.append(hamiltonian.get_gradient(p)[1])
    assert all(b <= a + 1e-9 for a, b in zip(e, e[1:])), e
    assert e[-1] < e[0]
