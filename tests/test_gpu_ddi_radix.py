"""Dipolar field on padded extents whose transforms run the mixed-radix Stockham path of the FFT
passes (register radices 2 ... 12 chosen by the device's cost planner), on one-row (2D: the
single-block b/c pass, several ka planes per block) and 3D layouts, against the FP64 oracle.

Extents (the zero-padded axes are 2N, 7-smooth here, so the oracle's padding is the same) and the
device's radix plans (power-of-two extents take the register power-of-two path):
  open 7 x 21 x 1    -> 14 x 42      (7*2, 7*6)
  open 15 x 10 x 1   -> 30 x 20      (6*5, 5*4)
  open 5 x 7 x 9     -> 10 x 14 x 18 (10, 7*2, 6*3)
  open 40 x 27 x 1   -> 80 x 54      (10*8, 9*6)
  open 18 x 6 x 6    -> 36 x 12 x 12 (9*4, 12, 12)
  periodic 12 x 9 x 3, no padding -> 12 x 9 x 3 (12, 9, 3)
  periodic 11 x 13 x 2, no padding -> 11 x 13 x 2 (prime lengths 11 and 13: direct-sum stages; 2)

Tolerances: FP64 gradient 1e-12 relative to max |g| (as the golden gradient cases); FP32 RK4
trajectory of 20 steps max |dm| <= 1e-5 against the FP64 oracle (the metric's bar).
"""
import numpy as np
import pytest

from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu

_OPEN = dict(bravais="sc", lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0], field=(0.8, (0, 0, 1)),
             anisotropy=(0.1, (0, 0, 1)), jij=[1.0], dij=[0.3], dm_chirality=2,
             ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1),
             llg=dict(dt=1e-3, damping=0.3, temperature=0.0))

CASES = {
    "open2d_7x21": dict(_OPEN, n_cells=[7, 21, 1]),
    "open2d_15x10": dict(_OPEN, n_cells=[15, 10, 1]),
    "open3d_5x7x9": dict(_OPEN, n_cells=[5, 7, 9], lattice_constant=3.0),
    "open2d_40x27": dict(_OPEN, n_cells=[40, 27, 1]),
    "open3d_18x6x6": dict(_OPEN, n_cells=[18, 6, 6], lattice_constant=3.0),
    "periodic_12x9x3": dict(_OPEN, n_cells=[12, 9, 3], bc=[1, 1, 1], lattice_constant=2.5,
                            ddi=dict(method="fft", n_periodic_images=[1, 1, 1], radius=0.0, pb_zero_padding=0)),
    "periodic_11x13x2": dict(_OPEN, n_cells=[11, 13, 2], bc=[1, 1, 1], lattice_constant=2.5,
                             ddi=dict(method="fft", n_periodic_images=[1, 1, 1], radius=0.0, pb_zero_padding=0)),
}


def _spins(spec, seed):
    from oracle.oracle import random_spins

    n = spec["n_cells"][0] * spec["n_cells"][1] * spec["n_cells"][2]
    return random_spins(n, seed)


@pytest.mark.parametrize("name", sorted(CASES))
def test_ddi_gradient_mixed_radix_fp64(name):
    from oracle.oracle import OracleSystem
    from spirit_gb300 import hamiltonian

    spec = CASES[name]
    s = _spins(spec, 31)
    ref, E_ref = OracleSystem(spec).gradient_and_energy(s)
    with make_state(spec, s, name="radix_" + name) as p:
        g, E = hamiltonian.get_gradient(p)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(g, ref, rtol=0, atol=1e-12 * scale)
    assert abs(E - E_ref) <= 1e-10 * abs(E_ref)


@pytest.mark.parametrize("name", sorted(CASES))
def test_ddi_rk4_mixed_radix_fp32(name):
    from oracle.oracle import OracleSystem
    from spirit_gb300 import simulation

    spec = CASES[name]
    s0 = _spins(spec, 32)
    ref, _ = OracleSystem(spec).llg(s0, "RK4", 20, dt=1e-3, damping=0.3)
    with make_state(spec, s0, precision=32, name="radix32_" + name) as p:
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_RK4, 20)
        s = spins_of(p)
    assert np.abs(s - ref).max() <= 1e-5


@pytest.mark.parametrize("n_cells", [[16, 16, 8], [12, 12, 6]])
def test_cluster_split_bitwise(n_cells, monkeypatch):
    """The fused b/c pass on one block per plane (K = 1) and split over clusters of K = 2, 4, 8
    blocks gives the same FP32 Heun trajectory bit for bit: 16 x 16 x 8 (z-padded to 16) takes the
    power-of-two index splits, 12 x 12 x 6 (Mb / K = 6, 3) the run-time divisions; shapes the plan
    cannot take (K > Nc) fall back to the tuned one.  The trajectory matches the FP64 oracle."""
    from cases import SC3D_DDI
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation

    spec = dict(SC3D_DDI, n_cells=n_cells, llg=dict(dt=5e-4, damping=0.1, temperature=0.0))
    n = n_cells[0] * n_cells[1] * n_cells[2]
    s0 = random_spins(n, 41)
    out = []
    for K in (1, 2, 4, 8):
        monkeypatch.setenv("SPIRIT_GB300_BC", "%d,512" % K)
        with make_state(spec, s0, precision=32, name="bc%d_%d" % (K, n)) as p:
            simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_HEUN, 20)
            out.append(spins_of(p))
    for o in out[1:]:
        np.testing.assert_array_equal(o, out[0])
    ref, _ = OracleSystem(spec).llg(s0, "Heun", 20, dt=5e-4, damping=0.1)
    assert np.abs(out[0] - ref).max() <= 1e-5
