"""GPU parity of the batched dipolar path: uneven open 2D (and one 3D) systems in one batch, their
dipolar fields from one shared FFT plan table.

Zero-padded axes of the device plan take the smallest even 7-smooth extent >= 2N (the field of a
zero-padded circular convolution equals the linear one for any extent >= 2N - 1); the oracle pads
to exactly 2N, as the reference does (Hamiltonian_Heisenberg.cpp:1501-1595).  Most edges here have
a 2N that is not 7-smooth (2 x 11, 13, 17, 19, 23, 29), so the device transforms a larger volume than
the oracle and the comparison checks that padding rule.

Tolerances:
  FP64 batched gradient: 1e-12 relative to the system's max |g|, energies 1e-11 relative;
  FP64 batched trajectories (Heun, 50 steps, T = 0): 1e-10;
  FP32 batched trajectories (stochastic SIB, 1000 steps, same Philox streams as the oracle):
  max |dm| <= 1e-5 per system (the metric's bar).
"""
import numpy as np
import pytest

from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu

# (n_cells, J, D, K, B, T): open boundaries, lattice constant 4 A, DDI by FFT with zero padding
SYSTEMS = [
    ([11, 11, 1], 1.0, 0.30, 0.10, 0.5, 5.0),
    ([13, 13, 1], 0.7, 0.10, 0.05, 1.5, 12.0),
    ([23, 23, 1], 1.3, 0.35, 0.15, 0.2, 2.0),
    ([29, 29, 1], 0.9, 0.05, 0.20, 1.0, 8.0),
    ([17, 17, 1], 1.2, 0.30, 0.02, 0.3, 1.0),
    ([16, 16, 1], 1.1, 0.25, 0.00, 0.0, 0.0),
    ([21, 21, 1], 0.6, 0.40, 0.12, 1.8, 15.0),
    ([19, 12, 1], 1.4, 0.20, 0.08, 0.7, 3.0),
    ([30, 30, 1], 1.0, 0.15, 0.18, 1.2, 20.0),
    ([11, 9, 3], 1.0, 0.20, 0.05, 0.5, 4.0),
]


def spec_of(k, n, J, D, K, B, T):
    return dict(bravais="sc", n_cells=n, lattice_constant=4.0, mu_s=[2.0], bc=[0, 0, 0],
                field=(B, (0, 0, 1)), anisotropy=(K, (0, 0, 1)), jij=[J], dij=[D], dm_chirality=2,
                ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1),
                llg=dict(dt=1e-3, damping=0.2, temperature=T, seed=700 + k))


def _states(stack, precision, seed_base, temperature=True):
    from oracle.oracle import random_spins

    specs, s0, ps = [], [], []
    for k, (n, J, D, K, B, T) in enumerate(SYSTEMS):
        sp = spec_of(k, n, J, D, K, B, T if temperature else 0.0)
        x = random_spins(n[0] * n[1] * n[2], seed_base + k)
        specs.append(sp)
        s0.append(x)
        ps.append(stack.enter_context(make_state(sp, x, precision=precision, name="bddi%d" % k)))
    return specs, s0, ps


def test_padded_extents_differ_from_2n():
    """Guard: the set contains edges whose exact 2N is not 7-smooth (so the device pads further)."""
    def smooth7(m):
        for r in (2, 3, 5, 7):
            while m % r == 0:
                m //= r
        return m == 1
    assert sum(not smooth7(2 * n[0]) for n, *_ in SYSTEMS) >= 4


def test_batched_gradient_fp64_vs_oracle():
    import contextlib

    from oracle.oracle import OracleSystem
    from spirit_gb300 import hamiltonian

    with contextlib.ExitStack() as st:
        specs, s0, ps = _states(st, 64, 9100)
        grads, energies = hamiltonian.get_gradient_batched(ps)
    for k, sp in enumerate(specs):
        g_ref, e_ref = OracleSystem(sp).gradient_and_energy(s0[k])
        scale = np.abs(g_ref).max()
        err = np.abs(grads[k] - g_ref).max() / scale
        assert err <= 1e-12, (k, SYSTEMS[k][0], err)
        assert abs(energies[k] - e_ref) <= 1e-11 * abs(e_ref), (k, energies[k], e_ref)


def test_batched_trajectories_fp64_vs_oracle():
    import contextlib

    from oracle.oracle import OracleSystem
    from spirit_gb300 import simulation

    n = 50
    with contextlib.ExitStack() as st:
        specs, s0, ps = _states(st, 64, 9200, temperature=False)
        simulation.start_batched(ps, simulation.SOLVER_HEUN, n)
        out = [spins_of(p) for p in ps]
    for k, sp in enumerate(specs):
        ref, _ = OracleSystem(sp).llg(s0[k], "Heun", n, dt=1e-3, damping=0.2, temperature=0.0)
        dm = np.abs(out[k] - ref).max()
        assert dm <= 1e-10, (k, SYSTEMS[k][0], dm)


def test_batched_trajectories_fp32_1000_steps_vs_oracle():
    """Stochastic SIB, 1000 steps, FP32 batched; system k of the batch draws noise stream k."""
    import contextlib

    from oracle.oracle import OracleSystem
    from spirit_gb300 import simulation

    n = 1000
    with contextlib.ExitStack() as st:
        specs, s0, ps = _states(st, 32, 9300)
        simulation.start_batched(ps, simulation.SOLVER_SIB, n)
        out = [spins_of(p) for p in ps]
    worst = 0.0
    for k, sp in enumerate(specs):
        ll = sp["llg"]
        ref, _ = OracleSystem(sp).llg(s0[k], "SIB", n, dt=1e-3, damping=0.2, temperature=ll["temperature"],
                                      seed=ll["seed"], stream=k)
        dm = np.abs(out[k] - ref).max()
        worst = max(worst, dm)
        assert dm <= 1e-5, (k, SYSTEMS[k][0], dm)
    print("batched dipolar FP32, 1000 SIB steps: max|dm| vs FP64 oracle = %.3e" % worst)
