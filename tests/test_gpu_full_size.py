"""GPU parity at the benchmark configurations' full sizes.

Fixtures (tests/golden/full_*.npz) come from the reference itself (make_golden.py): the plain-LLG
configuration exactly (SC 64 x 64 periodic, Neel DMI, Depondt, dt 1e-3 ps, alpha 0.3, 1000 steps)
and the dipolar configuration's system (SC 128 x 128 x 16, bulk DMI, DDI FFT zero-padded along c,
Heun, dt 5e-4 ps, alpha 0.1) over 100 steps, both at T = 0.  Inputs are regenerated from the
fixture's seed with oracle.portable_spins (bit-identical on every platform) and checked against
the stored sums.  Longer runs of the dipolar system are compared with the oracle (the CPU FP64
restatement pinned to these fixtures by tests/test_oracle_golden.py::test_llg_full_size).

Tolerances (max |dm| over all spins and components):
  FP64 device: 1e-10 after the fixture's steps; energy 1e-10 relative.
  FP32 device: 1e-5 after 1000 steps (the metric's bar) and after the fixture's 100 dipolar steps;
               the energy of the FP32 path is within 1e-8 meV per spin of the FP64 oracle.
"""
import numpy as np
import pytest

from cases import FULL_CASES
from conftest import golden
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu


def _case(name):
    from oracle.oracle import portable_spins

    (spec, sname, sid, n_iter, seed), = [c[1:] for c in FULL_CASES if c[0] == name]
    f = golden("full_%s.npz" % name)
    n = spec["n_cells"]
    s0 = portable_spins(n[0] * n[1] * n[2], seed)
    assert np.array_equal(s0[:64], f["spins_in_head"]) and np.array_equal(s0.sum(axis=0), f["spins_in_sum"])
    return f, spec, s0, sid, n_iter


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("name", ["c1_full", "c1_full_sib", "c1_full_heun", "c1_full_rk4"])
def test_c1_full_1000_steps(name, precision):
    """SC 64 x 64, 1000 steps against the reference run: Depondt (the configuration itself), SIB,
    Heun and RK4."""
    from spirit_gb300 import simulation, system

    f, spec, s0, sid, n_iter = _case(name)
    with make_state(spec, s0, precision=precision) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, n_iter)
        s = spins_of(p)
        it = simulation.get_iteration(p)
        E = system.get_energy_fp64(p)
    assert it == n_iter == int(f["iterations"])
    dm = np.abs(s - f["spins_out"]).max()
    print("%s FP%d: max|dm| vs reference after %d steps = %.3e" % (name, precision, n_iter, dm))
    if precision == 64:
        assert dm <= 1e-10, dm
        assert abs(E - f["energy"]) <= 1e-10 * abs(f["energy"])
    else:
        assert dm <= 1e-5, dm
        assert abs(E - f["energy"]) <= 1e-6 * abs(f["energy"])


@pytest.mark.parametrize("precision", [64, 32])
def test_c2_dipolar_100_steps(precision):
    """SC 128 x 128 x 16 with the dipolar interaction, Heun, 100 steps against the reference run."""
    from spirit_gb300 import simulation, system

    f, spec, s0, sid, n_iter = _case("c2_t0")
    with make_state(spec, s0, precision=precision) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, n_iter)
        s = spins_of(p)
        E = system.get_energy_fp64(p)
    dm16 = np.abs(s[::16] - f["spins_out_fp64_every16"]).max()
    dm = np.abs(s - f["spins_out"].astype(np.float64)).max()
    if precision == 64:
        assert dm16 <= 1e-10, dm16
        assert dm <= 1e-7, dm  # the full output is stored in FP32
        assert abs(E - f["energy"]) <= 1e-10 * abs(f["energy"])
    else:
        assert dm <= 1e-5, dm
        assert abs(E - f["energy"]) <= 1e-6 * abs(f["energy"])


def test_c2_dipolar_fp32_1000_steps_vs_oracle():
    """The metric's bar on the dipolar system: FP32 device, 1000 Heun steps at T = 0, max |dm|
    <= 1e-5 against the FP64 oracle (pinned to the reference at this size)."""
    from oracle.oracle import OracleSystem
    from spirit_gb300 import simulation

    f, spec, s0, sid, _ = _case("c2_t0")
    n = 1000
    ll = spec["llg"]
    ref, r = OracleSystem(spec).llg(s0, sid, n, dt=ll["dt"], damping=ll["damping"], temperature=0.0)
    with make_state(spec, s0, precision=32) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, n)
        s = spins_of(p)
    dm = np.abs(s - ref).max()
    print("C2 system, FP32, 1000 Heun steps: max|dm| vs FP64 oracle = %.3e" % dm)
    assert dm <= 1e-5, dm


@pytest.mark.parametrize("which", ["random", "after_100_steps"])
def test_c2_fp32_energy_error(which):
    """Energy of the FP32 path against the FP64 oracle on the full dipolar system (262,144 spins):
    the stage kernels' energy of a configuration (the probe evaluation a single-shot start makes:
    FP32 field and per-spin terms, compensated sums) against the oracle's FP64 energy of the same
    configuration -- a random one and the reference's configuration after 100 Heun steps.
    Bound: 1e-8 meV per spin (|E| / N is 0.05-0.5 meV here)."""
    from oracle.oracle import OracleSystem
    from spirit_gb300 import simulation, system

    f, spec, s0, sid, n_iter = _case("c2_t0")
    x = s0 if which == "random" else f["spins_out"].astype(np.float64)
    nos = x.shape[0]
    ref = OracleSystem(spec).energy(x)
    with make_state(spec, x, precision=32) as p:
        simulation.start(p, simulation.METHOD_LLG, sid, -1, -1, True)
        E = system.get_energy_fp64(p)
        simulation.stop(p)
    err = abs(E - ref) / nos
    print("FP32 path energy error (%s configuration): %.3e meV per spin, %.3e relative (E = %.6f meV)"
          % (which, err, abs(E - ref) / abs(ref), ref))
    assert err <= 1e-8, (E, ref)


@pytest.mark.parametrize("name", ["c1_full", "c2_t0"])
def test_compensated_state_accuracy(name, monkeypatch):
    """FP32 with the compensated state (spins kept as hi + lo float pairs, updates added with
    error-free transformations) against the plain FP32 state, both against the reference run:
    the compensated state removes the accumulated rounding of the stored spins."""
    from spirit_gb300 import simulation

    f, spec, s0, sid, n_iter = _case(name)
    ref = f["spins_out"].astype(np.float64)
    dm = {}
    for comp in ("1", "0"):
        monkeypatch.setenv("SPIRIT_GB300_COMP", comp)
        with make_state(spec, s0, precision=32, name="comp" + comp) as p:
            simulation.start(p, simulation.METHOD_LLG, sid, n_iter)
            dm[comp] = float(np.abs(spins_of(p) - ref).max())
    print("%s FP32 max|dm| vs reference: compensated %.3e, plain %.3e" % (name, dm["1"], dm["0"]))
    assert dm["1"] <= dm["0"] and dm["1"] <= 1e-5, dm
