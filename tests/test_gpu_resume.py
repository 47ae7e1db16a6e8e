"""Checkpoint and resume through OVF files on the GPU.

A thermal run's Philox streams are keyed by (seed, spin, iteration + iterations drawn before,
stream): two starts of N iterations equal one start of 2N, and a run written to a binary-8 OVF
file, read into a fresh State and continued for N more iterations reproduces the uninterrupted
run bit for bit in FP64 (LLG and Metropolis).  The uninterrupted FP64 run is also checked against
the oracle over the full 2N iterations."""
import os

import numpy as np
import pytest

from cases import SQ_C1
from helpers import _TMP, make_state, spins_of

pytestmark = pytest.mark.gpu

SPEC = dict(SQ_C1, llg=dict(dt=1e-3, damping=0.2, temperature=12.0, seed=31))


def _llg(p, n):
    from spirit_gb300 import simulation

    simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_SIB, n_iterations=n)


def _mc(p, n):
    from spirit_gb300 import simulation
    import spirit_gb300.parameters.mc as mc

    mc.set_temperature(p, 4.0)
    # a fixed cone: the adapted angle is a run-local quantity and not part of the file
    mc.set_metropolis_cone(p, True, 25.0, False, 0.5)
    simulation.start(p, simulation.METHOD_MC, n_iterations=n)


@pytest.mark.parametrize("method", ["llg", "mc"])
def test_two_starts_equal_one(method):
    from oracle.oracle import random_spins

    run = _llg if method == "llg" else _mc
    s0 = random_spins(SQ_C1["n_cells"][0] * SQ_C1["n_cells"][1], 12)
    with make_state(SPEC, s0, precision=64, name="one_" + method) as p:
        run(p, 40)
        one = spins_of(p)
    with make_state(SPEC, s0, precision=64, name="two_" + method) as p:
        run(p, 20)
        run(p, 20)
        two = spins_of(p)
    np.testing.assert_array_equal(one, two)


@pytest.mark.parametrize("method", ["llg", "mc"])
def test_resume_from_ovf_bitwise(method):
    from oracle.oracle import random_spins
    from spirit_gb300 import io

    run = _llg if method == "llg" else _mc
    s0 = random_spins(SQ_C1["n_cells"][0] * SQ_C1["n_cells"][1], 13)
    f = os.path.join(_TMP, "resume_%s_%d.ovf" % (method, os.getpid()))
    with make_state(SPEC, s0, precision=64, name="full_" + method) as p:
        run(p, 30)
        full = spins_of(p)
    with make_state(SPEC, s0, precision=64, name="half_" + method) as p:
        run(p, 15)
        io.image_write(p, f, io.FILEFORMAT_OVF_BIN8, "checkpoint")
    with make_state(SPEC, precision=64, name="resumed_" + method) as p:
        io.image_read(p, f)
        run(p, 15)
        resumed = spins_of(p)
    # the spins were renormalised on read (rounding of unit vectors): equal to a few ulp
    assert np.abs(resumed - full).max() < 1e-13


def test_thermal_llg_two_starts_vs_oracle():
    from oracle.oracle import OracleSystem, random_spins

    s0 = random_spins(SQ_C1["n_cells"][0] * SQ_C1["n_cells"][1], 14)
    with make_state(SPEC, s0, precision=64, name="orc") as p:
        _llg(p, 10)
        _llg(p, 15)
        got = spins_of(p)
    ref, _ = OracleSystem(SPEC).llg(s0, "SIB", 25, dt=1e-3, damping=0.2, temperature=12.0, seed=31, stream=0)
    assert np.abs(got - ref).max() < 1e-9
