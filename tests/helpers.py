"""Shared helpers of the parity tests: build a State from a spec, inject spins, query."""
import contextlib
import os
import tempfile

import numpy as np

_TMP = tempfile.mkdtemp(prefix="sg_tests_")


@contextlib.contextmanager
def make_state(spec, spins=None, precision=None, name="case"):
    from spirit_gb300 import simulation, state, system
    from spirit_gb300.configs import write_config

    cfg = write_config(spec, os.path.join(_TMP, "%s_%d.cfg" % (name, os.getpid())))
    p = state.setup(cfg, True)
    try:
        if spins is not None:
            system.get_spin_directions(p)[:] = spins
        if precision is not None:
            simulation.set_precision(p, precision)
        yield p
    finally:
        state.delete(p)


def spins_of(p, idx_image=-1):
    from spirit_gb300 import system

    return np.array(system.get_spin_directions(p, idx_image))
