"""OVF interchange with the reference itself, both ways (core/src/Spirit/IO.cpp:186-292,
core/src/io/OVF_File.cpp).

Fixtures (tests/golden/make_golden.py, reference Spirit v2.2.0 built from its sources):
  tests/golden/ovf/reference_<fmt>.ovf   the seeded spins written by the reference's IO_Image_Write
                                         in each data format (its double build writes "Binary 8"
                                         for the binary-4 request too);
  tests/golden/ovf/spirit_gb300_<fmt>.ovf  the same spins written by this library;
  tests/golden/ovf_interchange.npz       the spins, and what the reference's IO_Image_Read read
                                         from each of this library's files.
Tolerances: binary 8 and text to 1e-15 (text carries 17 significant digits here) -- reading
normalises each vector, which may move the last bit; binary 4 to FP32 rounding (1e-7).
"""
import os

import numpy as np
import pytest

from cases import OVF_FORMATS, OVF_SPEC
from conftest import GOLDEN, golden
from helpers import make_state, spins_of

TOL = {"bin4": 1e-7, "bin8": 1e-15, "text": 1e-12, "csv": 1e-12}


@pytest.mark.parametrize("fmt", sorted(OVF_FORMATS))
def test_read_reference_written_file(fmt):
    """IO_Image_Read of a file the reference wrote gives the spins the reference held."""
    from spirit_gb300 import configuration, io

    f = golden("ovf_interchange.npz")
    path = os.path.join(GOLDEN, "ovf", "reference_%s.ovf" % fmt)
    with make_state(OVF_SPEC) as p:
        configuration.plus_z(p)
        assert io.n_images_in_file(p, path) == 1
        io.image_read(p, path)
        s = spins_of(p)
    assert np.abs(s - f["spins"]).max() <= max(TOL[fmt], 1e-15), fmt


@pytest.mark.parametrize("fmt", sorted(OVF_FORMATS))
def test_reference_reads_our_file(fmt):
    """The reference's IO_Image_Read of a file this library wrote gives the spins we wrote; the
    committed file is also what this library writes for the same spins today (bit for bit after the
    header's title line)."""
    from spirit_gb300 import io, system
    from helpers import _TMP

    f = golden("ovf_interchange.npz")
    read = f["reference_read_" + fmt]
    assert np.abs(read - f["spins"]).max() <= TOL[fmt], fmt
    out = os.path.join(_TMP, "ours_%s_%d.ovf" % (fmt, os.getpid()))
    with make_state(OVF_SPEC) as p:
        system.get_spin_directions(p)[:] = f["spins"]
        io.image_write(p, out, OVF_FORMATS[fmt], "written by spirit_gb300")
    committed = open(os.path.join(GOLDEN, "ovf", "spirit_gb300_%s.ovf" % fmt), "rb").read()
    assert open(out, "rb").read() == committed
