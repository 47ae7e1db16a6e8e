"""OVF 2.0 input and output through the C API (reference tests: core/test/test_io.cpp:21-74,
core/python/test/io_test.py): write/read round trips in every format, appending and segment
counts, chains, vacancies and normalisation on read, files of other writers."""
import os
import struct

import numpy as np
import pytest

from cases import GRAD_CASES, SOLVERS
from helpers import _TMP, make_state, spins_of

FORMATS = {"bin": 0, "bin4": 1, "bin8": 2, "text": 3, "csv": 4}


def _path(name):
    return os.path.join(_TMP, "%s_%d.ovf" % (name, os.getpid()))


@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_image_round_trip_minus_z(fmt):
    from spirit_gb300 import configuration, io

    # test_io.cpp:41-67: write -z, set +z, read back, compare within 1e-12
    f = _path("mz_" + fmt)
    with make_state(GRAD_CASES["sq_c1"]) as p:
        configuration.minus_z(p)
        io.image_write(p, f, FORMATS[fmt], "io test")
        configuration.plus_z(p)
        io.image_read(p, f)
        s = spins_of(p)
        assert np.allclose(s, [0, 0, -1], atol=1e-12, rtol=0)


@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_image_round_trip_random(fmt):
    from spirit_gb300 import configuration, io

    f = _path("rnd_" + fmt)
    with make_state(GRAD_CASES["sc3d_ddi"]) as p:
        configuration.random(p)
        s0 = spins_of(p)
        io.image_write(p, f, FORMATS[fmt], "random")
        configuration.plus_z(p)
        io.image_read(p, f)
        s1 = spins_of(p)
        if fmt == "bin4":
            # 4-byte values, renormalised on read
            assert np.abs(s1 - s0).max() < 1e-6
        else:
            # 17 significant digits / 8-byte values; the read renormalises (rounding only)
            assert np.abs(s1 - s0).max() < 1e-15


def test_binary8_layout_and_header():
    from spirit_gb300 import configuration, geometry, io, system

    f = _path("layout")
    with make_state(GRAD_CASES["sc3d_ddi"]) as p:
        configuration.random(p)
        s0 = spins_of(p)
        io.image_write(p, f, io.FILEFORMAT_OVF_BIN8, "layout")
        raw = open(f, "rb").read()
        nos = system.get_nos(p)
        n = geometry.get_n_cells(p)
    head = raw[: raw.index(b"# Begin: Data Binary 8\n")].decode()
    assert head.startswith("# OOMMF OVF 2.0\n")
    assert "# Segment count: 000001\n" in head
    assert "# valuedim: 3" in head and "# meshtype: rectangular" in head
    assert "# xnodes: %d\n# ynodes: %d\n# znodes: %d\n" % tuple(n) in head
    p0 = raw.index(b"# Begin: Data Binary 8\n") + len(b"# Begin: Data Binary 8\n")
    assert struct.unpack("<d", raw[p0 : p0 + 8])[0] == 123456789012345.0
    data = np.frombuffer(raw[p0 + 8 : p0 + 8 + 24 * nos], dtype="<f8").reshape(-1, 3)
    assert np.array_equal(data, s0)
    assert raw.endswith(b"# End: Data Binary 8\n# End: Segment\n")


def test_append_counts_and_segments():
    from spirit_gb300 import configuration, io

    f = _path("append")
    if os.path.exists(f):
        os.remove(f)
    with make_state(GRAD_CASES["sq_c1"]) as p:
        configuration.plus_z(p)
        io.image_append(p, f, io.FILEFORMAT_OVF_TEXT, "a")
        configuration.minus_z(p)
        io.image_append(p, f, io.FILEFORMAT_OVF_BIN8, "b")
        configuration.random(p)
        s2 = spins_of(p)
        io.image_append(p, f, io.FILEFORMAT_OVF_CSV, "c")
        assert io.n_images_in_file(p, f) == 3
        assert b"# Segment count: 000003\n" in open(f, "rb").read()
        io.image_read(p, f, 1)
        assert np.allclose(spins_of(p), [0, 0, -1], atol=0)
        io.image_read(p, f, 0)
        assert np.allclose(spins_of(p), [0, 0, 1], atol=0)
        io.image_read(p, f, 2)
        assert np.abs(spins_of(p) - s2).max() < 1e-15
        # a segment that is not in the file leaves the image as it was
        io.image_read(p, f, 7)
        assert np.abs(spins_of(p) - s2).max() < 1e-15


def test_chain_write_read():
    from spirit_gb300 import chain, configuration, io

    f = _path("chain")
    with make_state(SOLVERS) as p:
        configuration.plus_z(p)
        chain.image_to_clipboard(p)
        for _ in range(3):
            chain.insert_image_after(p)
        ref = []
        for k in range(4):
            configuration.random(p, idx_image=k)
            ref.append(spins_of(p, k))
        io.chain_write(p, f, io.FILEFORMAT_OVF_BIN8, "chain")
        assert io.n_images_in_file(p, f) == 4
    with make_state(SOLVERS, name="chain2") as p:
        assert chain.get_noi(p) == 1
        io.chain_read(p, f, 0, -1, 0)
        assert chain.get_noi(p) == 4
        for k in range(4):
            assert np.abs(spins_of(p, k) - ref[k]).max() < 1e-15  # renormalised on read
        # appending doubles the file
        io.chain_append(p, f, io.FILEFORMAT_OVF_TEXT, "again")
        assert io.n_images_in_file(p, f) == 8
        io.chain_read(p, f, 6, 6, 1)
        assert np.abs(spins_of(p, 1) - ref[2]).max() < 1e-15


def test_foreign_file_vacancies_and_normalisation():
    """A text file in another writer's layout (different key order, comments, no description of
    random streams): vectors are normalised and near-zero vectors become +z
    (core/src/Spirit/IO.cpp:186-292)."""
    from spirit_gb300 import configuration, io, system

    with make_state(GRAD_CASES["sq_c1"]) as p:
        nos = system.get_nos(p)
        rng = np.random.default_rng(5)
        v = rng.normal(size=(nos, 3)) * 3.0
        v[1] = 0.0
        v[4] = [1e-7, 0, 0]
        lines = [
            "# OOMMF OVF 2.0",
            "# Segment count: 1",
            "# Begin: Segment",
            "# Begin: Header",
            "# Title: written elsewhere",
            "# meshtype: rectangular",
            "# meshunit: nm",
            "# xnodes: %d" % nos,
            "# ynodes: 1",
            "# znodes: 1",
            "# valuedim: 3   ## comment after the value",
            "# End: Header",
            "# Begin: Data Text",
        ]
        lines += ["%.17g %.17g %.17g" % tuple(r) for r in v]
        lines += ["# End: Data Text", "# End: Segment", ""]
        f = _path("foreign")
        open(f, "w").write("\n".join(lines))
        configuration.random(p)
        io.image_read(p, f)
        s = spins_of(p)
        want = v / np.linalg.norm(v, axis=1, keepdims=True)
        want[1] = want[4] = [0, 0, 1]
        assert np.abs(s - want).max() < 1e-15


def test_size_mismatch_reads_common_part():
    from spirit_gb300 import configuration, io, system

    f = _path("small")
    with make_state(GRAD_CASES["sq_c1"]) as p:
        n_small = system.get_nos(p)
        configuration.minus_z(p)
        io.image_write(p, f, io.FILEFORMAT_OVF_BIN8)
    with make_state(GRAD_CASES["sc3d_ddi"], name="big") as p:
        assert system.get_nos(p) > n_small
        configuration.plus_z(p)
        io.image_read(p, f)
        s = spins_of(p)
    assert np.allclose(s[:n_small], [0, 0, -1], atol=0)
    assert np.allclose(s[n_small:], [0, 0, 1], atol=0)


def test_positions_write():
    from spirit_gb300 import geometry, io

    f = _path("pos")
    with make_state(GRAD_CASES["sc3d_ddi"]) as p:
        io.positions_write(p, f, io.FILEFORMAT_OVF_BIN8)
        pos = np.array(geometry.get_positions(p))  # a copy: the getter's array belongs to the State
    raw = open(f, "rb").read()
    assert b"# valuelabels: position_x position_y position_z" in raw
    p0 = raw.index(b"# Begin: Data Binary 8\n") + len(b"# Begin: Data Binary 8\n")
    data = np.frombuffer(raw[p0 + 8 : p0 + 8 + 24 * len(pos)], dtype="<f8").reshape(-1, 3)
    assert np.array_equal(data, pos)


def test_stream_positions_round_trip_in_description():
    from spirit_gb300 import io

    f = _path("streams")
    with make_state(GRAD_CASES["sq_c1"]) as p:
        io.image_write(p, f, io.FILEFORMAT_OVF_TEXT, "note")
    txt = open(f).read()
    assert "# Desc: note\n" in txt
    assert "# Desc: spirit_gb300 llg_noise_drawn=0 mc_sweeps_drawn=0\n" in txt
