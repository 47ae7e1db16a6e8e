"""Pins the oracle (CPU FP64 restatement) against the reference's own outputs.

The fixtures in tests/golden/ come from the reference (Spirit v2.2.0 CPU/OpenMP FP64, kissFFT)
built from its sources by oracle/ref/Makefile and driven by tests/golden/make_golden.py.
Pair lists and positions must be bit-exact; FP64 gradients/energies agree to rounding; T=0
trajectories follow the same operations in the same order.
"""
import numpy as np
import pytest

from cases import FULL_CASES, GRAD_CASES, HTST_CASES, LLG_CASES, PAIR_GEOMETRIES, SOLVERS
from conftest import golden
from oracle.oracle import OracleSystem, image_types_auto, philox4x32, portable_spins


@pytest.mark.parametrize("name", sorted(PAIR_GEOMETRIES))
def test_pairs_bit_exact(name):
    f = golden("pairs_%s.npz" % name)
    o = OracleSystem(PAIR_GEOMETRIES[name])
    p, m = o.exchange_pairs()
    d, dm, dn = o.dmi_pairs()
    assert np.array_equal(p, f["exchange_pairs"])
    assert np.array_equal(m, f["exchange_magnitudes"])
    assert np.array_equal(d, f["dmi_pairs"])
    assert np.array_equal(dm, f["dmi_magnitudes"])
    assert np.array_equal(dn, f["dmi_normals"])
    assert np.array_equal(o.positions(), f["positions"])


@pytest.mark.parametrize("name", sorted(GRAD_CASES))
def test_gradient_and_energies(name):
    f = golden("grad_%s.npz" % name)
    o = OracleSystem(GRAD_CASES[name])
    s = f["spins"]
    scale = np.abs(f["gradient"]).max()
    np.testing.assert_allclose(o.gradient(s), f["gradient"], rtol=0, atol=1e-13 * scale)
    g, E = o.gradient_and_energy(s)
    np.testing.assert_allclose(g, f["gradient_ge"], rtol=0, atol=1e-13 * scale)
    assert abs(E - f["energy_ge"]) <= 1e-12 * abs(f["energy_ge"])
    assert abs(o.energy(s) - f["energy_total"]) <= 1e-12 * abs(f["energy_total"])
    contrib = o.energy_contributions(s)
    assert list(contrib) == [str(n) for n in f["term_names"]]
    for k in contrib:
        np.testing.assert_allclose(contrib[k], f["energy_" + k], rtol=0, atol=1e-12 * abs(f["energy_total"]))


def _padded_everywhere(spec):
    d = spec["ddi"]
    return all((not b) or d.get("pb_zero_padding", 1) or n == 1 for b, n in zip(spec["bc"], spec["n_cells"]))


@pytest.mark.parametrize("name", [n for n in sorted(GRAD_CASES) if GRAD_CASES[n].get("ddi")])
def test_ddi_direct_sum(name):
    """The O(N^2) direct sum with periodic images (Gradient_DDI_Direct) matches the reference;
    where every periodic direction is zero-padded, the FFT convolution equals it, which is the
    reference's own DDI check (core/test/test_physics.cpp:144-181).  Without padding the
    reference sums the images of a periodic direction asymmetrically, so FFT and direct differ
    there in the reference too."""
    f = golden("grad_%s.npz" % name)
    s = f["spins"]
    spec = dict(GRAD_CASES[name])
    spec["ddi"] = dict(spec["ddi"], method="cutoff", radius=-1.0)
    gd = OracleSystem(spec).gradient(s)
    np.testing.assert_allclose(gd, f["gradient_direct"], rtol=0, atol=1e-12 * np.abs(gd).max())
    if _padded_everywhere(GRAD_CASES[name]):
        g = OracleSystem(GRAD_CASES[name]).gradient(s)
        assert np.abs(g - gd).max() <= 1e-9 * np.abs(gd).max()


def full_case_input(name):
    """Fixture, spec and the regenerated input spins of a full-size case; the input is checked
    against the sums and first spins the fixture stored (the generator is platform-exact)."""
    (spec, sname, sid, n_iter, seed), = [c[1:] for c in FULL_CASES if c[0] == name]
    f = golden("full_%s.npz" % name)
    n = spec["n_cells"]
    s0 = portable_spins(n[0] * n[1] * n[2], seed)
    assert np.array_equal(s0[:64], f["spins_in_head"])
    assert np.array_equal(s0.sum(axis=0), f["spins_in_sum"])
    return f, spec, s0


@pytest.mark.parametrize("name", [c[0] for c in FULL_CASES])
def test_llg_full_size(name):
    """The benchmark configurations at full size against the reference: the plain-LLG
    configuration exactly (64 x 64, Depondt, 1000 steps) and the dipolar system (128 x 128 x 16,
    DDI zero-padded along c, Heun, 100 steps).  The large system's output is stored as FP32 (plus
    every 16th spin in FP64), so the full comparison is at FP32 rounding."""
    f, spec, s0 = full_case_input(name)
    ll = spec["llg"]
    s, r = OracleSystem(spec).llg(s0, int(f["solver"]), int(f["n_iter"]), dt=ll["dt"], damping=ll["damping"],
                                  temperature=0.0)
    assert r["iterations"] == int(f["iterations"])
    assert np.abs(s[::16] - f["spins_out_fp64_every16"]).max() <= 1e-11
    tol = 1e-11 if f["spins_out"].dtype == np.float64 else 1e-7
    assert np.abs(s - f["spins_out"]).max() <= tol
    assert abs(r["energy"] - f["energy"]) <= 1e-11 * abs(f["energy"])
    assert abs(r["max_torque"] - f["max_torque"]) <= 1e-8 * abs(f["max_torque"])


@pytest.mark.parametrize("case,solver,sid,n_iter", LLG_CASES)
def test_llg_trajectory(case, solver, sid, n_iter):
    f = golden("llg_%s_%s.npz" % (case, solver))
    spec = GRAD_CASES[case]
    o = OracleSystem(spec)
    ll = spec["llg"]
    s, r = o.llg(f["spins_in"], sid, n_iter, dt=ll["dt"], damping=ll["damping"], temperature=0.0)
    assert r["iterations"] == int(f["iterations"])
    assert np.abs(s - f["spins_out"]).max() <= 1e-12
    assert abs(r["energy"] - f["energy"]) <= 1e-12 * abs(f["energy"])
    assert abs(r["max_torque"] - f["max_torque"]) <= 1e-10 * abs(f["max_torque"])


@pytest.mark.parametrize("tag", ["gneb_vp", "gneb_vp_ci"])
def test_gneb_vp_short(tag):
    f = golden("%s.npz" % tag)
    o = OracleSystem(SOLVERS)
    c, r = o.gneb(f["chain_in"], int(f["n_iter"]), spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
    if int(f["n_iter_ci"]) > 0:
        t = image_types_auto(r["energies"], np.zeros(9))
        assert np.array_equal(t, f["image_type"])
        c, r = o.gneb(c, int(f["n_iter_ci"]), image_type=t, spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
    assert np.abs(c - f["chain_out"]).max() <= 1e-10
    np.testing.assert_allclose(r["energies"], f["energies"], rtol=1e-13)
    np.testing.assert_allclose(r["Rx"], f["Rx"], rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("tag", ["gneb_vp_oso", "gneb_lbfgs_oso", "gneb_lbfgs_oso_ci"])
def test_gneb_oso_short(tag):
    """GNEB with the exponential-transform solvers (Method_GNEB<VP_OSO>, Method_GNEB<LBFGS_OSO>)
    against the reference's own runs; a second start (climbing image) restarts the L-BFGS memory."""
    f = golden("%s.npz" % tag)
    o = OracleSystem(SOLVERS)
    sid = int(f["solver"])
    c, r = o.gneb(f["chain_in"], int(f["n_iter"]), spring_constant=1.0, force_convergence=1e-6, dt=1e-3, solver=sid)
    if int(f["n_iter_ci"]) > 0:
        t = image_types_auto(r["energies"], np.zeros(9))
        assert np.array_equal(t, f["image_type"])
        c, r = o.gneb(c, int(f["n_iter_ci"]), image_type=t, spring_constant=1.0, force_convergence=1e-6, dt=1e-3,
                      solver=sid)
    assert np.abs(c - f["chain_out"]).max() <= 1e-11
    np.testing.assert_allclose(r["energies"], f["energies"], rtol=1e-13)
    np.testing.assert_allclose(r["Rx"], f["Rx"], rtol=1e-11, atol=1e-12)
    assert abs(r["max_torque"] - float(f["max_torque"])) <= 1e-9 * float(f["max_torque"])


@pytest.mark.slow
def test_gneb_converged_saddle():
    """Converged skyrmion-collapse saddle; the reference test asserts -5811.5244140625 meV
    (core/test/test_solvers.cpp:85) with its own initial skyrmion."""
    f = golden("gneb_converged.npz")
    o = OracleSystem(SOLVERS)
    c, r = o.gneb(f["chain_in"], int(f["n_iter"]), spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
    t = image_types_auto(r["energies"], np.zeros(9))
    c, r = o.gneb(c, int(f["n_iter_ci"]), image_type=t, spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
    assert r["max_torque"] < 1e-6
    assert abs(r["energies"].max() - f["energies"].max()) < 1e-6
    assert np.float32(r["energies"].max()) == np.float32(-5811.5244140625)


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors published with the Random123 library (kat_vectors)."""
    assert list(philox4x32([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(philox4x32([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(philox4x32([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_thermal_noise_statistics():
    o = OracleSystem(GRAD_CASES["sq_c1"])
    xs = np.concatenate([o.thermal_noise(10.0, 0.3, 1e-3, 1234, 0, it) for it in range(200)])
    eps = np.sqrt(2 * 0.3 * 1e-3 * 0.1760859644 / 0.057883817555 * 0.08617330350) / (1 + 0.09)
    sigma = eps * np.sqrt(10.0 / 2.0)
    z = xs / sigma
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02


@pytest.mark.parametrize("name", [c[0] for c in HTST_CASES])
def test_htst_vs_reference(name):
    """HTST_Calculate of the reference (dense and sparse) on converged minimum / saddle pairs:
    prefactor constituents, full spectra, eigenvectors up to sign, perpendicular velocities."""
    f = golden("htst_%s.npz" % name)
    spec = [c[1] for c in HTST_CASES if c[0] == name][0]
    o = OracleSystem(spec)
    keys = [str(k) for k in f["keys"]]
    for sparse, ref in ((False, f["dense"]), (True, f["sparse"])):
        r = o.htst(f["spins_min"], f["spins_sp"], sparse=sparse)
        if not bool(f["completed"]):
            assert r["status"] == 4 and r["prefactor"] == 0  # higher-order saddle point: stops
            continue
        assert r["status"] == 0
        for k, v in zip(keys, ref):
            if sparse or k not in ("det_min", "det_sp"):
                assert abs(r[k] - v) <= 1e-10 * max(abs(v), 1.0), (sparse, k, r[k], v)
        if sparse:
            continue
        np.testing.assert_allclose(r["evalues_min"], f["evalues_min"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(r["evalues_sp"], f["evalues_sp"], rtol=0, atol=1e-12)
        # eigenvectors: reference stores them column-major [2N][2N] -> mode k is row k of the file
        # array read as (2N, 2N); compare up to sign where the eigenvalue is simple
        for which in ("min", "sp"):
            ev, ref_v = r["evectors_" + which], f["evectors_" + which]
            w = f["evalues_" + which]
            for k in range(len(w)):
                gap = min(abs(w[k] - w[j]) for j in range(len(w)) if j != k)
                if gap > 1e-6:
                    assert min(np.abs(ev[k] - ref_v[k]).max(), np.abs(ev[k] + ref_v[k]).max()) < 1e-8
        np.testing.assert_allclose(np.abs(r["velocities"]), np.abs(f["velocities"]), rtol=0, atol=1e-10)
