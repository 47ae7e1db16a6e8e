"""HTST prefactors on the GPU (HTST_Calculate) against the reference's own runs.

The fixtures hold converged minimum / first-order saddle-point pairs and the reference's
HTST_Calculate results, dense and sparse (tests/golden/make_golden.py).  The device computes the
geodesic Hessians and all their eigenpairs in FP64 (parallel Jacobi), so the prefactor
constituents agree to 1e-9 relative, spectra to 1e-10, eigenvectors up to sign, velocities up to
sign.  A tilted anisotropy axis makes the reference's Hessian see a higher-order saddle point; the
device stops the same way.
"""
import numpy as np
import pytest

from cases import HTST_CASES
from conftest import golden
from helpers import make_state

pytestmark = pytest.mark.gpu


def _load_pair(p, smin, ssp):
    from spirit_gb300 import chain, system

    chain.image_to_clipboard(p)
    chain.insert_image_after(p)
    system.get_spin_directions(p, 0)[:] = smin
    system.get_spin_directions(p, 1)[:] = ssp


@pytest.mark.parametrize("name", [c[0] for c in HTST_CASES])
@pytest.mark.parametrize("sparse", [False, True])
def test_htst_vs_reference(name, sparse):
    from spirit_gb300 import htst

    f = golden("htst_%s.npz" % name)
    spec = [c[1] for c in HTST_CASES if c[0] == name][0]
    keys = [str(k) for k in f["keys"]]
    ref = dict(zip(keys, (f["sparse"] if sparse else f["dense"]).tolist()))
    with make_state(spec, name="htst_" + name) as p:
        _load_pair(p, f["spins_min"], f["spins_sp"])
        pf = htst.calculate(p, 0, 1, -1, sparse)
        r = htst.get_result_fp64(p)
        info = htst.get_info_dict(p)
        if not sparse and bool(f["completed"]):
            ev32 = htst.get_eigenvalues_sp(p)
            assert np.abs(ev32 - f["evalues_sp"]).max() <= 1e-6 * np.abs(f["evalues_sp"]).max()
    if not bool(f["completed"]):
        assert r["status"] == 4 and pf == 0.0
        return
    assert r["status"] == 0
    assert abs(pf - ref["prefactor"]) <= 1e-6 * ref["prefactor"]  # float return value
    assert abs(info["prefactor"] - ref["prefactor"]) <= 1e-6 * ref["prefactor"]
    for k in keys:
        if sparse or k not in ("det_min", "det_sp"):
            assert abs(r[k] - ref[k]) <= 1e-9 * max(abs(ref[k]), 1.0), (k, r[k], ref[k])
    if sparse:
        return
    n2 = len(f["evalues_sp"])
    assert r["n_eigenmodes_keep"] == n2
    np.testing.assert_allclose(r["evalues_min"], f["evalues_min"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(r["evalues_sp"], f["evalues_sp"], rtol=0, atol=1e-10)
    for which in ("min", "sp"):
        w = f["evalues_" + which]
        for k in range(n2):
            gap = min(abs(w[k] - w[j]) for j in range(n2) if j != k)
            if gap > 1e-6:
                a, b = r["evectors_" + which][k], f["evectors_" + which][k]
                assert min(np.abs(a - b).max(), np.abs(a + b).max()) < 1e-8, (which, k)
    np.testing.assert_allclose(np.abs(r["velocities"]), np.abs(f["velocities"]), rtol=0, atol=1e-9)


def test_htst_rejects_unconverged_minimum():
    from oracle.oracle import random_spins
    from spirit_gb300 import htst

    name, spec, _ = HTST_CASES[1]
    f = golden("htst_%s.npz" % name)
    with make_state(spec, name="htst_bad") as p:
        _load_pair(p, random_spins(len(f["spins_min"]), 3), f["spins_sp"])
        assert htst.calculate(p, 0, 1) == 0.0
        assert htst.get_result_fp64(p)["status"] == 1


def test_htst_keep_fewer_modes():
    from spirit_gb300 import htst

    name, spec, _ = HTST_CASES[1]
    f = golden("htst_%s.npz" % name)
    with make_state(spec, name="htst_keep") as p:
        _load_pair(p, f["spins_min"], f["spins_sp"])
        htst.calculate(p, 0, 1, 3, False)
        v = htst.get_eigenvectors_min(p)
    assert v.shape == (3, len(f["evalues_min"]))
    for k in range(3):
        b = f["evectors_min"][k]
        assert min(np.abs(v[k] - b).max(), np.abs(v[k] + b).max()) < 1e-6
