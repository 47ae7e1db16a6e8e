"""The oracle's FFT dipolar field on the open (zero-padded) mixed-radix extents of
tests/test_gpu_ddi_radix.py against its direct O(N^2) sum (Gradient_DDI_Direct,
core/src/engine/Hamiltonian_Heisenberg.cpp:1016-1071): pins the oracle at the sizes where the
device is compared with it.  DDI-only systems (no pairs, field or anisotropy), FP64, CPU.

Tolerance: 1e-10 relative to max |g| (the FFT and the direct sum differ by rounding only).
"""
import numpy as np
import pytest

_BASE = dict(bravais="sc", lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0], field=(0.0, (0, 0, 1)),
             anisotropy=(0.0, (0, 0, 1)), pairs=[],
             ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1))

CASES = {
    "open2d_7x21": dict(_BASE, n_cells=[7, 21, 1]),
    "open2d_15x10": dict(_BASE, n_cells=[15, 10, 1]),
    "open3d_5x7x9": dict(_BASE, n_cells=[5, 7, 9], lattice_constant=3.0),
}
# Not here: periodic axes without padding.  There the reference's FFT field is the cyclic
# convolution over cell offsets 0..N-1 with the tensor summed over the periodic images
# (Hamiltonian_Heisenberg.cpp:1406-1499), which is not the direct sum over minimal images; the
# golden fixture grad_periodic_ddi pins that path to the reference's own output.


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_fft_ddi_equals_direct_sum(name):
    from oracle.oracle import OracleSystem, random_spins

    spec = CASES[name]
    n = spec["n_cells"][0] * spec["n_cells"][1] * spec["n_cells"][2]
    s = random_spins(n, 51)
    o = OracleSystem(spec)
    g_fft = o.gradient(s)
    g_dir = o.gradient_ddi_direct(s)
    scale = np.abs(g_dir).max()
    assert scale > 0
    np.testing.assert_allclose(g_fft, g_dir, rtol=0, atol=1e-10 * scale)
