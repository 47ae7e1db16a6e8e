"""Allocation-free gradient entry point Hamiltonian_Get_Gradient_NoAlloc against the engine's
Hamiltonian_Get_Gradient on the same spins (both FP64 on the device).

The caller owns every device buffer (allocated here with torch); the entry point itself uses a
static device scratch array.  Each case calls it twice in a row on the same buffers: nothing may
carry over between calls.  The file name puts it last in collection; it also passes alone.

Tolerance: gradients 1e-12 relative to max |g| (same per-spin arithmetic, only the energy
summation order differs), energies 1e-12 relative.
"""
import numpy as np
import pytest

from cases import FD_PAIRS, HEX2D, SQ_C1
from helpers import make_state, spins_of

pytestmark = pytest.mark.gpu

SC3D_OPEN_C = dict(  # stencil with wraps along a, cuts along b and c, two exchange shells
    bravais="sc", n_cells=[64, 48, 6], lattice_constant=1.0, mu_s=[2.0], bc=[1, 0, 0],
    field=(0.7, (0.3, 0, 1)), anisotropy=(0.2, (0, 0.6, 0.8)), jij=[1.0, 0.25], dij=[0.3], dm_chirality=1,
    llg=dict(dt=1e-3, damping=0.3, temperature=0.0),
)

CASES = {"sq_c1": SQ_C1, "hex2d": HEX2D, "fd_pairs": FD_PAIRS, "sc3d_open_c": SC3D_OPEN_C}


def _nos(spec):
    n = spec["n_cells"]
    return n[0] * n[1] * n[2] * len(spec["mu_s"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_gradient(name):
    torch = pytest.importorskip("torch")
    from oracle.oracle import random_spins
    from spirit_gb300 import hamiltonian

    spec = CASES[name]
    nos = _nos(spec)
    spins = random_spins(nos, 20240 + nos)
    with make_state(spec, spins) as p:
        g_ref, e_ref = hamiltonian.get_gradient(p)
        s = torch.tensor(np.ascontiguousarray(spins_of(p).T), dtype=torch.float64, device="cuda")
        g = torch.full_like(s, float("nan"))
        e = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            rc = hamiltonian.get_gradient_noalloc(p, s[0].data_ptr(), s[1].data_ptr(), s[2].data_ptr(),
                                                  g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                                  e.data_ptr(), stream)
            torch.cuda.synchronize()
            assert rc == 0
            got = g.T.cpu().numpy()
            scale = np.abs(g_ref).max()
            np.testing.assert_allclose(got, g_ref, rtol=0, atol=1e-12 * scale, err_msg="call %d" % call)
            assert abs(float(e.item()) - e_ref) <= 1e-12 * abs(e_ref), (call, float(e.item()), e_ref)


@pytest.mark.parametrize("name", ["sq_c1", "hex2d", "fd_pairs"])
def test_noalloc_matches_reference_fixture(name):
    """Directly against the reference: the gradient and energy the reference's own
    Gradient_and_Energy produced for the same spins (tests/golden/grad_<name>.npz), on two calls in
    a row.  Tolerance: gradients 1e-12 relative to max |g|, energies 1e-10 relative."""
    torch = pytest.importorskip("torch")
    from conftest import golden
    from spirit_gb300 import hamiltonian

    f = golden("grad_%s.npz" % name)
    spins = f["spins"]
    with make_state(CASES[name], spins) as p:
        s = torch.tensor(np.ascontiguousarray(spins.T), dtype=torch.float64, device="cuda")
        g = torch.full_like(s, float("nan"))
        e = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        for call in range(2):
            rc = hamiltonian.get_gradient_noalloc(p, s[0].data_ptr(), s[1].data_ptr(), s[2].data_ptr(),
                                                  g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                                  e.data_ptr(), torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            assert rc == 0
            scale = np.abs(f["gradient_ge"]).max()
            np.testing.assert_allclose(g.T.cpu().numpy(), f["gradient_ge"], rtol=0, atol=1e-12 * scale,
                                       err_msg="call %d" % call)
            assert abs(float(e.item()) - float(f["energy_total"])) <= 1e-10 * abs(float(f["energy_total"]))


@pytest.mark.parametrize("name", ["sq_c1", "sc3d_open_c"])
def test_noalloc_side_stream(name):
    """On a non-default stream the call is ordered on that stream alone: the result equals
    Hamiltonian_Get_Gradient's after the side stream is synchronised."""
    torch = pytest.importorskip("torch")
    from oracle.oracle import random_spins
    from spirit_gb300 import hamiltonian

    spec = CASES[name]
    nos = _nos(spec)
    spins = random_spins(nos, 31337 + nos)
    with make_state(spec, spins) as p:
        g_ref, e_ref = hamiltonian.get_gradient(p)
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            s = torch.tensor(np.ascontiguousarray(spins_of(p).T), dtype=torch.float64, device="cuda")
            g = torch.full_like(s, float("nan"))
            e = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        for call in range(2):
            rc = hamiltonian.get_gradient_noalloc(p, s[0].data_ptr(), s[1].data_ptr(), s[2].data_ptr(),
                                                  g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                                  e.data_ptr(), side.cuda_stream)
            assert rc == 0
            side.synchronize()
            got = g.T.cpu().numpy()
            np.testing.assert_allclose(got, g_ref, rtol=0, atol=1e-12 * np.abs(g_ref).max(), err_msg="call %d" % call)
            assert abs(float(e.item()) - e_ref) <= 1e-12 * abs(e_ref), (call, float(e.item()), e_ref)


def test_noalloc_rejects_null_buffer():
    """A null buffer is rejected (code 1) before anything is launched."""
    torch = pytest.importorskip("torch")
    from spirit_gb300 import hamiltonian

    nos = _nos(SQ_C1)
    with make_state(SQ_C1) as p:
        b = torch.zeros((7, nos), dtype=torch.float64, device="cuda")
        ptrs = [b[k].data_ptr() for k in range(7)]
        for k in range(7):
            args = list(ptrs)
            args[k] = 0
            assert hamiltonian.get_gradient_noalloc(p, *args) == 1, k


def test_noalloc_rejects_too_large():
    """More spins than the static scratch covers (4,194,304) are rejected (code 2) before any
    launch: the buffers given here are far too small for the system and are never touched."""
    torch = pytest.importorskip("torch")
    from spirit_gb300 import hamiltonian

    spec = dict(bravais="sc", n_cells=[2049, 2048, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                field=(0.5, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[1.0], dij=[0.0], dm_chirality=2)
    with make_state(spec) as p:
        b = torch.zeros((7, 4), dtype=torch.float64, device="cuda")
        rc = hamiltonian.get_gradient_noalloc(p, *[b[k].data_ptr() for k in range(7)])
        torch.cuda.synchronize()
    assert rc == 2


def test_noalloc_rejects_dipolar():
    torch = pytest.importorskip("torch")
    from cases import SC3D_DDI
    from spirit_gb300 import hamiltonian

    nos = _nos(SC3D_DDI)
    with make_state(SC3D_DDI) as p:
        b = torch.zeros((7, nos), dtype=torch.float64, device="cuda")
        rc = hamiltonian.get_gradient_noalloc(p, *[b[k].data_ptr() for k in range(7)])
        torch.cuda.synchronize()
    assert rc == 3
