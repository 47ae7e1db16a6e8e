"""Host-side logic of the library through its C API, without device compute: configuration
parsing, neighbour shells and DMI set-up, chains and transitions, spin configurations."""
import numpy as np
import pytest

from cases import GRAD_CASES, PAIR_GEOMETRIES, SOLVERS
from conftest import golden
from helpers import make_state, spins_of
from oracle.oracle import OracleSystem, transition_homogeneous


@pytest.mark.parametrize("name", sorted(PAIR_GEOMETRIES))
def test_pairs_and_positions_bit_exact(name):
    from spirit_gb300 import geometry, hamiltonian

    f = golden("pairs_%s.npz" % name)
    with make_state(PAIR_GEOMETRIES[name]) as p:
        idx, tr, J = hamiltonian.get_exchange_pairs(p)
        assert np.array_equal(np.concatenate([idx, tr], axis=1), f["exchange_pairs"])
        assert np.array_equal(J, f["exchange_magnitudes"].astype(np.float32))
        assert hamiltonian.get_dmi_n_pairs(p) == len(f["dmi_pairs"])
        assert np.array_equal(geometry.get_positions(p), f["positions"])


def test_config_parsing():
    from spirit_gb300 import geometry, hamiltonian
    import spirit_gb300.parameters.llg as llg

    spec = GRAD_CASES["sc3d_ddi"]
    with make_state(spec) as p:
        assert geometry.get_n_cells(p) == [8, 8, 4]
        assert hamiltonian.get_boundary_conditions(p) == [True, True, False]
        B, n = hamiltonian.get_field(p)
        assert abs(B - 0.5) < 1e-7 and n == [0, 0, 1]
        K, kn = hamiltonian.get_anisotropy(p)
        assert abs(K - 0.05) < 1e-7
        d = hamiltonian.get_ddi(p)
        assert d["ddi_method"] == 1 and d["n_periodic_images"] == [4, 4, 0] and not d["pb_zero_padding"]
        assert abs(llg.get_timestep(p) - 5e-4) < 1e-9 and abs(llg.get_damping(p) - 0.1) < 1e-7
        assert abs(geometry.get_mu_s(p)[0] - 2.0) < 1e-7


def test_state_setup_random_spins_are_unit_vectors():
    with make_state(GRAD_CASES["sq_c1"]) as p:
        s = spins_of(p)
        assert np.allclose(np.linalg.norm(s, axis=1), 1.0)


def test_transition_homogeneous_matches_oracle():
    from spirit_gb300 import chain, configuration, system, transition

    with make_state(SOLVERS) as p:
        configuration.plus_z(p)
        configuration.skyrmion(p, 5, phase=-90)
        chain.image_to_clipboard(p)
        for _ in range(6):
            chain.insert_image_after(p)
        assert chain.get_noi(p) == 7
        configuration.plus_z(p, idx_image=6)
        transition.homogeneous(p, 0, 6)
        c = np.stack([spins_of(p, i) for i in range(7)])
    ref = transition_homogeneous(c, 0, 6)
    assert np.abs(c - ref).max() < 1e-14


def test_chain_operations():
    from spirit_gb300 import chain

    with make_state(GRAD_CASES["sq_c1"]) as p:
        chain.image_to_clipboard(p)
        chain.insert_image_after(p)
        chain.push_back(p)
        assert chain.get_noi(p) == 3
        assert chain.jump_to_image(p, 2)
        assert chain.delete_image(p, 1)
        assert chain.get_noi(p) == 2
        chain.set_length(p, 5)
        assert chain.get_noi(p) == 5
        assert chain.pop_back(p)
        assert chain.get_noi(p) == 4


def test_domain_and_skyrmion_configurations():
    from spirit_gb300 import configuration, quantities

    with make_state(SOLVERS) as p:
        configuration.domain(p, [1, 1, 0])
        s = spins_of(p)
        assert np.allclose(s, [2 ** -0.5, 2 ** -0.5, 0])
        configuration.plus_z(p)
        configuration.skyrmion(p, 5, phase=-90)
        s = spins_of(p)
        assert np.allclose(np.linalg.norm(s, axis=1), 1.0)
        assert s[:, 2].min() < -0.9  # the core points down (no site sits exactly at the centre)
        m = quantities.get_magnetization(p)
        assert 0 < m[2] < 2


def test_invalid_indices_do_not_crash():
    from spirit_gb300 import simulation, system

    with make_state(GRAD_CASES["sq_c1"]) as p:
        assert system.get_nos(p, 7) == 0            # invalid image: logged, default returned
        simulation.start(p, simulation.METHOD_LLG, 99, 5)  # invalid solver: logged, nothing runs
        assert not simulation.running_on_image(p)
