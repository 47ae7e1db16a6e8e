"""Monte Carlo on the CPU side: the oracle's colouring and its Metropolis statistics.

The reference samples with a std::mt19937 in a sequential sweep (Method_MC.cpp), so there is no
reference trajectory to compare with; the oracle's Metropolis sweep is checked against exact
statistics instead: for non-interacting spins in a field B the mean z component is the Langevin
function L(x) = coth(x) - 1/x with x = mu_s mu_B B / (k_B T).
"""
import numpy as np

from cases import HEX2D, SQ_C1

MU_B = 0.057883817555
K_B = 0.08617330350


def test_colouring_is_proper_and_small():
    import ctypes

    from oracle.oracle import OracleSystem, lib

    # greedy in spin order: the checkerboard for the square lattice, at most 4 for the triangular
    for spec, expect in ((SQ_C1, 2), (HEX2D, 4)):
        o = OracleSystem(spec)
        c, n = o.mc_colors()
        assert n <= expect
        pairs, _ = o.exchange_pairs()
        nb = len(spec["mu_s"])
        for i in range(o.nos):
            for p in pairs:
                if p[0] != i % nb:
                    continue
                arr = (ctypes.c_int * 5)(*[int(x) for x in p])
                j = lib().og_idx_from_pair(o.h, i, arr)
                if j >= 0 and j != i:
                    assert c[i] != c[j], (i, j)


def test_langevin_statistics_of_free_spins():
    """T = 20 K, B = 2 T, mu_s = 2: x = 2*0.0579*2/(0.0862*20) = 0.1343..."""
    from oracle.oracle import OracleSystem, random_spins

    spec = dict(bravais="sc", n_cells=[32, 32, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                field=(2.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[], dij=[], dm_chirality=1,
                llg=dict(dt=1e-3, damping=0.3, temperature=0.0))
    T = 20.0
    o = OracleSystem(spec)
    s = random_spins(o.nos, 1)
    s, _ = o.mc(s, 200, temperature=T, seed=3)
    mz = []
    for k in range(60):
        s, _ = o.mc(s, 5, temperature=T, seed=100 + k)
        mz.append(s[:, 2].mean())
    x = 2.0 * MU_B * 2.0 / (K_B * T)
    L = 1.0 / np.tanh(x) - 1.0 / x
    err = np.std(mz) / np.sqrt(len(mz))
    assert abs(np.mean(mz) - L) < 5 * max(err, 1e-3), (np.mean(mz), L, err)
