"""The GNEB benchmark chain against the reference: 32 images of the periodic 96x96 triangular
lattice (J = 1, Neel D = 0.35, K = 0.08 meV, B = 1.5 T) between the relaxed Neel skyrmion and the
ferromagnet, VP with climbing image, converged to a max torque below 1e-6 meV (FP32 forces to
1e-5 meV, then FP64; `bench.run_gneb`).

Fixture (tests/golden/gneb_c3_barrier.npz, make_golden.py): the oracle relaxed and converged the
same chain in FP64; the reference itself then continued from it for 50 iterations with its own
climbing-image types, and its barrier is stored.  Tolerance: the device barrier within 1e-6 meV of
the reference's and of the oracle's (the barrier is ~1.5 meV).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_c3_chain_converges_to_the_reference_barrier():
    import bench

    f = golden("gneb_c3_barrier.npz")
    r = bench.run_gneb()
    print("C3: %d iterations (FP32 %d, FP64 %d), max torque %.3e, barrier %.10f meV; reference %.10f, oracle %.10f"
          % (r["iterations"], r["iterations_fp32"], r["iterations_fp64"], r["max_torque"], r["barrier_meV"],
             float(f["reference_barrier"]), float(f["oracle_barrier"])))
    assert r["converged"] and r["max_torque"] < 1e-6
    assert abs(r["barrier_meV"] - float(f["reference_barrier"])) <= 1e-6
    assert abs(r["barrier_meV"] - float(f["oracle_barrier"])) <= 1e-6
    assert r["saddle_image"] == int(np.argmax(f["reference_energies"]))
