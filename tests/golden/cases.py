"""Golden cases: small systems whose reference outputs are committed as fixtures.

Each case is a spec dictionary (spirit_gb300.configs) plus the operations run on it.  The
fixtures were produced by make_golden.py from the reference's own code (Spirit v2.2.0 CPU
build, FP64, OpenMP, kissFFT) and are read by the parity tests.  The cases cover the
lattices and terms of the benchmark configurations at sizes that finish in seconds.
"""

SQ_C1 = dict(  # 64x64 plain-LLG configuration, shrunk: SC 2D, periodic, Neel DMI
    bravais="sc", n_cells=[8, 8, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
    field=(1.0, (0, 0, 1)), anisotropy=(0.1, (0, 0, 1)), jij=[1.0], dij=[0.3], dm_chirality=2,
    llg=dict(dt=1e-3, damping=0.3, temperature=0.0),
)

SC3D_DDI = dict(  # 128x128x16 dipolar configuration, shrunk: bulk DMI, open z, DDI FFT z-padded
    bravais="sc", n_cells=[8, 8, 4], lattice_constant=4.0, mu_s=[2.0], bc=[1, 1, 0],
    field=(0.5, (0, 0, 1)), anisotropy=(0.05, (0, 0, 1)), jij=[1.0], dij=[0.2], dm_chirality=1,
    ddi=dict(method="fft", n_periodic_images=[4, 4, 0], radius=0.0, pb_zero_padding=0),
    llg=dict(dt=5e-4, damping=0.1, temperature=0.0),
)

HEX2D = dict(  # triangular GNEB configuration, shrunk
    bravais="hex2d60", n_cells=[12, 12, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
    field=(1.5, (0, 0, 1)), anisotropy=(0.08, (0, 0, 1)), jij=[1.0], dij=[0.35], dm_chirality=2,
    llg=dict(dt=1e-3, damping=0.3, temperature=0.0),
)

OPEN2D_DDI = dict(  # adjoint configuration, shrunk: open square lattice, padded 2D DDI
    bravais="sc", n_cells=[8, 8, 1], lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0],
    field=(0.8, (0, 0, 1)), anisotropy=(0.1, (0, 0, 1)), jij=[1.0], dij=[0.3], dm_chirality=2,
    ddi=dict(method="fft", n_periodic_images=[4, 4, 4], radius=0.0, pb_zero_padding=1),
    llg=dict(dt=1e-3, damping=0.3, temperature=0.0),
)

# reference test input core/test/input/physics_ddi.cfg: irregular 2-atom basis, DDI only
DDI_IRREGULAR = dict(
    bravais_vectors=[[3, 0, -1], [0, 1, 0], [0.3, -2, 1]], n_cells=[5, 5, 5],
    basis=[[0, 0, 0], [0.5, 0.2, 0.7]], lattice_constant=2.77, mu_s=[2.17, 2.17], bc=[1, 0, 0],
    field=(0.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), pairs=[],
    ddi=dict(method="fft", n_periodic_images=[4, 4, 4], radius=10.0, pb_zero_padding=1),
)

# periodic DDI with explicit zero padding on all periodic axes and several images
PERIODIC_DDI = dict(
    bravais="sc", n_cells=[6, 5, 3], lattice_constant=2.5, mu_s=[1.5], bc=[1, 1, 1],
    field=(0.3, (0, 1, 1)), anisotropy=(0.2, (1, 0, 1)), jij=[1.0, -0.2], dij=[0.3, 0.1], dm_chirality=-1,
    ddi=dict(method="fft", n_periodic_images=[2, 1, 3], radius=0.0, pb_zero_padding=0),
)

# reference test input core/test/input/fd_pairs.cfg: explicit pairs, open 2x2x1
FD_PAIRS = dict(
    bravais="sc", n_cells=[2, 2, 1], lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0],
    field=(25.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)),
    pairs=[(0, 0, 1, 0, 0, 10.0, 6.0, 0.0, 0.0), (0, 0, 0, 1, 0, 10.0, 0.0, 6.0, 0.0),
           (0, 0, 0, 0, 1, 10.0, 0.0, 0.0, 6.0)],
)

# reference test input core/test/input/solvers.cfg (16x16 SC, J=10, Bloch D=6, B=25 T)
SOLVERS = dict(
    bravais="sc", n_cells=[16, 16, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
    field=(25.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[10.0], dij=[6.0], dm_chirality=1,
    llg=dict(dt=1e-3, damping=0.3, temperature=0.0, force_convergence=1e-8),
    gneb=dict(spring_constant=1.0, force_convergence=1e-6),
)

# neighbour-shell geometries (pair lists must be bit-exact)
PAIR_GEOMETRIES = {
    "sc3d_3shells": dict(bravais="sc", n_cells=[5, 5, 5], bc=[1, 1, 1], jij=[1.0, 0.5, 0.25], dij=[0.1, 0.2, 0.3],
                         dm_chirality=1),
    "sc2d_open": dict(bravais="sc", n_cells=[4, 3, 1], bc=[0, 0, 0], jij=[1.0, 0.5], dij=[0.3], dm_chirality=2),
    "hex2d60_3shells": dict(bravais="hex2d60", n_cells=[6, 6, 1], bc=[1, 1, 0], jij=[1.0, 0.2, 0.1],
                            dij=[0.35, 0.1], dm_chirality=2),
    "hex2d120": dict(bravais="hex2d120", n_cells=[6, 6, 1], bc=[1, 1, 0], jij=[1.0], dij=[0.35],
                     dm_chirality=-2),
    "bcc_2shells": dict(bravais="bcc", n_cells=[4, 4, 4], bc=[1, 1, 1], jij=[1.0, 0.5], dij=[0.2],
                        dm_chirality=1),
    "fcc_2shells": dict(bravais="fcc", n_cells=[4, 4, 4], bc=[1, 1, 1], jij=[1.0, 0.5], dij=[0.2],
                        dm_chirality=-1),
    "irregular_2basis": dict(bravais_vectors=[[3, 0, -1], [0, 1, 0], [0.3, -2, 1]], n_cells=[5, 5, 5],
                             basis=[[0, 0, 0], [0.5, 0.2, 0.7]], lattice_constant=2.77, mu_s=[2.17, 2.17],
                             bc=[1, 0, 0], jij=[1.0, 0.5], dij=[0.3], dm_chirality=1),
    "chain1d": dict(bravais="sc", n_cells=[7, 1, 1], bc=[1, 0, 0], jij=[1.0, 0.3], dij=[0.2], dm_chirality=1),
    "lattice_const_hex": dict(bravais="hex2d", n_cells=[5, 4, 2], lattice_constant=2.5, bc=[1, 1, 0],
                              jij=[1.0, 0.5], dij=[0.2], dm_chirality=2),
}

GRAD_CASES = {
    "sq_c1": SQ_C1,
    "sc3d_ddi": SC3D_DDI,
    "hex2d": HEX2D,
    "open2d_ddi": OPEN2D_DDI,
    "ddi_irregular": DDI_IRREGULAR,
    "periodic_ddi": PERIODIC_DDI,
    "fd_pairs": FD_PAIRS,
}

# The benchmark configurations at their full sizes (T = 0): the plain-LLG configuration exactly
# (SC 64 x 64 periodic, Neel DMI, Depondt, 1000 steps) and the dipolar configuration's system
# (SC 128 x 128 x 16, bulk DMI, DDI FFT zero-padded along c, Heun) over 100 steps.  Input spins
# come from oracle.portable_spins(nos, seed), bit-identical on every platform.
C1_FULL = dict(SQ_C1, n_cells=[64, 64, 1])
C2_T0 = dict(SC3D_DDI, n_cells=[128, 128, 16])
# (name, spec, solver name, solver id, iterations, spin seed)
FULL_CASES = [
    ("c1_full", C1_FULL, "Depondt", 2, 1000, 101),
    ("c2_t0", C2_T0, "Heun", 3, 100, 102),
    # the plain-LLG configuration with the other integrators
    ("c1_full_sib", C1_FULL, "SIB", 1, 1000, 103),
    ("c1_full_heun", C1_FULL, "Heun", 3, 1000, 104),
    ("c1_full_rk4", C1_FULL, "RK4", 4, 1000, 105),
]

# (case, solver name, solver id, iterations)
LLG_CASES = [
    ("sq_c1", "Depondt", 2, 200),
    ("sq_c1", "Heun", 3, 200),
    ("sq_c1", "SIB", 1, 200),
    ("sq_c1", "RK4", 4, 200),
    ("sc3d_ddi", "Heun", 3, 50),
    ("open2d_ddi", "RK4", 4, 50),
    ("hex2d", "SIB", 1, 100),
    # direct minimisers with exponential transforms (Solver_VP_OSO.hpp, Solver_LBFGS_OSO.hpp)
    ("sq_c1", "VP_OSO", 7, 50),  # VP projections switch branch on rounding after ~100
    ("sq_c1", "LBFGS_OSO", 5, 200),
    ("sc3d_ddi", "LBFGS_OSO", 5, 60),
    ("open2d_ddi", "VP_OSO", 7, 60),
]

SPIN_SEED = {"sq_c1": 11, "sc3d_ddi": 12, "hex2d": 13, "open2d_ddi": 14, "ddi_irregular": 15,
             "periodic_ddi": 16, "fd_pairs": 17}

# HTST (HTST_Calculate) on converged minimum / first-order saddle pairs: an open chain (coherent
# reversal), an open 2D patch with DMI, and an open 2D patch with a tilted anisotropy axis and the
# dipolar interaction.  The field is tilted off the anisotropy axis so no continuous symmetry gives
# zero modes.  (name, spec, rng seed)
_HTST_BASE = dict(bravais="sc", lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0], jij=[1.0], dm_chirality=2,
                  llg=dict(dt=1e-3, damping=0.3, temperature=0.0, force_convergence=1e-12),
                  gneb=dict(spring_constant=1.0, force_convergence=1e-11))
HTST_CASES = [
    ("chain8", dict(_HTST_BASE, n_cells=[8, 1, 1], field=(4.0, (0.2, 0.0, -1.0)), anisotropy=(0.5, (0, 0, 1)),
                    dij=[0.0]), 3),
    ("dmi5x4", dict(_HTST_BASE, n_cells=[5, 4, 1], field=(3.0, (0.2, 0.0, -1.0)), anisotropy=(0.5, (0, 0, 1)),
                    dij=[0.3]), 3),
    ("ddi4x3", dict(_HTST_BASE, n_cells=[4, 3, 1], lattice_constant=3.0, field=(3.0, (0.2, 0.1, -1.0)),
                    anisotropy=(0.5, (0, 0, 1.0)), dij=[0.2],
                    ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1)), 5),
    # tilted anisotropy axis: the reference's Hessian puts the anisotropy's beta sum on the diagonal
    # (Hamiltonian_Heisenberg.cpp:1136-1146), which no longer matches the gradient for a tilted
    # axis; its HTST then sees a higher-order saddle and stops.  Pins that the same Hessian is used.
    ("tilted8", dict(_HTST_BASE, n_cells=[8, 1, 1], lattice_constant=3.0, field=(4.0, (0.2, 0.1, -1.0)),
                     anisotropy=(0.5, (0.1, 0.2, 1.0)), dij=[0.0]), 5),
]

# OVF interchange with the reference: files written by the reference's IO_Image_Write in each data
# format (reference format ids: binary 4 = 1, binary 8 = 2, text = 3, csv = 4) are committed under
# tests/golden/ovf/, and files written by this library are read back by the reference
OVF_SPEC = dict(bravais="sc", n_cells=[5, 4, 3], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                field=(0.5, (0, 0, 1)), anisotropy=(0.1, (0, 0, 1)), jij=[1.0], dij=[0.2], dm_chirality=2)
OVF_FORMATS = {"bin4": 1, "bin8": 2, "text": 3, "csv": 4}

# Thermal statistics against reference runs at T > 0 (the noise streams differ -- the reference
# draws from a host mt19937 -- so the comparison is of equilibrium averages within their
# statistical errors).  (name, spec, method, solver id, T [K], equilibration iterations, samples,
# iterations between samples, start: "random" (seeded) or "+z")
_FREE = dict(bravais="sc", n_cells=[32, 32, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
             field=(10.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[0.0], dij=[0.0], dm_chirality=2,
             llg=dict(dt=2e-3, damping=0.5, temperature=10.0, seed=5))
_FM = dict(bravais="sc", n_cells=[32, 32, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
           field=(2.0, (0, 0, 1)), anisotropy=(0.2, (0, 0, 1)), jij=[1.0], dij=[0.1], dm_chirality=2,
           llg=dict(dt=1e-3, damping=0.3, temperature=8.0, seed=6))
THERMAL_CASES = [
    # free spins in a field: <cos theta> = L(mu_s mu_B B / k_B T), the single-spin Langevin test
    ("free_spins_llg", _FREE, "llg", 1, 10.0, 3000, 4000, 10, "random"),
    # ordered 2D ferromagnet with anisotropy, field and weak DMI: <m_z>, <E>, var(E)
    ("fm_lattice_llg", _FM, "llg", 1, 8.0, 5000, 6000, 10, "+z"),
    ("fm_lattice_mc", _FM, "mc", 0, 8.0, 3000, 2000, 5, "+z"),
]
# The reference's Metropolis step (Method_MC.cpp:155-157) takes the old single-spin energy from the
# configuration at the start of the sweep and the new one from the configuration updated so far,
# so its chain does not sample the Boltzmann distribution exactly; this library's Monte Carlo is
# therefore held to the reference's equilibrium averages from LLG at the same temperature.
THERMAL_COMPARE = {"free_spins_llg": "free_spins_llg", "fm_lattice_llg": "fm_lattice_llg",
                   "fm_lattice_mc": "fm_lattice_llg"}
