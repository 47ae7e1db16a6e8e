/*
 * spirit_oracle.h -- CPU FP64 restatement of the reference's spin-dynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Results are compared against this library: the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it.  The product (libspirit_gb300)
 * never links, loads or calls it.
 *
 * Every function restates the algorithm of a reference function (Spirit v2.2.0, file:line
 * in the comments of spirit_oracle.c), in plain C with OpenMP, in FP64:
 *   geometry / neighbour shells / DMI normals  core/src/data/Geometry.cpp, core/src/engine/Neighbours.cpp
 *   Heisenberg gradient + energies              core/src/engine/Hamiltonian_Heisenberg.cpp
 *   dipole-dipole (zero-padded FFT convolution) core/src/engine/Hamiltonian_Heisenberg.cpp:920-1014,1373-1595
 *   LLG force and integrators                   core/src/engine/Method_LLG.cpp, core/include/engine/Solver_*.hpp
 *   GNEB force, tangents, VP solver             core/src/engine/Method_GNEB.cpp, Manifoldmath.cpp, Solver_VP.hpp
 * Thermal noise is NOT the reference's host mt19937 stream (which no GPU can reproduce);
 * it is the counter-based Philox4x32-10 stream defined in og_thermal_noise(), the same one
 * the CUDA kernels draw, so T>0 trajectories can be compared step for step.
 *
 * Parity of this restatement against the reference itself is pinned by the golden fixtures
 * in tests/golden/ (generated by tests/golden/make_golden.py from the reference's own code
 * built by oracle/ref/Makefile) and by the reference tests' own known answers.
 */
#ifndef SPIRIT_ORACLE_H
#define SPIRIT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OG_MAX_BASIS 8
#define OG_MAX_SHELLS 8

typedef struct og_system og_system;

/* Geometry + boundary conditions.  cell_atoms are in units of the Bravais vectors
 * (fractional), bravais is row-major [3][3], mu_s one value per basis atom. */
og_system * og_create(
    const int n_cells[3], int n_cell_atoms, const double bravais[9], const double * cell_atoms,
    double lattice_constant, const double * mu_s_basis, const int boundary_conditions[3] );
void og_free( og_system * s );
int og_nos( const og_system * s );
void og_positions( const og_system * s, double * out /* nos*3 */ );
void og_set_threads( int n );

/* Hamiltonian terms (Hamiltonian_Heisenberg members).  Field magnitude in Tesla. */
void og_set_field( og_system * s, double magnitude, const double normal[3] );
void og_set_anisotropy( og_system * s, int n, const int * indices, const double * magnitudes, const double * normals );
int og_set_exchange_shells( og_system * s, int n_shells, const double * jij );
int og_set_dmi_shells( og_system * s, int n_shells, const double * dij, int chirality );
/* explicit pair lists (heisenberg_pairs); pairs are (i, j, da, db, dc) */
int og_set_exchange_pairs( og_system * s, int n, const int * pairs, const double * jij );
int og_set_dmi_pairs( og_system * s, int n, const int * pairs, const double * dij, const double * normals );
/* method: 0 none, 1 fft, 3 cutoff (radius < 0 means the direct O(N^2) sum) */
void og_set_ddi( og_system * s, int method, const int n_periodic_images[3], double radius, int pb_zero_padding );

int og_n_exchange_pairs( const og_system * s );
int og_n_dmi_pairs( const og_system * s );
void og_get_exchange_pairs( const og_system * s, int * pairs, double * magnitudes );
void og_get_dmi_pairs( const og_system * s, int * pairs, double * magnitudes, double * normals );
int og_idx_from_pair( const og_system * s, int ispin, const int pair[5] );

/* Evaluation (FP64). */
void og_gradient( og_system * s, const double * spins, double * gradient );
double og_gradient_and_energy( og_system * s, const double * spins, double * gradient );
/* per-term, per-spin energies in the reference order (Zeeman, Anisotropy, Exchange, DMI, DDI);
 * returns the number of active terms, writes their names (comma separated) into names */
int og_energy_contributions( og_system * s, const double * spins, double * per_spin, char * names, int names_len );
double og_energy( og_system * s, const double * spins );
/* reference dipole gradient by the direct O(N^2) sum with periodic images (Gradient_DDI_Direct) */
void og_gradient_ddi_direct( og_system * s, const double * spins, double * gradient );

/* Thermal noise: xi[i][d] = epsilon * sqrt(T/mu_s) * N(0,1) with N from Philox4x32-10. */
void og_thermal_noise(
    const og_system * s, double temperature, double damping, double dt, uint64_t seed, uint32_t stream,
    uint32_t iteration, double * xi );
/* One Philox4x32-10 block (exposed for tests). */
void og_philox4x32( const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4] );

/* LLG.  solver ids follow Simulation.h: VP=0, SIB=1, Depondt=2, Heun=3, RK4=4. */
typedef struct og_llg_params
{
    double dt;
    double damping;
    double temperature;
    int direct_minimization;
    double force_convergence;
    uint64_t seed;
    uint32_t stream; /* system id inside a batch: part of the noise counter */
} og_llg_params;

/* Runs up to n_iter iterations (stops earlier on convergence, like Method::Iterate).
 * solver: 0 VP, 1 SIB, 2 Depondt, 3 Heun, 4 RK4, 5 LBFGS_OSO, 7 VP_OSO (Simulation.h ids).
 * spins in/out.  Returns the number of iterations done; energy = energy of the last force
 * evaluation (Spin_System::E after the run), max_torque as Simulation_Get_MaxTorqueNorm. */
int og_llg_run(
    og_system * s, const og_llg_params * p, int solver, int n_iter, double * spins, double * energy,
    double * max_torque );

/* GNEB with the VP solver (Method_GNEB<Solver::VP>).  chain = noi*nos*3 in/out,
 * image_type[noi] in (0 normal, 1 climbing, 2 falling, 3 stationary).
 * energies[noi], Rx[noi] out.  Returns iterations done. */
typedef struct og_gneb_params
{
    double spring_constant;
    double force_convergence;
    double dt; /* llg_parameters->dt of the images */
} og_gneb_params;
int og_gneb_run(
    og_system * s, const og_gneb_params * p, int noi, int n_iter, double * chain, const int * image_type,
    double * energies, double * Rx, double * max_torque );
/* GNEB with solver 0 (VP), 5 (LBFGS_OSO) or 7 (VP_OSO): Method_GNEB<solver> */
int og_gneb_run_solver(
    og_system * s, const og_gneb_params * p, int solver, int noi, int n_iter, double * chain,
    const int * image_type, double * energies, double * Rx, double * max_torque );
/* Parameters_GNEB_Set_Image_Type_Automatically */
void og_gneb_image_types_auto( int noi, const double * energies, int * image_type );
/* Transition_Homogeneous (geodesic interpolation between images idx_1 and idx_2) */
void og_transition_homogeneous( int nos, int noi, double * chain, int idx_1, int idx_2 );

/* HTST prefactor (HTST_Calculate, core/src/engine/HTST.cpp, Sparse_HTST.cpp).  Returns 0 or the
 * check that failed: 1 minimum / 2 saddle point not converged (torque > 1e-8), 3 no negative mode
 * at the saddle point, 4 higher-order saddle point, 5 negative mode at the minimum (dense only).
 * Dense (sparse = 0): evalues_* [2N] ascending, evectors_* [n_keep][2N] (mode-major),
 * velocities [2N]; sparse: those outputs are not written. */
typedef struct og_htst_info
{
    double temperature_exponent, me, Omega_0, s, volume_min, volume_sp, prefactor_dynamical, prefactor;
    double det_min, det_sp;
    int n_eigenmodes_keep, status;
} og_htst_info;
int og_htst(
    og_system * s, const double * spins_min, const double * spins_sp, int sparse, int n_keep, og_htst_info * info,
    double * evalues_min, double * evalues_sp, double * evectors_min, double * evectors_sp, double * velocities );

/* Monte Carlo (Method_MC, core/src/engine/Method_MC.cpp): Metropolis sweeps with cone sampling
 * and the adaptive cone.  A sweep visits the spins colour by colour (greedy colouring of the
 * interaction graph in spin order: spins of one colour never interact), drawing per spin and
 * sweep one Philox4x32-10 block (counter (i, sweep, stream, 0x4D435300), key = seed): u0 for
 * cos(theta), u1 for phi, u2 for the Metropolis test. */
typedef struct og_mc_params
{
    double temperature;
    int cone;
    double cone_angle_deg;
    int adaptive;
    double acceptance_target;
    uint64_t seed;
    uint32_t stream;
} og_mc_params;
/* colour of every spin (colors[nos]); returns the number of colours */
int og_mc_colors( const og_system * s, int * colors );
/* n_sweeps sweeps, spins in/out; cone_angle_deg_out / acceptance_out: state after the run */
int og_mc_run( og_system * s, const og_mc_params * p, int n_sweeps, double * spins, double * cone_angle_deg_out,
               double * acceptance_out );

#ifdef __cplusplus
}
#endif
#endif
