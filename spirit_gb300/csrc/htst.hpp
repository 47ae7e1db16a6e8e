// Harmonic transition-state theory prefactor on the device (HTST_Calculate,
// core/src/engine/HTST.cpp and Sparse_HTST.cpp).
#pragma once
#include "geometry.hpp"

#include <cuda_runtime.h>

#include <vector>

namespace sg
{

struct HtstResult
{
    // 0 done; the reference's checks: 1 minimum / 2 saddle point not converged (torque > 1e-8),
    // 3 no negative mode at the saddle point, 4 higher-order saddle point, 5 negative mode at the
    // minimum (dense only)
    int status   = -1;
    bool sparse  = false;
    int n_keep   = 0;
    int sweeps   = 0; // Jacobi sweeps of the two eigen-decompositions
    double temperature_exponent = 0, me = 0, Omega_0 = 0, s = 0, volume_min = 0, volume_sp = 0;
    double prefactor_dynamical = 0, prefactor = 0, det_min = 0, det_sp = 0;
    std::vector<double> evalues_min, evalues_sp; // 2N, ascending (dense)
    std::vector<double> evectors_min, evectors_sp; // [n_keep][2N] (dense)
    std::vector<double> velocities;               // 2N (dense)
};

// spins / gradients: AoS [nos][3] FP64 of the minimum and the saddle point (gradients with every
// term, as Hamiltonian::Gradient); each image with its own Hamiltonian, one geometry
HtstResult htst_calculate( const Geometry & g, const HamiltonianParams & h_min, const std::vector<double> & spins_min,
                           const std::vector<double> & grad_min, const HamiltonianParams & h_sp,
                           const std::vector<double> & spins_sp, const std::vector<double> & grad_sp, bool sparse,
                           int n_keep, cudaStream_t stream );

// Symmetric eigen-decomposition of the n x n row-major FP64 matrix d_A (n even; destroyed: its
// diagonal holds the unsorted eigenvalues on return), eigenvectors as the columns of d_V.
// Parallel cyclic Jacobi; returns the number of sweeps.
int jacobi_eigh( double * d_A, double * d_V, int n, cudaStream_t stream );

} // namespace sg
