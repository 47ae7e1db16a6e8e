// GNEB (chain of images; VP, VP_OSO or LBFGS_OSO) and the direct-minimisation / batched LLG
// drivers behind the C API.
#pragma once
#include "state.hpp"

#include <vector>

namespace sg
{

void gneb_start( State * st, Chain & chain, int solver, bool singleshot );
void gneb_n_shot( State * st, Chain & chain, int n );
void gneb_update_rx( Chain & chain );
const std::vector<double> & gneb_torques( Chain & chain );

// LLG direct minimisation on one image with VP (Solver_VP.hpp:28-114), VP_OSO or LBFGS_OSO
// (Solver_VP_OSO.hpp, Solver_LBFGS_OSO.hpp) under Method_LLG
void llg_vp_run( State * st, Image & img, int solver, bool singleshot );
void llg_vp_shot( State * st, Image & img, int n );

// batched LLG over the active images of several States (one device batch)
void llg_run_batched( State ** states, int n_states, int solver, int n_iterations, void * info, size_t info_size );
// caller-driven batched run: enqueue n_steps (first call uploads and starts), then finish
void llg_batched_launch( State ** states, int n_states, int solver, int n_steps );
void gradient_batched( State ** states, int n_states, double * gradients, double * energies );
void llg_batched_finish( State ** states, int n_states );

} // namespace sg
