// Adjoint of the T = 0 RK4 LLG trajectory (see adjoint.cu).
#pragma once
#include "engine.hpp"

namespace sg
{

struct AdjointInput
{
    const double * s0     = nullptr; // AoS [nos][3] initial spins
    const double * target = nullptr; // AoS [nos][3]
    int n_steps           = 0;
    int checkpoint        = 100;     // steps between stored states
    bool gradients        = true;
    // unit couplings for the parameter gradients: the system descriptor with every exchange pair
    // scaled by 1/J0 (DMI off), with every DMI vector scaled by 1/D0 (exchange off), the
    // anisotropy constants / K0 and mu_B n_B of the field
    SysDesc unit_J{};
    SysDesc unit_D{};
    double unit_K[MAX_BASIS] = {};
    double unit_B[3]         = {};
};

struct AdjointOutput
{
    double * grad_s0     = nullptr; // AoS [nos][3] (may be null)
    double grad_params[5] = { 0, 0, 0, 0, 0 }; // J, D, K, B, alpha
    double * final_spins = nullptr; // AoS [nos][3] (may be null)
};

// loss = mean_i |s_i(T) - target_i|^2 of system 0 of E; gradients when in.gradients
double adjoint_run( Engine & E, const AdjointInput & in, AdjointOutput & out, bool fp64 );

} // namespace sg
