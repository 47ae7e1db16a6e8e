// Monte Carlo (Metropolis) on the device engine's systems (see mc.cu).
#pragma once
#include "engine.hpp"

#include <vector>

namespace sg
{

// Parameters of one system's Metropolis run (Parameters_Method_MC, core/include/data/
// Parameters_Method_MC.hpp)
struct MCSettings
{
    double temperature        = 0;
    bool cone                 = true;
    double cone_angle_deg     = 30;
    bool adaptive             = true;
    double acceptance_target  = 0.5;
    unsigned long long seed   = 2006;
    unsigned int stream       = 0;
    int n_iterations          = 0;
    unsigned int rng_offset   = 0; // sweeps drawn before this run (the random stream continues)
};

struct MCStatus
{
    int iteration;
    double cone_angle_deg;
    double acceptance;
};

class MCRun
{
public:
    // colours every system of E (greedy colouring of the interaction graph in spin order)
    explicit MCRun( Engine & E );
    ~MCRun();
    MCRun( const MCRun & )             = delete;
    MCRun & operator=( const MCRun & ) = delete;
    void start( const std::vector<MCSettings> & settings );
    // enqueue n sweeps (no synchronisation); sweeps beyond a system's n_iterations do nothing
    void launch( int n_sweeps );
    std::vector<MCStatus> status();
    int n_colors() const
    {
        return n_colors_;
    }

private:
    template<typename R>
    void sweep_t();
    Engine & E_;
    int n_colors_ = 0;
    int * d_perm_ = nullptr;                 // spins ordered by (system, colour), local indices
    std::vector<int4 *> d_tables_;           // per colour: (system, first list index, count, 0)
    std::vector<int> n_blocks_;
    void * d_state_ = nullptr;               // per-system run state
    void * d_const_ = nullptr;               // per-system constants
    cudaGraphExec_t graph_ = nullptr;
    size_t n_sys_ = 0;
};

} // namespace sg
