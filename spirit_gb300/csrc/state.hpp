// Host data model behind the C API: a State holds one chain of images (spin systems); each
// image owns its geometry, Heisenberg parameters, LLG parameters and the host mirror of its
// spins in the API scalar type (double, AoS [nos][3], the buffer System_Get_Spin_Directions
// hands out).  Mirrors core/include/data/State.hpp, Spin_System.hpp, Spin_System_Chain.hpp.
#pragma once
#include "engine.hpp"
#include "geometry.hpp"
#include "util.hpp"

#include <atomic>
#include <chrono>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <vector>

namespace sg
{

struct LLGParams
{
    double dt                 = 1e-3;
    double damping            = 0.3;
    double beta               = 0;
    double temperature        = 0;
    double force_convergence  = 1e-10;
    bool direct_minimization  = false;
    long n_iterations         = 1000000;
    long n_iterations_log     = 1000;
    long max_walltime_sec     = 0;
    int rng_seed              = 2006;
    std::string output_folder = "output";
    std::string output_tag    = "<time>";
};

// Parameters_Method_MC (core/include/data/Parameters_Method_MC.hpp) and the generic method part
struct MCParams
{
    double temperature            = 0;
    int rng_seed                  = 2006;
    bool random_sample            = true;
    bool step_cone                = true;
    bool cone_adaptive            = true;
    double cone_angle             = 30; // degrees
    double acceptance_target      = 0.5;
    long n_iterations             = 1000000;
    long n_iterations_log         = 1000;
    long max_walltime_sec         = 0;
    std::string output_folder     = "output";
    std::string output_tag        = "<time>";
    bool output_any = false, output_initial = false, output_final = false;
    bool output_energy_step = false, output_energy_archive = false, output_energy_spin_resolved = false;
    bool output_energy_divide_by_nspins = true, output_energy_add_readability_lines = false;
    bool output_configuration_step = false, output_configuration_archive = false;
    int output_configuration_filetype = 3;
};

struct GNEBParams
{
    double spring_constant          = 1;
    double spring_force_ratio       = 0;
    double path_shortening_constant = 0;
    double force_convergence        = 1e-10;
    int n_E_interpolations          = 10;
    long n_iterations               = 1000000;
    long n_iterations_log           = 1000;
    long max_walltime_sec           = 0;
    bool moving_endpoints           = false;
    bool translating_endpoints      = false;
    double eq_delta_Rx_left = 1, eq_delta_Rx_right = 1;
    std::string output_folder = "output";
    std::string output_tag    = "<time>";
};

// per-run bookkeeping of a method (Method.hpp members the API reports)
struct MethodInfo
{
    std::string method = "None", solver = "None";
    int solver_id       = -1;
    int iteration       = 0;
    double time_ps      = 0;
    float max_torque    = 0;
    double ips          = 0;
    long long wall_ms   = 0;
    int n_iterations    = 0;
    std::chrono::steady_clock::time_point t_start;
};

struct Image
{
    std::shared_ptr<Geometry> geom;
    HamiltonianParams ham;
    LLGParams llg;
    MCParams mc;
    std::vector<double> spins;     // API mirror, AoS
    std::vector<double> eff_field; // AoS
    std::vector<double> positions; // AoS
    double E = 0;
    int gneb_type = 0; // GNEB_IMAGE_NORMAL
    std::atomic<bool> iteration_allowed{ false };
    bool singleshot_allowed = false;
    MethodInfo info;
    std::mt19937 prng{ 2006 };
    std::recursive_mutex mtx;
    // device engines (cached; rebuilt when `version` changes)
    long version = 0;
    std::unique_ptr<Engine> eval64;
    long eval64_version = -1;
    std::unique_ptr<Engine> run;
    long run_version  = -1;
    bool run_fp64     = false;
    std::shared_ptr<void> vp_run; // single-shot LLG run with the VP solver
    std::shared_ptr<void> mc_run; // Monte Carlo run (engine + colouring) of this image
    unsigned int mc_sweeps_drawn = 0; // Monte Carlo sweeps done so far (position in the random stream)
    unsigned int llg_noise_drawn = 0; // LLG iterations whose thermal noise was drawn (noise stream position)
    // page-locked registration of `spins` for single-shot transfers (declared after it: released first)
    HostPin spin_pin;

    int nos() const
    {
        return geom->nos();
    }
    void touch()
    {
        ++version;
    }
};

struct Chain
{
    std::vector<std::shared_ptr<Image>> images;
    GNEBParams gneb;
    std::vector<double> Rx, Rx_interpolated, E_interpolated;
    std::atomic<bool> iteration_allowed{ false };
    bool singleshot_allowed = false;
    MethodInfo info;
    std::recursive_mutex mtx;
    std::shared_ptr<void> gneb_run; // GNEB engine of a running/singleshot chain method
    std::vector<double> torques;    // per-image max torque of the last GNEB iteration
    std::shared_ptr<void> htst;     // result of the last HTST_Calculate (HtstResult)
};

struct State
{
    std::shared_ptr<Chain> chain;
    int idx_active_image = 0;
    std::shared_ptr<Image> clipboard;
    std::string config_file;
    bool quiet = false;
    int precision = 32; // device arithmetic of the LLG/GNEB step loop: 32 (FP32 bulk) or 64
    void * stream = nullptr; // caller-provided cudaStream_t for the device work (optional)
    std::string datetime;
    std::vector<std::string> log;
    int log_console_level = 2;
};

std::shared_ptr<Image> make_image_from_config( const std::string & cfg, State & st );
std::shared_ptr<Image> clone_image( const Image & src );
void refresh_positions( Image & img );
Engine & eval_engine( Image & img );
void log_msg( State * st, int level, const std::string & msg );

} // namespace sg
