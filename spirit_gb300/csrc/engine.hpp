// Device engine: one batch of independent spin systems resident in HBM, advanced together.
#pragma once
#include "common.hpp"
#include "ddi.hpp"
#include "geometry.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

#include <memory>
#include <vector>

namespace sg
{

struct SystemInput
{
    const Geometry * geom         = nullptr;
    const HamiltonianParams * ham = nullptr;
    double dt                     = 1e-3;
    double damping                = 0.3;
    double temperature            = 0;
    double force_convergence      = 1e-10;
    bool direct_minimization      = false;
    unsigned long long seed       = 2006;
    unsigned int stream           = 0;
    unsigned int noise_offset     = 0; // thermal-noise iterations drawn before this run
};

template<typename R>
struct StageArgs;
template<typename R>
struct SoA3;

// Host-side system descriptor of one system (spin_offset 0), as the engine builds it
void fill_system_desc( SysDesc & d, const SystemInput & in );

// Energy terms in the reference's order (Energy_Contributions_per_Spin, cpp:262-305)
enum Term
{
    TERM_ZEEMAN = 0,
    TERM_ANISOTROPY,
    TERM_EXCHANGE,
    TERM_DMI,
    TERM_DDI,
    N_TERMS
};

class Engine
{
public:
    Engine( const std::vector<SystemInput> & systems, bool fp64 );
    ~Engine();
    Engine( const Engine & )             = delete;
    Engine & operator=( const Engine & ) = delete;

    int n_sys() const
    {
        return (int)desc_.size();
    }
    int nos( int s ) const
    {
        return desc_[s].nos;
    }
    bool fp64() const
    {
        return fp64_;
    }
    long long total_spins() const
    {
        return total_;
    }

    // host AoS [nos][3] double <-> device SoA in the engine precision
    // sync = false: the copy and conversion are only enqueued (later launches on the engine's
    // stream see the new spins)
    void set_spins( int s, const double * aos, bool sync = true );
    void get_spins( int s, double * aos );
    // batched transfers of every system (one copy each way, converted on the device)
    void set_all_spins( const double * aos_concat );
    void get_all_spins( double * aos_concat );

    // Gradient, FP64 total energy and per-term energies of the current device spins of system s.
    void gradient( int s, double * grad_aos, double * energy, double * terms );
    // per-spin energy contributions [N_TERMS][nos] of system s
    void energy_per_spin( int s, double * per_term );

    // LLG: start a run (constructor probe: initial torque), then advance in steps.
    void llg_start( int solver, const std::vector<int> & n_iterations );
    // Launches n_steps steps (no host synchronisation).  Systems stop by themselves on
    // convergence or when their iteration budget is used up.
    void llg_launch( int n_steps );
    void sync();
    struct Status
    {
        int iteration;
        int active;
        float max_torque;
        double energy;
    };
    std::vector<Status> status();
    // the spins of system s (AoS, into aos) and its run status with a single synchronisation
    Status fetch( int s, double * aos );
    void set_params( int s, const SystemInput & in );
    // time one step of the current method on the stream with CUDA events (ms)
    cudaStream_t stream() const
    {
        return stream_;
    }
    // run on a caller's stream (e.g. a framework stream whose events time the kernels);
    // nullptr returns to the engine's own stream
    void set_stream( cudaStream_t s );
    int kernels_per_step() const;
    // tuned launch parameters: spins per thread of the stage kernels, lines / threads per block of
    // the FFT passes A, B, C, fused b/c pass (1 fused, 0 split), its cluster size and threads
    int tuning( int * out, int n ) const;
    // n steps launched kernel by kernel with CUDA events between launches on the engine stream;
    // before every step `flush_buf` is overwritten and `read_buf` read back (an L2 flush that
    // leaves clean lines; both may be null).
    // Adds per-kernel-id total ms and launch counts (arrays of N_KERNEL_IDS).
    void profile_steps( int n, void * flush_buf, size_t flush_bytes, void * read_buf, size_t read_bytes, double * ms,
                        int * count );
    // DDI field h of the current spins (tests)
    void ddi_field( int s, double * h_aos );

    // raw device pointers (component arrays) for the GNEB / Monte Carlo layers; their kernels
    // write the FP32 spins without the low parts of the compensated state, which therefore restart
    // from zero at the next LLG use
    void * spin_ptr( int comp ) const
    {
        lo_valid_ = false;
        return spins_[comp];
    }
    // FP32 LLG: keep the state compensated (hi + lo per component, see engine.cu)
    void enable_compensation();
    bool compensated() const
    {
        return comp_;
    }
    const SysDesc * d_desc() const
    {
        return d_desc_;
    }
    SysRun * d_runs() const
    {
        return d_runs_;
    }
    const int2 * d_blkmap() const
    {
        return d_blkmap_;
    }
    int n_blocks() const
    {
        return n_blocks_;
    }
    bool has_ddi() const
    {
        return any_ddi_;
    }
    void * field_ptr( int comp ) const
    {
        return field_[comp];
    }
    const SysDesc & desc( int s ) const
    {
        return desc_[s];
    }
    // dipolar field of the configuration cfg (3 component arrays) into field_ptr();
    // systems whose SysRun is inactive are skipped when runs != nullptr
    void run_ddi( void * const * cfg, const SysRun * runs )
    {
        if( any_ddi_ )
            ddi_.run( d_desc_, runs, cfg[0], cfg[1], cfg[2], field_[0], field_[1], field_[2], stream_ );
        w1_valid_ = false;
    }

    // A second dipolar lane: its own plan (work spectra), field arrays and stream, with the main
    // plan's tuned shapes, for dipolar fields computed beside the main stream (the adjoint's
    // recomputation of the previous segment).  Built on first use; null without dipolar systems.
    struct DdiLane
    {
        DDIPlan plan;
        void * field[3]     = { nullptr, nullptr, nullptr };
        cudaStream_t stream = nullptr;
    };
    DdiLane * ddi_lane();

private:
    void build_systems( const std::vector<SystemInput> & systems );
    void launch_step_kernels();
    template<typename R>
    void launch_step_t();
    template<typename R>
    void launch_probe_t();
    // close_iteration after the final stage of a step (or after the probe)
    void launch_close( int tune, int probe );
    template<typename R, int SOLVER, int STAGE>
    void launch_stage( StageArgs<R> a, cudaStream_t st );
    template<typename R, int SOLVER, int STAGE>
    void launch_stage_rows( StageArgs<R> a, cudaStream_t st );
    void build_row_map( int n_ddi );
    void ensure_spectrum();
    template<typename R>
    void launch_stages_t( StageArgs<R> & a, bool with_ddi );
    template<typename R>
    void tune_stages_t();
    template<typename R>
    void gradient_t( int s, double * grad_aos, double * energy, double * terms, double * per_spin );

    bool fp64_;
    size_t elem_;
    cudaStream_t stream_ = nullptr;
    cudaStream_t own_stream_ = nullptr;
    std::vector<SysDesc> desc_;
    std::vector<const Geometry *> geoms_;
    SysDesc * d_desc_ = nullptr;
    SysRun * d_runs_  = nullptr;
    long long total_  = 0; // padded total spins
    // SoA buffers (engine precision): state, predictor A/B, aux fv1, aux acc, DDI field
    void * spins_[3] = { nullptr, nullptr, nullptr };
    void * predA_[3] = { nullptr, nullptr, nullptr };
    void * predB_[3] = { nullptr, nullptr, nullptr };
    void * aux1_[3]  = { nullptr, nullptr, nullptr };
    void * aux2_[3]  = { nullptr, nullptr, nullptr };
    void * noise_[3] = { nullptr, nullptr, nullptr }; // thermal field of the current iteration
    void * field_[3] = { nullptr, nullptr, nullptr };
    void * lo_[3]    = { nullptr, nullptr, nullptr }; // low parts of the compensated FP32 state
    bool comp_       = false;
    mutable bool lo_valid_ = false; // lo_ belongs to the current high parts
    SoA3<float> lo_soa();
    SoA3<float> lo_valid() const;
    double * d_stage_ = nullptr; // AoS double staging for transfers
    double * d_red_   = nullptr; // reduction scratch (per-term sums)
    double * d_grad_  = nullptr; // AoS double gradient output
    int2 * d_blkmap_  = nullptr;
    int n_blocks_     = 0;
    int threads_      = 256;
    // block maps of the stage kernels for 1, 2, 4 spins per thread; spt_idx_ picks one (tuned)
    int2 * d_sblkmap_[3]  = { nullptr, nullptr, nullptr };
    int n_sblocks_[3]     = { 0, 0, 0 };
    int spt_idx_          = 0;
    int tuned_solver_     = -1;
    // TMA-staged persistent stage kernel (FP32 batches with a short stencil reach): tiles
    // (system, first spin, aligned window start, copies per component), tensor
    // maps of the three configuration buffers (state, predictor A, predictor B) x 3 components,
    // and an error flag the kernel sets when a copy does not arrive within its wait limit
    bool tma_           = false;
    int4 * d_tiles_     = nullptr;
    int n_tiles_        = 0;
    int * d_err_        = nullptr;
    CUtensorMap tmaps_[3][3];
    void build_tiles();
    void check_err();
    bool any_ddi_     = false;
    DDIPlan ddi_;
    std::vector<DDISystem> ddi_systems_;
    std::unique_ptr<DdiLane> lane_;
    // row-fused stages: the stage kernels do the passes along a (llg_stage_rows); the spectrum
    // then carries the configuration from one stage to the next b/c pass
    bool rows_          = false;
    bool w1_valid_      = false; // the spectrum holds the current state's (ready for a step)
    int4 * d_rowmap_    = nullptr;
    int n_rowblocks_    = 0;
    size_t rows_smem_   = 0;
    int solver_       = SOLVER_HEUN;
    cudaGraphExec_t graph_ = nullptr;
    cudaGraphExec_t graph1_ = nullptr; // single step
    std::vector<std::pair<int, cudaEvent_t>> * trace_ = nullptr;
    int graph_steps_       = 0;
    int graph_solver_      = -1;
};

} // namespace sg
