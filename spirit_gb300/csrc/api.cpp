// The C API (extern "C", noexcept): the reference's function names, signatures and argument
// meaning (core/include/Spirit/*.h), backed by the GB300 engine.  Declarations with their
// reference citations are in include/Spirit_gb300.h.
//
// Error behaviour: like the reference, every function catches everything and logs it
// (core/src/utility/Exception.cpp:70-110); unlike the reference, a CUDA error does not
// terminate the process -- the call logs, returns its default value, and the library stays
// usable.
#include "adjoint.hpp"
#include "config.hpp"
#include "gneb.hpp"
#include "htst.hpp"
#include "mc.hpp"
#include "ovf.hpp"
#include "state.hpp"
#include "util.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <thread>

using namespace sg;

// Simulation_Run_Info, core/include/Spirit/Simulation.h:57-71
struct Simulation_Run_Info
{
    int total_iterations = 0;
    int total_walltime   = 0;
    float total_ips      = 0;
    float max_torque     = 0;
    int n_history_iteration    = 0;
    int * history_iteration    = nullptr;
    int n_history_max_torque   = 0;
    float * history_max_torque = nullptr;
    int n_history_energy       = 0;
    float * history_energy     = nullptr;
};

namespace
{

constexpr double C_MU_B = 0.057883817555;

struct Idx
{
    std::shared_ptr<Image> img;
    std::shared_ptr<Chain> chain;
    int idx;
};

// from_indices (core/include/data/State.hpp:79-107): -1 selects the active image / chain
Idx from_indices( State * st, int idx_image, int idx_chain )
{
    if( !st || !st->chain )
        throw std::runtime_error( "The State pointer is invalid" );
    if( idx_chain > 0 )
        throw std::runtime_error( "Invalid chain index " + std::to_string( idx_chain ) );
    auto & ch = st->chain;
    int i     = idx_image < 0 ? st->idx_active_image : idx_image;
    if( i >= (int)ch->images.size() )
        throw std::runtime_error( "Invalid image index " + std::to_string( idx_image ) );
    return { ch->images[i], ch, i };
}

void handle( State * st, const char * where )
{
    try
    {
        throw;
    }
    catch( const std::exception & e )
    {
        log_msg( st, 1, std::string( where ) + ": " + e.what() );
    }
    catch( ... )
    {
        log_msg( st, 1, std::string( where ) + ": unknown error" );
    }
}

SystemInput input_of( const Image & img, unsigned int stream )
{
    SystemInput in;
    in.geom                = img.geom.get();
    in.ham                 = &img.ham;
    in.dt                  = img.llg.dt;
    in.damping             = img.llg.damping;
    in.temperature         = img.llg.temperature;
    in.force_convergence   = img.llg.force_convergence;
    in.direct_minimization = img.llg.direct_minimization;
    in.seed                = (unsigned long long)(unsigned)img.llg.rng_seed;
    in.stream              = stream;
    in.noise_offset        = img.llg_noise_drawn;
    return in;
}

Engine & run_engine( State * st, Image & img )
{
    bool fp64 = st->precision == 64;
    if( !img.run || img.run_version != img.version || img.run_fp64 != fp64 )
    {
        img.run.reset();
        img.run         = std::make_unique<Engine>( std::vector<SystemInput>{ input_of( img, 0 ) }, fp64 );
        img.run_version = img.version;
        img.run_fp64    = fp64;
        img.run->enable_compensation(); // FP32: compensated state of the LLG stage kernels
    }
    img.run->set_stream( (cudaStream_t)st->stream );
    return *img.run;
}

bool stop_file_present()
{
    std::ifstream f( "STOP" );
    return f.good();
}

const char * solver_name( int s )
{
    switch( s )
    {
    case 0:
        return "VP";
    case 1:
        return "SIB";
    case 2:
        return "Depondt";
    case 3:
        return "Heun";
    case 4:
        return "RK4";
    case 5:
        return "LBFGS_OSO";
    case 7:
        return "VP_OSO";
    default:
        return "None";
    }
}

Engine::Status finish_llg( Image & img, Engine & E )
{
    const Engine::Status s = E.fetch( 0, img.spins.data() );
    if( img.llg.temperature > 0 )
        img.llg_noise_drawn += (unsigned)( s.iteration - img.info.iteration );
    img.E               = s.energy;
    img.info.iteration  = s.iteration;
    img.info.max_torque = s.max_torque;
    img.info.time_ps    = s.iteration * img.llg.dt;
    auto now            = std::chrono::steady_clock::now();
    img.info.wall_ms    = std::chrono::duration_cast<std::chrono::milliseconds>( now - img.info.t_start ).count();
    img.info.ips        = img.info.wall_ms > 0 ? 1000.0 * s.iteration / img.info.wall_ms : 0.0;
    return s;
}

// Method::Iterate (core/src/engine/Method.cpp:57-113): the device stops a system by itself on
// convergence or at n_iterations; the host checks Simulation_Stop, the STOP file and the
// wall time between chunks of steps (growing from 8 up to 512 steps per chunk).
void iterate_llg( State * st, Image & img, Engine & E )
{
    int chunk = 8;
    auto t0   = std::chrono::steady_clock::now();
    while( true )
    {
        auto s = E.status()[0];
        if( !s.active || !img.iteration_allowed.load() || stop_file_present() )
            break;
        if( img.llg.max_walltime_sec > 0 )
        {
            double el = std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count();
            if( el > img.llg.max_walltime_sec )
                break;
        }
        E.llg_launch( chunk );
        E.sync();
        chunk = std::min( 512, chunk * 2 );
    }
    finish_llg( img, E );
    (void)st;
}

void update_data( Image & img )
{
    Engine & E = eval_engine( img );
    E.set_spins( 0, img.spins.data() );
    double Et;
    E.gradient( 0, img.eff_field.data(), &Et, nullptr );
    for( auto & v : img.eff_field )
        v = -v;
    img.E = Et;
}

void fill_run_info( Simulation_Run_Info * info, const MethodInfo & m )
{
    if( !info )
        return;
    info->total_iterations = m.iteration;
    info->total_walltime   = (int)m.wall_ms;
    info->total_ips        = (float)m.ips;
    info->max_torque       = m.max_torque;
}

std::function<bool( const double *, const double * )> make_filter( const double pos[3], const float rect[3], float cyl,
                                                                   float sph, bool inverted )
{
    Vec3 p{ pos[0], pos[1], pos[2] };
    float rc[3] = { rect ? rect[0] : -1.f, rect ? rect[1] : -1.f, rect ? rect[2] : -1.f };
    return [p, rc, cyl, sph, inverted]( const double *, const double * r ) {
        double d[3] = { r[0] - p[0], r[1] - p[1], r[2] - p[2] };
        double rcyl = std::sqrt( std::pow( r[0] - p[0], 2 ) + std::pow( r[1] - p[1], 2 ) );
        double rsph = std::sqrt( d[0] * d[0] + d[1] * d[1] + d[2] * d[2] );
        bool in = ( rc[0] < 0 || std::abs( d[0] ) < rc[0] ) && ( rc[1] < 0 || std::abs( d[1] ) < rc[1] )
                  && ( rc[2] < 0 || std::abs( d[2] ) < rc[2] ) && ( cyl < 0 || rcyl < cyl )
                  && ( sph < 0 || rsph < sph );
        return inverted ? !in : in;
    };
}

void centre_plus( const Image & img, const float * position, double out[3] )
{
    Vec3 c = img.geom->center();
    for( int e = 0; e < 3; ++e )
        out[e] = c[e] + ( position ? position[e] : 0.f );
}

void geometry_changed( State * st )
{
    // geometry setters act on every image of the chain (core/src/Spirit/Geometry.cpp:205-208)
    for( auto & img : st->chain->images )
    {
        update_interactions( *img->geom, img->ham );
        img->spin_pin.release(); // the buffer may move
        img->spins.assign( 3 * (size_t)img->nos(), 0.0 );
        for( int i = 0; i < img->nos(); ++i )
            img->spins[3 * i + 2] = 1.0;
        img->eff_field.assign( 3 * (size_t)img->nos(), 0.0 );
        refresh_positions( *img );
        img->touch();
    }
}

} // namespace

// OVF segment of an image (OVF_Segment(Spin_System), core/src/io/OVF_File.cpp: nodes
// (Na nb, Nb, Nc), bounds and step sizes in nm); the description carries the positions of the
// image's random streams so a run read back from the file continues them.
OvfSegment image_segment( const Image & img, const std::vector<double> & data, const char * comment )
{
    OvfSegment seg;
    const Geometry & g = *img.geom;
    seg.title          = std::string( "SPIRIT Version " ) + "2.2.0 (spirit_gb300)";
    seg.desc           = std::string( comment ? comment : "-" ) + "\nspirit_gb300 llg_noise_drawn=" +
               std::to_string( img.llg_noise_drawn ) + " mc_sweeps_drawn=" + std::to_string( img.mc_sweeps_drawn );
    seg.nodes          = { g.n_cells[0] * g.nb(), g.n_cells[1], g.n_cells[2] };
    const Vec3 lo = g.bounds_min(), hi = g.bounds_max();
    for( int e = 0; e < 3; ++e )
    {
        seg.bounds_min[e] = lo[e] * 0.1;
        seg.bounds_max[e] = hi[e] * 0.1;
        seg.base[e]       = 0;
        seg.step[e]       = g.lattice_constant * g.bravais[e][e] * 0.1;
    }
    seg.data = data;
    return seg;
}

// random-stream positions written by image_segment (absent in files of other writers)
void restore_streams( Image & img, const std::string & desc )
{
    auto grab = [&]( const char * key, unsigned int & out ) {
        size_t p = desc.find( key );
        if( p != std::string::npos )
            out = (unsigned int)std::stoul( desc.substr( p + std::strlen( key ) ) );
    };
    if( desc.find( "spirit_gb300" ) == std::string::npos )
        return;
    grab( "llg_noise_drawn=", img.llg_noise_drawn );
    grab( "mc_sweeps_drawn=", img.mc_sweeps_drawn );
}

// IO_Image_Read (core/src/Spirit/IO.cpp:186-292): copy min(N, nos) spins, normalise, vacancies -> +z
void read_image( Image & img, const OvfSegment & seg )
{
    if( seg.valuedim != 3 )
        throw std::runtime_error( "the OVF segment should have 3 columns, but has " + std::to_string( seg.valuedim ) );
    const size_t n = std::min( seg.data.size() / 3, (size_t)img.nos() );
    for( size_t i = 0; i < n; ++i )
    {
        double v[3] = { seg.data[3 * i], seg.data[3 * i + 1], seg.data[3 * i + 2] };
        double nn   = std::sqrt( v[0] * v[0] + v[1] * v[1] + v[2] * v[2] );
        for( int e = 0; e < 3; ++e )
            img.spins[3 * i + e] = nn < 1e-5 ? ( e == 2 ? 1.0 : 0.0 ) : v[e] / nn;
    }
    restore_streams( img, seg.desc );
}

// Monte Carlo run of one image: its own engine (precision of the State) and colouring
struct MCImageRun
{
    std::unique_ptr<Engine> eng;
    std::unique_ptr<MCRun> mc;
    long version = -1;
    bool fp64    = false;
};

MCImageRun & mc_image_run( State * st, Image & img )
{
    const bool fp64 = st->precision == 64;
    auto * r        = static_cast<MCImageRun *>( img.mc_run.get() );
    if( !r || r->version != img.version || r->fp64 != fp64 )
    {
        auto nr     = std::make_shared<MCImageRun>();
        nr->eng     = std::make_unique<Engine>( std::vector<SystemInput>{ input_of( img, 0 ) }, fp64 );
        nr->mc      = std::make_unique<MCRun>( *nr->eng );
        nr->version = img.version;
        nr->fp64    = fp64;
        img.mc_run  = nr;
        r           = nr.get();
    }
    r->eng->set_stream( (cudaStream_t)st->stream );
    return *r;
}

MCSettings mc_settings_of( const Image & img )
{
    MCSettings m;
    m.temperature       = img.mc.temperature;
    m.cone              = img.mc.step_cone;
    m.cone_angle_deg    = img.mc.cone_angle;
    m.adaptive          = img.mc.cone_adaptive;
    m.acceptance_target = img.mc.acceptance_target;
    m.seed              = (unsigned long long)(unsigned)img.mc.rng_seed;
    m.stream            = 0;
    m.n_iterations      = (int)img.mc.n_iterations;
    m.rng_offset        = img.mc_sweeps_drawn;
    return m;
}

void finish_mc( Image & img, MCImageRun & R )
{
    auto st = R.mc->status()[0];
    R.eng->get_spins( 0, img.spins.data() );
    img.mc_sweeps_drawn += (unsigned)( st.iteration - img.info.iteration );
    img.info.iteration = st.iteration;
    // the cone angle adapts during the run and is kept (Method_MC.cpp:85)
    if( img.mc.step_cone && img.mc.cone_adaptive )
        img.mc.cone_angle = st.cone_angle_deg;
    // the energy of the final state (Method_MC::Message_End -> UpdateEnergy)
    update_data( img );
    auto now         = std::chrono::steady_clock::now();
    img.info.wall_ms = std::chrono::duration_cast<std::chrono::milliseconds>( now - img.info.t_start ).count();
    img.info.ips     = img.info.wall_ms > 0 ? 1000.0 * st.iteration / img.info.wall_ms : 0.0;
}

// Method::Iterate for MC: sweeps in device chunks, host checks in between
void iterate_mc( Image & img, MCImageRun & R )
{
    int chunk = 8;
    auto t0   = std::chrono::steady_clock::now();
    while( true )
    {
        auto s = R.mc->status()[0];
        if( s.iteration >= img.mc.n_iterations || !img.iteration_allowed.load() || stop_file_present() )
            break;
        if( img.mc.max_walltime_sec > 0 )
        {
            double el = std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count();
            if( el > img.mc.max_walltime_sec )
                break;
        }
        R.mc->launch( chunk );
        chunk = std::min( 512, chunk * 2 );
    }
    finish_mc( img, R );
}

// adjoint driver behind Simulation_LLG_Adjoint / Simulation_LLG_Loss
namespace
{

// first-shell / reference value of a coupling family (0 when absent)
double first_of( const std::vector<double> & shells, const std::vector<double> & explicit_values, bool from_pairs )
{
    const auto & v = from_pairs ? explicit_values : shells;
    return v.empty() ? 0.0 : v[0];
}

double run_adjoint( State * state, const double * params, int n_steps, int checkpoint, const double * target,
                    double * grad_s0, double * grad_params, double * final_spins, int idx_image, int idx_chain,
                    bool gradients )
{
    auto I            = from_indices( state, idx_image, idx_chain );
    const Image & img = *I.img;
    if( !target )
        throw std::runtime_error( "target spins are required" );
    const HamiltonianParams & h0 = img.ham;
    const double J0 = first_of( h0.jij, h0.ex_J_in, h0.from_pairs );
    const double D0 = first_of( h0.dij, h0.dmi_D_in, h0.from_pairs );
    const double K0 = h0.aniso_K.empty() ? 0.0 : h0.aniso_K[0];
    const double Jv = params ? params[0] : J0, Dv = params ? params[1] : D0, Kv = params ? params[2] : K0;
    const double Bv = params ? params[3] : h0.B, av = params ? params[4] : img.llg.damping;
    auto scaled = []( double v, double ref ) {
        if( ref == 0.0 && v != 0.0 )
            throw std::runtime_error( "a coupling absent from the configuration cannot be set by the adjoint parameters" );
        return ref == 0.0 ? 0.0 : v / ref;
    };
    HamiltonianParams h = h0;
    const double sJ = scaled( Jv, J0 ), sD = scaled( Dv, D0 ), sK = scaled( Kv, K0 );
    for( auto & x : h.ex_J )
        x *= sJ;
    for( auto & x : h.dmi_D )
        x *= sD;
    for( auto & x : h.aniso_K )
        x *= sK;
    h.B = Bv;
    // unit couplings: d/dJ of every exchange pair, d/dD of every DMI vector (same merged pair order)
    HamiltonianParams hJ = h0, hD = h0;
    for( size_t k = 0; k < hJ.ex_J.size(); ++k )
        hJ.ex_J[k] = J0 != 0.0 ? h0.ex_J[k] / J0 : 0.0;
    for( auto & x : hJ.dmi_D )
        x = 0.0;
    for( auto & x : hD.ex_J )
        x = 0.0;
    for( size_t k = 0; k < hD.dmi_D.size(); ++k )
        hD.dmi_D[k] = D0 != 0.0 ? h0.dmi_D[k] / D0 : 0.0;
    SystemInput in;
    in.geom                = img.geom.get();
    in.ham                 = &h;
    in.dt                  = img.llg.dt;
    in.damping             = av;
    in.temperature         = img.llg.temperature;
    in.direct_minimization = img.llg.direct_minimization;
    in.force_convergence   = img.llg.force_convergence;
    AdjointInput A;
    A.s0         = img.spins.data();
    A.target     = target;
    A.n_steps    = n_steps;
    A.checkpoint = checkpoint > 0 ? checkpoint : 100;
    A.gradients  = gradients;
    SystemInput iJ = in, iD = in;
    iJ.ham         = &hJ;
    iD.ham         = &hD;
    fill_system_desc( A.unit_J, iJ );
    fill_system_desc( A.unit_D, iD );
    for( size_t k = 0; k < h0.aniso_K.size() && k < (size_t)MAX_BASIS; ++k )
        A.unit_K[k] = K0 != 0.0 ? h0.aniso_K[k] / K0 : 0.0;
    for( int e = 0; e < 3; ++e )
        A.unit_B[e] = C_MU_B * h.B_normal[e];
    Engine E( std::vector<SystemInput>{ in }, state->precision == 64 );
    if( state->stream )
        E.set_stream( (cudaStream_t)state->stream );
    AdjointOutput O;
    O.grad_s0     = grad_s0;
    O.final_spins = final_spins;
    const double loss = adjoint_run( E, A, O, state->precision == 64 );
    if( grad_params )
        for( int q = 0; q < 5; ++q )
            grad_params[q] = O.grad_params[q];
    return loss;
}

} // namespace

extern "C" {

// ============================================================== State (core/include/Spirit/State.h)
State * State_Setup( const char * config_file, bool quiet ) noexcept
{
    State * st = nullptr;
    try
    {
        st              = new State();
        st->quiet       = quiet;
        st->config_file = config_file ? config_file : "";
        {
            std::ifstream f( st->config_file );
            if( !st->config_file.empty() && !f.good() )
            {
                log_msg( st, 1, "Config file \"" + st->config_file + "\" could not be opened, using defaults" );
                st->config_file = "";
            }
        }
        auto img  = make_image_from_config( st->config_file, *st );
        st->chain = std::make_shared<Chain>();
        st->chain->images.push_back( img );
        st->chain->Rx.assign( 1, 0.0 );
        // GNEB parameters (Parameters_Method_GNEB_from_Config)
        if( !st->config_file.empty() )
        {
            ConfigFile cf;
            cf.load( st->config_file );
            auto & G = st->chain->gneb;
            cf.get( "gneb_spring_constant", G.spring_constant );
            cf.get( "gneb_force_convergence", G.force_convergence );
            cf.get( "gneb_n_iterations", G.n_iterations );
            cf.get( "gneb_n_iterations_log", G.n_iterations_log );
            cf.get( "gneb_n_energy_interpolations", G.n_E_interpolations );
            cf.get( "gneb_spring_force_ratio", G.spring_force_ratio );
            cf.get( "gneb_path_shortening_constant", G.path_shortening_constant );
        }
        auto now     = std::chrono::system_clock::now();
        std::time_t t = std::chrono::system_clock::to_time_t( now );
        char buf[64];
        std::strftime( buf, sizeof( buf ), "%Y-%m-%d_%H-%M-%S", std::localtime( &t ) );
        st->datetime = buf;
        return st;
    }
    catch( ... )
    {
        handle( st, "State_Setup" );
        return st;
    }
}

void State_Delete( State * state ) noexcept
{
    try
    {
        if( state && state->chain )
        {
            for( auto & img : state->chain->images )
                img->iteration_allowed = false;
            state->chain->iteration_allowed = false;
        }
        delete state;
    }
    catch( ... )
    {
        handle( nullptr, "State_Delete" );
    }
}

void State_Update( State * state ) noexcept
{
    try
    {
        for( auto & img : state->chain->images )
            img->touch();
    }
    catch( ... )
    {
        handle( state, "State_Update" );
    }
}

const char * State_DateTime( State * state ) noexcept
{
    try
    {
        return state->datetime.c_str();
    }
    catch( ... )
    {
        return "";
    }
}

void State_To_Config( State * state, const char * config_file, const char * comment ) noexcept
{
    try
    {
        auto I = from_indices( state, -1, -1 );
        auto & g = *I.img->geom;
        auto & h = I.img->ham;
        std::ofstream f( config_file );
        f << "# " << ( comment ? comment : "" ) << "\n";
        f << "bravais_vectors\n";
        for( auto & v : g.bravais )
            f << v[0] << " " << v[1] << " " << v[2] << "\n";
        f << "n_basis_cells " << g.n_cells[0] << " " << g.n_cells[1] << " " << g.n_cells[2] << "\n";
        f << "lattice_constant " << g.lattice_constant << "\n";
        f << "mu_s";
        for( double m : g.mu_s_basis )
            f << " " << m;
        f << "\nboundary_conditions " << h.bc[0] << " " << h.bc[1] << " " << h.bc[2] << "\n";
        f << "external_field_magnitude " << h.B << "\nexternal_field_normal " << h.B_normal[0] << " " << h.B_normal[1]
          << " " << h.B_normal[2] << "\n";
        f << "anisotropy_magnitude " << h.K << "\nanisotropy_normal " << h.K_normal[0] << " " << h.K_normal[1] << " "
          << h.K_normal[2] << "\n";
        f << "n_shells_exchange " << h.jij.size() << "\njij";
        for( double j : h.jij )
            f << " " << j;
        f << "\nn_shells_dmi " << h.dij.size() << "\ndij";
        for( double d : h.dij )
            f << " " << d;
        f << "\ndm_chirality " << h.dm_chirality << "\n";
        f << "ddi_method " << ( h.ddi_method == 1 ? "fft" : ( h.ddi_method == 3 ? "cutoff" : "none" ) ) << "\n";
        f << "llg_dt " << I.img->llg.dt << "\nllg_damping " << I.img->llg.damping << "\nllg_temperature "
          << I.img->llg.temperature << "\n";
    }
    catch( ... )
    {
        handle( state, "State_To_Config" );
    }
}

// ============================================================== Hamiltonian (core/include/Spirit/Hamiltonian.h)
void Hamiltonian_Set_Boundary_Conditions( State * state, const bool * periodical, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        // the reference does not regenerate interactions here (core/src/Spirit/Hamiltonian.cpp:22-51):
        // the stencil uses the new conditions, the DDI padding stays as it was prepared
        for( int d = 0; d < 3; ++d )
            I.img->ham.bc[d] = periodical[d] ? 1 : 0;
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_Boundary_Conditions" );
    }
}

void Hamiltonian_Set_Field( State * state, float magnitude, const float * normal, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        Vec3 n{ normal[0], normal[1], normal[2] };
        double l = std::sqrt( n[0] * n[0] + n[1] * n[1] + n[2] * n[2] );
        if( l > 0 )
            for( auto & x : n )
                x /= l;
        I.img->ham.B        = magnitude;
        I.img->ham.B_normal = n;
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_Field" );
    }
}

void Hamiltonian_Set_Anisotropy( State * state, float magnitude, const float * normal, int idx_image,
                                 int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        Vec3 n{ normal[0], normal[1], normal[2] };
        double l = std::sqrt( n[0] * n[0] + n[1] * n[1] + n[2] * n[2] );
        if( l > 0 )
            for( auto & x : n )
                x /= l;
        // every basis atom gets the anisotropy, even with magnitude 0 (Hamiltonian.cpp:110-135)
        h.K        = magnitude;
        h.K_normal = n;
        h.aniso_idx.clear();
        h.aniso_K.clear();
        h.aniso_n.clear();
        for( int i = 0; i < I.img->geom->nb(); ++i )
        {
            h.aniso_idx.push_back( i );
            h.aniso_K.push_back( magnitude );
            h.aniso_n.push_back( n );
        }
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_Anisotropy" );
    }
}

void Hamiltonian_Set_Cubic_Anisotropy( State * state, float magnitude, int idx_image, int idx_chain ) noexcept
{
    if( magnitude != 0 )
        log_msg( state, 2, "Hamiltonian_Set_Cubic_Anisotropy: cubic anisotropy is not part of this engine" );
    (void)idx_image;
    (void)idx_chain;
}

void Hamiltonian_Set_Exchange( State * state, int n_shells, const float * jij, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        h.jij.assign( jij, jij + n_shells );
        if( h.from_pairs )
        {
            h.from_pairs = false;
            h.dij.clear();
        }
        h.ex_pairs_in.clear();
        h.ex_J_in.clear();
        update_interactions( *I.img->geom, h );
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_Exchange" );
    }
}

void Hamiltonian_Set_DMI( State * state, int n_shells, const float * dij, int chirality, int idx_image,
                          int idx_chain ) noexcept
{
    try
    {
        if( chirality != 1 && chirality != 2 && chirality != -1 && chirality != -2 )
        {
            log_msg( state, 1, "Hamiltonian_Set_DMI: invalid chirality " + std::to_string( chirality ) );
            return;
        }
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        h.dij.assign( dij, dij + n_shells );
        h.dm_chirality = chirality;
        if( h.from_pairs )
        {
            h.from_pairs = false;
            h.jij.clear();
        }
        h.dmi_pairs_in.clear();
        h.dmi_D_in.clear();
        h.dmi_n_in.clear();
        update_interactions( *I.img->geom, h );
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_DMI" );
    }
}

void Hamiltonian_Set_DDI( State * state, int ddi_method, int n_periodic_images[3], float cutoff_radius,
                          bool pb_zero_padding, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        h.ddi_method = ddi_method;
        for( int d = 0; d < 3; ++d )
            h.ddi_images[d] = n_periodic_images[d];
        h.ddi_radius          = cutoff_radius;
        h.ddi_pb_zero_padding = pb_zero_padding;
        if( ddi_method == 3 )
            log_msg( state, 2, "Hamiltonian_Set_DDI: the cutoff/direct dipole sum is not part of this engine" );
        I.img->touch();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Set_DDI" );
    }
}

const char * Hamiltonian_Get_Name( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->ham.name.c_str();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Name" );
        return "";
    }
}

void Hamiltonian_Get_Boundary_Conditions( State * state, bool * periodical, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        for( int d = 0; d < 3; ++d )
            periodical[d] = I.img->ham.bc[d] != 0;
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Boundary_Conditions" );
    }
}

void Hamiltonian_Get_Field( State * state, float * magnitude, float * normal, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        *magnitude = (float)I.img->ham.B;
        for( int d = 0; d < 3; ++d )
            normal[d] = (float)I.img->ham.B_normal[d];
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Field" );
    }
}

void Hamiltonian_Get_Anisotropy( State * state, float * magnitude, float * normal, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        if( !h.aniso_idx.empty() )
        {
            *magnitude = (float)h.aniso_K[0];
            for( int d = 0; d < 3; ++d )
                normal[d] = (float)h.aniso_n[0][d];
        }
        else
        {
            *magnitude = 0;
            normal[0] = normal[1] = 0;
            normal[2]             = 1;
        }
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Anisotropy" );
    }
}

void Hamiltonian_Get_Cubic_Anisotropy( State * state, float * magnitude, int idx_image, int idx_chain ) noexcept
{
    (void)state;
    (void)idx_image;
    (void)idx_chain;
    *magnitude = 0;
}

void Hamiltonian_Get_Exchange_Shells( State * state, int * n_shells, float * jij, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I    = from_indices( state, idx_image, idx_chain );
        *n_shells = (int)I.img->ham.jij.size();
        for( size_t k = 0; k < I.img->ham.jij.size(); ++k )
            jij[k] = (float)I.img->ham.jij[k];
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Exchange_Shells" );
    }
}

int Hamiltonian_Get_Exchange_N_Pairs( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (int)from_indices( state, idx_image, idx_chain ).img->ham.ex_pairs.size();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Exchange_N_Pairs" );
        return 0;
    }
}

void Hamiltonian_Get_Exchange_Pairs( State * state, int idx[][2], int translations[][3], float * Jij, int idx_image,
                                     int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto & h = I.img->ham;
        for( size_t p = 0; p < h.ex_pairs.size(); ++p )
        {
            idx[p][0] = h.ex_pairs[p].i;
            idx[p][1] = h.ex_pairs[p].j;
            for( int d = 0; d < 3; ++d )
                translations[p][d] = h.ex_pairs[p].t[d];
            Jij[p] = (float)h.ex_J[p];
        }
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Exchange_Pairs" );
    }
}

void Hamiltonian_Get_DMI_Shells( State * state, int * n_shells, float * dij, int * chirality, int idx_image,
                                 int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        *n_shells  = (int)I.img->ham.dij.size();
        *chirality = I.img->ham.dm_chirality;
        for( size_t k = 0; k < I.img->ham.dij.size(); ++k )
            dij[k] = (float)I.img->ham.dij[k];
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_DMI_Shells" );
    }
}

int Hamiltonian_Get_DMI_N_Pairs( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (int)from_indices( state, idx_image, idx_chain ).img->ham.dmi_pairs.size();
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_DMI_N_Pairs" );
        return 0;
    }
}

void Hamiltonian_Get_DDI( State * state, int * ddi_method, int n_periodic_images[3], float * cutoff_radius,
                          bool * pb_zero_padding, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I      = from_indices( state, idx_image, idx_chain );
        auto & h    = I.img->ham;
        *ddi_method = h.ddi_method;
        for( int d = 0; d < 3; ++d )
            n_periodic_images[d] = h.ddi_images[d];
        *cutoff_radius   = (float)h.ddi_radius;
        *pb_zero_padding = h.ddi_pb_zero_padding;
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_DDI" );
    }
}

// ---- extensions (no reference C API counterpart; the reference reaches these through its
// C++ internals: Hamiltonian::Gradient / Gradient_and_Energy / Energy_Contributions_per_Spin)

// FP64 gradient of the image's current spins, AoS [nos][3]; returns the total FP64 energy
double Hamiltonian_Get_Gradient( State * state, double * gradient, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        Engine & E = eval_engine( *I.img );
        E.set_spins( 0, I.img->spins.data() );
        double Et = 0;
        E.gradient( 0, gradient, &Et, nullptr );
        return Et;
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Gradient" );
        return 0;
    }
}

// FP64 gradients (AoS, concatenated in the order of the States) and energies of the active images
// of n States, evaluated together by one batched FP64 engine (shared dipolar plan table)
void Hamiltonian_Get_Gradient_Batched( State ** states, int n_states, double * gradients, double * energies ) noexcept
{
    State * first = n_states > 0 ? states[0] : nullptr;
    try
    {
        gradient_batched( states, n_states, gradients, energies );
    }
    catch( ... )
    {
        handle( first, "Hamiltonian_Get_Gradient_Batched" );
    }
}

// FP64 energy per term (Zeeman, Anisotropy, Exchange, DMI, DDI); per_spin (optional) gets
// [5][nos].  Returns the total.
double Hamiltonian_Get_Energy_Contributions( State * state, double * terms, double * per_spin, int idx_image,
                                            int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        Engine & E = eval_engine( *I.img );
        E.set_spins( 0, I.img->spins.data() );
        double Et = 0, t[N_TERMS];
        E.gradient( 0, nullptr, &Et, t );
        if( terms )
            for( int k = 0; k < N_TERMS; ++k )
                terms[k] = t[k];
        if( per_spin )
            E.energy_per_spin( 0, per_spin );
        return Et;
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_Energy_Contributions" );
        return 0;
    }
}

// dipolar field h (the convolution D * mu s) of the current spins, AoS; FP64 engine
void Hamiltonian_Get_DDI_Field( State * state, double * field, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        Engine & E = eval_engine( *I.img );
        E.set_spins( 0, I.img->spins.data() );
        E.ddi_field( 0, field );
    }
    catch( ... )
    {
        handle( state, "Hamiltonian_Get_DDI_Field" );
    }
}

// ============================================================== Geometry (core/include/Spirit/Geometry.h)
void Geometry_Set_N_Cells( State * state, int n_cells[3] ) noexcept
{
    try
    {
        auto g = state->chain->images[0]->geom;
        g->n_cells = { n_cells[0], n_cells[1], n_cells[2] };
        geometry_changed( state );
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_N_Cells" );
    }
}

void Geometry_Set_mu_s( State * state, float mu_s, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        for( auto & m : I.img->geom->mu_s_basis )
            m = mu_s;
        for( auto & img : state->chain->images )
            img->touch();
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_mu_s" );
    }
}

void Geometry_Set_Lattice_Constant( State * state, float lattice_constant ) noexcept
{
    try
    {
        state->chain->images[0]->geom->lattice_constant = lattice_constant;
        geometry_changed( state );
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_Lattice_Constant" );
    }
}

void Geometry_Set_Bravais_Lattice_Type( State * state, int lattice_type ) noexcept
{
    try
    {
        // Bravais_Lattice_Type (Geometry.h:20-32): Irregular=0, Rectilinear=1, SC=2, Hex2D=3, Hex2D_60=4,
        // Hex2D_120=5, HCP=6, BCT=7, BCC=8, FCC=9
        const char * names[] = { nullptr, nullptr, "sc", "hex2d", "hex2d60", "hex2d120", nullptr, nullptr, "bcc", "fcc" };
        if( lattice_type < 0 || lattice_type > 9 || !names[lattice_type] )
        {
            log_msg( state, 1, "Geometry_Set_Bravais_Lattice_Type: unsupported lattice type" );
            return;
        }
        auto g          = state->chain->images[0]->geom;
        g->bravais      = bravais_preset( names[lattice_type] );
        g->bravais_name = names[lattice_type];
        geometry_changed( state );
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_Bravais_Lattice_Type" );
    }
}

void Geometry_Set_Bravais_Vectors( State * state, float ta[3], float tb[3], float tc[3] ) noexcept
{
    try
    {
        auto g          = state->chain->images[0]->geom;
        g->bravais      = { Vec3{ ta[0], ta[1], ta[2] }, Vec3{ tb[0], tb[1], tb[2] }, Vec3{ tc[0], tc[1], tc[2] } };
        g->bravais_name = "irregular";
        geometry_changed( state );
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_Bravais_Vectors" );
    }
}

void Geometry_Set_Cell_Atoms( State * state, int n_atoms, float ** atoms ) noexcept
{
    try
    {
        auto g = state->chain->images[0]->geom;
        g->cell_atoms.clear();
        for( int a = 0; a < n_atoms; ++a )
            g->cell_atoms.push_back( Vec3{ atoms[a][0], atoms[a][1], atoms[a][2] } );
        double m0 = g->mu_s_basis.empty() ? 1.0 : g->mu_s_basis[0];
        g->mu_s_basis.assign( n_atoms, m0 );
        for( auto & img : state->chain->images )
            set_uniform_anisotropy( *g, img->ham, img->ham.K, img->ham.K_normal );
        geometry_changed( state );
    }
    catch( ... )
    {
        handle( state, "Geometry_Set_Cell_Atoms" );
    }
}

int Geometry_Get_NOS( State * state ) noexcept
{
    try
    {
        return state->chain->images[0]->nos();
    }
    catch( ... )
    {
        return 0;
    }
}

double * Geometry_Get_Positions( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->positions.data();
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_Positions" );
        return nullptr;
    }
}

void Geometry_Get_Bounds( State * state, float min[3], float max[3], int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        auto a = I.img->geom->bounds_min(), b = I.img->geom->bounds_max();
        for( int d = 0; d < 3; ++d )
        {
            min[d] = (float)a[d];
            max[d] = (float)b[d];
        }
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_Bounds" );
    }
}

void Geometry_Get_Center( State * state, float center[3], int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto c = from_indices( state, idx_image, idx_chain ).img->geom->center();
        for( int d = 0; d < 3; ++d )
            center[d] = (float)c[d];
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_Center" );
    }
}

void Geometry_Get_Bravais_Vectors( State * state, float a[3], float b[3], float c[3], int idx_image,
                                   int idx_chain ) noexcept
{
    try
    {
        auto & br = from_indices( state, idx_image, idx_chain ).img->geom->bravais;
        for( int d = 0; d < 3; ++d )
        {
            a[d] = (float)br[0][d];
            b[d] = (float)br[1][d];
            c[d] = (float)br[2][d];
        }
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_Bravais_Vectors" );
    }
}

int Geometry_Get_Dimensionality( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->geom->dimensionality();
    }
    catch( ... )
    {
        return 0;
    }
}

void Geometry_Get_mu_s( State * state, float * mu_s, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        for( int i = 0; i < I.img->nos(); ++i )
            mu_s[i] = (float)I.img->geom->mu_s( i );
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_mu_s" );
    }
}

void Geometry_Get_N_Cells( State * state, int n_cells[3], int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto & n = from_indices( state, idx_image, idx_chain ).img->geom->n_cells;
        for( int d = 0; d < 3; ++d )
            n_cells[d] = n[d];
    }
    catch( ... )
    {
        handle( state, "Geometry_Get_N_Cells" );
    }
}

int Geometry_Get_N_Cell_Atoms( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->geom->nb();
    }
    catch( ... )
    {
        return 0;
    }
}

double Geometry_Get_Lattice_Constant( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->geom->lattice_constant;
    }
    catch( ... )
    {
        return 0;
    }
}

// ============================================================== Configurations (core/include/Spirit/Configurations.h)
static void apply_domain( State * state, Vec3 v, const float * position, const float * rect, float cyl, float sph,
                          bool inverted, int idx_image, int idx_chain )
{
    auto I = from_indices( state, idx_image, idx_chain );
    double p[3];
    centre_plus( *I.img, position, p );
    auto filter = make_filter( p, rect, cyl, sph, inverted );
    double n    = std::sqrt( v[0] * v[0] + v[1] * v[1] + v[2] * v[2] );
    if( n < 1e-8 )
        v = { 0, 0, 1 };
    else
        for( auto & x : v )
            x /= n;
    auto & S = I.img->spins;
    for( int i = 0; i < I.img->nos(); ++i )
        if( filter( &S[3 * i], &I.img->positions[3 * i] ) )
            for( int e = 0; e < 3; ++e )
                S[3 * i + e] = v[e];
}

void Configuration_Domain( State * state, const float direction[3], const float position[3],
                           const float r_cut_rectangular[3], float r_cut_cylindrical, float r_cut_spherical,
                           bool inverted, int idx_image, int idx_chain ) noexcept
{
    try
    {
        apply_domain( state, { direction[0], direction[1], direction[2] }, position, r_cut_rectangular,
                      r_cut_cylindrical, r_cut_spherical, inverted, idx_image, idx_chain );
    }
    catch( ... )
    {
        handle( state, "Configuration_Domain" );
    }
}

void Configuration_PlusZ( State * state, const float position[3], const float r_cut_rectangular[3],
                          float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                          int idx_chain ) noexcept
{
    try
    {
        apply_domain( state, { 0, 0, 1 }, position, r_cut_rectangular, r_cut_cylindrical, r_cut_spherical, inverted,
                      idx_image, idx_chain );
    }
    catch( ... )
    {
        handle( state, "Configuration_PlusZ" );
    }
}

void Configuration_MinusZ( State * state, const float position[3], const float r_cut_rectangular[3],
                           float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                           int idx_chain ) noexcept
{
    try
    {
        apply_domain( state, { 0, 0, -1 }, position, r_cut_rectangular, r_cut_cylindrical, r_cut_spherical, inverted,
                      idx_image, idx_chain );
    }
    catch( ... )
    {
        handle( state, "Configuration_MinusZ" );
    }
}

// Configurations::Random with the image's mt19937 (core/src/utility/Configurations.cpp:99-126)
void Configuration_Random( State * state, const float position[3], const float r_cut_rectangular[3],
                           float r_cut_cylindrical, float r_cut_spherical, bool inverted, bool external,
                           int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        double p[3];
        centre_plus( *I.img, position, p );
        auto filter = make_filter( p, r_cut_rectangular, r_cut_cylindrical, r_cut_spherical, inverted );
        std::uniform_real_distribution<double> dist( -1, 1 );
        auto & S = I.img->spins;
        (void)external;
        for( int i = 0; i < I.img->nos(); ++i )
            if( filter( &S[3 * i], &I.img->positions[3 * i] ) )
            {
                double vz  = dist( I.img->prng );
                double phi = dist( I.img->prng ) * M_PI;
                double r   = std::sqrt( 1 - vz * vz );
                S[3 * i]     = r * std::cos( phi );
                S[3 * i + 1] = r * std::sin( phi );
                S[3 * i + 2] = vz;
            }
    }
    catch( ... )
    {
        handle( state, "Configuration_Random" );
    }
}

// Configurations::Skyrmion (core/src/utility/Configurations.cpp:218-270), non-experimental profile
void Configuration_Skyrmion( State * state, float r, float order, float phase, bool upDown, bool achiral, bool rl,
                             const float position[3], const float r_cut_rectangular[3], float r_cut_cylindrical,
                             float r_cut_spherical, bool inverted, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        double p[3];
        centre_plus( *I.img, position, p );
        if( r_cut_cylindrical < 0 )
            r_cut_cylindrical = r;
        auto filter = make_filter( p, r_cut_rectangular, r_cut_cylindrical, r_cut_spherical, inverted );
        auto & S    = I.img->spins;
        auto & P    = I.img->positions;
        int ksi = ( (int)rl ) * 2 - 1, dir = ( (int)upDown ) * 2 - 1;
        for( int i = 0; i < I.img->nos(); ++i )
        {
            double distance = std::sqrt( std::pow( P[3 * i] - p[0], 2 ) + std::pow( P[3 * i + 1] - p[1], 2 ) );
            distance /= r;
            if( filter( &S[3 * i], &P[3 * i] ) )
            {
                double x     = ( P[3 * i] - p[0] ) / distance / r;
                double phi_i = std::acos( std::max( -1.0, std::min( 1.0, x ) ) );
                if( distance == 0 )
                    phi_i = 0;
                if( P[3 * i + 1] - p[1] < 0.0 )
                    phi_i = -phi_i;
                phi_i += phase / 180 * M_PI;
                double theta_i = M_PI - M_PI * distance;
                S[3 * i]       = ksi * std::sin( theta_i ) * std::cos( order * phi_i );
                S[3 * i + 1]   = ksi * std::sin( theta_i ) * std::sin( order * ( phi_i + achiral * M_PI ) );
                S[3 * i + 2]   = std::cos( theta_i ) * -dir;
            }
        }
        for( int i = 0; i < I.img->nos(); ++i )
        {
            double n2 = S[3 * i] * S[3 * i] + S[3 * i + 1] * S[3 * i + 1] + S[3 * i + 2] * S[3 * i + 2];
            if( n2 > 0 )
            {
                double n = std::sqrt( n2 );
                for( int e = 0; e < 3; ++e )
                    S[3 * i + e] /= n;
            }
        }
    }
    catch( ... )
    {
        handle( state, "Configuration_Skyrmion" );
    }
}

void Configuration_To_Clipboard( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I           = from_indices( state, idx_image, idx_chain );
        state->clipboard = clone_image( *I.img );
    }
    catch( ... )
    {
        handle( state, "Configuration_To_Clipboard" );
    }
}

void Configuration_From_Clipboard( State * state, const float position[3], const float r_cut_rectangular[3],
                                   float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                                   int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( !state->clipboard || state->clipboard->nos() != I.img->nos() )
            return;
        double p[3];
        centre_plus( *I.img, position, p );
        auto filter = make_filter( p, r_cut_rectangular, r_cut_cylindrical, r_cut_spherical, inverted );
        for( int i = 0; i < I.img->nos(); ++i )
            if( filter( &I.img->spins[3 * i], &I.img->positions[3 * i] ) )
                for( int e = 0; e < 3; ++e )
                    I.img->spins[3 * i + e] = state->clipboard->spins[3 * i + e];
    }
    catch( ... )
    {
        handle( state, "Configuration_From_Clipboard" );
    }
}

// ============================================================== Chain (core/include/Spirit/Chain.h)
int Chain_Get_NOI( State * state, int idx_chain ) noexcept
{
    try
    {
        (void)idx_chain;
        return (int)state->chain->images.size();
    }
    catch( ... )
    {
        return 0;
    }
}

bool Chain_Jump_To_Image( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I                  = from_indices( state, idx_image, idx_chain );
        state->idx_active_image = I.idx;
        return true;
    }
    catch( ... )
    {
        handle( state, "Chain_Jump_To_Image" );
        return false;
    }
}

bool Chain_next_Image( State * state, int idx_chain ) noexcept
{
    if( state->idx_active_image + 1 < (int)state->chain->images.size() )
        return Chain_Jump_To_Image( state, state->idx_active_image + 1, idx_chain );
    return false;
}

bool Chain_prev_Image( State * state, int idx_chain ) noexcept
{
    if( state->idx_active_image > 0 )
        return Chain_Jump_To_Image( state, state->idx_active_image - 1, idx_chain );
    return false;
}

void Chain_Image_to_Clipboard( State * state, int idx_image, int idx_chain ) noexcept
{
    Configuration_To_Clipboard( state, idx_image, idx_chain );
}

void Chain_Replace_Image( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( !state->clipboard )
            return;
        auto img                  = clone_image( *state->clipboard );
        img->geom                 = I.img->geom;
        state->chain->images[I.idx] = img;
    }
    catch( ... )
    {
        handle( state, "Chain_Replace_Image" );
    }
}

static void insert_image( State * state, int pos )
{
    if( !state->clipboard )
    {
        log_msg( state, 1, "Tried to insert an image, but the clipboard is empty" );
        return;
    }
    auto img  = clone_image( *state->clipboard );
    img->geom = state->chain->images[0]->geom;
    state->chain->images.insert( state->chain->images.begin() + pos, img );
    state->chain->Rx.assign( state->chain->images.size(), 0.0 );
}

void Chain_Insert_Image_Before( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        insert_image( state, I.idx );
        if( I.idx <= state->idx_active_image )
            ++state->idx_active_image;
    }
    catch( ... )
    {
        handle( state, "Chain_Insert_Image_Before" );
    }
}

void Chain_Insert_Image_After( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        insert_image( state, I.idx + 1 );
    }
    catch( ... )
    {
        handle( state, "Chain_Insert_Image_After" );
    }
}

void Chain_Push_Back( State * state, int idx_chain ) noexcept
{
    try
    {
        (void)idx_chain;
        insert_image( state, (int)state->chain->images.size() );
    }
    catch( ... )
    {
        handle( state, "Chain_Push_Back" );
    }
}

bool Chain_Delete_Image( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( state->chain->images.size() <= 1 )
            return false;
        state->chain->images.erase( state->chain->images.begin() + I.idx );
        if( state->idx_active_image >= (int)state->chain->images.size() )
            state->idx_active_image = (int)state->chain->images.size() - 1;
        state->chain->Rx.assign( state->chain->images.size(), 0.0 );
        return true;
    }
    catch( ... )
    {
        handle( state, "Chain_Delete_Image" );
        return false;
    }
}

bool Chain_Pop_Back( State * state, int idx_chain ) noexcept
{
    return Chain_Delete_Image( state, (int)state->chain->images.size() - 1, idx_chain );
}

void Chain_Set_Length( State * state, int n_images, int idx_chain ) noexcept
{
    try
    {
        if( n_images < 1 )
            return;
        if( !state->clipboard )
            Chain_Image_to_Clipboard( state, -1, idx_chain );
        while( (int)state->chain->images.size() < n_images )
            insert_image( state, (int)state->chain->images.size() );
        while( (int)state->chain->images.size() > n_images )
            state->chain->images.pop_back();
        if( state->idx_active_image >= n_images )
            state->idx_active_image = n_images - 1;
        state->chain->Rx.assign( state->chain->images.size(), 0.0 );
    }
    catch( ... )
    {
        handle( state, "Chain_Set_Length" );
    }
}

void Chain_Get_Rx( State * state, float * Rx, int idx_chain ) noexcept
{
    (void)idx_chain;
    for( size_t i = 0; i < state->chain->Rx.size(); ++i )
        Rx[i] = (float)state->chain->Rx[i];
}

void Chain_Get_Energy( State * state, float * energy, int idx_chain ) noexcept
{
    (void)idx_chain;
    for( size_t i = 0; i < state->chain->images.size(); ++i )
        energy[i] = (float)state->chain->images[i]->E;
}

void Chain_Get_Rx_Interpolated( State * state, float * Rx, int idx_chain ) noexcept
{
    (void)idx_chain;
    for( size_t i = 0; i < state->chain->Rx_interpolated.size(); ++i )
        Rx[i] = (float)state->chain->Rx_interpolated[i];
}

void Chain_Get_Energy_Interpolated( State * state, float * E, int idx_chain ) noexcept
{
    (void)idx_chain;
    for( size_t i = 0; i < state->chain->E_interpolated.size(); ++i )
        E[i] = (float)state->chain->E_interpolated[i];
}

void Chain_Update_Data( State * state, int idx_chain ) noexcept
{
    try
    {
        (void)idx_chain;
        auto & ch = *state->chain;
        for( auto & img : ch.images )
            update_data( *img );
        gneb_update_rx( ch );
    }
    catch( ... )
    {
        handle( state, "Chain_Update_Data" );
    }
}

void Chain_Setup_Data( State * state, int idx_chain ) noexcept
{
    Chain_Update_Data( state, idx_chain );
}

// ============================================================== Transitions (core/include/Spirit/Transitions.h)
// Homogeneous_Rotation (core/src/utility/Configuration_Chain.cpp:28-75); its antiparallel-axis
// test is always false in the reference, so antiparallel spins rotate about e_y -- kept as is.
void Transition_Homogeneous( State * state, int idx_1, int idx_2, int idx_chain ) noexcept
{
    try
    {
        (void)idx_chain;
        auto & imgs = state->chain->images;
        if( idx_1 < 0 || idx_2 >= (int)imgs.size() || idx_1 >= idx_2 )
        {
            log_msg( state, 1, "Transition_Homogeneous: invalid image indices" );
            return;
        }
        int nos            = imgs[0]->nos();
        const double * s1  = imgs[idx_1]->spins.data();
        const double * s2  = imgs[idx_2]->spins.data();
        for( int i = 0; i < nos; ++i )
        {
            const double * a = s1 + 3 * i;
            const double * b = s2 + 3 * i;
            double r         = std::fmax( -1.0, std::fmin( 1.0, a[0] * b[0] + a[1] * b[1] + a[2] * b[2] ) );
            double ang       = std::acos( r );
            double ax[3]     = { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
            double n2        = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
            if( n2 > 0 )
            {
                double n = std::sqrt( n2 );
                for( auto & x : ax )
                    x /= n;
            }
            if( std::abs( ang - M_PI ) < 1e-4 )
            {
                if( std::abs( a[0] ) - 1 > 1e-4 )
                {
                    ax[0] = 1;
                    ax[1] = ax[2] = 0;
                }
                else
                {
                    ax[1] = 1;
                    ax[0] = ax[2] = 0;
                }
            }
            for( int img = idx_1 + 1; img < idx_2; ++img )
            {
                double * o = imgs[img]->spins.data() + 3 * i;
                if( ang > 1e-8 )
                {
                    double angle = ang * double( img - idx_1 ) / double( idx_2 - idx_1 );
                    double c = std::cos( angle ), s = std::sin( angle );
                    double cr[3] = { ax[1] * a[2] - ax[2] * a[1], ax[2] * a[0] - ax[0] * a[2],
                                     ax[0] * a[1] - ax[1] * a[0] };
                    double ad    = ax[0] * a[0] + ax[1] * a[1] + ax[2] * a[2];
                    for( int e = 0; e < 3; ++e )
                        o[e] = a[e] * c + cr[e] * s + ax[e] * ad * ( 1 - c );
                }
                else
                    for( int e = 0; e < 3; ++e )
                        o[e] = a[e];
            }
        }
    }
    catch( ... )
    {
        handle( state, "Transition_Homogeneous" );
    }
}

// ============================================================== Parameters_LLG (core/include/Spirit/Parameters_LLG.h)
void Parameters_LLG_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_image,
                                      int idx_chain ) noexcept
{
    try
    {
        auto I                      = from_indices( state, idx_image, idx_chain );
        I.img->llg.n_iterations     = n_iterations;
        I.img->llg.n_iterations_log = n_iterations_log;
    }
    catch( ... )
    {
        handle( state, "Parameters_LLG_Set_N_Iterations" );
    }
}

void Parameters_LLG_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_image,
                                      int idx_chain ) noexcept
{
    try
    {
        auto I          = from_indices( state, idx_image, idx_chain );
        *iterations     = (int)I.img->llg.n_iterations;
        *iterations_log = (int)I.img->llg.n_iterations_log;
    }
    catch( ... )
    {
        handle( state, "Parameters_LLG_Get_N_Iterations" );
    }
}

#define LLG_SETTER( NAME, FIELD, TYPE )                                                                               \
    void Parameters_LLG_Set_##NAME( State * state, TYPE v, int idx_image, int idx_chain ) noexcept                    \
    {                                                                                                                 \
        try                                                                                                           \
        {                                                                                                             \
            from_indices( state, idx_image, idx_chain ).img->llg.FIELD = v;                                           \
        }                                                                                                             \
        catch( ... )                                                                                                  \
        {                                                                                                             \
            handle( state, "Parameters_LLG_Set_" #NAME );                                                             \
        }                                                                                                             \
    }
#define LLG_GETTER( NAME, FIELD, TYPE )                                                                               \
    TYPE Parameters_LLG_Get_##NAME( State * state, int idx_image, int idx_chain ) noexcept                           \
    {                                                                                                                 \
        try                                                                                                           \
        {                                                                                                             \
            return (TYPE)from_indices( state, idx_image, idx_chain ).img->llg.FIELD;                                  \
        }                                                                                                             \
        catch( ... )                                                                                                  \
        {                                                                                                             \
            handle( state, "Parameters_LLG_Get_" #NAME );                                                             \
            return TYPE( 0 );                                                                                         \
        }                                                                                                             \
    }

LLG_SETTER( Direct_Minimization, direct_minimization, bool )
LLG_SETTER( Convergence, force_convergence, float )
LLG_SETTER( Time_Step, dt, float )
LLG_SETTER( Damping, damping, float )
LLG_SETTER( Non_Adiabatic_Damping, beta, float )
LLG_SETTER( Temperature, temperature, float )
LLG_GETTER( Direct_Minimization, direct_minimization, bool )
LLG_GETTER( Convergence, force_convergence, float )
LLG_GETTER( Time_Step, dt, float )
LLG_GETTER( Damping, damping, float )
LLG_GETTER( Non_Adiabatic_Damping, beta, float )
LLG_GETTER( Temperature, temperature, float )

// thermal-noise seed: the reference reads it from the config file only (llg_seed); this
// extension sets it at run time (the Philox key of the thermal field)
void Parameters_LLG_Set_Seed( State * state, int seed, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I          = from_indices( state, idx_image, idx_chain );
        I.img->llg.rng_seed = seed;
        I.img->prng.seed( seed );
    }
    catch( ... )
    {
        handle( state, "Parameters_LLG_Set_Seed" );
    }
}

void Parameters_LLG_Set_Output_General( State * state, bool any, bool initial, bool final, int idx_image,
                                        int idx_chain ) noexcept
{
    (void)state;
    (void)any;
    (void)initial;
    (void)final;
    (void)idx_image;
    (void)idx_chain;
}

// ============================================================== Parameters_GNEB (core/include/Spirit/Parameters_GNEB.h)
void Parameters_GNEB_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_chain ) noexcept
{
    (void)idx_chain;
    state->chain->gneb.n_iterations     = n_iterations;
    state->chain->gneb.n_iterations_log = n_iterations_log;
}

void Parameters_GNEB_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_chain ) noexcept
{
    (void)idx_chain;
    *iterations     = (int)state->chain->gneb.n_iterations;
    *iterations_log = (int)state->chain->gneb.n_iterations_log;
}

void Parameters_GNEB_Set_Convergence( State * state, float convergence, int idx_image, int idx_chain ) noexcept
{
    (void)idx_image;
    (void)idx_chain;
    state->chain->gneb.force_convergence = convergence;
}

float Parameters_GNEB_Get_Convergence( State * state, int idx_image, int idx_chain ) noexcept
{
    (void)idx_image;
    (void)idx_chain;
    return (float)state->chain->gneb.force_convergence;
}

void Parameters_GNEB_Set_Spring_Constant( State * state, float spring_constant, int idx_image, int idx_chain ) noexcept
{
    (void)idx_image;
    (void)idx_chain;
    state->chain->gneb.spring_constant = spring_constant;
}

float Parameters_GNEB_Get_Spring_Constant( State * state, int idx_image, int idx_chain ) noexcept
{
    (void)idx_image;
    (void)idx_chain;
    return (float)state->chain->gneb.spring_constant;
}

void Parameters_GNEB_Set_Spring_Force_Ratio( State * state, float ratio, int idx_chain ) noexcept
{
    (void)idx_chain;
    state->chain->gneb.spring_force_ratio = ratio;
    if( ratio != 0 )
        log_msg( state, 2, "Parameters_GNEB_Set_Spring_Force_Ratio: energy-weighted springs are not part of this engine" );
}

float Parameters_GNEB_Get_Spring_Force_Ratio( State * state, int idx_chain ) noexcept
{
    (void)idx_chain;
    return (float)state->chain->gneb.spring_force_ratio;
}

void Parameters_GNEB_Set_Path_Shortening_Constant( State * state, float c, int idx_chain ) noexcept
{
    (void)idx_chain;
    state->chain->gneb.path_shortening_constant = c;
    if( c != 0 )
        log_msg( state, 2, "Parameters_GNEB_Set_Path_Shortening_Constant: path shortening is not part of this engine" );
}

float Parameters_GNEB_Get_Path_Shortening_Constant( State * state, int idx_chain ) noexcept
{
    (void)idx_chain;
    return (float)state->chain->gneb.path_shortening_constant;
}

void Parameters_GNEB_Set_Climbing_Falling( State * state, int image_type, int idx_image, int idx_chain ) noexcept
{
    try
    {
        from_indices( state, idx_image, idx_chain ).img->gneb_type = image_type;
    }
    catch( ... )
    {
        handle( state, "Parameters_GNEB_Set_Climbing_Falling" );
    }
}

int Parameters_GNEB_Get_Climbing_Falling( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->gneb_type;
    }
    catch( ... )
    {
        handle( state, "Parameters_GNEB_Get_Climbing_Falling" );
        return 0;
    }
}

// Parameters_GNEB_Set_Image_Type_Automatically (core/src/Spirit/Parameters_GNEB.cpp:338-363)
void Parameters_GNEB_Set_Image_Type_Automatically( State * state, int idx_chain ) noexcept
{
    (void)idx_chain;
    auto & imgs = state->chain->images;
    for( size_t i = 1; i + 1 < imgs.size(); ++i )
    {
        double E0 = imgs[i - 1]->E, E1 = imgs[i]->E, E2 = imgs[i + 1]->E;
        if( E0 < E1 && E1 > E2 )
            imgs[i]->gneb_type = 1;
        else if( E0 > E1 && E1 < E2 )
            imgs[i]->gneb_type = 2;
        else if( imgs[i]->gneb_type != 3 )
            imgs[i]->gneb_type = 0;
    }
}

void Parameters_GNEB_Set_N_Energy_Interpolations( State * state, int n, int idx_chain ) noexcept
{
    (void)idx_chain;
    state->chain->gneb.n_E_interpolations = n;
}

int Parameters_GNEB_Get_N_Energy_Interpolations( State * state, int idx_chain ) noexcept
{
    (void)idx_chain;
    return state->chain->gneb.n_E_interpolations;
}

void Parameters_GNEB_Set_Moving_Endpoints( State * state, bool moving, int idx_chain ) noexcept
{
    (void)idx_chain;
    state->chain->gneb.moving_endpoints = moving;
    if( moving )
        log_msg( state, 2, "Parameters_GNEB_Set_Moving_Endpoints: moving endpoints are not part of this engine" );
}

// ============================================================== Simulation (core/include/Spirit/Simulation.h)
void free_run_info( Simulation_Run_Info info ) noexcept
{
    delete[] info.history_iteration;
    delete[] info.history_max_torque;
    delete[] info.history_energy;
}

// Simulation_LLG_Start (core/src/Spirit/Simulation.cpp:134-217)
// Simulation_MC_Start (core/src/Spirit/Simulation.cpp:77-132)
void Simulation_MC_Start( State * state, int n_iterations, int n_iterations_log, bool singleshot,
                          Simulation_Run_Info * info, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I     = from_indices( state, idx_image, idx_chain );
        auto & img = *I.img;
        std::lock_guard<std::recursive_mutex> lk( img.mtx );
        if( img.iteration_allowed || I.chain->iteration_allowed )
        {
            log_msg( state, 2, "Tried to use Simulation_Start on an image, but there is already a simulation running." );
            return;
        }
        if( n_iterations > 0 )
            img.mc.n_iterations = n_iterations;
        if( n_iterations_log > 0 )
            img.mc.n_iterations_log = n_iterations_log;
        img.iteration_allowed  = true;
        img.singleshot_allowed = singleshot;
        img.info               = MethodInfo{};
        img.info.method        = "MC";
        img.info.solver        = "None";
        img.info.solver_id     = -1;
        img.info.n_iterations  = (int)img.mc.n_iterations;
        img.info.t_start       = std::chrono::steady_clock::now();
        MCImageRun & R         = mc_image_run( state, img );
        R.eng->set_spins( 0, img.spins.data() );
        R.mc->start( { mc_settings_of( img ) } );
        if( singleshot )
            return;
        iterate_mc( img, R );
        img.iteration_allowed = false;
        fill_run_info( info, img.info );
    }
    catch( ... )
    {
        handle( state, "Simulation_MC_Start" );
    }
}

void Simulation_LLG_Start( State * state, int solver_type, int n_iterations, int n_iterations_log, bool singleshot,
                           Simulation_Run_Info * info, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        auto & img = *I.img;
        std::lock_guard<std::recursive_mutex> lk( img.mtx );
        if( img.iteration_allowed || I.chain->iteration_allowed )
        {
            log_msg( state, 2, "Tried to use Simulation_Start on an image, but there is already a simulation running." );
            return;
        }
        if( solver_type != SOLVER_SIB && solver_type != SOLVER_HEUN && solver_type != SOLVER_DEPONDT
            && solver_type != SOLVER_RK4 && solver_type != SOLVER_VP && solver_type != SOLVER_VP_OSO
            && solver_type != SOLVER_LBFGS_OSO )
        {
            log_msg( state, 2, "Invalid solver_type " + std::to_string( solver_type ) );
            return;
        }
        if( n_iterations > 0 )
            img.llg.n_iterations = n_iterations;
        if( n_iterations_log > 0 )
            img.llg.n_iterations_log = n_iterations_log;
        img.iteration_allowed  = true;
        img.singleshot_allowed = singleshot;
        img.info               = MethodInfo{};
        img.info.method        = "LLG";
        img.info.solver        = solver_name( solver_type );
        img.info.solver_id     = solver_type;
        img.info.n_iterations  = (int)img.llg.n_iterations;
        img.info.t_start       = std::chrono::steady_clock::now();
        if( solver_type == SOLVER_VP || solver_type == SOLVER_VP_OSO || solver_type == SOLVER_LBFGS_OSO )
        {
            // direct minimisers on a single image: the chain-global projection / L-BFGS memory over
            // one image (Solver_VP.hpp:28-114, Solver_VP_OSO.hpp, Solver_LBFGS_OSO.hpp)
            llg_vp_run( state, img, solver_type, singleshot );
            if( !singleshot )
                fill_run_info( info, img.info );
            return;
        }
        Engine & E = run_engine( state, img );
        E.set_spins( 0, img.spins.data() );
        E.set_params( 0, input_of( img, 0 ) );
        E.llg_start( solver_type, { (int)img.llg.n_iterations } );
        if( singleshot )
        {
            // the start evaluated the field and energy of the current spins (the method's first
            // force evaluation): that is the image's energy until the first shot
            img.E = E.status()[0].energy;
            return;
        }
        iterate_llg( state, img, E );
        img.iteration_allowed = false;
        fill_run_info( info, img.info );
    }
    catch( ... )
    {
        try
        {
            auto I                    = from_indices( state, idx_image, idx_chain );
            I.img->iteration_allowed = false;
        }
        catch( ... )
        {
        }
        handle( state, "Simulation_LLG_Start" );
    }
}

// Simulation_N_Shot (core/src/Spirit/Simulation.cpp:454-540)
void Simulation_N_Shot( State * state, int N, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        auto & img = *I.img;
        if( I.chain->iteration_allowed && I.chain->singleshot_allowed )
        {
            gneb_n_shot( state, *I.chain, N );
            return;
        }
        if( !( img.iteration_allowed && img.singleshot_allowed ) )
        {
            log_msg( state, 2, "Tried to use Simulation_SingleShot but no SingleShot simulation has been started." );
            return;
        }
        if( img.info.method == "MC" )
        {
            MCImageRun & R = mc_image_run( state, img );
            R.eng->set_spins( 0, img.spins.data() );
            R.mc->launch( N );
            finish_mc( img, R );
            if( img.info.iteration >= img.mc.n_iterations || stop_file_present() )
            {
                img.iteration_allowed  = false;
                img.singleshot_allowed = false;
            }
            return;
        }
        if( img.info.solver_id == SOLVER_VP || img.info.solver_id == SOLVER_VP_OSO
            || img.info.solver_id == SOLVER_LBFGS_OSO )
        {
            llg_vp_shot( state, img, N );
            return;
        }
        Engine & E = *img.run;
        // the host spin buffer is the state: callers may have written into it since the last call.
        // Upload, steps and read-back are enqueued together with one synchronisation at the end
        // (steps of a converged or finished run are no-ops on the device).  The buffer is
        // page-locked on first use (direct DMA both ways).
        img.spin_pin.ensure( img.spins.data(), img.spins.size() * sizeof( double ) );
        E.set_spins( 0, img.spins.data(), false );
        E.llg_launch( N );
        const Engine::Status s = finish_llg( img, E );
        if( !s.active || stop_file_present() )
        {
            img.iteration_allowed  = false;
            img.singleshot_allowed = false;
        }
    }
    catch( ... )
    {
        handle( state, "Simulation_N_Shot" );
    }
}

void Simulation_SingleShot( State * state, int idx_image, int idx_chain ) noexcept
{
    Simulation_N_Shot( state, 1, idx_image, idx_chain );
}

void Simulation_Stop( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( I.img->iteration_allowed )
        {
            I.img->iteration_allowed  = false;
            I.img->singleshot_allowed = false;
        }
        else if( I.chain->iteration_allowed )
        {
            I.chain->iteration_allowed  = false;
            I.chain->singleshot_allowed = false;
        }
    }
    catch( ... )
    {
        handle( state, "Simulation_Stop" );
    }
}

void Simulation_Stop_All( State * state ) noexcept
{
    try
    {
        state->chain->iteration_allowed  = false;
        state->chain->singleshot_allowed = false;
        for( auto & img : state->chain->images )
        {
            img->iteration_allowed  = false;
            img->singleshot_allowed = false;
        }
    }
    catch( ... )
    {
        handle( state, "Simulation_Stop_All" );
    }
}

static const MethodInfo & info_of( State * state, int idx_image, int idx_chain )
{
    auto I = from_indices( state, idx_image, idx_chain );
    if( I.chain->info.method == "GNEB" && ( I.chain->iteration_allowed || I.img->info.method == "None" ) )
        return I.chain->info;
    return I.img->info;
}

float Simulation_Get_MaxTorqueNorm( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return info_of( state, idx_image, idx_chain ).max_torque;
    }
    catch( ... )
    {
        return 0;
    }
}

float Simulation_Get_MaxTorqueComponent( State * state, int idx_image, int idx_chain ) noexcept
{
    return Simulation_Get_MaxTorqueNorm( state, idx_image, idx_chain );
}

void Simulation_Get_Chain_MaxTorqueNorms( State * state, float * torques, int idx_chain ) noexcept
{
    (void)idx_chain;
    auto & ch = *state->chain;
    for( size_t i = 0; i < ch.images.size(); ++i )
        torques[i] = i < gneb_torques( ch ).size() ? (float)gneb_torques( ch )[i] : 0.f;
}

float Simulation_Get_IterationsPerSecond( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (float)info_of( state, idx_image, idx_chain ).ips;
    }
    catch( ... )
    {
        return 0;
    }
}

int Simulation_Get_Iteration( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return info_of( state, idx_image, idx_chain ).iteration;
    }
    catch( ... )
    {
        return 0;
    }
}

float Simulation_Get_Time( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (float)info_of( state, idx_image, idx_chain ).time_ps;
    }
    catch( ... )
    {
        return 0;
    }
}

int Simulation_Get_Wall_Time( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (int)info_of( state, idx_image, idx_chain ).wall_ms;
    }
    catch( ... )
    {
        return 0;
    }
}

const char * Simulation_Get_Solver_Name( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return info_of( state, idx_image, idx_chain ).solver.c_str();
    }
    catch( ... )
    {
        return "";
    }
}

const char * Simulation_Get_Method_Name( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return info_of( state, idx_image, idx_chain ).method.c_str();
    }
    catch( ... )
    {
        return "";
    }
}

bool Simulation_Running_On_Image( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->iteration_allowed.load();
    }
    catch( ... )
    {
        return false;
    }
}

bool Simulation_Running_On_Chain( State * state, int idx_chain ) noexcept
{
    (void)idx_chain;
    return state && state->chain && state->chain->iteration_allowed.load();
}

bool Simulation_Running_Anywhere_On_Chain( State * state, int idx_chain ) noexcept
{
    if( Simulation_Running_On_Chain( state, idx_chain ) )
        return true;
    for( auto & img : state->chain->images )
        if( img->iteration_allowed )
            return true;
    return false;
}

// Simulation_GNEB_Start (core/src/Spirit/Simulation.cpp:219-315)
void Simulation_GNEB_Start( State * state, int solver_type, int n_iterations, int n_iterations_log, bool singleshot,
                            Simulation_Run_Info * info, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, -1, idx_chain );
        if( I.chain->iteration_allowed || I.img->iteration_allowed )
        {
            log_msg( state, 2, "Tried to use Simulation_Start on the chain, but there is already a simulation running." );
            return;
        }
        if( Simulation_Running_Anywhere_On_Chain( state, idx_chain ) )
        {
            log_msg( state, 1, "There are still one or more simulations running on the specified chain!" );
            return;
        }
        if( I.chain->images.size() < 2 )
        {
            log_msg( state, 1, "There are less than 2 images in the specified chain!" );
            return;
        }
        if( solver_type != SOLVER_VP && solver_type != SOLVER_VP_OSO && solver_type != SOLVER_LBFGS_OSO )
        {
            log_msg( state, 2,
                     "Simulation_GNEB_Start: this engine runs GNEB with the VP, VP_OSO and LBFGS_OSO solvers" );
            return;
        }
        if( n_iterations > 0 )
            I.chain->gneb.n_iterations = n_iterations;
        if( n_iterations_log > 0 )
            I.chain->gneb.n_iterations_log = n_iterations_log;
        gneb_start( state, *I.chain, solver_type, singleshot );
        if( !singleshot )
            fill_run_info( info, I.chain->info );
    }
    catch( ... )
    {
        try
        {
            state->chain->iteration_allowed = false;
        }
        catch( ... )
        {
        }
        handle( state, "Simulation_GNEB_Start" );
    }
}

// ---- extensions
// Run the device work of this State on the caller's CUDA stream (nullptr: the engine's own).
void Simulation_Set_Stream( State * state, void * stream ) noexcept
{
    try
    {
        state->stream = stream;
        for( auto & img : state->chain->images )
            if( img->run )
                img->run->set_stream( (cudaStream_t)stream );
    }
    catch( ... )
    {
        handle( state, "Simulation_Set_Stream" );
    }
}

// Launch n steps of a started single-shot LLG run without host transfers or synchronisation
// (for pipelined callers and device-side timing); Simulation_SingleShot/N_Shot or
// System_Update_Spins_From_Device bring the spins back.
void Simulation_Launch_Steps( State * state, int n, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( !( I.img->iteration_allowed && I.img->singleshot_allowed ) || !I.img->run )
        {
            log_msg( state, 2, "Simulation_Launch_Steps needs a started single-shot LLG simulation" );
            return;
        }
        I.img->run->llg_launch( n );
    }
    catch( ... )
    {
        handle( state, "Simulation_Launch_Steps" );
    }
}

// Wait for the device work of the image and copy its spins into the host buffer.
void System_Update_Spins_From_Device( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( I.img->run )
        {
            I.img->run->sync();
            finish_llg( *I.img, *I.img->run );
        }
    }
    catch( ... )
    {
        handle( state, "System_Update_Spins_From_Device" );
    }
}

// Per-kernel device time of n steps of the started single-shot LLG run (CUDA events between the
// launches on the engine stream); ms[] and count[] have KERNEL_ID slots (stage, FFT passes A, B,
// C, B', A').  Before every step flush_buf is overwritten and read_buf read (L2 flush that leaves
// clean lines); both may be null.
void Simulation_Profile_Steps( State * state, int n, void * flush_buf, long long flush_bytes, void * read_buf,
                               long long read_bytes, double * ms, int * count, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        if( !I.img->run )
            return;
        I.img->run->profile_steps( n, flush_buf, (size_t)flush_bytes, read_buf, (size_t)read_bytes, ms, count );
    }
    catch( ... )
    {
        handle( state, "Simulation_Profile_Steps" );
    }
}

// Device kernels launched per step of the image's current LLG method.
int Simulation_Get_Kernels_Per_Step( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        return I.img->run ? I.img->run->kernels_per_step() : 0;
    }
    catch( ... )
    {
        return 0;
    }
}

// Tuned launch parameters of the image's LLG engine (see include/Spirit_gb300.h); returns how many
// values the engine reports (0 before a start).
int Simulation_Get_Tuning( State * state, int * values, int n, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        return I.img->run && values ? I.img->run->tuning( values, n ) : 0;
    }
    catch( ... )
    {
        return 0;
    }
}

void Simulation_Set_Precision( State * state, int bits ) noexcept
{
    if( bits == 32 || bits == 64 )
        state->precision = bits;
}

int Simulation_Get_Precision( State * state ) noexcept
{
    return state->precision;
}

// Batched LLG: every State's active image advances in one batched device launch sequence
// (no counterpart in the reference, which runs one image per method: Method_LLG.cpp:25-26).
// All states must use the same solver; each keeps its own geometry, Hamiltonian and LLG
// parameters.  The thermal-noise stream of state k is k (Philox counter), so replicas with the
// same seed draw independent noise.
void Simulation_LLG_Start_Batched( State ** states, int n_states, int solver_type, int n_iterations,
                                   Simulation_Run_Info * info ) noexcept
{
    State * first = n_states > 0 ? states[0] : nullptr;
    try
    {
        llg_run_batched( states, n_states, solver_type, n_iterations, info ? (void *)info : nullptr,
                         sizeof( Simulation_Run_Info ) );
        for( int k = 0; info && k < n_states; ++k )
            fill_run_info( info + k, states[k]->chain->images[states[k]->idx_active_image]->info );
    }
    catch( ... )
    {
        handle( first, "Simulation_LLG_Start_Batched" );
    }
}

// Enqueue n_steps of an open-ended batched LLG run of the States' active images on states[0]'s
// stream, without transfers or synchronisation (the first call uploads the spins and starts the
// batch).  Simulation_LLG_Batched_Finish brings the spins back and ends the run.
void Simulation_LLG_Batched_Launch_Steps( State ** states, int n_states, int solver_type, int n_steps ) noexcept
{
    State * first = n_states > 0 ? states[0] : nullptr;
    try
    {
        llg_batched_launch( states, n_states, solver_type, n_steps );
    }
    catch( ... )
    {
        handle( first, "Simulation_LLG_Batched_Launch_Steps" );
    }
}

void Simulation_LLG_Batched_Finish( State ** states, int n_states ) noexcept
{
    State * first = n_states > 0 ? states[0] : nullptr;
    try
    {
        llg_batched_finish( states, n_states );
    }
    catch( ... )
    {
        handle( first, "Simulation_LLG_Batched_Finish" );
    }
}

// ---------------------------------------------------------------- adjoint (no reference counterpart)

// Adjoint of a T = 0 RK4 LLG trajectory of the image: n_steps from the image's spins with the
// parameters params = (J, D, K [meV], B [T], alpha) replacing the configured first-shell exchange,
// first-shell DMI, anisotropy and field magnitudes (all shells / basis atoms scaled with them; the
// field direction stays) and the damping (params NULL: the configured values).  Returns the loss
// mean_i |s_i(T) - target_i|^2 (FP64); grad_s0 (AoS [nos][3]) and grad_params[5] receive its
// gradient; final_spins (optional) s(T).  checkpoint: steps between stored states.
double Simulation_LLG_Adjoint( State * state, const double * params, int n_steps, int checkpoint,
                               const double * target, double * grad_s0, double * grad_params, double * final_spins,
                               int idx_image, int idx_chain ) noexcept
{
    try
    {
        return run_adjoint( state, params, n_steps, checkpoint, target, grad_s0, grad_params, final_spins, idx_image,
                            idx_chain, true );
    }
    catch( ... )
    {
        handle( state, "Simulation_LLG_Adjoint" );
        return 0;
    }
}

// The loss of the same trajectory without gradients (finite differences, forward timing).
double Simulation_LLG_Loss( State * state, const double * params, int n_steps, const double * target,
                            double * final_spins, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return run_adjoint( state, params, n_steps, 1 << 30, target, nullptr, nullptr, final_spins, idx_image,
                            idx_chain, false );
    }
    catch( ... )
    {
        handle( state, "Simulation_LLG_Loss" );
        return 0;
    }
}

// ============================================================== HTST (core/include/Spirit/HTST.h)
static std::vector<double> fp64_gradient( Image & img )
{
    std::vector<double> g( 3 * (size_t)img.nos() );
    Engine & E = eval_engine( img );
    E.set_spins( 0, img.spins.data() );
    double Et = 0;
    E.gradient( 0, g.data(), &Et, nullptr );
    return g;
}

float HTST_Calculate( State * state, int idx_image_minimum, int idx_image_sp, int n_eigenmodes_keep, bool sparse,
                      int idx_chain ) noexcept
{
    try
    {
        auto Im = from_indices( state, idx_image_minimum, idx_chain );
        auto Is = from_indices( state, idx_image_sp, idx_chain );
        std::lock_guard<std::recursive_mutex> lk( Im.chain->mtx );
        Im.chain->htst.reset();
        auto gm = fp64_gradient( *Im.img );
        auto gs = fp64_gradient( *Is.img );
        cudaStream_t st;
        CUDA_CHECK( cudaStreamCreateWithFlags( &st, cudaStreamNonBlocking ) );
        std::shared_ptr<HtstResult> R;
        try
        {
            R = std::make_shared<HtstResult>( htst_calculate( *Im.img->geom, Im.img->ham, Im.img->spins, gm,
                                                              Is.img->ham, Is.img->spins, gs, sparse,
                                                              n_eigenmodes_keep, st ) );
        }
        catch( ... )
        {
            cudaStreamDestroy( st );
            throw;
        }
        CUDA_CHECK( cudaStreamDestroy( st ) );
        static const char * why[] = { "",
                                      "HTST: the initial configuration is not a converged minimum, its max. torque "
                                      "is above the threshold (1e-8)!",
                                      "HTST: the transition configuration is not a converged saddle point, its max. "
                                      "torque is above the threshold (1e-8)!",
                                      "HTST: the transition configuration is not a saddle point, its lowest "
                                      "eigenvalue is above the threshold (-1e-4)!",
                                      "HTST: the image you passed is a higher order saddle point!",
                                      "HTST: the initial configuration is not a minimum, its lowest eigenvalue is "
                                      "below the threshold (-1e-4)!" };
        if( R->status > 0 && R->status < 6 )
            log_msg( state, 1, why[R->status] );
        Im.chain->htst = R;
        return (float)R->prefactor;
    }
    catch( ... )
    {
        handle( state, "HTST_Calculate" );
        return 0;
    }
}

static std::shared_ptr<HtstResult> htst_of( State * state, int idx_chain, const char * who, bool eigen )
{
    auto I = from_indices( state, -1, idx_chain );
    auto R = std::static_pointer_cast<HtstResult>( I.chain->htst );
    if( !R )
        throw std::runtime_error( std::string( who ) + ": HTST_Calculate has not been called" );
    if( eigen && R->sparse )
    {
        log_msg( state, 1,
                 std::string( who )
                     + ": You tried to call this function after performing a sparse calculation. This is not allowed." );
        return nullptr;
    }
    return R;
}

void HTST_Get_Info( State * state, float * temperature_exponent, float * me, float * Omega_0, float * s,
                    float * volume_min, float * volume_sp, float * prefactor_dynamical, float * prefactor,
                    int * n_eigenmodes_keep, int idx_chain ) noexcept
{
    try
    {
        auto R = htst_of( state, idx_chain, "HTST_Get_Info", false );
        auto put = []( float * p, double v ) {
            if( p )
                *p = (float)v;
        };
        put( temperature_exponent, R->temperature_exponent );
        put( me, R->me );
        put( Omega_0, R->Omega_0 );
        put( s, R->s );
        put( volume_min, R->volume_min );
        put( volume_sp, R->volume_sp );
        put( prefactor_dynamical, R->prefactor_dynamical );
        put( prefactor, R->prefactor );
        if( n_eigenmodes_keep )
            *n_eigenmodes_keep = R->n_keep;
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Info" );
    }
}

static void htst_copy( State * state, float * out, int idx_chain, const char * who, int which )
{
    auto R = htst_of( state, idx_chain, who, true );
    if( !R )
        return;
    if( !out )
    {
        log_msg( state, 1, std::string( who ) + ": you passed a null pointer" );
        return;
    }
    const std::vector<double> & v = which == 0 ? R->evalues_min
                                  : which == 1 ? R->evectors_min
                                  : which == 2 ? R->evalues_sp
                                  : which == 3 ? R->evectors_sp
                                               : R->velocities;
    for( size_t i = 0; i < v.size(); ++i )
        out[i] = (float)v[i];
}

void HTST_Get_Eigenvalues_Min( State * state, float * eigenvalues_min, int idx_chain ) noexcept
{
    try
    {
        htst_copy( state, eigenvalues_min, idx_chain, "HTST_Get_Eigenvalues_Min", 0 );
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Eigenvalues_Min" );
    }
}

void HTST_Get_Eigenvectors_Min( State * state, float * eigenvectors_min, int idx_chain ) noexcept
{
    try
    {
        htst_copy( state, eigenvectors_min, idx_chain, "HTST_Get_Eigenvectors_Min", 1 );
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Eigenvectors_Min" );
    }
}

void HTST_Get_Eigenvalues_SP( State * state, float * eigenvalues_sp, int idx_chain ) noexcept
{
    try
    {
        htst_copy( state, eigenvalues_sp, idx_chain, "HTST_Get_Eigenvalues_SP", 2 );
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Eigenvalues_SP" );
    }
}

void HTST_Get_Eigenvectors_SP( State * state, float * eigenvectors_sp, int idx_chain ) noexcept
{
    try
    {
        htst_copy( state, eigenvectors_sp, idx_chain, "HTST_Get_Eigenvectors_SP", 3 );
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Eigenvectors_SP" );
    }
}

void HTST_Get_Velocities( State * state, float * velocities, int idx_chain ) noexcept
{
    try
    {
        htst_copy( state, velocities, idx_chain, "HTST_Get_Velocities", 4 );
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Velocities" );
    }
}

// FP64 copy of the last result: info[10] = temperature_exponent, me, Omega_0, s, volume_min,
// volume_sp, prefactor_dynamical, prefactor, det_min, det_sp; spectra / eigenvectors [n_keep][2N] /
// velocities as the float getters (NULL pointers skipped).  Returns the status (0 done, 1-5 the
// check that stopped the calculation, -1 none).
int HTST_Get_Result_FP64( State * state, double * info, double * eigenvalues_min, double * eigenvalues_sp,
                          double * eigenvectors_min, double * eigenvectors_sp, double * velocities,
                          int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, -1, idx_chain );
        auto R = std::static_pointer_cast<HtstResult>( I.chain->htst );
        if( !R )
            return -1;
        if( info )
        {
            const double v[10] = { R->temperature_exponent, R->me, R->Omega_0, R->s, R->volume_min, R->volume_sp,
                                   R->prefactor_dynamical, R->prefactor, R->det_min, R->det_sp };
            std::memcpy( info, v, sizeof( v ) );
        }
        auto cp = []( double * o, const std::vector<double> & v ) {
            if( o && !v.empty() )
                std::memcpy( o, v.data(), v.size() * sizeof( double ) );
        };
        cp( eigenvalues_min, R->evalues_min );
        cp( eigenvalues_sp, R->evalues_sp );
        cp( eigenvectors_min, R->evectors_min );
        cp( eigenvectors_sp, R->evectors_sp );
        cp( velocities, R->velocities );
        return R->status;
    }
    catch( ... )
    {
        handle( state, "HTST_Get_Result_FP64" );
        return -1;
    }
}

// ============================================================== IO (core/include/Spirit/IO.h)
int IO_N_Images_In_File( State * state, const char * file, int idx_image, int idx_chain ) noexcept
{
    (void)idx_image;
    (void)idx_chain;
    try
    {
        return ovf_count( file ? file : "" );
    }
    catch( ... )
    {
        handle( state, "IO_N_Images_In_File" );
        return 0;
    }
}

void IO_Image_Read( State * state, const char * file, int idx_image_infile, int idx_image_inchain,
                    int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image_inchain, idx_chain );
        std::lock_guard<std::recursive_mutex> lk( I.img->mtx );
        read_image( *I.img, ovf_read( file ? file : "", idx_image_infile ) );
    }
    catch( ... )
    {
        handle( state, "IO_Image_Read" );
    }
}

static void write_image( State * state, const char * file, int format, const char * comment, int idx_image,
                         int idx_chain, bool append )
{
    auto I = from_indices( state, idx_image, idx_chain );
    if( format < 0 || format > 4 )
        throw std::runtime_error( "Invalid file format index " + std::to_string( format ) );
    ovf_write( file ? file : "", image_segment( *I.img, I.img->spins, comment ), format, append );
}

void IO_Image_Write( State * state, const char * file, int format, const char * comment, int idx_image,
                     int idx_chain ) noexcept
{
    try
    {
        write_image( state, file, format, comment, idx_image, idx_chain, false );
    }
    catch( ... )
    {
        handle( state, "IO_Image_Write" );
    }
}

void IO_Image_Append( State * state, const char * file, int format, const char * comment, int idx_image,
                      int idx_chain ) noexcept
{
    try
    {
        write_image( state, file, format, comment, idx_image, idx_chain, true );
    }
    catch( ... )
    {
        handle( state, "IO_Image_Append" );
    }
}

void IO_Positions_Write( State * state, const char * file, int format, const char * comment, int idx_image,
                         int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto seg = image_segment( *I.img, I.img->positions, comment );
        seg.valuelabels = "position_x position_y position_z";
        seg.valueunits  = "Angstrom Angstrom Angstrom";
        ovf_write( file ? file : "", seg, format, false );
    }
    catch( ... )
    {
        handle( state, "IO_Positions_Write" );
    }
}

// IO_Chain_Read (core/src/Spirit/IO.cpp): segments [start, end] of the file into images
// insert_idx, insert_idx + 1, ... of the chain, appending images where the chain is too short
void IO_Chain_Read( State * state, const char * file, int start_image_infile, int end_image_infile, int insert_idx,
                    int idx_chain ) noexcept
{
    try
    {
        auto I         = from_indices( state, -1, idx_chain );
        auto & ch      = *I.chain;
        std::lock_guard<std::recursive_mutex> lk( ch.mtx );
        const int nseg = ovf_count( file ? file : "" );
        if( nseg == 0 )
            throw std::runtime_error( std::string( "no OVF segments in \"" ) + ( file ? file : "" ) + "\"" );
        if( insert_idx < 0 )
            insert_idx = state->idx_active_image;
        if( end_image_infile < 0 || end_image_infile >= nseg )
            end_image_infile = nseg - 1;
        for( int k = start_image_infile; k <= end_image_infile; ++k )
        {
            const int dst = insert_idx + ( k - start_image_infile );
            while( (int)ch.images.size() <= dst )
            {
                auto img  = clone_image( *ch.images.back() );
                img->geom = ch.images[0]->geom;
                ch.images.push_back( img );
            }
            read_image( *ch.images[dst], ovf_read( file, k ) );
        }
        ch.Rx.assign( ch.images.size(), 0.0 );
    }
    catch( ... )
    {
        handle( state, "IO_Chain_Read" );
    }
}

static void write_chain( State * state, const char * file, int format, const char * comment, int idx_chain,
                         bool append )
{
    auto I = from_indices( state, -1, idx_chain );
    if( format < 0 || format > 4 )
        throw std::runtime_error( "Invalid file format index " + std::to_string( format ) );
    bool first = !append;
    for( auto & img : I.chain->images )
    {
        ovf_write( file ? file : "", image_segment( *img, img->spins, comment ), format, !first );
        first = false;
    }
}

void IO_Chain_Write( State * state, const char * file, int format, const char * comment, int idx_chain ) noexcept
{
    try
    {
        write_chain( state, file, format, comment, idx_chain, false );
    }
    catch( ... )
    {
        handle( state, "IO_Chain_Write" );
    }
}

void IO_Chain_Append( State * state, const char * file, int format, const char * comment, int idx_chain ) noexcept
{
    try
    {
        write_chain( state, file, format, comment, idx_chain, true );
    }
    catch( ... )
    {
        handle( state, "IO_Chain_Append" );
    }
}

// ============================================================== Parameters_MC (core/include/Spirit/Parameters_MC.h)
#define MC_IMG( fn_name, body )                                                                                        \
    try                                                                                                                \
    {                                                                                                                  \
        auto I   = from_indices( state, idx_image, idx_chain );                                                        \
        auto & M = I.img->mc;                                                                                          \
        body;                                                                                                          \
    }                                                                                                                  \
    catch( ... )                                                                                                       \
    {                                                                                                                  \
        handle( state, fn_name );                                                                                      \
    }

void Parameters_MC_Set_Output_Tag( State * state, const char * tag, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Output_Tag", M.output_tag = tag ? tag : "" )
}
void Parameters_MC_Set_Output_Folder( State * state, const char * folder, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Output_Folder", M.output_folder = folder ? folder : "" )
}
void Parameters_MC_Set_Output_General( State * state, bool any, bool initial, bool final, int idx_image,
                                       int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Output_General", M.output_any = any; M.output_initial = initial; M.output_final = final )
}
void Parameters_MC_Set_Output_Energy( State * state, bool energy_step, bool energy_archive, bool energy_spin_resolved,
                                      bool energy_divide_by_nos, bool energy_add_readability_lines, int idx_image,
                                      int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Output_Energy", M.output_energy_step = energy_step;
            M.output_energy_archive = energy_archive; M.output_energy_spin_resolved = energy_spin_resolved;
            M.output_energy_divide_by_nspins = energy_divide_by_nos;
            M.output_energy_add_readability_lines = energy_add_readability_lines )
}
void Parameters_MC_Set_Output_Configuration( State * state, bool configuration_step, bool configuration_archive,
                                             int configuration_filetype, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Output_Configuration", M.output_configuration_step = configuration_step;
            M.output_configuration_archive = configuration_archive;
            M.output_configuration_filetype = configuration_filetype )
}
void Parameters_MC_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_image,
                                     int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_N_Iterations", M.n_iterations = n_iterations; M.n_iterations_log = n_iterations_log )
}
void Parameters_MC_Set_Temperature( State * state, float T, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Temperature", M.temperature = T )
}
void Parameters_MC_Set_Metropolis_Cone( State * state, bool cone, float cone_angle, bool adaptive_cone,
                                        float target_acceptance_ratio, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Metropolis_Cone", M.step_cone = cone; M.cone_angle = cone_angle;
            M.cone_adaptive = adaptive_cone; M.acceptance_target = target_acceptance_ratio )
}
void Parameters_MC_Set_Random_Sample( State * state, bool random_sample, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Set_Random_Sample", M.random_sample = random_sample )
}
const char * Parameters_MC_Get_Output_Tag( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->mc.output_tag.c_str();
    }
    catch( ... )
    {
        handle( state, "Parameters_MC_Get_Output_Tag" );
        return "";
    }
}
const char * Parameters_MC_Get_Output_Folder( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->mc.output_folder.c_str();
    }
    catch( ... )
    {
        handle( state, "Parameters_MC_Get_Output_Folder" );
        return "";
    }
}
void Parameters_MC_Get_Output_General( State * state, bool * any, bool * initial, bool * final, int idx_image,
                                       int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Get_Output_General", *any = M.output_any; *initial = M.output_initial;
            *final = M.output_final )
}
void Parameters_MC_Get_Output_Energy( State * state, bool * energy_step, bool * energy_archive,
                                      bool * energy_spin_resolved, bool * energy_divide_by_nos,
                                      bool * energy_add_readability_lines, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Get_Output_Energy", *energy_step = M.output_energy_step;
            *energy_archive = M.output_energy_archive; *energy_spin_resolved = M.output_energy_spin_resolved;
            *energy_divide_by_nos = M.output_energy_divide_by_nspins;
            *energy_add_readability_lines = M.output_energy_add_readability_lines )
}
void Parameters_MC_Get_Output_Configuration( State * state, bool * configuration_step, bool * configuration_archive,
                                             int * configuration_filetype, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Get_Output_Configuration", *configuration_step = M.output_configuration_step;
            *configuration_archive = M.output_configuration_archive;
            *configuration_filetype = M.output_configuration_filetype )
}
void Parameters_MC_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_image,
                                     int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Get_N_Iterations", *iterations = (int)M.n_iterations;
            *iterations_log = (int)M.n_iterations_log )
}
float Parameters_MC_Get_Temperature( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (float)from_indices( state, idx_image, idx_chain ).img->mc.temperature;
    }
    catch( ... )
    {
        handle( state, "Parameters_MC_Get_Temperature" );
        return 0;
    }
}
void Parameters_MC_Get_Metropolis_Cone( State * state, bool * cone, float * cone_angle, bool * adaptive_cone,
                                        float * target_acceptance_ratio, int idx_image, int idx_chain ) noexcept
{
    MC_IMG( "Parameters_MC_Get_Metropolis_Cone", *cone = M.step_cone; *cone_angle = (float)M.cone_angle;
            *adaptive_cone = M.cone_adaptive; *target_acceptance_ratio = (float)M.acceptance_target )
}
bool Parameters_MC_Get_Random_Sample( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->mc.random_sample;
    }
    catch( ... )
    {
        handle( state, "Parameters_MC_Get_Random_Sample" );
        return false;
    }
}
#undef MC_IMG

// ============================================================== System (core/include/Spirit/System.h)
int System_Get_Index( State * state ) noexcept
{
    return state ? state->idx_active_image : 0;
}

int System_Get_NOS( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->nos();
    }
    catch( ... )
    {
        handle( state, "System_Get_NOS" );
        return 0;
    }
}

double * System_Get_Spin_Directions( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->spins.data();
    }
    catch( ... )
    {
        handle( state, "System_Get_Spin_Directions" );
        return nullptr;
    }
}

double * System_Get_Effective_Field( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->eff_field.data();
    }
    catch( ... )
    {
        handle( state, "System_Get_Effective_Field" );
        return nullptr;
    }
}

float System_Get_Rx( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        return I.idx < (int)I.chain->Rx.size() ? (float)I.chain->Rx[I.idx] : 0.f;
    }
    catch( ... )
    {
        return 0;
    }
}

float System_Get_Energy( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return (float)from_indices( state, idx_image, idx_chain ).img->E;
    }
    catch( ... )
    {
        handle( state, "System_Get_Energy" );
        return 0;
    }
}

// FP64 energy of the image (Spin_System::E), extension of System_Get_Energy
double System_Get_Energy_FP64( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        return from_indices( state, idx_image, idx_chain ).img->E;
    }
    catch( ... )
    {
        handle( state, "System_Get_Energy_FP64" );
        return 0;
    }
}

static const char * term_names[N_TERMS] = { "Zeeman", "Anisotropy", "Exchange", "DMI", "DDI" };

static std::vector<int> active_terms( const Image & img )
{
    std::vector<int> t;
    auto & h = img.ham;
    if( std::abs( h.B * C_MU_B ) > 1e-60 )
        t.push_back( TERM_ZEEMAN );
    if( !h.aniso_idx.empty() )
        t.push_back( TERM_ANISOTROPY );
    if( !h.ex_pairs.empty() )
        t.push_back( TERM_EXCHANGE );
    if( !h.dmi_pairs.empty() )
        t.push_back( TERM_DMI );
    if( h.ddi_method != 0 )
        t.push_back( TERM_DDI );
    return t;
}

int System_Get_Energy_Array_Names( State * state, char * names, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I   = from_indices( state, idx_image, idx_chain );
        auto t   = active_terms( *I.img );
        std::string s;
        for( size_t k = 0; k < t.size(); ++k )
            s += std::string( k ? "|" : "" ) + term_names[t[k]];
        if( names )
            std::memcpy( names, s.c_str(), s.size() + 1 );
        return (int)s.size();
    }
    catch( ... )
    {
        handle( state, "System_Get_Energy_Array_Names" );
        return 0;
    }
}

int System_Get_Energy_Array( State * state, float * energies, bool divide_by_nspins, int idx_image,
                             int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        auto t = active_terms( *I.img );
        double terms[N_TERMS];
        Engine & E = eval_engine( *I.img );
        E.set_spins( 0, I.img->spins.data() );
        E.gradient( 0, nullptr, nullptr, terms );
        double div = divide_by_nspins ? I.img->nos() : 1.0;
        for( size_t k = 0; k < t.size(); ++k )
            energies[k] = (float)( terms[t[k]] / div );
        return (int)t.size();
    }
    catch( ... )
    {
        handle( state, "System_Get_Energy_Array" );
        return 0;
    }
}

void System_Print_Energy_Array( State * state, int idx_image, int idx_chain ) noexcept
{
    float e[N_TERMS];
    char names[256];
    int n = System_Get_Energy_Array( state, e, false, idx_image, idx_chain );
    System_Get_Energy_Array_Names( state, names, idx_image, idx_chain );
    std::printf( "Energy contributions: %s\n", names );
    for( int k = 0; k < n; ++k )
        std::printf( "  %g\n", e[k] );
}

// System_Update_Data: Spin_System::UpdateEnergy + UpdateEffectiveField (Spin_System.cpp:138-161)
void System_Update_Data( State * state, int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        update_data( *I.img );
    }
    catch( ... )
    {
        handle( state, "System_Update_Data" );
    }
}

// ============================================================== Quantities (core/include/Spirit/Quantities.h)
void Quantity_Get_Magnetization( State * state, float m[3], int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        double M[3] = { 0, 0, 0 };
        int n       = I.img->nos();
        for( int i = 0; i < n; ++i )
            for( int e = 0; e < 3; ++e )
                M[e] += I.img->spins[3 * i + e] * I.img->geom->mu_s( i );
        for( int e = 0; e < 3; ++e )
            m[e] = (float)( M[e] / n );
    }
    catch( ... )
    {
        handle( state, "Quantity_Get_Magnetization" );
    }
}

void Quantity_Get_Average_Spin( State * state, float s[3], int idx_image, int idx_chain ) noexcept
{
    try
    {
        auto I = from_indices( state, idx_image, idx_chain );
        double M[3] = { 0, 0, 0 };
        int n       = I.img->nos();
        for( int i = 0; i < n; ++i )
            for( int e = 0; e < 3; ++e )
                M[e] += I.img->spins[3 * i + e];
        for( int e = 0; e < 3; ++e )
            s[e] = (float)( M[e] / n );
    }
    catch( ... )
    {
        handle( state, "Quantity_Get_Average_Spin" );
    }
}

// ============================================================== Constants (core/include/Spirit/Constants.h)
double Constants_mu_B() noexcept
{
    return 0.057883817555;
}
double Constants_mu_0() noexcept
{
    return 2.0133545 * 1e-28;
}
double Constants_k_B() noexcept
{
    return 0.08617330350;
}
double Constants_hbar() noexcept
{
    return 0.6582119514;
}
double Constants_mRy() noexcept
{
    return 1.0 / 13.605693009;
}
double Constants_gamma() noexcept
{
    return 0.1760859644;
}
double Constants_g_e() noexcept
{
    return 2.00231930436182;
}
double Constants_Pi() noexcept
{
    return 3.141592653589793238462643383279502884197169399375105820974;
}

// ============================================================== Version / Log
const char * Spirit_Version() noexcept
{
    return "2.2.0";
}
const char * Spirit_Version_Full() noexcept
{
    return "2.2.0 (gb300)";
}
const char * Spirit_Scalar_Type() noexcept
{
    return "double";
}
const char * Spirit_Compiler_Full() noexcept
{
    return "nvcc sm_103a";
}
int Spirit_Cuda() noexcept
{
    return 1;
}

void Log_Send( State * state, int level, int sender, const char * message, int idx_image, int idx_chain ) noexcept
{
    (void)sender;
    (void)idx_image;
    (void)idx_chain;
    log_msg( state, level, message ? message : "" );
}

int Log_Get_N_Entries( State * state ) noexcept
{
    return state ? (int)state->log.size() : 0;
}

} // extern "C"
