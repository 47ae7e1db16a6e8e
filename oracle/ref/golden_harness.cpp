// Golden-vector harness for the reference (Spirit v2.2.0, CPU/OpenMP FP64, kissFFT).
//
// Test infrastructure only: links the reference library built by oracle/ref/Makefile
// and drives it exactly like the reference's own Catch tests do -- through its C API
// (State_Setup, Simulation_*_Start, System_Get_Spin_Directions, Chain_*) and, for the
// FP64 energies, through the Hamiltonian internals (core/test/test_physics.cpp:117-122).
// Input spins are injected through System_Get_Spin_Directions so the reference and the
// code under test see bit-identical states.
//
// Usage:
//   golden_harness pairs   <cfg> <out>                     neighbour/DMI pair lists
//   golden_harness grad    <cfg> <spins.bin> <out>         gradient, FP64 energy, per-term energies
//   golden_harness direct  <cfg> <spins.bin> <out>         same, after switching DDI to the direct sum
//   golden_harness llg     <cfg> <spins.bin> <out> <solver> <n_iter>
//   golden_harness ovfwrite <cfg> <spins.bin> <file> <format>   IO_Image_Write of the injected spins
//   golden_harness ovfread  <cfg> <file> <out.bin>               IO_Image_Read, then the spins it holds
//   golden_harness thermal <cfg> <spins.bin> <out> <llg|mc> <solver> <T> <n_equil> <n_samples> <stride>
//                                                        time series (E, m_x, m_y, m_z) every stride
//                                                        iterations after n_equil, at temperature T
//   golden_harness llgtime <cfg> <spins.bin> <solver> <n_iter>
//                                                        wall time of Simulation_LLG_Start only (stdout)
//   golden_harness gneb    <cfg> <chain.bin> <out> <noi> <solver> <n_iter> [<n_iter_ci>]
//   golden_harness htst    <cfg> <chain.bin> <out> <noi> <idx_min> <idx_sp> <sparse> <n_keep>
//                                                        HTST_Calculate on two images of a chain
//
// Binary files are little-endian float64 arrays; text outputs are whitespace separated.
#include <Spirit/Chain.h>
#include <Spirit/Configurations.h>
#include <Spirit/Geometry.h>
#include <Spirit/HTST.h>
#include <Spirit/IO.h>
#include <Spirit/Hamiltonian.h>
#include <Spirit/Parameters_GNEB.h>
#include <Spirit/Parameters_LLG.h>
#include <Spirit/Parameters_MC.h>
#include <Spirit/Simulation.h>
#include <Spirit/State.h>
#include <Spirit/System.h>
#include <data/State.hpp>
#include <engine/Hamiltonian_Heisenberg.hpp>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

static std::vector<double> read_bin( const char * path )
{
    FILE * f = std::fopen( path, "rb" );
    if( !f )
    {
        std::fprintf( stderr, "cannot open %s\n", path );
        std::exit( 2 );
    }
    std::fseek( f, 0, SEEK_END );
    long n = std::ftell( f ) / sizeof( double );
    std::fseek( f, 0, SEEK_SET );
    std::vector<double> v( n );
    if( std::fread( v.data(), sizeof( double ), n, f ) != (size_t)n )
        std::exit( 3 );
    std::fclose( f );
    return v;
}

static void write_bin( const std::string & path, const double * d, size_t n )
{
    FILE * f = std::fopen( path.c_str(), "wb" );
    std::fwrite( d, sizeof( double ), n, f );
    std::fclose( f );
}

static Engine::Hamiltonian_Heisenberg & heis( State * s )
{
    return *dynamic_cast<Engine::Hamiltonian_Heisenberg *>( s->active_image->hamiltonian.get() );
}

static void inject( State * s, const std::vector<double> & spins, int idx_image = -1 )
{
    double * d = System_Get_Spin_Directions( s, idx_image );
    int nos    = System_Get_NOS( s );
    if( (int)spins.size() < 3 * nos )
    {
        std::fprintf( stderr, "spin file too short\n" );
        std::exit( 4 );
    }
    std::memcpy( d, spins.data(), sizeof( double ) * 3 * nos );
}

static void dump_grad( State * s, const std::string & out )
{
    auto & ham   = heis( s );
    auto & spins = *s->active_image->spins;
    int nos      = s->nos;
    vectorfield g( nos ), g2( nos );
    scalar E = 0;
    ham.Gradient_and_Energy( spins, g, E );
    ham.Gradient( spins, g2 );
    write_bin( out + "_grad_and_energy_gradient.bin", g[0].data(), 3 * nos );
    write_bin( out + "_gradient.bin", g2[0].data(), 3 * nos );
    std::vector<std::pair<std::string, scalarfield>> contrib;
    ham.Energy_Contributions_per_Spin( spins, contrib );
    FILE * f = std::fopen( ( out + "_energy.txt" ).c_str(), "w" );
    std::fprintf( f, "grad_and_energy %.17g\n", E );
    std::fprintf( f, "total %.17g\n", ham.Energy( spins ) );
    for( auto & c : contrib )
    {
        double sum = 0;
        for( auto e : c.second )
            sum += e;
        std::string name = c.first;
        for( auto & ch : name )
            if( ch == ' ' )
                ch = '_';
        std::fprintf( f, "%s %.17g\n", name.c_str(), sum );
        write_bin( out + "_energy_" + name + ".bin", c.second.data(), nos );
    }
    std::fclose( f );
}

static void dump_pairs( State * s, const std::string & out )
{
    auto & ham = heis( s );
    FILE * f   = std::fopen( ( out + "_exchange.txt" ).c_str(), "w" );
    for( size_t p = 0; p < ham.exchange_pairs.size(); ++p )
    {
        auto & P = ham.exchange_pairs[p];
        std::fprintf(
            f, "%d %d %d %d %d %.17g\n", P.i, P.j, P.translations[0], P.translations[1], P.translations[2],
            ham.exchange_magnitudes[p] );
    }
    std::fclose( f );
    f = std::fopen( ( out + "_dmi.txt" ).c_str(), "w" );
    for( size_t p = 0; p < ham.dmi_pairs.size(); ++p )
    {
        auto & P = ham.dmi_pairs[p];
        auto & n = ham.dmi_normals[p];
        std::fprintf(
            f, "%d %d %d %d %d %.17g %.17g %.17g %.17g\n", P.i, P.j, P.translations[0], P.translations[1],
            P.translations[2], ham.dmi_magnitudes[p], n[0], n[1], n[2] );
    }
    std::fclose( f );
    auto & geo = *s->active_image->geometry;
    write_bin( out + "_positions.bin", geo.positions[0].data(), 3 * geo.nos );
}

int main( int argc, char ** argv )
{
    if( argc < 4 )
    {
        std::fprintf( stderr, "usage: see header\n" );
        return 1;
    }
    std::string op = argv[1];
    State * s      = State_Setup( argv[2], true );

    if( op == "pairs" )
    {
        dump_pairs( s, argv[3] );
    }
    else if( op == "grad" || op == "direct" )
    {
        inject( s, read_bin( argv[3] ) );
        if( op == "direct" )
        {
            int n_img[3] = { 4, 4, 4 };
            auto & ham   = heis( s );
            for( int i = 0; i < 3; ++i )
                n_img[i] = ham.ddi_n_periodic_images[i];
            Hamiltonian_Set_DDI( s, SPIRIT_DDI_METHOD_CUTOFF, n_img, -1 );
        }
        dump_grad( s, argv[4] );
    }
    else if( op == "llg" )
    {
        inject( s, read_bin( argv[3] ) );
        std::string out = argv[4];
        int solver      = std::atoi( argv[5] );
        int n_iter      = std::atoi( argv[6] );
        Simulation_LLG_Start( s, solver, n_iter, n_iter + 1 );
        int nos = System_Get_NOS( s );
        write_bin( out + "_spins.bin", System_Get_Spin_Directions( s ), 3 * nos );
        FILE * f = std::fopen( ( out + "_result.txt" ).c_str(), "w" );
        std::fprintf( f, "energy_image %.17g\n", (double)s->active_image->E );
        std::fprintf( f, "energy_float %.9g\n", (double)System_Get_Energy( s ) );
        auto method = s->method_image[s->idx_active_image];
        std::fprintf( f, "max_torque %.17g\n", (double)method->getTorqueMaxNorm() );
        std::fprintf( f, "iterations %d\n", method->getNIterations() );
        std::fclose( f );
        dump_grad( s, out + "_final" );
    }
    else if( op == "ovfwrite" )
    {
        inject( s, read_bin( argv[3] ) );
        IO_Image_Write( s, argv[4], std::atoi( argv[5] ), "written by the reference" );
    }
    else if( op == "ovfread" )
    {
        IO_Image_Read( s, argv[3] );
        write_bin( argv[4], System_Get_Spin_Directions( s ), 3 * (size_t)System_Get_NOS( s ) );
    }
    else if( op == "thermal" )
    {
        inject( s, read_bin( argv[3] ) );
        std::string out = argv[4];
        bool mc         = std::string( argv[5] ) == "mc";
        int solver      = std::atoi( argv[6] );
        float T         = (float)std::atof( argv[7] );
        int n_equil     = std::atoi( argv[8] );
        int n_samples   = std::atoi( argv[9] );
        int stride      = std::atoi( argv[10] );
        auto advance    = [&]( int n ) {
            if( n <= 0 )
                return;
            if( mc )
                Simulation_MC_Start( s, n, n + 1 );
            else
                Simulation_LLG_Start( s, solver, n, n + 1 );
        };
        if( mc )
            Parameters_MC_Set_Temperature( s, T );
        else
            Parameters_LLG_Set_Temperature( s, T );
        advance( n_equil );
        int nos = System_Get_NOS( s );
        std::vector<double> series;
        for( int k = 0; k < n_samples; ++k )
        {
            advance( stride );
            auto & spins = *s->active_image->spins;
            double m[3] = { 0, 0, 0 };
            for( int i = 0; i < nos; ++i )
                for( int e = 0; e < 3; ++e )
                    m[e] += spins[i][e];
            series.push_back( heis( s ).Energy( spins ) );
            for( int e = 0; e < 3; ++e )
                series.push_back( m[e] / nos );
        }
        write_bin( out + "_series.bin", series.data(), series.size() );
    }
    else if( op == "llgtime" )
    {
        inject( s, read_bin( argv[3] ) );
        int solver = std::atoi( argv[4] );
        int n_iter = std::atoi( argv[5] );
        auto t0    = std::chrono::steady_clock::now();
        Simulation_LLG_Start( s, solver, n_iter, n_iter + 1 );
        double dt = std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count();
        std::printf( "nos %d iterations %d seconds %.6f\n", System_Get_NOS( s ), n_iter, dt );
    }
    else if( op == "gneb" )
    {
        auto chain_in   = read_bin( argv[3] );
        std::string out = argv[4];
        int noi         = std::atoi( argv[5] );
        int solver      = std::atoi( argv[6] );
        int n_iter      = std::atoi( argv[7] );
        int n_iter_ci   = argc > 8 ? std::atoi( argv[8] ) : 0;
        Chain_Image_to_Clipboard( s );
        for( int i = 1; i < noi; ++i )
            Chain_Insert_Image_After( s );
        int nos = System_Get_NOS( s );
        for( int i = 0; i < noi; ++i )
        {
            double * d = System_Get_Spin_Directions( s, i );
            std::memcpy( d, chain_in.data() + (size_t)3 * nos * i, sizeof( double ) * 3 * nos );
        }
        Simulation_GNEB_Start( s, solver, n_iter, n_iter + 1 );
        if( n_iter_ci > 0 )
        {
            Parameters_GNEB_Set_Image_Type_Automatically( s );
            Simulation_GNEB_Start( s, solver, n_iter_ci, n_iter_ci + 1 );
        }
        std::vector<double> chain_out( (size_t)3 * nos * noi );
        for( int i = 0; i < noi; ++i )
            std::memcpy(
                chain_out.data() + (size_t)3 * nos * i, System_Get_Spin_Directions( s, i ),
                sizeof( double ) * 3 * nos );
        write_bin( out + "_chain.bin", chain_out.data(), chain_out.size() );
        FILE * f = std::fopen( ( out + "_result.txt" ).c_str(), "w" );
        for( int i = 0; i < noi; ++i )
            std::fprintf(
                f, "image %d E %.17g Rx %.17g type %d\n", i, (double)s->chain->images[i]->E,
                (double)s->chain->Rx[i], Parameters_GNEB_Get_Climbing_Falling( s, i ) );
        std::fprintf( f, "max_torque %.17g\n", (double)s->method_chain->getTorqueMaxNorm() );
        std::fprintf( f, "iterations %d\n", s->method_chain->getNIterations() );
        std::fclose( f );
    }
    else if( op == "htst" )
    {
        auto chain_in   = read_bin( argv[3] );
        std::string out = argv[4];
        int noi         = std::atoi( argv[5] );
        int idx_min     = std::atoi( argv[6] );
        int idx_sp      = std::atoi( argv[7] );
        bool sparse     = std::atoi( argv[8] ) != 0;
        int n_keep      = std::atoi( argv[9] );
        Chain_Image_to_Clipboard( s );
        for( int i = 1; i < noi; ++i )
            Chain_Insert_Image_After( s );
        int nos = System_Get_NOS( s );
        for( int i = 0; i < noi; ++i )
        {
            double * d = System_Get_Spin_Directions( s, i );
            std::memcpy( d, chain_in.data() + (size_t)3 * nos * i, sizeof( double ) * 3 * nos );
        }
        float pf    = HTST_Calculate( s, idx_min, idx_sp, n_keep, sparse );
        auto & info = s->chain->htst_info;
        FILE * f    = std::fopen( ( out + "_result.txt" ).c_str(), "w" );
        std::fprintf( f, "prefactor_float %.9g\n", (double)pf );
        std::fprintf( f, "temperature_exponent %.17g\n", (double)info.temperature_exponent );
        std::fprintf( f, "me %.17g\n", (double)info.me );
        std::fprintf( f, "Omega_0 %.17g\n", (double)info.Omega_0 );
        std::fprintf( f, "s %.17g\n", (double)info.s );
        std::fprintf( f, "volume_min %.17g\n", (double)info.volume_min );
        std::fprintf( f, "volume_sp %.17g\n", (double)info.volume_sp );
        std::fprintf( f, "prefactor_dynamical %.17g\n", (double)info.prefactor_dynamical );
        std::fprintf( f, "prefactor %.17g\n", (double)info.prefactor );
        std::fprintf( f, "det_min %.17g\n", (double)info.det_min );
        std::fprintf( f, "det_sp %.17g\n", (double)info.det_sp );
        std::fprintf( f, "n_eigenmodes_keep %d\n", info.n_eigenmodes_keep );
        std::fclose( f );
        if( !sparse )
        {
            write_bin( out + "_evalues_min.bin", info.eigenvalues_min.data(), info.eigenvalues_min.size() );
            write_bin( out + "_evalues_sp.bin", info.eigenvalues_sp.data(), info.eigenvalues_sp.size() );
            write_bin( out + "_evectors_min.bin", info.eigenvectors_min.data(), info.eigenvectors_min.size() );
            write_bin( out + "_evectors_sp.bin", info.eigenvectors_sp.data(), info.eigenvectors_sp.size() );
            write_bin(
                out + "_velocities.bin", info.perpendicular_velocity.data(), info.perpendicular_velocity.size() );
        }
    }
    State_Delete( s );
    return 0;
}
