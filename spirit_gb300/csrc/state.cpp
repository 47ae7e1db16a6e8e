#include "state.hpp"

#include "config.hpp"

#include <cmath>
#include <cstdio>
#include <sstream>

namespace sg
{

void log_msg( State * st, int level, const std::string & msg )
{
    if( !st )
    {
        std::fprintf( stderr, "[spirit_gb300] %s\n", msg.c_str() );
        return;
    }
    st->log.push_back( msg );
    if( st->log.size() > 10000 )
        st->log.erase( st->log.begin(), st->log.begin() + 5000 );
    // quiet mode keeps only errors (level <= 2) on the console, like the reference
    if( level <= ( st->quiet ? 2 : st->log_console_level ) )
        std::fprintf( stderr, "[spirit_gb300] %s\n", msg.c_str() );
}

static long parse_walltime( const std::string & s )
{
    int h = 0, m = 0, sec = 0;
    if( std::sscanf( s.c_str(), "%d:%d:%d", &h, &m, &sec ) == 3 )
        return 3600L * h + 60L * m + sec;
    return 0;
}

static Vec3 normalize_or( const Vec3 & v, const Vec3 & fallback )
{
    double n = std::sqrt( v[0] * v[0] + v[1] * v[1] + v[2] * v[2] );
    if( n < 1e-8 )
        return fallback;
    return { v[0] / n, v[1] / n, v[2] / n };
}

// Geometry_from_Config (core/src/io/Configparser.cpp:271-569), Hamiltonian_Heisenberg_from_Config
// (1256-1620), Parameters_Method_LLG_from_Config (701) and _GNEB_from_Config: the keywords the
// hot path uses, with the reference's defaults.
std::shared_ptr<Image> make_image_from_config( const std::string & path, State & st )
{
    auto img  = std::make_shared<Image>();
    auto geom = std::make_shared<Geometry>();
    ConfigFile cf;
    bool have = !path.empty() && cf.load( path );
    HamiltonianParams & h = img->ham;
    h.jij.clear();
    h.dij.clear();
    if( have )
    {
        // ---- geometry
        std::string lat;
        if( cf.get( "bravais_lattice", lat ) )
        {
            for( auto & c : lat )
                c = (char)std::tolower( c );
            bool ok;
            geom->bravais      = bravais_preset( lat, &ok );
            geom->bravais_name = ok ? lat : "sc";
        }
        else if( cf.find( "bravais_vectors" ) )
        {
            geom->bravais_name = "irregular";
            for( int k = 0; k < 3; ++k )
            {
                cf.next_line();
                double v[3] = { 0, 0, 0 };
                cf.read( v[0] );
                cf.read( v[1] );
                cf.read( v[2] );
                geom->bravais[k] = { v[0], v[1], v[2] };
            }
        }
        int nc[3];
        if( cf.get3( "n_basis_cells", nc ) )
            geom->n_cells = { nc[0], nc[1], nc[2] };
        if( cf.find( "basis" ) )
        {
            // the line after "basis" holds the number of atoms, then one line per atom
            int n = 0;
            if( cf.next_line() && cf.read( n ) && n > 0 )
            {
                geom->cell_atoms.clear();
                for( int a = 0; a < n; ++a )
                {
                    cf.next_line();
                    Vec3 p{ 0, 0, 0 };
                    cf.read( p[0] );
                    cf.read( p[1] );
                    cf.read( p[2] );
                    geom->cell_atoms.push_back( p );
                }
            }
        }
        cf.get( "lattice_constant", geom->lattice_constant );
        geom->mu_s_basis.assign( geom->nb(), 1.0 );
        if( cf.find( "mu_s" ) )
        {
            double first = 1.0;
            for( int a = 0; a < geom->nb(); ++a )
            {
                double v;
                if( cf.read( v ) )
                    geom->mu_s_basis[a] = v;
                else
                    geom->mu_s_basis[a] = first;
                if( a == 0 )
                    first = geom->mu_s_basis[0];
            }
        }
        // ---- Hamiltonian
        std::string htype = "heisenberg_neighbours";
        cf.get( "hamiltonian", htype );
        int bc[3] = { 0, 0, 0 };
        if( cf.get3( "boundary_conditions", bc ) )
            h.bc = { bc[0] != 0, bc[1] != 0, bc[2] != 0 };
        cf.get( "external_field_magnitude", h.B );
        double bn[3];
        if( cf.get3( "external_field_normal", bn ) )
            h.B_normal = normalize_or( { bn[0], bn[1], bn[2] }, { 0, 0, 1 } );
        double K = 0, kn[3] = { 0, 0, 1 };
        cf.get( "anisotropy_magnitude", K );
        cf.get3( "anisotropy_normal", kn );
        set_uniform_anisotropy( *geom, h, K, { kn[0], kn[1], kn[2] } );
        if( htype == "heisenberg_pairs" )
        {
            h.from_pairs = true;
            int n        = 0;
            if( cf.get( "n_interaction_pairs", n ) && n > 0 )
            {
                cf.next_line();
                std::vector<std::string> cols;
                {
                    std::string tok;
                    while( cf.read( tok ) )
                    {
                        for( auto & c : tok )
                            c = (char)std::tolower( c );
                        cols.push_back( tok );
                    }
                }
                for( int r = 0; r < n; ++r )
                {
                    if( !cf.next_line() )
                        break;
                    int i = 0, j = 0, t[3] = { 0, 0, 0 };
                    double J = 0, Dij = 0, D[3] = { 0, 0, 0 };
                    bool has_Dij = false;
                    for( auto & c : cols )
                    {
                        double v = 0;
                        cf.read( v );
                        if( c == "i" )
                            i = (int)v;
                        else if( c == "j" )
                            j = (int)v;
                        else if( c == "da" )
                            t[0] = (int)v;
                        else if( c == "db" )
                            t[1] = (int)v;
                        else if( c == "dc" )
                            t[2] = (int)v;
                        else if( c == "jij" )
                            J = v;
                        else if( c == "dij" )
                        {
                            Dij     = v;
                            has_Dij = true;
                        }
                        else if( c == "dijx" )
                            D[0] = v;
                        else if( c == "dijy" )
                            D[1] = v;
                        else if( c == "dijz" )
                            D[2] = v;
                    }
                    // Pairs_from_File (core/src/io/Dataparser.cpp:379-470): normalise the DMI vector,
                    // merge duplicate pairs
                    double dn = std::sqrt( std::pow( D[0], 2 ) + std::pow( D[1], 2 ) + std::pow( D[2], 2 ) );
                    if( dn != 0 )
                        for( auto & x : D )
                            x /= dn;
                    if( !has_Dij )
                        Dij = dn;
                    Pair P{ i, j, { t[0], t[1], t[2] } };
                    if( J != 0 )
                    {
                        bool merged = false;
                        for( size_t q = 0; q < h.ex_pairs_in.size(); ++q )
                        {
                            auto & p = h.ex_pairs_in[q];
                            if( ( p.i == i && p.j == j && p.t == P.t )
                                || ( p.i == j && p.j == i && p.t == std::array<int, 3>{ -t[0], -t[1], -t[2] } ) )
                            {
                                h.ex_J_in[q] += J;
                                merged = true;
                                break;
                            }
                        }
                        if( !merged )
                        {
                            h.ex_pairs_in.push_back( P );
                            h.ex_J_in.push_back( J );
                        }
                    }
                    if( Dij != 0 )
                    {
                        h.dmi_pairs_in.push_back( P );
                        h.dmi_D_in.push_back( Dij );
                        h.dmi_n_in.push_back( { D[0], D[1], D[2] } );
                    }
                }
            }
        }
        else
        {
            int ns = 0;
            if( cf.get( "n_shells_exchange", ns ) && ns > 0 )
            {
                h.jij.assign( ns, 0.0 );
                if( cf.find( "jij" ) )
                    for( int k = 0; k < ns; ++k )
                        cf.read( h.jij[k] );
            }
            int nd = 0;
            if( cf.get( "n_shells_dmi", nd ) && nd > 0 )
            {
                h.dij.assign( nd, 0.0 );
                if( cf.find( "dij" ) )
                    for( int k = 0; k < nd; ++k )
                        cf.read( h.dij[k] );
            }
            cf.get( "dm_chirality", h.dm_chirality );
        }
        std::string ddi = "none";
        cf.get( "ddi_method", ddi );
        h.ddi_method = ddi == "fft" ? 1 : ( ddi == "cutoff" ? 3 : 0 );
        int im[3];
        if( cf.get3( "ddi_n_periodic_images", im ) )
            h.ddi_images = { im[0], im[1], im[2] };
        int pb = 1;
        if( cf.get( "ddi_pb_zero_padding", pb ) )
            h.ddi_pb_zero_padding = pb != 0;
        cf.get( "ddi_radius", h.ddi_radius );
        // ---- LLG
        LLGParams & L = img->llg;
        cf.get( "llg_dt", L.dt );
        cf.get( "llg_damping", L.damping );
        cf.get( "llg_beta", L.beta );
        cf.get( "llg_temperature", L.temperature );
        cf.get( "llg_force_convergence", L.force_convergence );
        cf.get( "llg_n_iterations", L.n_iterations );
        cf.get( "llg_n_iterations_log", L.n_iterations_log );
        cf.get( "llg_seed", L.rng_seed );
        std::string wt;
        if( cf.get( "llg_max_walltime", wt ) )
            L.max_walltime_sec = parse_walltime( wt );
        cf.get( "llg_output_folder", L.output_folder );
        cf.get( "output_file_tag", L.output_tag );
        // ---- MC (Parameters_Method_MC_from_Config, core/src/io/Configparser.cpp:910-990)
        MCParams & M = img->mc;
        cf.get( "mc_seed", M.rng_seed );
        cf.get( "mc_n_iterations", M.n_iterations );
        cf.get( "mc_n_iterations_log", M.n_iterations_log );
        cf.get( "mc_temperature", M.temperature );
        cf.get( "mc_acceptance_ratio", M.acceptance_target );
        std::string mwt;
        if( cf.get( "mc_max_walltime", mwt ) )
            M.max_walltime_sec = parse_walltime( mwt );
        cf.get( "mc_output_folder", M.output_folder );
        cf.get( "output_file_tag", M.output_tag );
    }
    else
    {
        geom->mu_s_basis.assign( geom->nb(), 1.0 );
    }
    img->geom = geom;
    img->prng.seed( img->llg.rng_seed );
    update_interactions( *geom, h );
    img->spins.assign( 3 * (size_t)geom->nos(), 0.0 );
    img->eff_field.assign( 3 * (size_t)geom->nos(), 0.0 );
    refresh_positions( *img );
    // Configurations::Random on the whole system with the image's prng
    // (core/src/utility/Configurations.cpp:99-126, Vectormath.cpp:41-51)
    std::uniform_real_distribution<double> dist( -1, 1 );
    for( int i = 0; i < geom->nos(); ++i )
    {
        double vz   = dist( img->prng );
        double phi  = dist( img->prng ) * M_PI;
        double rxy  = std::sqrt( 1 - vz * vz );
        img->spins[3 * i + 0] = rxy * std::cos( phi );
        img->spins[3 * i + 1] = rxy * std::sin( phi );
        img->spins[3 * i + 2] = vz;
    }
    (void)st;
    return img;
}

void refresh_positions( Image & img )
{
    auto p = img.geom->positions();
    img.positions.resize( 3 * p.size() );
    for( size_t i = 0; i < p.size(); ++i )
        for( int e = 0; e < 3; ++e )
            img.positions[3 * i + e] = p[i][e];
}

std::shared_ptr<Image> clone_image( const Image & src )
{
    auto img       = std::make_shared<Image>();
    img->geom      = src.geom; // geometry is shared by all images of a chain
    img->ham       = src.ham;
    img->llg       = src.llg;
    img->mc        = src.mc;
    img->spins     = src.spins;
    img->eff_field = src.eff_field;
    img->positions = src.positions;
    img->E         = src.E;
    img->gneb_type = 0;
    img->prng      = src.prng;
    return img;
}

Engine & eval_engine( Image & img )
{
    if( !img.eval64 || img.eval64_version != img.version )
    {
        img.eval64.reset();
        SystemInput in;
        in.geom          = img.geom.get();
        in.ham           = &img.ham;
        img.eval64       = std::make_unique<Engine>( std::vector<SystemInput>{ in }, true );
        img.eval64_version = img.version;
    }
    return *img.eval64;
}

} // namespace sg
