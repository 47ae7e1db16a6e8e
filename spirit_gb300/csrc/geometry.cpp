#include "geometry.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <stdexcept>

namespace sg
{

static inline double norm( const Vec3 & v )
{
    return std::sqrt( v[0] * v[0] + v[1] * v[1] + v[2] * v[2] );
}

// Eigen's normalized(): a zero vector stays zero
static inline Vec3 normalized( const Vec3 & v )
{
    double n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if( n2 > 0 )
    {
        double n = std::sqrt( n2 );
        return { v[0] / n, v[1] / n, v[2] / n };
    }
    return v;
}

static inline Vec3 cross( const Vec3 & a, const Vec3 & b )
{
    return { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
}

// positions r = a_lat * ((n + cell_atom) . bravais)  (core/src/data/Geometry.cpp:141-160)
Vec3 Geometry::position( int ispin ) const
{
    int N  = nb();
    int ia = ispin % N;
    int cell = ispin / N;
    int da   = cell % n_cells[0];
    int db   = ( cell / n_cells[0] ) % n_cells[1];
    int dc   = cell / ( n_cells[0] * n_cells[1] );
    double fa = (double)da + cell_atoms[ia][0];
    double fb = (double)db + cell_atoms[ia][1];
    double fc = (double)dc + cell_atoms[ia][2];
    Vec3 r;
    for( int e = 0; e < 3; ++e )
        r[e] = lattice_constant * ( fa * bravais[0][e] + fb * bravais[1][e] + fc * bravais[2][e] );
    return r;
}

std::vector<Vec3> Geometry::positions() const
{
    std::vector<Vec3> p( nos() );
    for( int i = 0; i < nos(); ++i )
        p[i] = position( i );
    return p;
}

Vec3 Geometry::bounds_min() const
{
    Vec3 m{ DBL_MAX, DBL_MAX, DBL_MAX };
    for( int i = 0; i < nos(); ++i )
    {
        auto p = position( i );
        for( int e = 0; e < 3; ++e )
            m[e] = std::min( m[e], p[e] );
    }
    return m;
}

Vec3 Geometry::bounds_max() const
{
    Vec3 m{ -DBL_MAX, -DBL_MAX, -DBL_MAX };
    for( int i = 0; i < nos(); ++i )
    {
        auto p = position( i );
        for( int e = 0; e < 3; ++e )
            m[e] = std::max( m[e], p[e] );
    }
    return m;
}

Vec3 Geometry::center() const
{
    auto a = bounds_min(), b = bounds_max();
    return { 0.5 * ( a[0] + b[0] ), 0.5 * ( a[1] + b[1] ), 0.5 * ( a[2] + b[2] ) };
}

int Geometry::dimensionality() const
{
    int d = 0;
    for( int e = 0; e < 3; ++e )
        if( n_cells[e] > 1 )
            ++d;
    return d;
}

std::array<Vec3, 3> bravais_preset( const std::string & name, bool * ok )
{
    if( ok )
        *ok = true;
    const double h = 0.5 * std::sqrt( 3.0 );
    if( name == "sc" )
        return { Vec3{ 1, 0, 0 }, Vec3{ 0, 1, 0 }, Vec3{ 0, 0, 1 } };
    if( name == "fcc" )
        return { Vec3{ 0.5, 0.0, 0.5 }, Vec3{ 0.5, 0.5, 0.0 }, Vec3{ 0.0, 0.5, 0.5 } };
    if( name == "bcc" )
        return { Vec3{ 0.5, 0.5, -0.5 }, Vec3{ -0.5, 0.5, -0.5 }, Vec3{ 0.5, -0.5, -0.5 } };
    if( name == "hex2d" || name == "hex2d60" )
        return { Vec3{ h, -0.5, 0 }, Vec3{ h, 0.5, 0 }, Vec3{ 0, 0, 1 } };
    if( name == "hex2d120" )
        return { Vec3{ 0.5, -h, 0 }, Vec3{ 0.5, h, 0 }, Vec3{ 0, 0, 1 } };
    if( ok )
        *ok = false;
    return { Vec3{ 1, 0, 0 }, Vec3{ 0, 1, 0 }, Vec3{ 0, 0, 1 } };
}

// The shell search compares the fractional basis position cell_atoms[a1] with the Cartesian
// translation i*ta + j*tb + k*tc exactly as the reference does (Neighbours.cpp:56-66).
static void translation_bounds( const Geometry & g, int n_shells, Vec3 & ta, Vec3 & tb, Vec3 & tc, int & i_max,
                                int & j_max, int & k_max )
{
    for( int e = 0; e < 3; ++e )
    {
        ta[e] = g.lattice_constant * g.bravais[0][e];
        tb[e] = g.lattice_constant * g.bravais[1][e];
        tc[e] = g.lattice_constant * g.bravais[2][e];
    }
    int max_n = n_shells + 2;
    i_max     = std::min( max_n, g.n_cells[0] - 1 );
    j_max     = std::min( max_n, g.n_cells[1] - 1 );
    k_max     = std::min( max_n, g.n_cells[2] - 1 );
}

std::vector<double> shell_radii( const Geometry & g, int n_shells )
{
    const double min_shell_width = 1e-3;
    std::vector<double> radii( n_shells, 0.0 );
    Vec3 ta, tb, tc;
    int i_max, j_max, k_max;
    translation_bounds( g, n_shells, ta, tb, tc, i_max, j_max, k_max );
    if( norm( ta ) == 0.0 )
        i_max = 0;
    if( norm( tb ) == 0.0 )
        j_max = 0;
    if( norm( tc ) == 0.0 )
        k_max = 0;
    double outermost = 0, previous = 0;
    for( int ish = 0; ish < n_shells; ++ish )
    {
        previous  = outermost;
        outermost = DBL_MAX;
        for( int a1 = 0; a1 < g.nb(); ++a1 )
        {
            const Vec3 & p1 = g.cell_atoms[a1];
            for( int i = i_max; i >= 0; --i )
                for( int j = j_max; j >= -j_max; --j )
                    for( int k = k_max; k >= -k_max; --k )
                        for( int a2 = 0; a2 < g.nb(); ++a2 )
                        {
                            if( a1 == a2 && i == 0 && j == 0 && k == 0 )
                                continue;
                            Vec3 d;
                            for( int e = 0; e < 3; ++e )
                                d[e] = p1[e] - ( g.cell_atoms[a2][e] + i * ta[e] + j * tb[e] + k * tc[e] );
                            double delta = norm( d );
                            if( delta - previous > min_shell_width && delta < outermost )
                            {
                                outermost  = delta;
                                radii[ish] = delta;
                            }
                        }
        }
    }
    return radii;
}

void neighbours_in_shells( const Geometry & g, int n_shells, std::vector<Pair> & pairs, std::vector<int> & shells )
{
    const double min_shell_width = 1e-3;
    auto radii                   = shell_radii( g, n_shells );
    Vec3 ta, tb, tc;
    int i_max, j_max, k_max;
    translation_bounds( g, n_shells, ta, tb, tc, i_max, j_max, k_max );
    // lower bounds are fixed before the zero-vector checks (Neighbours.cpp:104-116)
    int i_min = -i_max, j_min = -j_max, k_min = -k_max;
    if( norm( ta ) == 0.0 )
        i_max = 0;
    if( norm( tb ) == 0.0 )
        j_max = 0;
    if( norm( tc ) == 0.0 )
        k_max = 0;
    pairs.clear();
    shells.clear();
    for( int a1 = 0; a1 < g.nb(); ++a1 )
    {
        const Vec3 & p1 = g.cell_atoms[a1];
        for( int ish = 0; ish < n_shells; ++ish )
            for( int i = i_max; i >= i_min; --i )
                for( int j = j_max; j >= j_min; --j )
                    for( int k = k_max; k >= k_min; --k )
                        for( int a2 = 0; a2 < g.nb(); ++a2 )
                        {
                            Vec3 d;
                            for( int e = 0; e < 3; ++e )
                                d[e] = p1[e] - ( g.cell_atoms[a2][e] + i * ta[e] + j * tb[e] + k * tc[e] );
                            if( std::abs( norm( d ) - radii[ish] ) < min_shell_width )
                            {
                                pairs.push_back( Pair{ a1, a2, { i, j, k } } );
                                shells.push_back( ish );
                            }
                        }
    }
}

Vec3 dmi_normal( const Geometry & g, const Pair & p, int chirality )
{
    Vec3 ipos = g.position( p.i ), jpos = g.position( p.j ), r;
    for( int e = 0; e < 3; ++e )
    {
        double ta = g.lattice_constant * g.bravais[0][e];
        double tb = g.lattice_constant * g.bravais[1][e];
        double tc = g.lattice_constant * g.bravais[2][e];
        jpos[e] += p.t[0] * ta + p.t[1] * tb + p.t[2] * tc;
        r[e] = jpos[e] - ipos[e];
    }
    const Vec3 ez{ 0, 0, 1 };
    if( chirality == 1 )
        return normalized( r );
    if( chirality == -1 )
        return normalized( Vec3{ -r[0], -r[1], -r[2] } );
    if( chirality == 2 )
        return cross( normalized( r ), ez );
    if( chirality == -2 )
        return cross( ez, normalized( r ) );
    return { 0, 0, 0 };
}

void set_uniform_anisotropy( const Geometry & g, HamiltonianParams & h, double K, const Vec3 & n )
{
    h.K        = K;
    h.K_normal = normalized( n );
    h.aniso_idx.clear();
    h.aniso_K.clear();
    h.aniso_n.clear();
    if( K != 0 )
        for( int i = 0; i < g.nb(); ++i )
        {
            h.aniso_idx.push_back( i );
            h.aniso_K.push_back( K );
            h.aniso_n.push_back( h.K_normal );
        }
}

void update_interactions( const Geometry & g, HamiltonianParams & h )
{
    h.ex_pairs.clear();
    h.ex_J.clear();
    h.dmi_pairs.clear();
    h.dmi_D.clear();
    h.dmi_n.clear();
    if( !h.from_pairs )
    {
        if( !h.jij.empty() )
        {
            std::vector<int> shells;
            neighbours_in_shells( g, (int)h.jij.size(), h.ex_pairs, shells );
            for( int s : shells )
                h.ex_J.push_back( h.jij[s] );
        }
        if( !h.dij.empty() )
        {
            std::vector<int> shells;
            neighbours_in_shells( g, (int)h.dij.size(), h.dmi_pairs, shells );
            for( size_t p = 0; p < h.dmi_pairs.size(); ++p )
            {
                h.dmi_n.push_back( dmi_normal( g, h.dmi_pairs[p], h.dm_chirality ) );
                h.dmi_D.push_back( h.dij[shells[p]] );
            }
        }
    }
    else
    {
        // explicit pairs + their redundant mirrors (Hamiltonian_Heisenberg.cpp:126-139, 160-173)
        h.ex_pairs = h.ex_pairs_in;
        h.ex_J     = h.ex_J_in;
        for( size_t p = 0; p < h.ex_pairs_in.size(); ++p )
        {
            auto & q = h.ex_pairs_in[p];
            h.ex_pairs.push_back( Pair{ q.j, q.i, { -q.t[0], -q.t[1], -q.t[2] } } );
            h.ex_J.push_back( h.ex_J_in[p] );
        }
        h.dmi_pairs = h.dmi_pairs_in;
        h.dmi_D     = h.dmi_D_in;
        h.dmi_n     = h.dmi_n_in;
        for( size_t p = 0; p < h.dmi_pairs_in.size(); ++p )
        {
            auto & q = h.dmi_pairs_in[p];
            h.dmi_pairs.push_back( Pair{ q.j, q.i, { -q.t[0], -q.t[1], -q.t[2] } } );
            h.dmi_D.push_back( h.dmi_D_in[p] );
            auto & n = h.dmi_n_in[p];
            h.dmi_n.push_back( Vec3{ -n[0], -n[1], -n[2] } );
        }
    }
}

int idx_from_pair( const Geometry & g, const std::array<int, 3> & bc, int ispin, const Pair & p )
{
    int N = g.nb();
    if( p.i != ispin % N )
        return -1;
    int Na = g.n_cells[0], Nb = g.n_cells[1], Nc = g.n_cells[2];
    if( std::abs( p.t[0] ) > Na || std::abs( p.t[1] ) > Nb || std::abs( p.t[2] ) > Nc )
        return -1;
    int nic = ispin / ( N * Na * Nb );
    int nib = ( ispin - nic * N * Na * Nb ) / ( N * Na );
    int nia = ( ispin - nic * N * Na * Nb - nib * N * Na ) / N;
    int n[3]    = { nia + p.t[0], nib + p.t[1], nic + p.t[2] };
    int lim[3]  = { Na, Nb, Nc };
    for( int d = 0; d < 3; ++d )
    {
        if( bc[d] || ( 0 <= n[d] && n[d] < lim[d] ) )
        {
            if( n[d] < 0 )
                n[d] += lim[d];
            if( n[d] >= lim[d] )
                n[d] -= lim[d];
        }
        else
            return -1;
    }
    return p.j + n[0] * N + n[1] * N * Na + n[2] * N * Na * Nb;
}

} // namespace sg
