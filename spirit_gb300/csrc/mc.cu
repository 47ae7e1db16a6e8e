// Metropolis Monte Carlo on the device (Method_MC, core/src/engine/Method_MC.cpp:54-190).
//
// The reference visits nos spins one after another (randomly drawn or in order) with one
// std::mt19937.  Here a sweep visits every spin once, colour by colour: the spins of one colour
// never interact (greedy colouring of the exchange/DMI graph in spin order), so a whole colour is
// one parallel step and the result does not depend on the order inside a colour.  Per spin and
// sweep one Philox4x32-10 block (counter (spin, sweep, stream, 0x4D435300), key = seed; the sweep
// count continues over successive runs of an image, like the reference's persistent generator) gives
// u0 -> cos(theta) of the cone sample, u1 -> phi, u2 -> the Metropolis test.  The single-spin
// energy is Energy_Single_Spin (Hamiltonian_Heisenberg.cpp:559-668; no dipolar term) with the
// current neighbours; the cone angle adapts once per sweep from the previous sweep's rejections
// (Method_MC.cpp:73-89).
#include "kernels.cuh"
#include "mc.hpp"
#include "util.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace sg
{

constexpr int MC_MAX_COLORS = 64;

struct MCConst
{
    double kT;
    double temperature;
    double target;
    unsigned long long seed;
    unsigned int stream;
    int cone;
    int adaptive;
    int n_iterations;
    int nos;
    int list_off; // first entry of the system in the permutation
    unsigned int rng_offset;
    int color_off[MC_MAX_COLORS + 1];
};

struct MCState
{
    double cone;     // radians
    double acc;      // acceptance ratio of the previous sweep
    double cos_cone;
    int n_rej;
    int iteration;
    int active;
    int pad;
};

// ------------------------------------------------------------------ kernels
__global__ void mc_adapt( MCState * st, const MCConst * k, int n_sys )
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if( s >= n_sys || !st[s].active )
        return;
    MCState & S       = st[s];
    const MCConst & K = k[s];
    const double dif  = 0.01;
    const double pi   = 3.14159265358979323846;
    if( K.cone && K.adaptive )
    {
        S.acc = 1.0 - (double)S.n_rej / (double)K.nos;
        if( S.acc < K.target && S.cone > dif )
            S.cone -= dif;
        if( S.acc > K.target && S.cone < pi - dif )
            S.cone += dif;
    }
    S.n_rej    = 0;
    S.cos_cone = cos( S.cone );
}

__global__ void mc_end( MCState * st, const MCConst * k, int n_sys )
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if( s >= n_sys || !st[s].active )
        return;
    st[s].iteration += 1;
    st[s].active = st[s].iteration < k[s].n_iterations;
}

template<typename R>
__device__ __forceinline__ R single_energy( const SysConst<R> & C, int ib, R mu, V3<R> v, V3<R> h )
{
    R E = 0;
    if( C.has_zeeman )
        E -= mu * ( C.zeeman[0] * v.x + C.zeeman[1] * v.y + C.zeeman[2] * v.z );
    for( int k = 0; k < C.n_aniso; ++k )
        if( C.aniso_idx[k] == ib )
        {
            const R d = C.aniso_n[k][0] * v.x + C.aniso_n[k][1] * v.y + C.aniso_n[k][2] * v.z;
            E -= C.aniso_K[k] * d * d;
        }
    E -= dot( v, h );
    return E;
}

// one colour of one sweep: block = (system, first list entry, count)
template<typename R>
__global__ void __launch_bounds__( 256 ) mc_color( const SysDesc * sd, SoA3<R> spins, const int * perm,
                                                   const int4 * table, MCState * st, const MCConst * kc )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red[32];
    const int4 blk = table[blockIdx.x];
    const int s    = blk.x;
    if( !st[s].active )
        return;
    const SysDesc & d = sd[s];
    const MCConst & K = kc[s];
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    __syncthreads();
    const int t      = threadIdx.x;
    const bool valid = t < blk.z;
    const int i      = valid ? perm[K.list_off + blk.y + t] : 0;
    int ib, a, b, c;
    cell_of( GS, i, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, valid );
    R rejected      = 0;
    if( valid )
    {
        const long long gi = GS.off + i;
        // field of the pairs: h = sum_p (J_p s_j + s_j x D_p)
        V3<R> h      = { 0, 0, 0 };
        const int p0 = GS.pair_begin[ib], p1 = GS.pair_begin[ib + 1];
        for( int q = p0; q < p1; ++q )
        {
            const PairR<R> P = pairs[q];
            long long j;
            if( smode == STENCIL_INTERIOR )
                j = gi + P.lin;
            else if( smode == STENCIL_ROW )
            {
                const int ja = a + P.da;
                j            = gi + P.lin;
                if( ja < 0 )
                    j = GS.bc[0] ? j + GS.row_len : -1;
                else if( ja >= GS.n[0] )
                    j = GS.bc[0] ? j - GS.row_len : -1;
            }
            else
                j = pair_index( GS, a, b, c, P.j, P.da, P.db, P.dc );
            if( j < 0 )
                continue;
            const V3<R> sj = spins.ld( j );
            const V3<R> cr = cross( sj, V3<R>{ P.Dx, P.Dy, P.Dz } );
            h.x += P.J * sj.x + cr.x;
            h.y += P.J * sj.y + cr.y;
            h.z += P.J * sj.z + cr.z;
        }
        const V3<R> so = spins.ld( gi );
        const uint4 x  = philox4x32( make_uint4( (unsigned)i, (unsigned)st[s].iteration + K.rng_offset, K.stream,
                                                 0x4D435300u ),
                                     make_uint2( (unsigned)K.seed, (unsigned)( K.seed >> 32 ) ) );
        const R sc     = R( 1.0 / 8388608.0 );
        const R u0     = ( R( x.x >> 9 ) + R( 0.5 ) ) * sc;
        const R u1     = ( R( x.y >> 9 ) + R( 0.5 ) ) * sc;
        const R u2     = ( R( x.z >> 9 ) + R( 0.5 ) ) * sc;
        V3<R> e0 = { 1, 0, 0 }, e1 = { 0, 1, 0 }, e2 = { 0, 0, 1 };
        R ct;
        if( K.cone )
        {
            // local basis with the spin as third axis (Method_MC.cpp:113-123)
            if( so.z < R( 1 - 1e-10 ) )
            {
                e2 = so;
                e0 = normalized( cross( e2, V3<R>{ 0, 0, 1 } ) );
                e1 = cross( e2, e0 );
            }
            ct = R( 1 ) - ( R( 1 ) - (R)st[s].cos_cone ) * u0;
        }
        else
            ct = u0; // the reference samples cos(theta) in [0, 1) here
        const R stt = sqrt( R( 1 ) - ct * ct );
        R sp, cp;
        sincospi( R( 2 ) * u1, &sp, &cp );
        const V3<R> l = { stt * cp, stt * sp, ct };
        const V3<R> v = { e0.x * l.x + e1.x * l.y + e2.x * l.z, e0.y * l.x + e1.y * l.y + e2.y * l.z,
                          e0.z * l.x + e1.z * l.y + e2.z * l.z };
        const R mu   = C.mu[ib];
        const R dE   = single_energy( C, ib, mu, v, h ) - single_energy( C, ib, mu, so, h );
        bool reject  = false;
        if( dE > R( 1e-14 ) )
        {
            if( K.temperature < 1e-12 )
                reject = true;
            else if( exp( -dE / (R)K.kT ) < u2 )
                reject = true;
        }
        if( reject )
            rejected = 1;
        else
            spins.st( gi, v );
    }
    const double nr = block_sum_w( rejected, red );
    if( threadIdx.x == 0 && nr > 0 )
        atomicAdd( &st[s].n_rej, (int)( nr + 0.5 ) );
}

// ================================================================== host
// neighbour index of the system's merged pair q at spin i (idx_from_pair, Vectormath.hpp:437-528)
static int host_pair_index( const SysDesc & d, int i, const PairEntry & q )
{
    const int nb = d.nb, Na = d.n_cells[0], Nb = d.n_cells[1], Nc = d.n_cells[2];
    const int cell = i / nb;
    const int a = cell % Na, b = ( cell / Na ) % Nb, c = cell / ( Na * Nb );
    const int t[3] = { q.da, q.db, q.dc }, n[3] = { Na, Nb, Nc };
    int x[3]       = { a + q.da, b + q.db, c + q.dc };
    for( int e = 0; e < 3; ++e )
    {
        if( std::abs( t[e] ) > n[e] )
            return -1;
        if( d.bc[e] || ( x[e] >= 0 && x[e] < n[e] ) )
        {
            if( x[e] < 0 )
                x[e] += n[e];
            if( x[e] >= n[e] )
                x[e] -= n[e];
        }
        else
            return -1;
    }
    return q.j + nb * ( x[0] + Na * ( x[1] + Nb * x[2] ) );
}

MCRun::MCRun( Engine & E ) : E_( E )
{
    n_sys_ = (size_t)E.n_sys();
    std::vector<int> perm;
    std::vector<MCConst> consts( n_sys_ );
    std::vector<std::vector<int4>> tables;
    for( size_t s = 0; s < n_sys_; ++s )
    {
        const SysDesc & d = E.desc( (int)s );
        std::vector<int> color( d.nos, -1 );
        int nc = 0;
        std::vector<int> used;
        for( int i = 0; i < d.nos; ++i )
        {
            used.assign( MC_MAX_COLORS + 1, 0 );
            const int ib = i % d.nb;
            for( int q = d.pair_begin[ib]; q < d.pair_begin[ib + 1]; ++q )
            {
                const int j = host_pair_index( d, i, d.pairs[q] );
                if( j >= 0 && j != i && color[j] >= 0 && color[j] <= MC_MAX_COLORS )
                    used[color[j]] = 1;
            }
            int c = 0;
            while( c < MC_MAX_COLORS && used[c] )
                ++c;
            if( c >= MC_MAX_COLORS )
                throw std::runtime_error( "Monte Carlo: more colours needed than supported" );
            color[i] = c;
            nc       = std::max( nc, c + 1 );
        }
        MCConst & K = consts[s];
        K           = MCConst{};
        K.nos       = d.nos;
        K.list_off  = (int)perm.size();
        std::vector<int> count( nc, 0 );
        for( int i = 0; i < d.nos; ++i )
            count[color[i]]++;
        K.color_off[0] = 0;
        for( int c = 0; c < nc; ++c )
            K.color_off[c + 1] = K.color_off[c] + count[c];
        for( int c = nc; c < MC_MAX_COLORS; ++c )
            K.color_off[c + 1] = K.color_off[c];
        for( int c = 0; c < nc; ++c )
            for( int i = 0; i < d.nos; ++i )
                if( color[i] == c )
                    perm.push_back( i );
        if( (int)tables.size() < nc )
            tables.resize( nc );
        for( int c = 0; c < nc; ++c )
            for( int f = K.color_off[c]; f < K.color_off[c + 1]; f += 256 )
                tables[c].push_back( make_int4( (int)s, f, std::min( 256, K.color_off[c + 1] - f ), 0 ) );
        n_colors_ = std::max( n_colors_, nc );
    }
    d_perm_ = dalloc<int>( std::max<size_t>( perm.size(), 1 ) );
    if( !perm.empty() )
        h2d( d_perm_, perm.data(), perm.size() );
    for( auto & t : tables )
    {
        int4 * p = dalloc<int4>( std::max<size_t>( t.size(), 1 ) );
        if( !t.empty() )
            h2d( p, t.data(), t.size() );
        d_tables_.push_back( p );
        n_blocks_.push_back( (int)t.size() );
    }
    d_const_ = dalloc<MCConst>( std::max<size_t>( n_sys_, 1 ) );
    d_state_ = dalloc<MCState>( std::max<size_t>( n_sys_, 1 ) );
    h2d( (MCConst *)d_const_, consts.data(), consts.size() );
}

MCRun::~MCRun()
{
    if( graph_ )
        cudaGraphExecDestroy( graph_ );
    dfree( d_perm_ );
    for( auto & p : d_tables_ )
        dfree( p );
    dfree( d_const_ );
    dfree( d_state_ );
}

void MCRun::start( const std::vector<MCSettings> & settings )
{
    std::vector<MCConst> consts( n_sys_ );
    d2h( consts.data(), (const MCConst *)d_const_, n_sys_ );
    std::vector<MCState> st( n_sys_ );
    for( size_t s = 0; s < n_sys_; ++s )
    {
        const MCSettings & m = settings.size() == 1 ? settings[0] : settings[s];
        MCConst & K          = consts[s];
        K.kT                 = 0.08617330350 * m.temperature; // k_B (Constants.hpp)
        K.temperature        = m.temperature;
        K.target             = m.acceptance_target;
        K.seed               = m.seed;
        K.stream             = m.stream + (unsigned)( settings.size() == 1 ? s : 0 );
        K.cone               = m.cone ? 1 : 0;
        K.adaptive           = m.adaptive ? 1 : 0;
        K.n_iterations       = m.n_iterations;
        K.rng_offset         = m.rng_offset;
        MCState & S          = st[s];
        S                    = MCState{};
        S.cone               = 3.14159265358979323846 * m.cone_angle_deg / 180.0;
        S.acc                = m.acceptance_target;
        S.cos_cone           = std::cos( S.cone );
        S.active             = m.n_iterations > 0;
    }
    h2d( (MCConst *)d_const_, consts.data(), consts.size() );
    h2d( (MCState *)d_state_, st.data(), st.size() );
}

template<typename R>
void MCRun::sweep_t()
{
    cudaStream_t stm = E_.stream();
    const int ns     = (int)n_sys_;
    mc_adapt<<<( ns + 127 ) / 128, 128, 0, stm>>>( (MCState *)d_state_, (const MCConst *)d_const_, ns );
    SoA3<R> sp = { (R *)E_.spin_ptr( 0 ), (R *)E_.spin_ptr( 1 ), (R *)E_.spin_ptr( 2 ) };
    for( int c = 0; c < n_colors_; ++c )
        if( n_blocks_[c] > 0 )
            mc_color<R><<<n_blocks_[c], 256, 0, stm>>>( E_.d_desc(), sp, d_perm_, d_tables_[c], (MCState *)d_state_,
                                                        (const MCConst *)d_const_ );
    mc_end<<<( ns + 127 ) / 128, 128, 0, stm>>>( (MCState *)d_state_, (const MCConst *)d_const_, ns );
    CUDA_CHECK( cudaGetLastError() );
}

void MCRun::launch( int n_sweeps )
{
    const int G      = 8;
    cudaStream_t stm = E_.stream();
    if( !graph_ )
    {
        cudaGraph_t g;
        CUDA_CHECK( cudaStreamBeginCapture( stm, cudaStreamCaptureModeThreadLocal ) );
        for( int k = 0; k < G; ++k )
        {
            if( E_.fp64() )
                sweep_t<double>();
            else
                sweep_t<float>();
        }
        CUDA_CHECK( cudaStreamEndCapture( stm, &g ) );
        CUDA_CHECK( cudaGraphInstantiate( &graph_, g, 0 ) );
        cudaGraphDestroy( g );
    }
    for( int k = 0; k < n_sweeps / G; ++k )
        CUDA_CHECK( cudaGraphLaunch( graph_, stm ) );
    for( int k = 0; k < n_sweeps % G; ++k )
    {
        if( E_.fp64() )
            sweep_t<double>();
        else
            sweep_t<float>();
    }
}

std::vector<MCStatus> MCRun::status()
{
    std::vector<MCState> st( n_sys_ );
    CUDA_CHECK( cudaStreamSynchronize( E_.stream() ) );
    d2h( st.data(), (const MCState *)d_state_, n_sys_ );
    std::vector<MCStatus> out( n_sys_ );
    for( size_t s = 0; s < n_sys_; ++s )
        out[s] = { st[s].iteration, st[s].cone * 180.0 / 3.14159265358979323846, st[s].acc };
    return out;
}

} // namespace sg
