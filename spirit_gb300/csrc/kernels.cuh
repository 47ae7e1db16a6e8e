// Device helpers shared by the LLG stage kernels (engine.cu) and the GNEB kernels (gneb.cu).
#pragma once
#include "common.hpp"

#include <cuda_runtime.h>

namespace sg
{

constexpr double C_MU_B  = 0.057883817555;
constexpr double C_K_B   = 0.08617330350;
constexpr double C_GAMMA = 0.1760859644;

template<typename R>
struct V3
{
    R x, y, z;
};
template<typename R>
__device__ __forceinline__ V3<R> cross( V3<R> a, V3<R> b )
{
    return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
template<typename R>
__device__ __forceinline__ R dot( V3<R> a, V3<R> b )
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
// Eigen normalize(): zero vectors stay zero
template<typename R>
__device__ __forceinline__ V3<R> normalized( V3<R> v )
{
    R n2 = dot( v, v );
    if( n2 > R( 0 ) )
    {
        R inv = R( 1 ) / sqrt( n2 );
        return { v.x * inv, v.y * inv, v.z * inv };
    }
    return v;
}

// Pair of the stencil in the kernels' working precision.  lin is the linear index offset of
// the neighbour, valid for cells whose whole stencil lies inside the system (no wrap, no cut).
// The couplings first and the record 16-byte aligned, so one pair reads as two or three vector
// loads from shared memory (J, D) and (lin, da, db, dc).
template<typename R>
struct alignas( 16 ) PairR
{
    R J, Dx, Dy, Dz;
    int lin, da, db, dc;
    int j;
};

template<typename R>
struct SoA3
{
    R * x;
    R * y;
    R * z;
    // I: long long, or int where the whole batch has fewer than 2^31 spins (one wide multiply-add
    // per address instead of a 64-bit add pair)
    template<typename I>
    __device__ __forceinline__ V3<R> ld( I i ) const
    {
        return { x[i], y[i], z[i] };
    }
    template<typename I>
    __device__ __forceinline__ void st( I i, V3<R> v ) const
    {
        x[i] = v.x;
        y[i] = v.y;
        z[i] = v.z;
    }
};

// ------------------------------------------------------------------ Philox4x32-10
// Salmon et al., SC'11.  Counter (spin, iteration, stream, 0x53504E00), key = seed.
__device__ __forceinline__ uint4 philox4x32( uint4 c, uint2 k )
{
#pragma unroll
    for( int r = 0; r < 10; ++r )
    {
        unsigned int hi0 = __umulhi( 0xD2511F53u, c.x ), lo0 = 0xD2511F53u * c.x;
        unsigned int hi1 = __umulhi( 0xCD9E8D57u, c.z ), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4( hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0 );
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// three standard normals for spin i: Box-Muller on 23-bit uniforms u = (x>>9 + 1/2) 2^-23
template<typename R>
__device__ __forceinline__ V3<R> gauss3( unsigned long long seed, unsigned int stream, unsigned int iteration,
                                         unsigned int i )
{
    uint4 x = philox4x32( make_uint4( i, iteration, stream, 0x53504E00u ),
                          make_uint2( (unsigned int)seed, (unsigned int)( seed >> 32 ) ) );
    const R sc = R( 1.0 / 8388608.0 );
    R u0 = ( R( x.x >> 9 ) + R( 0.5 ) ) * sc;
    R u1 = ( R( x.y >> 9 ) + R( 0.5 ) ) * sc;
    R u2 = ( R( x.z >> 9 ) + R( 0.5 ) ) * sc;
    R u3 = ( R( x.w >> 9 ) + R( 0.5 ) ) * sc;
    R r0 = sqrt( R( -2 ) * log( u0 ) );
    R r1 = sqrt( R( -2 ) * log( u2 ) );
    R s1, c1, s3, c3;
    sincospi( R( 2 ) * u1, &s1, &c1 );
    sincospi( R( 2 ) * u3, &s3, &c3 );
    return { r0 * c1, r0 * s1, r1 * c3 };
}

// Accumulation of one exchange + DMI pair, g -= J s_j + s_j x D.  FUSED (FP32 stage kernels):
// three FMAs per component (the products and the subtraction rounded together); otherwise the
// reference's order of operations.
template<typename R, bool FUSED>
__device__ __forceinline__ void pair_acc( V3<R> & g, R J, R Dx, R Dy, R Dz, V3<R> sj )
{
    if constexpr( FUSED )
    {
        g.x = fma( -J, sj.x, g.x );
        g.x = fma( -sj.y, Dz, g.x );
        g.x = fma( sj.z, Dy, g.x );
        g.y = fma( -J, sj.y, g.y );
        g.y = fma( -sj.z, Dx, g.y );
        g.y = fma( sj.x, Dz, g.y );
        g.z = fma( -J, sj.z, g.z );
        g.z = fma( -sj.x, Dy, g.z );
        g.z = fma( sj.y, Dx, g.z );
    }
    else
    {
        g.x -= J * sj.x;
        g.y -= J * sj.y;
        g.z -= J * sj.z;
        V3<R> cr = cross( sj, V3<R>{ Dx, Dy, Dz } );
        g.x -= cr.x;
        g.y -= cr.y;
        g.z -= cr.z;
    }
}

// Geometry scalars of one system, staged in shared memory by every kernel that walks pairs.
struct Geo
{
    int n[3];
    int bc[3];
    int nb;
    int nos;
    long long off;
    FastDiv div_nb, div_na, div_nbb;
    int pair_begin[MAX_BASIS + 1];
    int lo[3], hi[3]; // interior cells: lo[e] <= cell[e] < hi[e] on every axis
    int row_len;      // nb * Na: index distance of one wrap along a
    int a_single;     // every |da| < Na: one wrap along a reaches any neighbour
};

// Neighbour addressing of a warp: general (idx_from_pair), interior along b and c with the a-axis
// wrap done per lane, or fully interior (neighbour = spin index + lin).
enum StencilMode : int
{
    STENCIL_GENERAL = 0,
    STENCIL_ROW     = 1,
    STENCIL_INTERIOR = 2
};

__device__ __forceinline__ void load_geo( Geo & G, const SysDesc & d )
{
    if( threadIdx.x == 0 )
    {
        for( int e = 0; e < 3; ++e )
        {
            G.n[e]  = d.n_cells[e];
            G.bc[e] = d.bc[e];
        }
        G.nb      = d.nb;
        G.nos     = d.nos;
        G.off     = d.spin_offset;
        G.div_nb  = d.div_nb;
        G.div_na  = d.div_na;
        G.div_nbb = d.div_nbb;
        for( int b = 0; b <= d.nb; ++b )
            G.pair_begin[b] = d.pair_begin[b];
        for( int e = 0; e < 3; ++e )
        {
            G.lo[e] = d.max_t[e];
            G.hi[e] = d.n_cells[e] - d.max_t[e];
        }
        G.row_len  = d.nb * d.n_cells[0];
        G.a_single = d.max_t[0] < d.n_cells[0];
    }
}

// Stage the system's merged pairs in shared memory in the working precision (all threads).
template<typename R>
__device__ __forceinline__ void load_pairs_smem( PairR<R> * pairs, const SysDesc & d )
{
    const int nb = d.nb, Na = d.n_cells[0], Nb = d.n_cells[1];
    for( int p = threadIdx.x; p < d.n_pairs; p += blockDim.x )
    {
        const PairEntry & q = d.pairs[p];
        const int lin       = q.j - q.i + nb * ( q.da + Na * ( q.db + Nb * q.dc ) );
        pairs[p]            = { (R)q.J, (R)q.D[0], (R)q.D[1], (R)q.D[2], lin, q.da, q.db, q.dc, q.j };
    }
}

// Cell coordinates (a, b, c) and basis index ib of local spin index i
__device__ __forceinline__ void cell_of( const Geo & G, int i, int & ib, int & a, int & b, int & c )
{
    const int cell = (int)fdiv( (unsigned)i, G.div_nb );
    ib             = i - cell * G.nb;
    const int rest = (int)fdiv( (unsigned)cell, G.div_na );
    a              = cell - rest * G.n[0];
    c              = (int)fdiv( (unsigned)rest, G.div_nbb );
    b              = rest - c * G.n[1];
}

// Warp-uniform stencil mode: STENCIL_INTERIOR when every valid lane sits on an interior cell
// (neighbour of pair p = spin gi + lin_p), STENCIL_ROW when every valid lane is interior along b
// and c and one wrap along a suffices.  Called by all 32 lanes.
__device__ __forceinline__ int warp_stencil_mode( const Geo & G, int a, int b, int c, bool valid )
{
    const bool in_bc = !valid || ( b >= G.lo[1] && b < G.hi[1] && c >= G.lo[2] && c < G.hi[2] );
    const bool in_a  = !valid || ( a >= G.lo[0] && a < G.hi[0] );
    if( !__all_sync( 0xffffffffu, in_bc ) || !G.a_single )
        return STENCIL_GENERAL;
    return __all_sync( 0xffffffffu, in_a ) ? STENCIL_INTERIOR : STENCIL_ROW;
}

// ------------------------------------------------------------------ neighbour index
// idx_from_pair (core/include/engine/Vectormath.hpp:437-528) for a spin at cell (a, b, c): the
// batch index of the neighbour, -1 where an open boundary cuts the pair.  I: index type (int where
// the batch has fewer than 2^31 spins)
template<typename I = long long>
__device__ __forceinline__ I pair_index( const Geo & G, int a, int b, int c, int j, int da, int db, int dc )
{
    const int Na = G.n[0], Nb = G.n[1], Nc = G.n[2];
    if( abs( da ) > Na || abs( db ) > Nb || abs( dc ) > Nc )
        return -1;
    int ja = a + da, jb = b + db, jc = c + dc;
    if( G.bc[0] || ( ja >= 0 && ja < Na ) )
    {
        if( ja < 0 )
            ja += Na;
        if( ja >= Na )
            ja -= Na;
    }
    else
        return -1;
    if( G.bc[1] || ( jb >= 0 && jb < Nb ) )
    {
        if( jb < 0 )
            jb += Nb;
        if( jb >= Nb )
            jb -= Nb;
    }
    else
        return -1;
    if( G.bc[2] || ( jc >= 0 && jc < Nc ) )
    {
        if( jc < 0 )
            jc += Nc;
        if( jc >= Nc )
            jc -= Nc;
    }
    else
        return -1;
    return (I)G.off + j + (I)G.nb * ( ja + Na * ( jb + (I)Nb * jc ) );
}

// ------------------------------------------------------------------ block reductions
__device__ __forceinline__ double block_sum( double v, double * sh )
{
    for( int o = 16; o > 0; o >>= 1 )
        v += __shfl_down_sync( 0xffffffffu, v, o );
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if( l == 0 )
        sh[w] = v;
    __syncthreads();
    double r = 0;
    if( threadIdx.x < 32 )
    {
        r = threadIdx.x < ( blockDim.x >> 5 ) ? sh[threadIdx.x] : 0.0;
        for( int o = 16; o > 0; o >>= 1 )
            r += __shfl_down_sync( 0xffffffffu, r, o );
    }
    return r; // valid in thread 0
}

// Block sum of per-thread values of the working precision: a shuffle tree in R inside each
// warp, then the warp partials summed in FP64 by warp 0 (result valid in thread 0).
template<typename R>
__device__ __forceinline__ double block_sum_w( R v, double * sh )
{
    for( int o = 16; o > 0; o >>= 1 )
        v += __shfl_down_sync( 0xffffffffu, v, o );
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if( l == 0 )
        sh[w] = (double)v;
    __syncthreads();
    double r = 0;
    if( threadIdx.x < 32 )
    {
        r = threadIdx.x < ( blockDim.x >> 5 ) ? sh[threadIdx.x] : 0.0;
        for( int o = 16; o > 0; o >>= 1 )
            r += __shfl_down_sync( 0xffffffffu, r, o );
    }
    return r;
}

// Compensated accumulation s + c += x: in FP32 the rounding error of every addition is kept in c
// (TwoSum, Knuth: exact for round-to-nearest, no branch); FP64 accumulates plainly.
template<typename R>
__device__ __forceinline__ void comp_add( R & s, R & c, R x )
{
    if( sizeof( R ) == 4 )
    {
        const R t  = s + x;
        const R bp = t - s;
        c += ( s - ( t - bp ) ) + ( x - bp );
        s = t;
    }
    else
        s += x;
}

// Block sum of compensated FP32 partials (s, c): the shuffle tree inside each warp combines the
// pairs with TwoSum (the errors of the tree's additions join c), each warp's s + c is formed in
// FP64 and the warps are summed in FP64 by warp 0 (result valid in thread 0).  FP64 partials are
// summed as block_sum_w does.
template<typename R>
__device__ __forceinline__ double block_sum_comp( R v, R c, double * sh )
{
    if constexpr( sizeof( R ) != 4 )
        return block_sum_w( v, sh );
    for( int o = 16; o > 0; o >>= 1 )
    {
        const R v2 = __shfl_down_sync( 0xffffffffu, v, o );
        const R c2 = __shfl_down_sync( 0xffffffffu, c, o );
        const R t  = v + v2;
        const R bp = t - v;
        c += c2 + ( ( v - ( t - bp ) ) + ( v2 - bp ) );
        v = t;
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if( l == 0 )
        sh[w] = (double)v + (double)c;
    __syncthreads();
    double r = 0;
    if( threadIdx.x < 32 )
    {
        r = threadIdx.x < ( blockDim.x >> 5 ) ? sh[threadIdx.x] : 0.0;
        for( int o = 16; o > 0; o >>= 1 )
            r += __shfl_down_sync( 0xffffffffu, r, o );
    }
    return r;
}

__device__ __forceinline__ float block_max( float v, float * sh )
{
    for( int o = 16; o > 0; o >>= 1 )
        v = fmaxf( v, __shfl_down_sync( 0xffffffffu, v, o ) );
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if( l == 0 )
        sh[w] = v;
    __syncthreads();
    float r = 0;
    if( threadIdx.x < 32 )
    {
        r = threadIdx.x < ( blockDim.x >> 5 ) ? sh[threadIdx.x] : 0.f;
        for( int o = 16; o > 0; o >>= 1 )
            r = fmaxf( r, __shfl_down_sync( 0xffffffffu, r, o ) );
    }
    return r;
}

// Copy the per-system constants into shared memory (all threads; followed by __syncthreads by
// the caller).
template<typename R>
__device__ __forceinline__ void load_const( SysConst<R> & dst, const SysDesc & d )
{
    const unsigned int * src = reinterpret_cast<const unsigned int *>( &sys_const<R>( d ) );
    unsigned int * o         = reinterpret_cast<unsigned int *>( &dst );
    for( int w = threadIdx.x; w < (int)( sizeof( SysConst<R> ) / 4 ); w += blockDim.x )
        o[w] = src[w];
}

// Batch index of the neighbour of pair P for the spin gi at cell (a, b, c) under the warp's
// stencil mode; -1 where the pair is cut by an open boundary.
template<typename R, typename I>
__device__ __forceinline__ I neighbour_index( const Geo & d, const PairR<R> & P, int mode, I gi, int a, int b, int c )
{
    if( mode == STENCIL_INTERIOR )
        return gi + P.lin;
    if( mode == STENCIL_ROW )
    {
        const int ja = a + P.da;
        const I j    = gi + P.lin;
        if( ja < 0 )
            return d.bc[0] ? j + d.row_len : -1;
        if( ja >= d.n[0] )
            return d.bc[0] ? j - d.row_len : -1;
        return j;
    }
    return pair_index<I>( d, a, b, c, P.j, P.da, P.db, P.dc );
}

// Gradient of the Heisenberg Hamiltonian at spin i of configuration cfg (Gradient_and_Energy,
// Hamiltonian_Heisenberg.cpp:704-766: anisotropy, exchange + DMI pairs, dipolar field, then
// Zeeman), and the energy of that spin: 0.5 g_quadratic . s + Zeeman, in the working precision.
// hval, when given, is the dipolar field of the spin (instead of h[gi]).
// FUSED: FMA-fused pair accumulation (pair_acc); ENERGY: form e (false: e is left untouched).
// I: index type of gi and the neighbours (int for the stage kernels, whose batches have fewer
// than 2^31 spins).
template<typename R, bool FUSED = false, bool ENERGY = true, typename I = long long>
__device__ __forceinline__ V3<R> gradient_at( const Geo & d, const SysConst<R> & C, const PairR<R> * pairs,
                                              const SoA3<R> & cfg, const SoA3<R> & h, I gi, int ib, int a, int b,
                                              int c, V3<R> si, R mu, R & e, int mode = STENCIL_GENERAL,
                                              const V3<R> * hval = nullptr )
{
    V3<R> g = { 0, 0, 0 };
    for( int k = 0; k < C.n_aniso; ++k )
        if( C.aniso_idx[k] == ib )
        {
            V3<R> n = { C.aniso_n[k][0], C.aniso_n[k][1], C.aniso_n[k][2] };
            R sc    = R( 2 ) * C.aniso_K[k] * dot( n, si );
            g.x -= sc * n.x;
            g.y -= sc * n.y;
            g.z -= sc * n.z;
        }
    // one pair at a time and not unrolled: on the 256-system SIB ensemble (4 pairs per spin) this
    // ran 4 % faster than unrolled or chunked loops that issue several pairs' neighbour loads
    // together (the stage kernels are bound by issue and code size, not by these loads)
    const int p0 = d.pair_begin[ib], p1 = d.pair_begin[ib + 1];
#pragma unroll 1
    for( int p = p0; p < p1; ++p )
    {
        const I j      = neighbour_index( d, pairs[p], mode, gi, a, b, c );
        const V3<R> sj = j >= 0 ? cfg.ld( j ) : V3<R>{ 0, 0, 0 };
        if( j >= 0 )
        {
            const PairR<R> & P = pairs[p];
            pair_acc<R, FUSED>( g, P.J, P.Dx, P.Dy, P.Dz, sj );
        }
    }
    if( hval || h.x )
    {
        // dipolar field of the spin: given (computed by the caller) or from the field arrays
        V3<R> hh = hval ? *hval : h.ld( gi );
        g.x -= mu * hh.x;
        g.y -= mu * hh.y;
        g.z -= mu * hh.z;
    }
    if( ENERGY )
        e = R( 0.5 ) * ( g.x * si.x + g.y * si.y + g.z * si.z );
    if( C.has_zeeman )
    {
        V3<R> B = { C.zeeman[0], C.zeeman[1], C.zeeman[2] };
        g.x -= mu * B.x;
        g.y -= mu * B.y;
        g.z -= mu * B.z;
        if( ENERGY )
            e += -mu * ( B.x * si.x + B.y * si.y + B.z * si.z );
    }
    return g;
}

// Calculate_Force_Virtual for spin configuration c, force F = -g
template<typename R>
__device__ __forceinline__ V3<R> virtual_force( const SysConst<R> & C, V3<R> c, V3<R> g, R inv_mu, V3<R> xi )
{
    V3<R> F = { -g.x, -g.y, -g.z };
    if( C.direct )
    {
        V3<R> cr = cross( c, F );
        return { C.kdm * cr.x, C.kdm * cr.y, C.kdm * cr.z };
    }
    V3<R> cr = cross( c, F );
    V3<R> fv = { C.dtg * F.x, C.dtg * F.y, C.dtg * F.z };
    fv.x += C.dtga * cr.x;
    fv.y += C.dtga * cr.y;
    fv.z += C.dtga * cr.z;
    fv.x *= inv_mu;
    fv.y *= inv_mu;
    fv.z *= inv_mu;
    if( C.thermal )
    {
        V3<R> cx = cross( c, xi );
        fv.x += xi.x;
        fv.y += xi.y;
        fv.z += xi.z;
        fv.x += C.alpha * cx.x;
        fv.y += C.alpha * cx.y;
        fv.z += C.alpha * cx.z;
    }
    return fv;
}

// sib_transform (Solver_Kernels.cpp:15-48)
template<typename R>
__device__ __forceinline__ V3<R> sib( V3<R> e1, V3<R> f )
{
    V3<R> A  = { R( 0.5 ) * f.x, R( 0.5 ) * f.y, R( 0.5 ) * f.z };
    R nA     = sqrt( dot( A, A ) );
    R detAi  = R( 1 ) / ( R( 1 ) + nA * nA );
    V3<R> cr = cross( e1, A );
    V3<R> a2 = { e1.x - cr.x, e1.y - cr.y, e1.z - cr.z };
    V3<R> o;
    o.x = ( a2.x * ( A.x * A.x + R( 1 ) ) + a2.y * ( A.x * A.y - A.z ) + a2.z * ( A.x * A.z + A.y ) ) * detAi;
    o.y = ( a2.x * ( A.y * A.x + A.z ) + a2.y * ( A.y * A.y + R( 1 ) ) + a2.z * ( A.y * A.z - A.x ) ) * detAi;
    o.z = ( a2.x * ( A.z * A.x - A.y ) + a2.y * ( A.z * A.y + A.x ) + a2.z * ( A.z * A.z + R( 1 ) ) ) * detAi;
    return o;
}

// Rodrigues rotation (Vectormath::rotate, Vectormath.cpp:474-479)
template<typename R>
__device__ __forceinline__ V3<R> rotate( V3<R> v, V3<R> axis, R angle )
{
    R sn, cs;
    sincos( angle, &sn, &cs );
    V3<R> ax = cross( axis, v );
    R ad     = dot( axis, v );
    R omc    = R( 1 ) - cs;
    return { v.x * cs + ax.x * sn + axis.x * ad * omc, v.y * cs + ax.y * sn + axis.y * ad * omc,
             v.z * cs + ax.z * sn + axis.z * ad * omc };
}

template<typename R>
__device__ __forceinline__ R torque2( V3<R> fv, V3<R> s )
{
    R d      = dot( fv, s );
    V3<R> t  = { fv.x - d * s.x, fv.y - d * s.y, fv.z - d * s.z };
    return dot( t, t );
}


} // namespace sg
