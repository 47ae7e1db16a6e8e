// Hand-written adjoint of the T = 0 RK4 LLG trajectory (no counterpart in the reference).
//
// Forward step (identical arithmetic to the engine's RK4 stage kernels, llg_stage<R, RK4, m>,
// Solver_RK4.hpp:40-147):
//     c1 = s;  f_m = fv(c_m) (Method_LLG.cpp:132-226 at T = 0);  k_m = -(c_m x f_m)
//     p2 = s + k1/2, p3 = s + k2/2, p4 = s + k3;  c_m = N(p_m);  acc = s + k1/6 + k2/3 + k3/3 + k4/6
//     s' = N(acc)
// with fv(c) = (dtg Fo + dtga c x Fo) / mu, Fo = -g(c), g(c) = L c + z the Heisenberg gradient
// (L symmetric: anisotropy, exchange + DMI pairs of the redundant list, dipolar convolution with a
// symmetric tensor; z the Zeeman term).  Reverse mode, for lam' = dLoss/ds':
//     lam_acc = JN(acc) lam',  JN(x) = (I - x^ x^T) / |x|
//     lam_s += lam_acc, lam_k1 += lam_acc/6, lam_k2 += lam_acc/3, lam_k3 += lam_acc/3, lam_k4 += lam_acc/6
//     for m = 4..1:  lam_c  = lam_k x f_m                          (from k = -c x f)
//                    lam_f  = c_m x lam_k
//                    lam_Fo = (dtg lam_f + dtga lam_f x c_m) / mu
//                    lam_c += dtga (Fo_m x lam_f) / mu - L lam_Fo   (L lam_Fo: the same stencil and the
//                                                                     same dipolar convolution, transposed
//                                                                     = itself)
//                    m > 1: lam_p = JN(p_m) lam_c, lam_s += lam_p, lam_k(m-1) += lam_p (m = 4) or lam_p/2
//                    m = 1: lam_s += lam_c
// Parameter gradients (J, D, K: scale of all couplings of that kind relative to the configured
// first shell / anisotropy; B_z; alpha):
//     dLoss/dJ += lam_Fo . sum_p Jhat_p c_j,  dLoss/dD += lam_Fo . sum_p c_j x Dhat_p,
//     dLoss/dK += lam_Fo . 2 Khat (n . c) n,  dLoss/dB += mu lam_Fo . mu_B n_B,
//     dLoss/dalpha += lam_f . dfv/dalpha = lam_f . dtg/(mu (1 + a^2)) (-2 a Fo + (1 - a^2) c x Fo)
//
// Checkpointing: the forward pass keeps s every `checkpoint` steps; the backward pass recomputes
// one segment at a time from its checkpoint, recording every stage quantity of its steps in HBM,
// then runs the adjoint steps of the segment in reverse.  Cost: forward + recompute + adjoint.
#include "adjoint.hpp"
#include "kernels.cuh"
#include "util.hpp"

#include <cmath>
#include <cstring>
#include <stdexcept>

namespace sg
{

template<typename R>
struct AdjUnits
{
    R Jhat[MAX_PAIRS];
    R Dhat[MAX_PAIRS][3];
    R Khat[MAX_BASIS];
    R Bn[3]; // mu_B n_B
};

template<typename R>
struct AdjArgs
{
    const SysDesc * sd;
    SoA3<R> c[4];  // stage configurations, c[0] = s_n
    SoA3<R> f[4];  // virtual forces
    SoA3<R> Fo[4]; // -g
    SoA3<R> p[4];  // p[1..3]: predictors before normalisation
    SoA3<R> acc;   // RK4 sum
    SoA3<R> s_out; // s_{n+1}
    SoA3<R> h;     // dipolar field (of c_m forward, of lam_Fo backward)
    SoA3<R> lam_next; // dLoss/ds_{n+1}
    SoA3<R> lam_s;    // dLoss/ds_n (accumulated)
    SoA3<R> lam_k[4];
    SoA3<R> lam_Fo[2]; // stage m uses lam_Fo[m % 2] (the next stage's is written while neighbours read this)
    SoA3<R> lam_c;
    double * pgrad; // [5][n_blocks] per-block partial parameter gradients
    int n_blocks;
    int record;
    AdjUnits<R> u;
};

template<typename R>
__device__ __forceinline__ V3<R> operator_add( V3<R> a, V3<R> b )
{
    return { a.x + b.x, a.y + b.y, a.z + b.z };
}

template<typename R>
__device__ __forceinline__ V3<R> scale( V3<R> a, R s )
{
    return { a.x * s, a.y * s, a.z * s };
}

// JN(x)^T lam for the normalisation x -> x / |x| (symmetric Jacobian)
template<typename R>
__device__ __forceinline__ V3<R> jn_t( V3<R> x, V3<R> lam )
{
    const R n2 = dot( x, x );
    if( !( n2 > R( 0 ) ) )
        return lam;
    const R inv = R( 1 ) / sqrt( n2 );
    const V3<R> xh = scale( x, inv );
    const R d = dot( xh, lam );
    return { ( lam.x - d * xh.x ) * inv, ( lam.y - d * xh.y ) * inv, ( lam.z - d * xh.z ) * inv };
}

template<typename R>
__device__ __forceinline__ void setup_block( const SysDesc & d, PairR<R> * pairs, SysConst<R> & C, Geo & GS )
{
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    __syncthreads();
}

// ------------------------------------------------------------------ forward stage M
template<typename R, int M>
__global__ void __launch_bounds__( 256 ) adj_fwd( AdjArgs<R> A )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    const SysDesc & d = *A.sd;
    setup_block( d, pairs, C, GS );
    const int i      = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < d.nos;
    int ib, a, b, c;
    cell_of( GS, valid ? i : 0, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, valid );
    if( !valid )
        return;
    const long long gi = GS.off + i;
    const V3<R> ci     = A.c[M - 1].ld( gi );
    R e                = 0;
    const V3<R> g      = gradient_at<R>( GS, C, pairs, A.c[M - 1], A.h, gi, ib, a, b, c, ci, C.mu[ib], e, smode );
    const V3<R> fv     = virtual_force<R>( C, ci, g, C.inv_mu[ib], V3<R>{ 0, 0, 0 } );
    if( A.record )
    {
        A.f[M - 1].st( gi, fv );
        A.Fo[M - 1].st( gi, V3<R>{ -g.x, -g.y, -g.z } );
    }
    // the engine's RK4 stage arithmetic, in the same order
    const V3<R> cr = cross( ci, fv );
    const V3<R> k  = { R( -1 ) * cr.x, R( -1 ) * cr.y, R( -1 ) * cr.z };
    const V3<R> si = ( M == 1 ) ? ci : A.c[0].ld( gi );
    if( M == 1 )
    {
        V3<R> acc = si;
        R w6      = R( 1.0 / 6.0 );
        acc.x += w6 * k.x;
        acc.y += w6 * k.y;
        acc.z += w6 * k.z;
        A.acc.st( gi, acc );
        V3<R> p = { si.x + R( 0.5 ) * k.x, si.y + R( 0.5 ) * k.y, si.z + R( 0.5 ) * k.z };
        if( A.record )
            A.p[1].st( gi, p );
        A.c[1].st( gi, normalized( p ) );
    }
    else if( M == 2 || M == 3 )
    {
        V3<R> acc = A.acc.ld( gi );
        R w3      = R( 1.0 / 3.0 );
        acc.x += w3 * k.x;
        acc.y += w3 * k.y;
        acc.z += w3 * k.z;
        A.acc.st( gi, acc );
        R wn    = M == 2 ? R( 0.5 ) : R( 1 );
        V3<R> p = { si.x + wn * k.x, si.y + wn * k.y, si.z + wn * k.z };
        if( A.record )
            A.p[M].st( gi, p );
        A.c[M].st( gi, normalized( p ) );
    }
    else
    {
        V3<R> acc = A.acc.ld( gi );
        R w6      = R( 1.0 / 6.0 );
        acc.x += w6 * k.x;
        acc.y += w6 * k.y;
        acc.z += w6 * k.z;
        if( A.record )
            A.acc.st( gi, acc );
        A.s_out.st( gi, normalized( acc ) );
    }
}

// per-block sums of up to 5 values into pgrad[q * n_blocks + blockIdx.x] (deterministic order)
template<typename R>
__device__ __forceinline__ void block_accumulate( const AdjArgs<R> & A, const R * v, int q0, int nq, double * sh )
{
    for( int q = 0; q < nq; ++q )
    {
        const double s = block_sum_w( v[q], sh );
        if( threadIdx.x == 0 )
            A.pgrad[(size_t)( q0 + q ) * A.n_blocks + blockIdx.x] += s;
        __syncthreads();
    }
}

// Local part of the adjoint of stage m for one spin: from lam_k(m) to lam_Fo(m) (input of the
// transposed field, stored in lam_Fo[m % 2]) and the local part of lam_c(m) (stored); returns the
// spin's dLoss/dalpha contribution.
template<typename R>
__device__ __forceinline__ R stage_local( const AdjArgs<R> & A, const SysConst<R> & C, int m, long long gi, int ib,
                                          V3<R> lk )
{
    const V3<R> cm  = A.c[m - 1].ld( gi );
    const V3<R> fm  = A.f[m - 1].ld( gi );
    const V3<R> Fo  = A.Fo[m - 1].ld( gi );
    const R imu     = C.inv_mu[ib];
    V3<R> lc        = cross( lk, fm );
    const V3<R> lf  = cross( cm, lk );
    const V3<R> lfc = cross( lf, cm );
    const V3<R> lFo = { ( C.dtg * lf.x + C.dtga * lfc.x ) * imu, ( C.dtg * lf.y + C.dtga * lfc.y ) * imu,
                        ( C.dtg * lf.z + C.dtga * lfc.z ) * imu };
    const V3<R> Fl  = cross( Fo, lf );
    lc.x += C.dtga * imu * Fl.x;
    lc.y += C.dtga * imu * Fl.y;
    lc.z += C.dtga * imu * Fl.z;
    A.lam_Fo[m & 1].st( gi, lFo );
    A.lam_c.st( gi, lc );
    const R a2     = C.alpha * C.alpha;
    const V3<R> cF = cross( cm, Fo );
    const R sc     = C.dtg * imu / ( R( 1 ) + a2 );
    const V3<R> da = { sc * ( R( -2 ) * C.alpha * Fo.x + ( R( 1 ) - a2 ) * cF.x ),
                       sc * ( R( -2 ) * C.alpha * Fo.y + ( R( 1 ) - a2 ) * cF.y ),
                       sc * ( R( -2 ) * C.alpha * Fo.z + ( R( 1 ) - a2 ) * cF.z ) };
    return dot( lf, da );
}

// ------------------------------------------------------------------ backward: final normalisation + stage 4 local
template<typename R>
__global__ void __launch_bounds__( 256 ) adj_final( AdjArgs<R> A )
{
    __shared__ SysConst<R> C;
    __shared__ double red[32];
    const SysDesc & d = *A.sd;
    load_const( C, d );
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    R galpha    = 0;
    if( i < d.nos )
    {
        const long long gi = d.spin_offset + i;
        const V3<R> la     = jn_t( A.acc.ld( gi ), A.lam_next.ld( gi ) );
        const R w6 = R( 1.0 / 6.0 ), w3 = R( 1.0 / 3.0 );
        A.lam_s.st( gi, la );
        A.lam_k[2].st( gi, scale( la, w3 ) );
        A.lam_k[1].st( gi, scale( la, w3 ) );
        A.lam_k[0].st( gi, scale( la, w6 ) );
        galpha = stage_local( A, C, 4, gi, i % d.nb, scale( la, w6 ) );
    }
    block_accumulate( A, &galpha, 4, 1, red );
}

// ------------------------------------------------------------------ backward stage M, part 2
// lam_c -= L lam_Fo (stencil + anisotropy + dipolar field of lam_Fo in A.h), dLoss/d(J, D, K, B),
// then through the normalisation of c_m into lam_s and lam_k(M-1).
template<typename R, int M>
__global__ void __launch_bounds__( 256 ) adj_c( AdjArgs<R> A )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red[32];
    const SysDesc & d = *A.sd;
    setup_block( d, pairs, C, GS );
    const int i      = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < d.nos;
    int ib, a, b, c;
    cell_of( GS, valid ? i : 0, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, valid );
    R gp[5]         = { 0, 0, 0, 0, 0 }; // J, D, K, B, alpha (of stage M - 1)
    if( valid )
    {
        const long long gi = GS.off + i;
        const V3<R> lF     = A.lam_Fo[M & 1].ld( gi );
        const V3<R> cm     = A.c[M - 1].ld( gi );
        V3<R> Ll           = { 0, 0, 0 }; // -L lam_Fo
        // anisotropy
        for( int k = 0; k < C.n_aniso; ++k )
            if( C.aniso_idx[k] == ib )
            {
                const V3<R> n = { C.aniso_n[k][0], C.aniso_n[k][1], C.aniso_n[k][2] };
                const R sl    = R( 2 ) * C.aniso_K[k] * dot( n, lF );
                Ll.x += sl * n.x;
                Ll.y += sl * n.y;
                Ll.z += sl * n.z;
                gp[2] += R( 2 ) * A.u.Khat[k] * dot( n, cm ) * dot( n, lF );
            }
        // pairs: -L lam = sum_p (J_p lam_j + lam_j x D_p); parameter sums from c_j
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
            const V3<R> lj = A.lam_Fo[M & 1].ld( j );
            const V3<R> cj = A.c[M - 1].ld( j );
            const V3<R> D  = { P.Dx, P.Dy, P.Dz };
            const V3<R> lx = cross( lj, D );
            Ll.x += P.J * lj.x + lx.x;
            Ll.y += P.J * lj.y + lx.y;
            Ll.z += P.J * lj.z + lx.z;
            gp[0] += A.u.Jhat[q] * dot( lF, cj );
            const V3<R> Du = { A.u.Dhat[q][0], A.u.Dhat[q][1], A.u.Dhat[q][2] };
            gp[1] += dot( lF, cross( cj, Du ) );
        }
        // dipolar: g -= mu h(lam)  ->  -L lam += mu h
        const R mu = C.mu[ib];
        if( A.h.x )
        {
            const V3<R> hh = A.h.ld( gi );
            Ll.x += mu * hh.x;
            Ll.y += mu * hh.y;
            Ll.z += mu * hh.z;
        }
        gp[3] = mu * ( lF.x * A.u.Bn[0] + lF.y * A.u.Bn[1] + lF.z * A.u.Bn[2] );
        V3<R> lc = A.lam_c.ld( gi );
        lc.x += Ll.x;
        lc.y += Ll.y;
        lc.z += Ll.z;
        V3<R> ls = A.lam_s.ld( gi );
        if( M > 1 )
        {
            const V3<R> lp = jn_t( A.p[M - 1].ld( gi ), lc );
            ls             = operator_add( ls, lp );
            const R w      = ( M == 4 ) ? R( 1 ) : R( 0.5 );
            V3<R> lk       = A.lam_k[M - 2].ld( gi );
            lk.x += w * lp.x;
            lk.y += w * lp.y;
            lk.z += w * lp.z;
            // stage M - 1 starts here: its lam_k is final
            gp[4] = stage_local( A, C, M - 1, gi, ib, lk );
        }
        else
            ls = operator_add( ls, lc );
        A.lam_s.st( gi, ls );
    }
    block_accumulate( A, gp, 0, M > 1 ? 5 : 4, red );
}

// ================================================================== host driver
template<typename R>
static SoA3<R> soa_at( void * base, size_t total, size_t slot )
{
    R * p = static_cast<R *>( base ) + slot * 3 * total;
    return { p, p + total, p + 2 * total };
}

template<typename R>
struct AdjPlan
{
    size_t total = 0; // padded length of every component array
    int n_blocks = 0;
    // per recorded step: 16 slots (c0..c3, f0..f3, Fo0..Fo3, p1..p3, acc)
    static constexpr int SLOTS = 16;
    void * pool  = nullptr; // [k][SLOTS][3][total]
    void * work  = nullptr; // unrecorded forward: c0..c3, acc, s_out (6 slots) + adjoint: lam_next, lam_s,
                            // lam_k0..3, lam_Fo (2), lam_c (9 slots)
    void * ckpt  = nullptr; // [n_ckpt][3][total]
    double * pgrad = nullptr;

    // flip: the unrecorded state slots c0 / s_out and the adjoint slots lam_next / lam_s trade
    // places (ping-pong between steps instead of copying)
    AdjArgs<R> step_args( const SysDesc * sd, const AdjUnits<R> & u, int slot_base_step, bool recorded,
                          int flip_state = 0, int flip_lam = 0 ) const
    {
        AdjArgs<R> A{};
        A.sd       = sd;
        A.u        = u;
        A.pgrad    = pgrad;
        A.n_blocks = n_blocks;
        if( recorded )
        {
            const size_t b = (size_t)slot_base_step * SLOTS;
            for( int m = 0; m < 4; ++m )
            {
                A.c[m]  = soa_at<R>( pool, total, b + m );
                A.f[m]  = soa_at<R>( pool, total, b + 4 + m );
                A.Fo[m] = soa_at<R>( pool, total, b + 8 + m );
            }
            for( int m = 1; m < 4; ++m )
                A.p[m] = soa_at<R>( pool, total, b + 11 + m );
            A.acc    = soa_at<R>( pool, total, b + 15 );
            A.record = 1;
        }
        else
        {
            for( int m = 0; m < 4; ++m )
                A.c[m] = soa_at<R>( work, total, m );
            A.c[0]   = soa_at<R>( work, total, flip_state ? 5 : 0 );
            A.acc    = soa_at<R>( work, total, 4 );
            A.s_out  = soa_at<R>( work, total, flip_state ? 0 : 5 );
            A.record = 0;
        }
        A.lam_next = soa_at<R>( work, total, flip_lam ? 7 : 6 );
        A.lam_s    = soa_at<R>( work, total, flip_lam ? 6 : 7 );
        for( int m = 0; m < 4; ++m )
            A.lam_k[m] = soa_at<R>( work, total, 8 + m );
        A.lam_Fo[0] = soa_at<R>( work, total, 12 );
        A.lam_Fo[1] = soa_at<R>( work, total, 14 );
        A.lam_c     = soa_at<R>( work, total, 13 );
        return A;
    }
};

template<typename R>
static void copy3( SoA3<R> dst, SoA3<R> src, size_t n, cudaStream_t st )
{
    CUDA_CHECK( cudaMemcpyAsync( dst.x, src.x, n * sizeof( R ), cudaMemcpyDeviceToDevice, st ) );
    CUDA_CHECK( cudaMemcpyAsync( dst.y, src.y, n * sizeof( R ), cudaMemcpyDeviceToDevice, st ) );
    CUDA_CHECK( cudaMemcpyAsync( dst.z, src.z, n * sizeof( R ), cudaMemcpyDeviceToDevice, st ) );
}

// one forward RK4 step of A (c[0] -> s_out, or into the recorded slots); with a lane, on the
// lane's dipolar plan and field arrays (st is then the lane's stream)
template<typename R>
static void forward_step( Engine & E, AdjArgs<R> A, int nblk, cudaStream_t st, Engine::DdiLane * lane = nullptr )
{
    void * hf[3] = { E.field_ptr( 0 ), E.field_ptr( 1 ), E.field_ptr( 2 ) };
    if( lane )
        for( int c = 0; c < 3; ++c )
            hf[c] = lane->field[c];
    A.h        = E.has_ddi() ? SoA3<R>{ (R *)hf[0], (R *)hf[1], (R *)hf[2] } : SoA3<R>{ nullptr, nullptr, nullptr };
    auto field = [&]( const SoA3<R> & cfg ) {
        if( lane )
            lane->plan.run( E.d_desc(), nullptr, cfg.x, cfg.y, cfg.z, hf[0], hf[1], hf[2], st );
        else if( E.has_ddi() )
        {
            void * cp[3] = { cfg.x, cfg.y, cfg.z };
            E.run_ddi( cp, nullptr );
        }
    };
    field( A.c[0] );
    adj_fwd<R, 1><<<nblk, 256, 0, st>>>( A );
    field( A.c[1] );
    adj_fwd<R, 2><<<nblk, 256, 0, st>>>( A );
    field( A.c[2] );
    adj_fwd<R, 3><<<nblk, 256, 0, st>>>( A );
    field( A.c[3] );
    adj_fwd<R, 4><<<nblk, 256, 0, st>>>( A );
    CUDA_CHECK( cudaGetLastError() );
}

template<typename R>
static void backward_step( Engine & E, AdjArgs<R> A, int nblk, cudaStream_t st )
{
    void * hf[3] = { E.field_ptr( 0 ), E.field_ptr( 1 ), E.field_ptr( 2 ) };
    A.h          = E.has_ddi() ? SoA3<R>{ (R *)hf[0], (R *)hf[1], (R *)hf[2] } : SoA3<R>{ nullptr, nullptr, nullptr };
    auto field   = [&]( int m ) {
        if( E.has_ddi() )
        {
            void * cp[3] = { A.lam_Fo[m & 1].x, A.lam_Fo[m & 1].y, A.lam_Fo[m & 1].z };
            E.run_ddi( cp, nullptr );
        }
    };
    adj_final<R><<<nblk, 256, 0, st>>>( A );
    field( 4 );
    adj_c<R, 4><<<nblk, 256, 0, st>>>( A );
    field( 3 );
    adj_c<R, 3><<<nblk, 256, 0, st>>>( A );
    field( 2 );
    adj_c<R, 2><<<nblk, 256, 0, st>>>( A );
    field( 1 );
    adj_c<R, 1><<<nblk, 256, 0, st>>>( A );
    CUDA_CHECK( cudaGetLastError() );
}

template<typename R>
static AdjUnits<R> make_units( const AdjointInput & in )
{
    AdjUnits<R> u{};
    for( int q = 0; q < in.unit_J.n_pairs && q < MAX_PAIRS; ++q )
    {
        u.Jhat[q] = (R)in.unit_J.pairs[q].J;
        for( int e = 0; e < 3; ++e )
            u.Dhat[q][e] = (R)in.unit_D.pairs[q].D[e];
    }
    for( int k = 0; k < in.unit_J.n_aniso && k < MAX_BASIS; ++k )
        u.Khat[k] = (R)in.unit_K[k];
    for( int e = 0; e < 3; ++e )
        u.Bn[e] = (R)in.unit_B[e];
    return u;
}

template<typename R>
static double run_t( Engine & E, const AdjointInput & in, AdjointOutput & out )
{
    const SysDesc & d   = E.desc( 0 );
    const int nos       = d.nos;
    const size_t total  = ( (size_t)nos + SPIN_ALIGN - 1 ) / SPIN_ALIGN * SPIN_ALIGN + d.spin_offset;
    const int nblk      = ( nos + 255 ) / 256;
    const int K         = std::max( 1, std::min( in.checkpoint, std::max( 1, in.n_steps ) ) );
    const int n_ckpt    = ( in.n_steps + K - 1 ) / K + 1;
    cudaStream_t st     = E.stream();
    AdjPlan<R> P;
    P.total    = total;
    P.n_blocks = nblk;
    // Backward pass as a two-stream pipeline when there are several segments: the recomputation
    // of segment s - 1 (from its checkpoint, on a second stream with its own dipolar lane) runs
    // beside the adjoint steps of segment s; the recorded pool then has two halves of K steps.
    const int n_seg     = in.n_steps > 0 ? ( in.n_steps - 1 ) / K + 1 : 0;
    const char * penv   = std::getenv( "SPIRIT_GB300_ADJ_PIPE" );
    const bool pipe     = in.gradients && n_seg >= 2 && !( penv && penv[0] == '0' );
    Engine::DdiLane * lane = pipe ? E.ddi_lane() : nullptr;
    cudaStream_t st2       = pipe ? ( lane ? lane->stream : nullptr ) : nullptr;
    cudaStream_t own_st2   = nullptr;
    if( pipe && !st2 )
    {
        CUDA_CHECK( cudaStreamCreateWithFlags( &own_st2, cudaStreamNonBlocking ) );
        st2 = own_st2;
    }
    P.pool     = in.gradients ? dalloc_bytes( (size_t)( pipe ? 2 : 1 ) * K * AdjPlan<R>::SLOTS * 3 * total * sizeof( R ) )
                              : nullptr;
    P.work     = dalloc_bytes( (size_t)15 * 3 * total * sizeof( R ) );
    P.ckpt     = dalloc_bytes( (size_t)n_ckpt * 3 * total * sizeof( R ) );
    P.pgrad    = dalloc<double>( (size_t)5 * nblk );
    const AdjUnits<R> u  = make_units<R>( in );
    const SysDesc * d_sd = E.d_desc();
    double loss          = 0;
    try
    {
        // s0 (AoS FP64 host) -> work c0
        std::vector<R> soa( 3 * total, R( 0 ) );
        for( int i = 0; i < nos; ++i )
            for( int e = 0; e < 3; ++e )
                soa[e * total + d.spin_offset + i] = (R)in.s0[3 * (size_t)i + e];
        int fs       = 0; // which of the two unrecorded state slots holds the current state
        AdjArgs<R> W = P.step_args( d_sd, u, 0, false, fs );
        CUDA_CHECK( cudaMemcpyAsync( W.c[0].x, soa.data(), 3 * total * sizeof( R ), cudaMemcpyHostToDevice, st ) );
        // forward with checkpoints; with gradients, the last segment is recorded right away (the
        // backward pass then recomputes every segment but that one)
        const int last0 = in.n_steps > 0 ? ( ( in.n_steps - 1 ) / K ) * K : 0;
        for( int n = 0; n < in.n_steps; ++n )
        {
            W = P.step_args( d_sd, u, 0, false, fs );
            if( n % K == 0 )
                copy3( soa_at<R>( P.ckpt, total, n / K ), W.c[0], total, st );
            if( in.gradients && n >= last0 )
            {
                AdjArgs<R> A = P.step_args( d_sd, u, n - last0, true );
                if( n == last0 )
                    copy3( A.c[0], W.c[0], total, st );
                A.s_out = n + 1 < in.n_steps ? P.step_args( d_sd, u, n + 1 - last0, true ).c[0] : W.c[0];
                forward_step<R>( E, A, nblk, st );
            }
            else
            {
                forward_step<R>( E, W, nblk, st );
                fs ^= 1; // the new state is in the other slot
            }
        }
        W = P.step_args( d_sd, u, 0, false, fs );
        std::vector<R> fin( 3 * total );
        CUDA_CHECK( cudaMemcpyAsync( fin.data(), W.c[0].x, 3 * total * sizeof( R ), cudaMemcpyDeviceToHost, st ) );
        CUDA_CHECK( cudaStreamSynchronize( st ) );
        // loss = mean_i |s_i - t_i|^2 (FP64), lam_T = 2 (s - t) / N
        std::vector<R> lam( 3 * total, R( 0 ) );
        for( int i = 0; i < nos; ++i )
            for( int e = 0; e < 3; ++e )
            {
                const double sv = (double)fin[e * total + d.spin_offset + i];
                const double dv = sv - in.target[3 * (size_t)i + e];
                loss += dv * dv;
                lam[e * total + d.spin_offset + i] = (R)( 2.0 * dv / nos );
                if( out.final_spins )
                    out.final_spins[3 * (size_t)i + e] = sv;
            }
        loss /= nos;
        if( in.gradients )
        {
            CUDA_CHECK( cudaMemsetAsync( P.pgrad, 0, (size_t)5 * nblk * sizeof( double ), st ) );
            int fl = 1; // lam_s of flip 0 holds dLoss/ds_T: the first backward step reads it as lam_next
            CUDA_CHECK( cudaMemcpyAsync( P.step_args( d_sd, u, 0, false, 0, 0 ).lam_s.x, lam.data(),
                                         3 * total * sizeof( R ), cudaMemcpyHostToDevice, st ) );
            const int L = n_seg - 1; // the last segment, recorded by the forward pass into half 0
            auto half   = [&]( int seg ) { return pipe ? ( L - seg ) & 1 : 0; };
            // recompute segment seg from its checkpoint, recording every stage of its steps
            auto recompute = [&]( int seg, cudaStream_t s, Engine::DdiLane * ln ) {
                const int n0 = seg * K, n1 = std::min( in.n_steps, n0 + K ), hb = half( seg ) * K;
                copy3( P.step_args( d_sd, u, hb, true ).c[0], soa_at<R>( P.ckpt, total, seg ), total, s );
                for( int n = n0; n < n1; ++n )
                {
                    AdjArgs<R> A = P.step_args( d_sd, u, hb + n - n0, true );
                    if( n + 1 < n1 )
                        A.s_out = P.step_args( d_sd, u, hb + n + 1 - n0, true ).c[0];
                    else
                        A.s_out = P.step_args( d_sd, u, 0, false, fs ).s_out; // not needed further
                    forward_step<R>( E, A, nblk, s, ln );
                }
            };
            cudaEvent_t ev_rec = nullptr, ev_bwd = nullptr;
            if( pipe )
            {
                CUDA_CHECK( cudaEventCreateWithFlags( &ev_rec, cudaEventDisableTiming ) );
                CUDA_CHECK( cudaEventCreateWithFlags( &ev_bwd, cudaEventDisableTiming ) );
                // the checkpoints are written on the main stream
                CUDA_CHECK( cudaEventRecord( ev_bwd, st ) );
            }
            try
            {
                for( int seg = L; seg >= 0; --seg )
                {
                    const int n0 = seg * K, n1 = std::min( in.n_steps, n0 + K ), hb = half( seg ) * K;
                    if( pipe )
                    {
                        // segment seg was recomputed on the second stream (the last one: recorded)
                        if( seg != L )
                            CUDA_CHECK( cudaStreamWaitEvent( st, ev_rec, 0 ) );
                        // segment seg - 1 into the other half, once the adjoint of seg + 1 is done with it
                        if( seg >= 1 )
                        {
                            CUDA_CHECK( cudaStreamWaitEvent( st2, ev_bwd, 0 ) );
                            recompute( seg - 1, st2, lane );
                            CUDA_CHECK( cudaGetLastError() );
                            CUDA_CHECK( cudaEventRecord( ev_rec, st2 ) );
                        }
                    }
                    else if( n0 != last0 )
                        recompute( seg, st, nullptr );
                    // adjoint steps of the segment in reverse: lam_next holds dLoss/ds_{n+1} on entry
                    for( int n = n1 - 1; n >= n0; --n )
                    {
                        AdjArgs<R> A = P.step_args( d_sd, u, hb + n - n0, true, 0, fl );
                        backward_step<R>( E, A, nblk, st );
                        fl ^= 1; // lam_s of this step is lam_next of the previous one
                    }
                    if( pipe )
                        CUDA_CHECK( cudaEventRecord( ev_bwd, st ) );
                }
            }
            catch( ... )
            {
                if( pipe )
                {
                    cudaStreamSynchronize( st2 );
                    cudaEventDestroy( ev_rec );
                    cudaEventDestroy( ev_bwd );
                }
                throw;
            }
            if( pipe )
            {
                CUDA_CHECK( cudaEventDestroy( ev_rec ) );
                CUDA_CHECK( cudaEventDestroy( ev_bwd ) );
            }
            std::vector<R> g0( 3 * total );
            std::vector<double> pg( (size_t)5 * nblk );
            const SoA3<R> g_last = P.step_args( d_sd, u, 0, false, 0, fl ^ 1 ).lam_s;
            CUDA_CHECK( cudaMemcpyAsync( g0.data(), g_last.x, 3 * total * sizeof( R ), cudaMemcpyDeviceToHost, st ) );
            CUDA_CHECK( cudaMemcpyAsync( pg.data(), P.pgrad, pg.size() * sizeof( double ), cudaMemcpyDeviceToHost, st ) );
            CUDA_CHECK( cudaStreamSynchronize( st ) );
            if( out.grad_s0 )
                for( int i = 0; i < nos; ++i )
                    for( int e = 0; e < 3; ++e )
                        out.grad_s0[3 * (size_t)i + e] = (double)g0[e * total + d.spin_offset + i];
            for( int q = 0; q < 5; ++q )
            {
                double s = 0;
                for( int b = 0; b < nblk; ++b )
                    s += pg[(size_t)q * nblk + b];
                out.grad_params[q] = s;
            }
        }
    }
    catch( ... )
    {
        if( st2 )
            cudaStreamSynchronize( st2 );
        cudaStreamSynchronize( st );
        if( own_st2 )
            cudaStreamDestroy( own_st2 );
        dfree( P.pool );
        dfree( P.work );
        dfree( P.ckpt );
        dfree( P.pgrad );
        throw;
    }
    if( own_st2 )
        CUDA_CHECK( cudaStreamDestroy( own_st2 ) );
    dfree( P.pool );
    dfree( P.work );
    dfree( P.ckpt );
    dfree( P.pgrad );
    return loss;
}

double adjoint_run( Engine & E, const AdjointInput & in, AdjointOutput & out, bool fp64 )
{
    if( in.n_steps < 0 )
        throw std::runtime_error( "negative number of steps" );
    const SysDesc & d = E.desc( 0 );
    if( d.temperature != 0.0 || d.direct_minimization )
        throw std::runtime_error( "the adjoint covers deterministic dynamics only (T = 0, no direct minimisation)" );
    return fp64 ? run_t<double>( E, in, out ) : run_t<float>( E, in, out );
}

} // namespace sg
