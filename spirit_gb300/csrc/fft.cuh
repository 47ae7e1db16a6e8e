// Hand-written batched mixed-radix Stockham FFT for the dipole-dipole convolution.
//
// The reference computes the dipolar gradient as a zero-padded 3D convolution through
// kissFFT / cuFFT (core/src/engine/Hamiltonian_Heisenberg.cpp:920-1014, FFT.cu:23-80):
//     g_i -= mu_i * (1/T) IFFT( sum_b2 Dhat_{b1 b2}(k) . FFT(mu s)_{b2}(k) )
// Here the 3D transform is split into 1D passes along a (real-to-complex, half length),
// b and c, each done by a CTA on a group of lines held in shared memory:
//     A : R2C along a of every nonzero (b, c) row of mu*s        (zero padding is implicit)
//     B : C2C along b of every (ka, c) column, rows b >= Nb are implicit zeros
//     C : C2C along c, 6-component symmetric tensor product with Dhat, inverse along c;
//         only c < Nc of the result is kept (the padded half is never written)
//     B': inverse along b, only b < Nb kept
//     A': C2R along a, only a < Na kept, scaled by 1/T, written as the field h = D * (mu s)
// so the padded volume is never materialised.  Twiddles come from a table of exp(-2 pi i t / L)
// computed in FP64 on the host.
#pragma once
#include "common.hpp"

#include <cuda_runtime.h>

namespace sg
{

template<typename R>
struct cplx
{
    R x, y;
};

template<typename R>
__device__ __forceinline__ cplx<R> cmul( cplx<R> a, cplx<R> b )
{
    // explicit rounding: one product rounded, the other fused, the same in every kernel that
    // inlines the transform (left to the compiler, the choice of the fused product can differ
    // between kernels, and so would the transforms of the row-fused stages and of pass A / A')
    if constexpr( sizeof( R ) == 4 )
        return { __fmaf_rn( a.x, b.x, -__fmul_rn( a.y, b.y ) ), __fmaf_rn( a.x, b.y, __fmul_rn( a.y, b.x ) ) };
    else
        return { __fma_rn( a.x, b.x, -__dmul_rn( a.y, b.y ) ), __fma_rn( a.x, b.y, __dmul_rn( a.y, b.x ) ) };
}
template<typename R>
__device__ __forceinline__ cplx<R> cconj( cplx<R> a )
{
    return { a.x, -a.y };
}

// ------------------------------------------------------------------ register DFTs (radix 2..16)
// In-register DFT of N = 2, 4, 8, 16 points, X_m = sum_r v_r w^(r m), w = exp(-/+ 2 pi i / N).
// Constants are cos / sin of multiples of pi / 8.
template<typename R>
__device__ __forceinline__ cplx<R> mul_mi( cplx<R> a, bool inverse ) // a * (-i) forward, a * (+i) inverse
{
    return inverse ? cplx<R>{ -a.y, a.x } : cplx<R>{ a.y, -a.x };
}

template<typename R>
__device__ __forceinline__ void dft4( cplx<R> & v0, cplx<R> & v1, cplx<R> & v2, cplx<R> & v3, bool inverse )
{
    const cplx<R> s02 = { v0.x + v2.x, v0.y + v2.y }, d02 = { v0.x - v2.x, v0.y - v2.y };
    const cplx<R> s13 = { v1.x + v3.x, v1.y + v3.y }, d13 = { v1.x - v3.x, v1.y - v3.y };
    const cplx<R> id13 = mul_mi( d13, inverse );
    v0 = { s02.x + s13.x, s02.y + s13.y };
    v1 = { d02.x + id13.x, d02.y + id13.y };
    v2 = { s02.x - s13.x, s02.y - s13.y };
    v3 = { d02.x - id13.x, d02.y - id13.y };
}

// w16^k for k = 0..9 (forward sign), applied as multiplication (conjugated for the inverse)
template<typename R>
__device__ __forceinline__ cplx<R> w16( int k, bool inverse )
{
    const R c1 = R( 0.92387953251128675613 ), s1 = R( 0.38268343236508977173 ), c2 = R( 0.70710678118654752440 );
    cplx<R> w;
    switch( k )
    {
    case 0: w = { R( 1 ), R( 0 ) }; break;
    case 1: w = { c1, -s1 }; break;
    case 2: w = { c2, -c2 }; break;
    case 3: w = { s1, -c1 }; break;
    case 4: w = { R( 0 ), R( -1 ) }; break;
    case 6: w = { -c2, -c2 }; break;
    default: w = { -c1, s1 }; break; // k = 9
    }
    if( inverse )
        w.y = -w.y;
    return w;
}

template<typename R, int N>
__device__ __forceinline__ void dft_reg( cplx<R> * v, bool inverse )
{
    if constexpr( N == 2 )
    {
        const cplx<R> a = v[0], b = v[1];
        v[0] = { a.x + b.x, a.y + b.y };
        v[1] = { a.x - b.x, a.y - b.y };
    }
    else if constexpr( N == 4 )
        dft4( v[0], v[1], v[2], v[3], inverse );
    else if constexpr( N == 8 )
    {
        // two 4-point DFTs (even, odd inputs), then X_m = E_m + w8^m O_m, X_{m+4} = E_m - w8^m O_m
        cplx<R> e[4] = { v[0], v[2], v[4], v[6] }, o[4] = { v[1], v[3], v[5], v[7] };
        dft4( e[0], e[1], e[2], e[3], inverse );
        dft4( o[0], o[1], o[2], o[3], inverse );
        const R c2 = R( 0.70710678118654752440 );
        const cplx<R> t0 = o[0];
        const cplx<R> t1 = inverse ? cplx<R>{ c2 * ( o[1].x - o[1].y ), c2 * ( o[1].x + o[1].y ) }
                                   : cplx<R>{ c2 * ( o[1].x + o[1].y ), c2 * ( o[1].y - o[1].x ) };
        const cplx<R> t2 = mul_mi( o[2], inverse );
        const cplx<R> t3 = inverse ? cplx<R>{ -c2 * ( o[3].x + o[3].y ), c2 * ( o[3].x - o[3].y ) }
                                   : cplx<R>{ c2 * ( o[3].y - o[3].x ), -c2 * ( o[3].x + o[3].y ) };
        const cplx<R> t[4] = { t0, t1, t2, t3 };
#pragma unroll
        for( int m = 0; m < 4; ++m )
        {
            v[m]     = { e[m].x + t[m].x, e[m].y + t[m].y };
            v[m + 4] = { e[m].x - t[m].x, e[m].y - t[m].y };
        }
    }
    else
    {
        static_assert( N == 16, "radix 2, 4, 8 or 16" );
        // r = r1 + 4 r2:  Y[r1][m2] = DFT4_r2 v[r1 + 4 r2],  Y *= w16^(r1 m2),  X[m2 + 4 m1] = DFT4_r1 Y
        cplx<R> y[16];
#pragma unroll
        for( int r1 = 0; r1 < 4; ++r1 )
        {
            cplx<R> a0 = v[r1], a1 = v[r1 + 4], a2 = v[r1 + 8], a3 = v[r1 + 12];
            dft4( a0, a1, a2, a3, inverse );
            y[r1 * 4 + 0] = a0;
            y[r1 * 4 + 1] = r1 == 0 ? a1 : cmul( a1, w16<R>( r1, inverse ) );
            y[r1 * 4 + 2] = r1 == 0 ? a2 : cmul( a2, w16<R>( 2 * r1, inverse ) );
            y[r1 * 4 + 3] = r1 == 0 ? a3 : cmul( a3, w16<R>( 3 * r1, inverse ) );
        }
#pragma unroll
        for( int m2 = 0; m2 < 4; ++m2 )
        {
            cplx<R> b0 = y[0 * 4 + m2], b1 = y[1 * 4 + m2], b2 = y[2 * 4 + m2], b3 = y[3 * 4 + m2];
            dft4( b0, b1, b2, b3, inverse );
            v[m2]      = b0;
            v[m2 + 4]  = b1;
            v[m2 + 8]  = b2;
            v[m2 + 12] = b3;
        }
    }
}

// One Stockham stage of radix 2^LGR on lines of length 2^LGL (Ns = 2^LGNS), lines at l*ls,
// elements at t*es.  Twiddles: tw[t] = exp(-2 pi i t / L).
template<typename R, int LGL, int LGNS, int LGR, bool LINE_FAST>
__device__ __forceinline__ void stockham_stage( const cplx<R> * a, cplx<R> * b, int nl, const FastDiv & dnl, int ls,
                                               int es, const cplx<R> * tw, bool inverse )
{
    constexpr int RR   = 1 << LGR;
    constexpr int LGLR = LGL - LGR;
    constexpr int LR   = 1 << LGLR;
    constexpr int NS   = 1 << LGNS;
    constexpr int LGSP = LGL - LGNS - LGR;
    for( int idx = threadIdx.x; idx < ( nl << LGLR ); idx += blockDim.x )
    {
        int line, j;
        if( LINE_FAST )
        {
            j    = (int)fdiv( (unsigned)idx, dnl );
            line = idx - j * nl;
        }
        else
        {
            line = idx >> LGLR;
            j    = idx & ( LR - 1 );
        }
        const cplx<R> * src = a + line * ls;
        cplx<R> * dst       = b + line * ls;
        const int k         = j & ( NS - 1 );
        cplx<R> v[RR];
#pragma unroll
        for( int r = 0; r < RR; ++r )
        {
            const cplx<R> x = src[( j + r * LR ) * es];
            if( r == 0 || LGNS == 0 )
                v[r] = x;
            else
            {
                cplx<R> w = tw[( r * k ) << LGSP];
                if( inverse )
                    w.y = -w.y;
                v[r] = cmul( x, w );
            }
        }
        dft_reg<R, RR>( v, inverse );
        const int d0 = ( ( j >> LGNS ) << ( LGNS + LGR ) ) + k;
#pragma unroll
        for( int m = 0; m < RR; ++m )
            dst[( d0 + m * NS ) * es] = v[m];
    }
}

// Stockham FFT of length 2^LGL with radix-2^MAXLG register stages (the last stage takes the
// remainder).  Returns the buffer holding the result.
template<typename R, int LGL, int LGNS, int MAXLG, bool LINE_FAST>
__device__ __forceinline__ cplx<R> * stockham_reg( cplx<R> * a, cplx<R> * b, int nl, const FastDiv & dnl, int ls,
                                                  int es, const cplx<R> * tw, bool inverse )
{
    if constexpr( LGNS >= LGL )
        return a;
    else
    {
        constexpr int LGR = ( LGL - LGNS ) >= MAXLG ? MAXLG : ( LGL - LGNS );
        stockham_stage<R, LGL, LGNS, LGR, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
        __syncthreads();
        return stockham_reg<R, LGL, LGNS + LGR, MAXLG, LINE_FAST>( b, a, nl, dnl, ls, es, tw, inverse );
    }
}

// largest register radix: 8.  Radix 16 needs fewer shared-memory round trips but a quarter of the
// threads per line; the lines here are short and few per block, and radix 8 measured faster on
// the 128x128x16 dipolar workload (interleaved runs, ms/step: radix 8 everywhere 0.1035, 0.1037;
// radix 16 0.134, 0.111; radix 4 0.119, 0.106).
template<typename R>
struct MaxRadix
{
    static constexpr int LG = 3;
};


// Power-of-two lines: radix-4 stages (and one radix-2 stage if log2 L is odd) with shift/mask
// index arithmetic.
template<typename R>
__device__ cplx<R> * block_fft_pow2( cplx<R> * a, cplx<R> * b, int L, int ls, int nl, const cplx<R> * tw,
                                    bool inverse )
{
    const int lgL = __ffs( L ) - 1;
    int lgNs      = 0;
    while( lgNs < lgL )
    {
        const int lgR  = ( lgL - lgNs >= 2 ) ? 2 : 1;
        const int lgLR = lgL - lgR;
        const int LR   = 1 << lgLR;
        const int Ns   = 1 << lgNs;
        const int lgSp = lgL - lgNs - lgR;
        for( int idx = threadIdx.x; idx < ( nl << lgLR ); idx += blockDim.x )
        {
            const int line     = idx >> lgLR;
            const int j        = idx & ( LR - 1 );
            const cplx<R> * src = a + line * ls;
            cplx<R> * dst       = b + line * ls;
            const int k        = j & ( Ns - 1 );
            const int d0       = ( ( j >> lgNs ) << ( lgNs + lgR ) ) + k;
            if( lgR == 1 )
            {
                cplx<R> v0 = src[j];
                cplx<R> w  = tw[k << lgSp];
                if( inverse )
                    w = cconj( w );
                cplx<R> v1   = cmul( src[j + LR], w );
                dst[d0]      = { v0.x + v1.x, v0.y + v1.y };
                dst[d0 + Ns] = { v0.x - v1.x, v0.y - v1.y };
            }
            else
            {
                cplx<R> v[4];
                v[0] = src[j];
#pragma unroll
                for( int r = 1; r < 4; ++r )
                {
                    cplx<R> w = tw[( r * k ) << lgSp];
                    if( inverse )
                        w = cconj( w );
                    v[r] = cmul( src[j + r * LR], w );
                }
                cplx<R> s02  = { v[0].x + v[2].x, v[0].y + v[2].y };
                cplx<R> d02  = { v[0].x - v[2].x, v[0].y - v[2].y };
                cplx<R> s13  = { v[1].x + v[3].x, v[1].y + v[3].y };
                cplx<R> d13  = { v[1].x - v[3].x, v[1].y - v[3].y };
                cplx<R> id13 = inverse ? cplx<R>{ -d13.y, d13.x } : cplx<R>{ d13.y, -d13.x };
                dst[d0]          = { s02.x + s13.x, s02.y + s13.y };
                dst[d0 + Ns]     = { d02.x + id13.x, d02.y + id13.y };
                dst[d0 + 2 * Ns] = { s02.x - s13.x, s02.y - s13.y };
                dst[d0 + 3 * Ns] = { d02.x - id13.x, d02.y - id13.y };
            }
        }
        __syncthreads();
        cplx<R> * t = a;
        a           = b;
        b           = t;
        lgNs += lgR;
    }
    return a;
}

// Compile-time length version of block_fft_pow2 (the common extents 16..1024): constant
// strides and shifts, fully unrolled radix-4 butterflies.
template<typename R, int L>
__device__ __forceinline__ cplx<R> * block_fft_const( cplx<R> * a, cplx<R> * b, int ls, int nl, const cplx<R> * tw,
                                                     bool inverse )
{
    constexpr int lgL = ( L <= 1 ) ? 0 : ( L <= 2 ) ? 1 : ( L <= 4 ) ? 2 : ( L <= 8 ) ? 3 : ( L <= 16 ) ? 4
                        : ( L <= 32 ) ? 5 : ( L <= 64 ) ? 6 : ( L <= 128 ) ? 7 : ( L <= 256 ) ? 8 : ( L <= 512 ) ? 9 : 10;
#pragma unroll
    for( int lgNs = 0; lgNs < lgL; lgNs += 2 )
    {
        const int lgR  = ( lgL - lgNs >= 2 ) ? 2 : 1;
        const int lgLR = lgL - lgR;
        const int LR   = 1 << lgLR;
        const int Ns   = 1 << lgNs;
        const int lgSp = lgL - lgNs - lgR;
        for( int idx = threadIdx.x; idx < ( nl << lgLR ); idx += blockDim.x )
        {
            const int line     = idx >> lgLR;
            const int j        = idx & ( LR - 1 );
            const cplx<R> * src = a + line * ls;
            cplx<R> * dst       = b + line * ls;
            const int k        = j & ( Ns - 1 );
            const int d0       = ( ( j >> lgNs ) << ( lgNs + lgR ) ) + k;
            if( lgR == 1 )
            {
                cplx<R> v0 = src[j];
                cplx<R> w  = tw[k << lgSp];
                if( inverse )
                    w = cconj( w );
                cplx<R> v1   = cmul( src[j + LR], w );
                dst[d0]      = { v0.x + v1.x, v0.y + v1.y };
                dst[d0 + Ns] = { v0.x - v1.x, v0.y - v1.y };
            }
            else
            {
                cplx<R> v0 = src[j];
                cplx<R> w1 = tw[k << lgSp], w2 = tw[( 2 * k ) << lgSp], w3 = tw[( 3 * k ) << lgSp];
                if( inverse )
                {
                    w1 = cconj( w1 );
                    w2 = cconj( w2 );
                    w3 = cconj( w3 );
                }
                cplx<R> v1   = cmul( src[j + LR], w1 );
                cplx<R> v2   = cmul( src[j + 2 * LR], w2 );
                cplx<R> v3   = cmul( src[j + 3 * LR], w3 );
                cplx<R> s02  = { v0.x + v2.x, v0.y + v2.y };
                cplx<R> d02  = { v0.x - v2.x, v0.y - v2.y };
                cplx<R> s13  = { v1.x + v3.x, v1.y + v3.y };
                cplx<R> d13  = { v1.x - v3.x, v1.y - v3.y };
                cplx<R> id13 = inverse ? cplx<R>{ -d13.y, d13.x } : cplx<R>{ d13.y, -d13.x };
                dst[d0]          = { s02.x + s13.x, s02.y + s13.y };
                dst[d0 + Ns]     = { d02.x + id13.x, d02.y + id13.y };
                dst[d0 + 2 * Ns] = { s02.x - s13.x, s02.y - s13.y };
                dst[d0 + 3 * Ns] = { d02.x - id13.x, d02.y - id13.y };
            }
        }
        __syncthreads();
        cplx<R> * t = a;
        a           = b;
        b           = t;
        if( lgR == 1 )
            break; // the radix-2 stage is the last one
    }
    return a;
}

// Stockham stage loop over nl lines of length L in shared memory (a -> b -> a ...); line k
// starts at k * ls (ls = L, or L + 1 for power-of-two lengths to spread shared-memory banks).
// rad: 0-terminated radix list; tw: L twiddles exp(-2 pi i t/L) (in shared memory).
// Returns the buffer that holds the result.  Must be called by all threads of the block.
// power-of-two lines of 2^LGL with register stages of at most 2^MAXLG
template<typename R, int MAXLG>
__device__ __forceinline__ cplx<R> * block_fft_reg( cplx<R> * a, cplx<R> * b, int L, int ls, int nl,
                                                   const cplx<R> * tw, bool inverse, bool & done )
{
    done = true;
    const FastDiv one{ 1, 0, 0 };
    switch( L )
    {
    case 16:
        return stockham_reg<R, 4, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    case 32:
        return stockham_reg<R, 5, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    case 64:
        return stockham_reg<R, 6, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    case 128:
        return stockham_reg<R, 7, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    case 256:
        return stockham_reg<R, 8, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    case 512:
        return stockham_reg<R, 9, 0, MAXLG, false>( a, b, nl, one, ls, 1, tw, inverse );
    default:
        done = false;
        return a;
    }
}

template<typename R>
__device__ __noinline__ cplx<R> * mixed_fft( cplx<R> * a, cplx<R> * b, int L, int nl, int ls, int es,
                                             const RadixPlan & P, const cplx<R> * tw, bool inverse );

template<typename R>
__device__ cplx<R> * block_fft( cplx<R> * a, cplx<R> * b, int L, int ls, int nl, const RadixPlan & P,
                               const cplx<R> * tw, bool inverse )
{
    if( L == 1 )
        return a;
    bool done   = false;
    cplx<R> * r = block_fft_reg<R, MaxRadix<R>::LG>( a, b, L, ls, nl, tw, inverse, done );
    if( done )
        return r;
    if( ( L & ( L - 1 ) ) == 0 )
        return block_fft_pow2( a, b, L, ls, nl, tw, inverse );
    return mixed_fft<R>( a, b, L, nl, L, 1, P, tw, inverse );
}

// ------------------------------------------------------------------ strided line transforms
// Stockham FFT of nl lines in shared memory whose element t of line l sits at l*ls + t*es.
// LINE_FAST: consecutive threads take consecutive lines (for ls = 1, es > 1: a warp then touches
// consecutive words); otherwise consecutive threads take consecutive butterflies of one line.
// dnl = FastDiv of nl (used by LINE_FAST).  Returns the buffer that holds the result; must be
// called by all threads of the block.
template<typename R, int L, bool LINE_FAST>
__device__ __forceinline__ cplx<R> * sfft_const( cplx<R> * a, cplx<R> * b, int nl, const FastDiv & dnl, int ls,
                                                int es, const cplx<R> * tw, bool inverse )
{
    constexpr int lgL = ( L <= 1 ) ? 0 : ( L <= 2 ) ? 1 : ( L <= 4 ) ? 2 : ( L <= 8 ) ? 3 : ( L <= 16 ) ? 4
                        : ( L <= 32 ) ? 5 : ( L <= 64 ) ? 6 : ( L <= 128 ) ? 7 : ( L <= 256 ) ? 8 : ( L <= 512 ) ? 9 : 10;
#pragma unroll
    for( int lgNs = 0; lgNs < lgL; lgNs += 2 )
    {
        const int lgR  = ( lgL - lgNs >= 2 ) ? 2 : 1;
        const int lgLR = lgL - lgR;
        const int LR   = 1 << lgLR;
        const int Ns   = 1 << lgNs;
        const int lgSp = lgL - lgNs - lgR;
        for( int idx = threadIdx.x; idx < ( nl << lgLR ); idx += blockDim.x )
        {
            int line, j;
            if( LINE_FAST )
            {
                j    = (int)fdiv( (unsigned)idx, dnl );
                line = idx - j * nl;
            }
            else
            {
                line = idx >> lgLR;
                j    = idx & ( LR - 1 );
            }
            const cplx<R> * src = a + line * ls;
            cplx<R> * dst       = b + line * ls;
            const int k         = j & ( Ns - 1 );
            const int d0        = ( ( j >> lgNs ) << ( lgNs + lgR ) ) + k;
            if( lgR == 1 )
            {
                cplx<R> v0 = src[j * es];
                cplx<R> w  = tw[k << lgSp];
                if( inverse )
                    w = cconj( w );
                cplx<R> v1          = cmul( src[( j + LR ) * es], w );
                dst[d0 * es]        = { v0.x + v1.x, v0.y + v1.y };
                dst[( d0 + Ns ) * es] = { v0.x - v1.x, v0.y - v1.y };
            }
            else
            {
                cplx<R> v0 = src[j * es];
                cplx<R> w1 = tw[k << lgSp], w2 = tw[( 2 * k ) << lgSp], w3 = tw[( 3 * k ) << lgSp];
                if( inverse )
                {
                    w1 = cconj( w1 );
                    w2 = cconj( w2 );
                    w3 = cconj( w3 );
                }
                cplx<R> v1   = cmul( src[( j + LR ) * es], w1 );
                cplx<R> v2   = cmul( src[( j + 2 * LR ) * es], w2 );
                cplx<R> v3   = cmul( src[( j + 3 * LR ) * es], w3 );
                cplx<R> s02  = { v0.x + v2.x, v0.y + v2.y };
                cplx<R> d02  = { v0.x - v2.x, v0.y - v2.y };
                cplx<R> s13  = { v1.x + v3.x, v1.y + v3.y };
                cplx<R> d13  = { v1.x - v3.x, v1.y - v3.y };
                cplx<R> id13 = inverse ? cplx<R>{ -d13.y, d13.x } : cplx<R>{ d13.y, -d13.x };
                dst[d0 * es]              = { s02.x + s13.x, s02.y + s13.y };
                dst[( d0 + Ns ) * es]     = { d02.x + id13.x, d02.y + id13.y };
                dst[( d0 + 2 * Ns ) * es] = { s02.x - s13.x, s02.y - s13.y };
                dst[( d0 + 3 * Ns ) * es] = { d02.x - id13.x, d02.y - id13.y };
            }
        }
        __syncthreads();
        cplx<R> * t = a;
        a           = b;
        b           = t;
        if( lgR == 1 )
            break; // the radix-2 stage is the last one
    }
    return a;
}

// Element access of a complex line buffer.  GenBuf: through a generic pointer.  SmemBuf: by the
// buffer's 32-bit shared-window address with ld/st.shared of two components, for code that is
// handed generic pointers (a non-inlined function) which it has checked to point into shared
// memory, element-aligned -- it saves the generic-to-shared conversion and the 64-bit address
// arithmetic of every access.
template<typename R>
struct GenBuf
{
    cplx<R> * p;
    __device__ __forceinline__ cplx<R> ld( int i ) const
    {
        return p[i];
    }
    __device__ __forceinline__ void st( int i, cplx<R> v ) const
    {
        p[i] = v;
    }
};

template<typename R>
struct SmemBuf;

template<>
struct SmemBuf<float>
{
    unsigned int base;
    __device__ __forceinline__ cplx<float> ld( int i ) const
    {
        cplx<float> v;
        asm volatile( "ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"( v.x ), "=f"( v.y ) : "r"( base + 8u * (unsigned)i ) : "memory" );
        return v;
    }
    __device__ __forceinline__ void st( int i, cplx<float> v ) const
    {
        asm volatile( "st.shared.v2.f32 [%0], {%1, %2};" ::"r"( base + 8u * (unsigned)i ), "f"( v.x ), "f"( v.y ) : "memory" );
    }
};

template<>
struct SmemBuf<double>
{
    unsigned int base;
    __device__ __forceinline__ cplx<double> ld( int i ) const
    {
        cplx<double> v;
        asm volatile( "ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"( v.x ), "=d"( v.y ) : "r"( base + 16u * (unsigned)i ) : "memory" );
        return v;
    }
    __device__ __forceinline__ void st( int i, cplx<double> v ) const
    {
        asm volatile( "st.shared.v2.f64 [%0], {%1, %2};" ::"r"( base + 16u * (unsigned)i ), "d"( v.x ), "d"( v.y ) : "memory" );
    }
};

// Small-radix DFT helpers (the radix-3/5/7 butterflies): sums, differences, scaling by a real,
// and the rotation by -i (forward) / +i (inverse).
template<typename R>
__device__ __forceinline__ cplx<R> cadd( cplx<R> a, cplx<R> b )
{
    return { a.x + b.x, a.y + b.y };
}
template<typename R>
__device__ __forceinline__ cplx<R> csub( cplx<R> a, cplx<R> b )
{
    return { a.x - b.x, a.y - b.y };
}
template<typename R>
__device__ __forceinline__ cplx<R> caxpy( R s, cplx<R> a, cplx<R> y ) // y + s a
{
    return { y.x + s * a.x, y.y + s * a.y };
}
template<typename R>
__device__ __forceinline__ cplx<R> crot( cplx<R> u, bool inverse )
{
    return inverse ? cplx<R>{ -u.y, u.x } : cplx<R>{ u.y, -u.x };
}

// One Stockham stage of compile-time radix RR over nl lines (element t of line l at l*ls + t*es):
// butterfly j = 0 .. L/RR - 1 of every line, k = j mod Ns, twiddles W_L^(r k span) on the inputs,
// then the RR-point DFT in closed form: radix 2 and 4 by sums and +-i swaps; radix 3, 5, 7 by the
// symmetric pairs a_k = v_k + v_(RR-k), b_k = v_k - v_(RR-k):
//   y_m = v_0 + sum_k cos(2 pi k m / RR) a_k  -/+  i sum_k sin(2 pi k m / RR) b_k,
//   y_(RR-m) with the opposite sign of the i term,
// the cosines and sines read from the twiddle table (W_RR^q = tw[q L/RR]).
template<typename R, int RR, typename BUF>
__device__ __forceinline__ void mixed_stage( const BUF & a, const BUF & b, int nl, int ls, int es, int LR, int Ns,
                                             int span, const FastDiv & dlr, const FastDiv & dns, const BUF & tw,
                                             bool inverse )
{
    constexpr int NH = ( RR - 1 ) / 2;
    R cs[NH + 1], sn[NH + 1]; // cos(2 pi q / RR), sin(2 pi q / RR)
#pragma unroll
    for( int q = 1; q <= NH; ++q )
    {
        const cplx<R> w = tw.ld( q * LR );
        cs[q]           = w.x;
        sn[q]           = -w.y;
    }
    const int lres = LR * es, nses = Ns * es;
    for( int idx = threadIdx.x; idx < nl * LR; idx += blockDim.x )
    {
        const int line = (int)fdiv( (unsigned)idx, dlr );
        const int j    = idx - line * LR;
        const int jq   = (int)fdiv( (unsigned)j, dns );
        const int k    = j - jq * Ns;
        const int s0   = line * ls + j * es;                   // input r at s0 + r L/RR
        const int d0   = line * ls + ( jq * Ns * RR + k ) * es; // output m at d0 + m Ns
        const int ks   = k * span;
        cplx<R> v[RR];
        v[0] = a.ld( s0 );
#pragma unroll
        for( int r = 1; r < RR; ++r )
        {
            cplx<R> w = tw.ld( r * ks );
            if( inverse )
                w = cconj( w );
            v[r] = cmul( a.ld( s0 + r * lres ), w );
        }
        cplx<R> y[RR];
        if( RR == 2 )
        {
            y[0]      = cadd( v[0], v[1 % RR] );
            y[1 % RR] = csub( v[0], v[1 % RR] );
        }
        else if( RR == 4 )
        {
            const cplx<R> s02 = cadd( v[0], v[2 % RR] ), d02 = csub( v[0], v[2 % RR] );
            const cplx<R> s13 = cadd( v[1 % RR], v[3 % RR] ), d13 = crot( csub( v[1 % RR], v[3 % RR] ), inverse );
            y[0]      = cadd( s02, s13 );
            y[1 % RR] = cadd( d02, d13 );
            y[2 % RR] = csub( s02, s13 );
            y[3 % RR] = csub( d02, d13 );
        }
        else
        {
            cplx<R> ap[NH + 1], bm[NH + 1];
            y[0] = v[0];
#pragma unroll
            for( int q = 1; q <= NH; ++q )
            {
                ap[q] = cadd( v[q], v[RR - q] );
                bm[q] = csub( v[q], v[RR - q] );
                y[0]  = cadd( y[0], ap[q] );
            }
#pragma unroll
            for( int m = 1; m <= NH; ++m )
            {
                cplx<R> t = v[0], u = { 0, 0 };
#pragma unroll
                for( int q = 1; q <= NH; ++q )
                {
                    const int e  = ( q * m ) % RR; // angle index of cos/sin(2 pi q m / RR)
                    const int ef = e <= NH ? e : RR - e;
                    const R sg   = e <= NH ? R( 1 ) : R( -1 );
                    t            = caxpy( cs[ef], ap[q], t );
                    u            = caxpy( sg * sn[ef], bm[q], u );
                }
                const cplx<R> iu = crot( u, inverse );
                y[m]             = cadd( t, iu );
                y[RR - m]        = csub( t, iu );
            }
        }
#pragma unroll
        for( int m = 0; m < RR; ++m )
            b.st( d0 + m * nses, y[m] );
    }
}

// The stages of mixed_fft from buffer a into b (ping-pong); returns true when the result is in a.
template<typename R, typename BUF>
__device__ __forceinline__ bool mixed_stages( const BUF & A0, const BUF & B0, int L, int nl, int ls, int es,
                                              const RadixPlan & P, const BUF & tw, bool inverse )
{
    int Ns    = 1;
    bool in_a = true;
    for( int s = 0; s < 12 && P.radix[s] > 0; ++s )
    {
        const BUF & a     = in_a ? A0 : B0;
        const BUF & b     = in_a ? B0 : A0;
        const int Rr      = P.radix[s];
        const int LR      = L / Rr;
        const int span    = L / ( Ns * Rr );
        const FastDiv dlr = P.div_lr[s], dns = P.div_ns[s];
        switch( Rr )
        {
        case 2:
            mixed_stage<R, 2>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw, inverse );
            break;
        case 3:
            mixed_stage<R, 3>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw, inverse );
            break;
        case 4:
            mixed_stage<R, 4>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw, inverse );
            break;
        case 5:
            mixed_stage<R, 5>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw, inverse );
            break;
        case 7:
            mixed_stage<R, 7>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw, inverse );
            break;
        default:
            // other radices (not produced by the padded extents): runtime-radix direct sums
            for( int o = threadIdx.x; o < nl * L; o += blockDim.x )
            {
                const int line = o / L;
                const int q    = o - line * L;
                const int k    = q % Ns;
                const int m    = ( q / Ns ) % Rr;
                const int jhi  = q / ( Ns * Rr );
                const int j    = jhi * Ns + k;
                cplx<R> acc    = { 0, 0 };
                for( int r = 0; r < Rr; ++r )
                {
                    const int t = ( r * k * span + ( ( r * m ) % Rr ) * LR ) % L;
                    cplx<R> w   = tw.ld( t );
                    if( inverse )
                        w = cconj( w );
                    const cplx<R> p = cmul( a.ld( line * ls + ( j + r * LR ) * es ), w );
                    acc.x += p.x;
                    acc.y += p.y;
                }
                b.st( line * ls + q * es, acc );
            }
            break;
        }
        __syncthreads();
        in_a = !in_a;
        Ns *= Rr;
    }
    return in_a;
}

// Mixed-radix (any L) strided Stockham: element t of line l at l*ls + t*es, ping-pong between a
// and b; returns the buffer that holds the result.  Radices 2, 3, 4, 5, 7 (all that the padded
// extents produce) with closed-form compile-time butterflies and the stage divisors precomputed
// on the host (RadixPlan); others by runtime-radix direct sums.  Consecutive threads take
// consecutive butterflies of a line.  Not inlined (one copy serves every call site of a kernel):
// the buffers arrive as generic pointers and are accessed through the shared window when all three
// point into shared memory, element-aligned (every caller's do).
template<typename R>
__device__ __noinline__ cplx<R> * mixed_fft( cplx<R> * a, cplx<R> * b, int L, int nl, int ls, int es,
                                             const RadixPlan & P, const cplx<R> * tw, bool inverse )
{
    constexpr unsigned int EL = sizeof( cplx<R> );
    bool in_a;
    if( __isShared( a ) && __isShared( b ) && __isShared( tw ) )
    {
        const unsigned int sa = (unsigned int)__cvta_generic_to_shared( a );
        const unsigned int sb = (unsigned int)__cvta_generic_to_shared( b );
        const unsigned int st = (unsigned int)__cvta_generic_to_shared( tw );
        if( ( ( sa | sb | st ) & ( EL - 1 ) ) == 0 )
        {
            in_a = mixed_stages<R>( SmemBuf<R>{ sa }, SmemBuf<R>{ sb }, L, nl, ls, es, P, SmemBuf<R>{ st }, inverse );
            return in_a ? a : b;
        }
    }
    in_a = mixed_stages<R>( GenBuf<R>{ a }, GenBuf<R>{ b }, L, nl, ls, es, P, GenBuf<R>{ const_cast<cplx<R> *>( tw ) },
                            inverse );
    return in_a ? a : b;
}

template<typename R, bool LINE_FAST, int MAXLG = MaxRadix<R>::LG>
__device__ cplx<R> * sfft( cplx<R> * a, cplx<R> * b, int L, int nl, const FastDiv & dnl, int ls, int es,
                          const RadixPlan & P, const cplx<R> * tw, bool inverse )
{
    switch( L )
    {
    case 1:
        return a;
    case 2:
        return sfft_const<R, 2, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 4:
        return sfft_const<R, 4, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 8:
        return sfft_const<R, 8, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 16:
        return stockham_reg<R, 4, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 32:
        return stockham_reg<R, 5, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 64:
        return stockham_reg<R, 6, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 128:
        return stockham_reg<R, 7, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 256:
        return stockham_reg<R, 8, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 512:
        return stockham_reg<R, 9, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    case 1024:
        return stockham_reg<R, 10, 0, MAXLG, LINE_FAST>( a, b, nl, dnl, ls, es, tw, inverse );
    default:
        return mixed_fft<R>( a, b, L, nl, ls, es, P, tw, inverse );
    }
}

// copy a twiddle table into shared memory (all threads)
template<typename R>
__device__ __forceinline__ void load_tw( cplx<R> * dst, const cplx<R> * src, int L )
{
    for( int t = threadIdx.x; t < L; t += blockDim.x )
        dst[t] = src[t];
}

// shared-memory line stride for lines of length L
__host__ __device__ inline int line_stride( int L )
{
    return ( ( L & ( L - 1 ) ) == 0 && L >= 8 && L <= 64 ) ? L + 1 : L;
}

} // namespace sg
