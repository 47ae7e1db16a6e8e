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

#include <vector>

namespace sg
{

// Complex value, aligned to its size so that every load and store of one is a single vector
// access (every complex array here starts at a shared or global base aligned to 16 bytes and is
// indexed in whole elements).
template<typename R>
struct alignas( 2 * sizeof( R ) ) cplx
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
// starts at k * ls (ls = line_stride(L): L + 1 for even L, to spread shared-memory banks).
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
__device__ __forceinline__ cplx<R> * mixed_fft( cplx<R> * a, cplx<R> * b, int L, int nl, int ls, int es,
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
    return mixed_fft<R>( a, b, L, nl, ls, 1, P, tw, inverse );
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

// Small-DFT helpers: sums, differences, scaling by a real, and the rotation by -i (forward) / +i
// (inverse).
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
template<typename R, bool INV>
__device__ __forceinline__ cplx<R> crot( cplx<R> u )
{
    return INV ? cplx<R>{ -u.y, u.x } : cplx<R>{ u.y, -u.x };
}

// cos and sin of 2 pi e / N for the register radices N (0 <= e < N), exact where the angle makes
// them 0, +-1/2 or +-1.  Called with constant arguments only (the unrolled small DFTs), so every
// call folds to a literal.
__host__ __device__ constexpr double root_cos( int N, int e )
{
    constexpr double t3[] = { 1.0, -0.5, -0.5 };
    constexpr double t5[] = { 1.0, 0.309016994374947424102, -0.809016994374947424102, -0.809016994374947424102,
                              0.309016994374947424102 };
    constexpr double t6[] = { 1.0, 0.5, -0.5, -1.0, -0.5, 0.5 };
    constexpr double t7[] = { 1.0, 0.623489801858733530525, -0.222520933956314404289, -0.900968867902419126236,
                              -0.900968867902419126236, -0.222520933956314404289, 0.623489801858733530525 };
    constexpr double t8[] = { 1.0, 0.707106781186547524401, 0.0, -0.707106781186547524401, -1.0,
                              -0.707106781186547524401, 0.0, 0.707106781186547524401 };
    constexpr double t9[] = { 1.0, 0.766044443118978035202, 0.173648177666930348852, -0.5, -0.939692620785908384054,
                              -0.939692620785908384054, -0.5, 0.173648177666930348852, 0.766044443118978035202 };
    constexpr double t10[] = { 1.0, 0.809016994374947424102, 0.309016994374947424102, -0.309016994374947424102,
                               -0.809016994374947424102, -1.0, -0.809016994374947424102, -0.309016994374947424102,
                               0.309016994374947424102, 0.809016994374947424102 };
    constexpr double t12[] = { 1.0, 0.866025403784438646764, 0.5, 0.0, -0.5, -0.866025403784438646764, -1.0,
                               -0.866025403784438646764, -0.5, 0.0, 0.5, 0.866025403784438646764 };
    constexpr double t14[] = { 1.0, 0.900968867902419126236, 0.623489801858733530525, 0.222520933956314404289,
                               -0.222520933956314404289, -0.623489801858733530525, -0.900968867902419126236, -1.0,
                               -0.900968867902419126236, -0.623489801858733530525, -0.222520933956314404289,
                               0.222520933956314404289, 0.623489801858733530525, 0.900968867902419126236 };
    constexpr double t15[] = { 1.0, 0.913545457642600895502, 0.669130606358858213826, 0.309016994374947424102,
                               -0.1045284632676534714, -0.5, -0.809016994374947424102, -0.978147600733805637929,
                               -0.978147600733805637929, -0.809016994374947424102, -0.5, -0.1045284632676534714,
                               0.309016994374947424102, 0.669130606358858213826, 0.913545457642600895502 };
    constexpr double t16[] = { 1.0, 0.923879532511286756128, 0.707106781186547524401, 0.382683432365089771728, 0.0,
                               -0.382683432365089771728, -0.707106781186547524401, -0.923879532511286756128, -1.0,
                               -0.923879532511286756128, -0.707106781186547524401, -0.382683432365089771728, 0.0,
                               0.382683432365089771728, 0.707106781186547524401, 0.923879532511286756128 };
    switch( N )
    {
    case 3: return t3[e];
    case 5: return t5[e];
    case 6: return t6[e];
    case 7: return t7[e];
    case 8: return t8[e];
    case 9: return t9[e];
    case 10: return t10[e];
    case 12: return t12[e];
    case 14: return t14[e];
    case 15: return t15[e];
    case 16: return t16[e];
    default: return 1.0;
    }
}
__host__ __device__ constexpr double root_sin( int N, int e )
{
    constexpr double t3[] = { 0.0, 0.866025403784438646764, -0.866025403784438646764 };
    constexpr double t5[] = { 0.0, 0.951056516295153572116, 0.587785252292473129169, -0.587785252292473129169,
                              -0.951056516295153572116 };
    constexpr double t6[] = { 0.0, 0.866025403784438646764, 0.866025403784438646764, 0.0, -0.866025403784438646764,
                              -0.866025403784438646764 };
    constexpr double t7[] = { 0.0, 0.781831482468029808708, 0.974927912181823607018, 0.433883739117558120476,
                              -0.433883739117558120476, -0.974927912181823607018, -0.781831482468029808708 };
    constexpr double t8[] = { 0.0, 0.707106781186547524401, 1.0, 0.707106781186547524401, 0.0,
                              -0.707106781186547524401, -1.0, -0.707106781186547524401 };
    constexpr double t9[] = { 0.0, 0.642787609686539326323, 0.984807753012208059367, 0.866025403784438646764,
                              0.342020143325668733044, -0.342020143325668733044, -0.866025403784438646764,
                              -0.984807753012208059367, -0.642787609686539326323 };
    constexpr double t10[] = { 0.0, 0.587785252292473129169, 0.951056516295153572116, 0.951056516295153572116,
                               0.587785252292473129169, 0.0, -0.587785252292473129169, -0.951056516295153572116,
                               -0.951056516295153572116, -0.587785252292473129169 };
    constexpr double t12[] = { 0.0, 0.5, 0.866025403784438646764, 1.0, 0.866025403784438646764, 0.5, 0.0, -0.5,
                               -0.866025403784438646764, -1.0, -0.866025403784438646764, -0.5 };
    constexpr double t14[] = { 0.0, 0.433883739117558120476, 0.781831482468029808708, 0.974927912181823607018,
                               0.974927912181823607018, 0.781831482468029808708, 0.433883739117558120476, 0.0,
                               -0.433883739117558120476, -0.781831482468029808708, -0.974927912181823607018,
                               -0.974927912181823607018, -0.781831482468029808708, -0.433883739117558120476 };
    constexpr double t15[] = { 0.0, 0.406736643075800207754, 0.743144825477394235015, 0.951056516295153572116,
                               0.994521895368273336923, 0.866025403784438646764, 0.587785252292473129169,
                               0.207911690817759337102, -0.207911690817759337102, -0.587785252292473129169,
                               -0.866025403784438646764, -0.994521895368273336923, -0.951056516295153572116,
                               -0.743144825477394235015, -0.406736643075800207754 };
    constexpr double t16[] = { 0.0, 0.382683432365089771728, 0.707106781186547524401, 0.923879532511286756128, 1.0,
                               0.923879532511286756128, 0.707106781186547524401, 0.382683432365089771728, 0.0,
                               -0.382683432365089771728, -0.707106781186547524401, -0.923879532511286756128, -1.0,
                               -0.923879532511286756128, -0.707106781186547524401, -0.382683432365089771728 };
    switch( N )
    {
    case 3: return t3[e];
    case 5: return t5[e];
    case 6: return t6[e];
    case 7: return t7[e];
    case 8: return t8[e];
    case 9: return t9[e];
    case 10: return t10[e];
    case 12: return t12[e];
    case 14: return t14[e];
    case 15: return t15[e];
    case 16: return t16[e];
    default: return 0.0;
    }
}

// x * W_N^e (forward: W = exp(-2 pi i e / N); inverse: the conjugate) for constant N, e; the
// multiplications by 1, -1 and -+i are exact swaps and sign changes.
template<typename R, bool INV>
__device__ __forceinline__ cplx<R> twiddle_const( cplx<R> x, int N, int e )
{
    if( e == 0 )
        return x;
    if( 2 * e == N )
        return { -x.x, -x.y };
    if( 4 * e == N )
        return crot<R, INV>( x );
    if( 4 * e == 3 * N )
        return crot<R, !INV>( x );
    const R c = R( root_cos( N, e ) ), sn = R( root_sin( N, e ) );
    return cmul( x, cplx<R>{ c, INV ? sn : -sn } );
}

// In-register DFT of N points in natural order, N in {2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16}:
//   N = 2, 4, 8, 16: dft_reg;
//   N = 3, 5, 7: the symmetric pairs a_q = v_q + v_(N-q), b_q = v_q - v_(N-q),
//     X_m = v_0 + sum_q cos(2 pi q m / N) a_q -/+ i sum_q sin(2 pi q m / N) b_q, X_(N-m) the conjugate pattern;
//   N = P Q (6 = 2 3, 9 = 3 3, 10 = 2 5, 12 = 4 3, 14 = 2 7, 15 = 3 5): Cooley-Tukey in registers,
//     Q DFTs of P points over v[Q n1 + n2], twiddles W_N^(n2 k1), P DFTs of Q points, X[k1 + P k2].
template<int N>
struct SmallFactor
{
    static constexpr int P = ( N == 12 ) ? 4 : ( N % 2 == 0 ) ? 2 : 3;
};

template<typename R, int N, bool INV>
__device__ __forceinline__ void dft_small( cplx<R> * v )
{
    if constexpr( N == 1 )
        return;
    else if constexpr( N == 2 || N == 4 || N == 8 || N == 16 )
        dft_reg<R, N>( v, INV );
    else if constexpr( N == 3 || N == 5 || N == 7 )
    {
        constexpr int NH = ( N - 1 ) / 2;
        cplx<R> ap[NH + 1], bm[NH + 1], y[N];
        y[0] = v[0];
#pragma unroll
        for( int q = 1; q <= NH; ++q )
        {
            ap[q] = cadd( v[q], v[N - q] );
            bm[q] = csub( v[q], v[N - q] );
            y[0]  = cadd( y[0], ap[q] );
        }
#pragma unroll
        for( int m = 1; m <= NH; ++m )
        {
            cplx<R> t = v[0], u = { 0, 0 };
#pragma unroll
            for( int q = 1; q <= NH; ++q )
            {
                t = caxpy( R( root_cos( N, ( q * m ) % N ) ), ap[q], t );
                u = caxpy( R( root_sin( N, ( q * m ) % N ) ), bm[q], u );
            }
            const cplx<R> iu = crot<R, INV>( u );
            y[m]             = cadd( t, iu );
            y[N - m]         = csub( t, iu );
        }
#pragma unroll
        for( int m = 0; m < N; ++m )
            v[m] = y[m];
    }
    else
    {
        constexpr int P = SmallFactor<N>::P, Q = N / P;
        static_assert( P * Q == N && ( Q == 2 || Q == 3 || Q == 4 || Q == 5 || Q == 7 ), "register radix" );
        cplx<R> y[N];
#pragma unroll
        for( int n2 = 0; n2 < Q; ++n2 )
        {
            cplx<R> t[P];
#pragma unroll
            for( int n1 = 0; n1 < P; ++n1 )
                t[n1] = v[Q * n1 + n2];
            dft_small<R, P, INV>( t );
#pragma unroll
            for( int k1 = 0; k1 < P; ++k1 )
                y[k1 * Q + n2] = twiddle_const<R, INV>( t[k1], N, ( n2 * k1 ) % N );
        }
#pragma unroll
        for( int k1 = 0; k1 < P; ++k1 )
        {
            cplx<R> t[Q];
#pragma unroll
            for( int n2 = 0; n2 < Q; ++n2 )
                t[n2] = y[k1 * Q + n2];
            dft_small<R, Q, INV>( t );
#pragma unroll
            for( int k2 = 0; k2 < Q; ++k2 )
                v[k1 + P * k2] = t[k2];
        }
    }
}

// One Stockham stage of compile-time radix RR over nl lines (element t of line l at l*ls + t*es):
// butterfly j = 0 .. L/RR - 1 of every line, k = j mod Ns, twiddles W_L^(r k span) on the inputs
// (none in the first stage, Ns = 1), the RR-point DFT in registers, outputs at (j - k) RR + k + m Ns.
// Thread t takes butterflies t, t + T, t + 2T, ... (T threads) of the flattened (line, j) range; its
// position (line, j = jq Ns + k) advances by the precomputed step, so the loop divides nothing.
template<typename R, int RR, bool INV, bool FIRST, typename BUF>
__device__ __forceinline__ void mixed_stage( const BUF & a, const BUF & b, int nl, int ls, int es, int LR, int Ns,
                                             int span, const FastDiv & dlr, const FastDiv & dns, const BUF & tw )
{
    const int T   = blockDim.x;
    int line      = (int)fdiv( threadIdx.x, dlr );
    int j         = threadIdx.x - line * LR;
    int jq        = (int)fdiv( (unsigned)j, dns );
    int k         = j - jq * Ns;
    const int dl  = (int)fdiv( (unsigned)T, dlr );
    const int dj  = T - dl * LR;
    const int djq = (int)fdiv( (unsigned)dj, dns );
    const int dk  = dj - djq * Ns;
    const int lres = LR * es, nses = Ns * es, step = Ns * RR;
    while( line < nl )
    {
        const int s0 = line * ls + j * es;
        const int d0 = line * ls + ( jq * step + k ) * es;
        cplx<R> v[RR];
        v[0] = a.ld( s0 );
#pragma unroll
        for( int r = 1; r < RR; ++r )
        {
            v[r] = a.ld( s0 + r * lres );
            if( !FIRST )
            {
                cplx<R> w = tw.ld( r * k * span );
                if( INV )
                    w.y = -w.y;
                v[r] = cmul( v[r], w );
            }
        }
        dft_small<R, RR, INV>( v );
#pragma unroll
        for( int m = 0; m < RR; ++m )
            b.st( d0 + m * nses, v[m] );
        line += dl;
        j += dj;
        jq += djq;
        k += dk;
        if( k >= Ns )
        {
            k -= Ns;
            ++jq;
        }
        if( j >= LR )
        {
            j -= LR;
            ++line;
            jq -= span;
        }
    }
}

template<typename R, int RR, bool INV, typename BUF>
__device__ __forceinline__ void mixed_stage_any( const BUF & a, const BUF & b, int nl, int ls, int es, int LR, int Ns,
                                                 int span, const FastDiv & dlr, const FastDiv & dns, const BUF & tw )
{
    if( Ns == 1 )
        mixed_stage<R, RR, INV, true>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw );
    else
        mixed_stage<R, RR, INV, false>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw );
}

// The stages of mixed_fft from buffer a into b (ping-pong); returns true when the result is in a.
template<typename R, bool INV, typename BUF>
__device__ __forceinline__ bool mixed_stages( const BUF & A0, const BUF & B0, int L, int nl, int ls, int es,
                                              const RadixPlan & P, const BUF & tw )
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
#define SG_MIXED_CASE( RAD )                                                                                           \
    case RAD: mixed_stage_any<R, RAD, INV>( a, b, nl, ls, es, LR, Ns, span, dlr, dns, tw ); break;
            SG_MIXED_CASE( 2 )
            SG_MIXED_CASE( 3 )
            SG_MIXED_CASE( 4 )
            SG_MIXED_CASE( 5 )
            SG_MIXED_CASE( 6 )
            SG_MIXED_CASE( 7 )
            SG_MIXED_CASE( 8 )
            SG_MIXED_CASE( 9 )
            SG_MIXED_CASE( 10 )
            SG_MIXED_CASE( 12 )
#undef SG_MIXED_CASE
        default:
            // other radices (prime factors above 7 of unpadded periodic extents): direct sums
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
                    if( INV )
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
// and b; returns the buffer that holds the result.  The radix sequence (RadixPlan, chosen on the
// host by radix_plan) uses register DFTs of 2 ... 16 points; prime factors above 7 fall back to
// direct sums.  Not inlined (one copy per direction serves every call site of a kernel): the
// buffers arrive as generic pointers and are accessed through the shared window when all three
// point into shared memory, element-aligned (every caller's do).
template<typename R, bool INV>
__device__ __noinline__ cplx<R> * mixed_fft_dir( cplx<R> * a, cplx<R> * b, int L, int nl, int ls, int es,
                                                 const RadixPlan & P, const cplx<R> * tw )
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
            in_a = mixed_stages<R, INV>( SmemBuf<R>{ sa }, SmemBuf<R>{ sb }, L, nl, ls, es, P, SmemBuf<R>{ st } );
            return in_a ? a : b;
        }
    }
    in_a = mixed_stages<R, INV>( GenBuf<R>{ a }, GenBuf<R>{ b }, L, nl, ls, es, P,
                                 GenBuf<R>{ const_cast<cplx<R> *>( tw ) } );
    return in_a ? a : b;
}

template<typename R>
__device__ __forceinline__ cplx<R> * mixed_fft( cplx<R> * a, cplx<R> * b, int L, int nl, int ls, int es,
                                                const RadixPlan & P, const cplx<R> * tw, bool inverse )
{
    return inverse ? mixed_fft_dir<R, true>( a, b, L, nl, ls, es, P, tw )
                   : mixed_fft_dir<R, false>( a, b, L, nl, ls, es, P, tw );
}

// Radix sequence of a length-L transform for mixed_fft: the factorisation into register radices
// {2, ..., 16} of least estimated cost (per point and stage: a fixed part -- the shared-memory
// round trip, the twiddle and the index work -- plus the butterfly's arithmetic per point), found
// by dynamic programming over the divisors of L; prime factors above 7 become direct-sum stages.
// The stage divisors (L / radix and the product of the earlier radices) are filled in for the
// threads' start positions.
inline void radix_plan( int L, RadixPlan & P )
{
    const int cand[]   = { 12, 10, 9, 8, 7, 6, 5, 4, 3, 2 };
    const double fp[]  = { 12.3, 12.4, 13.3, 6.5, 12.0, 8.7, 8.0, 4.0, 5.3, 2.0 };
    const double fixed = 14.0;
    // L = smooth * rough: smooth has the prime factors 2, 3, 5, 7, rough the others
    int smooth = 1, rough = L;
    for( int p : { 2, 3, 5, 7 } )
        while( rough % p == 0 )
        {
            rough /= p;
            smooth *= p;
        }
    std::vector<double> best( smooth + 1, 1e300 );
    std::vector<int> pick( smooth + 1, 0 );
    best[1] = 0.0;
    for( int m = 2; m <= smooth; ++m )
    {
        if( smooth % m )
            continue;
        for( int c = 0; c < 10; ++c )
        {
            const int r = cand[c];
            if( m % r == 0 && best[m / r] + fixed + fp[c] < best[m] )
            {
                best[m] = best[m / r] + fixed + fp[c];
                pick[m] = r;
            }
        }
    }
    int ns = 0;
    for( int m = smooth; m > 1 && ns < 12; m /= pick[m] )
        P.radix[ns++] = pick[m];
    for( int p = 11; rough > 1 && ns < 12; p += 2 ) // rough has no factor below 11
        while( rough % p == 0 && ns < 12 )
        {
            P.radix[ns++] = p;
            rough /= p;
        }
    for( int s = ns; s < 12; ++s )
        P.radix[s] = 0;
    int prod = 1;
    for( int s = 0; s < ns; ++s )
    {
        P.div_lr[s] = make_fastdiv( (unsigned)( L / P.radix[s] ) );
        P.div_ns[s] = make_fastdiv( (unsigned)prod );
        prod *= P.radix[s];
    }
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

// Shared-memory line stride for lines of length L: odd, so that the transposed accesses of the
// passes (consecutive threads on consecutive lines at one frequency) spread over the banks -- an
// even stride puts many lanes of a half-warp on the same banks (16-way for 8-byte elements when L
// is a multiple of 16).
__host__ __device__ inline int line_stride( int L )
{
    return ( L % 2 == 0 ) ? L + 1 : L;
}

} // namespace sg
