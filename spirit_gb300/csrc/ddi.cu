// Dipole-dipole field of a batch of systems by zero-padded FFT convolution (see fft.cuh).
//
// Per system s with DDI, work arrays (complex, precision R):
//   W1[(cb*Cin + c)*Bin + b)*Mh + ka]   after pass A / before pass A'    (cb = ib*3 + comp)
//   W2[(cb*Cin + c)*Mb + kb)*Mh + ka]   after pass B / C / before B'
//   Dhat[((kb*Mh + ka)*npair + pair)*6 + comp6)*Mc + kc]   dipole spectrum, pair = b1*nb + b2
// Cin/Bin are the number of nonzero input rows: (Nc, Nb) for spins, (Mc, Mb) for the dense
// dipole tensor of the one-time precompute.
#include "ddi.hpp"
#include "fft.cuh"
#include "util.hpp"

#include <cooperative_groups.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace sg
{

template<typename R>
struct PassArgs
{
    const FFTDesc * fd;
    const SysDesc * sd;
    const SysRun * runs; // may be null (then every system is processed)
    const int4 * blocks; // (system, first group, n groups, 0)
    const cplx<R> * tw;  // twiddle tables
    cplx<R> * W1;
    cplx<R> * W2;
    const cplx<R> * Dhat;
    // spins of the stage configuration (pass A) / field output (pass A')
    const R * sx;
    const R * sy;
    const R * sz;
    R * hx;
    R * hy;
    R * hz;
    // dense real input for the dipole precompute (pass A mode 1)
    const R * dense;
    int mode; // 0: spin convolution, 1: dense forward transform
    int g;    // lines (pass B) / columns (pass C) per block; lines per block of pass A / A'
    FastDiv div_g;
    int ka_major; // W1 layout: 0 [row][b][ka] (split passes B, C, B'), 1 [ka][row][b] (fused pass BC)
    FastDiv div_gq; // (g + 1) / 2: line pairs per block of pass A
    int prefetch;   // fused b/c passes: prefetch the block's dipole-spectrum slice into L2 first
};

// Prefetch [p, p + bytes) into L2, one 128-byte line per request, spread over the block's threads
// (no completion: a later load simply finds the lines in L2)
__device__ __forceinline__ void prefetch_l2_lines( const void * p, size_t bytes, int lane, int nthreads )
{
    const char * c = static_cast<const char *>( p );
    for( size_t o = (size_t)lane * 128; o < bytes; o += (size_t)nthreads * 128 )
        asm volatile( "prefetch.global.L2 [%0];" ::"l"( c + o ) );
}

template<typename R>
__device__ __forceinline__ bool sys_inactive( const PassArgs<R> & p, int s )
{
    return p.runs && !p.runs[s].active;
}

// Block tables:
//   pass A / A' : (system, row = cb*Cin + c, first b, number of lines)
//   pass B / B' : (system, first line, number of lines) over the flattened lines (row, ka)
//   pass C      : (system, first column, number of columns) over the flattened columns kb*Mh + ka
// Passes B and C hold p.g lines (columns) per block; the block tables and p.g come from the
// autotuner of DDIPlan.
// ------------------------------------------------------------------ pass A: R2C along a
// Two real lines x, y go through one complex transform of z = x + i y:
//   X[k] = (Z[k] + conj Z[-k]) / 2,   Y[k] = (Z[k] - conj Z[-k]) / 2i
template<typename R>
__global__ void __launch_bounds__( 256, sizeof( R ) == 4 ? 4 : 2 ) pass_a( PassArgs<R> p )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    const FFTDesc & f = p.fd[s];
    const int Ma = f.M[0], Mh = f.Mh, nb = f.nb;
    const int Cin = p.mode ? f.M[2] : f.N[2];
    const int Bin = p.mode ? f.M[1] : f.N[1];
    const int Ain = p.mode ? f.M[0] : f.N[0];
    const int row = blk.y, b0 = blk.z, nl = blk.w;
    const int nq  = ( nl + 1 ) >> 1;
    const int ls  = line_stride( Ma );
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Ma;
    cplx<R> * b   = a + nq * ls;
    load_tw( tw, p.tw + f.tw_offset[0], Ma );
    pdl_wait();
    pdl_trigger();
    if( sys_inactive( p, s ) )
        return;
    if( p.mode == 0 )
    {
        const int cb = row / Cin, c = row - cb * Cin;
        const int ib = cb / 3, comp = cb - 3 * ib;
        const SysDesc & d    = p.sd[s];
        const R mu           = fft_mu<R>( f, ib );
        const R * src        = comp == 0 ? p.sx : ( comp == 1 ? p.sy : p.sz );
        const int rowlen     = nb * d.n_cells[0];
        // spin arrays of a batch hold fewer than 2^31 entries (the engine checks): 32-bit offsets
        const int base       = (int)d.spin_offset + ib + rowlen * ( b0 + d.n_cells[1] * c );
        // unrolled: the loads of several elements are in flight before the first lands in shared memory
#pragma unroll 4
        for( int e = threadIdx.x; e < nq * Ma; e += blockDim.x )
        {
            const int q = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - q * Ma;
            R x = 0, y = 0;
            if( t < Ain )
            {
                const int o = base + 2 * q * rowlen + nb * t;
                x           = mu * src[o];
                if( 2 * q + 1 < nl )
                    y = mu * src[o + rowlen];
            }
            a[q * ls + t] = { x, y };
        }
    }
    else
    {
        const R * src = p.dense + ( (size_t)row * Bin + b0 ) * Ma;
#pragma unroll 4
        for( int e = threadIdx.x; e < nq * Ma; e += blockDim.x )
        {
            const int q = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - q * Ma;
            const R x   = src[(size_t)( 2 * q ) * Ma + t];
            const R y   = 2 * q + 1 < nl ? src[(size_t)( 2 * q + 1 ) * Ma + t] : R( 0 );
            a[q * ls + t] = { x, y };
        }
    }
    __syncthreads();
    const cplx<R> * r = block_fft( a, b, Ma, ls, nq, f.plan[0], tw, false );
    if( !p.ka_major )
    {
        cplx<R> * W1 = p.W1 + f.spec_offset + ( (size_t)row * Bin + b0 ) * Mh;
        for( int e = threadIdx.x; e < nl * Mh; e += blockDim.x )
        {
            const int li      = (int)fdiv( (unsigned)e, f.div_Mh ), k = e - li * Mh;
            const cplx<R> * z = r + ( li >> 1 ) * ls;
            const cplx<R> zk = z[k], zm = z[k == 0 ? 0 : Ma - k];
            W1[e] = ( li & 1 ) ? cplx<R>{ R( 0.5 ) * ( zk.y + zm.y ), R( -0.5 ) * ( zk.x - zm.x ) }
                               : cplx<R>{ R( 0.5 ) * ( zk.x + zm.x ), R( 0.5 ) * ( zk.y - zm.y ) };
        }
    }
    else
    {
        // [ka][row][b]: consecutive threads -> consecutive b of one ka
        const int G     = p.g;
        const int rows  = 3 * nb * Cin;
        cplx<R> * W1    = p.W1 + f.spec_offset + (size_t)row * Bin + b0;
        for( int e = threadIdx.x; e < G * Mh; e += blockDim.x )
        {
            const int k = (int)fdiv( (unsigned)e, p.div_g ), li = e - k * G;
            if( li >= nl )
                continue;
            const cplx<R> * z = r + ( li >> 1 ) * ls;
            const cplx<R> zk = z[k], zm = z[k == 0 ? 0 : Ma - k];
            W1[(size_t)k * rows * Bin + li] = ( li & 1 ) ? cplx<R>{ R( 0.5 ) * ( zk.y + zm.y ), R( -0.5 ) * ( zk.x - zm.x ) }
                                                         : cplx<R>{ R( 0.5 ) * ( zk.x + zm.x ), R( 0.5 ) * ( zk.y - zm.y ) };
        }
    }
}

// ------------------------------------------------------------------ pass B: C2C along b
// block: p.g consecutive lines (row, ka) of the flattened line index row*Mh + ka.
// forward: W1 -> W2 (rows b >= Bin are zero), inverse: W2 -> W1 (only b < Nb kept).
template<typename R>
__global__ void __launch_bounds__( 256, sizeof( R ) == 4 ? 4 : 2 ) pass_b( PassArgs<R> p, int inverse )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mh = f.Mh;
    const int Bin   = p.mode ? f.M[1] : f.N[1];
    const int G     = p.g;
    const int line0 = blk.y, nl = blk.z;
    const int ls    = line_stride( Mb );
    cplx<R> * tw    = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a     = tw + Mb;
    cplx<R> * b     = a + G * ls;
    load_tw( tw, p.tw + f.tw_offset[1], Mb );
    const cplx<R> * W1 = p.W1 + f.spec_offset;
    const cplx<R> * W2 = p.W2 + f.spec_offset;
    for( int e = threadIdx.x; e < Mb * G; e += blockDim.x )
    {
        const int t = (int)fdiv( (unsigned)e, p.div_g ), li = e - t * G; // consecutive threads -> consecutive ka
        if( li >= nl )
            continue;
        const int line = line0 + li;
        const int row  = (int)fdiv( (unsigned)line, f.div_Mh ), ka = line - row * Mh;
        cplx<R> v      = { 0, 0 };
        if( !inverse )
        {
            if( t < Bin )
                v = W1[( (size_t)row * Bin + t ) * Mh + ka];
        }
        else
            v = W2[( (size_t)row * Mb + t ) * Mh + ka];
        a[li * ls + t] = v;
    }
    __syncthreads();
    const cplx<R> * r = block_fft( a, b, Mb, ls, nl, f.plan[1], tw, inverse != 0 );
    const int Bout    = inverse ? f.N[1] : Mb;
    cplx<R> * dst     = inverse ? p.W1 + f.spec_offset : p.W2 + f.spec_offset;
    for( int e = threadIdx.x; e < Bout * G; e += blockDim.x )
    {
        const int t = (int)fdiv( (unsigned)e, p.div_g ), li = e - t * G;
        if( li >= nl )
            continue;
        const int line = line0 + li;
        const int row  = (int)fdiv( (unsigned)line, f.div_Mh ), ka = line - row * Mh;
        dst[( (size_t)row * Bout + t ) * Mh + ka] = r[li * ls + t];
    }
}

// ------------------------------------------------------------------ pass C: along c + tensor product
// block: p.g consecutive columns col = kb*Mh + ka (contiguous in W2 and in Dhat), all 3*nb
// components (smem line cb*G + g).
template<typename R>
__global__ void __launch_bounds__( 256, sizeof( R ) == 4 ? 4 : 2 ) pass_c( PassArgs<R> p )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mc = f.M[2], Mh = f.Mh, nb = f.nb;
    const int ncb       = 3 * nb;
    const int Cin       = p.mode ? f.M[2] : f.N[2];
    const int G         = p.g;
    const int col0      = blk.y, ng = blk.z;
    const size_t plane  = (size_t)Mb * Mh;
    const int ls        = line_stride( Mc );
    const int nl        = ncb * G; // lines g >= ng (last block) are zeros, computed but never stored
    cplx<R> * tw        = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a         = tw + Mc;
    cplx<R> * b         = a + nl * ls;
    load_tw( tw, p.tw + f.tw_offset[2], Mc );
    cplx<R> * W2    = p.W2 + f.spec_offset + col0;
    const int total = nl * Mc;
    for( int e = threadIdx.x; e < total; e += blockDim.x )
    {
        // e -> (cb, c, g) with g fastest for coalescing
        const int rest = (int)fdiv( (unsigned)e, p.div_g ), g = e - rest * G;
        const int cb   = (int)fdiv( (unsigned)rest, f.div_Mc ), c = rest - cb * Mc;
        cplx<R> v      = { 0, 0 };
        if( c < Cin && g < ng )
            v = W2[( (size_t)cb * Cin + c ) * plane + g];
        a[( cb * G + g ) * ls + c] = v;
    }
    __syncthreads();
    cplx<R> * r = Mc > 1 ? block_fft( a, b, Mc, ls, nl, f.plan[2], tw, false ) : a;
    if( p.mode == 1 )
    {
        // dense forward transform: write every kc
        for( int e = threadIdx.x; e < total; e += blockDim.x )
        {
            const int rest = (int)fdiv( (unsigned)e, p.div_g ), g = e - rest * G;
            const int cb   = (int)fdiv( (unsigned)rest, f.div_Mc ), c = rest - cb * Mc;
            if( g < ng )
                W2[( (size_t)cb * Mc + c ) * plane + g] = r[( cb * G + g ) * ls + c];
        }
        return;
    }
    // tensor product H_b1 = sum_b2 D_b1b2 . S_b2 (FFT.hpp:42-49 mult3D rows: xx xy xz | xy yy yz | xz yz zz)
    cplx<R> * h        = ( r == a ) ? b : a;
    const int npair    = nb * nb;
    const cplx<R> * Dh = p.Dhat + f.dhat_offset + (size_t)col0 * npair * 6 * Mc;
    for( int e = threadIdx.x; e < nb * Mc * G; e += blockDim.x )
    {
        const int rest = (int)fdiv( (unsigned)e, p.div_g ), g = e - rest * G;
        const int b1   = (int)fdiv( (unsigned)rest, f.div_Mc ), kc = rest - b1 * Mc;
        if( g >= ng )
            continue;
        cplx<R> acc[3] = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for( int b2 = 0; b2 < nb; ++b2 )
        {
            const cplx<R> * D = Dh + ( (size_t)g * npair + b1 * nb + b2 ) * 6 * Mc + kc;
            cplx<R> d[6];
#pragma unroll
            for( int q = 0; q < 6; ++q )
                d[q] = D[q * Mc];
            const cplx<R> sx = r[( ( b2 * 3 + 0 ) * G + g ) * ls + kc];
            const cplx<R> sy = r[( ( b2 * 3 + 1 ) * G + g ) * ls + kc];
            const cplx<R> sz = r[( ( b2 * 3 + 2 ) * G + g ) * ls + kc];
            const int rw[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
#pragma unroll
            for( int c3 = 0; c3 < 3; ++c3 )
            {
                const cplx<R> d1 = d[rw[c3][0]], d2 = d[rw[c3][1]], d3 = d[rw[c3][2]];
                acc[c3].x += d1.x * sx.x + d2.x * sy.x + d3.x * sz.x - d1.y * sx.y - d2.y * sy.y - d3.y * sz.y;
                acc[c3].y += d1.x * sx.y + d2.x * sy.y + d3.x * sz.y + d1.y * sx.x + d2.y * sy.x + d3.y * sz.x;
            }
        }
#pragma unroll
        for( int c3 = 0; c3 < 3; ++c3 )
            h[( ( b1 * 3 + c3 ) * G + g ) * ls + kc] = acc[c3];
    }
    __syncthreads();
    cplx<R> * other = ( h == a ) ? b : a;
    const cplx<R> * o = Mc > 1 ? block_fft( h, other, Mc, ls, nl, f.plan[2], tw, true ) : h;
    const int Cout    = f.N[2];
    for( int e = threadIdx.x; e < total; e += blockDim.x )
    {
        const int rest = (int)fdiv( (unsigned)e, p.div_g ), g = e - rest * G;
        const int cb   = (int)fdiv( (unsigned)rest, f.div_Mc ), c = rest - cb * Mc;
        if( c < Cout && g < ng )
            W2[( (size_t)cb * Cin + c ) * plane + g] = o[( cb * G + g ) * ls + c];
    }
}

// ------------------------------------------------------------------ fused pass BC
// One block per (system, ka): the whole (c, b) plane of every component in shared memory,
// layout [c][cb][kb] (c-row = 3 nb Mb elements), twice for the Stockham ping-pong:
//   forward along b (lines c < Nc, cb), forward along c (lines cb, kb; rows c >= Nc are zero),
//   tensor product with Dhat (fused layout [ka][pair][6][kc][kb]), inverse along c, inverse
//   along b; W1 [ka][row][b] in and out (row = cb Nc + c).
template<typename R>
__global__ void __launch_bounds__( 1024 ) pass_bc( PassArgs<R> p )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mc = f.M[2], nb = f.nb;
    const int Nb = f.N[1], Nc = f.N[2];
    const int ncb   = 3 * nb;
    const int plane = ncb * Mb;
    const int vol   = Mc * plane;
    const int ka    = blk.y;
    // planes of the block: several consecutive ka when the system has one c row (Mc == 1: every
    // plane is ncb lines along b, and the planes lie one after another in W1 and in shared memory)
    const int G     = blk.w > 0 ? blk.w : 1;
    cplx<R> * twb   = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * twc   = twb + Mb;
    cplx<R> * A     = twc + Mc;
    cplx<R> * B     = A + G * vol;
    load_tw( twb, p.tw + f.tw_offset[1], Mb );
    load_tw( twc, p.tw + f.tw_offset[2], Mc );
    // the dipole spectrum is constant: its slice for these planes can stream into L2 while the
    // predecessor kernel finishes and the forward transforms run
    if( p.prefetch )
        prefetch_l2_lines( p.Dhat + f.dhat_offset + (size_t)ka * nb * nb * 6 * Mc * Mb,
                           sizeof( cplx<R> ) * (size_t)G * nb * nb * 6 * Mc * Mb, threadIdx.x, blockDim.x );
    for( int e = threadIdx.x; e < 2 * G * vol; e += blockDim.x )
        A[e] = { 0, 0 };
    __syncthreads();
    pdl_wait();
    pdl_trigger();
    if( sys_inactive( p, s ) )
        return;
    const int nin    = ncb * Nc * Nb;
    cplx<R> * W1     = p.W1 + f.spec_offset + (size_t)ka * nin;
    for( int e = threadIdx.x; e < G * nin; e += blockDim.x )
    {
        const int g = (int)fdiv( (unsigned)e, f.div_nin ), el = e - g * nin;
        const int row = (int)fdiv( (unsigned)el, f.div_Nb ), b = el - row * Nb;
        const int cb  = (int)fdiv( (unsigned)row, f.div_Nc ), c = row - cb * Nc;
        A[g * vol + c * plane + cb * Mb + b] = W1[e];
    }
    __syncthreads();
    const FastDiv none = { 1, 0, 0 };
    cplx<R> * r = sfft<R, false>( A, B, Mb, G * Nc * ncb, none, Mb, 1, f.plan[1], twb, false );
    cplx<R> * o = ( r == A ) ? B : A;
    r           = sfft<R, true>( r, o, Mc, plane, f.div_plane, 1, plane, f.plan[2], twc, false );
    o           = ( r == A ) ? B : A;
    // tensor product H_b1 = sum_b2 D_b1b2 . S_b2 (FFT.hpp:42-49 mult3D rows: xx xy xz | xy yy yz | xz yz zz)
    const int npair    = nb * nb;
    for( int e = threadIdx.x; e < G * nb * Mc * Mb; e += blockDim.x )
    {
        const int g = (int)fdiv( (unsigned)e, f.div_tens ), eg = e - g * ( nb * Mc * Mb );
        const cplx<R> * Dh = p.Dhat + f.dhat_offset + (size_t)( ka + g ) * npair * 6 * Mc * Mb;
        const int rest = (int)fdiv( (unsigned)eg, f.div_Mb ), kb = eg - rest * Mb;
        const int kc   = (int)fdiv( (unsigned)rest, f.div_nb ), b1 = rest - kc * nb;
        const cplx<R> * S = r + g * vol + kc * plane + kb;
        cplx<R> acc[3]    = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for( int b2 = 0; b2 < nb; ++b2 )
        {
            const cplx<R> * D = Dh + ( (size_t)( b1 * nb + b2 ) * 6 * Mc + kc ) * Mb + kb;
            cplx<R> d[6];
#pragma unroll
            for( int q = 0; q < 6; ++q )
                d[q] = D[(size_t)q * Mc * Mb];
            const cplx<R> sx = S[( b2 * 3 + 0 ) * Mb];
            const cplx<R> sy = S[( b2 * 3 + 1 ) * Mb];
            const cplx<R> sz = S[( b2 * 3 + 2 ) * Mb];
            const int rw[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
#pragma unroll
            for( int c3 = 0; c3 < 3; ++c3 )
            {
                const cplx<R> d1 = d[rw[c3][0]], d2 = d[rw[c3][1]], d3 = d[rw[c3][2]];
                acc[c3].x += d1.x * sx.x + d2.x * sy.x + d3.x * sz.x - d1.y * sx.y - d2.y * sy.y - d3.y * sz.y;
                acc[c3].y += d1.x * sx.y + d2.x * sy.y + d3.x * sz.y + d1.y * sx.x + d2.y * sy.x + d3.y * sz.x;
            }
        }
#pragma unroll
        for( int c3 = 0; c3 < 3; ++c3 )
            o[g * vol + kc * plane + ( b1 * 3 + c3 ) * Mb + kb] = acc[c3];
    }
    __syncthreads();
    r = sfft<R, true>( o, ( o == A ) ? B : A, Mc, plane, f.div_plane, 1, plane, f.plan[2], twc, true );
    o = ( r == A ) ? B : A;
    r = sfft<R, false>( r, o, Mb, G * Nc * ncb, none, Mb, 1, f.plan[1], twb, true );
    for( int e = threadIdx.x; e < G * nin; e += blockDim.x )
    {
        const int g = (int)fdiv( (unsigned)e, f.div_nin ), el = e - g * nin;
        const int row = (int)fdiv( (unsigned)el, f.div_Nb ), b = el - row * Nb;
        const int cb  = (int)fdiv( (unsigned)row, f.div_Nc ), c = row - cb * Nc;
        W1[e]         = r[g * vol + c * plane + cb * Mb + b];
    }
}

// ------------------------------------------------------------------ fused pass BC on a cluster
// The (c, b) plane of one ka split over a cluster of K blocks.  b-phase: block r owns the c-rows
// [r cq, r cq + nc) (cq = ceil(Nc / K)), layout [c_local][cb][kb]; c-phase: block r owns the kb
// range [r kq, (r + 1) kq) (kq = Mb / K) for every c (Mc rows, rows >= Nc zero), layout
// [c][cb][kb_local].  The two transposes between the phases go through distributed shared memory.
// Block table: (system, ka, rank, 0), the K blocks of a plane consecutive.
// Index splits of the clustered b/c pass.  POW2: Mb / K and ceil(Nc / K) are powers of two, Nc is
// a multiple of ceil(Nc / K) (every block of a plane that has c rows has ceil(Nc / K) of them) and
// the basis has one atom -- shifts and a division by the literal 3; the host checks this for every
// system of the plan.  Otherwise run-time divisions.
template<bool POW2>
struct ClusterSplit
{
    int kq, cq, nc, ncb, nb, lkq, lcq;
    __device__ __forceinline__ int by_kq( int n ) const
    {
        return POW2 ? n >> lkq : n / kq;
    }
    __device__ __forceinline__ int by_cq( int n ) const
    {
        return POW2 ? n >> lcq : n / cq;
    }
    __device__ __forceinline__ int by_nc( int n ) const // blocks with c rows only (nc > 0)
    {
        return POW2 ? n >> lcq : n / nc;
    }
    __device__ __forceinline__ int by_ncb( int n ) const
    {
        return POW2 ? n / 3 : n / ncb;
    }
    __device__ __forceinline__ int by_nb( int n ) const
    {
        return POW2 ? n : n / nb;
    }
};

template<typename R, bool POW2>
__global__ void __launch_bounds__( 512, 2 ) pass_bc_cl( PassArgs<R> p, int K )
{
    namespace cg = cooperative_groups;
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank            = (int)cluster.block_rank();
    const int4 blk            = p.blocks[blockIdx.x];
    const int s               = blk.x;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mc = f.M[2], nb = f.nb;
    const int Nb = f.N[1], Nc = f.N[2];
    const int ncb = 3 * nb;
    const int ka  = blk.y;
    const int cq  = ( Nc + K - 1 ) / K;
    const int c0  = rank * cq;
    const int nc  = max( 0, min( cq, Nc - c0 ) );
    const int kq  = Mb / K;
    const int kb0 = rank * kq;
    const int lb  = cq * ncb * Mb;  // b-phase buffer
    const int lc  = Mc * ncb * kq;  // c-phase buffer
    const int crow = ncb * kq;      // elements of one c-row in the c-phase
    const ClusterSplit<POW2> sp{ kq, cq, nc, ncb, nb, __ffs( kq ) - 1, __ffs( cq ) - 1 };
    cplx<R> * twb = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * twc = twb + Mb;
    cplx<R> * Bb0 = twc + Mc;
    cplx<R> * Bb1 = Bb0 + lb;
    cplx<R> * Bc0 = Bb1 + lb;
    cplx<R> * Bc1 = Bc0 + lc;
    load_tw( twb, p.tw + f.tw_offset[1], Mb );
    load_tw( twc, p.tw + f.tw_offset[2], Mc );
    if( p.prefetch )
    {
        // this block's kb range of the dipole spectrum: one contiguous run of kq elements per
        // (pair, component, kc) row; constant, so it is requested before the programmatic wait
        const cplx<R> * Dp = p.Dhat + f.dhat_offset + (size_t)ka * nb * nb * 6 * Mc * Mb + kb0;
        const int rows     = nb * nb * 6 * Mc;
        const int per_row  = ( kq * (int)sizeof( cplx<R> ) + 127 ) / 128;
        for( int e = threadIdx.x; e < rows * per_row; e += blockDim.x )
        {
            const int rw = e / per_row, ln = e - rw * per_row;
            asm volatile( "prefetch.global.L2 [%0];" ::"l"( reinterpret_cast<const char *>( Dp + (size_t)rw * Mb ) + ln * 128 ) );
        }
    }
    for( int e = threadIdx.x; e < lb; e += blockDim.x )
        Bb0[e] = { 0, 0 };
    for( int e = threadIdx.x; e < lc; e += blockDim.x )
        Bc0[e] = { 0, 0 };
    __syncthreads();
    pdl_wait();
    pdl_trigger();
    if( sys_inactive( p, s ) ) // uniform over the cluster: its blocks share the system
        return;
    const int nin    = ncb * Nc * Nb;
    cplx<R> * W1     = p.W1 + f.spec_offset + (size_t)ka * nin;
    for( int e = threadIdx.x; e < ncb * nc * Nb; e += blockDim.x )
    {
        const int rest = (int)fdiv( (unsigned)e, f.div_Nb ), b = e - rest * Nb;
        const int cb = sp.by_nc( rest ), cl = rest - cb * nc;
        Bb0[( cl * ncb + cb ) * Mb + b] = W1[( (size_t)cb * Nc + c0 + cl ) * Nb + b];
    }
    // every block's c-phase buffer is zero before any block writes into it
    cluster.sync();
    const FastDiv none = { 1, 0, 0 };
    cplx<R> * r = sfft<R, false>( Bb0, Bb1, Mb, nc * ncb, none, Mb, 1, f.plan[1], twb, false );
    // transpose 1: rows (c0 + cl, cb), all kb -> owner of kb
    for( int e = threadIdx.x; e < nc * ncb * Mb; e += blockDim.x )
    {
        const int l = (int)fdiv( (unsigned)e, f.div_Mb ), kb = e - l * Mb;
        const int cl = sp.by_ncb( l ), cb = l - cl * ncb;
        const int d = sp.by_kq( kb ), kbl = kb - d * kq;
        cplx<R> * dst = cluster.map_shared_rank( Bc0, d );
        dst[( c0 + cl ) * crow + cb * kq + kbl] = r[l * Mb + kb];
    }
    cluster.sync();
    const FastDiv dcrow = f.div_crow;
    r           = sfft<R, true>( Bc0, Bc1, Mc, crow, dcrow, 1, crow, f.plan[2], twc, false );
    cplx<R> * o = ( r == Bc0 ) ? Bc1 : Bc0;
    // tensor product at (kc, kb0 + kbl)
    const int npair    = nb * nb;
    const cplx<R> * Dh = p.Dhat + f.dhat_offset + (size_t)ka * npair * 6 * Mc * Mb;
    for( int e = threadIdx.x; e < nb * Mc * kq; e += blockDim.x )
    {
        const int rest = sp.by_kq( e ), kbl = e - rest * kq;
        const int kc = sp.by_nb( rest ), b1 = rest - kc * nb;
        const cplx<R> * S = r + kc * crow + kbl;
        cplx<R> acc[3]    = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for( int b2 = 0; b2 < nb; ++b2 )
        {
            const cplx<R> * D = Dh + ( (size_t)( b1 * nb + b2 ) * 6 * Mc + kc ) * Mb + kb0 + kbl;
            cplx<R> dd[6];
#pragma unroll
            for( int q = 0; q < 6; ++q )
                dd[q] = D[(size_t)q * Mc * Mb];
            const cplx<R> sx = S[( b2 * 3 + 0 ) * kq];
            const cplx<R> sy = S[( b2 * 3 + 1 ) * kq];
            const cplx<R> sz = S[( b2 * 3 + 2 ) * kq];
            const int rw[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
#pragma unroll
            for( int c3 = 0; c3 < 3; ++c3 )
            {
                const cplx<R> d1 = dd[rw[c3][0]], d2 = dd[rw[c3][1]], d3 = dd[rw[c3][2]];
                acc[c3].x += d1.x * sx.x + d2.x * sy.x + d3.x * sz.x - d1.y * sx.y - d2.y * sy.y - d3.y * sz.y;
                acc[c3].y += d1.x * sx.y + d2.x * sy.y + d3.x * sz.y + d1.y * sx.x + d2.y * sy.x + d3.y * sz.x;
            }
        }
#pragma unroll
        for( int c3 = 0; c3 < 3; ++c3 )
            o[kc * crow + ( b1 * 3 + c3 ) * kq + kbl] = acc[c3];
    }
    __syncthreads();
    r = sfft<R, true>( o, ( o == Bc0 ) ? Bc1 : Bc0, Mc, crow, dcrow, 1, crow, f.plan[2], twc, true );
    // transpose 2: rows c < Nc of the kb range -> owner of row c (its b-phase buffers are free)
    for( int e = threadIdx.x; e < Nc * ncb * kq; e += blockDim.x )
    {
        const int l = sp.by_kq( e ), kbl = e - l * kq;
        const int c = sp.by_ncb( l ), cb = l - c * ncb;
        const int d = sp.by_cq( c ), cl = c - d * cq;
        cplx<R> * dst = cluster.map_shared_rank( Bb0, d );
        dst[( cl * ncb + cb ) * Mb + kb0 + kbl] = r[c * crow + cb * kq + kbl];
    }
    cluster.sync();
    r = sfft<R, false>( Bb0, Bb1, Mb, nc * ncb, none, Mb, 1, f.plan[1], twb, true );
    for( int e = threadIdx.x; e < ncb * nc * Nb; e += blockDim.x )
    {
        const int rest = (int)fdiv( (unsigned)e, f.div_Nb ), b = e - rest * Nb;
        const int cb = sp.by_nc( rest ), cl = rest - cb * nc;
        W1[( (size_t)cb * Nc + c0 + cl ) * Nb + b] = r[( cl * ncb + cb ) * Mb + b];
    }
}

// ------------------------------------------------------------------ pass A': C2R along a -> field
// Two Hermitian half spectra X, Y go through one complex inverse transform of Z = X + i Y; the
// real part is x, the imaginary part y.  The imaginary parts of X and Y at k = 0 and k = Ma/2
// are dropped, as a real inverse transform does.
template<typename R>
__global__ void __launch_bounds__( 256, sizeof( R ) == 4 ? 4 : 2 ) pass_a_inv( PassArgs<R> p )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    const FFTDesc & f = p.fd[s];
    const SysDesc & d = p.sd[s];
    const int Ma = f.M[0], Mh = f.Mh, nb = f.nb;
    const int Nc = f.N[2], Nb = f.N[1], Na = f.N[0];
    const int row = blk.y, b0 = blk.z, nl = blk.w;
    const int nq  = ( nl + 1 ) >> 1;
    const int ls  = line_stride( Ma );
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Ma;
    cplx<R> * b   = a + nq * ls;
    load_tw( tw, p.tw + f.tw_offset[0], Ma );
    pdl_wait();
    pdl_trigger();
    if( sys_inactive( p, s ) )
        return;
    // element (line li, frequency kk) of W1 in either layout
    const size_t lstride = p.ka_major ? 1 : (size_t)Mh;
    const size_t kstride = p.ka_major ? (size_t)3 * nb * Nc * Nb : 1;
    const cplx<R> * W1   = p.W1 + f.spec_offset + ( p.ka_major ? (size_t)row * Nb + b0 : ( (size_t)row * Nb + b0 ) * Mh );
    // [row][b][ka]: consecutive threads take consecutive k of a line pair; [ka][row][b]:
    // consecutive threads take consecutive line pairs of one k (contiguous b)
    const int gq = p.ka_major ? ( p.g + 1 ) >> 1 : nq; // line pairs of a full block
#pragma unroll 4
    for( int e = threadIdx.x; e < gq * Ma; e += blockDim.x )
    {
        int q, k;
        if( p.ka_major )
        {
            k = (int)fdiv( (unsigned)e, p.div_gq );
            q = e - k * gq;
            if( q >= nq )
                continue;
        }
        else
        {
            q = (int)fdiv( (unsigned)e, f.div_Ma );
            k = e - q * Ma;
        }
        const bool hi = k >= Mh;
        const int kk  = hi ? Ma - k : k;
        cplx<R> x     = W1[( 2 * q ) * lstride + kk * kstride];
        cplx<R> y     = 2 * q + 1 < nl ? W1[( 2 * q + 1 ) * lstride + kk * kstride] : cplx<R>{ 0, 0 };
        if( hi )
        {
            x.y = -x.y;
            y.y = -y.y;
        }
        if( k == 0 || 2 * k == Ma )
        {
            x.y = 0;
            y.y = 0;
        }
        a[q * ls + k] = { x.x - y.y, x.y + y.x };
    }
    __syncthreads();
    const cplx<R> * r = block_fft( a, b, Ma, ls, nq, f.plan[0], tw, true );
    const R invT = fft_invT<R>( f );
    const int cb = row / Nc, c = row - cb * Nc;
    const int ib = cb / 3, comp = cb - 3 * ib;
    R * dst      = comp == 0 ? p.hx : ( comp == 1 ? p.hy : p.hz );
    const int rowlen     = nb * Na;
    const int base       = (int)d.spin_offset + ib + rowlen * ( b0 + Nb * c ); // < 2^31 (see pass_a)
    for( int e = threadIdx.x; e < nl * Ma; e += blockDim.x )
    {
        const int li = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - li * Ma;
        if( t < Na )
        {
            const cplx<R> v = r[( li >> 1 ) * ls + t];
            dst[base + li * rowlen + nb * t] = ( ( li & 1 ) ? v.y : v.x ) * invT;
        }
    }
}

// ------------------------------------------------------------------ Dhat re-layout
template<typename R, typename RS>
__global__ void dhat_relayout( const cplx<R> * W2, cplx<RS> * Dhat, int Mh, int Mb, int Mc, int npair, int fused )
{
    long long total = (long long)npair * 6 * Mc * Mb * Mh;
    for( long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x )
    {
        int ka = e % Mh;
        int kb = ( e / Mh ) % Mb;
        int kc = ( e / ( (long long)Mh * Mb ) ) % Mc;
        int pc = e / ( (long long)Mh * Mb * Mc ); // pair*6 + comp6
        cplx<R> v = W2[e];
        if( fused ) // [ka][pair*6 + comp6][kc][kb]
            Dhat[( ( (size_t)ka * npair * 6 + pc ) * Mc + kc ) * Mb + kb] = { (RS)v.x, (RS)v.y };
        else        // [kb*Mh + ka][pair*6 + comp6][kc]
            Dhat[( ( (size_t)kb * Mh + ka ) * npair * 6 + pc ) * Mc + kc] = { (RS)v.x, (RS)v.y };
    }
}

// ================================================================== host side
static size_t smem_bc( size_t elem, const FFTDesc & f, int G = 1 )
{
    return elem * ( f.M[1] + f.M[2] + 2 * (size_t)G * f.M[2] * 3 * f.nb * f.M[1] );
}

// fused pass split over a cluster of K blocks (pass_bc_cl)
static size_t smem_bcl( size_t elem, const FFTDesc & f, int K )
{
    const size_t cq = ( f.N[2] + K - 1 ) / K, kq = f.M[1] / K, ncb = 3 * f.nb;
    return elem * ( f.M[1] + f.M[2] + 2 * cq * ncb * f.M[1] + 2 * (size_t)f.M[2] * ncb * kq );
}

// largest dynamic shared memory of one block on the current device
static size_t smem_optin()
{
    int dev = 0, v = 0;
    CUDA_CHECK( cudaGetDevice( &dev ) );
    CUDA_CHECK( cudaDeviceGetAttribute( &v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev ) );
    return (size_t)v;
}


DDIPlan::~DDIPlan()
{
    release();
}

void DDIPlan::release()
{
    dfree( d_fd );
    dfree( d_tw );
    dfree( d_W1 );
    dfree( d_W2 );
    dfree( d_Dhat );
    for( int k = 0; k < 5; ++k )
        dfree( d_blocks[k] );
    n_sys = 0;
}

void DDIPlan::build( const std::vector<DDISystem> & systems, bool fp64, const SysDesc * d_sd, cudaStream_t stream )
{
    release();
    this->fp64  = fp64;
    size_t elem = fp64 ? sizeof( cplx<double> ) : sizeof( cplx<float> );
    std::vector<FFTDesc> fds;
    std::vector<double> tw_host; // interleaved re/im in FP64
    long long spec = 0, dhat = 0;
    sys_index.clear();
    for( size_t si = 0; si < systems.size(); ++si )
    {
        const DDISystem & S = systems[si];
        FFTDesc f{};
        for( int d = 0; d < 3; ++d )
        {
            f.N[d] = S.n_cells[d];
            f.M[d] = S.padded[d];
            if( f.M[d] > MAX_FFT_LEN )
                throw std::runtime_error( "DDI FFT extent exceeds the supported maximum" );
        }
        f.Mh = f.M[0] / 2 + 1;
        f.nb = S.nb;
        for( int b = 0; b < S.nb && b < MAX_BASIS; ++b )
        {
            f.mu_d[b] = S.mu_s[b];
            f.mu_f[b] = (float)S.mu_s[b];
        }
        f.invT_d = 1.0 / ( (double)f.M[0] * f.M[1] * f.M[2] );
        f.invT_f = (float)f.invT_d;
        f.div_Ma = make_fastdiv( f.M[0] );
        f.div_Mh = make_fastdiv( f.Mh );
        f.div_Mb = make_fastdiv( f.M[1] );
        f.div_Mc = make_fastdiv( f.M[2] );
        f.div_Nb    = make_fastdiv( f.N[1] );
        f.div_Nc    = make_fastdiv( f.N[2] );
        f.div_nb    = make_fastdiv( f.nb );
        f.div_plane = make_fastdiv( 3 * f.nb * f.M[1] );
        for( int d = 0; d < 3; ++d )
        {
            f.tw_offset[d] = (long long)tw_host.size() / 2;
            for( int t = 0; t < f.M[d]; ++t )
            {
                double ang = -2.0 * M_PI * (double)t / (double)f.M[d];
                tw_host.push_back( std::cos( ang ) );
                tw_host.push_back( std::sin( ang ) );
            }
            radix_plan( f.M[d], f.plan[d] );
        }
        f.spec_offset = spec;
        long long w2  = 3LL * f.nb * f.N[2] * f.M[1] * f.Mh;
        spec += ( w2 + 31 ) / 32 * 32;
        f.dhat_offset = dhat;
        dhat += (long long)f.nb * f.nb * 6 * f.M[2] * f.M[1] * f.Mh;
        fds.push_back( f );
        sys_index.push_back( S.sys );
    }
    n_sys = (int)fds.size();
    fd_host = fds;
    // FFTDesc table indexed by the batch's system index (so kernels use p.fd[s] with the SysDesc index)
    int n_batch = 0;
    for( auto & S : systems )
        n_batch = std::max( n_batch, S.sys + 1 );
    n_fd_slots = std::max( n_batch, 1 );
    std::vector<FFTDesc> fd_by_sys( n_fd_slots );
    for( size_t k = 0; k < systems.size(); ++k )
        fd_by_sys[systems[k].sys] = fds[k];
    d_fd = dalloc<FFTDesc>( fd_by_sys.size() );
    h2d( d_fd, fd_by_sys.data(), fd_by_sys.size() );
    // twiddles in the working precision
    size_t ntw = tw_host.size() / 2;
    if( fp64 )
    {
        d_tw = dalloc_bytes( ntw * sizeof( cplx<double> ) );
        h2d_bytes( d_tw, tw_host.data(), ntw * sizeof( cplx<double> ) );
    }
    else
    {
        std::vector<float> t( tw_host.begin(), tw_host.end() );
        d_tw = dalloc_bytes( ntw * sizeof( cplx<float> ) );
        h2d_bytes( d_tw, t.data(), ntw * sizeof( cplx<float> ) );
    }
    spec_elems = spec;
    d_W1       = dalloc_bytes( std::max<long long>( spec, 1 ) * elem );
    d_W2       = dalloc_bytes( std::max<long long>( spec, 1 ) * elem );
    d_Dhat     = dalloc_bytes( std::max<long long>( dhat, 1 ) * elem );
    // fused b/c pass when every system's (c, b) plane fits into one block's shared memory
    fused = !fds.empty();
    for( auto & f : fds )
        fused = fused && smem_bc( elem, f ) <= smem_optin();
    build_block_tables( systems );
    compute_dhat( systems, d_sd, stream );
}

// Shared memory of one block of each pass (twiddles + two ping-pong line buffers)
static size_t smem_a( size_t elem, int Ma, int nl )
{
    return elem * ( Ma + 2 * (size_t)( ( nl + 1 ) / 2 ) * line_stride( Ma ) );
}
static size_t smem_b( size_t elem, int Mb, int g )
{
    return elem * ( Mb + 2 * (size_t)g * line_stride( Mb ) );
}
static size_t smem_c( size_t elem, int Mc, int ncb, int g )
{
    return elem * ( Mc + 2 * (size_t)ncb * g * line_stride( Mc ) );
}

static constexpr size_t SMEM_MAX = 200 * 1024;



static void upload_table( int4 *& dst, int & n, const std::vector<int4> & t )
{
    dfree( dst );
    dst = dalloc<int4>( std::max<size_t>( t.size(), 1 ) );
    if( !t.empty() )
        h2d( dst, t.data(), t.size() );
    n = (int)t.size();
}

// Block tables for nl_a real lines per block in passes A / A', g_b lines per block in passes
// B / B' and g_c columns per block in pass C.
void DDIPlan::set_tiles( int nl_a, int g_b, int g_c )
{
    size_t elem = fp64 ? sizeof( cplx<double> ) : sizeof( cplx<float> );
    std::vector<int4> ta, tb, tc;
    max_smem_a = max_smem_b = max_smem_c = 0;
    for( size_t k = 0; k < fd_host.size(); ++k )
    {
        const FFTDesc & f = fd_host[k];
        const int s       = sys_index[k];
        const int rows    = 3 * f.nb * f.N[2];
        for( int row = 0; row < rows; ++row )
            for( int b0 = 0; b0 < f.N[1]; b0 += nl_a )
                ta.push_back( make_int4( s, row, b0, std::min( nl_a, f.N[1] - b0 ) ) );
        const int lines = rows * f.Mh;
        for( int l0 = 0; l0 < lines; l0 += g_b )
            tb.push_back( make_int4( s, l0, std::min( g_b, lines - l0 ), 0 ) );
        const int cols = f.M[1] * f.Mh;
        for( int c0 = 0; c0 < cols; c0 += g_c )
            tc.push_back( make_int4( s, c0, std::min( g_c, cols - c0 ), 0 ) );
        max_smem_a = std::max( max_smem_a, smem_a( elem, f.M[0], nl_a ) );
        max_smem_b = std::max( max_smem_b, smem_b( elem, f.M[1], g_b ) );
        max_smem_c = std::max( max_smem_c, smem_c( elem, f.M[2], 3 * f.nb, g_c ) );
    }
    if( max_smem_a > SMEM_MAX || max_smem_b > SMEM_MAX || max_smem_c > SMEM_MAX )
        throw std::runtime_error( "DDI FFT lines do not fit into shared memory (padded extent or basis too large)" );
    upload_table( d_blocks[0], n_blocks[0], ta );
    upload_table( d_blocks[1], n_blocks[1], tb );
    upload_table( d_blocks[2], n_blocks[2], tc );
    std::vector<int4> tbc;
    smem_bc_max = 0;
    bool pow2   = true;
    if( fused )
    {
        for( size_t k = 0; k < fd_host.size(); ++k )
        {
            // several ka planes per block for one-row systems (single-block kernel only)
            const int G = ( cluster_k == 1 && fd_host[k].M[2] == 1 ) ? planes_bc : 1;
            for( int ka = 0; ka < fd_host[k].Mh; ka += G )
                for( int r = 0; r < cluster_k; ++r )
                    tbc.push_back( make_int4( sys_index[k], ka, r, std::min( G, fd_host[k].Mh - ka ) ) );
            smem_bc_max = std::max( smem_bc_max, cluster_k == 1 ? smem_bc( elem, fd_host[k], G )
                                                                : smem_bcl( elem, fd_host[k], cluster_k ) );
            FFTDesc & g   = fd_host[k];
            g.div_crow    = make_fastdiv( 3 * g.nb * g.M[1] / cluster_k );
            const int kq  = g.M[1] / cluster_k, cq = ( g.N[2] + cluster_k - 1 ) / cluster_k;
            pow2          = pow2 && g.nb == 1 && ( kq & ( kq - 1 ) ) == 0 && ( cq & ( cq - 1 ) ) == 0
                   && g.N[2] % cq == 0;
            g.div_nin     = make_fastdiv( 3 * g.nb * g.N[2] * g.N[1] );
            g.div_tens    = make_fastdiv( g.nb * g.M[2] * g.M[1] );
        }
        // FFTDesc table indexed by the batch's system index
        std::vector<FFTDesc> by_sys( n_fd_slots );
        for( size_t k = 0; k < fd_host.size(); ++k )
            by_sys[sys_index[k]] = fd_host[k];
        h2d( d_fd, by_sys.data(), by_sys.size() );
    }
    upload_table( d_blocks[3], n_blocks[3], tbc );
    bc_pow2 = fused && cluster_k > 1 && pow2;
    tile[0] = nl_a;
    tile[1] = g_b;
    tile[2] = g_c;
}

void DDIPlan::copy_shape_from( const DDIPlan & o )
{
    if( o.fp64 != fp64 || o.fused != fused || o.fd_host.size() != fd_host.size() )
        throw std::runtime_error( "DDI plans of different systems" );
    for( int k = 0; k < 3; ++k )
        threads[k] = o.threads[k];
    threads_bc = o.threads_bc;
    cluster_k  = o.cluster_k;
    planes_bc  = o.planes_bc;
    set_tiles( o.tile[0], o.tile[1], o.tile[2] );
}

void DDIPlan::build_block_tables( const std::vector<DDISystem> & )
{
    // defaults until tune() measures better ones; shrink the groups until they fit (nl even)
    size_t elem = fp64 ? sizeof( cplx<double> ) : sizeof( cplx<float> );
    int nl = 8, gb = 8, gc = 8;
    for( auto & f : fd_host )
    {
        while( nl > 2 && smem_a( elem, f.M[0], nl ) > 64 * 1024 )
            nl /= 2;
        while( gb > 1 && smem_b( elem, f.M[1], gb ) > 64 * 1024 )
            gb /= 2;
        while( gc > 1 && smem_c( elem, f.M[2], 3 * f.nb, gc ) > 64 * 1024 )
            gc /= 2;
    }
    set_tiles( nl, gb, gc );
}

template<typename R>
static PassArgs<R> make_args( const DDIPlan & P, const SysDesc * d_sd, const SysRun * runs )
{
    PassArgs<R> a{};
    a.fd    = (const FFTDesc *)P.d_fd;
    a.sd    = d_sd;
    a.runs  = runs;
    a.tw    = (const cplx<R> *)P.d_tw;
    a.W1    = (cplx<R> *)P.d_W1;
    a.W2    = (cplx<R> *)P.d_W2;
    a.Dhat  = (const cplx<R> *)P.d_Dhat;
    static const int pf = [] {
        const char * e = std::getenv( "SPIRIT_GB300_DHAT_PREFETCH" );
        return ( e && e[0] == '0' ) ? 0 : 1;
    }();
    a.prefetch = pf;
    return a;
}

template<typename R>
static void set_smem_limits()
{
    static bool done = false;
    if( done )
        return;
    CUDA_CHECK( cudaFuncSetAttribute( pass_a<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024 ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_b<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024 ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_c<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024 ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_a_inv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024 ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_bc<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin() ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_bc_cl<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin() ) );
    CUDA_CHECK( cudaFuncSetAttribute( pass_bc_cl<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin() ) );
    done = true;
}

// One-time dipole spectrum (FFT_Dipole_Matrices, Hamiltonian_Heisenberg.cpp:1406-1499): the
// tensor D(r) is summed in FP64 on the host, transformed densely on the device in FP64 and
// stored in the engine's precision.
void DDIPlan::compute_dhat( const std::vector<DDISystem> & systems, const SysDesc * d_sd, cudaStream_t stream )
{
    set_smem_limits<double>();
    const double mult = 2.0133545e-28 * 0.057883817555 * 0.057883817555 / ( 4 * M_PI * 1e-30 );
    for( size_t k = 0; k < systems.size(); ++k )
    {
        const DDISystem & S = systems[k];
        const FFTDesc & f   = fd_host[k];
        const int Ma = f.M[0], Mb = f.M[1], Mc = f.M[2], Mh = f.Mh, nb = f.nb;
        const int npair = nb * nb;
        size_t vol      = (size_t)Ma * Mb * Mc;
        std::vector<double> Dr( (size_t)npair * 6 * vol, 0.0 );
        int img[3];
        for( int d = 0; d < 3; ++d )
            img[d] = S.bc[d] == 0 ? 0 : S.images[d];
        const int Na = f.N[0], Nb = f.N[1], Nc = f.N[2];
        for( int b1 = 0; b1 < nb; ++b1 )
            for( int b2 = 0; b2 < nb; ++b2 )
            {
                double * base = Dr.data() + (size_t)( b1 * nb + b2 ) * 6 * vol;
#pragma omp parallel for collapse( 2 )
                for( int c = 0; c < Mc; ++c )
                    for( int bb = 0; bb < Mb; ++bb )
                        for( int a = 0; a < Ma; ++a )
                        {
                            int a_idx = a < Na ? a : a - Ma;
                            int b_idx = bb < Nb ? bb : bb - Mb;
                            int c_idx = c < Nc ? c : c - Mc;
                            double Dxx = 0, Dxy = 0, Dxz = 0, Dyy = 0, Dyz = 0, Dzz = 0;
                            for( int ap = -img[0]; ap <= img[0]; ++ap )
                                for( int bp = -img[1]; bp <= img[1]; ++bp )
                                    for( int cp = -img[2]; cp <= img[2]; ++cp )
                                    {
                                        double fa = a_idx + ap * Na + S.cell_atoms[b1][0] - S.cell_atoms[b2][0];
                                        double fb = b_idx + bp * Nb + S.cell_atoms[b1][1] - S.cell_atoms[b2][1];
                                        double fc = c_idx + cp * Nc + S.cell_atoms[b1][2] - S.cell_atoms[b2][2];
                                        double r[3];
                                        for( int e = 0; e < 3; ++e )
                                            r[e] = S.lattice_constant
                                                   * ( fa * S.bravais[0][e] + fb * S.bravais[1][e]
                                                       + fc * S.bravais[2][e] );
                                        double dd = std::sqrt( r[0] * r[0] + r[1] * r[1] + r[2] * r[2] );
                                        if( dd > 1e-10 )
                                        {
                                            double d3 = dd * dd * dd, d5 = dd * dd * dd * dd * dd;
                                            Dxx += mult * ( 3 * r[0] * r[0] / d5 - 1 / d3 );
                                            Dxy += mult * 3 * r[0] * r[1] / d5;
                                            Dxz += mult * 3 * r[0] * r[2] / d5;
                                            Dyy += mult * ( 3 * r[1] * r[1] / d5 - 1 / d3 );
                                            Dyz += mult * 3 * r[1] * r[2] / d5;
                                            Dzz += mult * ( 3 * r[2] * r[2] / d5 - 1 / d3 );
                                        }
                                    }
                            size_t idx = (size_t)a + Ma * ( bb + (size_t)Mb * c );
                            double v[6] = { Dxx, Dxy, Dxz, Dyy, Dyz, Dzz };
                            for( int q = 0; q < 6; ++q )
                                base[q * vol + idx] = v[q];
                        }
            }
        // dense FP64 transform on the device: lines of (pair*6+q, c, b) in Dr layout [.][c][b][a]
        int nrows = npair * 6;
        double * d_dense   = (double *)dalloc_bytes( Dr.size() * sizeof( double ) );
        h2d_bytes( d_dense, Dr.data(), Dr.size() * sizeof( double ) );
        size_t wsz = (size_t)nrows * Mc * Mb * Mh;
        cplx<double> * dW1 = (cplx<double> *)dalloc_bytes( wsz * sizeof( cplx<double> ) );
        cplx<double> * dW2 = (cplx<double> *)dalloc_bytes( wsz * sizeof( cplx<double> ) );
        // a private FFTDesc for the dense transform (nb = nrows/3 so that 3*nb = nrows lines)
        FFTDesc fdd = f;
        fdd.nb          = 1; // unused by dense mode except through 3*nb below
        fdd.spec_offset = 0;
        FFTDesc * d_fdd = dalloc<FFTDesc>( 1 );
        h2d( d_fdd, &fdd, 1 );
        PassArgs<double> pa{};
        pa.fd    = d_fdd;
        pa.sd    = d_sd;
        pa.runs  = nullptr;
        pa.tw    = (const cplx<double> *)nullptr;
        pa.mode  = 1;
        pa.dense = d_dense;
        // twiddles in FP64
        std::vector<double> twh;
        FFTDesc fl = fdd;
        for( int d = 0; d < 3; ++d )
        {
            fl.tw_offset[d] = (long long)twh.size() / 2;
            for( int t = 0; t < fl.M[d]; ++t )
            {
                double ang = -2.0 * M_PI * (double)t / (double)fl.M[d];
                twh.push_back( std::cos( ang ) );
                twh.push_back( std::sin( ang ) );
            }
        }
        h2d( d_fdd, &fl, 1 );
        void * d_twd = dalloc_bytes( twh.size() * sizeof( double ) );
        h2d_bytes( d_twd, twh.data(), twh.size() * sizeof( double ) );
        pa.tw = (const cplx<double> *)d_twd;
        pa.W1 = dW1;
        pa.W2 = dW2;
        // pass A (dense): lines = nrows * Mc * Mb, each of length Ma
        {
            int nl = 16;
            while( nl > 1 && smem_a( sizeof( cplx<double> ), Ma, nl ) > 64 * 1024 )
                nl /= 2;
            std::vector<int4> t;
            for( int row = 0; row < nrows * Mc; ++row )
                for( int b0 = 0; b0 < Mb; b0 += nl )
                    t.push_back( make_int4( 0, row, b0, std::min( nl, Mb - b0 ) ) );
            int4 * dt = dalloc<int4>( t.size() );
            h2d( dt, t.data(), t.size() );
            pa.blocks = dt;
            size_t sm = smem_a( sizeof( cplx<double> ), Ma, nl );
            pass_a<double><<<(unsigned)t.size(), 256, sm, stream>>>( pa );
            CUDA_CHECK( cudaGetLastError() );
            CUDA_CHECK( cudaStreamSynchronize( stream ) );
            dfree( dt );
        }
        // pass B forward over the nrows * Mc rows (flattened lines row*Mh + ka)
        {
            int gb = 16;
            while( gb > 1 && smem_b( sizeof( cplx<double> ), Mb, gb ) > 64 * 1024 )
                gb /= 2;
            const int lines = nrows * Mc * Mh;
            std::vector<int4> t;
            for( int l0 = 0; l0 < lines; l0 += gb )
                t.push_back( make_int4( 0, l0, std::min( gb, lines - l0 ), 0 ) );
            int4 * dt = dalloc<int4>( t.size() );
            h2d( dt, t.data(), t.size() );
            pa.blocks = dt;
            pa.g      = gb;
            pa.div_g  = make_fastdiv( gb );
            pass_b<double><<<(unsigned)t.size(), 256, smem_b( sizeof( cplx<double> ), Mb, gb ), stream>>>( pa, 0 );
            CUDA_CHECK( cudaGetLastError() );
            CUDA_CHECK( cudaStreamSynchronize( stream ) );
            dfree( dt );
        }
        // pass C forward along c: every column; the 3*nb lines per column are the nrows rows
        {
            fl.nb = nrows / 3; // nrows = 6*npair is a multiple of 3
            h2d( d_fdd, &fl, 1 );
            int gc = 16;
            while( gc > 1 && smem_c( sizeof( cplx<double> ), Mc, nrows, gc ) > 120 * 1024 )
                gc /= 2;
            const size_t sm = smem_c( sizeof( cplx<double> ), Mc, nrows, gc );
            if( sm > SMEM_MAX )
                throw std::runtime_error( "DDI dipole tensor lines do not fit into shared memory" );
            const int cols = Mb * Mh;
            std::vector<int4> t;
            for( int c0 = 0; c0 < cols; c0 += gc )
                t.push_back( make_int4( 0, c0, std::min( gc, cols - c0 ), 0 ) );
            int4 * dt = dalloc<int4>( t.size() );
            h2d( dt, t.data(), t.size() );
            pa.blocks = dt;
            pa.g      = gc;
            pa.div_g  = make_fastdiv( gc );
            pass_c<double><<<(unsigned)t.size(), 256, sm, stream>>>( pa );
            CUDA_CHECK( cudaGetLastError() );
            CUDA_CHECK( cudaStreamSynchronize( stream ) );
            dfree( dt );
        }
        // W2 now holds [row][kc][kb][ka]; re-layout into Dhat[kb][ka][row][kc]
        if( fp64 )
            dhat_relayout<double, double><<<1024, 256, 0, stream>>>(
                dW2, (cplx<double> *)d_Dhat + f.dhat_offset, Mh, Mb, Mc, npair, fused ? 1 : 0 );
        else
            dhat_relayout<double, float><<<1024, 256, 0, stream>>>(
                dW2, (cplx<float> *)d_Dhat + f.dhat_offset, Mh, Mb, Mc, npair, fused ? 1 : 0 );
        CUDA_CHECK( cudaGetLastError() );
        CUDA_CHECK( cudaStreamSynchronize( stream ) );
        dfree( d_dense );
        dfree( dW1 );
        dfree( dW2 );
        dfree( d_fdd );
        dfree( d_twd );
    }
}

// pass k of the convolution: 0 A, 1 B, 2 C, 3 B', 4 A'
template<typename R>
void DDIPlan::launch_pass( int k, PassArgs<R> & a, cudaStream_t stream ) const
{
    a.ka_major = fused ? 1 : 0;
    switch( k )
    {
    case 0:
        a.blocks = d_blocks[0];
        a.g      = tile[0];
        a.div_g  = make_fastdiv( tile[0] );
        launch_pdl( pass_a<R>, dim3( n_blocks[0] ), dim3( threads[0] ), max_smem_a, stream, 1, a );
        break;
    case 1:
    case 3:
        a.blocks = d_blocks[1];
        a.g      = tile[1];
        a.div_g  = make_fastdiv( tile[1] );
        pass_b<R><<<n_blocks[1], threads[1], max_smem_b, stream>>>( a, k == 3 );
        break;
    case 2:
        a.blocks = d_blocks[2];
        a.g      = tile[2];
        a.div_g  = make_fastdiv( tile[2] );
        pass_c<R><<<n_blocks[2], threads[2], max_smem_c, stream>>>( a );
        break;
    case 5:
        a.blocks = d_blocks[3];
        if( cluster_k == 1 )
            launch_pdl( pass_bc<R>, dim3( n_blocks[3] ), dim3( threads_bc ), smem_bc_max, stream, 1, a );
        else
            launch_pdl( bc_pow2 ? pass_bc_cl<R, true> : pass_bc_cl<R, false>, dim3( n_blocks[3] ),
                        dim3( std::min( threads_bc, 512 ) ), smem_bc_max, stream,
                        cluster_k, a, cluster_k );
        break;
    default:
        a.blocks = d_blocks[0];
        a.g      = tile[0];
        a.div_g  = make_fastdiv( tile[0] );
        a.div_gq = make_fastdiv( ( tile[0] + 1 ) / 2 );
        launch_pdl( pass_a_inv<R>, dim3( n_blocks[0] ), dim3( threads[0] ), max_smem_a, stream, 1, a );
        break;
    }
}

// Autotuner: for each pass, time the candidate lines (columns) per block on the plan's own
// systems with CUDA events and keep the fastest.  Passes A/A' and B/B' share a table and are
// timed together.  Runs outside any stream capture; overwrites the field arrays and the work
// spectra only.
template<typename R>
void DDIPlan::tune_t( const SysDesc * d_sd, const R * sx, const R * sy, const R * sz, R * hx, R * hy, R * hz,
                      cudaStream_t stream )
{
    if( n_sys == 0 )
        return;
    set_smem_limits<R>();
    PassArgs<R> a = make_args<R>( *this, d_sd, nullptr );
    a.sx          = sx;
    a.sy          = sy;
    a.sz          = sz;
    a.hx          = hx;
    a.hy          = hy;
    a.hz          = hz;
    a.mode        = 0;
    const size_t elem = sizeof( cplx<R> );
    int maxN1 = 1, maxM0 = 1, maxM1 = 1, maxM2 = 1, maxnb = 1;
    long long lines_b = 0, cols_c = 0;
    for( auto & f : fd_host )
    {
        maxN1 = std::max( maxN1, f.N[1] );
        maxM0 = std::max( maxM0, f.M[0] );
        maxM1 = std::max( maxM1, f.M[1] );
        maxM2 = std::max( maxM2, f.M[2] );
        maxnb = std::max( maxnb, f.nb );
        lines_b += 3LL * f.nb * f.N[2] * f.Mh;
        cols_c += (long long)f.M[1] * f.Mh;
    }
    cudaEvent_t e0, e1;
    CUDA_CHECK( cudaEventCreate( &e0 ) );
    CUDA_CHECK( cudaEventCreate( &e1 ) );
    auto timed = [&]( std::initializer_list<int> passes ) {
        for( int k : passes )
            launch_pass<R>( k, a, stream );
        // the best of three timed groups of four (timings of short kernels are noisy)
        float best_ms = 1e30f;
        for( int trial = 0; trial < 3; ++trial )
        {
            CUDA_CHECK( cudaEventRecord( e0, stream ) );
            const int reps = 4;
            for( int r = 0; r < reps; ++r )
                for( int k : passes )
                    launch_pass<R>( k, a, stream );
            CUDA_CHECK( cudaEventRecord( e1, stream ) );
            CUDA_CHECK( cudaEventSynchronize( e1 ) );
            CUDA_CHECK( cudaGetLastError() );
            float ms = 0;
            CUDA_CHECK( cudaEventElapsedTime( &ms, e0, e1 ) );
            best_ms = std::min( best_ms, ms );
        }
        return best_ms;
    };
    // warm-up of the whole chain (first launches pay module loading)
    if( fused )
        timed( { 0, 5, 4 } );
    else
        timed( { 0, 1, 2, 3, 4 } );
    int best[3] = { tile[0], tile[1], tile[2] };
    int bthr[3] = { threads[0], threads[1], threads[2] };
    const int thread_opts[3] = { 64, 128, 256 };
    {
        float bt = 1e30f;
        for( int nl : { 2, 4, 6, 8, 12, 16, 24, 32, 48, 64 } )
        {
            // even counts only: lines are then always paired (even b, odd b) whatever the tile,
            // so the results do not depend on the tuner's choice.  At least 8 lines when the
            // systems allow: with the ka-major spectrum a block reads / writes runs of its lines
            // per frequency, and runs of 2-6 complex values (16-48 B) timed well back to back but
            // left pass A' 60 % stalled on those loads inside the step
            if( ( nl > maxN1 && nl > 2 ) || smem_a( elem, maxM0, nl ) > 96 * 1024 || ( nl < 8 && maxN1 >= 8 && fused ) )
                continue;
            set_tiles( nl, best[1], best[2] );
            for( int th : thread_opts )
            {
                threads[0] = th;
                float t    = timed( { 0, 4 } );
                if( t < bt )
                {
                    bt      = t;
                    best[0] = nl;
                    bthr[0] = th;
                }
            }
        }
        threads[0] = bthr[0];
        // override "lines,threads" (measurements, profiles)
        if( const char * e = std::getenv( "SPIRIT_GB300_A" ) )
        {
            int nl = 0, th = 0;
            if( std::sscanf( e, "%d,%d", &nl, &th ) == 2 && nl >= 2 && nl % 2 == 0 && nl <= 64
                && ( th == 64 || th == 128 || th == 256 ) && smem_a( elem, maxM0, nl ) <= 96 * 1024 )
            {
                best[0]    = nl;
                threads[0] = th;
            }
        }
    }
    if( fused )
    {
        // cluster size K (the plane split over K blocks) and threads per block; K = 1 is the
        // single-block kernel.  The arithmetic of every line is the same for every K.
        float bt = 1e30f, t_pref = 1e30f;
        int bthr_bc = threads_bc, bk = 1;
        for( int K : { 1, 2, 4, 8 } )
        {
            bool ok = true;
            for( auto & f : fd_host )
                ok = ok && ( K == 1 || ( f.M[1] % K == 0 && f.N[2] >= K && smem_bcl( elem, f, K ) <= smem_optin() ) );
            if( !ok )
                continue;
            cluster_k = K;
            set_tiles( best[0], best[1], best[2] );
            for( int th : { 128, 256, 512, 1024 } )
            {
                if( ( K > 1 && th > 512 ) || ( K == 1 && th < 256 ) )
                    continue;
                threads_bc = th;
                // timed inside the chain it runs in (A, b/c, A'): in isolation the same launches
                // overlap one another and favour other shapes
                float t = timed( { 0, 5, 4 } );
                if( K == 4 && th == 512 )
                    t_pref = t;
                if( t < bt )
                {
                    bt      = t;
                    bthr_bc = th;
                    bk      = K;
                }
            }
        }
        // Warm-L2 timings here rank the shapes within a few per cent of each other and not always
        // in the order of the step loop (cold dipole spectrum after other work): 4-block clusters
        // of 512 threads measured best there (128x128x16 Heun, fixed shapes interleaved: 0.1039
        // ms/step; 1 x 1024 0.105, 8 x 256 0.107, 2 x 512 0.107, 8 x 128 0.113, 4 x 256 0.115), so
        // they are kept unless another shape is more than 5 % faster here.
        if( t_pref <= 1.05f * bt )
        {
            bt      = t_pref;
            bthr_bc = 512;
            bk      = 4;
        }
        threads_bc = bthr_bc;
        cluster_k  = bk;
        // planes per block on one-row (2D) systems: their planes are only 3 nb lines of Mb points,
        // so one plane per block leaves most threads idle
        bool one_row = false;
        for( auto & f : fd_host )
            one_row = one_row || f.M[2] == 1;
        if( cluster_k == 1 && one_row )
        {
            float bg = 1e30f;
            int bgv  = 1;
            for( int G : { 1, 2, 4, 8, 16 } )
            {
                bool ok = true;
                for( auto & f : fd_host )
                    ok = ok && smem_bc( elem, f, f.M[2] == 1 ? G : 1 ) <= smem_optin();
                if( !ok )
                    continue;
                planes_bc = G;
                set_tiles( best[0], best[1], best[2] );
                float t = timed( { 0, 5, 4 } );
                if( t < bg )
                {
                    bg  = t;
                    bgv = G;
                }
            }
            planes_bc = bgv;
        }
        // override "K,threads" (measurements)
        if( const char * e = std::getenv( "SPIRIT_GB300_BC" ) )
        {
            int K = 0, th = 0;
            if( std::sscanf( e, "%d,%d", &K, &th ) == 2 && ( K == 1 || K == 2 || K == 4 || K == 8 )
                && ( th == 128 || th == 256 || th == 512 || ( th == 1024 && K == 1 ) ) )
            {
                bool ok = true;
                for( auto & f : fd_host )
                    ok = ok && ( K == 1 || ( f.M[1] % K == 0 && f.N[2] >= K && smem_bcl( elem, f, K ) <= smem_optin() ) );
                if( ok )
                {
                    cluster_k  = K;
                    threads_bc = th;
                }
            }
        }
    }
    else
    {
        float bt = 1e30f;
        for( int g : { 1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 24, 32 } )
        {
            if( g > lines_b || smem_b( elem, maxM1, g ) > 96 * 1024 )
                continue;
            set_tiles( best[0], g, best[2] );
            for( int th : thread_opts )
            {
                threads[1] = th;
                float t    = timed( { 1, 3 } );
                if( t < bt )
                {
                    bt      = t;
                    best[1] = g;
                    bthr[1] = th;
                }
            }
        }
        threads[1] = bthr[1];
    }
    if( !fused )
    {
        float bt = 1e30f;
        for( int g : { 1, 2, 3, 4, 5, 6, 8, 10, 12, 16 } )
        {
            if( g > cols_c || smem_c( elem, maxM2, 3 * maxnb, g ) > 96 * 1024 )
                continue;
            set_tiles( best[0], best[1], g );
            for( int th : thread_opts )
            {
                threads[2] = th;
                float t    = timed( { 2 } );
                if( t < bt )
                {
                    bt      = t;
                    best[2] = g;
                    bthr[2] = th;
                }
            }
        }
        threads[2] = bthr[2];
    }
    set_tiles( best[0], best[1], best[2] );
    CUDA_CHECK( cudaEventDestroy( e0 ) );
    CUDA_CHECK( cudaEventDestroy( e1 ) );
}

void DDIPlan::tune( const SysDesc * d_sd, const void * sx, const void * sy, const void * sz, void * hx, void * hy,
                    void * hz, cudaStream_t stream )
{
    if( fp64 )
        tune_t<double>( d_sd, (const double *)sx, (const double *)sy, (const double *)sz, (double *)hx, (double *)hy,
                        (double *)hz, stream );
    else
        tune_t<float>( d_sd, (const float *)sx, (const float *)sy, (const float *)sz, (float *)hx, (float *)hy,
                       (float *)hz, stream );
}

template<typename R>
void DDIPlan::run_t( const SysDesc * d_sd, const SysRun * runs, const R * sx, const R * sy, const R * sz, R * hx,
                     R * hy, R * hz, cudaStream_t stream, int only ) const
{
    if( n_sys == 0 )
        return;
    set_smem_limits<R>();
    PassArgs<R> a = make_args<R>( *this, d_sd, runs );
    a.sx          = sx;
    a.sy          = sy;
    a.sz          = sz;
    a.hx          = hx;
    a.hy          = hy;
    a.hz          = hz;
    a.mode        = 0;
    size_t elem   = sizeof( cplx<R> );
    (void)elem;
    auto mark = [&]( int id ) {
        if( trace )
        {
            cudaEvent_t e;
            CUDA_CHECK( cudaEventCreate( &e ) );
            CUDA_CHECK( cudaEventRecord( e, stream ) );
            trace->push_back( { id, e } );
        }
    };
    if( only >= 0 )
    {
        // one pass alone (the row-fused stage kernels do A and A' themselves)
        mark( only == 0 ? KERNEL_PASS_A : KERNEL_PASS_BC );
        launch_pass<R>( only, a, stream );
    }
    else if( fused )
    {
        static const int ks[3]  = { 0, 5, 4 };
        static const int ids[3] = { KERNEL_PASS_A, KERNEL_PASS_BC, KERNEL_PASS_A_INV };
        for( int q = 0; q < 3; ++q )
        {
            mark( ids[q] );
            launch_pass<R>( ks[q], a, stream );
        }
    }
    else
        for( int k = 0; k < 5; ++k )
        {
            static const int ids[5] = { KERNEL_PASS_A, KERNEL_PASS_B, KERNEL_PASS_C, KERNEL_PASS_B_INV, KERNEL_PASS_A_INV };
            mark( ids[k] );
            launch_pass<R>( k, a, stream );
        }
    CUDA_CHECK( cudaGetLastError() );
}

void DDIPlan::run( const SysDesc * d_sd, const SysRun * runs, const void * sx, const void * sy, const void * sz,
                   void * hx, void * hy, void * hz, cudaStream_t stream, int only ) const
{
    if( fp64 )
        run_t<double>( d_sd, runs, (const double *)sx, (const double *)sy, (const double *)sz, (double *)hx,
                       (double *)hy, (double *)hz, stream, only );
    else
        run_t<float>( d_sd, runs, (const float *)sx, (const float *)sy, (const float *)sz, (float *)hx, (float *)hy,
                      (float *)hz, stream, only );
}

} // namespace sg
