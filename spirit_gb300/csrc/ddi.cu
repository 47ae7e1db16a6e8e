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

#include <cmath>
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
};

template<typename R>
__device__ __forceinline__ void load_tw( cplx<R> * dst, const cplx<R> * src, int L )
{
    for( int t = threadIdx.x; t < L; t += blockDim.x )
        dst[t] = src[t];
}

template<typename R>
__device__ __forceinline__ bool sys_inactive( const PassArgs<R> & p, int s )
{
    return p.runs && !p.runs[s].active;
}

// Block tables:
//   pass A / A' : (system, row = cb*Cin + c, first b, number of lines)
//   pass B / C  : (system, group index, G = lines per group (a power of two), 0)
// ------------------------------------------------------------------ pass A: R2C along a
template<typename R>
__global__ void pass_a( PassArgs<R> p )
{
    extern __shared__ unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const int Ma = f.M[0], Mh = f.Mh, nb = f.nb;
    const int Cin = p.mode ? f.M[2] : f.N[2];
    const int Bin = p.mode ? f.M[1] : f.N[1];
    const int Ain = p.mode ? f.M[0] : f.N[0];
    const int row = blk.y, b0 = blk.z, nl = blk.w;
    const int ls  = line_stride( Ma );
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Ma;
    cplx<R> * b   = a + nl * ls;
    load_tw( tw, p.tw + f.tw_offset[0], Ma );
    const int cb = row / Cin, c = row - cb * Cin;
    const int ib = cb / 3, comp = cb - 3 * ib;
    if( p.mode == 0 )
    {
        const SysDesc & d  = p.sd[s];
        const R mu         = fft_mu<R>( f, ib );
        const R * src      = comp == 0 ? p.sx : ( comp == 1 ? p.sy : p.sz );
        const long long base = d.spin_offset + ib + (long long)nb * d.n_cells[0] * ( (long long)b0 + (long long)d.n_cells[1] * c );
        const int rowlen   = nb * d.n_cells[0];
        for( int e = threadIdx.x; e < nl * Ma; e += blockDim.x )
        {
            int li = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - li * Ma;
            R v    = 0;
            if( t < Ain )
                v = mu * src[base + (long long)li * rowlen + (long long)nb * t];
            a[li * ls + t] = { v, (R)0 };
        }
    }
    else
    {
        for( int e = threadIdx.x; e < nl * Ma; e += blockDim.x )
        {
            int li = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - li * Ma;
            a[li * ls + t] = { p.dense[( (size_t)row * Bin + b0 + li ) * Ma + t], (R)0 };
        }
    }
    __syncthreads();
    cplx<R> * r  = block_fft( a, b, Ma, ls, nl, f.radix[0], tw, false );
    cplx<R> * W1 = p.W1 + f.spec_offset + ( (size_t)row * Bin + b0 ) * Mh;
    for( int e = threadIdx.x; e < nl * Mh; e += blockDim.x )
    {
        int li = (int)fdiv( (unsigned)e, f.div_Mh ), k = e - li * Mh;
        W1[e]  = r[li * ls + k];
    }
}

// ------------------------------------------------------------------ pass B: C2C along b
// block: fixed row = (cb, c), a group of G consecutive ka.  forward: W1 -> W2, inverse: W2 -> W1.
template<typename R>
__global__ void pass_b( PassArgs<R> p, int inverse )
{
    extern __shared__ unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mh = f.Mh;
    const int Bin = p.mode ? f.M[1] : f.N[1];
    const int G   = blk.z;
    const int lgG = __ffs( G ) - 1;
    const int ngk = ( Mh + G - 1 ) >> lgG;
    const int row = blk.y / ngk;
    const int kg  = blk.y - row * ngk;
    const int ka0 = kg << lgG;
    const int nl  = min( G, Mh - ka0 );
    const int ls  = line_stride( Mb );
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Mb;
    cplx<R> * b   = a + G * ls;
    load_tw( tw, p.tw + f.tw_offset[1], Mb );
    cplx<R> * W1 = p.W1 + f.spec_offset;
    cplx<R> * W2 = p.W2 + f.spec_offset;
    for( int e = threadIdx.x; e < ( Mb << lgG ); e += blockDim.x )
    {
        int t = e >> lgG, li = e & ( G - 1 ); // consecutive threads -> consecutive ka (coalesced)
        if( li >= nl )
            continue;
        cplx<R> v = { 0, 0 };
        if( !inverse )
        {
            if( t < Bin )
                v = W1[( (size_t)row * Bin + t ) * Mh + ka0 + li];
        }
        else
            v = W2[( (size_t)row * Mb + t ) * Mh + ka0 + li];
        a[li * ls + t] = v;
    }
    __syncthreads();
    cplx<R> * r = block_fft( a, b, Mb, ls, nl, f.radix[1], tw, inverse != 0 );
    const int Bout = inverse ? f.N[1] : Mb;
    for( int e = threadIdx.x; e < ( Bout << lgG ); e += blockDim.x )
    {
        int t = e >> lgG, li = e & ( G - 1 );
        if( li >= nl )
            continue;
        if( !inverse )
            W2[( (size_t)row * Mb + t ) * Mh + ka0 + li] = r[li * ls + t];
        else
            W1[( (size_t)row * Bout + t ) * Mh + ka0 + li] = r[li * ls + t];
    }
}

// ------------------------------------------------------------------ pass C: along c + tensor product
// block: fixed kb, a group of G consecutive ka, all 3*nb components (line li = cb*G + g).
template<typename R>
__global__ void pass_c( PassArgs<R> p )
{
    extern __shared__ unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const int Mb = f.M[1], Mc = f.M[2], Mh = f.Mh, nb = f.nb;
    const int ncb = 3 * nb;
    const int Cin = p.mode ? f.M[2] : f.N[2];
    const int G   = blk.z;
    const int lgG = __ffs( G ) - 1;
    const int ngk = ( Mh + G - 1 ) >> lgG;
    const int kb  = blk.y / ngk;
    const int kg  = blk.y - kb * ngk;
    const int ka0 = kg << lgG;
    const int ng  = min( G, Mh - ka0 );
    const int ls  = line_stride( Mc );
    const int nl  = ncb << lgG; // lines g >= ng are computed but never stored
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Mc;
    cplx<R> * b   = a + nl * ls;
    load_tw( tw, p.tw + f.tw_offset[2], Mc );
    cplx<R> * W2 = p.W2 + f.spec_offset;
    const int total = nl * Mc;
    for( int e = threadIdx.x; e < total; e += blockDim.x )
    {
        // e -> (cb, c, g) with g fastest for coalescing
        int g    = e & ( G - 1 );
        int rest = e >> lgG;
        int cb   = (int)fdiv( (unsigned)rest, f.div_Mc );
        int c    = rest - cb * Mc;
        cplx<R> v = { 0, 0 };
        if( c < Cin && g < ng )
            v = W2[( ( (size_t)cb * Cin + c ) * Mb + kb ) * Mh + ka0 + g];
        a[( cb * G + g ) * ls + c] = v;
    }
    __syncthreads();
    cplx<R> * r = Mc > 1 ? block_fft( a, b, Mc, ls, nl, f.radix[2], tw, false ) : a;
    if( p.mode == 1 )
    {
        // dense forward transform: write every kc
        for( int e = threadIdx.x; e < total; e += blockDim.x )
        {
            int g    = e & ( G - 1 );
            int rest = e >> lgG;
            int cb   = (int)fdiv( (unsigned)rest, f.div_Mc );
            int c    = rest - cb * Mc;
            if( g < ng )
                W2[( ( (size_t)cb * Mc + c ) * Mb + kb ) * Mh + ka0 + g] = r[( cb * G + g ) * ls + c];
        }
        return;
    }
    // tensor product H_b1 = sum_b2 D_b1b2 . S_b2 (FFT.hpp:42-49 mult3D rows: xx xy xz | xy yy yz | xz yz zz)
    cplx<R> * h        = ( r == a ) ? b : a;
    const cplx<R> * Dh = p.Dhat + f.dhat_offset;
    const int npair    = nb * nb;
    for( int e = threadIdx.x; e < ( nb * Mc ) << lgG; e += blockDim.x )
    {
        int g    = e & ( G - 1 );
        int rest = e >> lgG;
        int b1   = (int)fdiv( (unsigned)rest, f.div_Mc );
        int kc   = rest - b1 * Mc;
        if( g >= ng )
            continue;
        cplx<R> acc[3] = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for( int b2 = 0; b2 < nb; ++b2 )
        {
            const cplx<R> * D = Dh + ( ( (size_t)kb * Mh + ka0 + g ) * npair + b1 * nb + b2 ) * 6 * Mc + kc;
            cplx<R> d[6];
#pragma unroll
            for( int q = 0; q < 6; ++q )
                d[q] = D[q * Mc];
            cplx<R> sx = r[( ( b2 * 3 + 0 ) * G + g ) * ls + kc];
            cplx<R> sy = r[( ( b2 * 3 + 1 ) * G + g ) * ls + kc];
            cplx<R> sz = r[( ( b2 * 3 + 2 ) * G + g ) * ls + kc];
            const int row[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
#pragma unroll
            for( int c3 = 0; c3 < 3; ++c3 )
            {
                cplx<R> d1 = d[row[c3][0]], d2 = d[row[c3][1]], d3 = d[row[c3][2]];
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
    cplx<R> * o     = Mc > 1 ? block_fft( h, other, Mc, ls, nl, f.radix[2], tw, true ) : h;
    const int Cout  = f.N[2];
    for( int e = threadIdx.x; e < total; e += blockDim.x )
    {
        int g    = e & ( G - 1 );
        int rest = e >> lgG;
        int cb   = (int)fdiv( (unsigned)rest, f.div_Mc );
        int c    = rest - cb * Mc;
        if( c < Cout && g < ng )
            W2[( ( (size_t)cb * Cin + c ) * Mb + kb ) * Mh + ka0 + g] = o[( cb * G + g ) * ls + c];
    }
}

// ------------------------------------------------------------------ pass A': C2R along a -> field
template<typename R>
__global__ void pass_a_inv( PassArgs<R> p )
{
    extern __shared__ unsigned char smem_raw[];
    const int4 blk = p.blocks[blockIdx.x];
    const int s    = blk.x;
    if( sys_inactive( p, s ) )
        return;
    const FFTDesc & f = p.fd[s];
    const SysDesc & d = p.sd[s];
    const int Ma = f.M[0], Mh = f.Mh, nb = f.nb;
    const int Nc = f.N[2], Nb = f.N[1], Na = f.N[0];
    const int row = blk.y, b0 = blk.z, nl = blk.w;
    const int ls  = line_stride( Ma );
    cplx<R> * tw  = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * a   = tw + Ma;
    cplx<R> * b   = a + nl * ls;
    load_tw( tw, p.tw + f.tw_offset[0], Ma );
    const cplx<R> * W1 = p.W1 + f.spec_offset + ( (size_t)row * Nb + b0 ) * Mh;
    for( int e = threadIdx.x; e < nl * Ma; e += blockDim.x )
    {
        int li = (int)fdiv( (unsigned)e, f.div_Ma ), k = e - li * Ma;
        cplx<R> v;
        if( k < Mh )
            v = W1[li * Mh + k];
        else
            v = cconj( W1[li * Mh + ( Ma - k )] );
        a[li * ls + k] = v;
    }
    __syncthreads();
    cplx<R> * r  = block_fft( a, b, Ma, ls, nl, f.radix[0], tw, true );
    const R invT = fft_invT<R>( f );
    const int cb = row / Nc, c = row - cb * Nc;
    const int ib = cb / 3, comp = cb - 3 * ib;
    R * dst      = comp == 0 ? p.hx : ( comp == 1 ? p.hy : p.hz );
    const long long base = d.spin_offset + ib + (long long)nb * Na * ( (long long)b0 + (long long)Nb * c );
    const int rowlen     = nb * Na;
    for( int e = threadIdx.x; e < nl * Ma; e += blockDim.x )
    {
        int li = (int)fdiv( (unsigned)e, f.div_Ma ), t = e - li * Ma;
        if( t < Na )
            dst[base + (long long)li * rowlen + (long long)nb * t] = r[li * ls + t].x * invT;
    }
}

// ------------------------------------------------------------------ Dhat re-layout
template<typename R, typename RS>
__global__ void dhat_relayout( const cplx<R> * W2, cplx<RS> * Dhat, int Mh, int Mb, int Mc, int npair )
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
        Dhat[( ( (size_t)kb * Mh + ka ) * npair * 6 + pc ) * Mc + kc] = { (RS)v.x, (RS)v.y };
    }
}

// ================================================================== host side
static void factorize( int L, int * rad )
{
    int n = 0;
    while( L % 4 == 0 && L > 4 )
    {
        rad[n++] = 4;
        L /= 4;
    }
    for( int p : { 4, 2, 3, 5, 7 } )
        while( L % p == 0 && L > 1 )
        {
            rad[n++] = p;
            L /= p;
        }
    for( int p = 11; L > 1; p += 2 )
        while( L % p == 0 )
        {
            rad[n++] = p;
            L /= p;
        }
    rad[n] = 0;
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
        for( int d = 0; d < 3; ++d )
        {
            f.tw_offset[d] = (long long)tw_host.size() / 2;
            for( int t = 0; t < f.M[d]; ++t )
            {
                double ang = -2.0 * M_PI * (double)t / (double)f.M[d];
                tw_host.push_back( std::cos( ang ) );
                tw_host.push_back( std::sin( ang ) );
            }
            factorize( f.M[d], f.radix[d] );
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
    std::vector<FFTDesc> fd_by_sys( std::max( n_batch, 1 ) );
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
    build_block_tables( systems );
    compute_dhat( systems, d_sd, stream );
}

// Lines per block: keep the two ping-pong buffers of a block within `budget` bytes; the result is
// a power of two (block tables of passes B and C rely on it).
static int group_for( int line_len, int lines_per_group, size_t elem, size_t budget, int cap )
{
    int ls = line_stride( line_len );
    int g  = (int)( budget / ( 2 * elem * (size_t)ls * lines_per_group ) );
    int p  = 1;
    while( p * 2 <= g && p * 2 <= cap )
        p *= 2;
    return p;
}

static size_t smem_a( size_t elem, int Ma, int nl )
{
    return elem * ( Ma + 2 * (size_t)nl * line_stride( Ma ) );
}

void DDIPlan::build_block_tables( const std::vector<DDISystem> & systems )
{
    size_t elem   = fp64 ? sizeof( cplx<double> ) : sizeof( cplx<float> );
    size_t budget = 16 * 1024;
    std::vector<int4> ta, tb, tc;
    max_smem_a = max_smem_b = max_smem_c = 0;
    for( size_t k = 0; k < systems.size(); ++k )
    {
        const FFTDesc & f = fd_host[k];
        int s             = systems[k].sys;
        int nl            = group_for( f.M[0], 1, elem, budget, 32 );
        for( int row = 0; row < 3 * f.nb * f.N[2]; ++row )
            for( int b0 = 0; b0 < f.N[1]; b0 += nl )
                ta.push_back( make_int4( s, row, b0, std::min( nl, f.N[1] - b0 ) ) );
        max_smem_a = std::max( max_smem_a, smem_a( elem, f.M[0], nl ) );
        int gb  = group_for( f.M[1], 1, elem, budget, 32 );
        int ngb = ( f.Mh + gb - 1 ) / gb;
        for( int g = 0; g < 3 * f.nb * f.N[2] * ngb; ++g )
            tb.push_back( make_int4( s, g, gb, 0 ) );
        max_smem_b = std::max( max_smem_b, elem * ( f.M[1] + 2 * (size_t)gb * line_stride( f.M[1] ) ) );
        int gc  = group_for( f.M[2], 3 * f.nb, elem, budget, 32 );
        int ngc = ( f.Mh + gc - 1 ) / gc;
        for( int g = 0; g < f.M[1] * ngc; ++g )
            tc.push_back( make_int4( s, g, gc, 0 ) );
        max_smem_c = std::max( max_smem_c, elem * ( f.M[2] + 2 * (size_t)3 * f.nb * gc * line_stride( f.M[2] ) ) );
    }
    n_blocks[0] = (int)ta.size();
    n_blocks[1] = (int)tb.size();
    n_blocks[2] = (int)tc.size();
    d_blocks[0] = dalloc<int4>( std::max<size_t>( ta.size(), 1 ) );
    d_blocks[1] = dalloc<int4>( std::max<size_t>( tb.size(), 1 ) );
    d_blocks[2] = dalloc<int4>( std::max<size_t>( tc.size(), 1 ) );
    if( !ta.empty() )
        h2d( (int4 *)d_blocks[0], ta.data(), ta.size() );
    if( !tb.empty() )
        h2d( (int4 *)d_blocks[1], tb.data(), tb.size() );
    if( !tc.empty() )
        h2d( (int4 *)d_blocks[2], tc.data(), tc.size() );
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
            int nl = group_for( Ma, 1, sizeof( cplx<double> ), 56 * 1024, 32 );
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
        // pass B forward: rows = nrows * Mc  (3*nb*Cin with nb=1 would be 3*Mc: use a row table)
        {
            int gb  = group_for( Mb, 1, sizeof( cplx<double> ), 56 * 1024, 32 );
            int ngk = ( Mh + gb - 1 ) / gb;
            std::vector<int4> t;
            for( int g = 0; g < nrows * Mc * ngk; ++g )
                t.push_back( make_int4( 0, g, gb, 0 ) );
            int4 * dt = dalloc<int4>( t.size() );
            h2d( dt, t.data(), t.size() );
            pa.blocks = dt;
            size_t sm = sizeof( cplx<double> ) * ( Mb + 2 * (size_t)gb * line_stride( Mb ) );
            pass_b<double><<<(unsigned)t.size(), 256, sm, stream>>>( pa, 0 );
            CUDA_CHECK( cudaGetLastError() );
            CUDA_CHECK( cudaStreamSynchronize( stream ) );
            dfree( dt );
        }
        // pass C forward along c: every (kb, ka-group); the 3*nb lines per group are the nrows rows
        {
            // nrows = 6*npair is a multiple of 3: the 3*nb lines of a group are the nrows rows
            fl.nb = nrows / 3;
            h2d( d_fdd, &fl, 1 );
            int gc  = group_for( Mc, nrows, sizeof( cplx<double> ), 120 * 1024, 32 );
            int ngk = ( Mh + gc - 1 ) / gc;
            std::vector<int4> t;
            for( int g = 0; g < Mb * ngk; ++g )
                t.push_back( make_int4( 0, g, gc, 0 ) );
            int4 * dt = dalloc<int4>( t.size() );
            h2d( dt, t.data(), t.size() );
            pa.blocks = dt;
            size_t sm = sizeof( cplx<double> ) * ( Mc + 2 * (size_t)nrows * gc * line_stride( Mc ) );
            pass_c<double><<<(unsigned)t.size(), 256, sm, stream>>>( pa );
            CUDA_CHECK( cudaGetLastError() );
            CUDA_CHECK( cudaStreamSynchronize( stream ) );
            dfree( dt );
        }
        // W2 now holds [row][kc][kb][ka]; re-layout into Dhat[kb][ka][row][kc]
        if( fp64 )
            dhat_relayout<double, double><<<1024, 256, 0, stream>>>(
                dW2, (cplx<double> *)d_Dhat + f.dhat_offset, Mh, Mb, Mc, npair );
        else
            dhat_relayout<double, float><<<1024, 256, 0, stream>>>(
                dW2, (cplx<float> *)d_Dhat + f.dhat_offset, Mh, Mb, Mc, npair );
        CUDA_CHECK( cudaGetLastError() );
        CUDA_CHECK( cudaStreamSynchronize( stream ) );
        dfree( d_dense );
        dfree( dW1 );
        dfree( dW2 );
        dfree( d_fdd );
        dfree( d_twd );
    }
}

template<typename R>
void DDIPlan::run_t( const SysDesc * d_sd, const SysRun * runs, const R * sx, const R * sy, const R * sz, R * hx,
                     R * hy, R * hz, cudaStream_t stream ) const
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
    a.blocks = (const int4 *)d_blocks[0];
    mark( KERNEL_PASS_A );
    pass_a<R><<<n_blocks[0], 256, max_smem_a, stream>>>( a );
    a.blocks = (const int4 *)d_blocks[1];
    mark( KERNEL_PASS_B );
    pass_b<R><<<n_blocks[1], 256, max_smem_b, stream>>>( a, 0 );
    a.blocks = (const int4 *)d_blocks[2];
    mark( KERNEL_PASS_C );
    pass_c<R><<<n_blocks[2], 256, max_smem_c, stream>>>( a );
    a.blocks = (const int4 *)d_blocks[1];
    mark( KERNEL_PASS_B_INV );
    pass_b<R><<<n_blocks[1], 256, max_smem_b, stream>>>( a, 1 );
    a.blocks = (const int4 *)d_blocks[0];
    mark( KERNEL_PASS_A_INV );
    pass_a_inv<R><<<n_blocks[0], 256, max_smem_a, stream>>>( a );
    CUDA_CHECK( cudaGetLastError() );
}

void DDIPlan::run( const SysDesc * d_sd, const SysRun * runs, const void * sx, const void * sy, const void * sz,
                   void * hx, void * hy, void * hz, cudaStream_t stream ) const
{
    if( fp64 )
        run_t<double>( d_sd, runs, (const double *)sx, (const double *)sy, (const double *)sz, (double *)hx,
                       (double *)hy, (double *)hz, stream );
    else
        run_t<float>( d_sd, runs, (const float *)sx, (const float *)sy, (const float *)sz, (float *)hx, (float *)hy,
                      (float *)hz, stream );
}

} // namespace sg
