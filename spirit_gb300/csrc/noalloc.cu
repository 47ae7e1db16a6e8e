// Allocation-free gradient entry point (no counterpart in the reference).
//
// Hamiltonian_Get_Gradient_NoAlloc evaluates the FP64 gradient and energy of the stencil terms
// (exchange, DMI, anisotropy, Zeeman: Gradient_and_Energy, Hamiltonian_Heisenberg.cpp:704-766,
// without the dipolar term) of spins that already sit on the device, and writes only into
// buffers the caller owns.  Its only scratch is the file-scope array below, so the call makes no
// device allocation at all.  It serves callers that cannot allocate while they run: programs
// whose device memory belongs to their own pool or caching allocator (a framework's allocator,
// a fixed arena of an embedded or real-time loop) and which must not have a library call
// cudaMalloc / cudaFree behind their back -- those calls also synchronise the device, which
// such callers cannot afford inside their step.
//
// Limits and rules:
//   * at most NOALLOC_MAX_SPINS spins (larger systems are rejected with an error code);
//   * no dipolar interaction (States with DDI are rejected);
//   * the scratch is shared by all calls on a device: calls that overlap in time (different
//     streams, or host threads without ordering) race on it and may return a wrong energy;
//   * nothing has to start at zero: every scratch entry the energy sum reads is written first by
//     the same call, in stream order;
//   * the first call in each CUDA context looks up the scratch address (cudaGetSymbolAddress),
//     which can load the module; make that first call before any stream capture.  The address is
//     cached per context (keyed on the driver's unique context id), not per device ordinal: after
//     cudaDeviceReset, or in a context other than the device's primary one, the module is loaded
//     anew and the symbol can sit at another address, so the lookup is repeated there;
//   * the system descriptor (SysDesc, several KB) is passed to the kernel by value: kernel
//     parameters above 4 KB need CUDA 12.1 or newer on sm_70+ (the limit is 32,764 bytes).
#include "engine.hpp"
#include "kernels.cuh"
#include "state.hpp"

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>

namespace sg
{

constexpr int NOALLOC_THREADS    = 256;
constexpr int NOALLOC_MAX_BLOCKS = 16384; // 128 KB of per-block energies
constexpr long long NOALLOC_MAX_SPINS = (long long)NOALLOC_MAX_BLOCKS * NOALLOC_THREADS; // 4,194,304

// per-block partial energies of one call
static __device__ __align__( 256 ) double g_noalloc_partials[NOALLOC_MAX_BLOCKS];

// the descriptor travels as a kernel parameter (by value): CUDA 12.1+ allows up to 32,764 bytes
static_assert( sizeof( SysDesc ) <= 32764, "SysDesc exceeds the kernel parameter limit" );

// Variant of the engine's evaluation kernel (engine.cu eval_kernel): SoA FP64 spins of one system
// at offset 0, gradient to SoA, and the block's energy sum into partials[blockIdx.x].
__global__ void __launch_bounds__( NOALLOC_THREADS )
    noalloc_gradient( const SysDesc d, const double * sx, const double * sy, const double * sz, double * gx,
                      double * gy, double * gz, double * partials )
{
    __shared__ PairR<double> pairs[MAX_PAIRS];
    __shared__ SysConst<double> C;
    __shared__ Geo GS;
    __shared__ double red[32];
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    __syncthreads();
    const int i      = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < d.nos;
    int ib, a, b, c;
    cell_of( GS, valid ? i : 0, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, valid );
    double e        = 0;
    if( valid )
    {
        const SoA3<double> cfg = { const_cast<double *>( sx ), const_cast<double *>( sy ), const_cast<double *>( sz ) };
        const SoA3<double> none = { nullptr, nullptr, nullptr };
        const V3<double> si     = cfg.ld( i );
        const V3<double> g = gradient_at<double>( GS, C, pairs, cfg, none, i, ib, a, b, c, si, C.mu[ib], e, smode );
        gx[i] = g.x;
        gy[i] = g.y;
        gz[i] = g.z;
    }
    const double es = block_sum_w( e, red );
    if( threadIdx.x == 0 )
        partials[blockIdx.x] = es;
}

// energy = sum of the n partials, in a fixed order (one block)
__global__ void __launch_bounds__( NOALLOC_THREADS ) noalloc_sum( const double * partials, int n, double * energy )
{
    __shared__ double red[32];
    double v = 0;
    for( int k = threadIdx.x; k < n; k += blockDim.x )
        v += partials[k];
    const double s = block_sum( v, red );
    if( threadIdx.x == 0 )
        *energy = s;
}

// Unique id of the calling thread's current CUDA context (cuCtxGetId through the runtime's
// driver entry point, so the library does not link the driver library itself); 0 when unknown.
static unsigned long long current_context_id()
{
    typedef int ( *GetCurrent )( void ** );
    typedef int ( *GetId )( void *, unsigned long long * );
    static GetCurrent get_current = nullptr;
    static GetId get_id           = nullptr;
    static std::once_flag once;
    std::call_once( once, [] {
        void * f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if( cudaGetDriverEntryPointByVersion( "cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q ) == cudaSuccess
            && q == cudaDriverEntryPointSuccess )
            get_current = reinterpret_cast<GetCurrent>( f );
        f = nullptr;
        if( cudaGetDriverEntryPointByVersion( "cuCtxGetId", &f, 12000, cudaEnableDefault, &q ) == cudaSuccess
            && q == cudaDriverEntryPointSuccess )
            get_id = reinterpret_cast<GetId>( f );
        cudaGetLastError();
    } );
    void * ctx             = nullptr;
    unsigned long long cid = 0;
    if( get_current && get_id && get_current( &ctx ) == 0 && ctx && get_id( ctx, &cid ) == 0 )
        return cid;
    return 0;
}

// Scratch address in the current context, looked up once per context.  A thread without a current
// context gets the device's primary one from the lookup itself (the runtime initialises it), and the
// address is cached under that context's id.
static double * noalloc_scratch( std::string & err )
{
    static std::mutex mu;
    static std::map<unsigned long long, double *> by_context;
    int dev       = -1;
    cudaError_t e = cudaGetDevice( &dev );
    if( e != cudaSuccess || dev < 0 )
    {
        err = "no usable current CUDA device";
        return nullptr;
    }
    std::lock_guard<std::mutex> lk( mu );
    unsigned long long cid = current_context_id();
    if( cid != 0 )
    {
        auto it = by_context.find( cid );
        if( it != by_context.end() )
            return it->second;
    }
    void * p = nullptr;
    e        = cudaGetSymbolAddress( &p, g_noalloc_partials );
    if( e != cudaSuccess )
    {
        err = std::string( "cudaGetSymbolAddress: " ) + cudaGetErrorString( e );
        return nullptr;
    }
    if( cid == 0 )
        cid = current_context_id();
    if( cid != 0 )
        by_context[cid] = static_cast<double *>( p );
    return static_cast<double *>( p );
}

} // namespace sg

using namespace sg;

// Return codes of Hamiltonian_Get_Gradient_NoAlloc
enum
{
    NOALLOC_OK          = 0,
    NOALLOC_BAD_ARGS    = 1, // invalid State, image index or null buffer
    NOALLOC_TOO_LARGE   = 2, // more than NOALLOC_MAX_SPINS spins
    NOALLOC_HAS_DDI     = 3, // dipolar interaction enabled
    NOALLOC_CUDA_ERROR  = 4,
    NOALLOC_HOST_ERROR  = 5
};

extern "C" int Hamiltonian_Get_Gradient_NoAlloc( State * state, const double * sx, const double * sy, const double * sz,
                                                double * gx, double * gy, double * gz, double * energy, void * stream,
                                                int idx_image, int idx_chain ) noexcept
{
    try
    {
        if( !state || !state->chain || idx_chain > 0 )
            return NOALLOC_BAD_ARGS;
        const int im = idx_image < 0 ? state->idx_active_image : idx_image;
        if( im >= (int)state->chain->images.size() )
            return NOALLOC_BAD_ARGS;
        if( !sx || !sy || !sz || !gx || !gy || !gz || !energy )
            return NOALLOC_BAD_ARGS;
        const Image & img = *state->chain->images[im];
        if( img.ham.ddi_method != 0 )
        {
            log_msg( state, 1, "Hamiltonian_Get_Gradient_NoAlloc: the dipolar interaction is not supported" );
            return NOALLOC_HAS_DDI;
        }
        const long long nos = img.geom->nos();
        if( nos > NOALLOC_MAX_SPINS )
        {
            log_msg( state, 1, "Hamiltonian_Get_Gradient_NoAlloc: " + std::to_string( nos ) + " spins exceed the maximum of "
                                   + std::to_string( NOALLOC_MAX_SPINS ) );
            return NOALLOC_TOO_LARGE;
        }
        SystemInput in;
        in.geom = img.geom.get();
        in.ham  = &img.ham;
        SysDesc d;
        fill_system_desc( d, in );
        d.spin_offset = 0;
        std::string err;
        double * scratch = noalloc_scratch( err );
        if( !scratch )
        {
            log_msg( state, 1, "Hamiltonian_Get_Gradient_NoAlloc: " + err );
            return NOALLOC_CUDA_ERROR;
        }
        const int nblk   = (int)( ( nos + NOALLOC_THREADS - 1 ) / NOALLOC_THREADS );
        cudaStream_t st  = static_cast<cudaStream_t>( stream );
        if( nblk > 0 )
            noalloc_gradient<<<nblk, NOALLOC_THREADS, 0, st>>>( d, sx, sy, sz, gx, gy, gz, scratch );
        noalloc_sum<<<1, NOALLOC_THREADS, 0, st>>>( scratch, nblk, energy );
        cudaError_t e = cudaGetLastError();
        if( e != cudaSuccess )
        {
            log_msg( state, 1, std::string( "Hamiltonian_Get_Gradient_NoAlloc: " ) + cudaGetErrorString( e ) );
            return NOALLOC_CUDA_ERROR;
        }
        return NOALLOC_OK;
    }
    catch( ... )
    {
        return NOALLOC_HOST_ERROR;
    }
}
