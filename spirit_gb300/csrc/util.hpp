// CUDA error handling and device-memory helpers.  Device errors become C++ exceptions on the
// host; the C API catches them per call (the reference logs and, for CUDA errors, exits the
// process: core/src/utility/Exception.cpp:70-110 -- here the API reports and returns instead).
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>

namespace sg
{

struct CudaError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

inline void cuda_check( cudaError_t e, const char * what, const char * file, int line )
{
    if( e != cudaSuccess )
        throw CudaError( std::string( "CUDA error in " ) + what + " (" + file + ":" + std::to_string( line )
                         + "): " + cudaGetErrorString( e ) );
}

#define CUDA_CHECK( x ) ::sg::cuda_check( ( x ), #x, __FILE__, __LINE__ )

inline void * dalloc_bytes( size_t bytes )
{
    void * p = nullptr;
    if( bytes == 0 )
        bytes = 16;
    CUDA_CHECK( cudaMalloc( &p, bytes ) );
    // zero-filled before any stream may use it: cudaMemset runs on the legacy stream and returns
    // early, and the engine streams are non-blocking (they would not wait for it)
    CUDA_CHECK( cudaMemset( p, 0, bytes ) );
    CUDA_CHECK( cudaStreamSynchronize( nullptr ) );
    return p;
}

template<typename T>
inline T * dalloc( size_t n )
{
    return static_cast<T *>( dalloc_bytes( n * sizeof( T ) ) );
}

template<typename T>
inline void dfree( T *& p )
{
    if( p )
        cudaFree( (void *)p );
    p = nullptr;
}

// Page-locked registration of a host buffer that outlives many transfers (an image's AoS spin
// mirror): the copy engines then move it directly, without the CUDA driver's staging through a pinned
// bounce buffer.  ensure() re-registers when the buffer has moved, release() before it is
// reallocated.  SPIRIT_GB300_PIN=0 leaves buffers pageable; a failed registration leaves the
// buffer pageable.
struct HostPin
{
    void * ptr   = nullptr;
    size_t bytes = 0;
    void ensure( void * p, size_t n )
    {
        if( p == ptr && n == bytes )
            return;
        release();
        const char * env = std::getenv( "SPIRIT_GB300_PIN" );
        if( !p || n == 0 || ( env && env[0] == '0' ) )
            return;
        if( cudaHostRegister( p, n, cudaHostRegisterPortable | cudaHostRegisterMapped ) == cudaSuccess )
        {
            ptr   = p;
            bytes = n;
        }
        else
            cudaGetLastError();
    }
    void release()
    {
        if( ptr )
        {
            cudaHostUnregister( ptr );
            cudaGetLastError();
        }
        ptr   = nullptr;
        bytes = 0;
    }
    HostPin() = default;
    HostPin( const HostPin & ) = delete;
    HostPin & operator=( const HostPin & ) = delete;
    ~HostPin()
    {
        release();
    }
};

template<typename T>
inline void h2d( T * d, const T * h, size_t n )
{
    // complete before return: later work runs on non-blocking streams, which a pageable copy's
    // outstanding DMA on the legacy stream would not order
    CUDA_CHECK( cudaMemcpy( d, h, n * sizeof( T ), cudaMemcpyHostToDevice ) );
    CUDA_CHECK( cudaStreamSynchronize( nullptr ) );
}

inline void h2d_bytes( void * d, const void * h, size_t n )
{
    CUDA_CHECK( cudaMemcpy( d, h, n, cudaMemcpyHostToDevice ) );
    CUDA_CHECK( cudaStreamSynchronize( nullptr ) );
}

template<typename T>
inline void d2h( T * h, const T * d, size_t n )
{
    CUDA_CHECK( cudaMemcpy( h, d, n * sizeof( T ), cudaMemcpyDeviceToHost ) );
}

// Programmatic dependent launch: the kernel may be launched while its predecessor in the stream
// is still running, so launch latency and its set-up (constants, twiddles, pair tables into
// shared memory) overlap the predecessor's tail; the kernel executes pdl_wait() (griddepcontrol
// .wait: the predecessor has completed and its writes are visible) before touching data an
// earlier kernel produced.  SPIRIT_GB300_PDL=0 launches without the attribute.
inline bool pdl_enabled()
{
    static const bool on = [] {
        const char * e = std::getenv( "SPIRIT_GB300_PDL" );
        return !( e && e[0] == '0' );
    }();
    return on;
}

template<typename... KArgs, typename... Args>
inline void launch_pdl( void ( *kern )( KArgs... ), dim3 grid, dim3 block, size_t smem, cudaStream_t st, int cluster,
                        Args &&... args )
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = grid;
    cfg.blockDim           = block;
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = st;
    cudaLaunchAttribute at[2];
    unsigned na = 0;
    if( pdl_enabled() )
    {
        at[na].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if( cluster > 1 )
    {
        at[na].id               = cudaLaunchAttributeClusterDimension;
        at[na].val.clusterDim.x = cluster;
        at[na].val.clusterDim.y = 1;
        at[na].val.clusterDim.z = 1;
        ++na;
    }
    cfg.attrs    = na ? at : nullptr;
    cfg.numAttrs = na;
    CUDA_CHECK( cudaLaunchKernelEx( &cfg, kern, std::forward<Args>( args )... ) );
}

} // namespace sg
