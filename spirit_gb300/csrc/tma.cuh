// Bulk tensor copies (TMA) into shared memory, completed on an mbarrier (sm_90+ PTX), with
// bounded waits.  Host side: tensor maps encoded through the driver entry point obtained from
// the runtime (the library does not link the driver library itself).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sg
{

#ifdef __CUDACC__
__device__ __forceinline__ unsigned smem_u32( const void * p )
{
    return (unsigned)__cvta_generic_to_shared( p );
}

__device__ __forceinline__ void mbar_init( uint64_t * bar, unsigned count )
{
    asm volatile( "mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"( smem_u32( bar ) ), "r"( count ) : "memory" );
}

// make the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile( "fence.mbarrier_init.release.cluster;" ::: "memory" );
}

// order earlier generic-proxy accesses of shared memory before later async-proxy writes to it
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile( "fence.proxy.async.shared::cta;" ::: "memory" );
}

__device__ __forceinline__ void mbar_arrive_expect_tx( uint64_t * bar, unsigned bytes )
{
    asm volatile( "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"( smem_u32( bar ) ), "r"( bytes )
                  : "memory" );
}

__device__ __forceinline__ bool mbar_try_wait( uint64_t * bar, unsigned phase )
{
    unsigned ok;
    asm volatile( "{\n\t.reg .pred p;\n\t"
                  "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                  "selp.u32 %0, 1, 0, p;\n\t}"
                  : "=r"( ok )
                  : "r"( smem_u32( bar ) ), "r"( phase )
                  : "memory" );
    return ok != 0;
}

// Wait for the phase with an iteration limit: false when the limit ran out (the caller records
// an error and returns instead of spinning forever).
__device__ __forceinline__ bool mbar_wait_bounded( uint64_t * bar, unsigned phase, unsigned limit = 1u << 22 )
{
    for( unsigned it = 0; it < limit; ++it )
        if( mbar_try_wait( bar, phase ) )
            return true;
    return false;
}

// One box of a rank-1 tensor map (elements [x, x + box) of the global array, zero-filled outside
// it) into shared memory at dst (128-byte aligned); x times the element size must be a multiple
// of 16 bytes.  Completes `bytes` of the barrier's expected transaction count.
__device__ __forceinline__ void tma_load_1d( void * dst, const CUtensorMap * map, int x, uint64_t * bar )
{
    asm volatile( "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];"
                  ::"r"( smem_u32( dst ) ), "l"( reinterpret_cast<uint64_t>( map ) ), "r"( x ), "r"( smem_u32( bar ) )
                  : "memory" );
}
#endif

// Rank-1 FP32 tensor map over n elements at base (16-byte aligned) with a box of `box` elements.
// Returns false when the driver entry point is missing or the encoding is refused.
bool encode_tensor_map_1d_f32( CUtensorMap * map, const void * base, unsigned long long n, unsigned box );

} // namespace sg
