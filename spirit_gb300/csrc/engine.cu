// Fused field + LLG stage kernels for a batch of spin systems (sm_103a).
//
// One launch per integrator stage evaluates, for every spin of every active system of the
// batch: the Heisenberg gradient at the stage configuration (anisotropy, merged exchange +
// DMI pair stencil, dipolar field from the FFT pipeline, Zeeman), the LLG virtual force with
// in-kernel Philox thermal noise, and the solver's update -- reading each spin once per stage.
// The last stage also reduces the FP64 energy of the evaluated configuration and the maximum
// torque |P_perp(s_new) fv_1| per system into per-system accumulators; a small kernel launched
// after it (close_iteration) finalises the iteration counter and the convergence flag on the
// device, so a whole step sequence can be captured in a CUDA graph and replayed without host
// round trips.
//
// Reference algorithms (file:line in Spirit v2.2.0):
//   gradient terms        core/src/engine/Hamiltonian_Heisenberg.cpp:704-864
//   virtual force         core/src/engine/Method_LLG.cpp:132-226
//   thermal field         core/src/engine/Method_LLG.cpp:65-110 (Philox stream instead of mt19937)
//   SIB                   core/include/engine/Solver_SIB.hpp:21-50, core/src/engine/Solver_Kernels.cpp:15-48
//   Depondt               core/include/engine/Solver_Depondt.hpp:28-77, Vectormath.cpp:474-485
//   Heun                  core/include/engine/Solver_Heun.hpp:29-80
//   RK4                   core/include/engine/Solver_RK4.hpp:40-147
//   max torque            core/include/engine/Method_Solver.hpp:225-230, Method_LLG.cpp:247-301
#include "engine.hpp"
#include "fft.cuh"
#include "kernels.cuh"
#include "tma.cuh"
#include "util.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <type_traits>

namespace sg
{

// ------------------------------------------------------------------ stage kernel
template<typename R>
struct StageArgs
{
    const SysDesc * sd;
    SysRun * runs;
    const int2 * blkmap;  // (system, first local spin)
    SoA3<R> s;            // state
    SoA3<R> cfg;          // stage configuration (neighbour reads)
    SoA3<R> out;          // predictor output
    SoA3<R> aux1;         // fv of stage 1
    SoA3<R> aux2;         // RK4 running sum
    SoA3<R> h;            // dipolar field of cfg (x == nullptr: none)
    SoA3<R> xi;           // thermal field of the iteration: written by stage 1, read by later stages
    SoA3<R> lo;           // FP32 compensated state: low parts of s (x == nullptr: plain FP32 state)
    int tune;             // 1: timing run of the tuner (ignores and keeps the run state)
};

// ------------------------------------------------------------------ compensated FP32 state
// With the compensated state an FP32 system keeps every spin as an unevaluated sum hi + lo of two
// floats (about 48 significant bits).  Fields and stage arithmetic stay FP32 and read hi only; the
// last stage of a step forms the solver's update as a small increment D of the state (s_new =
// normalise(s + D), D of the order dt |field| gamma), and adds it to (hi, lo) with error-free
// transformations: the rounding of the stored state -- about 3e-8 per step, which random-walks and
// dominates the FP32 deviation from an FP64 trajectory -- no longer accumulates; what remains is
// the FP32 error of D itself (1e-7 |D|).

// TwoSum (Knuth): a + b = s + err exactly, round-to-nearest, no branch
__device__ __forceinline__ float two_sum( float a, float b, float & err )
{
    const float s  = a + b;
    const float bp = s - a;
    err            = ( a - ( s - bp ) ) + ( b - bp );
    return s;
}

// (hi, lo) += x, renormalised so that hi carries the rounded sum
__device__ __forceinline__ void ff_add( float & hi, float & lo, float x )
{
    float e1, e2;
    const float s = two_sum( hi, x, e1 );
    const float l = lo + e1;
    hi            = two_sum( s, l, e2 );
    lo            = e2;
}

// Increment of a normalised update: s_new = (s + D) / |s + D| = s + E for s = hi + lo.
// |s + D|^2 = 1 + u with u = (|s|^2 - 1) + 2 s.D + |D|^2, the first term formed exactly enough from
// hi and lo (squares split by FMA, their sum by TwoSum; |hi|^2 is near 1, so subtracting 1 is
// exact); then 1 / |s + D| = 1 + delta, delta = -u / (r (1 + r)), r = sqrt(1 + u) (no cancellation),
// and E = D + delta (s + D).
__device__ __forceinline__ V3<float> ff_norm_increment( V3<float> h, V3<float> l, V3<float> D )
{
    const float px = h.x * h.x, py = h.y * h.y, pz = h.z * h.z;
    const float ex = fmaf( h.x, h.x, -px ), ey = fmaf( h.y, h.y, -py ), ez = fmaf( h.z, h.z, -pz );
    float e1, e2;
    float S       = two_sum( px, py, e1 );
    S             = two_sum( S, pz, e2 );
    const float eps = ( S - 1.f ) + ( ( e1 + e2 ) + ( ex + ey + ez ) ) + 2.f * ( h.x * l.x + h.y * l.y + h.z * l.z );
    const float u   = eps + 2.f * ( h.x * D.x + h.y * D.y + h.z * D.z ) + ( D.x * D.x + D.y * D.y + D.z * D.z );
    const float r   = sqrtf( 1.f + u );
    const float dl  = -u / ( r * ( 1.f + r ) );
    return { D.x + dl * ( h.x + D.x ), D.y + dl * ( h.y + D.y ), D.z + dl * ( h.z + D.z ) };
}

// s (= hi + lo at gi) <- normalise(s + D), stored back as hi and lo; returns the new hi
template<typename R>
__device__ __forceinline__ V3<float> ff_update( const StageArgs<R> & A, int gi, V3<float> h, V3<float> l,
                                                V3<float> D )
{
    const V3<float> E = ff_norm_increment( h, l, D );
    ff_add( h.x, l.x, E.x );
    ff_add( h.y, l.y, E.y );
    ff_add( h.z, l.z, E.z );
    A.lo.x[gi] = (R)l.x;
    A.lo.y[gi] = (R)l.y;
    A.lo.z[gi] = (R)l.z;
    return h;
}

enum
{
    ST_PROBE = 0
};

// spins per thread of the FP32 stage kernels (index = Engine::spt_idx_); FP64 uses 1
static const int SPT_OPTIONS[3] = { 1, 2, 4 };

// Per-spin part of a stage after the field g of configuration ci is known: thermal field, virtual
// force and the solver's update (Solver_SIB.hpp, Solver_Heun.hpp, Solver_Depondt.hpp,
// Solver_RK4.hpp); t2 takes the max squared torque.
// Thermal field of spin i at an iteration: epsilon sqrt(T / mu_s) times three standard normals
// from the spin's Philox block
template<typename R>
__device__ __forceinline__ V3<R> thermal_field( const SysConst<R> & C, const SysDesc & d, int ib, unsigned int counter,
                                                int i )
{
    const R sc    = C.noise[ib];
    const V3<R> z = gauss3<R>( d.seed, d.stream, counter, (unsigned int)i );
    return { sc * z.x, sc * z.y, sc * z.z };
}

// The per-spin arrays a stage reads besides the configuration: the state, the stage-1 virtual
// force, the thermal field, the RK4 sum and the low parts of a compensated state.  The stage
// kernels load them before the field is evaluated, so these loads are in flight together with the
// neighbour reads instead of being issued after them.
template<typename R>
struct StageIn
{
    V3<R> s, fv1, xi, acc;
    V3<float> lo;
};

template<typename R, int SOLVER, int STAGE>
__device__ __forceinline__ StageIn<R> stage_inputs( const StageArgs<R> & A, const SysConst<R> & C, int gi )
{
    constexpr bool LAST = ( SOLVER == SOLVER_RK4 ) ? ( STAGE == 4 ) : ( STAGE == 2 );
    StageIn<R> in{};
    if( STAGE >= 2 )
    {
        in.s = A.s.ld( gi );
        if( LAST )
            in.fv1 = A.aux1.ld( gi );
        if( C.thermal )
            in.xi = A.xi.ld( gi );
        if( SOLVER == SOLVER_RK4 )
            in.acc = A.aux2.ld( gi );
        if( LAST && sizeof( R ) == 4 && A.lo.x )
            in.lo = { (float)A.lo.x[gi], (float)A.lo.y[gi], (float)A.lo.z[gi] };
    }
    return in;
}

template<typename R, int SOLVER, int STAGE>
__device__ __forceinline__ void stage_update( const StageArgs<R> & A, const SysConst<R> & C, const SysDesc & d,
                                              int gi, int i, int ib, V3<R> ci, V3<R> g, int iteration,
                                              float & t2, const StageIn<R> & in )
{
    constexpr bool PROBE = STAGE == ST_PROBE;
    V3<R> xi             = { 0, 0, 0 };
    if( C.thermal )
    {
        // drawn once per iteration (Prepare_Thermal_Field, Method_LLG.cpp:65-110) by the first
        // stage and kept for the later stages of the same iteration
        if( PROBE || STAGE == 1 )
        {
            xi = thermal_field<R>( C, d, ib, PROBE ? 0xFFFFFFFFu : (unsigned int)iteration + d.noise_offset, i );
            if( STAGE == 1 )
                A.xi.st( gi, xi );
        }
        else
            xi = in.xi;
    }
    V3<R> fv = virtual_force<R>( C, ci, g, C.inv_mu[ib], xi );
    if( PROBE )
    {
        t2 = fmaxf( t2, (float)torque2( fv, ci ) );
    }
    else if( SOLVER == SOLVER_SIB )
    {
        const V3<R> si = ( STAGE == 1 ) ? ci : in.s;
        if( STAGE == 1 )
        {
            V3<R> p = sib( si, fv );
            p.x += si.x;
            p.y += si.y;
            p.z += si.z;
            p.x *= R( 0.5 );
            p.y *= R( 0.5 );
            p.z *= R( 0.5 );
            A.out.st( gi, p );
            A.aux1.st( gi, fv );
        }
        else
        {
            V3<R> sn;
            if( sizeof( R ) == 4 && A.lo.x )
            {
                // sib(s, fv) - s = 2 (A x s + A x (A x s)) / (1 + |A|^2), A = fv / 2
                const V3<R> Ah = { R( 0.5 ) * fv.x, R( 0.5 ) * fv.y, R( 0.5 ) * fv.z };
                const V3<R> c1 = cross( Ah, si );
                const V3<R> c2 = cross( Ah, c1 );
                const R w      = R( 2 ) / ( R( 1 ) + dot( Ah, Ah ) );
                const V3<float> D = { float( w * ( c1.x + c2.x ) ), float( w * ( c1.y + c2.y ) ),
                                      float( w * ( c1.z + c2.z ) ) };
                const V3<float> hn = ff_update( A, gi, V3<float>{ (float)si.x, (float)si.y, (float)si.z }, in.lo, D );
                sn                 = { (R)hn.x, (R)hn.y, (R)hn.z };
            }
            else
            {
                sn = sib( si, fv );
                // SIB preserves |s| only in exact arithmetic; in FP32 the rounding drift is removed
                if( sizeof( R ) == 4 )
                    sn = normalized( sn );
            }
            A.s.st( gi, sn );
            t2 = fmaxf( t2, (float)torque2( in.fv1, sn ) );
        }
    }
    else if( SOLVER == SOLVER_HEUN )
    {
        if( STAGE == 1 )
        {
            V3<R> cr = cross( ci, fv );
            V3<R> p  = { ci.x + R( -1 ) * cr.x, ci.y + R( -1 ) * cr.y, ci.z + R( -1 ) * cr.z };
            A.out.st( gi, normalized( p ) );
            A.aux1.st( gi, fv );
        }
        else
        {
            const V3<R> si  = in.s;
            const V3<R> fv1 = in.fv1;
            V3<R> c1        = cross( si, fv1 );
            V3<R> t1        = { R( -1 ) * c1.x, R( -1 ) * c1.y, R( -1 ) * c1.z };
            V3<R> c2        = cross( ci, fv );
            V3<R> sn;
            if( sizeof( R ) == 4 && A.lo.x )
            {
                const V3<float> D  = { float( R( 0.5 ) * t1.x - R( 0.5 ) * c2.x ), float( R( 0.5 ) * t1.y - R( 0.5 ) * c2.y ),
                                       float( R( 0.5 ) * t1.z - R( 0.5 ) * c2.z ) };
                const V3<float> hn = ff_update( A, gi, V3<float>{ (float)si.x, (float)si.y, (float)si.z }, in.lo, D );
                sn                 = { (R)hn.x, (R)hn.y, (R)hn.z };
            }
            else
            {
                V3<R> t = { t1.x * R( 0.5 ), t1.y * R( 0.5 ), t1.z * R( 0.5 ) };
                t.x += si.x;
                t.y += si.y;
                t.z += si.z;
                t.x += R( 0.5 ) * ( R( -1 ) * c2.x );
                t.y += R( 0.5 ) * ( R( -1 ) * c2.y );
                t.z += R( 0.5 ) * ( R( -1 ) * c2.z );
                sn = normalized( t );
            }
            A.s.st( gi, sn );
            t2 = fmaxf( t2, (float)torque2( fv1, sn ) );
        }
    }
    else if( SOLVER == SOLVER_DEPONDT )
    {
        if( STAGE == 1 )
        {
            R ang    = sqrt( dot( fv, fv ) );
            V3<R> ax = normalized( fv );
            A.out.st( gi, rotate( ci, ax, ang ) );
            A.aux1.st( gi, fv );
        }
        else
        {
            const V3<R> si  = in.s;
            const V3<R> fv1 = in.fv1;
            V3<R> ax        = { R( 0.5 ) * fv1.x, R( 0.5 ) * fv1.y, R( 0.5 ) * fv1.z };
            ax.x += R( 0.5 ) * fv.x;
            ax.y += R( 0.5 ) * fv.y;
            ax.z += R( 0.5 ) * fv.z;
            R ang = sqrt( dot( ax, ax ) );
            V3<R> sn;
            if( sizeof( R ) == 4 && A.lo.x )
            {
                // rotation by w = ax (angle |w|) as an increment:
                // D = (sin t / t) w x s + ((1 - cos t) / t^2) w x (w x s), both factors from sin / cos of t/2
                V3<float> D = { 0.f, 0.f, 0.f };
                if( ang > R( 0 ) )
                {
                    float sh, ch;
                    sincosf( 0.5f * (float)ang, &sh, &ch );
                    const float q     = sh / (float)ang;
                    const float f1    = 2.f * q * ch, f2 = 2.f * q * q;
                    const V3<R> c1    = cross( ax, si );
                    const V3<R> c2    = cross( ax, c1 );
                    D                 = { f1 * (float)c1.x + f2 * (float)c2.x, f1 * (float)c1.y + f2 * (float)c2.y,
                                          f1 * (float)c1.z + f2 * (float)c2.z };
                }
                const V3<float> hn = ff_update( A, gi, V3<float>{ (float)si.x, (float)si.y, (float)si.z }, in.lo, D );
                sn                 = { (R)hn.x, (R)hn.y, (R)hn.z };
            }
            else
            {
                sn = rotate( si, normalized( ax ), ang );
                // a rotation preserves |s| only in exact arithmetic; in FP32 the rounding drift is removed
                if( sizeof( R ) == 4 )
                    sn = normalized( sn );
            }
            A.s.st( gi, sn );
            t2 = fmaxf( t2, (float)torque2( fv1, sn ) );
        }
    }
    else if( SOLVER == SOLVER_RK4 )
    {
        // k_m = -(cfg_m x fv_m); cfg_{m+1} = normalize(s + w k_m); running sum acc = s + k1/6 + k2/3 + ...
        V3<R> cr = cross( ci, fv );
        V3<R> k  = { R( -1 ) * cr.x, R( -1 ) * cr.y, R( -1 ) * cr.z };
        const V3<R> si = ( STAGE == 1 ) ? ci : in.s;
        if( STAGE == 1 )
        {
            A.aux1.st( gi, fv );
            // compensated state: the running sum holds the increments only (s stays in (hi, lo))
            V3<R> acc = ( sizeof( R ) == 4 && A.lo.x ) ? V3<R>{ 0, 0, 0 } : si;
            R w6      = R( 1.0 / 6.0 );
            acc.x += w6 * k.x;
            acc.y += w6 * k.y;
            acc.z += w6 * k.z;
            A.aux2.st( gi, acc );
            V3<R> p = { si.x + R( 0.5 ) * k.x, si.y + R( 0.5 ) * k.y, si.z + R( 0.5 ) * k.z };
            A.out.st( gi, normalized( p ) );
        }
        else if( STAGE == 2 || STAGE == 3 )
        {
            V3<R> acc = in.acc;
            R w3      = R( 1.0 / 3.0 );
            acc.x += w3 * k.x;
            acc.y += w3 * k.y;
            acc.z += w3 * k.z;
            A.aux2.st( gi, acc );
            R wn    = STAGE == 2 ? R( 0.5 ) : R( 1 );
            V3<R> p = { si.x + wn * k.x, si.y + wn * k.y, si.z + wn * k.z };
            A.out.st( gi, normalized( p ) );
        }
        else
        {
            V3<R> acc = in.acc;
            R w6      = R( 1.0 / 6.0 );
            acc.x += w6 * k.x;
            acc.y += w6 * k.y;
            acc.z += w6 * k.z;
            V3<R> sn;
            if( sizeof( R ) == 4 && A.lo.x )
            {
                const V3<float> hn = ff_update( A, gi, V3<float>{ (float)si.x, (float)si.y, (float)si.z }, in.lo,
                                                V3<float>{ (float)acc.x, (float)acc.y, (float)acc.z } );
                sn                 = { (R)hn.x, (R)hn.y, (R)hn.z };
            }
            else
                sn = normalized( acc );
            A.s.st( gi, sn );
            t2 = fmaxf( t2, (float)torque2( in.fv1, sn ) );
        }
    }
}

// End of the final stage (or of the probe): the block's energy of the evaluated configuration (per
// warp a compensated FP32 sum -- plain in FP64 -- formed in FP64, the warps summed in FP64) and its
// max squared torque are added to the system's accumulators.  Nothing waits for the additions: no
// fence, no returned counter, one barrier; close_iteration, launched next on the same stream,
// closes the step.  A caller that reduces again reuses red_d / red_f only after another barrier.
template<typename R>
__device__ __forceinline__ void stage_reduce( SysRun * run, R e, R ec, float t2, double * red_d, float * red_f )
{
    for( int o = 16; o > 0; o >>= 1 )
    {
        const R e2 = __shfl_down_sync( 0xffffffffu, e, o );
        if constexpr( sizeof( R ) == 4 )
        {
            const R c2 = __shfl_down_sync( 0xffffffffu, ec, o );
            const R t  = e + e2;
            const R bp = t - e;
            ec += c2 + ( ( e - ( t - bp ) ) + ( e2 - bp ) );
            e = t;
        }
        else
            e += e2;
        t2 = fmaxf( t2, __shfl_down_sync( 0xffffffffu, t2, o ) );
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if( l == 0 )
    {
        red_d[w] = sizeof( R ) == 4 ? (double)e + (double)ec : (double)e;
        red_f[w] = t2;
    }
    __syncthreads();
    if( threadIdx.x < 32 )
    {
        const bool has = threadIdx.x < ( blockDim.x >> 5 );
        double r       = has ? red_d[threadIdx.x] : 0.0;
        float tm       = has ? red_f[threadIdx.x] : 0.f;
        for( int o = 16; o > 0; o >>= 1 )
        {
            r += __shfl_down_sync( 0xffffffffu, r, o );
            tm = fmaxf( tm, __shfl_down_sync( 0xffffffffu, tm, o ) );
        }
        if( threadIdx.x == 0 )
        {
            atomicAdd( &run->energy_acc, r );
            atomicMax( &run->torque_bits, __float_as_uint( tm ) );
        }
    }
}

// Closes the step of every system after the final stage (or the probe): max torque and energy from
// the accumulators the stage kernel's blocks added to (this launch follows that kernel on the
// stream, so all of them are complete and visible), accumulators reset, and -- outside tuner runs
// -- the iteration count and the active flag (budget and force convergence,
// Method_Solver.hpp:225-230).  Systems the stage kernel skipped as inactive are left as they are.
__global__ void close_iteration( SysRun * runs, const SysDesc * sd, int n_sys, int tune, int probe )
{
    pdl_wait();
    pdl_trigger();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if( s >= n_sys )
        return;
    SysRun * r = runs + s;
    if( !tune && !r->active )
        return;
    const float mt = sqrtf( __uint_as_float( r->torque_bits ) );
    r->max_torque  = mt;
    r->energy      = r->energy_acc;
    r->energy_acc  = 0;
    r->torque_bits = 0;
    if( !tune )
    {
        const int it = r->iteration + ( probe ? 0 : 1 );
        r->iteration = it;
        r->active    = ( it < sd[s].n_iterations ) && !( mt < (float)sd[s].force_convergence );
    }
}

// SOLVER / STAGE are compile-time; STAGE 0 is the constructor probe (initial torque + energy).
// A block of 256 threads covers SPT * 256 consecutive spins of one system (thread t: spins
// t, t + 256, ...), so the per-block set-up and reductions are shared by SPT spins per thread.
// FP32: at least 5 blocks of 256 threads per SM (48 registers, a few spilled): the 256-system SIB
// ensemble runs 0.287 ms per step against 0.309 at 4 blocks (64 registers) and 0.284 at 6 (40
// registers, more spills); the 128x128x16 dipolar step is unchanged (0.099 ms).
template<typename R, int SOLVER, int STAGE, int SPT>
__global__ void __launch_bounds__( 256, sizeof( R ) == 4 ? 5 : 1 ) llg_stage( StageArgs<R> A )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red_d[32];
    __shared__ float red_f[32];
    const int2 bm = A.blkmap[blockIdx.x];
    const int s   = bm.x;
    SysRun * run  = A.runs + s;
    const SysDesc & d = A.sd[s];
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    __syncthreads();
    pdl_wait(); // everything below reads what earlier kernels wrote
    pdl_trigger();
    if( !A.tune && !run->active )
        return;
    constexpr bool FINAL = ( SOLVER == SOLVER_RK4 ) ? ( STAGE == 4 ) : ( STAGE == 2 );
    constexpr bool PROBE = STAGE == ST_PROBE;
    const int iteration  = run->iteration;
    R e                  = 0;
    R ec                 = 0; // compensation of the energy sum
    float t2             = 0;
#pragma unroll
    for( int k = 0; k < SPT; ++k )
    {
    const int i      = bm.y + threadIdx.x + k * 256; // local spin index
    const bool valid = i < d.nos;
    int ib, a, b, c;
    cell_of( GS, valid ? i : 0, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, valid );
    if( valid )
    {
        const int gi         = (int)GS.off + i; // batches hold fewer than 2^31 spins
        const StageIn<R> pin = stage_inputs<R, SOLVER, STAGE>( A, C, gi );
        const R mu           = C.mu[ib];
        const V3<R> ci       = A.cfg.ld( gi );
        R ek                 = 0;
        V3<R> g = gradient_at<R, false, FINAL || PROBE>( GS, C, pairs, A.cfg, A.h, gi, ib, a, b, c, ci, mu,
                                                                    ek, smode );
        comp_add( e, ec, ek );
        stage_update<R, SOLVER, STAGE>( A, C, d, gi, i, ib, ci, g, iteration, t2, pin );
    }
    }
    if( !( FINAL || PROBE ) )
        return;
    stage_reduce<R>( run, e, ec, t2, red_d, red_f );
}

// ------------------------------------------------------------------ TMA-staged stage kernel (FP32)
// Persistent variant of llg_stage for FP32 batches whose stencil reaches only a few rows (2D
// lattices: the batched ensembles).  Each CTA walks a contiguous run of tiles (TT_SPINS
// consecutive spins of one system).  The stage configuration of a tile and its halo -- the index
// window [t0 - H, t0 + T + H), H the largest |linear offset| of a pair, which holds every
// neighbour of a cell that needs no wrap -- is brought into shared memory by bulk tensor copies
// (TMA: rank-1 boxes of TT_BOX floats of each component array, completed on an mbarrier), double
// buffered: the next tile's window streams in while the current tile is computed.  Neighbours
// outside the window (wraps along b or c, the far end of a system) are read from global memory.
// The arithmetic per spin is llg_stage's (same gradient terms and order, same stage update), so
// the two kernels give the same results.
constexpr int TT_SPINS = 1024; // spins per tile (4 per thread)
constexpr int TT_BOX   = 256;  // floats per tensor copy (largest box extent)
constexpr int TT_NCOPY = 8;    // tensor copies per component and window at most
constexpr int TT_WIN   = TT_BOX * TT_NCOPY;
constexpr size_t TT_SMEM = sizeof( float ) * 2 * 3 * TT_WIN; // two windows of three components

struct TileMaps
{
    CUtensorMap m[3]; // components x, y, z of the stage configuration: rank 1, box TT_BOX
};

// Gradient at spin gi (batch index) from the staged window (same terms and order as gradient_at).
template<bool ENERGY>
__device__ __forceinline__ V3<float> gradient_win( const Geo & d, const SysConst<float> & C, const PairR<float> * pairs,
                                                   const float * wx, const float * wy, const float * wz, int xs,
                                                   int wlen, const SoA3<float> & cfg, const SoA3<float> & h, int gi,
                                                   int ib, int a, int b, int c, V3<float> si, float mu, float & e,
                                                   int mode )
{
    V3<float> g = { 0, 0, 0 };
    for( int k = 0; k < C.n_aniso; ++k )
        if( C.aniso_idx[k] == ib )
        {
            V3<float> n = { C.aniso_n[k][0], C.aniso_n[k][1], C.aniso_n[k][2] };
            float sc    = 2.f * C.aniso_K[k] * dot( n, si );
            g.x -= sc * n.x;
            g.y -= sc * n.y;
            g.z -= sc * n.z;
        }
    const int p0 = d.pair_begin[ib], p1 = d.pair_begin[ib + 1];
#pragma unroll 6
    for( int p = p0; p < p1; ++p )
    {
        const PairR<float> P = pairs[p];
        int j;
        bool have = true, inwin = true;
        if( mode == STENCIL_INTERIOR )
            j = gi + P.lin;
        else
        {
            if( mode == STENCIL_ROW )
            {
                const int ja = a + P.da;
                j            = gi + P.lin;
                if( ja < 0 )
                {
                    j += d.row_len;
                    have = d.bc[0];
                }
                else if( ja >= d.n[0] )
                {
                    j -= d.row_len;
                    have = d.bc[0];
                }
            }
            else
            {
                const long long jj = pair_index( d, a, b, c, P.j, P.da, P.db, P.dc );
                have               = jj >= 0;
                j                  = (int)jj;
            }
            inwin = (unsigned)( j - xs ) < (unsigned)wlen;
        }
        if( have )
        {
            V3<float> sj;
            if( inwin )
            {
                const int w = j - xs;
                sj          = { wx[w], wy[w], wz[w] };
            }
            else
                sj = cfg.ld( j );
            pair_acc<float, false>( g, P.J, P.Dx, P.Dy, P.Dz, sj );
        }
    }
    if( h.x )
    {
        V3<float> hh = h.ld( gi );
        g.x -= mu * hh.x;
        g.y -= mu * hh.y;
        g.z -= mu * hh.z;
    }
    if( ENERGY )
        e = 0.5f * ( g.x * si.x + g.y * si.y + g.z * si.z );
    if( C.has_zeeman )
    {
        V3<float> B = { C.zeeman[0], C.zeeman[1], C.zeeman[2] };
        g.x -= mu * B.x;
        g.y -= mu * B.y;
        g.z -= mu * B.z;
        if( ENERGY )
            e += -mu * ( B.x * si.x + B.y * si.y + B.z * si.z );
    }
    return g;
}

// tiles[k] = (system, first local spin t0, aligned window start xs in the batch arrays, number
// of tensor copies per component); err: set to 1 when a copy did not arrive within the wait limit
template<int SOLVER, int STAGE>
__global__ void __launch_bounds__( 256, 4 )
    llg_stage_tma( StageArgs<float> A, const __grid_constant__ TileMaps M, const int4 * tiles, int n_tiles, int * err )
{
    extern __shared__ __align__( 128 ) float tt_win[]; // [2][3][TT_WIN]
    __shared__ __align__( 8 ) uint64_t bar[2];
    __shared__ PairR<float> pairs[MAX_PAIRS];
    __shared__ SysConst<float> C;
    __shared__ Geo GS;
    __shared__ double red_d[32];
    __shared__ float red_f[32];
    constexpr bool FINAL = ( SOLVER == SOLVER_RK4 ) ? ( STAGE == 4 ) : ( STAGE == 2 );
    const int k0 = (int)( (long long)blockIdx.x * n_tiles / gridDim.x );
    const int k1 = (int)( (long long)( blockIdx.x + 1 ) * n_tiles / gridDim.x );
    if( threadIdx.x == 0 )
    {
        mbar_init( &bar[0], 1 );
        mbar_init( &bar[1], 1 );
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait(); // the configuration and run state come from earlier kernels
    pdl_trigger();
    auto issue = [&]( int k, int buf ) {
        const int4 t = tiles[k];
        mbar_arrive_expect_tx( &bar[buf], 3u * (unsigned)t.w * TT_BOX * (unsigned)sizeof( float ) );
        for( int comp = 0; comp < 3; ++comp )
            for( int q = 0; q < t.w; ++q )
                tma_load_1d( tt_win + ( buf * 3 + comp ) * TT_WIN + q * TT_BOX, &M.m[comp], t.z + q * TT_BOX,
                             &bar[buf] );
    };
    if( threadIdx.x == 0 && k0 < k1 )
        issue( k0, 0 );
    unsigned phase = 0; // bit b: parity of the next completion of buffer b
    int cur        = -1;
    for( int k = k0; k < k1; ++k )
    {
        const int buf = ( k - k0 ) & 1;
        const int4 t  = tiles[k];
        if( threadIdx.x == 0 && k + 1 < k1 )
        {
            fence_proxy_async_smem(); // the other buffer was last read (generic proxy) by tile k - 1
            issue( k + 1, buf ^ 1 );
        }
        if( t.x != cur )
        {
            const SysDesc & d = A.sd[t.x];
            load_pairs_smem( pairs, d );
            load_const( C, d );
            load_geo( GS, d );
            __syncthreads();
            cur = t.x;
        }
        const bool ok = mbar_wait_bounded( &bar[buf], ( phase >> buf ) & 1u );
        phase ^= 1u << buf;
        if( __syncthreads_or( !ok ) )
        {
            // a copy did not arrive in time: record it, give the copies in flight a bounded
            // chance to land in this CTA's shared memory, and stop
            if( threadIdx.x == 0 )
            {
                atomicExch( err, 1 );
                mbar_wait_bounded( &bar[buf], ( ( phase >> buf ) & 1u ) ^ 1u );
                if( k + 1 < k1 )
                    mbar_wait_bounded( &bar[buf ^ 1], ( phase >> ( buf ^ 1 ) ) & 1u );
            }
            return;
        }
        const int s       = t.x;
        SysRun * run      = A.runs + s;
        const SysDesc & d = A.sd[s];
        if( !A.tune && !run->active )
        {
            __syncthreads(); // the window buffer is reused two tiles later
            continue;
        }
        const float * wx   = tt_win + ( buf * 3 + 0 ) * TT_WIN;
        const float * wy   = tt_win + ( buf * 3 + 1 ) * TT_WIN;
        const float * wz   = tt_win + ( buf * 3 + 2 ) * TT_WIN;
        const int xs       = t.z;
        const int wlen     = t.w * TT_BOX;
        const int iteration = run->iteration;
        float e = 0, ec = 0, t2 = 0;
#pragma unroll
        for( int q = 0; q < TT_SPINS / 256; ++q )
        {
            const int i      = t.y + threadIdx.x + q * 256; // local spin index
            const bool valid = i < GS.nos && threadIdx.x + q * 256 < TT_SPINS;
            int ib, a, b, c;
            cell_of( GS, valid ? i : t.y, ib, a, b, c );
            const int smode = warp_stencil_mode( GS, a, b, c, valid );
            if( valid )
            {
                const int gi   = (int)GS.off + i;
                const StageIn<float> pin = stage_inputs<float, SOLVER, STAGE>( A, C, gi );
                const float mu = C.mu[ib];
                const int w    = gi - xs;
                const V3<float> ci = { wx[w], wy[w], wz[w] };
                float ek           = 0;
                V3<float> g = gradient_win<FINAL>( GS, C, pairs, wx, wy, wz, xs, wlen, A.cfg, A.h, gi, ib, a, b, c, ci,
                                                   mu, ek, smode );
                comp_add( e, ec, ek );
                stage_update<float, SOLVER, STAGE>( A, C, d, gi, i, ib, ci, g, iteration, t2, pin );
            }
        }
        if( FINAL )
            stage_reduce<float>( run, e, ec, t2, red_d, red_f );
        __syncthreads(); // the window buffer and red_d / red_f are reused by later tiles
    }
}

// ------------------------------------------------------------------ row-fused stage kernel
// For systems whose dipolar spectrum is kept ka-major (fused b/c pass): a block owns whole rows
// along a -- (system, c, b0 .. b0+nr-1), every basis atom and component -- and does the passes
// along a itself:
//   prologue  the dipolar field of its rows: C2R along a of the spectrum after the b/c pass
//             (pass A' arithmetic, the same line pairs (b0 even): the field is bit for bit the one
//             pass A' writes);
//   main      the stage (gradient with that field, thermal field, solver update) as llg_stage;
//   epilogue  R2C along a of the configuration the next field evaluation needs (the predictor,
//             or the new state after the last stage) into the spectrum (pass A arithmetic).
// So one field evaluation is the b/c pass and this kernel: two launches instead of four, and the
// field arrays are neither written nor read.
template<typename R>
struct RowArgs
{
    const FFTDesc * fd; // per system
    const cplx<R> * tw; // twiddle tables
    cplx<R> * W1;       // ka-major spectra [ka][cb][c][b]
    const int4 * map;   // (system, c, first b, rows)
};

constexpr int ROW_SPT = 4; // spins per thread the row kernel holds (rows * row length <= 1024)

template<typename R, int SOLVER, int STAGE>
__global__ void __launch_bounds__( 256 ) llg_stage_rows( StageArgs<R> A, RowArgs<R> F )
{
    extern __shared__ __align__( 16 ) unsigned char smem_raw[];
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red_d[32];
    __shared__ float red_f[32];
    const int4 bm     = F.map[blockIdx.x];
    const int s       = bm.x, cc = bm.y, b0 = bm.z, nr = bm.w;
    SysRun * run      = A.runs + s;
    const SysDesc & d = A.sd[s];
    const FFTDesc & f = F.fd[s];
    const int Ma = f.M[0], Mh = f.Mh, nb = f.nb, Na = f.N[0], Nb = f.N[1], Nc = f.N[2];
    const int ncb    = 3 * nb;
    const int nrq    = ( nr + 1 ) >> 1; // line pairs per component row
    const int nq     = ncb * nrq;       // complex lines of the block
    const int ls     = line_stride( Ma );
    const int rowlen = nb * Na;
    cplx<R> * tw     = reinterpret_cast<cplx<R> *>( smem_raw );
    cplx<R> * ba     = tw + Ma;
    cplx<R> * bb     = ba + nq * ls;
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    load_tw( tw, F.tw + f.tw_offset[0], Ma );
    __syncthreads();
    pdl_wait(); // everything below reads what earlier kernels wrote
    pdl_trigger();
    if( !A.tune && !run->active )
        return;
    constexpr bool FINAL = ( SOLVER == SOLVER_RK4 ) ? ( STAGE == 4 ) : ( STAGE == 2 );
    const size_t kstride = (size_t)ncb * Nc * Nb;
    cplx<R> * W1         = F.W1 + f.spec_offset;
    // ---- prologue: C2R along a (pass_a_inv, ka-major branch)
    for( int e = threadIdx.x; e < nq * Ma; e += blockDim.x )
    {
        const int q = (int)fdiv( (unsigned)e, f.div_Ma ), k = e - q * Ma;
        const int cb = q / nrq, bl = 2 * ( q - cb * nrq );
        const bool hi  = k >= Mh;
        const int kk   = hi ? Ma - k : k;
        const size_t o = (size_t)kk * kstride + ( (size_t)cb * Nc + cc ) * Nb + b0 + bl;
        cplx<R> x      = W1[o];
        cplx<R> y      = bl + 1 < nr ? W1[o + 1] : cplx<R>{ 0, 0 };
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
        ba[q * ls + k] = { x.x - y.y, x.y + y.x };
    }
    __syncthreads();
    const cplx<R> * hr = block_fft( ba, bb, Ma, ls, nq, f.plan[0], tw, true );
    const R invT       = fft_invT<R>( f );
    // ---- main: the stage on the block's spins
    const int i0        = rowlen * ( b0 + Nb * cc ); // first local spin of the block
    const int n_spins   = nr * rowlen;
    const int iteration = run->iteration;
    R e                 = 0;
    float t2            = 0;
    V3<R> nx[ROW_SPT];
#pragma unroll
    for( int k = 0; k < ROW_SPT; ++k )
    {
        const int el     = threadIdx.x + k * 256;
        const bool valid = el < n_spins;
        const int i      = i0 + ( valid ? el : 0 );
        int ib, a, b, c;
        cell_of( GS, i, ib, a, b, c );
        const int smode = warp_stencil_mode( GS, a, b, c, valid );
        nx[k]           = { 0, 0, 0 };
        if( valid )
        {
            const int gi         = (int)GS.off + i; // batches hold fewer than 2^31 spins
            const StageIn<R> pin = stage_inputs<R, SOLVER, STAGE>( A, C, gi );
            const R mu           = C.mu[ib];
            const V3<R> ci       = A.cfg.ld( gi );
            const int lr         = b - b0;
            V3<R> hv;
            {
                const int qb      = lr >> 1;
                const bool odd    = lr & 1;
                const cplx<R> vx  = hr[( ( 3 * ib + 0 ) * nrq + qb ) * ls + a];
                const cplx<R> vy  = hr[( ( 3 * ib + 1 ) * nrq + qb ) * ls + a];
                const cplx<R> vz  = hr[( ( 3 * ib + 2 ) * nrq + qb ) * ls + a];
                hv                = { ( odd ? vx.y : vx.x ) * invT, ( odd ? vy.y : vy.x ) * invT,
                       ( odd ? vz.y : vz.x ) * invT };
            }
            R ek    = 0;
            V3<R> g = gradient_at<R, false, FINAL>( GS, C, pairs, A.cfg, A.h, gi, ib, a, b, c, ci, mu, ek,
                                                               smode, &hv );
            e += ek;
            stage_update<R, SOLVER, STAGE>( A, C, d, gi, i, ib, ci, g, iteration, t2, pin );
            const V3<R> v = FINAL ? A.s.ld( gi ) : A.out.ld( gi ); // this thread's own store
            nx[k]         = { mu * v.x, mu * v.y, mu * v.z };
        }
    }
    __syncthreads(); // the field buffer is free
    // ---- epilogue: R2C along a of the next configuration (pass_a, ka-major branch)
#pragma unroll
    for( int k = 0; k < ROW_SPT; ++k )
    {
        const int el = threadIdx.x + k * 256;
        if( el < n_spins )
        {
            const int lr = el / rowlen, rem = el - lr * rowlen;
            const int a = rem / nb, ib = rem - a * nb;
            const int qb = lr >> 1;
            R * px       = reinterpret_cast<R *>( ba + ( ( 3 * ib + 0 ) * nrq + qb ) * ls + a ) + ( lr & 1 );
            R * py       = reinterpret_cast<R *>( ba + ( ( 3 * ib + 1 ) * nrq + qb ) * ls + a ) + ( lr & 1 );
            R * pz       = reinterpret_cast<R *>( ba + ( ( 3 * ib + 2 ) * nrq + qb ) * ls + a ) + ( lr & 1 );
            *px          = nx[k].x;
            *py          = nx[k].y;
            *pz          = nx[k].z;
        }
    }
    // zero padding along a, and the second line of an unpaired last row
    for( int e2 = threadIdx.x; e2 < nq * Ma; e2 += blockDim.x )
    {
        const int q = (int)fdiv( (unsigned)e2, f.div_Ma ), t = e2 - q * Ma;
        const int bl = 2 * ( q % nrq );
        if( t >= Na )
            ba[q * ls + t] = { 0, 0 };
        else if( bl + 1 >= nr )
            ba[q * ls + t].y = 0;
    }
    __syncthreads();
    const cplx<R> * r = block_fft( ba, bb, Ma, ls, nq, f.plan[0], tw, false );
    for( int e2 = threadIdx.x; e2 < ncb * nr * Mh; e2 += blockDim.x )
    {
        const int lr = e2 % nr, rest = e2 / nr;
        const int cb = rest % ncb, k = rest / ncb;
        const cplx<R> * z = r + ( cb * nrq + ( lr >> 1 ) ) * ls;
        const cplx<R> zk = z[k], zm = z[k == 0 ? 0 : Ma - k];
        W1[(size_t)k * kstride + ( (size_t)cb * Nc + cc ) * Nb + b0 + lr]
            = ( lr & 1 ) ? cplx<R>{ R( 0.5 ) * ( zk.y + zm.y ), R( -0.5 ) * ( zk.x - zm.x ) }
                         : cplx<R>{ R( 0.5 ) * ( zk.x + zm.x ), R( 0.5 ) * ( zk.y - zm.y ) };
    }
    if( !FINAL )
        return;
    stage_reduce<R>( run, e, R( 0 ), t2, red_d, red_f );
}

// ------------------------------------------------------------------ evaluation kernel
// gradient (AoS double out), per-term energy sums (5 doubles per system) and optional per-spin
// per-term energies.  Used by the API getters and the parity tests.
template<typename R>
__global__ void __launch_bounds__( 256 ) eval_kernel( const SysDesc * sd, const int2 * blkmap, SoA3<R> spins,
                                                      SoA3<R> h, int only_sys, double * grad, double * term_sums,
                                                      double * per_spin )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red[32];
    const int2 bm = blkmap[blockIdx.x];
    const int s   = bm.x;
    if( s != only_sys )
        return;
    const SysDesc & d = sd[s];
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( GS, d );
    __syncthreads();
    const int i      = bm.y + threadIdx.x;
    double et[N_TERMS] = { 0, 0, 0, 0, 0 };
    if( i < d.nos )
    {
        const long long gi = GS.off + i;
        const int cell     = (int)fdiv( (unsigned)i, GS.div_nb );
        const int ib       = i - cell * GS.nb;
        const int rest     = (int)fdiv( (unsigned)cell, GS.div_na );
        const int a        = cell - rest * GS.n[0];
        const int c        = (int)fdiv( (unsigned)rest, GS.div_nbb );
        const int b        = rest - c * GS.n[1];
        const R mu      = C.mu[ib];
        const V3<R> si  = spins.ld( gi );
        R e             = 0;
        V3<R> g         = gradient_at<R>( GS, C, pairs, spins, h, gi, ib, a, b, c, si, mu, e );
        grad[3 * (size_t)i + 0] = g.x;
        grad[3 * (size_t)i + 1] = g.y;
        grad[3 * (size_t)i + 2] = g.z;
        // per-term energies (E_Zeeman, E_Anisotropy, E_Exchange, E_DMI, E_DDI; cpp:307-511)
        if( d.has_zeeman )
            et[TERM_ZEEMAN] = -(double)mu * ( d.zeeman[0] * si.x + d.zeeman[1] * si.y + d.zeeman[2] * si.z );
        for( int k = 0; k < d.n_aniso; ++k )
            if( d.aniso_idx[k] == ib )
            {
                double dd = d.aniso_n[k][0] * si.x + d.aniso_n[k][1] * si.y + d.aniso_n[k][2] * si.z;
                et[TERM_ANISOTROPY] -= d.aniso_K[k] * dd * dd;
            }
        for( int p = d.pair_begin[ib]; p < d.pair_begin[ib + 1]; ++p )
        {
            const PairR<R> P = pairs[p];
            long long j      = pair_index( GS, a, b, c, P.j, P.da, P.db, P.dc );
            if( j >= 0 )
            {
                V3<R> sj = spins.ld( j );
                et[TERM_EXCHANGE] -= 0.5 * (double)P.J * ( (double)si.x * sj.x + (double)si.y * sj.y + (double)si.z * sj.z );
                V3<R> cr = cross( si, sj );
                et[TERM_DMI] -= 0.5 * ( (double)P.Dx * cr.x + (double)P.Dy * cr.y + (double)P.Dz * cr.z );
            }
        }
        if( h.x )
        {
            V3<R> hh      = h.ld( gi );
            et[TERM_DDI]  = -0.5 * (double)mu * ( (double)hh.x * si.x + (double)hh.y * si.y + (double)hh.z * si.z );
        }
        if( per_spin )
            for( int t = 0; t < N_TERMS; ++t )
                per_spin[(size_t)t * d.nos + i] = et[t];
    }
    for( int t = 0; t < N_TERMS; ++t )
    {
        double v = block_sum( et[t], red );
        if( threadIdx.x == 0 )
            atomicAdd( &term_sums[t], v );
    }
}

// ------------------------------------------------------------------ transfers
// lo (x != nullptr, FP32 compensated state): also the low parts, x - (double)(float)x
template<typename R>
__global__ void aos_to_soa( const double * aos, SoA3<R> dst, long long off, int n, SoA3<R> lo )
{
    for( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
    {
        const double v[3] = { aos[3 * (size_t)i], aos[3 * (size_t)i + 1], aos[3 * (size_t)i + 2] };
        const V3<R> h     = { (R)v[0], (R)v[1], (R)v[2] };
        dst.st( off + i, h );
        if( lo.x )
            lo.st( off + i, V3<R>{ (R)( v[0] - (double)h.x ), (R)( v[1] - (double)h.y ), (R)( v[2] - (double)h.z ) } );
    }
}
template<typename R>
__global__ void soa_to_aos( SoA3<R> src, long long off, int n, double * aos, SoA3<R> lo )
{
    for( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x )
    {
        V3<R> v              = src.ld( off + i );
        double x = v.x, y = v.y, z = v.z;
        if( lo.x )
        {
            const V3<R> l = lo.ld( off + i );
            x += (double)l.x;
            y += (double)l.y;
            z += (double)l.z;
        }
        aos[3 * (size_t)i]     = x;
        aos[3 * (size_t)i + 1] = y;
        aos[3 * (size_t)i + 2] = z;
    }
}

// ================================================================== host
template<typename R>
static void fill_const( SysConst<R> & c, const SysDesc & d )
{
    const double a = d.damping;
    const double dtg = d.dt * C_GAMMA / C_MU_B / ( 1 + a * a );
    c.dtg            = (R)dtg;
    c.dtga           = (R)( dtg * a );
    c.alpha          = (R)a;
    c.kdm            = (R)( d.dt * C_GAMMA / C_MU_B );
    c.dt             = (R)d.dt;
    const double eps = std::sqrt( 2 * a * d.dt * C_GAMMA / C_MU_B * C_K_B ) / ( 1 + a * a );
    for( int b = 0; b < d.nb; ++b )
    {
        c.noise[b]  = (R)( eps * std::sqrt( d.temperature / d.mu_s[b] ) );
        c.mu[b]     = (R)d.mu_s[b];
        c.inv_mu[b] = (R)( 1.0 / d.mu_s[b] );
    }
    for( int e = 0; e < 3; ++e )
        c.zeeman[e] = (R)d.zeeman[e];
    c.has_zeeman = d.has_zeeman;
    c.n_aniso    = d.n_aniso;
    for( int k = 0; k < d.n_aniso; ++k )
    {
        c.aniso_idx[k] = d.aniso_idx[k];
        c.aniso_K[k]   = (R)d.aniso_K[k];
        for( int e = 0; e < 3; ++e )
            c.aniso_n[k][e] = (R)d.aniso_n[k][e];
    }
    c.thermal = d.temperature > 0 && !d.direct_minimization;
    c.direct  = d.direct_minimization;
}

static void fill_consts( SysDesc & d )
{
    fill_const( d.cf, d );
    fill_const( d.cd, d );
}

static void fill_desc( SysDesc & d, const SystemInput & in )
{
    const Geometry & g        = *in.geom;
    const HamiltonianParams & h = *in.ham;
    for( int e = 0; e < 3; ++e )
    {
        d.n_cells[e] = g.n_cells[e];
        d.bc[e]      = h.bc[e] ? 1 : 0;
    }
    d.nb      = g.nb();
    d.nos     = g.nos();
    d.div_nb  = make_fastdiv( d.nb );
    d.div_na  = make_fastdiv( d.n_cells[0] );
    d.div_nbb = make_fastdiv( d.n_cells[1] );
    if( d.nb > MAX_BASIS )
        throw std::runtime_error( "too many basis atoms for the device engine" );
    for( int b = 0; b < d.nb; ++b )
        d.mu_s[b] = g.mu_s_basis[b];
    // Zeeman: stored times mu_B (Hamiltonian_Heisenberg.cpp:35); active if |B mu_B| > 1e-60 (cpp:205)
    double Bm    = h.B * C_MU_B;
    d.has_zeeman = std::abs( Bm ) > 1e-60;
    for( int e = 0; e < 3; ++e )
        d.zeeman[e] = h.B_normal[e] * Bm;
    d.n_aniso = (int)h.aniso_idx.size();
    if( d.n_aniso > MAX_BASIS )
        throw std::runtime_error( "too many anisotropy entries" );
    for( int k = 0; k < d.n_aniso; ++k )
    {
        d.aniso_idx[k] = h.aniso_idx[k];
        d.aniso_K[k]   = h.aniso_K[k];
        for( int e = 0; e < 3; ++e )
            d.aniso_n[k][e] = h.aniso_n[k][e];
    }
    // merge exchange and DMI pairs per basis atom, keeping the reference's pair order
    std::vector<std::vector<PairEntry>> per( d.nb );
    auto add = [&]( const Pair & p, double J, const Vec3 * Dv ) {
        if( p.i < 0 || p.i >= d.nb || p.j < 0 || p.j >= d.nb )
            return;
        auto & L = per[p.i];
        for( auto & q : L )
            if( q.j == p.j && q.da == p.t[0] && q.db == p.t[1] && q.dc == p.t[2] )
            {
                q.J += J;
                if( Dv )
                    for( int e = 0; e < 3; ++e )
                        q.D[e] += ( *Dv )[e];
                return;
            }
        PairEntry q{};
        q.i  = p.i;
        q.j  = p.j;
        q.da = p.t[0];
        q.db = p.t[1];
        q.dc = p.t[2];
        q.J  = J;
        if( Dv )
            for( int e = 0; e < 3; ++e )
                q.D[e] = ( *Dv )[e];
        L.push_back( q );
    };
    for( size_t k = 0; k < h.ex_pairs.size(); ++k )
        add( h.ex_pairs[k], h.ex_J[k], nullptr );
    for( size_t k = 0; k < h.dmi_pairs.size(); ++k )
    {
        Vec3 Dv{ h.dmi_D[k] * h.dmi_n[k][0], h.dmi_D[k] * h.dmi_n[k][1], h.dmi_D[k] * h.dmi_n[k][2] };
        add( h.dmi_pairs[k], 0.0, &Dv );
    }
    int n = 0;
    d.max_t[0] = d.max_t[1] = d.max_t[2] = 0;
    for( int b = 0; b < d.nb; ++b )
    {
        d.pair_begin[b] = n;
        for( auto & q : per[b] )
        {
            if( n >= MAX_PAIRS )
                throw std::runtime_error( "too many interaction pairs for the device engine" );
            d.pairs[n++] = q;
            d.max_t[0]   = std::max( d.max_t[0], std::abs( q.da ) );
            d.max_t[1]   = std::max( d.max_t[1], std::abs( q.db ) );
            d.max_t[2]   = std::max( d.max_t[2], std::abs( q.dc ) );
        }
    }
    d.pair_begin[d.nb] = n;
    d.n_pairs          = n;
    d.dt                  = in.dt;
    d.damping             = in.damping;
    d.temperature         = in.temperature;
    d.direct_minimization = in.direct_minimization ? 1 : 0;
    d.force_convergence   = in.force_convergence;
    d.seed                = in.seed;
    d.stream              = in.stream;
    d.noise_offset        = in.noise_offset;
    d.n_iterations        = 0;
    d.ddi                 = ( h.ddi_method == 1 ) ? 1 : 0;
    fill_consts( d );
}

void fill_system_desc( SysDesc & d, const SystemInput & in )
{
    d = SysDesc{};
    fill_desc( d, in );
}

Engine::Engine( const std::vector<SystemInput> & systems, bool fp64 ) : fp64_( fp64 )
{
    elem_ = fp64 ? sizeof( double ) : sizeof( float );
    CUDA_CHECK( cudaStreamCreateWithFlags( &own_stream_, cudaStreamNonBlocking ) );
    stream_ = own_stream_;
    build_systems( systems );
}

Engine::~Engine()
{
    if( graph_ )
        cudaGraphExecDestroy( graph_ );
    if( graph1_ )
        cudaGraphExecDestroy( graph1_ );
    for( int c = 0; c < 3; ++c )
    {
        dfree( spins_[c] );
        dfree( predA_[c] );
        dfree( predB_[c] );
        dfree( aux1_[c] );
        dfree( aux2_[c] );
        dfree( noise_[c] );
        dfree( field_[c] );
        dfree( lo_[c] );
    }
    dfree( d_desc_ );
    dfree( d_runs_ );
    dfree( d_stage_ );
    dfree( d_red_ );
    dfree( d_grad_ );
    dfree( d_blkmap_ );
    for( int k = 0; k < 3; ++k )
    {
        dfree( d_sblkmap_[k] );
    }
    dfree( d_rowmap_ );
    dfree( d_tiles_ );
    dfree( d_err_ );
    if( lane_ )
    {
        for( int c = 0; c < 3; ++c )
            dfree( lane_->field[c] );
        if( lane_->stream )
            cudaStreamDestroy( lane_->stream );
    }
    if( own_stream_ )
        cudaStreamDestroy( own_stream_ );
}

Engine::DdiLane * Engine::ddi_lane()
{
    if( !any_ddi_ )
        return nullptr;
    if( !lane_ )
    {
        auto L = std::make_unique<DdiLane>();
        CUDA_CHECK( cudaStreamCreateWithFlags( &L->stream, cudaStreamNonBlocking ) );
        try
        {
            for( int c = 0; c < 3; ++c )
            {
                L->field[c] = dalloc_bytes( total_ * elem_ );
                CUDA_CHECK( cudaMemsetAsync( L->field[c], 0, total_ * elem_, stream_ ) );
            }
            L->plan.build( ddi_systems_, fp64_, d_desc_, stream_ );
            L->plan.copy_shape_from( ddi_ );
            CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
        }
        catch( ... )
        {
            for( int c = 0; c < 3; ++c )
                dfree( L->field[c] );
            cudaStreamDestroy( L->stream );
            throw;
        }
        lane_ = std::move( L );
    }
    return lane_.get();
}

void Engine::set_stream( cudaStream_t s )
{
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    stream_ = s ? s : own_stream_;
}

void Engine::build_systems( const std::vector<SystemInput> & systems )
{
    desc_.assign( systems.size(), SysDesc{} );
    geoms_.clear();
    long long off = 0;
    int max_nos   = 0;
    std::vector<int2> blkmap;
    std::vector<DDISystem> ddis;
    for( size_t s = 0; s < systems.size(); ++s )
    {
        fill_desc( desc_[s], systems[s] );
        desc_[s].spin_offset = off;
        off += ( desc_[s].nos + SPIN_ALIGN - 1 ) / SPIN_ALIGN * SPIN_ALIGN;
        max_nos = std::max( max_nos, desc_[s].nos );
        geoms_.push_back( systems[s].geom );
        int nbk = ( desc_[s].nos + threads_ - 1 ) / threads_;
        for( int k = 0; k < nbk; ++k )
            blkmap.push_back( make_int2( (int)s, k * threads_ ) );
        if( desc_[s].ddi )
        {
            const Geometry & g = *systems[s].geom;
            const auto & h     = *systems[s].ham;
            DDISystem D;
            D.sys              = (int)s;
            D.n_cells          = g.n_cells;
            D.bc               = { desc_[s].bc[0], desc_[s].bc[1], desc_[s].bc[2] };
            D.padded           = ddi_padding( g.n_cells, D.bc, h.ddi_pb_zero_padding );
            D.images           = h.ddi_images;
            D.nb               = g.nb();
            D.lattice_constant = g.lattice_constant;
            D.bravais          = g.bravais;
            D.cell_atoms       = g.cell_atoms;
            D.mu_s             = g.mu_s_basis;
            ddis.push_back( D );
            desc_[s].fft_slot = (int)ddis.size() - 1;
        }
    }
    total_    = std::max<long long>( off, SPIN_ALIGN );
    // the stage kernels index the batch with 32-bit integers
    if( total_ >= ( 1LL << 31 ) )
        throw std::runtime_error( "batch of 2^31 spins or more: not supported by the stage kernels" );
    n_blocks_ = (int)blkmap.size();
    for( int c = 0; c < 3; ++c )
    {
        spins_[c] = dalloc_bytes( total_ * elem_ );
        predA_[c] = dalloc_bytes( total_ * elem_ );
        predB_[c] = dalloc_bytes( total_ * elem_ );
        aux1_[c]  = dalloc_bytes( total_ * elem_ );
        aux2_[c]  = dalloc_bytes( total_ * elem_ );
        noise_[c] = dalloc_bytes( total_ * elem_ );
    }
    d_desc_     = dalloc<SysDesc>( desc_.size() );
    d_runs_     = dalloc<SysRun>( desc_.size() );
    d_stage_    = dalloc<double>( 3 * (size_t)total_ );
    d_grad_     = dalloc<double>( 3 * (size_t)std::max( max_nos, 1 ) );
    d_red_      = dalloc<double>( N_TERMS * 2 );
    d_blkmap_   = dalloc<int2>( std::max<size_t>( blkmap.size(), 1 ) );
    h2d( d_desc_, desc_.data(), desc_.size() );
    h2d( d_blkmap_, blkmap.data(), blkmap.size() );
    for( int k = 0; k < 3; ++k )
    {
        const int span = 256 * SPT_OPTIONS[k];
        std::vector<int2> m;
        for( size_t sy = 0; sy < desc_.size(); ++sy )
        {
            int nbk = ( desc_[sy].nos + span - 1 ) / span;
            for( int q = 0; q < nbk; ++q )
                m.push_back( make_int2( (int)sy, q * span ) );
        }
        n_sblocks_[k] = (int)m.size();
        d_sblkmap_[k] = dalloc<int2>( std::max<size_t>( m.size(), 1 ) );
        if( !m.empty() )
            h2d( d_sblkmap_[k], m.data(), m.size() );
    }
    any_ddi_ = !ddis.empty();
    if( any_ddi_ )
    {
        for( int c = 0; c < 3; ++c )
            field_[c] = dalloc_bytes( total_ * elem_ );
        ddi_.build( ddis, fp64_, d_desc_, stream_ );
        ddi_.tune( d_desc_, spins_[0], spins_[1], spins_[2], field_[0], field_[1], field_[2], stream_ );
        ddi_systems_ = ddis;
        build_row_map( (int)ddis.size() );
    }
    d_err_ = dalloc<int>( 1 );
    build_tiles();
}

bool encode_tensor_map_1d_f32( CUtensorMap * map, const void * base, unsigned long long n, unsigned box )
{
    typedef CUresult ( *Encode )( CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill );
    static Encode encode = [] {
        void * f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if( cudaGetDriverEntryPointByVersion( "cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q )
                != cudaSuccess
            || q != cudaDriverEntryPointSuccess )
        {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<Encode>( f );
    }();
    const bool debug = std::getenv( "SPIRIT_GB300_DEBUG" ) != nullptr;
    if( !encode || ( reinterpret_cast<uintptr_t>( base ) & 15 ) )
    {
        if( debug )
            std::fprintf( stderr, "spirit_gb300: no tensor-map encoder (%d) or unaligned base\n", encode != nullptr );
        return false;
    }
    const cuuint64_t dim[1]  = { n };
    const cuuint64_t str[1]  = { n * sizeof( float ) }; // rank 1: no stride is read
    const cuuint32_t bx[1]   = { box };
    const cuuint32_t estr[1] = { 1 };
    const CUresult r = encode( map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, const_cast<void *>( base ), dim, str, bx, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE );
    if( r != CUDA_SUCCESS && debug )
        std::fprintf( stderr, "spirit_gb300: cuTensorMapEncodeTiled returned %d\n", (int)r );
    return r == CUDA_SUCCESS;
}

// The TMA-staged stage kernel can serve FP32 batches in which every system's window (a tile of
// TT_SPINS spins plus the stencil reach H on both sides, aligned to 16 bytes) fits TT_NCOPY
// copies of TT_BOX floats; tiles never cross systems.  It is selected by SPIRIT_GB300_TMA=1: measured
// on the 256-system SIB ensemble it is slower than llg_stage (0.41 against 0.33 ms per step; the
// stage kernels are bound by instruction issue and the per-spin loads of the state, not by the
// neighbour reads it stages, and one-tile systems get a single CTA), so llg_stage is the default.
void Engine::build_tiles()
{
    tma_             = false;
    const char * env = std::getenv( "SPIRIT_GB300_TMA" );
    if( fp64_ || rows_ || !( env && env[0] == '1' ) || total_ >= ( 1LL << 30 ) )
        return;
    std::vector<int4> tiles;
    for( size_t s = 0; s < desc_.size(); ++s )
    {
        const SysDesc & d = desc_[s];
        long long H       = 0;
        for( int p = 0; p < d.n_pairs; ++p )
        {
            const PairEntry & q = d.pairs[p];
            const long long lin = q.j - q.i
                                  + (long long)d.nb
                                        * ( q.da + (long long)d.n_cells[0] * ( q.db + (long long)d.n_cells[1] * q.dc ) );
            H = std::max( H, std::abs( lin ) );
        }
        for( int t0 = 0; t0 < d.nos; t0 += TT_SPINS )
        {
            const int n          = std::min( TT_SPINS, d.nos - t0 );
            const long long lo   = d.spin_offset + t0 - H;
            const long long xs   = lo >= 0 ? lo / 4 * 4 : -( ( -lo + 3 ) / 4 * 4 ); // 16-byte aligned start
            const long long hi   = d.spin_offset + t0 + n + H;
            const long long ncpy = ( hi - xs + TT_BOX - 1 ) / TT_BOX;
            if( ncpy > TT_NCOPY )
            {
                if( std::getenv( "SPIRIT_GB300_DEBUG" ) )
                    std::fprintf( stderr, "spirit_gb300: system %zu reaches %lld spins: llg_stage\n", s, H );
                return; // a stencil reaching too far: llg_stage serves this batch
            }
            tiles.push_back( make_int4( (int)s, t0, (int)xs, (int)ncpy ) );
        }
    }
    void * const * bufs[3] = { spins_, predA_, predB_ };
    for( int b = 0; b < 3; ++b )
        for( int c = 0; c < 3; ++c )
            if( !encode_tensor_map_1d_f32( &tmaps_[b][c], bufs[b][c], (unsigned long long)total_, TT_BOX ) )
                return;
    d_tiles_ = dalloc<int4>( std::max<size_t>( tiles.size(), 1 ) );
    if( !tiles.empty() )
        h2d( d_tiles_, tiles.data(), tiles.size() );
    n_tiles_ = (int)tiles.size();
    tma_     = n_tiles_ > 0;
    if( std::getenv( "SPIRIT_GB300_DEBUG" ) )
        std::fprintf( stderr, "spirit_gb300: TMA-staged stage kernel, %d systems, %d tiles\n", (int)desc_.size(),
                      n_tiles_ );
}

void Engine::check_err()
{
    if( !d_err_ )
        return;
    int e = 0;
    CUDA_CHECK( cudaMemcpyAsync( &e, d_err_, sizeof( int ), cudaMemcpyDeviceToHost, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    if( e )
    {
        CUDA_CHECK( cudaMemsetAsync( d_err_, 0, sizeof( int ), stream_ ) );
        CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
        throw CudaError( "stage kernel: a tensor copy did not complete within the wait limit" );
    }
}

// Row-fused stages (llg_stage_rows), selected by SPIRIT_GB300_ROWS=1, when every system has the
// dipolar interaction on the fused (ka-major) b/c path and a block of whole rows fits: rows per
// block even (the line pairs of pass A / A'), rows * row length <= 1024 spins, the line buffers
// within the shared memory.  Not the default: on the 128x128x16 Heun workload the fused kernel
// (0.143 ms/step at 512 spins per block; 0.151 at 256, 0.171 at 1024) is slower than the
// separate passes (0.112 ms/step) -- each block runs its C2R, stage and R2C phases one after
// another with few lines to transform, where the separate kernels each fill the GPU.
void Engine::build_row_map( int n_ddi )
{
    rows_ = false;
    const char * env = std::getenv( "SPIRIT_GB300_ROWS" );
    if( !( env && env[0] == '1' ) )
        return;
    if( n_ddi != (int)desc_.size() || !ddi_.fused )
        return;
    std::vector<int4> m;
    size_t smem = 0;
    for( size_t s = 0; s < desc_.size(); ++s )
    {
        const FFTDesc & f = ddi_.fd_host[s];
        const int rowlen  = f.nb * f.N[0];
        int nr            = 2;
        const char * want = std::getenv( "SPIRIT_GB300_ROW_SPINS" ); // spins per block (experiments)
        const int target  = want ? std::atoi( want ) : 512;
        while( nr * 2 * rowlen <= target )
            nr *= 2;
        if( nr * rowlen > 256 * 4 )
            return;
        const int nq = 3 * f.nb * ( ( nr + 1 ) / 2 );
        smem         = std::max( smem, elem_ * 2 * ( f.M[0] + 2 * (size_t)nq * line_stride( f.M[0] ) ) );
        for( int c = 0; c < f.N[2]; ++c )
            for( int b0 = 0; b0 < f.N[1]; b0 += nr )
                m.push_back( make_int4( (int)s, c, b0, std::min( nr, f.N[1] - b0 ) ) );
    }
    if( smem > 96 * 1024 )
        return;
    d_rowmap_ = dalloc<int4>( m.size() );
    h2d( d_rowmap_, m.data(), m.size() );
    n_rowblocks_ = (int)m.size();
    rows_smem_   = smem;
    rows_        = true;
}

// the spectrum must hold the current state's before the first b/c pass of a step sequence
void Engine::ensure_spectrum()
{
    if( !rows_ || w1_valid_ )
        return;
    ddi_.run( d_desc_, d_runs_, spins_[0], spins_[1], spins_[2], field_[0], field_[1], field_[2], stream_, 0 );
    w1_valid_ = true;
}

void Engine::set_params( int s, const SystemInput & in )
{
    w1_valid_   = false;
    SysDesc & d = desc_[s];
    d.dt                  = in.dt;
    d.damping             = in.damping;
    d.temperature         = in.temperature;
    d.direct_minimization = in.direct_minimization ? 1 : 0;
    d.force_convergence   = in.force_convergence;
    d.seed                = in.seed;
    d.stream              = in.stream;
    d.noise_offset        = in.noise_offset;
    fill_consts( d );
    CUDA_CHECK( cudaMemcpyAsync( d_desc_ + s, &d, sizeof( SysDesc ), cudaMemcpyHostToDevice, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
}

template<typename R>
static SoA3<R> soa( void * const * p )
{
    return { (R *)p[0], (R *)p[1], (R *)p[2] };
}

// Low parts of the compensated FP32 state as kernel arguments: for writing (set_spins: the low parts
// of the host values) and for reading (only while they belong to the current high parts)
SoA3<float> Engine::lo_soa()
{
    if( !comp_ )
        return { nullptr, nullptr, nullptr };
    if( !lo_valid_ )
    {
        // high parts changed behind the state's back (spin_ptr): start the low parts from zero
        for( int c = 0; c < 3; ++c )
            CUDA_CHECK( cudaMemsetAsync( lo_[c], 0, total_ * sizeof( float ), stream_ ) );
        lo_valid_ = true;
    }
    return { (float *)lo_[0], (float *)lo_[1], (float *)lo_[2] };
}

SoA3<float> Engine::lo_valid() const
{
    if( comp_ && lo_valid_ )
        return { (float *)lo_[0], (float *)lo_[1], (float *)lo_[2] };
    return { nullptr, nullptr, nullptr };
}

// Keep FP32 spins as hi + lo pairs (the compensated state of the LLG stage kernels);
// SPIRIT_GB300_COMP=0 keeps the plain FP32 state.  No effect on FP64 engines.
void Engine::enable_compensation()
{
    if( fp64_ || comp_ )
        return;
    const char * env = std::getenv( "SPIRIT_GB300_COMP" );
    if( env && env[0] == '0' )
        return;
    for( int c = 0; c < 3; ++c )
        lo_[c] = dalloc_bytes( total_ * sizeof( float ) ); // zero: the current state is hi exactly
    comp_     = true;
    lo_valid_ = true;
}

void Engine::set_spins( int s, const double * aos, bool sync )
{
    w1_valid_         = false;
    const SysDesc & d = desc_[s];
    CUDA_CHECK( cudaMemcpyAsync( d_stage_, aos, sizeof( double ) * 3 * d.nos, cudaMemcpyHostToDevice, stream_ ) );
    int grid = std::min( 1024, ( d.nos + 255 ) / 256 );
    if( fp64_ )
        aos_to_soa<double><<<grid, 256, 0, stream_>>>( d_stage_, soa<double>( spins_ ), d.spin_offset, d.nos,
                                                        SoA3<double>{ nullptr, nullptr, nullptr } );
    else
        aos_to_soa<float><<<grid, 256, 0, stream_>>>( d_stage_, soa<float>( spins_ ), d.spin_offset, d.nos, lo_soa() );
    CUDA_CHECK( cudaGetLastError() );
    if( sync )
        CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
}

Engine::Status Engine::fetch( int s, double * aos )
{
    const SysDesc & d = desc_[s];
    int grid          = std::min( 1024, ( d.nos + 255 ) / 256 );
    if( fp64_ )
        soa_to_aos<double><<<grid, 256, 0, stream_>>>( soa<double>( spins_ ), d.spin_offset, d.nos, d_stage_,
                                                        SoA3<double>{ nullptr, nullptr, nullptr } );
    else
        soa_to_aos<float><<<grid, 256, 0, stream_>>>( soa<float>( spins_ ), d.spin_offset, d.nos, d_stage_,
                                                       lo_valid() );
    CUDA_CHECK( cudaGetLastError() );
    CUDA_CHECK( cudaMemcpyAsync( aos, d_stage_, sizeof( double ) * 3 * d.nos, cudaMemcpyDeviceToHost, stream_ ) );
    SysRun r;
    CUDA_CHECK( cudaMemcpyAsync( &r, d_runs_ + s, sizeof( SysRun ), cudaMemcpyDeviceToHost, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    return { r.iteration, r.active, r.max_torque, r.energy };
}

void Engine::get_spins( int s, double * aos )
{
    const SysDesc & d = desc_[s];
    int grid          = std::min( 1024, ( d.nos + 255 ) / 256 );
    if( fp64_ )
        soa_to_aos<double><<<grid, 256, 0, stream_>>>( soa<double>( spins_ ), d.spin_offset, d.nos, d_stage_,
                                                        SoA3<double>{ nullptr, nullptr, nullptr } );
    else
        soa_to_aos<float><<<grid, 256, 0, stream_>>>( soa<float>( spins_ ), d.spin_offset, d.nos, d_stage_,
                                                       lo_valid() );
    CUDA_CHECK( cudaGetLastError() );
    CUDA_CHECK( cudaMemcpyAsync( aos, d_stage_, sizeof( double ) * 3 * d.nos, cudaMemcpyDeviceToHost, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
}

void Engine::set_all_spins( const double * aos )
{
    w1_valid_ = false;
    // one host->device copy of the concatenated systems, then per-system conversion kernels
    size_t n = 0;
    for( auto & d : desc_ )
        n += 3 * (size_t)d.nos;
    CUDA_CHECK( cudaMemcpyAsync( d_stage_, aos, sizeof( double ) * n, cudaMemcpyHostToDevice, stream_ ) );
    size_t o = 0;
    for( auto & d : desc_ )
    {
        int grid = std::min( 1024, ( d.nos + 255 ) / 256 );
        if( fp64_ )
            aos_to_soa<double><<<grid, 256, 0, stream_>>>( d_stage_ + o, soa<double>( spins_ ), d.spin_offset, d.nos,
                                                            SoA3<double>{ nullptr, nullptr, nullptr } );
        else
            aos_to_soa<float><<<grid, 256, 0, stream_>>>( d_stage_ + o, soa<float>( spins_ ), d.spin_offset, d.nos,
                                                           lo_soa() );
        o += 3 * (size_t)d.nos;
    }
    CUDA_CHECK( cudaGetLastError() );
}

void Engine::get_all_spins( double * aos )
{
    size_t o = 0;
    for( auto & d : desc_ )
    {
        int grid = std::min( 1024, ( d.nos + 255 ) / 256 );
        if( fp64_ )
            soa_to_aos<double><<<grid, 256, 0, stream_>>>( soa<double>( spins_ ), d.spin_offset, d.nos, d_stage_ + o,
                                                            SoA3<double>{ nullptr, nullptr, nullptr } );
        else
            soa_to_aos<float><<<grid, 256, 0, stream_>>>( soa<float>( spins_ ), d.spin_offset, d.nos, d_stage_ + o,
                                                           lo_valid() );
        o += 3 * (size_t)d.nos;
    }
    CUDA_CHECK( cudaGetLastError() );
    CUDA_CHECK( cudaMemcpyAsync( aos, d_stage_, sizeof( double ) * o, cudaMemcpyDeviceToHost, stream_ ) );
}

template<typename R>
void Engine::gradient_t( int s, double * grad_aos, double * energy, double * terms, double * per_spin_host )
{
    const SysDesc & d = desc_[s];
    SoA3<R> h{ nullptr, nullptr, nullptr };
    if( d.ddi )
    {
        ddi_.run( d_desc_, nullptr, spins_[0], spins_[1], spins_[2], field_[0], field_[1], field_[2], stream_ );
        w1_valid_ = false;
        h = soa<R>( field_ );
    }
    CUDA_CHECK( cudaMemsetAsync( d_red_, 0, sizeof( double ) * N_TERMS, stream_ ) );
    double * d_ps = nullptr;
    if( per_spin_host )
        d_ps = dalloc<double>( (size_t)N_TERMS * d.nos );
    eval_kernel<R><<<n_blocks_, threads_, 0, stream_>>>( d_desc_, d_blkmap_, soa<R>( spins_ ), h, s, d_grad_, d_red_,
                                                         d_ps );
    CUDA_CHECK( cudaGetLastError() );
    double sums[N_TERMS];
    CUDA_CHECK( cudaMemcpyAsync( sums, d_red_, sizeof( sums ), cudaMemcpyDeviceToHost, stream_ ) );
    if( grad_aos )
        CUDA_CHECK( cudaMemcpyAsync( grad_aos, d_grad_, sizeof( double ) * 3 * d.nos, cudaMemcpyDeviceToHost, stream_ ) );
    if( per_spin_host )
        CUDA_CHECK( cudaMemcpyAsync( per_spin_host, d_ps, sizeof( double ) * N_TERMS * d.nos, cudaMemcpyDeviceToHost,
                                     stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    if( d_ps )
        dfree( d_ps );
    double E = 0;
    for( int t = 0; t < N_TERMS; ++t )
        E += sums[t];
    if( energy )
        *energy = E;
    if( terms )
        for( int t = 0; t < N_TERMS; ++t )
            terms[t] = sums[t];
}

void Engine::gradient( int s, double * grad_aos, double * energy, double * terms )
{
    if( fp64_ )
        gradient_t<double>( s, grad_aos, energy, terms, nullptr );
    else
        gradient_t<float>( s, grad_aos, energy, terms, nullptr );
}

void Engine::energy_per_spin( int s, double * per_term )
{
    if( fp64_ )
        gradient_t<double>( s, nullptr, nullptr, nullptr, per_term );
    else
        gradient_t<float>( s, nullptr, nullptr, nullptr, per_term );
}

void Engine::ddi_field( int s, double * h_aos )
{
    const SysDesc & d = desc_[s];
    if( !d.ddi )
    {
        std::fill( h_aos, h_aos + 3 * (size_t)d.nos, 0.0 );
        return;
    }
    ddi_.run( d_desc_, nullptr, spins_[0], spins_[1], spins_[2], field_[0], field_[1], field_[2], stream_ );
    w1_valid_ = false;
    int grid = std::min( 1024, ( d.nos + 255 ) / 256 );
    if( fp64_ )
        soa_to_aos<double><<<grid, 256, 0, stream_>>>( soa<double>( field_ ), d.spin_offset, d.nos, d_stage_,
                                                        SoA3<double>{ nullptr, nullptr, nullptr } );
    else
        soa_to_aos<float><<<grid, 256, 0, stream_>>>( soa<float>( field_ ), d.spin_offset, d.nos, d_stage_,
                                                       SoA3<float>{ nullptr, nullptr, nullptr } );
    CUDA_CHECK( cudaGetLastError() );
    CUDA_CHECK( cudaMemcpyAsync( h_aos, d_stage_, sizeof( double ) * 3 * d.nos, cudaMemcpyDeviceToHost, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
}

static void trace_mark( std::vector<std::pair<int, cudaEvent_t>> * trace, int id, cudaStream_t st )
{
    if( !trace )
        return;
    cudaEvent_t e;
    CUDA_CHECK( cudaEventCreate( &e ) );
    CUDA_CHECK( cudaEventRecord( e, st ) );
    trace->push_back( { id, e } );
}

template<typename R, int SOLVER, int STAGE>
void Engine::launch_stage_rows( StageArgs<R> a, cudaStream_t st )
{
    trace_mark( trace_, KERNEL_STAGE, st );
    static bool attr = false;
    if( !attr )
    {
        CUDA_CHECK( cudaFuncSetAttribute( llg_stage_rows<R, SOLVER, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          96 * 1024 ) );
        attr = true;
    }
    RowArgs<R> F;
    F.fd  = ddi_.d_fd;
    F.tw  = (const cplx<R> *)ddi_.d_tw;
    F.W1  = (cplx<R> *)ddi_.d_W1;
    F.map = d_rowmap_;
    launch_pdl( llg_stage_rows<R, SOLVER, STAGE>, dim3( n_rowblocks_ ), dim3( 256 ), rows_smem_, st, 1, a, F );
}

template<typename R, int SOLVER, int STAGE>
void Engine::launch_stage( StageArgs<R> a, cudaStream_t st )
{
    if( rows_ && a.h.x )
    {
        launch_stage_rows<R, SOLVER, STAGE>( a, st );
        return;
    }
    trace_mark( trace_, KERNEL_STAGE, st );
    if constexpr( std::is_same<R, float>::value )
    {
        int buf = -1;
        for( int b = 0; b < 3 && tma_; ++b )
        {
            void * const * bb = b == 0 ? spins_ : ( b == 1 ? predA_ : predB_ );
            if( (void *)a.cfg.x == bb[0] && (void *)a.cfg.y == bb[1] && (void *)a.cfg.z == bb[2] )
                buf = b;
        }
        if( buf >= 0 )
        {
            static int grid = 0;
            if( !grid )
            {
                CUDA_CHECK( cudaFuncSetAttribute( llg_stage_tma<SOLVER, STAGE>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_SMEM ) );
                int dev = 0, sms = 0, per = 0;
                CUDA_CHECK( cudaGetDevice( &dev ) );
                CUDA_CHECK( cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev ) );
                CUDA_CHECK( cudaOccupancyMaxActiveBlocksPerMultiprocessor( &per, llg_stage_tma<SOLVER, STAGE>, 256,
                                                                           TT_SMEM ) );
                grid = std::max( 1, sms * std::max( per, 1 ) );
            }
            TileMaps M;
            for( int c = 0; c < 3; ++c )
                M.m[c] = tmaps_[buf][c];
            launch_pdl( llg_stage_tma<SOLVER, STAGE>, dim3( std::min( grid, n_tiles_ ) ), dim3( 256 ), TT_SMEM, st, 1,
                        a, M, (const int4 *)d_tiles_, n_tiles_, d_err_ );
            return;
        }
    }
    const int k = sizeof( R ) == 8 ? 0 : spt_idx_;
    a.blkmap    = d_sblkmap_[k];
    const int n = n_sblocks_[k];
    if( k == 0 )
        launch_pdl( llg_stage<R, SOLVER, STAGE, 1>, dim3( n ), dim3( 256 ), 0, st, 1, a );
    else if( k == 1 )
        launch_pdl( llg_stage<R, SOLVER, STAGE, 2>, dim3( n ), dim3( 256 ), 0, st, 1, a );
    else
        launch_pdl( llg_stage<R, SOLVER, STAGE, 4>, dim3( n ), dim3( 256 ), 0, st, 1, a );
}

template<typename R>
void Engine::launch_probe_t()
{
    StageArgs<R> a{};
    a.sd       = d_desc_;
    a.runs     = d_runs_;
    a.blkmap   = d_blkmap_;
    a.s        = soa<R>( spins_ );
    a.cfg      = a.s;
    a.h        = { nullptr, nullptr, nullptr };
    if( any_ddi_ )
    {
        ddi_.run( d_desc_, d_runs_, spins_[0], spins_[1], spins_[2], field_[0], field_[1], field_[2], stream_ );
        w1_valid_ = false;
        a.h       = soa<R>( field_ );
    }
    // the probe uses the solver's force definition (direct minimisation / dynamics) only
    llg_stage<R, SOLVER_HEUN, ST_PROBE, 1><<<n_blocks_, 256, 0, stream_>>>( a );
    CUDA_CHECK( cudaGetLastError() );
    launch_close( 0, 1 );
}

void Engine::launch_close( int tune, int probe )
{
    const int n = (int)desc_.size();
    if( n == 0 )
        return;
    launch_pdl( close_iteration, dim3( ( n + 127 ) / 128 ), dim3( 128 ), 0, stream_, 1, d_runs_,
                (const SysDesc *)d_desc_, n, tune, probe );
}

// the stage kernels of one step of the current solver; with_ddi: the dipolar field of each
// stage configuration is computed before its stage
template<typename R>
void Engine::launch_stages_t( StageArgs<R> & a, bool with_ddi )
{
    SoA3<R> pA = soa<R>( predA_ ), pB = soa<R>( predB_ );
    auto field = [&]( const SoA3<R> & cfg ) {
        if( with_ddi && any_ddi_ )
            ddi_.run( d_desc_, d_runs_, cfg.x, cfg.y, cfg.z, field_[0], field_[1], field_[2], stream_, rows_ ? 5 : -1 );
    };
    if( !with_ddi && rows_ )
        a.h = { nullptr, nullptr, nullptr }; // timing runs of the tuner: plain stage kernels
    switch( solver_ )
    {
    case SOLVER_SIB:
    case SOLVER_HEUN:
    case SOLVER_DEPONDT:
    {
        a.cfg = a.s;
        a.out = pA;
        field( a.cfg );
        if( solver_ == SOLVER_SIB )
            launch_stage<R, SOLVER_SIB, 1>( a, stream_ );
        else if( solver_ == SOLVER_HEUN )
            launch_stage<R, SOLVER_HEUN, 1>( a, stream_ );
        else
            launch_stage<R, SOLVER_DEPONDT, 1>( a, stream_ );
        a.cfg = pA;
        field( a.cfg );
        if( solver_ == SOLVER_SIB )
            launch_stage<R, SOLVER_SIB, 2>( a, stream_ );
        else if( solver_ == SOLVER_HEUN )
            launch_stage<R, SOLVER_HEUN, 2>( a, stream_ );
        else
            launch_stage<R, SOLVER_DEPONDT, 2>( a, stream_ );
        launch_close( a.tune, 0 );
        break;
    }
    case SOLVER_RK4:
    {
        a.cfg = a.s;
        a.out = pA;
        field( a.cfg );
        launch_stage<R, SOLVER_RK4, 1>( a, stream_ );
        a.cfg = pA;
        a.out = pB;
        field( a.cfg );
        launch_stage<R, SOLVER_RK4, 2>( a, stream_ );
        a.cfg = pB;
        a.out = pA;
        field( a.cfg );
        launch_stage<R, SOLVER_RK4, 3>( a, stream_ );
        a.cfg = pA;
        field( a.cfg );
        launch_stage<R, SOLVER_RK4, 4>( a, stream_ );
        launch_close( a.tune, 0 );
        break;
    }
    default:
        throw std::runtime_error( "solver not supported by the LLG engine" );
    }
    CUDA_CHECK( cudaGetLastError() );
}

template<typename R>
void Engine::launch_step_t()
{
    StageArgs<R> a{};
    a.sd   = d_desc_;
    a.runs = d_runs_;
    a.s    = soa<R>( spins_ );
    a.aux1 = soa<R>( aux1_ );
    a.aux2 = soa<R>( aux2_ );
    a.h    = any_ddi_ ? soa<R>( field_ ) : SoA3<R>{ nullptr, nullptr, nullptr };
    a.xi   = soa<R>( noise_ );
    a.tune = 0;
    if constexpr( std::is_same<R, float>::value )
        a.lo = lo_soa();
    launch_stages_t<R>( a, true );
}

// Stage-kernel autotuner: times the stage kernels of one step of the current solver for 1, 2
// and 4 spins per thread and keeps the fastest.  Runs on scratch buffers (the state is not
// touched) with the run state ignored; the caller resets the run state afterwards.
template<typename R>
void Engine::tune_stages_t()
{
    if( tma_ )
        return; // the TMA-staged kernel has one shape
    StageArgs<R> a{};
    a.sd   = d_desc_;
    a.runs = d_runs_;
    a.s    = soa<R>( predB_ );
    a.aux1 = soa<R>( aux1_ );
    a.aux2 = soa<R>( aux2_ );
    a.h    = any_ddi_ ? soa<R>( field_ ) : SoA3<R>{ nullptr, nullptr, nullptr };
    a.xi   = soa<R>( noise_ );
    a.tune = 1;
    auto * saved = trace_;
    trace_       = nullptr;
    cudaEvent_t e0, e1;
    CUDA_CHECK( cudaEventCreate( &e0 ) );
    CUDA_CHECK( cudaEventCreate( &e1 ) );
    // 1 and 2 spins per thread only: 4 per thread (a quarter of the blocks) times well here, where
    // the stage launches run back to back and overlap, but measured 17 % slower inside the step
    // (128x128x16 Heun, interleaved: 1 -> 0.1033 / 0.1044, 2 -> 0.1030 / 0.1029, 4 -> 0.1207 /
    // 0.1213 ms/step); 2 is kept unless 1 is more than 5 % faster here.
    float best = 1e30f, t_two = 1e30f;
    int bi     = 0;
    for( int k = 0; k < 2; ++k )
    {
        spt_idx_ = k;
        launch_stages_t<R>( a, false );
        float ms = 1e30f;
        for( int trial = 0; trial < 3; ++trial ) // best of three groups of three steps
        {
            CUDA_CHECK( cudaEventRecord( e0, stream_ ) );
            for( int r = 0; r < 3; ++r )
                launch_stages_t<R>( a, false );
            CUDA_CHECK( cudaEventRecord( e1, stream_ ) );
            CUDA_CHECK( cudaEventSynchronize( e1 ) );
            float t = 0;
            CUDA_CHECK( cudaEventElapsedTime( &t, e0, e1 ) );
            ms = std::min( ms, t );
        }
        if( k == 1 )
            t_two = ms;
        if( ms < best )
        {
            best = ms;
            bi   = k;
        }
    }
    if( t_two <= 1.05f * best )
        bi = 1;
    spt_idx_ = bi;
    if( const char * e = std::getenv( "SPIRIT_GB300_SPT" ) ) // override (measurements): 1, 2 or 4
    {
        const int v = std::atoi( e );
        spt_idx_    = v == 1 ? 0 : ( v == 2 ? 1 : ( v == 4 ? 2 : spt_idx_ ) );
    }
    trace_   = saved;
    CUDA_CHECK( cudaEventDestroy( e0 ) );
    CUDA_CHECK( cudaEventDestroy( e1 ) );
}

void Engine::launch_step_kernels()
{
    if( fp64_ )
        launch_step_t<double>();
    else
        launch_step_t<float>();
}

// reads a buffer (so that L2 holds clean, unrelated lines afterwards)
__global__ void l2_read( const uint4 * p, size_t n, unsigned int * sink )
{
    unsigned int acc = 0;
    for( size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x )
    {
        uint4 v = p[i];
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if( acc == 0x9E3779B9u )
        *sink = acc;
}

void Engine::profile_steps( int n, void * flush_buf, size_t flush_bytes, void * read_buf, size_t read_bytes,
                            double * ms, int * count )
{
    std::vector<std::pair<int, cudaEvent_t>> tr;
    ensure_spectrum();
    for( int k = 0; k < n; ++k )
    {
        if( flush_buf && flush_bytes )
            CUDA_CHECK( cudaMemsetAsync( flush_buf, k & 0xff, flush_bytes, stream_ ) );
        if( read_buf && read_bytes >= 16 )
            l2_read<<<1216, 256, 0, stream_>>>( (const uint4 *)read_buf, read_bytes / 16, (unsigned int *)d_red_ );
        tr.clear();
        trace_    = &tr;
        ddi_.trace = &tr;
        launch_step_kernels();
        trace_mark( &tr, KERNEL_END, stream_ );
        trace_     = nullptr;
        ddi_.trace = nullptr;
        CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
        for( size_t e = 0; e + 1 < tr.size(); ++e )
        {
            float t = 0;
            CUDA_CHECK( cudaEventElapsedTime( &t, tr[e].second, tr[e + 1].second ) );
            ms[tr[e].first] += t;
            count[tr[e].first] += 1;
        }
        for( auto & x : tr )
            cudaEventDestroy( x.second );
    }
}

int Engine::tuning( int * out, int n ) const
{
    const int v[14] = { SPT_OPTIONS[fp64_ ? 0 : spt_idx_], ddi_.tile[0], ddi_.threads[0], ddi_.tile[1],
                        ddi_.threads[1], ddi_.tile[2], ddi_.threads[2], ddi_.fused ? 1 : 0,
                        ddi_.cluster_k, ddi_.threads_bc, any_ddi_ ? 1 : 0, rows_ ? 1 : 0, tma_ ? 1 : 0,
                        comp_ ? 1 : 0 };
    for( int k = 0; k < n && k < 14; ++k )
        out[k] = v[k];
    return 14;
}

int Engine::kernels_per_step() const
{
    int stages = solver_ == SOLVER_RK4 ? 4 : 2;
    // per stage: the stage kernel and the dipolar passes; per step: close_iteration
    return stages * ( 1 + ( any_ddi_ ? ( rows_ ? 1 : ( ddi_.fused ? 3 : 5 ) ) : 0 ) ) + 1;
}

void Engine::llg_start( int solver, const std::vector<int> & n_iterations )
{
    if( solver != SOLVER_SIB && solver != SOLVER_HEUN && solver != SOLVER_DEPONDT && solver != SOLVER_RK4 )
        throw std::runtime_error( "solver not supported by the LLG engine" );
    solver_ = solver;
    for( size_t s = 0; s < desc_.size(); ++s )
        desc_[s].n_iterations = n_iterations.size() == 1 ? n_iterations[0] : n_iterations[s];
    CUDA_CHECK( cudaMemcpyAsync( d_desc_, desc_.data(), sizeof( SysDesc ) * desc_.size(), cudaMemcpyHostToDevice,
                                 stream_ ) );
    if( !fp64_ && tuned_solver_ != solver_ )
    {
        tune_stages_t<float>();
        tuned_solver_ = solver_;
    }
    std::vector<SysRun> r( desc_.size() );
    for( auto & x : r )
    {
        std::memset( &x, 0, sizeof( x ) );
        x.active = 1; // the probe runs on every system
    }
    CUDA_CHECK( cudaMemcpyAsync( d_runs_, r.data(), sizeof( SysRun ) * r.size(), cudaMemcpyHostToDevice, stream_ ) );
    if( fp64_ )
        launch_probe_t<double>();
    else
        launch_probe_t<float>();
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
}

void Engine::llg_launch( int n_steps )
{
    // steps are replayed from CUDA graphs of G steps and of one step; steps beyond a system's
    // budget or after its convergence are no-ops on the device
    const int G = 8;
    ensure_spectrum();
    static const bool graphs = [] {
        const char * e = std::getenv( "SPIRIT_GB300_GRAPHS" ); // 0: direct launches (profilers)
        return !( e && e[0] == '0' );
    }();
    if( !graphs )
    {
        for( int k = 0; k < n_steps; ++k )
            launch_step_kernels();
        return;
    }
    if( !graph_ || graph_solver_ != solver_ )
    {
        if( graph_ )
            cudaGraphExecDestroy( graph_ );
        if( graph1_ )
            cudaGraphExecDestroy( graph1_ );
        for( int which = 0; which < 2; ++which )
        {
            cudaGraph_t g;
            CUDA_CHECK( cudaStreamBeginCapture( stream_, cudaStreamCaptureModeThreadLocal ) );
            for( int k = 0; k < ( which == 0 ? G : 1 ); ++k )
                launch_step_kernels();
            CUDA_CHECK( cudaStreamEndCapture( stream_, &g ) );
            CUDA_CHECK( cudaGraphInstantiate( which == 0 ? &graph_ : &graph1_, g, 0 ) );
            cudaGraphDestroy( g );
        }
        graph_solver_ = solver_;
        graph_steps_  = G;
    }
    int full = n_steps / G, rem = n_steps % G;
    for( int k = 0; k < full; ++k )
        CUDA_CHECK( cudaGraphLaunch( graph_, stream_ ) );
    for( int k = 0; k < rem; ++k )
        CUDA_CHECK( cudaGraphLaunch( graph1_, stream_ ) );
}

void Engine::sync()
{
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    if( tma_ )
        check_err();
}

std::vector<Engine::Status> Engine::status()
{
    std::vector<SysRun> r( desc_.size() );
    CUDA_CHECK( cudaMemcpyAsync( r.data(), d_runs_, sizeof( SysRun ) * r.size(), cudaMemcpyDeviceToHost, stream_ ) );
    CUDA_CHECK( cudaStreamSynchronize( stream_ ) );
    if( tma_ )
        check_err();
    std::vector<Status> out( r.size() );
    for( size_t s = 0; s < r.size(); ++s )
        out[s] = { r[s].iteration, r[s].active, r[s].max_torque, r[s].energy };
    return out;
}

} // namespace sg
