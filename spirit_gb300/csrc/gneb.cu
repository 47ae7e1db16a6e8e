// GNEB with the velocity-projection solver on a batch of images, and LLG with VP on one image.
//
// All images of the chain are one device batch (same geometry, SoA, 128-byte aligned).  One
// iteration is five launches:
//   K1 eval     gradient force G = -grad E at every spin, FP64 image energy, and the squared
//               geodesic angle to the previous image (Method_GNEB.cpp:95-128, Manifoldmath.cpp:66-72)
//   K2 scalars  one block: Rx, energy-weighted tangent coefficients (Manifoldmath.cpp:115-215),
//               spring coefficients k (Rx+ - 2 Rx + Rx-) (Method_GNEB.cpp:230-240)
//   K3 tangent  tangents (geodesic at the end points), P_perp of tangents and gradient forces,
//               per-image |t|^2 and F.t reductions
//   K4 force    climbing / falling / normal total force (Method_GNEB.cpp:176-256) and the VP
//               velocity update with chain-global v.F and F.F reductions (Solver_VP.hpp:55-80)
//   K5 update   VP projection and step, max torque per image (Hook_Post_Iteration 411-430) and the
//               in-place projection of the stored forces; the last block finalises the iteration
// Reductions are FP64 atomics of per-block partial sums.  The iteration counter and the
// convergence flag live on the device, so iterations replay from a CUDA graph.
//
// The exponential-transform minimisers replace K4/K5 (orthogonal spin optimisation,
// Solver_VP_OSO.hpp, Solver_LBFGS_OSO.hpp).  The reference writes them in permuted coordinates
// (g = T(-s x f) with the signed permutation T of oso_calc_gradients, Solver_Kernels.cpp:50-60,
// and the matching rotation matrix of oso_rotate, :62-95); T is orthogonal and applied to every
// vector alike, so here they run in physical coordinates: the search direction is the rotation
// vector itself and dot products are unchanged.
//   VP_OSO     K4' torque g = s x F, v += (g_prev + g)/2m, chain-global v.g and g.g;
//              K5' v = (v.g / g.g) g or 0, rotate s by dt v + dt g/2m
//   LBFGS_OSO  K4' gradient -(s x F), new difference dg[m], and the per-image Gram matrix of the
//              7 vectors {grad, da[0..2], dg[0..2]};
//              K6  one thread: the two-loop recursion of lbfgs_get_searchdir
//              (Solver_Kernels.hpp:44-189) on coefficients over those 7 vectors (every dot product
//              it needs is a Gram entry), and the rms-angle limit (maximum_rotation, :97-105)
//              from the per-image Grams;
//              K5' sd = sum c_j b_j, kept as the next da, rotate s by sd
// so one L-BFGS iteration reads the memory twice instead of once per recursion step.
#include "gneb.hpp"
#include "kernels.cuh"
#include "util.hpp"

#include <cmath>
#include <chrono>
#include <cstring>
#include <fstream>
#include <type_traits>

namespace sg
{

struct GnebImage
{
    double E, dist2, tt, ft;
    double cp, cm, spring, Rx;
    unsigned int torque_bits;
    int type;
    float torque;
    int pad;
};

struct GnebCtl
{
    int iteration, active, n_iterations, mode; // mode 0: GNEB, 1: LLG direct minimisation (single image)
    int noi, nos, aborted, solver;             // solver: SOLVER_VP, SOLVER_LBFGS_OSO, SOLVER_VP_OSO
    double force_convergence, m, proj, fn2;
    double hm; // 0.5 / m
    float max_torque;
    unsigned int blocks_done;
    unsigned int torque_bits;
    int fv_unit; // LLG virtual force s x F without the dt gamma / mu_B factor (LBFGS_OSO)
    // L-BFGS memory (3 pairs) and the coefficients of this iteration's search direction
    int local_iter, lb_store, pad3[2];
    double eps, maxmove;
    double rho[3], alpha[3], coef[7];
};

constexpr int LB_MEM  = 3;
constexpr int LB_VEC  = 1 + 2 * LB_MEM;                // grad, da[0..2], dg[0..2]
constexpr int LB_GRAM = LB_VEC * ( LB_VEC + 1 ) / 2;  // upper triangle

template<typename R>
struct GArgs
{
    const SysDesc * sd;
    const int2 * blkmap;
    int nblocks;
    SoA3<R> s, F, V, T, G, h;
    SoA3<R> Gb, DA[LB_MEM], DG[LB_MEM]; // L-BFGS: gradient, step and gradient-difference memory
    double * gram;                       // L-BFGS: per-image Gram matrices [noi][LB_GRAM]
    GnebImage * img;
    GnebCtl * ctl;
    double spring_constant;
};

template<typename R>
__device__ __forceinline__ void load_pairs( PairR<R> * pairs, SysConst<R> & C, Geo & G, const SysDesc & d )
{
    load_pairs_smem( pairs, d );
    load_const( C, d );
    load_geo( G, d );
    __syncthreads();
}

// K1 (and the LLG-VP probe when probe = 1)
template<typename R>
__global__ void __launch_bounds__( 256 ) gneb_eval( GArgs<R> A, int probe )
{
    __shared__ PairR<R> pairs[MAX_PAIRS];
    __shared__ SysConst<R> C;
    __shared__ Geo GS;
    __shared__ double red[32];
    if( !A.ctl->active )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const SysDesc & d = A.sd[im];
    load_pairs( pairs, C, GS, d );
    const int i = bm.y + threadIdx.x;
    R e         = 0;
    double a2   = 0;
    int ib, a, b, c;
    cell_of( GS, i < d.nos ? i : 0, ib, a, b, c );
    const int smode = warp_stencil_mode( GS, a, b, c, i < d.nos );
    if( i < d.nos )
    {
        const long long gi = GS.off + i;
        const R mu     = C.mu[ib];
        const V3<R> si = A.s.ld( gi );
        V3<R> g        = gradient_at<R>( GS, C, pairs, A.s, A.h, gi, ib, a, b, c, si, mu, e, smode );
        V3<R> f        = { -g.x, -g.y, -g.z };
        A.G.st( gi, f );
        if( A.ctl->mode == 0 && im > 0 )
        {
            const V3<R> sp = A.s.ld( A.sd[im - 1].spin_offset + i );
            double r       = (double)si.x * sp.x + (double)si.y * sp.y + (double)si.z * sp.z;
            r              = fmax( -1.0, fmin( 1.0, r ) );
            double ang     = acos( r );
            a2             = ang * ang;
        }
        if( A.ctl->mode == 1 )
        {
            // direct minimisation: virtual force fv = dt gamma/mu_B (s x F) (VP, VP_OSO) or s x F
            // (LBFGS_OSO; Method_LLG.cpp:161-168), kept in T for the torque
            R k      = A.ctl->fv_unit ? R( 1 ) : C.kdm;
            V3<R> cr = cross( si, f );
            V3<R> fv = { k * cr.x, k * cr.y, k * cr.z };
            A.T.st( gi, fv );
            if( probe )
            {
                // constructor: initial forces projected onto the tangent planes (Hook_Post_Iteration);
                // VP reuses them as its previous forces, the OSO solvers start from zero
                if( A.ctl->solver == SOLVER_VP )
                {
                    R dd = dot( f, si );
                    A.F.st( gi, V3<R>{ f.x - dd * si.x, f.y - dd * si.y, f.z - dd * si.z } );
                }
                float t2 = (float)torque2( fv, si );
                atomicMax( &A.img[im].torque_bits, __float_as_uint( t2 ) );
            }
        }
    }
    double es = block_sum( (double)e, red );
    double ds = block_sum( a2, red );
    if( threadIdx.x == 0 )
    {
        atomicAdd( &A.img[im].E, es );
        if( ds != 0 )
            atomicAdd( &A.img[im].dist2, ds );
    }
}

// K2: chain scalars (one thread)
__global__ void gneb_scalars( GnebImage * img, GnebCtl * ctl, double spring_constant )
{
    if( threadIdx.x != 0 || blockIdx.x != 0 || !ctl->active )
        return;
    const int noi = ctl->noi;
    img[0].Rx     = 0;
    for( int k = 1; k < noi; ++k )
    {
        img[k].Rx = img[k - 1].Rx + sqrt( img[k].dist2 );
        if( img[k].Rx - img[k - 1].Rx < 1e-10 )
            ctl->aborted = 1; // "The geodesic distance between two images is zero! Stopping..."
    }
    for( int k = 1; k < noi - 1; ++k )
    {
        double Em = img[k].E, Ep = img[k + 1].E, En = img[k - 1].E;
        double cp = 0, cm = 0;
        if( ( Ep < Em && Em > En ) || ( Ep > Em && Em < En ) )
        {
            double Emax = fmax( fabs( Ep - Em ), fabs( En - Em ) );
            double Emin = fmin( fabs( Ep - Em ), fabs( En - Em ) );
            if( Ep > En )
            {
                cp = Emax;
                cm = Emin;
            }
            else
            {
                cp = Emin;
                cm = Emax;
            }
        }
        else if( Ep > Em && Em > En )
            cp = 1;
        else if( Ep < Em && Em < En )
            cm = 1;
        else
        {
            cp = 1;
            cm = 1;
        }
        img[k].cp     = cp;
        img[k].cm     = cm;
        img[k].spring = spring_constant * ( img[k + 1].Rx - 2 * img[k].Rx + img[k - 1].Rx );
    }
    ctl->proj = 0;
    ctl->fn2  = 0;
}

// K3: tangents, projected gradient force, |t|^2 and F.t per image
template<typename R>
__global__ void __launch_bounds__( 256 ) gneb_tangent( GArgs<R> A )
{
    __shared__ double red[32];
    if( !A.ctl->active || A.ctl->aborted )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const int noi     = A.ctl->noi;
    const SysDesc & d = A.sd[im];
    const int i       = bm.y + threadIdx.x;
    double tt = 0, ft = 0;
    if( i < d.nos )
    {
        const long long gi = d.spin_offset + i;
        const V3<R> si     = A.s.ld( gi );
        V3<R> t;
        if( im == 0 || im == noi - 1 )
        {
            // Geodesic_Tangent (Manifoldmath.cpp:78-113): minus/plus images and the mid (= this) image
            V3<R> mn = im == 0 ? si : A.s.ld( A.sd[im - 1].spin_offset + i );
            V3<R> pl = im == 0 ? A.s.ld( A.sd[im + 1].spin_offset + i ) : si;
            V3<R> ax = cross( pl, mn );
            if( fabs( (double)dot( mn, pl ) + 1.0 ) < 1e-15 )
            {
                if( fabs( (double)si.x - 1.0 ) > 1e-15 )
                    ax = { 1, 0, 0 };
                else
                    ax = { 0, 1, 0 };
            }
            t = cross( si, ax );
        }
        else
        {
            const V3<R> sp = A.s.ld( A.sd[im + 1].spin_offset + i );
            const V3<R> sm = A.s.ld( A.sd[im - 1].spin_offset + i );
            V3<R> tp       = { sp.x - si.x, sp.y - si.y, sp.z - si.z };
            V3<R> tm       = { si.x - sm.x, si.y - sm.y, si.z - sm.z };
            R cp = (R)A.img[im].cp, cm = (R)A.img[im].cm;
            if( cp != R( 0 ) && cm != R( 0 ) )
                t = { cp * tp.x + cm * tm.x, cp * tp.y + cm * tm.y, cp * tp.z + cm * tm.z };
            else if( cp != R( 0 ) )
                t = { cp * tp.x, cp * tp.y, cp * tp.z };
            else
                t = { cm * tm.x, cm * tm.y, cm * tm.z };
            R dd = dot( t, si );
            t    = { t.x - dd * si.x, t.y - dd * si.y, t.z - dd * si.z };
            // P_perp of the gradient force (project_tangential(F_gradient, image))
            V3<R> f = A.G.ld( gi );
            R df    = dot( f, si );
            f       = { f.x - df * si.x, f.y - df * si.y, f.z - df * si.z };
            A.G.st( gi, f );
            ft = (double)f.x * t.x + (double)f.y * t.y + (double)f.z * t.z;
        }
        A.T.st( gi, t );
        tt = (double)t.x * t.x + (double)t.y * t.y + (double)t.z * t.z;
    }
    double a = block_sum( tt, red );
    double b = block_sum( ft, red );
    if( threadIdx.x == 0 )
    {
        atomicAdd( &A.img[im].tt, a );
        if( b != 0 )
            atomicAdd( &A.img[im].ft, b );
    }
}

// K4: total force and VP velocity (v += 0.5/m (F_prev + F)), global v.F and F.F
template<typename R>
__global__ void __launch_bounds__( 256 ) gneb_force( GArgs<R> A )
{
    __shared__ double red[32];
    if( !A.ctl->active || A.ctl->aborted )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const int noi     = A.ctl->noi;
    const SysDesc & d = A.sd[im];
    const int i       = bm.y + threadIdx.x;
    double vf = 0, ff = 0;
    if( i < d.nos )
    {
        const long long gi = d.spin_offset + i;
        V3<R> fnew         = { 0, 0, 0 };
        if( A.ctl->mode == 1 )
            fnew = A.G.ld( gi );
        else if( im > 0 && im < noi - 1 )
        {
            const GnebImage & I = A.img[im];
            const R inv         = R( 1 ) / sqrt( (R)I.tt );
            V3<R> t             = A.T.ld( gi );
            t                   = { t.x * inv, t.y * inv, t.z * inv };
            R ftn               = (R)I.ft * inv;
            V3<R> f             = A.G.ld( gi );
            if( I.type == 1 ) // climbing: invert the parallel component, no spring
                fnew = { f.x - R( 2 ) * ftn * t.x, f.y - R( 2 ) * ftn * t.y, f.z - R( 2 ) * ftn * t.z };
            else if( I.type == 2 ) // falling: no spring
                fnew = f;
            else if( I.type == 0 ) // normal: orthogonal gradient force + spring along the tangent
            {
                R sp = (R)I.spring;
                fnew = { f.x - ftn * t.x, f.y - ftn * t.y, f.z - ftn * t.z };
                fnew.x += sp * t.x;
                fnew.y += sp * t.y;
                fnew.z += sp * t.z;
            }
        }
        const V3<R> fp = A.F.ld( gi );
        V3<R> v        = A.V.ld( gi );
        const R hm     = (R)A.ctl->hm;
        v.x += hm * ( fp.x + fnew.x );
        v.y += hm * ( fp.y + fnew.y );
        v.z += hm * ( fp.z + fnew.z );
        A.V.st( gi, v );
        A.F.st( gi, fnew );
        vf = (double)v.x * fnew.x + (double)v.y * fnew.y + (double)v.z * fnew.z;
        ff = (double)fnew.x * fnew.x + (double)fnew.y * fnew.y + (double)fnew.z * fnew.z;
    }
    double a = block_sum( vf, red );
    double b = block_sum( ff, red );
    if( threadIdx.x == 0 )
    {
        atomicAdd( &A.ctl->proj, a );
        atomicAdd( &A.ctl->fn2, b );
    }
}

// last block of an iteration: per-image and maximum torques, iteration counter, convergence
template<typename R>
__device__ void finish_iteration( const GArgs<R> & A )
{
    __threadfence();
    volatile GnebCtl * vc   = A.ctl;
    volatile GnebImage * vi = A.img;
    float mt                = 0;
    for( int k = 0; k < vc->noi; ++k )
    {
        float tk          = sqrtf( __uint_as_float( vi[k].torque_bits ) );
        vi[k].torque      = tk;
        vi[k].torque_bits = 0;
        mt                = fmaxf( mt, tk );
    }
    vc->blocks_done = 0;
    if( vc->aborted )
    {
        vc->active = 0;
        return;
    }
    vc->max_torque = mt;
    int it         = vc->iteration + 1;
    vc->iteration  = it;
    vc->active     = ( it < vc->n_iterations ) && !( mt < (float)vc->force_convergence );
}

// K5: VP step, torques, projection of the stored forces, finalisation
template<typename R>
__global__ void __launch_bounds__( 256 ) gneb_update( GArgs<R> A )
{
    __shared__ float red[32];
    __shared__ int is_last;
    GnebCtl * ctl = A.ctl;
    if( !ctl->active )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const SysDesc & d = A.sd[im];
    const int i       = bm.y + threadIdx.x;
    float t2          = 0;
    const bool abort  = ctl->aborted != 0;
    if( i < d.nos && !abort )
    {
        const long long gi = d.spin_offset + i;
        V3<R> f            = A.F.ld( gi );
        V3<R> v;
        if( ctl->proj <= 0 )
            v = { 0, 0, 0 };
        else
        {
            R ratio = (R)ctl->proj / (R)ctl->fn2;
            v       = { f.x * ratio, f.y * ratio, f.z * ratio };
        }
        A.V.st( gi, v );
        const R dt   = sys_const<R>( d ).dt;
        const R hmdt = (R)ctl->hm * dt;
        V3<R> s      = A.s.ld( gi );
        V3<R> c      = { s.x + dt * v.x + hmdt * f.x, s.y + dt * v.y + hmdt * f.y, s.z + dt * v.z + hmdt * f.z };
        V3<R> sn     = normalized( c );
        A.s.st( gi, sn );
        // max torque: GNEB |P_perp F_total|, LLG-VP |P_perp fv| with fv from the force evaluation
        if( ctl->mode == 1 )
            t2 = (float)torque2( A.T.ld( gi ), sn );
        else
            t2 = (float)torque2( f, sn );
        R dd = dot( f, sn );
        A.F.st( gi, V3<R>{ f.x - dd * sn.x, f.y - dd * sn.y, f.z - dd * sn.z } );
    }
    float tm = block_max( t2, red );
    if( threadIdx.x == 0 )
    {
        atomicMax( &A.img[im].torque_bits, __float_as_uint( tm ) );
        __threadfence();
        unsigned int prev = atomicAdd( &ctl->blocks_done, 1u );
        is_last           = ( prev == (unsigned int)A.nblocks - 1 );
    }
    __syncthreads();
    if( is_last && threadIdx.x == 0 )
        finish_iteration( A );
}

// total force of an image's spin for the minimisers: GNEB climbing / falling / normal force
// (Method_GNEB.cpp:176-256; zero at the end points), LLG the gradient force
template<typename R>
__device__ __forceinline__ V3<R> total_force( const GArgs<R> & A, int im, long long gi )
{
    V3<R> fnew    = { 0, 0, 0 };
    const int noi = A.ctl->noi;
    if( A.ctl->mode == 1 )
        fnew = A.G.ld( gi );
    else if( im > 0 && im < noi - 1 )
    {
        const GnebImage & I = A.img[im];
        const R inv         = R( 1 ) / sqrt( (R)I.tt );
        V3<R> t             = A.T.ld( gi );
        t                   = { t.x * inv, t.y * inv, t.z * inv };
        R ftn               = (R)I.ft * inv;
        V3<R> f             = A.G.ld( gi );
        if( I.type == 1 )
            fnew = { f.x - R( 2 ) * ftn * t.x, f.y - R( 2 ) * ftn * t.y, f.z - R( 2 ) * ftn * t.z };
        else if( I.type == 2 )
            fnew = f;
        else if( I.type == 0 )
        {
            R sp = (R)I.spring;
            fnew = { f.x - ftn * t.x, f.y - ftn * t.y, f.z - ftn * t.z };
            fnew.x += sp * t.x;
            fnew.y += sp * t.y;
            fnew.z += sp * t.z;
        }
    }
    return fnew;
}

// K4' (VP_OSO, LBFGS_OSO)
template<typename R>
__global__ void __launch_bounds__( 256 ) oso_force( GArgs<R> A )
{
    __shared__ double red[8 * LB_GRAM];
    __shared__ double red1[32];
    GnebCtl * ctl = A.ctl;
    if( !ctl->active || ctl->aborted )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const SysDesc & d = A.sd[im];
    const int i       = bm.y + threadIdx.x;
    const bool lbfgs  = ctl->solver == SOLVER_LBFGS_OSO;
    double vf = 0, ff = 0;
    double b[LB_VEC][3];
#pragma unroll
    for( int k = 0; k < LB_VEC; ++k )
        b[k][0] = b[k][1] = b[k][2] = 0;
    if( i < d.nos )
    {
        const long long gi = d.spin_offset + i;
        const V3<R> fnew   = total_force( A, im, gi );
        if( ctl->mode == 0 )
            A.T.st( gi, fnew ); // F_total, for the torque after the step
        const V3<R> c = cross( A.s.ld( gi ), fnew );
        if( !lbfgs )
        {
            const V3<R> gp = A.F.ld( gi );
            V3<R> v        = A.V.ld( gi );
            const R hm     = (R)ctl->hm;
            v.x += hm * ( gp.x + c.x );
            v.y += hm * ( gp.y + c.y );
            v.z += hm * ( gp.z + c.z );
            A.V.st( gi, v );
            A.F.st( gi, c );
            vf = (double)v.x * c.x + (double)v.y * c.y + (double)v.z * c.z;
            ff = (double)c.x * c.x + (double)c.y * c.y + (double)c.z * c.z;
        }
        else
        {
            const V3<R> gr = { -c.x, -c.y, -c.z };
            const int m    = ctl->local_iter % LB_MEM;
            const bool upd = ctl->local_iter > 0;
            V3<R> dgm      = { 0, 0, 0 };
            if( upd )
            {
                // dg[m] = grad - grad_prev; da[m] already holds the previous step
                const V3<R> go = A.Gb.ld( gi );
                dgm            = { gr.x - go.x, gr.y - go.y, gr.z - go.z };
                A.DG[m].st( gi, dgm );
            }
            A.Gb.st( gi, gr );
            b[0][0] = gr.x;
            b[0][1] = gr.y;
            b[0][2] = gr.z;
#pragma unroll
            for( int k = 0; k < LB_MEM; ++k )
            {
                const V3<R> a = A.DA[k].ld( gi );
                const V3<R> g = ( upd && k == m ) ? dgm : A.DG[k].ld( gi );
                b[1 + k][0] = a.x;
                b[1 + k][1] = a.y;
                b[1 + k][2] = a.z;
                b[4 + k][0] = g.x;
                b[4 + k][1] = g.y;
                b[4 + k][2] = g.z;
            }
        }
    }
    if( !lbfgs )
    {
        double a  = block_sum( vf, red1 );
        double bb = block_sum( ff, red1 );
        if( threadIdx.x == 0 )
        {
            atomicAdd( &ctl->proj, a );
            atomicAdd( &ctl->fn2, bb );
        }
        return;
    }
    // per-block Gram partial sums (warp shuffles, then across the warps)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int k = 0;
#pragma unroll
    for( int p = 0; p < LB_VEC; ++p )
#pragma unroll
        for( int q = p; q < LB_VEC; ++q )
        {
            double x = b[p][0] * b[q][0] + b[p][1] * b[q][1] + b[p][2] * b[q][2];
#pragma unroll
            for( int o = 16; o > 0; o >>= 1 )
                x += __shfl_xor_sync( 0xffffffffu, x, o );
            if( lane == 0 )
                red[w * LB_GRAM + k] = x;
            ++k;
        }
    __syncthreads();
    if( threadIdx.x < LB_GRAM )
    {
        double t = 0;
        for( int j = 0; j < (int)( blockDim.x >> 5 ); ++j )
            t += red[j * LB_GRAM + threadIdx.x];
        if( t != 0 )
            atomicAdd( &A.gram[(size_t)im * LB_GRAM + threadIdx.x], t );
    }
}

// K6 (LBFGS_OSO): search-direction coefficients over {grad, da[0..2], dg[0..2]} -- one thread
__global__ void lbfgs_dir( GnebCtl * ctl, const double * gram )
{
    if( threadIdx.x != 0 || blockIdx.x != 0 || !ctl->active || ctl->aborted )
        return;
    const int noi = ctl->noi;
    double G[LB_VEC][LB_VEC];
    for( int p = 0; p < LB_VEC; ++p )
        for( int q = 0; q < LB_VEC; ++q )
            G[p][q] = 0;
    for( int im = 0; im < noi; ++im )
    {
        int k = 0;
        for( int p = 0; p < LB_VEC; ++p )
            for( int q = p; q < LB_VEC; ++q, ++k )
                G[p][q] += gram[(size_t)im * LB_GRAM + k];
    }
    for( int p = 0; p < LB_VEC; ++p )
        for( int q = 0; q < p; ++q )
            G[p][q] = G[q][p];
    const double eps = ctl->eps;
    int li           = ctl->local_iter;
    const int m      = li % LB_MEM;
    double sc[LB_VEC] = { 0, 0, 0, 0, 0, 0, 0 };
    bool gd           = li == 0;
    if( !gd )
    {
        const double rinv = G[4 + m][1 + m]; // dg[m] . da[m]
        if( rinv > eps )
            ctl->rho[m] = 1.0 / rinv;
        else
            gd = true; // restart from steepest descent
    }
    if( gd )
    {
        for( int k = 0; k < LB_MEM; ++k )
            ctl->rho[k] = 0;
        sc[0] = -1;
        li    = 1;
    }
    else
    {
        double qc[LB_VEC] = { 1, 0, 0, 0, 0, 0, 0 };
        for( int k = LB_MEM - 1; k > -1; --k )
        {
            const int c = ( k + m + 1 ) % LB_MEM;
            double x    = 0;
            for( int j = 0; j < LB_VEC; ++j )
                x += qc[j] * G[1 + c][j];
            const double a = ctl->rho[c] * x;
            ctl->alpha[c]  = a;
            qc[4 + c] -= a;
        }
        const double rhody2 = G[4 + m][4 + m] * ctl->rho[m];
        const double inv    = rhody2 > eps ? 1.0 / rhody2 : 1.0 / eps;
        for( int j = 0; j < LB_VEC; ++j )
            sc[j] = inv * qc[j];
        for( int k = 0; k < LB_MEM; ++k )
        {
            const int c = li < LB_MEM ? k : ( k + m + 1 ) % LB_MEM;
            double x    = 0;
            for( int j = 0; j < LB_VEC; ++j )
                x += sc[j] * G[4 + c][j];
            sc[1 + c] += ctl->alpha[c] - ctl->rho[c] * x;
        }
        for( int j = 0; j < LB_VEC; ++j )
            sc[j] = -sc[j];
        ++li;
    }
    // rms rotation angle of every image, limited to maxmove
    double scaling = 1;
    for( int im = 0; im < noi; ++im )
    {
        double th2 = 0;
        int k      = 0;
        for( int p = 0; p < LB_VEC; ++p )
            for( int q = p; q < LB_VEC; ++q, ++k )
                th2 += ( p == q ? 1.0 : 2.0 ) * sc[p] * sc[q] * gram[(size_t)im * LB_GRAM + k];
        const double th = sqrt( fmax( th2, 0.0 ) / ctl->nos );
        const double f  = th > ctl->maxmove ? ctl->maxmove / th : 1.0;
        scaling         = fmin( f, scaling );
    }
    for( int j = 0; j < LB_VEC; ++j )
        ctl->coef[j] = scaling * sc[j];
    ctl->local_iter = li;
    ctl->lb_store   = li % LB_MEM;
}

// rotation of s about the vector sd by |sd| (Rodrigues); no-op below 1e-20 (oso_rotate).  A
// rotation keeps |s| = 1 in exact arithmetic; in FP32 the rounding of the update (relative 6e-8
// per step) makes |s| drift over 1e5 iterations enough to move a saddle energy by 1e-2 meV, so
// the FP32 result is renormalised.  FP64 keeps the reference's arithmetic (no renormalisation).
template<typename R>
__device__ __forceinline__ V3<R> rotate_by( V3<R> s, V3<R> sd )
{
    const R th = sqrt( dot( sd, sd ) );
    if( !( th > R( 1e-20 ) ) )
        return s;
    const R inv = R( 1 ) / th;
    const V3<R> u = { sd.x * inv, sd.y * inv, sd.z * inv };
    R sn, cs;
    if constexpr( std::is_same<R, float>::value )
        sincosf( th, &sn, &cs );
    else
        sincos( th, &sn, &cs );
    const V3<R> x = cross( u, s );
    const R ud    = dot( u, s ) * ( R( 1 ) - cs );
    const V3<R> r = { s.x * cs + x.x * sn + u.x * ud, s.y * cs + x.y * sn + u.y * ud, s.z * cs + x.z * sn + u.z * ud };
    if constexpr( std::is_same<R, float>::value )
        return normalized( r );
    else
        return r;
}

// K5' (VP_OSO, LBFGS_OSO): step, rotation, torques, finalisation
template<typename R>
__global__ void __launch_bounds__( 256 ) oso_update( GArgs<R> A )
{
    __shared__ float red[32];
    __shared__ int is_last;
    GnebCtl * ctl = A.ctl;
    if( !ctl->active )
        return;
    const int2 bm     = A.blkmap[blockIdx.x];
    const int im      = bm.x;
    const SysDesc & d = A.sd[im];
    const int i       = bm.y + threadIdx.x;
    float t2          = 0;
    const bool abort  = ctl->aborted != 0;
    if( i < d.nos && !abort )
    {
        const long long gi = d.spin_offset + i;
        V3<R> sd;
        if( ctl->solver == SOLVER_VP_OSO )
        {
            const V3<R> g = A.F.ld( gi );
            V3<R> v;
            if( ctl->proj <= 0 )
                v = { 0, 0, 0 };
            else
            {
                const R ratio = (R)( ctl->proj / ctl->fn2 );
                v             = { g.x * ratio, g.y * ratio, g.z * ratio };
            }
            A.V.st( gi, v );
            const R dt   = sys_const<R>( d ).dt;
            const R hmdt = (R)ctl->hm * dt;
            sd           = { dt * v.x + hmdt * g.x, dt * v.y + hmdt * g.y, dt * v.z + hmdt * g.z };
        }
        else
        {
            R c[LB_VEC];
#pragma unroll
            for( int j = 0; j < LB_VEC; ++j )
                c[j] = (R)ctl->coef[j];
            const V3<R> g = A.Gb.ld( gi );
            sd            = { c[0] * g.x, c[0] * g.y, c[0] * g.z };
#pragma unroll
            for( int k = 0; k < LB_MEM; ++k )
            {
                const V3<R> a = A.DA[k].ld( gi );
                const V3<R> e = A.DG[k].ld( gi );
                sd.x += c[1 + k] * a.x + c[4 + k] * e.x;
                sd.y += c[1 + k] * a.y + c[4 + k] * e.y;
                sd.z += c[1 + k] * a.z + c[4 + k] * e.z;
            }
            A.DA[ctl->lb_store].st( gi, sd ); // the step becomes the next da
        }
        const V3<R> sn = rotate_by( A.s.ld( gi ), sd );
        A.s.st( gi, sn );
        // max torque: GNEB |P_perp F_total|, LLG |P_perp fv| (both kept in T)
        t2 = (float)torque2( A.T.ld( gi ), sn );
    }
    float tm = block_max( t2, red );
    if( threadIdx.x == 0 )
    {
        atomicMax( &A.img[im].torque_bits, __float_as_uint( tm ) );
        __threadfence();
        unsigned int prev = atomicAdd( &ctl->blocks_done, 1u );
        is_last           = ( prev == (unsigned int)A.nblocks - 1 );
    }
    __syncthreads();
    if( is_last && threadIdx.x == 0 )
        finish_iteration( A );
}

// clear the per-iteration accumulators (E, dist2, tt, ft; the L-BFGS Grams) -- one block
__global__ void gneb_clear( GnebImage * img, GnebCtl * ctl, double * gram )
{
    if( !ctl->active )
        return;
    for( int k = threadIdx.x; k < ctl->noi; k += blockDim.x )
    {
        img[k].E     = 0;
        img[k].dist2 = 0;
        img[k].tt    = 0;
        img[k].ft    = 0;
    }
    if( gram )
        for( int k = threadIdx.x; k < ctl->noi * LB_GRAM; k += blockDim.x )
            gram[k] = 0;
}

// LLG-VP has no chain scalars; only the global sums are reset
__global__ void gneb_scalars_vp( GnebCtl * ctl )
{
    if( threadIdx.x == 0 && ctl->active )
    {
        ctl->proj = 0;
        ctl->fn2  = 0;
    }
}

// LLG-VP probe finalisation: initial max torque and convergence flag
__global__ void vp_probe_finish( GnebImage * img, GnebCtl * ctl )
{
    float t            = sqrtf( __uint_as_float( img[0].torque_bits ) );
    img[0].torque_bits = 0;
    img[0].torque      = t;
    ctl->max_torque    = t;
    ctl->active        = ( 0 < ctl->n_iterations ) && !( t < (float)ctl->force_convergence );
}

// =================================================================== host driver
class GnebRun
{
public:
    GnebRun( const std::vector<Image *> & images, bool fp64, int mode, int solver ) : mode_( mode ), solver_( solver )
    {
        std::vector<SystemInput> in;
        for( auto * im : images )
        {
            SystemInput s;
            s.geom    = im->geom.get();
            s.ham     = &im->ham;
            s.dt      = im->llg.dt;
            s.damping = im->llg.damping;
            in.push_back( s );
        }
        eng   = std::make_unique<Engine>( in, fp64 );
        noi   = (int)images.size();
        size_t el = fp64 ? sizeof( double ) : sizeof( float );
        for( int c = 0; c < 3; ++c )
        {
            F[c] = dalloc_bytes( eng->total_spins() * el );
            V[c] = dalloc_bytes( eng->total_spins() * el );
            T[c] = dalloc_bytes( eng->total_spins() * el );
            G[c] = dalloc_bytes( eng->total_spins() * el );
        }
        d_img = dalloc<GnebImage>( noi );
        d_ctl = dalloc<GnebCtl>( 1 );
        if( solver_ == SOLVER_LBFGS_OSO )
        {
            for( int c = 0; c < 3; ++c )
            {
                Gb[c] = dalloc_bytes( eng->total_spins() * el );
                for( int k = 0; k < LB_MEM; ++k )
                {
                    DA[k][c] = dalloc_bytes( eng->total_spins() * el );
                    DG[k][c] = dalloc_bytes( eng->total_spins() * el );
                }
            }
            d_gram = dalloc<double>( (size_t)noi * LB_GRAM );
        }
    }
    ~GnebRun()
    {
        if( graph )
            cudaGraphExecDestroy( graph );
        for( int c = 0; c < 3; ++c )
        {
            dfree( F[c] );
            dfree( V[c] );
            dfree( T[c] );
            dfree( G[c] );
        }
        dfree( d_img );
        dfree( d_ctl );
        if( d_gram )
        {
            for( int c = 0; c < 3; ++c )
            {
                dfree( Gb[c] );
                for( int k = 0; k < LB_MEM; ++k )
                {
                    dfree( DA[k][c] );
                    dfree( DG[k][c] );
                }
            }
            dfree( d_gram );
        }
    }

    template<typename R>
    GArgs<R> args() const
    {
        GArgs<R> a{};
        a.sd      = eng->d_desc();
        a.blkmap  = eng->d_blkmap();
        a.nblocks = eng->n_blocks();
        a.s       = { (R *)eng->spin_ptr( 0 ), (R *)eng->spin_ptr( 1 ), (R *)eng->spin_ptr( 2 ) };
        a.F       = { (R *)F[0], (R *)F[1], (R *)F[2] };
        a.V       = { (R *)V[0], (R *)V[1], (R *)V[2] };
        a.T       = { (R *)T[0], (R *)T[1], (R *)T[2] };
        a.G       = { (R *)G[0], (R *)G[1], (R *)G[2] };
        a.h       = eng->has_ddi() ? SoA3<R>{ (R *)eng->field_ptr( 0 ), (R *)eng->field_ptr( 1 ),
                                            (R *)eng->field_ptr( 2 ) }
                                   : SoA3<R>{ nullptr, nullptr, nullptr };
        if( d_gram )
        {
            a.Gb = { (R *)Gb[0], (R *)Gb[1], (R *)Gb[2] };
            for( int k = 0; k < LB_MEM; ++k )
            {
                a.DA[k] = { (R *)DA[k][0], (R *)DA[k][1], (R *)DA[k][2] };
                a.DG[k] = { (R *)DG[k][0], (R *)DG[k][1], (R *)DG[k][2] };
            }
        }
        a.gram    = d_gram;
        a.img     = d_img;
        a.ctl     = d_ctl;
        a.spring_constant = spring;
        return a;
    }

    void start( const std::vector<int> & types, int n_iterations, double conv, double spring_k )
    {
        spring = spring_k;
        std::vector<GnebImage> im( noi );
        std::memset( im.data(), 0, sizeof( GnebImage ) * noi );
        for( int k = 0; k < noi; ++k )
            im[k].type = types.empty() ? 0 : types[k];
        h2d( d_img, im.data(), noi );
        GnebCtl c;
        std::memset( &c, 0, sizeof( c ) );
        c.n_iterations      = n_iterations;
        c.mode              = mode_;
        c.noi               = noi;
        c.nos               = eng->nos( 0 );
        c.force_convergence = conv;
        c.m                 = 1.0;
        c.hm                = 0.5 / c.m;
        c.active            = 1;
        c.solver            = solver_;
        c.fv_unit           = mode_ == 1 && solver_ == SOLVER_LBFGS_OSO;
        c.eps               = eng->fp64() ? 1e-300 : 1e-30; // lbfgs_get_searchdir epsilon
        c.maxmove           = 3.14159265358979323846 / 200.0;
        h2d( d_ctl, &c, 1 );
        size_t el = eng->fp64() ? sizeof( double ) : sizeof( float );
        for( int k = 0; k < 3; ++k )
        {
            // on the engine's (non-blocking) stream, ordered before the iterations
            CUDA_CHECK( cudaMemsetAsync( F[k], 0, eng->total_spins() * el, eng->stream() ) );
            CUDA_CHECK( cudaMemsetAsync( V[k], 0, eng->total_spins() * el, eng->stream() ) );
            if( d_gram )
            {
                CUDA_CHECK( cudaMemsetAsync( Gb[k], 0, eng->total_spins() * el, eng->stream() ) );
                for( int j = 0; j < LB_MEM; ++j )
                {
                    CUDA_CHECK( cudaMemsetAsync( DA[j][k], 0, eng->total_spins() * el, eng->stream() ) );
                    CUDA_CHECK( cudaMemsetAsync( DG[j][k], 0, eng->total_spins() * el, eng->stream() ) );
                }
            }
        }
        if( graph )
        {
            cudaGraphExecDestroy( graph );
            graph = nullptr;
        }
        if( mode_ == 1 )
        {
            // Method_LLG constructor with VP: initial forces, projected, and the initial torque
            if( eng->fp64() )
                probe_t<double>();
            else
                probe_t<float>();
        }
        CUDA_CHECK( cudaStreamSynchronize( eng->stream() ) );
    }

    template<typename R>
    void probe_t()
    {
        auto a  = args<R>();
        auto st = eng->stream();
        eng->run_ddi( eng_spins(), nullptr );
        gneb_clear<<<1, 64, 0, st>>>( d_img, d_ctl, d_gram );
        gneb_eval<R><<<eng->n_blocks(), 256, 0, st>>>( a, 1 );
        vp_probe_finish<<<1, 1, 0, st>>>( d_img, d_ctl );
        CUDA_CHECK( cudaGetLastError() );
    }

    void * const * eng_spins() const
    {
        static thread_local void * p[3];
        for( int c = 0; c < 3; ++c )
            p[c] = eng->spin_ptr( c );
        return p;
    }

    template<typename R>
    void iteration_t()
    {
        auto a  = args<R>();
        auto st = eng->stream();
        int nb  = eng->n_blocks();
        eng->run_ddi( eng_spins(), nullptr );
        gneb_clear<<<1, 256, 0, st>>>( d_img, d_ctl, d_gram );
        gneb_eval<R><<<nb, 256, 0, st>>>( a, 0 );
        if( mode_ == 0 )
        {
            gneb_scalars<<<1, 32, 0, st>>>( d_img, d_ctl, spring );
            gneb_tangent<R><<<nb, 256, 0, st>>>( a );
        }
        else
            gneb_scalars_vp<<<1, 32, 0, st>>>( d_ctl );
        if( solver_ == SOLVER_VP )
        {
            gneb_force<R><<<nb, 256, 0, st>>>( a );
            gneb_update<R><<<nb, 256, 0, st>>>( a );
        }
        else
        {
            oso_force<R><<<nb, 256, 0, st>>>( a );
            if( solver_ == SOLVER_LBFGS_OSO )
                lbfgs_dir<<<1, 32, 0, st>>>( d_ctl, d_gram );
            oso_update<R><<<nb, 256, 0, st>>>( a );
        }
        CUDA_CHECK( cudaGetLastError() );
    }

    void launch( int n )
    {
        const int Gs = 8;
        auto st      = eng->stream();
        if( !graph )
        {
            cudaGraph_t g;
            CUDA_CHECK( cudaStreamBeginCapture( st, cudaStreamCaptureModeThreadLocal ) );
            for( int k = 0; k < Gs; ++k )
                one();
            CUDA_CHECK( cudaStreamEndCapture( st, &g ) );
            CUDA_CHECK( cudaGraphInstantiate( &graph, g, 0 ) );
            cudaGraphDestroy( g );
        }
        for( int k = 0; k < n / Gs; ++k )
            CUDA_CHECK( cudaGraphLaunch( graph, st ) );
        for( int k = 0; k < n % Gs; ++k )
            one();
    }

    void one()
    {
        if( eng->fp64() )
            iteration_t<double>();
        else
            iteration_t<float>();
    }

    GnebCtl ctl()
    {
        GnebCtl c;
        CUDA_CHECK( cudaMemcpyAsync( &c, d_ctl, sizeof( c ), cudaMemcpyDeviceToHost, eng->stream() ) );
        CUDA_CHECK( cudaStreamSynchronize( eng->stream() ) );
        return c;
    }
    std::vector<GnebImage> images()
    {
        std::vector<GnebImage> v( noi );
        CUDA_CHECK( cudaMemcpyAsync( v.data(), d_img, sizeof( GnebImage ) * noi, cudaMemcpyDeviceToHost,
                                     eng->stream() ) );
        CUDA_CHECK( cudaStreamSynchronize( eng->stream() ) );
        return v;
    }

    std::unique_ptr<Engine> eng;
    int noi;
    int mode_;
    int solver_;
    double spring = 1;
    void * F[3] = {}, *V[3] = {}, *T[3] = {}, *G[3] = {};
    void * Gb[3] = {}, *DA[LB_MEM][3] = {}, *DG[LB_MEM][3] = {};
    double * d_gram = nullptr;
    GnebImage * d_img = nullptr;
    GnebCtl * d_ctl   = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<double> torques;
};

static bool stop_file()
{
    std::ifstream f( "STOP" );
    return f.good();
}

// Method::Iterate for a GNEB / VP run: chunks of iterations, host checks in between
static void iterate( GnebRun & R, const std::atomic<bool> & allowed, long max_walltime_sec )
{
    int chunk = 8;
    auto t0   = std::chrono::steady_clock::now();
    while( true )
    {
        auto c = R.ctl();
        if( !c.active || !allowed.load() || stop_file() )
            break;
        if( max_walltime_sec > 0
            && std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count() > max_walltime_sec )
            break;
        R.launch( chunk );
        R.eng->sync();
        chunk = std::min( 512, chunk * 2 );
    }
}

static void finish_chain( State * st, Chain & chain, GnebRun & R )
{
    auto c   = R.ctl();
    auto ims = R.images();
    for( int k = 0; k < R.noi; ++k )
    {
        R.eng->get_spins( k, chain.images[k]->spins.data() );
        chain.images[k]->E = ims[k].E;
    }
    chain.Rx.resize( R.noi );
    chain.torques.resize( R.noi );
    for( int k = 0; k < R.noi; ++k )
    {
        chain.Rx[k]      = ims[k].Rx;
        chain.torques[k] = ims[k].torque;
    }
    chain.Rx_interpolated = chain.Rx;
    chain.E_interpolated.resize( R.noi );
    for( int k = 0; k < R.noi; ++k )
        chain.E_interpolated[k] = ims[k].E;
    chain.info.iteration  = c.iteration;
    chain.info.max_torque = c.max_torque;
    auto now              = std::chrono::steady_clock::now();
    chain.info.wall_ms = std::chrono::duration_cast<std::chrono::milliseconds>( now - chain.info.t_start ).count();
    chain.info.ips     = chain.info.wall_ms > 0 ? 1000.0 * c.iteration / chain.info.wall_ms : 0;
    if( c.aborted )
        log_msg( st, 1, "The geodesic distance between two images is zero! Stopping..." );
}

void gneb_start( State * st, Chain & chain, int solver, bool singleshot )
{
    std::vector<Image *> ims;
    std::vector<int> types;
    for( auto & im : chain.images )
    {
        ims.push_back( im.get() );
        types.push_back( im->gneb_type );
    }
    auto R = std::make_shared<GnebRun>( ims, st->precision == 64, 0, solver );
    for( int k = 0; k < R->noi; ++k )
        R->eng->set_spins( k, ims[k]->spins.data() );
    R->start( types, (int)chain.gneb.n_iterations, chain.gneb.force_convergence, chain.gneb.spring_constant );
    chain.info              = MethodInfo{};
    chain.info.method       = "GNEB";
    chain.info.solver       = solver == SOLVER_VP ? "VP" : ( solver == SOLVER_VP_OSO ? "VP_OSO" : "LBFGS_OSO" );
    chain.info.solver_id    = solver;
    chain.info.n_iterations = (int)chain.gneb.n_iterations;
    chain.info.t_start      = std::chrono::steady_clock::now();
    chain.iteration_allowed  = true;
    chain.singleshot_allowed = singleshot;
    if( singleshot )
    {
        chain.gneb_run = R;
        return;
    }
    iterate( *R, chain.iteration_allowed, chain.gneb.max_walltime_sec );
    finish_chain( st, chain, *R );
    chain.iteration_allowed = false;
}

void gneb_n_shot( State * st, Chain & chain, int n )
{
    auto R = std::static_pointer_cast<GnebRun>( chain.gneb_run );
    if( !R )
        return;
    // the host spin buffers are the state: callers may have written into them since the last call
    for( int k = 0; k < R->noi; ++k )
        R->eng->set_spins( k, chain.images[k]->spins.data() );
    if( R->ctl().active )
    {
        R->launch( n );
        R->eng->sync();
    }
    finish_chain( st, chain, *R );
    if( !R->ctl().active || stop_file() )
    {
        chain.iteration_allowed  = false;
        chain.singleshot_allowed = false;
        chain.gneb_run.reset();
    }
}

// Rx of the host images (geodesic distances, Manifoldmath.cpp:66-72)
void gneb_update_rx( Chain & chain )
{
    size_t noi = chain.images.size();
    chain.Rx.assign( noi, 0.0 );
    for( size_t k = 1; k < noi; ++k )
    {
        auto & a = chain.images[k]->spins;
        auto & b = chain.images[k - 1]->spins;
        double d = 0;
        for( size_t i = 0; i + 2 < a.size(); i += 3 )
        {
            double r = std::fmax( -1.0, std::fmin( 1.0, a[i] * b[i] + a[i + 1] * b[i + 1] + a[i + 2] * b[i + 2] ) );
            double g = std::acos( r );
            d += g * g;
        }
        chain.Rx[k] = chain.Rx[k - 1] + std::sqrt( d );
    }
}

const std::vector<double> & gneb_torques( Chain & chain )
{
    return chain.torques;
}

static void finish_vp( Image & img, GnebRun & R )
{
    auto c   = R.ctl();
    auto ims = R.images();
    R.eng->get_spins( 0, img.spins.data() );
    img.E               = ims[0].E;
    img.info.iteration  = c.iteration;
    img.info.max_torque = c.max_torque;
    img.info.time_ps    = c.iteration * img.llg.dt;
    auto now            = std::chrono::steady_clock::now();
    img.info.wall_ms = std::chrono::duration_cast<std::chrono::milliseconds>( now - img.info.t_start ).count();
    img.info.ips     = img.info.wall_ms > 0 ? 1000.0 * c.iteration / img.info.wall_ms : 0;
}

void llg_vp_run( State * st, Image & img, int solver, bool singleshot )
{
    auto R = std::make_shared<GnebRun>( std::vector<Image *>{ &img }, st->precision == 64, 1, solver );
    R->eng->set_spins( 0, img.spins.data() );
    R->start( { 0 }, (int)img.llg.n_iterations, img.llg.force_convergence, 1.0 );
    if( singleshot )
    {
        img.vp_run = R;
        return;
    }
    iterate( *R, img.iteration_allowed, img.llg.max_walltime_sec );
    finish_vp( img, *R );
    img.iteration_allowed = false;
}

void llg_vp_shot( State * st, Image & img, int n )
{
    (void)st;
    auto R = std::static_pointer_cast<GnebRun>( img.vp_run );
    if( !R )
        return;
    R->eng->set_spins( 0, img.spins.data() );
    if( R->ctl().active )
    {
        R->launch( n );
        R->eng->sync();
    }
    finish_vp( img, *R );
    if( !R->ctl().active || stop_file() )
    {
        img.iteration_allowed  = false;
        img.singleshot_allowed = false;
        img.vp_run.reset();
    }
}

// ---------------------------------------------------------------- batched LLG
struct BatchCache
{
    std::vector<std::pair<const Image *, long>> key;
    bool fp64 = false;
    std::unique_ptr<Engine> eng;
    std::vector<double> host; // concatenated AoS spins (pinned)
    double * pinned = nullptr;
    size_t pinned_n = 0;
    ~BatchCache()
    {
        if( pinned )
            cudaFreeHost( pinned );
    }
};

static BatchCache & batch_cache()
{
    static BatchCache c;
    return c;
}

// Upload the active images of the States into the cached batch engine (rebuilt when the set of
// images or their versions changed) and start the LLG method of every system.
static Engine & batched_prepare( State ** states, int n_states, int solver, int n_iterations,
                                 std::vector<Image *> & ims )
{
    ims.clear();
    std::vector<std::pair<const Image *, long>> key;
    for( int k = 0; k < n_states; ++k )
    {
        State * s  = states[k];
        Image * im = s->chain->images[s->idx_active_image].get();
        if( im->iteration_allowed )
            throw std::runtime_error( "a simulation is already running on one of the batched images" );
        ims.push_back( im );
        key.push_back( { im, im->version } );
    }
    bool fp64 = states[0]->precision == 64;
    BatchCache & C = batch_cache();
    if( !C.eng || C.key != key || C.fp64 != fp64 )
    {
        C.eng.reset();
        std::vector<SystemInput> in;
        for( int k = 0; k < n_states; ++k )
        {
            SystemInput s;
            s.geom = ims[k]->geom.get();
            s.ham  = &ims[k]->ham;
            in.push_back( s );
        }
        C.eng  = std::make_unique<Engine>( in, fp64 );
        C.eng->enable_compensation(); // FP32: compensated state of the LLG stage kernels
        C.key  = key;
        C.fp64 = fp64;
    }
    Engine & E = *C.eng;
    E.set_stream( (cudaStream_t)states[0]->stream );
    size_t total = 0;
    for( auto * im : ims )
        total += im->spins.size();
    if( C.pinned_n < total )
    {
        if( C.pinned )
            cudaFreeHost( C.pinned );
        C.pinned = nullptr;
        CUDA_CHECK( cudaMallocHost( (void **)&C.pinned, total * sizeof( double ) ) );
        C.pinned_n = total;
    }
    size_t o = 0;
    for( int k = 0; k < n_states; ++k )
    {
        std::memcpy( C.pinned + o, ims[k]->spins.data(), ims[k]->spins.size() * sizeof( double ) );
        o += ims[k]->spins.size();
        SystemInput s;
        s.geom                = ims[k]->geom.get();
        s.ham                 = &ims[k]->ham;
        s.dt                  = ims[k]->llg.dt;
        s.damping             = ims[k]->llg.damping;
        s.temperature         = ims[k]->llg.temperature;
        s.force_convergence   = ims[k]->llg.force_convergence;
        s.direct_minimization = ims[k]->llg.direct_minimization;
        s.seed                = (unsigned long long)(unsigned)ims[k]->llg.rng_seed;
        s.stream              = (unsigned)k;
        s.noise_offset        = ims[k]->llg_noise_drawn;
        E.set_params( k, s );
        ims[k]->info           = MethodInfo{};
        ims[k]->info.method    = "LLG";
        ims[k]->info.solver    = solver == 1 ? "SIB" : solver == 2 ? "Depondt" : solver == 3 ? "Heun" : "RK4";
        ims[k]->info.solver_id = solver;
        ims[k]->info.t_start   = std::chrono::steady_clock::now();
        ims[k]->iteration_allowed = true;
    }
    E.set_all_spins( C.pinned );
    std::vector<int> nit( n_states );
    for( int k = 0; k < n_states; ++k )
        nit[k] = n_iterations > 0 ? n_iterations : (int)ims[k]->llg.n_iterations;
    E.llg_start( solver, nit );
    return E;
}

// Bring the batch's spins and run state back into the images and end their runs.
static void batched_finish( Engine & E, const std::vector<Image *> & ims )
{
    BatchCache & C = batch_cache();
    E.get_all_spins( C.pinned );
    E.sync();
    auto stv = E.status();
    size_t o = 0;
    auto now = std::chrono::steady_clock::now();
    for( size_t k = 0; k < ims.size(); ++k )
    {
        std::memcpy( ims[k]->spins.data(), C.pinned + o, ims[k]->spins.size() * sizeof( double ) );
        o += ims[k]->spins.size();
        ims[k]->E               = stv[k].energy;
        if( ims[k]->llg.temperature > 0 )
            ims[k]->llg_noise_drawn += (unsigned)stv[k].iteration;
        ims[k]->info.iteration  = stv[k].iteration;
        ims[k]->info.max_torque = stv[k].max_torque;
        ims[k]->info.time_ps    = stv[k].iteration * ims[k]->llg.dt;
        ims[k]->info.wall_ms = std::chrono::duration_cast<std::chrono::milliseconds>( now - ims[k]->info.t_start ).count();
        ims[k]->info.ips     = ims[k]->info.wall_ms > 0 ? 1000.0 * stv[k].iteration / ims[k]->info.wall_ms : 0;
        ims[k]->iteration_allowed = false;
    }
}

void llg_run_batched( State ** states, int n_states, int solver, int n_iterations, void * info, size_t info_size )
{
    (void)info;
    (void)info_size;
    if( n_states <= 0 )
        return;
    std::vector<Image *> ims;
    Engine & E = batched_prepare( states, n_states, solver, n_iterations, ims );
    // run until every system stopped (convergence / budget) or Simulation_Stop on the first state
    int chunk = 8;
    while( true )
    {
        auto stv = E.status();
        bool any = false;
        for( auto & s : stv )
            any = any || s.active;
        if( !any || !ims[0]->iteration_allowed.load() || stop_file() )
            break;
        E.llg_launch( chunk );
        E.sync();
        chunk = std::min( 512, chunk * 2 );
    }
    batched_finish( E, ims );
}

// FP64 gradients and energies of the States' active images evaluated as one batch: one FP64 engine
// over all systems, so the dipolar term of every system comes from the batch's shared FFT plan
// table (one launch per pass over all systems, each system on its own padded extents).
// gradients: AoS [sum nos][3] in the order of the States; energies[n_states].
void gradient_batched( State ** states, int n_states, double * gradients, double * energies )
{
    if( n_states <= 0 )
        return;
    std::vector<SystemInput> in;
    std::vector<double> all;
    for( int k = 0; k < n_states; ++k )
    {
        Image * im = states[k]->chain->images[states[k]->idx_active_image].get();
        SystemInput s;
        s.geom = im->geom.get();
        s.ham  = &im->ham;
        in.push_back( s );
        all.insert( all.end(), im->spins.begin(), im->spins.end() );
    }
    Engine E( in, true );
    E.set_all_spins( all.data() );
    size_t o = 0;
    for( int k = 0; k < n_states; ++k )
    {
        double e = 0;
        E.gradient( k, gradients ? gradients + o : nullptr, &e, nullptr );
        if( energies )
            energies[k] = e;
        o += 3 * (size_t)E.nos( k );
    }
}

// Open-ended batched run driven by the caller: the first call (or a call for another set of
// States) uploads and starts the batch; every call enqueues n_steps on the batch's stream
// (states[0]'s stream) without synchronising.  llg_batched_finish ends the run.
struct BatchedRun
{
    std::vector<State *> states;
    std::vector<Image *> ims;
    int solver   = -1;
    Engine * eng = nullptr;
};

static BatchedRun & batched_run()
{
    static BatchedRun r;
    return r;
}

void llg_batched_launch( State ** states, int n_states, int solver, int n_steps )
{
    if( n_states <= 0 )
        return;
    BatchedRun & R = batched_run();
    std::vector<State *> st( states, states + n_states );
    if( !R.eng || R.states != st || R.solver != solver )
    {
        if( R.eng )
            batched_finish( *R.eng, R.ims );
        R.eng    = nullptr;
        R.states = st;
        R.solver = solver;
        R.eng    = &batched_prepare( states, n_states, solver, std::numeric_limits<int>::max() / 2, R.ims );
    }
    R.eng->llg_launch( n_steps );
}

void llg_batched_finish( State ** states, int n_states )
{
    BatchedRun & R = batched_run();
    std::vector<State *> st( states, states + n_states );
    if( !R.eng || R.states != st )
        throw std::runtime_error( "no open batched run for these States" );
    batched_finish( *R.eng, R.ims );
    R = BatchedRun{};
}

} // namespace sg
