/*
 * spirit_oracle.c -- CPU FP64 restatement of the reference's spin-dynamics hot path.
 * TEST INFRASTRUCTURE ONLY (see spirit_oracle.h): the product never calls this code.
 *
 * Reference = Spirit v2.2.0 CPU build with OpenMP (redundant neighbour lists,
 * Hamiltonian_Heisenberg.cpp:101-109) and FP64 scalars.  File:line citations below are
 * relative to the reference project root.
 */
#include "spirit_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* core/include/utility/Constants.hpp:18-43 (SI-meV unit system) */
#define C_MU_B 0.057883817555
#define C_MU_0 ( 2.0133545 * 1e-28 )
#define C_K_B 0.08617330350
#define C_GAMMA 0.1760859644
#define C_PI 3.141592653589793238462643383279502884197169399375105820974

typedef struct
{
    int i, j, t[3];
} og_pair;

struct og_system
{
    int n_cells[3];
    int n_cell_atoms;
    int nos;
    int n_cells_total;
    double bravais[3][3];
    double cell_atoms[OG_MAX_BASIS][3];
    double lattice_constant;
    int bc[3];
    double * positions; /* nos*3 */
    double * mu_s;      /* nos */

    /* Zeeman: magnitude stored times mu_B (Hamiltonian_Heisenberg.cpp:35) */
    double field_mag, field_normal[3];
    /* uniaxial anisotropy */
    int n_aniso;
    int aniso_idx[OG_MAX_BASIS];
    double aniso_mag[OG_MAX_BASIS], aniso_normal[OG_MAX_BASIS][3];
    /* exchange and DMI (redundant lists) */
    int n_ex;
    og_pair * ex_pairs;
    double * ex_mag;
    int n_dmi;
    og_pair * dmi_pairs;
    double * dmi_mag;
    double * dmi_normal; /* n_dmi*3 */
    /* DDI */
    int ddi_method;
    int ddi_images[3];
    double ddi_radius;
    int ddi_pb_zero_padding;
    int ddi_ready;
    int pad[3];        /* padded FFT extents per lattice direction */
    int fft_total;     /* pad[0]*pad[1]*pad[2] */
    double * ddi_Dhat; /* [B][B][6][fft_total] complex (re,im interleaved) */
};

static int og_threads = 0;
void og_set_threads( int n )
{
    og_threads = n;
#ifdef _OPENMP
    if( n > 0 )
        omp_set_num_threads( n );
#endif
}

/* ---------------------------------------------------------------- small vector helpers */
static inline double dot3( const double * a, const double * b )
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cross3( const double * a, const double * b, double * o )
{
    double x = a[1] * b[2] - a[2] * b[1];
    double y = a[2] * b[0] - a[0] * b[2];
    double z = a[0] * b[1] - a[1] * b[0];
    o[0]     = x;
    o[1]     = y;
    o[2]     = z;
}
static inline double norm3( const double * a )
{
    return sqrt( dot3( a, a ) );
}
/* Eigen's normalize(): leaves a zero vector untouched */
static inline void normalize3( double * a )
{
    double n2 = dot3( a, a );
    if( n2 > 0 )
    {
        double n = sqrt( n2 );
        a[0] /= n;
        a[1] /= n;
        a[2] /= n;
    }
}

/* ---------------------------------------------------------------- geometry
 * positions: core/src/data/Geometry.cpp:141-160 */
og_system * og_create(
    const int n_cells[3], int n_cell_atoms, const double bravais[9], const double * cell_atoms,
    double lattice_constant, const double * mu_s_basis, const int boundary_conditions[3] )
{
    if( n_cell_atoms < 1 || n_cell_atoms > OG_MAX_BASIS )
        return NULL;
    og_system * s = (og_system *)calloc( 1, sizeof( og_system ) );
    for( int d = 0; d < 3; ++d )
    {
        s->n_cells[d] = n_cells[d];
        s->bc[d]      = boundary_conditions[d];
        for( int e = 0; e < 3; ++e )
            s->bravais[d][e] = bravais[3 * d + e];
    }
    s->n_cell_atoms = n_cell_atoms;
    for( int b = 0; b < n_cell_atoms; ++b )
        for( int e = 0; e < 3; ++e )
            s->cell_atoms[b][e] = cell_atoms[3 * b + e];
    s->lattice_constant = lattice_constant;
    s->n_cells_total    = n_cells[0] * n_cells[1] * n_cells[2];
    s->nos              = n_cell_atoms * s->n_cells_total;
    s->positions        = (double *)malloc( sizeof( double ) * 3 * s->nos );
    s->mu_s             = (double *)malloc( sizeof( double ) * s->nos );
    int N               = n_cell_atoms;
    for( int dc = 0; dc < n_cells[2]; ++dc )
        for( int db = 0; db < n_cells[1]; ++db )
            for( int da = 0; da < n_cells[0]; ++da )
                for( int ia = 0; ia < N; ++ia )
                {
                    int ispin = ia + dc * N * n_cells[1] * n_cells[0] + db * N * n_cells[0] + da * N;
                    double fa = (double)da + s->cell_atoms[ia][0];
                    double fb = (double)db + s->cell_atoms[ia][1];
                    double fc = (double)dc + s->cell_atoms[ia][2];
                    for( int e = 0; e < 3; ++e )
                        s->positions[3 * ispin + e]
                            = lattice_constant
                              * ( fa * s->bravais[0][e] + fb * s->bravais[1][e] + fc * s->bravais[2][e] );
                    s->mu_s[ispin] = mu_s_basis[ia];
                }
    s->ddi_images[0] = s->ddi_images[1] = s->ddi_images[2] = 4;
    return s;
}

void og_free( og_system * s )
{
    if( !s )
        return;
    free( s->positions );
    free( s->mu_s );
    free( s->ex_pairs );
    free( s->ex_mag );
    free( s->dmi_pairs );
    free( s->dmi_mag );
    free( s->dmi_normal );
    free( s->ddi_Dhat );
    free( s );
}

int og_nos( const og_system * s )
{
    return s->nos;
}

void og_positions( const og_system * s, double * out )
{
    memcpy( out, s->positions, sizeof( double ) * 3 * s->nos );
}

/* ---------------------------------------------------------------- neighbours
 * Get_Shell_Radii: core/src/engine/Neighbours.cpp:15-81.  Note the reference compares the
 * fractional basis position cell_atoms[a] with the Cartesian translation i*ta+j*tb+k*tc;
 * that is restated as is. */
static void shell_radii( const og_system * s, int n_shells, double * radii )
{
    const double min_shell_width = 1e-3;
    double ta[3], tb[3], tc[3];
    for( int e = 0; e < 3; ++e )
    {
        ta[e] = s->lattice_constant * s->bravais[0][e];
        tb[e] = s->lattice_constant * s->bravais[1][e];
        tc[e] = s->lattice_constant * s->bravais[2][e];
    }
    int max_n = n_shells + 2;
    int i_max = max_n < s->n_cells[0] - 1 ? max_n : s->n_cells[0] - 1;
    int j_max = max_n < s->n_cells[1] - 1 ? max_n : s->n_cells[1] - 1;
    int k_max = max_n < s->n_cells[2] - 1 ? max_n : s->n_cells[2] - 1;
    if( norm3( ta ) == 0.0 )
        i_max = 0;
    if( norm3( tb ) == 0.0 )
        j_max = 0;
    if( norm3( tc ) == 0.0 )
        k_max = 0;
    double outermost = 0, previous = 0;
    for( int ish = 0; ish < n_shells; ++ish )
    {
        previous  = outermost;
        outermost = DBL_MAX;
        radii[ish] = 0;
        for( int a1 = 0; a1 < s->n_cell_atoms; ++a1 )
        {
            const double * p1 = s->cell_atoms[a1];
            for( int i = i_max; i >= 0; --i )
                for( int j = j_max; j >= -j_max; --j )
                    for( int k = k_max; k >= -k_max; --k )
                        for( int a2 = 0; a2 < s->n_cell_atoms; ++a2 )
                        {
                            if( a1 == a2 && i == 0 && j == 0 && k == 0 )
                                continue;
                            double d[3];
                            for( int e = 0; e < 3; ++e )
                            {
                                double p2 = s->cell_atoms[a2][e] + i * ta[e] + j * tb[e] + k * tc[e];
                                d[e]      = p1[e] - p2;
                            }
                            double delta = norm3( d );
                            if( delta - previous > min_shell_width && delta < outermost )
                            {
                                outermost  = delta;
                                radii[ish] = delta;
                            }
                        }
        }
    }
}

/* Get_Neighbours_in_Shells with use_redundant_neighbours=true: Neighbours.cpp:83-156 */
static int neighbours_in_shells( const og_system * s, int n_shells, og_pair ** pairs_out, int ** shells_out )
{
    const double min_shell_width = 1e-3;
    double radii[OG_MAX_SHELLS];
    shell_radii( s, n_shells, radii );
    double ta[3], tb[3], tc[3];
    for( int e = 0; e < 3; ++e )
    {
        ta[e] = s->lattice_constant * s->bravais[0][e];
        tb[e] = s->lattice_constant * s->bravais[1][e];
        tc[e] = s->lattice_constant * s->bravais[2][e];
    }
    int max_n = n_shells + 2;
    int i_max = max_n < s->n_cells[0] - 1 ? max_n : s->n_cells[0] - 1;
    int j_max = max_n < s->n_cells[1] - 1 ? max_n : s->n_cells[1] - 1;
    int k_max = max_n < s->n_cells[2] - 1 ? max_n : s->n_cells[2] - 1;
    /* the lower bounds are taken before the zero-vector checks (Neighbours.cpp:104-116) */
    int i_min = -i_max, j_min = -j_max, k_min = -k_max;
    if( norm3( ta ) == 0.0 )
        i_max = 0;
    if( norm3( tb ) == 0.0 )
        j_max = 0;
    if( norm3( tc ) == 0.0 )
        k_max = 0;
    int cap = 64, n = 0;
    og_pair * pairs = (og_pair *)malloc( sizeof( og_pair ) * cap );
    int * shells    = (int *)malloc( sizeof( int ) * cap );
    for( int a1 = 0; a1 < s->n_cell_atoms; ++a1 )
    {
        const double * p1 = s->cell_atoms[a1];
        for( int ish = 0; ish < n_shells; ++ish )
        {
            double radius = radii[ish];
            for( int i = i_max; i >= i_min; --i )
                for( int j = j_max; j >= j_min; --j )
                    for( int k = k_max; k >= k_min; --k )
                        for( int a2 = 0; a2 < s->n_cell_atoms; ++a2 )
                        {
                            double d[3];
                            for( int e = 0; e < 3; ++e )
                            {
                                double p2 = s->cell_atoms[a2][e] + i * ta[e] + j * tb[e] + k * tc[e];
                                d[e]      = p1[e] - p2;
                            }
                            if( fabs( norm3( d ) - radius ) < min_shell_width )
                            {
                                if( n == cap )
                                {
                                    cap *= 2;
                                    pairs  = (og_pair *)realloc( pairs, sizeof( og_pair ) * cap );
                                    shells = (int *)realloc( shells, sizeof( int ) * cap );
                                }
                                pairs[n].i    = a1;
                                pairs[n].j    = a2;
                                pairs[n].t[0] = i;
                                pairs[n].t[1] = j;
                                pairs[n].t[2] = k;
                                shells[n]     = ish;
                                ++n;
                            }
                        }
        }
    }
    *pairs_out  = pairs;
    *shells_out = shells;
    return n;
}

/* DMI_Normal_from_Pair: Neighbours.cpp:249-286 */
static void dmi_normal( const og_system * s, const og_pair * p, int chirality, double * out )
{
    double ipos[3], jpos[3], r[3];
    for( int e = 0; e < 3; ++e )
    {
        double ta = s->lattice_constant * s->bravais[0][e];
        double tb = s->lattice_constant * s->bravais[1][e];
        double tc = s->lattice_constant * s->bravais[2][e];
        ipos[e]   = s->positions[3 * p->i + e];
        jpos[e]   = s->positions[3 * p->j + e] + p->t[0] * ta + p->t[1] * tb + p->t[2] * tc;
        r[e]      = jpos[e] - ipos[e];
    }
    const double ez[3] = { 0, 0, 1 };
    if( chirality == 1 )
    {
        normalize3( r );
        memcpy( out, r, sizeof( r ) );
    }
    else if( chirality == -1 )
    {
        r[0] = -r[0];
        r[1] = -r[1];
        r[2] = -r[2];
        normalize3( r );
        memcpy( out, r, sizeof( r ) );
    }
    else if( chirality == 2 )
    {
        normalize3( r );
        cross3( r, ez, out );
    }
    else if( chirality == -2 )
    {
        normalize3( r );
        cross3( ez, r, out );
    }
    else
        out[0] = out[1] = out[2] = 0;
}

int og_set_exchange_shells( og_system * s, int n_shells, const double * jij )
{
    free( s->ex_pairs );
    free( s->ex_mag );
    s->ex_pairs = NULL;
    s->ex_mag   = NULL;
    s->n_ex     = 0;
    if( n_shells <= 0 )
        return 0;
    int * shells;
    s->n_ex   = neighbours_in_shells( s, n_shells, &s->ex_pairs, &shells );
    s->ex_mag = (double *)malloc( sizeof( double ) * ( s->n_ex + 1 ) );
    for( int p = 0; p < s->n_ex; ++p )
        s->ex_mag[p] = jij[shells[p]];
    free( shells );
    return s->n_ex;
}

int og_set_dmi_shells( og_system * s, int n_shells, const double * dij, int chirality )
{
    free( s->dmi_pairs );
    free( s->dmi_mag );
    free( s->dmi_normal );
    s->dmi_pairs  = NULL;
    s->dmi_mag    = NULL;
    s->dmi_normal = NULL;
    s->n_dmi      = 0;
    if( n_shells <= 0 )
        return 0;
    int * shells;
    s->n_dmi      = neighbours_in_shells( s, n_shells, &s->dmi_pairs, &shells );
    s->dmi_mag    = (double *)malloc( sizeof( double ) * ( s->n_dmi + 1 ) );
    s->dmi_normal = (double *)malloc( sizeof( double ) * 3 * ( s->n_dmi + 1 ) );
    for( int p = 0; p < s->n_dmi; ++p )
    {
        s->dmi_mag[p] = dij[shells[p]];
        dmi_normal( s, &s->dmi_pairs[p], chirality, s->dmi_normal + 3 * p );
    }
    free( shells );
    return s->n_dmi;
}

/* explicit pairs + the redundant mirror (Hamiltonian_Heisenberg.cpp:126-139, 160-173) */
int og_set_exchange_pairs( og_system * s, int n, const int * pairs, const double * jij )
{
    free( s->ex_pairs );
    free( s->ex_mag );
    s->n_ex     = 2 * n;
    s->ex_pairs = (og_pair *)malloc( sizeof( og_pair ) * ( 2 * n + 1 ) );
    s->ex_mag   = (double *)malloc( sizeof( double ) * ( 2 * n + 1 ) );
    for( int p = 0; p < n; ++p )
    {
        const int * q        = pairs + 5 * p;
        og_pair a            = { q[0], q[1], { q[2], q[3], q[4] } };
        og_pair b            = { q[1], q[0], { -q[2], -q[3], -q[4] } };
        s->ex_pairs[p]       = a;
        s->ex_pairs[n + p]   = b;
        s->ex_mag[p]         = jij[p];
        s->ex_mag[n + p]     = jij[p];
    }
    return s->n_ex;
}

int og_set_dmi_pairs( og_system * s, int n, const int * pairs, const double * dij, const double * normals )
{
    free( s->dmi_pairs );
    free( s->dmi_mag );
    free( s->dmi_normal );
    s->n_dmi      = 2 * n;
    s->dmi_pairs  = (og_pair *)malloc( sizeof( og_pair ) * ( 2 * n + 1 ) );
    s->dmi_mag    = (double *)malloc( sizeof( double ) * ( 2 * n + 1 ) );
    s->dmi_normal = (double *)malloc( sizeof( double ) * 3 * ( 2 * n + 1 ) );
    for( int p = 0; p < n; ++p )
    {
        const int * q        = pairs + 5 * p;
        og_pair a            = { q[0], q[1], { q[2], q[3], q[4] } };
        og_pair b            = { q[1], q[0], { -q[2], -q[3], -q[4] } };
        s->dmi_pairs[p]      = a;
        s->dmi_pairs[n + p]  = b;
        s->dmi_mag[p]        = dij[p];
        s->dmi_mag[n + p]    = dij[p];
        for( int e = 0; e < 3; ++e )
        {
            s->dmi_normal[3 * p + e]       = normals[3 * p + e];
            s->dmi_normal[3 * ( n + p ) + e] = -normals[3 * p + e];
        }
    }
    return s->n_dmi;
}

int og_n_exchange_pairs( const og_system * s )
{
    return s->n_ex;
}
int og_n_dmi_pairs( const og_system * s )
{
    return s->n_dmi;
}
void og_get_exchange_pairs( const og_system * s, int * pairs, double * mag )
{
    for( int p = 0; p < s->n_ex; ++p )
    {
        pairs[5 * p + 0] = s->ex_pairs[p].i;
        pairs[5 * p + 1] = s->ex_pairs[p].j;
        for( int e = 0; e < 3; ++e )
            pairs[5 * p + 2 + e] = s->ex_pairs[p].t[e];
        mag[p] = s->ex_mag[p];
    }
}
void og_get_dmi_pairs( const og_system * s, int * pairs, double * mag, double * normals )
{
    for( int p = 0; p < s->n_dmi; ++p )
    {
        pairs[5 * p + 0] = s->dmi_pairs[p].i;
        pairs[5 * p + 1] = s->dmi_pairs[p].j;
        for( int e = 0; e < 3; ++e )
        {
            pairs[5 * p + 2 + e] = s->dmi_pairs[p].t[e];
            normals[3 * p + e]   = s->dmi_normal[3 * p + e];
        }
        mag[p] = s->dmi_mag[p];
    }
}

/* idx_from_pair: core/include/engine/Vectormath.hpp:437-528 (no defects: atom types always valid) */
static inline int idx_from_pair( const og_system * s, int ispin, const og_pair * p )
{
    int N = s->n_cell_atoms;
    if( p->i != ispin % N )
        return -1;
    int Na = s->n_cells[0], Nb = s->n_cells[1], Nc = s->n_cells[2];
    if( abs( p->t[0] ) > Na || abs( p->t[1] ) > Nb || abs( p->t[2] ) > Nc )
        return -1;
    int nic = ispin / ( N * Na * Nb );
    int nib = ( ispin - nic * N * Na * Nb ) / ( N * Na );
    int nia = ( ispin - nic * N * Na * Nb - nib * N * Na ) / N;
    int nja = nia + p->t[0], njb = nib + p->t[1], njc = nic + p->t[2];
    if( s->bc[0] || ( 0 <= nja && nja < Na ) )
    {
        if( nja < 0 )
            nja += Na;
        if( nja >= Na )
            nja -= Na;
    }
    else
        return -1;
    if( s->bc[1] || ( 0 <= njb && njb < Nb ) )
    {
        if( njb < 0 )
            njb += Nb;
        if( njb >= Nb )
            njb -= Nb;
    }
    else
        return -1;
    if( s->bc[2] || ( 0 <= njc && njc < Nc ) )
    {
        if( njc < 0 )
            njc += Nc;
        if( njc >= Nc )
            njc -= Nc;
    }
    else
        return -1;
    return p->j + nja * N + njb * N * Na + njc * N * Na * Nb;
}

int og_idx_from_pair( const og_system * s, int ispin, const int pair[5] )
{
    og_pair p = { pair[0], pair[1], { pair[2], pair[3], pair[4] } };
    return idx_from_pair( s, ispin, &p );
}

void og_set_field( og_system * s, double magnitude, const double normal[3] )
{
    s->field_mag = magnitude * C_MU_B;
    for( int e = 0; e < 3; ++e )
        s->field_normal[e] = normal[e];
}

void og_set_anisotropy( og_system * s, int n, const int * indices, const double * magnitudes, const double * normals )
{
    s->n_aniso = n;
    for( int k = 0; k < n; ++k )
    {
        s->aniso_idx[k] = indices[k];
        s->aniso_mag[k] = magnitudes[k];
        for( int e = 0; e < 3; ++e )
            s->aniso_normal[k][e] = normals[3 * k + e];
    }
}

/* ---------------------------------------------------------------- FFT (FP64, any length)
 * Mixed-radix decimation-in-time Cooley-Tukey, recursive, with an O(p^2) butterfly for each
 * prime factor p.  Unnormalised; sign = -1 forward, +1 inverse.  This replaces the
 * reference's kissFFT backend (core/thirdparty/kiss_fft, itself a mixed-radix Cooley-Tukey);
 * only the convolution result matters, which is basis-independent. */
typedef struct
{
    double re, im;
} cpx;

static void fft_rec( cpx * out, const cpx * in, int n, int stride, int sign, cpx * scratch )
{
    if( n == 1 )
    {
        out[0] = in[0];
        return;
    }
    int p = 2;
    while( p * p <= n && n % p )
        ++p;
    if( n % p )
        p = n;
    int m = n / p;
    /* sub-transforms of the p decimated sequences */
    for( int r = 0; r < p; ++r )
        fft_rec( scratch + r * m, in + r * stride, m, stride * p, sign, out );
    /* butterflies: X[k + q m] = sum_r W_n^{r(k+qm)} Y_r[k] */
    for( int k = 0; k < m; ++k )
    {
        for( int q = 0; q < p; ++q )
        {
            int kk   = k + q * m;
            double sr = 0, si = 0;
            for( int r = 0; r < p; ++r )
            {
                long long e  = ( (long long)r * kk ) % n;
                double ang   = sign * 2.0 * C_PI * (double)e / (double)n;
                double c     = cos( ang ), sn = sin( ang );
                cpx y        = scratch[r * m + k];
                sr += y.re * c - y.im * sn;
                si += y.re * sn + y.im * c;
            }
            out[kk].re = sr;
            out[kk].im = si;
        }
    }
}

/* power-of-two fast path: iterative radix-2 with exact twiddles */
static void fft_pow2( cpx * a, int n, int sign )
{
    for( int i = 1, j = 0; i < n; ++i )
    {
        int bit = n >> 1;
        for( ; j & bit; bit >>= 1 )
            j ^= bit;
        j ^= bit;
        if( i < j )
        {
            cpx t = a[i];
            a[i]  = a[j];
            a[j]  = t;
        }
    }
    for( int len = 2; len <= n; len <<= 1 )
    {
        int half = len >> 1;
        for( int k = 0; k < half; ++k )
        {
            double ang = sign * 2.0 * C_PI * (double)k / (double)len;
            double c = cos( ang ), sn = sin( ang );
            for( int i = 0; i < n; i += len )
            {
                cpx u      = a[i + k];
                cpx v      = a[i + k + half];
                double vr  = v.re * c - v.im * sn;
                double vi  = v.re * sn + v.im * c;
                a[i + k].re        = u.re + vr;
                a[i + k].im        = u.im + vi;
                a[i + k + half].re = u.re - vr;
                a[i + k + half].im = u.im - vi;
            }
        }
    }
}

static void fft_line( cpx * line, int n, int sign, cpx * w1, cpx * w2 )
{
    if( n <= 1 )
        return;
    if( ( n & ( n - 1 ) ) == 0 )
    {
        fft_pow2( line, n, sign );
        return;
    }
    memcpy( w1, line, sizeof( cpx ) * n );
    fft_rec( line, w1, n, 1, sign, w2 );
}

/* 3D transform of an [n2][n1][n0] array (index x0 + n0*(x1 + n1*x2)) along every axis */
static void fft3d( cpx * data, const int n[3], int sign )
{
    int total = n[0] * n[1] * n[2];
    for( int ax = 0; ax < 3; ++ax )
    {
        int len = n[ax];
        if( len <= 1 )
            continue;
        int stride = ax == 0 ? 1 : ( ax == 1 ? n[0] : n[0] * n[1] );
        int lines  = total / len;
#pragma omp parallel
        {
            cpx * buf = (cpx *)malloc( sizeof( cpx ) * len * 3 );
#pragma omp for schedule( static )
            for( int l = 0; l < lines; ++l )
            {
                int base;
                if( ax == 0 )
                    base = l * len;
                else if( ax == 1 )
                    base = ( l % n[0] ) + ( l / n[0] ) * n[0] * n[1];
                else
                    base = l;
                for( int t = 0; t < len; ++t )
                    buf[t] = data[base + t * stride];
                fft_line( buf, len, sign, buf + len, buf + 2 * len );
                for( int t = 0; t < len; ++t )
                    data[base + t * stride] = buf[t];
            }
            free( buf );
        }
    }
}

/* ---------------------------------------------------------------- DDI
 * Prepare_DDI (Hamiltonian_Heisenberg.cpp:1501-1595) + FFT_Dipole_Matrices (1406-1499).
 * Padding: a direction is doubled if n>1 and (open or pb_zero_padding).  The dipole tensor
 * D(r) = m (3 r r^T / r^5 - I / r^3), m = mu_0 mu_B^2 / (4 pi 1e-30), summed over the
 * periodic images of periodic directions, for every basis pair (b1, b2). */
void og_set_ddi( og_system * s, int method, const int n_periodic_images[3], double radius, int pb_zero_padding )
{
    s->ddi_method = method;
    for( int d = 0; d < 3; ++d )
        s->ddi_images[d] = n_periodic_images[d];
    s->ddi_radius          = radius;
    s->ddi_pb_zero_padding = pb_zero_padding;
    s->ddi_ready           = 0;
    free( s->ddi_Dhat );
    s->ddi_Dhat = NULL;
    if( method != 1 )
        return;
    for( int d = 0; d < 3; ++d )
    {
        s->pad[d] = s->n_cells[d];
        if( s->n_cells[d] > 1 && ( s->bc[d] == 0 || pb_zero_padding ) )
            s->pad[d] *= 2;
    }
    s->fft_total = s->pad[0] * s->pad[1] * s->pad[2];
    int B        = s->n_cell_atoms;
    int T        = s->fft_total;
    s->ddi_Dhat  = (double *)calloc( (size_t)B * B * 6 * T * 2, sizeof( double ) );
    const double mult = C_MU_0 * C_MU_B * C_MU_B / ( 4 * C_PI * 1e-30 );
    int img[3];
    for( int d = 0; d < 3; ++d )
        img[d] = s->bc[d] == 0 ? 0 : s->ddi_images[d];
    int Na = s->n_cells[0], Nb = s->n_cells[1], Nc = s->n_cells[2];
    for( int b1 = 0; b1 < B; ++b1 )
        for( int b2 = 0; b2 < B; ++b2 )
        {
            double * Dh = s->ddi_Dhat + (size_t)( b1 * B + b2 ) * 6 * T * 2;
#pragma omp parallel for collapse( 2 )
            for( int c = 0; c < s->pad[2]; ++c )
                for( int b = 0; b < s->pad[1]; ++b )
                    for( int a = 0; a < s->pad[0]; ++a )
                    {
                        int a_idx = a < Na ? a : a - s->pad[0];
                        int b_idx = b < Nb ? b : b - s->pad[1];
                        int c_idx = c < Nc ? c : c - s->pad[2];
                        double Dxx = 0, Dxy = 0, Dxz = 0, Dyy = 0, Dyz = 0, Dzz = 0;
                        for( int ap = -img[0]; ap <= img[0]; ++ap )
                            for( int bp = -img[1]; bp <= img[1]; ++bp )
                                for( int cp = -img[2]; cp <= img[2]; ++cp )
                                {
                                    double fa = a_idx + ap * Na + s->cell_atoms[b1][0] - s->cell_atoms[b2][0];
                                    double fb = b_idx + bp * Nb + s->cell_atoms[b1][1] - s->cell_atoms[b2][1];
                                    double fc = c_idx + cp * Nc + s->cell_atoms[b1][2] - s->cell_atoms[b2][2];
                                    double r[3];
                                    for( int e = 0; e < 3; ++e )
                                        r[e] = s->lattice_constant
                                               * ( fa * s->bravais[0][e] + fb * s->bravais[1][e]
                                                   + fc * s->bravais[2][e] );
                                    double d = norm3( r );
                                    if( d > 1e-10 )
                                    {
                                        double d3 = d * d * d, d5 = d * d * d * d * d;
                                        Dxx += mult * ( 3 * r[0] * r[0] / d5 - 1 / d3 );
                                        Dxy += mult * 3 * r[0] * r[1] / d5;
                                        Dxz += mult * 3 * r[0] * r[2] / d5;
                                        Dyy += mult * ( 3 * r[1] * r[1] / d5 - 1 / d3 );
                                        Dyz += mult * 3 * r[1] * r[2] / d5;
                                        Dzz += mult * ( 3 * r[2] * r[2] / d5 - 1 / d3 );
                                    }
                                }
                        size_t idx = (size_t)a + s->pad[0] * ( b + (size_t)s->pad[1] * c );
                        double v[6] = { Dxx, Dxy, Dxz, Dyy, Dyz, Dzz };
                        for( int comp = 0; comp < 6; ++comp )
                            Dh[2 * ( comp * (size_t)T + idx )] = v[comp];
                    }
            for( int comp = 0; comp < 6; ++comp )
                fft3d( (cpx *)( Dh + 2 * (size_t)comp * T ), s->pad, -1 );
        }
    s->ddi_ready = 1;
}

/* Gradient_DDI_FFT: Hamiltonian_Heisenberg.cpp:920-1014 (FFT_Spins 1373-1404): g_i -= mu_i * H_i,
 * H = (1/T) IFFT( sum_b2 Dhat_{b1 b2} . FFT(mu s)_b2 ). */
static void gradient_ddi_fft( og_system * s, const double * spins, double * grad )
{
    int B = s->n_cell_atoms, T = s->fft_total;
    int Na = s->n_cells[0], Nb = s->n_cells[1], Nc = s->n_cells[2];
    cpx * S = (cpx *)calloc( (size_t)B * 3 * T, sizeof( cpx ) );
    cpx * H = (cpx *)calloc( (size_t)B * 3 * T, sizeof( cpx ) );
    for( int c = 0; c < Nc; ++c )
        for( int b = 0; b < Nb; ++b )
            for( int a = 0; a < Na; ++a )
                for( int bi = 0; bi < B; ++bi )
                {
                    int io     = bi + B * ( a + Na * ( b + Nb * c ) );
                    size_t idx = (size_t)a + s->pad[0] * ( b + (size_t)s->pad[1] * c );
                    for( int e = 0; e < 3; ++e )
                        S[(size_t)( bi * 3 + e ) * T + idx].re = spins[3 * io + e] * s->mu_s[io];
                }
    for( int k = 0; k < 3 * B; ++k )
        fft3d( S + (size_t)k * T, s->pad, -1 );
#pragma omp parallel for
    for( long long q = 0; q < (long long)T; ++q )
    {
        for( int b1 = 0; b1 < B; ++b1 )
        {
            double hr[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
            for( int b2 = 0; b2 < B; ++b2 )
            {
                const cpx * D = (const cpx *)( s->ddi_Dhat + (size_t)( b1 * B + b2 ) * 6 * T * 2 );
                cpx d[6];
                for( int comp = 0; comp < 6; ++comp )
                    d[comp] = D[(size_t)comp * T + q];
                cpx sx = S[(size_t)( b2 * 3 + 0 ) * T + q], sy = S[(size_t)( b2 * 3 + 1 ) * T + q],
                    sz = S[(size_t)( b2 * 3 + 2 ) * T + q];
                /* rows of the symmetric tensor: (xx xy xz) (xy yy yz) (xz yz zz), FFT.hpp:42-49 */
                const int row[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
                for( int e = 0; e < 3; ++e )
                {
                    cpx d1 = d[row[e][0]], d2 = d[row[e][1]], d3 = d[row[e][2]];
                    hr[e] += d1.re * sx.re + d2.re * sy.re + d3.re * sz.re - d1.im * sx.im - d2.im * sy.im
                             - d3.im * sz.im;
                    hi[e] += d1.re * sx.im + d2.re * sy.im + d3.re * sz.im + d1.im * sx.re + d2.im * sy.re
                             + d3.im * sz.re;
                }
            }
            for( int e = 0; e < 3; ++e )
            {
                H[(size_t)( b1 * 3 + e ) * T + q].re = hr[e];
                H[(size_t)( b1 * 3 + e ) * T + q].im = hi[e];
            }
        }
    }
    for( int k = 0; k < 3 * B; ++k )
        fft3d( H + (size_t)k * T, s->pad, +1 );
    for( int c = 0; c < Nc; ++c )
        for( int b = 0; b < Nb; ++b )
            for( int a = 0; a < Na; ++a )
                for( int bi = 0; bi < B; ++bi )
                {
                    int io     = bi + B * ( a + Na * ( b + Nb * c ) );
                    size_t idx = (size_t)a + s->pad[0] * ( b + (size_t)s->pad[1] * c );
                    for( int e = 0; e < 3; ++e )
                        grad[3 * io + e] -= s->mu_s[io] * H[(size_t)( bi * 3 + e ) * T + idx].re / T;
                }
    free( S );
    free( H );
}

/* Gradient_DDI_Direct: Hamiltonian_Heisenberg.cpp:1016-1071 */
void og_gradient_ddi_direct( og_system * s, const double * spins, double * grad )
{
    const double mult = C_MU_0 * C_MU_B * C_MU_B / ( 4 * C_PI * 1e-30 );
    int img[3];
    for( int d = 0; d < 3; ++d )
        img[d] = s->bc[d] == 0 ? 0 : s->ddi_images[d];
#pragma omp parallel for schedule( dynamic, 16 )
    for( int i1 = 0; i1 < s->nos; ++i1 )
    {
        for( int i2 = 0; i2 < s->nos; ++i2 )
        {
            const double * m2 = spins + 3 * i2;
            double diff[3];
            for( int e = 0; e < 3; ++e )
                diff[e] = s->positions[3 * i2 + e] - s->positions[3 * i1 + e];
            double Dxx = 0, Dxy = 0, Dxz = 0, Dyy = 0, Dyz = 0, Dzz = 0;
            for( int ap = -img[0]; ap <= img[0]; ++ap )
                for( int bp = -img[1]; bp <= img[1]; ++bp )
                    for( int cp = -img[2]; cp <= img[2]; ++cp )
                    {
                        double r[3];
                        for( int e = 0; e < 3; ++e )
                            r[e] = diff[e] + ap * s->n_cells[0] * s->bravais[0][e] * s->lattice_constant
                                   + bp * s->n_cells[1] * s->bravais[1][e] * s->lattice_constant
                                   + cp * s->n_cells[2] * s->bravais[2][e] * s->lattice_constant;
                        double d = norm3( r );
                        if( d > 1e-10 )
                        {
                            double d3 = d * d * d, d5 = d * d * d * d * d;
                            Dxx += mult * ( 3 * r[0] * r[0] / d5 - 1 / d3 );
                            Dxy += mult * 3 * r[0] * r[1] / d5;
                            Dxz += mult * 3 * r[0] * r[2] / d5;
                            Dyy += mult * ( 3 * r[1] * r[1] / d5 - 1 / d3 );
                            Dyz += mult * 3 * r[1] * r[2] / d5;
                            Dzz += mult * ( 3 * r[2] * r[2] / d5 - 1 / d3 );
                        }
                    }
            double mm = s->mu_s[i1] * s->mu_s[i2];
            grad[3 * i1 + 0] -= ( Dxx * m2[0] + Dxy * m2[1] + Dxz * m2[2] ) * mm;
            grad[3 * i1 + 1] -= ( Dxy * m2[0] + Dyy * m2[1] + Dyz * m2[2] ) * mm;
            grad[3 * i1 + 2] -= ( Dxz * m2[0] + Dyz * m2[1] + Dzz * m2[2] ) * mm;
        }
    }
}

static void gradient_ddi( og_system * s, const double * spins, double * grad )
{
    if( s->ddi_method == 1 )
        gradient_ddi_fft( s, spins, grad );
    else if( s->ddi_method == 3 && s->ddi_radius < 0 )
        og_gradient_ddi_direct( s, spins, grad );
}

/* ---------------------------------------------------------------- local terms
 * Gradient_Zeeman 768-783, Gradient_Anisotropy 785-800, Gradient_Exchange 822-842,
 * Gradient_DMI 844-864 (redundant lists: only spin i is updated per pair) */
static void gradient_anisotropy( const og_system * s, const double * spins, double * g )
{
    int N = s->n_cell_atoms;
#pragma omp parallel for
    for( int ic = 0; ic < s->n_cells_total; ++ic )
        for( int k = 0; k < s->n_aniso; ++k )
        {
            int i              = ic * N + s->aniso_idx[k];
            const double * n   = s->aniso_normal[k];
            double sc          = 2.0 * s->aniso_mag[k] * dot3( n, spins + 3 * i );
            for( int e = 0; e < 3; ++e )
                g[3 * i + e] -= sc * n[e];
        }
}

static void gradient_exchange( const og_system * s, const double * spins, double * g )
{
#pragma omp parallel for
    for( int ic = 0; ic < s->n_cells_total; ++ic )
        for( int p = 0; p < s->n_ex; ++p )
        {
            int i = s->ex_pairs[p].i + ic * s->n_cell_atoms;
            int j = idx_from_pair( s, i, &s->ex_pairs[p] );
            if( j >= 0 )
                for( int e = 0; e < 3; ++e )
                    g[3 * i + e] -= s->ex_mag[p] * spins[3 * j + e];
        }
}

static void gradient_dmi( const og_system * s, const double * spins, double * g )
{
#pragma omp parallel for
    for( int ic = 0; ic < s->n_cells_total; ++ic )
        for( int p = 0; p < s->n_dmi; ++p )
        {
            int i = s->dmi_pairs[p].i + ic * s->n_cell_atoms;
            int j = idx_from_pair( s, i, &s->dmi_pairs[p] );
            if( j >= 0 )
            {
                double c[3];
                cross3( spins + 3 * j, s->dmi_normal + 3 * p, c );
                for( int e = 0; e < 3; ++e )
                    g[3 * i + e] -= s->dmi_mag[p] * c[e];
            }
        }
}

static void gradient_zeeman( const og_system * s, double * g )
{
#pragma omp parallel for
    for( int i = 0; i < s->nos; ++i )
        for( int e = 0; e < 3; ++e )
            g[3 * i + e] -= s->mu_s[i] * s->field_mag * s->field_normal[e];
}

static int has_zeeman( const og_system * s )
{
    return fabs( s->field_mag ) > 1e-60; /* Update_Energy_Contributions, cpp:205 */
}

/* Gradient: cpp:670-702 */
void og_gradient( og_system * s, const double * spins, double * g )
{
    memset( g, 0, sizeof( double ) * 3 * s->nos );
    if( has_zeeman( s ) )
        gradient_zeeman( s, g );
    if( s->n_aniso > 0 )
        gradient_anisotropy( s, spins, g );
    if( s->n_ex > 0 )
        gradient_exchange( s, spins, g );
    if( s->n_dmi > 0 )
        gradient_dmi( s, spins, g );
    if( s->ddi_method != 0 )
        gradient_ddi( s, spins, g );
}

/* Gradient_and_Energy: cpp:704-766.  E = sum 0.5 g.s over the quadratic terms, then the
 * Zeeman gradient and energy sum -mu_i B.s_i. */
double og_gradient_and_energy( og_system * s, const double * spins, double * g )
{
    memset( g, 0, sizeof( double ) * 3 * s->nos );
    if( s->n_aniso > 0 )
        gradient_anisotropy( s, spins, g );
    if( s->n_ex > 0 )
        gradient_exchange( s, spins, g );
    if( s->n_dmi > 0 )
        gradient_dmi( s, spins, g );
    if( s->ddi_method != 0 )
        gradient_ddi( s, spins, g );
    double E = 0;
#pragma omp parallel for reduction( + : E )
    for( int i = 0; i < s->nos; ++i )
        E += 0.5 * dot3( g + 3 * i, spins + 3 * i );
    if( has_zeeman( s ) )
    {
        gradient_zeeman( s, g );
        double Ez = 0;
#pragma omp parallel for reduction( + : Ez )
        for( int i = 0; i < s->nos; ++i )
        {
            double b[3] = { s->field_normal[0] * s->field_mag, s->field_normal[1] * s->field_mag,
                            s->field_normal[2] * s->field_mag };
            Ez += -s->mu_s[i] * dot3( b, spins + 3 * i );
        }
        E += Ez;
    }
    return E;
}

/* Energy_Contributions_per_Spin: cpp:262-305; E_Zeeman 307-322, E_Anisotropy 324-338,
 * E_Exchange 357-377, E_DMI 379-401, E_DDI_FFT 465-511 (0.5 s.g_DDI) */
int og_energy_contributions( og_system * s, const double * spins, double * out, char * names, int names_len )
{
    int nos = s->nos, n = 0;
    char buf[256] = { 0 };
    if( has_zeeman( s ) )
    {
        double * E = out + (size_t)n * nos;
        for( int i = 0; i < nos; ++i )
            E[i] = -s->mu_s[i] * s->field_mag * dot3( s->field_normal, spins + 3 * i );
        strcat( buf, "Zeeman," );
        ++n;
    }
    if( s->n_aniso > 0 )
    {
        double * E = out + (size_t)n * nos;
        memset( E, 0, sizeof( double ) * nos );
        for( int ic = 0; ic < s->n_cells_total; ++ic )
            for( int k = 0; k < s->n_aniso; ++k )
            {
                int i    = ic * s->n_cell_atoms + s->aniso_idx[k];
                double d = dot3( s->aniso_normal[k], spins + 3 * i );
                E[i] -= s->aniso_mag[k] * d * d;
            }
        strcat( buf, "Anisotropy," );
        ++n;
    }
    if( s->n_ex > 0 )
    {
        double * E = out + (size_t)n * nos;
        memset( E, 0, sizeof( double ) * nos );
#pragma omp parallel for
        for( int ic = 0; ic < s->n_cells_total; ++ic )
            for( int p = 0; p < s->n_ex; ++p )
            {
                int i = s->ex_pairs[p].i + ic * s->n_cell_atoms;
                int j = idx_from_pair( s, i, &s->ex_pairs[p] );
                if( j >= 0 )
                    E[i] -= 0.5 * s->ex_mag[p] * dot3( spins + 3 * i, spins + 3 * j );
            }
        strcat( buf, "Exchange," );
        ++n;
    }
    if( s->n_dmi > 0 )
    {
        double * E = out + (size_t)n * nos;
        memset( E, 0, sizeof( double ) * nos );
#pragma omp parallel for
        for( int ic = 0; ic < s->n_cells_total; ++ic )
            for( int p = 0; p < s->n_dmi; ++p )
            {
                int i = s->dmi_pairs[p].i + ic * s->n_cell_atoms;
                int j = idx_from_pair( s, i, &s->dmi_pairs[p] );
                if( j >= 0 )
                {
                    double c[3];
                    cross3( spins + 3 * i, spins + 3 * j, c );
                    E[i] -= 0.5 * s->dmi_mag[p] * dot3( s->dmi_normal + 3 * p, c );
                }
            }
        strcat( buf, "DMI," );
        ++n;
    }
    if( s->ddi_method != 0 )
    {
        double * E = out + (size_t)n * nos;
        double * g = (double *)calloc( (size_t)3 * nos, sizeof( double ) );
        gradient_ddi( s, spins, g );
        for( int i = 0; i < nos; ++i )
            E[i] = 0.5 * dot3( spins + 3 * i, g + 3 * i );
        free( g );
        strcat( buf, "DDI," );
        ++n;
    }
    if( names && names_len > 0 )
    {
        size_t l = strlen( buf );
        if( l > 0 )
            buf[l - 1] = 0;
        strncpy( names, buf, names_len - 1 );
        names[names_len - 1] = 0;
    }
    return n;
}

double og_energy( og_system * s, const double * spins )
{
    int nos    = s->nos;
    double * E = (double *)malloc( sizeof( double ) * 5 * nos );
    int n      = og_energy_contributions( s, spins, E, NULL, 0 );
    double sum = 0;
    for( int t = 0; t < n; ++t )
    {
        double part = 0;
        for( int i = 0; i < nos; ++i )
            part += E[(size_t)t * nos + i];
        sum += part;
    }
    free( E );
    return sum;
}

/* ---------------------------------------------------------------- Philox4x32-10
 * Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11):
 * 10 rounds of (mulhilo by 0xD2511F53 / 0xCD9E8D57, xor with key) with Weyl key
 * increments 0x9E3779B9 / 0xBB67AE85.  The CUDA kernels implement the same function. */
void og_philox4x32( const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4] )
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for( int r = 0; r < 10; ++r )
    {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)( p0 >> 32 ), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)( p1 >> 32 ), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Gaussian triple for spin i at a given iteration: counter (i, iteration, stream, 0x53504E00),
 * key (seed lo, seed hi); 23-bit uniforms u = ((x >> 9) + 1/2) 2^-23 (exact in FP32 and FP64);
 * Box-Muller on (u0,u1) and (u2,u3).  The CUDA kernels use the same mapping. */
static void gauss3( uint64_t seed, uint32_t stream, uint32_t iteration, uint32_t i, double * z )
{
    uint32_t ctr[4] = { i, iteration, stream, 0x53504E00u };
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)( seed >> 32 ) };
    uint32_t x[4];
    og_philox4x32( ctr, key, x );
    const double sc = 1.0 / 8388608.0;
    double u0 = ( (double)( x[0] >> 9 ) + 0.5 ) * sc;
    double u1 = ( (double)( x[1] >> 9 ) + 0.5 ) * sc;
    double u2 = ( (double)( x[2] >> 9 ) + 0.5 ) * sc;
    double u3 = ( (double)( x[3] >> 9 ) + 0.5 ) * sc;
    double r0 = sqrt( -2.0 * log( u0 ) );
    double r1 = sqrt( -2.0 * log( u2 ) );
    z[0]      = r0 * cos( 2.0 * C_PI * u1 );
    z[1]      = r0 * sin( 2.0 * C_PI * u1 );
    z[2]      = r1 * cos( 2.0 * C_PI * u3 );
}

/* Prepare_Thermal_Field: core/src/engine/Method_LLG.cpp:65-110 (homogeneous temperature) */
void og_thermal_noise(
    const og_system * s, double temperature, double damping, double dt, uint64_t seed, uint32_t stream,
    uint32_t iteration, double * xi )
{
    double eps = sqrt( 2 * damping * dt * C_GAMMA / C_MU_B * C_K_B ) / ( 1 + damping * damping );
#pragma omp parallel for
    for( int i = 0; i < s->nos; ++i )
    {
        double z[3];
        gauss3( seed, stream, iteration, (uint32_t)i, z );
        double sc = eps * sqrt( temperature / s->mu_s[i] );
        for( int e = 0; e < 3; ++e )
            xi[3 * i + e] = sc * z[e];
    }
}

/* ---------------------------------------------------------------- LLG
 * Calculate_Force_Virtual: Method_LLG.cpp:132-226.
 *  dynamics:             fv = (dtg F + dtg a s x F) / mu_s [+ xi + a s x xi],  dtg = dt g/mu_B/(1+a^2)
 *  direct min. and VP:   fv = dt g/mu_B (s x F) */
static void force_virtual(
    const og_system * s, const og_llg_params * p, int solver, const double * spins, const double * F,
    const double * xi, double * fv )
{
    double a   = p->damping;
    double dtg = p->dt * C_GAMMA / C_MU_B / ( 1 + a * a );
    int thermal = p->temperature > 0;
    if( solver == 5 ) /* LBFGS_OSO: s x F (Method_LLG.cpp:161-164) */
    {
#pragma omp parallel for
        for( int i = 0; i < s->nos; ++i )
            cross3( spins + 3 * i, F + 3 * i, fv + 3 * i );
        return;
    }
    if( p->direct_minimization || solver == 0 || solver == 7 )
    {
        double d = p->dt * C_GAMMA / C_MU_B;
#pragma omp parallel for
        for( int i = 0; i < s->nos; ++i )
        {
            double c[3];
            cross3( spins + 3 * i, F + 3 * i, c );
            for( int e = 0; e < 3; ++e )
                fv[3 * i + e] = d * c[e];
        }
        return;
    }
#pragma omp parallel for
    for( int i = 0; i < s->nos; ++i )
    {
        const double * si = spins + 3 * i;
        double c[3];
        cross3( si, F + 3 * i, c );
        for( int e = 0; e < 3; ++e )
        {
            double v = dtg * F[3 * i + e];
            v += dtg * a * c[e];
            fv[3 * i + e] = v / s->mu_s[i];
        }
        if( thermal )
        {
            double cx[3];
            cross3( si, xi + 3 * i, cx );
            for( int e = 0; e < 3; ++e )
            {
                fv[3 * i + e] += xi[3 * i + e];
                fv[3 * i + e] += a * cx[e];
            }
        }
    }
}

/* force = -gradient (Method_LLG::Calculate_Force, 113-129) */
static double calc_force( og_system * s, const double * spins, double * F )
{
    double E = og_gradient_and_energy( s, spins, F );
    for( int k = 0; k < 3 * s->nos; ++k )
        F[k] = -F[k];
    return E;
}

/* Vectormath::rotate (Vectormath.cpp:474-479), Rodrigues */
static inline void rotate3( const double * v, const double * axis, double angle, double * out )
{
    double c = cos( angle ), sn = sin( angle );
    double ax[3];
    cross3( axis, v, ax );
    double ad = dot3( axis, v );
    double r[3];
    for( int e = 0; e < 3; ++e )
        r[e] = v[e] * c + ax[e] * sn + axis[e] * ad * ( 1 - c );
    memcpy( out, r, sizeof( r ) );
}

/* sib_transform: core/src/engine/Solver_Kernels.cpp:15-48 */
static inline void sib_transform( const double * e1, const double * f, double * o )
{
    double A[3] = { 0.5 * f[0], 0.5 * f[1], 0.5 * f[2] };
    double nA   = norm3( A );
    double detAi = 1.0 / ( 1 + pow( nA, 2.0 ) );
    double c[3];
    cross3( e1, A, c );
    double a2[3] = { e1[0] - c[0], e1[1] - c[1], e1[2] - c[2] };
    double r[3];
    r[0] = ( a2[0] * ( A[0] * A[0] + 1 ) + a2[1] * ( A[0] * A[1] - A[2] ) + a2[2] * ( A[0] * A[2] + A[1] ) ) * detAi;
    r[1] = ( a2[0] * ( A[1] * A[0] + A[2] ) + a2[1] * ( A[1] * A[1] + 1 ) + a2[2] * ( A[1] * A[2] - A[0] ) ) * detAi;
    r[2] = ( a2[0] * ( A[2] * A[0] - A[1] ) + a2[1] * ( A[2] * A[1] + A[0] ) + a2[2] * ( A[2] * A[2] + 1 ) ) * detAi;
    memcpy( o, r, sizeof( r ) );
}

/* max_i |fv_i - (fv_i . s_i) s_i|  (MaxTorque_on_Image, Method_Solver.hpp:225-230) */
static double max_torque( int nos, const double * spins, const double * fv )
{
    double m2 = 0;
#pragma omp parallel for reduction( max : m2 )
    for( int i = 0; i < nos; ++i )
    {
        const double * si = spins + 3 * i;
        double d          = dot3( fv + 3 * i, si );
        double t[3]       = { fv[3 * i] - d * si[0], fv[3 * i + 1] - d * si[1], fv[3 * i + 2] - d * si[2] };
        double n2         = dot3( t, t );
        if( n2 > m2 )
            m2 = n2;
    }
    return sqrt( m2 );
}

/* One iteration per solver: Solver_SIB.hpp:21-50, Solver_Depondt.hpp:28-77,
 * Solver_Heun.hpp:29-80, Solver_RK4.hpp:40-147.  Returns the energy of the last force call. */
static double llg_iteration(
    og_system * s, const og_llg_params * p, int solver, double * spins, const double * xi, double * fv1,
    double * work )
{
    int nos    = s->nos;
    size_t n3  = (size_t)3 * nos;
    double * F  = work;
    double * fv = work + n3;
    double * pr = work + 2 * n3;
    double * t1 = work + 3 * n3;
    double * k1 = work + 4 * n3;
    double * k2 = work + 5 * n3;
    double * k3 = work + 6 * n3;
    double E    = calc_force( s, spins, F );
    force_virtual( s, p, solver, spins, F, xi, fv1 );
    if( solver == 1 ) /* SIB */
    {
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            sib_transform( spins + 3 * i, fv1 + 3 * i, pr + 3 * i );
            for( int e = 0; e < 3; ++e )
            {
                pr[3 * i + e] += spins[3 * i + e];
                pr[3 * i + e] *= 0.5;
            }
        }
        E = calc_force( s, pr, F );
        force_virtual( s, p, solver, pr, F, xi, fv );
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
            sib_transform( spins + 3 * i, fv + 3 * i, spins + 3 * i );
    }
    else if( solver == 2 ) /* Depondt */
    {
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double ax[3] = { fv1[3 * i], fv1[3 * i + 1], fv1[3 * i + 2] };
            double ang   = norm3( ax );
            normalize3( ax );
            rotate3( spins + 3 * i, ax, ang, pr + 3 * i );
        }
        E = calc_force( s, pr, F );
        force_virtual( s, p, solver, pr, F, xi, fv );
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double ax[3];
            for( int e = 0; e < 3; ++e )
            {
                ax[e] = 0.5 * fv1[3 * i + e];
                ax[e] += 0.5 * fv[3 * i + e];
            }
            double ang = norm3( ax );
            normalize3( ax );
            rotate3( spins + 3 * i, ax, ang, spins + 3 * i );
        }
    }
    else if( solver == 3 ) /* Heun */
    {
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double c[3];
            cross3( spins + 3 * i, fv1 + 3 * i, c );
            for( int e = 0; e < 3; ++e )
            {
                t1[3 * i + e] = -1 * c[e];
                pr[3 * i + e] = spins[3 * i + e] + t1[3 * i + e];
            }
            normalize3( pr + 3 * i );
        }
        E = calc_force( s, pr, F );
        force_virtual( s, p, solver, pr, F, xi, fv );
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double c[3], t[3];
            cross3( pr + 3 * i, fv + 3 * i, c );
            for( int e = 0; e < 3; ++e )
            {
                t[e] = t1[3 * i + e] * 0.5;
                t[e] += spins[3 * i + e];
                t[e] += 0.5 * ( -1 * c[e] );
            }
            normalize3( t );
            memcpy( spins + 3 * i, t, sizeof( t ) );
        }
    }
    else if( solver == 4 ) /* RK4 */
    {
        double * cfg   = pr;
        double * stage = t1;
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double c[3];
            cross3( spins + 3 * i, fv1 + 3 * i, c );
            for( int e = 0; e < 3; ++e )
            {
                k1[3 * i + e]  = -1 * c[e];
                cfg[3 * i + e] = spins[3 * i + e] + 0.5 * k1[3 * i + e];
            }
            normalize3( cfg + 3 * i );
        }
        double * ks[3] = { k2, k3, stage };
        const double wnext[2] = { 0.5, 1.0 };
        for( int st = 0; st < 3; ++st )
        {
            E = calc_force( s, cfg, F );
            force_virtual( s, p, solver, cfg, F, xi, fv );
            double * k = ks[st];
#pragma omp parallel for
            for( int i = 0; i < nos; ++i )
            {
                double c[3];
                cross3( cfg + 3 * i, fv + 3 * i, c );
                for( int e = 0; e < 3; ++e )
                    k[3 * i + e] = -1 * c[e];
            }
            if( st < 2 )
            {
#pragma omp parallel for
                for( int i = 0; i < nos; ++i )
                {
                    for( int e = 0; e < 3; ++e )
                        cfg[3 * i + e] = spins[3 * i + e] + wnext[st] * k[3 * i + e];
                    normalize3( cfg + 3 * i );
                }
            }
        }
#pragma omp parallel for
        for( int i = 0; i < nos; ++i )
        {
            double t[3];
            for( int e = 0; e < 3; ++e )
            {
                t[e] = spins[3 * i + e];
                t[e] += 1.0 / 6.0 * k1[3 * i + e];
                t[e] += 1.0 / 3.0 * k2[3 * i + e];
                t[e] += 1.0 / 3.0 * k3[3 * i + e];
                t[e] += 1.0 / 6.0 * stage[3 * i + e];
            }
            normalize3( t );
            memcpy( spins + 3 * i, t, sizeof( t ) );
        }
    }
    return E;
}

static double vdot( int n3, const double * a, const double * b )
{
    double r = 0;
#pragma omp parallel for reduction( + : r )
    for( int k = 0; k < n3; ++k )
        r += a[k] * b[k];
    return r;
}

/* ---------------------------------------------------------------- OSO direct minimisers
 * Orthogonal spin optimisation (A. Ivanov et al., arXiv:1904.02669) as the reference writes it,
 * in its coordinates: the "gradient" of an image is g = T (-s x f) with the signed permutation
 * T = [[0,0,1],[0,-1,0],[1,0,0]] (oso_calc_gradients, Solver_Kernels.cpp:50-60), a search
 * direction sd is applied as the rotation matrix of oso_rotate (Solver_Kernels.cpp:62-95), and
 * the step is limited to an rms angle of maxmove = pi/200 (maximum_rotation, :97-105).
 * VP_OSO: Solver_VP_OSO.hpp:28-114.  LBFGS_OSO: Solver_LBFGS_OSO.hpp:13-85 with
 * lbfgs_get_searchdir (Solver_Kernels.hpp:44-189), memory 3. */
typedef struct oso_state
{
    int noi, nos, solver;
    size_t n3;
    double *grad, *grad_pr, *v, *sd, *q;
    double *da[3], *dg[3];
    double rho[3], alpha[3];
    int local_iter;
} oso_state;

static void oso_init( oso_state * o, int solver, int noi, int nos )
{
    memset( o, 0, sizeof( *o ) );
    o->solver = solver;
    o->noi    = noi;
    o->nos    = nos;
    o->n3     = (size_t)3 * nos;
    size_t n  = noi * o->n3;
    o->grad    = (double *)calloc( n, sizeof( double ) );
    o->grad_pr = (double *)calloc( n, sizeof( double ) );
    o->v       = (double *)calloc( n, sizeof( double ) );
    o->sd      = (double *)calloc( n, sizeof( double ) );
    o->q       = (double *)calloc( n, sizeof( double ) );
    for( int k = 0; k < 3; ++k )
    {
        o->da[k] = (double *)calloc( n, sizeof( double ) );
        o->dg[k] = (double *)calloc( n, sizeof( double ) );
    }
}

static void oso_free( oso_state * o )
{
    free( o->grad );
    free( o->grad_pr );
    free( o->v );
    free( o->sd );
    free( o->q );
    for( int k = 0; k < 3; ++k )
    {
        free( o->da[k] );
        free( o->dg[k] );
    }
}

/* g = T (-s x f) */
static void oso_gradient( int nos, const double * spins, const double * f, double * g )
{
#pragma omp parallel for
    for( int i = 0; i < nos; ++i )
    {
        double c[3];
        cross3( spins + 3 * i, f + 3 * i, c );
        g[3 * i + 0] = -c[2];
        g[3 * i + 1] = c[1];
        g[3 * i + 2] = -c[0];
    }
}

static void oso_rotate( int nos, double * spins, const double * sd )
{
#pragma omp parallel for
    for( int i = 0; i < nos; ++i )
    {
        const double * d = sd + 3 * i;
        double * sp      = spins + 3 * i;
        double theta     = norm3( d );
        if( !( theta > 1.0e-20 ) )
            continue;
        double q = cos( theta ), w = 1 - q, sn = sin( theta );
        double x = -d[0] / theta, y = -d[1] / theta, z = -d[2] / theta;
        double a = -y * z * w, b = x * z * w, c = -x * y * w;
        double p1 = x * sn, p2 = y * sn, p3 = z * sn;
        double t1 = ( q + z * z * w ) * sp[0] + ( a + p1 ) * sp[1] + ( b + p2 ) * sp[2];
        double t2 = ( a - p1 ) * sp[0] + ( q + y * y * w ) * sp[1] + ( c + p3 ) * sp[2];
        double t3 = ( b - p2 ) * sp[0] + ( c - p3 ) * sp[1] + ( q + x * x * w ) * sp[2];
        sp[0] = t1;
        sp[1] = t2;
        sp[2] = t3;
    }
}

/* VP_OSO iteration on forces F (noi images) */
static void oso_vp_iteration( oso_state * o, double * chain, const double * F, double dt )
{
    const double m = 1.0;
    size_t n       = o->noi * o->n3;
    memcpy( o->grad_pr, o->grad, n * sizeof( double ) );
    for( int img = 0; img < o->noi; ++img )
    {
        double * g = o->grad + img * o->n3;
        oso_gradient( o->nos, chain + img * o->n3, F + img * o->n3, g );
        for( size_t k = 0; k < o->n3; ++k )
            g[k] *= -1.0;
    }
    double proj = 0, fn2 = 0;
    for( int img = 0; img < o->noi; ++img )
    {
        double * g  = o->grad + img * o->n3;
        double * gp = o->grad_pr + img * o->n3;
        double * v  = o->v + img * o->n3;
        for( size_t k = 0; k < o->n3; ++k )
            v[k] += 0.5 / m * ( gp[k] + g[k] );
        proj += vdot( (int)o->n3, v, g );
        fn2 += vdot( (int)o->n3, g, g );
    }
    for( int img = 0; img < o->noi; ++img )
    {
        double * g  = o->grad + img * o->n3;
        double * v  = o->v + img * o->n3;
        double * sd = o->sd + img * o->n3;
        double ratio = proj / fn2;
        if( proj <= 0 )
            memset( v, 0, o->n3 * sizeof( double ) );
        else
            for( size_t k = 0; k < o->n3; ++k )
                v[k] = g[k] * ratio;
        for( size_t k = 0; k < o->n3; ++k )
            sd[k] = dt * v[k] + 0.5 / m * dt * g[k];
    }
    for( int img = 0; img < o->noi; ++img )
        oso_rotate( o->nos, chain + img * o->n3, o->sd + img * o->n3 );
}

static double chain_dot( const oso_state * o, const double * a, const double * b )
{
    double r = 0;
    for( int img = 0; img < o->noi; ++img )
        r += vdot( (int)o->n3, a + img * o->n3, b + img * o->n3 );
    return r;
}

static void lbfgs_searchdir( oso_state * o )
{
    const int M     = 3;
    const double eps = 1e-300;
    size_t n        = o->noi * o->n3;
    int m           = o->local_iter % M;
    if( o->local_iter == 0 )
    {
        memcpy( o->grad_pr, o->grad, n * sizeof( double ) );
        for( size_t k = 0; k < n; ++k )
            o->sd[k] = -o->grad[k];
        for( int i = 0; i < M; ++i )
        {
            o->rho[i] = 0;
            memset( o->da[i], 0, n * sizeof( double ) );
            memset( o->dg[i], 0, n * sizeof( double ) );
        }
        o->local_iter++;
        return;
    }
    for( size_t k = 0; k < n; ++k )
    {
        o->da[m][k] = o->sd[k];
        o->dg[m][k] = o->grad[k] - o->grad_pr[k];
    }
    double rinv = chain_dot( o, o->dg[m], o->da[m] );
    if( rinv > eps )
        o->rho[m] = 1.0 / rinv;
    else
    {
        o->local_iter = 0;
        lbfgs_searchdir( o );
        return;
    }
    memcpy( o->q, o->grad, n * sizeof( double ) );
    for( int k = M - 1; k > -1; --k )
    {
        int c       = ( k + m + 1 ) % M;
        o->alpha[c] = o->rho[c] * chain_dot( o, o->da[c], o->q );
        for( size_t j = 0; j < n; ++j )
            o->q[j] += -o->alpha[c] * o->dg[c][j];
    }
    double dy2    = chain_dot( o, o->dg[m], o->dg[m] );
    double rhody2 = dy2 * o->rho[m];
    double inv    = rhody2 > eps ? 1.0 / rhody2 : 1.0 / eps;
    for( size_t j = 0; j < n; ++j )
        o->sd[j] = inv * o->q[j];
    for( int k = 0; k < M; ++k )
    {
        int c         = o->local_iter < M ? k : ( k + m + 1 ) % M;
        double rhopdg = o->rho[c] * chain_dot( o, o->dg[c], o->sd );
        for( size_t j = 0; j < n; ++j )
            o->sd[j] += ( o->alpha[c] - rhopdg ) * o->da[c][j];
    }
    for( size_t j = 0; j < n; ++j )
    {
        o->grad_pr[j] = o->grad[j];
        o->sd[j]      = -o->sd[j];
    }
    o->local_iter++;
}

/* LBFGS_OSO iteration on forces F */
static void oso_lbfgs_iteration( oso_state * o, double * chain, const double * F )
{
    const double maxmove = 3.14159265358979323846 / 200.0;
    for( int img = 0; img < o->noi; ++img )
        oso_gradient( o->nos, chain + img * o->n3, F + img * o->n3, o->grad + img * o->n3 );
    lbfgs_searchdir( o );
    double scaling = 1;
    for( int img = 0; img < o->noi; ++img )
    {
        double th = sqrt( vdot( (int)o->n3, o->sd + img * o->n3, o->sd + img * o->n3 ) / o->nos );
        double sc = th > maxmove ? maxmove / th : 1.0;
        scaling   = fmin( sc, scaling );
    }
    for( size_t k = 0; k < o->noi * o->n3; ++k )
        o->sd[k] *= scaling;
    for( int img = 0; img < o->noi; ++img )
        oso_rotate( o->nos, chain + img * o->n3, o->sd + img * o->n3 );
}

/* Method::Iterate (Method.cpp:57-113) + Method_LLG ctor (Method_LLG.cpp:22-63) and
 * Hook_Post_Iteration (247-301): the constructor evaluates the initial max torque, the loop
 * runs while iteration < n_iter and max_torque >= force_convergence. */
int og_llg_run(
    og_system * s, const og_llg_params * p, int solver, int n_iter, double * spins, double * energy,
    double * max_torque_out )
{
    int nos    = s->nos;
    size_t n3  = (size_t)3 * nos;
    double * work = (double *)calloc( 8 * n3, sizeof( double ) );
    double * xi   = (double *)calloc( n3, sizeof( double ) );
    double * fv1  = (double *)calloc( n3, sizeof( double ) );
    /* constructor: Prepare_Thermal_Field + force + virtual force + post hook on the initial state
     * (the constructor draws noise too; with Philox the draw is indexed, so it uses iteration
     * index 0xFFFFFFFF and never collides with the loop's draws) */
    if( p->temperature > 0 )
        og_thermal_noise( s, p->temperature, p->damping, p->dt, p->seed, p->stream, 0xFFFFFFFFu, xi );
    double E = calc_force( s, spins, work );
    force_virtual( s, p, solver, spins, work, xi, fv1 );
    double mt = max_torque( nos, spins, fv1 );
    int it    = 0;
    if( solver == 5 || solver == 7 )
    {
        /* direct minimisers: the force of the configuration before the step, its virtual force
         * (LBFGS_OSO: s x F; VP_OSO: dt gamma/mu_B s x F) for the torque after the step */
        oso_state o;
        oso_init( &o, solver, 1, nos );
        for( it = 0; it < n_iter && !( mt < p->force_convergence ); ++it )
        {
            E = calc_force( s, spins, work );
            force_virtual( s, p, solver, spins, work, xi, fv1 );
            if( solver == 7 )
                oso_vp_iteration( &o, spins, work, p->dt );
            else
                oso_lbfgs_iteration( &o, spins, work );
            mt = max_torque( nos, spins, fv1 );
        }
        oso_free( &o );
        goto done;
    }
    for( it = 0; it < n_iter && !( mt < p->force_convergence ); ++it )
    {
        if( p->temperature > 0 )
            og_thermal_noise( s, p->temperature, p->damping, p->dt, p->seed, p->stream, (uint32_t)it, xi );
        E  = llg_iteration( s, p, solver, spins, xi, fv1, work );
        mt = max_torque( nos, spins, fv1 );
    }
done:
    if( energy )
        *energy = E;
    if( max_torque_out )
        *max_torque_out = mt;
    free( work );
    free( xi );
    free( fv1 );
    return it;
}

/* ---------------------------------------------------------------- GNEB
 * Manifoldmath.cpp: project_tangential 59-64, dist_geodesic 66-72 (angle: Vectormath.cpp:434-441),
 * Geodesic_Tangent 78-113, Tangents 115-215, project_orthogonal 31-38, invert_parallel 40-47,
 * normalize 224-229.  Method_GNEB.cpp:88-357 (Calculate_Force, no spring-force ratio, no path
 * shortening, fixed endpoints), Solver_VP.hpp:28-114, Hook_Post_Iteration 411-456. */
static double dist_geodesic( int nos, const double * a, const double * b )
{
    double d = 0;
#pragma omp parallel for reduction( + : d )
    for( int i = 0; i < nos; ++i )
    {
        double r = dot3( a + 3 * i, b + 3 * i );
        r        = fmax( -1.0, fmin( 1.0, r ) );
        double ang = acos( r );
        d += pow( ang, 2 );
    }
    return sqrt( d );
}

static void project_tangential( int nos, double * v, const double * s )
{
#pragma omp parallel for
    for( int i = 0; i < nos; ++i )
    {
        double d = dot3( v + 3 * i, s + 3 * i );
        for( int e = 0; e < 3; ++e )
            v[3 * i + e] -= d * s[3 * i + e];
    }
}

static void normalize_3n( int n3, double * v )
{
    double sc = 1.0 / sqrt( vdot( n3, v, v ) );
    for( int k = 0; k < n3; ++k )
        v[k] *= sc;
}

static void geodesic_tangent( int nos, double * t, const double * im_minus, const double * im_plus, const double * mid )
{
    const double ex[3] = { 1, 0, 0 }, ey[3] = { 0, 1, 0 };
    const double epsilon = 1e-15;
#pragma omp parallel for
    for( int i = 0; i < nos; ++i )
    {
        double axis[3];
        cross3( im_plus + 3 * i, im_minus + 3 * i, axis );
        if( fabs( dot3( im_minus + 3 * i, im_plus + 3 * i ) + 1 ) < epsilon )
        {
            if( fabs( dot3( mid + 3 * i, ex ) - 1 ) > epsilon )
                memcpy( axis, ex, sizeof( axis ) );
            else
                memcpy( axis, ey, sizeof( axis ) );
        }
        cross3( mid + 3 * i, axis, t + 3 * i );
    }
    normalize_3n( 3 * nos, t );
}

static void tangents( int nos, int noi, const double * chain, const double * energies, double * tang )
{
    size_t n3 = (size_t)3 * nos;
    for( int img = 0; img < noi; ++img )
    {
        const double * im = chain + img * n3;
        double * t        = tang + img * n3;
        if( img == 0 )
            geodesic_tangent( nos, t, im, chain + n3, im );
        else if( img == noi - 1 )
            geodesic_tangent( nos, t, chain + ( img - 1 ) * n3, im, im );
        else
        {
            const double * ip = chain + ( img + 1 ) * n3;
            const double * imn = chain + ( img - 1 ) * n3;
            double Em = energies[img], Ep = energies[img + 1], En = energies[img - 1];
            double cp = 0, cm = 0; /* coefficients of t_plus and t_minus */
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
            for( size_t k = 0; k < n3; ++k )
            {
                double tp = ip[k] - im[k];
                double tm = im[k] - imn[k];
                if( cp != 0 && cm != 0 )
                {
                    double v = cp * tp;
                    v += cm * tm;
                    t[k] = v;
                }
                else if( cp != 0 )
                    t[k] = cp * tp;
                else
                    t[k] = cm * tm;
            }
            project_tangential( nos, t, im );
            normalize_3n( (int)n3, t );
        }
    }
}

/* Method_GNEB::Calculate_Force (Method_GNEB.cpp:88-357): gradient forces, energies, Rx,
 * tangents and total forces Ft (zero at the end points).  Returns 1 when two images coincide. */
static int gneb_forces(
    og_system * s, const og_gneb_params * p, int noi, const double * chain, const int * image_type, double * energies,
    double * Rx, double * Fg, double * T, double * Ft )
{
    int nos     = s->nos;
    size_t n3   = (size_t)3 * nos;
    int aborted = 0;
    for( int img = 0; img < noi; ++img )
    {
        double * g    = Fg + img * n3;
        energies[img] = og_gradient_and_energy( s, chain + img * n3, g );
        for( size_t k = 0; k < n3; ++k )
            g[k] *= -1;
        if( img == 0 )
            Rx[0] = 0;
        else
        {
            Rx[img] = Rx[img - 1] + dist_geodesic( nos, chain + img * n3, chain + ( img - 1 ) * n3 );
            if( Rx[img] - Rx[img - 1] < 1e-10 )
                aborted = 1;
        }
    }
    if( aborted )
        return 1;
    tangents( nos, noi, chain, energies, T );
    for( int img = 1; img < noi - 1; ++img )
    {
        double * g  = Fg + img * n3;
        double * t  = T + img * n3;
        double * ft = Ft + img * n3;
        project_tangential( nos, g, chain + img * n3 );
        if( image_type[img] == 1 )
        {
            double x = vdot( (int)n3, g, t );
            for( size_t k = 0; k < n3; ++k )
                g[k] -= 2 * x * t[k];
            memcpy( ft, g, sizeof( double ) * n3 );
        }
        else if( image_type[img] == 2 )
            memcpy( ft, g, sizeof( double ) * n3 );
        else if( image_type[img] == 0 )
        {
            double x = vdot( (int)n3, g, t );
            for( size_t k = 0; k < n3; ++k )
                g[k] -= x * t[k];
            double d = p->spring_constant * ( Rx[img + 1] - 2 * Rx[img] + Rx[img - 1] );
            for( size_t k = 0; k < n3; ++k )
            {
                double v = g[k];
                v += d * t[k];
                ft[k] = v;
            }
        }
        else
            memset( ft, 0, sizeof( double ) * n3 );
    }
    return 0;
}

/* max over images of max_i |P_perp F_total| (Method_GNEB::Hook_Post_Iteration, 411-430) */
static double gneb_max_torque( int nos, int noi, const double * chain, double * Ft )
{
    size_t n3 = (size_t)3 * nos;
    double mt = 0;
    for( int img = 0; img < noi; ++img )
    {
        double * ft = Ft + img * n3;
        project_tangential( nos, ft, chain + img * n3 );
        double m2 = 0;
        for( int i = 0; i < nos; ++i )
        {
            double n2 = dot3( ft + 3 * i, ft + 3 * i );
            if( n2 > m2 )
                m2 = n2;
        }
        if( sqrt( m2 ) > mt )
            mt = sqrt( m2 );
    }
    return mt;
}

int og_gneb_run_solver(
    og_system * s, const og_gneb_params * p, int solver, int noi, int n_iter, double * chain, const int * image_type,
    double * energies, double * Rx, double * max_torque_out )
{
    int nos   = s->nos;
    size_t n3 = (size_t)3 * nos;
    double * F  = (double *)calloc( noi * n3, sizeof( double ) ); /* forces (VP: F_total projected) */
    double * Fp = (double *)calloc( noi * n3, sizeof( double ) ); /* forces_previous */
    double * V  = (double *)calloc( noi * n3, sizeof( double ) );
    double * Fg = (double *)calloc( noi * n3, sizeof( double ) ); /* F_gradient */
    double * Ft = (double *)calloc( noi * n3, sizeof( double ) ); /* F_total */
    double * T  = (double *)calloc( noi * n3, sizeof( double ) );
    oso_state o;
    oso_init( &o, solver, solver == 0 ? 1 : noi, solver == 0 ? 1 : nos );
    const double m = 1.0;
    double mt      = p->force_convergence + 1.0;
    int it;
    for( it = 0; it < n_iter && !( mt < p->force_convergence ); ++it )
    {
        if( solver == 0 )
            memcpy( Fp, F, sizeof( double ) * noi * n3 );
        if( gneb_forces( s, p, noi, chain, image_type, energies, Rx, Fg, T, Ft ) )
            break;
        if( solver == 7 )
            oso_vp_iteration( &o, chain, Ft, p->dt );
        else if( solver == 5 )
            oso_lbfgs_iteration( &o, chain, Ft );
        else
        {
            for( int img = 1; img < noi - 1; ++img )
                memcpy( F + img * n3, Ft + img * n3, sizeof( double ) * n3 );
            /* Solver_VP::Iteration */
            double proj = 0, fn2 = 0;
            for( int img = 0; img < noi; ++img )
            {
                double * f  = F + img * n3;
                double * fp = Fp + img * n3;
                double * v  = V + img * n3;
                for( size_t k = 0; k < n3; ++k )
                    v[k] += 0.5 / m * ( fp[k] + f[k] );
                proj += vdot( (int)n3, v, f );
                fn2 += vdot( (int)n3, f, f );
            }
            for( int img = 0; img < noi; ++img )
            {
                double * f  = F + img * n3;
                double * v  = V + img * n3;
                double * sp = chain + img * n3;
                double ratio = proj / fn2;
                if( proj <= 0 )
                    memset( v, 0, sizeof( double ) * n3 );
                else
                    for( size_t k = 0; k < n3; ++k )
                        v[k] = f[k] * ratio;
                for( int i = 0; i < nos; ++i )
                {
                    double c[3];
                    for( int e = 0; e < 3; ++e )
                        c[e] = sp[3 * i + e] + p->dt * v[3 * i + e] + 0.5 / m * p->dt * f[3 * i + e];
                    normalize3( c );
                    memcpy( sp + 3 * i, c, sizeof( c ) );
                }
            }
            /* the post-iteration hook also projects the stored forces onto the new tangent
             * planes in place (Method_GNEB.cpp:428); VP reuses them as forces_previous */
            for( int img = 0; img < noi; ++img )
                project_tangential( nos, F + img * n3, chain + img * n3 );
        }
        mt = gneb_max_torque( nos, noi, chain, Ft );
    }
    if( max_torque_out )
        *max_torque_out = mt;
    oso_free( &o );
    free( F );
    free( Fp );
    free( V );
    free( Fg );
    free( Ft );
    free( T );
    return it;
}

int og_gneb_run(
    og_system * s, const og_gneb_params * p, int noi, int n_iter, double * chain, const int * image_type,
    double * energies, double * Rx, double * max_torque_out )
{
    return og_gneb_run_solver( s, p, 0, noi, n_iter, chain, image_type, energies, Rx, max_torque_out );
}

void og_gneb_image_types_auto( int noi, const double * E, int * type )
{
    for( int img = 1; img < noi - 1; ++img )
    {
        if( E[img - 1] < E[img] && E[img] > E[img + 1] )
            type[img] = 1;
        else if( E[img - 1] > E[img] && E[img] < E[img + 1] )
            type[img] = 2;
        else if( type[img] != 3 )
            type[img] = 0;
    }
}

/* Homogeneous_Rotation: core/src/utility/Configuration_Chain.cpp:28-75 (the antiparallel axis
 * test there is always false, so the axis is e_y for antiparallel spins; restated as is) */
void og_transition_homogeneous( int nos, int noi, double * chain, int idx_1, int idx_2 )
{
    size_t n3          = (size_t)3 * nos;
    const double * s1  = chain + idx_1 * n3;
    const double * s2  = chain + idx_2 * n3;
    const double ex[3] = { 1, 0, 0 }, ey[3] = { 0, 1, 0 };
    (void)noi;
    for( int i = 0; i < nos; ++i )
    {
        double r = dot3( s1 + 3 * i, s2 + 3 * i );
        r        = fmax( -1.0, fmin( 1.0, r ) );
        double rot_angle = acos( r );
        double axis[3];
        cross3( s1 + 3 * i, s2 + 3 * i, axis );
        normalize3( axis );
        if( fabs( rot_angle - C_PI ) < 1e-4 )
        {
            if( fabs( dot3( s1 + 3 * i, ex ) ) - 1 > 1e-4 )
                memcpy( axis, ex, sizeof( axis ) );
            else
                memcpy( axis, ey, sizeof( axis ) );
        }
        for( int img = idx_1 + 1; img < idx_2; ++img )
        {
            double * o = chain + img * n3 + 3 * i;
            if( rot_angle > 1e-8 )
            {
                double angle = rot_angle * (double)( img - idx_1 ) / (double)( idx_2 - idx_1 );
                rotate3( s1 + 3 * i, axis, angle, o );
            }
            else
                memcpy( o, s1 + 3 * i, sizeof( double ) * 3 );
        }
    }
}

/* ================================================================ Monte Carlo */
/* Neighbours of spin i over the exchange and DMI pair lists (both redundant), -1 skipped. */
static int mc_neighbours( const og_system * s, int i, int * out, int cap )
{
    int n  = 0;
    int ib = i % s->n_cell_atoms;
    for( int p = 0; p < s->n_ex && n < cap; ++p )
        if( s->ex_pairs[p].i == ib )
        {
            int j = idx_from_pair( s, i, &s->ex_pairs[p] );
            if( j >= 0 )
                out[n++] = j;
        }
    for( int p = 0; p < s->n_dmi && n < cap; ++p )
        if( s->dmi_pairs[p].i == ib )
        {
            int j = idx_from_pair( s, i, &s->dmi_pairs[p] );
            if( j >= 0 )
                out[n++] = j;
        }
    return n;
}

/* greedy colouring in spin order: the smallest colour no already coloured neighbour has */
int og_mc_colors( const og_system * s, int * colors )
{
    int nc = 0;
    int nbr[512];
    for( int i = 0; i < s->nos; ++i )
        colors[i] = -1;
    for( int i = 0; i < s->nos; ++i )
    {
        int n      = mc_neighbours( s, i, nbr, 512 );
        int c      = 0;
        int change = 1;
        while( change )
        {
            change = 0;
            for( int k = 0; k < n; ++k )
                if( nbr[k] != i && colors[nbr[k]] == c )
                {
                    ++c;
                    change = 1;
                }
        }
        colors[i] = c;
        if( c + 1 > nc )
            nc = c + 1;
    }
    return nc;
}

/* Energy_Single_Spin (Hamiltonian_Heisenberg.cpp:559-668, OpenMP build) of spin i set to v, the
 * other spins fixed: Zeeman, anisotropy, exchange and DMI pairs with pair.i == basis(i); no DDI.
 * The pair terms are written -v . h with h = sum_p (J_p s_j + D_p s_j x n_p). */
static double mc_energy_single( const og_system * s, const double * spins, int i, const double * v, const double * h )
{
    int ib   = i % s->n_cell_atoms;
    double E = 0;
    if( has_zeeman( s ) )
        E -= s->mu_s[i] * s->field_mag * dot3( s->field_normal, v );
    for( int k = 0; k < s->n_aniso; ++k )
        if( s->aniso_idx[k] == ib )
        {
            double d = dot3( s->aniso_normal[k], v );
            E -= s->aniso_mag[k] * d * d;
        }
    E -= dot3( v, h );
    (void)spins;
    return E;
}

static void mc_pair_field( const og_system * s, const double * spins, int i, double * h )
{
    int ib = i % s->n_cell_atoms;
    h[0] = h[1] = h[2] = 0;
    for( int p = 0; p < s->n_ex; ++p )
        if( s->ex_pairs[p].i == ib )
        {
            int j = idx_from_pair( s, i, &s->ex_pairs[p] );
            if( j >= 0 )
                for( int e = 0; e < 3; ++e )
                    h[e] += s->ex_mag[p] * spins[3 * j + e];
        }
    for( int p = 0; p < s->n_dmi; ++p )
        if( s->dmi_pairs[p].i == ib )
        {
            int j = idx_from_pair( s, i, &s->dmi_pairs[p] );
            if( j >= 0 )
            {
                double c[3];
                cross3( spins + 3 * j, s->dmi_normal + 3 * p, c );
                for( int e = 0; e < 3; ++e )
                    h[e] += s->dmi_mag[p] * c[e];
            }
        }
}

int og_mc_run( og_system * s, const og_mc_params * p, int n_sweeps, double * spins, double * cone_out, double * acc_out )
{
    int * colors = (int *)malloc( sizeof( int ) * (size_t)s->nos );
    int nc       = og_mc_colors( s, colors );
    double cone  = C_PI * p->cone_angle_deg / 180.0;
    double acc   = p->acceptance_target;
    long n_rej   = 0;
    const double kT  = C_K_B * p->temperature;
    const double dif = 0.01;
    uint32_t key[2]  = { (uint32_t)p->seed, (uint32_t)( p->seed >> 32 ) };
    for( int it = 0; it < n_sweeps; ++it )
    {
        /* cone angle feedback from the previous sweep's rejections (Method_MC.cpp:73-89) */
        if( p->cone && p->adaptive )
        {
            acc = 1.0 - (double)n_rej / (double)s->nos;
            if( acc < p->acceptance_target && cone > dif )
                cone -= dif;
            if( acc > p->acceptance_target && cone < C_PI - dif )
                cone += dif;
        }
        n_rej                 = 0;
        const double cos_cone = cos( cone );
        for( int c = 0; c < nc; ++c )
        {
#pragma omp parallel for reduction( + : n_rej )
            for( int i = 0; i < s->nos; ++i )
            {
                if( colors[i] != c )
                    continue;
                uint32_t ctr[4] = { (uint32_t)i, (uint32_t)it, p->stream, 0x4D435300u };
                uint32_t x[4];
                og_philox4x32( ctr, key, x );
                const double sc = 1.0 / 8388608.0;
                const double u0 = ( (double)( x[0] >> 9 ) + 0.5 ) * sc;
                const double u1 = ( (double)( x[1] >> 9 ) + 0.5 ) * sc;
                const double u2 = ( (double)( x[2] >> 9 ) + 0.5 ) * sc;
                double * so     = spins + 3 * i;
                double e0[3] = { 1, 0, 0 }, e1[3] = { 0, 1, 0 }, e2[3] = { 0, 0, 1 };
                double ct;
                if( p->cone )
                {
                    /* local basis with the spin as third axis (Method_MC.cpp:113-123) */
                    if( so[2] < 1 - 1e-10 )
                    {
                        const double ez[3] = { 0, 0, 1 };
                        e2[0] = so[0];
                        e2[1] = so[1];
                        e2[2] = so[2];
                        cross3( e2, ez, e0 );
                        normalize3( e0 );
                        cross3( e2, e0, e1 );
                    }
                    ct = 1 - ( 1 - cos_cone ) * u0;
                }
                else
                    ct = u0; /* the reference samples cos(theta) in [0, 1) here */
                const double st  = sqrt( 1 - ct * ct );
                const double phi = 2 * C_PI * u1;
                const double l[3] = { st * cos( phi ), st * sin( phi ), ct };
                double v[3];
                for( int e = 0; e < 3; ++e )
                    v[e] = e0[e] * l[0] + e1[e] * l[1] + e2[e] * l[2];
                double h[3];
                mc_pair_field( s, spins, i, h );
                const double Eold = mc_energy_single( s, spins, i, so, h );
                const double Enew = mc_energy_single( s, spins, i, v, h );
                const double dE   = Enew - Eold;
                int reject        = 0;
                if( dE > 1e-14 )
                {
                    if( p->temperature < 1e-12 )
                        reject = 1;
                    else if( exp( -dE / kT ) < u2 )
                        reject = 1;
                }
                if( reject )
                    ++n_rej;
                else
                    for( int e = 0; e < 3; ++e )
                        so[e] = v[e];
            }
        }
    }
    if( cone_out )
        *cone_out = cone * 180.0 / C_PI;
    if( acc_out )
        *acc_out = acc;
    free( colors );
    return n_sweeps;
}

/* ---------------------------------------------------------------- HTST
 * Harmonic transition-state theory prefactor (core/src/engine/HTST.cpp:29-346 dense,
 * Sparse_HTST.cpp:246-533 sparse), with Hamiltonian_Heisenberg::Hessian
 * (Hamiltonian_Heisenberg.cpp:1119-1275; the anisotropy term puts its beta sum on the diagonal as
 * the reference writes it), hessian_bordered_3N (HTST.cpp:484-503), tangent_basis_spherical
 * (Manifoldmath.cpp:254-287), Calculate_Dynamical_Matrix (HTST.cpp:425-482) and
 * Calculate_Zero_Volume (HTST.cpp:348-410).  The symmetric eigenproblems are solved by cyclic
 * Jacobi rotations; the sparse variant's log-determinants, lowest modes and linear solve are
 * evaluated from the same full decomposition (equal up to rounding). */
#define C_HBAR 0.6582119514
#define C_G_E 2.00231930436182

/* Hessian (3N x 3N row-major); the sparse variant's Sparse_Hessian (Hamiltonian_Heisenberg.cpp:
 * 1277-1371) has no dipolar block */
static void htst_hessian( const og_system * s, double * H, int with_ddi )
{
    int nos  = s->nos;
    size_t n = (size_t)3 * nos;
    int N    = s->n_cell_atoms;
    memset( H, 0, sizeof( double ) * n * n );
    for( int icell = 0; icell < s->n_cells_total; ++icell )
        for( int k = 0; k < s->n_aniso; ++k )
        {
            int i = icell * N + s->aniso_idx[k];
            for( int a = 0; a < 3; ++a )
                for( int b = 0; b < 3; ++b )
                    H[( 3 * i + a ) * n + 3 * i + a]
                        += -2.0 * s->aniso_mag[k] * s->aniso_normal[k][a] * s->aniso_normal[k][b];
        }
    for( int icell = 0; icell < s->n_cells_total; ++icell )
        for( int p = 0; p < s->n_ex; ++p )
        {
            int i = s->ex_pairs[p].i + icell * N;
            int j = idx_from_pair( s, i, &s->ex_pairs[p] );
            if( j < 0 )
                continue;
            for( int a = 0; a < 3; ++a )
                H[( 3 * i + a ) * n + 3 * j + a] += -s->ex_mag[p];
        }
    for( int icell = 0; icell < s->n_cells_total; ++icell )
        for( int p = 0; p < s->n_dmi; ++p )
        {
            int i = s->dmi_pairs[p].i + icell * N;
            int j = idx_from_pair( s, i, &s->dmi_pairs[p] );
            if( j < 0 )
                continue;
            const double d = s->dmi_mag[p], * nn = s->dmi_normal + 3 * p;
            size_t r = 3 * (size_t)i, c = 3 * (size_t)j;
            H[( r + 2 ) * n + c + 1] += d * nn[0];
            H[( r + 1 ) * n + c + 2] += -d * nn[0];
            H[( r + 0 ) * n + c + 2] += d * nn[1];
            H[( r + 2 ) * n + c + 0] += -d * nn[1];
            H[( r + 1 ) * n + c + 0] += d * nn[2];
            H[( r + 0 ) * n + c + 1] += -d * nn[2];
        }
    if( s->ddi_method != 0 && with_ddi )
    {
        const double mult = C_MU_0 * C_MU_B * C_MU_B / ( 4 * C_PI * 1e-30 );
        for( int i = 0; i < nos; ++i )
            for( int j = 0; j < nos; ++j )
            {
                double d[3];
                for( int e = 0; e < 3; ++e )
                    d[e] = s->positions[3 * j + e] - s->positions[3 * i + e];
                double r = norm3( d );
                double D[3][3] = { { 0 } };
                if( r > 1e-10 )
                {
                    double r3 = r * r * r, r5 = r3 * r * r;
                    for( int a = 0; a < 3; ++a )
                        for( int b = 0; b < 3; ++b )
                            D[a][b] = mult * ( 3 * d[a] * d[b] / r5 - ( a == b ? 1 / r3 : 0 ) );
                }
                double m = s->mu_s[i] * s->mu_s[j];
                for( int a = 0; a < 3; ++a )
                    for( int b = 0; b < 3; ++b )
                        H[( 3 * i + a ) * n + 3 * j + b] += -m * D[a][b];
            }
    }
}

/* columns 2i, 2i+1 of the tangent basis at spin i */
static void htst_basis( const double * sp, double e1[3], double e2[3] )
{
    double t1[3], t2[3];
    if( sp[2] > 1 - 1e-8 )
    {
        double a[3] = { 1, 0, 0 }, b[3] = { 0, 1, 0 };
        memcpy( t1, a, sizeof( a ) );
        memcpy( t2, b, sizeof( b ) );
    }
    else if( sp[2] < -1 + 1e-8 )
    {
        double a[3] = { 1, 0, 0 }, b[3] = { 0, -1, 0 };
        memcpy( t1, a, sizeof( a ) );
        memcpy( t2, b, sizeof( b ) );
    }
    else
    {
        double rxy = sqrt( 1 - sp[2] * sp[2] ), z = sp[2] / rxy;
        double a[3] = { sp[0] * z, sp[1] * z, -rxy }, b[3] = { -sp[1] / rxy, sp[0] / rxy, 0 };
        memcpy( t1, a, sizeof( a ) );
        memcpy( t2, b, sizeof( b ) );
    }
    double d1 = dot3( t1, sp ), d2 = dot3( t2, sp );
    for( int e = 0; e < 3; ++e )
    {
        e1[e] = t1[e] - d1 * sp[e];
        e2[e] = t2[e] - d2 * sp[e];
    }
    normalize3( e1 );
    normalize3( e2 );
}

/* out (2N x 2N) = B^T M B for a 3N x 3N row-major M */
static void htst_project( int nos, const double * B /* nos x 2 x 3 */, const double * M, double * out )
{
    size_t n3 = (size_t)3 * nos, n2 = (size_t)2 * nos;
#pragma omp parallel for
    for( int i = 0; i < nos; ++i )
        for( int j = 0; j < nos; ++j )
            for( int a = 0; a < 2; ++a )
                for( int b = 0; b < 2; ++b )
                {
                    double v = 0;
                    for( int x = 0; x < 3; ++x )
                        for( int y = 0; y < 3; ++y )
                            v += B[6 * i + 3 * a + x] * M[( 3 * i + x ) * n3 + 3 * j + y] * B[6 * j + 3 * b + y];
                    out[( 2 * i + a ) * n2 + 2 * j + b] = v;
                }
}

/* cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (destroyed); eigenvalues ascending,
 * eigenvectors as columns of V (row-major n x n) */
static void htst_eigh( int n, double * A, double * w, double * V )
{
    for( int i = 0; i < n; ++i )
        for( int j = 0; j < n; ++j )
            V[(size_t)i * n + j] = i == j;
    for( int sweep = 0; sweep < 100; ++sweep )
    {
        double off = 0, tot = 0;
        for( int i = 0; i < n; ++i )
            for( int j = 0; j < n; ++j )
            {
                double x = A[(size_t)i * n + j] * A[(size_t)i * n + j];
                tot += x;
                if( i != j )
                    off += x;
            }
        if( off <= 1e-30 * tot || off == 0 )
            break;
        for( int p = 0; p < n - 1; ++p )
            for( int q = p + 1; q < n; ++q )
            {
                double apq = A[(size_t)p * n + q];
                if( apq == 0 )
                    continue;
                double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                double th = ( aqq - app ) / ( 2 * apq );
                double t  = ( th >= 0 ? 1.0 : -1.0 ) / ( fabs( th ) + sqrt( th * th + 1 ) );
                double c = 1 / sqrt( t * t + 1 ), sn = t * c;
                for( int k = 0; k < n; ++k )
                {
                    double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - sn * akq;
                    A[(size_t)k * n + q] = sn * akp + c * akq;
                }
                for( int k = 0; k < n; ++k )
                {
                    double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - sn * aqk;
                    A[(size_t)q * n + k] = sn * apk + c * aqk;
                }
                for( int k = 0; k < n; ++k )
                {
                    double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - sn * vkq;
                    V[(size_t)k * n + q] = sn * vkp + c * vkq;
                }
            }
    }
    /* sort ascending (selection sort, swapping columns) */
    for( int i = 0; i < n; ++i )
        w[i] = A[(size_t)i * n + i];
    for( int i = 0; i < n; ++i )
    {
        int m = i;
        for( int j = i + 1; j < n; ++j )
            if( w[j] < w[m] )
                m = j;
        if( m != i )
        {
            double t = w[i];
            w[i]     = w[m];
            w[m]     = t;
            for( int k = 0; k < n; ++k )
            {
                double x             = V[(size_t)k * n + i];
                V[(size_t)k * n + i] = V[(size_t)k * n + m];
                V[(size_t)k * n + m] = x;
            }
        }
    }
}

/* geodesic (bordered, tangent-projected) Hessian of an image; returns max torque of the gradient */
static double htst_geodesic(
    og_system * s, const double * spins, double * H3, double * B, double * H2, double * g, int with_ddi )
{
    int nos  = s->nos;
    size_t n = (size_t)3 * nos;
    og_gradient( s, spins, g );
    double fm = 0;
    for( int i = 0; i < nos; ++i )
    {
        double f[3] = { g[3 * i], g[3 * i + 1], g[3 * i + 2] };
        double d    = dot3( f, spins + 3 * i );
        for( int e = 0; e < 3; ++e )
            f[e] -= d * spins[3 * i + e];
        fm = fmax( fm, norm3( f ) );
    }
    htst_hessian( s, H3, with_ddi );
    for( int i = 0; i < nos; ++i )
    {
        double u[3] = { spins[3 * i], spins[3 * i + 1], spins[3 * i + 2] };
        normalize3( u );
        double lam = dot3( u, g + 3 * i );
        for( int e = 0; e < 3; ++e )
            H3[( 3 * i + e ) * n + 3 * i + e] -= lam;
        htst_basis( spins + 3 * i, B + 6 * i, B + 6 * i + 3 );
    }
    htst_project( nos, B, H3, H2 );
    return fm;
}

/* Calculate_Zero_Volume */
static double htst_zero_volume( const og_system * s, const double * spins )
{
    int nos = s->nos, dim = 0;
    double len[3] = { 0, 0, 0 };
    double * sh   = (double *)malloc( sizeof( double ) * 3 * nos );
    for( int ib = 0; ib < 3; ++ib )
    {
        if( !( s->bc[ib] && s->n_cells[ib] > 1 ) )
            continue;
        int shift = ib == 0 ? s->n_cell_atoms
                            : ( ib == 1 ? s->n_cell_atoms * s->n_cells[0] : s->n_cell_atoms * s->n_cells[0] * s->n_cells[1] );
        for( int i = 0; i < nos; ++i )
            memcpy( sh + 3 * ( ( i + shift ) % nos ), spins + 3 * i, sizeof( double ) * 3 );
        len[ib] = dist_geodesic( nos, spins, sh );
        ++dim;
    }
    free( sh );
    double b[3][3];
    for( int k = 0; k < 3; ++k )
    {
        memcpy( b[k], s->bravais[k], sizeof( b[k] ) );
        normalize3( b[k] );
    }
    double c[3];
    cross3( b[0], b[1], c );
    if( dim == 1 )
        return len[0];
    if( dim == 2 )
        return len[0] * len[1] * norm3( c );
    if( dim == 3 )
        return len[0] * len[1] * len[2] * fabs( dot3( c, b[2] ) );
    return 1;
}

/* w = (B^T V B)^T q with V the dynamical matrix of the bordered Hessian H3 (Calculate_Dynamical_Matrix) */
static void htst_velocity_T( const og_system * s, const double * spins, const double * H3, const double * B,
                             const double * q, double * w )
{
    int nos  = s->nos;
    size_t n = (size_t)3 * nos;
    double * V = (double *)calloc( n * n, sizeof( double ) );
    for( int i = 0; i < nos; ++i )
    {
        const double * si = spins + 3 * i;
        double beff[3]    = { 0, 0, 0 };
        for( size_t c = 0; c < n; ++c )
        {
            double h[3] = { H3[( 3 * i ) * n + c], H3[( 3 * i + 1 ) * n + c], H3[( 3 * i + 2 ) * n + c] };
            V[( 3 * i ) * n + c]     = si[1] * h[2] - si[2] * h[1];
            V[( 3 * i + 1 ) * n + c] = si[2] * h[0] - si[0] * h[2];
            V[( 3 * i + 2 ) * n + c] = si[0] * h[1] - si[1] * h[0];
        }
        for( int j = 0; j < nos; ++j )
            for( int a = 0; a < 3; ++a )
                for( int b = 0; b < 3; ++b )
                    beff[a] -= H3[( 3 * i + a ) * n + 3 * j + b] * spins[3 * j + b];
        V[( 3 * i ) * n + 3 * i + 1] -= beff[2];
        V[( 3 * i ) * n + 3 * i + 2] += beff[1];
        V[( 3 * i + 1 ) * n + 3 * i] += beff[2];
        V[( 3 * i + 1 ) * n + 3 * i + 2] -= beff[0];
        V[( 3 * i + 2 ) * n + 3 * i] -= beff[1];
        V[( 3 * i + 2 ) * n + 3 * i + 1] += beff[0];
        for( int a = 0; a < 3; ++a )
            for( size_t c = 0; c < n; ++c )
                V[( 3 * i + a ) * n + c] /= s->mu_s[i];
    }
    double * V2 = (double *)malloc( sizeof( double ) * 4 * nos * nos );
    htst_project( nos, B, V, V2 );
    size_t n2 = (size_t)2 * nos;
    for( size_t c = 0; c < n2; ++c )
    {
        double x = 0;
        for( size_t r = 0; r < n2; ++r )
            x += V2[r * n2 + c] * q[r];
        w[c] = x;
    }
    free( V );
    free( V2 );
}

int og_htst(
    og_system * s, const double * spins_min, const double * spins_sp, int sparse, int n_keep, og_htst_info * info,
    double * evalues_min, double * evalues_sp, double * evectors_min, double * evectors_sp, double * velocities )
{
    const double eps = 1e-4, eps_force = 1e-8;
    int nos = s->nos, n2 = 2 * nos;
    size_t n = (size_t)3 * nos;
    memset( info, 0, sizeof( *info ) );
    if( n_keep < 0 )
        n_keep = n2;
    n_keep                  = n_keep < n2 ? n_keep : n2;
    info->n_eigenmodes_keep = sparse ? 0 : n_keep;
    double * H3 = (double *)malloc( sizeof( double ) * n * n );
    double * B  = (double *)malloc( sizeof( double ) * 6 * nos );
    double * H2 = (double *)malloc( sizeof( double ) * n2 * n2 );
    double * Q  = (double *)malloc( sizeof( double ) * n2 * n2 );
    double * ws = (double *)malloc( sizeof( double ) * n2 );
    double * wm = (double *)malloc( sizeof( double ) * n2 );
    double * g  = (double *)malloc( sizeof( double ) * n );
    double * q0 = (double *)malloc( sizeof( double ) * n2 );
    double * a  = (double *)malloc( sizeof( double ) * n2 );
    int status  = 0;
    if( htst_geodesic( s, spins_min, H3, B, H2, g, !sparse ) > eps_force )
    {
        status = 1; /* minimum not converged */
        goto out;
    }
    if( htst_geodesic( s, spins_sp, H3, B, H2, g, !sparse ) > eps_force )
    {
        status = 2; /* saddle point not converged */
        goto out;
    }
    /* saddle point (H3, B, H2 hold the saddle point's matrices) */
    htst_eigh( n2, H2, ws, Q );
    if( ws[0] > -eps )
    {
        status = 3;
        goto out;
    }
    {
        int n_neg = 0, lim = sparse ? ( n2 < 6 ? n2 : 6 ) : n2;
        for( int i = 0; i < lim; ++i )
            n_neg += ws[i] < -eps;
        if( n_neg > 1 )
        {
            status = 4;
            goto out;
        }
    }
    for( int r = 0; r < n2; ++r )
        q0[r] = Q[(size_t)r * n2];
    htst_velocity_T( s, spins_sp, H3, B, q0, a ); /* a = V2^T q0 */
    int n0_sp = 0;
    {
        int lim = sparse ? ( n2 < 6 ? n2 : 6 ) : n2;
        for( int i = 0; i < lim; ++i )
            n0_sp += fabs( ws[i] ) <= eps;
    }
    info->volume_sp = n0_sp > 0 ? htst_zero_volume( s, spins_sp ) : 1;
    if( !sparse )
    {
        /* perpendicular velocities a_k = (V2^T q0) . q_k */
        for( int k = 0; k < n2; ++k )
        {
            double x = 0;
            for( int r = 0; r < n2; ++r )
                x += a[r] * Q[(size_t)r * n2 + k];
            velocities[k] = x;
        }
        double s2 = 0;
        for( int i = n0_sp + 1; i < n2; ++i )
            s2 += velocities[i] * velocities[i] / ws[i];
        info->s = sqrt( s2 );
        memcpy( evalues_sp, ws, sizeof( double ) * n2 );
        for( int k = 0; k < n_keep; ++k )
            for( int r = 0; r < n2; ++r )
                evectors_sp[(size_t)k * n2 + r] = Q[(size_t)r * n2 + k];
    }
    else
    {
        /* s^2 = b . H^-1 b with b = V2^T q0; log|det| minus the unstable mode */
        double s2 = 0, ld = 0;
        for( int k = 0; k < n2; ++k )
        {
            double x = 0;
            for( int r = 0; r < n2; ++r )
                x += a[r] * Q[(size_t)r * n2 + k];
            s2 += x * x / ws[k];
            ld += log( fabs( ws[k] ) );
        }
        info->s      = sqrt( s2 );
        info->det_sp = ld - log( -ws[0] );
    }
    /* minimum */
    htst_geodesic( s, spins_min, H3, B, H2, g, !sparse );
    htst_eigh( n2, H2, wm, Q );
    if( !sparse && wm[0] < -eps )
    {
        status = 5;
        goto out;
    }
    int n0_min = 0;
    {
        int lim = sparse ? ( n2 < 6 ? n2 : 6 ) : n2;
        for( int i = 0; i < lim; ++i )
            n0_min += fabs( wm[i] ) <= eps;
    }
    info->volume_min = n0_min > 0 ? htst_zero_volume( s, spins_min ) : 1;
    info->temperature_exponent = 0.5 * ( n0_min - n0_sp );
    info->me                   = pow( 2 * C_PI * C_K_B, info->temperature_exponent );
    if( !sparse )
    {
        memcpy( evalues_min, wm, sizeof( double ) * n2 );
        for( int k = 0; k < n_keep; ++k )
            for( int r = 0; r < n2; ++r )
                evectors_min[(size_t)k * n2 + r] = Q[(size_t)r * n2 + k];
        double om = 1;
        if( n0_min > n0_sp + 1 )
            for( int i = n0_sp + 1; i < n0_min; ++i )
                om /= sqrt( ws[i] );
        else if( n0_min < n0_sp + 1 )
            for( int i = n0_min; i < n0_sp + 1; ++i )
                om *= sqrt( wm[i] );
        for( int i = ( n0_min > n0_sp + 1 ? n0_min : n0_sp + 1 ); i < n2; ++i )
            om *= sqrt( wm[i] / ws[i] );
        info->Omega_0 = om;
    }
    else
    {
        double ld = 0;
        for( int k = 0; k < n2; ++k )
            ld += log( fabs( wm[k] ) );
        info->det_min = ld;
        double om     = sqrt( exp( info->det_min - info->det_sp ) );
        double zf     = 1;
        for( int i = 0; i < n0_min; ++i )
            zf /= fabs( wm[i] );
        for( int i = 0; i < n0_sp; ++i )
            zf *= fabs( ws[i + 1] );
        info->Omega_0 = om * sqrt( zf );
    }
    info->prefactor_dynamical = info->me * info->volume_sp / info->volume_min * info->s;
    info->prefactor = C_G_E / ( C_HBAR * 1e-12 ) * info->Omega_0 * info->prefactor_dynamical / ( 2 * C_PI );
out:
    info->status = status;
    free( H3 );
    free( B );
    free( H2 );
    free( Q );
    free( ws );
    free( wm );
    free( g );
    free( q0 );
    free( a );
    return status;
}
