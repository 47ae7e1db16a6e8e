// Harmonic transition-state theory prefactor (HTST_Calculate; core/src/engine/HTST.cpp:29-346
// dense, Sparse_HTST.cpp:246-533 sparse), FP64 on the device.
//
// Per image (minimum, saddle point):
//   * host: the Hessian's non-zero 3x3 blocks as a CSR over spins (exchange -J I and DMI D[n]x of
//     the redundant pair lists; Hamiltonian_Heisenberg.cpp:1151-1210) and the anisotropy diagonal
//     as the reference writes it (its beta sum lands on the diagonal, :1136-1146);
//   * htst_setup: tangent basis (tangent_basis_spherical, Manifoldmath.cpp:254-287) and the
//     bordered-Hessian multipliers lambda_i = s_i . g_i (hessian_bordered_3N, HTST.cpp:484-503);
//   * htst_ddi_blocks + htst_local: the dense geodesic Hessian H2 = B^T (H - Lambda) B (2N x 2N),
//     every 2x2 block B_i^T H_ij B_j computed directly (the 3N x 3N Hessian is never stored); the
//     dipolar blocks are the direct sum of the reference's dense Hessian (no periodic images); the
//     sparse variant's Hessian has none (Sparse_Hessian, :1277-1371);
//   * jacobi_eigh: all eigenpairs by parallel cyclic Jacobi (round-robin pairing: n/2 disjoint
//     rotations per round, one launch for the rotation angles and one applying J^T A J blockwise
//     and V J), sweeps until the off-diagonal mass is below 1e-30 of the total;
//   * the saddle point's unstable mode q0 and w = V2^T q0 for the dynamical matrix
//     V = mu^-1 ([s]x H + [b]x), b = -H s (Calculate_Dynamical_Matrix, HTST.cpp:425-482), applied
//     matrix-free: (V^T u)_j = sum_i H_ji (u_i x s_i)/mu_i + (u_j x b_j)/mu_j;
//   * a = Q^T w, the perpendicular velocities (Calculate_Perpendicular_Velocity, :412-423).
// The host combines the spectra into Omega_0, s, the zero-mode volumes and the prefactor exactly
// as the reference.  The sparse variant's log-determinants, six lowest modes and the solve
// H2 x = V2^T q1 are evaluated from the same decomposition (equal up to rounding).
#include "htst.hpp"
#include "util.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace sg
{

namespace
{

constexpr double HT_PI    = 3.14159265358979323846;
constexpr double HT_MU_B  = 0.057883817555;
constexpr double HT_MU_0  = 2.0133545e-28;
constexpr double HT_K_B   = 0.08617330350;
constexpr double HT_HBAR  = 0.6582119514;
constexpr double HT_G_E   = 2.00231930436182;
constexpr double HT_EPS   = 1e-4;
constexpr double HT_FORCE = 1e-8;

struct HtDev
{
    int nos;
    const double * s;     // [nos][3]
    const double * pos;   // [nos][3]
    const double * mu;    // [nos]
    const double * B;     // [nos][2][3] tangent basis
    const double * lam;   // [nos] bordered-Hessian multipliers
    const double * diag;  // [nos][3] anisotropy diagonal
    const int * rowptr;   // CSR over spins
    const int * col;
    const double * J;     // exchange of the entry
    const double * Dv;    // [nnz][3] DMI vector of the entry
    int ddi;              // dipolar blocks present
    double ddi_mult;
};

__device__ __forceinline__ void ddi_tensor( const HtDev & d, int i, int j, double D[3][3] )
{
    double r[3] = { d.pos[3 * j] - d.pos[3 * i], d.pos[3 * j + 1] - d.pos[3 * i + 1], d.pos[3 * j + 2] - d.pos[3 * i + 2] };
    double rr   = sqrt( r[0] * r[0] + r[1] * r[1] + r[2] * r[2] );
    for( int a = 0; a < 3; ++a )
        for( int b = 0; b < 3; ++b )
            D[a][b] = 0;
    if( rr > 1e-10 )
    {
        const double r3 = rr * rr * rr, r5 = r3 * rr * rr;
        const double m  = -d.mu[i] * d.mu[j] * d.ddi_mult;
        for( int a = 0; a < 3; ++a )
            for( int b = 0; b < 3; ++b )
                D[a][b] = m * ( 3 * r[a] * r[b] / r5 - ( a == b ? 1 / r3 : 0 ) );
    }
}

// tangent basis and multipliers
__global__ void htst_setup( int nos, const double * s, const double * g, double * B, double * lam )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if( i >= nos )
        return;
    const double x = s[3 * i], y = s[3 * i + 1], z = s[3 * i + 2];
    double t1[3], t2[3];
    if( z > 1 - 1e-8 )
    {
        t1[0] = 1, t1[1] = 0, t1[2] = 0;
        t2[0] = 0, t2[1] = 1, t2[2] = 0;
    }
    else if( z < -1 + 1e-8 )
    {
        t1[0] = 1, t1[1] = 0, t1[2] = 0;
        t2[0] = 0, t2[1] = -1, t2[2] = 0;
    }
    else
    {
        const double rxy = sqrt( 1 - z * z ), zr = z / rxy;
        t1[0] = x * zr, t1[1] = y * zr, t1[2] = -rxy;
        t2[0] = -y / rxy, t2[1] = x / rxy, t2[2] = 0;
    }
    const double d1 = t1[0] * x + t1[1] * y + t1[2] * z, d2 = t2[0] * x + t2[1] * y + t2[2] * z;
    double e1[3] = { t1[0] - d1 * x, t1[1] - d1 * y, t1[2] - d1 * z };
    double e2[3] = { t2[0] - d2 * x, t2[1] - d2 * y, t2[2] - d2 * z };
    const double n1 = sqrt( e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2] );
    const double n2 = sqrt( e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2] );
    for( int c = 0; c < 3; ++c )
    {
        B[6 * i + c]     = e1[c] / n1;
        B[6 * i + 3 + c] = e2[c] / n2;
    }
    const double ns = sqrt( x * x + y * y + z * z );
    lam[i]          = ( x * g[3 * i] + y * g[3 * i + 1] + z * g[3 * i + 2] ) / ns;
}

// 2x2 block Bi^T M Bj of a 3x3 block M
__device__ __forceinline__ void project_block( const double * Bi, const double M[3][3], const double * Bj, double out[2][2] )
{
    for( int a = 0; a < 2; ++a )
    {
        double t[3];
        for( int y = 0; y < 3; ++y )
            t[y] = Bi[3 * a] * M[0][y] + Bi[3 * a + 1] * M[1][y] + Bi[3 * a + 2] * M[2][y];
        for( int b = 0; b < 2; ++b )
            out[a][b] = t[0] * Bj[3 * b] + t[1] * Bj[3 * b + 1] + t[2] * Bj[3 * b + 2];
    }
}

// dipolar 2x2 blocks of every spin pair (i, j): one thread per block; writes (not adds) the block
__global__ void htst_ddi_blocks( HtDev d, double * H2 )
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = d.nos;
    if( t >= n * n )
        return;
    const int i = (int)( t / n ), j = (int)( t % n );
    double D[3][3], o[2][2];
    ddi_tensor( d, i, j, D );
    project_block( d.B + 6 * i, D, d.B + 6 * j, o );
    const size_t n2 = 2 * (size_t)n;
    H2[( 2 * (size_t)i ) * n2 + 2 * j]         = o[0][0];
    H2[( 2 * (size_t)i ) * n2 + 2 * j + 1]     = o[0][1];
    H2[( 2 * (size_t)i + 1 ) * n2 + 2 * j]     = o[1][0];
    H2[( 2 * (size_t)i + 1 ) * n2 + 2 * j + 1] = o[1][1];
}

// neighbour and diagonal blocks of row block i (one thread per spin: it alone writes row block i)
__global__ void htst_local( HtDev d, double * H2 )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if( i >= d.nos )
        return;
    const size_t n2 = 2 * (size_t)d.nos;
    double M[3][3], o[2][2];
    for( int e = d.rowptr[i]; e < d.rowptr[i + 1]; ++e )
    {
        const int j = d.col[e];
        const double J = d.J[e], * v = d.Dv + 3 * e;
        M[0][0] = -J, M[0][1] = -v[2], M[0][2] = v[1];
        M[1][0] = v[2], M[1][1] = -J, M[1][2] = -v[0];
        M[2][0] = -v[1], M[2][1] = v[0], M[2][2] = -J;
        project_block( d.B + 6 * i, M, d.B + 6 * j, o );
        for( int a = 0; a < 2; ++a )
            for( int b = 0; b < 2; ++b )
                H2[( 2 * (size_t)i + a ) * n2 + 2 * j + b] += o[a][b];
    }
    for( int a = 0; a < 3; ++a )
        for( int b = 0; b < 3; ++b )
            M[a][b] = a == b ? d.diag[3 * i + a] - d.lam[i] : 0;
    project_block( d.B + 6 * i, M, d.B + 6 * i, o );
    for( int a = 0; a < 2; ++a )
        for( int b = 0; b < 2; ++b )
            H2[( 2 * (size_t)i + a ) * n2 + 2 * i + b] += o[a][b];
}

// y = (H - Lambda) x in the 3N representation, matrix-free
__global__ void htst_hmat( HtDev d, const double * x, double * y )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if( i >= d.nos )
        return;
    double r[3];
    for( int a = 0; a < 3; ++a )
        r[a] = ( d.diag[3 * i + a] - d.lam[i] ) * x[3 * i + a];
    for( int e = d.rowptr[i]; e < d.rowptr[i + 1]; ++e )
    {
        const int j       = d.col[e];
        const double J    = d.J[e], * v = d.Dv + 3 * e;
        const double * xj = x + 3 * j;
        // (-J I + [v]x) xj
        r[0] += -J * xj[0] + v[1] * xj[2] - v[2] * xj[1];
        r[1] += -J * xj[1] + v[2] * xj[0] - v[0] * xj[2];
        r[2] += -J * xj[2] + v[0] * xj[1] - v[1] * xj[0];
    }
    if( d.ddi )
        for( int j = 0; j < d.nos; ++j )
        {
            double D[3][3];
            ddi_tensor( d, i, j, D );
            for( int a = 0; a < 3; ++a )
                r[a] += D[a][0] * x[3 * j] + D[a][1] * x[3 * j + 1] + D[a][2] * x[3 * j + 2];
        }
    for( int a = 0; a < 3; ++a )
        y[3 * i + a] = r[a];
}

// u = B q (2N -> 3N) and c_i = (u_i x s_i) / mu_i
__global__ void htst_lift( HtDev d, const double * q, double * u, double * c )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if( i >= d.nos )
        return;
    const double * Bi = d.B + 6 * i;
    double v[3];
    for( int a = 0; a < 3; ++a )
        v[a] = Bi[a] * q[2 * i] + Bi[3 + a] * q[2 * i + 1];
    const double * s = d.s + 3 * i;
    const double m   = d.mu[i];
    for( int a = 0; a < 3; ++a )
        u[3 * i + a] = v[a];
    c[3 * i]     = ( v[1] * s[2] - v[2] * s[1] ) / m;
    c[3 * i + 1] = ( v[2] * s[0] - v[0] * s[2] ) / m;
    c[3 * i + 2] = ( v[0] * s[1] - v[1] * s[0] ) / m;
}

// w = B^T ( y + (u x b)/mu ) with b = -Hs  (hs = (H - Lambda) s)
__global__ void htst_velocity( HtDev d, const double * y, const double * u, const double * hs, double * w )
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if( j >= d.nos )
        return;
    const double * uj = u + 3 * j;
    const double b[3] = { -hs[3 * j], -hs[3 * j + 1], -hs[3 * j + 2] };
    const double m    = d.mu[j];
    double r[3]       = { y[3 * j] + ( uj[1] * b[2] - uj[2] * b[1] ) / m, y[3 * j + 1] + ( uj[2] * b[0] - uj[0] * b[2] ) / m,
                    y[3 * j + 2] + ( uj[0] * b[1] - uj[1] * b[0] ) / m };
    const double * Bj = d.B + 6 * j;
    w[2 * j]          = Bj[0] * r[0] + Bj[1] * r[1] + Bj[2] * r[2];
    w[2 * j + 1]      = Bj[3] * r[0] + Bj[4] * r[1] + Bj[5] * r[2];
}

// a_k = sum_r V[r][k] w[r]
__global__ void htst_gemv_t( const double * V, const double * w, double * a, int n )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if( k >= n )
        return;
    double x = 0;
    for( int r = 0; r < n; ++r )
        x += V[(size_t)r * n + k] * w[r];
    a[k] = x;
}

// ---------------------------------------------------------------- Jacobi
struct Rot
{
    int p, q;
    double c, s;
};

// round-robin pairing of round r: (r, n-1) and ((r+k) mod (n-1), (r-k) mod (n-1)), k = 1..n/2-1
__device__ __forceinline__ void pair_of( int r, int k, int n, int & p, int & q )
{
    const int m = n - 1;
    int a, b;
    if( k == 0 )
    {
        a = r % m;
        b = m;
    }
    else
    {
        a = ( r + k ) % m;
        b = ( r - k + m ) % m;
    }
    p = a < b ? a : b;
    q = a < b ? b : a;
}

__global__ void jac_params( const double * A, int n, int r, Rot * rot )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if( k >= n / 2 )
        return;
    int p, q;
    pair_of( r, k, n, p, q );
    const double apq = A[(size_t)p * n + q];
    double c = 1, s = 0;
    if( apq != 0 )
    {
        const double th = ( A[(size_t)q * n + q] - A[(size_t)p * n + p] ) / ( 2 * apq );
        double t;
        if( fabs( th ) > 1e150 )
            t = 0.5 / th;
        else
            t = ( th >= 0 ? 1.0 : -1.0 ) / ( fabs( th ) + sqrt( th * th + 1 ) );
        c = 1 / sqrt( t * t + 1 );
        s = t * c;
    }
    rot[k] = { p, q, c, s };
}

// A <- J^T A J (one thread per 2x2 block of two pairs), V <- V J (one thread per row and pair)
__global__ void jac_apply( double * A, double * V, int n, const Rot * rot )
{
    const long long h  = n / 2;
    const long long nb = h * h;
    const long long t  = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if( t < nb )
    {
        const Rot rk = rot[t / h], rl = rot[t % h];
        double * a00 = A + (size_t)rk.p * n + rl.p;
        double * a01 = A + (size_t)rk.p * n + rl.q;
        double * a10 = A + (size_t)rk.q * n + rl.p;
        double * a11 = A + (size_t)rk.q * n + rl.q;
        const double m00 = *a00, m01 = *a01, m10 = *a10, m11 = *a11;
        const double t00 = rk.c * m00 - rk.s * m10, t01 = rk.c * m01 - rk.s * m11;
        const double t10 = rk.s * m00 + rk.c * m10, t11 = rk.s * m01 + rk.c * m11;
        *a00 = t00 * rl.c - t01 * rl.s;
        *a01 = t00 * rl.s + t01 * rl.c;
        *a10 = t10 * rl.c - t11 * rl.s;
        *a11 = t10 * rl.s + t11 * rl.c;
        if( t / h == t % h )
        {
            *a01 = 0;
            *a10 = 0;
        }
        return;
    }
    const long long u = t - nb;
    if( u >= (long long)n * h )
        return;
    const long long row = u / h;
    const Rot rk        = rot[u % h];
    double * vp         = V + (size_t)row * n + rk.p;
    double * vq         = V + (size_t)row * n + rk.q;
    const double x = *vp, y = *vq;
    *vp = rk.c * x - rk.s * y;
    *vq = rk.s * x + rk.c * y;
}

// off-diagonal and total squared sums
__global__ void jac_norms( const double * A, int n, double * out )
{
    __shared__ double so[32], st[32];
    const long long nn = (long long)n * n;
    double o = 0, tt = 0;
    for( long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x )
    {
        const double x = A[e] * A[e];
        tt += x;
        if( e / n != e % n )
            o += x;
    }
    for( int s = 16; s > 0; s >>= 1 )
    {
        o += __shfl_xor_sync( 0xffffffffu, o, s );
        tt += __shfl_xor_sync( 0xffffffffu, tt, s );
    }
    if( ( threadIdx.x & 31 ) == 0 )
    {
        so[threadIdx.x >> 5] = o;
        st[threadIdx.x >> 5] = tt;
    }
    __syncthreads();
    if( threadIdx.x == 0 )
    {
        double a = 0, b = 0;
        for( int w = 0; w < (int)( blockDim.x >> 5 ); ++w )
        {
            a += so[w];
            b += st[w];
        }
        atomicAdd( out, a );
        atomicAdd( out + 1, b );
    }
}

__global__ void set_identity( double * V, int n )
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if( t < (long long)n * n )
        V[t] = ( t / n == t % n ) ? 1.0 : 0.0;
}

__global__ void get_diag( const double * A, int n, double * w )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if( k < n )
        w[k] = A[(size_t)k * n + k];
}

int blocks_for( long long n, int t )
{
    return (int)( ( n + t - 1 ) / t );
}

// one image's device data
struct HtImage
{
    int nos = 0;
    double *s = nullptr, *g = nullptr, *pos = nullptr, *mu = nullptr, *B = nullptr, *lam = nullptr, *diag = nullptr;
    int *rowptr = nullptr, *col = nullptr;
    double *J = nullptr, *Dv = nullptr;
    HtDev dev{};
    ~HtImage()
    {
        dfree( s );
        dfree( g );
        dfree( pos );
        dfree( mu );
        dfree( B );
        dfree( lam );
        dfree( diag );
        dfree( rowptr );
        dfree( col );
        dfree( J );
        dfree( Dv );
    }
};

void build_image( HtImage & im, const Geometry & g, const HamiltonianParams & h, const std::vector<double> & spins,
                  const std::vector<double> & grad, bool with_ddi, cudaStream_t st )
{
    const int nos = g.nos(), nb = g.nb();
    im.nos        = nos;
    // CSR of the neighbour blocks, in the order of the redundant pair lists
    std::vector<std::vector<std::pair<int, std::array<double, 4>>>> rows( nos );
    for( int i = 0; i < nos; ++i )
    {
        for( size_t p = 0; p < h.ex_pairs.size(); ++p )
            if( h.ex_pairs[p].i == i % nb )
            {
                int j = idx_from_pair( g, h.bc, i, h.ex_pairs[p] );
                if( j >= 0 )
                    rows[i].push_back( { j, { h.ex_J[p], 0, 0, 0 } } );
            }
        for( size_t p = 0; p < h.dmi_pairs.size(); ++p )
            if( h.dmi_pairs[p].i == i % nb )
            {
                int j = idx_from_pair( g, h.bc, i, h.dmi_pairs[p] );
                if( j >= 0 )
                    rows[i].push_back( { j, { 0, h.dmi_D[p] * h.dmi_n[p][0], h.dmi_D[p] * h.dmi_n[p][1],
                                              h.dmi_D[p] * h.dmi_n[p][2] } } );
            }
    }
    std::vector<int> rowptr( nos + 1, 0 ), col;
    std::vector<double> J, Dv;
    for( int i = 0; i < nos; ++i )
    {
        for( auto & e : rows[i] )
        {
            col.push_back( e.first );
            J.push_back( e.second[0] );
            Dv.push_back( e.second[1] );
            Dv.push_back( e.second[2] );
            Dv.push_back( e.second[3] );
        }
        rowptr[i + 1] = (int)col.size();
    }
    // anisotropy diagonal (Hamiltonian_Heisenberg.cpp:1136-1146)
    std::vector<double> diag( 3 * (size_t)nos, 0.0 );
    for( int i = 0; i < nos; ++i )
        for( size_t k = 0; k < h.aniso_idx.size(); ++k )
            if( h.aniso_idx[k] == i % nb )
            {
                const Vec3 & n = h.aniso_n[k];
                for( int a = 0; a < 3; ++a )
                    for( int b = 0; b < 3; ++b )
                        diag[3 * i + a] += -2.0 * h.aniso_K[k] * n[a] * n[b];
            }
    std::vector<double> pos( 3 * (size_t)nos ), mu( nos );
    auto P = g.positions();
    for( int i = 0; i < nos; ++i )
    {
        for( int a = 0; a < 3; ++a )
            pos[3 * i + a] = P[i][a];
        mu[i] = g.mu_s( i );
    }
    im.s      = dalloc<double>( 3 * (size_t)nos );
    im.g      = dalloc<double>( 3 * (size_t)nos );
    im.pos    = dalloc<double>( 3 * (size_t)nos );
    im.mu     = dalloc<double>( nos );
    im.B      = dalloc<double>( 6 * (size_t)nos );
    im.lam    = dalloc<double>( nos );
    im.diag   = dalloc<double>( 3 * (size_t)nos );
    im.rowptr = dalloc<int>( nos + 1 );
    im.col    = dalloc<int>( std::max<size_t>( col.size(), 1 ) );
    im.J      = dalloc<double>( std::max<size_t>( J.size(), 1 ) );
    im.Dv     = dalloc<double>( std::max<size_t>( Dv.size(), 1 ) );
    h2d( im.s, spins.data(), spins.size() );
    h2d( im.g, grad.data(), grad.size() );
    h2d( im.pos, pos.data(), pos.size() );
    h2d( im.mu, mu.data(), mu.size() );
    h2d( im.diag, diag.data(), diag.size() );
    h2d( im.rowptr, rowptr.data(), rowptr.size() );
    if( !col.empty() )
    {
        h2d( im.col, col.data(), col.size() );
        h2d( im.J, J.data(), J.size() );
        h2d( im.Dv, Dv.data(), Dv.size() );
    }
    htst_setup<<<blocks_for( nos, 128 ), 128, 0, st>>>( nos, im.s, im.g, im.B, im.lam );
    CUDA_CHECK( cudaGetLastError() );
    im.dev = { nos,    im.s,      im.pos, im.mu, im.B, im.lam, im.diag, im.rowptr, im.col,
               im.J,   im.Dv,     ( with_ddi && h.ddi_method != 0 ) ? 1 : 0,
               HT_MU_0 * HT_MU_B * HT_MU_B / ( 4 * HT_PI * 1e-30 ) };
}

void assemble( const HtImage & im, double * H2, cudaStream_t st )
{
    const long long n = im.nos;
    if( im.dev.ddi )
        htst_ddi_blocks<<<blocks_for( n * n, 256 ), 256, 0, st>>>( im.dev, H2 );
    else
        CUDA_CHECK( cudaMemsetAsync( H2, 0, sizeof( double ) * 4 * n * n, st ) );
    htst_local<<<blocks_for( n, 128 ), 128, 0, st>>>( im.dev, H2 );
    CUDA_CHECK( cudaGetLastError() );
}

double max_torque( const std::vector<double> & s, const std::vector<double> & g )
{
    double m = 0;
    for( size_t i = 0; i + 2 < s.size(); i += 3 )
    {
        const double d = s[i] * g[i] + s[i + 1] * g[i + 1] + s[i + 2] * g[i + 2];
        const double f[3] = { g[i] - d * s[i], g[i + 1] - d * s[i + 1], g[i + 2] - d * s[i + 2] };
        m = std::max( m, std::sqrt( f[0] * f[0] + f[1] * f[1] + f[2] * f[2] ) );
    }
    return m;
}

// Calculate_Zero_Volume (HTST.cpp:348-410)
double zero_volume( const Geometry & g, const std::array<int, 3> & bc, const std::vector<double> & s )
{
    const int nos = g.nos();
    int dim       = 0;
    double len[3] = { 0, 0, 0 };
    std::vector<double> sh( s.size() );
    for( int ib = 0; ib < 3; ++ib )
    {
        if( !( bc[ib] && g.n_cells[ib] > 1 ) )
            continue;
        const int shift = ib == 0 ? g.nb() : ( ib == 1 ? g.nb() * g.n_cells[0] : g.nb() * g.n_cells[0] * g.n_cells[1] );
        for( int i = 0; i < nos; ++i )
            for( int a = 0; a < 3; ++a )
                sh[3 * ( ( i + shift ) % nos ) + a] = s[3 * i + a];
        double d = 0;
        for( int i = 0; i < nos; ++i )
        {
            double r = s[3 * i] * sh[3 * i] + s[3 * i + 1] * sh[3 * i + 1] + s[3 * i + 2] * sh[3 * i + 2];
            r        = std::max( -1.0, std::min( 1.0, r ) );
            d += std::pow( std::acos( r ), 2 );
        }
        len[ib] = std::sqrt( d );
        ++dim;
    }
    Vec3 b[3];
    for( int k = 0; k < 3; ++k )
    {
        b[k]           = g.bravais[k];
        const double n = std::sqrt( b[k][0] * b[k][0] + b[k][1] * b[k][1] + b[k][2] * b[k][2] );
        for( int a = 0; a < 3; ++a )
            b[k][a] /= n;
    }
    const Vec3 c = { b[0][1] * b[1][2] - b[0][2] * b[1][1], b[0][2] * b[1][0] - b[0][0] * b[1][2],
                     b[0][0] * b[1][1] - b[0][1] * b[1][0] };
    if( dim == 1 )
        return len[0];
    if( dim == 2 )
        return len[0] * len[1] * std::sqrt( c[0] * c[0] + c[1] * c[1] + c[2] * c[2] );
    if( dim == 3 )
        return len[0] * len[1] * len[2] * std::fabs( c[0] * b[2][0] + c[1] * b[2][1] + c[2] * b[2][2] );
    return 1;
}

// eigen-decomposition of an image's geodesic Hessian: ascending eigenvalues, the permutation to
// the columns of d_V
struct Spectrum
{
    std::vector<double> w;
    std::vector<int> order;
};

Spectrum decompose( double * d_A, double * d_V, int n, cudaStream_t st, int & sweeps )
{
    sweeps += jacobi_eigh( d_A, d_V, n, st );
    double * d_w = dalloc<double>( n );
    get_diag<<<blocks_for( n, 256 ), 256, 0, st>>>( d_A, n, d_w );
    std::vector<double> w( n );
    CUDA_CHECK( cudaMemcpyAsync( w.data(), d_w, sizeof( double ) * n, cudaMemcpyDeviceToHost, st ) );
    CUDA_CHECK( cudaStreamSynchronize( st ) );
    dfree( d_w );
    Spectrum S;
    S.order.resize( n );
    std::iota( S.order.begin(), S.order.end(), 0 );
    std::stable_sort( S.order.begin(), S.order.end(), [&]( int a, int b ) { return w[a] < w[b]; } );
    S.w.resize( n );
    for( int k = 0; k < n; ++k )
        S.w[k] = w[S.order[k]];
    return S;
}

// columns `order[0..k)` of the row-major n x n d_V as [k][n]
std::vector<double> columns( const double * d_V, int n, const std::vector<int> & order, int k, cudaStream_t st )
{
    std::vector<double> V( (size_t)n * n ), out( (size_t)k * n );
    CUDA_CHECK( cudaMemcpyAsync( V.data(), d_V, sizeof( double ) * V.size(), cudaMemcpyDeviceToHost, st ) );
    CUDA_CHECK( cudaStreamSynchronize( st ) );
    for( int c = 0; c < k; ++c )
        for( int r = 0; r < n; ++r )
            out[(size_t)c * n + r] = V[(size_t)r * n + order[c]];
    return out;
}

} // namespace

int jacobi_eigh( double * d_A, double * d_V, int n, cudaStream_t st )
{
    if( n % 2 )
        throw std::runtime_error( "jacobi_eigh: the matrix order must be even" );
    Rot * d_rot   = dalloc<Rot>( n / 2 );
    double * d_nr = dalloc<double>( 2 );
    set_identity<<<blocks_for( (long long)n * n, 256 ), 256, 0, st>>>( d_V, n );
    const long long work = (long long)( n / 2 ) * ( n / 2 ) + (long long)n * ( n / 2 );
    int sweep            = 0;
    for( ; sweep < 60; ++sweep )
    {
        CUDA_CHECK( cudaMemsetAsync( d_nr, 0, 2 * sizeof( double ), st ) );
        jac_norms<<<std::min( 1024, blocks_for( (long long)n * n, 256 ) ), 256, 0, st>>>( d_A, n, d_nr );
        double nr[2];
        CUDA_CHECK( cudaMemcpyAsync( nr, d_nr, sizeof( nr ), cudaMemcpyDeviceToHost, st ) );
        CUDA_CHECK( cudaStreamSynchronize( st ) );
        if( nr[0] == 0 || nr[0] <= 1e-30 * nr[1] )
            break;
        for( int r = 0; r < n - 1; ++r )
        {
            jac_params<<<blocks_for( n / 2, 128 ), 128, 0, st>>>( d_A, n, r, d_rot );
            jac_apply<<<blocks_for( work, 256 ), 256, 0, st>>>( d_A, d_V, n, d_rot );
        }
        CUDA_CHECK( cudaGetLastError() );
    }
    dfree( d_rot );
    dfree( d_nr );
    return sweep;
}

HtstResult htst_calculate( const Geometry & g, const HamiltonianParams & h_min, const std::vector<double> & spins_min,
                           const std::vector<double> & grad_min, const HamiltonianParams & h_sp,
                           const std::vector<double> & spins_sp, const std::vector<double> & grad_sp, bool sparse,
                           int n_keep, cudaStream_t st )
{
    HtstResult R;
    R.sparse     = sparse;
    const int nos = g.nos(), n2 = 2 * nos;
    if( n_keep < 0 )
        n_keep = n2;
    n_keep   = std::min( n_keep, n2 );
    R.n_keep = sparse ? 0 : n_keep;
    if( max_torque( spins_min, grad_min ) > HT_FORCE )
    {
        R.status = 1;
        return R;
    }
    if( max_torque( spins_sp, grad_sp ) > HT_FORCE )
    {
        R.status = 2;
        return R;
    }
    const int lim = sparse ? std::min( n2, 6 ) : n2; // modes the checks look at (Spectra: 6 lowest)
    double * d_A  = dalloc<double>( (size_t)n2 * n2 );
    double * d_V  = dalloc<double>( (size_t)n2 * n2 );
    // ---- saddle point
    HtImage sp;
    build_image( sp, g, h_sp, spins_sp, grad_sp, !sparse, st );
    assemble( sp, d_A, st );
    Spectrum Ss = decompose( d_A, d_V, n2, st, R.sweeps );
    const auto & ws = Ss.w;
    int n_neg       = 0;
    for( int i = 0; i < lim; ++i )
        n_neg += ws[i] < -HT_EPS;
    if( ws[0] > -HT_EPS || n_neg > 1 )
    {
        R.status = ws[0] > -HT_EPS ? 3 : 4;
        dfree( d_A );
        dfree( d_V );
        return R;
    }
    // w = V2^T q0, a = Q^T w (unsorted order)
    std::vector<double> a( n2 );
    {
        double *d_q = dalloc<double>( n2 ), *d_u = dalloc<double>( 3 * (size_t)nos ), *d_c = dalloc<double>( 3 * (size_t)nos );
        double *d_y = dalloc<double>( 3 * (size_t)nos ), *d_hs = dalloc<double>( 3 * (size_t)nos );
        double *d_w = dalloc<double>( n2 ), *d_a = dalloc<double>( n2 );
        std::vector<double> q0 = columns( d_V, n2, Ss.order, 1, st );
        h2d( d_q, q0.data(), n2 );
        const int nb = blocks_for( nos, 128 );
        htst_lift<<<nb, 128, 0, st>>>( sp.dev, d_q, d_u, d_c );
        htst_hmat<<<nb, 128, 0, st>>>( sp.dev, d_c, d_y );
        htst_hmat<<<nb, 128, 0, st>>>( sp.dev, sp.s, d_hs );
        htst_velocity<<<nb, 128, 0, st>>>( sp.dev, d_y, d_u, d_hs, d_w );
        htst_gemv_t<<<blocks_for( n2, 128 ), 128, 0, st>>>( d_V, d_w, d_a, n2 );
        CUDA_CHECK( cudaGetLastError() );
        std::vector<double> au( n2 );
        CUDA_CHECK( cudaMemcpyAsync( au.data(), d_a, sizeof( double ) * n2, cudaMemcpyDeviceToHost, st ) );
        CUDA_CHECK( cudaStreamSynchronize( st ) );
        for( int k = 0; k < n2; ++k )
            a[k] = au[Ss.order[k]];
        for( double * p : { d_q, d_u, d_c, d_y, d_hs, d_w, d_a } )
            dfree( p );
    }
    int n0_sp = 0;
    for( int i = 0; i < lim; ++i )
        n0_sp += std::fabs( ws[i] ) <= HT_EPS;
    R.volume_sp = n0_sp > 0 ? zero_volume( g, h_sp.bc, spins_sp ) : 1;
    if( !sparse )
    {
        R.velocities = a;
        double s2    = 0;
        for( int i = n0_sp + 1; i < n2; ++i )
            s2 += a[i] * a[i] / ws[i];
        R.s           = std::sqrt( s2 );
        R.evalues_sp  = ws;
        R.evectors_sp = columns( d_V, n2, Ss.order, n_keep, st );
    }
    else
    {
        double s2 = 0, ld = 0;
        for( int k = 0; k < n2; ++k )
        {
            s2 += a[k] * a[k] / ws[k];
            ld += std::log( std::fabs( ws[k] ) );
        }
        R.s      = std::sqrt( s2 );
        R.det_sp = ld - std::log( -ws[0] );
    }
    // ---- minimum
    HtImage mn;
    build_image( mn, g, h_min, spins_min, grad_min, !sparse, st );
    assemble( mn, d_A, st );
    Spectrum Sm = decompose( d_A, d_V, n2, st, R.sweeps );
    const auto & wm = Sm.w;
    if( !sparse && wm[0] < -HT_EPS )
    {
        R.status = 5;
        dfree( d_A );
        dfree( d_V );
        return R;
    }
    int n0_min = 0;
    for( int i = 0; i < lim; ++i )
        n0_min += std::fabs( wm[i] ) <= HT_EPS;
    R.volume_min           = n0_min > 0 ? zero_volume( g, h_min.bc, spins_min ) : 1;
    R.temperature_exponent = 0.5 * ( n0_min - n0_sp );
    R.me                   = std::pow( 2 * HT_PI * HT_K_B, R.temperature_exponent );
    if( !sparse )
    {
        R.evalues_min  = wm;
        R.evectors_min = columns( d_V, n2, Sm.order, n_keep, st );
        double om      = 1;
        if( n0_min > n0_sp + 1 )
            for( int i = n0_sp + 1; i < n0_min; ++i )
                om /= std::sqrt( ws[i] );
        else if( n0_min < n0_sp + 1 )
            for( int i = n0_min; i < n0_sp + 1; ++i )
                om *= std::sqrt( wm[i] );
        for( int i = std::max( n0_min, n0_sp + 1 ); i < n2; ++i )
            om *= std::sqrt( wm[i] / ws[i] );
        R.Omega_0 = om;
    }
    else
    {
        double ld = 0;
        for( int k = 0; k < n2; ++k )
            ld += std::log( std::fabs( wm[k] ) );
        R.det_min = ld;
        double zf = 1;
        for( int i = 0; i < n0_min; ++i )
            zf /= std::fabs( wm[i] );
        for( int i = 0; i < n0_sp; ++i )
            zf *= std::fabs( ws[i + 1] );
        R.Omega_0 = std::sqrt( std::exp( R.det_min - R.det_sp ) ) * std::sqrt( zf );
    }
    R.prefactor_dynamical = R.me * R.volume_sp / R.volume_min * R.s;
    R.prefactor           = HT_G_E / ( HT_HBAR * 1e-12 ) * R.Omega_0 * R.prefactor_dynamical / ( 2 * HT_PI );
    R.status              = 0;
    dfree( d_A );
    dfree( d_V );
    return R;
}

} // namespace sg
