// Shared host/device definitions of the GB300 spin-dynamics engine.
//
// Device data layout (HBM): a "batch" holds any number of independent spin systems
// (ensemble members, parameter sweeps, GNEB images).  Spins are stored structure-of-arrays,
// one component array per direction (x[], y[], z[]), each system occupying the range
// [spin_offset, spin_offset + nos) of every component array; spin_offset is a multiple of
// 32 so every system starts on a 128-byte boundary.  Inside a system the spin index is the
// reference's ispin = ib + nb * (a + Na * (b + Nb * c)) (core/include/engine/Vectormath.hpp:61-74).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace sg
{

constexpr int MAX_BASIS        = 8;
constexpr int MAX_PAIRS        = 96; // merged exchange+DMI pairs over all basis atoms of one system
constexpr int SPIN_ALIGN       = 32;
constexpr int MAX_FFT_LEN      = 1024;

// kernel ids of the per-launch profiling trace
enum KernelId : int
{
    KERNEL_STAGE = 0,
    KERNEL_PASS_A,
    KERNEL_PASS_B,
    KERNEL_PASS_C,
    KERNEL_PASS_B_INV,
    KERNEL_PASS_A_INV,
    KERNEL_END,
    KERNEL_PASS_BC, // fused B, C, B'
    N_KERNEL_IDS
};

// Solver ids (core/include/Spirit/Simulation.h:33-53): VP=0, SIB=1, Depondt=2, Heun=3, RK4=4,
// LBFGS_OSO=5, VP_OSO=7 (LBFGS_Atlas=6 is not provided)
enum Solver : int
{
    SOLVER_VP        = 0,
    SOLVER_SIB       = 1,
    SOLVER_DEPONDT   = 2,
    SOLVER_HEUN      = 3,
    SOLVER_RK4       = 4,
    SOLVER_LBFGS_OSO = 5,
    SOLVER_VP_OSO    = 7,
};

// One interaction pair of basis atom i with atom j in the cell translated by (da, db, dc).
// Exchange (J) and DMI (D * normal) pairs with the same (i, j, t) are merged:
//   g_i -= J s_j + s_j x Dvec        (Hamiltonian_Heisenberg.cpp:822-864)
struct PairEntry
{
    int i, j, da, db, dc;
    double J;
    double D[3];
};

struct FFTDesc;

// Exact unsigned division by a runtime constant d >= 1 for dividends n < 2^31 (every index here is
// a non-negative int): q = (umulhi(n, m) + n) >> l with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1 (Granlund and Montgomery, PLDI 1994: the round-up method; the sum
// cannot overflow for n < 2^31) -- a multiply-high, an add and a shift, no branch (d = 1: m = 1, l = 0).
struct FastDiv
{
    unsigned int d;
    unsigned int m;
    unsigned int l;
    unsigned int pad;
};

__host__ __device__ inline FastDiv make_fastdiv( unsigned int d )
{
    FastDiv f;
    f.d   = d > 0 ? d : 1;
    f.pad = 0;
    f.l   = 0;
    while( ( 1ull << f.l ) < f.d )
        ++f.l;
    f.m = (unsigned int)( ( ( 1ull << 32 ) * ( ( 1ull << f.l ) - f.d ) ) / f.d + 1 );
    return f;
}

#ifdef __CUDACC__
__device__ __forceinline__ unsigned int fdiv( unsigned int n, const FastDiv & f )
{
    return ( __umulhi( n, f.m ) + n ) >> f.l;
}
#endif

// Per-system constants of the stage arithmetic, precomputed on the host in FP64 and kept in
// the precision of the kernel that reads them (no FP64 division or square root on the device).
template<typename R>
struct SysConst
{
    R dtg;                      // dt gamma / mu_B / (1 + alpha^2)          (Method_LLG.cpp:152)
    R dtga;                     // dtg * alpha
    R alpha;
    R kdm;                      // dt gamma / mu_B: direct minimisation / VP (Method_LLG.cpp:165)
    R dt;
    R noise[MAX_BASIS];         // epsilon sqrt(T / mu_s)                   (Method_LLG.cpp:72-107)
    R mu[MAX_BASIS];
    R inv_mu[MAX_BASIS];
    R zeeman[3];                // mu_B B n
    R aniso_K[MAX_BASIS];
    R aniso_n[MAX_BASIS][3];
    int aniso_idx[MAX_BASIS];
    int n_aniso;
    int has_zeeman;
    int thermal;
    int direct;
};

// Per-system constants.  Read by every kernel; double so the FP64 path loses nothing.
struct SysDesc
{
    int n_cells[3];
    int nb;
    int nos;
    int bc[3];
    long long spin_offset; // into the batch's component arrays
    int pair_begin[MAX_BASIS + 1]; // pairs of basis atom ib: [pair_begin[ib], pair_begin[ib+1]) in pairs[]
    int n_pairs;
    int max_t[3]; // largest |translation| along each axis (stencil halo)
    FastDiv div_nb, div_na, div_nbb; // division by nb, Na, Nb
    PairEntry pairs[MAX_PAIRS];
    double mu_s[MAX_BASIS];
    double zeeman[3];           // mu_B * B * normal: Zeeman gradient is -mu_s * zeeman
    int has_zeeman;
    int n_aniso;                // uniaxial anisotropy entries (one per basis atom at most)
    int aniso_idx[MAX_BASIS];
    double aniso_K[MAX_BASIS];
    double aniso_n[MAX_BASIS][3];
    // LLG
    double dt, damping, temperature;
    int direct_minimization;
    double force_convergence;
    unsigned long long seed;
    unsigned int stream;
    unsigned int noise_offset; // iterations drawn by earlier runs: the noise counter continues there
    int n_iterations;
    // DDI
    int ddi;                    // 0 none, 1 FFT
    int fft_slot;               // index into the batch's FFT plan table
    SysConst<float> cf;
    SysConst<double> cd;
};

template<typename R>
__host__ __device__ inline const SysConst<R> & sys_const( const SysDesc & d );
template<typename R>
__host__ __device__ inline R fft_mu( const FFTDesc & f, int ib );
template<typename R>
__host__ __device__ inline R fft_invT( const FFTDesc & f );
template<>
__host__ __device__ inline const SysConst<float> & sys_const<float>( const SysDesc & d )
{
    return d.cf;
}
template<>
__host__ __device__ inline const SysConst<double> & sys_const<double>( const SysDesc & d )
{
    return d.cd;
}

// Mutable per-system run state on the device.  The blocks of the last stage kernel of a step (or
// of the probe kernel) add to the accumulators; the closing kernel launched after it writes the
// rest, which every block of the following kernels reads.
struct SysRun
{
    int iteration;      // completed iterations
    int active;         // 1 while the method keeps iterating this system
    float max_torque;   // last max |P_perp fv| (Hook_Post_Iteration)
    unsigned int torque_bits; // running max of |t|^2 as float bits (non-negative floats order like uints)
    double energy;      // energy of the last force evaluation (Spin_System::E)
    double energy_acc;  // running sum of the current evaluation
    double reserved;
};

// Radix sequence of one axis (0-terminated) with the divisors of each Stockham stage s of a
// length-L transform: L / radix[s] (butterflies per line) and the product of the earlier radices.
struct RadixPlan
{
    int radix[12];
    FastDiv div_lr[12];
    FastDiv div_ns[12];
};

// FFT plan of one system's dipolar convolution.  Padded extents M[d] = N[d] or 2 N[d]
// (Hamiltonian_Heisenberg.cpp:1510-1518); the real-to-complex axis is a (half length Ma/2+1).
struct FFTDesc
{
    int N[3];      // original cells per axis
    int M[3];      // padded FFT extents
    int Mh;        // M[0] / 2 + 1
    int nb;        // basis atoms
    long long spec_offset;   // complex element offset of this system's spectrum work arrays
    long long dhat_offset;   // complex element offset of its dipole spectrum
    long long tw_offset[3];  // twiddle table offsets (one table of M[d] entries per axis)
    RadixPlan plan[3];       // radix sequence per axis
    float mu_f[MAX_BASIS];   // mu_s per basis atom
    double mu_d[MAX_BASIS];
    float invT_f;            // 1 / (Ma Mb Mc)
    double invT_d;
    FastDiv div_Ma, div_Mh, div_Mb, div_Mc;
    FastDiv div_Nb, div_Nc, div_nb;
    FastDiv div_plane; // 3 nb Mb: elements of one c-row of the fused b/c pass
    FastDiv div_crow;  // 3 nb Mb / K: one c-row of a block of the clustered b/c pass
    // index divisors of the single-block fused b/c pass (set with the tiles): 3 nb Nc Nb (one
    // input plane), nb Mc Mb (tensor points of one plane)
    FastDiv div_nin, div_tens;
};

template<>
__host__ __device__ inline float fft_mu<float>( const FFTDesc & f, int ib )
{
    return f.mu_f[ib];
}
template<>
__host__ __device__ inline double fft_mu<double>( const FFTDesc & f, int ib )
{
    return f.mu_d[ib];
}
template<>
__host__ __device__ inline float fft_invT<float>( const FFTDesc & f )
{
    return f.invT_f;
}
template<>
__host__ __device__ inline double fft_invT<double>( const FFTDesc & f )
{
    return f.invT_d;
}

#ifdef __CUDACC__
// griddepcontrol (sm_90+): wait for the programmatic predecessor grid (completed, writes visible);
// allow the dependent grid to be launched.  Both are no-ops for a kernel launched without the
// programmatic-serialization attribute.
__device__ __forceinline__ void pdl_wait()
{
    asm volatile( "griddepcontrol.wait;" ::: "memory" );
}
__device__ __forceinline__ void pdl_trigger()
{
    asm volatile( "griddepcontrol.launch_dependents;" ::: "memory" );
}
#endif

} // namespace sg
