// Dipolar FFT plan for a batch of systems (see fft.cuh / ddi.cu).
#pragma once
#include "common.hpp"

#include <cuda_runtime.h>

#include <array>
#include <utility>
#include <vector>

namespace sg
{

template<typename R>
struct PassArgs;

struct DDISystem
{
    int sys; // index of the system in the batch
    std::array<int, 3> n_cells;
    std::array<int, 3> padded;
    std::array<int, 3> bc;
    std::array<int, 3> images;
    int nb;
    double lattice_constant;
    std::array<std::array<double, 3>, 3> bravais;
    std::vector<std::array<double, 3>> cell_atoms;
    std::vector<double> mu_s; // per basis atom
};

class DDIPlan
{
public:
    ~DDIPlan();
    void build( const std::vector<DDISystem> & systems, bool fp64, const SysDesc * d_sd, cudaStream_t stream );
    // h = D * (mu s) for every DDI system of the batch whose SysRun is active (runs may be null);
    // only >= 0 launches that pass alone (0: A, the spectrum of s; 5: the fused b/c pass)
    void run( const SysDesc * d_sd, const SysRun * runs, const void * sx, const void * sy, const void * sz,
              void * hx, void * hy, void * hz, cudaStream_t stream, int only = -1 ) const;
    void release();
    // measure and keep the fastest lines (columns) per block of every pass (outside stream capture)
    void tune( const SysDesc * d_sd, const void * sx, const void * sy, const void * sz, void * hx, void * hy,
               void * hz, cudaStream_t stream );
    void set_tiles( int nl_a, int g_b, int g_c );
    // the tuned launch shapes of another plan built on the same systems (no timing runs)
    void copy_shape_from( const DDIPlan & o );
    // optional per-launch event trace (kernel id, event recorded before the launch)
    std::vector<std::pair<int, cudaEvent_t>> * trace = nullptr;
    int n_sys = 0;
    bool fp64 = false;

    // device tables (public for the pass launchers)
    FFTDesc * d_fd = nullptr;
    void * d_tw    = nullptr;
    void * d_W1    = nullptr;
    void * d_W2    = nullptr;
    void * d_Dhat  = nullptr;
    int4 * d_blocks[5] = { nullptr, nullptr, nullptr, nullptr, nullptr }; // A, B, C, BC
    int n_blocks[5]    = { 0, 0, 0, 0, 0 };
    int tile[3]        = { 8, 8, 8 }; // lines per block of A/A', lines per block of B/B', columns per block of C
    int threads[3]     = { 256, 256, 256 }; // threads per block of A/A', B/B', C
    bool fused         = false; // passes B, C, B' as one kernel per (system, ka) plane
    int threads_bc     = 1024;
    int cluster_k      = 1; // blocks per (system, ka) plane of the fused pass (cluster size)
    int planes_bc      = 1; // ka planes per block of the single-block fused pass on one-row (2D) systems
    bool bc_pow2       = false; // every system's cluster index splits are powers of two (pass_bc_cl<R, true>)
    int n_fd_slots     = 1;
    size_t smem_bc_max = 0;
    size_t max_smem_a = 0, max_smem_b = 0, max_smem_c = 0;
    long long spec_elems = 0;
    std::vector<FFTDesc> fd_host;
    std::vector<int> sys_index;

private:
    void build_block_tables( const std::vector<DDISystem> & systems );
    void compute_dhat( const std::vector<DDISystem> & systems, const SysDesc * d_sd, cudaStream_t stream );
    template<typename R>
    void tune_t( const SysDesc * d_sd, const R * sx, const R * sy, const R * sz, R * hx, R * hy, R * hz,
                 cudaStream_t stream );
    template<typename R>
    void launch_pass( int k, PassArgs<R> & a, cudaStream_t stream ) const;
    template<typename R>
    void run_t( const SysDesc * d_sd, const SysRun * runs, const R * sx, const R * sy, const R * sz, R * hx, R * hy,
                R * hz, cudaStream_t stream, int only ) const;
};

// smallest even number >= m whose prime factors are all <= 7
inline int ddi_smooth_even( int m )
{
    for( int v = m + ( m & 1 );; v += 2 )
    {
        int r = v;
        for( int p : { 2, 3, 5, 7 } )
            while( r % p == 0 )
                r /= p;
        if( r == 1 )
            return v;
    }
}

// Padded FFT extent per axis.  The reference (Prepare_DDI, Hamiltonian_Heisenberg.cpp:1510-1518)
// doubles an axis with more than one cell that is open or explicitly zero-padded, to 2N.  A
// zero-padded circular convolution of length M equals the linear one for every M >= 2N - 1 (the
// offsets between N and M - N are never paired), so here such an axis gets the smallest even
// 7-smooth M >= 2N: 2N itself when it is 7-smooth (powers of two, most sizes), else slightly more,
// which keeps every transform on radices <= 7 (2N = 2 * 251 would otherwise be a radix-251
// stage).  Periodic axes without padding keep M = N.  (Padding to the next power of two instead, so
// that every transform took the register power-of-two path, measured slower on the 256-system
// dipolar ensemble: 2.59 against 2.25 ms per step -- the extra cells cost more than the radices save.)
inline std::array<int, 3> ddi_padding( const std::array<int, 3> & n, const std::array<int, 3> & bc, bool pb_zero_padding )
{
    std::array<int, 3> m;
    for( int d = 0; d < 3; ++d )
        m[d] = ( n[d] > 1 && ( bc[d] == 0 || pb_zero_padding ) ) ? ddi_smooth_even( 2 * n[d] ) : n[d];
    return m;
}

} // namespace sg
