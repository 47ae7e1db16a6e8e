// Host-side lattice geometry, neighbour shells and interaction set-up of the Heisenberg
// Hamiltonian.  These run once per set-up (not in the step loop); the pair lists they produce
// must be identical to the reference's, entry for entry, because the redundant-pair order
// decides the floating-point summation order of the stencils.
#pragma once
#include <array>
#include <string>
#include <vector>

namespace sg
{

using Vec3 = std::array<double, 3>;

struct Pair
{
    int i, j;
    std::array<int, 3> t;
};

struct Geometry
{
    std::array<Vec3, 3> bravais{ Vec3{ 1, 0, 0 }, Vec3{ 0, 1, 0 }, Vec3{ 0, 0, 1 } };
    std::vector<Vec3> cell_atoms{ Vec3{ 0, 0, 0 } }; // fractional, in units of the Bravais vectors
    std::array<int, 3> n_cells{ 100, 100, 1 };
    double lattice_constant = 1.0;
    std::vector<double> mu_s_basis{ 1.0 };
    std::string bravais_name = "sc";

    int nb() const
    {
        return (int)cell_atoms.size();
    }
    int n_cells_total() const
    {
        return n_cells[0] * n_cells[1] * n_cells[2];
    }
    int nos() const
    {
        return nb() * n_cells_total();
    }
    double mu_s( int ispin ) const
    {
        return mu_s_basis[ispin % nb()];
    }
    Vec3 position( int ispin ) const;
    std::vector<Vec3> positions() const;
    Vec3 bounds_min() const;
    Vec3 bounds_max() const;
    Vec3 center() const;
    int dimensionality() const;
};

// Bravais presets (core/src/data/Geometry.cpp:446-487)
std::array<Vec3, 3> bravais_preset( const std::string & name, bool * ok = nullptr );

// core/src/engine/Neighbours.cpp:15-81 and :83-156 (redundant lists, as in the OpenMP build)
std::vector<double> shell_radii( const Geometry & g, int n_shells );
void neighbours_in_shells( const Geometry & g, int n_shells, std::vector<Pair> & pairs, std::vector<int> & shells );
// core/src/engine/Neighbours.cpp:249-286
Vec3 dmi_normal( const Geometry & g, const Pair & p, int chirality );

struct HamiltonianParams
{
    std::array<int, 3> bc{ 0, 0, 0 };
    double B = 0;                        // Tesla
    Vec3 B_normal{ 0, 0, 1 };
    double K = 0;                        // uniaxial anisotropy applied to every basis atom
    Vec3 K_normal{ 0, 0, 1 };
    std::vector<int> aniso_idx;
    std::vector<double> aniso_K;
    std::vector<Vec3> aniso_n;
    // exchange / DMI from shells ...
    std::vector<double> jij, dij;
    int dm_chirality = 1;
    // ... or from explicit pairs (heisenberg_pairs)
    bool from_pairs = false;
    std::vector<Pair> ex_pairs_in, dmi_pairs_in;
    std::vector<double> ex_J_in, dmi_D_in;
    std::vector<Vec3> dmi_n_in;
    // dipole-dipole
    int ddi_method = 0; // 0 none, 1 fft, 3 cutoff
    std::array<int, 3> ddi_images{ 4, 4, 4 };
    double ddi_radius        = 0;
    bool ddi_pb_zero_padding = true;
    std::string name         = "Heisenberg";

    // derived by update_interactions (Hamiltonian_Heisenberg::Update_Interactions, cpp:101-198)
    std::vector<Pair> ex_pairs, dmi_pairs;
    std::vector<double> ex_J, dmi_D;
    std::vector<Vec3> dmi_n;
};

void update_interactions( const Geometry & g, HamiltonianParams & h );
void set_uniform_anisotropy( const Geometry & g, HamiltonianParams & h, double K, const Vec3 & n );

// idx_from_pair (core/include/engine/Vectormath.hpp:437-528), host version used by the tests of
// the set-up and by the CPU-side bookkeeping
int idx_from_pair( const Geometry & g, const std::array<int, 3> & bc, int ispin, const Pair & p );

} // namespace sg
