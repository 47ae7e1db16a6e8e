/*
 * Spirit_gb300.h -- C ABI of libspirit_gb300.so, the GB300 (sm_103a) engine of the Spirit
 * spin-dynamics hot path.
 *
 * Drop-in boundary: the functions below keep the names, signatures (float parameters,
 * idx_image / idx_chain = -1 selecting the active image / chain) and argument meaning of the
 * reference's flat C API, so existing callers (the reference's ctypes bindings, C/C++ programs)
 * link against this library instead of libSpirit.so.  Every declaration names the reference
 * declaration it replaces as core/include/Spirit/<header>:<line>.  Declarations marked
 * EXTENSION have no counterpart in the reference.
 *
 * Types: `scalar` is double (the host mirror of the spins); the device computes in FP32 (default)
 * or FP64 (Simulation_Set_Precision).  Errors never terminate the process: a failing call logs
 * and returns its default value (the reference logs and, for CUDA errors, exits).
 */
#ifndef SPIRIT_GB300_H
#define SPIRIT_GB300_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double scalar;
struct State;
typedef struct State State;

/* core/include/Spirit/Simulation.h:57-71 */
typedef struct Simulation_Run_Info
{
    int total_iterations;
    int total_walltime;
    float total_ips;
    float max_torque;
    int n_history_iteration;
    int * history_iteration;
    int n_history_max_torque;
    float * history_max_torque;
    int n_history_energy;
    float * history_energy;
} Simulation_Run_Info;

/* solver ids: core/include/Spirit/Simulation.h:31-45 */
#define Solver_VP 0
#define Solver_SIB 1
#define Solver_Depondt 2
#define Solver_Heun 3
#define Solver_RungeKutta4 4
#define Solver_LBFGS_OSO 5 /* Simulation.h:48 (direct minimisation, LLG and GNEB) */
#define Solver_VP_OSO 7    /* Simulation.h:54 */

/* ================================================================ State (core/include/Spirit/State.h) */
State * State_Setup( const char * config_file, bool quiet );                  /* State.h:71 */
void State_Delete( State * state );                                            /* State.h:76 */
void State_Update( State * state );                                            /* State.h:81 */
void State_To_Config( State * state, const char * config_file, const char * comment ); /* State.h:87 */
const char * State_DateTime( State * state );                                  /* State.h:94 */

/* ================================================================ Hamiltonian (core/include/Spirit/Hamiltonian.h) */
void Hamiltonian_Set_Boundary_Conditions( State * state, const bool * periodical, int idx_image, int idx_chain ); /* :65 */
void Hamiltonian_Set_Field( State * state, float magnitude, const float * normal, int idx_image, int idx_chain );   /* :69 */
void Hamiltonian_Set_Anisotropy( State * state, float magnitude, const float * normal, int idx_image,
                                 int idx_chain );                                                                   /* :73 */
void Hamiltonian_Set_Cubic_Anisotropy( State * state, float magnitude, int idx_image, int idx_chain ); /* :77 (logs: not part of the engine) */
void Hamiltonian_Set_Exchange( State * state, int n_shells, const float * jij, int idx_image, int idx_chain ); /* :81 */
void Hamiltonian_Set_DMI( State * state, int n_shells, const float * dij, int chirality, int idx_image,
                          int idx_chain );                                                                 /* :85 */
void Hamiltonian_Set_DDI( State * state, int ddi_method, int n_periodic_images[3], float cutoff_radius,
                          bool pb_zero_padding, int idx_image, int idx_chain );                            /* :100 */
const char * Hamiltonian_Get_Name( State * state, int idx_image, int idx_chain );                         /* :110 */
void Hamiltonian_Get_Boundary_Conditions( State * state, bool * periodical, int idx_image, int idx_chain ); /* :113 */
void Hamiltonian_Get_Field( State * state, float * magnitude, float * normal, int idx_image, int idx_chain ); /* :117 */
void Hamiltonian_Get_Anisotropy( State * state, float * magnitude, float * normal, int idx_image,
                                 int idx_chain );                                                          /* :121 */
void Hamiltonian_Get_Cubic_Anisotropy( State * state, float * magnitude, int idx_image, int idx_chain ); /* :125 */
void Hamiltonian_Get_Exchange_Shells( State * state, int * n_shells, float * jij, int idx_image, int idx_chain ); /* :134 */
int Hamiltonian_Get_Exchange_N_Pairs( State * state, int idx_image, int idx_chain );                      /* :138 */
void Hamiltonian_Get_Exchange_Pairs( State * state, int idx[][2], int translations[][3], float * Jij, int idx_image,
                                     int idx_chain );                                                      /* :140 */
void Hamiltonian_Get_DMI_Shells( State * state, int * n_shells, float * dij, int * chirality, int idx_image,
                                 int idx_chain );                                                          /* :149 */
int Hamiltonian_Get_DMI_N_Pairs( State * state, int idx_image, int idx_chain );                           /* :153 */
void Hamiltonian_Get_DDI( State * state, int * ddi_method, int n_periodic_images[3], float * cutoff_radius,
                          bool * pb_zero_padding, int idx_image, int idx_chain );                          /* :164 */
/* EXTENSION: FP64 device gradient of the image's spins (AoS [nos][3]); returns the FP64 energy.
 * The reference reaches this only through Hamiltonian::Gradient_and_Energy (C++ internals). */
double Hamiltonian_Get_Gradient( State * state, double * gradient, int idx_image, int idx_chain );
/* EXTENSION: FP64 gradients and energies of the active images of n States evaluated as one batch
 * (one FP64 device engine over all systems; the dipolar term of every system from the batch's shared
 * FFT plan table, the path batched LLG runs take).  gradients: AoS [sum of nos][3] in the order of
 * the States (may be NULL); energies[n_states] (may be NULL).  No counterpart in the reference,
 * which evaluates one image per Hamiltonian call (Hamiltonian_Heisenberg.cpp:704-766). */
void Hamiltonian_Get_Gradient_Batched( State ** states, int n_states, double * gradients, double * energies );
/* EXTENSION: FP64 energy per term (Zeeman, Anisotropy, Exchange, DMI, DDI) into terms[5] and,
 * if per_spin != NULL, per spin into per_spin[5][nos]; returns the total (Energy_Contributions_per_Spin). */
double Hamiltonian_Get_Energy_Contributions( State * state, double * terms, double * per_spin, int idx_image,
                                            int idx_chain );
/* EXTENSION: dipolar field h = D * (mu s) of the image's spins, AoS [nos][3] (FP64 device FFT). */
void Hamiltonian_Get_DDI_Field( State * state, double * field, int idx_image, int idx_chain );
/* EXTENSION, no counterpart in the reference: allocation-free FP64 gradient and energy of the
 * stencil terms (exchange, DMI, anisotropy, Zeeman; no dipolar term) of the image's geometry and
 * Hamiltonian, for spins already on the device (SoA sx/sy/sz[nos]).  Writes gx/gy/gz[nos] and
 * energy[0] (all caller-owned device memory) asynchronously on `stream` (a cudaStream_t, NULL =
 * legacy default stream).  Makes no device allocation: its scratch is a static device array.
 * At most 4,194,304 spins.  Calls that overlap in time share that scratch and race.  The first
 * call on a device looks the scratch up and should precede any stream capture.  Returns 0 on
 * success, 1 bad arguments, 2 too many spins, 3 dipolar interaction enabled, 4 CUDA error,
 * 5 host error. */
int Hamiltonian_Get_Gradient_NoAlloc( State * state, const double * sx, const double * sy, const double * sz,
                                      double * gx, double * gy, double * gz, double * energy, void * stream,
                                      int idx_image, int idx_chain );

/* ================================================================ Geometry (core/include/Spirit/Geometry.h) */
void Geometry_Set_Bravais_Lattice_Type( State * state, int lattice_type );               /* :51 */
void Geometry_Set_N_Cells( State * state, int n_cells[3] );                               /* :56 */
void Geometry_Set_Cell_Atoms( State * state, int n_atoms, float ** atoms );               /* :62 */
void Geometry_Set_mu_s( State * state, float mu_s, int idx_image, int idx_chain );        /* :67 */
void Geometry_Set_Bravais_Vectors( State * state, float ta[3], float tb[3], float tc[3] ); /* :77 */
void Geometry_Set_Lattice_Constant( State * state, float lattice_constant );              /* :82 */
int Geometry_Get_NOS( State * state );                                                    /* :92 */
scalar * Geometry_Get_Positions( State * state, int idx_image, int idx_chain );           /* :97 */
void Geometry_Get_Bounds( State * state, float min[3], float max[3], int idx_image, int idx_chain ); /* :108 */
void Geometry_Get_Center( State * state, float center[3], int idx_image, int idx_chain ); /* :113 */
void Geometry_Get_Bravais_Vectors( State * state, float a[3], float b[3], float c[3], int idx_image,
                                   int idx_chain );                                       /* :124 */
int Geometry_Get_Dimensionality( State * state, int idx_image, int idx_chain );           /* :130 */
void Geometry_Get_mu_s( State * state, float * mu_s, int idx_image, int idx_chain );      /* :135 */
void Geometry_Get_N_Cells( State * state, int n_cells[3], int idx_image, int idx_chain ); /* :140 */
int Geometry_Get_N_Cell_Atoms( State * state, int idx_image, int idx_chain );             /* :155 */
/* EXTENSION: lattice constant in Angstrom */
double Geometry_Get_Lattice_Constant( State * state, int idx_image, int idx_chain );

/* ================================================================ Configurations (core/include/Spirit/Configurations.h) */
void Configuration_To_Clipboard( State * state, int idx_image, int idx_chain );           /* :42 */
void Configuration_From_Clipboard( State * state, const float position[3], const float r_cut_rectangular[3],
                                   float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                                   int idx_chain );                                       /* :45 */
void Configuration_Domain( State * state, const float direction[3], const float position[3],
                           const float r_cut_rectangular[3], float r_cut_cylindrical, float r_cut_spherical,
                           bool inverted, int idx_image, int idx_chain );                 /* :62 */
void Configuration_PlusZ( State * state, const float position[3], const float r_cut_rectangular[3],
                          float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                          int idx_chain );                                                /* :68 */
void Configuration_MinusZ( State * state, const float position[3], const float r_cut_rectangular[3],
                           float r_cut_cylindrical, float r_cut_spherical, bool inverted, int idx_image,
                           int idx_chain );                                               /* :74 */
void Configuration_Random( State * state, const float position[3], const float r_cut_rectangular[3],
                           float r_cut_cylindrical, float r_cut_spherical, bool inverted, bool external,
                           int idx_image, int idx_chain );                                /* :80 */
void Configuration_Skyrmion( State * state, float r, float order, float phase, bool upDown, bool achiral, bool rl,
                             const float position[3], const float r_cut_rectangular[3], float r_cut_cylindrical,
                             float r_cut_spherical, bool inverted, int idx_image, int idx_chain ); /* :118 */

/* ================================================================ Chain (core/include/Spirit/Chain.h) */
int Chain_Get_NOI( State * state, int idx_chain );                                        /* :22 */
bool Chain_next_Image( State * state, int idx_chain );                                    /* :34 */
bool Chain_prev_Image( State * state, int idx_chain );                                    /* :41 */
bool Chain_Jump_To_Image( State * state, int idx_image, int idx_chain );                  /* :48 */
void Chain_Set_Length( State * state, int n_images, int idx_chain );                      /* :63 */
void Chain_Image_to_Clipboard( State * state, int idx_image, int idx_chain );             /* :70 */
void Chain_Replace_Image( State * state, int idx_image, int idx_chain );                  /* :77 */
void Chain_Insert_Image_Before( State * state, int idx_image, int idx_chain );            /* :84 */
void Chain_Insert_Image_After( State * state, int idx_image, int idx_chain );             /* :91 */
void Chain_Push_Back( State * state, int idx_chain );                                     /* :98 */
bool Chain_Delete_Image( State * state, int idx_image, int idx_chain );                   /* :105 */
bool Chain_Pop_Back( State * state, int idx_chain );                                      /* :114 */
void Chain_Get_Rx( State * state, float * Rx, int idx_chain );                            /* :124 */
void Chain_Get_Rx_Interpolated( State * state, float * Rx_interpolated, int idx_chain );  /* :129 */
void Chain_Get_Energy( State * state, float * energy, int idx_chain );                    /* :134 */
void Chain_Get_Energy_Interpolated( State * state, float * E_interpolated, int idx_chain ); /* :139 */
void Chain_Update_Data( State * state, int idx_chain );                                   /* :151 */
void Chain_Setup_Data( State * state, int idx_chain );                                    /* :156 */

/* ================================================================ Transitions (core/include/Spirit/Transitions.h) */
void Transition_Homogeneous( State * state, int idx_1, int idx_2, int idx_chain );        /* :29 */

/* ================================================================ HTST (core/include/Spirit/HTST.h)
 * The Hessians and all eigenpairs are computed on the device in FP64 (parallel Jacobi); sparse =
 * true reports what the reference's sparse variant reports (log-determinants, no eigen output). */
float HTST_Calculate( State * state, int idx_image_minimum, int idx_image_sp, int n_eigenmodes_keep, bool sparse,
                      int idx_chain );                                                               /* :37 */
void HTST_Get_Info( State * state, float * temperature_exponent, float * me, float * Omega_0, float * s,
                    float * volume_min, float * volume_sp, float * prefactor_dynamical, float * prefactor,
                    int * n_eigenmodes_keep, int idx_chain );                                        /* :52 */
void HTST_Get_Eigenvalues_Min( State * state, float * eigenvalues_min, int idx_chain );             /* :61 */
void HTST_Get_Eigenvectors_Min( State * state, float * eigenvectors_min, int idx_chain );           /* :67 */
void HTST_Get_Eigenvalues_SP( State * state, float * eigenvalues_sp, int idx_chain );               /* :73 */
void HTST_Get_Eigenvectors_SP( State * state, float * eigenvectors_sp, int idx_chain );             /* :79 */
void HTST_Get_Velocities( State * state, float * velocities, int idx_chain );                       /* :86 */
/* EXTENSION: FP64 copy of the last HTST result.  info[10] = temperature_exponent, me, Omega_0, s,
 * volume_min, volume_sp, prefactor_dynamical, prefactor, det_min, det_sp; eigenvalues [2N];
 * eigenvectors [n_eigenmodes_keep][2N]; velocities [2N] (NULL pointers are skipped).  Returns 0
 * when the calculation completed, 1-5 for the check that stopped it (1 minimum / 2 saddle point
 * not converged, 3 no negative mode, 4 higher-order saddle point, 5 negative mode at the
 * minimum), -1 when there is no result. */
int HTST_Get_Result_FP64( State * state, double * info, double * eigenvalues_min, double * eigenvalues_sp,
                          double * eigenvectors_min, double * eigenvectors_sp, double * velocities, int idx_chain );

/* ================================================================ IO (core/include/Spirit/IO.h)
 * OVF 2.0 files; format: 0 binary in the API precision (8 bytes), 1 binary 4, 2 binary 8, 3 text,
 * 4 CSV (IO.h:26-38).  Segments written here carry the image's random-stream positions (LLG noise
 * iterations, Metropolis sweeps) in a Desc line; reading such a segment restores them, so a run
 * resumed from the file continues the same Philox streams. */
#define IO_Fileformat_OVF_bin 0
#define IO_Fileformat_OVF_bin4 1
#define IO_Fileformat_OVF_bin8 2
#define IO_Fileformat_OVF_text 3
#define IO_Fileformat_OVF_csv 4
void IO_Positions_Write( State * state, const char * file, int format, const char * comment, int idx_image,
                         int idx_chain );                                                  /* :50 */
int IO_N_Images_In_File( State * state, const char * file, int idx_image, int idx_chain ); /* :60 */
void IO_Image_Read( State * state, const char * file, int idx_image_infile, int idx_image_inchain,
                    int idx_chain );                                                       /* :63 */
void IO_Image_Write( State * state, const char * file, int format, const char * comment, int idx_image,
                     int idx_chain );                                                      /* :67 */
void IO_Image_Append( State * state, const char * file, int format, const char * comment, int idx_image,
                      int idx_chain );                                                     /* :72 */
void IO_Chain_Read( State * state, const char * file, int start_image_infile, int end_image_infile, int insert_idx,
                    int idx_chain );                                                       /* :87 */
void IO_Chain_Write( State * state, const char * file, int format, const char * comment, int idx_chain ); /* :92 */
void IO_Chain_Append( State * state, const char * file, int format, const char * comment, int idx_chain ); /* :97 */

/* ================================================================ Parameters_MC (core/include/Spirit/Parameters_MC.h) */
void Parameters_MC_Set_Output_Tag( State * state, const char * tag, int idx_image, int idx_chain );       /* :30 */
void Parameters_MC_Set_Output_Folder( State * state, const char * folder, int idx_image, int idx_chain ); /* :34 */
void Parameters_MC_Set_Output_General( State * state, bool any, bool initial, bool final, int idx_image,
                                       int idx_chain );                                                    /* :37 */
void Parameters_MC_Set_Output_Energy( State * state, bool energy_step, bool energy_archive, bool energy_spin_resolved,
                                      bool energy_divide_by_nos, bool energy_add_readability_lines, int idx_image,
                                      int idx_chain );                                                     /* :49 */
void Parameters_MC_Set_Output_Configuration( State * state, bool configuration_step, bool configuration_archive,
                                             int configuration_filetype, int idx_image, int idx_chain );   /* :60 */
void Parameters_MC_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_image,
                                     int idx_chain );                                                      /* :70 */
void Parameters_MC_Set_Temperature( State * state, float T, int idx_image, int idx_chain );                /* :79 */
void Parameters_MC_Set_Metropolis_Cone( State * state, bool cone, float cone_angle, bool adaptive_cone,
                                        float target_acceptance_ratio, int idx_image, int idx_chain );    /* :89 */
/* random_sample is stored; the device sweeps are colour-ordered in every case */
void Parameters_MC_Set_Random_Sample( State * state, bool random_sample, int idx_image, int idx_chain );  /* :94 */
const char * Parameters_MC_Get_Output_Tag( State * state, int idx_image, int idx_chain );                /* :103 */
const char * Parameters_MC_Get_Output_Folder( State * state, int idx_image, int idx_chain );             /* :106 */
void Parameters_MC_Get_Output_General( State * state, bool * any, bool * initial, bool * final, int idx_image,
                                       int idx_chain );                                                   /* :109 */
void Parameters_MC_Get_Output_Energy( State * state, bool * energy_step, bool * energy_archive,
                                      bool * energy_spin_resolved, bool * energy_divide_by_nos,
                                      bool * energy_add_readability_lines, int idx_image, int idx_chain ); /* :113 */
void Parameters_MC_Get_Output_Configuration( State * state, bool * configuration_step, bool * configuration_archive,
                                             int * configuration_filetype, int idx_image, int idx_chain ); /* :118 */
void Parameters_MC_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_image,
                                     int idx_chain );                                                     /* :123 */
float Parameters_MC_Get_Temperature( State * state, int idx_image, int idx_chain );                       /* :132 */
void Parameters_MC_Get_Metropolis_Cone( State * state, bool * cone, float * cone_angle, bool * adaptive_cone,
                                        float * target_acceptance_ratio, int idx_image, int idx_chain );  /* :142 */
bool Parameters_MC_Get_Random_Sample( State * state, int idx_image, int idx_chain );                      /* :147 */

/* ================================================================ Parameters_LLG (core/include/Spirit/Parameters_LLG.h) */
void Parameters_LLG_Set_Output_General( State * state, bool any, bool initial, bool final, int idx_image,
                                        int idx_chain );                                  /* :37 (accepted, no files written) */
void Parameters_LLG_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_image,
                                      int idx_chain );                                    /* :70 */
void Parameters_LLG_Set_Direct_Minimization( State * state, bool direct, int idx_image, int idx_chain ); /* :84 */
void Parameters_LLG_Set_Convergence( State * state, float convergence, int idx_image, int idx_chain );   /* :93 */
void Parameters_LLG_Set_Time_Step( State * state, float dt, int idx_image, int idx_chain );              /* :97 */
void Parameters_LLG_Set_Damping( State * state, float damping, int idx_image, int idx_chain );           /* :100 */
void Parameters_LLG_Set_Non_Adiabatic_Damping( State * state, float beta, int idx_image, int idx_chain ); /* :103 */
void Parameters_LLG_Set_Temperature( State * state, float T, int idx_image, int idx_chain );             /* :118 */
void Parameters_LLG_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_image,
                                      int idx_chain );                                    /* :155 */
bool Parameters_LLG_Get_Direct_Minimization( State * state, int idx_image, int idx_chain ); /* :164 */
float Parameters_LLG_Get_Convergence( State * state, int idx_image, int idx_chain );      /* :167 */
float Parameters_LLG_Get_Time_Step( State * state, int idx_image, int idx_chain );        /* :170 */
float Parameters_LLG_Get_Damping( State * state, int idx_image, int idx_chain );          /* :173 */
float Parameters_LLG_Get_Non_Adiabatic_Damping( State * state, int idx_image, int idx_chain ); /* :176 */
float Parameters_LLG_Get_Temperature( State * state, int idx_image, int idx_chain );      /* :179 */
/* EXTENSION: thermal-noise seed (Philox key); the reference reads it from the config file only
 * (llg_seed, core/include/data/Parameters_Method_LLG.hpp:22-24) */
void Parameters_LLG_Set_Seed( State * state, int seed, int idx_image, int idx_chain );

/* ================================================================ Parameters_GNEB (core/include/Spirit/Parameters_GNEB.h) */
void Parameters_GNEB_Set_N_Iterations( State * state, int n_iterations, int n_iterations_log, int idx_chain ); /* :86 */
void Parameters_GNEB_Set_Convergence( State * state, float convergence, int idx_image, int idx_chain ); /* :100 */
void Parameters_GNEB_Set_Spring_Constant( State * state, float spring_constant, int idx_image, int idx_chain ); /* :104 */
void Parameters_GNEB_Set_Spring_Force_Ratio( State * state, float ratio, int idx_chain );  /* :108 (0 supported) */
void Parameters_GNEB_Set_Path_Shortening_Constant( State * state, float c, int idx_chain ); /* :111 (0 supported) */
void Parameters_GNEB_Set_Moving_Endpoints( State * state, bool moving, int idx_chain );   /* :115 (fixed supported) */
void Parameters_GNEB_Set_Climbing_Falling( State * state, int image_type, int idx_image, int idx_chain ); /* :126 */
void Parameters_GNEB_Set_Image_Type_Automatically( State * state, int idx_chain );        /* :134 */
void Parameters_GNEB_Set_N_Energy_Interpolations( State * state, int n, int idx_chain );  /* :137 */
void Parameters_GNEB_Get_N_Iterations( State * state, int * iterations, int * iterations_log, int idx_chain ); /* :163 */
float Parameters_GNEB_Get_Convergence( State * state, int idx_image, int idx_chain );     /* :172 */
float Parameters_GNEB_Get_Spring_Constant( State * state, int idx_image, int idx_chain ); /* :175 */
float Parameters_GNEB_Get_Spring_Force_Ratio( State * state, int idx_chain );             /* :178 */
float Parameters_GNEB_Get_Path_Shortening_Constant( State * state, int idx_chain );       /* :181 */
int Parameters_GNEB_Get_Climbing_Falling( State * state, int idx_image, int idx_chain );  /* :198 */
int Parameters_GNEB_Get_N_Energy_Interpolations( State * state, int idx_chain );          /* :201 */

/* ================================================================ Simulation (core/include/Spirit/Simulation.h) */
void free_run_info( Simulation_Run_Info info );                                           /* :73 */
/* Monte Carlo: colour-ordered Metropolis sweeps on the device */
void Simulation_MC_Start( State * state, int n_iterations, int n_iterations_log, bool singleshot,
                          Simulation_Run_Info * info, int idx_image, int idx_chain );               /* :81 */
void Simulation_LLG_Start( State * state, int solver_type, int n_iterations, int n_iterations_log, bool singleshot,
                           Simulation_Run_Info * info, int idx_image, int idx_chain );    /* :86 */
void Simulation_GNEB_Start( State * state, int solver_type, int n_iterations, int n_iterations_log, bool singleshot,
                            Simulation_Run_Info * info, int idx_chain );                  /* :91 (VP solver) */
void Simulation_SingleShot( State * state, int idx_image, int idx_chain );                /* :111 */
void Simulation_N_Shot( State * state, int N, int idx_image, int idx_chain );             /* :119 */
void Simulation_Stop( State * state, int idx_image, int idx_chain );                      /* :122 */
void Simulation_Stop_All( State * state );                                                /* :125 */
float Simulation_Get_MaxTorqueComponent( State * state, int idx_image, int idx_chain );   /* :139 */
float Simulation_Get_MaxTorqueNorm( State * state, int idx_image, int idx_chain );        /* :155 */
void Simulation_Get_Chain_MaxTorqueNorms( State * state, float * torques, int idx_chain ); /* :162 */
float Simulation_Get_IterationsPerSecond( State * state, int idx_image, int idx_chain );  /* :171 */
int Simulation_Get_Iteration( State * state, int idx_image, int idx_chain );              /* :174 */
float Simulation_Get_Time( State * state, int idx_image, int idx_chain );                 /* :183 */
int Simulation_Get_Wall_Time( State * state, int idx_image, int idx_chain );              /* :186 */
const char * Simulation_Get_Solver_Name( State * state, int idx_image, int idx_chain );   /* :195 */
const char * Simulation_Get_Method_Name( State * state, int idx_image, int idx_chain );   /* :204 */
bool Simulation_Running_On_Image( State * state, int idx_image, int idx_chain );          /* :212 */
bool Simulation_Running_On_Chain( State * state, int idx_chain );                         /* :215 */
bool Simulation_Running_Anywhere_On_Chain( State * state, int idx_chain );                /* :218 */
/* EXTENSION: batched LLG -- the active images of n_states States advance together in one
 * device launch sequence (uneven sizes and parameters allowed, one solver); info: n_states entries
 * or NULL.  The reference iterates exactly one image per method (core/src/engine/Method_LLG.cpp:25-26). */
void Simulation_LLG_Start_Batched( State ** states, int n_states, int solver_type, int n_iterations,
                                   Simulation_Run_Info * info );
/* EXTENSION: enqueue n_steps of an open-ended batched LLG run of the States' active images on
 * states[0]'s stream (Simulation_Set_Stream), no transfers or synchronisation; the first call
 * uploads the spins and starts the batch.  Simulation_LLG_Batched_Finish copies the spins back
 * into the host buffers and ends the run. */
void Simulation_LLG_Batched_Launch_Steps( State ** states, int n_states, int solver_type, int n_steps );
void Simulation_LLG_Batched_Finish( State ** states, int n_states );
/* EXTENSION: adjoint of a T = 0 RK4 LLG trajectory of the image (the reference has none).
 * params = (J, D, K [meV], B [T], alpha) replace the configured first-shell exchange, first-shell
 * DMI, anisotropy and field magnitudes (other shells / basis atoms scale with them, the field
 * direction stays) and the damping; NULL keeps the configured values.  Runs n_steps from the
 * image's spins; returns loss = mean_i |s_i(T) - target_i|^2 (FP64) and writes its gradient with
 * respect to the initial spins (grad_s0, AoS [nos][3], may be NULL) and to params
 * (grad_params[5], may be NULL); final_spins (AoS, may be NULL) receives s(T).  States are kept
 * every `checkpoint` steps and each segment is recomputed once in the backward pass.  Device
 * arithmetic follows Simulation_Set_Precision. */
double Simulation_LLG_Adjoint( State * state, const double * params, int n_steps, int checkpoint,
                               const double * target, double * grad_s0, double * grad_params, double * final_spins,
                               int idx_image, int idx_chain );
/* EXTENSION: the loss of the same trajectory without gradients (finite differences, timing) */
double Simulation_LLG_Loss( State * state, const double * params, int n_steps, const double * target,
                            double * final_spins, int idx_image, int idx_chain );
/* EXTENSION: the autotuned launch parameters of the image's started LLG run, in this order:
 * spins per thread of the stage kernels; lines and threads per block of FFT pass A / A'; lines
 * and threads of pass B / B'; columns and threads of pass C; 1 if the fused b/c pass is used;
 * its cluster size and threads per block; 1 if the run has a dipolar term; 1 if the stage kernels
 * do the passes along a themselves (row-fused stages); 1 if the stage kernels stage each tile's
 * configuration window in shared memory by tensor copies (TMA); 1 if the FP32 state is kept
 * compensated (hi + lo float pairs).  Writes at most n values; returns the number the engine
 * reports (0 without a started run). */
int Simulation_Get_Tuning( State * state, int * values, int n, int idx_image, int idx_chain );
/* EXTENSION: device arithmetic of the step loop: 32 (FP32 bulk, default) or 64 */
void Simulation_Set_Precision( State * state, int bits );
int Simulation_Get_Precision( State * state );
/* EXTENSION: run the State's device work on the caller's cudaStream_t (NULL: engine stream) */
void Simulation_Set_Stream( State * state, void * stream );
/* EXTENSION: launch n steps of a started single-shot LLG run, no transfers, no synchronisation */
void Simulation_Launch_Steps( State * state, int n, int idx_image, int idx_chain );
/* EXTENSION: per-kernel device time (ms[] / count[] indexed stage, FFT passes A, B, C, B', A') of
 * n steps timed with CUDA events on the engine stream; before every step flush_buf is overwritten
 * and read_buf read (L2 flush); buffers may be NULL */
void Simulation_Profile_Steps( State * state, int n, void * flush_buf, long long flush_bytes, void * read_buf,
                               long long read_bytes, double * ms, int * count, int idx_image, int idx_chain );
/* EXTENSION: number of device kernels per step of the image's current LLG method */
int Simulation_Get_Kernels_Per_Step( State * state, int idx_image, int idx_chain );

/* ================================================================ System (core/include/Spirit/System.h) */
int System_Get_Index( State * state );                                                    /* :25 */
int System_Get_NOS( State * state, int idx_image, int idx_chain );                        /* :28 */
scalar * System_Get_Spin_Directions( State * state, int idx_image, int idx_chain );       /* :35 */
scalar * System_Get_Effective_Field( State * state, int idx_image, int idx_chain );       /* :42 */
float System_Get_Rx( State * state, int idx_image, int idx_chain );                       /* :52 */
float System_Get_Energy( State * state, int idx_image, int idx_chain );                   /* :55 */
int System_Get_Energy_Array_Names( State * state, char * names, int idx_image, int idx_chain ); /* :59 */
int System_Get_Energy_Array( State * state, float * energies, bool divide_by_nspins, int idx_image,
                             int idx_chain );                                             /* :63 */
void System_Print_Energy_Array( State * state, int idx_image, int idx_chain );            /* :70 */
void System_Update_Data( State * state, int idx_image, int idx_chain );                   /* :73 */
/* EXTENSION: the FP64 energy behind System_Get_Energy (Spin_System::E) */
double System_Get_Energy_FP64( State * state, int idx_image, int idx_chain );
/* EXTENSION: wait for the image's device work and copy its spins into the host buffer */
void System_Update_Spins_From_Device( State * state, int idx_image, int idx_chain );

/* ================================================================ Quantities (core/include/Spirit/Quantities.h) */
void Quantity_Get_Average_Spin( State * state, float s[3], int idx_image, int idx_chain ); /* :18 */
void Quantity_Get_Magnetization( State * state, float m[3], int idx_image, int idx_chain ); /* :21 */

/* ================================================================ Constants (core/include/Spirit/Constants.h) */
scalar Constants_mu_B( void );  /* :20 */
scalar Constants_mu_0( void );  /* :23 */
scalar Constants_k_B( void );   /* :26 */
scalar Constants_hbar( void );  /* :29 */
scalar Constants_mRy( void );   /* :32 */
scalar Constants_gamma( void ); /* :35 */
scalar Constants_g_e( void );   /* :38 */
scalar Constants_Pi( void );    /* :41 */

/* ================================================================ Version / Log (core/include/Spirit/Version.h, Log.h) */
const char * Spirit_Version( void );       /* Version.h:10 */
const char * Spirit_Version_Full( void );  /* Version.h:12 */
const char * Spirit_Compiler_Full( void ); /* Version.h:16 */
const char * Spirit_Scalar_Type( void );   /* Version.h:18 */
/* EXTENSION: 1 -- this library always runs the device engine */
int Spirit_Cuda( void );
void Log_Send( State * state, int level, int sender, const char * message, int idx_image, int idx_chain ); /* Log.h:57 */
int Log_Get_N_Entries( State * state );    /* Log.h:76 */

#ifdef __cplusplus
}
#endif
#endif
