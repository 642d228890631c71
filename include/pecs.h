/*
 * pecs.h -- C ABI of the GB300-native PECS drift-diffusion--Poisson time step.
 *
 * The reference (mdh266/PECS) is a single deal.II translation unit whose hot
 * path is driven by SolarCellProblem::run_full_system (source/SolarCell.cpp:
 * 1898-2095).  This header is the boundary that replaces, for that path:
 *
 *   - the class surface Poisson::PoissonData (include/Poisson.hpp:26-84),
 *     ChargeCarrierSpace::Carrier (include/Carrier.hpp:38-101) and
 *     ChargeCarrierSpace::CarrierPair (include/CarrierPair.hpp:30-110):
 *     pecs_lu_factor / pecs_lu_solve are set_solver() / solve();
 *   - the per-step stages of the IMEX loop (source/SolarCell.cpp:2055-2080):
 *     pecs_assemble_carrier_rhs, pecs_solve_carriers, pecs_assemble_poisson_rhs,
 *     pecs_solve_poisson, and pecs_step for the whole step;
 *   - the setup that deal.II performs once (meshes, DoF maps, the LDG and
 *     mixed matrices, UMFPACK factorisation): pecs_create.
 *
 * Conventions: every call returns 0 on success and a negative PECS_E* code on
 * failure; pecs_last_error() returns the message of the last failure on the
 * calling thread.  No call aborts the process.  Host buffers are owned by the
 * caller and copied; device memory is owned by the library.  Contexts are
 * independent; calls on one context must not overlap from several threads.
 * Any host thread may call into a context: every call that uses the GPU first
 * makes the context's device (pecs_options.device) the thread's current one,
 * and each context runs on its own stream, so contexts driven from separate
 * threads run at the same time (as the reference's four concurrent carrier
 * solves do, SolarCell.cpp:1763-1781).
 */
#ifndef PECS_H
#define PECS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes */
#define PECS_OK 0
#define PECS_E_ARG (-1)       /* invalid argument */
#define PECS_E_CUDA (-2)      /* CUDA runtime error */
#define PECS_E_SINGULAR (-3)  /* pivot below threshold during factorisation */
#define PECS_E_NONFINITE (-4) /* NaN/Inf detected in a state vector */
#define PECS_E_STATE (-5)     /* call out of sequence */
#define PECS_E_NODEVICE (-6)  /* no CUDA device available */

/* boundary ids, include/SolarCell.hpp:314-324 of the reference */
#define PECS_INTERFACE 0
#define PECS_DIRICHLET 1
#define PECS_NEUMANN 2
#define PECS_SCHOTTKY 3

/* fields of an instance's state */
#define PECS_FIELD_N 0       /* electrons  (semiconductor carrier_1) */
#define PECS_FIELD_P 1       /* holes      (semiconductor carrier_2) */
#define PECS_FIELD_R 2       /* reductants (electrolyte carrier_1)   */
#define PECS_FIELD_O 3       /* oxidants   (electrolyte carrier_2)   */
#define PECS_FIELD_POISSON 4 /* [D (RT) | Phi (DGQ_{k-1})]           */

/* matrices exported by pecs_get_matrix */
#define PECS_MAT_N 0
#define PECS_MAT_P 1
#define PECS_MAT_R 2
#define PECS_MAT_O 3
#define PECS_MAT_POISSON 4
#define PECS_MAT_MASS_SEMI 5
#define PECS_MAT_MASS_ELEC 6

/* solver precision */
#define PECS_PREC_FP64 0    /* FP64 factors and arithmetic, every solve refined once */
#define PECS_PREC_FP32_IR 1 /* FP32 factors + FP64-residual iterative refinement */
/* FP32 factors + refinement with FP32-pair ("double-float") residuals, RHS
 * quadrature terms in FP32 (constant and mass terms FP64), FP32 convergence
 * sums: the batched throughput mode (GB300 runs FP32 ~60x faster than FP64) */
#define PECS_PREC_FP32_MIXED 2

/*
 * Already-scaled parameters of one instance (the role of
 * ParameterSpace::Parameters, include/Parameters.hpp:27-289).  Profiles:
 * value[0] applies where x < junction_x, value[1] elsewhere.
 */
typedef struct pecs_params {
  int degree;      /* LDG degree k (1 or 2); Poisson element: see poisson_pairing */
  int full_system; /* 1: semiconductor + electrolyte; 0: semiconductor only */
  int nx_semi, nx_elec, ny;
  double x_semi0, x_semi1, x_elec1, height;
  int bc_semi[4], bc_elec[4], bc_poisson[4]; /* (left, right, bottom, top) */
  double lambda2;  /* scaled Debye length squared */
  double eps_semi, eps_elec;
  double mu[4];    /* mobilities: electrons, holes, reductants, oxidants */
  double dt, penalty;
  double k_et, k_ht;
  double junction_x;
  double nd[2], na[2], n_eq[2], p_eq[2];
  double r_eq, o_eq;
  int ic_kind;  /* 0: equilibrium densities, 1: doping profile */
  int gen_kind; /* 0 off, 1 alpha*G0*exp(alpha*(y-H)), 2 G0*exp(-alpha*(x_semi1-x)) */
  double G0, alpha;
  int srh;      /* 0: SRH returns 0 (reference), 1: documented SRH formula */
  double tau_n, tau_p, n_i;
  double phi_bi, phi_app; /* potential data phi_bi - phi_app where x == 0 */
  double s_n, s_p;        /* Schottky recombination velocities */
  double grading; /* widest / narrowest cell width of each region along x, cells narrowing
                     geometrically toward the interface x = x_semi1 (a boundary layer on a
                     tensor-product mesh in place of the reference's local refinement with
                     hanging nodes, Grid.cpp:71-111); 0 or 1: uniform */
  int bc_poisson_elec[4]; /* full system: ids of the Poisson mesh's outer faces over the
                             electrolyte (left unused, right, bottom, top), for layouts whose
                             sides change id at the interface (Grid.cpp:377-431); entries <= 0
                             take bc_poisson's id */
  int poisson_pairing;    /* Poisson element: 0 = RT_{k-1} x DGQ_{k-1}, the reference's pairing
                             (SolarCell.cpp:23-24); 1 = RT_k x DGQ_k, the pairing the benchmark
                             configurations name */
} pecs_params;

typedef struct pecs_options {
  int precision;     /* PECS_PREC_* */
  int leaf_cells;    /* nested-dissection leaf size in cells (0 = default) */
  int use_graphs;    /* capture a time step in a CUDA graph (1 = yes) */
  int ir_max_iters;  /* refinement sweeps per solve: FP64 residual, correction sweep
                        (0 = default: one for FP64 and FP32_MIXED, two for FP32_IR;
                        < 0 = none) */
  double ir_tol;     /* reserved: the refinement runs ir_max_iters sweeps; pecs_solve_residual
                        reports the relative residual they reached */
  int device;        /* CUDA device ordinal */
  int host_setup_only; /* 1: build meshes, matrices and factors on the host only
                          (no device work; for inspecting the setup) */
  int panel_chunk;     /* panel solve kernels (>= 32 right-hand sides per factor): staged
                          block columns per chunk (0 = default: 128 FP32, 64 FP64) */
  int panel_min_ctas;  /* panel solve kernels: CTAs a level must reach before shorter row
                          tiles or fewer right-hand sides per CTA are used (0 = default 152) */
  int autotune;        /* panel solve kernels: at creation, choose every tree level's
                          tiling by timing whole sweeps (1 = yes, the default;
                          0 = the heuristic above) */
  int gpu_factor_min_front; /* factorisation: fronts with at least this many rows are
                               factored in FP64 on the GPU (0 = default 1024; < 0 = all
                               on the host); host_setup_only contexts factor on the host */
  int flow_sweep;      /* solve sweeps: one persistent launch per sweep direction, nodes
                          started as soon as their children (forward) or parent (backward)
                          finish, instead of one launch per tree level (0 = default: when
                          the autotuner times it faster; 1 = wherever a flow plan applies;
                          -1 = never).  Panel banks: a flow plan applies where the sweep
                          vector rows are whole 128-byte lines; few-right-hand-side banks:
                          up to 16 (FP64: 8) right-hand sides per set */
  int increment_solves; /* PECS_PREC_FP32_MIXED: time steps solve for the increment from the
                           previous step's solution -- the residual b - K u_prev in FP32 pairs,
                           one FP32 sweep, u = u_prev + increment -- instead of a sweep and a
                           refinement sweep from zero; the residual vanishes at the fixed
                           point, which is therefore the refined mixed mode's.  Initial and
                           refill solves keep the refinement.  (1 = on, 0 = default: off) */
} pecs_options;

typedef struct pecs_info {
  int n_inst;
  int ndofs[5];            /* per field */
  long long factor_entries[3]; /* stored entries: semi carriers, elec carriers, Poisson */
  int factor_levels[3];
  int factor_nodes[3];
  long long factor_bytes;  /* device bytes of all factors */
  double setup_seconds;    /* host assembly + factorisation */
  int n_distinct_carrier_factors;
  int launches_per_step;   /* kernel launches of one step incl. steady-state test */
  double solve_bytes[2];   /* algorithmic bytes of one carrier / Poisson solve sweep */
  int solve_launches[2];   /* kernel launches of one carrier / Poisson solve sweep */
  int setup_launches;      /* kernel launches issued by pecs_create (tiling autotuner) */
  int initialize_launches; /* kernel launches of pecs_initialize */
  double tuned_sweep_ms[2]; /* autotuner: time of the tuned carrier / Poisson sweep (0: untuned) */
  int flow_rpl[2];         /* carrier / Poisson sweeps: right-hand sides per lane of the flow
                              sweep in use (0: one launch per tree level) */
  int flow_top[2];         /* carrier / Poisson sweeps: tree levels (from the root side) the
                              flow launches cover (0: none); the others are launched level
                              by level */
} pecs_info;

typedef struct pecs_ctx pecs_ctx;

const char* pecs_last_error(void);
void pecs_default_options(pecs_options* opt);

/* The reference's boundary layouts on p, replacing Grid::make_grids' id
 * assignment (Grid.cpp:112-131): every outer side Dirichlet and the
 * semiconductor-electrolyte faces Interface (make_Dirichlet_boundaries,
 * Grid.cpp:343-373); insulated != 0 adds make_Neumann_boundaries
 * (Grid.cpp:377-431: left side Neumann, top and bottom Neumann over the
 * electrolyte); schottky != 0 adds make_Schottky_boundaries (Grid.cpp:434-461:
 * the top of the semiconductor and Poisson meshes).  Sets bc_semi, bc_elec,
 * bc_poisson and bc_poisson_elec for p->full_system; no other field changes.
 * Host only. */
int pecs_apply_boundary_layout(pecs_params* p, int insulated, int schottky);

/* Physical parameters as input_file.prm gives them (the sections computational,
 * mesh, physical, electrons, holes, reductants, oxidants that
 * ParameterReader::declare_parameters declares, ParameterReader.cpp:29-208),
 * in the reference's units. */
typedef struct pecs_physical_params {
  double time_step;   /* computational/time step size (already scaled) */
  double mesh_height; /* mesh/mesh height (already scaled; the generation's incident line) */
  int illuminated;    /* physical/illumination status */
  double applied_bias, built_in_bias, schottky_bias; /* [V] */
  double characteristic_length;  /* [cm] */
  double characteristic_density; /* [cm^-3] */
  double characteristic_time;    /* [s] */
  double intrinsic_density;      /* [cm^-3] */
  double photon_flux;            /* [cm^-2 s^-1] */
  double absorption_coeff;       /* [cm^-1] */
  double semiconductor_permittivity, electrolyte_permittivity; /* relative */
  double electron_mobility, hole_mobility, reductant_mobility, oxidant_mobility; /* [cm^2/(V s)] */
  double electron_recombination_time, hole_recombination_time;         /* [s] */
  double electron_recombination_velocity, hole_recombination_velocity; /* [cm/s] */
  double electron_transfer_rate, hole_transfer_rate;                   /* [cm^4/s] */
} pecs_physical_params;

/* Scale factors the reference keeps beside the scaled values. */
typedef struct pecs_scales {
  double mobility_scale;  /* T V_t / L^2 */
  double rescale_current; /* q rho L / T: scaled current density -> [A cm^-2] */
  double rescaled_k_et, rescaled_k_ht; /* q k rho^2 with the unscaled rate constants */
  double schottky_bias;   /* scaled Schottky bias (no pecs_params field: the reference never
                             places its Schottky data, SolarCell.cpp:49-50) */
} pecs_scales;

/* The values of the reference's input_file.prm. */
void pecs_reference_physical_params(pecs_physical_params* ph);

/* Parameters::parse_and_scale_parameters (include/Parameters.hpp:117-287,
 * scaling 181-243) and the constructor's hand-off of the scaled values
 * (SolarCell.cpp:44-92): writes into p the scaled n_i, tau_n, tau_p, s_n, s_p,
 * G0, alpha and gen_kind (1 when illuminated, else 0 with G0 = alpha = 0),
 * lambda2, mu[0..3], k_et, k_ht, phi_app, phi_bi, eps_semi, eps_elec, dt and
 * height, evaluated in the reference's operation order; every other field of p
 * is left as it is.  scales may be NULL.  Host only. */
int pecs_scale_params(const pecs_physical_params* ph, pecs_params* p, pecs_scales* scales);

/* Setup: meshes, DoF maps, LDG + mixed matrices, LU factors, upload.
 * `params` holds n_inst instances; all must share the fields that enter the
 * matrices (mesh, degree, boundary layout, lambda2, eps, mu, dt, penalty). */
int pecs_create(const pecs_params* params, int n_inst, const pecs_options* opt, pecs_ctx** out);
void pecs_destroy(pecs_ctx* ctx);
int pecs_get_info(pecs_ctx* ctx, pecs_info* info);

/* CSR export of a setup matrix (which = PECS_MAT_*).  Call with NULL arrays to
 * query n and nnz. */
int pecs_get_matrix(pecs_ctx* ctx, int which, int* n, long long* nnz, int* rowptr, int* col,
                    double* val);

/* Host-computed per-instance vectors of the setup (also on host_setup_only
 * contexts), ndofs[field] doubles into out (n: its capacity in doubles):
 *   PECS_SETUP_CONST_RHS: the time-independent right-hand-side part of a field
 *     (generation and Dirichlet data of the carriers, SolarCell.cpp:1073-1401,
 *     1451-1726; doping and potential data of Poisson, SolarCell.cpp:487-815);
 *   PECS_SETUP_INITIAL: the projected initial density of a carrier field
 *     (SolarCell.cpp:1996-2027; currents zero), before the initial Poisson
 *     solve. */
#define PECS_SETUP_CONST_RHS 0
#define PECS_SETUP_INITIAL 1
int pecs_get_setup_vector(pecs_ctx* ctx, int kind, int field, int inst, double* out, long long n);

/* Cell edges of a mesh (the triangulations of Grid::make_grids, Grid.cpp:44-133):
 * nx + 1 x-coordinates into xs and ny + 1 y-coordinates into ys; cells are
 * numbered i + nx*j.  Call with NULL arrays to query nx and ny. */
#define PECS_MESH_SEMI 0
#define PECS_MESH_ELEC 1
#define PECS_MESH_POISSON 2
int pecs_get_mesh(pecs_ctx* ctx, int mesh, int* nx, int* ny, double* xs, double* ys);

/* Initial conditions (SolarCell.cpp:1996-2034): L2 projection of the initial
 * profiles, then the initial Poisson solve. */
int pecs_initialize(pecs_ctx* ctx);
int pecs_set_state(pecs_ctx* ctx, int inst, int field, const double* host, size_t n);
int pecs_get_state(pecs_ctx* ctx, int inst, int field, double* host, size_t n);
/* the same with device pointers (no host round trip) */
int pecs_get_state_device(pecs_ctx* ctx, int inst, int field, double* dst_dev);
int pecs_set_state_device(pecs_ctx* ctx, int inst, int field, const double* src_dev);
/* Replace the per-instance parameters of all n_inst instances (bias,
 * generation, doping, lifetimes, rate constants...): right-hand-side data and
 * initial states are rebuilt, matrices and factors are kept.  Fields that
 * enter the matrices must not change. */
int pecs_set_instances(pecs_ctx* ctx, const pecs_params* params, int n_inst);
/* right-hand side of the last assembly (field = PECS_FIELD_*) */
int pecs_get_rhs(pecs_ctx* ctx, int inst, int field, double* host, size_t n);

/* Stages of one IMEX step (SolarCell.cpp:2057-2075). */
int pecs_assemble_carrier_rhs(pecs_ctx* ctx); /* assemble_semiconductor_rhs + assemble_electrolyte_rhs */
int pecs_solve_carriers(pecs_ctx* ctx);       /* solve_full_system */
int pecs_assemble_poisson_rhs(pecs_ctx* ctx); /* assemble_Poisson_rhs */
int pecs_solve_poisson(pecs_ctx* ctx);        /* solve_Poisson */
int pecs_step(pecs_ctx* ctx, int n_steps);    /* n full steps */

/* March every instance until max over fields of ||u^{n+1}-u^n||/||u^{n+1}||
 * <= tol or max_steps; converged instances stop updating.  steps and
 * rel_change (n_inst entries each, may be NULL) receive per-instance results. */
int pecs_run_to_steady_state(pecs_ctx* ctx, int max_steps, double tol, int check_every,
                             int* steps, double* rel_change);
/* I_Sigma = int_Sigma [k_et (n-n_e) o - k_ht (p-p_e) r] ds per instance. */
int pecs_interface_current(pecs_ctx* ctx, double* out);
/* One I-V sweep end to end: initial state from host (n_inst x ndofs per field,
 * NULL = built-in initial conditions), run to steady state, copy back the
 * interface currents and (optionally) the final densities. */
int pecs_iv_sweep(pecs_ctx* ctx, const double* const* init_fields, int max_steps, double tol,
                  int check_every, double* currents, int* steps, double* const* final_fields);
/* Streamed I-V sweep: n_points parameter sets (same meshes and fixed matrices
 * as the context) marched through the context's n_inst slots.  Every
 * check_every steps, slots whose point converged (relative change <= tol) or
 * marched max_steps are harvested and refilled with the next points, so the
 * batch stays full until the list runs out.  init_n / init_p: NULL, or
 * n_points DEVICE pointers (entries may be NULL = built-in initial condition)
 * to full electron / hole vectors, e.g. a learned warm start.  Outputs per
 * point (host): steps (to convergence; max_steps when capped; negative when
 * the state became non-finite), currents (interface current) and, when
 * final_fields is not NULL, final_fields[f] -> n_points x ndofs[f] doubles
 * (NULL entries skipped).  No reference counterpart: the reference marches
 * one bias point per SolarCellProblem::run (source/SolarCell.cpp). */
int pecs_sweep_stream(pecs_ctx* ctx, int n_points, const pecs_params* params,
                      const double* const* init_n, const double* const* init_p, int max_steps, double tol,
                      int check_every, int* steps, double* currents, double* const* final_fields);
int pecs_synchronize(pecs_ctx* ctx);
/* Largest relative residual ||b - A x|| / ||b|| (FP64) over the instances and
 * fields of the latest carrier (which = 0) or Poisson (1) solve: b the last
 * assembled right-hand sides, x the state they were solved into.  Reports
 * what the refinement of the FP32 modes reached.  No reference counterpart
 * (UMFPACK's direct solves in Carrier.cpp:34-40 are not checked). */
int pecs_solve_residual(pecs_ctx* ctx, int which, double* max_rel);
/* Time steps executed by the last pecs_run_to_steady_state / pecs_iv_sweep
 * (including steps of a polling interval after the last instance converged). */
int pecs_last_run_steps(pecs_ctx* ctx);
/* CUDA stream the context launches on (cudaStream_t as void*). */
void* pecs_get_stream(pecs_ctx* ctx);
/* Mean device time (CUDA events on the context's stream) of `reps` back-to-back
 * applications of the carrier (which = 0) or Poisson (1) factors to all RHS. */
int pecs_time_solve(pecs_ctx* ctx, int which, int reps, double* ms_per_solve);
/* Mean device time (CUDA events on the context's stream) of the four stages of
 * `reps` full time steps, launched back to back after one untimed step: ms[0]
 * carrier right-hand sides, ms[1] carrier solves, ms[2] Poisson right-hand
 * side, ms[3] Poisson solve -- the sections the reference's TimerOutput times
 * inside its time loop (SolarCell.cpp:2057-2075).  The steps advance the
 * state. */
int pecs_time_stages(pecs_ctx* ctx, int reps, double* ms);

/* ---- element matrices of the reference's local assembly members ----------
 * Host only.  One axis-aligned cell (the data a deal.II cell iterator gives
 * the reference's assembly): its size, the boundary id of each face (left,
 * right, bottom, top; -1 = interior) and its material id (0, 1
 * semiconductor, 2, 3 electrolyte).  Outputs are row-major; carrier local
 * dofs [J_x (n1) | J_y (n1) | u (n1)], n1 = (k+1)^2; Poisson local dofs
 * [D_x | D_y | Phi] of the library's nodal RT basis.  pecs_element_sizes
 * gives the block sizes. */
typedef struct pecs_cell {
  double hx, hy;
  int boundary_id[4];
  int material_id;
} pecs_cell;
int pecs_element_sizes(int degree, int poisson_pairing, int* carrier_dofs, int* poisson_rt_dofs,
                       int* poisson_phi_dofs);
/* LDG::assemble_local_LDG_mass_matrix (LDG.cpp:40-83): (1/delta_t) v u on the
 * density block, zero elsewhere. */
int pecs_ldg_local_mass_matrix(int degree, const pecs_cell* cell, double delta_t, double* out);
/* LDG::assemble_local_LDG_cell_and_bc_terms (LDG.cpp:85-281) for both carriers
 * of a pair: (transient_or_steady/delta_t) v u + (1/mu) p.q - div(p) u -
 * grad(v).q, Dirichlet faces v (n.q + penalty/h u), other boundary faces
 * (p.n) u; h = the cell diagonal (cell->diameter(), LDG.cpp:117). */
int pecs_ldg_local_cell_and_bc_terms(int degree, const pecs_cell* cell, double mobility_1,
                                     double mobility_2, double delta_t, double transient_or_steady,
                                     double penalty, double* out_1, double* out_2);
/* LDG::assemble_local_flux_terms (LDG.cpp:429-622) on the face `face` of cell
 * (interior side i) shared with neighbor (exterior side e, its opposite
 * face): the blocks vi_ui, vi_ue, ve_ui, ve_ue with the reference's flux --
 * averages of p.n and v, beta.p with beta = (1,1)/sqrt(2) (LDG.cpp:455-501)
 * and penalty / min(h_i, h_e) -- as its assemble_flux_terms loop calls it
 * from the lower-numbered cell (the left / bottom one on these meshes). */
int pecs_ldg_local_flux_terms(int degree, const pecs_cell* cell, int face, const pecs_cell* neighbor,
                              double penalty, double* vi_ui, double* vi_ue, double* ve_ui, double* ve_ue);
/* MixedFEM::assemble_local_Poisson_matrix (MixedFEM.cpp:29-164):
 * p.(1/eps) D - div(p) Phi - lambda^2 v div(D), eps by the cell's material. */
int pecs_mixed_local_poisson_matrix(int degree, int poisson_pairing, const pecs_cell* cell,
                                    double semi_permittivity, double elec_permittivity,
                                    double scaled_debye_length, double* out);

/* ---- drop-in direct solver for an externally assembled matrix ------------
 * Carrier::set_solver / PoissonData::set_solver (Carrier.cpp:26-32,
 * Poisson.cpp:90-96) and their solve() (Carrier.cpp:34-40, Poisson.cpp:98-105).
 * dof_cell[i] names the mesh cell that owns dof i (faces: either neighbour),
 * cell_xy holds the cell centres (2 per cell) used by nested dissection,
 * dof_class[i] = 0 marks dofs whose diagonal blocks are cell-local and
 * mutually uncoupled across cells (the LDG current dofs), which are then
 * eliminated first; NULL = all dofs class 1. */
typedef struct pecs_lu pecs_lu;
int pecs_lu_factor(int n, const int* rowptr, const int* col, const double* val,
                   const int* dof_cell, const int* dof_class, int n_cells, const double* cell_xy,
                   int precision, int leaf_cells, pecs_lu** out);
/* Fronts of at least this many rows are factored in FP64 on the current GPU
 * by later pecs_lu_factor calls of this process (default 1024; < 0: always on
 * the host, as without a GPU).  Returns the previous value. */
int pecs_lu_set_gpu_factor_min_front(int rows);
int pecs_lu_solve(pecs_lu* lu, int nrhs, const double* b, double* x); /* host arrays, nrhs*n */
int pecs_lu_solve_device(pecs_lu* lu, int nrhs, const double* b_dev, double* x_dev, void* stream);
int pecs_lu_stats(pecs_lu* lu, long long* entries, int* levels, int* nodes, int* max_front);
void pecs_lu_destroy(pecs_lu* lu);

/* Same solve as pecs_lu_solve_device for callers that cannot allocate device
 * memory when they solve (their own pool owns the GPU's memory, or they run
 * under a fixed memory budget).  It has no counterpart in the reference.  The
 * sweeps' scratch lives in one file-scope device array of 2^20 doubles (8 MiB);
 * a solve needs nrhs*(n + update-vector length) doubles of it and nrhs <= 8,
 * larger requests return PECS_E_ARG.  Nothing is allocated: the factors must
 * already be on the current device (any earlier pecs_lu_solve or
 * pecs_lu_solve_device call on the handle uploads them), else PECS_E_STATE.
 * That upload also reserves the array on the device (CUDA loads the module
 * holding it then) and looks up its device address, so this call never
 * triggers a load; the device holds the array until the process exits.  The
 * call is synchronous: it returns when the solve has finished on `stream`.
 * All calls share the array and leave their contents in it (every value a
 * sweep reads is written earlier in the same sweep, so nothing needs
 * clearing); calls that overlap on the GPU race on it. */
int pecs_lu_solve_device_noalloc(pecs_lu* lu, int nrhs, const double* b_dev, double* x_dev,
                                 void* stream);

/* ---- learned warm start: neural operator (no counterpart in the reference) ----
 * A small MLP maps the parameters of an instance to coefficients of a fixed
 * low-rank basis of the steady-state fields; its prediction initialises the
 * time marching.  GEMM operands BF16, accumulation FP32, FP32 master weights,
 * Adam.  widths has n_layers+1 entries (input .. output); hidden layers use
 * tanh.  Parameters are packed per layer as W (out x in, row-major) then b.
 * All x/y/t pointers are device pointers to row-major (batch x width) FP32. */
typedef struct pecs_mlp pecs_mlp;
int pecs_mlp_create(int n_layers, const int* widths, unsigned long long seed, pecs_mlp** out);
void pecs_mlp_destroy(pecs_mlp* m);
int pecs_mlp_n_params(pecs_mlp* m, long long* n);
int pecs_mlp_get_params(pecs_mlp* m, float* host);
int pecs_mlp_set_params(pecs_mlp* m, const float* host);
int pecs_mlp_forward(pecs_mlp* m, int batch, const float* x_dev, float* y_dev, void* stream);
/* gradient of mean((y - t)^2) w.r.t. the packed parameters, no update */
int pecs_mlp_gradients(pecs_mlp* m, int batch, const float* x_dev, const float* t_dev, float* grad_host,
                       float* loss);
int pecs_mlp_train_step(pecs_mlp* m, int batch, const float* x_dev, const float* t_dev, float lr,
                        float* loss);
/* y (batch x n) = mean + c (batch x r) V^T with V (n x r); FP32 */
int pecs_decode(int batch, int r, int n, const float* c_dev, const float* V_dev, const float* mean_dev,
                float* y_dev, void* stream);
/* Warm-start carrier vectors from the network's coefficients c (batch x r):
 * y = mean + V c over the 2 n_u log-density outputs (V: 2 n_u x r, FP32), and
 * per row full electron / hole vectors (batch x nd doubles, device) with
 * exp(y) in the density block at u_off and zero currents.  Synchronous. */
int pecs_warm_start_vectors(int batch, int r, int n_u, const float* c_dev, const float* V_dev,
                            const float* mean_dev, int nd, int u_off, double* vn_dev, double* vp_dev,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PECS_H */
