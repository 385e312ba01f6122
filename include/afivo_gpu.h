/*
 * afivo_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of the
 * afivo-streamer per-timestep hot path.
 *
 * The reference is Fortran 2008 (MD-CWI/afivo-streamer).  Its callers stay as
 * they are; the bodies of the public afivo routines gain a branch that calls
 * these functions through ISO_C_BINDING interfaces.  Every
 * function returns an int status: AFG_OK (0) or a negative AFG_ERR_* code;
 * afg_last_error() gives a one-line reason.  Nothing here aborts or traps:
 * device-side failures are raised in a device error word that is read back on
 * synchronisation.
 *
 * Conventions honoured (afivo/src/m_af_types.f90):
 *   - box ids are 1-based, 0 = af_no_box, -1 = af_phys_boundary (38-41);
 *   - children in af_child_dix order (131,169-171);
 *   - neighbours lowx, highx, lowy, highy[, lowz, highz] (142-150,186-198);
 *   - neighbor_mat(-1:1,-1:1[,-1:1]) with the first index fastest (297);
 *   - per box, cell-centred data cc(0:nc+1, 0:nc+1[, 0:nc+1], n_var_cell)
 *     column-major (i fastest, then j, k, variable) (302,
 *     m_af_core.f90:548-550);
 *   - face-centred data fc(1:nc+1, 1:nc+1[, 1:nc+1], NDIM, n_var_face)
 *     (303, m_af_core.f90:549);
 *   - variable indices are 1-based like the Fortran tree%cc_names index.
 *
 * Threading: one context per tree, used from one host thread (the reference
 * calls these routines from serial code; its OpenMP is inside them).
 */
#ifndef AFIVO_GPU_H
#define AFIVO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define AFG_OK               0
#define AFG_ERR_ARG         -1  /* invalid argument / inconsistent tables   */
#define AFG_ERR_CUDA        -2  /* a CUDA runtime call failed               */
#define AFG_ERR_UNSUPPORTED -3  /* feature outside the GPU path (LSF, ...)  */
#define AFG_ERR_STATE       -4  /* call order violated (no tree, no mg ...) */
#define AFG_ERR_DEVICE      -5  /* a kernel raised its device error word    */
#define AFG_ERR_NOCONV      -6  /* iteration limit reached                  */
#define AFG_ERR_NOMEM       -7  /* device allocation failed                 */

/* ---- enumerations (values equal to afivo's constants) ------------------ */
#define AFG_XYZ 1               /* af_xyz, m_af_types.f90:47 */
#define AFG_CYL 2               /* af_cyl, m_af_types.f90:50 */

#define AFG_BC_DIRICHLET      -10   /* af_bc_dirichlet      (m_af_types.f90:57) */
#define AFG_BC_NEUMANN        -11   /* af_bc_neumann        (60) */
#define AFG_BC_CONTINUOUS     -12   /* af_bc_continuous     (63) */
#define AFG_BC_DIRICHLET_COPY -13   /* af_bc_dirichlet_copy (68) */

/* Refinement-boundary ghost rule of a cell-centred variable
 * (af_cc_methods%rb, m_af_types.f90:248-263). */
#define AFG_RB_MG_SIDES   0     /* mg_sides_rb        m_af_multigrid.f90:294-461 */
#define AFG_RB_INTERP     1     /* af_gc_interp       m_af_ghostcell.f90:394-498 */
#define AFG_RB_INTERP_LIM 2     /* af_gc_interp_lim   m_af_ghostcell.f90:503-612 */

/* Precision of a multigrid solve. */
#define AFG_FP64  0  /* plain FP64 FAS V-cycle, operation order of the reference */
#define AFG_MIXED 1  /* FP64 defect correction around an FP32 V-cycle            */

/* V-cycle smoothing stage (mg_cycle_down / mg_cycle_up, m_af_types.f90:544-545) */
#define AFG_CYCLE_DOWN 1
#define AFG_CYCLE_UP   3

typedef struct afg_ctx afg_ctx;

/* Tree tables: a flat view of af_t (m_af_types.f90:326-393).  Arrays are
 * indexed by (id-1); multi-valued entries are contiguous per box.  The level
 * lists are concatenated: level l (1-based) occupies
 * ids[ids_off[l-1] .. ids_off[l]-1]; same for leaves and parents. */
typedef struct afg_tree_desc {
  int ndim;                  /* 2 or 3 (NDIM)                                */
  int n_cell;                /* tree%n_cell (even, >= 2)                     */
  int coord;                 /* AFG_XYZ or AFG_CYL (2D only)                 */
  int n_boxes;               /* tree%highest_id                              */
  int highest_lvl;           /* tree%highest_lvl                             */
  int coarse_grid_size[3];   /* tree%coarse_grid_size                        */
  const int* lvl;            /* [n_boxes]            box%lvl                 */
  const int* ix;             /* [n_boxes][ndim]      box%ix                  */
  const int* parent;         /* [n_boxes]            box%parent              */
  const int* children;       /* [n_boxes][2^ndim]    box%children            */
  const int* neighbors;      /* [n_boxes][2*ndim]    box%neighbors           */
  const int* neighbor_mat;   /* [n_boxes][3^ndim]    box%neighbor_mat        */
  const double* r_min;       /* [n_boxes][ndim]      box%r_min               */
  const double* dr;          /* [n_boxes][ndim]      box%dr                  */
  const int* ids_off;     const int* ids;      /* tree%lvls(:)%ids     */
  const int* leaves_off;  const int* leaves;   /* tree%lvls(:)%leaves  */
  const int* parents_off; const int* parents;  /* tree%lvls(:)%parents */
} afg_tree_desc;

/* Boundary conditions of one cell-centred variable: per domain face
 * (lowx, highx, lowy, highy[, lowz, highz]) a kind and a value that is
 * constant over the face, plus the refinement-boundary rule.  This is what
 * the reference's bc callbacks return for the hot-path variables
 * (field_bc_homogeneous src/m_field.f90:590-610, photoi_helmh_bc
 * src/m_photoi_helmh.f90:210-228, af_bc_neumann_zero
 * afivo/src/m_af_ghostcell.f90:614-624), evaluated once on the host. */
typedef struct afg_gc_desc {
  int bc_type[6];
  double bc_val[6];
  int rb;                    /* AFG_RB_* */
} afg_gc_desc;

/* Multigrid options: the subset of mg_t (m_af_types.f90:572-665) used by the
 * default (mg_auto_*, normal-box) operators. */
typedef struct afg_mg_desc {
  int i_phi, i_rhs, i_tmp;   /* 1-based cell-centred variable indices        */
  int n_cycle_down;          /* mg%n_cycle_down (default 2)                  */
  int n_cycle_up;            /* mg%n_cycle_up   (default 2)                  */
  double helmholtz_lambda;   /* mg%helmholtz_lambda (lambda^2)               */
  int bc_type[6];            /* mg%sides_bc evaluated per domain face        */
  double bc_val[6];
  int precision;             /* AFG_FP64 or AFG_MIXED                        */
} afg_mg_desc;

/* ---- context and tree mirror ------------------------------------------- */

/* Create a context on CUDA device `device` (replaces nothing in the
 * reference: its state lives in af_t; this holds the device mirror). */
int afg_init(int device, afg_ctx** ctx);
int afg_finalize(afg_ctx* ctx);
const char* afg_last_error(const afg_ctx* ctx);

/* (Re)build the device mirror after af_init/mg_init and after every
 * af_adjust_refinement that added or removed boxes (src/streamer.f90:418).
 * Allocates n_var_cell cell-centred and n_var_face face-centred FP64 pools.
 * Data of variables is NOT kept across a sync: upload it again. */
int afg_tree_sync(afg_ctx* ctx, const afg_tree_desc* tree,
                  int n_var_cell, int n_var_face);

/* Batched independent instances (no counterpart in the reference, which runs
 * one tree per process): `tree` is a forest of n_inst trees with disjoint box
 * ids, box_inst[id-1] in 0..n_inst-1 the instance of box id.  No parent,
 * child or neighbour relation may cross instances, and the coarse grids
 * (level 1) must be alike: the same coarse_grid_size, with boxes at the same
 * ix with the same r_min and dr (the instances share one factored
 * coarse-grid operator; uneven grids differ in their number of levels).
 * Every level is then processed in one launch per stage for all instances.
 * Boundary values of a multigrid slot can differ per instance
 * (afg_mg_set_bc_values_inst); afg_field_compute_inst and afg_mg_solve_inst
 * converge each instance to its own threshold, freezing converged instances,
 * so each instance's result is the same as a run of its own tree.
 * Photoionization of batched instances is not supported. */
int afg_tree_sync_batched(afg_ctx* ctx, const afg_tree_desc* tree,
                          int n_var_cell, int n_var_face, int n_inst,
                          const int* box_inst);
/* number of instances of a batched tree (0 for a single tree) */
int afg_n_instances(const afg_ctx* ctx);

/* Copy cell-centred variable iv between host boxes and the device pool.
 * box_cc[id-1] points at box%cc(0,0[,0],1) of box id (NULL = skip); the data
 * of variable iv starts elem_offset doubles after it ((iv-1)*(nc+2)^ndim for
 * a Fortran box).  Ghost cells are copied too. */
int afg_cc_upload(afg_ctx* ctx, int iv, const double* const* box_cc,
                  long long elem_offset);
int afg_cc_download(afg_ctx* ctx, int iv, double* const* box_cc,
                    long long elem_offset);

/* Transfer paths of the four copy routines, when every box pointer is
 * non-NULL and the pointers are equally spaced:
 *   - all boxes inside one range page-locked by afg_host_register: the GPU
 *     reads/writes the mapped host memory directly (one kernel);
 *   - other page-locked memory (e.g. cudaMallocHost): one pitched DMA.
 * Otherwise the boxes are gathered/scattered by host threads through a
 * page-locked staging buffer, overlapped with the DMA in 32 MiB chunks.
 * Every copy has completed when the call returns. */

/* As afg_cc_download, but for boxes inside a range registered with
 * afg_host_register (equally spaced pointers) the copy is only started: it
 * runs on a transfer stream after all work issued so far and the call returns
 * at once, so it can overlap later work that does not write variable iv.
 * The caller must not write iv on the device, nor read or free the host
 * boxes, before afg_transfers_wait.  Other host memory: a synchronous copy.
 * No counterpart in the reference. */
int afg_cc_download_async(afg_ctx* ctx, int iv, double* const* box_cc,
                          long long elem_offset);
/* Autotuner: the work shape of the smoother (cells per thread, i.e. threads
 * per box) is timed on the largest level and the fastest kept.  It runs when
 * the first AFG_MIXED slot is set up on a tree (its FP32 buffers are the
 * scratch); afg_autotune repeats it for slot mg_id (AFG_MIXED).  All variants
 * compute the same values.  afg_tuning reports the choice: out[0] FP32,
 * out[1] FP64 cells per thread (0: not a tuned box size).  No counterpart in
 * the reference. */
int afg_autotune(afg_ctx* ctx, int mg_id);
int afg_tuning(const afg_ctx* ctx, int* out);
/* Set the smoother variants instead (in[0] FP32, in[1] FP64; 0 = default):
 * cells per thread 1, 2, 4, 8 (3D 8^3) or 1, 2, 4 (2D 16^2), or 16 + cells
 * per thread for the shared-memory-staged persistent variant (bulk copies of
 * each box's phi into shared memory, double-buffered; 3D: 18, 20; 2D: 17,
 * 18), plus 32 when the rhs block is staged as well (3D: 50, 52; 2D: 49,
 * 50).  afg_tuning reports the codes the same way.  With the compact FP32
 * layout (afg_set_fp32_layout, the default) in[0] selects among 0 (one box
 * per CTA, any box size) and 16 + 1, 2 or 4 cells per thread for the staged
 * persistent kernel (8^3 and 16^2 boxes). */
int afg_set_tuning(afg_ctx* ctx, const int* in);

/* Layout of the FP32 correction buffers of AFG_MIXED solves (internal to
 * the library): compact != 0 (the default) keeps each box's interior cells
 * in two colour halves of a red-black ordering with the ghost cells apart,
 * so a half sweep moves one contiguous half per box and operand; 0 keeps
 * the (nc+2)^D ghosted layout of the FP64 variables.  Both give the same
 * results bit for bit.  Takes effect for the next solves; call it before
 * afg_mg_setup so that the autotuner times the chosen layout.  No
 * counterpart in the reference. */
int afg_set_fp32_layout(afg_ctx* ctx, int compact);

/* Check of the device-side failure path: a kernel whose bounded mbarrier
 * wait cannot complete (copies announced, none issued) gives up after 1 s,
 * raises the context's error word and returns; the error is read back as
 * after every solve iteration and cleared.  Returns AFG_ERR_DEVICE when the
 * timeout was detected and reported (the expected outcome; the context stays
 * usable), waited_ms the kernel's duration.  No counterpart in the
 * reference. */
int afg_check_bounded_wait(afg_ctx* ctx, double* waited_ms);

/* Wait for the copies started by afg_cc_download_async. */
int afg_transfers_wait(afg_ctx* ctx);

/* Page-lock and map (cudaHostRegister) / release caller-owned host memory,
 * e.g. the storage behind the box arrays passed to the copy routines; the
 * context remembers the range until afg_host_unregister (same ptr).  No
 * counterpart in the reference (its data never leaves the host). */
int afg_host_register(afg_ctx* ctx, void* ptr, size_t bytes);
int afg_host_unregister(afg_ctx* ctx, void* ptr);

/* Same for face-centred variable ivf: box_fc[id-1] points at
 * box%fc(1,1[,1],1,1); elem_offset = (ivf-1)*NDIM*(nc+1)^ndim. */
int afg_fc_upload(afg_ctx* ctx, int ivf, const double* const* box_fc,
                  long long elem_offset);
int afg_fc_download(afg_ctx* ctx, int ivf, double* const* box_fc,
                    long long elem_offset);

/* Register the ghost-cell methods of variable iv (af_set_cc_methods,
 * afivo/src/m_af_core.f90:343-427). */
int afg_set_cc_methods(afg_ctx* ctx, int iv, const afg_gc_desc* gc);

/* af_gc_lvl / af_gc_tree (afivo/src/m_af_ghostcell.f90:24-61): fill ghost
 * cells of variable iv on level lvl (lvl = 0: all levels, coarse to fine),
 * with corner/edge ghosts when corners != 0. */
int afg_gc(afg_ctx* ctx, int iv, int lvl, int corners);

/* af_tree_maxabs_cc (afivo/src/m_af_utils.f90:773-784): max |cc(.., iv)|
 * over interior cells of the leaves (leaves_only != 0) or of all boxes. */
int afg_maxabs(afg_ctx* ctx, int iv, int leaves_only, double* result);

/* ---- multigrid (afivo/src/m_af_multigrid.f90) --------------------------- */

/* mg_init (43-109): store the operator of solver slot mg_id (0..15) and
 * factor its coarse-grid operator (replaces coarse_solver_initialize,
 * m_coarse_solver.f90:71-101, whose hypre PFMG is swapped for an exact
 * FP64 direct solve of the same matrix). */
int afg_mg_setup(afg_ctx* ctx, int mg_id, const afg_mg_desc* mg);

/* Change only the boundary values of slot mg_id (e.g. a new applied voltage,
 * field_set_voltage src/m_field.f90:551-586); kinds must stay the same. */
int afg_mg_set_bc_values(afg_ctx* ctx, int mg_id, const double* bc_val);
/* Batched trees: boundary values per instance, bc_val[q*6 + face]. */
int afg_mg_set_bc_values_inst(afg_ctx* ctx, int mg_id, const double* bc_val);

/* mg_fas_vcycle (185-264).  max_lvl <= 0 means tree%highest_lvl.  When
 * set_residual != 0 the residual is stored in i_tmp and, if max_res is not
 * NULL, max over leaves of |residual| is returned in it. */
int afg_mg_vcycle(afg_ctx* ctx, int mg_id, int set_residual, int max_lvl,
                  double* max_res);

/* mg_fas_fmg (137-180).  For an AFG_MIXED slot one call is one
 * defect-correction step: FP64 defect of phi (zero without a guess), FP32
 * FMG for the correction with homogeneous boundary values, phi += correction;
 * max_res is the FP64 defect's maximum over the leaves (i_tmp is not
 * written). */
int afg_mg_fmg(afg_ctx* ctx, int mg_id, int set_residual, int have_guess,
               double* max_res);

/* Run V-cycles until max|residual| over leaves < threshold or max_cycles is
 * reached (the loop of field_compute, src/m_field.f90:520-524).  With
 * precision AFG_MIXED each cycle is an FP64 residual + FP32 V-cycle on the
 * correction + FP64 update (defect correction).  n_done and the final
 * residual are returned; residuals[] (may be NULL) receives the history. */
int afg_mg_solve(afg_ctx* ctx, int mg_id, double threshold, int max_cycles,
                 int* n_done, double* residuals);
/* Batched trees: per instance until its residual < threshold[q];
 * n_done[q] iterations and residual[q] (either may be NULL).  On a batched
 * tree afg_mg_solve applies one threshold to all instances and reports the
 * most iterations (residuals[n_done-1] = the largest final residual). */
int afg_mg_solve_inst(afg_ctx* ctx, int mg_id, const double* threshold,
                      int max_cycles, int* n_done, double* residual);

/* Single stages, for parity testing of each kernel against the oracle:
 * gsrb_boxes (648-687), update_coarse (691-738), correct_children (624-646)
 * on the parents of level lvl-1 followed by af_gc_lvl(lvl), and the coarse
 * solve solve_coarse_grid (266-291).  Like the reference's multigrid
 * routines they need valid ghost cells of i_phi on entry (the smoother
 * evaluates the ghost rules on the fly between half sweeps). */
int afg_mg_gsrb_lvl(afg_ctx* ctx, int mg_id, int lvl, int cycle_type);
int afg_mg_update_coarse(afg_ctx* ctx, int mg_id, int lvl);
int afg_mg_correct_lvl(afg_ctx* ctx, int mg_id, int lvl);
int afg_mg_coarse_solve(afg_ctx* ctx, int mg_id);
/* residual_box (801-810) on all boxes of levels 1..max_lvl into i_tmp. */
int afg_mg_residual(afg_ctx* ctx, int mg_id, int max_lvl);

/* ---- drift-diffusion transport and sources (src/m_fluid.f90) ------------ */

#define AFG_MAX_SPECIES   16
#define AFG_MAX_REACTIONS 32
#define AFG_MAX_FLUX       8

/* Reaction-rate forms, values of rate_* in src/m_chemistry.f90:65-126.  Forms
 * that depend only on the (constant) gas temperature are evaluated on the
 * host and passed as AFG_RATE_CONSTANT. */
#define AFG_RATE_TABULATED_FIELD 1  /* c0 * LT(col, Td)                      */
#define AFG_RATE_CONSTANT        2  /* c0 * c1                               */
#define AFG_RATE_LINEAR          3  /* c0 * c1 * (Td - c2)                   */
#define AFG_RATE_EXP_V1          4  /* c0 * c1 * exp(-(c2/(c3 + Td))**2)     */
#define AFG_RATE_EXP_V2          5  /* c0 * c1 * exp(-(Td/c2)**2)            */
#define AFG_RATE_K1              6  /* c0 * c1 * (300/Te)**c2 with Te = 2 eV /
                                     * (3 kB) * LT(lt_col, Td), lt_col the mean
                                     * electron energy in eV (rate_analytic_k1) */
#define AFG_RATE_K13            18  /* c0 * c1 * exp(-(c2/(c3 + Td))**c4)    */
#define AFG_RATE_K14            19  /* c0 * c1 * exp(-(Td/c2)**c3)           */

/* Slope limiters (af_limiter_*_t, afivo/src/m_af_limiters.f90) used by the
 * two-layer refinement-boundary ghost cells (gc2_prolong_rb). */
#define AFG_LIMITER_VANLEER   1
#define AFG_LIMITER_KOREN     2
#define AFG_LIMITER_MINMOD    3
#define AFG_LIMITER_MC        4
#define AFG_LIMITER_GMINMOD43 5

typedef struct afg_reaction {
  int rate_type;           /* AFG_RATE_*                                    */
  int lt_col;              /* table column of a tabulated rate (0-based)    */
  double rate_factor;      /* reactions(n)%rate_factor                      */
  double c[4];             /* reactions(n)%rate_data                        */
  int n_in;                /* species consumed (gas species excluded)       */
  int ix_in[4];            /* indices into the species list (0-based)       */
  int n_out;
  int ix_out[4];
  int mult_out[4];         /* multiplicity_out                              */
} afg_reaction;

/* Transport model: the variables and tables m_fluid/m_chemistry use
 * (src/m_streamer.f90:17-71, src/m_transport_data.f90:61-220,
 * src/m_chemistry.f90:200-300).  All indices are 1-based tree variables
 * unless stated otherwise; the density of species s in time state st is
 * cc variable species_iv[s] + st. */
typedef struct afg_transport_desc {
  int n_species;
  int species_iv[AFG_MAX_SPECIES];
  double species_charge[AFG_MAX_SPECIES];
  int n_flux;                         /* [0] electrons (drift + diffusion), then mobile ions */
  int flux_species[AFG_MAX_FLUX];     /* 0-based index into the species list */
  int flux_fc[AFG_MAX_FLUX];          /* fc variable holding each flux (flux_variables) */
  double flux_charge_sign[AFG_MAX_FLUX];
  double ion_mobility_N[AFG_MAX_FLUX];/* mobility*N of mobile ions (entry 0 unused) */
  int i_electric_fld;                 /* cc |E|  */
  int i_efield_fc;                    /* fc E    (electric_fld) */
  int i_photo;                        /* cc photoionization source; 0 = none */
  int photoi_species;                 /* 0-based species that also gains the photo source */
  double gas_number_density;          /* N, m^-3 */
  afg_gc_desc species_gc;             /* bc_species + af_gc_interp_lim */
  int prolong_limiter;                /* AFG_LIMITER_* of gc2_prolong_rb */
  /* lookup table over the reduced field Td (td_tbl and chemtbl_fld share the
   * grid, src/m_chemistry.f90:348): linear x-spacing, rows_cols(n_points, n_cols) */
  int lt_n_points;
  double lt_x_min;
  double lt_inv_fac;
  int lt_n_cols;
  const double* lt_data;              /* [n_cols][n_points] (column after column) */
  int lt_col_mobility;                /* td_mobility: mu*N   */
  int lt_col_diffusion;               /* td_diffusion: D*N   */
  int lt_col_alpha;                   /* td_alpha: alpha/N (photoionization source) */
  int n_reactions;
  afg_reaction reactions[AFG_MAX_REACTIONS];
  double dt_chemistry_nmin;           /* dt_chemistry_nmin */
  int dt_chemistry_limit_loss;        /* dt_chemistry_limit_loss */
  /* AFG_FP64: the reference's arithmetic.  AFG_MIXED: the state stays FP64
   * but the per-cell arithmetic of the fluxes, the reaction sources, the
   * field gradient and the photon production is FP32; state differences,
   * the charge density and the final density sums stay FP64.  No counterpart
   * in the reference. */
  int precision;
} afg_transport_desc;

/* Store the transport model (transport_data_initialize, chemistry_initialize). */
int afg_transport_setup(afg_ctx* ctx, const afg_transport_desc* tr);

/* flux_upwind_tree (afivo/src/m_af_flux_schemes.f90:666-712) with the fluid
 * model's flux_upwind/flux_direction (src/m_fluid.f90:102-227) and the Koren
 * limiter, for densities of state s_deriv: restriction near refinement
 * boundaries, two-layer ghost cells, upwind fluxes into the flux fc
 * variables, af_consistent_fluxes.  dt_lim[0] = CFL limit (before
 * dt_cfl_number), dt_lim[1] = dielectric relaxation time. */
int afg_flux_upwind(afg_ctx* ctx, int s_deriv, double* dt_lim);

/* flux_update_densities (m_af_flux_schemes.f90:320-436) with
 * add_source_terms (src/m_fluid.f90:298-466): state s_out = sum_m w_prev[m] *
 * state s_prev[m] + dt * (chemistry + photoionization) + dt/dr * flux
 * divergence, on all leaves.  When last_step != 0, *dt_chem receives the
 * chemistry time-step limit. */
int afg_update_densities(afg_ctx* ctx, double dt, int s_deriv, int n_prev,
                         const int* s_prev, const double* w_prev, int s_out,
                         int last_step, double* dt_chem);

/* field_set_rhs (src/m_field.f90:406-444): rhs = -e/eps0 * sum q_s n_s
 * (state s_in) on leaves. */
int afg_field_set_rhs(afg_ctx* ctx, int i_rhs, int s_in);

/* field_from_potential (src/m_field.f90:531-548): E = -grad(phi) on faces
 * of all boxes (mg_compute_phi_gradient, m_af_multigrid.f90:1857-1994), |E|
 * at cell centres (mg_box_field_norm 2015-2045), then ghost cells of |E|. */
int afg_field_from_potential(afg_ctx* ctx, int i_phi);

/* field_compute (src/m_field.f90:448-528): rhs from the charges of state
 * s_in, boundary value `voltage` on the highest face of the last dimension,
 * FMG start when have_guess == 0, V-cycles until max|residual| < threshold
 * = max(1e-6, max|rhs|*max_rel_residual, 1e-10*|V|/(domain_len*dx_min)),
 * field from potential.  n_cycles and the final residual are returned.
 * With an AFG_MIXED slot the FMG start uses the defect-correction FMG of
 * afg_mg_fmg and its stall test ends it whatever the residual's magnitude;
 * the V-cycles of the mixed solve then reach the threshold. */
int afg_field_compute(afg_ctx* ctx, int mg_id, int s_in, int have_guess,
                      double voltage, double domain_len, double max_rel_residual,
                      int num_vcycles, int* n_cycles, double* residual);
/* Batched trees: field_compute of every instance with its own voltage[q]
 * (boundary value and threshold, with the instance's own max|rhs| and
 * finest dr); n_cycles[q] FMG + V-cycles and residual[q] per instance.  On
 * a batched tree afg_field_compute uses one voltage for all instances and
 * reports the most cycles and the largest residual. */
int afg_field_compute_inst(afg_ctx* ctx, int mg_id, int s_in, int have_guess,
                           const double* voltage, double domain_len,
                           double max_rel_residual, int num_vcycles,
                           int* n_cycles, double* residual);

/* photoionization_rate_from_alpha (src/m_photoi.f90:259-291) into i_rhs on
 * leaves (coeff = eta * quenching factor), then photoi_helmh_compute
 * (src/m_photoi_helmh.f90:162-204) with the Helmholtz modes in solver slots
 * mg_ids[0..n_modes-1] (their lambda^2 set at afg_mg_setup):
 * i_photo = -sum_n coeffs[n] * phi_n on leaves. */
int afg_photoi_helmh(afg_ctx* ctx, double coeff, int n_modes, const int* mg_ids,
                     const double* coeffs, double max_rel_residual,
                     int max_fmg_cycles);
/* How afg_photoi_helmh advances AFG_MIXED modes (at most 8, with the same
 * boundary conditions and cycle counts): on != 0 (default) in lockstep, as
 * multiple right-hand sides of one FMG whose every launch covers all modes
 * not yet converged; on == 0 as parallel CUDA-graph branches, one per mode.
 * Both give the same results.  No counterpart in the reference. */
int afg_set_photoi_lockstep(afg_ctx* ctx, int on);

/* Which kernel computes the AFG_MIXED fluxes of afg_flux_upwind for boxes of
 * 8^3 or 16^2 cells and at most two flux species: on != 0 (default) the one
 * that stages each box's |E| and densities in shared memory by bulk copies,
 * on == 0 the one that reads them from global memory.  Both give the same
 * results.  No counterpart in the reference. */
int afg_set_flux_staged(afg_ctx* ctx, int on);

/* af_tree_copy_cc (afivo/src/m_af_utils.f90:590-598): whole-array copy of
 * variable iv_from to iv_to on all boxes (used by copy_current_state,
 * src/streamer.f90:659-671). */
int afg_tree_copy_cc(afg_ctx* ctx, int iv_from, int iv_to);

/* ---- one stage of the explicit integrators (src/m_fluid.f90:21-99) -------
 * The module settings that forward_euler reads (m_field's solver and its
 * convergence settings, m_dt's dt_cfl_number and dt_max). */
typedef struct {
  int mg_id;                /* solver slot of the field (m_field's mg) */
  double domain_len;        /* length of the last dimension (the field's round-off threshold) */
  double max_rel_residual;  /* relative residual the field's V-cycles stop at */
  int num_vcycles;          /* V-cycle limit of the field */
  double dt_cfl_number;     /* dt_cfl_number (src/m_dt.f90:31) */
  double dt_max;            /* dt_max (src/m_dt.f90:40) */
} afg_stage_desc;
int afg_stage_setup(afg_ctx* ctx, const afg_stage_desc* d);

/* forward_euler (src/m_fluid.f90:21-99), the stage every explicit integrator
 * of af_advance (afivo/src/m_af_advance.f90:150-199) is made of: when
 * i_step > 1 the field of state s_deriv (afg_field_compute with a guess and
 * the boundary value `voltage`, the applied voltage at the stage's time), the
 * upwind fluxes of state s_deriv (afg_flux_upwind), then state s_out from
 * the previous states, the sources and the flux divergence
 * (afg_update_densities, the chemistry limit on the last step, i_step ==
 * n_steps).  *dt_lim = min(dt_max, dt_cfl_number * CFL limit, dielectric
 * relaxation time, chemistry limit of the last step); *n_cycles (optional)
 * = the field's FMG + V-cycles (0 when i_step == 1).  AFG_ERR_ARG without
 * afg_stage_setup; on a batched tree the field is the one-voltage
 * afg_field_compute. */
int afg_forward_euler(afg_ctx* ctx, double dt, double voltage, int s_deriv, int n_prev,
                      const int* s_prev, const double* w_prev, int s_out, int i_step,
                      int n_steps, double* dt_lim, int* n_cycles);

/* ---- adaptive refinement on the device (src/streamer.f90:397-428) -------
 * The refinement decision per cell and box, the prolongation into new boxes
 * and the move of the data to the new tree run on the GPU; the change of the
 * tree itself (af_adjust_refinement's 2:1 balancing and box bookkeeping,
 * afivo/src/m_af_core.f90:697-822) stays with the caller. */

#define AFG_MAX_REFINE_ITEMS 8
#define AFG_REF_RM   -1   /* af_rm_ref   (afivo/src/m_af_types.f90:23) */
#define AFG_REF_KEEP  0   /* af_keep_ref (26)                          */
#define AFG_REF_DO    1   /* af_do_ref   (29)                          */

/* default_refinement (src/m_refine.f90:197-298) with the constant gas
 * density; the time-dependent switches are evaluated by the caller: seeds are
 * passed only while global_time < refine_init_time, regions only while
 * global_time <= their stop time.  Boxes with an electrode surface are not
 * supported (no LSF boxes on this path). */
typedef struct afg_refine_desc {
  int i_electron;              /* cc variable of the electron density       */
  int i_electric_fld;          /* cc variable of |E|                        */
  int lt_col_alpha;            /* transport-table column of alpha/N          */
  int lt_col_eta;              /* ... of eta/N (use_alpha_effective)         */
  int use_alpha_effective;     /* refine_use_alpha_effective                */
  double gas_number_density;   /* gas_number_density                        */
  double adx;                  /* refine_adx                                */
  double adx_fac;              /* refine_adx_fac                            */
  double min_dens;             /* refine_min_dens                           */
  double derefine_dx;          /* derefine_dx                               */
  double max_dx;               /* refine_max_dx                             */
  double min_dx;               /* refine_min_dx                             */
  int ref_buffer;              /* refine_buffer_width (cells)               */
  int n_seeds;                 /* init_conds seeds (lines r0 - r1)          */
  double seed_r0[AFG_MAX_REFINE_ITEMS][3];
  double seed_r1[AFG_MAX_REFINE_ITEMS][3];
  double seed_width[AFG_MAX_REFINE_ITEMS];
  double init_fac;             /* refine_init_fac                           */
  int n_regions;               /* refine_regions_* (active ones)            */
  double region_rmin[AFG_MAX_REFINE_ITEMS][3];
  double region_rmax[AFG_MAX_REFINE_ITEMS][3];
  double region_dr[AFG_MAX_REFINE_ITEMS];
  int n_limits;                /* refine_limits_*                           */
  double limit_rmin[AFG_MAX_REFINE_ITEMS][3];
  double limit_rmax[AFG_MAX_REFINE_ITEMS][3];
  double limit_dr[AFG_MAX_REFINE_ITEMS];
  int electrode_mg;            /* multigrid slot of the field's electrode   */
  double electrode_dx;         /* current_electrode_dx: the electrode boxes
                                  of that slot refine while max_dx exceeds it
                                  (src/m_refine.f90:261-265); 0 = no rule  */
} afg_refine_desc;

/* The flag pass of consistent_ref_flags (afivo/src/m_af_core.f90:929-991)
 * with default_refinement as ref_subr and cell_to_ref_flags (1095-1149) for
 * the leaves and the parents of leaves: box_flags[id-1] receives -1
 * (af_rm_ref), 0 (af_keep_ref) or 1 (af_do_ref), the maximum over all
 * contributions as in the reference (boxes without any: 0).  The max-level
 * clamp and the 2:1 consistency passes follow on the host. */
int afg_refine_flags(afg_ctx* ctx, const afg_refine_desc* d, int* box_flags);

/* af_prolong_limit (afivo/src/m_af_prolong.f90:311-420) of variable iv into
 * the n boxes ids[] (1-based) from their parents, slopes limited with
 * AFG_LIMITER_* (m_af_limiters.f90:41-66); the children's interior is
 * overwritten.  As in the reference the parents' ghost cells of iv must be
 * valid; no box of ids[] may be the parent of another (the boxes are filled
 * concurrently). */
int afg_prolong_limit(afg_ctx* ctx, int iv, int n, const int* ids, int limiter);

/* af_prolong_linear with add = .false. (afivo/src/m_af_prolong.f90:531-679)
 * of variable iv into the n boxes ids[] (1-based) from their parents: bi- or
 * trilinear weights (9,3,3,1)/16 and (27,9,3,1)/64; used by auto_prolong
 * (afivo/src/m_af_core.f90:843-881) for variables whose prolongation method
 * is the default, e.g. phi and |E| of the streamer program.  Same
 * preconditions as afg_prolong_limit. */
int afg_prolong_linear(afg_ctx* ctx, int iv, int n, const int* ids);

/* af_restrict_tree (afivo/src/m_af_restrict.f90:50-59) of variable iv: from
 * the highest level down, every box restricted into its parent by
 * af_restrict_box with geometry (cylindrical weights in 2D axisymmetric
 * trees), as done for the densities before each refinement
 * (src/streamer.f90:405-406). */
int afg_restrict_tree(afg_ctx* ctx, int iv);

/* Mirror a new tree (after the caller's af_adjust_refinement) keeping the
 * data: old_id[id-1] is the id box id had in the previous tree, 0 for a new
 * box (whose data starts at zero and is then filled by afg_prolong_limit).
 * All cell- and face-centred variables move; operators, ghost-cell methods
 * and the transport model are set up again as after afg_tree_sync.  Not for
 * batched trees. */
int afg_tree_remap(afg_ctx* ctx, const afg_tree_desc* tree, const int* old_id);

/* Host-side mesh adjustment for a caller that does not keep afivo's own tree
 * code (a Fortran caller keeps af_adjust_refinement and needs none of this):
 * af_adjust_refinement (afivo/src/m_af_core.f90:697-1091) after the flag
 * pass, i.e. from the box flags of afg_refine_flags: max-level clamp,
 * ensure_two_one_balance, handle_derefinement_flags, then the new tree with
 * afivo's 2:1 balance over face neighbours, numbered level by level (level 1
 * in coordinate order, then children of refined parents in parent-id and
 * child order).  No CUDA call; needs no context.  *out is NULL when the mesh
 * does not change; otherwise query it with afg_tree_new_sizes, copy it out
 * with afg_tree_new_get (arrays laid out as in afg_tree_desc; any pointer may
 * be NULL to skip; dr_base receives ndim values) and release it with
 * afg_tree_new_free. */
typedef struct afg_tree_new afg_tree_new;
int afg_adjust_refinement(const afg_tree_desc* tree, const int* box_flags, int max_lvl,
                          afg_tree_new** out);
int afg_tree_new_sizes(const afg_tree_new* t, int* n_boxes, int* highest_lvl);
int afg_tree_new_get(const afg_tree_new* t, int* lvl, int* ix, int* parent, int* children,
                     int* neighbors, int* neighbor_mat, double* r_min, double* dr,
                     double* dr_base);
void afg_tree_new_free(afg_tree_new* t);

/* ---- accounting and timing (no counterpart in the reference, which keeps
 * wall-clock accumulators wc_time_* in src/m_streamer.f90:184-190) -------- */

/* out[0] kernel launches, out[1] smoother cell-updates (one GS relaxation of
 * one cell), out[2] transport cell-updates (leaf cells x species x stages),
 * out[3] V-cycles performed. */
int afg_counters(const afg_ctx* ctx, long long* out);

/* Record CUDA event `slot` (0..63) on the context's stream; elapsed time in
 * ms between two recorded events (synchronises on the second). */
int afg_event_record(afg_ctx* ctx, int slot);
int afg_event_elapsed(afg_ctx* ctx, int slot_a, int slot_b, float* ms);

/* Write `bytes` of scratch memory on the stream (evicts the L2 cache
 * between timed steps). */
int afg_flush_l2(afg_ctx* ctx, long long bytes);

/* Per-launch timing of one kernel class (AFG_KT_*): when enabled, each launch
 * of that class is bracketed by events; afg_kernel_stats returns the number
 * of launches, their summed device time (ms) and their summed algorithmic
 * bytes (interior cells only), then resets. */
#define AFG_KT_NONE     0
#define AFG_KT_GSRB     1  /* red-black half sweep                  */
#define AFG_KT_GHOST    2  /* ghost-cell fill                       */
#define AFG_KT_FLUX     3  /* Koren flux                            */
#define AFG_KT_UPDATE   4  /* density + source update               */
#define AFG_KT_RESIDUAL 5  /* residual (FP64 V-cycle)               */
#define AFG_KT_DEFECT   6  /* FP64 defect of the mixed solves       */
#define AFG_KT_RESTRICT 7  /* restriction, FAS right-hand side      */
#define AFG_KT_CORRECT  8  /* prolongation of corrections, phi += e */
#define AFG_KT_COARSE   9  /* coarse-grid solve                     */
#define AFG_KT_FIELD   10  /* field rhs, E from phi, photo source   */
#define AFG_KT_COPY    11  /* whole-variable copies, maxima         */
#define AFG_KT_NCLASS  12
#define AFG_KT_ALL     15  /* every class at once (afg_kernel_stats_all) */
int afg_kernel_timing(afg_ctx* ctx, int kernel_class);
int afg_kernel_stats(afg_ctx* ctx, long long* launches, double* ms, double* bytes);
/* With AFG_KT_ALL: per class c < AFG_KT_NCLASS the launches, device time
 * (ms) and algorithmic bytes recorded since afg_kernel_timing, then resets.
 * No counterpart in the reference. */
int afg_kernel_stats_all(afg_ctx* ctx, long long* launches, double* ms, double* bytes);

/* ---- reduction without device allocation -------------------------------
 * No counterpart in the reference.  For callers that may not call
 * cudaMalloc (they own their device arrays through their own allocator or
 * pool, or run under a fixed device-memory budget) and so cannot create a
 * context: max |v| over the interior cells of the boxes d_slots[0..n_slots-1]
 * (0-based box slots, in device memory) of a caller-owned device pool laid
 * out like one variable of this library's pools, d_pool[slot][(n_cell+2)^ndim]
 * (the same reduction as afg_maxabs; a NaN in the data is the result, as
 * there).  Nothing is allocated: the scratch is a file-scope device array of
 * AFG_NOALLOC_MAX_BOXES + 1 doubles (2 MiB) that every GPU loading this
 * library holds until the process exits; n_slots beyond
 * AFG_NOALLOC_MAX_BOXES returns AFG_ERR_ARG.  The first call on a device
 * looks up the array's device address with that device current.  Every call
 * copies the result into host memory and synchronises `stream`, so no call
 * may be made while any stream is being captured into a CUDA graph.  All
 * calls share the array, so calls that overlap on the GPU (other streams,
 * other threads) race; each call writes every entry it reads, so nothing
 * needs clearing.  A CUDA error left pending by earlier work is returned as
 * AFG_ERR_CUDA before anything is launched (and cleared, as
 * cudaGetLastError does).  Runs on `stream` (a cudaStream_t, NULL = default
 * stream); *result is a host double. */
#define AFG_NOALLOC_MAX_BOXES 262144
int afg_maxabs_noalloc(const double* d_pool, const int* d_slots, int n_slots,
                       int ndim, int n_cell, void* stream, double* result);

/* ---- electrode: internal Dirichlet boundary given by a level set --------
 * The electrode of the field solve (src/m_field.f90:255-390 with the shapes
 * of 672-904; afivo/src/m_af_multigrid.f90:954-1853): tree%mg_i_lsf,
 * mg%lsf, mg%lsf_dist => mg_lsf_dist_gss, mg%lsf_length_scale.
 * Coordinates are absolute (the reference's relative positions times the
 * domain length plus the origin). */
#define AFG_LSF_SPHERE         1   /* sphere_lsf: centre r0, radius          */
#define AFG_LSF_ROD            2   /* rod_lsf: segment r0-r1, radius         */
#define AFG_LSF_ROD_CONE_TOP   3   /* conical_rod_lsf                        */
#define AFG_LSF_ROD_ROD        4   /* rod_rod_lsf, rod_rod_get_potential     */
#define AFG_LSF_SPHERE_ROD     5   /* sphere_rod_lsf, sphere_rod_get_potential */
#define AFG_LSF_TWO_ROD_CONE   6   /* two_conical_rods_lsf / _get_potential  */
#define AFG_LSF_COAXIAL        7   /* coaxial_lsf, coaxial_get_potential     */

typedef struct afg_lsf_desc {
  int shape;                 /* AFG_LSF_*                                    */
  int i_lsf;                 /* 1-based cell variable receiving the level set */
  double r0[3], r1[3];       /* field_rod_r0 / field_rod_r1 (sphere: r0)      */
  double radius;             /* field_rod_radius                             */
  double r2_0[3], r2_1[3];   /* field_rod2_r0 / field_rod2_r1                */
  double radius2;            /* field_rod2_radius                            */
  double cone_tip_radius, cone_length_frac;    /* rod_cone_top, electrode 1  */
  double cone2_tip_radius, cone2_length_frac;  /* two_rod_cone_electrodes    */
  double center[3];          /* coaxial: the domain centre (axis position)   */
  int grounded, grounded2;   /* field_electrode_grounded / 2                 */
  double length_scale;       /* mg%lsf_length_scale (field_rod_radius)       */
  double gradient_safety_factor; /* mg%lsf_gradient_safety_factor (1.5)      */
  double tol;                /* mg%lsf_tol (1e-8)                            */
  double min_rel_distance;   /* mg%lsf_min_rel_distance (1e-4)               */
} afg_lsf_desc;

/* Electrode of an FP64 Poisson slot (helmholtz_lambda = 0), after
 * afg_mg_setup and again after every tree change: the level-set values of
 * every box (set_lsf_box, ghost cells included) into i_lsf, the boxes the
 * surface crosses (root mask, boundary distances by golden-section search
 * and bisection, mg_set_box_tag 1100-1145), their stencils
 * (mg_box_lsf_stencil 1779-1853), the coarse-grid matrix with those
 * stencils; boundary value 0 until afg_mg_set_lsf_voltage or
 * afg_field_compute (which passes its voltage).  AFG_ERR_ARG when no
 * level-1 box contains a boundary (check_coarse_representation_lsf
 * 2144-2161).  The electrode's custom prolongation
 * (mg%lsf_use_custom_prolongation, off by default) is not provided. */
int afg_mg_set_lsf(afg_ctx* ctx, int mg_id, const afg_lsf_desc* d);

/* current_voltage for the electrode boundary values: bc_correction =
 * f * boundary value (mg_set_operators_lvl 1169-1174). */
int afg_mg_set_lsf_voltage(afg_ctx* ctx, int mg_id, double voltage);

/* The electrode boxes of a slot: *n_boxes, and with non-NULL arrays their
 * ids (level order) and per box the stencil v[2*ndim+1][nc^ndim], the
 * boundary-value factor f, the rhs correction bcc and the distances
 * dd[2*ndim][nc^ndim] (cells i fastest). */
int afg_mg_lsf_info(afg_ctx* ctx, int mg_id, int* n_boxes, int* ids, double* v,
                    double* f, double* bcc, double* dd);

/* The electrode in the streamer's species update and initial state:
 * afg_transport_set_electrode(ctx, i_lsf) leaves the cells with level set
 * <= 0 out of afg_update_densities' flux and source terms (set_box_mask,
 * src/m_fluid.f90:469-515; a box without gas cells adds no chemistry time
 * step limit); i_lsf = 0 switches it off.  FP64 transport only. */
int afg_transport_set_electrode(afg_ctx* ctx, int i_lsf);

/* init_cond_set_box's electrode rule (src/m_init_cond.f90:284-288): every
 * cell (ghost cells included) of boxes ids[0..n-1] whose level set is <= 0
 * gets zero densities of all transport species (state 0). */
int afg_electrode_init_densities(afg_ctx* ctx, int mg_id, int n, const int* ids);

/* set_electrode_densities / electrode_species_bc (src/streamer.f90:
 * 590-656) on the electrode boxes of slot mg_id: cells with level set < 0
 * get zero densities (state 0); with neumann != 0 (bc_species =
 * af_bc_neumann_zero) a cell next to a gas cell gets the mean electron
 * density of its gas neighbours, and the ion (species index ion) the same. */
int afg_electrode_species_bc(afg_ctx* ctx, int mg_id, int electron, int ion, int neumann);

/* ---- output (afivo/src/m_af_output.f90) --------------------------------
 * The device-resident state written without a copy of the tree to the host:
 * the device gathers leaf cells, generates the mesh or interpolates, and
 * the host streams the result into the file in 64 MiB chunks.  Variables are
 * given as 1-based cell-centred indices ivs[0..n_iv-1] (at most 64) with
 * their names (tree%cc_names); the caller resolves cc_write_output
 * (get_output_vars, m_af_output.f90:1582-1597).  Ghost cells must be valid
 * where interpolation reads them, as in the reference. */

/* af_write_vtk (m_af_output.f90:556-752, m_vtk.f90): filename + ".vtu", a
 * VTK XML unstructured grid of all leaf cells, level by level in
 * tree%lvls(:)%leaves order: FieldData TIME (Float64) and CYCLE (Int32),
 * Float32 node coordinates (3 components, z = 0 in 2D), Int32 connectivity,
 * offsets and types (8 pixel / 11 voxel), one Float64 cell array per
 * variable, appended raw with 4-byte size headers (8-byte headers and
 * version 1.0 if an array exceeds 4 GiB).  The add_vars callback of the
 * reference has no counterpart: compute extra variables into spare
 * cell-centred variables first. */
int afg_write_vtk(afg_ctx* ctx, const char* filename, int n_cycle, double time,
                  int n_iv, const int* ivs, const char* const* names);

/* The cell data of variable iv on all leaves (the order and layout of the
 * CellData arrays of afg_write_vtk) into out[n_cells]; out = NULL returns
 * only *n_cells. */
int afg_leaf_cells(afg_ctx* ctx, int iv, double* out, long long* n_cells);

/* af_interp1 (m_af_interp.f90:43-105) at n_points points r[p][ndim]
 * (host arrays): the finest box containing the point (af_get_id_at without
 * a guess, m_af_utils.f90:266-313), multilinear interpolation between the
 * surrounding cell centres including ghost cells.  vals[p][v]; success[p]
 * (may be NULL) is 0 for a point outside the tree, whose values are 0. */
int afg_interp1(afg_ctx* ctx, long long n_points, const double* r, int n_iv,
                const int* ivs, double* vals, int* success);

/* af_write_line (m_af_output.f90:407-463): n_points points from r_min to
 * r_max (inclusive) into filename + ".txt": a "# x y[ z] names" header and
 * one row of coordinates and values per point.  A point outside the tree is
 * an error (AFG_ERR_ARG, no file), as the reference's error stop. */
int afg_write_line(afg_ctx* ctx, const char* filename, int n_iv, const int* ivs,
                   const char* const* names, const double* r_min,
                   const double* r_max, int n_points);

/* af_write_plane (m_af_output.f90:465-552): n_pixels[0] x n_pixels[1]
 * points spanning r_min..r_max (3D: the plane of the two coordinates that
 * differ most; the first of the smallest |r_max - r_min| is dropped) into
 * filename + ".vtk", legacy ASCII STRUCTURED_POINTS with the reference's
 * E20.8 number format. */
int afg_write_plane(afg_ctx* ctx, const char* filename, int n_iv, const int* ivs,
                    const char* const* names, const double* r_min,
                    const double* r_max, const int* n_pixels);

/* af_write_numpy (m_af_output.f90:756-901): the cell centres of a uniform
 * grid over r_min..r_max (NULL: the domain) with n_points[ndim] cells (NULL:
 * the spacing of the lowest level with a leaf in the region), interpolated.
 * filename ending in ".npy": one Fortran-ordered float64 array
 * (nx, ny[, nz], n_iv); ".npz": an uncompressed archive of one array per
 * variable under its name plus nx, r_min, r_max, dr, coord_t and
 * time_cycle. */
int afg_write_numpy(afg_ctx* ctx, const char* filename, const double* r_min,
                    const double* r_max, const int* n_points, int n_cycle,
                    double time, int n_iv, const int* ivs,
                    const char* const* names);

/* Synchronise the context's stream and check the device error word. */
int afg_sync(afg_ctx* ctx);

/* Kernel launches issued by this context since creation (for accounting). */
long long afg_launch_count(const afg_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* AFIVO_GPU_H */
