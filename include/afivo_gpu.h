/*
 * afivo_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of the
 * afivo-streamer per-timestep hot path.
 *
 * The reference is Fortran 2008 (MD-CWI/afivo-streamer).  Its callers stay as
 * they are; the bodies of the public afivo routines gain a branch that calls
 * these functions through ISO_C_BINDING (bindings in INTEGRATION.md).  Every
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

/* Copy cell-centred variable iv between host boxes and the device pool.
 * box_cc[id-1] points at box%cc(0,0[,0],1) of box id (NULL = skip); the data
 * of variable iv starts elem_offset doubles after it ((iv-1)*(nc+2)^ndim for
 * a Fortran box).  Ghost cells are copied too. */
int afg_cc_upload(afg_ctx* ctx, int iv, const double* const* box_cc,
                  long long elem_offset);
int afg_cc_download(afg_ctx* ctx, int iv, double* const* box_cc,
                    long long elem_offset);

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

/* mg_fas_vcycle (185-264).  max_lvl <= 0 means tree%highest_lvl.  When
 * set_residual != 0 the residual is stored in i_tmp and, if max_res is not
 * NULL, max over leaves of |residual| is returned in it. */
int afg_mg_vcycle(afg_ctx* ctx, int mg_id, int set_residual, int max_lvl,
                  double* max_res);

/* mg_fas_fmg (137-180). */
int afg_mg_fmg(afg_ctx* ctx, int mg_id, int set_residual, int have_guess,
               double* max_res);

/* Run V-cycles until max|residual| over leaves < threshold or max_cycles is
 * reached (the loop of field_compute, src/m_field.f90:520-524).  With
 * precision AFG_MIXED each cycle is an FP64 residual + FP32 V-cycle on the
 * correction + FP64 update (defect correction).  n_done and the final
 * residual are returned; residuals[] (may be NULL) receives the history. */
int afg_mg_solve(afg_ctx* ctx, int mg_id, double threshold, int max_cycles,
                 int* n_done, double* residuals);

/* Single stages, for parity testing of each kernel against the oracle:
 * gsrb_boxes (648-687), update_coarse (691-738), correct_children (624-646)
 * on the parents of level lvl-1 followed by af_gc_lvl(lvl), and the coarse
 * solve solve_coarse_grid (266-291). */
int afg_mg_gsrb_lvl(afg_ctx* ctx, int mg_id, int lvl, int cycle_type);
int afg_mg_update_coarse(afg_ctx* ctx, int mg_id, int lvl);
int afg_mg_correct_lvl(afg_ctx* ctx, int mg_id, int lvl);
int afg_mg_coarse_solve(afg_ctx* ctx, int mg_id);
/* residual_box (801-810) on all boxes of levels 1..max_lvl into i_tmp. */
int afg_mg_residual(afg_ctx* ctx, int mg_id, int max_lvl);

/* Synchronise the context's stream and check the device error word. */
int afg_sync(afg_ctx* ctx);

/* Kernel launches issued by this context since creation (for accounting). */
long long afg_launch_count(const afg_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* AFIVO_GPU_H */
