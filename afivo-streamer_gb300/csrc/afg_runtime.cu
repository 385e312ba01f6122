// afg_runtime.cu -- C-ABI implementation (include/afivo_gpu.h): device
// mirror of the afivo tree, variable pools, and the multigrid drivers
// (mg_fas_vcycle / mg_fas_fmg of afivo/src/m_af_multigrid.f90:137-264 and
// the V-cycle loop of field_compute, src/m_field.f90:520-524) as sequences
// of box-list kernels on one CUDA stream.
//
// There is no CPU fallback: every entry point either launches its kernels or
// returns an error code.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/afivo_gpu.h"
#include "afg_common.cuh"
#include "afg_lsf.h"
#include "afg_gc_kernels.cuh"
#include "afg_mg_kernels.cuh"
#include "afg_mg32.cuh"
#include "afg_transport.cuh"

using namespace afg;

namespace {

constexpr int kMaxMg = 16;
constexpr int kMaxCoarse = 4096;
constexpr int kModeSlot = 8, kMaxSlots = kMaxSlotsDev;  // device maxima slots (per instance)
constexpr int kMaxBranch = 8;                      // side streams

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Electrode (level-set) data of a multigrid slot (afg_lsf.cuh): per box
// crossed by the electrode surface the stencil, boundary-value factor,
// boundary values, rhs correction and distances; lists per level.
struct LsfState {
  afg_lsf::Electrode e{};
  int i_lsf = 0;
  double voltage = 0.0;
  int SI = 0;
  int n = 0;                  // electrode boxes
  std::vector<int> h_slots;   // [n]
  int* d_idx = nullptr;       // [n_boxes] electrode index or -1
  int* d_slots = nullptr;     // [n]
  double* d_v = nullptr;      // [n][2D+1][SI]
  double* d_f = nullptr;      // [n][SI]
  double* d_bcc = nullptr;    // [n][SI]
  double* d_bv = nullptr;     // [n][SI]
  double* d_dd = nullptr;     // [n][2D][SI]
  std::vector<double> h_v1;   // stencils of the level-1 electrode boxes (coarse matrix)
  std::vector<int> h_q1;      // their electrode indices
  std::vector<std::vector<int>> lvl_all, lvl_par, lvl_leaf;  // per level, slots
  int* d_lists = nullptr;
  std::vector<size_t> off_all, off_par, off_leaf;
  int n_cb = 0;               // level-1 electrode cells: coarse unknown, flat cell index
  int* d_cb_g = nullptr;
  int* d_cb_k = nullptr;
  ~LsfState() {
    for (void* p : {(void*)d_idx, (void*)d_slots, (void*)d_v, (void*)d_f, (void*)d_bcc, (void*)d_bv, (void*)d_dd,
                    (void*)d_lists, (void*)d_cb_g, (void*)d_cb_k})
      if (p) cudaFree(p);
  }
};

struct MgSlot {
  bool used = false;
  LsfState* lsf = nullptr;  // electrode of the field solve (afg_mg_set_lsf)
  afg_mg_desc d{};
  int n_coarse = 0;
  double* d_ainv = nullptr;
  double* d_b = nullptr;
  double* d_x = nullptr;
  double* d_b2r = nullptr;       // [n][2D]
  unsigned char* d_bmask = nullptr;
  // boundary values per instance row (one row for a single tree), then a
  // row of zeros (homogeneous): [(rows + 1)][6]
  double* d_bcval = nullptr;
  // coefficient tables (MgCoef): per box, and per radial index if cylindrical
  double* d_cb64 = nullptr;
  float* d_cb32 = nullptr;
  double* d_cy64 = nullptr;
  float* d_cy32 = nullptr;
  // FP32 inner-solver pools for AFG_MIXED (e, r, tmp)
  float* e32 = nullptr;
  float* r32 = nullptr;
  float* t32 = nullptr;
};

}  // namespace

struct afg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;
  // tree
  bool have_tree = false;
  int D = 2, nc = 16, n2 = 18, S = 324, NF = 289, coord = AFG_XYZ, n_boxes = 0, highest_lvl = 0;
  int cgs[3] = {1, 1, 1};
  std::vector<int> h_ix;      // [n][D]
  std::vector<int> h_nbr;     // [n][2D] raw Fortran ids
  std::vector<int> h_parent;  // [n] parent slot or -1
  std::vector<std::vector<int>> lvl_ids, lvl_leaves, lvl_parents;  // 0-based slots
  // device tables
  int *d_parent = nullptr, *d_children = nullptr, *d_nbr = nullptr, *d_pnb = nullptr, *d_nbmat = nullptr,
      *d_ix = nullptr;
  double *d_rmin = nullptr, *d_dr = nullptr, *d_idr = nullptr;
  float* d_idrf = nullptr;
  double* d_geo = nullptr;  // cylindrical geometry table (KTree::geo)
  int* d_lists = nullptr;  // all level lists concatenated
  int* d_rec = nullptr;    // per list entry: {slot, neighbour slots per face, pad} (8 ints)
  std::vector<size_t> off_ids, off_leaves, off_parents;  // per level offsets into d_lists
  // per level: boxes whose face ghosts a refinement-boundary rule of a finer
  // box reads (parents' neighbours across refinement faces), and offsets
  std::vector<std::vector<int>> lvl_rbsrc;
  std::vector<size_t> off_rbsrc;
  // per level: parents and refinement sources (the boxes whose ghost cells a
  // correction V-cycle reads after the level's up smoothing), and offsets
  std::vector<std::vector<int>> lvl_gcneed;
  std::vector<size_t> off_gcneed;
  size_t off_all = 0;       // list of all boxes, all levels (level order)
  size_t off_all_leaves = 0;
  int n_all = 0;            // boxes in all level lists
  int n_all_leaves = 0;
  unsigned char* d_is_leaf = nullptr;
  int* d_cslot = nullptr;   // coarse unknown -> slot (instance-major on batched trees)
  int* d_ccell = nullptr;   // coarse unknown -> cell index
  int* d_ccell_rb = nullptr;  // the same in the compact FP32 layout (interior block)
  // Batched independent instances (afg_tree_sync_batched); n_inst = 0 for a
  // single tree.  The coarse grids of all instances are alike (nloc
  // unknowns each) and share one inverse.
  int n_inst = 0;
  std::vector<int> h_inst;              // [n_boxes] instance of each slot
  std::vector<int> inst_hl;             // highest level per instance
  std::vector<double> inst_min_dr;      // finest dr per instance
  std::vector<std::vector<long long>> inst_cells;  // [instance][level] cells
  int* d_inst = nullptr;
  int* d_frozen = nullptr;       // flags the kernels read
  int* d_frozen_base = nullptr;  // instances whose solve has converged
  int* d_inst_hl = nullptr;
  int* h_frozen = nullptr;       // pinned staging of the flags
  int max_rows = 1;              // instance rows of d_max / h_max
  // pools
  int n_var = 0, n_var_face = 0;
  std::vector<double*> cc;  // [n_var]
  std::vector<double*> fc;  // [n_var_face]
  std::vector<GcDev> methods;
  std::vector<bool> has_method;
  // scratch
  // device maxima (bits of non-negative doubles): slots 0..7 by role, slots
  // kModeSlot + n per Helmholtz mode n
  unsigned long long* d_max = nullptr;
  unsigned long long* h_max = nullptr;  // pinned
  // error word raised by kernels whose bounded waits timed out, checked
  // whenever maxima are read back (pinned copy in h_err)
  unsigned* d_err = nullptr;
  unsigned* h_err = nullptr;
  // set when a kernel reported (error word bit 2) that it returned with
  // copies into its shared memory still outstanding after its bounded drain:
  // the context then refuses every further multigrid and transport call
  bool poisoned = false;
  int n_sm = 0;
  // side streams and events for independent branches (photoionization modes)
  cudaStream_t side[kMaxBranch] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kMaxBranch] = {};
  // smoother work shape (cells of a colour per thread) for the specialized
  // box sizes: [0] FP32, [1] FP64; picked by the autotuner, 0 = default
  int gsrb_cpt[3] = {0, 0, 0};  // [2]: FP32 on the compact layout
  // FP32 correction buffers of the mixed solves in the compact red-black
  // layout (afg_mg32.cuh); false: the ghosted (nc+2)^D layout
  bool rb32 = true;
  // lockstep problems (Helmholtz modes as multiple right-hand sides): while
  // ky > 1 every multigrid launch covers the slots grp[0..ky-1], blockIdx.y
  // selecting the slot; ky = 1 otherwise
  int ky = 1;
  MgSlot* grp[kMaxModes] = {};
  bool photoi_lockstep = true;  // Helmholtz modes in lockstep (else parallel branches)
  bool flux_staged = true;      // FP32 fluxes by k_flux32s where it applies (else k_flux32)
  // asynchronous downloads (afg_cc_download_async)
  cudaStream_t xfer_stream = nullptr;
  cudaEvent_t ev_xfer = nullptr;
  double* h_stage = nullptr;            // pinned staging
  size_t stage_elems = 0;
  MgSlot mg[kMaxMg];
  // transport state (afg_transport.cuh)
  TransportState tr;
  // integrator-stage settings (afg_stage_setup); stage.mg_id < 0 = unset
  afg_stage_desc stage{-1, 0.0, 0.0, 0, 0.0, 0.0};
  // accounting and timing
  long long ctr[4] = {0, 0, 0, 0};
  cudaEvent_t ev[64] = {};
  cudaEvent_t xfer_ev[2] = {};  // download pipeline
  std::vector<std::pair<uintptr_t, size_t>> host_regs;  // ranges page-locked by afg_host_register
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  int kt_class = 0;
  std::vector<cudaEvent_t> kt_ev;  // start/stop pairs
  size_t kt_used = 0;
  double kt_bytes = 0;
  std::vector<int> kt_cls;         // class of each recorded pair
  std::vector<double> kt_pbytes;   // algorithmic bytes of each recorded pair
  // CUDA graphs of fixed launch sequences (V-cycle iterations, transport
  // stages), keyed by what determines the sequence; cleared whenever the
  // tree, an operator or boundary values change
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0, ctr[4] = {0, 0, 0, 0};
  };
  std::map<std::string, Graph> graphs;
  bool use_graphs = true;
  bool fused_gsrb = true;
  // electrode boxes of the multigrid slot whose kernels are being launched
  // (KTree::lsf), set by LsfScope
  const int* cur_lsf = nullptr;
  bool capturing = false;
};

/* ------------------------------------------------------------------------- */
static int fail(afg_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(ctx, AFG_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                     \
  } while (0)

#define CKL()                                                                               \
  do {                                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                    \
    if (e_ != cudaSuccess)                                                                  \
      return fail(ctx, AFG_ERR_CUDA, "kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                      \
  } while (0)

#define RC(x)                 \
  do {                        \
    int rc_ = (x);            \
    if (rc_ != AFG_OK) return rc_; \
  } while (0)

template <typename T>
static cudaError_t dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc((void**)p, n * sizeof(T));
}

template <typename T>
static void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

static KTree ktree(const afg_ctx* c) {
  KTree t;
  t.D = c->D;
  t.nc = c->nc;
  t.n2 = c->n2;
  t.S = c->S;
  t.NF = c->NF;
  t.SI = c->D == 2 ? c->nc * c->nc : c->nc * c->nc * c->nc;
  t.nbox = c->n_boxes;
  t.parent = c->d_parent;
  t.children = c->d_children;
  t.nbr = c->d_nbr;
  t.pnb = c->d_pnb;
  t.nbmat = c->d_nbmat;
  t.ix = c->d_ix;
  t.r_min = c->d_rmin;
  t.dr = c->d_dr;
  t.geo = c->d_geo;
  t.idr = c->d_idr;
  t.idrf = c->d_idrf;
  t.inst = c->n_inst > 0 ? c->d_inst : nullptr;
  t.frozen = c->n_inst > 0 ? c->d_frozen : nullptr;
  t.lsf = c->cur_lsf;
  return t;
}

// the electrode boxes of slot m are skipped by the ordinary kernels launched
// while this scope lives
struct LsfScope {
  afg_ctx* c;
  const int* prev;
  LsfScope(afg_ctx* c_, const MgSlot& m) : c(c_), prev(c_->cur_lsf) { c->cur_lsf = m.lsf ? m.lsf->d_idx : nullptr; }
  ~LsfScope() { c->cur_lsf = prev; }
};

// instance rows of the per-instance tables (1 for a single tree)
static int inst_rows(const afg_ctx* c) { return c->n_inst > 0 ? c->n_inst : 1; }

template <typename T>
static MgCoef<T> coef_of(const MgSlot& m);
template <>
MgCoef<double> coef_of<double>(const MgSlot& m) {
  return MgCoef<double>{m.d_cb64, m.d_cy64};
}
template <>
MgCoef<float> coef_of<float>(const MgSlot& m) {
  return MgCoef<float>{m.d_cb32, m.d_cy32};
}
static MgCoef<double> coef64(const MgSlot& m) { return coef_of<double>(m); }

static const int* lst(const afg_ctx* c, size_t off) { return c->d_lists + off; }
// the box records of the entries of a list (a pointer into d_lists)
static const int* rec_of(const afg_ctx* c, const int* list) { return c->d_rec + (list - c->d_lists) * 8; }

// Per-launch timing of one kernel class (afg_kernel_timing): events around
// each launch of the selected class, algorithmic bytes summed on the host.
static bool kt_on(const afg_ctx* c, int cls) {
  return cls != AFG_KT_NONE && (c->kt_class == cls || c->kt_class == AFG_KT_ALL);
}
static void kt_begin(afg_ctx* c, int cls) {
  if (!kt_on(c, cls)) return;
  if (c->kt_used + 2 > c->kt_ev.size()) {
    if (c->kt_ev.size() >= 40000) return;
    const size_t old = c->kt_ev.size();
    c->kt_ev.resize(old + 2048);
    for (size_t q = old; q < c->kt_ev.size(); q++) cudaEventCreate(&c->kt_ev[q]);
  }
  cudaEventRecord(c->kt_ev[c->kt_used], c->stream);
}
static void kt_end(afg_ctx* c, int cls, double bytes) {
  if (!kt_on(c, cls)) return;
  if (c->kt_used + 2 > c->kt_ev.size()) return;
  cudaEventRecord(c->kt_ev[c->kt_used + 1], c->stream);
  c->kt_used += 2;
  c->kt_bytes += bytes;
  c->kt_cls.push_back(cls);
  c->kt_pbytes.push_back(bytes);
}
// events around the launches of one helper (a leaf: helpers with a scope do
// not call each other)
struct KtScope {
  afg_ctx* c;
  int cls;
  double bytes;
  KtScope(afg_ctx* c_, int cls_, double bytes_) : c(c_), cls(cls_), bytes(bytes_) { kt_begin(c, cls); }
  ~KtScope() { kt_end(c, cls, bytes); }
};
static double box_cells(const afg_ctx* c) { return c->D == 2 ? (double)c->nc * c->nc : (double)c->nc * c->nc * c->nc; }

static void clear_graphs(afg_ctx* c) {
  for (auto& kv : c->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  c->graphs.clear();
}

static void free_tree(afg_ctx* c) {
  clear_graphs(c);
  dfree(c->d_parent); dfree(c->d_children); dfree(c->d_nbr); dfree(c->d_pnb); dfree(c->d_nbmat);
  dfree(c->d_ix); dfree(c->d_rmin); dfree(c->d_dr); dfree(c->d_idr); dfree(c->d_idrf); dfree(c->d_lists); dfree(c->d_rec); dfree(c->d_is_leaf); dfree(c->d_geo);
  dfree(c->d_cslot); dfree(c->d_ccell); dfree(c->d_ccell_rb);
  dfree(c->d_inst); dfree(c->d_frozen); dfree(c->d_frozen_base); dfree(c->d_inst_hl);
  if (c->h_frozen) cudaFreeHost(c->h_frozen);
  c->h_frozen = nullptr;
  c->n_inst = 0;
  c->h_inst.clear();
  c->inst_hl.clear();
  c->inst_min_dr.clear();
  c->inst_cells.clear();
  for (auto& p : c->cc) dfree(p);
  for (auto& p : c->fc) dfree(p);
  c->cc.clear();
  c->fc.clear();
  for (auto& m : c->mg) {
    dfree(m.d_ainv); dfree(m.d_b); dfree(m.d_x); dfree(m.d_b2r); dfree(m.d_bmask); dfree(m.d_bcval);
    dfree(m.e32); dfree(m.r32); dfree(m.t32);
    dfree(m.d_cb64); dfree(m.d_cb32); dfree(m.d_cy64); dfree(m.d_cy32);
    delete m.lsf;
    m.lsf = nullptr;
    m.used = false;
  }
  transport_free(c->tr);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  c->h_stage = nullptr;
  c->stage_elems = 0;
  c->have_tree = false;
}

/* ------------------------------------------------------------------------- */
// Generic launchers dispatching on (D, cylindrical, T)

// the FP32 buffers of the mixed solves in the compact layout (afg_mg32.cuh)
template <typename T>
static bool rb_of(const afg_ctx* ctx) {
  return std::is_same<T, float>::value && ctx->rb32;
}

template <typename T>
static int launch_gc(afg_ctx* ctx, const int* list, int n, ModeArg<T> v, const GcDev& g, int corners) {
  if (n <= 0) return AFG_OK;
  KTree t = ktree(ctx);
  kt_begin(ctx, AFG_KT_GHOST);
  // four boxes per CTA (kGcLanes threads each)
  const int nb4 = (n + 3) / 4;
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      if (ctx->D == 2)
        AFG_NC2(NCV_, k_gc_rb<2, NCV_><<<dim3(nb4, ctx->ky), 4 * kGcLanes<2>, 0, ctx->stream>>>(t, rec_of(ctx, list), n,
                                                                                                v, g, corners));
      else
        AFG_NC3(NCV_, k_gc_rb<3, NCV_><<<dim3(nb4, ctx->ky), 4 * kGcLanes<3>, 0, ctx->stream>>>(t, rec_of(ctx, list), n,
                                                                                                v, g, corners));
      kt_end(ctx, AFG_KT_GHOST, 2.0 * sizeof(T) * n * ctx->ky * 2 * ctx->D * (box_cells(ctx) / ctx->nc));
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  if (ctx->D == 2)
    AFG_NC2(NCV_, k_gc<2, T, NCV_><<<dim3(nb4, ctx->ky), 4 * kGcLanes<2>, 0, ctx->stream>>>(t, rec_of(ctx, list), n, v,
                                                                                           g, corners));
  else
    AFG_NC3(NCV_, k_gc<3, T, NCV_><<<dim3(nb4, ctx->ky), 4 * kGcLanes<3>, 0, ctx->stream>>>(t, rec_of(ctx, list), n, v,
                                                                                           g, corners));
  kt_end(ctx, AFG_KT_GHOST, 2.0 * sizeof(T) * n * ctx->ky * 2 * ctx->D * (box_cells(ctx) / ctx->nc));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_gsrb(afg_ctx* ctx, const int* list, int n, T* phi, const T* rhs, int rb, MgCoef<T> lam) {
  if (n <= 0) return AFG_OK;
  if (rb_of<T>(ctx)) return fail(ctx, AFG_ERR_STATE, "the unfused smoother needs the ghosted FP32 layout");
  KTree t = ktree(ctx);
  const int threads = ctx->D == 2 ? std::min(256, ctx->nc * ctx->nc / 2) : std::min(256, ctx->nc * ctx->nc * ctx->nc / 2);
  kt_begin(ctx, AFG_KT_GSRB);
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_gsrb<3, false, T, NCV_><<<n, threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_gsrb<2, true, T, NCV_><<<n, threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam));
  else
    AFG_NC2(NCV_, k_gsrb<2, false, T, NCV_><<<n, threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam));
  // half sweep: 1.5 words per cell (read phi and rhs, write phi over two half sweeps)
  kt_end(ctx, AFG_KT_GSRB, 1.5 * sizeof(T) * n * box_cells(ctx));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

static bool gsrb_rec_specialized(const afg_ctx* ctx) {
  return (ctx->D == 3 && ctx->nc == 8) || (ctx->D == 2 && ctx->nc == 16);
}
template <typename T>
static int gsrb_cpt_of(const afg_ctx* ctx) {
  const int c = ctx->gsrb_cpt[sizeof(T) == 8 ? 1 : 0];
  return c > 0 ? c : (ctx->D == 3 ? 4 : 2);
}

// Persistent grid of the shared-memory-staged smoother: as many CTAs as fit
// on the GPU at once (occupancy of the instantiation with its shared memory)
template <int D, bool CYL, typename T, int NC, int CPT, bool SR>
static int launch_gsrb_tma(afg_ctx* ctx, const int* rec, int n, ModeArg<T> phi, ModeArg<const T> rhs, int rb,
                           ModeCoef<T> lam, const GcDev& g) {
  constexpr int TPB = (D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT;
  constexpr int S = D == 2 ? (NC + 2) * (NC + 2) : (NC + 2) * (NC + 2) * (NC + 2);
  constexpr size_t smem = (SR ? 4 : 2) * S * sizeof(T);
  static int per_sm = 0;
  if (per_sm == 0) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gsrb_tma<D, CYL, T, NC, CPT, SR>, TPB, smem));
    per_sm = std::max(1, per_sm);
  }
  const int grid = std::min(n, std::max(1, per_sm * ctx->n_sm / ctx->ky));
  k_gsrb_tma<D, CYL, T, NC, CPT, SR><<<dim3(grid, ctx->ky), TPB, smem, ctx->stream>>>(ktree(ctx), rec, n, phi, rhs,
                                                                                      rb, lam, g, ctx->d_err);
  return AFG_OK;
}

template <int D, bool CYL, typename T, int NC, int CPT>
static int launch_gsrb_tma(afg_ctx* ctx, bool sr, const int* rec, int n, ModeArg<T> phi, ModeArg<const T> rhs,
                           int rb, ModeCoef<T> lam, const GcDev& g) {
  return sr ? launch_gsrb_tma<D, CYL, T, NC, CPT, true>(ctx, rec, n, phi, rhs, rb, lam, g)
            : launch_gsrb_tma<D, CYL, T, NC, CPT, false>(ctx, rec, n, phi, rhs, rb, lam, g);
}

// record-driven half sweep with `cpt` cells of the colour per thread
// (3D 8^3: 1, 2, 4, 8; 2D 16^2: 1, 2, 4); cpt | kGsrbTma selects the
// shared-memory-staged persistent variant (3D: 2, 4; 2D: 1, 2), with
// | kGsrbTmaRhs the right-hand side staged too
constexpr int kGsrbTma = 16, kGsrbTmaRhs = 32;
template <typename T>
static int launch_gsrb_rec(afg_ctx* ctx, const int* rec, int n, ModeArg<T> phi, ModeArg<const T> rhs, int rb,
                           ModeCoef<T> lam, const GcDev& g, int cpt) {
  KTree t = ktree(ctx);
  if (cpt & kGsrbTma) {
    const int c = cpt & (kGsrbTma - 1);
    const bool sr = (cpt & kGsrbTmaRhs) != 0;
    int rc;
    if (ctx->D == 3)
      rc = c == 2 ? launch_gsrb_tma<3, false, T, 8, 2>(ctx, sr, rec, n, phi, rhs, rb, lam, g)
                  : launch_gsrb_tma<3, false, T, 8, 4>(ctx, sr, rec, n, phi, rhs, rb, lam, g);
    else if (ctx->coord == AFG_CYL)
      rc = c == 1 ? launch_gsrb_tma<2, true, T, 16, 1>(ctx, sr, rec, n, phi, rhs, rb, lam, g)
                  : launch_gsrb_tma<2, true, T, 16, 2>(ctx, sr, rec, n, phi, rhs, rb, lam, g);
    else
      rc = c == 1 ? launch_gsrb_tma<2, false, T, 16, 1>(ctx, sr, rec, n, phi, rhs, rb, lam, g)
                  : launch_gsrb_tma<2, false, T, 16, 2>(ctx, sr, rec, n, phi, rhs, rb, lam, g);
    if (rc != AFG_OK) return rc;
    CKL();
    return AFG_OK;
  }
  if (ctx->D == 3) {
    switch (cpt) {
      case 1: k_gsrb_rec<3, false, T, 8, 1><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      case 2: k_gsrb_rec<3, false, T, 8, 2><<<dim3(n, ctx->ky), 128, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      case 8: k_gsrb_rec<3, false, T, 8, 8><<<dim3(n, ctx->ky), 32, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      default: k_gsrb_rec<3, false, T, 8, 4><<<dim3(n, ctx->ky), 64, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
    }
  } else if (ctx->coord == AFG_CYL) {
    switch (cpt) {
      case 1: k_gsrb_rec<2, true, T, 16, 1><<<dim3(n, ctx->ky), 128, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      case 4: k_gsrb_rec<2, true, T, 16, 4><<<dim3(n, ctx->ky), 32, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      default: k_gsrb_rec<2, true, T, 16, 2><<<dim3(n, ctx->ky), 64, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
    }
  } else {
    switch (cpt) {
      case 1: k_gsrb_rec<2, false, T, 16, 1><<<dim3(n, ctx->ky), 128, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      case 4: k_gsrb_rec<2, false, T, 16, 4><<<dim3(n, ctx->ky), 32, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
      default: k_gsrb_rec<2, false, T, 16, 2><<<dim3(n, ctx->ky), 64, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g); break;
    }
  }
  CKL();
  return AFG_OK;
}

// Half sweep on the compact FP32 layout.  code: cpt | kGsrbTma selects the
// shared-memory-staged persistent kernel with cpt cells of the colour per
// thread (3D 8^3: 1, 2, 4; 2D 16^2: 1, 2, 4); anything else (and box sizes
// without a specialization) the one-box-per-CTA kernel.
template <int D, bool CYL, int NC, int CPT>
static int launch_gsrb_rb_tma(afg_ctx* ctx, const int* rec, int n, ModeArg<float> phi, ModeArg<const float> rhs,
                              int rb, ModeCoef<float> lam, const GcDev& g) {
  constexpr int TPB = (D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT;
  static int per_sm = 0;
  if (per_sm == 0) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gsrb_rb_tma<D, CYL, NC, CPT>, TPB, 0));
    per_sm = std::max(1, per_sm);
  }
  const int grid = std::min(n, std::max(1, per_sm * ctx->n_sm / ctx->ky));
  k_gsrb_rb_tma<D, CYL, NC, CPT><<<dim3(grid, ctx->ky), TPB, 0, ctx->stream>>>(ktree(ctx), rec, n, phi, rhs, rb, lam,
                                                                               g, ctx->d_err);
  return AFG_OK;
}

static int launch_gsrb_rb(afg_ctx* ctx, const int* rec, int n, ModeArg<float> phi, ModeArg<const float> rhs, int rb,
                          ModeCoef<float> lam, const GcDev& g, int code) {
  const KTree t = ktree(ctx);
  const int c = code & (kGsrbTma - 1);
  if ((code & kGsrbTma) && gsrb_rec_specialized(ctx) && (c == 1 || c == 2 || c == 4)) {
    int rc;
    if (ctx->D == 3) {
      if (c == 1) rc = launch_gsrb_rb_tma<3, false, 8, 1>(ctx, rec, n, phi, rhs, rb, lam, g);
      else if (c == 2) rc = launch_gsrb_rb_tma<3, false, 8, 2>(ctx, rec, n, phi, rhs, rb, lam, g);
      else rc = launch_gsrb_rb_tma<3, false, 8, 4>(ctx, rec, n, phi, rhs, rb, lam, g);
    } else if (ctx->coord == AFG_CYL) {
      if (c == 1) rc = launch_gsrb_rb_tma<2, true, 16, 1>(ctx, rec, n, phi, rhs, rb, lam, g);
      else if (c == 2) rc = launch_gsrb_rb_tma<2, true, 16, 2>(ctx, rec, n, phi, rhs, rb, lam, g);
      else rc = launch_gsrb_rb_tma<2, true, 16, 4>(ctx, rec, n, phi, rhs, rb, lam, g);
    } else {
      if (c == 1) rc = launch_gsrb_rb_tma<2, false, 16, 1>(ctx, rec, n, phi, rhs, rb, lam, g);
      else if (c == 2) rc = launch_gsrb_rb_tma<2, false, 16, 2>(ctx, rec, n, phi, rhs, rb, lam, g);
      else rc = launch_gsrb_rb_tma<2, false, 16, 4>(ctx, rec, n, phi, rhs, rb, lam, g);
    }
    RC(rc);
    CKL();
    return AFG_OK;
  }
  const int sh = (ctx->D == 2 ? ctx->nc * ctx->nc : ctx->nc * ctx->nc * ctx->nc) / 2;
  const int threads = std::max(32, std::min(256, sh));
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_gsrb_rb<3, false, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_gsrb_rb<2, true, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g));
  else
    AFG_NC2(NCV_, k_gsrb_rb<2, false, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec, phi, rhs, rb, lam, g));
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_gsrb_fused(afg_ctx* ctx, const int* list, int n, ModeArg<T> phi, ModeArg<const T> rhs, int rb,
                             ModeCoef<T> lam, const GcDev& g) {
  if (n <= 0) return AFG_OK;
  KTree t = ktree(ctx);
  const int threads = ctx->D == 2 ? std::min(256, ctx->nc * ctx->nc / 2) : std::min(256, ctx->nc * ctx->nc * ctx->nc / 2);
  kt_begin(ctx, AFG_KT_GSRB);
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      // untuned: the staged kernel with 2 cells per thread
      const int code = ctx->gsrb_cpt[2] == 0 ? (kGsrbTma | 2) : ctx->gsrb_cpt[2];
      RC(launch_gsrb_rb(ctx, rec_of(ctx, list), n, phi, rhs, rb, lam, g, code));
      kt_end(ctx, AFG_KT_GSRB, 1.5 * sizeof(T) * n * ctx->ky * box_cells(ctx));
      ctx->launches++;
      return AFG_OK;
    }
  }
  // the usual box sizes: several cells per thread (tuned), box records
  if (gsrb_rec_specialized(ctx) && ctx->cur_lsf == nullptr) {
    const int rc = launch_gsrb_rec<T>(ctx, rec_of(ctx, list), n, phi, rhs, rb, lam, g, gsrb_cpt_of<T>(ctx));
    if (rc != AFG_OK) return rc;
  } else if (ctx->D == 3)
    k_gsrb_fused<3, false, T, 0><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam, g);
  else if (ctx->coord == AFG_CYL)
    k_gsrb_fused<2, true, T, 0><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam, g);
  else
    k_gsrb_fused<2, false, T, 0><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, list, phi, rhs, rb, lam, g);
  // algorithmic bytes: 3 words per cell per full iteration (read phi and
  // rhs, write phi), 1.5 words per half sweep
  kt_end(ctx, AFG_KT_GSRB, 1.5 * sizeof(T) * n * ctx->ky * box_cells(ctx));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_residual(afg_ctx* ctx, const int* list, int n, const T* phi, const T* rhs, T* tmp, MgCoef<T> lam,
                           unsigned long long* maxbits) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_RESIDUAL, 3.0 * sizeof(T) * n * box_cells(ctx));
  if (rb_of<T>(ctx)) return fail(ctx, AFG_ERR_STATE, "no residual kernel on the compact FP32 layout");
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_residual<3, false, T, NCV_><<<n, 256, 0, ctx->stream>>>(t, list, phi, rhs, tmp, lam, ctx->d_is_leaf, maxbits));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_residual<2, true, T, NCV_><<<n, 256, 0, ctx->stream>>>(t, list, phi, rhs, tmp, lam, ctx->d_is_leaf, maxbits));
  else
    AFG_NC2(NCV_, k_residual<2, false, T, NCV_><<<n, 256, 0, ctx->stream>>>(t, list, phi, rhs, tmp, lam, ctx->d_is_leaf, maxbits));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_rrestrict(afg_ctx* ctx, const int* list, int n, ModeArg<T> phi, ModeArg<const T> rhs,
                            ModeArg<T> tmp, ModeCoef<T> lam, int store_child, const GcDev& g, int otf) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_RESTRICT, sizeof(T) * n * ctx->ky * box_cells(ctx) * (2.0 + 2.0 / (1 << ctx->D)));
  KTree t = ktree(ctx);
  const int hnc = ctx->nc / 2;
  const int threads = std::max(32, std::min(256, ctx->D == 2 ? hnc * hnc : hnc * hnc * hnc));
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      if (store_child || !otf) return fail(ctx, AFG_ERR_STATE, "compact FP32 restriction: face neighbours on the fly only");
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_residual_restrict_rb<3, false, NCV_><<<dim3(n, ctx->ky), threads, sizeof(float) * ctx->S, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      else if (ctx->coord == AFG_CYL)
        AFG_NC2(NCV_, k_residual_restrict_rb<2, true, NCV_><<<dim3(n, ctx->ky), threads, sizeof(float) * ctx->S, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      else
        AFG_NC2(NCV_, k_residual_restrict_rb<2, false, NCV_><<<dim3(n, ctx->ky), threads, sizeof(float) * ctx->S, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_residual_restrict<3, false, T, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, store_child, g, otf));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_residual_restrict<2, true, T, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, store_child, g, otf));
  else
    AFG_NC2(NCV_, k_residual_restrict<2, false, T, NCV_><<<dim3(n, ctx->ky), threads, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, store_child, g, otf));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_coarse_fas(afg_ctx* ctx, const int* list, int n, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp,
                             ModeCoef<T> lam, int copy_tmp, int fill, const GcDev& g) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_RESTRICT, 4.0 * sizeof(T) * n * ctx->ky * box_cells(ctx));
  KTree t = ktree(ctx);
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      if (!copy_tmp || !fill) return fail(ctx, AFG_ERR_STATE, "compact FP32 FAS update: fill and copy only");
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_coarse_fas_rb<3, false, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      else if (ctx->coord == AFG_CYL)
        AFG_NC2(NCV_, k_coarse_fas_rb<2, true, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      else
        AFG_NC2(NCV_, k_coarse_fas_rb<2, false, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, g));
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_coarse_fas<3, false, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, copy_tmp, fill, g));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_coarse_fas<2, true, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, copy_tmp, fill, g));
  else
    AFG_NC2(NCV_, k_coarse_fas<2, false, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, rec_of(ctx, list), phi, rhs, tmp, lam, copy_tmp, fill, g));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_correct(afg_ctx* ctx, const int* list, int n, ModeArg<T> phi, ModeArg<T> tmp) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_CORRECT, sizeof(T) * n * ctx->ky * box_cells(ctx) * (3.0 + 2.0 * (1 << ctx->D)));
  KTree t = ktree(ctx);
  const size_t sm = sizeof(T) * ctx->S;
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_correct_rb<3, NCV_><<<dim3(n, ctx->ky), 256, sm, ctx->stream>>>(t, list, phi, tmp));
      else
        AFG_NC2(NCV_, k_correct_rb<2, NCV_><<<dim3(n, ctx->ky), 256, sm, ctx->stream>>>(t, list, phi, tmp));
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_correct<3, T, NCV_><<<dim3(n, ctx->ky), 256, sm, ctx->stream>>>(t, list, phi, tmp));
  else
    AFG_NC2(NCV_, k_correct<2, T, NCV_><<<dim3(n, ctx->ky), 256, sm, ctx->stream>>>(t, list, phi, tmp));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_init_phi_rhs(afg_ctx* ctx, const int* list, int n, ModeArg<T> phi, ModeArg<T> rhs) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_RESTRICT, 2.0 * sizeof(T) * n * ctx->ky * box_cells(ctx));
  KTree t = ktree(ctx);
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_init_phi_rhs_rb<3, false, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
      else if (ctx->coord == AFG_CYL)
        AFG_NC2(NCV_, k_init_phi_rhs_rb<2, true, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
      else
        AFG_NC2(NCV_, k_init_phi_rhs_rb<2, false, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_init_phi_rhs<3, false, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_init_phi_rhs<2, true, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
  else
    AFG_NC2(NCV_, k_init_phi_rhs<2, false, T, NCV_><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(t, list, phi, rhs));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_copy(afg_ctx* ctx, const int* list, int n, ModeArg<const T> src, ModeArg<T> dst) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_COPY, 2.0 * sizeof(T) * n * ctx->ky * box_cells(ctx));
  if constexpr (std::is_same<T, float>::value) {
    if (ctx->rb32) {
      k_copy_rb<<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(ktree(ctx), list, src, dst);
      ctx->launches++;
      CKL();
      return AFG_OK;
    }
  }
  k_copy<T><<<dim3(n, ctx->ky), 256, 0, ctx->stream>>>(ktree(ctx), list, src, dst);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int launch_maxabs(afg_ctx* ctx, const int* list, int n, const T* v, unsigned long long* out) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_COPY, 1.0 * sizeof(T) * n * box_cells(ctx));
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    AFG_NC3(NCV_, k_maxabs<3, T, NCV_><<<n, 256, 0, ctx->stream>>>(t, list, v, out));
  else
    AFG_NC2(NCV_, k_maxabs<2, T, NCV_><<<n, 256, 0, ctx->stream>>>(t, list, v, out));
  ctx->launches++;
  CKL();
  return AFG_OK;
}


// Run a fixed launch sequence through a cached CUDA graph: captured on first
// use, replayed afterwards (one launch instead of hundreds).  The body must
// not synchronise.  Per-launch kernel timing bypasses the graphs.
template <typename F>
static int run_graph(afg_ctx* ctx, const std::string& key, F&& body) {
  if (!ctx->use_graphs || ctx->kt_class != AFG_KT_NONE || ctx->capturing) return body();
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    const long long l0 = ctx->launches;
    long long c0[4];
    for (int q = 0; q < 4; q++) c0[q] = ctx->ctr[q];
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    const int rc = body();
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
    if (rc != AFG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
    afg_ctx::Graph gr;
    const cudaError_t ei = cudaGraphInstantiate(&gr.exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ei));
    gr.launches = ctx->launches - l0;
    for (int q = 0; q < 4; q++) gr.ctr[q] = ctx->ctr[q] - c0[q];
    // the capture did not execute anything: undo the accounting, then replay
    ctx->launches = l0;
    for (int q = 0; q < 4; q++) ctx->ctr[q] = c0[q];
    it = ctx->graphs.emplace(key, gr).first;
  }
  CK(cudaGraphLaunch(it->second.exec, ctx->stream));
  ctx->launches += it->second.launches;
  for (int q = 0; q < 4; q++) ctx->ctr[q] += it->second.ctr[q];
  return AFG_OK;
}

static std::string gkey(const char* tag, int a = 0, int b = 0, int c = 0, int d = 0) {
  char buf[96];
  snprintf(buf, sizeof(buf), "%s:%d:%d:%d:%d", tag, a, b, c, d);
  return buf;
}

/* ------------------------------------------------------------------------- */
// Multigrid drivers (templated on the working precision T)

// Operator coefficients of slot m, or of every lockstep slot grp[0..ky-1]
// (grp[0] is m) for a launch covering them
template <typename T>
static ModeCoef<T> coefs(const afg_ctx* ctx, const MgSlot& m) {
  ModeCoef<T> c(coef_of<T>(m));
  for (int k = 1; k < ctx->ky; k++) {
    const MgCoef<T> q = coef_of<T>(*ctx->grp[k]);
    c.cb[k] = q.cb;
    c.cy[k] = q.cy;
  }
  return c;
}

// a per-slot buffer (member `f` of MgSlot) of m, or of every lockstep slot
template <typename T>
static ModeArg<T> slot_bufs(const afg_ctx* ctx, const MgSlot& m, T* MgSlot::*f) {
  ModeArg<T> a(m.*f);
  for (int k = 1; k < ctx->ky; k++) a.p[k] = ctx->grp[k]->*f;
  return a;
}

// Ghost-cell method of a multigrid slot's phi; on batched trees the boundary
// values are read per instance from the slot's device rows.
static GcDev mg_gc(const afg_ctx* ctx, const MgSlot& m, bool homogeneous) {
  GcDev g;
  for (int n = 0; n < 6; n++) {
    g.bc_type[n] = m.d.bc_type[n];
    g.bc_val[n] = homogeneous ? 0.0 : m.d.bc_val[n];
  }
  g.rb = AFG_RB_MG_SIDES;
  g.ival = ctx->n_inst > 0 && !homogeneous ? m.d_bcval : nullptr;
  return g;
}

#include "afg_lsf.cuh"

// the electrode boxes' part of the restriction and of the FAS update (FP64)
template <typename T>
static int lsf_rrestrict(afg_ctx* ctx, const MgSlot& m, int lvl, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp,
                         int store_child, const GcDev& g, int otf) {
  if (!m.lsf) return AFG_OK;
  if constexpr (std::is_same<T, double>::value) {
    return launch_lsf_rrestrict(ctx, m, lvl, phi.p[0], rhs.p[0], tmp.p[0], store_child, g, otf);
  } else {
    return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode boxes in an FP32 solve");
  }
}
template <typename T>
static int lsf_coarse_fas(afg_ctx* ctx, const MgSlot& m, int plvl, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp,
                          int copy_tmp, int fill, const GcDev& g) {
  if (!m.lsf) return AFG_OK;
  if constexpr (std::is_same<T, double>::value) {
    return launch_lsf_coarse_fas(ctx, m, plvl, phi.p[0], rhs.p[0], tmp.p[0], copy_tmp, fill, g);
  } else {
    return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode boxes in an FP32 solve");
  }
}

template <typename T>
static int mg_gc_lvl(afg_ctx* ctx, int lvl, ModeArg<T> phi, const GcDev& g, int corners) {
  return launch_gc<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, g, corners);
}

// gsrb_boxes, m_af_multigrid.f90:648-687
template <typename T>
static int mg_gsrb_boxes(afg_ctx* ctx, const MgSlot& m, int lvl, int type, ModeArg<T> phi, ModeArg<const T> rhs,
                         const GcDev& g, bool fill_down = true, bool fill_needed_only = false,
                         bool stored_first = false) {
  const int n_cycle = type == AFG_CYCLE_DOWN ? m.d.n_cycle_down : m.d.n_cycle_up;
  const int* list = lst(ctx, ctx->off_ids[lvl - 1]);
  const int n = (int)ctx->lvl_ids[lvl - 1].size();
  ctx->ctr[1] += (long long)n * (long long)box_cells(ctx) * n_cycle * ctx->ky;
  LsfScope lsc(ctx, m);
  // the electrode boxes' half sweep after the ordinary boxes' (otf: ghost
  // values on the fly as the fused smoother's, else the stored ones)
  auto lsf_sweep = [&](int it, int otf) -> int {
    if (!m.lsf) return AFG_OK;
    if constexpr (std::is_same<T, double>::value) {
      return launch_lsf_gsrb(ctx, m, lvl, phi.p[0], const_cast<double*>(rhs.p[0]), it, g, otf);
    } else {
      return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode boxes in an FP32 solve");
    }
  };
  if (ctx->fused_gsrb) {
    int it0 = 1;
    if (stored_first) {
      // the first half sweep with the ghost cells as they are stored, then
      // the fill that follows it in the reference (gsrb_boxes)
      if (ctx->ky != 1 || rb_of<T>(ctx)) return fail(ctx, AFG_ERR_STATE, "stored-ghost half sweep: one FP64 problem");
      RC(launch_gsrb<T>(ctx, list, n, phi.p[0], rhs.p[0], 1, coef_of<T>(m)));
      RC(lsf_sweep(1, 0));
      RC(launch_gc<T>(ctx, list, n, phi, g, 0));
      it0 = 2;
    }
    for (int it = it0; it <= 2 * n_cycle; it++) {
      RC(launch_gsrb_fused<T>(ctx, list, n, phi, rhs, it, coefs<T>(ctx, m), g));
      RC(lsf_sweep(it, 1));
    }
    if (type == AFG_CYCLE_DOWN && !fill_down) return AFG_OK;
    if (type != AFG_CYCLE_DOWN && fill_needed_only)
      return launch_gc<T>(ctx, lst(ctx, ctx->off_gcneed[lvl - 1]), (int)ctx->lvl_gcneed[lvl - 1].size(), phi, g, 1);
    return launch_gc<T>(ctx, list, n, phi, g, type != AFG_CYCLE_DOWN ? 1 : 0);
  }
  // unfused reference order (one problem at a time)
  for (int it = 1; it <= 2 * n_cycle; it++) {
    RC(launch_gsrb<T>(ctx, list, n, phi.p[0], rhs.p[0], it, coef_of<T>(m)));
    RC(lsf_sweep(it, 0));
    const int corners = (type != AFG_CYCLE_DOWN && it == 2 * n_cycle) ? 1 : 0;
    RC(launch_gc<T>(ctx, list, n, phi, g, corners));
  }
  return AFG_OK;
}

// update_coarse (m_af_multigrid.f90:691-738): residual of lvl restricted to
// the parents, phi restricted, then the parents' ghost fill fused with the
// FAS right-hand side.  otf: the residual's neighbours across box faces are
// computed on the fly, so lvl needs no ghost fill after its down smoothing
// (the V-cycle); otherwise the stored ghost cells are used as they are.
template <typename T>
static int mg_update_coarse(afg_ctx* ctx, const MgSlot& m, int lvl, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp,
                            const GcDev& g, bool otf = true) {
  LsfScope lsc(ctx, m);
  RC(launch_rrestrict<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, rhs, tmp,
                         coefs<T>(ctx, m), 0, g, otf ? 1 : 0));
  RC(lsf_rrestrict<T>(ctx, m, lvl, phi, rhs, tmp, 0, g, otf ? 1 : 0));
  RC(launch_coarse_fas<T>(ctx, lst(ctx, ctx->off_parents[lvl - 2]), (int)ctx->lvl_parents[lvl - 2].size(), phi, rhs,
                          tmp, coefs<T>(ctx, m), 1, 1, g));
  RC(lsf_coarse_fas<T>(ctx, m, lvl - 1, phi, rhs, tmp, 1, 1, g));
  return AFG_OK;
}

// set_coarse_phi_rhs, m_af_multigrid.f90:742-776
template <typename T>
static int mg_set_coarse_phi_rhs(afg_ctx* ctx, const MgSlot& m, int lvl, ModeArg<T> phi, ModeArg<T> rhs,
                                 ModeArg<T> tmp, const GcDev& g) {
  LsfScope lsc(ctx, m);
  if (lvl == ctx->highest_lvl) RC(mg_gc_lvl<T>(ctx, lvl, phi, g, 1));
  RC(launch_rrestrict<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, rhs, tmp,
                         coefs<T>(ctx, m), 1, g, 0));
  RC(lsf_rrestrict<T>(ctx, m, lvl, phi, rhs, tmp, 1, g, 0));
  RC(mg_gc_lvl<T>(ctx, lvl - 1, phi, g, 1));
  RC(launch_coarse_fas<T>(ctx, lst(ctx, ctx->off_parents[lvl - 2]), (int)ctx->lvl_parents[lvl - 2].size(), phi, rhs,
                          tmp, coefs<T>(ctx, m), 0, 0, g));
  RC(lsf_coarse_fas<T>(ctx, m, lvl - 1, phi, rhs, tmp, 0, 0, g));
  return AFG_OK;
}

// correct_children(parents of lvl-1) + af_gc_lvl(lvl).  Inside the V-cycle
// and FMG the next operation on lvl is the fused smoother, which computes the
// face ghosts it reads from the neighbours' current values (the same values
// af_gc_lvl would store) and fills all ghosts when it ends; there the ghost
// fill is skipped (fill = false), the stored ghost cells of lvl being read
// by nothing in between.
template <typename T>
static int mg_correct(afg_ctx* ctx, int lvl, ModeArg<T> phi, ModeArg<T> tmp, const GcDev& g, bool fill = true) {
  RC(launch_correct<T>(ctx, lst(ctx, ctx->off_parents[lvl - 2]), (int)ctx->lvl_parents[lvl - 2].size(), phi, tmp));
  if (fill) RC(mg_gc_lvl<T>(ctx, lvl, phi, g, 1));
  return AFG_OK;
}

// solve_coarse_grid, m_af_multigrid.f90:266-291 (exact FP64 solve)
// (batched trees: every instance's coarse grid with the shared inverse and
// its own boundary values; lockstep slots: each its own inverse and vectors,
// the boundary tables and values those of m, equal for all of them)
template <typename T>
static int mg_coarse_solve(afg_ctx* ctx, MgSlot& m, ModeArg<T> phi, ModeArg<const T> rhs, const GcDev& g,
                           bool homogeneous) {
  const int nloc = m.n_coarse, rows = inst_rows(ctx), n = nloc * rows;
  {
  KtScope kts(ctx, AFG_KT_COARSE, 0.0);
  const double* bcv = m.d_bcval + (homogeneous ? 6 * rows : 0);
  const int stride = homogeneous ? 0 : 6;
  const ModeArg<double> b = slot_bufs(ctx, m, &MgSlot::d_b), x = slot_bufs(ctx, m, &MgSlot::d_x);
  ModeArg<const double> ainv(m.d_ainv);
  for (int k = 1; k < ctx->ky; k++) ainv.p[k] = ctx->grp[k]->d_ainv;
  const dim3 g128((n + 127) / 128, ctx->ky), g8((n + 7) / 8, ctx->ky);
  const bool rbl = rb_of<T>(ctx);
  const int* ccell = rbl ? ctx->d_ccell_rb : ctx->d_ccell;
  const int cstride = rbl ? (int)ktree(ctx).SI : ctx->S;
  k_coarse_gather<T><<<g128, 128, 0, ctx->stream>>>(n, nloc, ctx->D, ctx->d_cslot, ccell, m.d_b2r, m.d_bmask,
                                                    bcv, stride, rhs, cstride, b);
  ctx->launches++;
  CKL();
  if (m.lsf && !homogeneous) RC(launch_lsf_coarse_bcc(ctx, m, m.d_b));
  k_coarse_matvec<<<g8, 256, 0, ctx->stream>>>(n, nloc, ainv, ModeArg<const double>(b), x);
  ctx->launches++;
  CKL();
  k_coarse_scatter<T><<<g128, 128, 0, ctx->stream>>>(ktree(ctx), n, ctx->d_cslot, ccell, cstride,
                                                     ModeArg<const double>(x), phi);
  ctx->launches++;
  CKL();
  }
  return mg_gc_lvl<T>(ctx, 1, phi, g, 1);
}

// Freeze flags seen by the kernels of a batched tree: converged instances
// plus those whose highest level is outside [lo, hi] (no-op on one tree).
static int inst_mask(afg_ctx* ctx, int lo, int hi) {
  if (ctx->n_inst <= 0) return AFG_OK;
  k_inst_mask<<<(ctx->n_inst + 127) / 128, 128, 0, ctx->stream>>>(ctx->n_inst, ctx->d_frozen_base, ctx->d_inst_hl, lo,
                                                                  hi, ctx->d_frozen);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

template <typename T>
static int mg_residual_lvls(afg_ctx* ctx, const MgSlot& m, int max_lvl, const T* phi, const T* rhs, T* tmp,
                            unsigned long long* maxbits) {
  LsfScope lsc(ctx, m);
  if (m.lsf) {
    if constexpr (std::is_same<T, double>::value) {
      const GcDev g = mg_gc(ctx, m, false);
      for (int lvl = 1; lvl <= max_lvl; lvl++) RC(launch_lsf_residual(ctx, m, lvl, phi, rhs, tmp, g, maxbits));
    } else {
      return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode boxes in an FP32 solve");
    }
  }
  if (max_lvl == ctx->highest_lvl)  // boxes are independent: one launch over all levels
    return launch_residual<T>(ctx, lst(ctx, ctx->off_all), ctx->n_all, phi, rhs, tmp, coef_of<T>(m), maxbits);
  for (int lvl = 1; lvl <= max_lvl; lvl++)
    RC(launch_residual<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, rhs, tmp,
                          coef_of<T>(m), maxbits));
  return AFG_OK;
}

// mg_fas_vcycle, m_af_multigrid.f90:185-264 (the residual, set_residual,
// for one problem at a time)
//
// stored_first: the first half sweep on max_lvl reads the ghost cells as
// they are stored, as the reference's does.  A V-cycle called on its own
// cannot know whether they are current: a mesh change leaves old ghost
// values next to changed neighbours, and the reference's first half sweep
// uses them.  Every later half sweep sees freshly filled (or equal on-the-fly)
// values, in the reference as here.  Inside FMG the level was just corrected
// and filled in the reference, so its ghost values are current there.
template <typename T>
static int mg_vcycle(afg_ctx* ctx, MgSlot& m, int max_lvl, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp,
                     bool set_residual, bool homogeneous, unsigned long long* maxbits, bool stored_first = false) {
  const GcDev g = mg_gc(ctx, m, homogeneous);
  ctx->ctr[3] += ctx->ky;
  for (int lvl = max_lvl; lvl >= 2; lvl--) {
    // the restriction below computes the face neighbours it needs itself
    RC(mg_gsrb_boxes<T>(ctx, m, lvl, AFG_CYCLE_DOWN, phi, rhs, g, false, false, stored_first && lvl == max_lvl));
    RC(mg_update_coarse<T>(ctx, m, lvl, phi, rhs, tmp, g));
  }
  RC(mg_coarse_solve<T>(ctx, m, phi, rhs, g, homogeneous));
  // A correction V-cycle (homogeneous, no residual: the mixed path's inner
  // cycles) fills after the up smoothing only the ghost cells read later:
  // those of parents (prolongation to the next level) and of refinement
  // sources (the next level's refinement rules).
  const bool needed_only = homogeneous && !set_residual;
  for (int lvl = 2; lvl <= max_lvl; lvl++) {
    RC(mg_correct<T>(ctx, lvl, phi, tmp, g, !ctx->fused_gsrb));
    RC(mg_gsrb_boxes<T>(ctx, m, lvl, AFG_CYCLE_UP, phi, rhs, g, true, needed_only));
  }
  if (set_residual) RC(mg_residual_lvls<T>(ctx, m, max_lvl, phi.p[0], rhs.p[0], tmp.p[0], maxbits));
  return AFG_OK;
}

// mg_fas_fmg, m_af_multigrid.f90:137-180
template <typename T>
static int mg_fmg(afg_ctx* ctx, MgSlot& m, ModeArg<T> phi, ModeArg<T> rhs, ModeArg<T> tmp, bool set_residual,
                  bool have_guess, unsigned long long* maxbits, bool homogeneous = false) {
  const GcDev g = mg_gc(ctx, m, homogeneous);
  const int H = ctx->highest_lvl;
  if (have_guess) {
    for (int lvl = H; lvl >= 2; lvl--) RC(mg_set_coarse_phi_rhs<T>(ctx, m, lvl, phi, rhs, tmp, g));
  } else {
    for (int lvl = H; lvl >= 2; lvl--)
      RC(launch_init_phi_rhs<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, rhs));
  }
  RC(launch_copy<T>(ctx, lst(ctx, ctx->off_ids[0]), (int)ctx->lvl_ids[0].size(), phi, tmp));
  if (ctx->n_inst <= 0) {
    RC(mg_vcycle<T>(ctx, m, 1, phi, rhs, tmp, set_residual && H == 1, homogeneous, maxbits));
    for (int lvl = 2; lvl <= H; lvl++) {
      RC(launch_copy<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, tmp));
      RC(mg_correct<T>(ctx, lvl, phi, tmp, g, !ctx->fused_gsrb));
      RC(mg_vcycle<T>(ctx, m, lvl, phi, rhs, tmp, set_residual && lvl == H, homogeneous, maxbits));
    }
    return AFG_OK;
  }
  // Batched instances of different depths: the V-cycle at level lvl runs on
  // the instances that have that level (an instance's FMG ends at its own
  // highest level), and the residual of an instance is taken after its last
  // V-cycle; then the flags return to the converged set.
  for (int lvl = 1; lvl <= H; lvl++) {
    RC(inst_mask(ctx, lvl, INT_MAX));
    if (lvl > 1) {
      RC(launch_copy<T>(ctx, lst(ctx, ctx->off_ids[lvl - 1]), (int)ctx->lvl_ids[lvl - 1].size(), phi, tmp));
      RC(mg_correct<T>(ctx, lvl, phi, tmp, g, !ctx->fused_gsrb));
    }
    RC(mg_vcycle<T>(ctx, m, lvl, phi, rhs, tmp, false, homogeneous, maxbits));
    if (set_residual) {
      RC(inst_mask(ctx, lvl, lvl));
      RC(mg_residual_lvls<T>(ctx, m, lvl, phi.p[0], rhs.p[0], tmp.p[0], maxbits));
    }
  }
  return inst_mask(ctx, 0, INT_MAX);
}

// Slots of the device maxima: 0 right-hand side / max-norm, 1 V-cycle and
// FMG residual, 2 defect, 3-4 transport limits, 5 chemistry limit, from
// kModeSlot per Helmholtz mode.  On batched trees the residual-type slots
// hold one word per instance (row q at d_max + q * kMaxSlots); the
// transport limits stay global (row 0).
static bool inst_slot(const afg_ctx* ctx, int slot) { return ctx->n_inst > 0 && (slot < 3 || slot > 5); }

static double bits_to_double(unsigned long long b) {
  double v;
  memcpy(&v, &b, sizeof(double));
  return v;
}

// value of slot for instance q after read_max (batched trees)
static double inst_value(const afg_ctx* ctx, int slot, int q) {
  return bits_to_double(ctx->h_max[(size_t)q * kMaxSlots + slot]);
}

// the slot's maximum (over all instances of a batched tree)
static int wait_failed(afg_ctx* ctx) {
  if (*ctx->h_err & 2u) {
    ctx->poisoned = true;
    return fail(ctx, AFG_ERR_CUDA, "a bounded wait on a copy into shared memory timed out and the copies did "
                                   "not drain; the context is unusable");
  }
  return fail(ctx, AFG_ERR_CUDA, "a bounded wait on a copy into shared memory timed out");
}

static int read_max(afg_ctx* ctx, int slot, double* out) {
  CK(cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  if (!inst_slot(ctx, slot)) {
    CK(cudaMemcpyAsync(ctx->h_max + slot, ctx->d_max + slot, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (*ctx->h_err) return wait_failed(ctx);
    *out = bits_to_double(ctx->h_max[slot]);
    return AFG_OK;
  }
  const size_t pitch = kMaxSlots * sizeof(unsigned long long);
  CK(cudaMemcpy2DAsync(ctx->h_max + slot, pitch, ctx->d_max + slot, pitch, sizeof(unsigned long long), ctx->n_inst,
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (*ctx->h_err) return wait_failed(ctx);
  double mx = 0;
  for (int q = 0; q < ctx->n_inst; q++) mx = std::max(mx, inst_value(ctx, slot, q));
  *out = mx;
  return AFG_OK;
}

static int reset_max(afg_ctx* ctx, int slot) {
  if (!inst_slot(ctx, slot)) {
    CK(cudaMemsetAsync(ctx->d_max + slot, 0, sizeof(unsigned long long), ctx->stream));
    return AFG_OK;
  }
  const size_t pitch = kMaxSlots * sizeof(unsigned long long);
  CK(cudaMemset2DAsync(ctx->d_max + slot, pitch, 0, sizeof(unsigned long long), ctx->n_inst, ctx->stream));
  return AFG_OK;
}

// Autotuner of the compact-layout FP32 smoother: the staged kernel with 1, 2
// or 4 cells per thread and the one-box-per-CTA kernel, timed like the
// ghosted-layout variants below on the level with the most boxes.
static int autotune_gsrb_rb(afg_ctx* ctx, MgSlot& m) {
  int best_l = 0;
  for (int l = 0; l < ctx->highest_lvl; l++)
    if (ctx->lvl_ids[l].size() > ctx->lvl_ids[best_l].size()) best_l = l;
  const int n = (int)ctx->lvl_ids[best_l].size();
  if (n < 256) return AFG_OK;  // too small to time; the default stays
  const int* rec = rec_of(ctx, lst(ctx, ctx->off_ids[best_l]));
  const GcDev g = mg_gc(ctx, m, true);
  const int cands[] = {kGsrbTma | 1, kGsrbTma | 2, kGsrbTma | 4, -1};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_c = kGsrbTma | 2;
  int rc = AFG_OK;
  for (int q = 0; q < 4 && rc == AFG_OK; q++) {
    float tmin = 1e30f;
    for (int r = 0; r < 8 && rc == AFG_OK; r++) {
      cudaEventRecord(e0, ctx->stream);
      rc = launch_gsrb_rb(ctx, rec, n, m.e32, m.r32, 1 + (r & 1), coef_of<float>(m), g, cands[q]);
      cudaEventRecord(e1, ctx->stream);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0) tmin = std::min(tmin, ms);
    }
    if (tmin < best) {
      best = tmin;
      best_c = cands[q];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  RC(rc);
  ctx->gsrb_cpt[2] = best_c;
  const size_t N = (size_t)ctx->n_boxes * (ktree(ctx).SI + ctx->S);
  CK(cudaMemsetAsync(m.e32, 0, N * sizeof(float), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

// Autotuner of the smoother's work shape: on the level with the most boxes,
// time every cells-per-thread variant of the FP32 half sweep (CUDA events,
// best of 7 after a warm-up) on the slot's FP32 buffers, which are scratch
// outside a solve, and keep the fastest.  All variants do the same
// arithmetic, so the choice changes speed only.
static int autotune_gsrb(afg_ctx* ctx, MgSlot& m) {
  if (!gsrb_rec_specialized(ctx) || !m.e32) return AFG_OK;
  if (ctx->rb32) return autotune_gsrb_rb(ctx, m);
  int best_l = 0;
  for (int l = 0; l < ctx->highest_lvl; l++)
    if (ctx->lvl_ids[l].size() > ctx->lvl_ids[best_l].size()) best_l = l;
  const int n = (int)ctx->lvl_ids[best_l].size();
  if (n < 256) return AFG_OK;  // too small to time; the default stays
  const int* rec = rec_of(ctx, lst(ctx, ctx->off_ids[best_l]));
  const GcDev g = mg_gc(ctx, m, true);
  const int S = kGsrbTma, R = kGsrbTma | kGsrbTmaRhs;
  const int cands3[] = {1, 2, 4, 8, S | 2, S | 4, R | 2, R | 4}, cands2[] = {1, 2, 4, S | 1, S | 2, R | 1, R | 2};
  const int* cands = ctx->D == 3 ? cands3 : cands2;
  const int nc = ctx->D == 3 ? 8 : 7;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_c = gsrb_cpt_of<float>(ctx);
  int rc = AFG_OK;
  for (int q = 0; q < nc && rc == AFG_OK; q++) {
    float tmin = 1e30f;
    for (int r = 0; r < 8 && rc == AFG_OK; r++) {
      cudaEventRecord(e0, ctx->stream);
      rc = launch_gsrb_rec<float>(ctx, rec, n, m.e32, m.r32, 1 + (r & 1), coef_of<float>(m), g, cands[q]);
      cudaEventRecord(e1, ctx->stream);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0) tmin = std::min(tmin, ms);
    }
    if (tmin < best) {
      best = tmin;
      best_c = cands[q];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  RC(rc);
  ctx->gsrb_cpt[0] = best_c;
  // the correction buffers were only smoothed with zero data; clear them
  const size_t N = (size_t)ctx->n_boxes * ctx->S;
  CK(cudaMemsetAsync(m.e32, 0, N * sizeof(float), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

#include "afg_mixed.cuh"

/* ------------------------------------------------------------------------- */
// Batched independent instances: per-instance convergence.  A solve loop
// freezes the instances that have converged while the others continue
// (kernels skip their boxes), so every instance ends exactly where a solve
// of its own tree would; replayed graphs stay valid because the flags live
// in device memory.

// base freeze flags (converged instances) from the host, also as the flags
// the kernels read; the pinned copy may change again after the next sync
static int set_frozen(afg_ctx* ctx, const std::vector<char>& done) {
  if (ctx->n_inst <= 0) return AFG_OK;
  for (int q = 0; q < ctx->n_inst; q++) ctx->h_frozen[q] = done[q] ? 1 : 0;
  CK(cudaMemcpyAsync(ctx->d_frozen_base, ctx->h_frozen, sizeof(int) * ctx->n_inst, cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_frozen, ctx->d_frozen_base, sizeof(int) * ctx->n_inst, cudaMemcpyDeviceToDevice,
                     ctx->stream));
  return AFG_OK;
}

// smoother cell updates of one V-cycle of instance q (levels 2..its highest)
static long long inst_vcycle_work(const afg_ctx* ctx, const MgSlot& m, int q) {
  long long w = 0;
  for (int l = 2; l <= ctx->inst_hl[q]; l++) w += ctx->inst_cells[q][l - 1];
  return w * (m.d.n_cycle_down + m.d.n_cycle_up);
}

// ... of one FMG of instance q (a V-cycle up to each of its levels)
static long long inst_fmg_work(const afg_ctx* ctx, const MgSlot& m, int q) {
  long long w = 0;
  for (int top = 2; top <= ctx->inst_hl[q]; top++)
    for (int l = 2; l <= top; l++) w += ctx->inst_cells[q][l - 1];
  return w * (m.d.n_cycle_down + m.d.n_cycle_up);
}

// The cell-update counter of a V-cycle or FMG launch sequence counts every
// box of the levels it visits; on a batched tree remove the updates that
// frozen instances, and instances past the end of their own FMG, skipped.
static void inst_uncount(afg_ctx* ctx, const MgSlot& m, bool fmg) {
  if (ctx->n_inst <= 0) return;
  const int H = ctx->highest_lvl;
  for (int q = 0; q < ctx->n_inst; q++) {
    const long long V = inst_vcycle_work(ctx, m, q), extra = fmg ? (H - ctx->inst_hl[q]) * V : 0;
    ctx->ctr[1] -= extra + (ctx->h_frozen[q] ? (fmg ? inst_fmg_work(ctx, m, q) : V) : 0);
  }
}

// the launch sequences of one solve iteration (shared by the single-tree
// and the batched loops, so both replay the same graphs)
// first: the first V-cycle of a solve (its first half sweep reads the stored
// ghost cells, which a mesh change may have left behind; after it they are
// current and on-the-fly values equal them)
static int vcycle_graph(afg_ctx* ctx, MgSlot& m, bool first) {
  const int mg_id = (int)(&m - ctx->mg);
  double* phi = ctx->cc[m.d.i_phi - 1];
  double* rhs = ctx->cc[m.d.i_rhs - 1];
  double* tmp = ctx->cc[m.d.i_tmp - 1];
  RC(run_graph(ctx, gkey(first ? "vcycle" : "vcycle_next", mg_id, ctx->highest_lvl, 1), [&]() -> int {
    RC(reset_max(ctx, 1));
    return mg_vcycle<double>(ctx, m, ctx->highest_lvl, phi, rhs, tmp, true, false, ctx->d_max + 1, first);
  }));
  inst_uncount(ctx, m, false);
  return AFG_OK;
}

static int mixed_defect_graph(afg_ctx* ctx, MgSlot& m) {
  const int mg_id = (int)(&m - ctx->mg);
  double* phi = ctx->cc[m.d.i_phi - 1];
  double* rhs = ctx->cc[m.d.i_rhs - 1];
  return run_graph(ctx, gkey("defect", mg_id), [&]() -> int {
    RC(mixed_prepare(ctx, m, phi));
    RC(reset_max(ctx, 2));
    return launch_defect(ctx, m, phi, rhs, ctx->d_max + 2);
  });
}

static int mixed_iter_graph(afg_ctx* ctx, MgSlot& m) {
  const int mg_id = (int)(&m - ctx->mg);
  double* phi = ctx->cc[m.d.i_phi - 1];
  double* rhs = ctx->cc[m.d.i_rhs - 1];
  RC(run_graph(ctx, gkey("mixed_iter", mg_id), [&]() -> int {
    RC(mg_vcycle<float>(ctx, m, ctx->highest_lvl, m.e32, m.r32, m.t32, false, true, nullptr));
    // leaves only: mixed_prepare restricts the parents from them
    RC(launch_add_correction(ctx, lst(ctx, ctx->off_all_leaves), ctx->n_all_leaves, phi, m.e32));
    RC(mixed_prepare(ctx, m, phi));
    RC(reset_max(ctx, 2));
    return launch_defect(ctx, m, phi, rhs, ctx->d_max + 2);
  }));
  inst_uncount(ctx, m, false);
  return AFG_OK;
}

// afg_mg_solve of a mixed-precision slot on one tree: FP64 defect, then
// iterations of FP32 V-cycle on the correction, update and new defect until
// the defect is below the threshold; all ghost cells of phi at the end.
static int mixed_solve(afg_ctx* ctx, MgSlot& m, double threshold, int max_cycles, int* n_done, double* residuals) {
  double* phi = ctx->cc[m.d.i_phi - 1];
  double r = 0;
  int n = 0;
  const int mg_id = (int)(&m - ctx->mg);
  RC(mixed_defect_graph(ctx, m));
  RC(read_max(ctx, 2, &r));
  while (n < max_cycles) {
    RC(mixed_iter_graph(ctx, m));
    RC(read_max(ctx, 2, &r));
    if (residuals) residuals[n] = r;
    n++;
    if (r < threshold) break;
  }
  RC(run_graph(ctx, gkey("mixed_finish", mg_id), [&]() -> int { return mixed_finish(ctx, m, phi); }));
  if (n_done) *n_done = n;
  return r < threshold ? AFG_OK : AFG_ERR_NOCONV;
}

// Solve loop of a batched tree: per instance until its residual is below
// thr[q] (at most max_cycles iterations); n_done[q] iterations and the last
// residual res[q] per instance (either may be null).
static int mg_solve_inst(afg_ctx* ctx, MgSlot& m, const double* thr, int max_cycles, int* n_done, double* res) {
  const int Q = ctx->n_inst;
  const bool mixed = m.d.precision == AFG_MIXED;
  const int slot = mixed ? 2 : 1;
  std::vector<char> done(Q, 0);
  std::vector<int> cyc(Q, 0);
  std::vector<double> r(Q, 0.0);
  double mx;
  RC(set_frozen(ctx, done));
  if (mixed) {
    // the defect of the current phi; as on one tree, at least one
    // iteration follows
    RC(mixed_defect_graph(ctx, m));
    RC(read_max(ctx, 2, &mx));
    for (int q = 0; q < Q; q++) r[q] = inst_value(ctx, 2, q);
  }
  auto all_done = [&]() {
    for (int q = 0; q < Q; q++)
      if (!done[q]) return false;
    return true;
  };
  for (int it = 0; it < max_cycles && !all_done(); it++) {
    RC(set_frozen(ctx, done));
    RC(mixed ? mixed_iter_graph(ctx, m) : vcycle_graph(ctx, m, it == 0));
    RC(read_max(ctx, slot, &mx));
    for (int q = 0; q < Q; q++) {
      if (done[q]) continue;
      r[q] = inst_value(ctx, slot, q);
      cyc[q]++;
      done[q] = r[q] < thr[q];
    }
  }
  const bool ok = all_done();
  std::fill(done.begin(), done.end(), 0);
  RC(set_frozen(ctx, done));
  if (mixed) {
    const int mg_id = (int)(&m - ctx->mg);
    double* phi = ctx->cc[m.d.i_phi - 1];
    RC(run_graph(ctx, gkey("mixed_finish", mg_id), [&]() -> int { return mixed_finish(ctx, m, phi); }));
  }
  for (int q = 0; q < Q; q++) {
    if (n_done) n_done[q] = cyc[q];
    if (res) res[q] = r[q];
  }
  return ok ? AFG_OK : AFG_ERR_NOCONV;
}

/* ========================================================================= */
extern "C" {

int afg_init(int device, afg_ctx** out) {
  afg_ctx* ctx = nullptr;
  if (!out) return AFG_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return AFG_ERR_CUDA;
  if (device < 0 || device >= ndev) return AFG_ERR_ARG;
  ctx = new afg_ctx();
  ctx->device = device;
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(dalloc(&ctx->d_max, kMaxSlots));
  CK(cudaMallocHost((void**)&ctx->h_max, kMaxSlots * sizeof(unsigned long long)));
  CK(dalloc(&ctx->d_err, 1));
  CK(cudaMemset(ctx->d_err, 0, sizeof(unsigned)));
  CK(cudaMallocHost((void**)&ctx->h_err, sizeof(unsigned)));
  *ctx->h_err = 0;
  CK(cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device));
  for (auto& st : ctx->side) CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->xfer_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->ev_xfer, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  for (auto& e : ctx->ev_join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto& e : ctx->xfer_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  *out = ctx;
  return AFG_OK;
}

int afg_finalize(afg_ctx* ctx) {
  if (!ctx) return AFG_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_tree(ctx);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->kt_ev) cudaEventDestroy(e);
  for (auto& e : ctx->xfer_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->flush_buf) cudaFree(ctx->flush_buf);
  dfree(ctx->d_max);
  if (ctx->h_max) cudaFreeHost(ctx->h_max);
  dfree(ctx->d_err);
  if (ctx->h_err) cudaFreeHost(ctx->h_err);
  if (ctx->xfer_stream) {
    cudaStreamSynchronize(ctx->xfer_stream);
    cudaStreamDestroy(ctx->xfer_stream);
  }
  if (ctx->ev_xfer) cudaEventDestroy(ctx->ev_xfer);
  for (auto& st : ctx->side)
    if (st) cudaStreamDestroy(st);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  for (auto& e : ctx->ev_join)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return AFG_OK;
}

const char* afg_last_error(const afg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long afg_launch_count(const afg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int afg_check_bounded_wait(afg_ctx* ctx, double* waited_ms) {
  if (!ctx) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  cudaEventRecord(e0, ctx->stream);
  k_wait_check<<<1, 32, 0, ctx->stream>>>(256u, ctx->d_err);
  cudaEventRecord(e1, ctx->stream);
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "bounded-wait check: %s", cudaGetErrorString(e));
  if (waited_ms) *waited_ms = ms;
  // the error word is read like after every solve iteration, then cleared
  double unused;
  const int rc = read_max(ctx, 1, &unused);
  CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (rc == AFG_OK) return fail(ctx, AFG_ERR_STATE, "the timed-out wait was not reported");
  return rc == AFG_ERR_CUDA ? AFG_ERR_DEVICE : rc;
}

int afg_sync(afg_ctx* ctx) {
  if (!ctx) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

int afg_tree_sync(afg_ctx* ctx, const afg_tree_desc* t, int n_var_cell, int n_var_face) {
  return afg_tree_sync_batched(ctx, t, n_var_cell, n_var_face, 0, nullptr);
}

int afg_tree_sync_batched(afg_ctx* ctx, const afg_tree_desc* t, int n_var_cell, int n_var_face, int n_inst,
                          const int* box_inst) {
  if (!ctx || !t) return AFG_ERR_ARG;
  if (n_inst < 0 || (n_inst > 0 && !box_inst)) return fail(ctx, AFG_ERR_ARG, "bad instance table");
  if (t->ndim != 2 && t->ndim != 3) return fail(ctx, AFG_ERR_ARG, "ndim must be 2 or 3");
  if (t->n_cell < 2 || (t->n_cell & 1) || t->n_cell > 64) return fail(ctx, AFG_ERR_ARG, "bad n_cell %d", t->n_cell);
  if (t->coord == AFG_CYL && t->ndim != 2) return fail(ctx, AFG_ERR_ARG, "cylindrical needs ndim=2");
  if (t->n_boxes <= 0 || t->highest_lvl <= 0 || n_var_cell <= 0) return fail(ctx, AFG_ERR_ARG, "empty tree");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  free_tree(ctx);
  const int D = t->ndim, nc = t->n_cell, n = t->n_boxes;
  ctx->D = D;
  ctx->nc = nc;
  ctx->n2 = nc + 2;
  ctx->S = D == 2 ? (nc + 2) * (nc + 2) : (nc + 2) * (nc + 2) * (nc + 2);
  ctx->NF = D == 2 ? (nc + 1) * (nc + 1) : (nc + 1) * (nc + 1) * (nc + 1);
  ctx->coord = t->coord;
  ctx->n_boxes = n;
  ctx->highest_lvl = t->highest_lvl;
  for (int d = 0; d < 3; d++) ctx->cgs[d] = d < D ? t->coarse_grid_size[d] : 1;
  const int nch = 1 << D, nnb = 2 * D, nm = D == 2 ? 9 : 27;
  // host tables converted to slots
  std::vector<int> parent(n), children((size_t)n * nch), nbr((size_t)n * nnb), pnb((size_t)n * nnb, -1),
      nbmat((size_t)n * nm);
  for (int b = 0; b < n; b++) {
    const int p = t->parent[b];
    if (p < 0 || p > n) return fail(ctx, AFG_ERR_ARG, "bad parent of box %d", b + 1);
    parent[b] = p - 1;
    for (int c = 0; c < nch; c++) {
      const int v = t->children[(size_t)b * nch + c];
      if (v < 0 || v > n) return fail(ctx, AFG_ERR_ARG, "bad child of box %d", b + 1);
      children[(size_t)b * nch + c] = v - 1;
    }
    for (int k = 0; k < nm; k++) {
      const int v = t->neighbor_mat[(size_t)b * nm + k];
      if (v > n) return fail(ctx, AFG_ERR_ARG, "bad neighbor_mat of box %d", b + 1);
      nbmat[(size_t)b * nm + k] = v > 0 ? v - 1 : -1;
    }
  }
  for (int b = 0; b < n; b++)
    for (int nb = 0; nb < nnb; nb++) {
      const int v = t->neighbors[(size_t)b * nnb + nb];
      if (v > n || v < -1) return fail(ctx, AFG_ERR_ARG, "bad neighbor of box %d", b + 1);
      if (v > 0) {
        nbr[(size_t)b * nnb + nb] = v - 1;
      } else if (v == 0) {
        nbr[(size_t)b * nnb + nb] = kNbRefine;
        const int p = parent[b];
        if (p < 0) return fail(ctx, AFG_ERR_ARG, "level-1 box %d has a refinement boundary", b + 1);
        const int pn = t->neighbors[(size_t)p * nnb + nb];
        if (pn <= 0) return fail(ctx, AFG_ERR_ARG, "parent of box %d lacks neighbour %d (2:1 balance)", b + 1, nb + 1);
        pnb[(size_t)b * nnb + nb] = pn - 1;
      } else {
        nbr[(size_t)b * nnb + nb] = kNbPhys;
      }
    }
  ctx->h_ix.assign(t->ix, t->ix + (size_t)n * D);
  ctx->h_parent = parent;
  ctx->h_nbr.assign(t->neighbors, t->neighbors + (size_t)n * nnb);
  // independent instances: every relation of a box stays inside its instance
  if (n_inst > 0) {
    ctx->h_inst.assign(box_inst, box_inst + n);
    for (int b = 0; b < n; b++) {
      const int q = box_inst[b];
      if (q < 0 || q >= n_inst) return fail(ctx, AFG_ERR_ARG, "box %d: instance %d out of range", b + 1, q);
      if (parent[b] >= 0 && box_inst[parent[b]] != q) return fail(ctx, AFG_ERR_ARG, "box %d: parent in another instance", b + 1);
      for (int c = 0; c < nch; c++) {
        const int v = children[(size_t)b * nch + c];
        if (v >= 0 && box_inst[v] != q) return fail(ctx, AFG_ERR_ARG, "box %d: child in another instance", b + 1);
      }
      for (int k = 0; k < nnb; k++) {
        const int v = nbr[(size_t)b * nnb + k];
        if (v >= 0 && box_inst[v] != q) return fail(ctx, AFG_ERR_ARG, "box %d: neighbour in another instance", b + 1);
      }
      for (int k = 0; k < nm; k++) {
        const int v = nbmat[(size_t)b * nm + k];
        if (v >= 0 && box_inst[v] != q) return fail(ctx, AFG_ERR_ARG, "box %d: neighbor_mat in another instance", b + 1);
      }
    }
  }
  const int rows = n_inst > 0 ? n_inst : 1;
  // level lists
  ctx->lvl_ids.assign(t->highest_lvl, {});
  ctx->lvl_leaves.assign(t->highest_lvl, {});
  ctx->lvl_parents.assign(t->highest_lvl, {});
  std::vector<int> all;
  std::vector<unsigned char> is_leaf(n, 0);
  for (int l = 0; l < t->highest_lvl; l++) {
    for (int k = t->ids_off[l]; k < t->ids_off[l + 1]; k++) {
      const int id = t->ids[k];
      if (id < 1 || id > n) return fail(ctx, AFG_ERR_ARG, "bad id in level list %d", l + 1);
      ctx->lvl_ids[l].push_back(id - 1);
    }
    for (int k = t->leaves_off[l]; k < t->leaves_off[l + 1]; k++) {
      const int id = t->leaves[k];
      if (id < 1 || id > n) return fail(ctx, AFG_ERR_ARG, "bad id in leaf list %d", l + 1);
      ctx->lvl_leaves[l].push_back(id - 1);
      is_leaf[id - 1] = 1;
    }
    for (int k = t->parents_off[l]; k < t->parents_off[l + 1]; k++) {
      const int id = t->parents[k];
      if (id < 1 || id > n) return fail(ctx, AFG_ERR_ARG, "bad id in parent list %d", l + 1);
      ctx->lvl_parents[l].push_back(id - 1);
    }
  }
  std::vector<int> lists;
  ctx->off_ids.assign(t->highest_lvl, 0);
  ctx->off_leaves.assign(t->highest_lvl, 0);
  ctx->off_parents.assign(t->highest_lvl, 0);
  for (int l = 0; l < t->highest_lvl; l++) {
    ctx->off_ids[l] = lists.size();
    lists.insert(lists.end(), ctx->lvl_ids[l].begin(), ctx->lvl_ids[l].end());
    ctx->off_leaves[l] = lists.size();
    lists.insert(lists.end(), ctx->lvl_leaves[l].begin(), ctx->lvl_leaves[l].end());
    ctx->off_parents[l] = lists.size();
    lists.insert(lists.end(), ctx->lvl_parents[l].begin(), ctx->lvl_parents[l].end());
  }
  ctx->off_all = lists.size();
  ctx->n_all = 0;
  for (int l = 0; l < t->highest_lvl; l++) {
    lists.insert(lists.end(), ctx->lvl_ids[l].begin(), ctx->lvl_ids[l].end());
    ctx->n_all += (int)ctx->lvl_ids[l].size();
  }
  {
    std::vector<unsigned char> src(n, 0);
    for (int b = 0; b < n; b++)
      for (int nb = 0; nb < nnb; nb++)
        if (nbr[(size_t)b * nnb + nb] == kNbRefine) src[pnb[(size_t)b * nnb + nb]] = 1;
    ctx->lvl_rbsrc.assign(t->highest_lvl, {});
    ctx->off_rbsrc.assign(t->highest_lvl, 0);
    ctx->lvl_gcneed.assign(t->highest_lvl, {});
    ctx->off_gcneed.assign(t->highest_lvl, 0);
    for (int l = 0; l < t->highest_lvl; l++) {
      for (int sl : ctx->lvl_ids[l]) {
        if (src[sl]) ctx->lvl_rbsrc[l].push_back(sl);
        if (src[sl] || !is_leaf[sl]) ctx->lvl_gcneed[l].push_back(sl);
      }
      ctx->off_rbsrc[l] = lists.size();
      lists.insert(lists.end(), ctx->lvl_rbsrc[l].begin(), ctx->lvl_rbsrc[l].end());
      ctx->off_gcneed[l] = lists.size();
      lists.insert(lists.end(), ctx->lvl_gcneed[l].begin(), ctx->lvl_gcneed[l].end());
    }
  }
  ctx->off_all_leaves = lists.size();
  ctx->n_all_leaves = 0;
  for (int l = 0; l < t->highest_lvl; l++) {
    lists.insert(lists.end(), ctx->lvl_leaves[l].begin(), ctx->lvl_leaves[l].end());
    ctx->n_all_leaves += (int)ctx->lvl_leaves[l].size();
  }
  // coarse grid map (level 1); a batched tree stacks the instances' coarse
  // grids (instance-major), which must be alike: same boxes at the same
  // places with the same geometry
  const long nloc = (long)ctx->cgs[0] * ctx->cgs[1] * ctx->cgs[2];
  const long ncoarse = nloc * rows;
  std::vector<int> cslot(ncoarse, -1), ccell(ncoarse, 0);
  if (nloc <= kMaxCoarse) {
    std::vector<int> first(nloc, -1);  // instance-0 box of each coarse cell
    for (int s : ctx->lvl_ids[0]) {
      const long q = n_inst > 0 ? box_inst[s] : 0;
      const int kn = D == 3 ? nc : 1;
      for (int k = 1; k <= kn; k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) {
            long I = (long)(t->ix[(size_t)s * D + 0] - 1) * nc + (i - 1);
            long J = (long)(t->ix[(size_t)s * D + 1] - 1) * nc + (j - 1);
            long K = D == 3 ? (long)(t->ix[(size_t)s * D + 2] - 1) * nc + (k - 1) : 0;
            if (I >= ctx->cgs[0] || J >= ctx->cgs[1] || K >= ctx->cgs[2])
              return fail(ctx, AFG_ERR_ARG, "level-1 box outside coarse_grid_size");
            const long gl = I + ctx->cgs[0] * (J + (long)ctx->cgs[1] * K), g = q * nloc + gl;
            if (cslot[g] >= 0) return fail(ctx, AFG_ERR_ARG, "level-1 boxes overlap");
            cslot[g] = s;
            ccell[g] = i + ctx->n2 * (j + ctx->n2 * (D == 3 ? k : 0));
            if (q == 0) first[gl] = s;
          }
    }
    if (n_inst > 0)
      for (long g = 0; g < ncoarse; g++) {
        const int s = cslot[g], s0 = first[g % nloc];
        if (s < 0 || s0 < 0) continue;
        for (int d = 0; d < D; d++)
          if (t->dr[(size_t)s * D + d] != t->dr[(size_t)s0 * D + d] ||
              t->r_min[(size_t)s * D + d] != t->r_min[(size_t)s0 * D + d])
            return fail(ctx, AFG_ERR_UNSUPPORTED, "instances need alike coarse grids (box %d)", s + 1);
      }
    for (long g = 0; g < ncoarse; g++)
      if (cslot[g] < 0) return fail(ctx, AFG_ERR_ARG, "coarse grid not covered by level-1 boxes");
  }
  // upload tables
  CK(dalloc(&ctx->d_parent, n));
  CK(dalloc(&ctx->d_children, (size_t)n * nch));
  CK(dalloc(&ctx->d_nbr, (size_t)n * nnb));
  CK(dalloc(&ctx->d_pnb, (size_t)n * nnb));
  CK(dalloc(&ctx->d_nbmat, (size_t)n * nm));
  CK(dalloc(&ctx->d_ix, (size_t)n * D));
  CK(dalloc(&ctx->d_rmin, (size_t)n * D));
  CK(dalloc(&ctx->d_dr, (size_t)n * D));
  CK(dalloc(&ctx->d_lists, lists.size()));
  CK(dalloc(&ctx->d_is_leaf, n));
  CK(dalloc(&ctx->d_cslot, ncoarse));
  CK(dalloc(&ctx->d_ccell, ncoarse));
  CK(cudaMemcpy(ctx->d_parent, parent.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_children, children.data(), sizeof(int) * children.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_nbr, nbr.data(), sizeof(int) * nbr.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_pnb, pnb.data(), sizeof(int) * pnb.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_nbmat, nbmat.data(), sizeof(int) * nbmat.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_ix, t->ix, sizeof(int) * (size_t)n * D, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_rmin, t->r_min, sizeof(double) * (size_t)n * D, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_dr, t->dr, sizeof(double) * (size_t)n * D, cudaMemcpyHostToDevice));
  {
    std::vector<double> idr((size_t)n * D);
    std::vector<float> idrf((size_t)n * D);
    for (size_t q = 0; q < idr.size(); q++) {
      idr[q] = 1.0 / t->dr[q];
      idrf[q] = (float)idr[q];
    }
    CK(dalloc(&ctx->d_idr, idr.size()));
    CK(dalloc(&ctx->d_idrf, idrf.size()));
    CK(cudaMemcpy(ctx->d_idr, idr.data(), sizeof(double) * idr.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_idrf, idrf.data(), sizeof(float) * idrf.size(), cudaMemcpyHostToDevice));
  }
  if (!lists.empty()) CK(cudaMemcpy(ctx->d_lists, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice));
  {
    // box records: a kernel walking a list gets the slot and the face
    // neighbours of its box in one 32-byte load
    std::vector<unsigned char> src(n, 0);
    for (int b = 0; b < n; b++)
      for (int nb = 0; nb < nnb; nb++)
        if (nbr[(size_t)b * nnb + nb] == kNbRefine) src[pnb[(size_t)b * nnb + nb]] = 1;
    std::vector<int> rec(std::max<size_t>(1, lists.size()) * 8, kNbPhys);
    for (size_t q = 0; q < lists.size(); q++) {
      const int sl = lists[q];
      rec[q * 8] = sl;
      for (int nb = 0; nb < nnb; nb++) rec[q * 8 + 1 + nb] = nbr[(size_t)sl * nnb + nb];
      rec[q * 8 + 7] = src[sl];  // 1: the box is a refinement-boundary source
    }
    CK(dalloc(&ctx->d_rec, rec.size()));
    CK(cudaMemcpy(ctx->d_rec, rec.data(), sizeof(int) * rec.size(), cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(ctx->d_is_leaf, is_leaf.data(), n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_cslot, cslot.data(), sizeof(int) * ncoarse, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_ccell, ccell.data(), sizeof(int) * ncoarse, cudaMemcpyHostToDevice));
  {
    // the coarse unknowns' cells in the compact FP32 layout (interior block)
    std::vector<int> crb(ncoarse);
    const int n2c = nc + 2, hn = nc / 2, sh = (D == 2 ? nc * nc : nc * nc * nc) / 2;
    for (long g = 0; g < ncoarse; g++) {
      const int x = ccell[g], i = x % n2c, r = x / n2c;
      const int j = D == 2 ? r : r % n2c, k = D == 2 ? 0 : r / n2c;
      const int row = D == 2 ? j - 1 : (k - 1) * nc + (j - 1);
      crb[g] = (((i + j + k) & 1) ? sh : 0) + row * hn + ((i - 1) >> 1);
    }
    CK(dalloc(&ctx->d_ccell_rb, ncoarse));
    CK(cudaMemcpy(ctx->d_ccell_rb, crb.data(), sizeof(int) * ncoarse, cudaMemcpyHostToDevice));
  }
  // per-instance tables: depth, finest dr (af_min_dr), cells per level
  ctx->inst_hl.assign(rows, 0);
  ctx->inst_min_dr.assign(rows, 0.0);
  ctx->inst_cells.assign(rows, std::vector<long long>(t->highest_lvl, 0));
  const long long cells_box = D == 2 ? (long long)nc * nc : (long long)nc * nc * nc;
  for (int l = 0; l < t->highest_lvl; l++)
    for (int s : ctx->lvl_ids[l]) {
      const int q = n_inst > 0 ? box_inst[s] : 0;
      ctx->inst_cells[q][l] += cells_box;
      if (l + 1 > ctx->inst_hl[q]) {
        ctx->inst_hl[q] = l + 1;
        double mdr = t->dr[(size_t)s * D];
        for (int d = 1; d < D; d++) mdr = std::min(mdr, t->dr[(size_t)s * D + d]);
        ctx->inst_min_dr[q] = mdr;
      }
    }
  for (int q = 0; q < rows; q++)
    if (ctx->inst_hl[q] == 0) return fail(ctx, AFG_ERR_ARG, "instance %d has no boxes", q);
  if (rows > ctx->max_rows) {
    dfree(ctx->d_max);
    cudaFreeHost(ctx->h_max);
    ctx->h_max = nullptr;
    CK(dalloc(&ctx->d_max, (size_t)rows * kMaxSlots));
    CK(cudaMallocHost((void**)&ctx->h_max, (size_t)rows * kMaxSlots * sizeof(unsigned long long)));
    ctx->max_rows = rows;
  }
  CK(cudaMemset(ctx->d_max, 0, (size_t)ctx->max_rows * kMaxSlots * sizeof(unsigned long long)));
  if (n_inst > 0) {
    CK(dalloc(&ctx->d_inst, n));
    CK(dalloc(&ctx->d_frozen, n_inst));
    CK(dalloc(&ctx->d_frozen_base, n_inst));
    CK(dalloc(&ctx->d_inst_hl, n_inst));
    CK(cudaMallocHost((void**)&ctx->h_frozen, sizeof(int) * n_inst));
    memset(ctx->h_frozen, 0, sizeof(int) * n_inst);
    CK(cudaMemcpy(ctx->d_inst, box_inst, sizeof(int) * n, cudaMemcpyHostToDevice));
    CK(cudaMemset(ctx->d_frozen, 0, sizeof(int) * n_inst));
    CK(cudaMemset(ctx->d_frozen_base, 0, sizeof(int) * n_inst));
    CK(cudaMemcpy(ctx->d_inst_hl, ctx->inst_hl.data(), sizeof(int) * n_inst, cudaMemcpyHostToDevice));
    ctx->n_inst = n_inst;
  }
  // cylindrical geometry table
  if (ctx->coord == AFG_CYL) {
    CK(dalloc(&ctx->d_geo, (size_t)n * nc * 4));
    k_setup_geo<<<(n * nc + 255) / 256, 256, 0, ctx->stream>>>(n, nc, ctx->d_rmin, ctx->d_dr, ctx->d_geo);
    ctx->launches++;
    CKL();
  }
  // pools
  ctx->n_var = n_var_cell;
  ctx->n_var_face = n_var_face;
  ctx->cc.assign(n_var_cell, nullptr);
  ctx->fc.assign(std::max(0, n_var_face), nullptr);
  for (int v = 0; v < n_var_cell; v++) {
    if (dalloc(&ctx->cc[v], (size_t)n * ctx->S) != cudaSuccess)
      return fail(ctx, AFG_ERR_NOMEM, "cannot allocate cell pool %d", v + 1);
    CK(cudaMemsetAsync(ctx->cc[v], 0, sizeof(double) * (size_t)n * ctx->S, ctx->stream));
  }
  for (int v = 0; v < n_var_face; v++) {
    if (dalloc(&ctx->fc[v], (size_t)n * D * ctx->NF) != cudaSuccess)
      return fail(ctx, AFG_ERR_NOMEM, "cannot allocate face pool %d", v + 1);
    CK(cudaMemsetAsync(ctx->fc[v], 0, sizeof(double) * (size_t)n * D * ctx->NF, ctx->stream));
  }
  ctx->methods.assign(n_var_cell, GcDev{});
  ctx->has_method.assign(n_var_cell, false);
  ctx->stage_elems = (size_t)n * std::max(ctx->S, D * ctx->NF);
  CK(cudaMallocHost((void**)&ctx->h_stage, sizeof(double) * ctx->stage_elems));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->gsrb_cpt[0] = ctx->gsrb_cpt[1] = 0;  // a new tree is tuned again
  ctx->have_tree = true;
  return AFG_OK;
}

static int check_var(afg_ctx* ctx, int iv) {
  if (!ctx) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree: call afg_tree_sync first");
  if (iv < 1 || iv > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad cc variable %d", iv);
  return AFG_OK;
}

/* ---- host <-> device transfers ------------------------------------------ */

// Boxes per staged chunk: the gather of chunk c+1 overlaps the DMA of chunk c.
static const size_t kXferChunkBytes = 32u << 20;

static bool is_page_locked(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// All boxes present, equally spaced by a pitch >= E elements, and the whole
// span page-locked: one pitched DMA moves every box with no host copy.
static bool pitched_boxes(int n, size_t E, const double* const* box, long long off, size_t* pitch) {
  if (n <= 0 || !box[0]) return false;
  if (n == 1) {
    *pitch = E;
  } else {
    if (!box[1] || box[1] <= box[0]) return false;
    const ptrdiff_t d = box[1] - box[0];
    if ((size_t)d < E) return false;
    for (int b = 2; b < n; b++)
      if (!box[b] || box[b] - box[b - 1] != d) return false;
    *pitch = (size_t)d;
  }
  return is_page_locked(box[0] + off) && is_page_locked(box[n - 1] + off + E - 1);
}

// Box copies between a device pool and host boxes in mapped page-locked
// memory, done by the GPU itself (loads/stores over the host link).
__global__ void __launch_bounds__(256) k_gather_pitched(double* __restrict__ dst, const double* __restrict__ src,
                                                        size_t pitch, int E, int n, int vec2) {
  for (int b = blockIdx.x; b < n; b += gridDim.x) {
    const double* s = src + (size_t)b * pitch;
    double* d = dst + (size_t)b * E;
    if (vec2) {
      const double2* s2 = reinterpret_cast<const double2*>(s);
      double2* d2 = reinterpret_cast<double2*>(d);
      for (int x = threadIdx.x; x < E / 2; x += blockDim.x) d2[x] = s2[x];
    } else {
      for (int x = threadIdx.x; x < E; x += blockDim.x) d[x] = s[x];
    }
  }
}
__global__ void __launch_bounds__(256) k_scatter_pitched(double* __restrict__ dst, const double* __restrict__ src,
                                                         size_t pitch, int E, int n, int vec2) {
  for (int b = blockIdx.x; b < n; b += gridDim.x) {
    const double* s = src + (size_t)b * E;
    double* d = dst + (size_t)b * pitch;
    if (vec2) {
      const double2* s2 = reinterpret_cast<const double2*>(s);
      double2* d2 = reinterpret_cast<double2*>(d);
      for (int x = threadIdx.x; x < E / 2; x += blockDim.x) d2[x] = s2[x];
    } else {
      for (int x = threadIdx.x; x < E; x += blockDim.x) d[x] = s[x];
    }
  }
}

// The same scatter with a small grid for copies that overlap other work: few
// blocks (the link, not the SMs, is the limit), each thread moving one
// double2 of four boxes at a time so enough bytes are in flight.
constexpr int kXferAsyncBlocks = 64;
__global__ void __launch_bounds__(256) k_scatter_pitched_narrow(double* __restrict__ dst,
                                                                const double* __restrict__ src, size_t pitch, int E,
                                                                int n) {
  const int G = gridDim.x, h = E / 2;
  for (int b0 = blockIdx.x; b0 < n; b0 += 4 * G) {
    for (int x = threadIdx.x; x < h; x += blockDim.x) {
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int b = b0 + u * G;
        if (b < n) v[u] = reinterpret_cast<const double2*>(src + (size_t)b * E)[x];
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int b = b0 + u * G;
        if (b < n) reinterpret_cast<double2*>(dst + (size_t)b * pitch)[x] = v[u];
      }
    }
  }
}

// Device address of [p, p + bytes) when the whole span lies inside one range
// page-locked by afg_host_register (mapped, so the GPU may access it);
// nullptr otherwise.
static const void* registered_span(afg_ctx* ctx, const void* p, size_t bytes) {
  const uintptr_t a = (uintptr_t)p;
  for (const auto& r : ctx->host_regs)
    if (a >= r.first && a + bytes <= r.first + r.second) {
      void* dev = nullptr;
      if (cudaHostGetDevicePointer(&dev, const_cast<void*>(p), 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      return dev;
    }
  return nullptr;
}

static int xfer_grid(int n) { return std::max(1, std::min(n, 152 * 16)); }

// Boxes 0..n-1 of a device pool with E elements per box <- host box arrays
// (null entries skipped: their device data is left as it is).
static int h2d_boxes(afg_ctx* ctx, double* dst, size_t E, const double* const* box, long long off) {
  const int n = ctx->n_boxes;
  size_t pitch = 0;
  CK(cudaStreamSynchronize(ctx->stream));
  if (pitched_boxes(n, E, box, off, &pitch)) {
    const double* first = box[0] + off;
    const void* dev = registered_span(ctx, first, sizeof(double) * ((size_t)(n - 1) * pitch + E));
    if (dev) {
      const int vec2 = ((uintptr_t)dev % 16 == 0) && pitch % 2 == 0 && E % 2 == 0;
      k_gather_pitched<<<xfer_grid(n), 256, 0, ctx->stream>>>(dst, (const double*)dev, pitch, (int)E, n, vec2);
      CK(cudaGetLastError());
    } else {
      CK(cudaMemcpy2DAsync(dst, E * sizeof(double), first, pitch * sizeof(double), E * sizeof(double), n,
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return AFG_OK;
  }
  const int per = (int)std::max<size_t>(1, kXferChunkBytes / (E * sizeof(double)));
  for (int b0 = 0; b0 < n; b0 += per) {
    const int b1 = std::min(n, b0 + per);
#pragma omp parallel for schedule(static)
    for (int b = b0; b < b1; b++)
      if (box[b]) memcpy(ctx->h_stage + (size_t)b * E, box[b] + off, sizeof(double) * E);
    int b = b0;
    while (b < b1) {
      if (!box[b]) { b++; continue; }
      int e = b;
      while (e < b1 && box[e]) e++;
      CK(cudaMemcpyAsync(dst + (size_t)b * E, ctx->h_stage + (size_t)b * E, sizeof(double) * E * (e - b),
                         cudaMemcpyHostToDevice, ctx->stream));
      b = e;
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

// Host box arrays <- boxes 0..n-1 of a device pool (null entries skipped).
static int d2h_boxes(afg_ctx* ctx, const double* src, size_t E, double* const* box, long long off) {
  const int n = ctx->n_boxes;
  size_t pitch = 0;
  if (pitched_boxes(n, E, box, off, &pitch)) {
    double* first = box[0] + off;
    const void* dev = registered_span(ctx, first, sizeof(double) * ((size_t)(n - 1) * pitch + E));
    if (dev) {
      const int vec2 = ((uintptr_t)dev % 16 == 0) && pitch % 2 == 0 && E % 2 == 0;
      k_scatter_pitched<<<xfer_grid(n), 256, 0, ctx->stream>>>((double*)dev, src, pitch, (int)E, n, vec2);
      CK(cudaGetLastError());
    } else {
      CK(cudaMemcpy2DAsync(first, pitch * sizeof(double), src, E * sizeof(double), E * sizeof(double), n,
                           cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return AFG_OK;
  }
  const int per = (int)std::max<size_t>(1, kXferChunkBytes / (E * sizeof(double)));
  const int nch = (n + per - 1) / per;
  auto issue = [&](int c) -> cudaError_t {
    const int b0 = c * per, b1 = std::min(n, b0 + per);
    cudaError_t e = cudaMemcpyAsync(ctx->h_stage + (size_t)b0 * E, src + (size_t)b0 * E,
                                    sizeof(double) * E * (b1 - b0), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return e;
    return cudaEventRecord(ctx->xfer_ev[c & 1], ctx->stream);
  };
  CK(issue(0));
  for (int c = 0; c < nch; c++) {
    if (c + 1 < nch) CK(issue(c + 1));
    CK(cudaEventSynchronize(ctx->xfer_ev[c & 1]));
    const int b0 = c * per, b1 = std::min(n, b0 + per);
#pragma omp parallel for schedule(static)
    for (int b = b0; b < b1; b++)
      if (box[b]) memcpy(box[b] + off, ctx->h_stage + (size_t)b * E, sizeof(double) * E);
  }
  return AFG_OK;
}

int afg_cc_download_async(afg_ctx* ctx, int iv, double* const* box_cc, long long off) {
  RC(check_var(ctx, iv));
  if (!box_cc) return fail(ctx, AFG_ERR_ARG, "null box_cc");
  const size_t E = ctx->S;
  const int n = ctx->n_boxes;
  size_t pitch = 0;
  if (pitched_boxes(n, E, box_cc, off, &pitch)) {
    double* first = box_cc[0] + off;
    const void* dev = registered_span(ctx, first, sizeof(double) * ((size_t)(n - 1) * pitch + E));
    if (dev) {
      // ordered after all work issued so far on the context's stream
      CK(cudaEventRecord(ctx->ev_xfer, ctx->stream));
      CK(cudaStreamWaitEvent(ctx->xfer_stream, ctx->ev_xfer, 0));
      const int vec2 = ((uintptr_t)dev % 16 == 0) && pitch % 2 == 0 && E % 2 == 0;
      if (vec2)
        k_scatter_pitched_narrow<<<kXferAsyncBlocks, 256, 0, ctx->xfer_stream>>>((double*)dev, ctx->cc[iv - 1],
                                                                                 pitch, (int)E, n);
      else
        k_scatter_pitched<<<kXferAsyncBlocks, 256, 0, ctx->xfer_stream>>>((double*)dev, ctx->cc[iv - 1], pitch,
                                                                          (int)E, n, 0);
      CK(cudaGetLastError());
      return AFG_OK;
    }
  }
  return d2h_boxes(ctx, ctx->cc[iv - 1], E, box_cc, off);
}

int afg_transfers_wait(afg_ctx* ctx) {
  if (!ctx) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->xfer_stream));
  return AFG_OK;
}

int afg_cc_upload(afg_ctx* ctx, int iv, const double* const* box_cc, long long off) {
  RC(check_var(ctx, iv));
  if (!box_cc) return fail(ctx, AFG_ERR_ARG, "null box_cc");
  return h2d_boxes(ctx, ctx->cc[iv - 1], ctx->S, box_cc, off);
}

int afg_cc_download(afg_ctx* ctx, int iv, double* const* box_cc, long long off) {
  RC(check_var(ctx, iv));
  if (!box_cc) return fail(ctx, AFG_ERR_ARG, "null box_cc");
  return d2h_boxes(ctx, ctx->cc[iv - 1], ctx->S, box_cc, off);
}

int afg_fc_upload(afg_ctx* ctx, int ivf, const double* const* box_fc, long long off) {
  if (!ctx || !ctx->have_tree) return AFG_ERR_STATE;
  if (ivf < 1 || ivf > ctx->n_var_face || !box_fc) return fail(ctx, AFG_ERR_ARG, "bad fc variable %d", ivf);
  return h2d_boxes(ctx, ctx->fc[ivf - 1], (size_t)ctx->D * ctx->NF, box_fc, off);
}

int afg_fc_download(afg_ctx* ctx, int ivf, double* const* box_fc, long long off) {
  if (!ctx || !ctx->have_tree) return AFG_ERR_STATE;
  if (ivf < 1 || ivf > ctx->n_var_face || !box_fc) return fail(ctx, AFG_ERR_ARG, "bad fc variable %d", ivf);
  return d2h_boxes(ctx, ctx->fc[ivf - 1], (size_t)ctx->D * ctx->NF, box_fc, off);
}

int afg_host_register(afg_ctx* ctx, void* ptr, size_t bytes) {
  if (!ctx || !ptr || bytes == 0) return AFG_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable));
  ctx->host_regs.emplace_back((uintptr_t)ptr, bytes);
  return AFG_OK;
}

int afg_host_unregister(afg_ctx* ctx, void* ptr) {
  if (!ctx || !ptr) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t q = 0; q < ctx->host_regs.size(); q++)
    if (ctx->host_regs[q].first == (uintptr_t)ptr) {
      ctx->host_regs.erase(ctx->host_regs.begin() + q);
      break;
    }
  CK(cudaHostUnregister(ptr));
  return AFG_OK;
}

int afg_set_cc_methods(afg_ctx* ctx, int iv, const afg_gc_desc* gc) {
  RC(check_var(ctx, iv));
  if (!gc || gc->rb < 0 || gc->rb > 2) return fail(ctx, AFG_ERR_ARG, "bad ghost-cell method");
  clear_graphs(ctx);
  GcDev g;
  for (int n = 0; n < 6; n++) {
    g.bc_type[n] = gc->bc_type[n];
    g.bc_val[n] = gc->bc_val[n];
    if (n < 2 * ctx->D && (g.bc_type[n] > -10 || g.bc_type[n] < -13))
      return fail(ctx, AFG_ERR_ARG, "bad bc type %d on face %d", g.bc_type[n], n + 1);
  }
  g.rb = gc->rb;
  ctx->methods[iv - 1] = g;
  ctx->has_method[iv - 1] = true;
  return AFG_OK;
}

int afg_gc(afg_ctx* ctx, int iv, int lvl, int corners) {
  RC(check_var(ctx, iv));
  if (!ctx->has_method[iv - 1]) return fail(ctx, AFG_ERR_STATE, "no ghost-cell methods for variable %d", iv);
  if (lvl > ctx->highest_lvl) return fail(ctx, AFG_ERR_ARG, "bad level %d", lvl);
  const GcDev& g = ctx->methods[iv - 1];
  const int l0 = lvl <= 0 ? 1 : lvl, l1 = lvl <= 0 ? ctx->highest_lvl : lvl;
  for (int l = l0; l <= l1; l++)
    RC(launch_gc<double>(ctx, lst(ctx, ctx->off_ids[l - 1]), (int)ctx->lvl_ids[l - 1].size(), ctx->cc[iv - 1], g,
                         corners));
  return AFG_OK;
}

int afg_maxabs(afg_ctx* ctx, int iv, int leaves_only, double* result) {
  RC(check_var(ctx, iv));
  if (!result) return AFG_ERR_ARG;
  RC(reset_max(ctx, 0));
  if (leaves_only)
    RC(launch_maxabs<double>(ctx, lst(ctx, ctx->off_all_leaves), ctx->n_all_leaves, ctx->cc[iv - 1], ctx->d_max));
  else
    RC(launch_maxabs<double>(ctx, lst(ctx, ctx->off_all), ctx->n_all, ctx->cc[iv - 1], ctx->d_max));
  return read_max(ctx, 0, result);
}

/* ---- multigrid ---------------------------------------------------------- */

// Dense coarse matrix with boundary conditions folded in and its inverse
// (hypre_set_matrix + stencil_handle_boundaries, m_coarse_solver.f90:104-194,
// 442-491); the inverse replaces hypre's PFMG solve.
static int build_coarse(afg_ctx* ctx, MgSlot& m) {
  const int D = ctx->D, nc = ctx->nc;
  const long n = (long)ctx->cgs[0] * ctx->cgs[1] * ctx->cgs[2];
  if (n > kMaxCoarse)
    return fail(ctx, AFG_ERR_UNSUPPORTED, "coarse grid of %ld unknowns exceeds the direct solver limit %d", n,
                kMaxCoarse);
  std::vector<double> A((size_t)n * n, 0.0), b2r((size_t)n * 2 * D, 0.0);
  std::vector<unsigned char> mask(n, 0);
  std::vector<double> dr(D), rmin(D);
  for (int s : ctx->lvl_ids[0]) {
    // batched trees: the coarse grids are alike; the first one defines it
    if (ctx->n_inst > 0 && ctx->h_inst[s] != 0) continue;
    // per-box coefficients, mg_box_lpl_stencil
    double h[3], c[7];
    std::vector<double> hdr((size_t)D), hrm((size_t)D);
    CK(cudaMemcpy(hdr.data(), ctx->d_dr + (size_t)s * D, sizeof(double) * D, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hrm.data(), ctx->d_rmin + (size_t)s * D, sizeof(double) * D, cudaMemcpyDeviceToHost));
    for (int d = 0; d < D; d++) h[d] = hdr[d];
    double inv[3];
    for (int d = 0; d < D; d++) inv[d] = 1 / (h[d] * h[d]);
    for (int d = 0; d < D; d++) c[1 + 2 * d] = c[2 + 2 * d] = inv[d];
    double sum = 0;
    for (int k = 1; k <= 2 * D; k++) sum += c[k];
    c[0] = -sum - m.d.helmholtz_lambda;
    const bool cyl = ctx->coord == AFG_CYL;
    const int kn = D == 3 ? nc : 1;
    // electrode boxes: their own variable stencil (no cylindrical factors:
    // the axisymmetric term is part of it)
    const double* vq = nullptr;
    if (m.lsf) {
      const LsfState& L = *m.lsf;
      for (size_t p = 0; p < L.lvl_all[0].size(); p++)
        if (L.lvl_all[0][p] == s) vq = L.h_v1.data() + p * (size_t)(2 * D + 1) * L.SI;
    }
    for (int k = 1; k <= kn; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          double st[7];
          for (int q = 0; q < 7; q++) st[q] = c[q];
          if (vq) {
            const int cix = (i - 1) + nc * ((j - 1) + nc * (k - 1));
            const int SI = m.lsf->SI;
            for (int q = 0; q < 7; q++) st[q] = q <= 2 * D ? vq[(size_t)q * SI + cix] : 0.0;
          } else if (cyl) {
            const double r = hrm[0] + (i - 0.5) * h[0];
            const double inv_r = 1 / r;
            const double f1 = (r - 0.5 * h[0]) * inv_r, f2 = (r + 0.5 * h[0]) * inv_r;
            st[1] = f1 * c[1];
            st[2] = f2 * c[2];
            st[0] = c[0] - (st[1] - c[1]) - (st[2] - c[2]);
          }
          const long I = (long)(ctx->h_ix[(size_t)s * D] - 1) * nc + (i - 1);
          const long J = (long)(ctx->h_ix[(size_t)s * D + 1] - 1) * nc + (j - 1);
          const long K = D == 3 ? (long)(ctx->h_ix[(size_t)s * D + 2] - 1) * nc + (k - 1) : 0;
          const long g = I + ctx->cgs[0] * (J + (long)ctx->cgs[1] * K);
          const int cidx[3] = {i, j, k};
          for (int nb = 0; nb < 2 * D; nb++) {
            if (ctx->h_nbr[(size_t)s * 2 * D + nb] >= 0) continue;
            const int d = nb / 2;
            const bool low = (nb % 2) == 0;
            if (cidx[d] != (low ? 1 : nc)) continue;
            if (m.d.bc_type[nb] == AFG_BC_DIRICHLET) {
              st[0] = st[0] - st[nb + 1];
              b2r[(size_t)g * 2 * D + nb] = -2 * st[nb + 1];
              st[nb + 1] = 0.0;
            } else if (m.d.bc_type[nb] == AFG_BC_NEUMANN) {
              st[0] = st[0] + st[nb + 1];
              b2r[(size_t)g * 2 * D + nb] = -(st[nb + 1] * h[d]) * (low ? -1 : 1);
              st[nb + 1] = 0.0;
            } else {
              return fail(ctx, AFG_ERR_UNSUPPORTED, "coarse solver supports Dirichlet/Neumann only");
            }
            mask[g] |= (unsigned char)(1u << nb);
          }
          A[(size_t)g * n + g] += st[0];
          const long G[3] = {I, J, K};
          for (int nb = 0; nb < 2 * D; nb++) {
            if (st[nb + 1] == 0.0) continue;
            long H[3] = {G[0], G[1], G[2]};
            H[nb / 2] += (nb % 2) ? 1 : -1;
            if (H[nb / 2] < 0 || H[nb / 2] >= ctx->cgs[nb / 2])
              return fail(ctx, AFG_ERR_UNSUPPORTED, "periodic coarse grids are not supported");
            const long hh = H[0] + ctx->cgs[0] * (H[1] + (long)ctx->cgs[1] * H[2]);
            A[(size_t)g * n + hh] += st[nb + 1];
          }
        }
  }
  // Gauss-Jordan with partial pivoting (same steps as the CPU oracle)
  std::vector<double> Inv((size_t)n * n, 0.0);
  for (long r = 0; r < n; r++) Inv[(size_t)r * n + r] = 1.0;
  for (long col = 0; col < n; col++) {
    long piv = col;
    double best = std::fabs(A[(size_t)col * n + col]);
    for (long r = col + 1; r < n; r++) {
      const double v = std::fabs(A[(size_t)r * n + col]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) return fail(ctx, AFG_ERR_ARG, "singular coarse-grid operator (all-Neumann Poisson?)");
    if (piv != col)
      for (long q = 0; q < n; q++) {
        std::swap(A[(size_t)col * n + q], A[(size_t)piv * n + q]);
        std::swap(Inv[(size_t)col * n + q], Inv[(size_t)piv * n + q]);
      }
    const double iv = 1.0 / A[(size_t)col * n + col];
    for (long q = 0; q < n; q++) {
      A[(size_t)col * n + q] *= iv;
      Inv[(size_t)col * n + q] *= iv;
    }
    for (long r = 0; r < n; r++) {
      if (r == col) continue;
      const double f = A[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (long q = 0; q < n; q++) {
        A[(size_t)r * n + q] -= f * A[(size_t)col * n + q];
        Inv[(size_t)r * n + q] -= f * Inv[(size_t)col * n + q];
      }
    }
  }
  m.n_coarse = (int)n;
  const int rows = inst_rows(ctx);
  CK(dalloc(&m.d_ainv, (size_t)n * n));
  CK(dalloc(&m.d_b, (size_t)n * rows));
  CK(dalloc(&m.d_x, (size_t)n * rows));
  CK(dalloc(&m.d_b2r, (size_t)n * 2 * D));
  CK(dalloc(&m.d_bmask, n));
  CK(dalloc(&m.d_bcval, (size_t)(rows + 1) * 6));
  CK(cudaMemcpy(m.d_ainv, Inv.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m.d_b2r, b2r.data(), sizeof(double) * b2r.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m.d_bmask, mask.data(), n, cudaMemcpyHostToDevice));
  std::vector<double> bcv((size_t)(rows + 1) * 6, 0.0);
  for (int r = 0; r < rows; r++)
    for (int q = 0; q < 6; q++) bcv[(size_t)r * 6 + q] = m.d.bc_val[q];
  CK(cudaMemcpy(m.d_bcval, bcv.data(), sizeof(double) * bcv.size(), cudaMemcpyHostToDevice));
  return AFG_OK;
}

static int get_mg(afg_ctx* ctx, int mg_id, MgSlot** out) {
  if (!ctx) return AFG_ERR_ARG;
  if (ctx->poisoned) return fail(ctx, AFG_ERR_CUDA, "context unusable after a failed drain of shared-memory copies");
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree");
  if (mg_id < 0 || mg_id >= kMaxMg || !ctx->mg[mg_id].used) return fail(ctx, AFG_ERR_STATE, "mg slot %d not set up", mg_id);
  *out = &ctx->mg[mg_id];
  return AFG_OK;
}

int afg_mg_setup(afg_ctx* ctx, int mg_id, const afg_mg_desc* d) {
  if (!ctx || !d) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree");
  if (mg_id < 0 || mg_id >= kMaxMg) return fail(ctx, AFG_ERR_ARG, "mg_id out of range");
  for (int v : {d->i_phi, d->i_rhs, d->i_tmp})
    if (v < 1 || v > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad mg variable %d", v);
  if (d->i_phi == d->i_rhs || d->i_phi == d->i_tmp || d->i_rhs == d->i_tmp)
    return fail(ctx, AFG_ERR_ARG, "i_phi, i_rhs and i_tmp must differ");
  if (d->n_cycle_down < 1 || d->n_cycle_up < 1) return fail(ctx, AFG_ERR_ARG, "n_cycle must be >= 1");
  if (d->precision != AFG_FP64 && d->precision != AFG_MIXED) return fail(ctx, AFG_ERR_ARG, "bad precision");
  for (int n = 0; n < 2 * ctx->D; n++)
    if (d->bc_type[n] != AFG_BC_DIRICHLET && d->bc_type[n] != AFG_BC_NEUMANN)
      return fail(ctx, AFG_ERR_UNSUPPORTED, "multigrid needs Dirichlet or Neumann sides");
  clear_graphs(ctx);
  MgSlot& m = ctx->mg[mg_id];
  dfree(m.d_ainv); dfree(m.d_b); dfree(m.d_x); dfree(m.d_b2r); dfree(m.d_bmask); dfree(m.d_bcval);
  dfree(m.e32); dfree(m.r32); dfree(m.t32);
  dfree(m.d_cb64); dfree(m.d_cb32); dfree(m.d_cy64); dfree(m.d_cy32);
  delete m.lsf;
  m.lsf = nullptr;
  m.used = false;
  m.d = *d;
  RC(build_coarse(ctx, m));
  {
    const int n = ctx->n_boxes, cyl = ctx->coord == AFG_CYL;
    const size_t ny = cyl ? (size_t)n * ctx->nc * 4 : 1;
    CK(dalloc(&m.d_cb64, (size_t)n * 8));
    CK(dalloc(&m.d_cb32, (size_t)n * 8));
    CK(dalloc(&m.d_cy64, ny));
    CK(dalloc(&m.d_cy32, ny));
    KTree t = ktree(ctx);
    if (ctx->D == 3)
      k_setup_coef<3><<<(n + 127) / 128, 128, 0, ctx->stream>>>(t, n, d->helmholtz_lambda, 0, m.d_cb64, m.d_cb32,
                                                               m.d_cy64, m.d_cy32);
    else
      k_setup_coef<2><<<(n + 127) / 128, 128, 0, ctx->stream>>>(t, n, d->helmholtz_lambda, cyl, m.d_cb64, m.d_cb32,
                                                               m.d_cy64, m.d_cy32);
    ctx->launches++;
    CKL();
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if (d->precision == AFG_MIXED) {
    // room for either FP32 layout: interior blocks plus ghost blocks
    const size_t N = (size_t)ctx->n_boxes * (ktree(ctx).SI + ctx->S);
    if (dalloc(&m.e32, N) != cudaSuccess || dalloc(&m.r32, N) != cudaSuccess || dalloc(&m.t32, N) != cudaSuccess)
      return fail(ctx, AFG_ERR_NOMEM, "cannot allocate FP32 pools");
    CK(cudaMemset(m.e32, 0, N * sizeof(float)));
    CK(cudaMemset(m.r32, 0, N * sizeof(float)));
    CK(cudaMemset(m.t32, 0, N * sizeof(float)));
    if (ctx->gsrb_cpt[ctx->rb32 ? 2 : 0] == 0) RC(autotune_gsrb(ctx, m));
  }
  m.used = true;
  // mg_init: phi gets the multigrid ghost-cell methods
  GcDev g = mg_gc(ctx, m, false);
  ctx->methods[d->i_phi - 1] = g;
  ctx->has_method[d->i_phi - 1] = true;
  return AFG_OK;
}

int afg_mg_set_bc_values(afg_ctx* ctx, int mg_id, const double* v) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!v) return AFG_ERR_ARG;
  bool same = true;
  for (int q = 0; q < 6; q++) same = same && m->d.bc_val[q] == v[q];
  if (same) return AFG_OK;
  clear_graphs(ctx);  // boundary values are kernel parameters of captured graphs
  for (int q = 0; q < 6; q++) m->d.bc_val[q] = v[q];
  const int rows = inst_rows(ctx);
  std::vector<double> bcv((size_t)rows * 6);
  for (int r = 0; r < rows; r++)
    for (int q = 0; q < 6; q++) bcv[(size_t)r * 6 + q] = v[q];
  CK(cudaMemcpyAsync(m->d_bcval, bcv.data(), sizeof(double) * bcv.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->methods[m->d.i_phi - 1] = mg_gc(ctx, *m, false);
  return AFG_OK;
}

int afg_mg_set_bc_values_inst(afg_ctx* ctx, int mg_id, const double* v) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!v) return AFG_ERR_ARG;
  if (ctx->n_inst <= 0) return afg_mg_set_bc_values(ctx, mg_id, v);
  // read by the kernels from device memory: captured graphs stay valid
  CK(cudaMemcpyAsync(m->d_bcval, v, sizeof(double) * 6 * ctx->n_inst, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

#define MG_VARS(m)                                 \
  double* phi = ctx->cc[(m)->d.i_phi - 1];         \
  double* rhs = ctx->cc[(m)->d.i_rhs - 1];         \
  double* tmp = ctx->cc[(m)->d.i_tmp - 1];

int afg_mg_gsrb_lvl(afg_ctx* ctx, int mg_id, int lvl, int type) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (lvl < 1 || lvl > ctx->highest_lvl) return fail(ctx, AFG_ERR_ARG, "bad level");
  MG_VARS(m);
  (void)tmp;
  // a call on its own: the first half sweep reads the stored ghost cells,
  // as the reference's gsrb_boxes does
  return mg_gsrb_boxes<double>(ctx, *m, lvl, type, phi, rhs, mg_gc(ctx, *m, false), true, false, true);
}

int afg_mg_update_coarse(afg_ctx* ctx, int mg_id, int lvl) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (lvl < 2 || lvl > ctx->highest_lvl) return fail(ctx, AFG_ERR_ARG, "bad level");
  MG_VARS(m);
  const GcDev g = mg_gc(ctx, *m, false);
  RC(mg_update_coarse<double>(ctx, *m, lvl, phi, rhs, tmp, g, false));
  // the reference fills the whole coarser level, leaves included
  return mg_gc_lvl<double>(ctx, lvl - 1, phi, g, 1);
}

int afg_mg_correct_lvl(afg_ctx* ctx, int mg_id, int lvl) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (lvl < 2 || lvl > ctx->highest_lvl) return fail(ctx, AFG_ERR_ARG, "bad level");
  MG_VARS(m);
  (void)rhs;
  return mg_correct<double>(ctx, lvl, phi, tmp, mg_gc(ctx, *m, false));
}

int afg_mg_coarse_solve(afg_ctx* ctx, int mg_id) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  MG_VARS(m);
  (void)tmp;
  return mg_coarse_solve<double>(ctx, *m, phi, rhs, mg_gc(ctx, *m, false), false);
}

int afg_mg_residual(afg_ctx* ctx, int mg_id, int max_lvl) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  MG_VARS(m);
  return mg_residual_lvls<double>(ctx, *m, max_lvl <= 0 ? ctx->highest_lvl : std::min(max_lvl, ctx->highest_lvl),
                                  phi, rhs, tmp, nullptr);
}

int afg_mg_vcycle(afg_ctx* ctx, int mg_id, int set_residual, int max_lvl, double* max_res) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  MG_VARS(m);
  const int ml = max_lvl <= 0 ? ctx->highest_lvl : std::min(max_lvl, ctx->highest_lvl);
  RC(run_graph(ctx, gkey("vcycle", mg_id, ml, set_residual != 0), [&]() -> int {
    RC(reset_max(ctx, 1));
    return mg_vcycle<double>(ctx, *m, ml, phi, rhs, tmp, set_residual != 0, false, ctx->d_max + 1, true);
  }));
  inst_uncount(ctx, *m, false);
  if (set_residual && max_res) return read_max(ctx, 1, max_res);
  return AFG_OK;
}

int afg_mg_fmg(afg_ctx* ctx, int mg_id, int set_residual, int have_guess, double* max_res) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  MG_VARS(m);
  RC(run_graph(ctx, gkey("fmg", mg_id, set_residual != 0, have_guess != 0), [&]() -> int {
    RC(reset_max(ctx, 1));
    if (m->d.precision == AFG_MIXED)
      return mixed_fmg(ctx, *m, phi, rhs, set_residual != 0, have_guess != 0, ctx->d_max + 1);
    return mg_fmg<double>(ctx, *m, phi, rhs, tmp, set_residual != 0, have_guess != 0, ctx->d_max + 1);
  }));
  inst_uncount(ctx, *m, true);
  if (set_residual && max_res) return read_max(ctx, 1, max_res);
  return AFG_OK;
}

int afg_mg_solve(afg_ctx* ctx, int mg_id, double threshold, int max_cycles, int* n_done, double* residuals) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (max_cycles < 1) return fail(ctx, AFG_ERR_ARG, "max_cycles < 1");
  if (ctx->n_inst > 0) {
    // the same threshold for every instance; the most iterations and the
    // largest final residual are reported
    std::vector<double> thr(ctx->n_inst, threshold), res(ctx->n_inst);
    std::vector<int> nd(ctx->n_inst);
    const int rc = mg_solve_inst(ctx, *m, thr.data(), max_cycles, nd.data(), res.data());
    if (rc != AFG_OK && rc != AFG_ERR_NOCONV) return rc;
    const int n = *std::max_element(nd.begin(), nd.end());
    if (n_done) *n_done = n;
    if (residuals && n > 0) residuals[n - 1] = *std::max_element(res.begin(), res.end());
    return rc;
  }
  if (m->d.precision == AFG_MIXED) return mixed_solve(ctx, *m, threshold, max_cycles, n_done, residuals);
  int n = 0;
  double r = 0;
  for (n = 0; n < max_cycles;) {
    RC(vcycle_graph(ctx, *m, n == 0));
    RC(read_max(ctx, 1, &r));
    if (residuals) residuals[n] = r;
    n++;
    if (r < threshold) break;
  }
  if (n_done) *n_done = n;
  return r < threshold ? AFG_OK : AFG_ERR_NOCONV;
}

}  // extern "C"

extern "C" {

int afg_mg_solve_inst(afg_ctx* ctx, int mg_id, const double* threshold, int max_cycles, int* n_done,
                      double* residual) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (ctx->n_inst <= 0) return fail(ctx, AFG_ERR_STATE, "not a batched tree");
  if (max_cycles < 1 || !threshold) return fail(ctx, AFG_ERR_ARG, "bad solve arguments");
  return mg_solve_inst(ctx, *m, threshold, max_cycles, n_done, residual);
}

int afg_n_instances(const afg_ctx* ctx) { return ctx ? ctx->n_inst : 0; }

int afg_set_photoi_lockstep(afg_ctx* ctx, int on) {
  if (!ctx) return AFG_ERR_ARG;
  ctx->photoi_lockstep = on != 0;
  return AFG_OK;
}

int afg_tree_copy_cc(afg_ctx* ctx, int iv_from, int iv_to) {
  RC(check_var(ctx, iv_from));
  RC(check_var(ctx, iv_to));
  // every box of the tree: one copy of the whole pool (slots of boxes not in
  // use hold no data anyone reads)
  if (iv_from == iv_to) return AFG_OK;
  KtScope kts(ctx, AFG_KT_COPY, 16.0 * (size_t)ctx->n_boxes * ctx->S);
  CK(cudaMemcpyAsync(ctx->cc[iv_to - 1], ctx->cc[iv_from - 1], sizeof(double) * (size_t)ctx->n_boxes * ctx->S,
                     cudaMemcpyDeviceToDevice, ctx->stream));
  return AFG_OK;
}

int afg_autotune(afg_ctx* ctx, int mg_id) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (m->d.precision != AFG_MIXED) return fail(ctx, AFG_ERR_ARG, "autotuning needs a mixed-precision slot (scratch)");
  clear_graphs(ctx);
  return autotune_gsrb(ctx, *m);
}

int afg_set_tuning(afg_ctx* ctx, const int* in) {
  if (!ctx || !in) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree");
  const int S = kGsrbTma, R = kGsrbTma | kGsrbTmaRhs;
  const int ok3[] = {0, 1, 2, 4, 8, S | 2, S | 4, R | 2, R | 4}, ok2[] = {0, 1, 2, 4, S | 1, S | 2, R | 1, R | 2};
  for (int k = ctx->rb32 ? 1 : 0; k < 2; k++) {
    bool ok = false;
    for (int v : (ctx->D == 3 ? std::vector<int>(ok3, ok3 + 9) : std::vector<int>(ok2, ok2 + 8))) ok = ok || in[k] == v;
    if (!ok) return fail(ctx, AFG_ERR_ARG, "bad smoother variant %d", in[k]);
  }
  clear_graphs(ctx);  // launch shapes are part of captured graphs
  if (ctx->rb32) {
    const int T = kGsrbTma;
    if (in[0] != 0 && in[0] != (T | 1) && in[0] != (T | 2) && in[0] != (T | 4))
      return fail(ctx, AFG_ERR_ARG, "bad compact-layout smoother variant %d", in[0]);
    ctx->gsrb_cpt[2] = in[0] == 0 ? -1 : in[0];  // -1: the one-box-per-CTA kernel, kept by the autotuner
  } else {
    ctx->gsrb_cpt[0] = in[0];
  }
  ctx->gsrb_cpt[1] = in[1];
  return AFG_OK;
}

int afg_set_fp32_layout(afg_ctx* ctx, int compact) {
  if (!ctx) return AFG_ERR_ARG;
  clear_graphs(ctx);
  ctx->rb32 = compact != 0;
  return AFG_OK;
}

int afg_tuning(const afg_ctx* ctx, int* out) {
  if (!ctx || !out) return AFG_ERR_ARG;
  const bool sp = gsrb_rec_specialized(ctx);
  out[0] = sp ? (ctx->rb32 ? std::max(0, ctx->gsrb_cpt[2]) : gsrb_cpt_of<float>(ctx)) : 0;
  out[1] = sp ? gsrb_cpt_of<double>(ctx) : 0;
  return AFG_OK;
}

int afg_counters(const afg_ctx* ctx, long long* out) {
  if (!ctx || !out) return AFG_ERR_ARG;
  out[0] = ctx->launches;
  for (int q = 1; q < 4; q++) out[q] = ctx->ctr[q];
  return AFG_OK;
}

int afg_event_record(afg_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 64) return AFG_ERR_ARG;
  if (!ctx->ev[slot]) CK(cudaEventCreate(&ctx->ev[slot]));
  CK(cudaEventRecord(ctx->ev[slot], ctx->stream));
  return AFG_OK;
}

int afg_event_elapsed(afg_ctx* ctx, int a, int b, float* ms) {
  if (!ctx || a < 0 || b < 0 || a >= 64 || b >= 64 || !ms || !ctx->ev[a] || !ctx->ev[b]) return AFG_ERR_ARG;
  CK(cudaEventSynchronize(ctx->ev[b]));
  CK(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
  return AFG_OK;
}

int afg_flush_l2(afg_ctx* ctx, long long bytes) {
  if (!ctx || bytes <= 0) return AFG_ERR_ARG;
  if ((size_t)bytes > ctx->flush_bytes) {
    if (ctx->flush_buf) cudaFree(ctx->flush_buf);
    ctx->flush_buf = nullptr;
    CK(cudaMalloc(&ctx->flush_buf, (size_t)bytes));
    ctx->flush_bytes = (size_t)bytes;
  }
  CK(cudaMemsetAsync(ctx->flush_buf, (int)(ctx->launches & 0xff), (size_t)bytes, ctx->stream));
  return AFG_OK;
}

int afg_kernel_timing(afg_ctx* ctx, int cls) {
  if (!ctx || cls < 0 || (cls >= AFG_KT_NCLASS && cls != AFG_KT_ALL)) return AFG_ERR_ARG;
  ctx->kt_class = cls;
  ctx->kt_used = 0;
  ctx->kt_bytes = 0;
  ctx->kt_cls.clear();
  ctx->kt_pbytes.clear();
  return AFG_OK;
}

int afg_kernel_stats_all(afg_ctx* ctx, long long* launches, double* ms, double* bytes) {
  if (!ctx || !launches || !ms || !bytes) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < AFG_KT_NCLASS; c++) {
    launches[c] = 0;
    ms[c] = 0;
    bytes[c] = 0;
  }
  for (size_t q = 0; q + 1 < ctx->kt_used; q += 2) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, ctx->kt_ev[q], ctx->kt_ev[q + 1]));
    const int c = ctx->kt_cls[q / 2];
    launches[c]++;
    ms[c] += t;
    bytes[c] += ctx->kt_pbytes[q / 2];
  }
  ctx->kt_used = 0;
  ctx->kt_bytes = 0;
  ctx->kt_cls.clear();
  ctx->kt_pbytes.clear();
  return AFG_OK;
}

int afg_kernel_stats(afg_ctx* ctx, long long* launches, double* ms, double* bytes) {
  if (!ctx) return AFG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  double tot = 0;
  for (size_t q = 0; q + 1 < ctx->kt_used; q += 2) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, ctx->kt_ev[q], ctx->kt_ev[q + 1]));
    tot += t;
  }
  if (launches) *launches = (long long)(ctx->kt_used / 2);
  if (ms) *ms = tot;
  if (bytes) *bytes = ctx->kt_bytes;
  ctx->kt_used = 0;
  ctx->kt_bytes = 0;
  ctx->kt_cls.clear();
  ctx->kt_pbytes.clear();
  return AFG_OK;
}

}  // extern "C"

#include "afg_transport_api.cuh"
#include "afg_amr.cuh"
#include "afg_output.cuh"
#include "afg_lsf_api.cuh"
