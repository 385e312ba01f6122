// afg_common.cuh -- device data model shared by all kernels of the afivo hot
// path on sm_103a.
//
// HBM layout: one pool per cell-centred variable, box-major:
//   pool[slot][(nc+2)^D], slot = box id - 1, cell (i,j[,k]) at
//   i + (nc+2)*(j + (nc+2)*k), i.e. exactly the per-box, per-variable block of
//   the reference's box%cc(0:nc+1, ..., iv) (afivo/src/m_af_types.f90:302).
// Face-centred variables: pool[slot][dim][(nc+1)^D] (box%fc, 303).
// Box tables are int arrays indexed by slot with neighbour/child/parent ids
// converted to slots (negative = none, see KTree).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace afg {

constexpr int kNbPhys = -2;   // physical boundary (af_phys_boundary)
constexpr int kNbRefine = -1; // refinement boundary (af_no_box)

// Device view of the tree tables, passed to kernels by value.
struct KTree {
  int D, nc, n2, S, NF;
  int SI;         // interior cells per box, nc^D
  long long nbox; // boxes in the pools (compact FP32 buffers: ghost blocks follow nbox interior blocks)
  const int* parent;    // [n] parent slot or -1
  const int* children;  // [n][2^D] child slot or -1
  const int* nbr;       // [n][2D] neighbour slot, kNbRefine or kNbPhys
  const int* pnb;       // [n][2D] slot of parent's neighbour (refinement faces)
  const int* nbmat;     // [n][3^D] same-level box at each offset (or -1)
  const int* ix;        // [n][D]  box%ix (1-based)
  const double* r_min;  // [n][D]
  const double* dr;     // [n][D]
  // cylindrical geometry per (box, radial index i=1..nc), 2D only:
  // [n][nc][4] = flux factors (r -/+ dr/2)/r (af_cyl_flux_factors,
  // m_af_types.f90:1199-1211) and child weights 1 -/+ dr/(4r)
  // (af_cyl_child_weights, 1187-1196); null for Cartesian trees
  const double* geo;
  // 1/dr per box and dimension, computed on the host ([n][D]); a correctly
  // rounded division, so identical to 1 / dr evaluated on the device
  const double* idr;
  const float* idrf;  // the same rounded to FP32
  // Batched independent instances (null for a single tree): instance of
  // each slot, and per instance a flag that freezes it (set for instances
  // whose solve has converged while others continue): kernels of the solve
  // loops leave the boxes of a frozen instance untouched.
  const int* inst;
  const int* frozen;
  // electrode boxes of the solve in progress (index of the box's electrode
  // data or -1; null without an electrode): the kernels of ordinary boxes
  // skip them, the electrode kernels (afg_lsf.cuh) process them
  const int* lsf;
};

// maxima slots per instance in the device maxima array ([instance][slot])
constexpr int kMaxSlotsDev = 24;

// an electrode box of the solve in progress (handled by afg_lsf.cuh)
__device__ __forceinline__ bool lsf_box(const KTree& t, int slot) { return t.lsf != nullptr && t.lsf[slot] >= 0; }

__device__ __forceinline__ bool box_frozen(const KTree& t, int slot) {
  return t.frozen != nullptr && t.frozen[t.inst[slot]] != 0;
}
// the maxima word of the box's instance (batched trees) or the word itself
__device__ __forceinline__ unsigned long long* inst_max(const KTree& t, unsigned long long* m, int slot) {
  return t.inst != nullptr ? m + (size_t)t.inst[slot] * kMaxSlotsDev : m;
}

// Box records: per entry of a box list, {slot, neighbour slot of faces
// 0..2D-1, ..., source flag} in 8 ints, read as two int4 (one 32-byte load);
// the last int is 1 when a refinement-boundary rule of a finer box reads the
// box's face ghosts.
__device__ __forceinline__ void load_rec(const int* __restrict__ rec, int e, int4& r0, int4& r1) {
  r0 = reinterpret_cast<const int4*>(rec)[2 * e];
  r1 = reinterpret_cast<const int4*>(rec)[2 * e + 1];
}
// neighbour slot of face nb from a record (selects, no local memory)
__device__ __forceinline__ int rec_nb(const int4& r0, const int4& r1, int nb) {
  return nb == 0 ? r0.y : nb == 1 ? r0.z : nb == 2 ? r0.w : nb == 3 ? r1.x : nb == 4 ? r1.y : r1.z;
}

// Box size as a compile-time constant: kernels carry a template parameter NC
// (0 = take the sizes from the tree) and start with t = fix_dims<D, NC>(t0).
// With NC > 0 the sizes are constants, so the index arithmetic (divisions by
// nc and nc + 2 in the flat cell and face loops) compiles to shifts and
// multiplications.
template <int D, int NC>
__device__ __forceinline__ KTree fix_dims(KTree t) {
  if (NC > 0) {
    t.nc = NC;
    t.n2 = NC + 2;
    t.S = D == 2 ? (NC + 2) * (NC + 2) : (NC + 2) * (NC + 2) * (NC + 2);
    t.NF = D == 2 ? (NC + 1) * (NC + 1) : (NC + 1) * (NC + 1) * (NC + 1);
    t.SI = D == 2 ? NC * NC : NC * NC * NC;
  }
  return t;
}

// Launch-site dispatch on the box size: 8^3-cell boxes in 3D and 16^2-cell
// boxes in 2D (the usual afivo-streamer sizes) get their own instantiation,
// other sizes the generic one.  `ctx` must be in scope.
#define AFG_NC3(NCV, ...)         \
  do {                            \
    if (ctx->nc == 8) {           \
      constexpr int NCV = 8;      \
      __VA_ARGS__;                \
    } else {                      \
      constexpr int NCV = 0;      \
      __VA_ARGS__;                \
    }                             \
  } while (0)
#define AFG_NC2(NCV, ...)         \
  do {                            \
    if (ctx->nc == 16) {          \
      constexpr int NCV = 16;     \
      __VA_ARGS__;                \
    } else {                      \
      constexpr int NCV = 0;      \
      __VA_ARGS__;                \
    }                             \
  } while (0)

// Double <-> float conversions by IEEE-754 bit manipulation, for the FP32
// arithmetic of the mixed-precision kernels: integer instructions only, so
// the conversions do not queue on the FP64 pipe.  d2f truncates the mantissa
// toward zero (error below one FP32 ulp) and returns signed zero for
// magnitudes below the FP32 normal range and signed infinity above it (NaN
// stays NaN); f2d is exact for normal numbers, zero, infinity and NaN and
// flushes FP32 subnormals to signed zero.
__device__ __forceinline__ float d2f(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned ah = hi & 0x7FFFFFFFu;
  // normal range (biased FP64 exponent 897..1150): the FP32 exponent and the
  // top 23 mantissa bits are the high word less the bias difference, shifted
  // left by 3 with the low word's top 3 bits
  unsigned r = __funnelshift_l(lo, ah - (896u << 20), 3);
  if (ah < (897u << 20)) r = 0u;  // below the FP32 normal range
  if (ah >= (1151u << 20)) {      // above it, infinity or NaN
    const bool nan = ah > 0x7FF00000u || (ah == 0x7FF00000u && lo != 0u);
    r = 0x7F800000u | (nan ? 0x400000u : 0u);
  }
  return __uint_as_float(r | (hi & 0x80000000u));
}
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned mant = u & 0x7FFFFFu;
  unsigned hi, lo;
  if (e == 0u) {
    hi = sign;
    lo = 0u;
  } else if (e == 0xFFu) {
    hi = sign | 0x7FF00000u | (mant >> 3);
    lo = mant << 29;
  } else {
    hi = sign | ((e + 896u) << 20) | (mant >> 3);
    lo = mant << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// Operator coefficients of one multigrid slot, precomputed per box:
// cb[n][8] = c(1..2D+1) of mg_box_lpl_stencil and 1/c(1); for cylindrical
// trees cy[n][nc][4] = corrected c(1), c(2), c(3) and 1/c(1) per radial index.
template <typename T>
struct MgCoef {
  const T* cb;
  const T* cy;
};

// Several multigrid problems on the same tree advanced in lockstep (the
// Helmholtz modes of photoionization as multiple right-hand sides): a launch
// carries one pointer per problem and blockIdx.y selects it.  A single
// pointer converts to an argument holding it in every element (one problem,
// or a buffer all problems share).  The element is picked by selects on
// constant indices, so the parameter array is never indexed dynamically (no
// local-memory copy).
constexpr int kMaxModes = 8;
template <typename T>
struct ModeArg {
  T* p[kMaxModes] = {};
  ModeArg() = default;
  __host__ __device__ ModeArg(T* q) {  // the same pointer for every problem
    for (int k = 0; k < kMaxModes; k++) p[k] = q;
  }
  template <typename U>  // the same pointers with added const
  __host__ __device__ ModeArg(const ModeArg<U>& o) {
    for (int k = 0; k < kMaxModes; k++) p[k] = o.p[k];
  }
  __device__ __forceinline__ T* get() const {
    const unsigned y = blockIdx.y;
    T* r = p[0];
#pragma unroll
    for (unsigned k = 1; k < kMaxModes; k++)
      if (y == k) r = p[k];
    return r;
  }
};
template <typename T>
struct ModeCoef {
  const T* cb[kMaxModes] = {};
  const T* cy[kMaxModes] = {};
  ModeCoef() = default;
  __host__ __device__ ModeCoef(MgCoef<T> q) {  // the same tables for every problem
    for (int k = 0; k < kMaxModes; k++) {
      cb[k] = q.cb;
      cy[k] = q.cy;
    }
  }
  __device__ __forceinline__ MgCoef<T> get() const {
    const unsigned y = blockIdx.y;
    MgCoef<T> r{cb[0], cy[0]};
#pragma unroll
    for (unsigned k = 1; k < kMaxModes; k++)
      if (y == k) r = MgCoef<T>{cb[k], cy[k]};
    return r;
  }
};

// Ghost-cell method of one variable (bc per domain face + refinement rule).
struct GcDev {
  int bc_type[6];
  double bc_val[6];
  int rb;
  // batched trees: boundary values per instance [instance][6] in device
  // memory, replacing bc_val (null: bc_val holds them)
  const double* ival = nullptr;
};

// bc_type[nb] / bc_val[nb] of a ghost-cell method for a run-time face index,
// through selects so that the kernel parameter is not copied to local memory
__device__ __forceinline__ int gc_type(const GcDev& g, int nb) {
  int r = g.bc_type[0];
#pragma unroll
  for (int k = 1; k < 6; k++)
    if (nb == k) r = g.bc_type[k];
  return r;
}
__device__ __forceinline__ double gc_val(const GcDev& g, int nb) {
  double r = g.bc_val[0];
#pragma unroll
  for (int k = 1; k < 6; k++)
    if (nb == k) r = g.bc_val[k];
  return r;
}
// boundary value of face nb for box `slot` (its instance's on batched trees)
__device__ __forceinline__ double gc_val(const GcDev& g, int nb, const KTree& t, int slot) {
  return g.ival != nullptr ? g.ival[t.inst[slot] * 6 + nb] : gc_val(g, nb);
}

__device__ __forceinline__ int at2(int n2, int i, int j) { return i + n2 * j; }
__device__ __forceinline__ int at3(int n2, int i, int j, int k) { return i + n2 * (j + n2 * k); }

// cell with normal dimension d at normal index x, tangential indices p (the
// lower remaining dimension) and q (the higher one)
template <int D>
__device__ __forceinline__ int face_at(int n2, int d, int x, int p, int q) {
  if (D == 2) return d == 0 ? at2(n2, x, p) : at2(n2, p, x);
  if (d == 0) return at3(n2, x, p, q);
  if (d == 1) return at3(n2, p, x, q);
  return at3(n2, p, q, x);
}

__device__ __forceinline__ int child_offset(const KTree& t, int slot, int d) {
  return ((t.ix[slot * t.D + d] - 1) & 1) * (t.nc / 2);
}

// Non-negative doubles order like their bit patterns: max via atomicMax.
// mx = max(mx, |v|) for non-NaN values; for doubles the magnitudes are
// compared as integers (the IEEE-754 order of non-negative numbers), which
// keeps the comparison off the FP64 pipe and returns the same value.
__device__ __forceinline__ void acc_absmax(double& mx, double v) {
  const long long b = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFll;
  const long long m = __double_as_longlong(mx);
  mx = __longlong_as_double(b > m ? b : m);
}
// FP32: the same maximum, a NaN kept once seen (fmaxf would drop it)
__device__ __forceinline__ void acc_absmax(float& mx, float v) {
  const float a = fabsf(v);
  mx = (mx != mx || mx > a) ? mx : a;
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// CTA-wide maximum of non-negative values; a NaN of any thread is the
// result (a diverged residual must not read as converged)
template <typename T>
__device__ __forceinline__ T nan_max(T v, T w) {
  return (v != v || v > w) ? v : w;
}
template <typename T>
__device__ __forceinline__ T block_max(T v, T* sbuf) {
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = nan_max(v, w);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sbuf[warp] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (warp == 0) {
    v = lane < nw ? sbuf[lane] : T(0);
    for (int o = 16; o > 0; o >>= 1) {
      T w = __shfl_xor_sync(0xffffffffu, v, o);
      v = nan_max(v, w);
    }
  }
  return v;  // valid in thread 0
}

}  // namespace afg
