// Output writers on the device-resident state (afivo/src/m_af_output.f90):
// the device gathers the leaf cells and generates the mesh (af_write_vtk),
// or locates and interpolates points (af_interp1 for af_write_line,
// af_write_plane, af_write_numpy); the host only streams bytes into files
// (afg_output_host.cpp).  Large outputs go through the host in chunks of
// leaf boxes: a kernel fills one of two device buffers while the previous
// chunk's page-locked copy is written out.
//
// Included by afg_runtime.cu after the context definition.
#pragma once

#include "afg_output_host.h"

namespace {

constexpr int kMaxOutVars = 64;
struct OutPools {
  const double* p[kMaxOutVars];
};

// cells of one variable of leaf boxes g0 .. g0+gridDim.x-1 (list order),
// i fastest within a box: cc_vars of af_write_vtk (m_af_output.f90:659-718)
template <int D>
__global__ void k_out_cells(KTree t, const int* __restrict__ leaves, long long g0, const double* __restrict__ pool,
                            double* __restrict__ out) {
  const int nc = t.nc, n2 = t.n2;
  const int cpb = D == 2 ? nc * nc : nc * nc * nc;
  const int slot = leaves[g0 + blockIdx.x];
  const double* src = pool + (size_t)slot * t.S;
  double* dst = out + (size_t)blockIdx.x * cpb;
  for (int c = threadIdx.x; c < cpb; c += blockDim.x) {
    const int i = c % nc, j = (c / nc) % nc, k = D == 3 ? c / (nc * nc) : 0;
    const size_t idx = (size_t)(i + 1) + (size_t)(j + 1) * n2 + (D == 3 ? (size_t)(k + 1) * n2 * n2 : 0);
    dst[c] = src[idx];
  }
}

// box nodes r_min + (i-1) dr, i = 1..nc+1 per dimension (i fastest), as 3
// Float32 components (zero z in 2D): coords of af_write_vtk and the
// single-precision copy of vtk_unstr_geo_xml (m_vtk.f90:66-88)
template <int D>
__global__ void k_out_points(KTree t, const int* __restrict__ leaves, long long g0, float* __restrict__ out) {
  const int bn = t.nc + 1;
  const int npb = D == 2 ? bn * bn : bn * bn * bn;
  const int slot = leaves[g0 + blockIdx.x];
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  float* dst = out + (size_t)blockIdx.x * npb * 3;
  for (int n = threadIdx.x; n < npb; n += blockDim.x) {
    const int i = n % bn, j = (n / bn) % bn, k = D == 3 ? n / (bn * bn) : 0;
    dst[3 * n + 0] = (float)(rm[0] + (double)i * dr[0]);
    dst[3 * n + 1] = (float)(rm[1] + (double)j * dr[1]);
    dst[3 * n + 2] = D == 3 ? (float)(rm[D == 3 ? 2 : 0] + (double)k * dr[D == 3 ? 2 : 0]) : 0.0f;
  }
}

// connectivity of the cells of leaf boxes g0..: the pixel / voxel corner
// nodes of each cell (0-based node numbers of the whole file)
template <int D>
__global__ void k_out_connect(int nc, long long g0, int* __restrict__ out) {
  const int bn = nc + 1, bn2 = bn * bn;
  const int cpb = D == 2 ? nc * nc : nc * nc * nc;
  const int npb = D == 2 ? bn2 : bn2 * bn;
  const long long node0 = (g0 + blockIdx.x) * (long long)npb;
  int* dst = out + (size_t)blockIdx.x * cpb * (1 << D);
  for (int c = threadIdx.x; c < cpb; c += blockDim.x) {
    const int i = c % nc, j = (c / nc) % nc, k = D == 3 ? c / (nc * nc) : 0;
    const int n = (int)(node0 + (long long)k * bn2 + j * bn + i);
    int* o = dst + (size_t)c * (1 << D);
    o[0] = n;
    o[1] = n + 1;
    o[2] = n + bn;
    o[3] = n + bn + 1;
    if (D == 3) {
      o[4] = n + bn2;
      o[5] = n + bn2 + 1;
      o[6] = n + bn2 + bn;
      o[7] = n + bn2 + bn + 1;
    }
  }
}

// offsets (2^D times the 1-based cell number) or types (8 pixel, 11 voxel)
// of the cells c0 .. c0+n-1
template <int D>
__global__ void k_out_cellint(long long c0, long long n, int types, int* __restrict__ out) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
    out[c] = types ? (D == 2 ? 8 : 11) : (int)((c0 + c + 1) * (1 << D));
}

// Points where af_interp1 evaluates: an explicit list r[p][D], or the cell
// centres of a uniform grid, r = r_min + (i - 0.5) dr with i = 1..nx per
// dimension, i fastest (af_write_numpy, m_af_output.f90:842-869)
struct OutGrid {
  double rmin[3], dr[3];
  long long nx[3];
};

// af_get_id_at without a guess (m_af_utils.f90:266-313): the first level-1
// box (list order) that contains r (af_r_inside, bounds inclusive,
// m_af_utils.f90:248-261), then the child that contains r
// (child_that_contains, 340-356) while the box has children.  -1 if none.
template <int D>
__device__ int out_locate(const KTree& t, const int* __restrict__ lvl1, int n1, const double* r) {
  const int nch = 1 << D;
  int s = -1;
  for (int q = 0; q < n1 && s < 0; q++) {
    const int b = lvl1[q];
    bool in = true;
    for (int d = 0; d < D; d++) {
      const double lo = t.r_min[(size_t)b * D + d];
      const double hi = lo + t.dr[(size_t)b * D + d] * (double)t.nc;
      in = in && r[d] >= lo && r[d] <= hi;
    }
    if (in) s = b;
  }
  if (s < 0) return -1;
  while (t.children[(size_t)s * nch] >= 0) {
    int ch = 0;
    for (int d = 0; d < D; d++) {
      const double c = t.r_min[(size_t)s * D + d] + t.dr[(size_t)s * D + d] * (double)(t.nc >> 1);
      if (r[d] > c) ch += 1 << d;
    }
    s = t.children[(size_t)s * nch + ch];
  }
  return s;
}

// af_interp1 (afivo/src/m_af_interp.f90:43-105): multilinear interpolation
// between the cell centres around r in the finest box containing r (ghost
// cells included); vals[p][v], ok[p] = 0 and zero values outside the tree.
// With gvar >= 0 only variable gvar is evaluated and stored at vals[p]
// (one variable of a uniform grid at a time).
template <int D>
__global__ void k_interp1(KTree t, const int* __restrict__ lvl1, int n1, long long n_pts, long long p0,
                          const double* __restrict__ rlist, OutGrid grid, int n_iv, OutPools pools, int gvar,
                          double* __restrict__ vals, int* __restrict__ ok) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n_pts) return;
  const long long p = p0 + q;
  double r[3] = {0, 0, 0};
  if (rlist) {
    for (int d = 0; d < D; d++) r[d] = rlist[(size_t)p * D + d];
  } else {
    long long rem = p;
    for (int d = 0; d < D; d++) {
      const long long i = rem % grid.nx[d] + 1;
      rem /= grid.nx[d];
      r[d] = grid.rmin[d] + ((double)i - 0.5) * grid.dr[d];
    }
  }
  const int s = out_locate<D>(t, lvl1, n1, r);
  const int v0 = gvar >= 0 ? gvar : 0, v1 = gvar >= 0 ? gvar + 1 : n_iv;
  double* o = gvar >= 0 ? vals + q : vals + (size_t)q * n_iv;
  if (ok) ok[q] = s >= 0;
  if (s < 0) {
    for (int v = v0; v < v1; v++) o[v - v0] = 0.0;
    return;
  }
  int ix[3] = {0, 0, 0};
  double dv[3] = {0, 0, 0}, ov[3] = {1, 1, 1};
  for (int d = 0; d < D; d++) {
    const double rm = t.r_min[(size_t)s * D + d], dr = t.dr[(size_t)s * D + d];
    ix[d] = (int)round((r[d] - rm) / dr);  // nint: halves away from zero
    const double rloc = rm + ((double)ix[d] - 0.5) * dr;
    dv[d] = (r[d] - rloc) / dr;
    ov[d] = 1.0 - dv[d];
  }
  // weights in the order of the Fortran array w(1:2, 1:2[, 1:2])
  double w[8];
  if (D == 2) {
    w[0] = ov[0] * ov[1];
    w[1] = dv[0] * ov[1];
    w[2] = ov[0] * dv[1];
    w[3] = dv[0] * dv[1];
  } else {
    w[0] = ov[0] * ov[1] * ov[2];
    w[1] = dv[0] * ov[1] * ov[2];
    w[2] = ov[0] * dv[1] * ov[2];
    w[3] = dv[0] * dv[1] * ov[2];
    w[4] = ov[0] * ov[1] * dv[2];
    w[5] = dv[0] * ov[1] * dv[2];
    w[6] = ov[0] * dv[1] * dv[2];
    w[7] = dv[0] * dv[1] * dv[2];
  }
  const int n2 = t.n2;
  const size_t base = (size_t)s * t.S + ix[0] + (size_t)ix[1] * n2 + (D == 3 ? (size_t)ix[2] * n2 * n2 : 0);
  for (int v = v0; v < v1; v++) {
    const double* c = pools.p[v] + base;
    // sum(w * cc(ix:ix+1, ...)) accumulated in array element order from 0
    double acc = 0.0;
    for (int e = 0; e < (1 << D); e++) {
      const size_t off = (e & 1) + ((e >> 1) & 1) * (size_t)n2 + (D == 3 ? ((e >> 2) & 1) * (size_t)n2 * n2 : 0);
      acc = acc + w[e] * c[off];
    }
    o[v - v0] = acc;
  }
}

// number of zero flags among ok[0..n-1], added to *count
__global__ void k_count_zero(const int* __restrict__ ok, long long n, unsigned* count) {
  unsigned z = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z += ok[i] == 0;
  if (z) atomicAdd(count, z);
}

// Two device buffers and two page-locked host buffers for chunked output
struct OutStream {
  afg_ctx* ctx = nullptr;
  void* d[2] = {nullptr, nullptr};
  void* h[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  size_t cap = 0;
  ~OutStream() {
    for (int k = 0; k < 2; k++) {
      if (d[k]) cudaFree(d[k]);
      if (h[k]) cudaFreeHost(h[k]);
      if (ev[k]) cudaEventDestroy(ev[k]);
    }
  }
  cudaError_t init(afg_ctx* c, size_t bytes) {
    ctx = c;
    cap = bytes;
    for (int k = 0; k < 2; k++) {
      cudaError_t e = cudaMalloc(&d[k], bytes);
      if (e == cudaSuccess) e = cudaHostAlloc(&h[k], bytes, cudaHostAllocDefault);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
};

constexpr size_t kOutChunkBytes = 64ull << 20;

// Streams one array of n_items items of item_bytes bytes through the two
// buffers: fill(i0, n, dbuf) launches the kernels producing items
// i0..i0+n-1 into dbuf; put(hbuf, bytes) consumes the host copy in order.
template <typename Fill, typename Put>
static int out_stream(OutStream& st, long long n_items, size_t item_bytes, Fill fill, Put put) {
  afg_ctx* ctx = st.ctx;
  const long long per = std::max<long long>(1, (long long)(st.cap / item_bytes));
  long long prev_n = 0;
  int k = 0;
  for (long long i0 = 0; i0 < n_items; i0 += per, k ^= 1) {
    const long long n = std::min(per, n_items - i0);
    fill(i0, n, st.d[k]);
    ctx->launches++;
    CKL();
    CK(cudaMemcpyAsync(st.h[k], st.d[k], (size_t)n * item_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(st.ev[k], ctx->stream));
    if (prev_n > 0) {
      CK(cudaEventSynchronize(st.ev[k ^ 1]));
      if (!put(st.h[k ^ 1], (size_t)prev_n * item_bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
    }
    prev_n = n;
  }
  if (prev_n > 0) {
    CK(cudaEventSynchronize(st.ev[k ^ 1]));
    if (!put(st.h[k ^ 1], (size_t)prev_n * item_bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
  }
  return AFG_OK;
}

static int check_out_vars(afg_ctx* ctx, int n_iv, const int* ivs, const char* const* names) {
  if (!ctx) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree: call afg_tree_sync first");
  if (n_iv < 0 || n_iv > kMaxOutVars || (n_iv > 0 && !ivs))
    return fail(ctx, AFG_ERR_ARG, "bad variable list (at most %d variables)", kMaxOutVars);
  for (int v = 0; v < n_iv; v++) {
    if (ivs[v] < 1 || ivs[v] > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "wrong indices given: %d", ivs[v]);
    if (names && !names[v]) return fail(ctx, AFG_ERR_ARG, "missing name of variable %d", ivs[v]);
  }
  return AFG_OK;
}

static OutPools out_pools(afg_ctx* ctx, int n_iv, const int* ivs) {
  OutPools p{};
  for (int v = 0; v < n_iv; v++) p.p[v] = ctx->cc[ivs[v] - 1];
  return p;
}

// af_interp1 at n points: explicit r (host array) or a uniform grid, into
// host vals/ok
static int out_interp(afg_ctx* ctx, long long n, const double* h_r, const OutGrid* grid, int n_iv, const int* ivs,
                      double* vals, int* ok) {
  if (n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  const int n1 = (int)ctx->lvl_ids[0].size();
  const int* l1 = lst(ctx, ctx->off_ids[0]);
  OutPools pools = out_pools(ctx, n_iv, ivs);
  double *d_r = nullptr, *d_v = nullptr;
  int* d_ok = nullptr;
  cudaError_t e = cudaSuccess;
  if (h_r) e = dalloc(&d_r, (size_t)n * ctx->D);
  if (e == cudaSuccess) e = dalloc(&d_v, (size_t)n * std::max(1, n_iv));
  if (e == cudaSuccess) e = dalloc(&d_ok, (size_t)n);
  if (e == cudaSuccess && h_r)
    e = cudaMemcpyAsync(d_r, h_r, sizeof(double) * n * ctx->D, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    const OutGrid g = grid ? *grid : OutGrid{};
    const int tpb = 128;
    const long long nb = (n + tpb - 1) / tpb;
    if (ctx->D == 3)
      k_interp1<3><<<(unsigned)nb, tpb, 0, ctx->stream>>>(t, l1, n1, n, 0, d_r, g, n_iv, pools, -1, d_v, d_ok);
    else
      k_interp1<2><<<(unsigned)nb, tpb, 0, ctx->stream>>>(t, l1, n1, n, 0, d_r, g, n_iv, pools, -1, d_v, d_ok);
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n_iv > 0)
    e = cudaMemcpyAsync(vals, d_v, sizeof(double) * n * n_iv, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && ok) e = cudaMemcpyAsync(ok, d_ok, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dfree(d_r);
  dfree(d_v);
  dfree(d_ok);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "interpolation: %s", cudaGetErrorString(e));
  return AFG_OK;
}

}  // namespace

/* ---- C-ABI --------------------------------------------------------------- */

int afg_interp1(afg_ctx* ctx, long long n_points, const double* r, int n_iv, const int* ivs, double* vals,
                int* success) {
  RC(check_out_vars(ctx, n_iv, ivs, nullptr));
  if (n_points < 0 || (n_points > 0 && (!r || (n_iv > 0 && !vals))))
    return fail(ctx, AFG_ERR_ARG, "bad point list");
  if (n_points > (long long)INT_MAX * 128) return fail(ctx, AFG_ERR_ARG, "too many points");
  return out_interp(ctx, n_points, r, nullptr, n_iv, ivs, vals, success);
}

int afg_write_vtk(afg_ctx* ctx, const char* filename, int n_cycle, double time, int n_iv, const int* ivs,
                  const char* const* names) {
  RC(check_out_vars(ctx, n_iv, ivs, names));
  if (!filename) return fail(ctx, AFG_ERR_ARG, "no file name");
  if (n_iv > 0 && !names) return fail(ctx, AFG_ERR_ARG, "no variable names");
  if (ctx->poisoned) return fail(ctx, AFG_ERR_DEVICE, "context unusable: copies outstanding");
  const int D = ctx->D, nc = ctx->nc, bn = nc + 1;
  const long long n_leaf = ctx->n_all_leaves;
  const long long cpb = D == 2 ? nc * nc : (long long)nc * nc * nc;
  const long long npb = D == 2 ? (long long)bn * bn : (long long)bn * bn * bn;
  const long long n_cells = n_leaf * cpb, n_nodes = n_leaf * npb;
  if (n_nodes > INT_MAX || n_cells * (1 << D) > INT_MAX)
    return fail(ctx, AFG_ERR_ARG, "mesh too large for Int32 connectivity (%lld cells)", n_cells);
  std::vector<afg_out::VtuArray> arrays;
  arrays.push_back({"Points", "Float32", "Points", 3, (uint64_t)n_nodes * 12});
  arrays.push_back({"Cells", "Int32", "connectivity", 1, (uint64_t)n_cells * (4u << D)});
  arrays.push_back({"Cells", "Int32", "offsets", 1, (uint64_t)n_cells * 4});
  arrays.push_back({"Cells", "Int32", "types", 1, (uint64_t)n_cells * 4});
  for (int v = 0; v < n_iv; v++) arrays.push_back({"CellData", "Float64", names[v], 1, (uint64_t)n_cells * 8});
  const std::string path = std::string(filename) + ".vtu";
  afg_out::VtuFile vf;
  if (!vf.open(path, time, n_cycle, n_nodes, n_cells, arrays))
    return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  OutStream st;
  CK(st.init(ctx, kOutChunkBytes));
  KTree t = ktree(ctx);
  const int* leaves = lst(ctx, ctx->off_all_leaves);
  auto put = [&](const void* h, size_t b) { return vf.write(h, b); };
  // points, per leaf box
  if (!vf.begin(arrays[0].bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
  RC(out_stream(st, n_leaf, (size_t)npb * 12, [&](long long g0, long long n, void* d) {
    if (D == 3) k_out_points<3><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, (float*)d);
    else k_out_points<2><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, (float*)d);
  }, put));
  if (!vf.begin(arrays[1].bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
  RC(out_stream(st, n_leaf, (size_t)cpb * (4u << D), [&](long long g0, long long n, void* d) {
    if (D == 3) k_out_connect<3><<<(unsigned)n, 128, 0, ctx->stream>>>(nc, g0, (int*)d);
    else k_out_connect<2><<<(unsigned)n, 128, 0, ctx->stream>>>(nc, g0, (int*)d);
  }, put));
  for (int types = 0; types < 2; types++) {
    if (!vf.begin(arrays[2 + types].bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
    RC(out_stream(st, n_cells, 4, [&](long long c0, long long n, void* d) {
      const unsigned nb = (unsigned)std::min<long long>((n + 255) / 256, 16LL * std::max(1, ctx->n_sm));
      if (D == 3) k_out_cellint<3><<<nb, 256, 0, ctx->stream>>>(c0, n, types, (int*)d);
      else k_out_cellint<2><<<nb, 256, 0, ctx->stream>>>(c0, n, types, (int*)d);
    }, put));
  }
  for (int v = 0; v < n_iv; v++) {
    if (!vf.begin(arrays[4 + v].bytes)) return fail(ctx, AFG_ERR_ARG, "write error");
    const double* pool = ctx->cc[ivs[v] - 1];
    RC(out_stream(st, n_leaf, (size_t)cpb * 8, [&](long long g0, long long n, void* d) {
      if (D == 3) k_out_cells<3><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, pool, (double*)d);
      else k_out_cells<2><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, pool, (double*)d);
    }, put));
  }
  if (!vf.close()) return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  return AFG_OK;
}

int afg_leaf_cells(afg_ctx* ctx, int iv, double* out, long long* n_cells) {
  RC(check_var(ctx, iv));
  const int D = ctx->D, nc = ctx->nc;
  const long long cpb = D == 2 ? nc * nc : (long long)nc * nc * nc;
  const long long n_leaf = ctx->n_all_leaves;
  if (n_cells) *n_cells = n_leaf * cpb;
  if (!out) return AFG_OK;
  OutStream st;
  CK(st.init(ctx, kOutChunkBytes));
  KTree t = ktree(ctx);
  const int* leaves = lst(ctx, ctx->off_all_leaves);
  const double* pool = ctx->cc[iv - 1];
  char* dst = reinterpret_cast<char*>(out);
  return out_stream(st, n_leaf, (size_t)cpb * 8, [&](long long g0, long long n, void* d) {
    if (D == 3) k_out_cells<3><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, pool, (double*)d);
    else k_out_cells<2><<<(unsigned)n, 128, 0, ctx->stream>>>(t, leaves, g0, pool, (double*)d);
  }, [&](const void* h, size_t b) {
    memcpy(dst, h, b);
    dst += b;
    return true;
  });
}

int afg_write_line(afg_ctx* ctx, const char* filename, int n_iv, const int* ivs, const char* const* names,
                   const double* r_min, const double* r_max, int n_points) {
  RC(check_out_vars(ctx, n_iv, ivs, names));
  if (!filename || !r_min || !r_max || n_points < 1 || (n_iv > 0 && !names))
    return fail(ctx, AFG_ERR_ARG, "bad line arguments");
  const int D = ctx->D;
  // r = r_min + (i-1) dr_vec, dr_vec = (r_max - r_min) / max(1, n_points-1)
  // (af_write_line, m_af_output.f90:407-463)
  double drv[3];
  for (int d = 0; d < D; d++) drv[d] = (r_max[d] - r_min[d]) / (double)std::max(1, n_points - 1);
  std::vector<double> r((size_t)n_points * D), vals((size_t)n_points * std::max(1, n_iv));
  std::vector<int> ok(n_points);
  for (int i = 0; i < n_points; i++)
    for (int d = 0; d < D; d++) r[(size_t)i * D + d] = r_min[d] + (double)i * drv[d];
  RC(out_interp(ctx, n_points, r.data(), nullptr, n_iv, ivs, vals.data(), ok.data()));
  for (int i = 0; i < n_points; i++)
    if (!ok[i]) return fail(ctx, AFG_ERR_ARG, "af_write_line: interpolation error (point %d outside the tree)", i + 1);
  const std::string path = std::string(filename) + ".txt";
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  fputs(D == 2 ? "# x y" : "# x y z", f);
  for (int v = 0; v < n_iv; v++) fprintf(f, " %s", names[v]);
  fputs("\n", f);
  for (int i = 0; i < n_points; i++) {
    for (int d = 0; d < D; d++) fprintf(f, " %24.17E", r[(size_t)i * D + d]);
    for (int v = 0; v < n_iv; v++) fprintf(f, " %24.17E", vals[(size_t)i * n_iv + v]);
    fputs("\n", f);
  }
  if (fclose(f) != 0) return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  return AFG_OK;
}

int afg_write_plane(afg_ctx* ctx, const char* filename, int n_iv, const int* ivs, const char* const* names,
                    const double* r_min, const double* r_max, const int* n_pixels) {
  RC(check_out_vars(ctx, n_iv, ivs, names));
  if (!filename || !r_min || !r_max || !n_pixels || n_pixels[0] < 2 || n_pixels[1] < 2 || (n_iv > 0 && !names))
    return fail(ctx, AFG_ERR_ARG, "bad plane arguments");
  const int D = ctx->D;
  // af_write_plane (m_af_output.f90:465-552): two spanning vectors over the
  // coordinates in which r_min and r_max differ (3D: all but the first
  // minimum of |r_max - r_min|)
  double dvec[3] = {0, 0, 0}, v1[3] = {0, 0, 0}, v2[3] = {0, 0, 0};
  long long npts[3];
  for (int d = 0; d < D; d++) dvec[d] = r_max[d] - r_min[d];
  const double n1 = (double)(n_pixels[0] - 1), n2 = (double)(n_pixels[1] - 1);
  if (D == 2) {
    v1[0] = dvec[0] / n1;
    v1[1] = 0.0 / n1;
    v2[0] = 0.0 / n2;
    v2[1] = dvec[1] / n2;
    npts[0] = n_pixels[0], npts[1] = n_pixels[1], npts[2] = 1;
  } else {
    int un = 0;
    for (int d = 1; d < 3; d++)
      if (std::fabs(dvec[d]) < std::fabs(dvec[un])) un = d;
    const int a = un == 0 ? 1 : 0, b = un == 2 ? 1 : 2;
    for (int d = 0; d < 3; d++) {
      v1[d] = (d == a ? dvec[d] : 0.0) / n1;
      v2[d] = (d == b ? dvec[d] : 0.0) / n2;
    }
    npts[0] = un == 0 ? 1 : n_pixels[0];
    npts[1] = un == 0 ? n_pixels[0] : un == 1 ? 1 : n_pixels[1];
    npts[2] = un == 2 ? 1 : n_pixels[1];
  }
  const long long np = (long long)n_pixels[0] * n_pixels[1];
  std::vector<double> r((size_t)np * D), vals((size_t)np * std::max(1, n_iv));
  std::vector<int> ok(np);
  for (int j = 0; j < n_pixels[1]; j++)
    for (int i = 0; i < n_pixels[0]; i++)
      for (int d = 0; d < D; d++)
        r[((size_t)j * n_pixels[0] + i) * D + d] = r_min[d] + (double)i * v1[d] + (double)j * v2[d];
  RC(out_interp(ctx, np, r.data(), nullptr, n_iv, ivs, vals.data(), ok.data()));
  for (long long p = 0; p < np; p++)
    if (!ok[p]) return fail(ctx, AFG_ERR_ARG, "af_write_plane: interpolation error (pixel %lld outside the tree)", p + 1);
  const std::string path = std::string(filename) + ".vtk";
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  fprintf(f, "# vtk DataFile Version 2.0\n%s\nASCII\nDATASET STRUCTURED_POINTS\n", filename);
  fprintf(f, "DIMENSIONS %10lld%10lld%10lld\n", npts[0], npts[1], npts[2]);
  double org[3] = {r_min[0], r_min[1], D == 3 ? r_min[2] : 0.0};
  double spc[3] = {v1[0] + v2[0], v1[1] + v2[1], D == 3 ? v1[2] + v2[2] : 0.0};
  fputs("ORIGIN ", f);
  for (int d = 0; d < 3; d++) fputs(afg_out::fortran_e(org[d], 20, 8).c_str(), f);
  fputs("\nSPACING ", f);
  for (int d = 0; d < 3; d++) fputs(afg_out::fortran_e(spc[d], 20, 8).c_str(), f);
  fprintf(f, "\nPOINT_DATA %lld\n", np);
  std::string row;
  for (int v = 0; v < n_iv; v++) {
    fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", names[v]);
    for (int j = 0; j < n_pixels[1]; j++) {
      row.clear();
      for (int i = 0; i < n_pixels[0]; i++)
        row += afg_out::fortran_e(vals[((size_t)j * n_pixels[0] + i) * n_iv + v], 20, 8);
      row += "\n";
      fputs(row.c_str(), f);
    }
  }
  if (fclose(f) != 0) return fail(ctx, AFG_ERR_ARG, "cannot write %s", path.c_str());
  return AFG_OK;
}

int afg_write_numpy(afg_ctx* ctx, const char* filename, const double* r_min, const double* r_max,
                    const int* n_points, int n_cycle, double time, int n_iv, const int* ivs,
                    const char* const* names) {
  RC(check_out_vars(ctx, n_iv, ivs, names));
  if (!filename || (n_iv > 0 && !names)) return fail(ctx, AFG_ERR_ARG, "bad numpy arguments");
  const std::string fn(filename);
  const bool npz = fn.size() >= 4 && fn.compare(fn.size() - 4, 4, ".npz") == 0;
  const bool npy = fn.size() >= 4 && fn.compare(fn.size() - 4, 4, ".npy") == 0;
  if (!npz && !npy) return fail(ctx, AFG_ERR_ARG, "Unknown file extension");
  const int D = ctx->D, nc = ctx->nc;
  // r_base and dr_base: the level-1 box with ix = 1 in every dimension
  std::vector<double> h_rmin((size_t)ctx->n_boxes * D), h_dr((size_t)ctx->n_boxes * D);
  CK(cudaMemcpy(h_rmin.data(), ctx->d_rmin, sizeof(double) * h_rmin.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(h_dr.data(), ctx->d_dr, sizeof(double) * h_dr.size(), cudaMemcpyDeviceToHost));
  int base = -1;
  for (int s : ctx->lvl_ids[0]) {
    bool one = true;
    for (int d = 0; d < D; d++) one = one && ctx->h_ix[(size_t)s * D + d] == 1;
    if (one) base = s;
  }
  if (base < 0) return fail(ctx, AFG_ERR_STATE, "no level-1 box at ix = 1");
  double rmin[3], rmax[3], dr[3];
  long long nx[3] = {1, 1, 1};
  for (int d = 0; d < D; d++) {
    const double rb = h_rmin[(size_t)base * D + d], db = h_dr[(size_t)base * D + d];
    rmin[d] = r_min ? r_min[d] : rb;
    rmax[d] = r_max ? r_max[d] : rb + db * (double)ctx->cgs[d];
  }
  if (n_points) {
    for (int d = 0; d < D; d++) nx[d] = n_points[d];
  } else {
    // the lowest level with a leaf in the region (m_af_output.f90:813-829)
    int lvl = 1;
    for (; lvl <= ctx->highest_lvl - 1; lvl++) {
      bool found = false;
      for (int s : ctx->lvl_leaves[lvl - 1]) {
        bool in = true;
        for (int d = 0; d < D; d++) {
          const double lo = h_rmin[(size_t)s * D + d];
          in = in && lo <= rmax[d] && lo + (double)nc * h_dr[(size_t)s * D + d] >= rmin[d];
        }
        if (in) {
          found = true;
          break;
        }
      }
      if (found) break;
    }
    for (int d = 0; d < D; d++) {
      double ldr = h_dr[(size_t)base * D + d];
      for (int l = 1; l < lvl; l++) ldr *= 0.5;
      nx[d] = (long long)std::llround((rmax[d] - rmin[d]) / ldr);
    }
  }
  long long np = 1;
  for (int d = 0; d < D; d++) {
    if (nx[d] < 1) return fail(ctx, AFG_ERR_ARG, "bad number of points");
    dr[d] = (rmax[d] - rmin[d]) / (double)nx[d];
    np *= nx[d];
  }
  OutGrid g{};
  for (int d = 0; d < D; d++) g.rmin[d] = rmin[d], g.dr[d] = dr[d], g.nx[d] = nx[d];
  // one variable after the other (the Fortran order of cc(nx.., n_cc)),
  // in chunks of points; a point outside the tree fails the whole call
  KTree t = ktree(ctx);
  const int n1 = (int)ctx->lvl_ids[0].size();
  const int* l1 = lst(ctx, ctx->off_ids[0]);
  OutPools pools = out_pools(ctx, n_iv, ivs);
  OutStream st;
  CK(st.init(ctx, kOutChunkBytes));
  int* d_ok = nullptr;
  CK(dalloc(&d_ok, (size_t)(kOutChunkBytes / 8)));
  unsigned* d_bad = nullptr;
  cudaError_t e = dalloc(&d_bad, 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(unsigned), ctx->stream);
  std::vector<std::string> blobs(std::max(1, n_iv));
  int rc = AFG_OK;
  for (int v = 0; v < n_iv && rc == AFG_OK && e == cudaSuccess; v++) {
    std::string& blob = blobs[v];
    blob.reserve((size_t)np * 8);
    rc = out_stream(st, np, 8, [&](long long p0, long long n, void* d) {
      const int tpb = 128;
      if (D == 3)
        k_interp1<3><<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, ctx->stream>>>(t, l1, n1, n, p0, nullptr, g, n_iv,
                                                                                pools, v, (double*)d, d_ok);
      else
        k_interp1<2><<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, ctx->stream>>>(t, l1, n1, n, p0, nullptr, g, n_iv,
                                                                                pools, v, (double*)d, d_ok);
      k_count_zero<<<(unsigned)std::min<long long>((n + 255) / 256, 1024), 256, 0, ctx->stream>>>(d_ok, n, d_bad);
      ctx->launches++;
    }, [&](const void* h, size_t b) {
      blob.append(static_cast<const char*>(h), b);
      return true;
    });
  }
  unsigned bad = 0;
  if (e == cudaSuccess && rc == AFG_OK) e = cudaMemcpy(&bad, d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost);
  dfree(d_ok);
  dfree(d_bad);
  if (rc != AFG_OK) return rc;
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "numpy output: %s", cudaGetErrorString(e));
  if (bad) return fail(ctx, AFG_ERR_ARG, "af_write_numpy: interpolation error (%u points outside the tree)", bad);
  std::vector<long long> shape(nx, nx + D);
  if (npy) {
    shape.push_back(n_iv);
    FILE* f = fopen(filename, "wb");
    if (!f) return fail(ctx, AFG_ERR_ARG, "cannot write %s", filename);
    const std::string h = afg_out::npy_header("<f8", shape);
    bool okw = fwrite(h.data(), 1, h.size(), f) == h.size();
    for (int v = 0; v < n_iv && okw; v++) okw = fwrite(blobs[v].data(), 1, blobs[v].size(), f) == blobs[v].size();
    okw = (fclose(f) == 0) && okw;
    if (!okw) return fail(ctx, AFG_ERR_ARG, "cannot write %s", filename);
    return AFG_OK;
  }
  // .npz: one array per variable plus the grid description, stored
  // uncompressed under their names (m_af_output.f90:876-897)
  afg_out::ZipStore z;
  if (!z.open(filename)) return fail(ctx, AFG_ERR_ARG, "cannot write %s", filename);
  bool okw = true;
  for (int v = 0; v < n_iv && okw; v++) okw = z.add(names[v], afg_out::npy_header("<f8", shape) + blobs[v]);
  auto vec_f8 = [&](const double* x, int n) {
    return afg_out::npy_header("<f8", {n}) + std::string(reinterpret_cast<const char*>(x), sizeof(double) * n);
  };
  auto vec_i4 = [&](const int* x, int n) {
    return afg_out::npy_header("<i4", {n}) + std::string(reinterpret_cast<const char*>(x), sizeof(int) * n);
  };
  int nxi[3] = {(int)nx[0], (int)nx[1], (int)nx[2]};
  const int coord = ctx->coord;
  const double tc[2] = {time, (double)n_cycle};
  if (okw) okw = z.add("nx", vec_i4(nxi, D));
  if (okw) okw = z.add("r_min", vec_f8(rmin, D));
  if (okw) okw = z.add("r_max", vec_f8(rmax, D));
  if (okw) okw = z.add("dr", vec_f8(dr, D));
  if (okw) okw = z.add("coord_t", vec_i4(&coord, 1));
  if (okw) okw = z.add("time_cycle", vec_f8(tc, 2));
  okw = z.close() && okw;
  if (!okw) return fail(ctx, AFG_ERR_ARG, "cannot write %s", filename);
  return AFG_OK;
}
