// afg_noalloc.cu -- a reduction entry point that allocates no device memory.
//
// afg_maxabs (afg_runtime.cu) keeps its reduction word in memory that
// afg_init allocated.  Some callers may not call cudaMalloc at all: code that
// owns its device arrays through its own allocator or memory pool (a Fortran
// host using CUDA Fortran/OpenACC data regions, a solver running under a
// fixed device-memory budget) and only wants the max-norm of a box pool.
// afg_maxabs_noalloc serves them: it works on caller-owned device buffers
// and needs no context, and its scratch lives in the file-scope array below,
// which every GPU that loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/afivo_gpu.h"

namespace {

constexpr int kMaxDevices = 64;

// Per-box maxima, then the final value at index AFG_NOALLOC_MAX_BOXES.
static __device__ __align__(256) double g_noalloc_scratch[AFG_NOALLOC_MAX_BOXES + 1];

// Device address of g_noalloc_scratch per device.  In host code the array's
// name is only a host-side stand-in, so the address is looked up once per
// device, with that device current, and passed to the kernels.
double* g_scratch_ptr[kMaxDevices] = {};
std::once_flag g_once[kMaxDevices];
cudaError_t g_setup_err[kMaxDevices] = {};

// Maxima of non-negative values (magnitudes, NaN included) compared as
// integers: the IEEE-754 bit patterns of non-negative doubles order like the
// numbers, and a NaN magnitude (exponent all ones, mantissa non-zero) sorts
// above infinity, so a NaN anywhere in the data is the result, exactly as
// with afg_maxabs.  fmax would drop it.
__device__ __forceinline__ double max_bits(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return __longlong_as_double(x > y ? x : y);
}
__device__ __forceinline__ double abs_bits(double v) {
  return __longlong_as_double(__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFll);
}

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = max_bits(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ double block_max_nonneg(double v) {
  __shared__ double s[32];
  v = warp_max(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s[warp] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (warp == 0 && lane < nw) ? s[lane] : 0.0;
  if (warp == 0) v = warp_max(v);
  return v;  // valid in thread 0
}

// Pass 1: max |v| over the interior cells of box slots[b] into scratch[b]
// (the per-box part of k_maxabs).
__global__ void __launch_bounds__(256) k_maxabs_boxes(const double* __restrict__ pool, const int* __restrict__ slots,
                                                      int ndim, int nc, double* __restrict__ scratch) {
  const int n2 = nc + 2;
  const size_t S = ndim == 2 ? (size_t)n2 * n2 : (size_t)n2 * n2 * n2;
  const double* a = pool + (size_t)slots[blockIdx.x] * S;
  const int count = ndim == 2 ? nc * nc : nc * nc * nc;
  double mx = 0.0;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = ndim == 2 ? r + 1 : r % nc + 1, k = ndim == 2 ? 0 : r / nc + 1;
    mx = max_bits(mx, abs_bits(a[i + n2 * (j + n2 * k)]));
  }
  mx = block_max_nonneg(mx);
  if (threadIdx.x == 0) scratch[blockIdx.x] = mx;
}

// Pass 2: one CTA folds the n per-box maxima into scratch[AFG_NOALLOC_MAX_BOXES].
__global__ void __launch_bounds__(1024) k_maxabs_fold(int n, double* __restrict__ scratch) {
  double mx = 0.0;
  for (int b = threadIdx.x; b < n; b += blockDim.x) mx = max_bits(mx, scratch[b]);
  mx = block_max_nonneg(mx);
  if (threadIdx.x == 0) scratch[AFG_NOALLOC_MAX_BOXES] = mx;
}

void setup_device(int dev) {
  void* p = nullptr;
  g_setup_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (g_setup_err[dev] == cudaSuccess) g_scratch_ptr[dev] = static_cast<double*>(p);
}

}  // namespace

extern "C" int afg_maxabs_noalloc(const double* d_pool, const int* d_slots, int n_slots, int ndim, int n_cell,
                                  void* stream, double* result) {
  if (!d_pool || !d_slots || !result) return AFG_ERR_ARG;
  if (ndim != 2 && ndim != 3) return AFG_ERR_ARG;
  if (n_cell < 2 || n_cell > 64 || (n_cell & 1)) return AFG_ERR_ARG;
  if (n_slots < 0 || n_slots > AFG_NOALLOC_MAX_BOXES) return AFG_ERR_ARG;  // beyond the scratch array
  if (n_slots == 0) {
    *result = 0.0;
    return AFG_OK;
  }
  // an error left pending by earlier work of the caller is reported here,
  // before any launch, so that the launch checks below see only this call's
  if (cudaGetLastError() != cudaSuccess) return AFG_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AFG_ERR_CUDA;
  std::call_once(g_once[dev], setup_device, dev);
  if (g_setup_err[dev] != cudaSuccess || !g_scratch_ptr[dev]) return AFG_ERR_CUDA;
  double* scratch = g_scratch_ptr[dev];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_maxabs_boxes<<<n_slots, 256, 0, s>>>(d_pool, d_slots, ndim, n_cell, scratch);
  if (cudaGetLastError() != cudaSuccess) return AFG_ERR_CUDA;
  k_maxabs_fold<<<1, 1024, 0, s>>>(n_slots, scratch);
  if (cudaGetLastError() != cudaSuccess) return AFG_ERR_CUDA;
  double v = 0.0;
  if (cudaMemcpyAsync(&v, scratch + AFG_NOALLOC_MAX_BOXES, sizeof(double), cudaMemcpyDeviceToHost, s) !=
      cudaSuccess)
    return AFG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return AFG_ERR_CUDA;
  *result = v;
  return AFG_OK;
}
