// afg_species_update.cu -- launchers of the species-update kernels
// (flux_update_densities + add_source_terms: k_update, k_update32 of
// afg_transport.cuh / afg_transport32.cuh), in a translation unit of their
// own: the kernels are instantiated for every dimension, coordinate system,
// box size and compile-time species bound, and compile in parallel with the
// runtime.  Called by afg_update_densities (afg_transport_api.cuh).
#include <cuda_runtime.h>

#include "afg_transport32.cuh"

namespace afg {

namespace {

// D, cylindrical and compile-time box size (8^3 and 16^2 specialised)
template <int NSM, bool F32, typename Args>
void launch_update_ns(int D, bool cyl, int nc, int n, const KTree& t, const int* list, const Args& a, size_t smem,
                      cudaStream_t st) {
  if constexpr (F32) {
    if (D == 3 && nc == 8) k_update32<3, false, NSM, 8><<<n, 128, smem, st>>>(t, list, a);
    else if (D == 3) k_update32<3, false, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
    else if (cyl && nc == 16) k_update32<2, true, NSM, 16><<<n, 128, smem, st>>>(t, list, a);
    else if (cyl) k_update32<2, true, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
    else if (nc == 16) k_update32<2, false, NSM, 16><<<n, 128, smem, st>>>(t, list, a);
    else k_update32<2, false, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
  } else {
    if (D == 3 && nc == 8) k_update<3, false, NSM, 8><<<n, 128, smem, st>>>(t, list, a);
    else if (D == 3) k_update<3, false, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
    else if (cyl && nc == 16) k_update<2, true, NSM, 16><<<n, 128, smem, st>>>(t, list, a);
    else if (cyl) k_update<2, true, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
    else if (nc == 16) k_update<2, false, NSM, 16><<<n, 128, smem, st>>>(t, list, a);
    else k_update<2, false, NSM, 0><<<n, 128, smem, st>>>(t, list, a);
  }
}

}  // namespace

// FP32 arithmetic: compile-time species bounds close to the model's count,
// so that the unrolled species loops carry no dead guarded iterations; smem
// = the reaction records (dynamic shared memory)
void launch_update32(int D, bool cyl, int nc, int ns, int n, const KTree& t, const int* list, const UpdateArgs32& u,
                     size_t smem, cudaStream_t st) {
  if (ns <= 3) launch_update_ns<3, true>(D, cyl, nc, n, t, list, u, smem, st);
  else if (ns <= 4) launch_update_ns<4, true>(D, cyl, nc, n, t, list, u, smem, st);
  else if (ns <= 5) launch_update_ns<5, true>(D, cyl, nc, n, t, list, u, smem, st);
  else if (ns <= 6) launch_update_ns<6, true>(D, cyl, nc, n, t, list, u, smem, st);
  else if (ns <= 8) launch_update_ns<8, true>(D, cyl, nc, n, t, list, u, smem, st);
  else launch_update_ns<16, true>(D, cyl, nc, n, t, list, u, smem, st);
}

// FP64 arithmetic (the reference's)
void launch_update64(int D, bool cyl, int nc, int ns, int n, const KTree& t, const int* list, const UpdateArgs& a,
                     cudaStream_t st) {
  if (ns <= 4) launch_update_ns<4, false>(D, cyl, nc, n, t, list, a, 0, st);
  else if (ns <= 8) launch_update_ns<8, false>(D, cyl, nc, n, t, list, a, 0, st);
  else launch_update_ns<16, false>(D, cyl, nc, n, t, list, a, 0, st);
}

}  // namespace afg
