// mbir_sweep_f32_hbm.cu -- FP32 ICD sweep kernels (HAADF) for voxel slices too large for
// shared memory (the slice's detector rows are used in place in HBM), and the FP32
// reference-order kernel.  The bright-field ones are in mbir_sweep_f32_hbm_bf.cu.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_hbm(const SweepArgs& a, int nb, size_t smem, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a.bf ? launch_sweep_f32_hbm_bf(a, nb, smem, stream)
              : sweep::launch_sweep_f32_pick<false, false>(a, nb, smem, s);
}

int launch_ref_order_f32(const RefOrderArgs& a, int nb, void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nb == 3) return launch_ref_t<float, 3, 5>(a, s);
  if (nb == 5) return launch_ref_t<float, 5, 5>(a, s);
  if (nb == 9) return launch_ref_t<float, 9, 5>(a, s);
  return -7;
}

}  // namespace mbir
