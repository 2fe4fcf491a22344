// mbir_sweep_f32_hbm_bf.cu -- FP32 bright-field ICD sweep kernels for voxel slices too large for
// shared memory (the slice's detector rows and selector bytes used in place in HBM).
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_hbm_bf(const SweepArgs& a, int nb, size_t smem, void* stream) {
  return sweep::launch_sweep_f32_pick<false, true>(a, nb, smem, static_cast<cudaStream_t>(stream));
}

}  // namespace mbir
