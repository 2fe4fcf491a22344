// mbir_sweep_f32.cu -- FP32 ICD sweep kernels (HAADF) with the voxel slice staged in shared
// memory.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_smem_haadf(const SweepArgs& a, int nb, size_t smem, void* stream) {
  return sweep::launch_sweep_f32_pick<true, false>(a, nb, smem,
                                                   static_cast<cudaStream_t>(stream));
}

}  // namespace mbir
