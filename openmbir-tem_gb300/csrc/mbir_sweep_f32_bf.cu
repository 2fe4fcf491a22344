// mbir_sweep_f32_bf.cu -- FP32 ICD sweep kernels (bright field) with the voxel slice and its
// Bragg selector rows staged in shared memory.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_smem_bf(const SweepArgs& a, int nb, size_t smem, void* stream) {
  return sweep::launch_sweep_f32_pick<true, true>(a, nb, smem, static_cast<cudaStream_t>(stream));
}

int launch_acol_f32(const DevGeom& g, const DevTables& tab, int nb, float4* out, void* stream) {
  return sweep::launch_acol_t(g, tab, nb, out, static_cast<cudaStream_t>(stream));
}

}  // namespace mbir
