// mbir_sweep_f32.cu -- FP32 ICD sweep kernels with the voxel slice staged in shared memory,
// and the FP32 reference-order kernel.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_smem(const SweepArgs& a, int nb, size_t smem, void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int vpl = a.g.n_theta <= 64 ? 4 : (a.g.n_theta <= 128 ? 8 : 10);
  if (nb == 3 && vpl == 4) return launch_sweep_t<float, 3, 16, 4, true>(a, smem, s);
  if (nb == 3 && vpl == 8) return launch_sweep_t<float, 3, 16, 8, true>(a, smem, s);
  if (nb == 3 && vpl == 10) return launch_sweep_t<float, 3, 16, 10, true>(a, smem, s);
  if (nb == 5 && vpl == 4) return launch_sweep_t<float, 5, 16, 4, true>(a, smem, s);
  if (nb == 5 && vpl == 8) return launch_sweep_t<float, 5, 16, 8, true>(a, smem, s);
  if (nb == 5 && vpl == 10) return launch_sweep_t<float, 5, 16, 10, true>(a, smem, s);
  if (nb == 9) return launch_sweep_t<float, 9, 32, 5, true>(a, smem, s);
  return -7;
}

int launch_batch_sweep(const BatchArgs& b, int nb, int vpl, size_t smem, int grid,
                       void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nb == 3 && vpl == 4) return launch_batch_t<3, 16, 4>(b, smem, grid, s);
  if (nb == 3 && vpl == 8) return launch_batch_t<3, 16, 8>(b, smem, grid, s);
  if (nb == 3 && vpl == 10) return launch_batch_t<3, 16, 10>(b, smem, grid, s);
  if (nb == 5 && vpl == 4) return launch_batch_t<5, 16, 4>(b, smem, grid, s);
  if (nb == 5 && vpl == 8) return launch_batch_t<5, 16, 8>(b, smem, grid, s);
  if (nb == 5 && vpl == 10) return launch_batch_t<5, 16, 10>(b, smem, grid, s);
  return -7;
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
