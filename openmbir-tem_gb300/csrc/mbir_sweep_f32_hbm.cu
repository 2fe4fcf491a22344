// mbir_sweep_f32_hbm.cu -- FP32 ICD sweep kernels for voxel slices too large for shared
// memory: the slice's detector rows are used in place in HBM.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f32_hbm(const SweepArgs& a, int nb, size_t smem, void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int vpl = a.g.n_theta <= 64 ? 4 : (a.g.n_theta <= 128 ? 8 : 10);
  if (nb == 3 && vpl == 4) return launch_sweep_t<float, 3, 16, 4, false>(a, smem, s);
  if (nb == 3 && vpl == 8) return launch_sweep_t<float, 3, 16, 8, false>(a, smem, s);
  if (nb == 3 && vpl == 10) return launch_sweep_t<float, 3, 16, 10, false>(a, smem, s);
  if (nb == 5 && vpl == 4) return launch_sweep_t<float, 5, 16, 4, false>(a, smem, s);
  if (nb == 5 && vpl == 8) return launch_sweep_t<float, 5, 16, 8, false>(a, smem, s);
  if (nb == 5 && vpl == 10) return launch_sweep_t<float, 5, 16, 10, false>(a, smem, s);
  if (nb == 9) return launch_sweep_t<float, 9, 32, 5, false>(a, smem, s);
  return -7;
}

}  // namespace mbir
