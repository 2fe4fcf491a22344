// mbir_sweep_f32_batch3.cu -- persistent batched sweep kernels, three-bin footprints.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_batch_sweep_nb3(const BatchArgs& b, int group, int threads, size_t smem, int grid,
                            void* stream) {
  return sweep::launch_batch_pick<3>(b, group, threads, smem, grid,
                                     static_cast<cudaStream_t>(stream));
}

}  // namespace mbir
