// mbir_sweep_f32_batch5.cu -- persistent batched sweep kernels, five-bin footprints.
#include "mbir_sweep.cuh"

namespace mbir {

int launch_batch_sweep_nb5(const BatchArgs& b, int group, int threads, size_t smem, int grid,
                            void* stream) {
  return sweep::launch_batch_pick<5>(b, group, threads, smem, grid,
                                     static_cast<cudaStream_t>(stream));
}

}  // namespace mbir
