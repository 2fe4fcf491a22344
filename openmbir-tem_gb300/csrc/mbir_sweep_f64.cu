// mbir_sweep_f64.cu -- FP64 instantiations of the sweep and reference-order kernels (the
// reference's own precision; used for order-exact parity and precision studies).
#include "mbir_sweep.cuh"

namespace mbir {

int launch_sweep_f64(const SweepArgs& a, int nb, size_t smem, void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool st = a.smem_rows != 0;
  if (a.g.n_theta > kMaxViewsShaped) {  // 32 lanes x 8 views, slices in HBM
    if (st) return -7;
    if (nb == 3) return launch_sweep_m<double, 3, 32, 8, false>(a, smem, s);
    if (nb == 5) return launch_sweep_m<double, 5, 32, 8, false>(a, smem, s);
    if (nb == 9) return launch_sweep_m<double, 9, 32, 8, false>(a, smem, s);
    return -7;
  }
  if (nb == 3)
    return st ? launch_sweep_m<double, 3, 32, 5, true>(a, smem, s)
              : launch_sweep_m<double, 3, 32, 5, false>(a, smem, s);
  if (nb == 5)
    return st ? launch_sweep_m<double, 5, 32, 5, true>(a, smem, s)
              : launch_sweep_m<double, 5, 32, 5, false>(a, smem, s);
  if (nb == 9)
    return st ? launch_sweep_m<double, 9, 32, 5, true>(a, smem, s)
              : launch_sweep_m<double, 9, 32, 5, false>(a, smem, s);
  return -7;
}

int launch_ref_order_f64(const RefOrderArgs& a, int nb, void* stream) {
  using namespace sweep;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nb == 3) return launch_ref_t<double, 3, 5>(a, s);
  if (nb == 5) return launch_ref_t<double, 5, 5>(a, s);
  if (nb == 9) return launch_ref_t<double, 9, 5>(a, s);
  return -7;
}

size_t sweep_smem_bytes(int n_theta, int n_x, int n_rs, int t_rows, int bins, int fp64,
                        int n_sp, bool sched) {
  return sweep::smem_layout(n_theta, n_x, n_rs, t_rows, bins, n_rs > 0, fp64 ? 8 : 4, n_sp, sched)
      .total;
}

}  // namespace mbir
