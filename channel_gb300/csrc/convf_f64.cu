// Register-blocked transform kernels (convf.cuh) instantiated for double.
#include "convf.cuh"

namespace chgpu {

template <>
bool launch_convolutions_r<double>(const ConvLaunch& L, cudaStream_t s, int stage) {
  return launch_convolutions_r_impl<double>(L, s, stage);
}
template <>
cudaError_t convr_set_smem_limits<double>() {
  return set_limits_type<double>();
}

}  // namespace chgpu
