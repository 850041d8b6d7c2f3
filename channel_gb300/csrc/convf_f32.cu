// Register-blocked transform kernels (convf.cuh) instantiated for float.
#include "convf.cuh"

namespace chgpu {

template <>
bool launch_convolutions_r<float>(const ConvLaunch& L, cudaStream_t s, int stage) {
  return launch_convolutions_r_impl<float>(L, s, stage);
}
template <>
cudaError_t convr_set_smem_limits<float>() {
  return set_limits_type<float>();
}

}  // namespace chgpu
