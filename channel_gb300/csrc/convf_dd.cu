// Register-blocked transform kernels (convf.cuh) instantiated for dd.
#include "convf.cuh"

namespace chgpu {

template <>
bool launch_convolutions_r<dd>(const ConvLaunch& L, cudaStream_t s, int stage) {
  return launch_convolutions_r_impl<dd>(L, s, stage);
}
template <>
cudaError_t convr_set_smem_limits<dd>() {
  return set_limits_type<dd>();
}

}  // namespace chgpu
