// Statistics of the field on the device: running sums for the mean and
// variance profiles that the reference's post-processing defines
// (postpro/history/var_history.f90:37-84):
//   mean_c(y) = < Re V(y, kx=0, kz=0, c) >
//   var_c(y)  = < sum_{ix,iz} f_ix |V(y,iz,ix,c) - delta_{ix,0} delta_{iz,0} mean_c(y)|^2 >
// with f_ix = 1 for ix = 0 and 2 otherwise (the kx<0 half of the spectrum).
// Expanding the square gives var = <S2> - mean^2 with S2 = sum f |V|^2, so one
// pass per sample accumulates S1 = Re V00 and S2; sums over samples are
// compensated (Kahan), the per-plane sum over modes is a thread-level Kahan
// sum followed by a pairwise tree.
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ void kahan_add(double& sum, double& comp, double x) {
  const double y = x - comp;
  const double t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

__global__ void __launch_bounds__(256) k_stats_accumulate(const double2* __restrict__ V, Dims d, double* acc) {
  // acc: [4][3][nplanes] = S1, compensation of S1, S2, compensation of S2
  const int plane = blockIdx.x, c = blockIdx.y;
  const double2* row = V + ((size_t)c * d.nplanes + plane) * d.nmodes;
  double sum = 0.0, comp = 0.0;
  for (int m = threadIdx.x; m < d.nmodes; m += blockDim.x) {
    const double f = (m < d.nzt) ? 1.0 : 2.0;  // modes m < 2nz+1 have ix = 0
    const double2 v = row[m];
    kahan_add(sum, comp, f * (v.x * v.x + v.y * v.y));
  }
  __shared__ double red[256];
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const size_t n = (size_t)3 * d.nplanes, k = (size_t)c * d.nplanes + plane;
    kahan_add(acc[k], acc[n + k], row[d.nz].x);
    kahan_add(acc[2 * n + k], acc[3 * n + k], red[0]);
  }
}

}  // namespace

void launch_stats_accumulate(const double2* V, const Dims& d, double* acc, cudaStream_t s) {
  k_stats_accumulate<<<dim3(d.nplanes, 3), 256, 0, s>>>(V, d, acc);
}

}  // namespace chgpu
