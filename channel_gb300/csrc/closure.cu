// Velocity gradients of the coarse field for the learned closure.
//
// k_grad_xz: d/dx and d/dz, the products with i alfa0 kx and i beta0 kz,
// one thread per value.  k_grad: one thread per (mode, velocity component
// c), d/dy by the compact
// derivative COMPLEXderiv (dnsdata.f90:339-373): the d1 stencil with the
// one-sided wall values d140/d14m1/d14n/d14np1 folded in, then the two
// sweeps of the D0mat factorisation (LeftLU5divStep1 bottom-up,
// LeftLU5divStep2 top-down; rbparmat_blocking.f90:57-100).  G holds nine
// fields in the layout of V: G[3c + 0, 1, 2] = d/dx, d/dy, d/dz of V[c].
#include <cuda_runtime.h>

#include "chgpu_internal.h"
#include "kernels.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ size_t gidx(const Dims& d, int c, int iy, int m) {
  return ((size_t)c * d.nplanes + (iy + 1)) * d.nmodes + m;
}
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 rm(double s, double2 a) { return make_double2(s * a.x, s * a.y); }

// d/dx and d/dz: one thread per (component, plane, mode)
__global__ void k_grad_xz(const double2* __restrict__ V, double2* __restrict__ G, Dims d) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_c = (size_t)d.nplanes * d.nmodes;
  if (t >= 3 * per_c) return;
  const int c = (int)(t / per_c);
  const size_t r = t - c * per_c;
  const int m = (int)(r % d.nmodes);
  const int ix = m / d.nzt, kz = m - ix * d.nzt - d.nz;
  const double ka = d.alfa0 * ix, kb = d.beta0 * kz;
  const double2 v = V[t];
  G[(size_t)(3 * c) * per_c + r] = make_double2(-ka * v.y, ka * v.x);
  G[(size_t)(3 * c + 2) * per_c + r] = make_double2(-kb * v.y, kb * v.x);
}

// d/dy: one thread per (mode, component), the two sweeps along y
__global__ void k_grad(const double2* __restrict__ V, double2* __restrict__ G, const double* __restrict__ der,
                       const double* __restrict__ d0lu, BcRows bc, Dims d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * d.nmodes) return;
  const int c = t / d.nmodes, m = t - c * d.nmodes;
  const int ny = d.ny;
  // d/dy: wall values, then Step1 bottom-up parked in the d/dy slot, then Step2
  auto dot5 = [&](int iy0, const double* w) {
    double2 a = rm(w[0], V[gidx(d, c, iy0, m)]);
    for (int j = 1; j < 5; ++j) a = a + rm(w[j], V[gidx(d, c, iy0 + j, m)]);
    return a;
  };
  const double2 f0 = dot5(-1, bc.d140), fm1 = dot5(-1, bc.d14m1);
  const double2 fn = dot5(ny - 3, bc.d14n), fn1 = dot5(ny - 3, bc.d14np1);
  double2* out = G + gidx(d, 3 * c + 1, 0, m) - (size_t)d.nmodes;  // out[(iy+1)*nmodes] = d/dy at iy
  double2 x1 = make_double2(0.0, 0.0), x2 = x1;
  for (int iy = ny - 1; iy >= 1; --iy) {
    const double* dr = der + (size_t)iy * 20;
    double2 f = rm(dr[5], V[gidx(d, c, iy - 2, m)]);
    for (int j = 1; j < 5; ++j) f = f + rm(dr[5 + j], V[gidx(d, c, iy - 2 + j, m)]);
    if (iy == ny - 1) f = f - (rm(dr[3], fn) + rm(dr[4], fn1));
    if (iy == ny - 2) f = f - rm(dr[4], fn);
    if (iy == 1) f = f - (rm(dr[1], f0) + rm(dr[0], fm1));
    if (iy == 2) f = f - rm(dr[0], f0);
    const double* lu = d0lu + (size_t)(iy - 1) * 5;
    const double2 s = rm(lu[3], x1) + rm(lu[4], x2);
    const double2 x = rm(lu[2], f - s);
    x2 = x1;
    x1 = x;
    out[(size_t)(iy + 1) * d.nmodes] = x;
  }
  double2 bm2 = make_double2(0.0, 0.0), bm1 = fm1;
  for (int iy = -1; iy <= ny + 1; ++iy) {
    double2 vp;
    if (iy == -1) vp = fm1;
    else if (iy == 0) vp = f0;
    else if (iy == ny) vp = fn;
    else if (iy == ny + 1) vp = fn1;
    else {
      const double* lu = d0lu + (size_t)(iy - 1) * 5;
      vp = out[(size_t)(iy + 1) * d.nmodes] - (rm(lu[0], bm2) + rm(lu[1], bm1));
    }
    if (iy >= 0 && iy <= ny - 1) {
      bm2 = bm1;
      bm1 = vp;
    }
    out[(size_t)(iy + 1) * d.nmodes] = vp;
  }
}

}  // namespace

void launch_gradients(const double2* V, double2* G, const double* der, const double* d0lu, const BcRows& bc,
                      const Dims& d, cudaStream_t s) {
  const size_t nxz = (size_t)3 * d.nplanes * d.nmodes;
  k_grad_xz<<<(unsigned)((nxz + 255) / 256), 256, 0, s>>>(V, G, d);
  const int n = 3 * d.nmodes;
  k_grad<<<(n + 63) / 64, 64, 0, s>>>(V, G, der, d0lu, bc, d);
}

}  // namespace chgpu
