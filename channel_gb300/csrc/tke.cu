// Spanwise spectra of the Reynolds-stress budgets on the device: the
// per-snapshot accumulation of the reference's post-processing program
// postpro/tke/uiuj_spectra.f90 (:161-240), from the handle's current field.
//
//   k_tke_prep   : the fluctuation u' = V with the mean profiles U(y), W(y)
//                  taken off the (0,0) mode (:172-174) into fields 0..2 of
//                  the work buffer W; fields 3 + 3i + k then receive
//                  du'_i/dx_k from launch_gradients (get_gradient_33,
//                  :469-486: i alfa0 kx, compact d/dy, i beta0 kz).
//   k_tke_zinv / k_tke_x / k_tke_zfwd : the convective term
//                  N_i = F(sum_k u'_k du'_i/dx_k) formed on the 3/2-padded
//                  physical grid and brought back to the kept modes with
//                  `factor`, in chunks of planes (the ttrsp block, :182-227;
//                  the sum over k is taken before the forward transform,
//                  which the linearity of the transform and of cprod allows).
//   k_tke_accum  : one thread per (plane, kz), the sum over kx with weight
//                  c = 1 (kx = 0), 2 of var, prod, psdiss, ttrsp and, with a
//                  pressure field, pstrain and PHIptrsp for the six pairs
//                  uu, vv, ww, uv, vw, uw (:161-180, :230-233), added to
//                  the running sums acc[term][pair][plane][kz].
// Everything is FP64 (the reference's arithmetic), in every precision path.
#include <cuda_runtime.h>

#include "chgpu_internal.h"
#include "cplx.cuh"
#include "kernels.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ double cprod(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }  // Re(conj(a) b)

__global__ void k_tke_prep(const double2* __restrict__ V, double2* __restrict__ W, const double* __restrict__ mean,
                           Dims d) {
  const size_t per_c = (size_t)d.nplanes * d.nmodes;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * per_c) return;
  const int c = (int)(t / per_c);
  const size_t r = t - (size_t)c * per_c;
  const int plane = (int)(r / d.nmodes);
  const int m = (int)(r - (size_t)plane * d.nmodes);
  double2 v = V[t];
  if (m == d.nz && c != 1) v.x -= mean[(c == 0 ? 0 : d.nplanes) + plane];  // mode (0,0): U and W
  W[t] = v;
}

// the pressure's mean profile off its (0,0) mode
__global__ void k_tke_pmean(double2* __restrict__ P, const double* __restrict__ meanp, Dims d) {
  const int plane = blockIdx.x * blockDim.x + threadIdx.x;
  if (plane < d.nplanes) P[(size_t)plane * d.nmodes + d.nz].x -= meanp[plane];
}

// z-inverse of one column of field f at one plane of the chunk
__global__ void __launch_bounds__(256) k_tke_zinv(const double2* __restrict__ W, double2* __restrict__ Zt,
                                                  const double2* __restrict__ twz, Dims d, RadixDev rz, int p0,
                                                  int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nzd = d.nzd, nz = d.nz, nxp = d.nx + 1;
  double2* a = reinterpret_cast<double2*>(smem_raw);
  double2* b = a + pad32_size(nzd);
  const int ix = blockIdx.x, pl = blockIdx.y, f = blockIdx.z;
  const double2* src = W + ((size_t)f * d.nplanes + p0 + pl) * d.nmodes + (size_t)ix * d.nzt;
  for (int jz = threadIdx.x; jz < nzd; jz += blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (jz <= nz) v = src[nz + jz];
    else if (jz >= nzd - nz) v = src[jz - nzd + nz];
    a[pad32(jz)] = v;
  }
  __syncthreads();
  double2* res = fft_block<+1>(a, b, 1, rz, twz);
  double2* out = Zt + (((size_t)f * C + pl) * nxp + ix) * nzd;
  for (int jz = threadIdx.x; jz < nzd; jz += blockDim.x) out[jz] = res[pad32(jz)];
}

// One plane row jz: for k = 0..2, the c2r of u'_k and du'_i/dx_k (i = 0..2)
// and N_i += u'_k du'_i/dx_k; then the r2c of N_0..2 with `factor`
// (g = factor/2 and twh[2M + k] = (factor/2) e^{-i pi k/M}, as in k_xrow).
__global__ void __launch_bounds__(256) k_tke_x(const double2* __restrict__ Zt, double2* __restrict__ Xt,
                                               const double2* __restrict__ twx, const double2* __restrict__ twh,
                                               Dims d, RadixDev rx, double g, int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = d.nxd, nx = d.nx, nxp = nx + 1, nzd = d.nzd;
  const int jz = blockIdx.x, pl = blockIdx.y;
  double2* Cb = reinterpret_cast<double2*>(smem_raw);
  double2* A = Cb + pad32_size(4 * M);
  double2* B = A + pad32_size(4 * M);
  double2* N = B + pad32_size(4 * M);
  for (int i = threadIdx.x; i < 3 * M; i += blockDim.x) N[pad32(i)] = make_double2(0.0, 0.0);
  for (int k = 0; k < 3; ++k) {
    // rows: u'_k, then du'_i/dx_k for i = 0..2 (work-buffer fields k, 3 + 3i + k)
    for (int idx = threadIdx.x; idx < 4 * M; idx += blockDim.x) {
      const int q = idx / M, kx = idx - q * M;
      const int f = q == 0 ? k : 3 + 3 * (q - 1) + k;
      double2 v = make_double2(0.0, 0.0);
      if (kx <= nx) v = Zt[(((size_t)f * C + pl) * nxp + kx) * nzd + jz];
      Cb[pad32(idx)] = v;
    }
    __syncthreads();
    // c2r packing (as k_xrow): Z = (X_k + conj X_{M-k}) + i (X_k - conj X_{M-k}) e^{+i pi k/M}
    for (int idx = threadIdx.x; idx < 4 * M; idx += blockDim.x) {
      const int q = idx / M, kx = idx - q * M;
      double2 xk = Cb[pad32(idx)];
      double2 xm = make_double2(0.0, 0.0);
      if (kx == 0) xk.y = 0.0;
      else xm = conjg(Cb[pad32(q * M + M - kx)]);
      const double2 e = xk + xm, o = cmul_s<+1>(xk - xm, twh[kx]);
      A[pad32(idx)] = e + mul_is<+1>(o);
    }
    __syncthreads();
    double2* U = fft_block<+1>(A, B, 4, rx, twx);
    for (int idx = threadIdx.x; idx < 3 * M; idx += blockDim.x) {
      const int i = idx / M, m = idx - i * M;
      const double2 u = U[pad32(m)], gi = U[pad32((1 + i) * M + m)];
      double2& n = N[pad32(idx)];
      n = make_double2(n.x + u.x * gi.x, n.y + u.y * gi.y);
    }
    __syncthreads();
  }
  double2* P = fft_block<-1>(N, A, 3, rx, twx);
  for (int idx = threadIdx.x; idx < 3 * nxp; idx += blockDim.x) {
    const int i = idx / nxp, kx = idx - i * nxp;
    const double2 zk = P[pad32(i * M + kx)];
    const double2 zm = conjg(P[pad32(i * M + (kx == 0 ? 0 : M - kx))]);
    const double2 sm = zk + zm, df = zk - zm;
    const double2 w = twh[2 * M + kx];
    Xt[(((size_t)i * C + pl) * nxp + kx) * nzd + jz] =
        make_double2(fma(g, sm.x, fma(w.x, df.y, w.y * df.x)), fma(g, sm.y, fma(w.y, df.y, -(w.x * df.x))));
  }
}

// z-forward of one column of N_i, truncated to |kz| <= nz
__global__ void __launch_bounds__(256) k_tke_zfwd(const double2* __restrict__ Xt, double2* __restrict__ N3,
                                                  const double2* __restrict__ twz, Dims d, RadixDev rz, int p0,
                                                  int C) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nzd = d.nzd, nz = d.nz, nxp = d.nx + 1;
  double2* a = reinterpret_cast<double2*>(smem_raw);
  double2* b = a + pad32_size(nzd);
  const int ix = blockIdx.x, pl = blockIdx.y, i = blockIdx.z;
  const double2* src = Xt + (((size_t)i * C + pl) * nxp + ix) * nzd;
  for (int jz = threadIdx.x; jz < nzd; jz += blockDim.x) a[pad32(jz)] = src[jz];
  __syncthreads();
  double2* res = fft_block<-1>(a, b, 1, rz, twz);
  double2* out = N3 + ((size_t)i * d.nplanes + p0 + pl) * d.nmodes + (size_t)ix * d.nzt;
  for (int izp = threadIdx.x; izp < d.nzt; izp += blockDim.x) {
    const int iz = izp - nz;
    out[izp] = res[pad32(iz >= 0 ? iz : nzd + iz)];
  }
}

// terms accumulated per snapshot (the rest follow at the end by y derivatives)
constexpr int kTkeTerms = 6;  // var, prod, psdiss, ttrsp, pstrain, PHIptrsp

__global__ void __launch_bounds__(128) k_tke_accum(const double2* __restrict__ W, const double2* __restrict__ N3,
                                                   const double2* __restrict__ P, double* __restrict__ acc,
                                                   const double* __restrict__ mgrad, Dims d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int S = d.nplanes * d.nzt;
  if (t >= S) return;
  const int plane = t / d.nzt, izp = t - plane * d.nzt;
  const size_t FS = (size_t)d.nplanes * d.nmodes;
  const double ni = d.ni;
  const double Uy = mgrad[plane], Wy = mgrad[d.nplanes + plane];
  // mean velocity gradient M[j][k] (get_mean_grad): M[0][1] = dU/dy, M[2][1] = dW/dy
  const double Mj1[3] = {Uy, 0.0, Wy};
  double a[kTkeTerms][6];
#pragma unroll
  for (int q = 0; q < kTkeTerms; ++q)
#pragma unroll
    for (int r = 0; r < 6; ++r) a[q][r] = 0.0;
  constexpr int PI_[6] = {0, 1, 2, 0, 1, 0}, PJ_[6] = {0, 1, 2, 1, 2, 2};
  for (int ix = 0; ix <= d.nx; ++ix) {
    const double c = ix == 0 ? 1.0 : 2.0;
    const size_t base = (size_t)plane * d.nmodes + (size_t)ix * d.nzt + izp;
    double2 u[3], n[3], gr[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      u[i] = W[i * FS + base];
      n[i] = N3[i * FS + base];
#pragma unroll
      for (int k = 0; k < 3; ++k) gr[i][k] = W[(size_t)(3 + 3 * i + k) * FS + base];
    }
    const double2 p = P ? P[base] : make_double2(0.0, 0.0);
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const int i = PI_[r], j = PJ_[r];
      a[0][r] = a[0][r] + c * cprod(u[i], u[j]);
      // the reference sums over k with the mean gradient's zero entries too
      a[1][r] = a[1][r] - c * (cprod(u[i], u[1]) * Mj1[j] + cprod(u[j], u[1]) * Mj1[i]);
#pragma unroll
      for (int k = 0; k < 3; ++k) a[2][r] = a[2][r] - 2.0 * ni * c * cprod(gr[i][k], gr[j][k]);
      a[3][r] = a[3][r] - c * cprod(n[i], u[j]) - c * cprod(n[j], u[i]);
      if (P) {
        a[4][r] = a[4][r] + c * cprod(p, gr[i][j] + gr[j][i]);
        if (r == 1) a[5][r] = a[5][r] - c * (cprod(p, u[1]) + cprod(u[1], p));
        if (r == 3) a[5][r] = a[5][r] - c * cprod(p, u[0]);
        if (r == 4) a[5][r] = a[5][r] - c * cprod(p, u[2]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kTkeTerms; ++q)
#pragma unroll
    for (int r = 0; r < 6; ++r) acc[(size_t)(q * 6 + r) * S + t] += a[q][r];
}

}  // namespace

size_t tke_z_smem(int nzd) { return 2 * (size_t)pad32_size(nzd) * sizeof(double2); }
size_t tke_x_smem(int nxd) { return (3 * (size_t)pad32_size(4 * nxd) + pad32_size(3 * nxd)) * sizeof(double2); }

cudaError_t tke_set_smem_limits(int nzd, int nxd) {
  cudaError_t e = cudaFuncSetAttribute(k_tke_zinv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tke_z_smem(nzd));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tke_zfwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tke_z_smem(nzd));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tke_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tke_x_smem(nxd));
  return e;
}

void launch_tke_snapshot(const TkeLaunch& L, cudaStream_t s) {
  const Dims& d = L.d;
  const size_t per_c = (size_t)d.nplanes * d.nmodes;
  k_tke_prep<<<(unsigned)((3 * per_c + 255) / 256), 256, 0, s>>>(L.V, L.W, L.mean, d);
  if (L.P) k_tke_pmean<<<(d.nplanes + 127) / 128, 128, 0, s>>>(L.P, L.mean + 2 * d.nplanes, d);
  launch_gradients(L.W, L.W + 3 * per_c, L.der, L.d0lu, L.bc, d, s);
  const int nxp = d.nx + 1;
  for (int p0 = 0; p0 < d.nplanes; p0 += L.chunk) {
    const int C = d.nplanes - p0 < L.chunk ? d.nplanes - p0 : L.chunk;
    k_tke_zinv<<<dim3(nxp, C, 12), 256, tke_z_smem(d.nzd), s>>>(L.W, L.Zt, L.twz, d, L.rz, p0, L.chunk);
    k_tke_x<<<dim3(d.nzd, C), 256, tke_x_smem(d.nxd), s>>>(L.Zt, L.Xt, L.twx, L.twh, d, L.rx, 0.5 * d.factor,
                                                          L.chunk);
    k_tke_zfwd<<<dim3(nxp, C, 3), 256, tke_z_smem(d.nzd), s>>>(L.Xt, L.N3, L.twz, d, L.rz, p0, L.chunk);
  }
  const int S = d.nplanes * d.nzt;
  k_tke_accum<<<(S + 127) / 128, 128, 0, s>>>(L.W, L.N3, L.P, L.acc, L.mean + 3 * d.nplanes, d);
}

}  // namespace chgpu
