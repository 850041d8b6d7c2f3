// Physical-space export of the field: the un-dealiased transform of the
// reference's exporter (out_exporter/out2bin.f90:141-203) on the device.
//
// For each y-plane iy = 0..ny and component c:
//   z pass  (k_export_z): the 2nz+1 spanwise modes of every kx, in FFT order
//           (kz = 0..nz, -nz..-1, out2bin.f90:169-170), after the optional
//           removal of the mean mode (:151-153) and the spanwise filter
//           (filter_vfield, :338-347), go through the unnormalised exp(+i)
//           DFT of length Nz = 2nz+1 (:172);
//   x pass  (k_export_x): per physical z index l, the nx+1 values X_kx give
//           the real signal of odd length Nx = 2nx+1 by the c2r rule
//           u_j = Re X_0 + 2 Re sum_{k=1..nx} X_k e^{+2 pi i jk/Nx} (:184);
//           two l columns share one complex transform (a + i b holds both
//           Hermitian spectra);
//   sample  (k_export_interp): the nxtot x nztot output grid of
//           xz_interpolation (:236-275), written as vec(3, nxtot, 0:ny, nztot)
//           in Fortran order, i.e. [zz][iy][xx][c] with c fastest.
// Nx and Nz are odd and may have any prime factors, so the transforms are
// Stockham stages of arbitrary radix p: each output of a stage is a length-p
// DFT whose inner and inter-stage twiddles combine into one power of the
// length-n root (w_{Ns p}^{r (k + q Ns)}), read from a table of the n roots.
#include <cuda_runtime.h>

#include <algorithm>

#include "cplx.cuh"
#include "kernels.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ double2 cfma(double2 acc, double2 a, double2 w) {
  return make_double2(fma(a.x, w.x, fma(-a.y, w.y, acc.x)), fma(a.x, w.y, fma(a.y, w.x, acc.y)));
}

// One Stockham stage of radix p over B transforms of length n held
// contiguously in src; results to dst.  Ns = product of the earlier radices.
// sign > 0: exp(+i); tw = forward roots exp(-2 pi i m/n).
__device__ void stage_any(const double2* __restrict__ src, double2* __restrict__ dst, int B, int n, int p, int Ns,
                          int sign, const double2* __restrict__ tw) {
  const int nb = n / p;
  const int twstep = n / (Ns * p);
  const FastDiv by_n(n), by_nb(nb), by_Ns(Ns);
  for (int item = threadIdx.x; item < B * n; item += blockDim.x) {
    const int t = by_n.div(item);
    const int rem = item - t * n;
    const int q = by_nb.div(rem);
    const int j = rem - q * nb;
    const int k = j - by_Ns.div(j) * Ns;
    const int e = (k + q * Ns) * twstep;  // < n
    const double2* s = src + (size_t)t * n + j;
    double2 acc = s[0];
    int idx = 0;
    for (int r = 1; r < p; ++r) {
      idx += e;
      if (idx >= n) idx -= n;
      double2 w = __ldg(tw + idx);
      if (sign > 0) w.y = -w.y;
      acc = cfma(acc, s[(size_t)r * nb], w);
    }
    dst[(size_t)t * n + (size_t)(j - k) * p + k + (size_t)q * Ns] = acc;
  }
}

// B transforms of length rad.n in a (b is scratch of the same size); returns
// the buffer holding the result.  Every thread of the block calls it.
__device__ double2* fft_any(double2* a, double2* b, int B, const RadixDev& rad, int sign,
                            const double2* __restrict__ tw) {
  int Ns = 1;
  for (int st = 0; st < rad.nst; ++st) {
    stage_any(a, b, B, rad.n, rad.r[st], Ns, sign, tw);
    __syncthreads();
    double2* t = a;
    a = b;
    b = t;
    Ns *= rad.r[st];
  }
  return a;
}

__device__ __forceinline__ bool mode_dropped(const ExportLaunch& L, int ix, int iz) {
  if (L.fluct_only && ix == 0 && iz == 0) return true;
  if (L.part == 0) return false;
  const double k = fabs(L.beta0 * (double)iz);
  const double thr = (double)L.z_threshold;
  return (k <= thr && L.part == 2) || (k > thr && L.part == 1);
}

// grid (ceil((nx+1)/zcols), planes of the chunk, 3); W[c][iy-iy0][ix][l]
__global__ void __launch_bounds__(256) k_export_z(ExportLaunch L, int iy0) {
  extern __shared__ double2 smem[];
  const int Nz = L.rz.n, nz = L.d.nz, nx1 = L.d.nx + 1;
  const int ix0 = blockIdx.x * L.zcols;
  const int nb = min(L.zcols, nx1 - ix0);
  const int iy = iy0 + blockIdx.y, c = blockIdx.z;
  double2* a = smem;
  double2* b = smem + (size_t)L.zcols * Nz;
  const double2* row = L.V + ((size_t)c * L.d.nplanes + (iy + 1)) * L.d.nmodes;
  const FastDiv by_Nz(Nz);
  for (int e = threadIdx.x; e < nb * Nz; e += blockDim.x) {
    const int t = by_Nz.div(e);
    const int pos = e - t * Nz;
    const int iz = pos <= nz ? pos : pos - Nz;
    const int ix = ix0 + t;
    a[e] = mode_dropped(L, ix, iz) ? make_double2(0.0, 0.0) : row[(size_t)ix * Nz + iz + nz];
  }
  __syncthreads();
  const double2* r = fft_any(a, b, nb, L.rz, +1, L.twz);
  double2* w = L.W + (((size_t)c * L.chunk + blockIdx.y) * nx1 + ix0) * Nz;
  for (int e = threadIdx.x; e < nb * Nz; e += blockDim.x) w[e] = r[e];
}

// grid (ceil(Nz/(2 xpairs)), planes of the chunk, 3); P[c][iy-iy0][l][j]
__global__ void __launch_bounds__(256) k_export_x(ExportLaunch L) {
  extern __shared__ double2 smem[];
  const int Nx = L.rx.n, Nz = L.rz.n, nx1 = L.d.nx + 1, nx = L.d.nx;
  const int P = L.xpairs, Q = 2 * P;
  const int l0 = blockIdx.x * Q;
  const int np = min(P, (Nz - l0 + 1) / 2);
  const int c = blockIdx.z;
  double2* S = smem;                      // staged X[kx][q], (nx+1) x 2P
  double2* a = smem + (size_t)Q * nx1;    // P transforms of length Nx
  double2* b = a + (size_t)P * Nx;
  const double2* w = L.W + ((size_t)c * L.chunk + blockIdx.y) * nx1 * (size_t)Nz;
  for (int e = threadIdx.x; e < nx1 * Q; e += blockDim.x) {
    const int kx = e / Q, q = e - kx * Q, l = l0 + q;
    S[e] = l < Nz ? w[(size_t)kx * Nz + l] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  // Z_k = A_k + i B_k over the Hermitian extensions of columns 2t and 2t+1
  const FastDiv by_Nx(Nx);
  for (int e = threadIdx.x; e < np * Nx; e += blockDim.x) {
    const int t = by_Nx.div(e);
    const int k = e - t * Nx;
    double2 z;
    if (k == 0) {
      z = make_double2(S[2 * t].x, S[2 * t + 1].x);
    } else if (k <= nx) {
      const double2 xa = S[k * Q + 2 * t], xb = S[k * Q + 2 * t + 1];
      z = make_double2(xa.x - xb.y, xa.y + xb.x);
    } else {
      const double2 xa = S[(Nx - k) * Q + 2 * t], xb = S[(Nx - k) * Q + 2 * t + 1];
      z = make_double2(xa.x + xb.y, xb.x - xa.y);
    }
    a[e] = z;
  }
  __syncthreads();
  const double2* r = fft_any(a, b, np, L.rx, +1, L.twx);
  double* out = L.P + ((size_t)c * L.chunk + blockIdx.y) * (size_t)Nz * Nx;
  for (int e = threadIdx.x; e < np * Nx; e += blockDim.x) {
    const int t = by_Nx.div(e);
    const int j = e - t * Nx;
    const int l = l0 + 2 * t;
    out[(size_t)l * Nx + j] = r[e].x;
    if (l + 1 < Nz) out[(size_t)(l + 1) * Nx + j] = r[e].y;
  }
}

// Fortran index map and weights of xz_interpolation, in the reference's
// precisions: the ratio in real*4 (:296), the weights in real*8 (:250-263).
struct Tap {
  int c, f;  // 0-based, wrapped onto the periodic grid
  double wc, wf;
};
__device__ __forceinline__ Tap tap(int n_full, int n_tot, int i1) {
  const float s = __fdiv_rn((float)n_full, (float)n_tot);
  const double prj = (double)__fadd_rn(__fmul_rn(s, __fsub_rn((float)i1, 1.0f)), 1.0f);
  const int c = (int)ceil(prj), f = (int)floor(prj);
  Tap t;
  if (c == f) {
    t.wc = 0.5;
    t.wf = 0.5;
  } else {
    const double d = (double)(c - f);
    t.wc = fabs((double)(float)f - prj) / d;
    t.wf = fabs((double)(float)c - prj) / d;
  }
  t.c = (c - 1) % n_full;
  t.f = (f - 1) % n_full;
  return t;
}

// one thread per output value; out holds planes iy0..iy0+chunk-1 as
// [zz][iy-iy0][xx][c]
__global__ void __launch_bounds__(256) k_export_interp(ExportLaunch L, int nplanes_chunk) {
  const size_t total = (size_t)L.nztot * nplanes_chunk * L.nxtot * 3;
  const int Nx = L.rx.n, Nz = L.rz.n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % 3);
    size_t r = e / 3;
    const int xx = (int)(r % L.nxtot);
    r /= L.nxtot;
    const int iy = (int)(r % nplanes_chunk);
    const int zz = (int)(r / nplanes_chunk);
    const Tap tx = tap(Nx, L.nxtot, xx + 1), tz = tap(Nz, L.nztot, zz + 1);
    const double* u = L.P + ((size_t)c * L.chunk + iy) * (size_t)Nz * Nx;
    const double ucc = u[(size_t)tz.c * Nx + tx.c], uff = u[(size_t)tz.f * Nx + tx.f];
    const double ucf = u[(size_t)tz.f * Nx + tx.c], ufc = u[(size_t)tz.c * Nx + tx.f];
    const double wcc = __dmul_rn(tx.wc, tz.wc), wff = __dmul_rn(tx.wf, tz.wf);
    const double wcf = __dmul_rn(tx.wc, tz.wf), wfc = __dmul_rn(tx.wf, tz.wc);
    double v = __dmul_rn(ucc, wcc);
    v = __dadd_rn(v, __dmul_rn(uff, wff));
    v = __dadd_rn(v, __dmul_rn(ufc, wfc));
    v = __dadd_rn(v, __dmul_rn(ucf, wcf));
    L.out[e] = v;
  }
}

}  // namespace

size_t export_z_smem(int zcols, int Nz) { return (size_t)2 * zcols * Nz * sizeof(double2); }
size_t export_x_smem(int xpairs, int nx, int Nx) {
  return ((size_t)2 * xpairs * (nx + 1) + (size_t)2 * xpairs * Nx) * sizeof(double2);
}

int export_set_smem_limits() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
  cudaFuncAttributes fz, fx;
  if (cudaFuncGetAttributes(&fz, k_export_z) != cudaSuccess || cudaFuncGetAttributes(&fx, k_export_x) != cudaSuccess)
    return -1;
  const int lim = optin - (int)std::max(fz.sharedSizeBytes, fx.sharedSizeBytes);
  if (cudaFuncSetAttribute(k_export_z, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess ||
      cudaFuncSetAttribute(k_export_x, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess)
    return -1;
  return lim;
}

void launch_export_chunk(const ExportLaunch& L, int iy0, int nplanes_chunk, cudaStream_t s) {
  const int nx1 = L.d.nx + 1, Nz = L.rz.n, Nx = L.rx.n;
  k_export_z<<<dim3((nx1 + L.zcols - 1) / L.zcols, nplanes_chunk, 3), 256, export_z_smem(L.zcols, Nz), s>>>(L, iy0);
  k_export_x<<<dim3((Nz + 2 * L.xpairs - 1) / (2 * L.xpairs), nplanes_chunk, 3), 256,
               export_x_smem(L.xpairs, L.d.nx, Nx), s>>>(L);
  const size_t total = (size_t)L.nztot * nplanes_chunk * L.nxtot * 3;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)152 * 16);
  k_export_interp<<<blocks, 256, 0, s>>>(L, nplanes_chunk);
}

}  // namespace chgpu
