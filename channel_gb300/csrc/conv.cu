// The nonlinear terms of every y-plane: `convolutions` of the reference
// (dnsdata.f90:487-602) as three batched shared-memory FFT kernels.
//
//   k_zinv : z-backward transform of u,v,w per (plane, column kx), with the
//            3/2 zero band inserted while loading (dnsdata.f90:504-510).
//            Writes Zb[c][plane][ix][jz] (physical z, spectral x).
//   k_xrow : per (plane, rows jz): c2r in x of u,v,w (dnsdata.f90:533-535,
//            real-to-complex packing into half-length transforms), the CFL
//            maximum (:552-556), the six products times `factor`
//            (:581-584), r2c of the products keeping kx<=nx (:586) -- the
//            z<->x pencil transposes (mpi_transpose.f90:50-117) are the
//            strided loads/stores of this kernel.  Writes Pb[p][plane][ix][jz].
//   k_zfwd : z-forward transform of the six products per (plane, column),
//            keeping |kz|<=nz (:590, truncation read by buildrhs :609).
//            Writes VV[p][plane][mode].
//
// T is the arithmetic type: double (plain FP64 step) or float (mixed step).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "chgpu_internal.h"
#include "cplx.cuh"
#include "kernels.cuh"
#include "async.cuh"

namespace chgpu {

// c2r packing term (X_k + conj X_{M-k}) + i (X_k - conj X_{M-k}) conj(w_k):
// the product and the sum as four fused multiply-adds (FP64 and FP32);
// double-float through its complex operations
template <typename V2> __device__ __forceinline__ V2 c2r_pack(V2 xk, V2 xm, V2 w) {
  const V2 e = xk + xm, d = xk - xm;
  if constexpr (std::is_same<V2, cdd>::value) {
    return e + mul_is<+1>(cmul_s<+1>(d, w));
  } else {
    return mk<V2>(fma(d.x, w.y, fma(-d.y, w.x, e.x)), fma(d.y, w.y, fma(d.x, w.x, e.y)));
  }
}

__device__ __forceinline__ void block_max_atomic(double v, double* target) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double wmax[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wmax[wid] = (double)v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = wmax[i] > m ? wmax[i] : m;
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(target), (unsigned long long)__double_as_longlong(m));
  }
}

// an FP32 pair of the closure's stresses in the transform type
template <typename V2> __device__ __forceinline__ V2 tau2(float2 t);
template <> __device__ __forceinline__ double2 tau2<double2>(float2 t) { return make_double2(t.x, t.y); }
template <> __device__ __forceinline__ float2 tau2<float2>(float2 t) { return t; }
template <> __device__ __forceinline__ cdd tau2<cdd>(float2 t) { return cdd{dd(t.x), dd(t.y)}; }

// MINB: resident 256-thread blocks per SM the register allocation is capped
// for (the autotuner picks the variant and the rows per block together)
// TAU: the closure's subgrid stresses tau[p][plane][jz][x] (FP32, physical,
// x pairs packed like the transform) are added to the six products.
template <typename T, int MINB, bool TAU = false>
__global__ void __launch_bounds__(256, MINB) k_xrow(const typename C2<T>::t* __restrict__ Zb, typename C2<T>::t* __restrict__ Pb,
                                              const typename C2<T>::t* __restrict__ twx,
                                              const typename C2<T>::t* __restrict__ twh, const T* __restrict__ cst,
                                              Dims d, RadixDev rx, int nrows, int plane0, int compute_cfl,
                                              DevScalars* sc, const float2* __restrict__ tau) {
  using V2 = typename C2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = d.nxd, nx = d.nx, nxp = nx + 1, nzd = d.nzd;
  const int plane = plane0 + blockIdx.y;
  const int jz0 = blockIdx.x * nrows;
  const int S = 3 * nrows * M;  // one buffer group: [3][nrows][M]
  const int lgr = __ffs(nrows) - 1;  // nrows is 1, 2 or 4
  const FastDiv by_M(M), by_nxp(nxp);
  V2* A = reinterpret_cast<V2*>(smem_raw);
  V2* B = A + pad32_size(S);
  V2* Cb = B + pad32_size(S);
  // load the three spectra rows (zTOx, x zero band; dnsdata.f90:533-535)
  for (int idx = threadIdx.x; idx < 3 * M * nrows; idx += blockDim.x) {
    const int r = idx & (nrows - 1);
    const int ck = idx >> lgr;
    const int c = by_M.div(ck);
    const int k = ck - c * M;
    V2 val = czero<V2>();
    if (k <= nx) val = Zb[(((size_t)c * d.nplanes + plane) * nxp + k) * nzd + jz0 + r];
    Cb[pad32((c * nrows + r) * M + k)] = val;
  }
  __syncthreads();
  // c2r packing: Z[k] = (X[k]+conj(X[M-k])) + i (X[k]-conj(X[M-k])) e^{+i pi k/M}
  for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
    const int cr = by_M.div(idx);
    const int k = idx - cr * M;
    V2 xk = Cb[pad32(cr * M + k)];
    V2 xm = czero<V2>();
    if (k == 0) xk.y = T();  // the c2r reads only Re of the kx=0 entry
    else xm = conjg(Cb[pad32(cr * M + M - k)]);
    A[pad32(idx)] = c2r_pack(xk, xm, twh[k]);
  }
  __syncthreads();
  V2* U = fft_block<+1, V2, true>(A, B, 3 * nrows, rx, twx);
  V2* freeb = (U == A) ? B : A;
  // CFL (dnsdata.f90:552-556) and products uu,vv,ww (:584); their factor
  // (:581-584) is applied in the r2c unpacking below (the transform is linear)
  const T g = cst[0];  // factor / 2
  T cfl = T();
  bool bad = false;
  const bool do_cfl = compute_cfl && plane >= 2 && plane <= d.ny;
  const T rdx = cst[1], rdz = cst[2];
  const T rdy = do_cfl ? cst[3 + plane] : T();
  for (int idx = threadIdx.x; idx < nrows * M; idx += blockDim.x) {
    const int r = by_M.div(idx), m = idx - r * M;
    V2 u = U[pad32((0 * nrows + r) * M + m)];
    V2 v = U[pad32((1 * nrows + r) * M + m)];
    V2 w = U[pad32((2 * nrows + r) * M + m)];
    if (do_cfl) {
      using N = Num<T>;
      T c0 = N::abs(u.x) * rdx + N::abs(v.x) * rdy + N::abs(w.x) * rdz;
      T c1 = N::abs(u.y) * rdx + N::abs(v.y) * rdy + N::abs(w.y) * rdz;
      cfl = N::max(cfl, N::max(c0, c1));
      bad = bad || !N::finite(c0) || !N::finite(c1);
    }
    V2 puu = mk<V2>(u.x * u.x, u.y * u.y), pvv = mk<V2>(v.x * v.x, v.y * v.y), pww = mk<V2>(w.x * w.x, w.y * w.y);
    if constexpr (TAU) {
      const size_t tb = ((size_t)plane * nzd + jz0 + r) * M + m, ts = (size_t)d.nplanes * nzd * M;
      puu = puu + tau2<V2>(tau[tb]);
      pvv = pvv + tau2<V2>(tau[tb + ts]);
      pww = pww + tau2<V2>(tau[tb + 2 * ts]);
    }
    Cb[pad32((0 * nrows + r) * M + m)] = puu;
    Cb[pad32((1 * nrows + r) * M + m)] = pvv;
    Cb[pad32((2 * nrows + r) * M + m)] = pww;
  }
  if (bad) cfl = T((float)INFINITY);  // a non-finite velocity shows up as an infinite CFL
  if (compute_cfl) block_max_atomic(Num<T>::to_double(cfl), &sc->cfl);
  __syncthreads();
  for (int half = 0; half < 2; ++half) {
    if (half == 1) {  // products uv, vw, uw (dnsdata.f90:581-583)
      for (int idx = threadIdx.x; idx < nrows * M; idx += blockDim.x) {
        const int r = by_M.div(idx), m = idx - r * M;
        V2 u = U[pad32((0 * nrows + r) * M + m)];
        V2 v = U[pad32((1 * nrows + r) * M + m)];
        V2 w = U[pad32((2 * nrows + r) * M + m)];
        V2 puv = mk<V2>(u.x * v.x, u.y * v.y), pvw = mk<V2>(v.x * w.x, v.y * w.y), puw = mk<V2>(u.x * w.x, u.y * w.y);
        if constexpr (TAU) {
          const size_t tb = ((size_t)plane * nzd + jz0 + r) * M + m, ts = (size_t)d.nplanes * nzd * M;
          puv = puv + tau2<V2>(tau[tb + 3 * ts]);
          pvw = pvw + tau2<V2>(tau[tb + 4 * ts]);
          puw = puw + tau2<V2>(tau[tb + 5 * ts]);
        }
        Cb[pad32((0 * nrows + r) * M + m)] = puv;
        Cb[pad32((1 * nrows + r) * M + m)] = pvw;
        Cb[pad32((2 * nrows + r) * M + m)] = puw;
      }
      __syncthreads();
    }
    V2* P = fft_block<-1, V2, true>(Cb, freeb, 3 * nrows, rx, twx);
    // r2c unpacking, kx = 0..nx (HFT + xTOz, dnsdata.f90:586-588)
    for (int idx = threadIdx.x; idx < 3 * nxp * nrows; idx += blockDim.x) {
      const int r = idx & (nrows - 1);
      const int pk = idx >> lgr;
      const int p = by_nxp.div(pk);
      const int k = pk - p * nxp;
      const int zb = (p * nrows + r) * M;
      V2 zk = P[pad32(zb + k)];
      V2 zm = conjg(P[pad32(zb + (k == 0 ? 0 : M - k))]);
      // X = factor (Z_k + conj Z_{M-k})/2 + (factor/2) w_k (-i)(Z_k - conj Z_{M-k}),
      // with the second table twh[2M + k] = (factor/2) w_k
      const V2 sm = zk + zm, df = zk - zm;
      const V2 w = twh[2 * M + k];
      // o = (-i) df = (df.y, -df.x); X = g sm + w o, fused
      V2 X;
      if constexpr (std::is_same<T, dd>::value) {
        X = scale(sm, g) + cmul(w, mk<V2>(df.y, T() - df.x));
      } else {
        X = mk<V2>(fma(g, sm.x, fma(w.x, df.y, w.y * df.x)), fma(g, sm.y, fma(w.y, df.y, -(w.x * df.x))));
      }
      Pb[(((size_t)(3 * half + p) * d.nplanes + plane) * nxp + k) * nzd + jz0 + r] = X;
    }
    __syncthreads();
    if (P != Cb) {  // keep Cb as the product buffer of the second half
      V2* t = Cb;
      Cb = P;
      freeb = t;
    }
  }
}


// x-inverse alone: the physical rows of ncomp fields after their z-inverse
// (the c2r of k_xrow), for the closure's velocity gradients.  Blocks:
// (groups of nrows z rows, planes, groups of 3 fields).  Writes
// out[c][plane][jz][m], the pairs x = 2m, 2m+1 packed as in the transform.
template <typename T>
__global__ void __launch_bounds__(256) k_xphys(const typename C2<T>::t* __restrict__ Zb, typename C2<T>::t* __restrict__ out,
                                               const typename C2<T>::t* __restrict__ twx,
                                               const typename C2<T>::t* __restrict__ twh, Dims d, RadixDev rx,
                                               int nrows, int plane0) {
  using V2 = typename C2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = d.nxd, nx = d.nx, nxp = nx + 1, nzd = d.nzd;
  const int plane = plane0 + blockIdx.y;
  const int jz0 = blockIdx.x * nrows;
  const int c0 = 3 * blockIdx.z;
  const int S = 3 * nrows * M;
  const int lgr = __ffs(nrows) - 1;
  const FastDiv by_M(M);
  V2* A = reinterpret_cast<V2*>(smem_raw);
  V2* B = A + pad32_size(S);
  V2* Cb = B + pad32_size(S);
  for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
    const int r = idx & (nrows - 1);
    const int ck = idx >> lgr;
    const int c = by_M.div(ck);
    const int k = ck - c * M;
    V2 val = czero<V2>();
    if (k <= nx) val = Zb[(((size_t)(c0 + c) * d.nplanes + plane) * nxp + k) * nzd + jz0 + r];
    Cb[pad32((c * nrows + r) * M + k)] = val;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
    const int cr = by_M.div(idx);
    const int k = idx - cr * M;
    V2 xk = Cb[pad32(cr * M + k)];
    V2 xm = czero<V2>();
    if (k == 0) xk.y = T();
    else xm = conjg(Cb[pad32(cr * M + M - k)]);
    A[pad32(idx)] = c2r_pack(xk, xm, twh[k]);
  }
  __syncthreads();
  V2* U = fft_block<+1, V2, true>(A, B, 3 * nrows, rx, twx);
  for (int idx = threadIdx.x; idx < S; idx += blockDim.x) {
    const int cr = by_M.div(idx), m = idx - cr * M;
    const int c = cr >> lgr, r = cr & (nrows - 1);
    out[(((size_t)(c0 + c) * d.nplanes + plane) * nzd + jz0 + r) * M + m] = U[pad32(idx)];
  }
}

// z-inverse of u, v, w per (plane, column group).  The block's columns of V
// are one contiguous run of complex doubles: one bulk copy brings them into
// the scratch buffer (sized for the raw columns when T is 8 bytes), the
// conversion pass places them with the 3/2 zero band in the padded layout.
template <typename T>
__global__ void __launch_bounds__(256) k_zinv(const double2* __restrict__ V, typename C2<T>::t* __restrict__ Zb,
                                              const typename C2<T>::t* __restrict__ twz, Dims d, RadixDev rz,
                                              int nb_cols, int plane0, int ix_lo, int ix_hi,
                                              DevScalars* __restrict__ sc) {
  using V2 = typename C2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar;
  const int nzd = d.nzd, nz = d.nz, nxp = d.nx + 1, nzt = d.nzt;
  V2* bufA = reinterpret_cast<V2*>(smem_raw);
  V2* bufB = bufA + pad32_size(nb_cols * nzd);
  const double2* raw = reinterpret_cast<const double2*>(bufB);
  const int c = blockIdx.z;
  const int plane = plane0 + blockIdx.y;
  const int ix0 = ix_lo + blockIdx.x * nb_cols;
  const int nb = min(nb_cols, ix_hi - ix0);
  const size_t colbase = ((size_t)c * d.nplanes + plane) * nxp;
  const unsigned bytes = (unsigned)((size_t)nb * nzt * sizeof(double2));
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) bulk_copy_g2s(const_cast<double2*>(raw), V + (colbase + ix0) * nzt, bytes, &bar);
  if (!mbar_wait(&bar, 0, sc->first_wait > 0 ? sc->first_wait - 1 : kBulkWaitPolls)) {
    if (threadIdx.x == 0) atomicOr(&sc->error, 2);
    mbar_wait(&bar, 0, kBulkWaitPolls);  // the copy in flight, with the full limit
    return;
  }
  const FastDiv by_nzd(nzd);
  for (int idx = threadIdx.x; idx < nb * nzd; idx += blockDim.x) {
    const int b = by_nzd.div(idx);
    const int jz = idx - b * nzd;
    V2 val = czero<V2>();
    int izp = -1;
    if (jz <= nz) izp = nz + jz;
    else if (jz >= nzd - nz) izp = jz - nzd + nz;
    if (izp >= 0) {
      const double2 x = raw[b * nzt + izp];
      val = mk<V2>(Num<T>::from_double(x.x), Num<T>::from_double(x.y));
    }
    bufA[pad32(idx)] = val;
  }
  __syncthreads();
  V2* res = fft_block<+1>(bufA, bufB, nb, rz, twz);
  V2* out = Zb + (colbase + ix0) * nzd;
  for (int idx = threadIdx.x; idx < nb * nzd; idx += blockDim.x) out[idx] = res[pad32(idx)];
}

template <typename T>
__global__ void __launch_bounds__(256) k_zfwd(const typename C2<T>::t* __restrict__ Pb, typename C2<T>::t* __restrict__ VV,
                                              const typename C2<T>::t* __restrict__ twz, Dims d, RadixDev rz,
                                              int nb_cols, int plane0, DevScalars* __restrict__ sc) {
  using V2 = typename C2<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar;
  const int nzd = d.nzd, nz = d.nz, nxp = d.nx + 1, nzt = d.nzt;
  V2* bufA = reinterpret_cast<V2*>(smem_raw);
  V2* bufB = bufA + pad32_size(nb_cols * nzd);
  const int p = blockIdx.z;
  const int plane = plane0 + blockIdx.y;
  const int ix0 = blockIdx.x * nb_cols;
  const int nb = min(nb_cols, nxp - ix0);
  const size_t colbase = ((size_t)p * d.nplanes + plane) * nxp;
  const V2* in = Pb + (colbase + ix0) * nzd;
  // the block's columns are one contiguous run of Pb (nzd even: 16-byte
  // aligned, a multiple of 16 bytes): one bulk copy into the scratch buffer,
  // then into the padded transform layout
  const unsigned bytes = (unsigned)((size_t)nb * nzd * sizeof(V2));
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) bulk_copy_g2s(bufB, in, bytes, &bar);
  if (!mbar_wait(&bar, 0, sc->first_wait > 0 ? sc->first_wait - 1 : kBulkWaitPolls)) {
    if (threadIdx.x == 0) atomicOr(&sc->error, 2);
    mbar_wait(&bar, 0, kBulkWaitPolls);  // the copy in flight, with the full limit
    return;
  }
  for (int idx = threadIdx.x; idx < nb * nzd; idx += blockDim.x) bufA[pad32(idx)] = bufB[idx];
  __syncthreads();
  V2* res = fft_block<-1>(bufA, bufB, nb, rz, twz);
  const FastDiv by_nzt(nzt);
  for (int idx = threadIdx.x; idx < nb * nzt; idx += blockDim.x) {
    const int b = by_nzt.div(idx);
    const int izp = idx - b * nzt;
    const int iz = izp - nz;
    const int jz = iz >= 0 ? iz : nzd + iz;
    VV[(colbase + ix0 + b) * nzt + izp] = res[pad32(b * nzd + jz)];
  }
}

size_t conv_z_smem(int zcols, int nzd, size_t ts) { return 2 * (size_t)pad32_size(zcols * nzd) * ts; }
size_t conv_zinv_smem(int zcols, int nzd, int nzt, size_t ts) {
  const size_t buf = (size_t)pad32_size(zcols * nzd) * ts;
  return buf + std::max(buf, (size_t)zcols * nzt * sizeof(double2));
}
size_t conv_x_smem(int xrows, int nxd, size_t ts) { return 3 * (size_t)pad32_size(3 * xrows * nxd) * ts; }

template <typename T>
void launch_convolutions(const ConvLaunch& L, cudaStream_t s, int stage) {
  using V2 = typename C2<T>::t;
  const Dims& d = L.d;
  const int nxp = d.nx + 1;
  // lengths with a register-blocked plan (the closure's stresses go through
  // the x-row kernel below)
  if ((stage == 1 ? (L.xfast && !L.tau) : L.zfast) && launch_convolutions_r<T>(L, s, stage)) return;
  if (stage == 0) {
    const int ncol = L.ix_hi - L.ix_lo;
    dim3 grid((ncol + L.zcols - 1) / L.zcols, L.nplanes, 3);
    size_t sm = conv_zinv_smem(L.zcols, d.nzd, d.nzt, sizeof(V2));
    k_zinv<T><<<grid, L.zthreads, sm, s>>>(L.V, (V2*)L.Zb, (const V2*)L.twz, d, L.rz, L.zcols, L.plane0, L.ix_lo,
                                           L.ix_hi, L.sc);
  }
  if (stage == 1) {
    dim3 grid(d.nzd / L.xrows, L.nplanes);
    size_t sm = conv_x_smem(L.xrows, d.nxd, sizeof(V2));
    auto kern = L.tau ? k_xrow<T, 2, true> : L.xminb == 1 ? k_xrow<T, 1> : L.xminb == 3 ? k_xrow<T, 3> : k_xrow<T, 2>;
    kern<<<grid, L.xthreads, sm, s>>>((const V2*)L.Zb, (V2*)L.Pb, (const V2*)L.twx, (const V2*)L.twh, (const T*)L.cst, d, L.rx,
                               L.xrows, L.plane0, L.compute_cfl, L.sc, L.tau);
  }
  if (stage == 2) {
    dim3 grid((nxp + L.zcols - 1) / L.zcols, L.nplanes, 6);
    size_t sm = conv_z_smem(L.zcols, d.nzd, sizeof(V2));
    k_zfwd<T><<<grid, L.zthreads, sm, s>>>((const V2*)L.Pb, (V2*)L.VV, (const V2*)L.twz, d, L.rz, L.zcols, L.plane0,
                                           L.sc);
  }
}

// z-inverse and x-inverse of ncomp (a multiple of 3) fields in the field
// layout, FP32, all planes: src [c][plane][mode] -> zb -> out [c][plane][jz][m]
void launch_physical_fields(const double2* src, int ncomp, float2* zb, float2* out, const float2* twz,
                            const float2* twx, const float2* twh, const Dims& d, const RadixDev& rz,
                            const RadixDev& rx, int zcols, int xrows, DevScalars* sc, cudaStream_t s) {
  const int nxp = d.nx + 1;
  dim3 gz((nxp + zcols - 1) / zcols, d.nplanes, ncomp);
  k_zinv<float><<<gz, 256, conv_zinv_smem(zcols, d.nzd, d.nzt, sizeof(float2)), s>>>(src, zb, twz, d, rz, zcols, 0, 0,
                                                                                      nxp, sc);
  dim3 gx(d.nzd / xrows, d.nplanes, ncomp / 3);
  k_xphys<float><<<gx, 256, conv_x_smem(xrows, d.nxd, sizeof(float2)), s>>>(zb, out, twx, twh, d, rx, xrows, 0);
}

template void launch_convolutions<double>(const ConvLaunch&, cudaStream_t, int);
template void launch_convolutions<float>(const ConvLaunch&, cudaStream_t, int);
template void launch_convolutions<dd>(const ConvLaunch&, cudaStream_t, int);

namespace {
template <typename K>
cudaError_t allow_max_smem(K* kernel, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}
}  // namespace

cudaError_t conv_set_smem_limits() {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if ((e = allow_max_smem(k_zinv<double>, optin))) return e;
  if ((e = allow_max_smem(k_zinv<float>, optin))) return e;
  if ((e = allow_max_smem(k_zinv<dd>, optin))) return e;
  if ((e = allow_max_smem(k_zfwd<double>, optin))) return e;
  if ((e = allow_max_smem(k_zfwd<float>, optin))) return e;
  if ((e = allow_max_smem(k_zfwd<dd>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<double, 1>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<double, 2>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<double, 3>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<float, 1>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<float, 2>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<float, 3>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<dd, 1>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<dd, 2>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<dd, 3>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<double, 2, true>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<float, 2, true>, optin))) return e;
  if ((e = allow_max_smem(k_xrow<dd, 2, true>, optin))) return e;
  if ((e = allow_max_smem(k_xphys<float>, optin))) return e;
  if ((e = convr_set_smem_limits<float>())) return e;
  if ((e = convr_set_smem_limits<double>())) return e;
  return convr_set_smem_limits<dd>();
}

}  // namespace chgpu
