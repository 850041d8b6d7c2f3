// The three transform kernels of `convolutions` (dnsdata.f90:487-602) for
// the transform lengths with a compile-time register-blocked plan
// (rfft.cuh): the same work as k_zinv / k_xrow / k_zfwd in conv.cu, which
// remain the kernels of every other length.
//
//   k_zinv_r : one group of TPR threads per (plane, component, column kx):
//              the column's 2nz+1 modes are loaded straight into registers
//              in the transform's input distribution (consecutive threads,
//              consecutive modes: coalesced), the 3/2 zero band is left
//              zero (dnsdata.f90:504-510), the backward z transform runs in
//              registers and the last pass writes the physical-z column to
//              Zb[c][plane][ix][jz] (consecutive jz per thread group).
//   k_xrow_r : one group per plane row jz, NR rows per block.  The block
//              stages its rows' spectra (Zb[c][plane][kx][jz0..jz0+NR-1],
//              NR consecutive values per kx: the zTOx transpose of
//              mpi_transpose.f90:50-117) through shared memory with
//              coalesced loads; each group packs its row for the
//              half-length c2r (dnsdata.f90:533-535), transforms u, v, w,
//              keeps them in shared memory, forms the six products
//              (:581-584) and the CFL maximum (:552-556), transforms each
//              product forward, unpacks kx = 0..nx (:586-588); the block then
//              writes the products' rows back transposed (xTOz) with
//              coalesced stores to Pb[p][plane][kx][jz].
//   k_zfwd_r : one group per (plane, product, column): the column of Pb in
//              registers, the forward z transform, the last pass storing
//              only |kz| <= nz (:590) into VV[p][plane][mode].
//
// T: double (FP64 step), float (mixed step) or dd (double-float step); one
// translation unit per type (convf_f32.cu, convf_f64.cu, convf_dd.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "chgpu_internal.h"
#include "cplx.cuh"
#include "kernels.cuh"
#include "rfft.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ void rblock_max_atomic(double v, double* target) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double wmax[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wmax[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = wmax[i] > m ? wmax[i] : m;
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(target), (unsigned long long)__double_as_longlong(m));
  }
}

// blocks of the z kernels: 256 threads, at most 32 columns
template <int TPR> constexpr int z_cols() { return (256 / TPR) < 32 ? (256 / TPR) : 32; }
// shared memory per x row: u, v (and w without WREG) in physical space,
// the padded exchange buffer, one bank shift
template <int M, int TPR, bool WREG> constexpr int x_row_stride() { return (WREG ? 3 : 4) * M + TPR + 1; }
// rows per x block: as many as keep the block's shared memory within 74 KB
// with w in registers (three resident blocks per SM) or 102 KB without (two),
// at least one warp, at most 256 threads
template <int M, int TPR, bool WREG, int S> constexpr int x_rows() {
  int nr = 32;
  const int budget = (WREG ? 74 : 102) * 1024;
  while (nr > 1 && (nr * x_row_stride<M, TPR, WREG>() * S > budget || nr * TPR > 256)) nr /= 2;
  while (nr * TPR < 32) nr *= 2;
  return nr;
}
// resident blocks per SM the x-row kernel's registers are capped for: as
// many as its shared memory lets share an SM (1 KB reserved per block), at
// most CAP (tiles x-row variant 4: 3, variant 5: 4; the autotuner times both)
template <int M, int TPR, bool WREG, int S, int CAP> constexpr int x_minb() {
  if (!WREG) return 1;  // no register cap: two blocks' shared memory set the residency
  const int bytes = x_rows<M, TPR, WREG, S>() * x_row_stride<M, TPR, WREG>() * S + 1024;
  const int by_smem = 233472 / bytes;
  const int b = by_smem < CAP ? by_smem : CAP;
  return b < 1 ? 1 : b;
}

}  // namespace

template <typename T, int E, int TPR, int NC>
__global__ void __launch_bounds__(NC * TPR) k_zinv_r(const double2* __restrict__ V, typename C2<T>::t* __restrict__ Zb,
                                                     const typename C2<T>::t* __restrict__ tw, Dims d, int plane0,
                                                     int ix_lo, int ix_hi) {
  using V2 = typename C2<T>::t;
  constexpr int N = E * TPR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V2* buf = reinterpret_cast<V2*>(smem_raw) + (threadIdx.x / TPR) * rbuf_size<E, TPR>();
  const int t = threadIdx.x % TPR;
  const int c = blockIdx.z, plane = plane0 + blockIdx.y;
  const int ix = ix_lo + blockIdx.x * NC + (int)(threadIdx.x / TPR);
  const bool active = ix < ix_hi;
  const int nz = d.nz, nzt = d.nzt;
  const size_t col = ((size_t)c * d.nplanes + plane) * (d.nx + 1) + (active ? ix : ix_lo);
  const double2* src = V + col * nzt;
  V2 a[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int jz = t + TPR * e;
    const int izp = jz <= nz ? nz + jz : (jz >= N - nz ? jz - N + nz : -1);
    V2 v = czero<V2>();
    if (active && izp >= 0) {
      const double2 x = __ldg(src + izp);
      v = mk<V2>(Num<T>::from_double(x.x), Num<T>::from_double(x.y));
    }
    a[e] = v;
  }
  V2* dst = Zb + col * N;
  rfft<E, TPR, +1>(a, buf, t, tw, [&](int o, V2 v) {
    if (active) dst[o] = v;
  });
}

template <typename T, int E, int TPR, int NC>
__global__ void __launch_bounds__(NC * TPR) k_zfwd_r(const typename C2<T>::t* __restrict__ Pb,
                                                     typename C2<T>::t* __restrict__ VV,
                                                     const typename C2<T>::t* __restrict__ tw, Dims d, int plane0) {
  using V2 = typename C2<T>::t;
  constexpr int N = E * TPR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V2* buf = reinterpret_cast<V2*>(smem_raw) + (threadIdx.x / TPR) * rbuf_size<E, TPR>();
  const int t = threadIdx.x % TPR;
  const int p = blockIdx.z, plane = plane0 + blockIdx.y;
  const int nxp = d.nx + 1;
  const int ix = blockIdx.x * NC + (int)(threadIdx.x / TPR);
  const bool active = ix < nxp;
  const int nz = d.nz, nzt = d.nzt;
  const size_t col = ((size_t)p * d.nplanes + plane) * nxp + (active ? ix : 0);
  const V2* src = Pb + col * N;
  V2 a[E];
#pragma unroll
  for (int e = 0; e < E; ++e) a[e] = active ? ldg_v(src + t + TPR * e) : czero<V2>();
  V2* dst = VV + col * nzt + nz;
  rfft<E, TPR, -1>(a, buf, t, tw, [&](int o, V2 v) {
    if (!active) return;
    if (o <= nz) dst[o] = v;
    else if (o >= N - nz) dst[o - N] = v;
  });
}

// Row layout in shared memory: u and v in physical space (M each), then the
// padded exchange buffer X (M + TPR), which first holds the row's w
// spectrum; without WREG w's physical values take a third slot before X.  With WREG w stays in registers after its transform: the last pass
// leaves each thread exactly the elements the products' forward transforms
// start from, so only u and v need shared memory.
template <typename T, int E, int TPR, int NR, int MINB, bool WREG>
__global__ void __launch_bounds__(NR * TPR, MINB) k_xrow_r(const typename C2<T>::t* __restrict__ Zb,
                                                           typename C2<T>::t* __restrict__ Pb,
                                                           const typename C2<T>::t* __restrict__ tw,
                                                           const typename C2<T>::t* __restrict__ twh,
                                                           const T* __restrict__ cst, Dims d, int plane0,
                                                           int compute_cfl, DevScalars* sc) {
  using V2 = typename C2<T>::t;
  constexpr int M = E * TPR;
  constexpr int RS = x_row_stride<M, TPR, WREG>();
  constexpr int NT = NR * TPR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V2* S = reinterpret_cast<V2*>(smem_raw);
  const int row = threadIdx.x / TPR, t = threadIdx.x % TPR;
  V2* U = S + row * RS;
  V2* Vv = U + M;
  V2* X = U + (WREG ? 2 : 3) * M;  // the exchange buffer; without WREG w's slot sits before it
  const int nx = d.nx, nxp = nx + 1, nzd = d.nzd;
  const int plane = plane0 + blockIdx.y;
  const int jz0 = blockIdx.x * NR;
  const int nrow = min(NR, nzd - jz0);
  // the block's rows of the three spectra (zTOx): NR consecutive jz per kx,
  // u into U, v into V, w into X (with WREG) or into its own slot W
  V2* Wp = U + 2 * M;  // w in physical space without WREG
  for (int c = 0; c < 3; ++c) {
    const V2* src = Zb + ((size_t)c * d.nplanes + plane) * nxp * nzd + jz0;
    const int off = c * M;
    for (int i = threadIdx.x; i < nxp * NR; i += NT) {
      const int r = i % NR, k = i / NR;
      V2 v = czero<V2>();
      if (r < nrow) v = ldg_v(src + (size_t)k * nzd + r);
      S[r * RS + off + k] = v;
    }
  }
  __syncthreads();
  // c2r by the half-length packing
  //   Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) e^{+i pi k / M}
  // (only Re of the kx = 0 entry; the x zero band kx > nx, dnsdata.f90:535)
  auto pack = [&](const V2* F, V2 (&a)[E]) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int n = t + TPR * e;
      V2 xk = n <= nx ? F[n] : czero<V2>();
      V2 xm = czero<V2>();
      if (n == 0) xk.y = T();
      else if (M - n <= nx) xm = conjg(F[M - n]);
      const V2 ev = xk + xm, od = cmul_s<+1>(xk - xm, ldg_v(twh + n));
      a[e] = ev + mul_is<+1>(od);
    }
  };
  V2 w[WREG ? E : 1];  // with WREG: w in physical space, w[e] at x pair t + TPR e
  if constexpr (WREG) {
    pack(X, w);
    group_sync<TPR>();  // every read of the w spectrum before X becomes the exchange buffer
    rfft_regs<E, TPR, +1>(w, X, t, tw);
  }
#pragma unroll 1
  for (int c = 0; c < (WREG ? 2 : 3); ++c) {
    V2* F = c == 0 ? U : (c == 1 ? Vv : Wp);
    V2 a[E];
    pack(F, a);
    rfft<E, TPR, +1>(a, X, t, tw, [&](int o, V2 v) { F[o] = v; });
  }
  group_sync<TPR>();
  // w at pair t + TPR e
  auto wv = [&](int e) -> V2 {
    if constexpr (WREG) return w[e];
    else return Wp[t + TPR * e];
  };
  // CFL (dnsdata.f90:552-556) over the physical values of this row
  if (compute_cfl) {
    T cfl = T();
    bool bad = false;
    if (plane >= 2 && plane <= d.ny && row < nrow) {
      using Nm = Num<T>;
      const T rdx = cst[1], rdz = cst[2], rdy = cst[3 + plane];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = t + TPR * e;
        const V2 u = U[n], v = Vv[n], ww = wv(e);
        const T c0 = Nm::abs(u.x) * rdx + Nm::abs(v.x) * rdy + Nm::abs(ww.x) * rdz;
        const T c1 = Nm::abs(u.y) * rdx + Nm::abs(v.y) * rdy + Nm::abs(ww.y) * rdz;
        cfl = Nm::max(cfl, Nm::max(c0, c1));
        bad = bad || !Nm::finite(c0) || !Nm::finite(c1);
      }
    }
    double cd = Num<T>::to_double(cfl);
    if (bad) cd = (double)INFINITY;  // a non-finite velocity shows up as an infinite CFL
    rblock_max_atomic(cd, &sc->cfl);
  }
  // products (dnsdata.f90:581-584), those with w first (w then dies):
  // ww, vw, uw, uu, vv, uv -> Pb slots 2, 4, 5, 0, 1, 3; `factor` enters in
  // the unpacking, g = factor/2 and twh[2M + k] = (factor/2) e^{-i pi k/M}
  const T g = cst[0];
#pragma unroll 1
  for (int q = 0; q < 6; ++q) {
    // with WREG the products with w first (w then dies): ww, vw, uw, uu, vv, uv
    const int p = !WREG ? q : (q == 0 ? 2 : q == 1 ? 4 : q == 2 ? 5 : q == 3 ? 0 : q == 4 ? 1 : 3);
    V2 a[E];
    if constexpr (!WREG) {
      // factors of product p (uu, vv, ww, uv, vw, uw) from the u, v, w slots
      const int fa = p < 3 ? p : (p == 5 ? 0 : p - 3);
      const int fb = p < 3 ? p : (p == 3 ? 1 : 2);
      const V2* A = U + fa * M;
      const V2* B = U + fb * M;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = t + TPR * e;
        const V2 x = A[n], y = B[n];
        a[e] = mk<V2>(x.x * y.x, x.y * y.y);
      }
    } else if (q < 3) {
      const V2* B = q == 1 ? Vv : U;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const V2 y = wv(e), x = q == 0 ? y : B[t + TPR * e];
        a[e] = mk<V2>(x.x * y.x, x.y * y.y);
      }
    } else {
      const V2* A = q == 4 ? Vv : U;
      const V2* B = q == 3 ? U : Vv;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = t + TPR * e;
        const V2 x = A[n], y = B[n];
        a[e] = mk<V2>(x.x * y.x, x.y * y.y);
      }
    }
    rfft<E, TPR, -1>(a, X, t, tw, [&](int o, V2 v) { X[o] = v; });
    group_sync<TPR>();
    // r2c unpacking, kx = 0..nx (HFT, dnsdata.f90:586):
    //   X = g (Z_k + conj Z_{M-k}) + (g w_k) (-i) (Z_k - conj Z_{M-k})
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int k = t + TPR * e;
      if (k <= nx) {
        const V2 zk = X[k];
        const V2 zm = conjg(X[k == 0 ? 0 : M - k]);
        const V2 sm = zk + zm, df = zk - zm;
        const V2 wk = ldg_v(twh + 2 * M + k);
        if constexpr (std::is_same<T, dd>::value) {
          a[e] = scale(sm, g) + cmul(wk, mk<V2>(df.y, T() - df.x));
        } else {
          a[e] = mk<V2>(fma(g, sm.x, fma(wk.x, df.y, wk.y * df.x)), fma(g, sm.y, fma(wk.y, df.y, -(wk.x * df.x))));
        }
      }
    }
    group_sync<TPR>();
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int k = t + TPR * e;
      if (k <= nx) X[k] = a[e];
    }
    __syncthreads();
    // xTOz: the block's rows of product p, NR consecutive jz per kx
    V2* dst = Pb + ((size_t)p * d.nplanes + plane) * nxp * nzd + jz0;
    for (int i = threadIdx.x; i < nxp * NR; i += NT) {
      const int r = i % NR, k = i / NR;
      if (r < nrow) dst[(size_t)k * nzd + r] = S[r * RS + (WREG ? 2 : 3) * M + k];
    }
    __syncthreads();
  }
}

namespace {

template <typename T, int N>
void launch_z_len(const ConvLaunch& L, cudaStream_t s, int stage) {
  using V2 = typename C2<T>::t;
  constexpr int E = RLen<N>::E, TPR = RLen<N>::TPR, NC = z_cols<TPR>();
  const size_t sm = (size_t)NC * rbuf_size<E, TPR>() * sizeof(V2);
  const Dims& d = L.d;
  if (stage == 0) {
    const int ncol = L.ix_hi - L.ix_lo;
    dim3 grid((ncol + NC - 1) / NC, L.nplanes, 3);
    k_zinv_r<T, E, TPR, NC><<<grid, NC * TPR, sm, s>>>(L.V, (V2*)L.Zb, (const V2*)L.twzr, d, L.plane0, L.ix_lo,
                                                        L.ix_hi);
  } else {
    dim3 grid((d.nx + 1 + NC - 1) / NC, L.nplanes, 6);
    k_zfwd_r<T, E, TPR, NC><<<grid, NC * TPR, sm, s>>>((const V2*)L.Pb, (V2*)L.VV, (const V2*)L.twzr, d, L.plane0);
  }
}

template <typename T, int M, int CAP>
void launch_x_len(const ConvLaunch& L, cudaStream_t s) {
  using V2 = typename C2<T>::t;
  constexpr int E = XLen<M>::E, TPR = XLen<M>::TPR;
  constexpr bool WREG = XLen<M>::WREG;
  constexpr int NR = x_rows<M, TPR, WREG, (int)sizeof(V2)>();
  constexpr int MINB = x_minb<M, TPR, WREG, (int)sizeof(V2), CAP>();
  const size_t sm = (size_t)NR * x_row_stride<M, TPR, WREG>() * sizeof(V2);
  const Dims& d = L.d;
  dim3 grid((d.nzd + NR - 1) / NR, L.nplanes);
  k_xrow_r<T, E, TPR, NR, MINB, WREG><<<grid, NR * TPR, sm, s>>>((const V2*)L.Zb, (V2*)L.Pb, (const V2*)L.twxr, (const V2*)L.twh,
                                                      (const T*)L.cst, d, L.plane0, L.compute_cfl, L.sc);
}

// x lengths: nxd <= 768 for every workload (a 1536-point x row would need
// 48 KB of registers and shared memory per row)
template <int N> constexpr bool x_plan() { return N <= 768; }

template <typename T, int N>
bool launch_len(const ConvLaunch& L, cudaStream_t s, int stage) {
  if (stage == 1) {
    if constexpr (x_plan<N>()) {
      if (L.xminb == 5) launch_x_len<T, N, 4>(L, s);
      else launch_x_len<T, N, 3>(L, s);
    } else {
      return false;
    }
  } else {
    launch_z_len<T, N>(L, s, stage);
  }
  return true;
}

// carveout: the x-row kernel with w in registers asks for the largest
// shared-memory carveout (three or four 74 KB blocks); the others keep the default,
// whose larger L1 serves their twiddle loads (the largest carveout made
// z-forward 30% slower)
template <typename K>
cudaError_t allow_smem(K* kernel, size_t bytes, bool max_carveout = false) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess && max_carveout)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
}

template <typename T, int N>
cudaError_t set_limits_len() {
  using V2 = typename C2<T>::t;
  constexpr int E = RLen<N>::E, TPR = RLen<N>::TPR, NC = z_cols<TPR>();
  cudaError_t e = allow_smem(k_zinv_r<T, E, TPR, NC>, (size_t)NC * rbuf_size<E, TPR>() * sizeof(V2));
  if (e == cudaSuccess) e = allow_smem(k_zfwd_r<T, E, TPR, NC>, (size_t)NC * rbuf_size<E, TPR>() * sizeof(V2));
  if constexpr (x_plan<N>()) {
    constexpr int XE = XLen<N>::E, XT = XLen<N>::TPR;
    constexpr bool WR = XLen<N>::WREG;
    constexpr int XNR = x_rows<N, XT, WR, (int)sizeof(V2)>();
    constexpr size_t xsm = (size_t)XNR * x_row_stride<N, XT, WR>() * sizeof(V2);
    constexpr int MB3 = x_minb<N, XT, WR, (int)sizeof(V2), 3>(), MB4 = x_minb<N, XT, WR, (int)sizeof(V2), 4>();
    if (e == cudaSuccess) e = allow_smem(k_xrow_r<T, XE, XT, XNR, MB3, WR>, xsm, WR);
    if (e == cudaSuccess) e = allow_smem(k_xrow_r<T, XE, XT, XNR, MB4, WR>, xsm, WR);
  }
  return e;
}

template <typename T>
cudaError_t set_limits_type() {
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = set_limits_len<T, 32>();
  if (e == cudaSuccess) e = set_limits_len<T, 48>();
  if (e == cudaSuccess) e = set_limits_len<T, 64>();
  if (e == cudaSuccess) e = set_limits_len<T, 96>();
  if (e == cudaSuccess) e = set_limits_len<T, 192>();
  if (e == cudaSuccess) e = set_limits_len<T, 384>();
  if (e == cudaSuccess) e = set_limits_len<T, 768>();
  if (e == cudaSuccess) e = set_limits_len<T, 1536>();
  return e;
}

}  // namespace

template <typename T>
bool launch_convolutions_r_impl(const ConvLaunch& L, cudaStream_t s, int stage) {
  const int n = stage == 1 ? L.d.nxd : L.d.nzd;
  switch (n) {
    case 32: return launch_len<T, 32>(L, s, stage);
    case 48: return launch_len<T, 48>(L, s, stage);
    case 64: return launch_len<T, 64>(L, s, stage);
    case 96: return launch_len<T, 96>(L, s, stage);
    case 192: return launch_len<T, 192>(L, s, stage);
    case 384: return launch_len<T, 384>(L, s, stage);
    case 768: return launch_len<T, 768>(L, s, stage);
    case 1536: return launch_len<T, 1536>(L, s, stage);
    default: return false;
  }
}

}  // namespace chgpu
