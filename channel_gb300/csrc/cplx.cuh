// Small complex helpers over CUDA's double2/float2 and the shared-memory
// Stockham FFT used by every transform of the step.
#pragma once

#include <cuda_runtime.h>

#include "dd.cuh"

namespace chgpu {

template <typename T> struct C2;
template <> struct C2<double> { using t = double2; };
template <> struct C2<float> { using t = float2; };
template <> struct C2<dd> { using t = cdd; };

template <typename V> __device__ __forceinline__ V mk(decltype(V::x) a, decltype(V::x) b) { V r; r.x = a; r.y = b; return r; }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename V> __device__ __forceinline__ V conjg(V a) { return mk<V>(a.x, -a.y); }
template <typename V> __device__ __forceinline__ V czero() { return mk<V>(decltype(V::x)(), decltype(V::x)()); }
template <typename V> __device__ __forceinline__ V scale(V a, decltype(V::x) s) { return mk<V>(a.x * s, a.y * s); }
// a * (sign * i)
template <typename V> __device__ __forceinline__ V mul_i(V a, int sign) {
  return sign > 0 ? mk<V>(-a.y, a.x) : mk<V>(a.y, -a.x);
}

// Radix plan passed by value to kernels.
struct RadixDev {
  int n, nst;
  int r[24];
};

// Batched in-shared-memory Stockham FFT (Govindaraju et al. 2008 formulation):
// `B` transforms of length rad.n, contiguous, in `a`; `b` is scratch of the
// same size. Unnormalised; sign -1: exp(-i...), +1: exp(+i...). `tw` holds
// the forward roots exp(-2 pi i m / n), m<n. Returns the buffer holding the
// result. Every thread of the block must call it.
template <typename V>
__device__ V* fft_block(V* a, V* b, int B, const RadixDev& rad, int sign, const V* __restrict__ tw) {
  using T = decltype(V::x);
  const int n = rad.n;
  int Ns = 1;
  const T h3 = Num<T>::sqrt3_2();
  for (int st = 0; st < rad.nst; ++st) {
    const int R = rad.r[st];
    const int nb = n / R;
    const int total = B * nb;
    const int twstep = n / (Ns * R);
    for (int item = threadIdx.x; item < total; item += blockDim.x) {
      const int t = item / nb;
      const int j = item - t * nb;
      const V* src = a + (size_t)t * n;
      V* dst = b + (size_t)t * n;
      const int k = j % Ns;
      V v0 = src[j], v1 = src[j + nb], v2, v3;
      if (R >= 3) v2 = src[j + 2 * nb];
      if (R == 4) v3 = src[j + 3 * nb];
      if (k != 0) {
        V w = tw[k * twstep];
        if (sign > 0) w = conjg(w);
        v1 = cmul(v1, w);
        if (R >= 3) {
          V w2 = tw[2 * k * twstep];
          if (sign > 0) w2 = conjg(w2);
          v2 = cmul(v2, w2);
        }
        if (R == 4) {
          V w3 = tw[3 * k * twstep];
          if (sign > 0) w3 = conjg(w3);
          v3 = cmul(v3, w3);
        }
      }
      const int idxD = (j - k) * R + k;
      if (R == 2) {
        dst[idxD] = v0 + v1;
        dst[idxD + Ns] = v0 - v1;
      } else if (R == 4) {
        V t0 = v0 + v2, t1 = v0 - v2, t2 = v1 + v3, t3 = mul_i(v1 - v3, sign);
        dst[idxD] = t0 + t2;
        dst[idxD + Ns] = t1 + t3;
        dst[idxD + 2 * Ns] = t0 - t2;
        dst[idxD + 3 * Ns] = t1 - t3;
      } else {
        V t1 = v1 + v2;
        V t2 = v0 - scale(t1, T(0.5f));
        V t3 = mul_i(scale(v1 - v2, h3), sign);
        dst[idxD] = v0 + t1;
        dst[idxD + Ns] = t2 + t3;
        dst[idxD + 2 * Ns] = t2 - t3;
      }
    }
    __syncthreads();
    V* tmp = a;
    a = b;
    b = tmp;
    Ns *= R;
  }
  return a;
}

}  // namespace chgpu
