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

// x / d for 0 <= x, x*d < 2^32 by a multiply-high (integer division by a
// value unknown at compile time costs tens of instructions).  magic =
// floor((2^32-1)/d) + 1 over-estimates the quotient by at most one, which the
// final compare removes; d = 1 (magic would be 2^32) is taken apart.
struct FastDiv {
  int d;
  unsigned magic;
  __device__ __forceinline__ explicit FastDiv(int dv) : d(dv), magic(dv > 1 ? 0xFFFFFFFFu / (unsigned)dv + 1u : 0u) {}
  __device__ __forceinline__ int div(int x) const {
    if (magic == 0u) return x;
    int q = (int)__umulhi((unsigned)x, magic);
    return (q * d > x) ? q - 1 : q;
  }
};

// Radix plan passed by value to kernels: radices 16, then one of 8/4/2, then
// 3 (lengths 2^a 3^b, b <= 1), so every stride before the last stage is a
// power of two.
struct RadixDev {
  int n, nst;
  int r[24];
};

// In-register DFTs of length R (natural order in and out), sign -1: exp(-i),
// +1: exp(+i).  Internal twiddles are constants of the type.
template <typename V> __device__ __forceinline__ void dft4(V& a0, V& a1, V& a2, V& a3, int sign) {
  const V t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_i(a1 - a3, sign);
  a0 = t0 + t2;
  a1 = t1 + t3;
  a2 = t0 - t2;
  a3 = t1 - t3;
}

template <int R, typename V> struct Dft;
template <typename V> struct Dft<2, V> {
  __device__ static void run(V* a, int) {
    const V t = a[0] - a[1];
    a[0] = a[0] + a[1];
    a[1] = t;
  }
};
template <typename V> struct Dft<3, V> {
  __device__ static void run(V* a, int sign) {
    using T = decltype(V::x);
    const V t1 = a[1] + a[2];
    const V t2 = a[0] - scale(t1, T(0.5f));
    const V t3 = mul_i(scale(a[1] - a[2], Num<T>::sqrt3_2()), sign);
    a[0] = a[0] + t1;
    a[1] = t2 + t3;
    a[2] = t2 - t3;
  }
};
template <typename V> struct Dft<4, V> {
  __device__ static void run(V* a, int sign) { dft4(a[0], a[1], a[2], a[3], sign); }
};
template <typename V> struct Dft<8, V> {
  // r = 2 r1 + r2, k = k1 + 4 k2: DFT4 over r1, twiddle w8^(r2 k1), DFT2 over r2
  __device__ static void run(V* a, int sign) {
    using T = decltype(V::x);
    const T r2 = Num<T>::sqrt1_2();
    const T sr2 = sign > 0 ? r2 : -r2;
    dft4(a[0], a[2], a[4], a[6], sign);
    dft4(a[1], a[3], a[5], a[7], sign);
    a[3] = cmul(a[3], mk<V>(r2, sr2));   // w8^1
    a[5] = mul_i(a[5], sign);            // w8^2
    a[7] = cmul(a[7], mk<V>(-r2, sr2));  // w8^3
    V y[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      y[k1] = a[2 * k1] + a[2 * k1 + 1];
      y[k1 + 4] = a[2 * k1] - a[2 * k1 + 1];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = y[k];
  }
};
template <typename V> struct Dft<16, V> {
  // r = 4 r1 + r2, k = k1 + 4 k2: DFT4 over r1, twiddle w16^(r2 k1), DFT4 over r2
  __device__ static void run(V* a, int sign) {
    using T = decltype(V::x);
    const T c = Num<T>::cos_pi8(), s = Num<T>::sin_pi8(), r2 = Num<T>::sqrt1_2();
    const T ss = sign > 0 ? s : -s, sc = sign > 0 ? c : -c, sr2 = sign > 0 ? r2 : -r2;
#pragma unroll
    for (int q = 0; q < 4; ++q) dft4(a[q], a[q + 4], a[q + 8], a[q + 12], sign);
    // b[r2][k1] sits in a[r2 + 4 k1]
    a[1 + 4] = cmul(a[1 + 4], mk<V>(c, ss));     // w^1
    a[1 + 8] = cmul(a[1 + 8], mk<V>(r2, sr2));   // w^2
    a[1 + 12] = cmul(a[1 + 12], mk<V>(s, sc));   // w^3
    a[2 + 4] = cmul(a[2 + 4], mk<V>(r2, sr2));   // w^2
    a[2 + 8] = mul_i(a[2 + 8], sign);            // w^4
    a[2 + 12] = cmul(a[2 + 12], mk<V>(-r2, sr2));  // w^6
    a[3 + 4] = cmul(a[3 + 4], mk<V>(s, sc));     // w^3
    a[3 + 8] = cmul(a[3 + 8], mk<V>(-r2, sr2));  // w^6
    a[3 + 12] = cmul(a[3 + 12], mk<V>(-c, -ss));  // w^9
    V y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      V b0 = a[4 * k1], b1 = a[4 * k1 + 1], b2 = a[4 * k1 + 2], b3 = a[4 * k1 + 3];
      dft4(b0, b1, b2, b3, sign);
      y[k1] = b0;
      y[k1 + 4] = b1;
      y[k1 + 8] = b2;
      y[k1 + 12] = b3;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = y[k];
  }
};

// One Stockham stage (Govindaraju et al. 2008 formulation) with radix R over
// B transforms of length n: item j of a transform reads R points at stride
// n/R, twiddles them by w_{Ns R}^{r k} (k = j mod Ns), transforms them in
// registers and writes them at stride Ns.  Ns is a power of two.
template <int R, typename V>
__device__ __forceinline__ void stockham_stage(const V* __restrict__ src, V* __restrict__ dst, int B, int n, int Ns,
                                               int sign, const V* __restrict__ tw) {
  const int nb = n / R;
  const int total = B * nb;
  const int twstep = n / (Ns * R);
  const FastDiv by_nb(nb);
  for (int item = threadIdx.x; item < total; item += blockDim.x) {
    const int t = by_nb.div(item);
    const int j = item - t * nb;
    const int k = j & (Ns - 1);
    const V* s = src + (size_t)t * n;
    V* d = dst + (size_t)t * n;
    V a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = s[j + r * nb];
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        V w = tw[r * k * twstep];
        if (sign > 0) w = conjg(w);
        a[r] = cmul(a[r], w);
      }
    }
    Dft<R, V>::run(a, sign);
    const int idxD = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[idxD + r * Ns] = a[r];
  }
}

// Batched in-shared-memory FFT: `B` transforms of length rad.n, contiguous,
// in `a`; `b` is scratch of the same size. Unnormalised; sign -1: exp(-i...),
// +1: exp(+i...). `tw` holds the forward roots exp(-2 pi i m / n), m<n.
// Returns the buffer holding the result. Every thread of the block calls it.
template <typename V>
__device__ V* fft_block(V* a, V* b, int B, const RadixDev& rad, int sign, const V* __restrict__ tw) {
  const int n = rad.n;
  int Ns = 1;
  for (int st = 0; st < rad.nst; ++st) {
    const int R = rad.r[st];
    switch (R) {
      case 16: stockham_stage<16>(a, b, B, n, Ns, sign, tw); break;
      case 8: stockham_stage<8>(a, b, B, n, Ns, sign, tw); break;
      case 4: stockham_stage<4>(a, b, B, n, Ns, sign, tw); break;
      case 2: stockham_stage<2>(a, b, B, n, Ns, sign, tw); break;
      default: stockham_stage<3>(a, b, B, n, Ns, sign, tw); break;
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
