// Small complex helpers over CUDA's double2/float2 and the shared-memory
// Stockham FFT used by every transform of the step.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

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
// power of two.  twoff[st] is the offset of stage st's twiddles in the
// per-length table (see stockham_stage).
struct RadixDev {
  int n, nst;
  int r[24];
  int twoff[24];
};

// Shared-memory index with one pad slot per 32 elements: the stores of a
// Stockham stage with small Ns run at stride R, which without padding puts a
// whole warp on one bank; with it every warp access needs only the minimum
// number of wavefronts for 8- and 16-byte elements.
__device__ __forceinline__ int pad32(int i) { return i + (i >> 5); }
// even, so that a buffer placed after one of 8-byte elements starts on a
// 16-byte boundary (what bulk copies into it need)
__host__ __device__ constexpr int pad32_size(int n) { return (n + (n >> 5) + 2) & ~1; }

// a * (SIGN * i)
template <int SIGN, typename V> __device__ __forceinline__ V mul_is(V a) {
  return SIGN > 0 ? mk<V>(-a.y, a.x) : mk<V>(a.y, -a.x);
}
// a * w (SIGN < 0) or a * conj(w) (SIGN > 0): the tables hold forward roots
template <int SIGN, typename V> __device__ __forceinline__ V cmul_s(V a, V w) {
  return SIGN < 0 ? cmul(a, w) : mk<V>(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
template <int SIGN> __device__ __forceinline__ cdd cmul_s(cdd a, cdd w) {
  return SIGN < 0 ? cmul(a, w) : cdd{dd_dot2(a.x, w.x, a.y, w.y), dd_dot2(a.y, w.x, -a.x, w.y)};
}
// products that feed only further sums inside a register DFT: for
// double-float without the final renormalisation
template <typename V> __device__ __forceinline__ V cmul_inner(V a, V b) { return cmul(a, b); }
__device__ __forceinline__ cdd cmul_inner(cdd a, cdd b) { return cmul_nr(a, b); }
template <int SIGN, typename V> __device__ __forceinline__ V cmul_s_inner(V a, V w) { return cmul_s<SIGN>(a, w); }
template <int SIGN> __device__ __forceinline__ cdd cmul_s_inner(cdd a, cdd w) {
  return SIGN < 0 ? cmul_nr(a, w) : cdd{dd_dot2_nr(a.x, w.x, a.y, w.y), dd_dot2_nr(a.y, w.x, -a.x, w.y)};
}

// w_N^m = exp(SIGN 2 pi i m / N) for N dividing 24 (m fixed at compile
// time after unrolling), from the constants of the type: angles are
// multiples of 15 degrees.
template <int N, int SIGN, typename V> __device__ __forceinline__ V root(int m) {
  using T = decltype(V::x);
  const int e = (m * (24 / N)) % 24;  // in units of 15 degrees
  const T c15 = Num<T>::cos_pi12(), s15 = Num<T>::sin_pi12(), c30 = Num<T>::sqrt3_2(), h = T(0.5f);
  const T r2 = Num<T>::sqrt1_2(), one = T(1.0f), zero = T();
  // cos and sin of e * 15 degrees for e in [0, 6], then quadrant by symmetry
  const int q = e / 6, f = e % 6;
  T c, s;
  switch (f) {
    case 0: c = one; s = zero; break;
    case 1: c = c15; s = s15; break;
    case 2: c = c30; s = h; break;
    case 3: c = r2; s = r2; break;
    case 4: c = h; s = c30; break;
    default: c = s15; s = c15; break;
  }
  // rotate by q quarter turns: (c, s) -> (-s, c)
  for (int i = 0; i < q; ++i) {
    const T t = c;
    c = zero - s;
    s = t;
  }
  return mk<V>(c, SIGN > 0 ? s : zero - s);
}

// In-register DFTs of length R (natural order in and out), SIGN -1: exp(-i),
// +1: exp(+i).  Internal twiddles are constants of the type.
template <int SIGN, typename V> __device__ __forceinline__ void dft4(V& a0, V& a1, V& a2, V& a3) {
  const V t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_is<SIGN>(a1 - a3);
  a0 = t0 + t2;
  a1 = t1 + t3;
  a2 = t0 - t2;
  a3 = t1 - t3;
}
// radix-4 butterfly whose outputs feed only further arithmetic inside a
// larger register DFT: for double-float no sum is renormalised
template <int SIGN, typename V> __device__ __forceinline__ void dft4_inner(V& a0, V& a1, V& a2, V& a3) {
  dft4<SIGN>(a0, a1, a2, a3);
}
template <int SIGN> __device__ __forceinline__ void dft4_inner(cdd& a0, cdd& a1, cdd& a2, cdd& a3) {
  const cdd t0 = add_nr(a0, a2), t1 = sub_nr(a0, a2), t2 = add_nr(a1, a3), t3 = mul_is<SIGN>(sub_nr(a1, a3));
  a0 = add_nr(t0, t2);
  a1 = add_nr(t1, t3);
  a2 = sub_nr(t0, t2);
  a3 = sub_nr(t1, t3);
}
// double-float: the first-level sums feed only the second level, so they
// skip the renormalisation; the outputs are normalised
template <int SIGN> __device__ __forceinline__ void dft4(cdd& a0, cdd& a1, cdd& a2, cdd& a3) {
  const cdd t0 = add_nr(a0, a2), t1 = sub_nr(a0, a2), t2 = add_nr(a1, a3), t3 = mul_is<SIGN>(sub_nr(a1, a3));
  a0 = t0 + t2;
  a1 = t1 + t3;
  a2 = t0 - t2;
  a3 = t1 - t3;
}

template <int R, typename V> struct Dft;
template <typename V> struct Dft<2, V> {
  template <int SIGN> __device__ static void run(V* a) {
    const V t = a[0] - a[1];
    a[0] = a[0] + a[1];
    a[1] = t;
  }
};
template <typename V> struct Dft<3, V> {
  template <int SIGN> __device__ static void run(V* a) {
    using T = decltype(V::x);
    const V t1 = a[1] + a[2];
    if constexpr (std::is_same<V, cdd>::value) {
      const V t2 = a[0] - scale(t1, T(0.5f));
      const V t3 = mul_is<SIGN>(scale(a[1] - a[2], Num<T>::sqrt3_2()));
      a[0] = a[0] + t1;
      a[1] = t2 + t3;
      a[2] = t2 - t3;
    } else {
      // m +- SIGN i (sqrt3/2) d as four fused multiply-adds onto m = a0 - t1/2
      const V d = a[1] - a[2];
      const T s = SIGN > 0 ? Num<T>::sqrt3_2() : -Num<T>::sqrt3_2();
      const V m = mk<V>(fma(T(-0.5f), t1.x, a[0].x), fma(T(-0.5f), t1.y, a[0].y));
      a[0] = a[0] + t1;
      a[1] = mk<V>(fma(-s, d.y, m.x), fma(s, d.x, m.y));
      a[2] = mk<V>(fma(s, d.y, m.x), fma(-s, d.x, m.y));
    }
  }
};
template <typename V> struct Dft<4, V> {
  template <int SIGN> __device__ static void run(V* a) { dft4<SIGN>(a[0], a[1], a[2], a[3]); }
};
template <typename V> struct Dft<8, V> {
  // r = 2 r1 + r2, k = k1 + 4 k2: DFT4 over r1, twiddle w8^(r2 k1), DFT2 over r2
  template <int SIGN> __device__ static void run(V* a) {
    using T = decltype(V::x);
    const T r2 = Num<T>::sqrt1_2();
    const T sr2 = SIGN > 0 ? r2 : -r2;
    dft4_inner<SIGN>(a[0], a[2], a[4], a[6]);
    dft4_inner<SIGN>(a[1], a[3], a[5], a[7]);
    a[3] = cmul_inner(a[3], mk<V>(r2, sr2));   // w8^1
    a[5] = mul_is<SIGN>(a[5]);           // w8^2
    a[7] = cmul_inner(a[7], mk<V>(-r2, sr2));  // w8^3
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
  template <int SIGN> __device__ static void run(V* a) {
    using T = decltype(V::x);
    const T c = Num<T>::cos_pi8(), s = Num<T>::sin_pi8(), r2 = Num<T>::sqrt1_2();
    const T ss = SIGN > 0 ? s : -s, sc = SIGN > 0 ? c : -c, sr2 = SIGN > 0 ? r2 : -r2;
#pragma unroll
    for (int q = 0; q < 4; ++q) dft4_inner<SIGN>(a[q], a[q + 4], a[q + 8], a[q + 12]);
    // b[r2][k1] sits in a[r2 + 4 k1]
    a[1 + 4] = cmul_inner(a[1 + 4], mk<V>(c, ss));      // w^1
    a[1 + 8] = cmul_inner(a[1 + 8], mk<V>(r2, sr2));    // w^2
    a[1 + 12] = cmul_inner(a[1 + 12], mk<V>(s, sc));    // w^3
    a[2 + 4] = cmul_inner(a[2 + 4], mk<V>(r2, sr2));    // w^2
    a[2 + 8] = mul_is<SIGN>(a[2 + 8]);            // w^4
    a[2 + 12] = cmul_inner(a[2 + 12], mk<V>(-r2, sr2));  // w^6
    a[3 + 4] = cmul_inner(a[3 + 4], mk<V>(s, sc));      // w^3
    a[3 + 8] = cmul_inner(a[3 + 8], mk<V>(-r2, sr2));   // w^6
    a[3 + 12] = cmul_inner(a[3 + 12], mk<V>(-c, -ss));  // w^9
    V y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      V b0 = a[4 * k1], b1 = a[4 * k1 + 1], b2 = a[4 * k1 + 2], b3 = a[4 * k1 + 3];
      dft4<SIGN>(b0, b1, b2, b3);
      y[k1] = b0;
      y[k1 + 4] = b1;
      y[k1 + 8] = b2;
      y[k1 + 12] = b3;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = y[k];
  }
};

// Composite register DFTs of length 3 P (P = 2, 4, 8): r = P r1 + r2,
// k = k1 + 3 k2 -- DFT3 over r1 for each r2, twiddle w_{3P}^(r2 k1), DFT_P
// over r2 for each k1.  w(m) is w_{3P}^m for the transform's sign.
template <int P, typename V> struct DftComposite {
  template <int SIGN> __device__ static void run(V* a) {
    using T = decltype(V::x);
    constexpr int N = 3 * P;
#pragma unroll
    for (int r2 = 0; r2 < P; ++r2) {
      V b[3] = {a[r2], a[P + r2], a[2 * P + r2]};
      Dft<3, V>::template run<SIGN>(b);
      a[r2] = b[0];
      a[P + r2] = b[1];
      a[2 * P + r2] = b[2];
    }
    // a[k1 P + r2] holds the DFT3 output k1 of column r2
#pragma unroll
    for (int k1 = 1; k1 < 3; ++k1)
#pragma unroll
      for (int r2 = 1; r2 < P; ++r2) a[k1 * P + r2] = cmul(a[k1 * P + r2], root<N, SIGN, V>(r2 * k1));
    V y[N];
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      V c[P];
#pragma unroll
      for (int r2 = 0; r2 < P; ++r2) c[r2] = a[k1 * P + r2];
      Dft<P, V>::template run<SIGN>(c);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) y[k1 + 3 * k2] = c[k2];
    }
#pragma unroll
    for (int k = 0; k < N; ++k) a[k] = y[k];
    (void)sizeof(T);
  }
};
template <typename V> struct Dft<6, V> : DftComposite<2, V> {};
template <typename V> struct Dft<12, V> : DftComposite<4, V> {};
template <typename V> struct Dft<24, V> : DftComposite<8, V> {};

// read-only load of a complex value of any of the three types
template <typename V> __device__ __forceinline__ V ldg_v(const V* p) { return __ldg(p); }
template <> __device__ __forceinline__ cdd ldg_v<cdd>(const cdd* p) {
  const float4 f = __ldg(reinterpret_cast<const float4*>(p));
  return cdd{dd(f.x, f.y), dd(f.z, f.w)};
}

// ---------------------------------------------------------------------------
// FP64 twiddled DFTs with fused multiply-adds (Linzer and Feig, "Modified
// FFTs for fused multiply-add architectures", Math. Comp. 60, 1993).  A
// twiddle w is held as (c, t) with w = c (1 + i t) or w = i c (1 + i t)
// (whichever gives |t| <= 1; the choice q is the lowest significand bit of
// c, a perturbation of at most one ulp), so that a butterfly a +- w b is
//   P + i Q = (1 + i t) b          two FMAs
//   a +- c (P + i Q)  or  a +- i c (P + i Q)   four FMAs
// -- six FP64 operations where a complex product and two complex additions
// take eight.  The rotation by i only swaps P and Q and flips a sign of c,
// which are integer selects, off the FP64 pipe.  SIGN > 0 uses conj(w).
// ---------------------------------------------------------------------------
template <int SIGN> __device__ __forceinline__ void lf_butterfly(double2& a, double2& b, double2 w) {
  const int lo = __double2loint(w.x);
  const bool q = (lo & 1) != 0;
  const double t = w.y;
  const double P = SIGN < 0 ? fma(-t, b.y, b.x) : fma(t, b.y, b.x);
  const double Q = SIGN < 0 ? fma(t, b.x, b.y) : fma(-t, b.x, b.y);
  const double X = q ? Q : P, Y = q ? P : Q;
  const double cneg = __hiloint2double(__double2hiint(w.x) ^ (int)0x80000000, lo);
  const double cx = (SIGN < 0 && q) ? cneg : w.x;
  const double cy = (SIGN > 0 && q) ? cneg : w.x;
  const double2 o1 = make_double2(fma(cx, X, a.x), fma(cy, Y, a.y));
  b = make_double2(fma(-cx, X, a.x), fma(-cy, Y, a.y));
  a = o1;
}
__host__ __device__ constexpr int ilog2c(int r) { return r <= 1 ? 0 : 1 + ilog2c(r / 2); }
__host__ __device__ constexpr bool is_pow2c(int r) { return r >= 2 && (r & (r - 1)) == 0; }
// position of partial transform m (l bits) in the in-place radix-2 cascade
// of an R-point DFT: bit i of m at R / 2^(i+1)
__host__ __device__ constexpr int lf_pos(int m, int l, int R) {
  int o = 0;
  for (int i = 0; i < l; ++i)
    if ((m >> i) & 1) o += R >> (i + 1);
  return o;
}
// X_m = sum_r a_r W_{Ns R}^{r k} W_R^{r m} for R = 2^L, natural order in and
// out, as L levels of radix-2 decimation in time: level l combines pairs at
// distance R / 2^l with the twiddles W_{2^l Ns}^{k + Ns m'} (m' < 2^(l-1)),
// which are w[2^(l-1) - 1 + m'] (R - 1 values per k, in that order).
template <int R, int SIGN> __device__ __forceinline__ void lf_dft(double2* a, const double2* __restrict__ w) {
  constexpr int L = ilog2c(R);
#pragma unroll
  for (int l = 1; l <= L; ++l) {
    const int h = R >> l;
#pragma unroll
    for (int mp = 0; mp < (1 << (l - 1)); ++mp) {
      const double2 tw = __ldg(w + (1 << (l - 1)) - 1 + mp);
      const int off = lf_pos(mp, l - 1, R);
#pragma unroll
      for (int r = 0; r < h; ++r) lf_butterfly<SIGN>(a[off + r], a[off + r + h], tw);
    }
  }
  double2 y[R];
#pragma unroll
  for (int m = 0; m < R; ++m) y[m] = a[lf_pos(m, L, R)];
#pragma unroll
  for (int m = 0; m < R; ++m) a[m] = y[m];
}

// A 16-point DFT without external twiddles as Dft<16> splits it (DFT4 over
// r1, twiddles w16^(r2 k1), DFT4 over r2), with the twiddled DFT4s of k1 =
// 1..3 as lf_dft<4> (their twiddles are those of a radix-4 pass with Ns = 4
// at k = k1): w holds their 3 x 3 pairs
template <int SIGN> __device__ __forceinline__ void lf_dft16_first(double2* a, const double2* __restrict__ w) {
#pragma unroll
  for (int q = 0; q < 4; ++q) dft4_inner<SIGN>(a[q], a[q + 4], a[q + 8], a[q + 12]);
  double2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    double2 c[4] = {a[4 * k1], a[4 * k1 + 1], a[4 * k1 + 2], a[4 * k1 + 3]};
    if (k1 == 0) dft4<SIGN>(c[0], c[1], c[2], c[3]);
    else lf_dft<4, SIGN>(c, w + 3 * (k1 - 1));
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = c[k2];
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = y[k];
}

// One Stockham stage (Govindaraju et al. 2008 formulation) with radix R over
// B transforms of length n held in padded shared memory (pad32): item j of
// a transform reads R points at stride n/R, twiddles them by
// w_{Ns R}^{r k} (k = j mod Ns), transforms them in registers and writes
// them at stride Ns.  Ns is a power of two.  twst holds this stage's forward
// twiddles, R-1 consecutive values per k (twst[k (R-1) + r-1]), so one item
// reads one contiguous run.
template <int R, int SIGN, typename V>
__device__ __forceinline__ void stockham_stage(const V* __restrict__ src, V* __restrict__ dst, int B, int n, int Ns,
                                               const V* __restrict__ twst) {
  const int nb = n / R;
  const int total = B * nb;
  const FastDiv by_nb(nb);
  for (int item = threadIdx.x; item < total; item += blockDim.x) {
    const int t = by_nb.div(item);
    const int j = item - t * nb;
    const int k = j & (Ns - 1);
    const int sbase = t * n + j;
    V a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = src[pad32(sbase + r * nb)];
    if constexpr (std::is_same<V, double2>::value && is_pow2c(R)) {
      // FP64: the twiddles in the fused multiply-add form (lf_dft); a
      // first radix-16 stage twiddles only inside its DFT (lf_dft16_first)
      if (Ns > 1) lf_dft<R, SIGN>(a, twst + k * (R - 1));
      else if constexpr (R == 16) lf_dft16_first<SIGN>(a, twst);
      else Dft<R, V>::template run<SIGN>(a);
    } else {
      if (Ns > 1) {
        const V* w = twst + k * (R - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) a[r] = cmul_s_inner<SIGN>(a[r], ldg_v(w + r - 1));
      }
      Dft<R, V>::template run<SIGN>(a);
    }
    const int dbase = t * n + (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[pad32(dbase + r * Ns)] = a[r];
  }
}

// Batched in-shared-memory FFT: B transforms of length rad.n, contiguous in
// the padded layout, in `a`; `b` is scratch of the same size.  Unnormalised;
// SIGN -1: exp(-i...), +1: exp(+i...).  `tw` is the per-stage twiddle table
// of this length.  COMPOSITE compiles the 6/12/24-point tail stages in (FP32
// only; their registers would cost the other kernels occupancy).  Returns the
// buffer holding the result.  Every thread of the block calls it.
template <int SIGN, typename V, bool COMPOSITE = false>
__device__ V* fft_block(V* a, V* b, int B, const RadixDev& rad, const V* __restrict__ tw) {
  const int n = rad.n;
  int Ns = 1;
  for (int st = 0; st < rad.nst; ++st) {
    const int R = rad.r[st];
    const V* twst = tw + rad.twoff[st];
    if constexpr (COMPOSITE && std::is_same<V, float2>::value) {  // composite tails: FP32 x plans only
      if (R == 24 || R == 12 || R == 6) {
        if (R == 24) stockham_stage<24, SIGN>(a, b, B, n, Ns, twst);
        else if (R == 12) stockham_stage<12, SIGN>(a, b, B, n, Ns, twst);
        else stockham_stage<6, SIGN>(a, b, B, n, Ns, twst);
        __syncthreads();
        V* tmp = a;
        a = b;
        b = tmp;
        Ns *= R;
        continue;
      }
    }
    switch (R) {
      case 16: stockham_stage<16, SIGN>(a, b, B, n, Ns, twst); break;
      case 8: stockham_stage<8, SIGN>(a, b, B, n, Ns, twst); break;
      case 4: stockham_stage<4, SIGN>(a, b, B, n, Ns, twst); break;
      case 2: stockham_stage<2, SIGN>(a, b, B, n, Ns, twst); break;
      default: stockham_stage<3, SIGN>(a, b, B, n, Ns, twst); break;
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
