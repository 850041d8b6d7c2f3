// Register-blocked Stockham FFT with compile-time lengths, the core of the
// transform kernels for the lengths the workloads use (32 ... 1536).
//
// A length N = E * TPR transform belongs to a group of TPR consecutive
// threads; thread t of the group holds the E elements x[t + TPR e] in
// registers.  Pass 1 is one radix-E register DFT per thread (its inputs are
// exactly the thread's own elements, at stride TPR).  Every later pass, of
// radix R dividing E, does E/R butterflies per thread: butterfly j = t +
// TPR i (i < E/R) takes x[j + r N/R] = the thread's element i + r E/R,
// multiplies by w_{Ns R}^{r k} (k = j mod Ns, Ns the product of the earlier
// radices), transforms in registers and writes its outputs to
// (j - k) R + k + r Ns of the group's shared-memory buffer; after a group
// barrier each thread reads back x'[t + TPR e].  Each pass thus costs one
// shared-memory store and one load per element, and no index arithmetic
// beyond compile-time constants.  The output of the last pass is in natural
// order at j + r Ns (j < Ns), consecutive over the group's threads, so it can
// go straight to global memory or to an unpadded buffer.
//
// Exchange buffers are padded with one slot per E elements: pass 1 writes
// at stride E across the threads, which without the pad puts a warp on two
// banks (stride E+1 spreads it over all of them); the loads and the later
// passes' stores are consecutive runs either way.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "cplx.cuh"

namespace chgpu {

// radix of pass p (p >= 1) for elements per thread E and threads per group
// TPR: the largest power of two dividing E that still divides what is left
// of TPR
__host__ __device__ constexpr int rplan_radix(int E, int TPR, int p) {
  int rem = TPR;
  int r = 1;
  const int rmax = (E % 16 == 0) ? 16 : (E % 8 == 0 ? 8 : (E % 4 == 0 ? 4 : 2));
  for (int q = 1; q <= p; ++q) {
    if (rem <= 1) return 1;
    r = rmax;
    while (r > rem) r /= 2;
    rem /= r;
  }
  return r;
}
__host__ __device__ constexpr int rplan_passes(int E, int TPR) {
  int n = 1, rem = TPR;
  const int rmax = (E % 16 == 0) ? 16 : (E % 8 == 0 ? 8 : (E % 4 == 0 ? 4 : 2));
  while (rem > 1) {
    int r = rmax;
    while (r > rem) r /= 2;
    rem /= r;
    ++n;
  }
  return n;
}
// Ns before pass p (p = 0 is the radix-E pass)
__host__ __device__ constexpr int rplan_ns(int E, int TPR, int p) {
  int ns = E;
  for (int q = 1; q < p; ++q) ns *= rplan_radix(E, TPR, q);
  return p == 0 ? 1 : ns;
}
// table entries per butterfly position k of a radix-R pass: the R-1
// twiddles, padded to R in FP32 tables so that twiddle pairs are 16-byte
// loads (load_twiddles)
template <typename V> __host__ __device__ constexpr int tw_per_k(int R) {
  return std::is_same<V, float2>::value ? R : R - 1;
}
// offset of pass p's twiddles in the plan's table: tw_per_k values per k < Ns
template <typename V> __host__ __device__ constexpr int rplan_twoff(int E, int TPR, int p) {
  int off = 0;
  for (int q = 1; q < p; ++q) off += rplan_ns(E, TPR, q) * tw_per_k<V>(rplan_radix(E, TPR, q));
  return off;
}
template <typename V> __host__ __device__ constexpr int rplan_twsize(int E, int TPR) {
  return rplan_twoff<V>(E, TPR, rplan_passes(E, TPR));
}

// padded index of an exchange buffer
template <int E> __device__ __forceinline__ int rpad(int i) { return i + i / E; }
template <int E, int TPR> __host__ __device__ constexpr int rbuf_size() { return E * TPR + TPR; }

// barrier over one transform group: the warp (or sub-warp groups of one
// warp, which all run the same passes), or a named barrier of TPR threads
template <int TPR> __device__ __forceinline__ void group_sync() {
  if constexpr (TPR <= 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / TPR)), "r"(TPR) : "memory");
  }
}

// pass 1: one radix-E register DFT per thread.  FP64 with E = 3P: the
// composite DFT's two twiddled P-point DFTs (twiddles W_{3P}^{r k1}, k1 = 1,
// 2) in the fused multiply-add form, from the 2 (P-1) pairs at the end of
// the plan's table
template <int E, int TPR, int SIGN, typename V>
__device__ __forceinline__ void rpass_first(V (&a)[E], const V* __restrict__ tw) {
  if constexpr (std::is_same<V, double2>::value && E % 3 == 0 && is_pow2c(E / 3)) {
    constexpr int P = E / 3;
    const V* tail = tw + rplan_twsize<V>(E, TPR);
#pragma unroll
    for (int r2 = 0; r2 < P; ++r2) {
      V b[3] = {a[r2], a[P + r2], a[2 * P + r2]};
      Dft<3, V>::template run<SIGN>(b);
      a[r2] = b[0];
      a[P + r2] = b[1];
      a[2 * P + r2] = b[2];
    }
    V y[E];
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      V c[P];
#pragma unroll
      for (int r2 = 0; r2 < P; ++r2) c[r2] = a[k1 * P + r2];
      if (k1 == 0) Dft<P, V>::template run<SIGN>(c);
      else lf_dft<P, SIGN>(c, tail + (k1 - 1) * (P - 1));
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) y[k1 + 3 * k2] = c[k2];
    }
#pragma unroll
    for (int k = 0; k < E; ++k) a[k] = y[k];
  } else {
    Dft<E, V>::template run<SIGN>(a);
  }
}
// entries after the per-pass twiddles: FP64 composite first passes only
__host__ __device__ constexpr int rplan_tailsize(int E) {
  return (E % 3 == 0 && E / 3 >= 2 && ((E / 3) & (E / 3 - 1)) == 0) ? 2 * (E / 3 - 1) : 0;
}

// The R-1 twiddles w^1..w^(R-1) of one butterfly from its run of the
// table.  TW_PRODUCTS (FP32 only, whose runs are padded to R entries): a
// radix-8 butterfly loads w^1..w^4 as two 16-byte loads and forms w^5, w^6,
// w^7 as products with w^4 (one more rounding, ~1e-7), a radix-4 one loads
// w^1, w^2 as one and forms w^3; fewer loads for these latency-limited
// kernels (products in place of loads measured 3-4% faster on GB300; the
// paired loads measured even).  FP64 and double-float load every value
// (their multiplications bound them).
constexpr bool TW_PRODUCTS = true;
template <int R, typename V> __device__ __forceinline__ void load_twiddles(const V* w, V (&tw)[R]) {
  if constexpr (TW_PRODUCTS && std::is_same<V, float2>::value && R == 8) {
    // w^1..w^4 as two 16-byte loads (the run is padded to 8 entries)
    const float4 a = __ldg(reinterpret_cast<const float4*>(w));
    const float4 b = __ldg(reinterpret_cast<const float4*>(w + 2));
    tw[1] = make_float2(a.x, a.y);
    tw[2] = make_float2(a.z, a.w);
    tw[3] = make_float2(b.x, b.y);
    tw[4] = make_float2(b.z, b.w);
    tw[5] = cmul(tw[1], tw[4]);
    tw[6] = cmul(tw[2], tw[4]);
    tw[7] = cmul(tw[3], tw[4]);
  } else if constexpr (TW_PRODUCTS && std::is_same<V, float2>::value && R == 4) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(w));
    tw[1] = make_float2(a.x, a.y);
    tw[2] = make_float2(a.z, a.w);
    tw[3] = cmul(tw[1], tw[2]);
  } else {
#pragma unroll
    for (int r = 1; r < R; ++r) tw[r] = ldg_v(w + r - 1);
  }
}

// One butterfly of a pass p >= 1: the R-1 twiddles of its run of the table,
// then the R-point DFT; FP64 in the fused multiply-add form (lf_dft, whose
// tables hold (c, t) pairs in its order)
template <int R, int SIGN, typename V> __device__ __forceinline__ void twiddled_dft(V (&b)[R], const V* w) {
  static_assert(is_pow2c(R), "passes after the first have power-of-two radices");
  if constexpr (std::is_same<V, double2>::value) {
    lf_dft<R, SIGN>(b, w);
  } else {
    V tw_[R];
    load_twiddles<R>(w, tw_);
#pragma unroll
    for (int r = 1; r < R; ++r) b[r] = cmul_s_inner<SIGN>(b[r], tw_[r]);
    Dft<R, V>::template run<SIGN>(b);
  }
}

// Writes the outputs of a pass whose inputs are in a[] (pass p >= 1) or the
// outputs of pass 1 (p == 0, a[] already transformed) to buf.
template <int E, int TPR, int P, int SIGN, bool PADDED, typename V>
__device__ __forceinline__ void rpass_store(V (&a)[E], V* buf, int t, const V* __restrict__ tw) {
  if constexpr (P == 0) {
    // pass 1 outputs: butterfly j = t, outputs at t E + r
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int o = t * E + r;
      buf[PADDED ? rpad<E>(o) : o] = a[r];
    }
  } else {
    constexpr int R = rplan_radix(E, TPR, P);
    constexpr int Ns = rplan_ns(E, TPR, P);
    constexpr int B = E / R;
    const V* twp = tw + rplan_twoff<V>(E, TPR, P);
#pragma unroll
    for (int i = 0; i < B; ++i) {
      const int j = t + TPR * i;
      const int k = j % Ns;
      V b[R];
#pragma unroll
      for (int r = 0; r < R; ++r) b[r] = a[i + r * B];
      twiddled_dft<R, SIGN>(b, twp + k * tw_per_k<V>(R));
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int o = base + r * Ns;
        buf[PADDED ? rpad<E>(o) : o] = b[r];
      }
    }
  }
}

template <int E, int TPR, typename V> __device__ __forceinline__ void rload(V (&a)[E], const V* buf, int t) {
#pragma unroll
  for (int e = 0; e < E; ++e) a[e] = buf[rpad<E>(t + TPR * e)];
}

// The last pass's butterflies.  Their outputs j + r Ns (j = t + TPR i < Ns =
// N/R) are the elements x[t + TPR e], e = i + r E/R, of the same thread: the
// output distribution equals the input distribution.  TO_REGS keeps them
// in a[] (a[e] = x[t + TPR e]); otherwise each goes to sink(index, value).
template <int E, int TPR, int SIGN, bool TO_REGS, typename V, typename Sink>
__device__ __forceinline__ void rpass_last_any(V (&a)[E], int t, const V* __restrict__ tw, Sink sink) {
  constexpr int NP = rplan_passes(E, TPR);
  if constexpr (NP == 1) {
    // the only pass: a[r] is output r of butterfly t = 0 (TPR == 1)
    if constexpr (!TO_REGS) {
#pragma unroll
      for (int r = 0; r < E; ++r) sink(r, a[r]);
    }
  } else {
    constexpr int P = NP - 1;
    constexpr int R = rplan_radix(E, TPR, P);
    constexpr int Ns = rplan_ns(E, TPR, P);
    constexpr int B = E / R;
    static_assert(Ns * R == E * TPR, "last pass");
    const V* twp = tw + rplan_twoff<V>(E, TPR, P);
#pragma unroll
    for (int i = 0; i < B; ++i) {
      const int j = t + TPR * i;  // < Ns, so k = j
      V b[R];
#pragma unroll
      for (int r = 0; r < R; ++r) b[r] = a[i + r * B];
      twiddled_dft<R, SIGN>(b, twp + j * tw_per_k<V>(R));
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if constexpr (TO_REGS) a[i + r * B] = b[r];
        else sink(j + r * Ns, b[r]);
      }
    }
  }
}

// Every pass but the last: a[] holds the input distribution on entry and the
// last pass's inputs on return; buf is the group's padded exchange buffer
// (rbuf_size elements).  Every thread of the group calls it.
template <int E, int TPR, int SIGN, typename V>
__device__ __forceinline__ void rfft_head(V (&a)[E], V* buf, int t, const V* __restrict__ tw) {
  constexpr int NP = rplan_passes(E, TPR);
  rpass_first<E, TPR, SIGN>(a, tw);
  if constexpr (NP >= 2) {
    rpass_store<E, TPR, 0, SIGN, true>(a, buf, t, tw);
    group_sync<TPR>();
    rload<E, TPR>(a, buf, t);
    group_sync<TPR>();
  }
  if constexpr (NP >= 3) {
    rpass_store<E, TPR, 1, SIGN, true>(a, buf, t, tw);
    group_sync<TPR>();
    rload<E, TPR>(a, buf, t);
    group_sync<TPR>();
  }
  if constexpr (NP >= 4) {
    rpass_store<E, TPR, 2, SIGN, true>(a, buf, t, tw);
    group_sync<TPR>();
    rload<E, TPR>(a, buf, t);
    group_sync<TPR>();
  }
  static_assert(NP <= 4, "at most four passes");
}

// Whole transform, a[] holding the input distribution (x[t + TPR e]) on
// entry, the outputs handed to sink(index, value).  The caller synchronises
// the group before reusing buf.
template <int E, int TPR, int SIGN, typename V, typename Sink>
__device__ __forceinline__ void rfft(V (&a)[E], V* buf, int t, const V* __restrict__ tw, Sink sink) {
  rfft_head<E, TPR, SIGN>(a, buf, t, tw);
  rpass_last_any<E, TPR, SIGN, false>(a, t, tw, sink);
}

// Whole transform with the outputs left in a[] (a[e] = x[t + TPR e]).
template <int E, int TPR, int SIGN, typename V>
__device__ __forceinline__ void rfft_regs(V (&a)[E], V* buf, int t, const V* __restrict__ tw) {
  rfft_head<E, TPR, SIGN>(a, buf, t, tw);
  rpass_last_any<E, TPR, SIGN, true>(a, t, tw, [](int, V) {});
}

// Compile-time plans of the lengths with register-blocked kernels.
template <int N> struct RLen;
template <> struct RLen<32> { static constexpr int E = 16, TPR = 2; };
template <> struct RLen<48> { static constexpr int E = 24, TPR = 2; };
template <> struct RLen<64> { static constexpr int E = 16, TPR = 4; };
template <> struct RLen<96> { static constexpr int E = 24, TPR = 4; };
template <> struct RLen<192> { static constexpr int E = 24, TPR = 8; };
template <> struct RLen<384> { static constexpr int E = 24, TPR = 16; };
template <> struct RLen<768> { static constexpr int E = 24, TPR = 32; };
template <> struct RLen<1536> { static constexpr int E = 24, TPR = 64; };

// Plans of the x-row kernel.  WREG: w's physical values stay in registers
// next to the transform being computed (12 elements per thread, 8 for the
// power-of-two lengths, so that three or four blocks share an SM); without
// it w too sits in shared memory and a thread holds 24 elements (measured
// faster at 768 points, where two 64-thread groups per row would need named
// barriers at every exchange).
template <int N> struct XLen;
template <> struct XLen<32> { static constexpr int E = 8, TPR = 4; static constexpr bool WREG = true; };
template <> struct XLen<48> { static constexpr int E = 12, TPR = 4; static constexpr bool WREG = true; };
template <> struct XLen<64> { static constexpr int E = 8, TPR = 8; static constexpr bool WREG = true; };
template <> struct XLen<96> { static constexpr int E = 12, TPR = 8; static constexpr bool WREG = true; };
template <> struct XLen<192> { static constexpr int E = 12, TPR = 16; static constexpr bool WREG = true; };
template <> struct XLen<384> { static constexpr int E = 12, TPR = 32; static constexpr bool WREG = true; };
template <> struct XLen<768> { static constexpr int E = 24, TPR = 32; static constexpr bool WREG = false; };

inline bool xlen_plan(int n, int* E, int* TPR) {
  switch (n) {
    case 32: *E = 8; *TPR = 4; return true;
    case 48: *E = 12; *TPR = 4; return true;
    case 64: *E = 8; *TPR = 8; return true;
    case 96: *E = 12; *TPR = 8; return true;
    case 192: *E = 12; *TPR = 16; return true;
    case 384: *E = 12; *TPR = 32; return true;
    case 768: *E = 24; *TPR = 32; return true;
    default: return false;
  }
}

// host side: does a length have a register-blocked plan, and its (E, TPR)
inline bool rlen_plan(int n, int* E, int* TPR) {
  switch (n) {
    case 32: *E = 16; *TPR = 2; return true;
    case 48: *E = 24; *TPR = 2; return true;
    case 64: *E = 16; *TPR = 4; return true;
    case 96: *E = 24; *TPR = 4; return true;
    case 192: *E = 24; *TPR = 8; return true;
    case 384: *E = 24; *TPR = 16; return true;
    case 768: *E = 24; *TPR = 32; return true;
    case 1536: *E = 24; *TPR = 64; return true;
    default: return false;
  }
}

}  // namespace chgpu
