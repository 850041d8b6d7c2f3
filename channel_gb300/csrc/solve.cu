// The wall-normal half of the step: buildrhs rows and linsolve.
//
// k_rhs      : one thread per (mode, y-row): the five-point stencils of the
//              six product spectra and of the field, the RK3/CN combination
//              `timescheme` and the RK history update (dnsdata.f90:609-661).
//              Results go to a separate buffer, which is what the reference's
//              newrhs ring and write-back achieve (dnsdata.f90:667-670).
// k_linsolve : one thread per pair of modes (kx, +kz) and (kx, -kz), whose
//              matrices are equal because k^2 is: the pentadiagonal matrices
//              are assembled, boundary-folded and factored once per row and
//              applied to both modes (linsolve_blocking.inc:11-49), fused as
//   pass A (iy=ny-1..1): assemble, applybc_n/applybc_0 (dnsdata.f90:458-472),
//            LU5decompStep row, LeftLU5divStep1 row (rbparmat_blocking.f90:35-43,70-72)
//   pass B (iy=1..ny-1): LeftLU5divStep2 (rbparmat_blocking.f90:93-95), then
//            wall/ghost values (linsolve_blocking.inc:50-61)
//   mean mode: U/W split, unit-forcing response, flow rates and the
//            constant-flow-rate / CPI correction (linsolve_blocking.inc:62-97)
//   pass C (iy=ny-1..1): COMPLEXderiv of v with LeftLU5divStep1(D0mat) (dnsdata.f90:339-373)
//   pass D (iy=-1..ny+1): LeftLU5divStep2(D0mat) and u,w recovery (linsolve_blocking.inc:99-103)
// The recurrences of each mode are sequential in y; parallelism is across modes.
// k_factor + k_solve : the same solve for grids with fewer than 65 536 pairs:
//              pass A's factorisation alone (two threads per pair, factors to
//              global memory), then Step1, Step2, walls, mean flow, v' and
//              u, w with one thread per (system, mode) -- twice the threads
//              of the fused kernel where it has too few to hide latency.
#include <cuda_runtime.h>

#include <cstdio>

#include <type_traits>

#include "async.cuh"
#include "chgpu_internal.h"
#include "cplx.cuh"
#include "kernels.cuh"

namespace chgpu {

namespace {

__device__ __forceinline__ double2 cz() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double2 rmul(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cdivr(double2 a, double s) { return make_double2(a.x / s, a.y / s); }
// (0 + i a) * z, the product with ialfa/ibeta of the reference (the zero real
// part contributes exact zeros)
template <typename V> __device__ __forceinline__ V mul_ia(decltype(V::x) a, V z) { return mk<V>(-(a * z.y), a * z.x); }
// a * b + c in the arithmetic type: one FMA for FP64 and FP32, the
// double-float product and sum for double-float
template <typename T> __device__ __forceinline__ T fmaT(T a, T b, T c) { return fma(a, b, c); }
template <> __device__ __forceinline__ dd fmaT<dd>(dd a, dd b, dd c) { return a * b + c; }

__device__ __forceinline__ size_t vidx(const Dims& d, int c, int iy, int m) {
  return ((size_t)c * d.nplanes + (iy + 1)) * d.nmodes + m;
}

}  // namespace

// ---------------------------------------------------------------------------
// buildrhs rows
// ---------------------------------------------------------------------------
// Type of the linear terms of the field in buildrhs: FP64, except in the
// mixed path, where double-float keeps them FP64-accurate (~1e-14) on the
// FP32 pipes.
template <typename T> struct LinT { using t = double; };
template <> struct LinT<float> { using t = dd; };

// real * complex in the linear-term type
__device__ __forceinline__ double2 lmul(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ cdd lmul(dd s, cdd a) { return cdd{s * a.x, s * a.y}; }
// FP64 field value in the linear-term type
template <typename LV> __device__ __forceinline__ LV cvt2(double2 v);
template <> __device__ __forceinline__ double2 cvt2<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ cdd cvt2<cdd>(double2 v) { return cdd{dd_from_double(v.x), dd_from_double(v.y)}; }
// explicit-term or history value in the linear-term type
template <typename L> __device__ __forceinline__ L conv(double x);
template <typename L> __device__ __forceinline__ L conv(float x);
template <typename L> __device__ __forceinline__ L conv(dd x);
template <> __device__ __forceinline__ double conv<double>(double x) { return x; }
template <> __device__ __forceinline__ double conv<double>(dd x) { return dd_to_double(x); }
template <> __device__ __forceinline__ dd conv<dd>(float x) { return dd(x); }
// linear-term value stored in the history type
template <typename OT> __device__ __forceinline__ OT store_as(double x) { return (OT)x; }
template <typename OT> __device__ __forceinline__ OT store_as(dd x);
template <> __device__ __forceinline__ float store_as<float>(dd x) { return __fadd_rn(x.hi, x.lo); }


// Storage type of the RK history (the explicit term of the previous
// substep): FP32 in the mixed path, FP64 otherwise.
template <typename T> struct HistT { using t = typename C2<T>::t; };
template <> struct HistT<dd> { using t = double2; };

// resident 128-thread blocks per SM the registers are capped for
template <typename T> struct RhsBlocks { static constexpr int value = 4; };
template <> struct RhsBlocks<float> { static constexpr int value = 3; };
template <> struct RhsBlocks<dd> { static constexpr int value = 5; };

// RB consecutive rows per thread: the five-row windows of the products and
// of the field slide down the rows, so each row is loaded (and, in the mixed
// path, converted to double-float) once instead of five times.
template <typename T, int RB>
__global__ void __launch_bounds__(128, RhsBlocks<T>::value) k_rhs(const double2* __restrict__ V, const typename C2<T>::t* __restrict__ VV,
                                             typename HistT<T>::t* __restrict__ old, double2* __restrict__ rhs,
                                             const typename LinT<T>::t* __restrict__ derL, const T* __restrict__ derT,
                                             Dims d, double ode1, double ode2, double ode3,
                                             const DevScalars* __restrict__ sc, const double2* __restrict__ F,
                                             int m_lo, int m_hi) {
  using V2 = typename C2<T>::t;
  using O2 = typename HistT<T>::t;
  using OT = decltype(O2::x);
  const int m = m_lo + blockIdx.x * blockDim.x + threadIdx.x;
  const int iy0 = blockIdx.y * RB + 1;
  const int nrows = min(RB, d.ny - iy0);
  // ---- linear terms of the field in L (FP64, or double-float in the mixed
  //      path: the FP64 pipe is 1/58 of FP32 here) ----
  // The reference evaluates unkn and impl as separate stencils and combines
  // them; the combined coefficients agree to rounding (one five-point stencil
  // per equation instead of three).
  // timescheme (dnsdata.f90:486) combines ODE(1)/deltat * unkn + impl, which
  // for D2v (:647) is, with S_k = Dk(V2) and lambda = ODE(1)/deltat,
  //   lambda (S2 - k2 S0) + ni (S4 - 2 k2 S2 + k2^2 S0) = sum_j (A_j + k2 B_j + k2^2 C_j) V2_j
  // and for eta (:658) with w = i kz V1 - i kx V3
  //   lambda S0(w) + ni (S2(w) - k2 S0(w)) = sum_j (D_j + k2 E_j) w_j,
  // the mean mode (:653) being the k2 = 0 case on (U, W).  The per-row
  // coefficients A..E are formed once per block and row.
  using L = typename LinT<T>::t;
  using LV = typename C2<L>::t;
  const size_t tailL = (size_t)(d.ny + 1) * 20;  // der rows, then alfa0, beta0, ni
  __shared__ __align__(16) unsigned char cf_raw[RB * 25 * sizeof(L)];
  L* cf = reinterpret_cast<L*>(cf_raw);
  for (int t = threadIdx.x; t < 5 * nrows; t += blockDim.x) {
    const int j = t % 5, rr = t / 5;
    const L* dr = derL + (size_t)(iy0 + rr) * 20;
    const L c0 = dr[j], c2 = dr[10 + j], c4 = dr[15 + j];
    const L lam = Num<L>::from_double(ode1 * sc->rdt);  // ODE(1)/deltat
    const L nu = derL[tailL + 2];
    L* c = cf + rr * 25;
    c[j] = lam * c2 + nu * c4;
    c[5 + j] = L() - (lam * c0 + (nu + nu) * c2);
    c[10 + j] = nu * c0;
    c[15 + j] = lam * c0 + nu * c2;
    c[20 + j] = L() - nu * c0;
  }
  __syncthreads();
  if (m >= m_hi) return;
  const int ix = m / d.nzt;
  const int iz = m - ix * d.nzt - d.nz;
  // wavenumbers (derT holds der in T, then alfa0, beta0; derL likewise in L, then ni)
  const size_t tail = (size_t)(d.ny + 1) * 20;
  const T ta = T((float)ix) * derT[tail], tb = T((float)iz) * derT[tail + 1];
  const T tk2 = ta * ta + tb * tb;
  const L a = L((float)ix) * derL[tailL], b = L((float)iz) * derL[tailL + 1];
  const L k2 = a * a + b * b;
  const L lode2 = Num<L>::from_double(ode2), lode3 = Num<L>::from_double(ode3);
  // STAGED (FP32 path): the next D rows' products (plane iy+3), field rows
  // iy+2 and RK history at iy are copied into a per-thread ring in shared
  // memory while the current row is computed (cp.async), instead of loaded
  // at the top of each row into registers the window already fills
  constexpr bool STAGED = std::is_same<T, float>::value;
  constexpr int D = 2;
  constexpr int SLOT = 128 * (6 * (int)sizeof(V2) + 3 * 16 + 2 * (int)sizeof(O2));
  __shared__ __align__(16) unsigned char stage_raw[STAGED ? (D + 1) * SLOT : 16];
  const int tid = threadIdx.x;
  auto s_vv = [&](int s, int k) { return reinterpret_cast<V2*>(stage_raw + s * SLOT) + k * 128 + tid; };
  auto s_v = [&](int s, int c) {
    return reinterpret_cast<double2*>(stage_raw + s * SLOT + 128 * 6 * (int)sizeof(V2)) + c * 128 + tid;
  };
  auto s_old = [&](int s, int c) {
    return reinterpret_cast<O2*>(stage_raw + s * SLOT + 128 * (6 * (int)sizeof(V2) + 3 * 16)) + c * 128 + tid;
  };
  // issue the copies of row rr of this block's run (none past its rows), then close the group
  auto stage = [&](int rr) {
    if constexpr (STAGED) {
      if (rr < nrows) {
        const int iy = iy0 + rr, s = rr % (D + 1);
#pragma unroll
        for (int k = 0; k < 6; ++k) cp_async8(s_vv(s, k), &VV[((size_t)k * d.nplanes + (iy + 3)) * d.nmodes + m]);
#pragma unroll
        for (int c = 0; c < 3; ++c) cp_async16(s_v(s, c), &V[vidx(d, c, iy + 2, m)]);
        cp_async8(s_old(s, 0), &old[((size_t)0 * (d.ny - 1) + (iy - 1)) * d.nmodes + m]);
        cp_async8(s_old(s, 1), &old[((size_t)1 * (d.ny - 1) + (iy - 1)) * d.nmodes + m]);
      }
      cp_async_commit();
    }
  };
  // windows over rows iy-2..iy+2: the six product spectra (plane = row + 1) and the field
  V2 vv[6][5];
  LV v1[5], v2[5], v3[5];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
#pragma unroll
    for (int k = 0; k < 6; ++k) vv[k][j + 1] = VV[((size_t)k * d.nplanes + (iy0 - 1 + j)) * d.nmodes + m];
    v1[j + 1] = cvt2<LV>(V[vidx(d, 0, iy0 - 2 + j, m)]);
    v2[j + 1] = cvt2<LV>(V[vidx(d, 1, iy0 - 2 + j, m)]);
    v3[j + 1] = cvt2<LV>(V[vidx(d, 2, iy0 - 2 + j, m)]);
  }
#pragma unroll
  for (int q = 0; q < D; ++q) stage(q);
#pragma unroll 1
  for (int rr = 0; rr < RB; ++rr) {
  if (rr >= nrows) break;
  const int iy = iy0 + rr;
  const L* cfr = cf + rr * 25;
  // slide the windows one row down and load row iy+2
#pragma unroll
  for (int j = 0; j < 4; ++j) {
#pragma unroll
    for (int k = 0; k < 6; ++k) vv[k][j] = vv[k][j + 1];
    v1[j] = v1[j + 1];
    v2[j] = v2[j + 1];
    v3[j] = v3[j + 1];
  }
  O2 o_eta, o_d2v;  // RK history at this row
  if constexpr (STAGED) {
    cp_async_wait<D - 1>();  // this row's group has landed
    const int s = rr % (D + 1);
#pragma unroll
    for (int k = 0; k < 6; ++k) vv[k][4] = *s_vv(s, k);
    v1[4] = cvt2<LV>(*s_v(s, 0));
    v2[4] = cvt2<LV>(*s_v(s, 1));
    v3[4] = cvt2<LV>(*s_v(s, 2));
    o_eta = *s_old(s, 0);
    o_d2v = *s_old(s, 1);
    stage(rr + D);  // into the slot of row rr-1, already read
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) vv[k][4] = VV[((size_t)k * d.nplanes + (iy + 3)) * d.nmodes + m];
    v1[4] = cvt2<LV>(V[vidx(d, 0, iy + 2, m)]);
    v2[4] = cvt2<LV>(V[vidx(d, 1, iy + 2, m)]);
    v3[4] = cvt2<LV>(V[vidx(d, 2, iy + 2, m)]);
    o_eta = old[((size_t)0 * (d.ny - 1) + (iy - 1)) * d.nmodes + m];
    o_d2v = old[((size_t)1 * (d.ny - 1) + (iy - 1)) * d.nmodes + m];
  }
  // stencil coefficients of this row in T
  const T* drT = derT + (size_t)iy * 20;
  T e0[5], e1[5], e2[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    e0[j] = drT[j];
    e1[j] = drT[5 + j];
    e2[j] = drT[10 + j];
  }
  // DD(f,k) (dnsdata.f90:609-610) on product k (0-based) at rows iy-2..iy+2
  auto DD = [&](const T* c, int k) -> V2 {
    V2 s = mk<V2>(c[0] * vv[k][0].x, c[0] * vv[k][0].y);
#pragma unroll
    for (int j = 1; j < 5; ++j) s = s + mk<V2>(c[j] * vv[k][j].x, c[j] * vv[k][j].y);
    return s;
  };
  const V2 DD0_6 = DD(e0, 5), DD1_6 = DD(e1, 5);
  // rhsu = -i ta DD0(uu) - DD1(uv) - i tb DD0(uw) (dnsdata.f90:636-638), and
  // rhsv, rhsw alike: with i a z = (-a z.y, a z.x), each component two
  // fused multiply-adds (a leading 0 - ... would block the fusion)
  auto rhs3 = [&](V2 X, V2 Y, V2 Z) {
    return mk<V2>(fmaT(tb, Z.y, fmaT(ta, X.y, -Y.x)), fmaT(-tb, Z.x, fmaT(-ta, X.x, -Y.y)));
  };
  const V2 rhsu = rhs3(DD(e0, 0), DD(e1, 3), DD0_6);
  const V2 rhsv = rhs3(DD(e0, 3), DD(e1, 1), DD(e0, 4));
  const V2 rhsw = rhs3(DD0_6, DD(e1, 4), DD(e0, 2));
  // expl_v = i ta (i ta D1uu + D2uv + i tb D1uw) + i tb (i ta D1uw + D2vw + i tb D1ww) - k2 rhsv (:639-640)
  auto ia_sum = [&](V2 X, V2 Y, V2 Z) {  // i ta X + Y + i tb Z
    return mk<V2>(fmaT(-tb, Z.y, fmaT(-ta, X.y, Y.x)), fmaT(tb, Z.x, fmaT(ta, X.x, Y.y)));
  };
  const V2 in1 = ia_sum(DD(e1, 0), DD(e2, 3), DD1_6), in2 = ia_sum(DD1_6, DD(e2, 4), DD(e1, 2));
  const V2 explv = mk<V2>(fmaT(-tk2, rhsv.x, fmaT(-ta, in1.y, -(tb * in2.y))),
                          fmaT(-tk2, rhsv.y, fmaT(ta, in1.x, tb * in2.x)));
  // body-force terms (dnsdata.f90:644, 651, 658): fv for the v equation,
  // fe for eta (or the mean mode's D0 of Re F1, Re F3)
  LV fv = czero<LV>(), fe = czero<LV>();
  if (F) {
    LV D0f1 = czero<LV>(), D0f2 = czero<LV>(), D0f3 = czero<LV>(), D1f1 = czero<LV>(), D1f3 = czero<LV>();
    L r1 = L(), r3 = L();
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const L c0 = derL[(size_t)iy * 20 + j], c1 = derL[(size_t)iy * 20 + 5 + j];
      const LV f1 = cvt2<LV>(F[vidx(d, 0, iy - 2 + j, m)]);
      const LV f2 = cvt2<LV>(F[vidx(d, 1, iy - 2 + j, m)]);
      const LV f3 = cvt2<LV>(F[vidx(d, 2, iy - 2 + j, m)]);
      D0f1 = D0f1 + lmul(c0, f1);
      D0f2 = D0f2 + lmul(c0, f2);
      D0f3 = D0f3 + lmul(c0, f3);
      D1f1 = D1f1 + lmul(c1, f1);
      D1f3 = D1f3 + lmul(c1, f3);
      r1 = r1 + c0 * f1.x;
      r3 = r3 + c0 * f3.x;
    }
    fv = czero<LV>() - lmul(k2, D0f2) - mul_ia<LV>(a, D1f1) - mul_ia<LV>(b, D1f3);
    fe = (ix == 0 && iz == 0) ? mk<LV>(r1, r3) : mul_ia<LV>(b, D0f1) - mul_ia<LV>(a, D0f3);
  }
  const size_t r0 = ((size_t)0 * (d.ny - 1) + (iy - 1)) * d.nmodes + m;  // eta
  const size_t r1 = ((size_t)1 * (d.ny - 1) + (iy - 1)) * d.nmodes + m;  // d2v
  {
    LV r = lmul(cfr[0] + k2 * (cfr[5] + k2 * cfr[10]), v2[0]);
#pragma unroll
    for (int j = 1; j < 5; ++j) r = r + lmul(cfr[j] + k2 * (cfr[5 + j] + k2 * cfr[10 + j]), v2[j]);
    const O2 o = o_d2v;
    LV e = mk<LV>(conv<L>(explv.x), conv<L>(explv.y));
    if (F) e = e + fv;
    r = r + lmul(lode2, e);
    r = r - lmul(lode3, mk<LV>(conv<L>(o.x), conv<L>(o.y)));
    old[r1] = mk<O2>(store_as<OT>(e.x), store_as<OT>(e.y));
    rhs[r1] = make_double2(Num<L>::to_double(r.x), Num<L>::to_double(r.y));
  }
  if (ix == 0 && iz == 0) {  // mean flow U + iW (:648-654)
    LV e = mk<LV>(conv<L>(rhsu.x) + Num<L>::from_double(sc->meanpx),
                  conv<L>(rhsw.x) + Num<L>::from_double(sc->meanpz));
    if (F) e = e + fe;
    L su = cfr[15] * v1[0].x, sw = cfr[15] * v3[0].x;
#pragma unroll
    for (int j = 1; j < 5; ++j) {
      su = su + cfr[15 + j] * v1[j].x;
      sw = sw + cfr[15 + j] * v3[j].x;
    }
    LV r = mk<LV>(su, sw);
    const O2 o = o_eta;
    r = r + lmul(lode2, e);
    r = r - lmul(lode3, mk<LV>(conv<L>(o.x), conv<L>(o.y)));
    old[r0] = mk<O2>(store_as<OT>(e.x), store_as<OT>(e.y));
    rhs[r0] = make_double2(Num<L>::to_double(r.x), Num<L>::to_double(r.y));
  } else {  // eta (:656-661): with w = i kz V1 - i kx V3, unkn = D0(w), impl = ni (D2(w) - k2 D0(w))
    // i tb rhsu - i ta rhsw (:654)
    const V2 ee = mk<V2>(fmaT(ta, rhsw.y, -(tb * rhsu.y)), fmaT(-ta, rhsw.x, tb * rhsu.x));
    L nj = cfr[15] + k2 * cfr[20];
    LV s1 = lmul(nj, v1[0]), s3 = lmul(nj, v3[0]);
#pragma unroll
    for (int j = 1; j < 5; ++j) {
      nj = cfr[15 + j] + k2 * cfr[20 + j];
      s1 = s1 + lmul(nj, v1[j]);
      s3 = s3 + lmul(nj, v3[j]);
    }
    LV r = mk<LV>(fmaT(a, s3.y, -(b * s1.y)), fmaT(-a, s3.x, b * s1.x));  // i kz s1 - i kx s3
    const O2 o = o_eta;
    LV e = mk<LV>(conv<L>(ee.x), conv<L>(ee.y));
    if (F) e = e + fe;
    r = r + lmul(lode2, e);
    r = r - lmul(lode3, mk<LV>(conv<L>(o.x), conv<L>(o.y)));
    old[r0] = mk<O2>(store_as<OT>(e.x), store_as<OT>(e.y));
    rhs[r0] = make_double2(Num<L>::to_double(r.x), Num<L>::to_double(r.y));
  }
  }  // rows
}

// rows per thread: several where the kernel waits on loads (the FP32 path),
// one where the FP64 pipe binds it and registers are dear
template <typename T> struct RhsRows { static constexpr int value = 1; };
template <> struct RhsRows<float> { static constexpr int value = 16; };

template <typename T>
void launch_rhs(const SolveLaunch& L, cudaStream_t s) {
  using V2 = typename C2<T>::t;
  using O2 = typename HistT<T>::t;
  constexpr int RB = RhsRows<T>::value;
  if (L.m_hi <= L.m_lo) return;
  dim3 grid((L.m_hi - L.m_lo + 127) / 128, (L.d.ny - 1 + RB - 1) / RB);
  using LT = typename LinT<T>::t;
  k_rhs<T, RB><<<grid, 128, 0, s>>>(L.V, (const V2*)L.VV, (O2*)L.old, L.rhs, (const LT*)L.derL, (const T*)L.derT, L.d,
                                L.ode[0], L.ode[1], L.ode[2], L.sc, L.F, L.m_lo, L.m_hi);
}
template void launch_rhs<double>(const SolveLaunch&, cudaStream_t);
template void launch_rhs<float>(const SolveLaunch&, cudaStream_t);
template void launch_rhs<dd>(const SolveLaunch&, cudaStream_t);

// ---------------------------------------------------------------------------
// linsolve
// ---------------------------------------------------------------------------
namespace {

// One row of the two pentadiagonal matrices (linsolve_blocking.inc:12-13),
//   D2vmat = lambda (d2 - k2 d0) - ni (d4 - 2 k2 d2 + k2^2 d0)
//          = cv4 d4 + cv2 d2 + cv0 d0,
//   etamat = lambda d0 - ni (d2 - k2 d0) = ce0 d0 + ce2 d2,
// with the per-mode scalars of AsmCoef.
struct AsmCoef {
  double cv4, cv2, cv0, ce0, ce2;
};
__device__ __forceinline__ AsmCoef asm_coef(double lambda, double k2, double ni) {
  AsmCoef c;
  c.cv4 = -ni;
  c.cv2 = lambda + 2.0 * ni * k2;
  c.cv0 = -(lambda * k2 + ni * k2 * k2);
  c.ce0 = lambda + ni * k2;
  c.ce2 = -ni;
  return c;
}
// applybc_n rows ny-1 / ny-2 and applybc_0 rows 1 / 2 (dnsdata.f90:458-472)
__device__ __forceinline__ void bc_top1(double A[5], const double* bcn, const double* bcnp1) {
  double e = A[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) A[j] = A[j] - e * bcnp1[j] / bcnp1[4];
  e = A[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) A[j] = A[j] - e * bcn[j] / bcn[3];
}
__device__ __forceinline__ void bc_top2(double A[5], const double* bcn) {
  const double e = A[4];
#pragma unroll
  for (int j = 1; j < 4; ++j) A[j] = A[j] - e * bcn[j - 1] / bcn[3];
}
__device__ __forceinline__ void bc_bot1(double A[5], const double* bc0, const double* bc0m1) {
  double e = A[0];
#pragma unroll
  for (int j = 1; j < 5; ++j) A[j] = A[j] - e * bc0m1[j] / bc0m1[0];
  e = A[1];
#pragma unroll
  for (int j = 2; j < 5; ++j) A[j] = A[j] - e * bc0[j] / bc0[1];
}
__device__ __forceinline__ void bc_bot2(double A[5], const double* bc0) {
  const double e = A[0];
#pragma unroll
  for (int j = 1; j < 4; ++j) A[j] = A[j] - e * bc0[j + 1] / bc0[1];
}

// Reciprocal of a pivot by Newton-Raphson iteration (the reciprocal
// iteration of Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Develop. 34(1), 1990): the start
// is the FP32 approximate reciprocal (relative error <= 2^-23) of x's
// leading 24 significand bits (truncation error < 2^-23), scaled by x's
// binary exponent through the exponent field; two steps y <- y + y (1 - x y)
// square the error twice (2^-22 -> 2^-44 -> 2^-88), so the result is 1/x
// rounded once, within half an ulp plus 2^-88 relative.  Four FP64 fused
// multiply-adds, on a GPU whose FP64 pipe bounds these solves.  x with a
// biased exponent outside [1, 2044] (zero, subnormal, |x| >= 2^1022, Inf,
// NaN) takes the IEEE division.
__device__ __forceinline__ double rcp_nr(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 1 || e > 2044) return 1.0 / x;
  const unsigned hi = (unsigned)(b >> 32);
  const float mf = __uint_as_float(0x3f800000u | ((hi & 0xfffffu) << 3) | (unsigned)((b >> 29) & 0x7u));  // [1, 2)
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(mf));  // (0.5, 1]
  const unsigned u = __float_as_uint(rf);
  const unsigned long long ey = (unsigned long long)((int)((u >> 23) & 0xffu) - 127 + 2046 - e);  // in [1, 2046]
  double y = __longlong_as_double(
      (long long)(((unsigned long long)(hi & 0x80000000u) << 32) | (ey << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
  double r = fma(-x, y, 1.0);
  y = fma(y, r, y);
  r = fma(-x, y, 1.0);
  return fma(y, r, y);
}

// LU5decompStep for one row given the (scaled) lower entries of the two rows
// below: L1 = row+1 (j=-2,-1), L2 = row+2.
__device__ __forceinline__ void lu_row(double A[5], const double L1[2], const double L2[2]) {
  double piv = A[4];
  A[3] = A[3] - piv * L2[1];
  A[2] = A[2] - piv * L2[0];
  piv = A[3];
  A[2] = A[2] - piv * L1[1];
  A[1] = A[1] - piv * L1[0];
  piv = rcp_nr(A[2]);
  A[2] = piv;
  A[0] = A[0] * piv;
  A[1] = A[1] * piv;
}

// LeftLU5divStep1 row, x = (b - u1 x(+1) - u2 x(+2)) / d with A[2] = 1/d:
// the two differences as fused multiply-adds (three FP64 operations per
// component where the sum-then-subtract order of the reference takes four)
__device__ __forceinline__ double2 step1u(double2 b, double rd, double u1, double u2, double2 x1, double2 x2) {
  return make_double2(rd * fma(-u2, x2.x, fma(-u1, x1.x, b.x)), rd * fma(-u2, x2.y, fma(-u1, x1.y, b.y)));
}
__device__ __forceinline__ double2 step1(double2 b, const double A[5], double2 x1, double2 x2) {
  return step1u(b, A[2], A[3], A[4], x1, x2);
}

// LeftLU5divStep2 row, b - l2 b(-2) - l1 b(-1), as two fused multiply-adds
// per component
__device__ __forceinline__ double2 step2(double2 b, double lm2, double lm1, double2 bm2, double2 bm1) {
  return make_double2(fma(-lm1, bm1.x, fma(-lm2, bm2.x, b.x)), fma(-lm1, bm1.y, fma(-lm2, bm2.y, b.y)));
}

__device__ __forceinline__ double2 dot3(const double2* v, const double* c) {  // sum(v(1:3)*c(0:2))
  double2 s = rmul(c[0], v[0]);
  s = s + rmul(c[1], v[1]);
  return s + rmul(c[2], v[2]);
}
__device__ __forceinline__ double2 dot4(const double2* v, const double* c) {
  double2 s = rmul(c[0], v[0]);
  s = s + rmul(c[1], v[1]);
  s = s + rmul(c[2], v[2]);
  return s + rmul(c[3], v[3]);
}
__device__ __forceinline__ double2 dot5(const double2* v, const double* c) {
  double2 s = rmul(c[0], v[0]);
#pragma unroll
  for (int j = 1; j < 5; ++j) s = s + rmul(c[j], v[j]);
  return s;
}

}  // namespace

// Arithmetic of the v' / u, w pass: FP64, or double-float in the mixed and
// double-float paths (the FP64 pipe is the bound of this kernel).  The Step1
// result is parked in the field's w slot between the two sweeps (16 bytes
// either way).
template <typename R> struct DerivOps;
template <> struct DerivOps<double> {
  using C = double2;
  __device__ static C in(double2 v) { return v; }
  __device__ static double scal(double v) { return v; }
  __device__ static C rm(double c, C x) { return make_double2(c * x.x, c * x.y); }
  __device__ static void park(double2* p, C x) { *p = x; }
  __device__ static C unpark(const double2* p) { return *p; }
  __device__ static double2 out(C x) { return x; }
  // coefficient tables: d1 and d0 rows of der, D0mat factors
  __device__ static double d1(const double* der, const dd*, int iy, int j) { return __ldg(der + (size_t)iy * 20 + 5 + j); }
  __device__ static double d0(const double* der, const dd*, int iy, int j) { return __ldg(der + (size_t)iy * 20 + j); }
  __device__ static double lu(const double* d0lu, const dd*, int iy, int j) { return __ldg(d0lu + (size_t)(iy - 1) * 5 + j); }
};
template <> struct DerivOps<dd> {
  using C = cdd;
  __device__ static C in(double2 v) { return cdd{dd_from_double(v.x), dd_from_double(v.y)}; }
  __device__ static dd scal(double v) { return dd_from_double(v); }
  __device__ static C rm(dd c, C x) { return cdd{c * x.x, c * x.y}; }
  __device__ static void park(double2* p, C x) { *reinterpret_cast<cdd*>(p) = x; }
  __device__ static C unpark(const double2* p) { return *reinterpret_cast<const cdd*>(p); }
  __device__ static double2 out(C x) { return make_double2(dd_to_double_int(x.x), dd_to_double_int(x.y)); }
  __device__ static dd ld(const dd* t) {
    const float2 f = __ldg(reinterpret_cast<const float2*>(t));
    return dd(f.x, f.y);
  }
  __device__ static dd d1(const double*, const dd* t, int iy, int j) { return ld(t + (size_t)iy * 15 + j); }
  __device__ static dd d0(const double*, const dd* t, int iy, int j) { return ld(t + (size_t)iy * 15 + 10 + j); }
  __device__ static dd lu(const double*, const dd* t, int iy, int j) { return ld(t + (size_t)iy * 15 + 5 + j); }
};

// One mode per thread: COMPLEXderiv + Step1(D0mat) bottom-up, then
// Step2(D0mat) and u, w top-down (dnsdata.f90:339-373,
// linsolve_blocking.inc:99-103).  lindd: per row y, the d1 row, the D0mat
// factors and the d0 row in double-float (15 values).
template <typename R>
__device__ __forceinline__ void deriv_uw(double2* __restrict__ V, const double* __restrict__ der,
                                         const double* __restrict__ d0lu, const dd* __restrict__ lindd,
                                         const BcRows& bc, const Dims& d, int m, double ka, double kz, double k2) {
  using O = DerivOps<R>;
  using C = typename O::C;
  const int ny = d.ny;
  const double rk2 = 1.0 / k2;
  const R au = O::scal(ka * rk2), bu = O::scal(kz * rk2);
  C vlo[5], vhi[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    vlo[j] = O::in(V[vidx(d, 1, -1 + j, m)]);
    vhi[j] = O::in(V[vidx(d, 1, ny - 3 + j, m)]);
  }
  auto dot5r = [&](const C* v, const double* c) {
    C acc = O::rm(O::scal(c[0]), v[0]);
#pragma unroll
    for (int j = 1; j < 5; ++j) acc = acc + O::rm(O::scal(c[j]), v[j]);
    return acc;
  };
  const C f0 = dot5r(vlo, bc.d140), fm1 = dot5r(vlo, bc.d14m1);
  const C fn = dot5r(vhi, bc.d14n), fn1 = dot5r(vhi, bc.d14np1);
  {
    C win[5];  // v(iy-2..iy+2) sliding downwards
    win[1] = vhi[1];
    win[2] = vhi[2];
    win[3] = vhi[3];
    win[4] = vhi[4];
    C x1 = C(), x2 = C();
    x1.x = R(); x1.y = R(); x2 = x1;
    double2 wnext = V[vidx(d, 1, ny - 3, m)];  // v one row ahead
    for (int iy = ny - 1; iy >= 1; --iy) {
      win[0] = O::in(wnext);
      if (iy > 1) wnext = V[vidx(d, 1, iy - 3, m)];
      C f = O::rm(O::d1(der, lindd, iy, 0), win[0]);
#pragma unroll
      for (int j = 1; j < 5; ++j) f = f + O::rm(O::d1(der, lindd, iy, j), win[j]);
      if (iy == ny - 1) f = f - (O::rm(O::d0(der, lindd, iy, 3), fn) + O::rm(O::d0(der, lindd, iy, 4), fn1));
      if (iy == ny - 2) f = f - O::rm(O::d0(der, lindd, iy, 4), fn);
      if (iy == 1) f = f - (O::rm(O::d0(der, lindd, iy, 1), f0) + O::rm(O::d0(der, lindd, iy, 0), fm1));
      if (iy == 2) f = f - O::rm(O::d0(der, lindd, iy, 0), f0);
      // Step1 of D0mat: x = A2 (f - A3 x1 - A4 x2)
      C x;
      if constexpr (std::is_same<R, double>::value) {
        x = step1u(f, O::lu(d0lu, lindd, iy, 2), O::lu(d0lu, lindd, iy, 3), O::lu(d0lu, lindd, iy, 4), x1, x2);
      } else {
        const C s = O::rm(O::lu(d0lu, lindd, iy, 3), x1) + O::rm(O::lu(d0lu, lindd, iy, 4), x2);
        x = O::rm(O::lu(d0lu, lindd, iy, 2), f - s);
      }
      x2 = x1;
      x1 = x;
      O::park(&V[vidx(d, 2, iy, m)], x);
#pragma unroll
      for (int j = 4; j > 0; --j) win[j] = win[j - 1];
    }
  }
  {
    C bm2 = fm1, bm1 = fm1;
    bm2.x = R(); bm2.y = R();
    double2 etn = V[vidx(d, 0, -1, m)], xn = make_double2(0.0, 0.0);  // eta and Step1 results one row ahead
    for (int iy = -1; iy <= ny + 1; ++iy) {
      const C et = O::in(etn);
      const double2 xs = xn;
      if (iy < ny + 1) etn = V[vidx(d, 0, iy + 1, m)];
      if (iy + 1 >= 1 && iy + 1 <= ny - 1) xn = V[vidx(d, 2, iy + 1, m)];
      C vp;
      if (iy == -1) vp = fm1;
      else if (iy == 0) vp = f0;
      else if (iy == ny) vp = fn;
      else if (iy == ny + 1) vp = fn1;
      else if constexpr (std::is_same<R, double>::value)  // Step2 of D0mat: vp = x - (l2 bm2 + l1 bm1)
        vp = step2(O::unpark(&xs), O::lu(d0lu, lindd, iy, 0), O::lu(d0lu, lindd, iy, 1), bm2, bm1);
      else
        vp = O::unpark(&xs) - (O::rm(O::lu(d0lu, lindd, iy, 0), bm2) + O::rm(O::lu(d0lu, lindd, iy, 1), bm1));
      if (iy >= 0 && iy <= ny - 1) {
        bm2 = bm1;
        bm1 = vp;
      }
      // u = (i kx v' - i kz eta)/k2, w = (i kz v' + i kx eta)/k2; in FP64 with
      // explicit fused multiply-adds, so that the per-component kernel
      // (deriv_uw_c) rounds exactly alike
      C u, w;
      if constexpr (std::is_same<R, double>::value) {
        u.x = fma(bu, et.y, -(au * vp.y));
        u.y = fma(au, vp.x, -(bu * et.x));
        w.x = fma(-au, et.y, -(bu * vp.y));
        w.y = fma(bu, vp.x, au * et.x);
      } else {
        u.x = bu * et.y - au * vp.y;
        u.y = au * vp.x - bu * et.x;
        w.x = R() - bu * vp.y - au * et.y;
        w.y = bu * vp.x + au * et.x;
      }
      V[vidx(d, 0, iy, m)] = O::out(u);
      V[vidx(d, 2, iy, m)] = O::out(w);
    }
  }
}

// Two threads per pair (kx, +-kz): role 0 owns the v system (D2vmat), role 1
// the eta system (etamat; for the mean mode also the unit-forcing response).
// A block holds 32 pairs: warp 0 the v systems, warp 1 the eta systems.  After
// both have written v and eta, role r takes mode (kx, (1-2r)|kz|) for v' and
// the u, w recovery.
// registers capped for 8 resident 64-thread blocks per SM: at 147 456 pairs
// (383x384x383) the extra warps hide the recurrences' latency (-19% per
// launch); at 16 384 pairs the grid, not the registers, limits residency.
// FACTORED: the factorisation ran before (k_factor, kFacPerRow values per
// row and pair, the mean mode's wall terms in sc->wallrhs); pass A loads each
// row's 1/d, u1, u2 and pass B its l2, l1 instead of assembling and
// factoring.
template <bool FACTORED>
__global__ void __launch_bounds__(64, 8) k_linsolve(double2* __restrict__ V, const double2* rhs, size_t rcs, int roff,
                                                 double* __restrict__ fac, const double* __restrict__ der,
                                                 const double* __restrict__ d0lu, const double* __restrict__ yint,
                                                 BcRows bc, Dims d, double lambda_in, double ode1,
                                                 int lambda_from_dt, DevScalars* __restrict__ sc,
                                                 const dd* __restrict__ lindd, const double* __restrict__ nud,
                                                 int q_lo, int q_hi) {
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;
  const int q = q_lo + blockIdx.x * 32 + lane;
  const bool active = q < q_hi;
  const int ny = d.ny, nz = d.nz;
  const int ix = active ? q / (nz + 1) : 0;
  const int a = active ? q - ix * (nz + 1) : 0;
  const int nm = (a == 0) ? 1 : 2;
  int mm[2];
  mm[0] = ix * d.nzt + nz + a;
  mm[1] = ix * d.nzt + nz - a;
  const bool is00 = (ix == 0 && a == 0);
  const double ka = ix * d.alfa0, kb = a * d.beta0;
  const double k2 = ka * ka + kb * kb;
  const double lambda = lambda_from_dt ? ode1 / sc->deltat : lambda_in;
  const double ni = d.ni;
  const size_t P = d.npairs;
  const int vc = role == 0 ? 1 : 0;  // field component this role solves for (v or eta)
  // boundary rows of this role's system, selected element by element
  double bot[5], botm1[5], top[5], topp1[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    bot[j] = role ? bc.eta0bc[j] : bc.v0bc[j];
    botm1[j] = role ? bc.eta0m1bc[j] : bc.v0m1bc[j];
    top[j] = role ? bc.etanbc[j] : bc.vnbc[j];
    topp1[j] = role ? bc.etanp1bc[j] : bc.vnp1bc[j];
  }
  // wall values: zero except the mean mode's packed U+iW (channel.f90:122-124)
  const double bval0 = (role == 1 && is00) ? sc->u0 : 0.0;
  const double bvaln = (role == 1 && is00) ? sc->uN : 0.0;
  const bool ucor = role == 1 && is00;
  const AsmCoef ac = asm_coef(lambda, k2, ni);

  // fac layout: kFacPerRow values per row (l2, l1, 1/d, u1, u2 of each
  // system) when factored ahead, else the fused kernel's own l2, l1
  constexpr int FS = FACTORED ? kFacPerRow : kFacPerRowFused, RS = FACTORED ? 5 : 2;
  if (active) {
    // ---- pass A: bottom-up assembly + BC fold + factor + Step1 ----
    double L1[2] = {0, 0}, L2[2] = {0, 0};
    double2 x1[2] = {cz(), cz()}, x2[2] = {cz(), cz()};
    double2 xc1 = cz(), xc2 = cz();
    const double2* rsrc = rhs + (role == 0 ? rcs : 0);
    // right-hand sides (and factors) one row ahead of the recurrence
    // (global-load latency)
    double2 bnext[2] = {cz(), cz()};
#pragma unroll
    for (int t = 0; t < 2; ++t)
      if (t < nm) bnext[t] = rsrc[(size_t)(ny - 1 + roff) * d.nmodes + mm[t]];
    double fnext[3] = {0, 0, 0};
    if constexpr (FACTORED) {
      const double* f = fac + ((size_t)(ny - 2) * FS + RS * role + 2) * P + q;
      fnext[0] = f[0];
      fnext[1] = f[P];
      fnext[2] = f[2 * P];
    }
    for (int iy = ny - 1; iy >= 1; --iy) {
      const double* dr = der + (size_t)iy * 20;
      double2 b[2] = {bnext[0], bnext[1]};
      double A[5];
      if constexpr (FACTORED) {
        A[2] = fnext[0];
        A[3] = fnext[1];
        A[4] = fnext[2];
      }
      if (iy > 1) {
#pragma unroll
        for (int t = 0; t < 2; ++t)
          if (t < nm) bnext[t] = rsrc[(size_t)(iy - 1 + roff) * d.nmodes + mm[t]];
        if constexpr (FACTORED) {
          const double* f = fac + ((size_t)(iy - 2) * FS + RS * role + 2) * P + q;
          fnext[0] = f[0];
          fnext[1] = f[P];
          fnext[2] = f[2 * P];
        }
      }
      if constexpr (FACTORED) {
        if (role == 1 && is00) {  // the wall terms k_factor stored (linsolve_blocking.inc:26-27,40-41)
          if (iy == 1) b[0] = b[0] - make_double2(sc->wallrhs[0], sc->wallrhs[1]);
          if (iy == 2) b[0] = b[0] - make_double2(sc->wallrhs[2], sc->wallrhs[3]);
          if (iy == ny - 2) b[0] = b[0] - make_double2(sc->wallrhs[4], sc->wallrhs[5]);
          if (iy == ny - 1) b[0] = b[0] - make_double2(sc->wallrhs[6], sc->wallrhs[7]);
        }
      } else {
        // warp-uniform: each warp assembles only its own matrix; the products
        // -ni d4 and -ni d2, the same for every mode, come from the per-row
        // table nud when there is one
        if (role) {
#pragma unroll
          for (int j = 0; j < 5; ++j) {
            const double p2 = nud ? __ldg(nud + (size_t)iy * 10 + 5 + j) : ac.ce2 * __ldg(dr + 10 + j);
            A[j] = fma(ac.ce0, __ldg(dr + j), p2);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 5; ++j) {
            const double p4 = nud ? __ldg(nud + (size_t)iy * 10 + j) : ac.cv4 * __ldg(dr + 15 + j);
            A[j] = fma(ac.cv0, __ldg(dr + j), fma(ac.cv2, __ldg(dr + 10 + j), p4));
          }
        }
        if (iy == ny - 1) bc_top1(A, top, topp1);
        if (iy == ny - 2) bc_top2(A, top);
        if (iy == 1) bc_bot1(A, bot, botm1);
        if (iy == 2) bc_bot2(A, bot);
        if (role == 1 && is00) {  // the packed wall velocity enters rows 1, 2, ny-2, ny-1 (linsolve_blocking.inc:26-27,40-41)
          if (iy == 1) b[0] = b[0] - make_double2(A[1] * bval0 / bot[1], A[1] * 0.0 / bot[1]);
          if (iy == 2) b[0] = b[0] - make_double2(A[0] * bval0 / bot[1], A[0] * 0.0 / bot[1]);
          if (iy == ny - 1) b[0] = b[0] - make_double2(A[3] * bvaln / top[3], A[3] * 0.0 / top[3]);
          if (iy == ny - 2) b[0] = b[0] - make_double2(A[4] * bvaln / top[3], A[4] * 0.0 / top[3]);
        }
        if (iy == ny - 1) { A[3] = 0; A[4] = 0; }  // rbparmat_blocking.f90:29
        if (iy == ny - 2) A[4] = 0;
        lu_row(A, L1, L2);
      }
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        if (t < nm) {
          const double2 nx_ = step1(b[t], A, x1[t], x2[t]);
          x2[t] = x1[t];
          x1[t] = nx_;
          V[vidx(d, vc, iy, mm[t])] = nx_;
        }
      }
      if (ucor) {
        const double2 nc = step1(make_double2(1.0, 0.0), A, xc1, xc2);
        xc2 = xc1;
        xc1 = nc;
        V[vidx(d, 2, iy, mm[0])] = nc;
      }
      if constexpr (!FACTORED) {
        L2[0] = L1[0]; L2[1] = L1[1];
        L1[0] = A[0]; L1[1] = A[1];
        if (iy == 1) { A[0] = 0; A[1] = 0; }  // rbparmat_blocking.f90:45
        if (iy == 2) A[0] = 0;
        double* f = fac + ((size_t)(iy - 1) * FS + RS * role) * P + q;
        f[0] = A[0];
        f[P] = A[1];
      }
    }
    // ---- pass B: top-down Step2; rows 1..3 and ny-3..ny-1 kept for the walls ----
    double2 lo[2][3], hi[2][3], clo[3], chi[3];
    {
      double2 m2[2] = {cz(), cz()}, m1[2] = {cz(), cz()}, c2 = cz(), c1 = cz();
      // factors and Step1 results one row ahead
      const double* f1 = fac + ((size_t)0 * FS + RS * role) * P + q;
      double l2n = f1[0], l1n = f1[P];
      double2 vn[2] = {cz(), cz()};
#pragma unroll
      for (int t = 0; t < 2; ++t)
        if (t < nm) vn[t] = V[vidx(d, vc, 1, mm[t])];
      for (int iy = 1; iy <= ny - 1; ++iy) {
        const double l2 = l2n, l1 = l1n;
        const double2 vcur[2] = {vn[0], vn[1]};
        if (iy < ny - 1) {
          const double* f = fac + ((size_t)iy * FS + RS * role) * P + q;
          l2n = f[0];
          l1n = f[P];
#pragma unroll
          for (int t = 0; t < 2; ++t)
            if (t < nm) vn[t] = V[vidx(d, vc, iy + 1, mm[t])];
        }
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          if (t < nm) {
            const double2 nv = step2(vcur[t], l2, l1, m2[t], m1[t]);
            V[vidx(d, vc, iy, mm[t])] = nv;
            m2[t] = m1[t];
            m1[t] = nv;
            if (iy == 1) lo[t][0] = nv;
            if (iy == 2) lo[t][1] = nv;
            if (iy == 3) lo[t][2] = nv;
            if (iy == ny - 3) hi[t][0] = nv;
            if (iy == ny - 2) hi[t][1] = nv;
            if (iy == ny - 1) hi[t][2] = nv;
          }
        }
        if (ucor) {
          const double2 nc = step2(V[vidx(d, 2, iy, mm[0])], l2, l1, c2, c1);
          V[vidx(d, 2, iy, mm[0])] = nc;
          c2 = c1;
          c1 = nc;
          if (iy == 1) clo[0] = nc;
          if (iy == 2) clo[1] = nc;
          if (iy == 3) clo[2] = nc;
          if (iy == ny - 3) chi[0] = nc;
          if (iy == ny - 2) chi[1] = nc;
          if (iy == ny - 1) chi[2] = nc;
        }
      }
    }
    // wall and ghost values (linsolve_blocking.inc:50-61)
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (t < nm) {
        const double2 w0 = cdivr(make_double2(bval0, 0.0) - dot3(lo[t], bot + 2), bot[1]);
        const double2 rb[4] = {w0, lo[t][0], lo[t][1], lo[t][2]};
        const double2 wm1 = cdivr(cz() - dot4(rb, botm1 + 1), botm1[0]);
        const double2 wn = cdivr(make_double2(bvaln, 0.0) - dot3(hi[t], top), top[3]);
        const double2 rt[4] = {hi[t][0], hi[t][1], hi[t][2], wn};
        const double2 wn1 = cdivr(cz() - dot4(rt, topp1), topp1[4]);
        V[vidx(d, vc, -1, mm[t])] = wm1;
        V[vidx(d, vc, 0, mm[t])] = w0;
        V[vidx(d, vc, ny, mm[t])] = wn;
        V[vidx(d, vc, ny + 1, mm[t])] = wn1;
      }
    }
    if (ucor) {  // mean flow (linsolve_blocking.inc:62-97)
      const int m = mm[0];
      const double2 c0 = cdivr(cz() - dot3(clo, bot + 2), bot[1]);
      const double2 rb[4] = {c0, clo[0], clo[1], clo[2]};
      const double2 cm1 = cdivr(cz() - dot4(rb, botm1 + 1), botm1[0]);
      const double2 cn = cdivr(cz() - dot3(chi, top), top[3]);
      const double2 rt[4] = {chi[0], chi[1], chi[2], cn};
      const double2 cn1 = cdivr(cz() - dot4(rt, topp1), topp1[4]);
      V[vidx(d, 2, -1, m)] = cm1;
      V[vidx(d, 2, 0, m)] = c0;
      V[vidx(d, 2, ny, m)] = cn;
      V[vidx(d, 2, ny + 1, m)] = cn1;
      // flow rates by the non-uniform Simpson rule (dnsdata.f90:312-324)
      double fu = 0.0, fw = 0.0, fc = 0.0;
      for (int iy = 1, k = 0; iy <= ny - 1; iy += 2, ++k) {
        const double a1 = yint[3 * k], a2 = yint[3 * k + 1], a3 = yint[3 * k + 2];
        const double2 e0 = V[vidx(d, 0, iy - 1, m)], e1 = V[vidx(d, 0, iy, m)], e2 = V[vidx(d, 0, iy + 1, m)];
        const double2 u0 = V[vidx(d, 2, iy - 1, m)], u1 = V[vidx(d, 2, iy, m)], u2 = V[vidx(d, 2, iy + 1, m)];
        fu = fu + a1 * e0.x + a2 * e1.x + a3 * e2.x;
        fw = fw + a1 * e0.y + a2 * e1.y + a3 * e2.y;
        fc = fc + a1 * u0.x + a2 * u1.x + a3 * u2.x;
      }
      double corrpx = sc->corrpx, corrpz = sc->corrpz;
      const bool cx = fabs(d.meanflowx) > 1.0e-7 && !d.cpi;
      const bool cz_ = fabs(d.meanflowz) > 1.0e-7 && !d.cpi;
      if (cx) corrpx = (d.meanflowx - fu) / fc;
      if (cz_) corrpz = (d.meanflowz - fw) / fc;
      for (int iy = -1; iy <= ny + 1; ++iy) {
        const double2 et = V[vidx(d, 0, iy, m)];
        const double uc = V[vidx(d, 2, iy, m)].x;
        double U = et.x, W = et.y;
        if (cx) U = U + corrpx * uc;
        if (cz_) W = W + corrpz * uc;
        V[vidx(d, 0, iy, m)] = make_double2(U, 0.0);
        V[vidx(d, 2, iy, m)] = make_double2(W, 0.0);
      }
      sc->fr[0] = fu; sc->fr[1] = fw; sc->fr[2] = fc;
      sc->corrpx = corrpx; sc->corrpz = corrpz;
      if (d.cpi) {
        if (d.cpi_type == 0) sc->meanpx = (1 - d.gamma) * 6 * ni / fu;
        else sc->meanpx = (1.5 / d.gamma) * fu * ni;
      }
    }
  }
  __syncthreads();  // v and eta of this block's pairs are in V
  if (!active || is00 || role >= nm) return;

  if (lindd) deriv_uw<dd>(V, der, d0lu, lindd, bc, d, mm[role], ka, (role == 0 ? 1.0 : -1.0) * kb, k2);
  else deriv_uw<double>(V, der, d0lu, lindd, bc, d, mm[role], ka, (role == 0 ? 1.0 : -1.0) * kb, k2);
}

// The same solves in two kernels, for grids with few pairs (the fused kernel
// has too few warps per SM there to hide its recurrences' latency):
//
// k_factor: two threads per pair (kx, +-kz), whose matrices are equal because
// k^2 is: role 0 the v system (D2vmat), role 1 the eta system (etamat).
// Bottom-up (iy = ny-1..1): assemble, fold the boundary rows, LU5decompStep
// row; each row's factors go to fac[iy-1][5 role + {l2, l1, 1/d, u1, u2}][q]
// (l2, l1 the scaled lower entries LeftLU5divStep2 reads, 1/d, u1, u2 the
// reciprocal pivot and upper entries LeftLU5divStep1 reads).  The eta thread
// of the mean mode also stores the wall-velocity terms of its right-hand side
// (rows 1, 2, ny-2, ny-1; linsolve_blocking.inc:26-27,40-41).
// Registers capped for 8 resident 64-thread blocks per SM.
__global__ void __launch_bounds__(64, 8) k_factor(double* __restrict__ fac, const double* __restrict__ der,
                                                  BcRows bc, Dims d, double lambda_in, double ode1,
                                                  int lambda_from_dt, DevScalars* __restrict__ sc,
                                                  const double* __restrict__ nud, int q_lo, int q_hi) {
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;
  const int q = q_lo + blockIdx.x * 32 + lane;
  if (q >= q_hi) return;
  const int ny = d.ny, nz = d.nz;
  const int ix = q / (nz + 1);
  const int a = q - ix * (nz + 1);
  const bool is00 = (ix == 0 && a == 0);
  const double ka = ix * d.alfa0, kb = a * d.beta0;
  const double k2 = ka * ka + kb * kb;
  const double lambda = lambda_from_dt ? ode1 / sc->deltat : lambda_in;
  const size_t P = d.npairs;
  double bot[5], botm1[5], top[5], topp1[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    bot[j] = role ? bc.eta0bc[j] : bc.v0bc[j];
    botm1[j] = role ? bc.eta0m1bc[j] : bc.v0m1bc[j];
    top[j] = role ? bc.etanbc[j] : bc.vnbc[j];
    topp1[j] = role ? bc.etanp1bc[j] : bc.vnp1bc[j];
  }
  const bool wallrhs = role == 1 && is00;  // the packed wall velocity U+iW (channel.f90:122-124)
  const double bval0 = wallrhs ? sc->u0 : 0.0, bvaln = wallrhs ? sc->uN : 0.0;
  const AsmCoef ac = asm_coef(lambda, k2, d.ni);
  double L1[2] = {0, 0}, L2[2] = {0, 0};
  for (int iy = ny - 1; iy >= 1; --iy) {
    const double* dr = der + (size_t)iy * 20;
    // warp-uniform: each warp assembles only its own matrix; the products
    // -ni d4 and -ni d2, the same for every mode, come from the per-row
    // table nud when there is one
    double A[5];
    if (role) {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const double p2 = nud ? __ldg(nud + (size_t)iy * 10 + 5 + j) : ac.ce2 * __ldg(dr + 10 + j);
        A[j] = fma(ac.ce0, __ldg(dr + j), p2);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const double p4 = nud ? __ldg(nud + (size_t)iy * 10 + j) : ac.cv4 * __ldg(dr + 15 + j);
        A[j] = fma(ac.cv0, __ldg(dr + j), fma(ac.cv2, __ldg(dr + 10 + j), p4));
      }
    }
    if (iy == ny - 1) bc_top1(A, top, topp1);
    if (iy == ny - 2) bc_top2(A, top);
    if (iy == 1) bc_bot1(A, bot, botm1);
    if (iy == 2) bc_bot2(A, bot);
    if (wallrhs) {  // subtracted from the right-hand side of these rows by k_solve
      if (iy == 1) { sc->wallrhs[0] = A[1] * bval0 / bot[1]; sc->wallrhs[1] = A[1] * 0.0 / bot[1]; }
      if (iy == 2) { sc->wallrhs[2] = A[0] * bval0 / bot[1]; sc->wallrhs[3] = A[0] * 0.0 / bot[1]; }
      if (iy == ny - 2) { sc->wallrhs[4] = A[4] * bvaln / top[3]; sc->wallrhs[5] = A[4] * 0.0 / top[3]; }
      if (iy == ny - 1) { sc->wallrhs[6] = A[3] * bvaln / top[3]; sc->wallrhs[7] = A[3] * 0.0 / top[3]; }
    }
    if (iy == ny - 1) { A[3] = 0; A[4] = 0; }  // rbparmat_blocking.f90:29
    if (iy == ny - 2) A[4] = 0;
    lu_row(A, L1, L2);
    L2[0] = L1[0]; L2[1] = L1[1];
    L1[0] = A[0]; L1[1] = A[1];
    if (iy == 1) { A[0] = 0; A[1] = 0; }  // rbparmat_blocking.f90:45
    if (iy == 2) A[0] = 0;
    double* f = fac + ((size_t)(iy - 1) * kFacPerRow + 5 * role) * P + q;
    f[0] = A[0];
    f[P] = A[1];
    f[2 * P] = A[2];
    f[3 * P] = A[3];
    f[4 * P] = A[4];
  }
}

// L1 prefetch of a line the thread will load some rows later (no register
// is held for it); every address passed is inside its buffer
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
constexpr int kSolvePrefetch = 6;  // rows ahead

// k_solve: four threads per pair, one per (system, mode): warp 0 (v, +kz),
// warp 1 (v, -kz), warp 2 (eta, +kz), warp 3 (eta, -kz).  The (eta, -kz)
// thread of the mean pair, whose mode does not exist, solves the mean
// mode's unit-forcing response instead.  Each: LeftLU5divStep1 bottom-up and
// LeftLU5divStep2 top-down with the factors of k_factor (rbparmat_blocking.f90:
// 57-100), then the wall and ghost values (linsolve_blocking.inc:50-61).
// After a block barrier the mean pair's eta thread makes the mean-flow
// correction (:62-97), and warps 0 and 1 take v' and the u, w recovery of
// the +kz and -kz modes (:99-103).
__global__ void __launch_bounds__(128, 4) k_solve(double2* __restrict__ V, const double2* rhs, size_t rcs, int roff,
                                                  const double* __restrict__ fac, const double* __restrict__ der,
                                                  const double* __restrict__ d0lu, const double* __restrict__ yint,
                                                  BcRows bc, Dims d, DevScalars* __restrict__ sc,
                                                  const dd* __restrict__ lindd, int q_lo, int q_hi) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sys = w >> 1, t = w & 1;
  const int q = q_lo + blockIdx.x * 32 + lane;
  const bool active = q < q_hi;
  const int ny = d.ny, nz = d.nz;
  const int ix = active ? q / (nz + 1) : 0;
  const int a = active ? q - ix * (nz + 1) : 0;
  const int nm = (a == 0) ? 1 : 2;
  int mm[2];
  mm[0] = ix * d.nzt + nz + a;
  mm[1] = ix * d.nzt + nz - a;
  const bool is00 = (ix == 0 && a == 0);
  const double ka = ix * d.alfa0, kb = a * d.beta0;
  const double k2 = ka * ka + kb * kb;
  const double ni = d.ni;
  const size_t P = d.npairs;
  const bool ucor = active && is00 && sys == 1 && t == 1;  // unit-forcing response (linsolve_blocking.inc:62-68)
  const bool mine = active && t < nm;
  const int m = mm[ucor ? 0 : t];
  const int vc = ucor ? 2 : (sys == 0 ? 1 : 0);  // field slot written
  const bool wallrhs = mine && sys == 1 && is00;
  double bot[5], botm1[5], top[5], topp1[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    bot[j] = sys ? bc.eta0bc[j] : bc.v0bc[j];
    botm1[j] = sys ? bc.eta0m1bc[j] : bc.v0m1bc[j];
    top[j] = sys ? bc.etanbc[j] : bc.vnbc[j];
    topp1[j] = sys ? bc.etanp1bc[j] : bc.vnp1bc[j];
  }
  const double bval0 = wallrhs ? sc->u0 : 0.0, bvaln = wallrhs ? sc->uN : 0.0;
  if (mine || ucor) {
    const double* fs = fac + (size_t)5 * sys * P + q;  // this system's factors of row 1
    const size_t frow = (size_t)kFacPerRow * P;
    // ---- Step1 bottom-up: x = (b - u1 x(+1) - u2 x(+2)) / d ----
    const double2* rsrc = rhs + (sys == 0 ? rcs : 0);
    double2 x1 = cz(), x2 = cz();
    double2 bn = ucor ? make_double2(1.0, 0.0) : rsrc[(size_t)(ny - 1 + roff) * d.nmodes + m];
    const double* f = fs + (size_t)(ny - 2) * frow;
    double dn = f[2 * P], u1n = f[3 * P], u2n = f[4 * P];
    for (int iy = ny - 1; iy >= 1; --iy) {
      double2 b = bn;
      const double dv = dn, u1 = u1n, u2 = u2n;
      if (iy > 1) {  // one row ahead (global-load latency)
        if (!ucor) bn = rsrc[(size_t)(iy - 1 + roff) * d.nmodes + m];
        f -= frow;
        dn = f[2 * P];
        u1n = f[3 * P];
        u2n = f[4 * P];
      }
      if (iy - kSolvePrefetch >= 1) {  // and the lines of a row further down
        const double* fp = f - (size_t)(kSolvePrefetch - 1) * frow;
        prefetch_l1(fp + 2 * P);
        prefetch_l1(fp + 3 * P);
        prefetch_l1(fp + 4 * P);
        if (!ucor) prefetch_l1(rsrc + (size_t)(iy - kSolvePrefetch + roff) * d.nmodes + m);
      }
      if (wallrhs) {
        if (iy == 1) b = b - make_double2(sc->wallrhs[0], sc->wallrhs[1]);
        if (iy == 2) b = b - make_double2(sc->wallrhs[2], sc->wallrhs[3]);
        if (iy == ny - 2) b = b - make_double2(sc->wallrhs[4], sc->wallrhs[5]);
        if (iy == ny - 1) b = b - make_double2(sc->wallrhs[6], sc->wallrhs[7]);
      }
      const double2 x = step1u(b, dv, u1, u2, x1, x2);
      x2 = x1;
      x1 = x;
      V[vidx(d, vc, iy, m)] = x;
    }
    // ---- Step2 top-down: v = x - l2 v(-2) - l1 v(-1); rows 1..3 and ny-3..ny-1 kept ----
    double2 lo[3], hi[3];
    double2 m2 = cz(), m1 = cz();
    f = fs;
    double l2n = f[0], l1n = f[P];
    double2 vn = V[vidx(d, vc, 1, m)];
    for (int iy = 1; iy <= ny - 1; ++iy) {
      const double l2 = l2n, l1 = l1n;
      const double2 vcur = vn;
      if (iy < ny - 1) {
        f += frow;
        l2n = f[0];
        l1n = f[P];
        vn = V[vidx(d, vc, iy + 1, m)];
      }
      if (iy + kSolvePrefetch <= ny - 1) {
        const double* fp = f + (size_t)(kSolvePrefetch - 1) * frow;
        prefetch_l1(fp);
        prefetch_l1(fp + P);
        prefetch_l1(&V[vidx(d, vc, iy + kSolvePrefetch, m)]);
      }
      const double2 nv = step2(vcur, l2, l1, m2, m1);
      V[vidx(d, vc, iy, m)] = nv;
      m2 = m1;
      m1 = nv;
      if (iy == 1) lo[0] = nv;
      if (iy == 2) lo[1] = nv;
      if (iy == 3) lo[2] = nv;
      if (iy == ny - 3) hi[0] = nv;
      if (iy == ny - 2) hi[1] = nv;
      if (iy == ny - 1) hi[2] = nv;
    }
    // wall and ghost values (linsolve_blocking.inc:50-61)
    const double2 w0 = cdivr(make_double2(bval0, 0.0) - dot3(lo, bot + 2), bot[1]);
    const double2 rb[4] = {w0, lo[0], lo[1], lo[2]};
    const double2 wm1 = cdivr(cz() - dot4(rb, botm1 + 1), botm1[0]);
    const double2 wn = cdivr(make_double2(bvaln, 0.0) - dot3(hi, top), top[3]);
    const double2 rt[4] = {hi[0], hi[1], hi[2], wn};
    const double2 wn1 = cdivr(cz() - dot4(rt, topp1), topp1[4]);
    V[vidx(d, vc, -1, m)] = wm1;
    V[vidx(d, vc, 0, m)] = w0;
    V[vidx(d, vc, ny, m)] = wn;
    V[vidx(d, vc, ny + 1, m)] = wn1;
  }
  __syncthreads();  // v, eta (and the unit response) of this block's pairs are in V
  if (wallrhs) {  // mean flow (linsolve_blocking.inc:62-97)
    // flow rates by the non-uniform Simpson rule (dnsdata.f90:312-324)
    double fu = 0.0, fw = 0.0, fc = 0.0;
    for (int iy = 1, k = 0; iy <= ny - 1; iy += 2, ++k) {
      const double a1 = yint[3 * k], a2 = yint[3 * k + 1], a3 = yint[3 * k + 2];
      const double2 e0 = V[vidx(d, 0, iy - 1, m)], e1 = V[vidx(d, 0, iy, m)], e2 = V[vidx(d, 0, iy + 1, m)];
      const double2 u0 = V[vidx(d, 2, iy - 1, m)], u1 = V[vidx(d, 2, iy, m)], u2 = V[vidx(d, 2, iy + 1, m)];
      fu = fu + a1 * e0.x + a2 * e1.x + a3 * e2.x;
      fw = fw + a1 * e0.y + a2 * e1.y + a3 * e2.y;
      fc = fc + a1 * u0.x + a2 * u1.x + a3 * u2.x;
    }
    double corrpx = sc->corrpx, corrpz = sc->corrpz;
    const bool cx = fabs(d.meanflowx) > 1.0e-7 && !d.cpi;
    const bool cz_ = fabs(d.meanflowz) > 1.0e-7 && !d.cpi;
    if (cx) corrpx = (d.meanflowx - fu) / fc;
    if (cz_) corrpz = (d.meanflowz - fw) / fc;
    for (int iy = -1; iy <= ny + 1; ++iy) {
      const double2 et = V[vidx(d, 0, iy, m)];
      const double uc = V[vidx(d, 2, iy, m)].x;
      double U = et.x, W = et.y;
      if (cx) U = U + corrpx * uc;
      if (cz_) W = W + corrpz * uc;
      V[vidx(d, 0, iy, m)] = make_double2(U, 0.0);
      V[vidx(d, 2, iy, m)] = make_double2(W, 0.0);
    }
    sc->fr[0] = fu; sc->fr[1] = fw; sc->fr[2] = fc;
    sc->corrpx = corrpx; sc->corrpz = corrpz;
    if (d.cpi) {
      if (d.cpi_type == 0) sc->meanpx = (1 - d.gamma) * 6 * ni / fu;
      else sc->meanpx = (1.5 / d.gamma) * fu * ni;
    }
  }
  if (!active || is00 || sys != 0 || t >= nm) return;
  if (lindd) deriv_uw<dd>(V, der, d0lu, lindd, bc, d, mm[t], ka, (t == 0 ? 1.0 : -1.0) * kb, k2);
  else deriv_uw<double>(V, der, d0lu, lindd, bc, d, mm[t], ka, (t == 0 ? 1.0 : -1.0) * kb, k2);
}

// ---------------------------------------------------------------------------
// The substitutions with eight threads per (kx, +-kz) pair: the systems'
// coefficients are real, so the real and imaginary parts of every
// recurrence are independent and each (system, mode) thread of k_solve
// splits into two, one per component, with the same operations on each (the
// results are bit-identical to k_solve's).  Twice the warps for a kernel
// whose y recurrences are latency-bound.  Only the u, w recovery mixes the
// components (i kx v', i kz eta): each thread takes its partner's values by
// a shuffle, so no thread reads the half of a slot its partner writes.
// ---------------------------------------------------------------------------
namespace {
// component c of a complex128 in memory
__device__ __forceinline__ const double* cptr(const double2* p, int c) { return reinterpret_cast<const double*>(p) + c; }
__device__ __forceinline__ double* cptr(double2* p, int c) { return reinterpret_cast<double*>(p) + c; }

// one component of DerivOps' arithmetic
template <typename R> struct DerivC;
template <> struct DerivC<double> {
  using S = double;
  __device__ static S in(double v) { return v; }
  __device__ static double scal(double v) { return v; }
  __device__ static S rm(double c, S x) { return c * x; }
  __device__ static void park(double2* p, int c, S x) { *cptr(p, c) = x; }
  __device__ static S unpark(const double2* p, int c) { return *cptr(p, c); }
  __device__ static double out(S x) { return x; }
  __device__ static S partner(S x, unsigned mask) { return __shfl_xor_sync(mask, x, 1); }
};
template <> struct DerivC<dd> {
  using S = dd;
  __device__ static S in(double v) { return dd_from_double(v); }
  __device__ static dd scal(double v) { return dd_from_double(v); }
  __device__ static S rm(dd c, S x) { return c * x; }
  __device__ static void park(double2* p, int c, S x) { reinterpret_cast<float2*>(p)[c] = make_float2(x.hi, x.lo); }
  __device__ static S unpark(const double2* p, int c) {
    const float2 f = reinterpret_cast<const float2*>(p)[c];
    return dd(f.x, f.y);
  }
  __device__ static double out(S x) { return dd_to_double_int(x); }
  __device__ static S partner(S x, unsigned mask) {
    return dd(__shfl_xor_sync(mask, x.hi, 1), __shfl_xor_sync(mask, x.lo, 1));
  }
};

// deriv_uw for component c of mode m (the partner lane, lane ^ 1, holds the
// other component of the same mode; mask: the lanes taking part)
template <typename R>
__device__ __forceinline__ void deriv_uw_c(double2* __restrict__ V, const double* __restrict__ der,
                                           const double* __restrict__ d0lu, const dd* __restrict__ lindd,
                                           const BcRows& bc, const Dims& d, int m, double ka, double kz, double k2,
                                           int c, unsigned mask) {
  using O = DerivOps<R>;
  using Q = DerivC<R>;
  using S = typename Q::S;
  const int ny = d.ny;
  const double rk2 = 1.0 / k2;
  const R au = O::scal(ka * rk2), bu = O::scal(kz * rk2);
  S vlo[5], vhi[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    vlo[j] = Q::in(*cptr(&V[vidx(d, 1, -1 + j, m)], c));
    vhi[j] = Q::in(*cptr(&V[vidx(d, 1, ny - 3 + j, m)], c));
  }
  auto dot5r = [&](const S* v, const double* cf) {
    S acc = Q::rm(Q::scal(cf[0]), v[0]);
#pragma unroll
    for (int j = 1; j < 5; ++j) acc = acc + Q::rm(Q::scal(cf[j]), v[j]);
    return acc;
  };
  const S f0 = dot5r(vlo, bc.d140), fm1 = dot5r(vlo, bc.d14m1);
  const S fn = dot5r(vhi, bc.d14n), fn1 = dot5r(vhi, bc.d14np1);
  {
    S win[5];
    win[1] = vhi[1];
    win[2] = vhi[2];
    win[3] = vhi[3];
    win[4] = vhi[4];
    S x1 = S(), x2 = S();
    double wnext = *cptr(&V[vidx(d, 1, ny - 3, m)], c);
    for (int iy = ny - 1; iy >= 1; --iy) {
      win[0] = Q::in(wnext);
      if (iy > 1) wnext = *cptr(&V[vidx(d, 1, iy - 3, m)], c);
      S f = Q::rm(O::d1(der, lindd, iy, 0), win[0]);
#pragma unroll
      for (int j = 1; j < 5; ++j) f = f + Q::rm(O::d1(der, lindd, iy, j), win[j]);
      if (iy == ny - 1) f = f - (Q::rm(O::d0(der, lindd, iy, 3), fn) + Q::rm(O::d0(der, lindd, iy, 4), fn1));
      if (iy == ny - 2) f = f - Q::rm(O::d0(der, lindd, iy, 4), fn);
      if (iy == 1) f = f - (Q::rm(O::d0(der, lindd, iy, 1), f0) + Q::rm(O::d0(der, lindd, iy, 0), fm1));
      if (iy == 2) f = f - Q::rm(O::d0(der, lindd, iy, 0), f0);
      S x;
      if constexpr (std::is_same<R, double>::value) {
        x = O::lu(d0lu, lindd, iy, 2) * fma(-O::lu(d0lu, lindd, iy, 4), x2, fma(-O::lu(d0lu, lindd, iy, 3), x1, f));
      } else {
        const S s = Q::rm(O::lu(d0lu, lindd, iy, 3), x1) + Q::rm(O::lu(d0lu, lindd, iy, 4), x2);
        x = Q::rm(O::lu(d0lu, lindd, iy, 2), f - s);
      }
      x2 = x1;
      x1 = x;
      Q::park(&V[vidx(d, 2, iy, m)], c, x);
#pragma unroll
      for (int j = 4; j > 0; --j) win[j] = win[j - 1];
    }
  }
  {
    S bm2 = S(), bm1 = fm1;
    double etn = *cptr(&V[vidx(d, 0, -1, m)], c);
    S xn = S();
    for (int iy = -1; iy <= ny + 1; ++iy) {
      const S et = Q::in(etn);
      const S xs = xn;
      if (iy < ny + 1) etn = *cptr(&V[vidx(d, 0, iy + 1, m)], c);
      if (iy + 1 >= 1 && iy + 1 <= ny - 1) xn = Q::unpark(&V[vidx(d, 2, iy + 1, m)], c);
      S vp;
      if (iy == -1) vp = fm1;
      else if (iy == 0) vp = f0;
      else if (iy == ny) vp = fn;
      else if (iy == ny + 1) vp = fn1;
      else if constexpr (std::is_same<R, double>::value)
        vp = fma(-O::lu(d0lu, lindd, iy, 1), bm1, fma(-O::lu(d0lu, lindd, iy, 0), bm2, xs));
      else
        vp = xs - (Q::rm(O::lu(d0lu, lindd, iy, 0), bm2) + Q::rm(O::lu(d0lu, lindd, iy, 1), bm1));
      if (iy >= 0 && iy <= ny - 1) {
        bm2 = bm1;
        bm1 = vp;
      }
      // u = (i kx v' - i kz eta)/k2, w = (i kz v' + i kx eta)/k2: each
      // component takes the other component of v' and eta
      const S vo = Q::partner(vp, mask), eo = Q::partner(et, mask);
      S u, w;
      if constexpr (std::is_same<R, double>::value) {  // deriv_uw's fused forms
        if (c == 0) {
          u = fma(bu, eo, -(au * vo));
          w = fma(-au, eo, -(bu * vo));
        } else {
          u = fma(au, vo, -(bu * eo));
          w = fma(bu, vo, au * eo);
        }
      } else if (c == 0) {
        u = bu * eo - au * vo;
        w = R() - bu * vo - au * eo;
      } else {
        u = au * vo - bu * eo;
        w = bu * vo + au * eo;
      }
      *cptr(&V[vidx(d, 0, iy, m)], c) = Q::out(u);
      *cptr(&V[vidx(d, 2, iy, m)], c) = Q::out(w);
    }
  }
}
}  // namespace

// Eight threads per pair: warp w is the role of k_solve's warp w (system w/2,
// mode w%2); lane l takes pair l/2 of the block's 16 and component l%2.
__global__ void __launch_bounds__(128, 4) k_solve_ri(double2* __restrict__ V, const double2* rhs, size_t rcs,
                                                     int roff, const double* __restrict__ fac,
                                                     const double* __restrict__ der, const double* __restrict__ d0lu,
                                                     const double* __restrict__ yint, BcRows bc, Dims d,
                                                     DevScalars* __restrict__ sc, const dd* __restrict__ lindd,
                                                     int q_lo, int q_hi) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sys = w >> 1, t = w & 1, c = lane & 1;
  const int q = q_lo + blockIdx.x * 16 + (lane >> 1);
  const bool active = q < q_hi;
  const int ny = d.ny, nz = d.nz;
  const int ix = active ? q / (nz + 1) : 0;
  const int a = active ? q - ix * (nz + 1) : 0;
  const int nm = (a == 0) ? 1 : 2;
  int mm[2];
  mm[0] = ix * d.nzt + nz + a;
  mm[1] = ix * d.nzt + nz - a;
  const bool is00 = (ix == 0 && a == 0);
  const double ka = ix * d.alfa0, kb = a * d.beta0;
  const double k2 = ka * ka + kb * kb;
  const double ni = d.ni;
  const size_t P = d.npairs;
  const bool ucor = active && is00 && sys == 1 && t == 1;  // unit-forcing response (linsolve_blocking.inc:62-68)
  const bool mine = active && t < nm;
  const int m = mm[ucor ? 0 : t];
  const int vc = ucor ? 2 : (sys == 0 ? 1 : 0);  // field slot written
  const bool wallrhs = mine && sys == 1 && is00;
  double bot[5], botm1[5], top[5], topp1[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    bot[j] = sys ? bc.eta0bc[j] : bc.v0bc[j];
    botm1[j] = sys ? bc.eta0m1bc[j] : bc.v0m1bc[j];
    top[j] = sys ? bc.etanbc[j] : bc.vnbc[j];
    topp1[j] = sys ? bc.etanp1bc[j] : bc.vnp1bc[j];
  }
  // the wall velocity enters the real component only
  const double bval0 = (wallrhs && c == 0) ? sc->u0 : 0.0, bvaln = (wallrhs && c == 0) ? sc->uN : 0.0;
  if (mine || ucor) {
    const double* fs = fac + (size_t)5 * sys * P + q;
    const size_t frow = (size_t)kFacPerRow * P;
    // ---- Step1 bottom-up: x = (b - u1 x(+1) - u2 x(+2)) / d ----
    const double2* rsrc = rhs + (sys == 0 ? rcs : 0);
    double x1 = 0.0, x2 = 0.0;
    double bn = ucor ? (c == 0 ? 1.0 : 0.0) : *cptr(&rsrc[(size_t)(ny - 1 + roff) * d.nmodes + m], c);
    const double* f = fs + (size_t)(ny - 2) * frow;
    double dn = f[2 * P], u1n = f[3 * P], u2n = f[4 * P];
    for (int iy = ny - 1; iy >= 1; --iy) {
      double b = bn;
      const double dv = dn, u1 = u1n, u2 = u2n;
      if (iy > 1) {  // one row ahead (global-load latency)
        if (!ucor) bn = *cptr(&rsrc[(size_t)(iy - 1 + roff) * d.nmodes + m], c);
        f -= frow;
        dn = f[2 * P];
        u1n = f[3 * P];
        u2n = f[4 * P];
      }
      if (iy - kSolvePrefetch >= 1) {  // and the lines of a row further down
        const double* fp = f - (size_t)(kSolvePrefetch - 1) * frow;
        prefetch_l1(fp + 2 * P);
        prefetch_l1(fp + 3 * P);
        prefetch_l1(fp + 4 * P);
        if (!ucor) prefetch_l1(rsrc + (size_t)(iy - kSolvePrefetch + roff) * d.nmodes + m);
      }
      if (wallrhs) {
        if (iy == 1) b = b - sc->wallrhs[0 + c];
        if (iy == 2) b = b - sc->wallrhs[2 + c];
        if (iy == ny - 2) b = b - sc->wallrhs[4 + c];
        if (iy == ny - 1) b = b - sc->wallrhs[6 + c];
      }
      const double x = dv * fma(-u2, x2, fma(-u1, x1, b));
      x2 = x1;
      x1 = x;
      *cptr(&V[vidx(d, vc, iy, m)], c) = x;
    }
    // ---- Step2 top-down: v = x - l2 v(-2) - l1 v(-1); rows 1..3 and ny-3..ny-1 kept ----
    double lo[3], hi[3];
    double m2 = 0.0, m1 = 0.0;
    f = fs;
    double l2n = f[0], l1n = f[P];
    double vn = *cptr(&V[vidx(d, vc, 1, m)], c);
    for (int iy = 1; iy <= ny - 1; ++iy) {
      const double l2 = l2n, l1 = l1n;
      const double vcur = vn;
      if (iy < ny - 1) {
        f += frow;
        l2n = f[0];
        l1n = f[P];
        vn = *cptr(&V[vidx(d, vc, iy + 1, m)], c);
      }
      if (iy + kSolvePrefetch <= ny - 1) {
        const double* fp = f + (size_t)(kSolvePrefetch - 1) * frow;
        prefetch_l1(fp);
        prefetch_l1(fp + P);
        prefetch_l1(&V[vidx(d, vc, iy + kSolvePrefetch, m)]);
      }
      const double nv = fma(-l1, m1, fma(-l2, m2, vcur));
      *cptr(&V[vidx(d, vc, iy, m)], c) = nv;
      m2 = m1;
      m1 = nv;
      if (iy == 1) lo[0] = nv;
      if (iy == 2) lo[1] = nv;
      if (iy == 3) lo[2] = nv;
      if (iy == ny - 3) hi[0] = nv;
      if (iy == ny - 2) hi[1] = nv;
      if (iy == ny - 1) hi[2] = nv;
    }
    // wall and ghost values (linsolve_blocking.inc:50-61), per component as dot3/dot4/cdivr
    auto d3 = [](const double* v, const double* cf) {
      double s = cf[0] * v[0];
      s = s + cf[1] * v[1];
      return s + cf[2] * v[2];
    };
    auto d4 = [](const double* v, const double* cf) {
      double s = cf[0] * v[0];
      s = s + cf[1] * v[1];
      s = s + cf[2] * v[2];
      return s + cf[3] * v[3];
    };
    const double w0 = (bval0 - d3(lo, bot + 2)) / bot[1];
    const double rb[4] = {w0, lo[0], lo[1], lo[2]};
    const double wm1 = (0.0 - d4(rb, botm1 + 1)) / botm1[0];
    const double wn = (bvaln - d3(hi, top)) / top[3];
    const double rt[4] = {hi[0], hi[1], hi[2], wn};
    const double wn1 = (0.0 - d4(rt, topp1)) / topp1[4];
    *cptr(&V[vidx(d, vc, -1, m)], c) = wm1;
    *cptr(&V[vidx(d, vc, 0, m)], c) = w0;
    *cptr(&V[vidx(d, vc, ny, m)], c) = wn;
    *cptr(&V[vidx(d, vc, ny + 1, m)], c) = wn1;
  }
  __syncthreads();  // v, eta (and the unit response) of this block's pairs are in V
  if (wallrhs && c == 0) {  // mean flow (linsolve_blocking.inc:62-97), both components
    double fu = 0.0, fw = 0.0, fc = 0.0;
    for (int iy = 1, k = 0; iy <= ny - 1; iy += 2, ++k) {
      const double a1 = yint[3 * k], a2 = yint[3 * k + 1], a3 = yint[3 * k + 2];
      const double2 e0 = V[vidx(d, 0, iy - 1, m)], e1 = V[vidx(d, 0, iy, m)], e2 = V[vidx(d, 0, iy + 1, m)];
      const double2 u0 = V[vidx(d, 2, iy - 1, m)], u1 = V[vidx(d, 2, iy, m)], u2 = V[vidx(d, 2, iy + 1, m)];
      fu = fu + a1 * e0.x + a2 * e1.x + a3 * e2.x;
      fw = fw + a1 * e0.y + a2 * e1.y + a3 * e2.y;
      fc = fc + a1 * u0.x + a2 * u1.x + a3 * u2.x;
    }
    double corrpx = sc->corrpx, corrpz = sc->corrpz;
    const bool cx = fabs(d.meanflowx) > 1.0e-7 && !d.cpi;
    const bool cz_ = fabs(d.meanflowz) > 1.0e-7 && !d.cpi;
    if (cx) corrpx = (d.meanflowx - fu) / fc;
    if (cz_) corrpz = (d.meanflowz - fw) / fc;
    for (int iy = -1; iy <= ny + 1; ++iy) {
      const double2 et = V[vidx(d, 0, iy, m)];
      const double uc = V[vidx(d, 2, iy, m)].x;
      double U = et.x, W = et.y;
      if (cx) U = U + corrpx * uc;
      if (cz_) W = W + corrpz * uc;
      V[vidx(d, 0, iy, m)] = make_double2(U, 0.0);
      V[vidx(d, 2, iy, m)] = make_double2(W, 0.0);
    }
    sc->fr[0] = fu; sc->fr[1] = fw; sc->fr[2] = fc;
    sc->corrpx = corrpx; sc->corrpz = corrpz;
    if (d.cpi) {
      if (d.cpi_type == 0) sc->meanpx = (1 - d.gamma) * 6 * ni / fu;
      else sc->meanpx = (1.5 / d.gamma) * fu * ni;
    }
  }
  const bool takes = active && !is00 && sys == 0 && t < nm;  // the same for both lanes of a pair
  const unsigned mask = __ballot_sync(0xffffffffu, takes);
  if (!takes) return;
  if (lindd) deriv_uw_c<dd>(V, der, d0lu, lindd, bc, d, mm[t], ka, (t == 0 ? 1.0 : -1.0) * kb, k2, c, mask);
  else deriv_uw_c<double>(V, der, d0lu, lindd, bc, d, mm[t], ka, (t == 0 ? 1.0 : -1.0) * kb, k2, c, mask);
}

void launch_factor(const SolveLaunch& L, cudaStream_t s) {
  if (L.q_hi <= L.q_lo) return;
  const unsigned grid = (unsigned)((L.q_hi - L.q_lo + 31) / 32);
  k_factor<<<grid, 64, 0, s>>>(L.fac, L.der, L.bc, L.d, L.lambda, L.ode[0], L.lambda_from_dt, L.sc, L.nud, L.q_lo,
                               L.q_hi);
}

void launch_linsolve(const SolveLaunch& L, cudaStream_t s) {
  if (L.q_hi <= L.q_lo) return;
  const unsigned grid = (unsigned)((L.q_hi - L.q_lo + 31) / 32);
  if (!L.split_solve) {
    k_linsolve<false><<<grid, 64, 0, s>>>(L.V, L.rhs_src, L.rhs_cstride, L.rhs_plane_off, L.fac, L.der, L.d0lu, L.yint,
                                          L.bc, L.d, L.lambda, L.ode[0], L.lambda_from_dt, L.sc, (const dd*)L.lindd,
                                          L.nud, L.q_lo, L.q_hi);
    return;
  }
  if (!L.factored) launch_factor(L, s);
  if (L.split_solve == 3) {
    k_solve_ri<<<(unsigned)((L.q_hi - L.q_lo + 15) / 16), 128, 0, s>>>(
        L.V, L.rhs_src, L.rhs_cstride, L.rhs_plane_off, L.fac, L.der, L.d0lu, L.yint, L.bc, L.d, L.sc,
        (const dd*)L.lindd, L.q_lo, L.q_hi);
    return;
  }
  if (L.split_solve == 2) {
    k_linsolve<true><<<grid, 64, 0, s>>>(L.V, L.rhs_src, L.rhs_cstride, L.rhs_plane_off, L.fac, L.der, L.d0lu, L.yint,
                                         L.bc, L.d, L.lambda, L.ode[0], L.lambda_from_dt, L.sc, (const dd*)L.lindd,
                                         L.nud, L.q_lo, L.q_hi);
    return;
  }
  k_solve<<<grid, 128, 0, s>>>(L.V, L.rhs_src, L.rhs_cstride, L.rhs_plane_off, L.fac, L.der, L.d0lu, L.yint, L.bc,
                               L.d, L.sc, (const dd*)L.lindd, L.q_lo, L.q_hi);
}

// ---------------------------------------------------------------------------
// small scalar kernels
// ---------------------------------------------------------------------------
__global__ void k_advance_time(DevScalars* sc, double coef, int new_step) {
  if (new_step) sc->istep += 1;
  sc->time = sc->time + coef * sc->deltat;  // channel.f90:128,141,154
}

void launch_advance_time(DevScalars* sc, double coef, int new_step, cudaStream_t s) {
  k_advance_time<<<1, 1, 0, s>>>(sc, coef, new_step);
}

// outstats without file output (dnsdata.f90:861-879)
__global__ void k_outstats(const double2* __restrict__ V, Dims d, BcRows bc, DevScalars* sc) {
  const double rg = sc->cfl;
  sc->cfl = 0.0;
  if (d.cflmax > 0) {
    sc->deltat = d.cflmax / rg;
    sc->rdt = 1.0 / sc->deltat;
  }
  const int m = d.nz;  // ix=0, iz=0
  const int ny = d.ny;
  double lo1[5], lo3[5], hi1[5], hi3[5];
  for (int j = 0; j < 5; ++j) {
    lo1[j] = V[vidx(d, 0, -1 + j, m)].x;
    lo3[j] = V[vidx(d, 2, -1 + j, m)].x;
    hi1[j] = V[vidx(d, 0, ny - 3 + j, m)].x;
    hi3[j] = V[vidx(d, 2, ny - 3 + j, m)].x;
  }
  double d11 = bc.d140[0] * lo1[0], d21 = bc.d140[0] * lo3[0], d12 = bc.d14n[0] * hi1[0], d22 = bc.d14n[0] * hi3[0];
  for (int j = 1; j < 5; ++j) {
    d11 = d11 + bc.d140[j] * lo1[j];
    d21 = d21 + bc.d140[j] * lo3[j];
    d12 = d12 + bc.d14n[j] * hi1[j];
    d22 = d22 + bc.d14n[j] * hi3[j];
  }
  double* o = sc->line;
  o[0] = sc->time;
  o[1] = d11; o[2] = -d12; o[3] = d21; o[4] = -d22;
  o[5] = sc->fr[0] + sc->corrpx * sc->fr[2];
  o[6] = sc->meanpx + sc->corrpx;
  o[7] = sc->fr[1] + sc->corrpz * sc->fr[2];
  o[8] = sc->meanpz + sc->corrpz;
  o[9] = rg * sc->deltat;
  o[10] = sc->deltat;
  sc->runtime_global = rg;
  bool bad = !isfinite(rg);
  for (int i = 0; i < 11; ++i) bad = bad || !isfinite(o[i]);
  if (bad) sc->error |= 1;
}

void launch_outstats(const SolveLaunch& L, cudaStream_t s) { k_outstats<<<1, 1, 0, s>>>(L.V, L.d, L.bc, L.sc); }

// initial flow rate and CPI gradient (channel.f90:101-115)
__global__ void k_flowrate(const double2* __restrict__ V, const double* __restrict__ yint, Dims d, DevScalars* sc) {
  const int m = d.nz;
  double fu = 0.0, fw = 0.0;
  for (int iy = 1, k = 0; iy <= d.ny - 1; iy += 2, ++k) {
    const double a1 = yint[3 * k], a2 = yint[3 * k + 1], a3 = yint[3 * k + 2];
    fu = fu + a1 * V[vidx(d, 0, iy - 1, m)].x + a2 * V[vidx(d, 0, iy, m)].x + a3 * V[vidx(d, 0, iy + 1, m)].x;
    fw = fw + a1 * V[vidx(d, 2, iy - 1, m)].x + a2 * V[vidx(d, 2, iy, m)].x + a3 * V[vidx(d, 2, iy + 1, m)].x;
  }
  sc->fr[0] = fu;
  sc->fr[1] = fw;
  sc->fr[2] = 0.0;  // the driver's frl(3) is never assigned
  if (d.cpi) {
    if (d.cpi_type == 0) sc->meanpx = (1 - d.gamma) * 6 * d.ni / fu;
    else sc->meanpx = (1.5 / d.gamma) * fu * d.ni;
  }
}

void launch_flowrate(const SolveLaunch& L, cudaStream_t s) { k_flowrate<<<1, 1, 0, s>>>(L.V, L.yint, L.d, L.sc); }

// ---------------------------------------------------------------------------
// body-force ghost rows as buildrhs sets them (dnsdata.f90:617-628):
// F(0)=F(ny)=0, F(-1) = -D4(F)/d4(-2) at iy=1, F(ny+1) = -D4(F)/d4(2) at iy=ny-1
// ---------------------------------------------------------------------------
__global__ void k_force_ghosts(double2* __restrict__ F, const double* __restrict__ der, Dims d) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (m >= d.nmodes) return;
  const int ny = d.ny;
  F[vidx(d, c, -1, m)] = cz();
  F[vidx(d, c, 0, m)] = cz();
  F[vidx(d, c, ny, m)] = cz();
  F[vidx(d, c, ny + 1, m)] = cz();
  const double* d4b = der + (size_t)1 * 20 + 15;
  const double* d4t = der + (size_t)(ny - 1) * 20 + 15;
  double2 lo[5], hi[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    lo[j] = F[vidx(d, c, -1 + j, m)];
    hi[j] = F[vidx(d, c, ny - 3 + j, m)];
  }
  F[vidx(d, c, -1, m)] = cdivr(cz() - dot5(lo, d4b), d4b[0]);
  F[vidx(d, c, ny + 1, m)] = cdivr(cz() - dot5(hi, d4t), d4t[4]);
}

void launch_force_ghosts(double2* F, const double* der, const Dims& d, cudaStream_t s) {
  k_force_ghosts<<<dim3((d.nmodes + 127) / 128, 3), 128, 0, s>>>(F, der, d);
}

// ---------------------------------------------------------------------------
// layout transposes between the restart-file order (y fastest) and the
// device order (mode fastest): batch of [rows][cols] -> [cols][rows]
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_transpose(const double2* __restrict__ in, double2* __restrict__ out, int rows,
                                                   int cols) {
  __shared__ double2 tile[32][33];
  const size_t base = (size_t)blockIdx.z * rows * cols;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[base + (size_t)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[base + (size_t)c * rows + r] = tile[threadIdx.x][i];
  }
}

void launch_transpose(const double2* in, double2* out, int rows, int cols, int batch, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch);
  k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, out, rows, cols);
}

}  // namespace chgpu

// ---------------------------------------------------------------------------
// the pivot reciprocal over caller values, for its accuracy test
// ---------------------------------------------------------------------------
namespace chgpu {
__global__ void k_rcp_values(const double* __restrict__ x, double* __restrict__ y, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = rcp_nr(x[i]);
}
}  // namespace chgpu

extern "C" int chgpu_pivot_reciprocal(const double* x, double* y, size_t n, char* err, size_t errlen) {
  if (!x || !y) {
    if (err && errlen) snprintf(err, errlen, "null buffer");
    return CHGPU_E_PARAM;
  }
  if (n == 0) return CHGPU_OK;
  double* dx = nullptr;
  cudaError_t e = cudaMalloc(&dx, 2 * n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    chgpu::k_rcp_values<<<(unsigned)((n + 255) / 256), 256>>>(dx, dx + n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(y, dx + n, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (dx) cudaFree(dx);
  if (e != cudaSuccess) {
    if (err && errlen) snprintf(err, errlen, "pivot reciprocal: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? CHGPU_E_NOMEM : CHGPU_E_CUDA;
  }
  return CHGPU_OK;
}
