// extern "C" entry points of libchgpu.so (declared in include/chgpu.h).
//
// One handle = one channel run on the current device: the field V in a
// plane-major layout [component][y-plane][mode] (mode = ix*(2nz+1)+iz+nz,
// contiguous), the RK history, the spectra of the six products of every
// plane, the x/z work buffers of the transforms, the y-discretisation tables
// and the module scalars (time, deltat, flow rates, pressure-gradient
// corrections, CFL), all resident on the device.  A whole time step
// (channel.f90:118-167) is a fixed sequence of launches reading every
// dynamic value (deltat, lambda) from device memory, captured once into a
// CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/chgpu.h"
#include "../../include/chgpu_closure.h"
#include "chgpu_internal.h"
#include "kernels.cuh"
#include "rfft.cuh"
#include "mlp.cuh"

using namespace chgpu;

namespace {

constexpr double RK[3][3] = {
    {120.0 / 32.0, 2.0, 0.0},
    {120.0 / 8.0, 50.0 / 8.0, 34.0 / 8.0},
    {120.0 / 20.0, 90.0 / 20.0, 50.0 / 20.0}};  // dnsdata.f90:70-72

thread_local std::string g_create_error;

}  // namespace

struct chgpu_handle {
  chgpu_params p{};
  Dims d{};
  BcRows bc{};
  Tables tab;
  RadixDev rz{}, rx{};
  int prec = CHGPU_FP64;  // CHGPU_FP64, CHGPU_MIXED or CHGPU_FP64DD
  int zcols = 1, xrows = 1;
  int xminb = 2;  // register-cap variant of the x-row kernel
  int zthreads = 256, xthreads = 256;  // threads per block of the transform kernels
  bool tuned = false;
  cudaStream_t stream = nullptr;
  // the step in two kx halves (rhs / solve / next z-inverse of one half
  // overlapping the other's): side stream and its fork / join events.  Used
  // from 65 536 (kx, +-kz) pairs on: at 16 384 the halved solves leave the
  // GPU emptier than they overlap (mixed path 10.0 -> 11.2 ms at 127x192x127),
  // at 147 456 the overlap gains ~1%.
  int halves = 1;
  // the banded solves as two kernels (factorisation, then one thread per
  // mode and system) below 65 536 pairs: at 16 384 the fused kernel has ~7
  // warps per SM and the split is 14-17% faster; at 147 456 the fused kernel
  // hides its latency and the split is 4-19% slower (extra factor traffic,
  // half the warps idle during v')
  // 1: fused (k_linsolve); 2: split (k_factor, k_solve); 3: split with each
  // substep's factorisation on a third stream, started with the substep (it
  // needs only dt and the RK coefficient), so that the FP64-pipe bound
  // k_factor runs beside the FP32 / memory-bound transforms and k_rhs; 4: the
  // factorisation ahead as in 3, the substitutions by the fused kernel's two
  // threads per pair reading the factors; 5: the factorisation ahead, the
  // substitutions with eight threads per pair (k_solve_ri: one per system,
  // mode and real / imaginary component)
  int solve_form = 1;
  cudaStream_t stream2 = nullptr, stream3 = nullptr;
  cudaEvent_t ev_vv = nullptr, ev_solved = nullptr, ev_fac_fork = nullptr, ev_factored = nullptr;
  cudaEvent_t ev_copy_fork = nullptr, ev_copy_join = nullptr;  // the two-stream field upload
  // device buffers
  double2* V = nullptr;
  void* old = nullptr;
  void* VV = nullptr;
  void* Zb = nullptr;
  void* Pb = nullptr;
  double2* rhs = nullptr;
  double2* F = nullptr;  // body force, plane-major like V
  bool use_F = false;
  double* fac = nullptr;
  double* der = nullptr;
  void* derT = nullptr;
  void* derL = nullptr;
  void* cst = nullptr;  // transform-type constants: factor, 1/dx, 1/dz, 1/dy per plane
  double* d0lu = nullptr;
  double* nud = nullptr;  // per row: -ni d4, -ni d2 (the mode-independent matrix terms)
  void* lindd = nullptr;  // double-float d1 / D0mat / d0 rows for v' and u, w (mixed and double-float paths)
  double* yint = nullptr;
  double* dy = nullptr;
  void* twz = nullptr;
  void* twx = nullptr;
  void* twh = nullptr;
  // register-blocked transform kernels (convf.cu), used for the lengths with
  // a compile-time plan: their per-pass twiddle tables
  void* twzr = nullptr;
  void* twxr = nullptr;
  bool zfast = false, xfast = false;
  int xrvar = 4;  // register-blocked x-row variant: 4 (registers for 3 blocks per SM) or 5 (for 4)
  DevScalars* sc = nullptr;
  DevScalars* sc_host = nullptr;  // pinned
  cudaGraphExec_t graph = nullptr;
  long long version = 0;  // bumped whenever the launch sequence of a step changes
  bool field_set = false;
  // on-device statistics: [S1, comp S1, S2, comp S2][3][nplanes]
  double* stats_acc = nullptr;
  long long stats_n = 0;
  // asynchronous snapshots: device staging, pinned host copy, side stream
  double2* snap_stage = nullptr;
  double* snap_host = nullptr;
  cudaStream_t snap_stream = nullptr;
  cudaEvent_t snap_read = nullptr, snap_done = nullptr;
  bool snap_pending = false;
  // physical-space export: per-chunk work buffers and root tables
  double2* ex_W = nullptr;
  double* ex_P = nullptr;
  double* ex_out = nullptr;
  double2* ex_twz = nullptr;
  double2* ex_twx = nullptr;
  size_t ex_out_cap = 0;  // doubles
  int ex_chunk = 0, ex_zcols = 0, ex_xpairs = 0;
  RadixDev ex_rz{}, ex_rx{};
  // learned closure: gradient spectra [9][plane][mode], their z-inverse
  // [9][plane][kx][z] and physical values [9][plane][z][x] (FP32, x pairs
  // packed), the stresses [6][plane][z][x], wall distance per plane, FP32
  // transform tables
  chgpu_mlp* cl_mlp = nullptr;
  bool cl_on = false;     // the network evaluates tau in every convolution pass
  bool cl_fixed = false;  // a prescribed tau (chgpu_closure_set_tau)
  double2* cl_G = nullptr;
  float2* cl_Z = nullptr;
  float2* cl_P = nullptr;
  float2* cl_tau = nullptr;
  float* cl_wd = nullptr;
  void *cl_twz = nullptr, *cl_twx = nullptr, *cl_twh = nullptr;
  // Reynolds-stress budget spectra (allocated by the first chgpu_tke_reset)
  double2 *tke_W = nullptr, *tke_N = nullptr, *tke_P = nullptr, *tke_Zt = nullptr, *tke_Xt = nullptr;
  double *tke_acc = nullptr, *tke_mean = nullptr;
  void *tke_twz = nullptr, *tke_twx = nullptr, *tke_twh = nullptr;
  RadixDev tke_rz{}, tke_rx{};
  int tke_chunk = 0;
  long long tke_n = 0;
  bool tke_ready = false, tke_pressure = false;
  std::vector<double> tke_meanh;  // U, W, dU/dy, dW/dy, d2U/dy2, d2W/dy2, P per plane
  int nsm = 0;
  // per-kernel timing
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  double kind_ms[CHGPU_NKINDS] = {0};
  long long kind_n[CHGPU_NKINDS] = {0};
  long long launches = 0;
  long long step_launches = 19;  // kernels in one captured step
  std::string err;
};

namespace {

int fail(chgpu_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(chgpu_handle* h, cudaError_t e, const char* where) {
  return fail(h, e == cudaErrorMemoryAllocation ? CHGPU_E_NOMEM : CHGPU_E_CUDA,
              std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define CK(h, call)                                         \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
  } while (0)

// element size of the transform buffers and spectra (and of the RK history)
size_t tsize(const chgpu_handle* h) { return h->prec == CHGPU_MIXED ? sizeof(float2) : sizeof(double2); }

// value of a long double in each arithmetic type (double-float: split in extended precision)
template <typename T> T from_ld(long double v) { return (T)v; }
template <> dd from_ld<dd>(long double v) {
  const float hi = (float)v;
  return dd(hi, (float)(v - (long double)hi));
}

template <typename V2>
std::vector<V2> roots(int n) {  // forward roots exp(-2 pi i m/n), from the mathematics in extended precision
  using T = decltype(V2::x);
  std::vector<V2> w(n);
  for (int m = 0; m < n; ++m) {
    long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)n;
    w[m].x = from_ld<T>(cosl(ang));
    w[m].y = from_ld<T>(-sinl(ang));
  }
  return w;
}

// der and the wavenumber units in the nonlinear-term type: [(ny+1)*20] then alfa0, beta0
template <typename T>
int upload_derT(chgpu_handle* h) {
  const std::vector<double>& der = h->tab.der;
  std::vector<T> t(der.size() + 2);
  for (size_t i = 0; i < der.size(); ++i) t[i] = from_ld<T>((long double)der[i]);
  t[der.size()] = from_ld<T>((long double)h->p.alfa0);
  t[der.size() + 1] = from_ld<T>((long double)h->p.beta0);
  CK(h, cudaMalloc(&h->derT, sizeof(T) * t.size()));
  CK(h, cudaMemcpy(h->derT, t.data(), sizeof(T) * t.size(), cudaMemcpyHostToDevice));
  // constants of the x-row pass: factor/2, 1/dx, 1/dz (dnsdata.f90:124), 1/dy(iy) per plane (:155)
  std::vector<T> c(3 + h->d.nplanes, T());
  c[0] = from_ld<T>(0.5L * (long double)h->d.factor);
  c[1] = from_ld<T>((long double)h->d.rdx);
  c[2] = from_ld<T>((long double)h->d.rdz);
  for (int iy = 1; iy <= h->p.ny - 1; ++iy) c[3 + iy + 1] = from_ld<T>(1.0L / (long double)h->tab.dy[iy]);
  CK(h, cudaMalloc(&h->cst, sizeof(T) * c.size()));
  CK(h, cudaMemcpy(h->cst, c.data(), sizeof(T) * c.size(), cudaMemcpyHostToDevice));
  return 0;
}

// der in the linear-term type of buildrhs (double-float in the mixed path,
// FP64 otherwise), then alfa0, beta0, ni
template <typename L>
int upload_derL(chgpu_handle* h) {
  const std::vector<double>& der = h->tab.der;
  std::vector<L> t(der.size() + 3);
  for (size_t i = 0; i < der.size(); ++i) t[i] = from_ld<L>((long double)der[i]);
  t[der.size()] = from_ld<L>((long double)h->p.alfa0);
  t[der.size() + 1] = from_ld<L>((long double)h->p.beta0);
  t[der.size() + 2] = from_ld<L>((long double)h->p.ni);
  CK(h, cudaMalloc(&h->derL, sizeof(L) * t.size()));
  CK(h, cudaMemcpy(h->derL, t.data(), sizeof(L) * t.size(), cudaMemcpyHostToDevice));
  return 0;
}

// per-stage twiddles of a radix plan (the layout stockham_stage reads):
// stage st at twoff[st], R-1 values w_{Ns R}^{r k} (r = 1..R-1) per k < Ns
void set_twiddle_offsets(RadixDev& r) {
  int Ns = 1, off = 0;
  for (int st = 0; st < r.nst; ++st) {
    r.twoff[st] = off;
    off += Ns * (r.r[st] - 1);
    Ns *= r.r[st];
  }
}

// FP64 twiddle of the fused multiply-add butterflies (lf_butterfly, cplx.cuh):
// w = exp(-2 pi i phi) as (c, t) with w = c (1 + i t), or w = i c (1 + i t)
// marked by c's lowest significand bit, whichever gives |t| <= 1
double2 lf_entry(long double phi) {
  const long double ang = 2.0L * 3.14159265358979323846264338327950288L * phi;
  const long double wx = cosl(ang), wy = -sinl(ang);
  const bool q = fabsl(wy) > fabsl(wx);
  const long double c = q ? wy : wx, t = q ? -wx / wy : wy / wx;
  double cd = (double)c;
  unsigned long long bits;
  std::memcpy(&bits, &cd, sizeof bits);
  bits = (bits & ~1ull) | (q ? 1ull : 0ull);
  std::memcpy(&cd, &bits, sizeof bits);
  return make_double2(cd, (double)t);
}
// the R-1 entries of one k of a power-of-two radix-R stage, in lf_dft's
// order: level l = 1..log2 R, m' < 2^(l-1): W_{2^l Ns}^{k + Ns m'}
void lf_stage_entries(double2* out, int Ns, int R, int k) {
  int i = 0;
  for (int half = 1; half < R; half *= 2)  // half = 2^(l-1)
    for (int mp = 0; mp < half; ++mp)
      out[i++] = lf_entry((long double)(k + Ns * mp) / (long double)(2 * half * Ns));
}
template <typename V2> constexpr bool lf_format(int R) { return std::is_same<V2, double2>::value && is_pow2c(R); }

template <typename V2>
int upload_stage_twiddles(chgpu_handle* h, void** dst, const RadixDev& rad) {
  using T = decltype(V2::x);
  std::vector<V2> w(std::max(1, rad.n));
  int Ns = 1;
  for (int st = 0; st < rad.nst; ++st) {
    const int R = rad.r[st];
    if constexpr (std::is_same<V2, double2>::value) {
      if (lf_format<V2>(R)) {
        if (Ns == 1 && R == 16) {  // the first stage's inner twiddled DFT4s (lf_dft16_first)
          for (int k1 = 1; k1 <= 3; ++k1) lf_stage_entries(&w[rad.twoff[st] + 3 * (k1 - 1)], 4, 4, k1);
        } else {
          for (int k = 0; k < Ns; ++k) lf_stage_entries(&w[rad.twoff[st] + k * (R - 1)], Ns, R, k);
        }
        Ns *= R;
        continue;
      }
    }
    for (int k = 0; k < Ns; ++k)
      for (int r = 1; r < R; ++r) {
        const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)(r * k) /
                                (long double)(Ns * R);
        V2& e = w[rad.twoff[st] + k * (R - 1) + r - 1];
        e.x = from_ld<T>(cosl(ang));
        e.y = from_ld<T>(-sinl(ang));
      }
    Ns *= R;
  }
  CK(h, cudaMalloc(dst, sizeof(V2) * w.size()));
  CK(h, cudaMemcpy(*dst, w.data(), sizeof(V2) * w.size(), cudaMemcpyHostToDevice));
  return 0;
}

// roots of 2 nxd for the real-to-complex packing, then the same scaled by
// factor/2 for the unpacking of the products (factor = dnsdata.f90:124)
template <typename V2>
int upload_pack_roots(chgpu_handle* h, void** dst, int n, long double scale) {
  using T = decltype(V2::x);
  std::vector<V2> w(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)n;
    w[m].x = from_ld<T>(cosl(ang));
    w[m].y = from_ld<T>(-sinl(ang));
    w[n + m].x = from_ld<T>(scale * cosl(ang));
    w[n + m].y = from_ld<T>(-scale * sinl(ang));
  }
  CK(h, cudaMalloc(dst, sizeof(V2) * w.size()));
  CK(h, cudaMemcpy(*dst, w.data(), sizeof(V2) * w.size(), cudaMemcpyHostToDevice));
  return 0;
}

// per-pass twiddles of a register-blocked plan (rfft.cuh): pass p >= 1 at
// rplan_twoff(p), R-1 forward roots w_{Ns R}^{r k} (r = 1..R-1) per k < Ns,
// padded to R per k in FP32 tables
template <typename V2>
int upload_rplan_twiddles(chgpu_handle* h, void** dst, int n, bool xplan = false) {
  using T = decltype(V2::x);
  int E = 0, TPR = 0;
  if (!(xplan ? xlen_plan(n, &E, &TPR) : rlen_plan(n, &E, &TPR))) return 0;
  const int np = rplan_passes(E, TPR);
  const int tail = std::is_same<V2, double2>::value ? rplan_tailsize(E) : 0;
  std::vector<V2> w(std::max(1, rplan_twsize<V2>(E, TPR) + tail));
  if constexpr (std::is_same<V2, double2>::value) {  // the composite first pass's twiddled DFTs (rpass_first)
    for (int k1 = 1; k1 <= 2 && tail > 0; ++k1)
      lf_stage_entries(&w[rplan_twsize<V2>(E, TPR) + (k1 - 1) * (E / 3 - 1)], 3, E / 3, k1);
  }
  for (int p = 1; p < np; ++p) {
    const int R = rplan_radix(E, TPR, p), Ns = rplan_ns(E, TPR, p), off = rplan_twoff<V2>(E, TPR, p);
    if constexpr (std::is_same<V2, double2>::value) {  // every pass after the first has a power-of-two radix
      for (int k = 0; k < Ns; ++k) lf_stage_entries(&w[off + k * (R - 1)], Ns, R, k);
      continue;
    }
    for (int k = 0; k < Ns; ++k)
      for (int r = 1; r < R; ++r) {
        const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)(r * k) /
                                (long double)(Ns * R);
        V2& e = w[off + k * tw_per_k<V2>(R) + r - 1];
        e.x = from_ld<T>(cosl(ang));
        e.y = from_ld<T>(-sinl(ang));
      }
  }
  CK(h, cudaMalloc(dst, sizeof(V2) * w.size()));
  CK(h, cudaMemcpy(*dst, w.data(), sizeof(V2) * w.size(), cudaMemcpyHostToDevice));
  return 0;
}

cudaEvent_t take_event(chgpu_handle* h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets the launches of `fn` with an event pair when profiling.
template <typename F>
void timed(chgpu_handle* h, int kind, F fn) {
  if (!h->profiling) {
    fn();
    return;
  }
  cudaEvent_t a = take_event(h), b = take_event(h);
  cudaEventRecord(a, h->stream);
  fn();
  cudaEventRecord(b, h->stream);
  h->ev_pending.push_back({kind, {a, b}});
}

ConvLaunch conv_launch(chgpu_handle* h, int compute_cfl, int products, int plane0, int nplanes) {
  ConvLaunch L{};
  L.d = h->d;
  L.rz = h->rz;
  L.rx = h->rx;
  L.V = h->V;
  L.Zb = h->Zb;
  L.Pb = h->Pb;
  L.VV = h->VV;
  L.twz = h->twz;
  L.twx = h->twx;
  L.twh = h->twh;
  L.dy = h->dy;
  L.cst = h->cst;
  L.sc = h->sc;
  L.zcols = h->zcols;
  L.xrows = h->xrows;
  L.xminb = h->xfast ? h->xrvar : h->xminb;
  L.zthreads = h->zthreads;
  L.xthreads = h->xthreads;
  L.ix_lo = 0;
  L.ix_hi = h->d.nx + 1;
  L.plane0 = plane0;
  L.nplanes = nplanes;
  L.compute_cfl = compute_cfl;
  L.products = products;
  L.twzr = h->twzr;
  L.twxr = h->twxr;
  L.zfast = h->zfast;
  L.xfast = h->xfast;
  return L;
}

SolveLaunch solve_launch(chgpu_handle* h, const double* ode) {
  SolveLaunch L{};
  L.d = h->d;
  L.bc = h->bc;
  L.V = h->V;
  L.VV = h->VV;
  L.old = h->old;
  L.rhs = h->rhs;
  L.F = h->use_F ? h->F : nullptr;
  L.fac = h->fac;
  L.der = h->der;
  L.derT = h->derT;
  L.derL = h->derL;
  L.d0lu = h->d0lu;
  L.lindd = h->lindd;
  L.nud = h->nud;
  L.m_lo = 0;
  L.m_hi = h->d.nmodes;
  L.q_lo = 0;
  L.q_hi = h->d.npairs;
  L.yint = h->yint;
  L.sc = h->sc;
  if (ode) {
    L.ode[0] = ode[0];
    L.ode[1] = ode[1];
    L.ode[2] = ode[2];
  }
  return L;
}

// the closure's stresses for the current field: velocity gradients ->
// physical -> network -> tau at the points of the planes iy = 1..ny-1
void enqueue_closure(chgpu_handle* h) {
  const Dims& d = h->d;
  launch_gradients(h->V, h->cl_G, h->der, h->d0lu, h->bc, d, h->stream);
  launch_physical_fields(h->cl_G, 9, h->cl_Z, h->cl_P, (const float2*)h->cl_twz, (const float2*)h->cl_twx,
                         (const float2*)h->cl_twh, d, h->rz, h->rx, h->zcols, h->xrows, h->sc, h->stream);
  launch_mlp_closure(h->cl_mlp, reinterpret_cast<const float*>(h->cl_P), reinterpret_cast<float*>(h->cl_tau),
                     h->cl_wd, (long long)d.nzd * 2 * d.nxd, d.nplanes, d.ny, &h->sc->error, 4, h->nsm, h->stream);
  h->launches += 5;
}

void run_convolutions(chgpu_handle* h, int compute_cfl, int products, int plane0, int nplanes, int stage_lo = 0,
                      int stage_hi = 3, int ix_lo = 0, int ix_hi = -1) {
  ConvLaunch L = conv_launch(h, compute_cfl, products, plane0, nplanes);
  if (ix_hi >= 0) {
    L.ix_lo = ix_lo;
    L.ix_hi = ix_hi;
  }
  if (products && (h->cl_on || h->cl_fixed)) L.tau = h->cl_tau;
  if (products && h->cl_on && stage_lo == 0) enqueue_closure(h);
  const int nst = products ? 3 : 2;
  for (int stage = stage_lo; stage < std::min(nst, stage_hi); ++stage) {
    timed(h, stage, [&] {
      if (h->prec == CHGPU_MIXED) launch_convolutions<float>(L, h->stream, stage);
      else if (h->prec == CHGPU_FP64DD) launch_convolutions<dd>(L, h->stream, stage);
      else launch_convolutions<double>(L, h->stream, stage);
    });
    h->launches += 1;
  }
}

void run_rhs(chgpu_handle* h, const double* ode, cudaStream_t s = nullptr, int m_lo = 0, int m_hi = -1) {
  SolveLaunch L = solve_launch(h, ode);
  if (m_hi >= 0) {
    L.m_lo = m_lo;
    L.m_hi = m_hi;
  }
  if (!s) s = h->stream;
  timed(h, 3, [&] {
    if (h->prec == CHGPU_MIXED) launch_rhs<float>(L, s);
    else if (h->prec == CHGPU_FP64DD) launch_rhs<dd>(L, s);
    else launch_rhs<double>(L, s);
  });
  h->launches += 1;
}

// rhs_in_field: read the right-hand sides from V (the reference's in-place
// convention) instead of the separate buffer k_rhs writes.
// k_factor of one substep on the third stream, after everything enqueued on
// the main stream so far (the previous substep's k_solve, which reads fac,
// and for a step's first substep the outstats that set dt) and, with two
// halves, after half B's solve; k_solve waits for ev_factored.
void enqueue_factor(chgpu_handle* h, double ode1, bool after_half_b) {
  SolveLaunch L = solve_launch(h, nullptr);
  L.ode[0] = ode1;
  L.lambda_from_dt = 1;
  cudaEventRecord(h->ev_fac_fork, h->stream);
  cudaStreamWaitEvent(h->stream3, h->ev_fac_fork, 0);
  if (after_half_b) cudaStreamWaitEvent(h->stream3, h->ev_solved, 0);
  launch_factor(L, h->stream3);
  cudaEventRecord(h->ev_factored, h->stream3);
  h->launches += 1;
}

void run_linsolve(chgpu_handle* h, double ode1, double lambda, int from_dt, bool rhs_in_field,
                  cudaStream_t s = nullptr, int q_lo = 0, int q_hi = -1, bool factored = false) {
  SolveLaunch L = solve_launch(h, nullptr);
  L.ode[0] = ode1;
  L.lambda = lambda;
  L.lambda_from_dt = from_dt;
  if (q_hi >= 0) {
    L.q_lo = q_lo;
    L.q_hi = q_hi;
  }
  if (rhs_in_field) {
    L.rhs_src = h->V;
    L.rhs_cstride = (size_t)h->d.nplanes * h->d.nmodes;
    L.rhs_plane_off = 1;
  } else {
    L.rhs_src = h->rhs;
    L.rhs_cstride = (size_t)(h->d.ny - 1) * h->d.nmodes;
    L.rhs_plane_off = -1;
  }
  if (!s) s = h->stream;
  L.split_solve = h->solve_form == 1 ? 0 : (h->solve_form == 4 ? 2 : (h->solve_form == 5 ? 3 : 1));
  L.factored = factored && h->solve_form >= 2 ? 1 : 0;
  if (L.factored) cudaStreamWaitEvent(s, h->ev_factored, 0);
  timed(h, 4, [&] { launch_linsolve(L, s); });
  h->launches += h->solve_form >= 2 && !L.factored ? 2 : 1;
}

void run_outstats(chgpu_handle* h) {
  SolveLaunch L = solve_launch(h, nullptr);
  timed(h, 5, [&] { launch_outstats(L, h->stream); });
  h->launches += 1;
}

// One time-loop iteration (channel.f90:118-167) on the stream.
//
// With halves = 2 (and no per-kernel timing) the kx columns split in two
// halves A (kx < KA, holding the mean mode) and B: k_rhs, k_linsolve and the
// next substep's z-inverse touch only the modes of their half, so half B's
// rhs and solve run on the side stream, started after half A's rhs, while
// half A's solve and next z-inverse run on the main one -- the
// latency-bound solve of one half overlaps the other half's work.  The x pass, which needs every kx, joins
// both; so does the end of the step.  Nothing half B's kernels read is
// written by half A's (the mean-mode scalars are read only for the mean mode).
//
// With the factorisation ahead (solve forms 3 and 4, no per-kernel timing) each substep's
// k_factor is enqueued first on the third stream and overlaps the substep's
// transforms and k_rhs; the solves wait for it.
void enqueue_step(chgpu_handle* h) {
  const bool split = h->halves == 2 && !h->profiling && h->d.nx >= 1 && !h->cl_on && !h->cl_fixed;
  const bool ahead = h->solve_form >= 3 && !h->profiling;
  const int KA = (h->d.nx + 1 + 1) / 2, nxp = h->d.nx + 1;
  const int mA = KA * h->d.nzt, qA = KA * (h->d.nz + 1);
  for (int k = 0; k < 3; ++k) {
    if (ahead) enqueue_factor(h, RK[k][0], split && k > 0);
    timed(h, 5, [&] { launch_advance_time(h->sc, 2.0 / RK[k][0], k == 0, h->stream); });
    h->launches += 1;
    if (!split) {
      run_convolutions(h, k == 2, 1, 0, h->d.nplanes);
      run_rhs(h, RK[k]);
      run_linsolve(h, RK[k][0], 0.0, 1, false, nullptr, 0, -1, ahead);
      continue;
    }
    if (k == 0) {
      run_convolutions(h, 0, 1, 0, h->d.nplanes, 0, 1);  // z-inverse, all kx
    } else {
      run_convolutions(h, 0, 1, 0, h->d.nplanes, 0, 1, 0, KA);  // half A (its solve is done)
      cudaStreamWaitEvent(h->stream, h->ev_solved, 0);
      run_convolutions(h, 0, 1, 0, h->d.nplanes, 0, 1, KA, nxp);  // half B
    }
    run_convolutions(h, k == 2, 1, 0, h->d.nplanes, 1, 3);  // x pass and z-forward, all kx
    // staggered: half B's rhs starts when half A's is done, so it overlaps
    // half A's solve, and half A's next z-inverse overlaps half B's solve
    run_rhs(h, RK[k], h->stream, 0, mA);
    cudaEventRecord(h->ev_vv, h->stream);
    cudaStreamWaitEvent(h->stream2, h->ev_vv, 0);
    run_rhs(h, RK[k], h->stream2, mA, h->d.nmodes);
    run_linsolve(h, RK[k][0], 0.0, 1, false, h->stream2, qA, h->d.npairs, ahead);
    cudaEventRecord(h->ev_solved, h->stream2);
    run_linsolve(h, RK[k][0], 0.0, 1, false, h->stream, 0, qA, ahead);
  }
  if (split) cudaStreamWaitEvent(h->stream, h->ev_solved, 0);
  run_outstats(h);
}

void fill_stats(const chgpu_handle* h, chgpu_stats* st) {
  const DevScalars& s = *h->sc_host;
  std::memcpy(st->line, s.line, sizeof st->line);
  std::memcpy(st->fr, s.fr, sizeof st->fr);
  st->corrpx = s.corrpx;
  st->corrpz = s.corrpz;
  st->meanpx = s.meanpx;
  st->meanpz = s.meanpz;
  st->cfl = s.runtime_global;
  st->deltat = s.deltat;
  st->time = s.time;
  st->istep = s.istep;
}

int pull_scalars(chgpu_handle* h) {
  CK(h, cudaMemcpyAsync(h->sc_host, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (h->sc_host->error & 2) return fail(h, CHGPU_E_CUDA, "a bulk copy into shared memory did not complete in time");
  if (h->sc_host->error & 4) return fail(h, CHGPU_E_CUDA, "a tensor-core completion wait of the closure ran out");
  if (h->sc_host->error & 1) return fail(h, CHGPU_E_NONFINITE, "non-finite CFL or statistics (flow field blew up)");
  return 0;
}

void release(chgpu_handle* h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (auto& pe : h->ev_pending) {
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  void* bufs[] = {h->V, h->F, h->old, h->VV, h->Zb, h->Pb, h->rhs, h->fac, h->der, h->derT, h->derL, h->cst, h->d0lu, h->nud, h->lindd, h->yint, h->dy,
                  h->twz, h->twx, h->twh, h->twzr, h->twxr, h->sc, h->ex_W, h->ex_P, h->ex_out, h->ex_twz, h->ex_twx,
                  h->cl_G, h->cl_Z, h->cl_P, h->cl_tau, h->cl_wd, h->cl_twz, h->cl_twx, h->cl_twh,
                  h->tke_W, h->tke_N, h->tke_P, h->tke_Zt, h->tke_Xt, h->tke_acc, h->tke_mean,
                  h->tke_twz, h->tke_twx, h->tke_twh};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (h->sc_host) cudaFreeHost(h->sc_host);
  if (h->stats_acc) cudaFree(h->stats_acc);
  if (h->snap_stage) cudaFree(h->snap_stage);
  if (h->snap_host) cudaFreeHost(h->snap_host);
  if (h->snap_read) cudaEventDestroy(h->snap_read);
  if (h->snap_done) cudaEventDestroy(h->snap_done);
  if (h->snap_stream) cudaStreamDestroy(h->snap_stream);
  if (h->ev_vv) cudaEventDestroy(h->ev_vv);
  if (h->ev_solved) cudaEventDestroy(h->ev_solved);
  if (h->ev_fac_fork) cudaEventDestroy(h->ev_fac_fork);
  if (h->ev_copy_fork) cudaEventDestroy(h->ev_copy_fork);
  if (h->ev_copy_join) cudaEventDestroy(h->ev_copy_join);
  if (h->ev_factored) cudaEventDestroy(h->ev_factored);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->stream3) cudaStreamDestroy(h->stream3);
  if (h->stream) cudaStreamDestroy(h->stream);
}

}  // namespace

extern "C" {

const char* chgpu_last_error(const chgpu_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int chgpu_create(const chgpu_params* p, chgpu_handle** out) {
  if (!p || !out) return fail(nullptr, CHGPU_E_PARAM, "chgpu_create: null argument");
  *out = nullptr;
  if (p->nx < 1 || p->nz < 1 || p->ny < 8)
    return fail(nullptr, CHGPU_E_PARAM, "chgpu_create: need nx>=1, nz>=1, ny>=8");
  if (!(p->ymax > p->ymin) || !(p->a > 0) || !(p->alfa0 > 0) || !(p->beta0 > 0) || !(p->ni > 0))
    return fail(nullptr, CHGPU_E_PARAM, "chgpu_create: need ymax>ymin, a>0, alfa0>0, beta0>0, ni>0");
  if (p->precision != CHGPU_FP64 && p->precision != CHGPU_MIXED && p->precision != CHGPU_FP64DD)
    return fail(nullptr, CHGPU_E_PARAM, "chgpu_create: precision must be CHGPU_FP64, CHGPU_MIXED or CHGPU_FP64DD");
  if (p->cpi && p->cpi_type != 0 && p->cpi_type != 1)
    return fail(nullptr, CHGPU_E_PARAM, "Wrong selection of CPI_Type");  // linsolve_blocking.inc:93-95
  chgpu_handle* h = new (std::nothrow) chgpu_handle();
  if (!h) return fail(nullptr, CHGPU_E_NOMEM, "chgpu_create: host allocation failed");
  h->p = *p;
  h->prec = p->precision;
  int nxd, nzd;
  padded_sizes(p->nx, p->nz, &nxd, &nzd);
  Dims& d = h->d;
  d.nx = p->nx; d.ny = p->ny; d.nz = p->nz;
  d.nzt = 2 * p->nz + 1;
  d.nxd = nxd; d.nzd = nzd;
  d.nplanes = p->ny + 3;
  d.nmodes = (p->nx + 1) * d.nzt;
  d.npairs = (p->nx + 1) * (p->nz + 1);
  d.alfa0 = p->alfa0; d.beta0 = p->beta0; d.ni = p->ni;
  const double PI = 3.1415926535897932384626433832795028841971;
  const double dx = PI / (p->alfa0 * nxd), dz = 2.0 * PI / (p->beta0 * nzd);
  d.factor = 1.0 / (2.0 * nxd * nzd);  // dnsdata.f90:124
  d.rdx = 1.0 / dx;
  d.rdz = 1.0 / dz;
  d.meanflowx = p->meanflowx; d.meanflowz = p->meanflowz;
  d.cflmax = p->cflmax; d.gamma = p->gamma;
  d.cpi = p->cpi; d.cpi_type = p->cpi_type;
  compute_tables(*p, h->tab);
  const Tables& t = h->tab;
  std::memcpy(h->bc.v0bc, t.v0bc, 40); std::memcpy(h->bc.v0m1bc, t.v0m1bc, 40);
  std::memcpy(h->bc.eta0bc, t.eta0bc, 40); std::memcpy(h->bc.eta0m1bc, t.eta0m1bc, 40);
  std::memcpy(h->bc.vnbc, t.vnbc, 40); std::memcpy(h->bc.vnp1bc, t.vnp1bc, 40);
  std::memcpy(h->bc.etanbc, t.etanbc, 40); std::memcpy(h->bc.etanp1bc, t.etanp1bc, 40);
  std::memcpy(h->bc.d140, t.d140, 40); std::memcpy(h->bc.d14m1, t.d14m1, 40);
  std::memcpy(h->bc.d14n, t.d14n, 40); std::memcpy(h->bc.d14np1, t.d14np1, 40);
  // composite tail stage where measured faster: the FP32 x transforms (the
  // z ones lose occupancy to its registers)
  Radix rz = make_radix(nzd, false), rx = make_radix(nxd, h->prec == CHGPU_MIXED);
  if (rz.nst < 0 || rx.nst < 0) { delete h; return fail(nullptr, CHGPU_E_PARAM, "unsupported FFT length"); }
  {
    // register-blocked transforms where they measured faster (GB300, 127x192x127
    // and 383x384x383): FP32 z and x passes (x-row 92 -> 59 ms, z-forward
    // 20 -> 10.5 ms per step at 383x384x383); FP64 z passes (even with the
    // generic kernels; the FP64 x-row kernel stays generic, 977 vs 1017 ms);
    // double-float keeps the generic kernels (its register-blocked x-row
    // kernel spills: 820 vs 354 ms)
    int e_ = 0, tpr_ = 0;
    h->zfast = rlen_plan(nzd, &e_, &tpr_) && h->prec != CHGPU_FP64DD;
    h->xfast = xlen_plan(nxd, &e_, &tpr_) && h->prec == CHGPU_MIXED;
  }
  h->halves = d.npairs >= 65536 ? 2 : 1;
  h->solve_form = d.npairs < 65536 ? 3 : 1;
  h->rz.n = rz.n; h->rz.nst = rz.nst; std::memcpy(h->rz.r, rz.r, sizeof rz.r);
  h->rx.n = rx.n; h->rx.nst = rx.nst; std::memcpy(h->rx.r, rx.r, sizeof rx.r);
  set_twiddle_offsets(h->rz);
  set_twiddle_offsets(h->rx);
  // tiles: columns per z-transform block and rows per x block, from the
  // shared-memory budget (two ping-pong buffers; nine row buffers)
  const size_t ts = tsize(h);
  h->zcols = 8;
  while (h->zcols > 1 && conv_zinv_smem(h->zcols, nzd, d.nzt, ts) > 100 * 1024) --h->zcols;
  // rows per x block: the most that keep two resident blocks per SM (228 KB
  // of shared memory per SM, 1 KB reserved per block); chgpu_autotune may
  // choose otherwise by timing
  const size_t xbudget = 233472 / 2 - 1024 - 512;
  h->xrows = 1;
  while (h->xrows < 4 && conv_x_smem(2 * h->xrows, nxd, ts) <= xbudget && nzd % (2 * h->xrows) == 0)
    h->xrows *= 2;
  if (conv_x_smem(h->xrows, nxd, ts) > 227 * 1024 || conv_zinv_smem(1, nzd, d.nzt, ts) > 227 * 1024) {
    delete h;
    return fail(nullptr, CHGPU_E_PARAM, "transform length too large for one thread block");
  }
  int rc = 0;
  auto dev_alloc = [&](void** ptr, size_t bytes, const char* what) -> int {
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) return cuda_fail(h, e, what);
    return 0;
  };
  const size_t nplanes = d.nplanes, nmodes = d.nmodes, nxp = p->nx + 1;
  do {
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_vv, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_solved, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream3, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fac_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_factored, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_copy_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_copy_join, cudaEventDisableTiming);
    if (e != cudaSuccess) { rc = cuda_fail(h, e, "cudaStreamCreate"); break; }
    e = conv_set_smem_limits();
    if (e != cudaSuccess) { rc = cuda_fail(h, e, "cudaFuncSetAttribute"); break; }
    if ((rc = dev_alloc((void**)&h->V, sizeof(double2) * 3 * nplanes * nmodes, "field"))) break;
    if ((rc = dev_alloc(&h->old, ts * 2 * (p->ny - 1) * nmodes, "RK history"))) break;
    if ((rc = dev_alloc(&h->VV, ts * 6 * nplanes * nmodes, "product spectra"))) break;
    if ((rc = dev_alloc(&h->Zb, ts * 3 * nplanes * nxp * nzd, "z work buffer"))) break;
    if ((rc = dev_alloc(&h->Pb, std::max(ts * 6 * nplanes * nxp * nzd, sizeof(double2) * 3 * nplanes * nmodes),
                        "x work buffer"))) break;
    if ((rc = dev_alloc((void**)&h->rhs, sizeof(double2) * 2 * (p->ny - 1) * nmodes, "rhs"))) break;
    if ((rc = dev_alloc((void**)&h->fac,
                        sizeof(double) * kFacPerRow * (p->ny - 1) *
                            (size_t)d.npairs,
                        "factors")))
      break;
    if ((rc = dev_alloc((void**)&h->der, sizeof(double) * t.der.size(), "der"))) break;
    if ((rc = dev_alloc((void**)&h->d0lu, sizeof(double) * t.d0lu.size(), "D0mat"))) break;
    if ((rc = dev_alloc((void**)&h->yint, sizeof(double) * std::max<size_t>(3, t.yint.size()), "yint"))) break;
    if ((rc = dev_alloc((void**)&h->dy, sizeof(double) * t.dy.size(), "dy"))) break;
    if ((rc = dev_alloc((void**)&h->sc, sizeof(DevScalars), "scalars"))) break;
    e = cudaMallocHost((void**)&h->sc_host, sizeof(DevScalars));
    if (e != cudaSuccess) { rc = cuda_fail(h, e, "cudaMallocHost"); break; }
    if (h->prec == CHGPU_MIXED) {
      if ((rc = upload_stage_twiddles<float2>(h, &h->twz, h->rz))) break;
      if ((rc = upload_stage_twiddles<float2>(h, &h->twx, h->rx))) break;
      if ((rc = upload_pack_roots<float2>(h, &h->twh, 2 * nxd, 0.5L * (long double)d.factor))) break;
      if ((rc = upload_rplan_twiddles<float2>(h, &h->twzr, nzd))) break;
      if ((rc = upload_rplan_twiddles<float2>(h, &h->twxr, nxd, true))) break;
      if ((rc = upload_derT<float>(h))) break;
      if ((rc = upload_derL<dd>(h))) break;
    } else if (h->prec == CHGPU_FP64DD) {
      if ((rc = upload_stage_twiddles<cdd>(h, &h->twz, h->rz))) break;
      if ((rc = upload_stage_twiddles<cdd>(h, &h->twx, h->rx))) break;
      if ((rc = upload_pack_roots<cdd>(h, &h->twh, 2 * nxd, 0.5L * (long double)d.factor))) break;
      if ((rc = upload_rplan_twiddles<cdd>(h, &h->twzr, nzd))) break;
      if ((rc = upload_rplan_twiddles<cdd>(h, &h->twxr, nxd, true))) break;
      if ((rc = upload_derT<dd>(h))) break;
      if ((rc = upload_derL<double>(h))) break;
    } else {
      if ((rc = upload_stage_twiddles<double2>(h, &h->twz, h->rz))) break;
      if ((rc = upload_stage_twiddles<double2>(h, &h->twx, h->rx))) break;
      if ((rc = upload_pack_roots<double2>(h, &h->twh, 2 * nxd, 0.5L * (long double)d.factor))) break;
      if ((rc = upload_rplan_twiddles<double2>(h, &h->twzr, nzd))) break;
      if ((rc = upload_rplan_twiddles<double2>(h, &h->twxr, nxd, true))) break;
      if ((rc = upload_derT<double>(h))) break;
      if ((rc = upload_derL<double>(h))) break;
    }
    // mixed and double-float paths: v' and u, w in double-float; per y row:
    // d1 row, D0mat factors (rows 1..ny-1), d0 row
    if (h->prec != CHGPU_FP64) {
      std::vector<dd> ld((size_t)(p->ny + 1) * 15, dd());
      for (int iy = 0; iy <= p->ny; ++iy)
        for (int j = 0; j < 5; ++j) {
          ld[(size_t)iy * 15 + j] = from_ld<dd>((long double)t.der[(size_t)iy * 20 + 5 + j]);
          ld[(size_t)iy * 15 + 10 + j] = from_ld<dd>((long double)t.der[(size_t)iy * 20 + j]);
          if (iy >= 1 && iy <= p->ny - 1)
            ld[(size_t)iy * 15 + 5 + j] = from_ld<dd>((long double)t.d0lu[(size_t)(iy - 1) * 5 + j]);
        }
      if ((rc = dev_alloc(&h->lindd, sizeof(dd) * ld.size(), "double-float derivative rows"))) break;
      cudaMemcpy(h->lindd, ld.data(), sizeof(dd) * ld.size(), cudaMemcpyHostToDevice);
    }
    {
      std::vector<double> nu((size_t)(p->ny + 1) * 10, 0.0);
      const double mni = -p->ni;
      for (int iy = 0; iy <= p->ny; ++iy)
        for (int j = 0; j < 5; ++j) {
          nu[(size_t)iy * 10 + j] = mni * t.der[(size_t)iy * 20 + 15 + j];
          nu[(size_t)iy * 10 + 5 + j] = mni * t.der[(size_t)iy * 20 + 10 + j];
        }
      if ((rc = dev_alloc((void**)&h->nud, sizeof(double) * nu.size(), "viscous rows"))) break;
      cudaMemcpy(h->nud, nu.data(), sizeof(double) * nu.size(), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(h->der, t.der.data(), sizeof(double) * t.der.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(h->d0lu, t.d0lu.data(), sizeof(double) * t.d0lu.size(), cudaMemcpyHostToDevice);
    if (!t.yint.empty()) cudaMemcpy(h->yint, t.yint.data(), sizeof(double) * t.yint.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(h->dy, t.dy.data(), sizeof(double) * t.dy.size(), cudaMemcpyHostToDevice);
    cudaMemset(h->V, 0, sizeof(double2) * 3 * nplanes * nmodes);
    cudaMemset(h->old, 0, ts * 2 * (p->ny - 1) * nmodes);  // oldrhs starts at zero (RK1 has ODE(3)=0)
    DevScalars s{};
    s.deltat = p->deltat;
    s.rdt = 1.0 / p->deltat;
    s.time = p->time;
    s.meanpx = p->meanpx;
    s.meanpz = p->meanpz;
    s.u0 = p->u0;
    s.uN = p->uN;
    *h->sc_host = s;
    e = cudaMemcpy(h->sc, &s, sizeof s, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { rc = cuda_fail(h, e, "upload scalars"); break; }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { rc = cuda_fail(h, e, "set-up"); break; }
  } while (0);
  if (rc) {
    g_create_error = h->err;
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return 0;
}

int chgpu_destroy(chgpu_handle* h) {
  if (!h) return 0;
  // work in flight on any of the handle's streams (a snapshot copy into the
  // pinned buffer, a half of the split step) ends before anything is freed
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->stream3) cudaStreamSynchronize(h->stream3);
  if (h->snap_stream) cudaStreamSynchronize(h->snap_stream);
  release(h);
  delete h;
  return 0;
}

size_t chgpu_field_doubles(const chgpu_handle* h) { return h ? (size_t)2 * 3 * h->d.nplanes * h->d.nmodes : 0; }

int chgpu_upload_field(chgpu_handle* h, const double* V) {
  if (!h || !V) return fail(h, CHGPU_E_PARAM, "chgpu_upload_field: null argument");
  const size_t n = (size_t)3 * h->d.nplanes * h->d.nmodes;
  double2* stage = reinterpret_cast<double2*>(h->Pb);
  // the two halves on two streams: one host-to-device copy of pinned memory
  // measured ~110 GB/s on GB300, two concurrent ones ~210 GB/s; both start
  // after the work already on the handle's stream (the staging buffer is
  // step scratch) and the transposes wait for both
  const size_t half = n / 2;
  CK(h, cudaEventRecord(h->ev_copy_fork, h->stream));
  CK(h, cudaStreamWaitEvent(h->stream2, h->ev_copy_fork, 0));
  CK(h, cudaMemcpyAsync(stage, V, sizeof(double2) * half, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(stage + half, V + 2 * half, sizeof(double2) * (n - half), cudaMemcpyHostToDevice,
                        h->stream2));
  CK(h, cudaEventRecord(h->ev_copy_join, h->stream2));
  CK(h, cudaStreamWaitEvent(h->stream, h->ev_copy_join, 0));
  // restart order per component: [mode][iy] -> device [iy][mode]
  launch_transpose(stage, h->V, h->d.nmodes, h->d.nplanes, 3, h->stream);
  h->launches += 1;
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  h->field_set = true;
  return 0;
}

int chgpu_download_field(chgpu_handle* h, double* V) {
  if (!h || !V) return fail(h, CHGPU_E_PARAM, "chgpu_download_field: null argument");
  const size_t n = (size_t)3 * h->d.nplanes * h->d.nmodes;
  double2* stage = reinterpret_cast<double2*>(h->Pb);
  launch_transpose(h->V, stage, h->d.nplanes, h->d.nmodes, 3, h->stream);
  h->launches += 1;
  CK(h, cudaGetLastError());
  CK(h, cudaMemcpyAsync(V, stage, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int chgpu_start(chgpu_handle* h, double time, double deltat, chgpu_stats* st) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_start: null handle");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_start: upload the field first");
  if (deltat == 0) deltat = 1.0;  // channel.f90:97
  DevScalars s = *h->sc_host;
  CK(h, cudaMemcpyAsync(h->sc_host, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  s = *h->sc_host;
  s.time = time;
  s.deltat = deltat;
  s.rdt = 1.0 / deltat;
  s.cfl = 0.0;
  s.istep = 0;
  *h->sc_host = s;
  CK(h, cudaMemcpyAsync(h->sc, h->sc_host, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
  run_convolutions(h, 1, 0, 2, h->d.ny - 1);  // planes iy=1..ny-1 (channel.f90:96-99)
  SolveLaunch L = solve_launch(h, nullptr);
  launch_flowrate(L, h->stream);
  h->launches += 1;
  run_outstats(h);
  CK(h, cudaGetLastError());
  int rc = pull_scalars(h);
  if (st) fill_stats(h, st);
  return rc;
}

int chgpu_set_wall_velocity(chgpu_handle* h, double u0, double uN) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  double v[2] = {u0, uN};
  CK(h, cudaMemcpyAsync(&h->sc->u0, v, sizeof v, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int chgpu_buildrhs(chgpu_handle* h, const double ode[3], int compute_cfl) {
  if (!h || !ode) return fail(h, CHGPU_E_PARAM, "chgpu_buildrhs: null argument");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_buildrhs: upload the field first");
  run_convolutions(h, compute_cfl ? 1 : 0, 1, 0, h->d.nplanes);
  run_rhs(h, ode);
  // write-back of the new right-hand sides into V(1:ny-1, :, :, 1:2) (dnsdata.f90:667-670)
  const size_t rows = (size_t)(h->d.ny - 1) * h->d.nmodes;
  for (int c = 0; c < 2; ++c)
    CK(h, cudaMemcpyAsync(h->V + ((size_t)c * h->d.nplanes + 2) * h->d.nmodes, h->rhs + c * rows,
                          sizeof(double2) * rows, cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaGetLastError());
  return 0;
}

int chgpu_linsolve(chgpu_handle* h, double lambda) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_linsolve: null handle");
  run_linsolve(h, 0.0, lambda, 0, true);
  CK(h, cudaGetLastError());
  return 0;
}

int chgpu_outstats(chgpu_handle* h, chgpu_stats* st) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_outstats: null handle");
  run_outstats(h);
  CK(h, cudaGetLastError());
  int rc = pull_scalars(h);
  if (st) fill_stats(h, st);
  return rc;
}

int chgpu_step(chgpu_handle* h, chgpu_stats* st) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_step: null handle");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_step: upload the field first");
  if (h->profiling) {
    enqueue_step(h);
    CK(h, cudaGetLastError());
    if (st) {
      int rc = pull_scalars(h);
      fill_stats(h, st);
      return rc;
    }
    return 0;
  }
  if (!h->graph) {
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = h->launches;
    enqueue_step(h);
    h->step_launches = h->launches - before;
    h->launches = before;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      h->graph = nullptr;
      return cuda_fail(h, e, "cudaGraphInstantiate");
    }
  }
  CK(h, cudaGraphLaunch(h->graph, h->stream));
  h->launches += h->step_launches;
  if (st) {
    int rc = pull_scalars(h);
    fill_stats(h, st);
    return rc;
  }
  return 0;
}

int chgpu_get_stats(chgpu_handle* h, chgpu_stats* st) {
  if (!h || !st) return fail(h, CHGPU_E_PARAM, "chgpu_get_stats: null argument");
  int rc = pull_scalars(h);
  fill_stats(h, st);
  return rc;
}

int chgpu_synchronize(chgpu_handle* h) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  return pull_scalars(h);
}

int chgpu_set_profiling(chgpu_handle* h, int on) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  h->profiling = on != 0;
  for (int k = 0; k < CHGPU_NKINDS; ++k) {
    h->kind_ms[k] = 0;
    h->kind_n[k] = 0;
  }
  return 0;
}

int chgpu_kernel_times(chgpu_handle* h, double ms[CHGPU_NKINDS], long long launches[CHGPU_NKINDS]) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  CK(h, cudaStreamSynchronize(h->stream));
  for (auto& pe : h->ev_pending) {
    float t = 0.f;
    CK(h, cudaEventElapsedTime(&t, pe.second.first, pe.second.second));
    h->kind_ms[pe.first] += t;
    h->kind_n[pe.first] += 1;
    h->ev_pool.push_back(pe.second.first);
    h->ev_pool.push_back(pe.second.second);
  }
  h->ev_pending.clear();
  for (int k = 0; k < CHGPU_NKINDS; ++k) {
    if (ms) ms[k] = h->kind_ms[k];
    if (launches) launches[k] = h->kind_n[k];
  }
  return 0;
}

const char* chgpu_kernel_kind_name(int kind) {
  static const char* names[CHGPU_NKINDS] = {"k_zinv", "k_xrow", "k_zfwd", "k_rhs", "k_linsolve", "scalars"};
  return (kind >= 0 && kind < CHGPU_NKINDS) ? names[kind] : "?";
}

// ---------------------------------------------------------------------------
// ensemble of independent runs: one graph launch per step for all members
// ---------------------------------------------------------------------------
struct chgpu_ensemble {
  std::vector<chgpu_handle*> m;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t graph = nullptr;
  std::vector<long long> versions;  // member versions the graph was captured with
  std::string err;
};

namespace {

int ens_fail(chgpu_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  else g_create_error = msg;
  return code;
}

#define CKE(e, call)                                                                             \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return ens_fail((e), e_ == cudaErrorMemoryAllocation ? CHGPU_E_NOMEM : CHGPU_E_CUDA,        \
                      std::string(#call) + ": " + cudaGetErrorName(e_) + " (" + cudaGetErrorString(e_) + ")"); \
  } while (0)

void ens_release(chgpu_ensemble* e) {
  if (e->graph) cudaGraphExecDestroy(e->graph);
  for (cudaEvent_t ev : e->join)
    if (ev) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->stream) cudaStreamDestroy(e->stream);
  for (chgpu_handle* h : e->m)
    if (h) chgpu_destroy(h);
}

}  // namespace

int chgpu_ensemble_create(const chgpu_params* params, int n, chgpu_ensemble** out) {
  if (!out) return ens_fail(nullptr, CHGPU_E_PARAM, "chgpu_ensemble_create: null output");
  *out = nullptr;
  if (!params || n < 1) return ens_fail(nullptr, CHGPU_E_PARAM, "chgpu_ensemble_create: need n >= 1 parameter sets");
  chgpu_ensemble* e = new (std::nothrow) chgpu_ensemble;
  if (!e) return ens_fail(nullptr, CHGPU_E_NOMEM, "chgpu_ensemble_create: out of host memory");
  e->m.assign(n, nullptr);
  e->join.assign(n, nullptr);
  for (int i = 0; i < n; ++i) {
    if (int rc = chgpu_create(&params[i], &e->m[i])) {
      const std::string msg = "member " + std::to_string(i) + ": " + chgpu_last_error(nullptr);
      ens_release(e);
      delete e;
      return ens_fail(nullptr, rc, msg);
    }
  }
  cudaError_t c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (c == cudaSuccess) c = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  for (int i = 0; i < n && c == cudaSuccess; ++i) c = cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming);
  if (c != cudaSuccess) {
    ens_release(e);
    delete e;
    return ens_fail(nullptr, CHGPU_E_CUDA, std::string("chgpu_ensemble_create: ") + cudaGetErrorString(c));
  }
  *out = e;
  return 0;
}

int chgpu_ensemble_destroy(chgpu_ensemble* e) {
  if (!e) return 0;
  if (e->stream) cudaStreamSynchronize(e->stream);
  ens_release(e);
  delete e;
  return 0;
}

int chgpu_ensemble_size(const chgpu_ensemble* e) { return e ? (int)e->m.size() : 0; }

chgpu_handle* chgpu_ensemble_member(chgpu_ensemble* e, int i) {
  return (e && i >= 0 && i < (int)e->m.size()) ? e->m[i] : nullptr;
}

int chgpu_ensemble_step(chgpu_ensemble* e, chgpu_stats* st) {
  if (!e) return ens_fail(e, CHGPU_E_PARAM, "chgpu_ensemble_step: null ensemble");
  const int n = (int)e->m.size();
  bool stale = !e->graph || (int)e->versions.size() != n;
  for (int i = 0; i < n; ++i) {
    if (!e->m[i]->field_set) return ens_fail(e, CHGPU_E_STATE, "chgpu_ensemble_step: member without a field");
    if (!stale && e->versions[i] != e->m[i]->version) stale = true;
  }
  if (stale) {
    if (e->graph) {
      cudaGraphExecDestroy(e->graph);
      e->graph = nullptr;
    }
    // fork from the ensemble stream into every member's stream, enqueue each
    // member's step there, join back: one graph whose branches run together
    cudaGraph_t g = nullptr;
    CKE(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    CKE(e, cudaEventRecord(e->fork, e->stream));
    for (int i = 0; i < n; ++i) {
      chgpu_handle* h = e->m[i];
      const bool prof = h->profiling;
      h->profiling = false;
      const long long before = h->launches;
      cudaStreamWaitEvent(h->stream, e->fork, 0);
      enqueue_step(h);
      cudaEventRecord(e->join[i], h->stream);
      cudaStreamWaitEvent(e->stream, e->join[i], 0);
      h->step_launches = h->launches - before;
      h->launches = before;
      h->profiling = prof;
    }
    cudaError_t c = cudaStreamEndCapture(e->stream, &g);
    if (c != cudaSuccess) return ens_fail(e, CHGPU_E_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(c));
    c = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (c != cudaSuccess) {
      e->graph = nullptr;
      return ens_fail(e, CHGPU_E_CUDA, std::string("ensemble graph: ") + cudaGetErrorString(c));
    }
    e->versions.resize(n);
    for (int i = 0; i < n; ++i) e->versions[i] = e->m[i]->version;
  }
  CKE(e, cudaGraphLaunch(e->graph, e->stream));
  for (chgpu_handle* h : e->m) h->launches += h->step_launches;
  if (!st) return 0;
  for (chgpu_handle* h : e->m)
    CKE(e, cudaMemcpyAsync(h->sc_host, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, e->stream));
  CKE(e, cudaStreamSynchronize(e->stream));
  int rc = 0;
  for (int i = 0; i < n; ++i) {
    fill_stats(e->m[i], &st[i]);
    if ((e->m[i]->sc_host->error & 1) && rc == 0)
      rc = ens_fail(e, CHGPU_E_NONFINITE, "member " + std::to_string(i) + ": non-finite CFL or statistics");
  }
  return rc;
}

int chgpu_ensemble_synchronize(chgpu_ensemble* e) {
  if (!e) return ens_fail(e, CHGPU_E_PARAM, "null ensemble");
  CKE(e, cudaStreamSynchronize(e->stream));
  return 0;
}

void* chgpu_ensemble_stream(chgpu_ensemble* e) { return e ? (void*)e->stream : nullptr; }

const char* chgpu_ensemble_last_error(const chgpu_ensemble* e) { return e ? e->err.c_str() : g_create_error.c_str(); }

// ---------------------------------------------------------------------------
// autotuner of the transform tiles
// ---------------------------------------------------------------------------
namespace {

// average device time of `reps` launches of one convolution stage over all
// planes with the handle's current tiles (after one untimed launch)
int time_conv_stage(chgpu_handle* h, int stage, int reps, float* ms) {
  ConvLaunch L = conv_launch(h, 0, 1, 0, h->d.nplanes);
  auto launch = [&] {
    if (h->prec == CHGPU_MIXED) launch_convolutions<float>(L, h->stream, stage);
    else if (h->prec == CHGPU_FP64DD) launch_convolutions<dd>(L, h->stream, stage);
    else launch_convolutions<double>(L, h->stream, stage);
  };
  cudaEvent_t a = take_event(h), b = take_event(h);
  launch();
  CK(h, cudaEventRecord(a, h->stream));
  for (int i = 0; i < reps; ++i) launch();
  CK(h, cudaEventRecord(b, h->stream));
  CK(h, cudaGetLastError());
  CK(h, cudaEventSynchronize(b));
  CK(h, cudaEventElapsedTime(ms, a, b));
  *ms /= (float)reps;
  h->ev_pool.push_back(a);
  h->ev_pool.push_back(b);
  h->launches += reps + 1;
  return 0;
}

}  // namespace

namespace {

// The banded solves as one fused kernel (two threads per (kx, +-kz) pair,
// one per system), as the factorisation kernel and a substitution kernel
// with four threads per pair (one per system and mode), as those two with
// the factorisation on a third stream beside the substep's transforms, or
// with the factorisation ahead and the fused kernel's two threads per pair
// substituting, or with the factorisation ahead and eight threads per pair
// substituting (one per system, mode and component); and the step on one
// stream or in two kx halves on two streams: the ten combinations timed as
// whole steps on this handle's sizes, the fastest kept.  All ten perform the
// same operations in the same order (the results are bit-identical).  The field, the RK history and the
// module scalars are saved first and put back.
int tune_solve_and_halves(chgpu_handle* h) {
  const Dims& d = h->d;
  const size_t vbytes = sizeof(double2) * 3 * (size_t)d.nplanes * d.nmodes;
  const size_t obytes = tsize(h) * 2 * (size_t)(d.ny - 1) * d.nmodes;
  void *sv = nullptr, *so = nullptr, *ss = nullptr;
  if (cudaMalloc(&sv, vbytes) != cudaSuccess || cudaMalloc(&so, obytes) != cudaSuccess ||
      cudaMalloc(&ss, sizeof(DevScalars)) != cudaSuccess) {
    // no room for the saved state: keep the current choice
    cudaGetLastError();
    if (sv) cudaFree(sv);
    if (so) cudaFree(so);
    return 0;
  }
  CK(h, cudaMemcpyAsync(sv, h->V, vbytes, cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(so, h->old, obytes, cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(ss, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToDevice, h->stream));
  const bool prof = h->profiling;
  h->profiling = false;
  float best = 1e30f;
  int best_form = h->solve_form, best_halves = h->halves;
  cudaEvent_t a = take_event(h), b = take_event(h);
  int rc = 0;
  for (int c = 0; c < 10 && rc == 0; ++c) {
    h->solve_form = 1 + c % 5;
    h->halves = c >= 5 ? 2 : 1;
    enqueue_step(h);  // warm-up
    cudaEventRecord(a, h->stream);
    enqueue_step(h);
    cudaEventRecord(b, h->stream);
    cudaError_t e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e != cudaSuccess) {
      rc = cuda_fail(h, e, "chgpu_autotune: timing the solve forms");
      break;
    }
    if (ms < best) {
      best = ms;
      best_form = h->solve_form;
      best_halves = h->halves;
    }
  }
  h->ev_pool.push_back(a);
  h->ev_pool.push_back(b);
  h->solve_form = best_form;
  h->halves = best_halves;
  h->profiling = prof;
  cudaMemcpyAsync(h->V, sv, vbytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(h->old, so, obytes, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(h->sc, ss, sizeof(DevScalars), cudaMemcpyDeviceToDevice, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(sv);
  cudaFree(so);
  cudaFree(ss);
  if (rc == 0 && e != cudaSuccess) rc = cuda_fail(h, e, "chgpu_autotune: restoring the state");
  return rc;
}

}  // namespace

int chgpu_autotune(chgpu_handle* h) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  int dev = 0, optin = 0;
  CK(h, cudaGetDevice(&dev));
  CK(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t ts = tsize(h), lim = (size_t)optin - 1024;
  const int nzd = h->d.nzd, nxd = h->d.nxd;
  const int reps = 2;
  float ms = 0;
  // valid spectra in the work buffers before timing the later stages
  if (int rc = time_conv_stage(h, 0, 1, &ms)) return rc;
  if (int rc = time_conv_stage(h, 1, 1, &ms)) return rc;
  // columns per block of the two z-transform kernels, then their block size
  int best_z = h->zcols;
  float best = 1e30f;
  auto time_z = [&](float* t) -> int {
    float m0 = 0, m2 = 0;
    if (int rc = time_conv_stage(h, 0, reps, &m0)) return rc;
    if (int rc = time_conv_stage(h, 2, reps, &m2)) return rc;
    *t = m0 + m2;
    return 0;
  };
  // the register-blocked kernels have compile-time tiles; the generic
  // kernels' tiles are tuned where those run (switching between the two
  // would change the rounding of the step, so the tuner keeps the choice)
  if (!h->zfast) {
    h->zthreads = 256;
    for (int zc = 1; zc <= 8; zc *= 2) {
      if (conv_zinv_smem(zc, nzd, h->d.nzt, ts) > lim) break;
      h->zcols = zc;
      if (int rc = time_z(&ms)) return rc;
      if (ms < best) {
        best = ms;
        best_z = zc;
      }
  }
  h->zcols = best_z;
  int best_zt = 256;
  for (int zt : {128, 192}) {
    h->zthreads = zt;
    if (int rc = time_z(&ms)) return rc;
    if (ms < best) {
      best = ms;
      best_zt = zt;
    }
  }
  h->zthreads = best_zt;
  }
  // the register-blocked x-row kernel's register cap (3 or 4 resident blocks)
  if (h->xfast) {
    float best_v = 1e30f;
    int bv = h->xrvar;
    for (int v = 4; v <= 5; ++v) {
      h->xrvar = v;
      if (int rc = time_conv_stage(h, 1, reps, &ms)) return rc;
      if (ms < best_v) {
        best_v = ms;
        bv = v;
      }
    }
    h->xrvar = bv;
  }
  // rows per block and register-cap variant of the x-row kernel, then its block size
  if (!h->xfast) {
    int best_r = h->xrows, best_b = h->xminb;
    best = 1e30f;
    h->xthreads = 256;
    for (int xb = 1; xb <= 3; ++xb)
      for (int xr = 1; xr <= 4; xr *= 2) {
        if (nzd % xr != 0 || conv_x_smem(xr, nxd, ts) > lim) continue;
        h->xrows = xr;
        h->xminb = xb;
        if (int rc = time_conv_stage(h, 1, reps, &ms)) return rc;
        if (ms < best) {
          best = ms;
          best_r = xr;
          best_b = xb;
        }
      }
    h->xrows = best_r;
    h->xminb = best_b;
    int best_xt = 256;
    for (int xt : {128, 192}) {
      h->xthreads = xt;
      if (int rc = time_conv_stage(h, 1, reps, &ms)) return rc;
      if (ms < best) {
        best = ms;
        best_xt = xt;
      }
  }
  h->xthreads = best_xt;
  }
  if (int rc = tune_solve_and_halves(h)) return rc;
  h->tuned = true;
  ++h->version;
  if (h->graph) {  // the captured step holds the old launch shapes
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return 0;
}

int chgpu_set_tiles(chgpu_handle* h, const int tiles[CHGPU_NTILES]) {
  if (!h || !tiles) return fail(h, CHGPU_E_PARAM, "chgpu_set_tiles: null argument");
  int dev = 0, optin = 0;
  CK(h, cudaGetDevice(&dev));
  CK(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t ts = tsize(h), lim = (size_t)optin - 1024;
  const int zc = tiles[0], xr = tiles[1], xb = tiles[2], zt = tiles[3], xt = tiles[4], sf = tiles[5], hv = tiles[6];
  auto threads_ok = [](int t) { return t >= 64 && t <= 256 && t % 32 == 0; };
  int e_ = 0, tpr_ = 0;
  const bool zplan = rlen_plan(h->d.nzd, &e_, &tpr_), xplan = xlen_plan(h->d.nxd, &e_, &tpr_);
  if ((zc == 0 && !zplan) || (zc != 0 && (zc < 1 || zc > 8 || conv_zinv_smem(zc, h->d.nzd, h->d.nzt, ts) > lim)) ||
      (xr != 1 && xr != 2 && xr != 4) || h->d.nzd % xr != 0 || conv_x_smem(xr, h->d.nxd, ts) > lim ||
      (xb >= 4 && !xplan) || xb < 1 || xb > 5 || !threads_ok(zt) || !threads_ok(xt) || sf < 1 || sf > 5 ||
      (hv != 1 && hv != 2))
    return fail(h, CHGPU_E_PARAM, "chgpu_set_tiles: tiles outside what this handle's sizes allow");
  h->zfast = zc == 0;
  if (zc != 0) h->zcols = zc;
  h->xrows = xr;
  h->xfast = xb >= 4;
  if (xb >= 4) h->xrvar = xb;
  else h->xminb = xb;
  h->zthreads = zt;
  h->xthreads = xt;
  h->solve_form = sf;
  h->halves = hv;
  ++h->version;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return 0;
}

int chgpu_set_wait_limit(chgpu_handle* h, int polls) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  const int v = polls < 0 ? 0 : polls + 1;
  h->sc_host->first_wait = v;  // the host copy is uploaded whole by chgpu_start
  CK(h, cudaMemcpyAsync(&h->sc->first_wait, &v, sizeof v, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int chgpu_set_step_halves(chgpu_handle* h, int halves) {
  if (!h || (halves != 1 && halves != 2)) return fail(h, CHGPU_E_PARAM, "chgpu_set_step_halves: 1 or 2");
  if (h->halves != halves) {
    h->halves = halves;
    ++h->version;
    if (h->graph) {
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
  }
  return 0;
}

int chgpu_tiles(const chgpu_handle* h, int tiles[CHGPU_NTILES]) {
  if (!h || !tiles) return CHGPU_E_PARAM;
  tiles[0] = h->zfast ? 0 : h->zcols;
  tiles[1] = h->xrows;
  tiles[2] = h->xfast ? h->xrvar : h->xminb;
  tiles[3] = h->zthreads;
  tiles[4] = h->xthreads;
  tiles[5] = h->solve_form;
  tiles[6] = h->halves;
  return 0;
}

// ---------------------------------------------------------------------------
// physical-space export (out_exporter/out2bin.f90)
// ---------------------------------------------------------------------------
namespace {

int fortran_nint(float x) { return x >= 0.f ? (int)std::floor(x + 0.5f) : -(int)std::floor(-x + 0.5f); }

// out2bin.f90:76-78: nint(xcent_undersample * (2n+1)) with the product in real*4
int export_len(int n, float undersample) {
  volatile float prod = undersample * (float)(2 * n + 1);
  return fortran_nint(prod);
}

RadixDev prime_radices(int n) {
  RadixDev r{};
  r.n = n;
  int m = n;
  for (int p = 2; m > 1; ++p) {
    if ((long long)p * p > m) p = m;
    while (m % p == 0) {
      r.r[r.nst++] = p;
      m /= p;
    }
  }
  return r;
}

int export_setup(chgpu_handle* h) {
  if (h->ex_W) return 0;
  const int Nx = 2 * h->d.nx + 1, Nz = 2 * h->d.nz + 1;
  const int lim = export_set_smem_limits();
  if (lim <= 0) return fail(h, CHGPU_E_CUDA, "export: shared-memory limits");
  h->ex_zcols = 8;
  while (h->ex_zcols > 1 && export_z_smem(h->ex_zcols, Nz) > (size_t)lim) --h->ex_zcols;
  h->ex_xpairs = 4;
  while (h->ex_xpairs > 1 && export_x_smem(h->ex_xpairs, h->d.nx, Nx) > (size_t)lim) --h->ex_xpairs;
  if (export_z_smem(h->ex_zcols, Nz) > (size_t)lim || export_x_smem(h->ex_xpairs, h->d.nx, Nx) > (size_t)lim)
    return fail(h, CHGPU_E_PARAM, "export: 2nx+1 or 2nz+1 too long for one transform in shared memory");
  h->ex_rz = prime_radices(Nz);
  h->ex_rx = prime_radices(Nx);
  // planes per chunk: W and P of a chunk within 256 MiB
  const size_t per_plane = (size_t)3 * (h->d.nx + 1) * Nz * sizeof(double2) + (size_t)3 * Nz * Nx * sizeof(double);
  h->ex_chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)h->d.ny + 1, (1ull << 28) / per_plane));
  CK(h, cudaMalloc((void**)&h->ex_W, (size_t)3 * h->ex_chunk * (h->d.nx + 1) * Nz * sizeof(double2)));
  CK(h, cudaMalloc((void**)&h->ex_P, (size_t)3 * h->ex_chunk * Nz * Nx * sizeof(double)));
  const std::vector<double2> wz = roots<double2>(Nz), wx = roots<double2>(Nx);
  CK(h, cudaMalloc((void**)&h->ex_twz, sizeof(double2) * Nz));
  CK(h, cudaMalloc((void**)&h->ex_twx, sizeof(double2) * Nx));
  CK(h, cudaMemcpy(h->ex_twz, wz.data(), sizeof(double2) * Nz, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->ex_twx, wx.data(), sizeof(double2) * Nx, cudaMemcpyHostToDevice));
  return 0;
}

}  // namespace

int chgpu_export_dims(const chgpu_handle* h, float undersample, int dims[3]) {
  if (!h || !dims || !(undersample > 0.f)) return CHGPU_E_PARAM;
  dims[0] = export_len(h->d.nx, undersample);
  dims[1] = h->d.ny + 1;
  dims[2] = export_len(h->d.nz, undersample);
  return (dims[0] >= 1 && dims[2] >= 1) ? 0 : CHGPU_E_PARAM;
}

int chgpu_export_physical(chgpu_handle* h, const chgpu_export_opts* o, double* out) {
  if (!h || !out) return fail(h, CHGPU_E_PARAM, "chgpu_export_physical: null argument");
  chgpu_export_opts opt{0, CHGPU_EXPORT_ALL, 0, 1.0f};
  if (o) opt = *o;
  int dims[3];
  if (chgpu_export_dims(h, opt.undersample, dims) != 0)
    return fail(h, CHGPU_E_PARAM, "chgpu_export_physical: undersample factor gives an empty grid");
  if (opt.part < CHGPU_EXPORT_ALL || opt.part > CHGPU_EXPORT_SMALL)
    return fail(h, CHGPU_E_PARAM, "chgpu_export_physical: part must be CHGPU_EXPORT_ALL, _LARGE or _SMALL");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_export_physical: no field uploaded");
  if (int rc = export_setup(h)) return rc;
  const int nxtot = dims[0], nytot = dims[1], nztot = dims[2];
  const size_t need = (size_t)nztot * h->ex_chunk * nxtot * 3;
  if (need > h->ex_out_cap) {
    if (h->ex_out) CK(h, cudaFree(h->ex_out));
    h->ex_out = nullptr;
    h->ex_out_cap = 0;
    CK(h, cudaMalloc((void**)&h->ex_out, need * sizeof(double)));
    h->ex_out_cap = need;
  }
  ExportLaunch L{};
  L.V = h->V;
  L.d = h->d;
  L.W = h->ex_W;
  L.P = h->ex_P;
  L.out = h->ex_out;
  L.twz = h->ex_twz;
  L.twx = h->ex_twx;
  L.rz = h->ex_rz;
  L.rx = h->ex_rx;
  L.zcols = h->ex_zcols;
  L.xpairs = h->ex_xpairs;
  L.chunk = h->ex_chunk;
  L.nxtot = nxtot;
  L.nztot = nztot;
  L.fluct_only = opt.fluct_only ? 1 : 0;
  L.part = opt.part;
  L.z_threshold = opt.z_threshold;
  L.beta0 = h->p.beta0;
  const size_t row = (size_t)nxtot * 3 * sizeof(double);
  for (int iy0 = 0; iy0 < nytot; iy0 += h->ex_chunk) {
    const int nc = std::min(h->ex_chunk, nytot - iy0);
    launch_export_chunk(L, iy0, nc, h->stream);
    h->launches += 3;
    CK(h, cudaGetLastError());
    // [zz][iy][xx][c]: the chunk's planes are one strided block per zz
    CK(h, cudaMemcpy2DAsync(out + (size_t)iy0 * nxtot * 3, row * nytot, h->ex_out, row * nc, row * nc, nztot,
                            cudaMemcpyDeviceToHost, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int chgpu_set_body_force(chgpu_handle* h, const double* F) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  const bool was = h->use_F;
  if (!F) {
    h->use_F = false;
  } else {
    const size_t n = (size_t)3 * h->d.nplanes * h->d.nmodes;
    if (!h->F) CK(h, cudaMalloc((void**)&h->F, sizeof(double2) * n));
    double2* stage = reinterpret_cast<double2*>(h->Pb);
    CK(h, cudaMemcpyAsync(stage, F, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
    launch_transpose(stage, h->F, h->d.nmodes, h->d.nplanes, 3, h->stream);
    launch_force_ghosts(h->F, h->der, h->d, h->stream);
    h->launches += 2;
    CK(h, cudaGetLastError());
    CK(h, cudaStreamSynchronize(h->stream));
    h->use_F = true;
  }
  if (was != h->use_F) ++h->version;
  if (was != h->use_F && h->graph) {  // the captured step holds the old launch parameters
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return 0;
}

int chgpu_stats_reset(chgpu_handle* h) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  const size_t n = (size_t)4 * 3 * h->d.nplanes;
  if (!h->stats_acc) CK(h, cudaMalloc((void**)&h->stats_acc, sizeof(double) * n));
  CK(h, cudaMemsetAsync(h->stats_acc, 0, sizeof(double) * n, h->stream));
  h->stats_n = 0;
  return 0;
}

int chgpu_stats_accumulate(chgpu_handle* h) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  if (!h->stats_acc) {
    int rc = chgpu_stats_reset(h);
    if (rc) return rc;
  }
  launch_stats_accumulate(h->V, h->d, h->stats_acc, h->stream);
  h->launches += 1;
  CK(h, cudaGetLastError());
  h->stats_n += 1;
  return 0;
}

int chgpu_profiles(chgpu_handle* h, double* mean, double* var, long long* nsamples) {
  if (!h || !mean || !var) return fail(h, CHGPU_E_PARAM, "chgpu_profiles: null argument");
  if (!h->stats_acc || h->stats_n == 0) return fail(h, CHGPU_E_STATE, "chgpu_profiles: no samples accumulated");
  const size_t n = (size_t)3 * h->d.nplanes;
  std::vector<double> acc(4 * n);
  CK(h, cudaMemcpyAsync(acc.data(), h->stats_acc, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  const double N = (double)h->stats_n;
  for (size_t k = 0; k < n; ++k) {
    mean[k] = acc[k] / N;
    var[k] = acc[2 * n + k] / N - mean[k] * mean[k];
  }
  if (nsamples) *nsamples = h->stats_n;
  return 0;
}

// ---------------------------------------------------------------------------
// Reynolds-stress budget spectra (postpro/tke/uiuj_spectra.f90)
// ---------------------------------------------------------------------------
int chgpu_tke_reset(chgpu_handle* h, const double* mean) {
  if (!h || !mean) return fail(h, CHGPU_E_PARAM, "chgpu_tke_reset: null argument");
  const Dims& d = h->d;
  const int np = d.nplanes;
  const size_t FS = (size_t)np * d.nmodes, nxp = (size_t)d.nx + 1;
  if (!h->tke_ready) {
    int dev = 0, optin = 0;
    CK(h, cudaGetDevice(&dev));
    CK(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (tke_x_smem(d.nxd) > (size_t)optin || tke_z_smem(d.nzd) > (size_t)optin)
      return fail(h, CHGPU_E_PARAM, "chgpu_tke_reset: transform length too large for the budget kernels");
    // planes per chunk of the padded-grid work: the z-inverted fields of a chunk within ~2 GB
    const size_t per_plane = 12 * nxp * (size_t)d.nzd * sizeof(double2);
    h->tke_chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)np, ((size_t)2 << 30) / per_plane));
    const size_t C = (size_t)h->tke_chunk;
    CK(h, cudaMalloc((void**)&h->tke_W, sizeof(double2) * 12 * FS));
    CK(h, cudaMalloc((void**)&h->tke_N, sizeof(double2) * 3 * FS));
    CK(h, cudaMalloc((void**)&h->tke_P, sizeof(double2) * FS));
    CK(h, cudaMalloc((void**)&h->tke_Zt, sizeof(double2) * 12 * C * nxp * d.nzd));
    CK(h, cudaMalloc((void**)&h->tke_Xt, sizeof(double2) * 3 * C * nxp * d.nzd));
    CK(h, cudaMalloc((void**)&h->tke_acc, sizeof(double) * 36 * (size_t)np * d.nzt));
    CK(h, cudaMalloc((void**)&h->tke_mean, sizeof(double) * 5 * (size_t)np));
    Radix rz = make_radix(d.nzd, false), rx = make_radix(d.nxd, false);
    h->tke_rz.n = rz.n; h->tke_rz.nst = rz.nst; std::memcpy(h->tke_rz.r, rz.r, sizeof rz.r);
    h->tke_rx.n = rx.n; h->tke_rx.nst = rx.nst; std::memcpy(h->tke_rx.r, rx.r, sizeof rx.r);
    set_twiddle_offsets(h->tke_rz);
    set_twiddle_offsets(h->tke_rx);
    if (int rc = upload_stage_twiddles<double2>(h, &h->tke_twz, h->tke_rz)) return rc;
    if (int rc = upload_stage_twiddles<double2>(h, &h->tke_twx, h->tke_rx)) return rc;
    if (int rc = upload_pack_roots<double2>(h, &h->tke_twh, 2 * d.nxd, 0.5L * (long double)d.factor)) return rc;
    CK(h, tke_set_smem_limits(d.nzd, d.nxd));
    h->tke_ready = true;
  }
  // mean profiles and their y derivatives (uiuj_spectra.f90:152-155)
  std::vector<double>& m = h->tke_meanh;
  m.assign(7 * (size_t)np, 0.0);
  for (int q = 0; q < np; ++q) {
    m[q] = mean[q];
    m[(size_t)np + q] = mean[(size_t)np + q];
    m[6 * (size_t)np + q] = mean[2 * (size_t)np + q];
  }
  real_deriv(h->tab, &m[0], &m[2 * (size_t)np], 1);
  real_deriv(h->tab, &m[(size_t)np], &m[3 * (size_t)np], 1);
  real_deriv(h->tab, &m[0], &m[4 * (size_t)np], 2);
  real_deriv(h->tab, &m[(size_t)np], &m[5 * (size_t)np], 2);
  std::vector<double> dm(5 * (size_t)np);  // U, W, P, dU/dy, dW/dy
  for (int q = 0; q < np; ++q) {
    dm[q] = m[q];
    dm[(size_t)np + q] = m[(size_t)np + q];
    dm[2 * (size_t)np + q] = m[6 * (size_t)np + q];
    dm[3 * (size_t)np + q] = m[2 * (size_t)np + q];
    dm[4 * (size_t)np + q] = m[3 * (size_t)np + q];
  }
  CK(h, cudaMemcpyAsync(h->tke_mean, dm.data(), sizeof(double) * dm.size(), cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemsetAsync(h->tke_acc, 0, sizeof(double) * 36 * (size_t)np * d.nzt, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->tke_n = 0;
  h->tke_pressure = false;
  return 0;
}

int chgpu_tke_accumulate(chgpu_handle* h, const double* pressure) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  if (!h->tke_ready) return fail(h, CHGPU_E_STATE, "chgpu_tke_accumulate: chgpu_tke_reset first");
  if (h->tke_n > 0 && (pressure != nullptr) != h->tke_pressure)
    return fail(h, CHGPU_E_PARAM, "chgpu_tke_accumulate: give a pressure field with every sample or with none");
  const Dims& d = h->d;
  const size_t FS = (size_t)d.nplanes * d.nmodes;
  if (pressure) {
    // restart-file layout (iy fastest) to the plane-major layout, through the x work buffer
    double2* stage = reinterpret_cast<double2*>(h->Pb);
    CK(h, cudaMemcpyAsync(stage, pressure, sizeof(double2) * FS, cudaMemcpyHostToDevice, h->stream));
    launch_transpose(stage, h->tke_P, d.nmodes, d.nplanes, 1, h->stream);
  }
  TkeLaunch L{};
  L.d = d;
  L.bc = h->bc;
  L.V = h->V;
  L.W = h->tke_W;
  L.N3 = h->tke_N;
  L.P = pressure ? h->tke_P : nullptr;
  L.Zt = h->tke_Zt;
  L.Xt = h->tke_Xt;
  L.acc = h->tke_acc;
  L.mean = h->tke_mean;
  L.der = h->der;
  L.d0lu = h->d0lu;
  L.twz = (const double2*)h->tke_twz;
  L.twx = (const double2*)h->tke_twx;
  L.twh = (const double2*)h->tke_twh;
  L.rz = h->tke_rz;
  L.rx = h->tke_rx;
  L.chunk = h->tke_chunk;
  launch_tke_snapshot(L, h->stream);
  CK(h, cudaGetLastError());
  const int nchunks = (d.nplanes + h->tke_chunk - 1) / h->tke_chunk;
  h->launches += 3 + (pressure ? 2 : 0) + 3 * nchunks;
  h->tke_pressure = pressure != nullptr;
  h->tke_n += 1;
  return 0;
}

int chgpu_tke_result(chgpu_handle* h, int timestwo, double* mean7, double* spectra, double* profiles,
                     long long* nsamples) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  if (!h->tke_ready || h->tke_n == 0) return fail(h, CHGPU_E_STATE, "chgpu_tke_result: no samples accumulated");
  const Dims& d = h->d;
  const int np = d.nplanes, nzt = d.nzt;
  const size_t S = (size_t)np * nzt;
  std::vector<double> acc(36 * S);
  CK(h, cudaMemcpyAsync(acc.data(), h->tke_acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  const double N = (double)h->tke_n;
  // spectra(irs, term, iz, iy) in the reference's order (irs fastest); the
  // accumulated terms var, prod, psdiss, ttrsp, pstrain, PHIptrsp sit at
  // term 0, 1, 2, 3, 5, 9 (uiuj_spectra.f90:13-14, :70)
  static const int kAccTerm[6] = {0, 1, 2, 3, 5, 9};
  std::vector<double> sp((size_t)60 * S, 0.0);
  auto SP = [&](int irs, int term, int izp, int plane) -> double& {
    return sp[(size_t)irs + 6 * ((size_t)term + 10 * ((size_t)izp + (size_t)nzt * plane))];
  };
  for (int q = 0; q < 6; ++q)
    for (int irs = 0; irs < 6; ++irs)
      for (int plane = 0; plane < np; ++plane)
        for (int izp = 0; izp < nzt; ++izp)
          SP(irs, kAccTerm[q], izp, plane) = acc[(size_t)(q * 6 + irs) * S + (size_t)plane * nzt + izp] / N;
  // flux derivatives (:243-259): PHIvdiff = ni d/dy var, vdiff = ni d2/dy2 var, ptrsp = d/dy PHIptrsp
  std::vector<double> f0(np), f1(np);
  for (int izp = 0; izp < nzt; ++izp)
    for (int irs = 0; irs < 6; ++irs) {
      for (int q = 0; q < np; ++q) f0[q] = SP(irs, 0, izp, q);
      real_deriv(h->tab, f0.data(), f1.data(), 1);
      for (int q = 0; q < np; ++q) SP(irs, 8, izp, q) = f1[q] * d.ni;
      real_deriv(h->tab, f0.data(), f1.data(), 2);
      for (int q = 0; q < np; ++q) SP(irs, 4, izp, q) = f1[q] * d.ni;
      for (int q = 0; q < np; ++q) f0[q] = SP(irs, 9, izp, q);
      real_deriv(h->tab, f0.data(), f1.data(), 1);
      for (int q = 0; q < np; ++q) SP(irs, 6, izp, q) = f1[q];
    }
  if (timestwo)  // -two (:262)
    for (int plane = 0; plane < np; ++plane)
      for (int izp = 0; izp < nzt; ++izp)
        for (int irs = 0; irs < 6; ++irs) SP(irs, 0, izp, plane) *= 2.0;
  if (spectra) std::memcpy(spectra, sp.data(), sizeof(double) * sp.size());
  if (profiles)
    for (int plane = 0; plane < np; ++plane)
      for (int term = 0; term < 10; ++term)
        for (int irs = 0; irs < 6; ++irs) {
          double s = 0.0;
          for (int izp = 0; izp < nzt; ++izp) s += SP(irs, term, izp, plane);
          profiles[(size_t)irs + 6 * ((size_t)term + 10 * (size_t)plane)] = s;
        }
  if (mean7)
    for (int plane = 0; plane < np; ++plane)
      for (int q = 0; q < 7; ++q) mean7[(size_t)q + 7 * (size_t)plane] = h->tke_meanh[(size_t)q * np + plane];
  if (nsamples) *nsamples = h->tke_n;
  return 0;
}

int chgpu_snapshot_async(chgpu_handle* h) {
  if (!h) return fail(h, CHGPU_E_PARAM, "null handle");
  if (h->snap_pending) return fail(h, CHGPU_E_STATE, "chgpu_snapshot_async: previous snapshot not collected");
  const size_t n = (size_t)3 * h->d.nplanes * h->d.nmodes;
  if (!h->snap_stage) {
    CK(h, cudaMalloc((void**)&h->snap_stage, sizeof(double2) * n));
    CK(h, cudaMallocHost((void**)&h->snap_host, sizeof(double2) * n));
    CK(h, cudaStreamCreateWithFlags(&h->snap_stream, cudaStreamNonBlocking));
    CK(h, cudaEventCreateWithFlags(&h->snap_read, cudaEventDisableTiming));
    CK(h, cudaEventCreateWithFlags(&h->snap_done, cudaEventDisableTiming));
  }
  // the transpose reads V in stream order; later steps wait only for it, the
  // device-to-host copy runs on the side stream while they compute
  launch_transpose(h->V, h->snap_stage, h->d.nplanes, h->d.nmodes, 3, h->stream);
  h->launches += 1;
  CK(h, cudaGetLastError());
  CK(h, cudaEventRecord(h->snap_read, h->stream));
  CK(h, cudaStreamWaitEvent(h->snap_stream, h->snap_read, 0));
  CK(h, cudaMemcpyAsync(h->snap_host, h->snap_stage, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->snap_stream));
  CK(h, cudaEventRecord(h->snap_done, h->snap_stream));
  h->snap_pending = true;
  return 0;
}

int chgpu_snapshot_wait(chgpu_handle* h, const double** V) {
  if (!h || !V) return fail(h, CHGPU_E_PARAM, "chgpu_snapshot_wait: null argument");
  if (!h->snap_pending) return fail(h, CHGPU_E_STATE, "chgpu_snapshot_wait: no snapshot in flight");
  CK(h, cudaEventSynchronize(h->snap_done));
  h->snap_pending = false;
  *V = h->snap_host;
  return 0;
}

void* chgpu_stream(chgpu_handle* h) { return h ? (void*)h->stream : nullptr; }

long long chgpu_launch_count(const chgpu_handle* h) { return h ? h->launches : 0; }

// ---------------------------------------------------------------------------
// learned closure (include/chgpu_closure.h)
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

long long closure_plane_pts(const chgpu_handle* h) { return (long long)h->d.nzd * 2 * h->d.nxd; }

void drop_graph(chgpu_handle* h) {  // the captured step holds the old launch sequence
  if (h->graph) {
    cudaStreamSynchronize(h->stream);
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  ++h->version;
}

void closure_free(chgpu_handle* h) {
  void** bufs[] = {(void**)&h->cl_G, (void**)&h->cl_Z, (void**)&h->cl_P, (void**)&h->cl_tau, (void**)&h->cl_wd,
                   &h->cl_twz, &h->cl_twx, &h->cl_twh};
  for (void** b : bufs) {
    if (*b) cudaFree(*b);
    *b = nullptr;
  }
}

int closure_alloc_all(chgpu_handle* h);

// buffers and FP32 tables of the closure, on first use; all or nothing
int closure_alloc(chgpu_handle* h) {
  if (h->cl_twh) return 0;  // the last one made
  const int rc = closure_alloc_all(h);
  if (rc) closure_free(h);
  return rc;
}

int closure_alloc_all(chgpu_handle* h) {
  const Dims& d = h->d;
  const size_t np = d.nplanes, nm = d.nmodes, nxp = d.nx + 1;
  const size_t phys = (size_t)9 * np * d.nzd * d.nxd * sizeof(float2);
  // cl_P also stages host spectra (up to 9 fields, complex128) for chgpu_closure_physical
  const size_t stage = (size_t)9 * np * nm * sizeof(double2);
  int dev = 0;
  CK(h, cudaGetDevice(&dev));
  CK(h, cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, dev));
  if (mlp_set_smem_limits() != 0) return fail(h, CHGPU_E_CUDA, "closure: shared-memory limit refused");
  auto alloc = [&](void** ptr, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(ptr, bytes);
    return e == cudaSuccess ? 0 : fail(h, CHGPU_E_NOMEM, "closure: device allocation failed");
  };
  if (int rc = alloc((void**)&h->cl_G, (size_t)9 * np * nm * sizeof(double2))) return rc;
  if (int rc = alloc((void**)&h->cl_Z, (size_t)9 * np * nxp * d.nzd * sizeof(float2))) return rc;
  if (int rc = alloc((void**)&h->cl_P, std::max(phys, stage))) return rc;
  if (int rc = alloc((void**)&h->cl_tau, (size_t)6 * np * d.nzd * d.nxd * sizeof(float2))) return rc;
  if (int rc = alloc((void**)&h->cl_wd, np * sizeof(float))) return rc;
  CK(h, cudaMemset(h->cl_tau, 0, (size_t)6 * np * d.nzd * d.nxd * sizeof(float2)));
  std::vector<float> wd(np);
  for (size_t k = 0; k < np; ++k) {
    const double y = h->tab.y[k];
    wd[k] = (float)std::min(y - h->p.ymin, h->p.ymax - y);
  }
  CK(h, cudaMemcpy(h->cl_wd, wd.data(), np * sizeof(float), cudaMemcpyHostToDevice));
  if (int rc = upload_stage_twiddles<float2>(h, &h->cl_twz, h->rz)) return rc;
  if (int rc = upload_stage_twiddles<float2>(h, &h->cl_twx, h->rx)) return rc;
  return upload_pack_roots<float2>(h, &h->cl_twh, 2 * d.nxd, 1.0L);
}

// interior planes (iy = 1..ny-1) of ncomp physical fields in cl_P -> out[ncomp][npts]
int copy_closure_points(chgpu_handle* h, int ncomp, float* out) {
  const long long pp = closure_plane_pts(h), n = (long long)(h->d.ny - 1) * pp;
  const float* P = reinterpret_cast<const float*>(h->cl_P);
  for (int c = 0; c < ncomp; ++c)
    CK(h, cudaMemcpyAsync(out + (size_t)c * n, P + ((size_t)c * h->d.nplanes + 2) * pp, sizeof(float) * n,
                          cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

template <typename V2>
__global__ void k_to_double2(const V2* __restrict__ in, double2* __restrict__ out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

}  // namespace

extern "C" {

int chgpu_closure_dims(chgpu_handle* h, int dims[3]) {
  if (!h || !dims) return fail(h, CHGPU_E_PARAM, "chgpu_closure_dims: null argument");
  dims[0] = 2 * h->d.nxd;
  dims[1] = h->d.nzd;
  dims[2] = h->d.ny - 1;
  return 0;
}

int chgpu_closure_attach(chgpu_handle* h, chgpu_mlp* m, int enable) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_closure_attach: null handle");
  if (enable && !m) return fail(h, CHGPU_E_PARAM, "chgpu_closure_attach: enable needs a network");
  if (int rc = closure_alloc(h)) return rc;
  h->cl_mlp = m;
  const bool on = enable && m;
  if (on != h->cl_on) {
    h->cl_on = on;
    drop_graph(h);
  }
  return 0;
}

int chgpu_closure_set_tau(chgpu_handle* h, const float* tau) {
  if (!h) return fail(h, CHGPU_E_PARAM, "chgpu_closure_set_tau: null handle");
  if (int rc = closure_alloc(h)) return rc;
  const long long pp = closure_plane_pts(h), n = (long long)(h->d.ny - 1) * pp;
  float* T = reinterpret_cast<float*>(h->cl_tau);
  CK(h, cudaStreamSynchronize(h->stream));
  CK(h, cudaMemset(T, 0, sizeof(float) * 6 * h->d.nplanes * pp));
  if (tau)
    for (int o = 0; o < 6; ++o)
      CK(h, cudaMemcpy(T + ((size_t)o * h->d.nplanes + 2) * pp, tau + (size_t)o * n, sizeof(float) * n,
                       cudaMemcpyHostToDevice));
  const bool fixed = tau != nullptr;
  if (fixed != h->cl_fixed) {
    h->cl_fixed = fixed;
    drop_graph(h);
  }
  return 0;
}

int chgpu_closure_features(chgpu_handle* h, float* feat) {
  if (!h || !feat) return fail(h, CHGPU_E_PARAM, "chgpu_closure_features: null argument");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_closure_features: upload the field first");
  if (int rc = closure_alloc(h)) return rc;
  const Dims& d = h->d;
  launch_gradients(h->V, h->cl_G, h->der, h->d0lu, h->bc, d, h->stream);
  launch_physical_fields(h->cl_G, 9, h->cl_Z, h->cl_P, (const float2*)h->cl_twz, (const float2*)h->cl_twx,
                         (const float2*)h->cl_twh, d, h->rz, h->rx, h->zcols, h->xrows, h->sc, h->stream);
  h->launches += 4;
  CK(h, cudaGetLastError());
  if (int rc = copy_closure_points(h, 9, feat)) return rc;
  if (int rc = pull_scalars(h)) return rc;
  const long long pp = closure_plane_pts(h), n = (long long)(d.ny - 1) * pp;
  float* w = feat + (size_t)9 * n;
  for (int iy = 1; iy <= d.ny - 1; ++iy) {
    const double y = h->tab.y[iy + 1];
    const float v = (float)std::min(y - h->p.ymin, h->p.ymax - y);
    std::fill(w + (size_t)(iy - 1) * pp, w + (size_t)iy * pp, v);
  }
  return 0;
}

int chgpu_closure_physical(chgpu_handle* h, const double* spec, int ncomp, float* out) {
  if (!h || !spec || !out) return fail(h, CHGPU_E_PARAM, "chgpu_closure_physical: null argument");
  if (ncomp != 3 && ncomp != 6 && ncomp != 9) return fail(h, CHGPU_E_PARAM, "chgpu_closure_physical: ncomp must be 3, 6 or 9");
  if (int rc = closure_alloc(h)) return rc;
  const Dims& d = h->d;
  const size_t n = (size_t)ncomp * d.nplanes * d.nmodes;
  double2* stage = reinterpret_cast<double2*>(h->cl_P);
  CK(h, cudaMemcpyAsync(stage, spec, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
  launch_transpose(stage, h->cl_G, d.nmodes, d.nplanes, ncomp, h->stream);
  launch_physical_fields(h->cl_G, ncomp, h->cl_Z, h->cl_P, (const float2*)h->cl_twz, (const float2*)h->cl_twx,
                         (const float2*)h->cl_twh, d, h->rz, h->rx, h->zcols, h->xrows, h->sc, h->stream);
  h->launches += 3;
  CK(h, cudaGetLastError());
  if (int rc = copy_closure_points(h, ncomp, out)) return rc;
  return pull_scalars(h);
}

int chgpu_products(chgpu_handle* h, double* out) {
  if (!h || !out) return fail(h, CHGPU_E_PARAM, "chgpu_products: null argument");
  if (!h->field_set) return fail(h, CHGPU_E_STATE, "chgpu_products: upload the field first");
  if (int rc = closure_alloc(h)) return rc;
  const Dims& d = h->d;
  const bool on = h->cl_on, fixed = h->cl_fixed;
  h->cl_on = h->cl_fixed = false;  // the resolved products alone
  run_convolutions(h, 0, 1, 0, d.nplanes);
  h->cl_on = on;
  h->cl_fixed = fixed;
  const size_t n = (size_t)6 * d.nplanes * d.nmodes;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (h->prec == CHGPU_MIXED) k_to_double2<float2><<<blocks, 256, 0, h->stream>>>((const float2*)h->VV, h->cl_G, n);
  else if (h->prec == CHGPU_FP64DD)
    k_to_double2<cdd><<<blocks, 256, 0, h->stream>>>((const cdd*)h->VV, h->cl_G, n);
  else CK(h, cudaMemcpyAsync(h->cl_G, h->VV, sizeof(double2) * n, cudaMemcpyDeviceToDevice, h->stream));
  double2* stage = reinterpret_cast<double2*>(h->cl_P);
  launch_transpose(h->cl_G, stage, d.nplanes, d.nmodes, 6, h->stream);
  h->launches += 2;
  CK(h, cudaGetLastError());
  CK(h, cudaMemcpyAsync(out, stage, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return pull_scalars(h);
}

}  // extern "C"
