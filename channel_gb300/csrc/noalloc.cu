// chgpu_linsolve_noalloc: the implicit solve of one RK substep for callers
// that cannot allocate device memory.
//
// Some hosts of this solver own every byte of device memory themselves: a
// code that runs inside a fixed memory arena handed out by its framework, a
// driver that reserved the GPU's memory at start-up, or a caller that must
// not trigger an allocation between launches.  They cannot let a library call
// cudaMalloc.  This entry point runs the fused solve kernel of
// chgpu_linsolve on the caller's field buffer, and keeps everything else it
// needs -- the pentadiagonal factors (the kernel's scratch), the
// wall-normal tables and the mean-flow scalars -- in the file-scope device
// arrays below.  Those arrays belong to the library image: every GPU that
// loads the library holds them (64 MiB of factor scratch, CHGPU_NOALLOC_
// SCRATCH_BYTES, plus 0.2 MiB of tables) until the process exits.
//
// All calls share the arrays: calls that overlap on the GPU (different
// streams, threads or devices sharing a context) race on them.  Each call
// rewrites every word of the arrays it later reads (tables, scalars, and each
// factor row before the substitution that reads it), so nothing from a
// previous call leaks into the next and nothing needs clearing.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/chgpu.h"
#include "chgpu_internal.h"
#include "kernels.cuh"

namespace {

using chgpu::StaticTables;

constexpr size_t kFactorDoubles = CHGPU_NOALLOC_SCRATCH_BYTES / sizeof(double);
constexpr size_t kDerDoubles = (size_t)(StaticTables::kMaxNy + 1) * 20;
constexpr size_t kD0Doubles = (size_t)(StaticTables::kMaxNy + 1) * 5;
constexpr size_t kYintDoubles = 3 * (size_t)(StaticTables::kMaxNy / 2 + 1);
constexpr size_t kTableDoubles = kDerDoubles + kD0Doubles + kYintDoubles;

// the kernel's scratch: lower factors of the v and eta matrices, [row][4][pair]
static __device__ __align__(256) double g_noalloc_factors[kFactorDoubles];
// der (20 per row), the factored D0mat (5 per row), Simpson weights
static __device__ __align__(256) double g_noalloc_tables[kTableDoubles];
static __device__ __align__(256) chgpu::DevScalars g_noalloc_scalars;

struct DeviceAddresses {
  double* factors = nullptr;
  double* tables = nullptr;
  chgpu::DevScalars* scalars = nullptr;
};
std::mutex g_mutex;         // guards the host staging below
StaticTables g_host_tables;  // host staging of the tables (no heap)
double g_host_pack[kTableDoubles];
thread_local char* g_err = nullptr;  // the caller's message buffer, if any
thread_local size_t g_errlen = 0;

int error(int code, const char* msg) {
  if (g_err && g_errlen) std::snprintf(g_err, g_errlen, "%s", msg);
  return code;
}

int cuda_error(cudaError_t e, const char* where) {
  if (g_err && g_errlen) std::snprintf(g_err, g_errlen, "%s: %s", where, cudaGetErrorString(e));
  return CHGPU_E_CUDA;
}

// Host code cannot use the arrays' names as device addresses: they are
// resolved with the caller's device current, on every call (a lookup, no
// allocation), so that a context torn down and created again -- where the
// module, and with it the arrays, may be loaded at other addresses -- is
// never handed stale pointers.
int resolve_addresses(DeviceAddresses* a) {
  cudaError_t e = cudaGetSymbolAddress((void**)&a->factors, g_noalloc_factors);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(factors)");
  e = cudaGetSymbolAddress((void**)&a->tables, g_noalloc_tables);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(tables)");
  e = cudaGetSymbolAddress((void**)&a->scalars, g_noalloc_scalars);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scalars)");
  return 0;
}

}  // namespace

extern "C" int chgpu_linsolve_noalloc(const chgpu_params* p, double lambda, double* field, double* scalars,
                                      void* stream, char* err, size_t errlen) {
  g_err = err;
  g_errlen = errlen;
  if (err && errlen) err[0] = '\0';
  if (!p || !field || !scalars) return error(CHGPU_E_PARAM, "chgpu_linsolve_noalloc: null argument");
  if (p->nx < 1 || p->nz < 1 || p->ny < 8 || p->ny > StaticTables::kMaxNy)
    return error(CHGPU_E_PARAM, "chgpu_linsolve_noalloc: need nx>=1, nz>=1, 8<=ny<=1024");
  const size_t npairs = (size_t)(p->nx + 1) * (p->nz + 1);
  const size_t need = chgpu::kFacPerRowFused * (size_t)(p->ny - 1) * npairs;
  if (need > kFactorDoubles) {
    if (err && errlen)
      std::snprintf(err, errlen,
                    "chgpu_linsolve_noalloc: 4*(ny-1)*(nx+1)*(nz+1) = %zu factor doubles exceed the %zu-byte static "
                    "scratch (CHGPU_NOALLOC_SCRATCH_BYTES)",
                    need, (size_t)CHGPU_NOALLOC_SCRATCH_BYTES);
    return CHGPU_E_PARAM;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceAddresses addr;
  DeviceAddresses* a = &addr;
  int rc = resolve_addresses(a);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  StaticTables& t = g_host_tables;
  if (!chgpu::compute_tables_static(*p, t)) return error(CHGPU_E_PARAM, "chgpu_linsolve_noalloc: bad ny");
  const int ny = p->ny;
  // pack der | D0 factors | Simpson weights at fixed offsets
  std::memcpy(g_host_pack, t.der, sizeof(double) * (size_t)(ny + 1) * 20);
  std::memcpy(g_host_pack + kDerDoubles, t.d0lu, sizeof(double) * (size_t)(ny + 1) * 5);
  std::memcpy(g_host_pack + kDerDoubles + kD0Doubles, t.yint, sizeof(double) * 3 * (size_t)t.nyint);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  e = cudaMemcpyAsync(a->tables, g_host_pack, sizeof(double) * kTableDoubles, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "copy tables");
  chgpu::DevScalars sc{};
  sc.u0 = p->u0;
  sc.uN = p->uN;
  sc.corrpx = scalars[3];
  sc.corrpz = scalars[4];
  sc.meanpx = scalars[5];
  sc.meanpz = scalars[6];
  e = cudaMemcpyAsync(a->scalars, &sc, sizeof sc, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_error(e, "copy scalars");

  chgpu::SolveLaunch L{};
  chgpu::Dims& d = L.d;
  int nxd = 0, nzd = 0;
  chgpu::padded_sizes(p->nx, p->nz, &nxd, &nzd);
  d.nx = p->nx; d.ny = ny; d.nz = p->nz;
  d.nzt = 2 * p->nz + 1;
  d.nxd = nxd; d.nzd = nzd;
  d.nplanes = ny + 3;
  d.nmodes = (p->nx + 1) * d.nzt;
  d.npairs = (int)npairs;
  d.alfa0 = p->alfa0; d.beta0 = p->beta0; d.ni = p->ni;
  d.meanflowx = p->meanflowx; d.meanflowz = p->meanflowz;
  d.cflmax = p->cflmax; d.gamma = p->gamma;
  d.cpi = p->cpi; d.cpi_type = p->cpi_type;
  L.q_lo = 0;
  L.q_hi = (int)npairs;
  L.m_lo = 0;
  L.m_hi = d.nmodes;
  std::memcpy(L.bc.v0bc, t.v0bc, 40); std::memcpy(L.bc.v0m1bc, t.v0m1bc, 40);
  std::memcpy(L.bc.eta0bc, t.eta0bc, 40); std::memcpy(L.bc.eta0m1bc, t.eta0m1bc, 40);
  std::memcpy(L.bc.vnbc, t.vnbc, 40); std::memcpy(L.bc.vnp1bc, t.vnp1bc, 40);
  std::memcpy(L.bc.etanbc, t.etanbc, 40); std::memcpy(L.bc.etanp1bc, t.etanp1bc, 40);
  std::memcpy(L.bc.d140, t.d140, 40); std::memcpy(L.bc.d14m1, t.d14m1, 40);
  std::memcpy(L.bc.d14n, t.d14n, 40); std::memcpy(L.bc.d14np1, t.d14np1, 40);
  L.V = reinterpret_cast<double2*>(field);
  L.rhs_src = L.V;  // right-hand sides in place, as buildrhs leaves them
  L.rhs_cstride = (size_t)d.nplanes * d.nmodes;
  L.rhs_plane_off = 1;
  L.fac = a->factors;
  L.der = a->tables;
  L.d0lu = a->tables + kDerDoubles;
  L.yint = a->tables + kDerDoubles + kD0Doubles;
  L.sc = a->scalars;
  L.lambda = lambda;
  L.lambda_from_dt = 0;
  chgpu::launch_linsolve(L, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "k_linsolve launch");
  e = cudaMemcpyAsync(&sc, a->scalars, sizeof sc, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_error(e, "read scalars");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_error(e, "k_linsolve");
  scalars[0] = sc.fr[0];
  scalars[1] = sc.fr[1];
  scalars[2] = sc.fr[2];
  scalars[3] = sc.corrpx;
  scalars[4] = sc.corrpz;
  scalars[5] = sc.meanpx;
  scalars[6] = sc.meanpz;
  return 0;
}
