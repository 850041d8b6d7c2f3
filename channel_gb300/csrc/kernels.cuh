// Launch descriptors shared by the kernel files and the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include "chgpu_internal.h"
#include "cplx.cuh"

namespace chgpu {

// Sizes and physics constants passed by value to every kernel.
struct Dims {
  int nx, ny, nz, nzt, nxd, nzd;
  int nplanes;  // ny+3 (iy=-1..ny+1 -> plane iy+1)
  int nmodes;   // (nx+1)(2nz+1): mode m = ix*(2nz+1) + iz+nz
  int npairs;   // (nx+1)(nz+1): pair (ix, |iz|)
  double alfa0, beta0, ni, factor, rdx, rdz;
  double meanflowx, meanflowz, cflmax, gamma;
  int cpi, cpi_type;
};

// Boundary rows of setup_boundary_conditions and the one-sided wall
// stencils (dnsdata.f90:259-308), by value.
struct BcRows {
  double v0bc[5], v0m1bc[5], eta0bc[5], eta0m1bc[5];
  double vnbc[5], vnp1bc[5], etanbc[5], etanp1bc[5];
  double d140[5], d14m1[5], d14n[5], d14np1[5];
};

struct ConvLaunch {
  Dims d;
  RadixDev rz, rx;
  const double2* V;
  void* Zb;
  void* Pb;
  void* VV;
  const void* twz;
  const void* twx;
  const void* twh;
  const double* dy;
  const void* cst;  // in the transform type: factor, 1/dx, 1/dz, then 1/dy(iy) at [3 + plane]
  DevScalars* sc;
  int zcols, xrows;
  int xminb;  // register-cap variant of the x-row kernel (1, 2 or 3 blocks per SM)
  int zthreads, xthreads;  // threads per block of the z-transform and x-row kernels (<= 256)
  int ix_lo, ix_hi;        // kx columns of the z-inverse pass (all: 0, nx+1)
  int plane0, nplanes;
  int compute_cfl;
  int products;  // 0: stop after the x pass (the start-up CFL pass)
  const float2* tau;  // closure stresses added to the products, or null
  // register-blocked kernels (convf.cu) for the lengths with a compile-time
  // plan: their twiddle tables, and whether they run the z / x stages
  const void* twzr;
  const void* twxr;
  int zfast, xfast;
};

// stage 0: z-inverse, 1: x rows, 2: z-forward
template <typename T> void launch_convolutions(const ConvLaunch& L, cudaStream_t s, int stage);
cudaError_t conv_set_smem_limits();
// the register-blocked stage kernels; false when the stage's length has no plan
template <typename T> bool launch_convolutions_r(const ConvLaunch& L, cudaStream_t s, int stage);
template <typename T> cudaError_t convr_set_smem_limits();
// defined in convf_f32.cu, convf_f64.cu, convf_dd.cu
template <> bool launch_convolutions_r<float>(const ConvLaunch& L, cudaStream_t s, int stage);
template <> bool launch_convolutions_r<double>(const ConvLaunch& L, cudaStream_t s, int stage);
template <> bool launch_convolutions_r<dd>(const ConvLaunch& L, cudaStream_t s, int stage);
template <> cudaError_t convr_set_smem_limits<float>();
template <> cudaError_t convr_set_smem_limits<double>();
template <> cudaError_t convr_set_smem_limits<dd>();
// dynamic shared memory of the z-transform and x-row kernels (padded buffers)
size_t conv_z_smem(int zcols, int nzd, size_t ts);                     // z-forward
size_t conv_zinv_smem(int zcols, int nzd, int nzt, size_t ts);         // z-inverse (raw field copy)
size_t conv_x_smem(int xrows, int nxd, size_t ts);
void launch_physical_fields(const double2* src, int ncomp, float2* zb, float2* out, const float2* twz,
                            const float2* twx, const float2* twh, const Dims& d, const RadixDev& rz,
                            const RadixDev& rx, int zcols, int xrows, DevScalars* sc, cudaStream_t s);
// the closure's velocity gradients: G[3c + {0,1,2}] = d/dx, d/dy, d/dz of V[c]
void launch_gradients(const double2* V, double2* G, const double* der, const double* d0lu, const BcRows& bc,
                      const Dims& d, cudaStream_t s);

// factor doubles per y row and (kx, +-kz) pair: the fused solve keeps l2, l1
// of the v and eta matrices; the split solve (k_factor + k_solve) l2, l1,
// 1/d, u1, u2 of both
constexpr int kFacPerRowFused = 4, kFacPerRow = 10;

struct SolveLaunch {
  Dims d;
  BcRows bc;
  double2* V;
  const void* VV;
  void* old;
  double2* rhs;
  const double2* F;        // body force (plane-major like V) or null
  const double2* rhs_src;  // where k_linsolve reads its right-hand sides
  size_t rhs_cstride;      // component stride of rhs_src
  int rhs_plane_off;       // row iy lives at plane iy+rhs_plane_off
  double* fac;
  const double* der;
  const void* derT;  // der in the nonlinear-term type, then alfa0, beta0
  const void* derL;  // der in the linear-term type, then alfa0, beta0, ni
  const double* d0lu;
  const double* yint;
  DevScalars* sc;
  double ode[3];
  double lambda;  // used when lambda_from_dt == 0
  int lambda_from_dt;
  const void* lindd;  // double-float d1 row, D0mat factors, d0 row per y row: v' and u, w in
                      // double-float; null: FP64
  const double* nud;  // per y row: -ni d4 (5), -ni d2 (5); null: formed in the kernel
  int m_lo, m_hi;     // modes of k_rhs (all: 0, nmodes); a range of whole kx columns
  int q_lo, q_hi;     // (kx, +-kz) pairs of k_linsolve (all: 0, npairs)
  int split_solve;    // 0: the fused k_linsolve; 1: k_factor then k_solve (fac holds kFacPerRow per row);
                      // 2: k_factor then k_linsolve reading the factors (two threads per pair);
                      // 3: k_factor then k_solve_ri (eight threads per pair)
  int factored;       // split form: fac already holds this substep's factors (k_factor ran ahead), k_solve only
};

template <typename T> void launch_rhs(const SolveLaunch& L, cudaStream_t s);
void launch_linsolve(const SolveLaunch& L, cudaStream_t s);
void launch_factor(const SolveLaunch& L, cudaStream_t s);  // k_factor alone, pairs q_lo..q_hi
void launch_advance_time(DevScalars* sc, double coef, int new_step, cudaStream_t s);
void launch_outstats(const SolveLaunch& L, cudaStream_t s);
void launch_flowrate(const SolveLaunch& L, cudaStream_t s);
void launch_transpose(const double2* in, double2* out, int rows, int cols, int batch, cudaStream_t s);
// physical-space export (export.cu)
struct ExportLaunch {
  const double2* V;
  Dims d;
  double2* W;    // z-transformed planes of a chunk: [3][chunk][nx+1][Nz]
  double* P;     // physical planes of a chunk: [3][chunk][Nz][Nx]
  double* out;   // sampled output of a chunk: [nztot][planes of the chunk][nxtot][3]
  const double2* twz;  // forward roots of Nz = 2nz+1
  const double2* twx;  // forward roots of Nx = 2nx+1
  RadixDev rz, rx;     // prime factors of Nz and Nx
  int zcols, xpairs, chunk;
  int nxtot, nztot;
  int fluct_only, part, z_threshold;
  double beta0;
};
size_t export_z_smem(int zcols, int Nz);
size_t export_x_smem(int xpairs, int nx, int Nx);
int export_set_smem_limits();  // dynamic shared memory allowed per block, or -1
void launch_export_chunk(const ExportLaunch& L, int iy0, int nplanes_chunk, cudaStream_t s);
void launch_force_ghosts(double2* F, const double* der, const Dims& d, cudaStream_t s);
// Reynolds-stress budget spectra (tke.cu): one snapshot's accumulation
struct TkeLaunch {
  Dims d;
  BcRows bc;
  const double2* V;  // the field
  double2* W;        // work: u', v', w' then du'_i/dx_k at field 3 + 3i + k (12 fields, V's layout)
  double2* N3;       // the convective terms N_0..2 (3 fields, V's layout)
  double2* P;        // pressure (V's layout, one field), or null
  double2* Zt;       // z-inverted fields of a chunk of planes: [12][chunk][nx+1][nzd]
  double2* Xt;       // x-forward N_i of a chunk: [3][chunk][nx+1][nzd]
  double* acc;       // running sums [6 terms][6 pairs][plane][kz]
  const double* mean;  // U, W, P, dU/dy, dW/dy per plane
  const double* der;
  const double* d0lu;
  const double2* twz;  // FP64 per-stage roots of the z plan and of the x plan, pack roots
  const double2* twx;
  const double2* twh;
  RadixDev rz, rx;
  int chunk;  // planes per chunk
};
void launch_tke_snapshot(const TkeLaunch& L, cudaStream_t s);
cudaError_t tke_set_smem_limits(int nzd, int nxd);
size_t tke_z_smem(int nzd);
size_t tke_x_smem(int nxd);
void launch_stats_accumulate(const double2* V, const Dims& d, double* acc, cudaStream_t s);

}  // namespace chgpu
