// Internal declarations of the channel-flow step library (libchgpu.so).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/chgpu.h"

namespace chgpu {

// Host-side tables of the wall-normal discretisation, computed once per run
// in FP64 exactly as setup_derivatives / setup_boundary_conditions do
// (dnsdata.f90:241-308) and uploaded to the device.
struct Tables {
  int ny = 0;
  std::vector<double> y;    // y(iy), iy=-1..ny+1 at index iy+1       (dnsdata.f90:153)
  std::vector<double> dy;   // dy(iy), iy=0..ny (entries 1..ny-1 used) (dnsdata.f90:155)
  std::vector<double> der;  // der(iy): [iy][d0,d1,d2,d4][5], iy=0..ny (1..ny-1 used)
  double d040[5], d140[5], d240[5], d14m1[5], d24m1[5];
  double d04n[5], d14n[5], d24n[5], d14np1[5], d24np1[5];
  double v0bc[5], v0m1bc[5], eta0bc[5], eta0m1bc[5];
  double vnbc[5], vnp1bc[5], etanbc[5], etanp1bc[5];
  std::vector<double> d0lu;  // LU5decompStep(D0mat): rows iy=1..ny+1 -> [(iy-1)*5 + j+2]
  std::vector<double> yint;  // yintegr weights: [(iy-1)/2][3] for odd iy    (dnsdata.f90:317-323)
};

// The same tables in fixed-capacity arrays (no heap), for the entry point
// that allocates nothing; ny <= kMaxNy.
struct StaticTables {
  static constexpr int kMaxNy = 1024;
  int ny = 0, nyint = 0;
  double y[kMaxNy + 3];
  double der[(kMaxNy + 1) * 20];
  double d0lu[(kMaxNy + 1) * 5];
  double yint[3 * (kMaxNy / 2 + 1)];
  double d140[5], d14m1[5], d14n[5], d14np1[5];
  double v0bc[5], v0m1bc[5], eta0bc[5], eta0m1bc[5];
  double vnbc[5], vnp1bc[5], etanbc[5], etanp1bc[5];
};
bool compute_tables_static(const chgpu_params& p, StaticTables& t);

bool fft_fit(int n);                       // ffts.f90:78-86
void padded_sizes(int nx, int nz, int* nxd, int* nzd);  // dnsdata.f90:110-114
void compute_tables(const chgpu_params& p, Tables& t);
// REALderiv / REALderiv2 (dnsdata.f90:419-451): compact first (order 1) or
// second (order 2) y derivative of a real line f0[iy+1], iy = -1..ny+1
void real_deriv(const Tables& t, const double* f0, double* f1, int order);

// Radix plan of a length-n transform (n = 2^a or 3*2^a).
struct Radix {
  int n = 0, nst = 0;
  int r[24];
};
// radices 16, then 8/4/2, then 3; with composite, a tail of 6, 12 or 24
// points is one stage
Radix make_radix(int n, bool composite = false);

// Scalars the reference keeps as module globals, resident on the device so
// that whole steps (including the CFL-driven time step) run without the host.
struct DevScalars {
  double deltat;
  double rdt;  // 1/deltat
  double time;
  double cfl;  // running max over planes (non-negative: ordered as u64 bits)
  double fr[3];
  double corrpx, corrpz, meanpx, meanpz;
  double u0, uN;
  double line[11];
  double runtime_global;
  double wallrhs[8];  // the mean mode's wall-velocity terms of the eta right-hand side, rows 1, 2, ny-2, ny-1
  long long istep;
  int error;  // bit 0: non-finite CFL or statistics; bit 1: a bulk-copy wait ran out;
              // bit 2: a tensor-core completion wait of the closure ran out
  int first_wait;  // 0: the full poll limit; k > 0: a generic z kernel's first bulk-copy wait
                   // makes k-1 polls (chgpu_set_wait_limit, for tests of the time-out path)
};

}  // namespace chgpu
