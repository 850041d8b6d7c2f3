// Host-side set-up of the wall-normal discretisation (FP64).
//
// Restates setup_derivatives (dnsdata.f90:241-286) with LUdecomp/.bs.
// (rbmat.f90:60-76, 201-215), setup_boundary_conditions (dnsdata.f90:290-308,
// full channel), the y grid (dnsdata.f90:153-155) and the factorisation of
// D0mat by LU5decompStep (rbparmat_blocking.f90:20-51, single y-domain).
// The arithmetic follows the Fortran expressions term by term: powers with a
// real exponent go through pow(), sums run left to right.
#include <cmath>
#include <cstring>

#include "chgpu_internal.h"

namespace chgpu {

bool fft_fit(int n) {
  int j = n;
  while (j % 2 == 0) j >>= 1;
  return j == 1 || j == 3;
}

void padded_sizes(int nx, int nz, int* nxd, int* nzd) {
  int a = 3 * (nx + 1) / 2, b = 3 * nz;
  while (!fft_fit(a)) ++a;
  while (!fft_fit(b)) ++b;
  *nxd = a;
  *nzd = b;
}

Radix make_radix(int n, bool composite) {
  Radix r;
  r.n = n;
  int m = n;
  while (m % 16 == 0) { r.r[r.nst++] = 16; m /= 16; }
  // the tail 2^b * 3 (b = 1..3) as one register DFT of 6, 12 or 24 points
  if (composite && (m == 6 || m == 12 || m == 24)) { r.r[r.nst++] = m; m = 1; }
  if (m % 8 == 0) { r.r[r.nst++] = 8; m /= 8; }
  else if (m % 4 == 0) { r.r[r.nst++] = 4; m /= 4; }
  else if (m % 2 == 0) { r.r[r.nst++] = 2; m /= 2; }
  if (m % 3 == 0) { r.r[r.nst++] = 3; m /= 3; }
  if (m != 1) r.nst = -1;
  return r;
}

namespace {

// rbmat.f90:60-76, 5x5, 1-based indices mapped to 0-based storage.
void lu_decomp5(double A[5][5]) {
  for (int i = 5; i >= 2; --i) {
    double piv = 1.0 / A[i - 1][i - 1];
    A[i - 1][i - 1] = piv;
    for (int j = 1; j <= i - 1; ++j) A[i - 1][j - 1] *= piv;
    for (int k = 1; k <= i - 1; ++k) {
      piv = A[k - 1][i - 1];
      for (int j = 1; j <= i - 1; ++j) A[k - 1][j - 1] = A[k - 1][j - 1] - piv * A[i - 1][j - 1];
    }
  }
  A[0][0] = 1.0 / A[0][0];
}

// rbmat.f90:201-215: x = A .bs. b
void lu_solve5(double A[5][5], const double b[5], double x[5]) {
  x[4] = b[4] * A[4][4];
  for (int i = 4; i >= 1; --i) {
    double s = 0.0;
    for (int j = i + 1; j <= 5; ++j) s += A[i - 1][j - 1] * x[j - 1];
    x[i - 1] = (b[i - 1] - s) * A[i - 1][i - 1];
  }
  for (int i = 2; i <= 5; ++i) {
    double s = 0.0;
    for (int j = 1; j <= i - 1; ++j) s += A[i - 1][j - 1] * x[j - 1];
    x[i - 1] = x[i - 1] - s;
  }
}

// Vandermonde-like matrix of the compact stencils: M(i,j) = (y(c+j)-y0)^(4-i).
void vander(const std::vector<double>& y, int first, double y0, double M[5][5], const double* scale) {
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      double v = std::pow(y[first + j + 1] - y0, 4.0 - i);
      M[i][j] = scale ? scale[i] * v : v;
    }
}

// LU5decompStep with first=last=.TRUE. on rows r=0..nrow-1 (row r <-> iy=r+1).
void lu5_decomp(std::vector<double>& A, int nrow) {
  auto a = [&](int i, int j) -> double& { return A[(size_t)i * 5 + j + 2]; };
  const int HI1 = nrow - 1, HI2 = 2;
  a(HI1 - 2, 1) = 0; a(HI1 - 2, 2) = 0; a(HI1 - 3, 2) = 0;
  for (int i = HI1 - HI2; i >= 0; --i) {
    for (int k = HI2; k >= 1; --k) {
      double piv = a(i, k);
      for (int j = -1; j >= -2; --j) {
        double below = (i + k <= HI1 - HI2) ? a(i + k, j) : 0.0;  // unassigned rows drop out
        a(i, j + k) = a(i, j + k) - piv * below;
      }
    }
    double piv = 1.0 / a(i, 0);
    a(i, 0) = piv;
    a(i, -2) *= piv;
    a(i, -1) *= piv;
  }
  a(0, -2) = 0; a(0, -1) = 0; a(1, -2) = 0;
}

}  // namespace

void compute_tables(const chgpu_params& p, Tables& t) {
  const int ny = p.ny;
  t.ny = ny;
  t.y.assign(ny + 3, 0.0);
  for (int iy = -1; iy <= ny + 1; ++iy)
    t.y[iy + 1] = p.ymin + 0.5 * (p.ymax - p.ymin) *
                               (std::tanh(p.a * (2.0 * (double)iy / (double)ny - 1)) / std::tanh(p.a) + 1);
  t.dy.assign(ny + 1, 0.0);
  for (int iy = 1; iy <= ny - 1; ++iy) t.dy[iy] = 0.5 * (t.y[iy + 2] - t.y[iy]);
  t.der.assign((size_t)(ny + 1) * 20, 0.0);
  const std::vector<double>& y = t.y;
  double M[5][5], rhs[5];
  for (int iy = 1; iy <= ny - 1; ++iy) {
    double* d0 = &t.der[(size_t)iy * 20 + 0];
    double* d1 = &t.der[(size_t)iy * 20 + 5];
    double* d2 = &t.der[(size_t)iy * 20 + 10];
    double* d4 = &t.der[(size_t)iy * 20 + 15];
    const double yc = y[iy + 1];
    vander(y, iy - 2, yc, M, nullptr);
    lu_decomp5(M);
    std::memset(rhs, 0, sizeof rhs);
    rhs[0] = 24;
    lu_solve5(M, rhs, d4);
    double sc[5];
    for (int i = 0; i < 5; ++i) sc[i] = (5.0 - i) * (6.0 - i) * (7.0 - i) * (8.0 - i);
    vander(y, iy - 2, yc, M, sc);
    lu_decomp5(M);
    for (int i = 0; i < 5; ++i) {
      double acc = d4[0] * std::pow(y[iy - 1] - yc, 8.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d4[j] * std::pow(y[iy - 1 + j] - yc, 8.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d0);
    vander(y, iy - 2, yc, M, nullptr);
    lu_decomp5(M);
    std::memset(rhs, 0, sizeof rhs);
    for (int i = 0; i <= 2; ++i) {
      double acc = d0[0] * (4.0 - i) * (3.0 - i) * std::pow(y[iy - 1] - yc, 2.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d0[j] * (4.0 - i) * (3.0 - i) * std::pow(y[iy - 1 + j] - yc, 2.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d2);
    std::memset(rhs, 0, sizeof rhs);
    for (int i = 0; i <= 3; ++i) {
      double acc = d0[0] * (4.0 - i) * std::pow(y[iy - 1] - yc, 3.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d0[j] * (4.0 - i) * std::pow(y[iy - 1 + j] - yc, 3.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d1);
  }
  // one-sided wall stencils (dnsdata.f90:259-276)
  vander(y, -1, y[1], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1.0; lu_solve5(M, rhs, t.d140);
  std::memset(rhs, 0, sizeof rhs); rhs[2] = 2.0; lu_solve5(M, rhs, t.d240);
  vander(y, -1, y[0], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1.0; lu_solve5(M, rhs, t.d14m1);
  std::memset(rhs, 0, sizeof rhs); rhs[2] = 2.0; lu_solve5(M, rhs, t.d24m1);
  std::memset(t.d040, 0, sizeof t.d040); t.d040[1] = 1;
  vander(y, ny - 3, y[ny + 1], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1; lu_solve5(M, rhs, t.d14n);
  std::memset(rhs, 0, sizeof rhs); rhs[2] = 2; lu_solve5(M, rhs, t.d24n);
  vander(y, ny - 3, y[ny + 2], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1; lu_solve5(M, rhs, t.d14np1);
  std::memset(rhs, 0, sizeof rhs); rhs[2] = 2; lu_solve5(M, rhs, t.d24np1);
  std::memset(t.d04n, 0, sizeof t.d04n); t.d04n[3] = 1;
  // D0mat and its factorisation (dnsdata.f90:277-284); rows ny, ny+1 zero
  t.d0lu.assign((size_t)(ny + 1) * 5, 0.0);
  for (int iy = 1; iy <= ny - 1; ++iy)
    for (int j = 0; j < 5; ++j) t.d0lu[(size_t)(iy - 1) * 5 + j] = t.der[(size_t)iy * 20 + j];
  lu5_decomp(t.d0lu, ny + 1);
  // boundary-condition rows (dnsdata.f90:290-308)
  std::memcpy(t.v0bc, t.d040, 40);
  std::memcpy(t.v0m1bc, t.d140, 40);
  std::memcpy(t.eta0bc, t.d040, 40);
  std::memcpy(t.eta0m1bc, &t.der[(size_t)1 * 20 + 15], 40);
  {
    double v[5], e[5];
    std::memcpy(v, t.v0bc, 40); std::memcpy(e, t.eta0bc, 40);
    for (int j = 1; j < 5; ++j) t.v0bc[j] = v[j] - v[0] * t.v0m1bc[j] / t.v0m1bc[0];
    for (int j = 1; j < 5; ++j) t.eta0bc[j] = e[j] - e[0] * t.eta0m1bc[j] / t.eta0m1bc[0];
  }
  std::memcpy(t.vnbc, t.d04n, 40);
  std::memcpy(t.vnp1bc, t.d14n, 40);
  std::memcpy(t.etanbc, t.d04n, 40);
  std::memcpy(t.etanp1bc, &t.der[(size_t)(ny - 1) * 20 + 15], 40);
  {
    double v[5], e[5];
    std::memcpy(v, t.vnbc, 40); std::memcpy(e, t.etanbc, 40);
    for (int j = 0; j < 4; ++j) t.vnbc[j] = v[j] - v[4] * t.vnp1bc[j] / t.vnp1bc[4];
    for (int j = 0; j < 4; ++j) t.etanbc[j] = e[j] - e[4] * t.etanp1bc[j] / t.etanp1bc[4];
  }
  // yintegr weights (dnsdata.f90:317-321)
  t.yint.clear();
  for (int iy = 1; iy <= ny - 1; iy += 2) {
    double yp1 = y[iy + 2] - y[iy + 1], ym1 = y[iy] - y[iy + 1];
    double a1 = -1.0 / 3.0 * ym1 + 1.0 / 6.0 * yp1 + 1.0 / 6.0 * yp1 * yp1 / ym1;
    double a3 = +1.0 / 3.0 * yp1 - 1.0 / 6.0 * ym1 - 1.0 / 6.0 * ym1 * ym1 / yp1;
    double a2 = yp1 - ym1 - a1 - a3;
    t.yint.push_back(a1);
    t.yint.push_back(a2);
    t.yint.push_back(a3);
  }
}

namespace {

// LU5decompStep of rows r=0..nrow-1 held in a plain array (see lu5_decomp).
void lu5_decomp_array(double* A, int nrow) {
  auto a = [&](int i, int j) -> double& { return A[(size_t)i * 5 + j + 2]; };
  const int HI1 = nrow - 1, HI2 = 2;
  a(HI1 - 2, 1) = 0; a(HI1 - 2, 2) = 0; a(HI1 - 3, 2) = 0;
  for (int i = HI1 - HI2; i >= 0; --i) {
    for (int k = HI2; k >= 1; --k) {
      double piv = a(i, k);
      for (int j = -1; j >= -2; --j) {
        double below = (i + k <= HI1 - HI2) ? a(i + k, j) : 0.0;
        a(i, j + k) = a(i, j + k) - piv * below;
      }
    }
    double piv = 1.0 / a(i, 0);
    a(i, 0) = piv;
    a(i, -2) *= piv;
    a(i, -1) *= piv;
  }
  a(0, -2) = 0; a(0, -1) = 0; a(1, -2) = 0;
}

void vander_array(const double* y, int first, double y0, double M[5][5], const double* scale) {
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      double v = std::pow(y[first + j + 1] - y0, 4.0 - i);
      M[i][j] = scale ? scale[i] * v : v;
    }
}

}  // namespace

// Same arithmetic as compute_tables, into fixed arrays.
void real_deriv(const Tables& t, const double* f0, double* f1, int order) {
  const int ny = t.ny;
  auto F0 = [&](int iy) { return f0[iy + 1]; };
  auto sum5 = [&](const double* c, int iy0) {
    double s = c[0] * F0(iy0);
    for (int j = 1; j < 5; ++j) s = s + c[j] * F0(iy0 + j);
    return s;
  };
  const int dk = order == 2 ? 10 : 5;  // d2 or d1 row of der
  // COMPLEXderiv / COMPLEXderiv2 (dnsdata.f90:339-414) on a real line
  double* x = f1;  // x[iy+1]
  x[0 + 1] = sum5(order == 2 ? t.d240 : t.d140, -1);
  x[-1 + 1] = sum5(order == 2 ? t.d24m1 : t.d14m1, -1);
  x[ny + 1] = sum5(order == 2 ? t.d24n : t.d14n, ny - 3);
  x[ny + 1 + 1] = sum5(order == 2 ? t.d24np1 : t.d14np1, ny - 3);
  for (int iy = 1; iy <= ny - 1; ++iy) x[iy + 1] = sum5(&t.der[(size_t)iy * 20 + dk], iy - 2);
  const double* d0 = t.der.data();
  x[1 + 1] = x[1 + 1] - (d0[1 * 20 + 1] * x[0 + 1] + d0[1 * 20 + 0] * x[-1 + 1]);
  x[2 + 1] = x[2 + 1] - d0[2 * 20 + 0] * x[0 + 1];
  x[ny - 1 + 1] = x[ny - 1 + 1] - (d0[(size_t)(ny - 1) * 20 + 3] * x[ny + 1] + d0[(size_t)(ny - 1) * 20 + 4] * x[ny + 1 + 1]);
  x[ny - 2 + 1] = x[ny - 2 + 1] - d0[(size_t)(ny - 2) * 20 + 4] * x[ny + 1];
  // LeftLU5divStep1 and Step2 with the factored D0mat (rbparmat_blocking.f90:57-100);
  // row r of the factors is y row iy = r + 1, and x(r) = x[r + 1 + 1]
  const int nrow = ny + 1;
  const double* A = t.d0lu.data();
  for (int r = nrow - 3; r >= 0; --r) {
    const double* a = A + (size_t)r * 5 + 2;
    double s = a[1] * x[r + 1 + 2];
    s = s + a[2] * x[r + 2 + 2];
    x[r + 2] = (x[r + 2] - s) * a[0];
  }
  for (int r = 0; r <= nrow - 1; ++r) {
    const double* a = A + (size_t)r * 5 + 2;
    double s = a[-2] * x[r - 2 + 2];
    s = s + a[-1] * x[r - 1 + 2];
    x[r + 2] = x[r + 2] - s;
  }
}

bool compute_tables_static(const chgpu_params& p, StaticTables& t) {
  const int ny = p.ny;
  if (ny < 8 || ny > StaticTables::kMaxNy) return false;
  t.ny = ny;
  double* y = t.y;
  for (int iy = -1; iy <= ny + 1; ++iy)
    y[iy + 1] = p.ymin + 0.5 * (p.ymax - p.ymin) * (std::tanh(p.a * (2.0 * (double)iy / (double)ny - 1)) / std::tanh(p.a) + 1);
  std::memset(t.der, 0, sizeof(double) * (size_t)(ny + 1) * 20);
  double M[5][5], rhs[5];
  for (int iy = 1; iy <= ny - 1; ++iy) {
    double* d0 = &t.der[(size_t)iy * 20 + 0];
    double* d1 = &t.der[(size_t)iy * 20 + 5];
    double* d2 = &t.der[(size_t)iy * 20 + 10];
    double* d4 = &t.der[(size_t)iy * 20 + 15];
    const double yc = y[iy + 1];
    vander_array(y, iy - 2, yc, M, nullptr);
    lu_decomp5(M);
    std::memset(rhs, 0, sizeof rhs);
    rhs[0] = 24;
    lu_solve5(M, rhs, d4);
    double sc[5];
    for (int i = 0; i < 5; ++i) sc[i] = (5.0 - i) * (6.0 - i) * (7.0 - i) * (8.0 - i);
    vander_array(y, iy - 2, yc, M, sc);
    lu_decomp5(M);
    for (int i = 0; i < 5; ++i) {
      double acc = d4[0] * std::pow(y[iy - 1] - yc, 8.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d4[j] * std::pow(y[iy - 1 + j] - yc, 8.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d0);
    vander_array(y, iy - 2, yc, M, nullptr);
    lu_decomp5(M);
    std::memset(rhs, 0, sizeof rhs);
    for (int i = 0; i <= 2; ++i) {
      double acc = d0[0] * (4.0 - i) * (3.0 - i) * std::pow(y[iy - 1] - yc, 2.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d0[j] * (4.0 - i) * (3.0 - i) * std::pow(y[iy - 1 + j] - yc, 2.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d2);
    std::memset(rhs, 0, sizeof rhs);
    for (int i = 0; i <= 3; ++i) {
      double acc = d0[0] * (4.0 - i) * std::pow(y[iy - 1] - yc, 3.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d0[j] * (4.0 - i) * std::pow(y[iy - 1 + j] - yc, 3.0 - i);
      rhs[i] = acc;
    }
    lu_solve5(M, rhs, d1);
  }
  double d040[5] = {0, 1, 0, 0, 0}, d04n[5] = {0, 0, 0, 1, 0};
  vander_array(y, -1, y[1], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1.0; lu_solve5(M, rhs, t.d140);
  vander_array(y, -1, y[0], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1.0; lu_solve5(M, rhs, t.d14m1);
  vander_array(y, ny - 3, y[ny + 1], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1; lu_solve5(M, rhs, t.d14n);
  vander_array(y, ny - 3, y[ny + 2], M, nullptr);
  lu_decomp5(M);
  std::memset(rhs, 0, sizeof rhs); rhs[3] = 1; lu_solve5(M, rhs, t.d14np1);
  std::memset(t.d0lu, 0, sizeof(double) * (size_t)(ny + 1) * 5);
  for (int iy = 1; iy <= ny - 1; ++iy)
    for (int j = 0; j < 5; ++j) t.d0lu[(size_t)(iy - 1) * 5 + j] = t.der[(size_t)iy * 20 + j];
  lu5_decomp_array(t.d0lu, ny + 1);
  std::memcpy(t.v0bc, d040, 40);
  std::memcpy(t.v0m1bc, t.d140, 40);
  std::memcpy(t.eta0bc, d040, 40);
  std::memcpy(t.eta0m1bc, &t.der[(size_t)1 * 20 + 15], 40);
  {
    double v[5], e[5];
    std::memcpy(v, t.v0bc, 40); std::memcpy(e, t.eta0bc, 40);
    for (int j = 1; j < 5; ++j) t.v0bc[j] = v[j] - v[0] * t.v0m1bc[j] / t.v0m1bc[0];
    for (int j = 1; j < 5; ++j) t.eta0bc[j] = e[j] - e[0] * t.eta0m1bc[j] / t.eta0m1bc[0];
  }
  std::memcpy(t.vnbc, d04n, 40);
  std::memcpy(t.vnp1bc, t.d14n, 40);
  std::memcpy(t.etanbc, d04n, 40);
  std::memcpy(t.etanp1bc, &t.der[(size_t)(ny - 1) * 20 + 15], 40);
  {
    double v[5], e[5];
    std::memcpy(v, t.vnbc, 40); std::memcpy(e, t.etanbc, 40);
    for (int j = 0; j < 4; ++j) t.vnbc[j] = v[j] - v[4] * t.vnp1bc[j] / t.vnp1bc[4];
    for (int j = 0; j < 4; ++j) t.etanbc[j] = e[j] - e[4] * t.etanp1bc[j] / t.etanp1bc[4];
  }
  t.nyint = 0;
  for (int iy = 1; iy <= ny - 1; iy += 2) {
    double yp1 = y[iy + 2] - y[iy + 1], ym1 = y[iy] - y[iy + 1];
    double a1 = -1.0 / 3.0 * ym1 + 1.0 / 6.0 * yp1 + 1.0 / 6.0 * yp1 * yp1 / ym1;
    double a3 = +1.0 / 3.0 * yp1 - 1.0 / 6.0 * ym1 - 1.0 / 6.0 * ym1 * ym1 / yp1;
    double a2 = yp1 - ym1 - a1 - a3;
    t.yint[3 * t.nyint] = a1;
    t.yint[3 * t.nyint + 1] = a2;
    t.yint[3 * t.nyint + 2] = a3;
    ++t.nyint;
  }
  return true;
}

}  // namespace chgpu
