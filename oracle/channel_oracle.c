/*
 * channel_oracle.c -- CPU oracle for the channel RK3/CN step (TEST
 * INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's
 * CPU-baseline leg load it as the checker; the product never does).
 *
 * A plain-C FP64 restatement of the reference hot path.  Each routine cites
 * the reference lines it follows; per output value the arithmetic is the one
 * the Fortran expression spells out (left-to-right sums, real*complex as two
 * real products, complex/real as two divisions).  Build with
 * -ffp-contract=off -fcx-fortran-rules so the compiler does not re-associate.
 *
 * Loop structure differs from the reference where that does not change any
 * value: buildrhs convolves every plane first and writes the new right-hand
 * sides back after all rows are computed, which is what the reference's
 * five-plane ring and three-plane newrhs ring compute (dnsdata.f90:630-671).
 *
 * Rows iy=ny,ny+1 of D0mat are never assigned by the reference
 * (dnsdata.f90:277); they are treated as zero here, so LeftLU5divStep2 leaves
 * the one-sided wall derivatives of COMPLEXderiv unchanged in those rows.
 *
 * Parity is unpinned against the reference binary (no reference golden
 * vectors exist; see channel_oracle.h).
 */
#include "channel_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ------------------------------------------------------------------ */
/* FFT: mixed radix 4/2/3 Stockham, unnormalised, FFTW sign convention. */
/* ------------------------------------------------------------------ */
typedef struct fftplan {
  int n, sign, nst;
  int radix[32];
  cplx* tw; /* tw[m] = exp(sign*2*pi*i*m/n) */
} fftplan;

static void fftplan_init(fftplan* p, int n, int sign) {
  p->n = n;
  p->sign = sign;
  p->nst = 0;
  int m = n;
  while (m % 4 == 0) { p->radix[p->nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p->radix[p->nst++] = 2; m /= 2; }
  while (m % 3 == 0) { p->radix[p->nst++] = 3; m /= 3; }
  if (m != 1) abort(); /* lengths are 2^a or 3*2^a (ffts.f90:78-86) */
  p->tw = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  for (int k = 0; k < n; ++k) {
    /* twiddles from the mathematics, in extended precision */
    long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)n;
    double c = (double)cosl(ang), s = (double)sinl(ang);
    p->tw[k] = CMPLX(c, sign * s);
  }
}

static void fftplan_free(fftplan* p) { free(p->tw); }

static inline cplx cmul(cplx a, cplx b) {
  return CMPLX(creal(a) * creal(b) - cimag(a) * cimag(b),
               creal(a) * cimag(b) + cimag(a) * creal(b));
}
static inline cplx mul_i(cplx a, int sign) { /* a * (sign*i) */
  return sign > 0 ? CMPLX(-cimag(a), creal(a)) : CMPLX(cimag(a), -creal(a));
}

/* x: n complex, work: n complex scratch. Result in x. */
static void fft_exec(const fftplan* p, cplx* x, cplx* work) {
  const int n = p->n;
  cplx* src = x;
  cplx* dst = work;
  int Ns = 1;
  const double h3 = 0.86602540378443864676372317075294; /* sqrt(3)/2 */
  for (int st = 0; st < p->nst; ++st) {
    const int R = p->radix[st];
    const int nR = n / R;
    const int twstep = n / (Ns * R);
    for (int j = 0; j < nR; ++j) {
      const int k = j % Ns;
      cplx a[4];
      for (int r = 0; r < R; ++r) a[r] = src[j + r * nR];
      if (k != 0)
        for (int r = 1; r < R; ++r) a[r] = cmul(a[r], p->tw[(r * k * twstep) % n]);
      cplx y[4];
      if (R == 2) {
        y[0] = a[0] + a[1];
        y[1] = a[0] - a[1];
      } else if (R == 4) {
        cplx t0 = a[0] + a[2], t1 = a[0] - a[2];
        cplx t2 = a[1] + a[3], t3 = mul_i(a[1] - a[3], p->sign);
        y[0] = t0 + t2;
        y[2] = t0 - t2;
        y[1] = t1 + t3;
        y[3] = t1 - t3;
      } else { /* R == 3 */
        cplx t1 = a[1] + a[2];
        cplx t2 = a[0] - 0.5 * t1;
        cplx t3 = mul_i(h3 * (a[1] - a[2]), p->sign);
        y[0] = a[0] + t1;
        y[1] = t2 + t3;
        y[2] = t2 - t3;
      }
      const int idxD = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) dst[idxD + r * Ns] = y[r];
    }
    cplx* t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(cplx) * (size_t)n);
}

void orc_fft(int n, int sign, int howmany, double* data) {
  fftplan p;
  fftplan_init(&p, n, sign);
  cplx* work = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  for (int b = 0; b < howmany; ++b) fft_exec(&p, (cplx*)data + (size_t)b * n, work);
  free(work);
  fftplan_free(&p);
}

/* ------------------------------------------------------------------ */
/* Parameters                                                          */
/* ------------------------------------------------------------------ */
int orc_fftfit(int i) { /* ffts.f90:78-86 */
  int j = i;
  while (j % 2 == 0) j >>= 1;
  return j == 1 || j == 3;
}

void orc_sizes(const orc_params* p, int* nxd, int* nzd) { /* dnsdata.f90:110-114 */
  int a = 3 * (p->nx + 1) / 2, b = 3 * p->nz;
  while (!orc_fftfit(a)) ++a;
  while (!orc_fftfit(b)) ++b;
  *nxd = a;
  *nzd = b;
}

/* ------------------------------------------------------------------ */
/* State                                                               */
/* ------------------------------------------------------------------ */
typedef struct { double d0[5], d1[5], d2[5], d4[5]; } Di; /* typedef.f90:28-30 */

struct orc_state {
  orc_params p;
  int nx, ny, nz, nxd, nzd, nzt, nthreads;
  double dx, dz, factor;
  double* y;   /* y[iy+1], iy=-1..ny+1 */
  double* dy;  /* dy[iy], iy=1..ny-1 (index 0 unused) */
  Di* der;     /* der[iy], iy=1..ny-1 */
  double d040[5], d140[5], d240[5], d14m1[5], d24m1[5];
  double d04n[5], d14n[5], d24n[5], d14np1[5], d24np1[5];
  double v0bc[5], v0m1bc[5], eta0bc[5], eta0m1bc[5];
  double vnbc[5], vnp1bc[5], etanbc[5], etanp1bc[5];
  double* D0mat; /* rows iy=1..ny+1 -> D0mat[(iy-1)*5 + j+2] */
  cplx* V;       /* Fortran order (ny+3, 2nz+1, nx+1, 3) */
  cplx* old_eta; /* oldrhs(iy=1..ny-1, iz, ix)%eta */
  cplx* old_d2v;
  cplx* VV;      /* per plane: [plane][6][ix][iz] truncated spectra */
  cplx* newrhs_eta;
  cplx* newrhs_d2v;
  cplx* F;       /* body force, V's layout, or NULL */
  double* tau;   /* closure stresses [6][iy=1..ny-1][nzd][2nxd], or NULL */
  double* k2;    /* k2[ix*(2nz+1)+iz+nz] */
  fftplan pz_f, pz_b, px_f, px_b;
  /* module scalars */
  double cfl, fr[3], corrpx, corrpz, meanpx, meanpz;
  double time, deltat, time0;
  long long istep;
};

#define YI(iy) ((iy) + 1)
#define VIDX(s, iy, iz, ix, ic) \
  ((size_t)YI(iy) + (size_t)((s)->ny + 3) * ((size_t)((iz) + (s)->nz) + (size_t)(s)->nzt * ((size_t)(ix) + (size_t)((s)->nx + 1) * (size_t)((ic) - 1))))
#define V_(s, iy, iz, ix, ic) ((s)->V[VIDX(s, iy, iz, ix, ic)])
#define RIDX(s, iy, iz, ix) ((size_t)((iy) - 1) + (size_t)((s)->ny - 1) * ((size_t)((iz) + (s)->nz) + (size_t)(s)->nzt * (size_t)(ix)))
#define K2(s, iz, ix) ((s)->k2[(size_t)(ix) * (s)->nzt + (iz) + (s)->nz])

/* rbmat.f90:60-76  in-place decomposition of a 5x5 matrix (A 1-based). */
static void LUdecomp5(double A[5][5]) {
  const int HI = 5;
  for (int i = HI; i >= 2; --i) {
    double piv = 1.0 / A[i - 1][i - 1];
    A[i - 1][i - 1] = piv;
    for (int j = 1; j <= i - 1; ++j) A[i - 1][j - 1] = A[i - 1][j - 1] * piv;
    for (int k = 1; k <= i - 1; ++k) {
      piv = A[k - 1][i - 1];
      for (int j = 1; j <= i - 1; ++j) A[k - 1][j - 1] = A[k - 1][j - 1] - piv * A[i - 1][j - 1];
    }
  }
  A[0][0] = 1.0 / A[0][0];
}

/* rbmat.f90:201-215  x = A .bs. b */
static void LLUdiv5(double A[5][5], const double b[5], double x[5]) {
  const int HI = 5;
  x[HI - 1] = b[HI - 1] * A[HI - 1][HI - 1];
  for (int i = HI - 1; i >= 1; --i) {
    double s = 0.0;
    for (int j = i + 1; j <= HI; ++j) s += A[i - 1][j - 1] * x[j - 1];
    x[i - 1] = (b[i - 1] - s) * A[i - 1][i - 1];
  }
  for (int i = 2; i <= HI; ++i) {
    double s = 0.0;
    for (int j = 1; j <= i - 1; ++j) s += A[i - 1][j - 1] * x[j - 1];
    x[i - 1] = x[i - 1] - s;
  }
}

static double ypow(double b, double e) { return pow(b, e); }

/* rbparmat_blocking.f90:20-51 with first=last=.TRUE. A has nrow rows
 * (row r <-> iy=r+1) of 5 bands (j=-2..2 -> index j+2). Rows nrow-2,nrow-1
 * (iy=ny,ny+1) are not touched by the loop. */
static void LU5decompStep(double* A, int nrow) {
  const int HI1 = nrow - 1, HI2 = 2;
#define A_(i, j) A[(size_t)(i) * 5 + (j) + 2]
  A_(HI1 - 2, 1) = 0; A_(HI1 - 2, 2) = 0; A_(HI1 - 3, 2) = 0;
  for (int i = HI1 - HI2; i >= 0; --i) {
    for (int k = HI2; k >= 1; --k) {
      double piv = A_(i, k);
      for (int j = -1; j >= -2; --j) {
        /* rows i+k > HI1-HI2 are the unassigned rows iy=ny,ny+1: their
         * coefficients are multiplied by the zeroed piv and drop out */
        double aik = (i + k <= HI1 - HI2) ? A_(i + k, j) : 0.0;
        A_(i, j + k) = A_(i, j + k) - piv * aik;
      }
    }
    double piv = 1.0 / A_(i, 0);
    A_(i, 0) = piv;
    A_(i, -2) = A_(i, -2) * piv;
    A_(i, -1) = A_(i, -1) * piv;
  }
  A_(0, -2) = 0; A_(0, -1) = 0; A_(1, -2) = 0;
#undef A_
}

/* rbparmat_blocking.f90:57-77 (in place: x is b). x indexed from -2 (x[0]
 * is x(-2)). */
static void LeftLU5divStep1(cplx* x, const double* A, int nrow) {
  const int HI1 = nrow - 1, HI2 = 2;
  for (int i = HI1 - HI2; i >= 0; --i) {
    const double* a = A + (size_t)i * 5 + 2;
    cplx s = a[1] * x[i + 1 + 2];
    s = s + a[2] * x[i + 2 + 2];
    x[i + 2] = (x[i + 2] - s) * a[0];
  }
}

/* rbparmat_blocking.f90:82-100 */
static void LeftLU5divStep2(const double* A, cplx* b, int nrow) {
  const int HI1 = nrow - 1;
  for (int i = 0; i <= HI1; ++i) {
    const double* a = A + (size_t)i * 5 + 2;
    cplx s = a[-2] * b[i - 2 + 2];
    s = s + a[-1] * b[i - 1 + 2];
    b[i + 2] = b[i + 2] - s;
  }
}

static double sum5(const double* c, const double* f) { /* sum(c(-2:2)*f(...)) */
  double s = c[0] * f[0];
  for (int j = 1; j < 5; ++j) s = s + c[j] * f[j];
  return s;
}
static cplx csum5(const double* c, const cplx* f) {
  cplx s = c[0] * f[0];
  for (int j = 1; j < 5; ++j) s = s + c[j] * f[j];
  return s;
}

/* dnsdata.f90:241-286 */
static void setup_derivatives(orc_state* s) {
  const int ny = s->ny;
  double M[5][5], t[5];
  const double* y = s->y;
#define Y(iy) y[YI(iy)]
  for (int iy = 1; iy <= ny - 1; ++iy) {
    Di* d = &s->der[iy];
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(iy - 2 + j) - Y(iy), 4.0 - i);
    LUdecomp5(M);
    memset(t, 0, sizeof t); t[0] = 24;
    LLUdiv5(M, t, d->d4);
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j)
        M[i][j] = (5.0 - i) * (6.0 - i) * (7.0 - i) * (8.0 - i) * ypow(Y(iy - 2 + j) - Y(iy), 4.0 - i);
    LUdecomp5(M);
    for (int i = 0; i < 5; ++i) {
      double acc = d->d4[0] * ypow(Y(iy - 2) - Y(iy), 8.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d->d4[j] * ypow(Y(iy - 2 + j) - Y(iy), 8.0 - i);
      t[i] = acc;
    }
    LLUdiv5(M, t, d->d0);
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(iy - 2 + j) - Y(iy), 4.0 - i);
    LUdecomp5(M);
    memset(t, 0, sizeof t);
    for (int i = 0; i <= 2; ++i) {
      double acc = d->d0[0] * (4.0 - i) * (3.0 - i) * ypow(Y(iy - 2) - Y(iy), 2.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d->d0[j] * (4.0 - i) * (3.0 - i) * ypow(Y(iy - 2 + j) - Y(iy), 2.0 - i);
      t[i] = acc;
    }
    LLUdiv5(M, t, d->d2);
    memset(t, 0, sizeof t);
    for (int i = 0; i <= 3; ++i) {
      double acc = d->d0[0] * (4.0 - i) * ypow(Y(iy - 2) - Y(iy), 3.0 - i);
      for (int j = 1; j < 5; ++j) acc = acc + d->d0[j] * (4.0 - i) * ypow(Y(iy - 2 + j) - Y(iy), 3.0 - i);
      t[i] = acc;
    }
    LLUdiv5(M, t, d->d1);
  }
  /* first */
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(-1 + j) - Y(0), 4.0 - i);
  LUdecomp5(M);
  memset(t, 0, sizeof t); t[3] = 1.0; LLUdiv5(M, t, s->d140);
  memset(t, 0, sizeof t); t[2] = 2.0; LLUdiv5(M, t, s->d240);
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(-1 + j) - Y(-1), 4.0 - i);
  LUdecomp5(M);
  memset(t, 0, sizeof t); t[3] = 1.0; LLUdiv5(M, t, s->d14m1);
  memset(t, 0, sizeof t); t[2] = 2.0; LLUdiv5(M, t, s->d24m1);
  memset(s->d040, 0, sizeof s->d040); s->d040[1] = 1;
  /* last */
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(ny - 3 + j) - Y(ny), 4.0 - i);
  LUdecomp5(M);
  memset(t, 0, sizeof t); t[3] = 1; LLUdiv5(M, t, s->d14n);
  memset(t, 0, sizeof t); t[2] = 2; LLUdiv5(M, t, s->d24n);
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) M[i][j] = ypow(Y(ny - 3 + j) - Y(ny + 1), 4.0 - i);
  LUdecomp5(M);
  memset(t, 0, sizeof t); t[3] = 1; LLUdiv5(M, t, s->d14np1);
  memset(t, 0, sizeof t); t[2] = 2; LLUdiv5(M, t, s->d24np1);
  memset(s->d04n, 0, sizeof s->d04n); s->d04n[3] = 1;
  /* D0mat rows iy=1..ny-1 from d0, rows ny,ny+1 zero */
  memset(s->D0mat, 0, sizeof(double) * 5 * (size_t)(ny + 1));
  for (int iy = 1; iy <= ny - 1; ++iy)
    for (int j = 0; j < 5; ++j) s->D0mat[(size_t)(iy - 1) * 5 + j] = s->der[iy].d0[j];
  LU5decompStep(s->D0mat, ny + 1);
#undef Y
}

/* dnsdata.f90:290-308 (full channel) */
static void setup_boundary_conditions(orc_state* s) {
  const int ny = s->ny;
  memcpy(s->v0bc, s->d040, sizeof s->v0bc);
  memcpy(s->v0m1bc, s->d140, sizeof s->v0m1bc);
  memcpy(s->eta0bc, s->d040, sizeof s->eta0bc);
  memcpy(s->eta0m1bc, s->der[1].d4, sizeof s->eta0m1bc);
  {
    double v[5], e[5];
    memcpy(v, s->v0bc, sizeof v); memcpy(e, s->eta0bc, sizeof e);
    for (int j = 1; j < 5; ++j) s->v0bc[j] = v[j] - v[0] * s->v0m1bc[j] / s->v0m1bc[0];
    for (int j = 1; j < 5; ++j) s->eta0bc[j] = e[j] - e[0] * s->eta0m1bc[j] / s->eta0m1bc[0];
  }
  memcpy(s->vnbc, s->d04n, sizeof s->vnbc);
  memcpy(s->vnp1bc, s->d14n, sizeof s->vnp1bc);
  memcpy(s->etanbc, s->d04n, sizeof s->etanbc);
  memcpy(s->etanp1bc, s->der[ny - 1].d4, sizeof s->etanp1bc);
  {
    double v[5], e[5];
    memcpy(v, s->vnbc, sizeof v); memcpy(e, s->etanbc, sizeof e);
    for (int j = 0; j < 4; ++j) s->vnbc[j] = v[j] - v[4] * s->vnp1bc[j] / s->vnp1bc[4];
    for (int j = 0; j < 4; ++j) s->etanbc[j] = e[j] - e[4] * s->etanp1bc[j] / s->etanp1bc[4];
  }
}

orc_state* orc_create(const orc_params* p, int nthreads) {
  const int ny = p->ny, nx = p->nx, nz = p->nz, nzt = 2 * nz + 1;
  if (ny < 8 || nx < 1 || nz < 1) return NULL;
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  s->p = *p;
  s->nx = p->nx; s->ny = p->ny; s->nz = p->nz;
  orc_sizes(p, &s->nxd, &s->nzd);
  s->nzt = 2 * p->nz + 1;
  s->nthreads = nthreads > 0 ? nthreads : 1;
  const double PI = 3.1415926535897932384626433832795028841971;
  s->dx = PI / (p->alfa0 * s->nxd);
  s->dz = 2.0 * PI / (p->beta0 * s->nzd);
  s->factor = 1.0 / (2.0 * s->nxd * s->nzd);
  /* dnsdata.f90:153-158 */
  s->y = (double*)malloc(sizeof(double) * (size_t)(ny + 3));
  for (int iy = -1; iy <= ny + 1; ++iy)
    s->y[YI(iy)] = p->ymin + 0.5 * (p->ymax - p->ymin) *
                   (tanh(p->a * (2.0 * (double)(float)iy / (double)(float)ny - 1)) / tanh(p->a) + 1);
  s->dy = (double*)calloc((size_t)ny + 1, sizeof(double));
  for (int iy = 1; iy <= ny - 1; ++iy) s->dy[iy] = 0.5 * (s->y[YI(iy + 1)] - s->y[YI(iy - 1)]);
  s->k2 = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * nzt);
  for (int ix = 0; ix <= nx; ++ix)
    for (int iz = -nz; iz <= nz; ++iz)
      K2(s, iz, ix) = pow(p->alfa0 * ix, 2.0) + pow(p->beta0 * iz, 2.0);
  s->der = (Di*)calloc((size_t)(ny + 1), sizeof(Di));
  s->D0mat = (double*)calloc((size_t)(ny + 1) * 5, sizeof(double));
  setup_derivatives(s);
  setup_boundary_conditions(s);
  const size_t nV = (size_t)(ny + 3) * nzt * (nx + 1) * 3;
  s->V = (cplx*)calloc(nV, sizeof(cplx));
  const size_t nR = (size_t)(ny - 1) * nzt * (nx + 1);
  s->old_eta = (cplx*)calloc(nR, sizeof(cplx));
  s->old_d2v = (cplx*)calloc(nR, sizeof(cplx));
  s->newrhs_eta = (cplx*)calloc(nR, sizeof(cplx));
  s->newrhs_d2v = (cplx*)calloc(nR, sizeof(cplx));
  s->VV = (cplx*)calloc((size_t)(ny + 3) * 6 * (nx + 1) * nzt, sizeof(cplx));
  fftplan_init(&s->pz_f, s->nzd, -1);
  fftplan_init(&s->pz_b, s->nzd, +1);
  fftplan_init(&s->px_f, 2 * s->nxd, -1);
  fftplan_init(&s->px_b, 2 * s->nxd, +1);
  s->meanpx = p->meanpx; s->meanpz = p->meanpz;
  s->time = p->time; s->deltat = p->deltat;
  return s;
}

void orc_destroy(orc_state* s) {
  if (!s) return;
  free(s->y); free(s->dy); free(s->k2); free(s->der); free(s->D0mat);
  free(s->V); free(s->old_eta); free(s->old_d2v); free(s->newrhs_eta); free(s->newrhs_d2v);
  free(s->VV);
  free(s->F);
  free(s->tau);
  fftplan_free(&s->pz_f); fftplan_free(&s->pz_b); fftplan_free(&s->px_f); fftplan_free(&s->px_b);
  free(s);
}

long long orc_field_len(const orc_state* s) {
  return (long long)(s->ny + 3) * s->nzt * (s->nx + 1) * 3;
}
void orc_set_field(orc_state* s, const double* V) {
  memcpy(s->V, V, sizeof(cplx) * (size_t)orc_field_len(s));
}
void orc_get_field(const orc_state* s, double* V) {
  memcpy(V, s->V, sizeof(cplx) * (size_t)orc_field_len(s));
}

void orc_tables(const orc_state* s, double* y, double* der, double* wall, double* bc, double* d0mat) {
  const int ny = s->ny;
  if (y) memcpy(y, s->y, sizeof(double) * (size_t)(ny + 3));
  if (der)
    for (int iy = 1; iy <= ny - 1; ++iy) {
      memcpy(der + (size_t)(iy - 1) * 20 + 0, s->der[iy].d0, 40);
      memcpy(der + (size_t)(iy - 1) * 20 + 5, s->der[iy].d1, 40);
      memcpy(der + (size_t)(iy - 1) * 20 + 10, s->der[iy].d2, 40);
      memcpy(der + (size_t)(iy - 1) * 20 + 15, s->der[iy].d4, 40);
    }
  if (wall) {
    const double* w[10] = {s->d040, s->d140, s->d240, s->d14m1, s->d24m1, s->d04n, s->d14n, s->d24n, s->d14np1, s->d24np1};
    for (int k = 0; k < 10; ++k) memcpy(wall + 5 * k, w[k], 40);
  }
  if (bc) {
    const double* w[8] = {s->v0bc, s->v0m1bc, s->eta0bc, s->eta0m1bc, s->vnbc, s->vnp1bc, s->etanbc, s->etanp1bc};
    for (int k = 0; k < 8; ++k) memcpy(bc + 5 * k, w[k], 40);
  }
  if (d0mat) memcpy(d0mat, s->D0mat, sizeof(double) * 5 * (size_t)(ny + 1));
}

/* ------------------------------------------------------------------ */
/* convolutions (dnsdata.f90:487-602), one plane, into out[6][ix][iz]  */
/* ------------------------------------------------------------------ */
typedef struct conv_ws {
  cplx* zc;    /* [3 or 6][nx+1][nzd] z columns */
  double* xr;  /* [6][nzd][2nxd] physical rows */
  cplx* row;   /* 2nxd complex */
  cplx* work;  /* max(nzd, 2nxd) */
} conv_ws;

static void conv_ws_init(const orc_state* s, conv_ws* w) {
  const int nxp = s->nx + 1, nzd = s->nzd, n2 = 2 * s->nxd;
  w->zc = (cplx*)calloc((size_t)6 * nxp * nzd, sizeof(cplx));
  w->xr = (double*)calloc((size_t)6 * nzd * n2, sizeof(double));
  w->row = (cplx*)calloc((size_t)n2, sizeof(cplx));
  int m = nzd > n2 ? nzd : n2;
  w->work = (cplx*)calloc((size_t)m, sizeof(cplx));
}
static void conv_ws_free(conv_ws* w) { free(w->zc); free(w->xr); free(w->row); free(w->work); }

static double convolve_plane(orc_state* s, int iy, int compute_cfl, cplx* out, conv_ws* w) {
  const int nx = s->nx, nz = s->nz, nzd = s->nzd, nxd = s->nxd, n2 = 2 * nxd, nzt = s->nzt;
  const int nxp = nx + 1;
  /* dnsdata.f90:504-505: pad in z */
  for (int c = 0; c < 3; ++c)
    for (int ix = 0; ix <= nx; ++ix) {
      cplx* col = w->zc + ((size_t)c * nxp + ix) * nzd;
      for (int jz = 0; jz < nzd; ++jz) col[jz] = 0;
      for (int iz = 0; iz <= nz; ++iz) col[iz] = V_(s, iy, iz, ix, c + 1);
      for (int iz = -nz; iz <= -1; ++iz) col[nzd + iz] = V_(s, iy, iz, ix, c + 1);
      fft_exec(&s->pz_b, col, w->work); /* IFT, dnsdata.f90:510 */
    }
  /* zTOx, x-pad, RFT (dnsdata.f90:533-535): c2r of length 2nxd; the c2r
   * uses only the real part of the kx=0 entry; the Nyquist entry is 0. */
  for (int c = 0; c < 3; ++c)
    for (int jz = 0; jz < nzd; ++jz) {
      cplx* r = w->row;
      for (int k = 0; k < n2; ++k) r[k] = 0;
      r[0] = creal(w->zc[((size_t)c * nxp + 0) * nzd + jz]);
      for (int ix = 1; ix <= nx; ++ix) {
        cplx X = w->zc[((size_t)c * nxp + ix) * nzd + jz];
        r[ix] = X;
        r[n2 - ix] = conj(X);
      }
      fft_exec(&s->px_b, r, w->work);
      double* xr = w->xr + ((size_t)c * nzd + jz) * n2;
      for (int k = 0; k < n2; ++k) xr[k] = creal(r[k]);
    }
  double cfl = 0;
  if (compute_cfl && iy >= 1 && iy <= s->ny - 1) { /* dnsdata.f90:552-556 */
    const double dyi = s->dy[iy];
    for (int jz = 0; jz < nzd; ++jz)
      for (int k = 0; k < n2; ++k) {
        double u = w->xr[((size_t)0 * nzd + jz) * n2 + k];
        double v = w->xr[((size_t)1 * nzd + jz) * n2 + k];
        double ww = w->xr[((size_t)2 * nzd + jz) * n2 + k];
        double c = fabs(u) / s->dx + fabs(v) / dyi + fabs(ww) / s->dz;
        if (c > cfl) cfl = c;
      }
  }
  /* products (dnsdata.f90:581-584): 4=uv 5=vw 6=uw, then 1..3 squares */
  const double f = s->factor;
  for (int jz = 0; jz < nzd; ++jz)
    for (int k = 0; k < n2; ++k) {
      double* u = w->xr + ((size_t)0 * nzd + jz) * n2 + k;
      double* v = w->xr + ((size_t)1 * nzd + jz) * n2 + k;
      double* ww = w->xr + ((size_t)2 * nzd + jz) * n2 + k;
      double U = *u, Vv = *v, W = *ww;
      w->xr[((size_t)3 * nzd + jz) * n2 + k] = U * Vv * f;
      w->xr[((size_t)4 * nzd + jz) * n2 + k] = Vv * W * f;
      w->xr[((size_t)5 * nzd + jz) * n2 + k] = U * W * f;
      *u = U * U * f;
      *v = Vv * Vv * f;
      *ww = W * W * f;
    }
  /* a prescribed subgrid stress enters with the products it belongs to */
  if (s->tau && iy >= 1 && iy <= s->ny - 1) {
    const size_t pp = (size_t)nzd * n2, np = (size_t)(s->ny - 1) * pp;
    for (int c = 0; c < 6; ++c)
      for (size_t q = 0; q < pp; ++q) w->xr[(size_t)c * pp + q] += s->tau[(size_t)c * np + (size_t)(iy - 1) * pp + q] * f;
  }
  /* HFT, xTOz, FFT (dnsdata.f90:585-590) */
  for (int c = 0; c < 6; ++c) {
    for (int jz = 0; jz < nzd; ++jz) {
      cplx* r = w->row;
      const double* xr = w->xr + ((size_t)c * nzd + jz) * n2;
      for (int k = 0; k < n2; ++k) r[k] = xr[k];
      fft_exec(&s->px_f, r, w->work);
      for (int ix = 0; ix <= nx; ++ix) w->zc[((size_t)c * nxp + ix) * nzd + jz] = r[ix];
    }
    for (int ix = 0; ix <= nx; ++ix) {
      cplx* col = w->zc + ((size_t)c * nxp + ix) * nzd;
      fft_exec(&s->pz_f, col, w->work);
      cplx* o = out + ((size_t)c * nxp + ix) * nzt;
      for (int iz = -nz; iz <= nz; ++iz) o[iz + nz] = col[iz >= 0 ? iz : nzd + iz];
    }
  }
  return cfl;
}

double orc_convolve_plane(orc_state* s, int iy, double* out) {
  conv_ws w;
  conv_ws_init(s, &w);
  double c = convolve_plane(s, iy, 1, (cplx*)out, &w);
  conv_ws_free(&w);
  return c;
}

/* ------------------------------------------------------------------ */
/* buildrhs (dnsdata.f90:611-673)                                      */
/* ------------------------------------------------------------------ */
#define F_(s, iy, iz, ix, ic) ((s)->F[VIDX(s, iy, iz, ix, ic)])

void orc_set_body_force(orc_state* s, const double* F) {
  if (!F) {
    free(s->F);
    s->F = NULL;
    return;
  }
  if (!s->F) s->F = (cplx*)malloc(sizeof(cplx) * (size_t)orc_field_len(s));
  memcpy(s->F, F, sizeof(cplx) * (size_t)orc_field_len(s));
}

void orc_set_tau(orc_state* s, const double* tau) {
  const size_t n = (size_t)6 * (s->ny - 1) * s->nzd * 2 * s->nxd;
  if (!tau) {
    free(s->tau);
    s->tau = NULL;
    return;
  }
  if (!s->tau) s->tau = (double*)malloc(sizeof(double) * n);
  memcpy(s->tau, tau, sizeof(double) * n);
}

/* dnsdata.f90:617-628: F(-1:0)=0, then F(-1) = -D4(F)/d4(-2) at iy=1; same at the top */
static void body_force_ghosts(orc_state* s) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  for (int ic = 1; ic <= 3; ++ic)
    for (int ix = 0; ix <= nx; ++ix)
      for (int iz = -nz; iz <= nz; ++iz) {
        F_(s, -1, iz, ix, ic) = 0;
        F_(s, 0, iz, ix, ic) = 0;
        F_(s, ny, iz, ix, ic) = 0;
        F_(s, ny + 1, iz, ix, ic) = 0;
      }
  for (int ic = 1; ic <= 3; ++ic)
    for (int ix = 0; ix <= nx; ++ix)
      for (int iz = -nz; iz <= nz; ++iz) {
        cplx f[5];
        for (int j = 0; j < 5; ++j) f[j] = F_(s, 1 - 2 + j, iz, ix, ic);
        F_(s, -1, iz, ix, ic) = -csum5(s->der[1].d4, f) / s->der[1].d4[0];
        for (int j = 0; j < 5; ++j) f[j] = F_(s, ny - 1 - 2 + j, iz, ix, ic);
        F_(s, ny + 1, iz, ix, ic) = -csum5(s->der[ny - 1].d4, f) / s->der[ny - 1].d4[4];
      }
}

static cplx fstencil(const orc_state* s, const double* c, int iy, int iz, int ix, int ic) {
  cplx f[5];
  for (int j = 0; j < 5; ++j) f[j] = F_(s, iy - 2 + j, iz, ix, ic);
  return csum5(c, f);
}

#define VVP(s, iy, k, ix, iz) \
  ((s)->VV[(((size_t)YI(iy) * 6 + (size_t)((k) - 1)) * ((s)->nx + 1) + (size_t)(ix)) * (s)->nzt + (size_t)((iz) + (s)->nz)])

/* DD(f,k) of dnsdata.f90:609-610: five-point stencil on product k at row iy */
static cplx dd_stencil(const orc_state* s, const double* c, int iy, int k, int ix, int iz) {
  cplx f[5];
  for (int j = 0; j < 5; ++j) f[j] = VVP(s, iy - 2 + j, k, ix, iz);
  return csum5(c, f);
}

void orc_buildrhs(orc_state* s, const double ode[3], int compute_cfl) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const int nthr = s->nthreads;
  double cflmax = s->cfl;
  /* convolutions of planes -1..ny+1 (dnsdata.f90:630-632) */
#pragma omp parallel num_threads(nthr) reduction(max : cflmax)
  {
    conv_ws w;
    conv_ws_init(s, &w);
#pragma omp for schedule(dynamic, 1)
    for (int iy = -1; iy <= ny + 1; ++iy) {
      double c = convolve_plane(s, iy, compute_cfl, &VVP(s, iy, 1, 0, -nz), &w);
      if (c > cflmax) cflmax = c;
    }
    conv_ws_free(&w);
  }
  s->cfl = cflmax;
  if (s->F) body_force_ghosts(s);
  const double dt = s->deltat, ni = s->p.ni;
  const double meanpx = s->meanpx, meanpz = s->meanpz;
#pragma omp parallel for num_threads(nthr) schedule(static)
  for (int iy = 1; iy <= ny - 1; ++iy) {
    const Di* d = &s->der[iy];
    for (int iz = -nz; iz <= nz; ++iz)
      for (int ix = 0; ix <= nx; ++ix) {
        const cplx ialfa = CMPLX(0.0, ix * s->p.alfa0);
        const cplx ibeta = CMPLX(0.0, iz * s->p.beta0);
        const double k2 = K2(s, iz, ix);
#define DD(cf, k) dd_stencil(s, d->cf, iy, k, ix, iz)
        const cplx DD0_6 = DD(d0, 6), DD1_6 = DD(d1, 6);
        const cplx rhsu = -(cmul(ialfa, DD(d0, 1))) - DD(d1, 4) - cmul(ibeta, DD0_6);
        const cplx rhsv = -(cmul(ialfa, DD(d0, 4))) - DD(d1, 2) - cmul(ibeta, DD(d0, 5));
        const cplx rhsw = -(cmul(ialfa, DD0_6)) - DD(d1, 5) - cmul(ibeta, DD(d0, 3));
        cplx expl = cmul(ialfa, cmul(ialfa, DD(d1, 1)) + DD(d2, 4) + cmul(ibeta, DD1_6)) +
                    cmul(ibeta, cmul(ialfa, DD1_6) + DD(d2, 5) + cmul(ibeta, DD(d1, 3))) - k2 * rhsv;
        if (s->F) /* dnsdata.f90:644 */
          expl = expl - k2 * fstencil(s, d->d0, iy, iz, ix, 2) - cmul(ialfa, fstencil(s, d->d1, iy, iz, ix, 1)) -
                 cmul(ibeta, fstencil(s, d->d1, iy, iz, ix, 3));
#undef DD
        cplx v2[5], v1[5], v3[5];
        for (int j = 0; j < 5; ++j) {
          v1[j] = V_(s, iy - 2 + j, iz, ix, 1);
          v2[j] = V_(s, iy - 2 + j, iz, ix, 2);
          v3[j] = V_(s, iy - 2 + j, iz, ix, 3);
        }
        const size_t r = RIDX(s, iy, iz, ix);
        /* timescheme for D2v (dnsdata.f90:486,647) */
        {
          cplx unkn = csum5(d->d2, v2) - k2 * csum5(d->d0, v2);
          cplx impl;
          {
            double os0 = ni * (d->d4[0] - 2.0 * k2 * d->d2[0] + k2 * k2 * d->d0[0]);
            impl = os0 * v2[0];
            for (int j = 1; j < 5; ++j) {
              double os = ni * (d->d4[j] - 2.0 * k2 * d->d2[j] + k2 * k2 * d->d0[j]);
              impl = impl + os * v2[j];
            }
          }
          cplx rhs = (ode[0] * unkn) / dt + impl + ode[1] * expl - ode[2] * s->old_d2v[r];
          s->old_d2v[r] = expl;
          s->newrhs_d2v[r] = rhs;
        }
        if (ix == 0 && iz == 0) { /* dnsdata.f90:648-654 */
          expl = CMPLX(creal(rhsu) + meanpx, creal(rhsw) + meanpz);
          if (s->F) { /* dnsdata.f90:651: rD0(F,1,3) */
            double r1[5], r3[5];
            for (int j = 0; j < 5; ++j) { r1[j] = creal(F_(s, iy - 2 + j, iz, ix, 1)); r3[j] = creal(F_(s, iy - 2 + j, iz, ix, 3)); }
            expl = expl + CMPLX(sum5(d->d0, r1), sum5(d->d0, r3));
          }
          double r1[5], r3[5];
          for (int j = 0; j < 5; ++j) { r1[j] = creal(v1[j]); r3[j] = creal(v3[j]); }
          cplx unkn = CMPLX(sum5(d->d0, r1), sum5(d->d0, r3));
          cplx impl = ni * CMPLX(sum5(d->d2, r1), sum5(d->d2, r3));
          cplx rhs = (ode[0] * unkn) / dt + impl + ode[1] * expl - ode[2] * s->old_eta[r];
          s->old_eta[r] = expl;
          s->newrhs_eta[r] = rhs;
        } else { /* dnsdata.f90:655-661 */
          expl = cmul(ibeta, rhsu) - cmul(ialfa, rhsw);
          if (s->F) /* dnsdata.f90:658 */
            expl = expl + cmul(ibeta, fstencil(s, d->d0, iy, iz, ix, 1)) - cmul(ialfa, fstencil(s, d->d0, iy, iz, ix, 3));
          cplx unkn = cmul(ibeta, csum5(d->d0, v1)) - cmul(ialfa, csum5(d->d0, v3));
          cplx impl;
          {
            double sq0 = ni * (d->d2[0] - k2 * d->d0[0]);
            impl = sq0 * (cmul(ibeta, v1[0]) - cmul(ialfa, v3[0]));
            for (int j = 1; j < 5; ++j) {
              double sq = ni * (d->d2[j] - k2 * d->d0[j]);
              impl = impl + sq * (cmul(ibeta, v1[j]) - cmul(ialfa, v3[j]));
            }
          }
          cplx rhs = (ode[0] * unkn) / dt + impl + ode[1] * expl - ode[2] * s->old_eta[r];
          s->old_eta[r] = expl;
          s->newrhs_eta[r] = rhs;
        }
      }
  }
  /* write-back (dnsdata.f90:667-670) */
  for (int iy = 1; iy <= ny - 1; ++iy)
    for (int ix = 0; ix <= nx; ++ix)
      for (int iz = -nz; iz <= nz; ++iz) {
        const size_t r = RIDX(s, iy, iz, ix);
        V_(s, iy, iz, ix, 1) = s->newrhs_eta[r];
        V_(s, iy, iz, ix, 2) = s->newrhs_d2v[r];
      }
}

/* ------------------------------------------------------------------ */
/* linsolve (linsolve_blocking.inc:3-107)                              */
/* ------------------------------------------------------------------ */
double orc_yintegr(const orc_state* s, const double* f) { /* dnsdata.f90:312-324, f indexed iy+1 */
  double II = 0.0;
  const double* y = s->y;
  for (int iy = 1; iy <= s->ny - 1; iy += 2) {
    double yp1 = y[YI(iy + 1)] - y[YI(iy)], ym1 = y[YI(iy - 1)] - y[YI(iy)];
    double a1 = -1.0 / 3.0 * ym1 + 1.0 / 6.0 * yp1 + 1.0 / 6.0 * yp1 * yp1 / ym1;
    double a3 = +1.0 / 3.0 * yp1 - 1.0 / 6.0 * ym1 - 1.0 / 6.0 * ym1 * ym1 / yp1;
    double a2 = yp1 - ym1 - a1 - a3;
    II = II + a1 * f[YI(iy - 1)] + a2 * f[YI(iy)] + a3 * f[YI(iy + 1)];
  }
  return II;
}

/* COMPLEXderiv (dnsdata.f90:339-373) followed by LeftLU5divStep2(D0mat). */
static void complex_deriv(const orc_state* s, const cplx* f0, cplx* f1) {
  const int ny = s->ny;
#define F0(iy) f0[YI(iy)]
#define F1(iy) f1[YI(iy)]
  F1(0) = csum5(s->d140, &F0(-1));
  F1(-1) = csum5(s->d14m1, &F0(-1));
  F1(ny) = csum5(s->d14n, &F0(ny - 3));
  F1(ny + 1) = csum5(s->d14np1, &F0(ny - 3));
  for (int iy = 1; iy <= ny - 1; ++iy) F1(iy) = csum5(s->der[iy].d1, &F0(iy - 2));
  F1(1) = F1(1) - (s->der[1].d0[1] * F1(0) + s->der[1].d0[0] * F1(-1));
  F1(2) = F1(2) - s->der[2].d0[0] * F1(0);
  F1(ny - 1) = F1(ny - 1) - (s->der[ny - 1].d0[3] * F1(ny) + s->der[ny - 1].d0[4] * F1(ny + 1));
  F1(ny - 2) = F1(ny - 2) - s->der[ny - 2].d0[4] * F1(ny);
  LeftLU5divStep1(f1, s->D0mat, ny + 1);
  LeftLU5divStep2(s->D0mat, f1, ny + 1);
#undef F0
#undef F1
}

void orc_deriv(const orc_state* s, const double* f0, double* f1) {
  complex_deriv(s, (const cplx*)f0, (cplx*)f1);
}

/* COMPLEXderiv2 (dnsdata.f90:378-414) followed by LeftLU5divStep2(D0mat):
 * the compact second derivative (REALderiv2, dnsdata.f90:438-451, is this on
 * a real line). */
static void complex_deriv2(const orc_state* s, const cplx* f0, cplx* f1) {
  const int ny = s->ny;
#define F0(iy) f0[YI(iy)]
#define F1(iy) f1[YI(iy)]
  F1(0) = csum5(s->d240, &F0(-1));
  F1(-1) = csum5(s->d24m1, &F0(-1));
  F1(ny) = csum5(s->d24n, &F0(ny - 3));
  F1(ny + 1) = csum5(s->d24np1, &F0(ny - 3));
  for (int iy = 1; iy <= ny - 1; ++iy) F1(iy) = csum5(s->der[iy].d2, &F0(iy - 2));
  F1(1) = F1(1) - (s->der[1].d0[1] * F1(0) + s->der[1].d0[0] * F1(-1));
  F1(2) = F1(2) - s->der[2].d0[0] * F1(0);
  F1(ny - 1) = F1(ny - 1) - (s->der[ny - 1].d0[3] * F1(ny) + s->der[ny - 1].d0[4] * F1(ny + 1));
  F1(ny - 2) = F1(ny - 2) - s->der[ny - 2].d0[4] * F1(ny);
  LeftLU5divStep1(f1, s->D0mat, ny + 1);
  LeftLU5divStep2(s->D0mat, f1, ny + 1);
#undef F0
#undef F1
}

void orc_deriv2(const orc_state* s, const double* f0, double* f1) {
  complex_deriv2(s, (const cplx*)f0, (cplx*)f1);
}

static void applybc_0(double* EQ, const double* bc0, const double* bc0m1) { /* dnsdata.f90:458-464 */
  /* EQ rows iy=1.. : EQ[(iy-1)*5 + j+2] */
  double* r1 = EQ;
  double* r2 = EQ + 5;
  double e = r1[0];
  for (int j = 1; j < 5; ++j) r1[j] = r1[j] - e * bc0m1[j] / bc0m1[0];
  e = r1[1];
  for (int j = 2; j < 5; ++j) r1[j] = r1[j] - e * bc0[j] / bc0[1];
  e = r2[0];
  for (int j = 1; j < 4; ++j) r2[j] = r2[j] - e * bc0[j + 1] / bc0[1];
}

static void applybc_n(double* EQ, int ny, const double* bcn, const double* bcnp1) { /* dnsdata.f90:466-472 */
  double* rn1 = EQ + (size_t)(ny - 2) * 5; /* iy=ny-1 */
  double* rn2 = EQ + (size_t)(ny - 3) * 5; /* iy=ny-2 */
  double e = rn1[4];
  for (int j = 0; j < 4; ++j) rn1[j] = rn1[j] - e * bcnp1[j] / bcnp1[4];
  e = rn1[3];
  for (int j = 0; j < 3; ++j) rn1[j] = rn1[j] - e * bcn[j] / bcn[3];
  e = rn2[4];
  for (int j = 1; j < 4; ++j) rn2[j] = rn2[j] - e * bcn[j - 1] / bcn[3];
}

void orc_linsolve(orc_state* s, double lambda) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const double ni = s->p.ni;
  const int nrow = ny + 1;
#pragma omp parallel num_threads(s->nthreads)
  {
    double* D2v = (double*)malloc(sizeof(double) * 5 * (size_t)nrow);
    double* eta = (double*)malloc(sizeof(double) * 5 * (size_t)nrow);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * (size_t)(ny + 3));
    cplx* lv = (cplx*)malloc(sizeof(cplx) * (size_t)(ny + 3));
    cplx* le = (cplx*)malloc(sizeof(cplx) * (size_t)(ny + 3));
    cplx* lw = (cplx*)malloc(sizeof(cplx) * (size_t)(ny + 3));
#pragma omp for schedule(dynamic, 1) collapse(2)
    for (int ix = 0; ix <= nx; ++ix)
      for (int iz = -nz; iz <= nz; ++iz) {
        const double k2 = K2(s, iz, ix);
        const cplx ialfa = CMPLX(0.0, ix * s->p.alfa0);
        const cplx ibeta = CMPLX(0.0, iz * s->p.beta0);
        memset(D2v, 0, sizeof(double) * 5 * (size_t)nrow);
        memset(eta, 0, sizeof(double) * 5 * (size_t)nrow);
        for (int iy = 1; iy <= ny - 1; ++iy) { /* :11-14 */
          const Di* d = &s->der[iy];
          for (int j = 0; j < 5; ++j) {
            double os = ni * (d->d4[j] - 2.0 * k2 * d->d2[j] + k2 * k2 * d->d0[j]);
            double sq = ni * (d->d2[j] - k2 * d->d0[j]);
            D2v[(size_t)(iy - 1) * 5 + j] = lambda * (d->d2[j] - k2 * d->d0[j]) - os;
            eta[(size_t)(iy - 1) * 5 + j] = lambda * d->d0[j] - sq;
          }
        }
        /* this mode's y-lines, iy=-1..ny+1 (index iy+1) */
        for (int iy = -1; iy <= ny + 1; ++iy) {
          lv[YI(iy)] = V_(s, iy, iz, ix, 2);
          le[YI(iy)] = V_(s, iy, iz, ix, 1);
        }
        /* boundary values (:15-42): walls at rest except the mean mode's
         * packed U+iW (channel.f90:122-124) */
        cplx b0v = 0, b0vy = 0, b0eta = 0, bnv = 0, bnvy = 0, bneta = 0;
        if (ix == 0 && iz == 0) {
          b0eta = CMPLX(s->p.u0, 0.0);
          bneta = CMPLX(s->p.uN, 0.0);
        } else {
          /* bc%vy = -ialfa*u - ibeta*w, bc%eta = ibeta*u - ialfa*w with u=w=0 */
        }
        b0v = b0v - s->v0bc[0] * b0vy / s->v0m1bc[0];
        applybc_0(D2v, s->v0bc, s->v0m1bc);
        lv[YI(1)] = lv[YI(1)] - D2v[0 * 5 + 0] * b0vy / s->v0m1bc[0] - D2v[0 * 5 + 1] * b0v / s->v0bc[1];
        lv[YI(2)] = lv[YI(2)] - D2v[1 * 5 + 0] * b0v / s->v0bc[1];
        applybc_0(eta, s->eta0bc, s->eta0m1bc);
        le[YI(1)] = le[YI(1)] - eta[0 * 5 + 1] * b0eta / s->eta0bc[1];
        le[YI(2)] = le[YI(2)] - eta[1 * 5 + 0] * b0eta / s->eta0bc[1];
        bnv = bnv - s->vnbc[4] * bnvy / s->vnp1bc[4];
        applybc_n(D2v, ny, s->vnbc, s->vnp1bc);
        lv[YI(ny - 1)] = lv[YI(ny - 1)] - D2v[(size_t)(ny - 2) * 5 + 4] * bnvy / s->vnp1bc[4] -
                         D2v[(size_t)(ny - 2) * 5 + 3] * bnv / s->vnbc[3];
        lv[YI(ny - 2)] = lv[YI(ny - 2)] - D2v[(size_t)(ny - 3) * 5 + 4] * bnv / s->vnbc[3];
        applybc_n(eta, ny, s->etanbc, s->etanp1bc);
        le[YI(ny - 1)] = le[YI(ny - 1)] - eta[(size_t)(ny - 2) * 5 + 3] * bneta / s->etanbc[3];
        le[YI(ny - 2)] = le[YI(ny - 2)] - eta[(size_t)(ny - 3) * 5 + 4] * bneta / s->etanbc[3];
        LU5decompStep(D2v, nrow);
        LU5decompStep(eta, nrow);
        LeftLU5divStep1(lv, D2v, nrow);
        LeftLU5divStep1(le, eta, nrow);
        LeftLU5divStep2(D2v, lv, nrow);
        LeftLU5divStep2(eta, le, nrow);
        /* wall and ghost values (:50-61) */
#define L(a, iy) a[YI(iy)]
        {
          cplx acc = L(lv, 1) * s->v0bc[2]; acc = acc + L(lv, 2) * s->v0bc[3]; acc = acc + L(lv, 3) * s->v0bc[4];
          L(lv, 0) = (b0v - acc) / s->v0bc[1];
          acc = L(lv, 0) * s->v0m1bc[1]; acc = acc + L(lv, 1) * s->v0m1bc[2]; acc = acc + L(lv, 2) * s->v0m1bc[3]; acc = acc + L(lv, 3) * s->v0m1bc[4];
          L(lv, -1) = (b0vy - acc) / s->v0m1bc[0];
          acc = L(le, 1) * s->eta0bc[2]; acc = acc + L(le, 2) * s->eta0bc[3]; acc = acc + L(le, 3) * s->eta0bc[4];
          L(le, 0) = (b0eta - acc) / s->eta0bc[1];
          acc = L(le, 0) * s->eta0m1bc[1]; acc = acc + L(le, 1) * s->eta0m1bc[2]; acc = acc + L(le, 2) * s->eta0m1bc[3]; acc = acc + L(le, 3) * s->eta0m1bc[4];
          L(le, -1) = -acc / s->eta0m1bc[0];
          acc = L(lv, ny - 3) * s->vnbc[0]; acc = acc + L(lv, ny - 2) * s->vnbc[1]; acc = acc + L(lv, ny - 1) * s->vnbc[2];
          L(lv, ny) = (bnv - acc) / s->vnbc[3];
          acc = L(lv, ny - 3) * s->vnp1bc[0]; acc = acc + L(lv, ny - 2) * s->vnp1bc[1]; acc = acc + L(lv, ny - 1) * s->vnp1bc[2]; acc = acc + L(lv, ny) * s->vnp1bc[3];
          L(lv, ny + 1) = (bnvy - acc) / s->vnp1bc[4];
          acc = L(le, ny - 3) * s->etanbc[0]; acc = acc + L(le, ny - 2) * s->etanbc[1]; acc = acc + L(le, ny - 1) * s->etanbc[2];
          L(le, ny) = (bneta - acc) / s->etanbc[3];
          acc = L(le, ny - 3) * s->etanp1bc[0]; acc = acc + L(le, ny - 2) * s->etanp1bc[1]; acc = acc + L(le, ny - 1) * s->etanp1bc[2]; acc = acc + L(le, ny) * s->etanp1bc[3];
          L(le, ny + 1) = -acc / s->etanp1bc[4];
        }
        if (ix == 0 && iz == 0) { /* :62-97 */
          double fU[ny + 3], fW[ny + 3], fc[ny + 3];
          for (int iy = -1; iy <= ny + 1; ++iy) {
            lw[YI(iy)] = CMPLX(cimag(L(le, iy)), 0.0);
            L(le, iy) = CMPLX(creal(L(le, iy)), 0.0);
          }
          for (int iy = -1; iy <= ny + 1; ++iy) tmp[YI(iy)] = (iy >= 1 && iy <= ny - 1) ? 1.0 : 0.0;
          LeftLU5divStep1(tmp, eta, nrow);
          LeftLU5divStep2(eta, tmp, nrow);
          {
            cplx acc = L(tmp, 1) * s->eta0bc[2]; acc = acc + L(tmp, 2) * s->eta0bc[3]; acc = acc + L(tmp, 3) * s->eta0bc[4];
            L(tmp, 0) = -acc / s->eta0bc[1];
            acc = L(tmp, 0) * s->eta0m1bc[1]; acc = acc + L(tmp, 1) * s->eta0m1bc[2]; acc = acc + L(tmp, 2) * s->eta0m1bc[3]; acc = acc + L(tmp, 3) * s->eta0m1bc[4];
            L(tmp, -1) = -acc / s->eta0m1bc[0];
            acc = L(tmp, ny - 3) * s->etanbc[0]; acc = acc + L(tmp, ny - 2) * s->etanbc[1]; acc = acc + L(tmp, ny - 1) * s->etanbc[2];
            L(tmp, ny) = -acc / s->etanbc[3];
            acc = L(tmp, ny - 3) * s->etanp1bc[0]; acc = acc + L(tmp, ny - 2) * s->etanp1bc[1]; acc = acc + L(tmp, ny - 1) * s->etanp1bc[2]; acc = acc + L(tmp, ny) * s->etanp1bc[3];
            L(tmp, ny + 1) = -acc / s->etanp1bc[4];
          }
          for (int iy = -1; iy <= ny + 1; ++iy) {
            fU[YI(iy)] = creal(L(le, iy));
            fW[YI(iy)] = creal(L(lw, iy));
            fc[YI(iy)] = creal(L(tmp, iy));
          }
          s->fr[0] = orc_yintegr(s, fU);
          s->fr[1] = orc_yintegr(s, fW);
          s->fr[2] = orc_yintegr(s, fc);
          if (fabs(s->p.meanflowx) > 1.0e-7 && !s->p.cpi) {
            s->corrpx = (s->p.meanflowx - s->fr[0]) / s->fr[2];
            for (int iy = -1; iy <= ny + 1; ++iy)
              L(le, iy) = CMPLX(creal(L(le, iy)) + s->corrpx * creal(L(tmp, iy)), cimag(L(le, iy)));
          }
          if (fabs(s->p.meanflowz) > 1.0e-7 && !s->p.cpi) {
            s->corrpz = (s->p.meanflowz - s->fr[1]) / s->fr[2];
            for (int iy = -1; iy <= ny + 1; ++iy)
              L(lw, iy) = CMPLX(creal(L(lw, iy)) + s->corrpz * creal(L(tmp, iy)), cimag(L(lw, iy)));
          }
          if (s->p.cpi) {
            if (s->p.cpi_type == 0) s->meanpx = (1 - s->p.gamma) * 6 * ni / s->fr[0];
            else s->meanpx = (1.5 / s->p.gamma) * s->fr[0] * ni;
          }
          for (int iy = -1; iy <= ny + 1; ++iy) {
            V_(s, iy, iz, ix, 1) = L(le, iy);
            V_(s, iy, iz, ix, 2) = L(lv, iy);
            V_(s, iy, iz, ix, 3) = L(lw, iy);
          }
        } else { /* :98-104 */
          complex_deriv(s, lv, lw);
          for (int iy = -1; iy <= ny + 1; ++iy) {
            cplx v3 = L(lw, iy), v1 = L(le, iy);
            cplx t = (cmul(ialfa, v3) - cmul(ibeta, v1)) / k2;
            cplx w = (cmul(ibeta, v3) + cmul(ialfa, v1)) / k2;
            V_(s, iy, iz, ix, 1) = t;
            V_(s, iy, iz, ix, 2) = L(lv, iy);
            V_(s, iy, iz, ix, 3) = w;
          }
        }
#undef L
      }
    free(D2v); free(eta); free(tmp); free(lv); free(le); free(lw);
  }
}

/* ------------------------------------------------------------------ */
/* Driver pieces (channel.f90, outstats)                               */
/* ------------------------------------------------------------------ */
double orc_initial_cfl(orc_state* s) { /* channel.f90:96-99 */
  const int ny = s->ny;
  double cflmax = s->cfl;
#pragma omp parallel num_threads(s->nthreads) reduction(max : cflmax)
  {
    conv_ws w;
    conv_ws_init(s, &w);
    cplx* out = (cplx*)malloc(sizeof(cplx) * 6 * (size_t)(s->nx + 1) * s->nzt);
#pragma omp for schedule(dynamic, 1)
    for (int iy = 1; iy <= ny - 1; ++iy) {
      double c = convolve_plane(s, iy, 1, out, &w);
      if (c > cflmax) cflmax = c;
    }
    free(out);
    conv_ws_free(&w);
  }
  s->cfl = cflmax;
  return cflmax;
}

void orc_initial_flowrate(orc_state* s) { /* channel.f90:101-115 */
  const int ny = s->ny;
  double fU[ny + 3], fW[ny + 3];
  for (int iy = -1; iy <= ny + 1; ++iy) {
    fU[YI(iy)] = creal(V_(s, iy, 0, 0, 1));
    fW[YI(iy)] = creal(V_(s, iy, 0, 0, 3));
  }
  s->fr[0] = orc_yintegr(s, fU);
  s->fr[1] = orc_yintegr(s, fW);
  s->fr[2] = 0.0; /* frl(3) of the driver is never assigned */
  if (s->p.cpi) {
    if (s->p.cpi_type == 0) s->meanpx = (1 - s->p.gamma) * 6 * s->p.ni / s->fr[0];
    else s->meanpx = (1.5 / s->p.gamma) * s->fr[0] * s->p.ni;
  }
}

void orc_outstats(orc_state* s, orc_line* line) { /* dnsdata.f90:853-880 */
  const int ny = s->ny;
  double runtime_global = s->cfl;
  s->cfl = 0;
  if (s->p.cflmax > 0) s->deltat = s->p.cflmax / runtime_global;
  double r[5];
  for (int j = 0; j < 5; ++j) r[j] = creal(V_(s, ny - 3 + j, 0, 0, 1));
  double d12 = -sum5(s->d14n, r);
  for (int j = 0; j < 5; ++j) r[j] = creal(V_(s, ny - 3 + j, 0, 0, 3));
  double d22 = -sum5(s->d14n, r);
  for (int j = 0; j < 5; ++j) r[j] = creal(V_(s, -1 + j, 0, 0, 1));
  double d11 = sum5(s->d140, r);
  for (int j = 0; j < 5; ++j) r[j] = creal(V_(s, -1 + j, 0, 0, 3));
  double d21 = sum5(s->d140, r);
  double* o = line->v;
  o[0] = s->time;
  o[1] = d11; o[2] = d12; o[3] = d21; o[4] = d22;
  o[5] = s->fr[0] + s->corrpx * s->fr[2];
  o[6] = s->meanpx + s->corrpx;
  o[7] = s->fr[1] + s->corrpz * s->fr[2];
  o[8] = s->meanpz + s->corrpz;
  o[9] = runtime_global * s->deltat;
  o[10] = s->deltat;
}

static const double RK[3][3] = {
    {120.0 / 32.0, 2.0, 0.0},
    {120.0 / 8.0, 50.0 / 8.0, 34.0 / 8.0},
    {120.0 / 20.0, 90.0 / 20.0, 50.0 / 20.0}}; /* dnsdata.f90:70-72 */

void orc_start(orc_state* s, orc_line* line) { /* channel.f90:64-116 */
  s->time0 = s->time;
  if (s->deltat == 0) s->deltat = 1.0; /* channel.f90:97 */
  orc_initial_cfl(s);
  orc_initial_flowrate(s);
  orc_outstats(s, line);
}

void orc_step(orc_state* s, orc_line* line) { /* channel.f90:118-167 */
  s->istep++;
  for (int k = 0; k < 3; ++k) {
    s->time = s->time + 2.0 / RK[k][0] * s->deltat;
    orc_buildrhs(s, RK[k], k == 2);
    orc_linsolve(s, RK[k][0] / s->deltat);
  }
  orc_outstats(s, line);
}

void orc_get_scalars(const orc_state* s, orc_scalars* o) {
  o->time = s->time; o->deltat = s->deltat; o->cfl = s->cfl;
  memcpy(o->fr, s->fr, sizeof o->fr);
  o->corrpx = s->corrpx; o->corrpz = s->corrpz; o->meanpx = s->meanpx; o->meanpz = s->meanpz;
  o->istep = s->istep;
}
void orc_set_scalars(orc_state* s, const orc_scalars* i) {
  s->time = i->time; s->deltat = i->deltat; s->cfl = i->cfl;
  memcpy(s->fr, i->fr, sizeof s->fr);
  s->corrpx = i->corrpx; s->corrpz = i->corrpz; s->meanpx = i->meanpx; s->meanpz = i->meanpz;
  s->istep = i->istep;
}
