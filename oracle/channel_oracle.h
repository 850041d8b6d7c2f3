/*
 * channel_oracle.h -- CPU oracle (test infrastructure only).
 *
 * A plain-C FP64 restatement of davecats/channel's RK3/Crank-Nicolson time
 * step in the v-eta formulation.  It exists to check the CUDA library: only
 * the tests, the smoke check and the CPU-baseline leg of the benchmark may
 * load it.  Nothing in the product links against it.
 *
 * Parity status: the reference (Fortran + MPI + FFTW) ships no golden vectors
 * or known-answer tests, and cannot be built where this oracle is developed,
 * so the oracle is pinned by analytic known answers (polynomial exactness of
 * the compact stencils, FFT round trips against numpy, laminar Poiseuille
 * Runtimedata values, dealiased products of band-limited modes) and by
 * committed fixtures it generated itself.  Parity to the reference binary is
 * unpinned.
 *
 * Conventions (all follow the reference):
 *   - V is complex128, Fortran order V(iy,iz,ix,ic): iy=-1..ny+1 fastest,
 *     then iz=-nz..nz, ix=0..nx, ic=1..3 (u/eta, v, w)   [dnsdata.f90:132]
 *   - transforms are unnormalised with FFTW sign conventions:
 *     forward exp(-i), backward exp(+i)                  [ffts.f90:70-75]
 */
#ifndef CHANNEL_ORACLE_H
#define CHANNEL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* The twelve lines of dns.in after read_dnsin (dnsdata.f90:98-125). `ni` is
 * stored as read_dnsin leaves it, i.e. already inverted (1/Re). */
typedef struct orc_params {
  int nx, ny, nz;
  double alfa0, beta0;
  double ni;
  double a, ymin, ymax;
  int cpi, cpi_type;
  double gamma;
  double meanpx, meanpz;
  double meanflowx, meanflowz;
  double u0, uN;
  double deltat, cflmax, time;
  double dt_field, dt_save, t_max;
  int time_from_restart;
  long long nstep;
  int npy;
} orc_params;

typedef struct orc_state orc_state;

/* One Runtimedata line (dnsdata.f90:878): 11 doubles. */
typedef struct orc_line { double v[11]; } orc_line;

int orc_fftfit(int n);                                  /* ffts.f90:78-86 */
void orc_sizes(const orc_params* p, int* nxd, int* nzd);  /* dnsdata.f90:110-114 */

orc_state* orc_create(const orc_params* p, int nthreads);
void orc_destroy(orc_state* s);

/* Field access: interleaved complex128 in the restart-file order. */
void orc_set_field(orc_state* s, const double* V);
void orc_get_field(const orc_state* s, double* V);
long long orc_field_len(const orc_state* s); /* number of complex values */

/* Setup tables, for known-answer tests. Arrays are filled if non-NULL:
 *  y[ny+3] (iy=-1..ny+1), der[(ny-1)*20] (iy=1..ny-1: d0,d1,d2,d4 each 5),
 *  wall[10*5] = d040,d140,d240,d14m1,d24m1,d04n,d14n,d24n,d14np1,d24np1,
 *  bc[8*5] = v0bc,v0m1bc,eta0bc,eta0m1bc,vnbc,vnp1bc,etanbc,etanp1bc,
 *  d0mat[(ny+1)*5] (rows iy=1..ny+1 after LU5decompStep). */
void orc_tables(const orc_state* s, double* y, double* der, double* wall,
                double* bc, double* d0mat);

/* Hot-path pieces, following the reference routines one to one. */
void orc_buildrhs(orc_state* s, const double ode[3], int compute_cfl); /* dnsdata.f90:611 */
void orc_linsolve(orc_state* s, double lambda);        /* linsolve_blocking.inc:3 */
double orc_initial_cfl(orc_state* s);                  /* channel.f90:96-99 */
void orc_initial_flowrate(orc_state* s);               /* channel.f90:101-115 */
double orc_yintegr(const orc_state* s, const double* f); /* dnsdata.f90:312 */

/* Products of one y-plane (convolutions, dnsdata.f90:487-602): writes the
 * six truncated spectra uu,vv,ww,uv,vw,uw as out[6][nx+1][2nz+1] complex
 * (iz fastest, iz=-nz..nz) and returns the plane's CFL maximum. */
double orc_convolve_plane(orc_state* s, int iy, double* out);

/* Scalars that the reference keeps as module globals. */
typedef struct orc_scalars {
  double time, deltat, cfl;
  double fr[3];
  double corrpx, corrpz, meanpx, meanpz;
  long long istep;
} orc_scalars;
void orc_get_scalars(const orc_state* s, orc_scalars* out);
void orc_set_scalars(orc_state* s, const orc_scalars* in);

/* outstats (dnsdata.f90:853-880) without file output: fills one line. */
void orc_outstats(orc_state* s, orc_line* line);

/* One RK3 step of the time loop (channel.f90:118-167), including outstats. */
void orc_step(orc_state* s, orc_line* line);

/* The driver's start-up (channel.f90:64-116) given the field already set:
 * initial CFL pass, flow rate and CPI, first outstats line. */
void orc_start(orc_state* s, orc_line* line);

/* Body force F (bodyforce hook, dnsdata.f90:617-659): F has V's layout;
 * NULL switches it off.  buildrhs first rebuilds F's ghost rows
 * (dnsdata.f90:617-628) and adds F's terms to the explicit parts. */
void orc_set_body_force(orc_state* s, const double* F);

/* A subgrid stress tau[6][iy=1..ny-1][nzd][2nxd] (physical, the order of
 * the products uu vv ww uv vw uw) added to the products of the planes
 * iy = 1..ny-1 before their forward transforms -- the closure's insertion
 * point (no counterpart in the reference); NULL switches it off. */
void orc_set_tau(orc_state* s, const double* tau);

/* COMPLEXderiv followed by LeftLU5divStep2(D0mat) on one y-line
 * (dnsdata.f90:339-373): f0, f1 hold ny+3 complex values (iy=-1..ny+1). */
void orc_deriv(const orc_state* s, const double* f0, double* f1);
void orc_deriv2(const orc_state* s, const double* f0, double* f1);

/* Batched complex FFT of length n (n = 2^a or 3*2^a), unnormalised;
 * sign=-1 forward, +1 backward; data interleaved complex, `howmany` rows of
 * length n, contiguous. */
void orc_fft(int n, int sign, int howmany, double* data);

#ifdef __cplusplus
}
#endif
#endif
