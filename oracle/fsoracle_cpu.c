/*
 * fsoracle_cpu.c -- f64 restatement of the reference CPU solver.
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never the product.
 *
 * Each function names the reference function it restates (fluid-sim paths).
 * Floating-point operations are kept in the reference's order; the file is
 * compiled with -ffp-contract=off so no a*b+c is fused, which keeps results
 * identical on x86-64 and aarch64 hosts.
 */
#include "fsoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void fso_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
#define OMP_ROWS _Pragma("omp parallel for schedule(static) num_threads(g_threads) if(g_threads > 1)")

/* JavaScript Math.round: floor(x + 0.5) (ties toward +inf). */
static double js_round(double x) { return floor(x + 0.5); }

/* ================================================================ grid.js */

/* src/core/grid.js:51-69 */
void fso_grid_init(fso_grid* g, int nx, int ny, double lx, double ly) {
  g->nx = nx; g->ny = ny; g->lx = lx; g->ly = ly;
  g->dx = lx / nx; g->dy = ly / ny;
}

/* src/core/grid.js:40 */
int fso_wrap(int i, int n) { return ((i % n) + n) % n; }

static inline int64_t wrap64(int64_t i, int64_t n) { return ((i % n) + n) % n; }

/* test/core.test.js:94-98: s = (s*1103515245 + 12345) & 0x7fffffff in JS doubles.
 * The product exceeds 2^53 and is rounded as a double before ToInt32 wraps it
 * mod 2^32; fmod on the (integer-valued) double reproduces that exactly. */
static inline uint32_t js_lcg_next(uint32_t s) {
  double t = (double)s * 1103515245.0;
  t = t + 12345.0;
  double m = fmod(t, 4294967296.0);
  uint32_t lo = (uint32_t)m;
  return lo & 0x7fffffffu;
}

uint32_t fso_lcg_fill(uint32_t seed, int64_t n, double* out) {
  uint32_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    s = js_lcg_next(s);
    out[i] = (double)s / 2147483647.0 - 0.5;
  }
  return s;
}

uint32_t fso_lcg_fill_uv(uint32_t seed, int64_t n, double* u, double* v) {
  uint32_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    s = js_lcg_next(s);
    u[i] = (double)s / 2147483647.0 - 0.5;
    s = js_lcg_next(s);
    v[i] = (double)s / 2147483647.0 - 0.5;
  }
  return s;
}

/* src/core/grid.js:147-164 */
double fso_bilerp(const double* arr, int nx, int ny, double gx, double gy) {
  double fi0 = floor(gx), fj0 = floor(gy);
  double fx = gx - fi0, fy = gy - fj0;
  int64_t i0 = (int64_t)fi0, j0 = (int64_t)fj0;
  int64_t i0w = wrap64(i0, nx), i1w = wrap64(i0 + 1, nx);
  int64_t j0w = wrap64(j0, ny), j1w = wrap64(j0 + 1, ny);
  double a = arr[j0w * nx + i0w];
  double b = arr[j0w * nx + i1w];
  double c = arr[j1w * nx + i0w];
  double d = arr[j1w * nx + i1w];
  double top = a + (b - a) * fx;
  double bot = c + (d - c) * fx;
  return top + (bot - top) * fy;
}

/* src/core/grid.js:167-180 */
double fso_sample_u(const fso_grid* g, const double* u, double x, double y) {
  return fso_bilerp(u, g->nx, g->ny, x / g->dx, y / g->dy - 0.5);
}
double fso_sample_v(const fso_grid* g, const double* v, double x, double y) {
  return fso_bilerp(v, g->nx, g->ny, x / g->dx - 0.5, y / g->dy);
}
double fso_sample_p(const fso_grid* g, const double* p, double x, double y) {
  return fso_bilerp(p, g->nx, g->ny, x / g->dx - 0.5, y / g->dy - 0.5);
}

#define IDX(g, i, j) ((int64_t)fso_wrap((j), (g)->ny) * (g)->nx + fso_wrap((i), (g)->nx))
static inline double uX(const fso_grid* g, int i) { return i * g->dx; }
static inline double uY(const fso_grid* g, int j) { return (j + 0.5) * g->dy; }
static inline double vX(const fso_grid* g, int i) { return (i + 0.5) * g->dx; }
static inline double vY(const fso_grid* g, int j) { return j * g->dy; }
static inline double pX(const fso_grid* g, int i) { return (i + 0.5) * g->dx; }
static inline double pY(const fso_grid* g, int j) { return (j + 0.5) * g->dy; }

/* src/core/grid.js:191-206 */
void fso_divergence(const fso_grid* g, const double* u, const double* v, double* out) {
  const int nx = g->nx, ny = g->ny;
  const double dx = g->dx, dy = g->dy;
  OMP_ROWS
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      double uL = u[IDX(g, i, j)], uR = u[IDX(g, i + 1, j)];
      double vB = v[IDX(g, i, j)], vT = v[IDX(g, i, j + 1)];
      out[IDX(g, i, j)] = (uR - uL) / dx + (vT - vB) / dy;
    }
  }
}

/* src/core/grid.js:209-218 */
void fso_subtract_gradient(const fso_grid* g, double* u, double* v, const double* p, double scale) {
  const int nx = g->nx, ny = g->ny;
  OMP_ROWS
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      u[IDX(g, i, j)] -= scale * (p[IDX(g, i, j)] - p[IDX(g, i - 1, j)]) / g->dx;
      v[IDX(g, i, j)] -= scale * (p[IDX(g, i, j)] - p[IDX(g, i, j - 1)]) / g->dy;
    }
  }
}

/* src/core/grid.js:228-239 */
void fso_vorticity_corner(const fso_grid* g, const double* u, const double* v, double* out) {
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double dvdx = (v[IDX(g, i, j)] - v[IDX(g, i - 1, j)]) / g->dx;
      double dudy = (u[IDX(g, i, j)] - u[IDX(g, i, j - 1)]) / g->dy;
      out[(int64_t)j * g->nx + i] = dvdx - dudy;
    }
  }
}

/* src/core/grid.js:242-257 */
void fso_vorticity_center(const fso_grid* g, const double* u, const double* v, double* out) {
  const int nx = g->nx, ny = g->ny;
  double* c = (double*)malloc(sizeof(double) * (size_t)nx * ny);
  fso_vorticity_corner(g, u, v, c);
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      out[IDX(g, i, j)] = 0.25 * (c[(int64_t)fso_wrap(j, ny) * nx + fso_wrap(i, nx)] +
                                  c[(int64_t)fso_wrap(j, ny) * nx + fso_wrap(i + 1, nx)] +
                                  c[(int64_t)fso_wrap(j + 1, ny) * nx + fso_wrap(i, nx)] +
                                  c[(int64_t)fso_wrap(j + 1, ny) * nx + fso_wrap(i + 1, nx)]);
    }
  }
  free(c);
}

/* src/core/grid.js:267-278 */
void fso_velocity_at_centers(const fso_grid* g, const double* u, const double* v, double* cu, double* cv) {
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      cu[IDX(g, i, j)] = 0.5 * (u[IDX(g, i, j)] + u[IDX(g, i + 1, j)]);
      cv[IDX(g, i, j)] = 0.5 * (v[IDX(g, i, j)] + v[IDX(g, i, j + 1)]);
    }
  }
}

/* src/core/grid.js:290-295 */
double fso_kinetic_energy(const fso_grid* g, const double* u, const double* v) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* cu = (double*)malloc(sizeof(double) * n);
  double* cv = (double*)malloc(sizeof(double) * n);
  fso_velocity_at_centers(g, u, v, cu, cv);
  double s = 0;
  for (int64_t k = 0; k < n; k++) s += cu[k] * cu[k] + cv[k] * cv[k];
  free(cu); free(cv);
  return 0.5 * s / n;
}

/* src/core/grid.js:298-303 */
double fso_enstrophy(const fso_grid* g, const double* u, const double* v) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* w = (double*)malloc(sizeof(double) * n);
  fso_vorticity_center(g, u, v, w);
  double s = 0;
  for (int64_t k = 0; k < n; k++) s += w[k] * w[k];
  free(w);
  return 0.5 * s / n;
}

/* src/core/grid.js:306-311 */
double fso_max_divergence(const fso_grid* g, const double* u, const double* v) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* d = (double*)malloc(sizeof(double) * n);
  fso_divergence(g, u, v, d);
  double m = 0;
  for (int64_t k = 0; k < n; k++) m = fmax(m, fabs(d[k]));
  free(d);
  return m;
}

/* src/core/grid.js:314-319 */
double fso_l2_divergence(const fso_grid* g, const double* u, const double* v) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* d = (double*)malloc(sizeof(double) * n);
  fso_divergence(g, u, v, d);
  double s = 0;
  for (int64_t k = 0; k < n; k++) s += d[k] * d[k];
  free(d);
  return sqrt(s / n);
}

/* src/core/grid.js:322-327 */
double fso_cfl(const fso_grid* g, const double* u, const double* v, double dt) {
  int64_t n = (int64_t)g->nx * g->ny;
  double mu = 0, mv = 0;
  for (int64_t k = 0; k < n; k++) mu = fmax(mu, fabs(u[k]));
  for (int64_t k = 0; k < n; k++) mv = fmax(mv, fabs(v[k]));
  return dt * (mu / g->dx + mv / g->dy);
}

/* ============================================================ analytic.js */

/* src/core/analytic.js:42-43,67-71 */
void fso_tg_init(const fso_grid* g, double* u, double* v, double t, double nu) {
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double x = uX(g, i), y = uY(g, j);
      u[IDX(g, i, j)] = sin(x) * cos(y) * exp(-2 * nu * t);
    }
  }
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double x = vX(g, i), y = vY(g, j);
      v[IDX(g, i, j)] = -cos(x) * sin(y) * exp(-2 * nu * t);
    }
  }
}

/* src/core/analytic.js:195-206 */
double fso_tg_velocity_error(const fso_grid* g, const double* u, const double* v, double t, double nu) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* eu = (double*)malloc(sizeof(double) * n);
  double* ev = (double*)malloc(sizeof(double) * n);
  fso_tg_init(g, eu, ev, t, nu);
  double num = 0, den = 0;
  for (int64_t k = 0; k < n; k++) {
    double du = u[k] - eu[k], dv = v[k] - ev[k];
    num += du * du + dv * dv;
    den += eu[k] * eu[k] + ev[k] * ev[k];
  }
  free(eu); free(ev);
  if (den < 1e-300) return sqrt(num / (2 * n));
  return sqrt(num / den);
}

/* src/core/analytic.js:155-167 */
double fso_rel_l2(const double* a, const double* exact, int64_t n) {
  double num = 0, den = 0;
  for (int64_t k = 0; k < n; k++) {
    double d = a[k] - exact[k];
    num += d * d;
    den += exact[k] * exact[k];
  }
  if (den < 1e-300) return sqrt(num / n);
  return sqrt(num / den);
}

/* src/core/analytic.js:109-124 */
double fso_gaussian_scalar(double x, double y, double t, double sigma, double ax, double ay,
                           double cx, double cy) {
  const double L = 2 * M_PI;
  double mx = cx + ax * t, my = cy + ay * t;
  double s = 0;
  for (int p = -3; p <= 3; p++) {
    for (int q = -3; q <= 3; q++) {
      double dx = x - mx + p * L;
      double dy = y - my + q * L;
      s += exp(-(dx * dx + dy * dy) / (2 * sigma * sigma));
    }
  }
  return s;
}

/* ================================================================= fft.js */

/* src/core/fft.js:24-26 */
int fso_is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* src/core/fft.js:33-69: bit reversal then butterflies with a twiddle recurrence */
void fso_fft_inplace(double* re, double* im, int n, int sign) {
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    double ang = sign * 2 * M_PI / len;
    double wr = cos(ang), wi = sin(ang);
    int half = len / 2;
    for (int i = 0; i < n; i += len) {
      double cr = 1, ci = 0;
      for (int k = 0; k < half; k++) {
        double ar = re[i + k], ai = im[i + k];
        double br = re[i + k + half], bi = im[i + k + half];
        double dr = br * cr - bi * ci;
        double di = br * ci + bi * cr;
        re[i + k] = ar + dr; im[i + k] = ai + di;
        re[i + k + half] = ar - dr;
        im[i + k + half] = ai - di;
        double ncr = cr * wr - ci * wi;
        ci = cr * wi + ci * wr;
        cr = ncr;
      }
    }
  }
}

/* src/core/fft.js:90-106 */
void fso_dft_naive(const double* re_in, const double* im_in, double* re, double* im, int n, int sign) {
  for (int k = 0; k < n; k++) {
    double sr = 0, si = 0;
    for (int t = 0; t < n; t++) {
      double a = sign * 2 * M_PI * k * t / n;
      double c = cos(a), s = sin(a);
      double i0 = im_in ? im_in[t] : 0.0;
      sr += re_in[t] * c - i0 * s;
      si += re_in[t] * s + i0 * c;
    }
    re[k] = sr; im[k] = si;
  }
}

static void fft2_core(double* re, double* im, int nx, int ny, int sign) {
  OMP_ROWS
  for (int j = 0; j < ny; j++) fso_fft_inplace(re + (int64_t)j * nx, im + (int64_t)j * nx, nx, sign);
  OMP_ROWS
  for (int i = 0; i < nx; i++) {
    double* colR = (double*)malloc(sizeof(double) * ny);
    double* colI = (double*)malloc(sizeof(double) * ny);
    for (int j = 0; j < ny; j++) { colR[j] = re[(int64_t)j * nx + i]; colI[j] = im[(int64_t)j * nx + i]; }
    fso_fft_inplace(colR, colI, ny, sign);
    for (int j = 0; j < ny; j++) { re[(int64_t)j * nx + i] = colR[j]; im[(int64_t)j * nx + i] = colI[j]; }
    free(colR); free(colI);
  }
}

/* src/core/fft.js:112-133 */
int fso_fft2(const double* field, int nx, int ny, double* re, double* im) {
  if (!fso_is_pow2(nx) || !fso_is_pow2(ny)) return -1;
  int64_t n = (int64_t)nx * ny;
  memcpy(re, field, sizeof(double) * n);
  memset(im, 0, sizeof(double) * n);
  fft2_core(re, im, nx, ny, -1);
  return 0;
}

/* src/core/fft.js:138-157 */
int fso_ifft2(const double* re0, const double* im0, int nx, int ny, double* re, double* im) {
  if (!fso_is_pow2(nx) || !fso_is_pow2(ny)) return -1;
  int64_t n = (int64_t)nx * ny;
  memcpy(re, re0, sizeof(double) * n);
  memcpy(im, im0, sizeof(double) * n);
  fft2_core(re, im, nx, ny, +1);
  for (int64_t i = 0; i < n; i++) { re[i] /= n; im[i] /= n; }
  return 0;
}

static inline int freq_index(int i, int n) { return i <= n / 2 ? i : i - n; }

/* src/core/fft.js:196-234 */
int fso_energy_spectrum(const double* cu, const double* cv, int nx, int ny, double* E, int32_t* counts) {
  if (!fso_is_pow2(nx) || !fso_is_pow2(ny)) return -1;
  int64_t N = (int64_t)nx * ny;
  double* ur = (double*)malloc(sizeof(double) * N); double* ui = (double*)malloc(sizeof(double) * N);
  double* vr = (double*)malloc(sizeof(double) * N); double* vi = (double*)malloc(sizeof(double) * N);
  fso_fft2(cu, nx, ny, ur, ui);
  fso_fft2(cv, nx, ny, vr, vi);
  int kmax = (nx < ny ? nx : ny) / 2;
  for (int k = 0; k <= kmax; k++) { E[k] = 0; counts[k] = 0; }
  double NN = (double)N * (double)N;
  for (int j = 0; j < ny; j++) {
    int ky = freq_index(j, ny);
    for (int i = 0; i < nx; i++) {
      int kx = freq_index(i, nx);
      int64_t idx = (int64_t)j * nx + i;
      double pu = (ur[idx] * ur[idx] + ui[idx] * ui[idx]) / NN;
      double pv = (vr[idx] * vr[idx] + vi[idx] * vi[idx]) / NN;
      double e = 0.5 * (pu + pv);
      double kmag = sqrt((double)kx * kx + (double)ky * ky);
      int shell = (int)js_round(kmag);
      if (shell <= kmax) { E[shell] += e; counts[shell]++; }
    }
  }
  free(ur); free(ui); free(vr); free(vi);
  return kmax;
}

/* ============================================================== advect.js */

/* src/cpu/advect.js:46-54: RK2 midpoint backward trace */
static inline void trace_back(const fso_grid* g, const double* u, const double* v, double x, double y,
                              double dt, double* ox, double* oy) {
  double u1 = fso_sample_u(g, u, x, y);
  double v1 = fso_sample_v(g, v, x, y);
  double xm = x - 0.5 * dt * u1;
  double ym = y - 0.5 * dt * v1;
  double u2 = fso_sample_u(g, u, xm, ym);
  double v2 = fso_sample_v(g, v, xm, ym);
  *ox = x - dt * u2;
  *oy = y - dt * v2;
}

/* src/cpu/advect.js:61-71 */
static void advect_scalar_sl(const fso_grid* g, const double* u, const double* v, const double* q,
                             double* out, double dt) {
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double x, y;
      trace_back(g, u, v, pX(g, i), pY(g, j), dt, &x, &y);
      out[IDX(g, i, j)] = fso_sample_p(g, q, x, y);
    }
  }
}

/* src/cpu/advect.js:74-97: u and v traced from their own staggered positions */
static void advect_velocity_sl(const fso_grid* g, const double* u, const double* v, double* ou,
                               double* ov, double dt) {
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double x, y;
      trace_back(g, u, v, uX(g, i), uY(g, j), dt, &x, &y);
      ou[IDX(g, i, j)] = fso_sample_u(g, u, x, y);
    }
  }
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double x, y;
      trace_back(g, u, v, vX(g, i), vY(g, j), dt, &x, &y);
      ov[IDX(g, i, j)] = fso_sample_v(g, v, x, y);
    }
  }
}

/* src/cpu/advect.js:104-111 */
static inline void interp_bounds(const double* arr, int nx, int ny, double gx, double gy, double* lo,
                                 double* hi) {
  int64_t i0 = (int64_t)floor(gx), j0 = (int64_t)floor(gy);
  int64_t i0w = wrap64(i0, nx), i1w = wrap64(i0 + 1, nx);
  int64_t j0w = wrap64(j0, ny), j1w = wrap64(j0 + 1, ny);
  double a = arr[j0w * nx + i0w], b = arr[j0w * nx + i1w];
  double c = arr[j1w * nx + i0w], d = arr[j1w * nx + i1w];
  *lo = fmin(fmin(a, b), fmin(c, d));
  *hi = fmax(fmax(a, b), fmax(c, d));
}

static inline double clamp_js(double c, double lo, double hi) { return c < lo ? lo : c > hi ? hi : c; }

/* src/cpu/advect.js:120-146 */
static void advect_scalar_mc(const fso_grid* g, const double* u, const double* v, const double* q,
                             double* out, double dt) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* fwd = (double*)malloc(sizeof(double) * n);
  double* back = (double*)malloc(sizeof(double) * n);
  advect_scalar_sl(g, u, v, q, fwd, dt);
  advect_scalar_sl(g, u, v, fwd, back, -dt);
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      int64_t k = IDX(g, i, j);
      double corrected = fwd[k] + 0.5 * (q[k] - back[k]);
      double x, y, lo, hi;
      trace_back(g, u, v, pX(g, i), pY(g, j), dt, &x, &y);
      interp_bounds(q, g->nx, g->ny, x / g->dx - 0.5, y / g->dy - 0.5, &lo, &hi);
      out[k] = clamp_js(corrected, lo, hi);
    }
  }
  free(fwd); free(back);
}

/* src/cpu/advect.js:192-206 */
static void advect_component_with(const fso_grid* g, const double* u, const double* v,
                                  const double* field, double* out, double dt, int is_u) {
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double px = is_u ? uX(g, i) : vX(g, i);
      double py = is_u ? uY(g, j) : vY(g, j);
      double x, y;
      trace_back(g, u, v, px, py, dt, &x, &y);
      out[IDX(g, i, j)] = is_u ? fso_bilerp(field, g->nx, g->ny, x / g->dx, y / g->dy - 0.5)
                               : fso_bilerp(field, g->nx, g->ny, x / g->dx - 0.5, y / g->dy);
    }
  }
}

/* src/cpu/advect.js:149-185 */
static void advect_velocity_mc(const fso_grid* g, const double* u, const double* v, double* ou,
                               double* ov, double dt) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* fu = (double*)malloc(sizeof(double) * n); double* fv = (double*)malloc(sizeof(double) * n);
  double* bu = (double*)malloc(sizeof(double) * n); double* bv = (double*)malloc(sizeof(double) * n);
  advect_velocity_sl(g, u, v, fu, fv, dt);
  advect_component_with(g, u, v, fu, bu, -dt, 1);
  advect_component_with(g, u, v, fv, bv, -dt, 0);
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      int64_t k = IDX(g, i, j);
      double corrected = fu[k] + 0.5 * (u[k] - bu[k]);
      double x, y, lo, hi;
      trace_back(g, u, v, uX(g, i), uY(g, j), dt, &x, &y);
      interp_bounds(u, g->nx, g->ny, x / g->dx, y / g->dy - 0.5, &lo, &hi);
      ou[k] = clamp_js(corrected, lo, hi);
    }
  }
  OMP_ROWS
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      int64_t k = IDX(g, i, j);
      double corrected = fv[k] + 0.5 * (v[k] - bv[k]);
      double x, y, lo, hi;
      trace_back(g, u, v, vX(g, i), vY(g, j), dt, &x, &y);
      interp_bounds(v, g->nx, g->ny, x / g->dx - 0.5, y / g->dy, &lo, &hi);
      ov[k] = clamp_js(corrected, lo, hi);
    }
  }
  free(fu); free(fv); free(bu); free(bv);
}

/* src/cpu/advect.js:208-221 */
void fso_advect_velocity(const fso_grid* g, int scheme, const double* u, const double* v,
                         double* out_u, double* out_v, double dt) {
  if (scheme == FSO_MACCORMACK) advect_velocity_mc(g, u, v, out_u, out_v, dt);
  else advect_velocity_sl(g, u, v, out_u, out_v, dt);
}
void fso_advect_scalar(const fso_grid* g, int scheme, const double* u, const double* v,
                       const double* q, double* out, double dt) {
  if (scheme == FSO_MACCORMACK) advect_scalar_mc(g, u, v, q, out, dt);
  else advect_scalar_sl(g, u, v, q, out, dt);
}

/* ========================================================== projection.js */

/* src/cpu/projection.js:48-62 */
void fso_laplacian(const fso_grid* g, const double* p, double* out) {
  const int nx = g->nx, ny = g->ny;
  const double ix = 1 / (g->dx * g->dx), iy = 1 / (g->dy * g->dy);
  OMP_ROWS
  for (int j = 0; j < ny; j++) {
    int64_t jm = (int64_t)fso_wrap(j - 1, ny) * nx, jp = (int64_t)fso_wrap(j + 1, ny) * nx, j0 = (int64_t)j * nx;
    for (int i = 0; i < nx; i++) {
      int im = fso_wrap(i - 1, nx), ip = fso_wrap(i + 1, nx);
      out[j0 + i] = (p[j0 + im] - 2 * p[j0 + i] + p[j0 + ip]) * ix +
                    (p[jm + i] - 2 * p[j0 + i] + p[jp + i]) * iy;
    }
  }
}

static double dot(const double* a, const double* b, int64_t n) {
  double s = 0;
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* src/cpu/projection.js:70-76 */
static double remove_mean(double* a, int64_t n) {
  double s = 0;
  for (int64_t i = 0; i < n; i++) s += a[i];
  double m = s / n;
  for (int64_t i = 0; i < n; i++) a[i] -= m;
  return m;
}

/* src/cpu/projection.js:87-139 */
int fso_poisson_cg(const fso_grid* g, const double* rhs, double* p, double tol, int max_iter,
                   double* residual_out, double* history, int history_cap) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* work = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  double* Ap = (double*)malloc(sizeof(double) * n);
  double* d = (double*)malloc(sizeof(double) * n);
  memcpy(work, rhs, sizeof(double) * n);
  remove_mean(work, n);
  memcpy(r, work, sizeof(double) * n);
  fso_laplacian(g, p, Ap);
  for (int64_t i = 0; i < n; i++) r[i] -= Ap[i];
  remove_mean(r, n);
  memcpy(d, r, sizeof(double) * n);
  double rr = dot(r, r, n);
  double rhs_norm = sqrt(dot(work, work, n));
  if (rhs_norm == 0) rhs_norm = 1;
  int iter = 0, nh = 0;
  double residual = sqrt(rr) / rhs_norm;
  if (residual <= tol) {
    if (history && history_cap > 0) history[0] = residual;
    if (residual_out) *residual_out = residual;
    free(work); free(r); free(Ap); free(d);
    return 0;
  }
  for (; iter < max_iter; iter++) {
    fso_laplacian(g, d, Ap);
    remove_mean(Ap, n);
    double dAd = dot(d, Ap, n);
    if (fabs(dAd) < 1e-300) break;
    double alpha = rr / dAd;
    for (int64_t i = 0; i < n; i++) {
      p[i] += alpha * d[i];
      r[i] -= alpha * Ap[i];
    }
    double rr_new = dot(r, r, n);
    residual = sqrt(rr_new) / rhs_norm;
    if (history && nh < history_cap) history[nh++] = residual;
    if (residual <= tol) { iter++; break; }
    double beta = rr_new / rr;
    for (int64_t i = 0; i < n; i++) d[i] = r[i] + beta * d[i];
    rr = rr_new;
  }
  remove_mean(p, n);
  if (residual_out) *residual_out = residual;
  free(work); free(r); free(Ap); free(d);
  return iter;
}

/* src/cpu/projection.js:239-248 */
double fso_poisson_residual(const fso_grid* g, const double* p, const double* rhs) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* Ap = (double*)malloc(sizeof(double) * n);
  fso_laplacian(g, p, Ap);
  double num = 0, den = 0;
  for (int64_t i = 0; i < n; i++) {
    double d = Ap[i] - rhs[i];
    num += d * d;
    den += rhs[i] * rhs[i];
  }
  free(Ap);
  double sd = sqrt(den);
  return sqrt(num) / (sd == 0 ? 1 : sd);
}

/* src/cpu/projection.js:151-180 */
int fso_poisson_jacobi(const fso_grid* g, const double* rhs, double* p, int iterations, double omega,
                       double* residual_out, double* history, int history_cap) {
  const int nx = g->nx, ny = g->ny;
  int64_t n = (int64_t)nx * ny;
  double h2 = g->dx * g->dx;
  double* cur = p;
  double* next = (double*)calloc(n, sizeof(double));
  double* spare = next;
  double* work = (double*)malloc(sizeof(double) * n);
  memcpy(work, rhs, sizeof(double) * n);
  remove_mean(work, n);
  double last = NAN;
  for (int it = 0; it < iterations; it++) {
    OMP_ROWS
    for (int j = 0; j < ny; j++) {
      int64_t jm = (int64_t)fso_wrap(j - 1, ny) * nx, jp = (int64_t)fso_wrap(j + 1, ny) * nx, j0 = (int64_t)j * nx;
      for (int i = 0; i < nx; i++) {
        int im = fso_wrap(i - 1, nx), ip = fso_wrap(i + 1, nx);
        double sum = cur[j0 + im] + cur[j0 + ip] + cur[jm + i] + cur[jp + i];
        double jac = (sum - h2 * work[j0 + i]) * 0.25;
        next[j0 + i] = cur[j0 + i] + omega * (jac - cur[j0 + i]);
      }
    }
    double* t = cur; cur = next; next = t;
    last = fso_poisson_residual(g, cur, work);
    if (history && it < history_cap) history[it] = last;
  }
  if (cur != p) memcpy(p, cur, sizeof(double) * n);
  remove_mean(p, n);
  if (residual_out) *residual_out = last;
  free(spare);
  free(work);
  return iterations;
}

/* src/cpu/projection.js:208-236: exact solve with the discrete eigenvalues */
int fso_poisson_fft(const fso_grid* g, const double* rhs, double* p) {
  const int nx = g->nx, ny = g->ny;
  if (!fso_is_pow2(nx) || !fso_is_pow2(ny)) return -1;
  int64_t n = (int64_t)nx * ny;
  double* re = (double*)malloc(sizeof(double) * n);
  double* im = (double*)malloc(sizeof(double) * n);
  fso_fft2(rhs, nx, ny, re, im);
  OMP_ROWS
  for (int j = 0; j < ny; j++) {
    double sy = sin(M_PI * j / ny);
    double ly = -4 * sy * sy / (g->dy * g->dy);
    for (int i = 0; i < nx; i++) {
      double sx = sin(M_PI * i / nx);
      double lx = -4 * sx * sx / (g->dx * g->dx);
      double lam = lx + ly;
      int64_t k = (int64_t)j * nx + i;
      if (i == 0 && j == 0) { re[k] = 0; im[k] = 0; }
      else { re[k] /= lam; im[k] /= lam; }
    }
  }
  double* pr = (double*)malloc(sizeof(double) * n);
  double* pi = (double*)malloc(sizeof(double) * n);
  fso_ifft2(re, im, nx, ny, pr, pi);
  memcpy(p, pr, sizeof(double) * n);
  free(re); free(im); free(pr); free(pi);
  return 1;
}

/* src/cpu/projection.js:259-266 */
int fso_project(const fso_grid* g, double* u, double* v, double* p, double tol, int max_iter,
                double* residual) {
  int64_t n = (int64_t)g->nx * g->ny;
  double* div = (double*)malloc(sizeof(double) * n);
  fso_divergence(g, u, v, div);
  int it = fso_poisson_cg(g, div, p, tol, max_iter, residual, NULL, 0);
  fso_subtract_gradient(g, u, v, p, 1);
  free(div);
  return it;
}

/* ============================================================== solver.js */

/* src/cpu/solver.js:52-112 */
int fso_diffuse(const fso_grid* g, const double* field, double* out, double nu, double dt,
                int explicit_, double tol, double* residual_out) {
  const int nx = g->nx, ny = g->ny;
  int64_t n = (int64_t)nx * ny;
  if (nu <= 0) {
    memcpy(out, field, sizeof(double) * n);
    if (residual_out) *residual_out = 0;
    return 0;
  }
  if (explicit_) {
    double alpha = nu * dt / (g->dx * g->dx);
    double beta = nu * dt / (g->dy * g->dy);
    OMP_ROWS
    for (int j = 0; j < ny; j++) {
      int64_t jm = (int64_t)fso_wrap(j - 1, ny) * nx, jp = (int64_t)fso_wrap(j + 1, ny) * nx, j0 = (int64_t)j * nx;
      for (int i = 0; i < nx; i++) {
        int im = fso_wrap(i - 1, nx), ip = fso_wrap(i + 1, nx);
        out[j0 + i] = field[j0 + i]
          + alpha * (field[j0 + im] - 2 * field[j0 + i] + field[j0 + ip])
          + beta * (field[jm + i] - 2 * field[j0 + i] + field[jp + i]);
      }
    }
    if (residual_out) *residual_out = 0;
    return 1;
  }
  /* CG on (I - nu dt lap), warm-started from the field */
  double k = nu * dt;
  double* r = (double*)calloc((size_t)n, sizeof(double));
  double* Ap = (double*)malloc(sizeof(double) * n);
  double* d = (double*)malloc(sizeof(double) * n);
  memcpy(out, field, sizeof(double) * n);
  fso_laplacian(g, out, Ap);
  for (int64_t i = 0; i < n; i++) Ap[i] = out[i] - k * Ap[i];
  for (int64_t i = 0; i < n; i++) r[i] = field[i] - Ap[i];
  memcpy(d, r, sizeof(double) * n);
  double rr = 0;
  for (int64_t i = 0; i < n; i++) rr += r[i] * r[i];
  double bsum = 0;
  for (int64_t i = 0; i < n; i++) bsum = bsum + field[i] * field[i];
  double b_norm = sqrt(bsum);
  if (b_norm == 0) b_norm = 1;
  int iterations = 0;
  for (int it = 0; it < 400; it++) {
    if (sqrt(rr) / b_norm <= tol) break;
    fso_laplacian(g, d, Ap);
    for (int64_t i = 0; i < n; i++) Ap[i] = d[i] - k * Ap[i];
    double dAd = 0;
    for (int64_t i = 0; i < n; i++) dAd += d[i] * Ap[i];
    if (fabs(dAd) < 1e-300) break;
    double alpha = rr / dAd;
    double rr_new = 0;
    for (int64_t i = 0; i < n; i++) {
      out[i] += alpha * d[i];
      r[i] -= alpha * Ap[i];
      rr_new += r[i] * r[i];
    }
    double beta = rr_new / rr;
    for (int64_t i = 0; i < n; i++) d[i] = r[i] + beta * d[i];
    rr = rr_new;
    iterations = it + 1;
  }
  if (residual_out) *residual_out = sqrt(rr) / b_norm;
  free(r); free(Ap); free(d);
  return iterations;
}

/* src/cpu/solver.js:232-237 */
void fso_linear_drag(double* u, double* v, int64_t n, double alpha, double dt) {
  if (alpha <= 0) return;
  double f = exp(-alpha * dt);
  for (int64_t i = 0; i < n; i++) u[i] *= f;
  for (int64_t i = 0; i < n; i++) v[i] *= f;
}

/* src/cpu/solver.js:179-217 */
void fso_band_forcing(const fso_grid* g, double* u, double* v, double kf, double width, double amp,
                      uint32_t seed, double dt) {
  uint32_t s = seed;
  struct { double kx, ky, phase; } modes[24];
  for (int n = 0; n < 24; n++) {
    s = (uint32_t)((uint64_t)s * 1664525u + 1013904223u); double r1 = s / 4294967296.0;
    double theta = 2 * M_PI * r1;
    s = (uint32_t)((uint64_t)s * 1664525u + 1013904223u); double r2 = s / 4294967296.0;
    double kmag = kf + (r2 - 0.5) * 2 * width;
    s = (uint32_t)((uint64_t)s * 1664525u + 1013904223u); double r3 = s / 4294967296.0;
    modes[n].kx = js_round(kmag * cos(theta));
    modes[n].ky = js_round(kmag * sin(theta));
    modes[n].phase = 2 * M_PI * r3;
  }
  double scale = amp * dt / sqrt(24.0);
  for (int m = 0; m < 24; m++) {
    if (modes[m].kx == 0 && modes[m].ky == 0) continue;
    double kk = modes[m].kx * modes[m].kx + modes[m].ky * modes[m].ky;
    for (int j = 0; j < g->ny; j++) {
      for (int i = 0; i < g->nx; i++) {
        double xu = uX(g, i), yu = uY(g, j);
        u[IDX(g, i, j)] += scale * (modes[m].ky / sqrt(kk)) *
                           cos(modes[m].kx * xu + modes[m].ky * yu + modes[m].phase);
        double xv = vX(g, i), yv = vY(g, j);
        v[IDX(g, i, j)] += scale * (-modes[m].kx / sqrt(kk)) *
                           cos(modes[m].kx * xv + modes[m].ky * yv + modes[m].phase);
      }
    }
  }
}

/* Philox4x32-10: ten rounds of two 32x32->64 multiplies (multipliers
 * 0xD2511F53, 0xCD9E8D57) with the Weyl key schedule (0x9E3779B9, 0xBB67AE85) */
void fso_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void fso_gauss_band_forcing(const fso_grid* g, double* u, double* v, double kf, double width, double amp,
                            uint64_t key, uint32_t counter, double dt) {
  const double lo = kf - width, hi = kf + width;
  const int K = (int)ceil(hi);
  int M = 0;
  for (int ky = -K; ky <= K; ky++)
    for (int kx = -K; kx <= K; kx++) {
      double kk = (double)kx * kx + (double)ky * ky;
      if (kk != 0 && kk >= lo * lo && kk <= hi * hi) M++;
    }
  if (M == 0) return;
  const double scale = amp * dt / sqrt((double)M);
  const uint32_t kw[2] = {(uint32_t)key, (uint32_t)(key >> 32)};
  int m = 0;
  for (int ky = -K; ky <= K; ky++)
    for (int kx = -K; kx <= K; kx++) {
      double kk = (double)kx * kx + (double)ky * ky;
      if (kk == 0 || kk < lo * lo || kk > hi * hi) continue;
      uint32_t ctr[4] = {counter, (uint32_t)m, 0u, 0u}, r[4];
      fso_philox4x32_10(ctr, kw, r);
      m++;
      double u1 = ((double)r[0] + 0.5) / 4294967296.0, u2 = ((double)r[1] + 0.5) / 4294967296.0;
      double A = sqrt(-2.0 * log(u1)), phi = 2 * M_PI * u2, k = sqrt(kk);
      for (int j = 0; j < g->ny; j++)
        for (int i = 0; i < g->nx; i++) {
          u[IDX(g, i, j)] += scale * A * (ky / k) * cos(kx * uX(g, i) + ky * uY(g, j) + phi);
          v[IDX(g, i, j)] += scale * A * (-kx / k) * cos(kx * vX(g, i) + ky * vY(g, j) + phi);
        }
    }
}

/* The GPU backend's FORCING kernel (src/gpu/shaders.js:532-566) in f64:
 * drag and forcing fused, drag applied to the incoming velocity. */
void fso_forcing_modes(const fso_grid* g, double* u, double* v, const fso_mode* modes, int m,
                       double amp, double drag, double drift_phase, double dt) {
  double scale = amp * dt / sqrt((double)m);
  double damp = exp(-drag * dt);
  for (int j = 0; j < g->ny; j++) {
    for (int i = 0; i < g->nx; i++) {
      double pux = i * g->dx, puy = (j + 0.5) * g->dy;
      double pvx = (i + 0.5) * g->dx, pvy = j * g->dy;
      double fu = 0, fv = 0;
      for (int k = 0; k < m; k++) {
        double kk = sqrt(modes[k].kx * modes[k].kx + modes[k].ky * modes[k].ky);
        if (kk < 1e-6) continue;
        fu = fu + (modes[k].ky / kk) * cos(modes[k].kx * pux + modes[k].ky * puy + modes[k].phase + drift_phase);
        fv = fv - (modes[k].kx / kk) * cos(modes[k].kx * pvx + modes[k].ky * pvy + modes[k].phase + drift_phase);
      }
      int64_t c = (int64_t)j * g->nx + i;
      u[c] = u[c] * damp + scale * fu;
      v[c] = v[c] * damp + scale * fv;
    }
  }
}

/* =============================================================== solid.js */

/* src/cpu/solid.js:38-40 */
static inline double wrap_delta(double d, double L) { return d - L * js_round(d / L); }

/* src/cpu/solid.js:53-94 */
void fso_disk_init(fso_disk* d, double x, double y, double r, double density, double vx, double vy,
                   double omega, int fixed, int added_mass_correction) {
  memset(d, 0, sizeof(*d));
  d->x = x; d->y = y; d->r = r; d->density = density;
  d->vx = vx; d->vy = vy; d->omega = omega; d->fixed = fixed;
  d->mass = density * M_PI * r * r;
  d->inertia = 0.5 * d->mass * r * r;
  d->added_mass_correction = added_mass_correction;
  d->added_mass = M_PI * r * r;
  d->effective_mass = d->mass + (added_mass_correction ? d->added_mass : 0);
  d->effective_inertia = d->inertia + (added_mass_correction ? 0.5 * d->added_mass * r * r : 0);
}

/* src/cpu/solid.js:101-106 */
double fso_disk_mask(const fso_disk* d, double px, double py, double lx, double ly, double width) {
  double dx = wrap_delta(px - d->x, lx);
  double dy = wrap_delta(py - d->y, ly);
  double dd = hypot(dx, dy) - d->r;
  return 0.5 * (1 - tanh(dd / width));
}

/* src/cpu/solid.js:117-128 */
void fso_disk_integrate(fso_disk* d, double dt, double gravity) {
  if (d->fixed) return;
  d->vx += (d->force[0] / d->effective_mass) * dt;
  d->vy += (d->force[1] / d->effective_mass) * dt + gravity * dt;
  d->omega += (d->torque / d->effective_inertia) * dt;
  d->x += d->vx * dt;
  d->y += d->vy * dt;
}

/* src/cpu/solid.js:165-233: direct forcing, multi-pass, Newton-3 reaction */
void fso_apply_coupling(const fso_grid* g, double* u, double* v, fso_disk* solids, int n_solids,
                        double dt, double mask_width, int passes, double* impulse_out) {
  const double lx = g->lx, ly = g->ly;
  const double width = mask_width * g->dx;
  const double dA = g->dx * g->dy;
  double impulse_x = 0, impulse_y = 0;
  for (int pass = 0; pass < passes; pass++) {
    for (int si = 0; si < n_solids; si++) {
      fso_disk* s = &solids[si];
      double fx = 0, fy = 0, tq = 0;
      for (int j = 0; j < g->ny; j++) {
        for (int i = 0; i < g->nx; i++) {
          double px = uX(g, i), py = uY(g, j);
          double chi = fso_disk_mask(s, px, py, lx, ly, width);
          if (chi < 1e-6) continue;
          int64_t k = IDX(g, i, j);
          double ddy = wrap_delta(py - s->y, ly);
          double su = s->vx - s->omega * ddy;
          double du = chi * (su - u[k]);
          u[k] += du;
          fx += du * dA;
          tq += -ddy * du * dA;
        }
      }
      for (int j = 0; j < g->ny; j++) {
        for (int i = 0; i < g->nx; i++) {
          double px = vX(g, i), py = vY(g, j);
          double chi = fso_disk_mask(s, px, py, lx, ly, width);
          if (chi < 1e-6) continue;
          int64_t k = IDX(g, i, j);
          double ddx = wrap_delta(px - s->x, lx);
          double sv = s->vy + s->omega * ddx;
          double dv = chi * (sv - v[k]);
          v[k] += dv;
          fy += dv * dA;
          tq += ddx * dv * dA;
        }
      }
      if (pass == 0) {
        s->last_impulse[0] = fx; s->last_impulse[1] = fy;
        s->force[0] = 0; s->force[1] = 0; s->torque = 0;
      } else {
        s->last_impulse[0] = s->last_impulse[0] + fx;
        s->last_impulse[1] = s->last_impulse[1] + fy;
      }
      s->force[0] = s->force[0] - fx / dt;
      s->force[1] = s->force[1] - fy / dt;
      s->torque -= tq / dt;
      impulse_x += fx;
      impulse_y += fy;
    }
  }
  if (impulse_out) { impulse_out[0] = impulse_x; impulse_out[1] = impulse_y; }
}

/* ============================================================ FluidSolver */

#define FSO_MAX_SOLIDS 64
struct fso_solver {
  fso_params prm;
  fso_grid g;
  double *u, *v, *dye, *p, *tu, *tv, *tq;
  double t;
  int steps;
  int last_iterations;
  double last_residual;
  int n_solids;
  fso_disk solids[FSO_MAX_SOLIDS];
  int n_modes;
  fso_mode* modes;
  double mode_amp, mode_drag, mode_drift;
  int channel_on;
  fso_channel channel;
};

/* defaults of src/cpu/solver.js:250-260 */
void fso_params_default(fso_params* p) {
  p->nx = 64; p->ny = 64;
  p->lx = 2 * M_PI; p->ly = 2 * M_PI;
  p->nu = 0.01;
  p->advection = FSO_SL;
  p->explicit_diffusion = 0;
  p->projection = FSO_PROJ_CG;
  p->proj_tol = 1e-10;
  p->proj_max_iter = 2000;
  p->mask_width = 1.5;
  p->coupling_passes = 2;
}

void fso_step_opts_default(fso_step_opts* o) {
  memset(o, 0, sizeof(*o));
  o->advect_dye = 1;
}

/* src/cpu/solver.js:250-323 (validation guards included) */
fso_solver* fso_create(const fso_params* p, int* err) {
  if (err) *err = 0;
  if (p->nx < 2 || p->ny < 2) { if (err) *err = 1; return NULL; }
  if (p->advection != FSO_SL && p->advection != FSO_MACCORMACK) { if (err) *err = 2; return NULL; }
  if (p->projection < 0 || p->projection > 2) { if (err) *err = 3; return NULL; }
  if (p->projection == FSO_PROJ_FFT && !(fso_is_pow2(p->nx) && fso_is_pow2(p->ny))) { if (err) *err = 4; return NULL; }
  fso_solver* s = (fso_solver*)calloc(1, sizeof(fso_solver));
  s->prm = *p;
  fso_grid_init(&s->g, p->nx, p->ny, p->lx, p->ly);
  int64_t n = (int64_t)p->nx * p->ny;
  s->u = (double*)calloc(n, sizeof(double)); s->v = (double*)calloc(n, sizeof(double));
  s->dye = (double*)calloc(n, sizeof(double)); s->p = (double*)calloc(n, sizeof(double));
  s->tu = (double*)calloc(n, sizeof(double)); s->tv = (double*)calloc(n, sizeof(double));
  s->tq = (double*)calloc(n, sizeof(double));
  return s;
}

void fso_destroy(fso_solver* s) {
  if (!s) return;
  free(s->u); free(s->v); free(s->dye); free(s->p); free(s->tu); free(s->tv); free(s->tq);
  free(s->modes);
  free(s);
}

double* fso_field(fso_solver* s, int which) {
  switch (which) {
    case 0: return s->u;
    case 1: return s->v;
    case 2: return s->p;
    case 3: return s->dye;
    default: return NULL;
  }
}
const fso_grid* fso_solver_grid(fso_solver* s) { return &s->g; }
int fso_add_solid(fso_solver* s, const fso_disk* d) {
  if (s->n_solids >= FSO_MAX_SOLIDS) return -1;
  s->solids[s->n_solids] = *d;
  return s->n_solids++;
}
fso_disk* fso_get_solid(fso_solver* s, int i) { return (i >= 0 && i < s->n_solids) ? &s->solids[i] : NULL; }

void fso_set_modes(fso_solver* s, const fso_mode* modes, int m, double amp, double drag, double drift) {
  free(s->modes);
  s->modes = NULL; s->n_modes = 0;
  if (m <= 0) return;
  s->modes = (fso_mode*)malloc(sizeof(fso_mode) * m);
  memcpy(s->modes, modes, sizeof(fso_mode) * m);
  s->n_modes = m; s->mode_amp = amp; s->mode_drag = drag; s->mode_drift = drift;
}

void fso_set_channel(fso_solver* s, const fso_channel* c) {
  s->channel_on = c != NULL;
  if (c) s->channel = *c;
}

/* 1/2 (1 - tanh((|d| - half) / w)), the disk mask's profile across a slab */
static double slab_chi(double d, double half, double w) { return 0.5 * (1 - tanh((fabs(d) - half) / w)); }

void fso_channel_forcing(const fso_grid* g, double* u, double* v, const fso_channel* c, double mask_width) {
  const double w = mask_width * g->dx;
  for (int j = 0; j < g->ny; j++)
    for (int i = 0; i < g->nx; i++) {
      int64_t k = IDX(g, i, j);
      double cu = slab_chi(wrap_delta(uX(g, i) - c->fringe_x, g->lx), c->fringe_half, c->fringe_ramp);
      double cv = slab_chi(wrap_delta(vX(g, i) - c->fringe_x, g->lx), c->fringe_half, c->fringe_ramp);
      if (cu >= 1e-6) u[k] += cu * (c->inflow_u - u[k]);
      if (cv >= 1e-6) v[k] += cv * (0.0 - v[k]);
      cu = slab_chi(wrap_delta(uY(g, j) - c->wall_y, g->ly), c->wall_half, w);
      cv = slab_chi(wrap_delta(vY(g, j) - c->wall_y, g->ly), c->wall_half, w);
      if (cu >= 1e-6) u[k] += cu * (0.0 - u[k]);
      if (cv >= 1e-6) v[k] += cv * (0.0 - v[k]);
    }
}

static void swap_ptr(double** a, double** b) { double* t = *a; *a = *b; *b = t; }

/* src/cpu/solver.js:336-398 */
void fso_step(fso_solver* s, double dt, const fso_step_opts* o) {
  fso_step_opts def;
  if (!o) { fso_step_opts_default(&def); o = &def; }
  const fso_grid* g = &s->g;
  int64_t n = (int64_t)g->nx * g->ny;

  fso_advect_velocity(g, s->prm.advection, s->u, s->v, s->tu, s->tv, dt);
  swap_ptr(&s->u, &s->tu); swap_ptr(&s->v, &s->tv);

  if (s->prm.nu > 0) {
    fso_diffuse(g, s->u, s->tu, s->prm.nu, dt, s->prm.explicit_diffusion, 1e-12, NULL);
    fso_diffuse(g, s->v, s->tv, s->prm.nu, dt, s->prm.explicit_diffusion, 1e-12, NULL);
    swap_ptr(&s->u, &s->tu); swap_ptr(&s->v, &s->tv);
  }

  if (o->band_forcing && o->band_kind == 1)
    fso_gauss_band_forcing(g, s->u, s->v, o->band_kf, o->band_width, o->band_amp, o->band_key, o->band_counter, dt);
  else if (o->band_forcing)
    fso_band_forcing(g, s->u, s->v, o->band_kf, o->band_width, o->band_amp, o->band_seed, dt);
  if (s->n_modes > 0)
    fso_forcing_modes(g, s->u, s->v, s->modes, s->n_modes, s->mode_amp, s->mode_drag,
                      s->mode_drift * s->t, dt);
  if (o->drag > 0) fso_linear_drag(s->u, s->v, n, o->drag, dt);
  if (s->channel_on) fso_channel_forcing(g, s->u, s->v, &s->channel, s->prm.mask_width);

  if (s->n_solids) {
    fso_apply_coupling(g, s->u, s->v, s->solids, s->n_solids, dt, s->prm.mask_width,
                       s->prm.coupling_passes, NULL);
    for (int i = 0; i < s->n_solids; i++) fso_disk_integrate(&s->solids[i], dt, o->gravity);
  }

  double* div = (double*)malloc(sizeof(double) * n);
  fso_divergence(g, s->u, s->v, div);
  memset(s->p, 0, sizeof(double) * n);
  double res = 0;
  if (s->prm.projection == FSO_PROJ_FFT) {
    s->last_iterations = fso_poisson_fft(g, div, s->p);
    res = 0;
  } else if (s->prm.projection == FSO_PROJ_JACOBI) {
    s->last_iterations = fso_poisson_jacobi(g, div, s->p, s->prm.proj_max_iter, 1.0, &res, NULL, 0);
  } else {
    s->last_iterations = fso_poisson_cg(g, div, s->p, s->prm.proj_tol, s->prm.proj_max_iter, &res, NULL, 0);
  }
  s->last_residual = res;
  fso_subtract_gradient(g, s->u, s->v, s->p, 1);
  free(div);

  if (o->advect_dye) {
    fso_advect_scalar(g, s->prm.advection, s->u, s->v, s->dye, s->tq, dt);
    swap_ptr(&s->dye, &s->tq);
  }
  s->t += dt;
  s->steps++;
}

double fso_time(fso_solver* s) { return s->t; }
int fso_steps(fso_solver* s) { return s->steps; }
int fso_last_iterations(fso_solver* s) { return s->last_iterations; }
double fso_last_residual(fso_solver* s) { return s->last_residual; }

/* src/cpu/solver.js:409-417 */
int fso_is_blown_up(fso_solver* s) {
  int64_t n = (int64_t)s->g.nx * s->g.ny;
  for (int64_t i = 0; i < n; i++) if (!isfinite(s->u[i])) return 1;
  for (int64_t i = 0; i < n; i++) if (!isfinite(s->v[i])) return 1;
  return 0;
}
