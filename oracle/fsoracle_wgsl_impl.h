/*
 * fsoracle_wgsl_impl.h -- restatement of the reference's GPU algorithm.
 * TEST INFRASTRUCTURE ONLY.  Included twice by fsoracle_wgsl.c with
 * REAL = float (suffix f32) and REAL = double (suffix f64).
 *
 * Kernels follow src/gpu/shaders.js and src/gpu/multigrid.js one function per
 * WGSL entry point, with the WGSL expression order (mix(), clamp(), the
 * copy-through red-black pass, ping-pong buffers).  The orchestration follows
 * src/gpu/solver.js (step, _encodeAdvection, _encodeProjection, _encodePoisson,
 * poissonResidualAfter, maxDivergence) and src/gpu/multigrid.js (Multigrid,
 * encodeVCycle).  Uniform parameters are rounded to REAL exactly as
 * `new Float32Array(...).set([...])` rounds them in src/gpu/solver.js:249-256.
 */
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(CAT(fsw_, SUF), CAT(_, name))
#define ST CAT(fsw_solver_, SUF)
#define K(name) CAT(CAT(k_, SUF), CAT(_, name))

typedef struct {
  int nx, ny;
  REAL dx, dy, dt, nu, a, b;
} CAT(params_, SUF);
#define PRM CAT(params_, SUF)

typedef struct {
  int n;
  double dx;
  REAL* x[2];
  int xi;
  REAL* rhs; /* borrowed for level 0 */
  REAL* res;
} CAT(level_, SUF);
#define LEV CAT(level_, SUF)

struct ST {
  int nx, ny;
  double dx, dy, nu, mask_width;
  int advection, solver, iterations;
  double relax; /* param_a of every JACOBI / RED_BLACK_GS dispatch (1.0 as the reference) */
  REAL *u, *v, *un, *vn, *fu, *fv, *bu, *bv;
  REAL *p, *pn, *div;
  int n_modes;
  REAL* modes;
  double amp, drag, drift;
  int solid_on;
  double sx, sy, svx, svy, somega, sr;
  REAL *imp_x, *imp_y, *imp_t;
  int nlev;
  LEV lev[24];
  double t;
  int steps;
};

static inline int K(wrapi)(int i, int n) { return ((i % n) + n) % n; }
static inline REAL K(ld)(const REAL* f, int nx, int ny, int i, int j) {
  return f[(int64_t)K(wrapi)(j, ny) * nx + K(wrapi)(i, nx)];
}
/* WGSL mix(e1, e2, e3) = e1 * (1 - e3) + e2 * e3 */
static inline REAL K(mix)(REAL a, REAL b, REAL t) { return a * ((REAL)1 - t) + b * t; }
/* WGSL round() is round-half-to-even */
static inline REAL K(wrap_delta)(REAL d, REAL L) { return d - L * (REAL)rint((double)(d / L)); }

/* shaders.js:89-101 */
static inline REAL K(bilerp)(const REAL* t, int nx, int ny, REAL gx, REAL gy) {
  REAL fgx = (REAL)floor((double)gx), fgy = (REAL)floor((double)gy);
  int i0 = (int)fgx, j0 = (int)fgy;
  REAL fx = gx - fgx, fy = gy - fgy;
  REAL a = K(ld)(t, nx, ny, i0, j0), b = K(ld)(t, nx, ny, i0 + 1, j0);
  REAL c = K(ld)(t, nx, ny, i0, j0 + 1), d = K(ld)(t, nx, ny, i0 + 1, j0 + 1);
  REAL top = K(mix)(a, b, fx), bot = K(mix)(c, d, fx);
  return K(mix)(top, bot, fy);
}
/* shaders.js:104-109 */
static inline REAL K(sample_u)(const PRM* P, const REAL* u, REAL x, REAL y) {
  return K(bilerp)(u, P->nx, P->ny, x / P->dx, y / P->dy - (REAL)0.5);
}
static inline REAL K(sample_v)(const PRM* P, const REAL* v, REAL x, REAL y) {
  return K(bilerp)(v, P->nx, P->ny, x / P->dx - (REAL)0.5, y / P->dy);
}
/* shaders.js:117-122 */
static inline void K(trace)(const PRM* P, const REAL* u, const REAL* v, REAL x, REAL y, REAL dt,
                            REAL* ox, REAL* oy) {
  REAL v1x = K(sample_u)(P, u, x, y), v1y = K(sample_v)(P, v, x, y);
  REAL h = (REAL)0.5 * dt;
  REAL pmx = x - h * v1x, pmy = y - h * v1y;
  REAL v2x = K(sample_u)(P, u, pmx, pmy), v2y = K(sample_v)(P, v, pmx, pmy);
  *ox = x - dt * v2x;
  *oy = y - dt * v2y;
}
static inline REAL K(pux)(const PRM* P, int i) { return (REAL)i * P->dx; }
static inline REAL K(puy)(const PRM* P, int j) { return ((REAL)j + (REAL)0.5) * P->dy; }
static inline REAL K(pvx)(const PRM* P, int i) { return ((REAL)i + (REAL)0.5) * P->dx; }
static inline REAL K(pvy)(const PRM* P, int j) { return (REAL)j * P->dy; }

/* ADVECT_VELOCITY, shaders.js:126-145 */
static void K(advect_velocity)(const PRM* P, const REAL* u, const REAL* v, REAL* ou, REAL* ov) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL ax, ay, bx, by;
      K(trace)(P, u, v, K(pux)(P, i), K(puy)(P, j), P->dt, &ax, &ay);
      K(trace)(P, u, v, K(pvx)(P, i), K(pvy)(P, j), P->dt, &bx, &by);
      int64_t c = (int64_t)j * P->nx + i;
      ou[c] = K(sample_u)(P, u, ax, ay);
      ov[c] = K(sample_v)(P, v, bx, by);
    }
}

/* ADVECT_FIELD_BY, shaders.js:155-171 */
static void K(advect_field_by)(const PRM* P, const REAL* u, const REAL* v, const REAL* su,
                               const REAL* sv, REAL* ou, REAL* ov) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL ax, ay, bx, by;
      K(trace)(P, u, v, K(pux)(P, i), K(puy)(P, j), P->dt, &ax, &ay);
      K(trace)(P, u, v, K(pvx)(P, i), K(pvy)(P, j), P->dt, &bx, &by);
      int64_t c = (int64_t)j * P->nx + i;
      ou[c] = K(bilerp)(su, P->nx, P->ny, ax / P->dx, ay / P->dy - (REAL)0.5);
      ov[c] = K(bilerp)(sv, P->nx, P->ny, bx / P->dx - (REAL)0.5, by / P->dy);
    }
}

static inline REAL K(clampw)(REAL e, REAL lo, REAL hi) {
  REAL m = e > lo ? e : lo;
  return m < hi ? m : hi;
}

/* MACCORMACK_COMBINE, shaders.js:187-231 */
static void K(maccormack_combine)(const PRM* P, const REAL* u, const REAL* v, const REAL* fu,
                                  const REAL* fv, const REAL* bu, const REAL* bv, REAL* ou, REAL* ov) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      int64_t c = (int64_t)j * P->nx + i;
      REAL cx = fu[c] + (REAL)0.5 * (u[c] - bu[c]);
      REAL cy = fv[c] + (REAL)0.5 * (v[c] - bv[c]);
      REAL ax, ay, bx, by;
      K(trace)(P, u, v, K(pux)(P, i), K(puy)(P, j), P->dt, &ax, &ay);
      K(trace)(P, u, v, K(pvx)(P, i), K(pvy)(P, j), P->dt, &bx, &by);
      REAL gx = ax / P->dx, gy = ay / P->dy - (REAL)0.5;
      int ix = (int)floor((double)gx), iy = (int)floor((double)gy);
      REAL lo = (REAL)1e30, hi = (REAL)-1e30;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          REAL s = K(ld)(u, P->nx, P->ny, ix + di, iy + dj);
          lo = lo < s ? lo : s; hi = hi > s ? hi : s;
        }
      cx = K(clampw)(cx, lo, hi);
      gx = bx / P->dx - (REAL)0.5; gy = by / P->dy;
      ix = (int)floor((double)gx); iy = (int)floor((double)gy);
      lo = (REAL)1e30; hi = (REAL)-1e30;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          REAL s = K(ld)(v, P->nx, P->ny, ix + di, iy + dj);
          lo = lo < s ? lo : s; hi = hi > s ? hi : s;
        }
      cy = K(clampw)(cy, lo, hi);
      ou[c] = cx; ov[c] = cy;
    }
}

/* DIFFUSE, shaders.js:401-425 */
static void K(diffuse)(const PRM* P, const REAL* u, const REAL* v, REAL* ou, REAL* ov) {
  REAL a = P->nu * P->dt / (P->dx * P->dx);
  REAL bb = P->nu * P->dt / (P->dy * P->dy);
  for (int pass = 0; pass < 2; pass++) {
    const REAL* s = pass ? v : u;
    REAL* o = pass ? ov : ou;
    for (int j = 0; j < P->ny; j++)
      for (int i = 0; i < P->nx; i++) {
        REAL c = K(ld)(s, P->nx, P->ny, i, j);
        REAL l = K(ld)(s, P->nx, P->ny, i - 1, j), r = K(ld)(s, P->nx, P->ny, i + 1, j);
        REAL b = K(ld)(s, P->nx, P->ny, i, j - 1), t = K(ld)(s, P->nx, P->ny, i, j + 1);
        o[(int64_t)j * P->nx + i] = c + a * (l + r - (REAL)2 * c) + bb * (b + t - (REAL)2 * c);
      }
  }
}

/* FORCING, shaders.js:532-566 (param_a = amplitude, nu = drag, param_b = drift*t) */
static void K(forcing)(const PRM* P, const REAL* modes, int count, const REAL* u, const REAL* v,
                       REAL* ou, REAL* ov) {
  REAL scale = P->a * P->dt / (REAL)sqrt((double)(REAL)count);
  REAL damp = (REAL)exp((double)(-P->nu * P->dt));
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL pux = K(pux)(P, i), puy = K(puy)(P, j), pvx = K(pvx)(P, i), pvy = K(pvy)(P, j);
      REAL fu = 0, fv = 0;
      for (int m = 0; m < count; m++) {
        REAL kx = modes[3 * m], ky = modes[3 * m + 1], ph = modes[3 * m + 2];
        REAL kk = (REAL)sqrt((double)(kx * kx + ky * ky));
        if (kk < (REAL)1e-6) continue;
        fu = fu + (ky / kk) * (REAL)cos((double)(kx * pux + ky * puy + ph + P->b));
        fv = fv - (kx / kk) * (REAL)cos((double)(kx * pvx + ky * pvy + ph + P->b));
      }
      int64_t c = (int64_t)j * P->nx + i;
      ou[c] = u[c] * damp + scale * fu;
      ov[c] = v[c] * damp + scale * fv;
    }
}

/* SOLID_COUPLE, shaders.js:587-653 */
static REAL K(mask_at)(const PRM* P, const REAL* S, REAL px, REAL py) {
  REAL Lx = (REAL)P->nx * P->dx, Ly = (REAL)P->ny * P->dy;
  REAL dx = K(wrap_delta)(px - S[0], Lx), dy = K(wrap_delta)(py - S[1], Ly);
  REAL len = (REAL)sqrt((double)(dx * dx + dy * dy));
  REAL t = K(clampw)((len - S[5]) / S[6], (REAL)-10, (REAL)10);
  return (REAL)0.5 * ((REAL)1 - (REAL)tanh((double)t));
}
static void K(solid_couple)(const PRM* P, const REAL* S, const REAL* u, const REAL* v, REAL* ou,
                            REAL* ov, REAL* ix, REAL* iy, REAL* it) {
  REAL Lx = (REAL)P->nx * P->dx, Ly = (REAL)P->ny * P->dy;
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      int64_t c = (int64_t)j * P->nx + i;
      REAL pux = K(pux)(P, i), puy = K(puy)(P, j);
      REAL cu = K(mask_at)(P, S, pux, puy);
      REAL dux = K(wrap_delta)(pux - S[0], Lx), duy = K(wrap_delta)(puy - S[1], Ly);
      (void)dux;
      REAL su = S[2] - S[4] * duy;
      REAL dU = cu * (su - u[c]);
      REAL pvx = K(pvx)(P, i), pvy = K(pvy)(P, j);
      REAL cv = K(mask_at)(P, S, pvx, pvy);
      REAL dvx = K(wrap_delta)(pvx - S[0], Lx);
      REAL sv = S[3] + S[4] * dvx;
      REAL dV = cv * (sv - v[c]);
      ou[c] = u[c] + dU;
      ov[c] = v[c] + dV;
      ix[c] = dU; iy[c] = dV; it[c] = -duy * dU + dvx * dV;
    }
}

/* DIVERGENCE, shaders.js:269-288 */
static void K(divergence)(const PRM* P, const REAL* u, const REAL* v, REAL* d) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL uL = K(ld)(u, P->nx, P->ny, i, j), uR = K(ld)(u, P->nx, P->ny, i + 1, j);
      REAL vB = K(ld)(v, P->nx, P->ny, i, j), vT = K(ld)(v, P->nx, P->ny, i, j + 1);
      d[(int64_t)j * P->nx + i] = (uR - uL) / P->dx + (vT - vB) / P->dy;
    }
}

/* JACOBI, shaders.js:302-325 */
static void K(jacobi)(const PRM* P, const REAL* p, const REAL* d, REAL* o) {
  REAL h2 = P->dx * P->dx;
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL l = K(ld)(p, P->nx, P->ny, i - 1, j), r = K(ld)(p, P->nx, P->ny, i + 1, j);
      REAL b = K(ld)(p, P->nx, P->ny, i, j - 1), t = K(ld)(p, P->nx, P->ny, i, j + 1);
      REAL dd = d[(int64_t)j * P->nx + i];
      REAL jac = (l + r + b + t - h2 * dd) * (REAL)0.25;
      REAL cur = p[(int64_t)j * P->nx + i];
      o[(int64_t)j * P->nx + i] = cur + P->a * (jac - cur);
    }
}

/* RED_BLACK_GS, shaders.js:340-372: one colour, the other copied through */
static void K(red_black)(const PRM* P, const REAL* p, const REAL* d, REAL* o) {
  REAL h2 = P->dx * P->dx;
  unsigned colour_want = (unsigned)P->b;
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      int64_t c = (int64_t)j * P->nx + i;
      REAL cur = p[c];
      if ((unsigned)((i + j) % 2) != colour_want) { o[c] = cur; continue; }
      REAL l = K(ld)(p, P->nx, P->ny, i - 1, j), r = K(ld)(p, P->nx, P->ny, i + 1, j);
      REAL b = K(ld)(p, P->nx, P->ny, i, j - 1), t = K(ld)(p, P->nx, P->ny, i, j + 1);
      REAL gs = (l + r + b + t - h2 * d[c]) * (REAL)0.25;
      o[c] = cur + P->a * (gs - cur);
    }
}

/* SUBTRACT_GRADIENT, shaders.js:375-398 */
static void K(subtract_gradient)(const PRM* P, const REAL* u, const REAL* v, const REAL* p, REAL* ou,
                                 REAL* ov) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      int64_t c = (int64_t)j * P->nx + i;
      REAL pc = p[c], pl = K(ld)(p, P->nx, P->ny, i - 1, j), pb = K(ld)(p, P->nx, P->ny, i, j - 1);
      ou[c] = u[c] - (pc - pl) / P->dx;
      ov[c] = v[c] - (pc - pb) / P->dy;
    }
}

/* RESIDUAL, multigrid.js:48-66 */
static void K(residual)(const PRM* P, const REAL* x, const REAL* rhs, REAL* o) {
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL l = K(ld)(x, P->nx, P->ny, i - 1, j), r = K(ld)(x, P->nx, P->ny, i + 1, j);
      REAL b = K(ld)(x, P->nx, P->ny, i, j - 1), t = K(ld)(x, P->nx, P->ny, i, j + 1);
      int64_t c = (int64_t)j * P->nx + i;
      REAL lap = (l + r + b + t - (REAL)4 * x[c]) / (P->dx * P->dx);
      o[c] = rhs[c] - lap;
    }
}

/* RESTRICT, multigrid.js:72-93 (P describes the coarse grid) */
static void K(restrict_)(const PRM* P, const REAL* fine, REAL* o) {
  int fnx = P->nx * 2, fny = P->ny * 2;
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL s = 0;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          int x = ((2 * i + di) % fnx + fnx) % fnx, y = ((2 * j + dj) % fny + fny) % fny;
          s = s + fine[(int64_t)y * fnx + x];
        }
      o[(int64_t)j * P->nx + i] = s * (REAL)0.25;
    }
}

/* PROLONG, multigrid.js:99-131 (P describes the fine grid) */
static void K(prolong)(const PRM* P, const REAL* coarse, const REAL* fine_in, REAL* o) {
  int cnx = P->nx / 2, cny = P->ny / 2;
  for (int j = 0; j < P->ny; j++)
    for (int i = 0; i < P->nx; i++) {
      REAL gx = ((REAL)i + (REAL)0.5) * (REAL)0.5 - (REAL)0.5;
      REAL gy = ((REAL)j + (REAL)0.5) * (REAL)0.5 - (REAL)0.5;
      REAL fgx = (REAL)floor((double)gx), fgy = (REAL)floor((double)gy);
      int i0 = (int)fgx, j0 = (int)fgy;
      REAL fx = gx - fgx, fy = gy - fgy;
      int x0 = ((i0 % cnx) + cnx) % cnx, x1 = (((i0 + 1) % cnx) + cnx) % cnx;
      int y0 = ((j0 % cny) + cny) % cny, y1 = (((j0 + 1) % cny) + cny) % cny;
      REAL a = coarse[(int64_t)y0 * cnx + x0], b = coarse[(int64_t)y0 * cnx + x1];
      REAL c = coarse[(int64_t)y1 * cnx + x0], d = coarse[(int64_t)y1 * cnx + x1];
      REAL corr = K(mix)(K(mix)(a, b, fx), K(mix)(c, d, fx), fy);
      int64_t k = (int64_t)j * P->nx + i;
      o[k] = fine_in[k] + corr;
    }
}

/* ------------------------------------------------------------ orchestration */

static PRM K(params)(const ST* s, double dt, double a, double b) {
  PRM P;
  P.nx = s->nx; P.ny = s->ny;
  P.dx = (REAL)s->dx; P.dy = (REAL)s->dy; P.dt = (REAL)dt; P.nu = (REAL)s->nu;
  P.a = (REAL)a; P.b = (REAL)b;
  return P;
}
/* Multigrid._levelParams, multigrid.js:217-225 */
static PRM K(level_params)(const LEV* lv, double a, double b) {
  PRM P;
  P.nx = lv->n; P.ny = lv->n;
  P.dx = (REAL)lv->dx; P.dy = (REAL)lv->dx; P.dt = 0; P.nu = 0;
  P.a = (REAL)a; P.b = (REAL)b;
  return P;
}

#define ALLOC(n) ((REAL*)calloc((size_t)(n), sizeof(REAL)))

ST* FN(create)(int nx, int ny, double lx, double ly, double nu, int advection, int pressure_solver,
               int iterations, double solid_mask_width) {
  ST* s = (ST*)calloc(1, sizeof(ST));
  int64_t n = (int64_t)nx * ny;
  s->nx = nx; s->ny = ny; s->dx = lx / nx; s->dy = ly / ny; s->nu = nu;
  s->advection = advection; s->solver = pressure_solver; s->iterations = iterations;
  s->relax = 1.0;
  s->mask_width = solid_mask_width;
  s->u = ALLOC(n); s->v = ALLOC(n); s->un = ALLOC(n); s->vn = ALLOC(n);
  s->fu = ALLOC(n); s->fv = ALLOC(n); s->bu = ALLOC(n); s->bv = ALLOC(n);
  s->p = ALLOC(n); s->pn = ALLOC(n); s->div = ALLOC(n);
  s->imp_x = ALLOC(n); s->imp_y = ALLOC(n); s->imp_t = ALLOC(n);
  if (pressure_solver == FSW_MULTIGRID) {
    /* multigrid.js:177-197, minSize 8 */
    int m = nx;
    s->nlev = 0;
    while (m >= 8 && s->nlev < 24) {
      LEV* lv = &s->lev[s->nlev];
      lv->n = m;
      lv->dx = (s->dx * nx) / m;
      lv->x[0] = ALLOC((int64_t)m * m); lv->x[1] = ALLOC((int64_t)m * m);
      lv->xi = 0;
      lv->rhs = s->nlev == 0 ? NULL : ALLOC((int64_t)m * m);
      lv->res = ALLOC((int64_t)m * m);
      s->nlev++;
      if (m / 2 < 8) break;
      m = m / 2;
    }
  }
  return s;
}

void FN(destroy)(ST* s) {
  if (!s) return;
  free(s->u); free(s->v); free(s->un); free(s->vn); free(s->fu); free(s->fv); free(s->bu); free(s->bv);
  free(s->p); free(s->pn); free(s->div); free(s->imp_x); free(s->imp_y); free(s->imp_t);
  free(s->modes);
  for (int i = 0; i < s->nlev; i++) {
    free(s->lev[i].x[0]); free(s->lev[i].x[1]); free(s->lev[i].res);
    if (i) free(s->lev[i].rhs);
  }
  free(s);
}

void FN(upload_velocity)(ST* s, const double* u, const double* v) {
  int64_t n = (int64_t)s->nx * s->ny;
  for (int64_t i = 0; i < n; i++) { s->u[i] = (REAL)u[i]; s->v[i] = (REAL)v[i]; }
}
void FN(read_velocity)(ST* s, double* u, double* v) {
  int64_t n = (int64_t)s->nx * s->ny;
  for (int64_t i = 0; i < n; i++) { u[i] = (double)s->u[i]; v[i] = (double)s->v[i]; }
}
void FN(read_pressure)(ST* s, double* p) {
  int64_t n = (int64_t)s->nx * s->ny;
  for (int64_t i = 0; i < n; i++) p[i] = (double)s->p[i];
}
void FN(read_divergence)(ST* s, double* d) {
  int64_t n = (int64_t)s->nx * s->ny;
  for (int64_t i = 0; i < n; i++) d[i] = (double)s->div[i];
}
void FN(read_impulse)(ST* s, double* fx, double* fy, double* tq) {
  int64_t n = (int64_t)s->nx * s->ny;
  for (int64_t i = 0; i < n; i++) { fx[i] = s->imp_x[i]; fy[i] = s->imp_y[i]; tq[i] = s->imp_t[i]; }
}
void FN(set_iterations)(ST* s, int iterations) { s->iterations = iterations; }
/* the relaxation factor the reference's callers fix at 1.0 (solver.js:716,729,
   multigrid.js:261), applied to every sweep including the coarsest level's */
void FN(set_relax)(ST* s, double relax) { s->relax = relax; }

/* setForcing, solver.js:370-385 */
void FN(set_forcing)(ST* s, const double* modes, int m, double amp, double drag, double drift) {
  free(s->modes); s->modes = NULL; s->n_modes = 0;
  if (!modes || m <= 0) return;
  s->modes = ALLOC(3 * m);
  for (int i = 0; i < 3 * m; i++) s->modes[i] = (REAL)modes[i];
  s->n_modes = m; s->amp = amp; s->drag = drag; s->drift = drift;
}

void FN(set_solid)(ST* s, int on, double x, double y, double vx, double vy, double omega, double r) {
  s->solid_on = on; s->sx = x; s->sy = y; s->svx = vx; s->svy = vy; s->somega = omega; s->sr = r;
}

static void K(swapvel)(ST* s) {
  REAL* t = s->u; s->u = s->un; s->un = t;
  t = s->v; s->v = s->vn; s->vn = t;
}
static void K(swappres)(ST* s) { REAL* t = s->p; s->p = s->pn; s->pn = t; }

/* _encodeAdvection, solver.js:604-647 */
static void K(do_advect)(ST* s, double dt) {
  if (s->advection == 1) {
    PRM P = K(params)(s, dt, 0, 0);
    K(advect_velocity)(&P, s->u, s->v, s->fu, s->fv);
    PRM Pb = K(params)(s, -dt, 0, 0);
    K(advect_field_by)(&Pb, s->u, s->v, s->fu, s->fv, s->bu, s->bv);
    K(maccormack_combine)(&P, s->u, s->v, s->fu, s->fv, s->bu, s->bv, s->un, s->vn);
    K(swapvel)(s);
    return;
  }
  PRM P = K(params)(s, dt, 0, 0);
  K(advect_velocity)(&P, s->u, s->v, s->un, s->vn);
  K(swapvel)(s);
}

static void K(do_diffuse)(ST* s, double dt) {
  PRM P = K(params)(s, dt, 0, 0);
  K(diffuse)(&P, s->u, s->v, s->un, s->vn);
  K(swapvel)(s);
}

/* _encodeForcing, solver.js:387-414 */
static void K(do_forcing)(ST* s, double dt) {
  if (!s->n_modes) return;
  PRM P = K(params)(s, dt, s->amp, s->drift * s->t);
  P.nu = (REAL)s->drag;
  K(forcing)(&P, s->modes, s->n_modes, s->u, s->v, s->un, s->vn);
  K(swapvel)(s);
}

/* _encodeSolid, solver.js:440-465 */
static void K(do_solid)(ST* s, double dt) {
  if (!s->solid_on) return;
  REAL S[8] = {(REAL)s->sx, (REAL)s->sy, (REAL)s->svx, (REAL)s->svy, (REAL)s->somega, (REAL)s->sr,
               (REAL)(s->mask_width * s->dx), 0};
  PRM P = K(params)(s, dt, 0, 0);
  K(solid_couple)(&P, S, s->u, s->v, s->un, s->vn, s->imp_x, s->imp_y, s->imp_t);
  K(swapvel)(s);
}

static void K(do_divergence)(ST* s, double dt) {
  PRM P = K(params)(s, dt, 0, 0);
  K(divergence)(&P, s->u, s->v, s->div);
}

/* Multigrid._smooth, multigrid.js:256-270 */
static void K(mg_smooth)(LEV* lv, const REAL* rhs, int sweeps, double relax) {
  for (int k = 0; k < sweeps; k++)
    for (int colour = 0; colour < 2; colour++) {
      PRM P = K(level_params)(lv, relax, colour);
      K(red_black)(&P, lv->x[lv->xi], rhs, lv->x[1 - lv->xi]);
      lv->xi = 1 - lv->xi;
    }
}

/* Multigrid.encodeVCycle, multigrid.js:277-330 (pre 2, post 2, coarse 40) */
static void K(vcycle)(ST* s, REAL* rhs) {
  LEV* L = s->lev;
  int nl = s->nlev;
  L[0].rhs = rhs;
  for (int i = 0; i < nl - 1; i++) {
    LEV* lv = &L[i];
    LEV* nx = &L[i + 1];
    K(mg_smooth)(lv, lv->rhs, 2, s->relax);
    PRM P = K(level_params)(lv, 0, 0);
    K(residual)(&P, lv->x[lv->xi], lv->rhs, lv->res);
    PRM Pc = K(level_params)(nx, 0, 0);
    K(restrict_)(&Pc, lv->res, nx->rhs);
    memset(nx->x[nx->xi], 0, sizeof(REAL) * (size_t)nx->n * nx->n);
    memset(nx->x[1 - nx->xi], 0, sizeof(REAL) * (size_t)nx->n * nx->n);
  }
  LEV* last = &L[nl - 1];
  K(mg_smooth)(last, last->rhs, 40, s->relax);
  for (int i = nl - 2; i >= 0; i--) {
    LEV* lv = &L[i];
    LEV* below = &L[i + 1];
    PRM P = K(level_params)(lv, 0, 0);
    K(prolong)(&P, below->x[below->xi], lv->x[lv->xi], lv->x[1 - lv->xi]);
    lv->xi = 1 - lv->xi;
    K(mg_smooth)(lv, lv->rhs, 2, s->relax);
  }
  L[0].rhs = NULL;
}

/* _encodePoisson, solver.js:686-738 */
static void K(do_poisson)(ST* s, double dt, int iterations) {
  int64_t n = (int64_t)s->nx * s->ny;
  if (s->solver == FSW_MULTIGRID) {
    LEV* l0 = &s->lev[0];
    memset(l0->x[0], 0, sizeof(REAL) * n);
    memset(l0->x[1], 0, sizeof(REAL) * n);
    for (int k = 0; k < iterations; k++) K(vcycle)(s, s->div);
    memcpy(s->p, l0->x[l0->xi], sizeof(REAL) * n);
    return;
  }
  if (s->solver == FSW_RED_BLACK) {
    for (int k = 0; k < iterations; k++)
      for (int colour = 0; colour < 2; colour++) {
        PRM P = K(params)(s, dt, s->relax, colour);
        K(red_black)(&P, s->p, s->div, s->pn);
        K(swappres)(s);
      }
    return;
  }
  for (int k = 0; k < iterations; k++) {
    PRM P = K(params)(s, dt, s->relax, 0);
    K(jacobi)(&P, s->p, s->div, s->pn);
    K(swappres)(s);
  }
}

static void K(do_subtract)(ST* s, double dt) {
  PRM P = K(params)(s, dt, 0, 0);
  K(subtract_gradient)(&P, s->u, s->v, s->p, s->un, s->vn);
  K(swapvel)(s);
}

/* _encodeProjection, solver.js:658-684 */
static void K(do_project)(ST* s, double dt) {
  int64_t n = (int64_t)s->nx * s->ny;
  K(do_divergence)(s, dt);
  memset(s->p, 0, sizeof(REAL) * n);
  K(do_poisson)(s, dt, s->iterations);
  K(do_subtract)(s, dt);
}

/* step, solver.js:518-591 (dye, splats and confinement are not part of this path) */
void FN(step)(ST* s, double dt) {
  K(do_advect)(s, dt);
  if (s->nu > 0) K(do_diffuse)(s, dt);
  K(do_forcing)(s, dt);
  K(do_solid)(s, dt);
  K(do_project)(s, dt);
  s->t += dt;
  s->steps++;
}

void FN(stage)(ST* s, int stage, double dt) {
  int64_t n = (int64_t)s->nx * s->ny;
  switch (stage) {
    case FSW_STAGE_ADVECT: K(do_advect)(s, dt); break;
    case FSW_STAGE_DIFFUSE: K(do_diffuse)(s, dt); break;
    case FSW_STAGE_FORCING: K(do_forcing)(s, dt); break;
    case FSW_STAGE_SOLID: K(do_solid)(s, dt); break;
    case FSW_STAGE_DIVERGENCE: K(do_divergence)(s, dt); break;
    case FSW_STAGE_PRESSURE:
      memset(s->p, 0, sizeof(REAL) * n);
      K(do_poisson)(s, dt, s->iterations);
      break;
    case FSW_STAGE_SUBTRACT_GRADIENT: K(do_subtract)(s, dt); break;
    case FSW_STAGE_PROJECT: K(do_project)(s, dt); break;
    default: break;
  }
}

/* poissonResidualAfter, solver.js:857-896: residual evaluated in f64 on the host */
double FN(poisson_residual_after)(ST* s, int iterations, double dt) {
  int64_t n = (int64_t)s->nx * s->ny;
  K(do_divergence)(s, dt);
  memset(s->p, 0, sizeof(REAL) * n);
  K(do_poisson)(s, dt, iterations);
  const int nx = s->nx, ny = s->ny;
  const double h2 = s->dx * s->dx;
#define AT(arr, i, j) ((double)(arr)[(int64_t)(((j) % ny + ny) % ny) * nx + (((i) % nx) + nx) % nx])
  double num = 0, den = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double lap = (AT(s->p, i - 1, j) + AT(s->p, i + 1, j) + AT(s->p, i, j - 1) + AT(s->p, i, j + 1) -
                    4 * AT(s->p, i, j)) / h2;
      double r = lap - AT(s->div, i, j);
      num += r * r;
      den += AT(s->div, i, j) * AT(s->div, i, j);
    }
#undef AT
  double sd = sqrt(den);
  return sqrt(num) / (sd == 0 ? 1 : sd);
}

/* maxDivergence, solver.js:835-850 */
double FN(max_divergence)(ST* s) {
  int64_t n = (int64_t)s->nx * s->ny;
  K(do_divergence)(s, 0);
  double m = 0;
  for (int64_t i = 0; i < n; i++) m = fmax(m, fabs((double)s->div[i]));
  return m;
}

double FN(time)(ST* s) { return s->t; }

#undef ALLOC
#undef PRM
#undef LEV
#undef ST
#undef FN
#undef K
