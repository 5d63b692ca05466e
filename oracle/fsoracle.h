/*
 * fsoracle.h -- CPU oracle for the stable-fluids step.  TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker that the CUDA path is measured against.  It is
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg, and by nothing in the product path.
 *
 * Two restatements live here, both written from the reference's published
 * algorithm (fluid-sim, JavaScript):
 *
 *  fso_*   f64 restatement of the CPU reference solver
 *          (src/core/grid.js, src/core/analytic.js, src/core/fft.js,
 *           src/cpu/advect.js, src/cpu/projection.js, src/cpu/solver.js,
 *           src/cpu/solid.js).  Every loop keeps the reference's order of
 *           floating-point operations, so on identical inputs the results are
 *           bit-identical to the JavaScript except where libm and V8 differ in
 *           the last ulp of sin/cos/exp/tanh/hypot.  Compiled with
 *           -ffp-contract=off so no multiply-add is fused on either host.
 *
 *  fsw_*   restatement of the reference's GPU algorithm (the WGSL kernels in
 *          src/gpu/shaders.js and src/gpu/multigrid.js orchestrated as in
 *          src/gpu/solver.js), compiled twice: fsw_f32_* in float arithmetic
 *          (what the WebGPU backend computes) and fsw_f64_* in double (the same
 *          algorithm without f32 rounding).
 *
 * Parity is pinned by tests/test_oracle_golden.py against the reference's own
 * committed run outputs (results/validation.json, results/gpu-verify.json).
 */
#ifndef FSORACLE_H
#define FSORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ grid */
typedef struct {
  int nx, ny;
  double lx, ly, dx, dy;
} fso_grid;

void fso_grid_init(fso_grid* g, int nx, int ny, double lx, double ly);

/* ((i % n) + n) % n  -- src/core/grid.js:40 */
int fso_wrap(int i, int n);

/* JavaScript LCG used by every reference fixture:
 * s = (s*1103515245 + 12345) & 0x7fffffff evaluated in double then ToInt32,
 * value = s/0x7fffffff - 0.5 (test/core.test.js:94-98).  Fills out[0..n).
 * Returns the final state. */
uint32_t fso_lcg_fill(uint32_t seed, int64_t n, double* out);
/* Same generator, filling u and v alternately (u[0],v[0],u[1],v[1],...) as
 * tools/gputest.html:116,158,196 do. */
uint32_t fso_lcg_fill_uv(uint32_t seed, int64_t n, double* u, double* v);

double fso_bilerp(const double* a, int nx, int ny, double gx, double gy);
double fso_sample_u(const fso_grid* g, const double* u, double x, double y);
double fso_sample_v(const fso_grid* g, const double* v, double x, double y);
double fso_sample_p(const fso_grid* g, const double* p, double x, double y);

void fso_divergence(const fso_grid* g, const double* u, const double* v, double* out);
void fso_subtract_gradient(const fso_grid* g, double* u, double* v, const double* p, double scale);
void fso_vorticity_corner(const fso_grid* g, const double* u, const double* v, double* out);
void fso_vorticity_center(const fso_grid* g, const double* u, const double* v, double* out);
void fso_velocity_at_centers(const fso_grid* g, const double* u, const double* v, double* cu, double* cv);
double fso_kinetic_energy(const fso_grid* g, const double* u, const double* v);
double fso_enstrophy(const fso_grid* g, const double* u, const double* v);
double fso_max_divergence(const fso_grid* g, const double* u, const double* v);
double fso_l2_divergence(const fso_grid* g, const double* u, const double* v);
double fso_cfl(const fso_grid* g, const double* u, const double* v, double dt);

/* ------------------------------------------------------------- analytic */
void fso_tg_init(const fso_grid* g, double* u, double* v, double t, double nu);
double fso_tg_velocity_error(const fso_grid* g, const double* u, const double* v, double t, double nu);
double fso_rel_l2(const double* a, const double* exact, int64_t n);
double fso_gaussian_scalar(double x, double y, double t, double sigma, double ax, double ay, double cx, double cy);

/* ------------------------------------------------------------------ fft */
int fso_is_pow2(int n);
void fso_fft_inplace(double* re, double* im, int n, int sign);
void fso_dft_naive(const double* re_in, const double* im_in, double* re, double* im, int n, int sign);
int fso_fft2(const double* field, int nx, int ny, double* re, double* im);
int fso_ifft2(const double* re0, const double* im0, int nx, int ny, double* re, double* im);
/* E has kmax+1 = min(nx,ny)/2+1 entries */
int fso_energy_spectrum(const double* cu, const double* cv, int nx, int ny, double* E, int32_t* counts);

/* ------------------------------------------------------------ advection */
enum { FSO_SL = 0, FSO_MACCORMACK = 1 };
void fso_advect_velocity(const fso_grid* g, int scheme, const double* u, const double* v,
                         double* out_u, double* out_v, double dt);
void fso_advect_scalar(const fso_grid* g, int scheme, const double* u, const double* v,
                       const double* q, double* out, double dt);

/* ----------------------------------------------------------- projection */
void fso_laplacian(const fso_grid* g, const double* p, double* out);
/* returns iterations; *residual gets the final relative residual */
int fso_poisson_cg(const fso_grid* g, const double* rhs, double* p, double tol, int max_iter,
                   double* residual, double* history, int history_cap);
int fso_poisson_jacobi(const fso_grid* g, const double* rhs, double* p, int iterations,
                       double omega, double* residual, double* history, int history_cap);
int fso_poisson_fft(const fso_grid* g, const double* rhs, double* p);
double fso_poisson_residual(const fso_grid* g, const double* p, const double* rhs);
/* divergence -> CG -> subtract gradient (src/cpu/projection.js:259) */
int fso_project(const fso_grid* g, double* u, double* v, double* p, double tol, int max_iter,
                double* residual);

/* ----------------------------------------------------- diffusion, forces */
int fso_diffuse(const fso_grid* g, const double* field, double* out, double nu, double dt,
                int explicit_, double tol, double* residual);
void fso_linear_drag(double* u, double* v, int64_t n, double alpha, double dt);
/* bandForcing (src/cpu/solver.js:179) */
void fso_band_forcing(const fso_grid* g, double* u, double* v, double kf, double width,
                      double amp, uint32_t seed, double dt);
/* Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11) */
void fso_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Band forcing with a complex Gaussian amplitude per lattice mode (the forced-
 * turbulence configuration; no reference counterpart, the reference draws 24
 * LCG modes): every integer (kx, ky) with kf-width <= |k| <= kf+width, ky then
 * kx ascending; mode m draws Philox(ctr = {counter, m, 0, 0}, key = {key lo,
 * key hi}) -> u1 = (x0 + 1/2)/2^32, u2 = (x1 + 1/2)/2^32, A = sqrt(-2 ln u1),
 * phi = 2 pi u2, and adds the curl of A cos(k.x + phi) scaled by amp dt/sqrt(M)
 * exactly as bandForcing does with its modes. */
void fso_gauss_band_forcing(const fso_grid* g, double* u, double* v, double kf, double width, double amp,
                            uint64_t key, uint32_t counter, double dt);
/* GPU FORCING semantics (src/gpu/shaders.js:532-566): u = u*exp(-drag dt) + amp dt/sqrt(M) sum */
typedef struct { double kx, ky, phase; } fso_mode;
void fso_forcing_modes(const fso_grid* g, double* u, double* v, const fso_mode* modes, int m,
                       double amp, double drag, double drift_phase, double dt);

/* ---------------------------------------------------------------- solid */
typedef struct {
  double x, y, r, density, vx, vy, omega;
  int fixed, added_mass_correction;
  double mass, inertia, added_mass, effective_mass, effective_inertia;
  double force[2], torque, last_impulse[2];
} fso_disk;
void fso_disk_init(fso_disk* d, double x, double y, double r, double density, double vx,
                   double vy, double omega, int fixed, int added_mass_correction);
double fso_disk_mask(const fso_disk* d, double px, double py, double lx, double ly, double width);
void fso_disk_integrate(fso_disk* d, double dt, double gravity);
void fso_apply_coupling(const fso_grid* g, double* u, double* v, fso_disk* solids, int n_solids,
                        double dt, double mask_width, int passes, double* impulse_out);

/* A channel on the periodic grid (no reference counterpart; the reference is
 * periodic only): a fringe strip driving (u, v) to (inflow_u, 0), then a
 * no-slip wall slab, both as direct forcing with the reference disks' tanh
 * mask (src/cpu/solid.js:101-114,165-233) on a slab instead of a disk. */
typedef struct {
  double wall_y, wall_half, fringe_x, fringe_half, fringe_ramp, inflow_u;
} fso_channel;
void fso_channel_forcing(const fso_grid* g, double* u, double* v, const fso_channel* c, double mask_width);

/* --------------------------------------------------------------- solver */
enum { FSO_PROJ_CG = 0, FSO_PROJ_FFT = 1, FSO_PROJ_JACOBI = 2 };
typedef struct {
  int nx, ny;
  double lx, ly, nu;
  int advection, explicit_diffusion, projection;
  double proj_tol;
  int proj_max_iter;
  double mask_width;
  int coupling_passes;
} fso_params;

typedef struct fso_solver fso_solver;
void fso_params_default(fso_params* p);
/* returns NULL and sets *err on invalid parameters (fft on non-pow2 etc.) */
fso_solver* fso_create(const fso_params* p, int* err);
void fso_destroy(fso_solver* s);
double* fso_field(fso_solver* s, int which); /* 0 u, 1 v, 2 p, 3 dye */
const fso_grid* fso_solver_grid(fso_solver* s);
int fso_add_solid(fso_solver* s, const fso_disk* d);
fso_disk* fso_get_solid(fso_solver* s, int i);
void fso_set_modes(fso_solver* s, const fso_mode* modes, int m, double amp, double drag, double drift);
/* c == NULL removes it; applied after the forces and drag, before the disks */
void fso_set_channel(fso_solver* s, const fso_channel* c);
/* step: advect, diffuse, forces (gpu-style modes if set), drag, solids, project, dye.
 * band_seed > 0 applies bandForcing(kf, width, amp) as opts.force. */
typedef struct {
  int advect_dye;
  double drag;
  double gravity;
  int band_forcing;
  double band_kf, band_width, band_amp;
  uint32_t band_seed;
  int band_kind;          /* 0: bandForcing with band_seed; 1: fso_gauss_band_forcing */
  uint64_t band_key;      /* kind 1: Philox key */
  uint32_t band_counter;  /* kind 1: Philox counter word 0 (the step) */
} fso_step_opts;
void fso_step_opts_default(fso_step_opts* o);
void fso_step(fso_solver* s, double dt, const fso_step_opts* o);
double fso_time(fso_solver* s);
int fso_steps(fso_solver* s);
int fso_last_iterations(fso_solver* s);
double fso_last_residual(fso_solver* s);
int fso_is_blown_up(fso_solver* s);
void fso_set_threads(int n);

/* ------------------------------------- reference GPU algorithm restatement */
#define FSW_DECLARE(SUF)                                                                  \
  typedef struct fsw_solver_##SUF fsw_solver_##SUF;                                      \
  fsw_solver_##SUF* fsw_##SUF##_create(int nx, int ny, double lx, double ly, double nu,     \
                                       int advection, int pressure_solver, int iterations,  \
                                       double solid_mask_width);                            \
  void fsw_##SUF##_destroy(fsw_solver_##SUF* s);                                          \
  void fsw_##SUF##_upload_velocity(fsw_solver_##SUF* s, const double* u, const double* v); \
  void fsw_##SUF##_read_velocity(fsw_solver_##SUF* s, double* u, double* v);               \
  void fsw_##SUF##_read_pressure(fsw_solver_##SUF* s, double* p);                          \
  void fsw_##SUF##_read_divergence(fsw_solver_##SUF* s, double* d);                        \
  void fsw_##SUF##_set_forcing(fsw_solver_##SUF* s, const double* modes, int m, double amp, \
                               double drag, double drift);                                  \
  void fsw_##SUF##_set_solid(fsw_solver_##SUF* s, int on, double x, double y, double vx,    \
                             double vy, double omega, double r);                            \
  void fsw_##SUF##_read_impulse(fsw_solver_##SUF* s, double* fx, double* fy, double* tq);  \
  void fsw_##SUF##_set_iterations(fsw_solver_##SUF* s, int iterations);                    \
  void fsw_##SUF##_set_relax(fsw_solver_##SUF* s, double relax);                           \
  void fsw_##SUF##_step(fsw_solver_##SUF* s, double dt);                                   \
  void fsw_##SUF##_stage(fsw_solver_##SUF* s, int stage, double dt);                       \
  double fsw_##SUF##_poisson_residual_after(fsw_solver_##SUF* s, int iterations, double dt);\
  double fsw_##SUF##_max_divergence(fsw_solver_##SUF* s);                                  \
  double fsw_##SUF##_time(fsw_solver_##SUF* s);

/* stages for fsw_*_stage */
enum {
  FSW_STAGE_ADVECT = 0, FSW_STAGE_DIFFUSE = 1, FSW_STAGE_FORCING = 2, FSW_STAGE_SOLID = 3,
  FSW_STAGE_DIVERGENCE = 4, FSW_STAGE_PRESSURE = 5, FSW_STAGE_SUBTRACT_GRADIENT = 6,
  FSW_STAGE_PROJECT = 7
};
enum { FSW_JACOBI = 0, FSW_RED_BLACK = 1, FSW_MULTIGRID = 2 };

FSW_DECLARE(f32)
FSW_DECLARE(f64)

#ifdef __cplusplus
}
#endif
#endif
