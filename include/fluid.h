/*
 * fluid.h -- C ABI of libfluidcuda.so, the GB300 (sm_103a) stable-fluids step.
 *
 * This is the drop-in boundary for fluid-sim's GPU backend, the JavaScript
 * class GPUFluidSolver in src/gpu/solver.js.  Each entry point below names the
 * reference member it replaces.  The signatures carry only plain C types
 * (pointers, sizes, enums, PODs) so any FFI -- an N-API addon for the
 * reference's Node host, ctypes, C/C++ -- can bind them.
 *
 * Conventions
 *  - Every function returns an int status (fs_status; 0 = FS_OK) unless
 *    stated otherwise.  On failure fs_last_error() returns a message.
 *  - Fields are row-major n = nx*ny arrays, i fastest: u[j*nx+i] is u on the
 *    LEFT face of cell (i,j), v[j*nx+i] on its BOTTOM face, p at its centre
 *    (src/core/grid.js:95-105).  Inputs are copied; outputs are written to
 *    caller memory.
 *  - A solver owns its device memory and one CUDA stream.  Calls on one
 *    handle are not thread-safe; distinct handles are independent.  Work is
 *    enqueued asynchronously; every read-back call synchronises the stream.
 *  - Unknown enum values are rejected with FS_ERR_INVALID_ARGUMENT (the
 *    reference silently falls back to semi-Lagrangian / Jacobi,
 *    src/gpu/solver.js:606,687; this boundary is deliberately stricter).
 *  - Nothing here falls back to the CPU: with no usable CUDA device fs_create
 *    fails with FS_ERR_NO_DEVICE.
 */
#ifndef FLUIDCUDA_H
#define FLUIDCUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define FS_API __declspec(dllexport)
#else
#define FS_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fs_solver fs_solver;

typedef enum fs_status {
  FS_OK = 0,
  FS_ERR_INVALID_ARGUMENT = 1,
  FS_ERR_CUDA = 2,
  FS_ERR_OUT_OF_MEMORY = 3,
  FS_ERR_NOT_CONVERGED = 4, /* tolerance not met within max_cycles (state is still advanced) */
  FS_ERR_NONFINITE = 5,     /* a residual reduction saw NaN or Inf */
  FS_ERR_UNSUPPORTED = 6,
  FS_ERR_NO_DEVICE = 7
} fs_status;

/* advection option of src/gpu/solver.js:68 */
typedef enum fs_advection { FS_ADVECT_SEMI_LAGRANGIAN = 0, FS_ADVECT_MACCORMACK = 1 } fs_advection;

/* pressureSolver option of src/gpu/solver.js:70 */
typedef enum fs_pressure_solver {
  FS_PRESSURE_JACOBI = 0,
  FS_PRESSURE_RED_BLACK = 1,
  FS_PRESSURE_MULTIGRID = 2
} fs_pressure_solver;

/* Arithmetic of the step.
 *  F32:   every field f32, as the reference WebGPU backend computes.
 *  MIXED: velocity, pressure and divergence held in f64; advection, forcing
 *         and the Poisson corrections (V-cycles / sweeps) in f32 inside an
 *         iterative refinement whose residual and pressure accumulation are
 *         f64.  Needed for max|div u| <= 1e-6 and below at large n, where an
 *         f32-stored velocity alone floors max|div| near 1e-5. */
typedef enum fs_precision { FS_PRECISION_F32 = 0, FS_PRECISION_MIXED = 1 } fs_precision;

typedef enum fs_dtype { FS_DTYPE_F32 = 0, FS_DTYPE_F64 = 1 } fs_dtype;

typedef enum fs_field {
  FS_FIELD_U = 0,
  FS_FIELD_V = 1,
  FS_FIELD_PRESSURE = 2,   /* last projection's pressure (readTexture(presCur)) */
  FS_FIELD_DIVERGENCE = 3, /* last computed divergence (readTexture(div)) */
  FS_FIELD_IMPULSE_X = 4,  /* last solid-coupling impulse per cell (impulseTex .x/.y/.z) */
  FS_FIELD_IMPULSE_Y = 5,
  FS_FIELD_IMPULSE_TORQUE = 6
} fs_field;

/* One stage of the step, for fs_run_stage (the verification harness's reach
 * into private _bind/_dispatch, tools/gputest.html:91-100, made public). */
typedef enum fs_stage {
  FS_STAGE_ADVECT = 0,            /* _encodeAdvection, solver.js:604-647 */
  FS_STAGE_DIFFUSE = 1,           /* DIFFUSE pass, solver.js:532-540 */
  FS_STAGE_FORCING = 2,           /* _encodeForcing, solver.js:387-414 */
  FS_STAGE_SOLID = 3,             /* _encodeSolid, solver.js:440-465 */
  FS_STAGE_DIVERGENCE = 4,        /* DIVERGENCE pass, solver.js:659-664 */
  FS_STAGE_PRESSURE = 5,          /* zero p + _encodePoisson, solver.js:669-674 */
  FS_STAGE_SUBTRACT_GRADIENT = 6, /* SUBTRACT_GRADIENT pass, solver.js:676-683 */
  FS_STAGE_PROJECT = 7            /* _encodeProjection, solver.js:658-684 */
} fs_stage;

/* Constructor options of GPUFluidSolver (src/gpu/solver.js:65-72) plus the
 * tolerance loop, precision and multigrid settings.  Fill with
 * fs_params_default() first; it sets the reference defaults. */
typedef struct fs_params {
  int32_t nx, ny;             /* cells (default 256 x 256) */
  double lx, ly;              /* domain (default 2*pi x 2*pi) */
  double nu;                  /* viscosity, explicit diffusion (default 0) */
  double confinement;         /* must be 0: vorticity confinement is not on this path */
  int32_t advection;          /* fs_advection (default MacCormack) */
  double solid_mask_width;    /* mask width in cells (default 1.5) */
  int32_t pressure_solver;    /* fs_pressure_solver (default Jacobi) */
  int32_t pressure_iterations;/* pressure_tol == 0: sweeps (Jacobi, red-black) or
                                 V-cycles (multigrid) per projection (default 40);
                                 pressure_tol > 0: sweeps per cycle (Jacobi, red-black) */
  int32_t precision;          /* fs_precision (default F32) */
  double pressure_tol;        /* > 0: repeat cycles until max|div u| <= tol; a cycle is
                                 one V-cycle (multigrid) or pressure_iterations sweeps.
                                 In MIXED precision every cycle ends with the
                                 double-float update p += e, r = d - lap p. */
  int32_t max_cycles;         /* cap of the tolerance loop (default 50) */
  int32_t mg_pre_smooth;      /* red-black sweeps before restriction (default 2) */
  int32_t mg_post_smooth;     /* red-black sweeps after prolongation (default 2) */
  int32_t mg_coarse_sweeps;   /* sweeps on the coarsest level (default 40) */
  int32_t mg_min_size;        /* stop coarsening below this size (default 8) */
  int32_t warm_start;         /* 1: start each projection from the previous pressure
                                 instead of zero (the reference zeroes it,
                                 solver.js:669-672) */
  int32_t device;             /* CUDA device ordinal (default 0) */
  int32_t kernel_variant;     /* 0: fused multigrid kernels (default); 1: one kernel per
                                 reference pass (RBGS colour, residual, restriction,
                                 prolongation), kept to cross-check the fused cycle */
  double dye_fade;            /* dyeFade (solver.js:67,82): dye *= 1 - dye_fade per step
                                 (default 0); dye advection runs once a dye field is
                                 uploaded (fs_upload_dye) */
  double relax;               /* relaxation factor w of every Jacobi / red-black sweep,
                                 including the multigrid smoothers: cur + w (gs - cur),
                                 param_a of JACOBI / RED_BLACK_GS (shaders.js:322,368).
                                 Default 1.0, the value the reference's callers pass
                                 (solver.js:716,729, multigrid.js:261); w = 1 rounds
                                 exactly like the plain update.  Must lie in (0, 2). */
  int32_t pressure_tol_relative; /* 1: the tolerance loop stops at max|r| <= pressure_tol
                                 times the max residual the projection started from
                                 (a relative residual), 0 (default): at max|div u| <=
                                 pressure_tol */
  int32_t mg_first_pre;       /* red-black sweeps on the finest level before restriction
                                 in the first V-cycle of each MIXED projection, 0 ..
                                 mg_pre_smooth; -1 (default): mg_pre_smooth, as every
                                 cycle of the reference.  Fused multigrid only. */
  int32_t mg_first_post;      /* likewise after prolongation, 0 .. mg_post_smooth;
                                 -1 (default): mg_post_smooth */
} fs_params;

/* one forcing mode, as setForcing's {kx, ky, phase} (solver.js:370-385) */
typedef struct fs_mode {
  double kx, ky, phase;
} fs_mode;

/* an immersed rigid disk (src/cpu/solid.js:42-146 RigidDisk: centre, radius,
 * velocity, angular velocity); the step applies its direct forcing */
typedef struct fs_disk {
  double x, y, r, vx, vy, omega;
} fs_disk;

typedef struct fs_step_stats {
  int32_t cycles;            /* cycles (sweeps or V-cycles) the last projection ran */
  int32_t converged;         /* 1 if pressure_tol was met (always 1 when tol == 0) */
  double residual_max;       /* max|div u| after the last projection, -1 if not measured */
  double residual_initial;   /* max|div u| entering the last projection, -1 if not measured */
} fs_step_stats;

/* per-kernel timing from fs_profile_step */
typedef struct fs_kernel_time {
  char name[48];
  int32_t launches;
  double total_ms;
  double bytes;              /* algorithmic bytes moved by those launches */
} fs_kernel_time;

/* ---------------------------------------------------------------- lifecycle */
FS_API void fs_params_default(fs_params* params);
/* new GPUFluidSolver(device, opts) + createDevice (solver.js:43-98) */
FS_API int fs_create(const fs_params* params, fs_solver** out);
/* destroy() (solver.js:898-911) */
FS_API void fs_destroy(fs_solver* s);
/* Message of the last failure on s; with s == NULL, of the last failed
 * fs_create on this thread.  Valid until the next call on the same handle. */
FS_API const char* fs_last_error(const fs_solver* s);
FS_API const char* fs_status_string(int status);
FS_API int fs_get_params(const fs_solver* s, fs_params* out);

/* -------------------------------------------------------------- field I/O */
/* uploadVelocity(u, v) (solver.js:301-315); dtype selects f32 or f64 input.
 * Returns once u and v have been read (the caller may reuse them), as the
 * reference copies them at the call. */
FS_API int fs_upload_velocity(fs_solver* s, const void* u, const void* v, int dtype);
/* readVelocity() (solver.js:356-362); synchronises */
FS_API int fs_read_velocity(fs_solver* s, void* u, void* v, int dtype);
/* readTexture(tex) for the other fields (solver.js:336-353); synchronises */
FS_API int fs_read_field(fs_solver* s, int field, void* out, int dtype);
/* set the pressure a warm-started projection starts from (FS_FIELD_PRESSURE only) */
FS_API int fs_upload_field(fs_solver* s, int field, const void* data, int dtype);

/* ----------------------------------------------------- forces and solids */
/* setForcing(modes, {amplitude, drag, phaseDrift}) (solver.js:370-385);
 * count == 0 disables the forcing pass */
FS_API int fs_set_forcing(fs_solver* s, const fs_mode* modes, int count, double amplitude,
                          double drag, double phase_drift);
/* Band-limited random forcing renewed every step, plus linear drag: the
 * forced-turbulence driver of the reference (bandForcing + linearDrag,
 * src/cpu/solver.js:179-237, passed to FluidSolver.step as opts.force /
 * opts.drag with a seed that grows by one per step,
 * validate/longrun-spectrum.js:65-67).  Each step adds the curl of
 * psi = sum_m A_m cos(kx_m x + ky_m y + phi_m), scaled by amplitude*dt/sqrt(M),
 * to the velocity after diffusion, then multiplies it by exp(-drag dt); the
 * fixed-mode forcing of fs_set_forcing, if also set, follows. */
typedef enum fs_band_kind {
  /* bandForcing itself: 24 modes drawn by its 32-bit LCG from seed + step,
   * |k| = kf + (r - 1/2) 2 width at a random angle, rounded; A = 1 */
  FS_BAND_REFERENCE = 0,
  /* every integer (kx, ky) with kf - width <= |k| <= kf + width (ky, then kx
   * ascending), each with a complex Gaussian amplitude (sigma 1 per part)
   * from Philox4x32-10, key = seed, counter = (step, mode index, 0, 0) */
  FS_BAND_GAUSSIAN = 1
} fs_band_kind;

typedef struct fs_band {
  int32_t kind;       /* fs_band_kind */
  double kf, width;   /* the band: centre and half-width in wave numbers */
  double amplitude;   /* amp of bandForcing */
  uint64_t seed;      /* draws of the solver's k-th forced step use seed + k
                         (REFERENCE) or counter k (GAUSSIAN) */
  double drag;        /* linear drag alpha >= 0 (linearDrag) */
} fs_band;

/* band == NULL removes it.  Setting it restarts the step counter of the
 * draws at 0.  Drops the captured step. */
FS_API int fs_set_band_forcing(fs_solver* s, const fs_band* band);

/* A channel with inflow, outflow and no-slip walls on the periodic grid.  No
 * counterpart in the reference, which is periodic only (README.md:139); the
 * walls use the reference's immersed-disk direct forcing
 * (src/cpu/solid.js:165-233) on a slab instead of a disk, and the inflow /
 * outflow a fringe strip (the fringe-region method of spectral channel
 * codes).  Each step, after the forces and before the disks:
 *   fringe: chi_f = 1/2 (1 - tanh((|x - fringe_x| - fringe_half) / fringe_ramp))
 *           u += chi_f (inflow_u - u), v += chi_f (0 - v)   where chi_f >= 1e-6
 *   walls:  chi_w = 1/2 (1 - tanh((|y - wall_y| - wall_half) / w)),
 *           w = solid_mask_width cells;
 *           u += chi_w (0 - u), v += chi_w (0 - v)          where chi_w >= 1e-6
 * at each face's position (distances periodic).  The slab's two edges are
 * the walls; flow leaves through the fringe and re-enters past it as the
 * uniform inflow u = inflow_u.  The pressure stays periodic. */
typedef struct fs_channel {
  double wall_y, wall_half;                     /* wall slab centre and half-thickness (y) */
  double fringe_x, fringe_half, fringe_ramp;    /* fringe centre, half-width, ramp width (x) */
  double inflow_u;                              /* U_in */
} fs_channel;
/* c == NULL removes it; drops the captured step */
FS_API int fs_set_channel(fs_solver* s, const fs_channel* c);

/* setSolid(disk) (solver.js:425-438), generalised to count disks applied in
 * order (src/cpu/solid.js:181-230); count == 0 removes them */
FS_API int fs_set_solids(fs_solver* s, const fs_disk* disks, int count);
/* Impulse the last coupling pass gave the fluid, per disk: out[3k+0..2] =
 * (sum du dA, sum dv dA, sum torque dA), reduced on the device (replaces the
 * readback + CPU sum of integrateSolid, solver.js:477-510); synchronises */
FS_API int fs_solid_impulse(fs_solver* s, double* out, int count);

/* ------------------------------------------------------------------ step */
/* step(dt) (solver.js:518-591): advect, diffuse, force, solids, project.
 * Fused multigrid configurations (kernel_variant 0) run the step as one CUDA
 * graph, captured on the first call for a given dt; its tolerance loop is a
 * conditional node decided on the device, so fs_step never waits, and a
 * tolerance failure is reported by fs_last_stats.  Other configurations run
 * eagerly; with pressure_tol > 0 they read one residual word per cycle and
 * return FS_ERR_NOT_CONVERGED / FS_ERR_NONFINITE themselves (the step is
 * still applied). */
FS_API int fs_step(fs_solver* s, double dt);
/* nsteps consecutive steps */
FS_API int fs_advance(fs_solver* s, double dt, int nsteps);
FS_API int fs_sync(fs_solver* s);
/* statistics of the last projection; synchronises.  Returns
 * FS_ERR_NOT_CONVERGED / FS_ERR_NONFINITE when that projection's tolerance
 * loop failed inside a captured step. */
FS_API int fs_last_stats(fs_solver* s, fs_step_stats* out);
/* simulation time and step count (the public fields t and steps) */
FS_API int fs_get_time(const fs_solver* s, double* t, int64_t* steps);
/* run one stage of the step by itself (see fs_stage) */
FS_API int fs_run_stage(fs_solver* s, int stage, double dt);

/* ------------------------------------------------------------ diagnostics */
/* maxDivergence() (solver.js:835-850), reduced on the device; synchronises */
FS_API int fs_max_divergence(fs_solver* s, double* out);
/* poissonResidualAfter(iterations, dt) (solver.js:857-896): divergence, zero
 * pressure, `iterations` sweeps / V-cycles, then ||lap p - div|| / ||div||
 * reduced in f64 on the device; synchronises */
FS_API int fs_poisson_residual_after(fs_solver* s, int iterations, double dt, double* out);

/* -------------------------------------------------------------- measurement */
/* Time nsteps steps with CUDA events recorded on the solver's stream; writes
 * the elapsed milliseconds.  Synchronises. */
FS_API int fs_time_steps(fs_solver* s, double dt, int nsteps, double* elapsed_ms);
/* Run nsteps steps with a CUDA event pair around every kernel launch and
 * return per-kernel launch counts, total times and algorithmic bytes
 * (out has room for cap entries; *count gets the number written). */
FS_API int fs_profile_step(fs_solver* s, double dt, int nsteps, fs_kernel_time* out, int cap,
                           int* count);
/* Number of kernels this handle has run since creation (graph replays
 * included; synchronises when a captured tolerance loop has to be counted). */
FS_API int64_t fs_launch_count(const fs_solver* s);
/* Page-locked host memory for fast uploads and read-backs (cudaMallocHost). */
FS_API void* fs_host_alloc(size_t bytes);
FS_API void fs_host_free(void* p);

/* ---------------------------------------------------- allocation-free entry */
/* No counterpart in the reference.  max|div u| of an f32 MAC velocity field
 * that the caller already holds on the CURRENT device (d_u, d_v: nx*ny floats,
 * row-major), written as one double to the device pointer d_out, enqueued on
 * `stream` (a cudaStream_t; NULL = the legacy default stream).
 *
 * For callers that cannot allocate device memory while they run -- hosts that
 * reserve the GPU through their own pool, frame loops that must not call
 * cudaMalloc/cudaFree (they can synchronise the device).  It calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch (per-block
 * maxima and an arrival counter) is a static device array of 65536 + 64
 * floats (256 KB) that every GPU loading the library holds until the process
 * exits.
 *
 *  - Grids are limited to 65536 blocks of 32x8 cells (at most 16,777,216
 *    cells, e.g. 4096 x 4096) and to ny <= 524280 (65535 block rows); other
 *    grids return FS_ERR_INVALID_ARGUMENT before anything is enqueued.
 *  - The first call on a device looks up the device address of that array
 *    (with the device current) and keeps it; make that first call before any
 *    stream capture begins.  The kept address is stale after cudaDeviceReset
 *    of that device: do not call this entry point on a device after resetting
 *    it.
 *  - All calls share the one array: calls that can overlap on the GPU
 *    (different streams, no ordering between them) race and may return
 *    wrong maxima.  Each call clears the counter it needs before its kernel.
 *  - On failure fs_last_error(NULL) returns the message. */
FS_API int fs_max_divergence_noalloc(const float* d_u, const float* d_v, int32_t nx, int32_t ny, double lx,
                                     double ly, double* d_out, void* stream);

/* ------------------------------------------------------------------------
 * Tensor-core building blocks of the learned pressure guess.  No counterpart
 * in the reference (which has no learned component); these sit beside the
 * solver, not in place of any reference function.
 * ------------------------------------------------------------------------ */

/* 3x3 periodic convolution of NHWC bf16 images on the tcgen05 tensor cores:
 *   out[b,y,x,co] = bias[co] + sum_{ky,kx,ci} w[co,ci,ky,kx] in[b, y+ky-1, x+kx-1, ci]
 * with x, y wrapped.  d_wpacked holds w as bf16 in the layout
 * [ky*3+kx][ci/8][co][ci%8].  epilogue 0: bf16 out, 1: bf16 out after ReLU,
 * 2: f32 planar [b][y][x] of output channel 0 only (c_out must be 16).
 * Instantiated channel pairs: 16->16, 16->32, 32->16, 32->64, 64->32,
 * 64->128, 128->64.  Buffers 16-byte aligned; device pointers; enqueued on
 * `stream`.  *d_err is set to 1 if a tensor-core completion wait timed out. */
FS_API int fs_conv3x3_bf16(const void* d_in, const void* d_wpacked, const float* d_bias, void* d_out, int32_t batch,
                           int32_t h, int32_t w, int32_t c_in, int32_t c_out, int32_t epilogue, int32_t* d_err,
                           void* stream);

/* One 128 x n tile D = A B^T (A 128 x k, B n x k, row-major bf16; D f32
 * row-major) through the same tcgen05 path: a device self-check of the
 * descriptors and the accumulator read-back.  n in {16, 64}, k in {16..64}. */
FS_API int fs_tc_gemm_check(const void* d_a, const void* d_b, float* d_d, int32_t n, int32_t k, int32_t* d_err,
                            void* stream);

/* ------------------------------------------------------------------------
 * Learned pressure guess: a periodic U-Net (4 levels, 16/32/64/128 channels,
 * 3x3 convolutions, ReLU, 2x2 average pooling, nearest upsampling with
 * additive skips; bf16 weights and activations, f32 accumulation) mapping
 * the divergence and the solid mask at half the grid resolution to an
 * initial pressure.  With a guess attached, the multigrid projection starts
 * from it instead of zero and still iterates to pressure_tol, so plain
 * multigrid stays both the fallback and the yardstick.  No reference counterpart.
 *
 * Network inputs at its own resolution H x W (multiples of 8):
 *   div_n = h^2 d / sigma, sigma = RMS(h^2 d) per sample (h = grid spacing),
 *   mask  = solid mask in [0, 1];
 * output p / sigma (pressure up to a constant).  Parameters: f32, flattened
 * layer by layer (A..J) as w[c_out][c_in][3][3] then b[c_out].  Data pointers
 * of predict / loss_grad / train_step are device pointers, f32 [B][H][W].
 * ------------------------------------------------------------------------ */
typedef struct fs_guess fs_guess;

/* He-normal initial weights from `seed` (SplitMix64 + Box-Muller). */
FS_API int fs_guess_create(int32_t device, uint64_t seed, fs_guess** out);
FS_API void fs_guess_destroy(fs_guess* g);
FS_API int64_t fs_guess_num_params(const fs_guess* g);
FS_API int fs_guess_get_params(fs_guess* g, float* host, int64_t n);
/* also resets the Adam moments and step count */
FS_API int fs_guess_set_params(fs_guess* g, const float* host, int64_t n);
FS_API int fs_guess_predict(fs_guess* g, const float* d_div_n, const float* d_mask, int32_t batch, int32_t h,
                            int32_t w, float* d_out);
/* loss = mean over batch and pixels of w_p (e - mean_b e)^2 + w_r (lap e)^2,
 * e = out - target (weights from fs_guess_set_loss);
 * d_grad (nullable, n floats on the device) receives dloss/dparams */
FS_API int fs_guess_loss_grad(fs_guess* g, const float* d_div_n, const float* d_mask, const float* d_target,
                              int32_t batch, int32_t h, int32_t w, double* loss, float* d_grad);
/* loss_grad then one Adam step (beta1 0.9, beta2 0.999, eps 1e-8, bias
 * corrected).  With loss == NULL the call does not synchronise. */
FS_API int fs_guess_train_step(fs_guess* g, const float* d_div_n, const float* d_mask, const float* d_target,
                               int32_t batch, int32_t h, int32_t w, float lr, double* loss);
/* Loss weights (default 1, 0): w_pressure on the mean-free squared pressure
 * error, w_residual on the squared periodic 5-point Laplacian of the error
 * (l + r + b + t - 4c, unscaled), which in the network's units is the initial
 * residual of the projection the guess seeds. */
FS_API int fs_guess_set_loss(fs_guess* g, double w_pressure, double w_residual);
FS_API int fs_guess_sync(fs_guess* g);
FS_API int64_t fs_guess_launch_count(const fs_guess* g);

/* Attach (or with NULL detach) a guess to a multigrid solver.  The network
 * runs at 1/factor of the grid resolution (factor 1 or 2; nx, ny multiples of
 * 8 * factor); the divergence is block-averaged in and the output
 * prolongated back (bilinear, the multigrid stencil) for factor 2.  The
 * solver does not own g; keep g alive while attached. */
FS_API int fs_set_guess(fs_solver* s, fs_guess* g, int32_t factor);

/* The training pair of the last projection: divergence, solid mask and
 * pressure averaged over factor x factor cells (mask at the coarse cell
 * centres), host f32 arrays of (nx/factor) x (ny/factor).  Synchronises. */
FS_API int fs_dump_pair(fs_solver* s, int32_t factor, float* div, float* mask, float* p);
/* The same pair into device buffers the caller owns (f32, (nx/factor) x
 * (ny/factor) each), enqueued on the solver's stream without synchronising:
 * a training loop streams pairs straight from the solver into its batches. */
FS_API int fs_dump_pair_device(fs_solver* s, int32_t factor, float* d_div, float* d_mask, float* d_p);

/* Training-pair file ("FSPAIR" v1): 40-byte header {magic "FSPAIR\0\1",
 * u32 version = 1, u32 nx, u32 ny, u32 dtype = 0 (f32), f64 dx, u32 nfields =
 * 3, u32 0} then div, mask, p as f32 [ny][nx], little-endian.  Reading with
 * div == NULL fills only nx, ny, dx. */
FS_API int fs_write_pair_file(const char* path, int32_t nx, int32_t ny, double dx, const float* div,
                              const float* mask, const float* p);
FS_API int fs_read_pair_file(const char* path, int32_t* nx, int32_t* ny, double* dx, float* div, float* mask,
                             float* p);


/* ------------------------------------------------------------------------
 * Dye (uploadDye, solver.js:317-323; ADVECT_SCALAR, shaders.js:234-266): an
 * RGBA f32 field at the cell centres, [ny][nx][4].  Once uploaded, every step
 * advects it semi-Lagrangian through the projected velocity, fades it by
 * dye_fade and clamps it to [0, 1], as the reference does.
 * ------------------------------------------------------------------------ */
FS_API int fs_upload_dye(fs_solver* s, const float* rgba);
FS_API int fs_read_dye(fs_solver* s, float* rgba);

/* The arithmetic of the reference's RENDER pass (shaders.js:677-768) into a
 * buffer instead of a swapchain (no graphics API): linear RGBA f32 per cell,
 * [ny][nx][4], host array.  mode 0 colours the centre vorticity
 * tanh(w * exposure) on a magenta / cyan ramp, mode 1 the speed; both add the
 * exposure-scaled speed glow and, if uploaded, the dim dye lift.  exposure is
 * the reference's param_a.  Synchronises. */
FS_API int fs_render(fs_solver* s, int32_t mode, double exposure, float* rgba);

/* Multigrid sweep counts of an existing solver (drops the captured step). */
FS_API int fs_set_mg_sweeps(fs_solver* s, int32_t pre, int32_t post);
/* refinement cycles run by every projection of the tolerance loop since
 * creation (a device counter; synchronises) */
FS_API int fs_total_cycles(fs_solver* s, int64_t* cycles);
/* Record of every tolerance-loop projection the solver's steps have run
 * since creation: how many, how many ended without meeting pressure_tol
 * (max_cycles reached or a non-finite residual), and the largest final
 * max|div u| among them (+inf if one was non-finite).  fs_last_stats reports
 * only the last projection; this covers every step of a long run, including
 * steps replayed from a captured graph whose loop ran on the device.  No
 * counterpart in the reference (its projection runs a fixed count and never
 * reports convergence).  Synchronises. */
FS_API int fs_convergence_record(fs_solver* s, int64_t* steps, int64_t* failed_steps, double* worst_residual);
/* Autotuner: times nsteps steps of dt for every (pre, post) sweep pair the
 * fused kernels take (1..3 each), from the same saved state each time, and
 * keeps the fastest that still meets pressure_tol; the state, dye, time and
 * pressure are restored afterwards.  No reference counterpart. */
FS_API int fs_autotune(fs_solver* s, double dt, int32_t nsteps, int32_t* pre, int32_t* post, double* ms_per_step);
/* Tile sides (16, 32 or 64 cells) of the fused multigrid kernels of each tile
 * level (the levels above the bottom solve); 0 = the built-in rule (64 where
 * that gives >= 1024 CTAs, else 32 where that gives >= 256, else 16).  A side
 * larger than half its level is not used there (the built-in rule applies;
 * fs_get_mg_tiles reports the side in use).  The tiles give the same values
 * whatever their size, so they change only the speed. */
FS_API int fs_set_mg_tiles(fs_solver* s, const int32_t* tiles, int32_t count);
/* the sides in use, one per tile level (*count = number of tile levels) */
FS_API int fs_get_mg_tiles(fs_solver* s, int32_t* tiles, int32_t cap, int32_t* count);
/* Greedy per level: every tile level tries 64, 32 and 16 (the others fixed),
 * each timed over nsteps steps from the same saved state; keeps the fastest.
 * The state and time are restored; tiles_out gets the picks (0 = rule kept). */
FS_API int fs_autotune_tiles(fs_solver* s, double dt, int32_t nsteps, int32_t* tiles_out, int32_t cap,
                             int32_t* count, double* ms_per_step);

/* ------------------------------------------------------------------------
 * Diagnostics on the device (the reference reads the fields back and loops
 * on the CPU: src/core/grid.js:280-327, src/core/fft.js:196-254).
 * ------------------------------------------------------------------------ */
typedef struct fs_diagnostics {
  double kinetic_energy; /* 1/2 <cu^2 + cv^2>, velocity at cell centres */
  double enstrophy;      /* 1/2 <w^2>, w = mean of the 4 corner vorticities */
  double max_divergence; /* max |div u| */
  double l2_divergence;  /* sqrt(<div u^2>) */
} fs_diagnostics;
/* all four in one reduction kernel, per-cell values in f32 and sums in
 * double (fs_max_divergence is the double-float-exact divergence check);
 * synchronises */
FS_API int fs_diagnose(fs_solver* s, fs_diagnostics* out);
/* Shell-averaged energy spectrum E[k], k = 0..kmax = n/2 (square power-of-two
 * grids 8..8192): E[k] = sum over modes with round(|k|) = k of
 * 1/2 (|U|^2 + |V|^2) / N^2, counts[k] the modes per shell (cap >= kmax + 1).
 * parseval (nullable, 2 doubles): sum E and the kinetic energy it should
 * match (modes beyond kmax are dropped, as in the reference).  Synchronises. */
FS_API int fs_energy_spectrum(fs_solver* s, double* E, int32_t* counts, int32_t cap, int32_t* kmax,
                              double* parseval);

/* ------------------------------------------------------------------------
 * Batches: many independent simulations of uneven sizes advanced by one CUDA
 * graph launch per step (each member's step, with its own tolerance loop, is
 * an independent branch of the graph; the branches overlap on the GPU).  No
 * reference counterpart (the reference steps one solver per submit).
 * Members need the fused multigrid step (pressure_solver = MULTIGRID,
 * kernel_variant = 0, nx == ny).  Member handles are owned by the batch (do
 * not fs_destroy them); use them for upload / read-back / solids / stats.
 * Eager calls on members and batch steps share one stream, so they are
 * ordered without further synchronisation.
 * ------------------------------------------------------------------------ */
typedef struct fs_batch fs_batch;
FS_API int fs_batch_create(const fs_params* params, int32_t count, fs_batch** out);
FS_API void fs_batch_destroy(fs_batch* b);
FS_API int32_t fs_batch_size(const fs_batch* b);
FS_API fs_solver* fs_batch_member(fs_batch* b, int32_t index);
FS_API const char* fs_batch_last_error(const fs_batch* b);
/* one step of every member; dt[i] per member.  The graph is re-captured when
 * a dt changes or a member's forcing / solids / guess changed. */
FS_API int fs_batch_step(fs_batch* b, const double* dt);
FS_API int fs_batch_sync(fs_batch* b);
/* nsteps batch steps between two events on the batch stream (capture first) */
FS_API int fs_batch_time_steps(fs_batch* b, const double* dt, int32_t nsteps, double* elapsed_ms);
FS_API int64_t fs_batch_launch_count(fs_batch* b);
/* tile sides per size class and tile level, greedy, each candidate timed as
 * nsteps whole batch steps from the same saved state of every member (which
 * is restored); the picks are set on the members (fs_get_mg_tiles) */
FS_API int fs_batch_autotune_tiles(fs_batch* b, const double* dt, int32_t nsteps, double* ms_per_step);
/* the (pre, post) sweep pair of each size class, timed the same way; the
 * picks are set on the members (fs_params mg_pre_smooth / mg_post_smooth) */
FS_API int fs_batch_autotune(fs_batch* b, const double* dt, int32_t nsteps, double* ms_per_step);

#ifdef __cplusplus
}
#endif
#endif
