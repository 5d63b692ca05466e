// fs_api.cu -- the C ABI of libfluidcuda (include/fluid.h): solver lifecycle,
// field I/O, the step orchestration and diagnostics.
//
// Reference: the GPUFluidSolver class, src/gpu/solver.js:64-912, and the
// Multigrid hierarchy of src/gpu/multigrid.js:159-205.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "fs_internal.cuh"

struct fs_solver {
  fs::Solver s;
};

namespace fs {

static thread_local std::string g_create_error;

// message for fs_last_error(NULL) from entry points that take no handle
void record_error(const std::string& msg) { g_create_error = msg; }

// ------------------------------------------------------------------ errors
static int fail(Solver* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  else g_create_error = msg;
  return code;
}
int fail_status(Solver* s, int code, const std::string& msg) { return fail(s, code, msg); }

#define CU(S, call)                                                                          \
  do {                                                                                       \
    cudaError_t _e = (call);                                                                 \
    if (_e != cudaSuccess)                                                                   \
      return fail((S), _e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(_e));                       \
  } while (0)

static int check_launch(Solver* s) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(s, FS_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return FS_OK;
}

// --------------------------------------------------------------- profiling
void prof_begin(Solver* s, const char* name, double bytes, int* slot, cudaEvent_t* a) {
  int idx = -1;
  for (size_t k = 0; k < s->kstats.size(); k++)
    if (s->kstats[k].name == name) { idx = (int)k; break; }
  if (idx < 0) {
    s->kstats.push_back(KernelStat{name, 0, 0.0, 0.0});
    idx = (int)s->kstats.size() - 1;
  }
  s->kstats[idx].launches++;
  s->kstats[idx].bytes += bytes;
  cudaEventCreate(a);
  cudaEventRecord(*a, s->stream);
  *slot = idx;
}

void prof_end(Solver* s, int slot, cudaEvent_t a) {
  cudaEvent_t b;
  cudaEventCreate(&b);
  cudaEventRecord(b, s->stream);
  s->pending.push_back(Solver::Pending{slot, a, b});
}

static void prof_collect(Solver* s) {
  cudaStreamSynchronize(s->stream);
  for (auto& p : s->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    s->kstats[p.stat].ms += ms;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  s->pending.clear();
}

// ---------------------------------------------------------------- helpers
static bool is_pow2_multiple(int n, int levels) { return n % (1 << (levels - 1)) == 0; }

template <class T>
static int dalloc(Solver* s, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return FS_OK;
  CU(s, cudaMalloc((void**)p, count * sizeof(T)));
  return FS_OK;
}

static void free_all(Solver* s) {
  auto f = [](void* p) { if (p) cudaFree(p); };
  f(s->u); f(s->v); f(s->wu); f(s->wv); f(s->tu); f(s->tv); f(s->fu); f(s->fv);
  f(s->ulo); f(s->vlo); f(s->mc_bounds);
  f(s->p32); f(s->p32b); f(s->div32); f(s->ph); f(s->pl); f(s->pbh); f(s->pbl); f(s->dh); f(s->dl);
  f(s->r32); f(s->e32); f(s->e32b); f(s->scratch);
  for (size_t l = 1; l < s->lev.size(); l++) { f(s->lev[l].x); f(s->lev[l].x2); f(s->lev[l].rhs); }
  f(s->stage);
  f(s->red_partials); f(s->red_out); f(s->modes); f(s->imp); f(s->d_impulse);
  f(s->dev); f(s->d_disks); f(s->d_tiles); f(s->d_tile_masks); f(s->dye); f(s->dye2);
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->h_red) cudaFreeHost(s->h_red);
  diag_free(s);
  band_free(s);
  if (s->body_stream) cudaStreamDestroy(s->body_stream);
  if (s->own_stream) {
    cudaStreamDestroy(s->own_stream);  // batch member: s->stream is the batch's
  } else if (s->stream) {
    cudaStreamDestroy(s->stream);
  }
}

static int sync(Solver* s) {
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

// read the reduction words back (synchronises)
static int read_red(Solver* s, double* a, double* b = nullptr) {
  CU(s, cudaMemcpyAsync(s->h_red, s->red_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CU(s, cudaStreamSynchronize(s->stream));
  if (a) *a = s->h_red[0];
  if (b) *b = s->h_red[1];
  return FS_OK;
}

// -------------------------------------------------------------- creation
static int create(const fs_params* prm, Solver* s) {
  s->prm = *prm;
  const fs_params& P = s->prm;
  if (P.nx < 2 || P.ny < 2) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "grid must be at least 2x2");
  if ((int64_t)P.nx * P.ny > (int64_t)1 << 30) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "grid larger than 2^30 cells");
  if (!(P.lx > 0) || !(P.ly > 0)) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "domain size must be positive");
  if (!(P.nu >= 0)) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "nu must be >= 0");
  if (!(P.dye_fade >= 0) || !(P.dye_fade <= 1)) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "dye_fade must be in [0, 1]");
  if (!(P.relax > 0) || !(P.relax < 2)) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "relax must be in (0, 2)");
  if (P.pressure_tol_relative != 0 && P.pressure_tol_relative != 1)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "pressure_tol_relative must be 0 or 1");
  if (P.confinement != 0)
    return fail(nullptr, FS_ERR_UNSUPPORTED, "vorticity confinement is not part of this path (it must stay off)");
  if (P.advection != FS_ADVECT_SEMI_LAGRANGIAN && P.advection != FS_ADVECT_MACCORMACK)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "unknown advection scheme");
  if (P.pressure_solver < FS_PRESSURE_JACOBI || P.pressure_solver > FS_PRESSURE_MULTIGRID)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "unknown pressure solver");
  if (P.precision != FS_PRECISION_F32 && P.precision != FS_PRECISION_MIXED)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "unknown precision");
  if (P.pressure_iterations < 0 || P.max_cycles < 1 || !(P.pressure_tol >= 0))
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "bad iteration settings");
  if (P.mg_pre_smooth < 0 || P.mg_post_smooth < 0 || P.mg_coarse_sweeps < 0 || P.mg_min_size < 2)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "bad multigrid settings");
  if (P.mg_first_pre < -1 || P.mg_first_pre > P.mg_pre_smooth || P.mg_first_post < -1 ||
      P.mg_first_post > P.mg_post_smooth)
    return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "mg_first_pre / mg_first_post must be -1 or 0 .. the cycle's sweeps");
  if ((P.mg_first_pre >= 0 || P.mg_first_post >= 0) && P.kernel_variant != 0)
    return fail(nullptr, FS_ERR_UNSUPPORTED, "mg_first_pre / mg_first_post need the fused multigrid kernels");
  if (!(P.solid_mask_width > 0)) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "solid_mask_width must be > 0");
  if (P.kernel_variant < 0 || P.kernel_variant > 1) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "unknown kernel_variant");

  s->mixed = P.precision == FS_PRECISION_MIXED;
  s->odd = (P.nx & 1) || (P.ny & 1);
  s->n = (int64_t)P.nx * P.ny;
  Grid& g = s->g;
  g.nx = P.nx; g.ny = P.ny;
  g.dxd = P.lx / P.nx; g.dyd = P.ly / P.ny;
  g.idxd = 1.0 / g.dxd; g.idyd = 1.0 / g.dyd;
  g.dx = (float)g.dxd; g.dy = (float)g.dyd;
  g.idx = (float)g.idxd; g.idy = (float)g.idyd;

  // multigrid hierarchy (multigrid.js:177-197): square, n -> n/2 while >= min
  if (P.pressure_solver == FS_PRESSURE_MULTIGRID) {
    if (P.nx != P.ny) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "multigrid needs a square grid");
    int m = P.nx, count = 0;
    while (m >= P.mg_min_size) {
      count++;
      if (m / 2 < P.mg_min_size) break;
      if (m & 1) break;
      m /= 2;
    }
    if (count < 1) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "grid smaller than mg_min_size");
    if (!is_pow2_multiple(P.nx, count))
      return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "multigrid needs n divisible by 2^(levels-1)");
    int n = P.nx;
    double fine = g.dxd * P.nx;
    for (int l = 0; l < count; l++, n /= 2) {
      Level L{};
      L.n = n;
      L.dx = (float)(fine / n);
      L.h2 = L.dx * L.dx;
      s->lev.push_back(L);
    }
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, FS_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (P.device < 0 || P.device >= ndev) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "device ordinal out of range");
  s->device = P.device;
  if (cudaSetDevice(s->device) != cudaSuccess) return fail(nullptr, FS_ERR_CUDA, "cudaSetDevice failed");

  CU(nullptr, cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  const int64_t n = s->n;
  int rc;
#define A(ptr, T, cnt) if ((rc = dalloc(s, (T**)&(ptr), (size_t)(cnt))) != FS_OK) return rc
  A(s->u, float, n); A(s->v, float, n);
  if (s->mixed) {
    A(s->ulo, float, n); A(s->vlo, float, n);
    A(s->ph, float, n); A(s->pl, float, n); A(s->pbh, float, n); A(s->pbl, float, n);
    A(s->dh, float, n); A(s->dl, float, n);
    A(s->r32, float, n); A(s->e32, float, n); A(s->e32b, float, n);
  } else {
    A(s->p32, float, n); A(s->p32b, float, n); A(s->div32, float, n);
  }
  A(s->wu, float, n); A(s->wv, float, n); A(s->tu, float, n); A(s->tv, float, n);
  if (P.advection == FS_ADVECT_MACCORMACK) {
    A(s->fu, float, n);
    A(s->fv, float, n);
    A(s->mc_bounds, float, 4 * n);
  }
  if (!s->lev.empty()) {
    A(s->scratch, float, n);
    s->lev[0].x = s->mixed ? s->e32 : s->p32;
    s->lev[0].x2 = s->mixed ? s->e32b : s->p32b;
    s->lev[0].rhs = s->mixed ? s->r32 : s->div32;
    for (size_t l = 1; l < s->lev.size(); l++) {
      int64_t m = (int64_t)s->lev[l].n * s->lev[l].n;
      A(s->lev[l].x, float, m); A(s->lev[l].rhs, float, m); A(s->lev[l].x2, float, m);
    }
    s->fused = P.kernel_variant == 0 && mg_fused_supported(s);
  }
  // reductions: partial buffer for the largest grid launch plus the counter word
  int64_t blocks = (int64_t)((P.nx + 31) / 32) * ((P.ny + 7) / 8);
  s->red_cap = (int)std::max<int64_t>(blocks, 4096);
  // [2*cap f64 sums][cap f32 maxima][counter word]
  A(s->red_partials, double, 2 * (int64_t)s->red_cap + (s->red_cap + 2) / 2 + 1);
  A(s->red_out, double, 4);
  A(s->dev, DevState, 1);
#undef A
  CU(s, cudaMemsetAsync(s->red_partials, 0, (2 * (size_t)s->red_cap + (s->red_cap + 2) / 2 + 1) * sizeof(double),
                        s->stream));
  CU(s, cudaMallocHost((void**)&s->h_red, 4 * sizeof(double)));
  CU(s, cudaMemsetAsync(s->dev, 0, sizeof(DevState), s->stream));
  CU(s, cudaStreamCreateWithFlags(&s->body_stream, cudaStreamNonBlocking));
  // every field starts at zero
  CU(s, cudaMemsetAsync(s->u, 0, n * 4, s->stream));
  CU(s, cudaMemsetAsync(s->v, 0, n * 4, s->stream));
  if (s->mixed) {
    for (float* q : {s->ulo, s->vlo, s->ph, s->pl, s->dh, s->dl}) CU(s, cudaMemsetAsync(q, 0, n * 4, s->stream));
  } else {
    CU(s, cudaMemsetAsync(s->p32, 0, n * 4, s->stream));
    CU(s, cudaMemsetAsync(s->div32, 0, n * 4, s->stream));
  }
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

// -------------------------------------------------------- the projection
// F32 Poisson solve on (p32, div32): `iterations` sweeps or V-cycles
// (_encodePoisson, solver.js:686-738)
static void poisson_f32(Solver* s, int iterations, bool p_nonzero) {
  const fs_params& P = s->prm;
  const Grid& g = s->g;
  float h2 = g.dx * g.dx;
  if (P.pressure_solver == FS_PRESSURE_MULTIGRID) {
    s->lev[0].x = s->p32;
    s->lev[0].x2 = s->p32b;
    for (int k = 0; k < iterations; k++) {
      if (s->fused) mg_vcycle_fused(s, p_nonzero || k > 0);
      else mg_vcycle(s);
    }
    s->p32 = s->lev[0].x;
    s->p32b = s->lev[0].x2;
    return;
  } else if (P.pressure_solver == FS_PRESSURE_RED_BLACK) {
    for (int k = 0; k < iterations; k++)
      for (int colour = 0; colour < 2; colour++) {
        if (!s->odd) {
          launch_rb_half(s, s->p32, s->div32, s->p32, h2, colour, g.nx, g.ny);
        } else {
          launch_rb_half(s, s->p32, s->div32, s->p32b, h2, colour, g.nx, g.ny);
          std::swap(s->p32, s->p32b);
        }
      }
  } else {
    for (int k = 0; k < iterations; k++) {
      launch_jacobi(s, s->p32, s->div32, s->p32b, h2, g.nx, g.ny);
      std::swap(s->p32, s->p32b);
    }
  }
}

// correction solve of the MIXED mode: e32 from r32 starting at zero
static void correction_solve(Solver* s, int iterations) {
  const fs_params& P = s->prm;
  const Grid& g = s->g;
  float h2 = g.dx * g.dx;
  if (P.pressure_solver == FS_PRESSURE_MULTIGRID) {
    s->lev[0].x = s->e32;
    s->lev[0].x2 = s->e32b;
    if (!s->fused) launch_fill(s, s->e32, 0.f, s->n);  // the fused cycle starts from zero itself
    for (int k = 0; k < iterations; k++) {
      if (s->fused) mg_vcycle_fused(s, k > 0);
      else mg_vcycle(s);
    }
    s->e32 = s->lev[0].x;
    s->e32b = s->lev[0].x2;
    return;
  }
  launch_fill(s, s->e32, 0.f, s->n);
  if (P.pressure_solver == FS_PRESSURE_RED_BLACK) {
    for (int k = 0; k < iterations; k++)
      for (int colour = 0; colour < 2; colour++) {
        if (!s->odd) {
          launch_rb_half(s, s->e32, s->r32, s->e32, h2, colour, g.nx, g.ny);
        } else {
          launch_rb_half(s, s->e32, s->r32, s->e32b, h2, colour, g.nx, g.ny);
          std::swap(s->e32, s->e32b);
        }
      }
  } else {
    for (int k = 0; k < iterations; k++) {
      launch_jacobi(s, s->e32, s->r32, s->e32b, h2, g.nx, g.ny);
      std::swap(s->e32, s->e32b);
    }
  }
}

// One cycle of the multigrid tolerance loop (both precisions):
//   F32:   one V-cycle on (p32, div32) from the current p [+ max|div - lap p|]
//   MIXED: one V-cycle on (r32 -> e) from zero, p += e (double-float), then
//          r = d - lap p -> r32 and max|r|.
// The fused F32 cycle always reads p (the zero-initial-guess shortcut would
// change the kernel sequence from the first cycle to the next, which a
// replayed loop body cannot do); reading a zero p gives the same bits.
static void mg_cycle(Solver* s, bool residual) {
  if (s->mixed) {
    s->lev[0].x = s->e32;
    s->lev[0].x2 = s->e32b;
    if (s->fused) {
      mg_vcycle_fused(s, false, s->ph, s->pl);
      launch_refine_init(s, s->dh, s->dl, s->ph, s->pl, s->r32, false);
    } else {
      launch_fill(s, s->e32, 0.f, s->n);
      mg_vcycle(s);
      launch_refine_update(s, s->ph, s->pl, s->e32, s->dh, s->dl, s->pbh, s->pbl, s->r32);
      std::swap(s->ph, s->pbh);
      std::swap(s->pl, s->pbl);
    }
    return;
  }
  s->lev[0].x = s->p32;
  s->lev[0].x2 = s->p32b;
  if (s->fused) mg_vcycle_fused(s, true);
  else mg_vcycle(s);
  s->p32 = s->lev[0].x;
  s->p32b = s->lev[0].x2;
  if (residual) launch_absmax_residual32(s, s->p32, s->div32);
}

// One cycle of the flat solvers: `iterations` sweeps; MIXED adds the
// double-float update p += e, r = d - lap p.
static void flat_cycle(Solver* s, int iterations, bool residual) {
  if (s->mixed) {
    correction_solve(s, iterations);
    launch_refine_update(s, s->ph, s->pl, s->e32, s->dh, s->dl, s->pbh, s->pbl, s->r32);
    std::swap(s->ph, s->pbh);
    std::swap(s->pl, s->pbl);
    return;
  }
  poisson_f32(s, iterations, true);
  if (residual) launch_absmax_residual32(s, s->p32, s->div32);
}

// Records the tolerance loop into a conditional WHILE node of the step graph
// being captured on s->stream: k_cond (init) sets the condition from the
// initial residual, the body is one cycle followed by k_cond (step) -- for
// the fused MIXED multigrid cycle, the residual kernel's finishing thread
// does k_cond's step itself (one launch less per cycle).
static int capture_tolerance_loop(Solver* s) {
  cudaStreamCaptureStatus cst;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CU(s, cudaStreamGetCaptureInfo(s->stream, &cst, nullptr, &cg, &deps, nullptr, &nd));
  cudaGraphConditionalHandle h;
  CU(s, cudaGraphConditionalHandleCreate(&h, cg, 0, 0));
  launch_cond_init(s, h, true);
  CU(s, cudaStreamGetCaptureInfo(s->stream, &cst, nullptr, &cg, &deps, nullptr, &nd));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CU(s, cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CU(s, cudaStreamUpdateCaptureDependencies(s->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  CU(s, cudaStreamBeginCaptureToGraph(s->body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  cudaStream_t main = s->stream;
  s->stream = s->body_stream;
  int64_t l0 = s->launches;
  if (s->prm.pressure_solver == FS_PRESSURE_MULTIGRID && s->mixed && s->fused) {
    // the fused MIXED cycle; its residual kernel also does k_cond's step
    s->lev[0].x = s->e32;
    s->lev[0].x2 = s->e32b;
    mg_vcycle_fused(s, false, s->ph, s->pl);
    if (!launch_refine_init(s, s->dh, s->dl, s->ph, s->pl, s->r32, false, &h)) launch_cond_step(s, h, true);
  } else {
    mg_cycle(s, true);
    launch_cond_step(s, h, true);
  }
  s->graph_launches_body = s->launches - l0;
  s->stream = main;
  cudaGraph_t tmp = nullptr;
  CU(s, cudaStreamEndCapture(s->body_stream, &tmp));
  return check_launch(s);
}

// Pressure solve from the divergence already in div32 / (dh, dl).
//  pressure_tol == 0: multigrid runs pressure_iterations cycles (V-cycles);
//    Jacobi / red-black run pressure_iterations sweeps (MIXED: then one update).
//  pressure_tol > 0: cycles (one V-cycle, or pressure_iterations sweeps) until
//    max|div u| <= tol or max_cycles.  In a captured step the loop is a
//    conditional node evaluated on the device; otherwise the host reads the
//    residual after every cycle.
// started: launch_div_start has already set the zero-pressure residual, the
// zeroed pressure and max|r| (MIXED, no guess, no warm start).
static int pressure_solve(Solver* s, bool capture, bool defer = false, bool started = false) {
  const fs_params& P = s->prm;
  const int iters = P.pressure_iterations;
  const bool tol = P.pressure_tol > 0;
  const bool mg = P.pressure_solver == FS_PRESSURE_MULTIGRID;
  s->stats = fs_step_stats{0, 1, -1.0, -1.0};
  s->stats_on_device = false;
  if (s->guess) {
    // learned initial pressure; the cycles below correct it to the tolerance
    int rc = guess_enqueue(s, s->guess, s->guess_factor);
    if (rc) return rc;
    if (s->mixed) launch_refine_init(s, s->dh, s->dl, s->ph, s->pl, s->r32, false);
    else if (tol) launch_absmax_residual32(s, s->p32, s->div32);
  } else if (started) {
    // nothing left to start
  } else if (s->mixed) {
    launch_refine_init(s, s->dh, s->dl, s->ph, s->pl, s->r32, !P.warm_start);
    if (!P.warm_start) {
      launch_fill(s, s->ph, 0.f, s->n);
      launch_fill(s, s->pl, 0.f, s->n);
    }
  } else {
    if (!P.warm_start) launch_fill(s, s->p32, 0.f, s->n);
    if (tol) launch_absmax_residual32(s, s->p32, s->div32);
  }
  if (!tol) {
    if (mg) {
      for (int k = 0; k < iters; k++) {
        s->mg_cycle_index = k;
        mg_cycle(s, false);
      }
      s->mg_cycle_index = -1;
    } else if (s->mixed) {
      flat_cycle(s, iters, false);
    } else {
      poisson_f32(s, iters, P.warm_start != 0);
    }
    s->stats.cycles = mg ? iters : (s->mixed ? 1 : iters);
    return check_launch(s);
  }
  if (capture) {
    s->stats_on_device = true;
    if (defer) {
      // a batch runs the loop for a whole size class (batch_build): only the
      // statistics of the initial residual are set here
      launch_cond_init(s, 0, false);
      return check_launch(s);
    }
    return capture_tolerance_loop(s);
  }
  double m;
  int rc = read_red(s, &m);
  if (rc) return rc;
  s->stats.residual_initial = m;
  const double lim = P.pressure_tol_relative ? P.pressure_tol * m : P.pressure_tol;
  int c = 0;
  while (!(m <= lim) && c < P.max_cycles && std::isfinite(m)) {
    s->mg_cycle_index = c;
    if (mg) mg_cycle(s, true);
    else flat_cycle(s, iters, true);
    s->mg_cycle_index = -1;
    if ((rc = read_red(s, &m))) return rc;
    c++;
  }
  s->stats.cycles = c;
  s->stats.residual_max = m;
  s->stats.converged = m <= lim;
  if (!std::isfinite(m)) return fail(s, FS_ERR_NONFINITE, "non-finite Poisson residual");
  if (!s->stats.converged) return fail(s, FS_ERR_NOT_CONVERGED, "pressure tolerance not met within max_cycles");
  return check_launch(s);
}

// divergence of (wu, wv) -> solve -> state velocity = w - grad p
static int project_finish(Solver* s, const float* wu, const float* wv) {
  if (s->mixed) launch_subgrad_df(s, wu, nullptr, wv, nullptr, s->ph, s->pl, s->u, s->ulo, s->v, s->vlo);
  else launch_subtract_gradient_f32(s, wu, wv, s->p32, s->u, s->v);
  return check_launch(s);
}

// defer: stop after the start of the pressure solve (see pressure_solve)
static int project_from(Solver* s, const float* wu, const float* wv, bool capture, bool defer = false) {
  const bool start = s->mixed && !s->guess && !s->prm.warm_start;
  if (start) launch_div_start(s, wu, wv);
  else if (s->mixed) launch_div_df(s, wu, nullptr, wv, nullptr, s->dh, s->dl);
  else launch_divergence<float, float>(s, wu, wv, s->div32);
  int rc = pressure_solve(s, capture, defer, start);
  if (defer) return rc;
  int rc2 = project_finish(s, wu, wv);
  return rc ? rc : rc2;
}

// advection of the state into (wu, wv)
static void advect_into(Solver* s, float dt, float* ou, float* ov) {
  // the MIXED state is advected from its f32 hi planes
  if (s->prm.advection == FS_ADVECT_MACCORMACK) launch_advect_mc<float>(s, s->u, s->v, s->fu, s->fv, ou, ov, dt);
  else launch_advect_sl<float>(s, s->u, s->v, ou, ov, dt);
}

// A step split around its tolerance loop (batched size classes): the velocity
// the gradient subtraction reads.
struct StepSplit {
  const float* wu = nullptr;
  const float* wv = nullptr;
};

// step(dt), solver.js:518-591, enqueued on s->stream (eagerly or under capture).
// With split, it stops where the tolerance loop would start; the rest is
// enqueue_step_back.
static int enqueue_step(Solver* s, double dt, bool capture, StepSplit* split = nullptr) {
  float fdt = (float)dt;
  advect_into(s, fdt, s->wu, s->wv);
  float *cu = s->wu, *cv = s->wv;
  if (s->prm.nu > 0) {
    launch_diffuse(s, cu, cv, s->tu, s->tv, fdt);
    cu = s->tu; cv = s->tv;
  }
  if (s->band) launch_band(s, cu, cv, fdt);
  if (s->n_modes > 0) launch_forcing(s, cu, cv, fdt);
  if (s->channel_on) launch_channel(s, cu, cv);
  if (!s->disks.empty()) launch_solids(s, cu, cv, fdt, false);
  int rc = project_from(s, cu, cv, capture, split != nullptr);
  if (split) {
    split->wu = cu;
    split->wv = cv;
    return rc;
  }
  // dye through the now divergence-free field (solver.js:516, 577-586)
  if (s->dye) launch_advect_dye(s, fdt);
  launch_step_finish(s, dt);
  return rc;
}

static int enqueue_step_back(Solver* s, double dt, const StepSplit& split) {
  int rc = project_finish(s, split.wu, split.wv);
  if (s->dye) launch_advect_dye(s, (float)dt);
  launch_step_finish(s, dt);
  return rc;
}

static void drop_graph(Solver* s) {
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  s->graph_exec = nullptr;
  s->graph_ok = false;
  s->batch_dirty = true;
}

// Capture one step into a CUDA graph (the fused multigrid configurations):
// every kernel argument is fixed for a given dt, the time the forcing needs
// and the loop statistics live on the device.
static int build_step_graph(Solver* s, double dt) {
  drop_graph(s);
  // each failed capture leaves its partial graph behind (below): after a few
  // the handle stops capturing, so that a caller retrying in a loop cannot
  // make the leak grow without bound
  if (s->failed_captures >= kMaxFailedCaptures)
    return fail(s, FS_ERR_CUDA, "step capture failed " + std::to_string(s->failed_captures) +
                                    " times on this handle; it no longer captures (recreate the solver)");
  int64_t l0 = s->launches;
  CU(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(s, dt, true);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != FS_OK) {
    // a failed capture (a launch refused inside the tolerance loop's body)
    // leaves its partial graph alone: destroying a graph whose conditional
    // body was being captured when the capture failed is not relied on
    cudaGetLastError();
    s->failed_captures++;
    return rc;
  }
  if (e != cudaSuccess) return fail(s, FS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&s->graph_exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(s, FS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  int64_t captured = s->launches - l0;
  s->graph_launches_fixed = captured - (s->prm.pressure_tol > 0 ? s->graph_launches_body : 0);
  if (s->prm.pressure_tol <= 0) s->graph_launches_body = 0;
  s->launches = l0;  // launches are counted when the graph runs
  s->graph_dt = dt;
  s->graph_ok = true;
  return FS_OK;
}

static int step(Solver* s, double dt) {
  if (s->fused && !s->profiling) {
    if (!s->graph_ok || s->graph_dt != dt) {
      int rc = build_step_graph(s, dt);
      if (rc) return rc;
    }
    CU(s, cudaGraphLaunch(s->graph_exec, s->stream));
    s->graph_replays++;
    s->stats_on_device = s->prm.pressure_tol > 0;
    if (!s->stats_on_device) s->stats = fs_step_stats{s->prm.pressure_iterations, 1, -1.0, -1.0};
    s->t += dt;
    s->steps++;
    return FS_OK;
  }
  int rc = enqueue_step(s, dt, false);
  s->t += dt;
  s->steps++;
  if (s->prm.pressure_tol > 0 && !s->stats_on_device) {
    // the eager tolerance loop ran on the host: keep the record here
    s->host_rec_steps++;
    if (!s->stats.converged) s->host_rec_failed++;
    const double m = std::isfinite(s->stats.residual_max) ? s->stats.residual_max : INFINITY;
    if (!(m <= s->host_rec_worst)) s->host_rec_worst = m;
  }
  return rc;
}

// state <-> working f32 copies for the stage-by-stage entry point
static void state_to_w(Solver* s) {
  if (s->mixed) {
    launch_df_to_f(s, s->u, s->ulo, s->wu, s->n);
    launch_df_to_f(s, s->v, s->vlo, s->wv, s->n);
  } else {
    cudaMemcpyAsync(s->wu, s->u, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->wv, s->v, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
  }
}
static void w_to_state(Solver* s, const float* a, const float* b) {
  cudaMemcpyAsync(s->u, a, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
  cudaMemcpyAsync(s->v, b, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (s->mixed) {
    cudaMemsetAsync(s->ulo, 0, s->n * 4, s->stream);
    cudaMemsetAsync(s->vlo, 0, s->n * 4, s->stream);
  }
}

static int run_stage(Solver* s, int stage, double dt) {
  float fdt = (float)dt;
  switch (stage) {
    case FS_STAGE_ADVECT:
      advect_into(s, fdt, s->tu, s->tv);
      w_to_state(s, s->tu, s->tv);
      break;
    case FS_STAGE_DIFFUSE:
      state_to_w(s);
      launch_diffuse(s, s->wu, s->wv, s->tu, s->tv, fdt);
      w_to_state(s, s->tu, s->tv);
      break;
    case FS_STAGE_FORCING:
      if (s->n_modes == 0 && !s->band) break;
      state_to_w(s);
      if (s->band) launch_band(s, s->wu, s->wv, fdt);
      if (s->n_modes > 0) launch_forcing(s, s->wu, s->wv, fdt);
      w_to_state(s, s->wu, s->wv);
      break;
    case FS_STAGE_SOLID:
      if (s->disks.empty() && !s->channel_on) break;
      state_to_w(s);
      if (s->channel_on) launch_channel(s, s->wu, s->wv);
      if (!s->disks.empty()) launch_solids(s, s->wu, s->wv, fdt, s->imp != nullptr);
      w_to_state(s, s->wu, s->wv);
      break;
    case FS_STAGE_DIVERGENCE:
      if (s->mixed) launch_div_df(s, s->u, s->ulo, s->v, s->vlo, s->dh, s->dl);
      else launch_divergence<float, float>(s, s->u, s->v, s->div32);
      break;
    case FS_STAGE_PRESSURE: {
      int rc = pressure_solve(s, false);
      if (rc) return rc;
      break;
    }
    case FS_STAGE_SUBTRACT_GRADIENT:
      if (s->mixed) {
        // keep the full df state: copy it aside, then u = w - grad p
        cudaMemcpyAsync(s->wu, s->u, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->wv, s->v, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->tu, s->ulo, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->tv, s->vlo, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        launch_subgrad_df(s, s->wu, s->tu, s->wv, s->tv, s->ph, s->pl, s->u, s->ulo, s->v, s->vlo);
      } else {
        state_to_w(s);
        launch_subtract_gradient_f32(s, s->wu, s->wv, s->p32, s->u, s->v);
      }
      break;
    case FS_STAGE_PROJECT: {
      if (s->mixed) {
        cudaMemcpyAsync(s->wu, s->u, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->wv, s->v, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->tu, s->ulo, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->tv, s->vlo, s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
        launch_div_df(s, s->wu, s->tu, s->wv, s->tv, s->dh, s->dl);
        int rc = pressure_solve(s, false);
        launch_subgrad_df(s, s->wu, s->tu, s->wv, s->tv, s->ph, s->pl, s->u, s->ulo, s->v, s->vlo);
        if (rc) return rc;
      } else {
        state_to_w(s);
        int rc = project_from(s, s->wu, s->wv, false);
        if (rc) return rc;
      }
      break;
    }
    default:
      return fail(s, FS_ERR_INVALID_ARGUMENT, "unknown stage");
  }
  return check_launch(s);
}

}  // namespace fs

using namespace fs;

// =================================================================== C ABI
extern "C" {

FS_API void fs_params_default(fs_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->nx = 256; p->ny = 256;
  p->lx = 2 * M_PI; p->ly = 2 * M_PI;
  p->nu = 0.0;
  p->confinement = 0.0;
  p->advection = FS_ADVECT_MACCORMACK;
  p->solid_mask_width = 1.5;
  p->pressure_solver = FS_PRESSURE_JACOBI;
  p->pressure_iterations = 40;
  p->precision = FS_PRECISION_F32;
  p->pressure_tol = 0.0;
  p->max_cycles = 50;
  p->mg_pre_smooth = 2;
  p->mg_post_smooth = 2;
  p->mg_coarse_sweeps = 40;
  p->mg_min_size = 8;
  p->warm_start = 0;
  p->device = 0;
  p->kernel_variant = 0;
  p->dye_fade = 0.0;
  p->relax = 1.0;
  p->pressure_tol_relative = 0;
  p->mg_first_pre = -1;
  p->mg_first_post = -1;
}

FS_API int fs_create(const fs_params* params, fs_solver** out) {
  if (!out) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!params) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "params is NULL");
  fs_solver* h = new (std::nothrow) fs_solver();
  if (!h) return fail(nullptr, FS_ERR_OUT_OF_MEMORY, "host allocation failed");
  int rc = create(params, &h->s);
  if (rc != FS_OK) {
    if (!h->s.err.empty()) g_create_error = h->s.err;
    free_all(&h->s);
    delete h;
    return rc;
  }
  *out = h;
  return FS_OK;
}

FS_API void fs_destroy(fs_solver* h) {
  if (!h) return;
  cudaSetDevice(h->s.device);
  cudaStreamSynchronize(h->s.stream);
  for (auto& p : h->s.pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  free_all(&h->s);
  delete h;
}

FS_API const char* fs_last_error(const fs_solver* h) {
  if (!h) return g_create_error.c_str();
  return h->s.err.c_str();
}

FS_API const char* fs_status_string(int st) {
  switch (st) {
    case FS_OK: return "ok";
    case FS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FS_ERR_CUDA: return "CUDA error";
    case FS_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FS_ERR_NOT_CONVERGED: return "pressure tolerance not met";
    case FS_ERR_NONFINITE: return "non-finite residual";
    case FS_ERR_UNSUPPORTED: return "unsupported";
    case FS_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

FS_API int fs_get_params(const fs_solver* h, fs_params* out) {
  if (!h || !out) return FS_ERR_INVALID_ARGUMENT;
  *out = h->s.prm;
  return FS_OK;
}

#define SOLVER(h)                                                          \
  if (!h) return fail(nullptr, FS_ERR_INVALID_ARGUMENT, "solver is NULL"); \
  Solver* s = &h->s;                                                       \
  if (cudaSetDevice(s->device) != cudaSuccess) return fail(s, FS_ERR_CUDA, "cudaSetDevice failed")

// persistent device staging buffer for dtype conversion on upload / read-back
static int staging(Solver* s, void** out) {
  if (!s->stage) CU(s, cudaMalloc(&s->stage, (size_t)s->n * 8));
  *out = s->stage;
  return FS_OK;
}

// host array -> device field; lo == nullptr means an f32 field, otherwise a
// double-float pair (hi, lo)
static int upload_to(Solver* s, const void* src, int dtype, float* hi, float* lo) {
  if (dtype != FS_DTYPE_F32 && dtype != FS_DTYPE_F64) return fail(s, FS_ERR_INVALID_ARGUMENT, "unknown dtype");
  const size_t n = (size_t)s->n;
  if (dtype == FS_DTYPE_F32) {
    CU(s, cudaMemcpyAsync(hi, src, n * 4, cudaMemcpyHostToDevice, s->stream));
    if (lo) CU(s, cudaMemsetAsync(lo, 0, n * 4, s->stream));
  } else {
    void* st;
    int rc = staging(s, &st);
    if (rc) return rc;
    CU(s, cudaMemcpyAsync(st, src, n * 8, cudaMemcpyHostToDevice, s->stream));
    if (lo) launch_d_to_df(s, (const double*)st, hi, lo, s->n);
    else launch_convert(s, st, 1, hi, 0, s->n);
  }
  return check_launch(s);
}

// device field -> host array (synchronises unless sync is false; later work on
// the stream may reuse the staging buffer, the stream orders it after the copy)
static int download_from(Solver* s, const float* hi, const float* lo, void* dst, int dtype, bool sync = true) {
  if (dtype != FS_DTYPE_F32 && dtype != FS_DTYPE_F64) return fail(s, FS_ERR_INVALID_ARGUMENT, "unknown dtype");
  const size_t n = (size_t)s->n;
  if (dtype == FS_DTYPE_F32 && !lo) {
    CU(s, cudaMemcpyAsync(dst, hi, n * 4, cudaMemcpyDeviceToHost, s->stream));
  } else {
    void* st;
    int rc = staging(s, &st);
    if (rc) return rc;
    if (dtype == FS_DTYPE_F32) {
      launch_df_to_f(s, hi, lo, (float*)st, s->n);
      CU(s, cudaMemcpyAsync(dst, st, n * 4, cudaMemcpyDeviceToHost, s->stream));
    } else {
      launch_df_to_d(s, hi, lo, (double*)st, s->n);
      CU(s, cudaMemcpyAsync(dst, st, n * 8, cudaMemcpyDeviceToHost, s->stream));
    }
  }
  if (sync) CU(s, cudaStreamSynchronize(s->stream));
  return check_launch(s);
}

// Uploads return once the caller's arrays have been read, as the reference's
// writeTexture copies them at the call (src/gpu/solver.js:300-315): a copy from
// page-locked memory is asynchronous, so the stream is synchronised.
FS_API int fs_upload_velocity(fs_solver* h, const void* u, const void* v, int dtype) {
  SOLVER(h);
  if (!u || !v) return fail(s, FS_ERR_INVALID_ARGUMENT, "u or v is NULL");
  int rc = upload_to(s, u, dtype, s->u, s->ulo);
  if (rc) return rc;
  if ((rc = upload_to(s, v, dtype, s->v, s->vlo))) return rc;
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

// The double-float velocity is always a normalised pair -- written by the
// error-free sums of the gradient subtraction (hi = RN(hi + lo) by
// construction) or by an upload (hi = RN(x), lo the exact remainder, or lo =
// 0) -- so its f32 value RN(hi + lo) is hi itself: an f32 read-back copies the
// hi planes, with no conversion kernel.
FS_API int fs_read_velocity(fs_solver* h, void* u, void* v, int dtype) {
  SOLVER(h);
  if (!u || !v) return fail(s, FS_ERR_INVALID_ARGUMENT, "u or v is NULL");
  const bool hi_only = dtype == FS_DTYPE_F32;
  int rc = download_from(s, s->u, hi_only ? nullptr : s->ulo, u, dtype, false);  // one synchronisation for both
  if (rc) return rc;
  return download_from(s, s->v, hi_only ? nullptr : s->vlo, v, dtype);
}

FS_API int fs_read_field(fs_solver* h, int field, void* out, int dtype) {
  SOLVER(h);
  if (!out) return fail(s, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  switch (field) {
    case FS_FIELD_U: return download_from(s, s->u, s->ulo, out, dtype);
    case FS_FIELD_V: return download_from(s, s->v, s->vlo, out, dtype);
    case FS_FIELD_PRESSURE:
      return s->mixed ? download_from(s, s->ph, s->pl, out, dtype) : download_from(s, s->p32, nullptr, out, dtype);
    case FS_FIELD_DIVERGENCE:
      return s->mixed ? download_from(s, s->dh, s->dl, out, dtype) : download_from(s, s->div32, nullptr, out, dtype);
    case FS_FIELD_IMPULSE_X:
    case FS_FIELD_IMPULSE_Y:
    case FS_FIELD_IMPULSE_TORQUE:
      if (!s->imp) return fail(s, FS_ERR_INVALID_ARGUMENT, "no solid attached");
      return download_from(s, s->imp + (int64_t)(field - FS_FIELD_IMPULSE_X) * s->n, nullptr, out, dtype);
    default:
      return fail(s, FS_ERR_INVALID_ARGUMENT, "unknown field");
  }
}

FS_API int fs_upload_field(fs_solver* h, int field, const void* data, int dtype) {
  SOLVER(h);
  if (!data) return fail(s, FS_ERR_INVALID_ARGUMENT, "data is NULL");
  if (field != FS_FIELD_PRESSURE) return fail(s, FS_ERR_INVALID_ARGUMENT, "only the pressure can be uploaded");
  int rc = s->mixed ? upload_to(s, data, dtype, s->ph, s->pl) : upload_to(s, data, dtype, s->p32, nullptr);
  if (rc) return rc;
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

FS_API int fs_set_forcing(fs_solver* h, const fs_mode* modes, int count, double amplitude, double drag,
                          double phase_drift) {
  SOLVER(h);
  if (count < 0 || (count > 0 && !modes)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad mode list");
  if (count > 4096) return fail(s, FS_ERR_INVALID_ARGUMENT, "at most 4096 forcing modes");
  CU(s, cudaStreamSynchronize(s->stream));
  drop_graph(s);  // the captured step has or lacks a forcing kernel
  if (s->modes) { cudaFree(s->modes); s->modes = nullptr; }
  s->n_modes = 0;
  if (count == 0) return FS_OK;
  std::vector<float> hm(3 * (size_t)count);
  for (int k = 0; k < count; k++) {
    hm[3 * k] = (float)modes[k].kx; hm[3 * k + 1] = (float)modes[k].ky; hm[3 * k + 2] = (float)modes[k].phase;
  }
  CU(s, cudaMalloc((void**)&s->modes, hm.size() * sizeof(float)));
  CU(s, cudaMemcpy(s->modes, hm.data(), hm.size() * sizeof(float), cudaMemcpyHostToDevice));
  s->n_modes = count;
  s->amp = amplitude; s->drag = drag; s->drift = phase_drift;
  return FS_OK;
}

FS_API int fs_set_band_forcing(fs_solver* h, const fs_band* band) {
  SOLVER(h);
  if (band) {
    if (band->kind != FS_BAND_REFERENCE && band->kind != FS_BAND_GAUSSIAN)
      return fail(s, FS_ERR_INVALID_ARGUMENT, "unknown band forcing kind");
    if (!(band->kf > 0) || !(band->width >= 0) || !(band->kf + band->width <= 256) ||
        !std::isfinite(band->amplitude) || !(band->drag >= 0) || !std::isfinite(band->drag))
      return fail(s, FS_ERR_INVALID_ARGUMENT, "band forcing needs kf > 0, width >= 0, kf + width <= 256, "
                                              "a finite amplitude and drag >= 0");
  }
  CU(s, cudaStreamSynchronize(s->stream));
  drop_graph(s);  // the captured step has or lacks the band kernels
  int rc = band_set(s, band);
  if (rc) return rc;
  // the draws start again from step 0
  CU(s, cudaMemsetAsync(&s->dev->band_step, 0, sizeof(unsigned long long), s->stream));
  return FS_OK;
}

FS_API int fs_set_channel(fs_solver* h, const fs_channel* c) {
  SOLVER(h);
  if (c) {
    const double v[6] = {c->wall_y, c->wall_half, c->fringe_x, c->fringe_half, c->fringe_ramp, c->inflow_u};
    for (double x : v)
      if (!std::isfinite(x)) return fail(s, FS_ERR_INVALID_ARGUMENT, "channel parameters must be finite");
    if (!(c->wall_half > 0) || !(c->wall_half < 0.5 * s->prm.ly) || !(c->fringe_half > 0) ||
        !(c->fringe_half < 0.5 * s->prm.lx) || !(c->fringe_ramp > 0))
      return fail(s, FS_ERR_INVALID_ARGUMENT,
                  "channel needs 0 < wall_half < ly/2, 0 < fringe_half < lx/2 and fringe_ramp > 0");
  }
  CU(s, cudaStreamSynchronize(s->stream));
  drop_graph(s);  // the captured step has or lacks the channel kernel
  return channel_set(s, c);
}

FS_API int fs_set_solids(fs_solver* h, const fs_disk* disks, int count) {
  SOLVER(h);
  if (count < 0 || (count > 0 && !disks)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad disk list");
  if (count > 64) return fail(s, FS_ERR_INVALID_ARGUMENT, "at most 64 disks");
  for (int k = 0; k < count; k++)
    if (!(disks[k].r > 0) || !std::isfinite(disks[k].x) || !std::isfinite(disks[k].y))
      return fail(s, FS_ERR_INVALID_ARGUMENT, "disk needs a finite centre and r > 0");
  CU(s, cudaStreamSynchronize(s->stream));
  drop_graph(s);  // the captured step has or lacks a solids kernel
  s->disks.assign(disks, disks + count);
  if (count > 0) {
    if (!s->imp) {
      CU(s, cudaMalloc((void**)&s->imp, 3 * (size_t)s->n * sizeof(float)));
      CU(s, cudaMemsetAsync(s->imp, 0, 3 * (size_t)s->n * sizeof(float), s->stream));
    }
    if (s->imp_cap < count) {
      if (s->d_impulse) cudaFree(s->d_impulse);
      CU(s, cudaMalloc((void**)&s->d_impulse, 3 * 64 * sizeof(double)));
      CU(s, cudaMemsetAsync(s->d_impulse, 0, 3 * 64 * sizeof(double), s->stream));
      s->imp_cap = 64;
    }
    if (upload_disks(s) != 0) return fail(s, FS_ERR_CUDA, "uploading the disk parameters failed");
  }
  return FS_OK;
}

FS_API int fs_solid_impulse(fs_solver* h, double* out, int count) {
  SOLVER(h);
  if (!out || count < (int)s->disks.size()) return fail(s, FS_ERR_INVALID_ARGUMENT, "out too small");
  if (s->disks.empty()) return FS_OK;
  CU(s, cudaMemcpyAsync(out, s->d_impulse, 3 * s->disks.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

FS_API int fs_set_guess(fs_solver* h, fs_guess* g, int32_t factor) {
  SOLVER(h);
  if (g && factor != 1 && factor != 2) return fail(s, FS_ERR_INVALID_ARGUMENT, "fs_set_guess: factor must be 1 or 2");
  if (g && !guess_supported(s, factor))
    return fail(s, FS_ERR_UNSUPPORTED, "the pressure guess needs nx and ny multiples of 8 * factor");
  if (g && s->prm.pressure_solver != FS_PRESSURE_MULTIGRID)
    return fail(s, FS_ERR_UNSUPPORTED, "the pressure guess seeds multigrid cycles only");
  CU(s, cudaStreamSynchronize(s->stream));
  if (g) {
    int rc = guess_prepare(s, g, factor);
    if (rc) return rc;
  }
  drop_graph(s);  // the captured step gains or loses the guess
  s->guess = g;
  s->guess_factor = g ? factor : 2;
  return FS_OK;
}

FS_API int fs_dump_pair(fs_solver* h, int32_t factor, float* div, float* mask, float* p) {
  SOLVER(h);
  if (!div || !mask || !p) return fail(s, FS_ERR_INVALID_ARGUMENT, "fs_dump_pair: NULL output");
  if (factor < 1 || s->g.nx % factor || s->g.ny % factor)
    return fail(s, FS_ERR_INVALID_ARGUMENT, "fs_dump_pair: factor must divide nx and ny");
  return dump_pair(s, factor, div, mask, p);
}

FS_API int fs_dump_pair_device(fs_solver* h, int32_t factor, float* d_div, float* d_mask, float* d_p) {
  SOLVER(h);
  if (!d_div || !d_mask || !d_p) return fail(s, FS_ERR_INVALID_ARGUMENT, "fs_dump_pair_device: NULL output");
  if (factor < 1 || s->g.nx % factor || s->g.ny % factor)
    return fail(s, FS_ERR_INVALID_ARGUMENT, "fs_dump_pair_device: factor must divide nx and ny");
  return dump_pair_device(s, factor, d_div, d_mask, d_p);
}

FS_API int fs_upload_dye(fs_solver* h, const float* rgba) {
  SOLVER(h);
  if (!rgba) return fail(s, FS_ERR_INVALID_ARGUMENT, "rgba is NULL");
  if (!s->dye) {
    CU(s, cudaStreamSynchronize(s->stream));
    CU(s, cudaMalloc(&s->dye, (size_t)s->n * 16));
    CU(s, cudaMalloc(&s->dye2, (size_t)s->n * 16));
    drop_graph(s);  // the captured step gains the dye pass
  }
  CU(s, cudaMemcpyAsync(s->dye, rgba, (size_t)s->n * 16, cudaMemcpyHostToDevice, s->stream));
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

FS_API int fs_read_dye(fs_solver* h, float* rgba) {
  SOLVER(h);
  if (!rgba) return fail(s, FS_ERR_INVALID_ARGUMENT, "rgba is NULL");
  if (!s->dye) return fail(s, FS_ERR_INVALID_ARGUMENT, "no dye uploaded");
  CU(s, cudaMemcpyAsync(rgba, s->dye, (size_t)s->n * 16, cudaMemcpyDeviceToHost, s->stream));
  CU(s, cudaStreamSynchronize(s->stream));
  return FS_OK;
}

FS_API int fs_render(fs_solver* h, int32_t mode, double exposure, float* rgba) {
  SOLVER(h);
  if (!rgba) return fail(s, FS_ERR_INVALID_ARGUMENT, "rgba is NULL");
  if (!std::isfinite(exposure)) return fail(s, FS_ERR_INVALID_ARGUMENT, "exposure must be finite");
  return render(s, mode, (float)exposure, rgba);
}

FS_API int fs_diagnose(fs_solver* h, fs_diagnostics* out) {
  SOLVER(h);
  if (!out) return fail(s, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  return diagnostics(s, out, false);
}

FS_API int fs_energy_spectrum(fs_solver* h, double* E, int32_t* counts, int32_t cap, int32_t* kmax,
                              double* parseval) {
  SOLVER(h);
  if (!E || !counts) return fail(s, FS_ERR_INVALID_ARGUMENT, "E and counts must be given");
  int km = 0;
  int rc = energy_spectrum(s, E, counts, cap, &km, parseval);
  if (kmax) *kmax = km;
  return rc;
}

FS_API int fs_step(fs_solver* h, double dt) {
  SOLVER(h);
  if (!std::isfinite(dt)) return fail(s, FS_ERR_INVALID_ARGUMENT, "dt must be finite");
  return step(s, dt);
}

FS_API int fs_advance(fs_solver* h, double dt, int nsteps) {
  SOLVER(h);
  if (!std::isfinite(dt) || nsteps < 0) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad dt or nsteps");
  for (int k = 0; k < nsteps; k++) {
    int rc = step(s, dt);
    if (rc) return rc;
  }
  return FS_OK;
}

FS_API int fs_sync(fs_solver* h) {
  SOLVER(h);
  return sync(s);
}

FS_API int fs_last_stats(fs_solver* h, fs_step_stats* out) {
  SOLVER(h);
  if (!out) return fail(s, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  int rc = sync(s);
  if (rc) return rc;
  DevState d;
  CU(s, cudaMemcpy(&d, s->dev, sizeof(DevState), cudaMemcpyDeviceToHost));
  if (d.async_err) return fail(s, FS_ERR_CUDA, "an asynchronous tile copy did not complete (bounded wait)");
  if (s->stats_on_device) {
    // the last projection's loop ran inside a captured step
    s->stats = fs_step_stats{d.cycles, d.converged, d.res_max, d.res_initial};
    *out = s->stats;
    if (d.nonfinite) return fail(s, FS_ERR_NONFINITE, "non-finite Poisson residual in the last step");
    if (!d.converged) return fail(s, FS_ERR_NOT_CONVERGED, "pressure tolerance not met within max_cycles in the last step");
    return FS_OK;
  }
  *out = s->stats;
  return FS_OK;
}

FS_API int fs_get_time(const fs_solver* h, double* t, int64_t* steps) {
  if (!h) return FS_ERR_INVALID_ARGUMENT;
  if (t) *t = h->s.t;
  if (steps) *steps = h->s.steps;
  return FS_OK;
}

FS_API int fs_run_stage(fs_solver* h, int stage, double dt) {
  SOLVER(h);
  return run_stage(s, stage, dt);
}

FS_API int fs_max_divergence(fs_solver* h, double* out) {
  SOLVER(h);
  if (!out) return fail(s, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  if (s->mixed) {
    launch_div_df(s, s->u, s->ulo, s->v, s->vlo, s->dh, s->dl);
    launch_absmax<float>(s, s->dh, s->n, s->red_out);
  } else {
    launch_divergence<float, float>(s, s->u, s->v, s->div32);
    launch_absmax<float>(s, s->div32, s->n, s->red_out);
  }
  int rc = check_launch(s);
  if (rc) return rc;
  return read_red(s, out);
}

FS_API int fs_poisson_residual_after(fs_solver* h, int iterations, double dt, double* out) {
  SOLVER(h);
  (void)dt;
  if (!out || iterations < 0) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  if (s->mixed) return fail(s, FS_ERR_UNSUPPORTED, "poisson_residual_after measures the F32 solver");
  launch_divergence<float, float>(s, s->u, s->v, s->div32);
  launch_fill(s, s->p32, 0.f, s->n);
  poisson_f32(s, iterations, false);
  launch_poisson_norms(s, s->p32, s->div32, s->g.dx * s->g.dx, s->g.dxd * s->g.dxd);
  int rc = check_launch(s);
  if (rc) return rc;
  double num, den;
  if ((rc = read_red(s, &num, &den))) return rc;
  double sd = sqrt(den);
  *out = sqrt(num) / (sd == 0 ? 1 : sd);
  return FS_OK;
}

FS_API int fs_time_steps(fs_solver* h, double dt, int nsteps, double* elapsed_ms) {
  SOLVER(h);
  if (!elapsed_ms || nsteps < 0) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  cudaEvent_t a, b;
  CU(s, cudaEventCreate(&a));
  CU(s, cudaEventCreate(&b));
  CU(s, cudaStreamSynchronize(s->stream));
  CU(s, cudaEventRecord(a, s->stream));
  int rc = FS_OK;
  for (int k = 0; k < nsteps && rc == FS_OK; k++) rc = step(s, dt);
  CU(s, cudaEventRecord(b, s->stream));
  CU(s, cudaEventSynchronize(b));
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *elapsed_ms = ms;
  return rc;
}

FS_API int fs_set_mg_sweeps(fs_solver* h, int32_t pre, int32_t post) {
  SOLVER(h);
  if (s->prm.pressure_solver != FS_PRESSURE_MULTIGRID) return fail(s, FS_ERR_UNSUPPORTED, "multigrid only");
  if (pre < 1 || pre > 8 || post < 1 || post > 8) return fail(s, FS_ERR_INVALID_ARGUMENT, "sweeps in 1..8");
  CU(s, cudaStreamSynchronize(s->stream));
  const fs_params old = s->prm;
  s->prm.mg_pre_smooth = pre;
  s->prm.mg_post_smooth = post;
  if (s->fused && !mg_fused_supported(s)) {  // the fused tile kernels take 1..3
    s->prm = old;
    return fail(s, FS_ERR_UNSUPPORTED, "the fused multigrid kernels take 1 to 3 sweeps");
  }
  drop_graph(s);
  return FS_OK;
}

// Autotuner of the multigrid sweep counts: every (pre, post) pair the fused
// kernels take is timed over `nsteps` steps from the same state (the state,
// dye, time and pressure are saved on the device and restored between
// candidates and at the end), and the fastest is kept.  Ties in time go to
// fewer sweeps.  Returns the choice and its ms per step.
// ------------------------------------------------------------- autotuning
// A solver's step-changing state saved on the device, so that every candidate
// setting is timed from the same state, and the timing of one candidate.
struct TuneState {
  Solver* s = nullptr;
  std::vector<std::pair<void*, size_t>> planes;  // device plane, bytes per cell
  char* save = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  double t0 = 0;
  int64_t steps0 = 0, l0 = 0, r0 = 0;
};

static cudaError_t tune_copy(TuneState& T, bool to_save) {
  Solver* s = T.s;
  size_t off = 0;
  for (auto& p : T.planes) {
    const size_t b = p.second * (size_t)s->n;
    cudaError_t e = to_save ? cudaMemcpyAsync(T.save + off, p.first, b, cudaMemcpyDeviceToDevice, s->stream)
                            : cudaMemcpyAsync(p.first, T.save + off, b, cudaMemcpyDeviceToDevice, s->stream);
    if (e != cudaSuccess) return e;
    off += b;
  }
  return to_save ? cudaMemcpyAsync(T.save + off, s->dev, sizeof(DevState), cudaMemcpyDeviceToDevice, s->stream)
                 : cudaMemcpyAsync(s->dev, T.save + off, sizeof(DevState), cudaMemcpyDeviceToDevice, s->stream);
}

static cudaError_t tune_begin(Solver* s, TuneState& T) {
  T.s = s;
  T.planes = {{s->u, 4}, {s->v, 4}};
  if (s->mixed) {
    T.planes.push_back({s->ulo, 4});
    T.planes.push_back({s->vlo, 4});
    T.planes.push_back({s->ph, 4});
    T.planes.push_back({s->pl, 4});
  } else {
    T.planes.push_back({s->p32, 4});
  }
  if (s->dye) T.planes.push_back({s->dye, 16});
  size_t total = sizeof(DevState);
  for (auto& p : T.planes) total += p.second * (size_t)s->n;
  T.t0 = s->t;
  T.steps0 = s->steps;
  T.l0 = s->launches;
  T.r0 = s->graph_replays;
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess) e = cudaMalloc(&T.save, total);
  if (e == cudaSuccess) e = cudaEventCreate(&T.a);
  if (e == cudaSuccess) e = cudaEventCreate(&T.b);
  if (e == cudaSuccess) e = tune_copy(T, true);
  return e;
}

// restores the saved state and the host-side counters
static void tune_end(TuneState& T) {
  Solver* s = T.s;
  if (T.save) tune_copy(T, false);
  cudaStreamSynchronize(s->stream);
  if (T.a) cudaEventDestroy(T.a);
  if (T.b) cudaEventDestroy(T.b);
  if (T.save) cudaFree(T.save);
  T.save = nullptr;
  s->t = T.t0;
  s->steps = T.steps0;
  s->launches = T.l0;
  s->graph_replays = T.r0;
}

// ms per step of nsteps steps of the current settings from the saved state
// (the graph is captured before the timing); 1e30 if the tolerance was missed
static int tune_time(TuneState& T, double dt, int nsteps, double* per, cudaError_t* err) {
  Solver* s = T.s;
  drop_graph(s);
  int rc = step(s, dt);
  cudaError_t e = cudaSuccess;
  if (rc == FS_OK) e = tune_copy(T, false);
  if (rc == FS_OK && e == cudaSuccess) e = cudaEventRecord(T.a, s->stream);
  for (int k = 0; k < nsteps && rc == FS_OK && e == cudaSuccess; k++) rc = step(s, dt);
  if (e == cudaSuccess) e = cudaEventRecord(T.b, s->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(T.b);
  float ms = 0;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, T.a, T.b);
  if (rc == FS_OK && e == cudaSuccess && s->stats_on_device) {
    DevState d;
    e = cudaMemcpy(&d, s->dev, sizeof d, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && (!d.converged || d.nonfinite)) ms = 1e30f;  // must still meet the tolerance
  }
  if (e == cudaSuccess) e = tune_copy(T, false);
  *per = ms / nsteps;
  *err = e;
  return rc;
}

FS_API int fs_autotune(fs_solver* h, double dt, int32_t nsteps, int32_t* pre_out, int32_t* post_out,
                       double* ms_out) {
  SOLVER(h);
  if (s->prm.pressure_solver != FS_PRESSURE_MULTIGRID || !s->fused)
    return fail(s, FS_ERR_UNSUPPORTED, "fs_autotune tunes the fused multigrid step");
  if (nsteps < 1 || !std::isfinite(dt)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad dt or nsteps");
  TuneState T;
  cudaError_t e = tune_begin(s, T);
  const fs_params orig = s->prm;
  int best_pre = orig.mg_pre_smooth, best_post = orig.mg_post_smooth, rc = FS_OK;
  double best = 1e300;
  for (int pre = 1; pre <= 3 && e == cudaSuccess && rc == FS_OK; pre++) {
    for (int post = 1; post <= 3 && e == cudaSuccess && rc == FS_OK; post++) {
      s->prm.mg_pre_smooth = pre;
      s->prm.mg_post_smooth = post;
      double per = 0;
      rc = tune_time(T, dt, nsteps, &per, &e);
      if (rc == FS_OK && e == cudaSuccess && per < best * 0.999) {
        best = per;
        best_pre = pre;
        best_post = post;
      }
    }
  }
  tune_end(T);
  s->prm = orig;
  s->prm.mg_pre_smooth = best_pre;
  s->prm.mg_post_smooth = best_post;
  drop_graph(s);
  if (rc != FS_OK) return rc;
  if (e != cudaSuccess) return fail(s, FS_ERR_CUDA, std::string("fs_autotune: ") + cudaGetErrorString(e));
  if (pre_out) *pre_out = best_pre;
  if (post_out) *post_out = best_post;
  if (ms_out) *ms_out = best;
  return FS_OK;
}

// the levels that run the tile kernels (the fused cycle's levels above its bottom solve)
static int tile_levels(const Solver* s) { return s->fused ? bottom_first_level(s) : 0; }

FS_API int fs_set_mg_tiles(fs_solver* h, const int32_t* tiles, int32_t count) {
  SOLVER(h);
  if (count < 0 || count > 16 || (count > 0 && !tiles)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad tiles");
  for (int l = 0; l < count; l++)
    if (tiles[l] != 0 && tiles[l] != 16 && tiles[l] != 32 && tiles[l] != 64)
      return fail(s, FS_ERR_INVALID_ARGUMENT, "a tile side is 16, 32, 64 or 0 (the built-in rule)");
  for (int l = 0; l < 16; l++) s->tile_level[l] = l < count ? tiles[l] : 0;
  drop_graph(s);
  return FS_OK;
}

FS_API int fs_get_mg_tiles(fs_solver* h, int32_t* tiles, int32_t cap, int32_t* count) {
  SOLVER(h);
  if (!count || cap < 0 || (cap > 0 && !tiles)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  const int nl = tile_levels(s);
  *count = nl;
  for (int l = 0; l < nl && l < cap; l++) tiles[l] = mg_tile(s, l);
  return FS_OK;
}

// Greedy per level: each tile level tries 64, 32 and 16 with the others fixed
// (the tiles give the same values whatever their size, so only time counts).
FS_API int fs_autotune_tiles(fs_solver* h, double dt, int32_t nsteps, int32_t* tiles_out, int32_t cap,
                             int32_t* count, double* ms_out) {
  SOLVER(h);
  if (!s->fused) return fail(s, FS_ERR_UNSUPPORTED, "fs_autotune_tiles tunes the fused multigrid step");
  if (nsteps < 1 || !std::isfinite(dt) || !count || cap < 0 || (cap > 0 && !tiles_out))
    return fail(s, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  const int nl = tile_levels(s);
  TuneState T;
  cudaError_t e = tune_begin(s, T);
  int rc = FS_OK;
  double best = 1e300;
  // the current choice first; another side must be 0.5% faster to replace it
  for (int l = 0; l < nl && l < 16 && e == cudaSuccess && rc == FS_OK; l++) {
    const int start = mg_tile(s, l);
    int pick = start;
    double here = 1e300;
    for (int t : {start, 64, 32, 16}) {
      if (t == start && here < 1e300) continue;
      s->tile_level[l] = t;
      double per = 0;
      rc = tune_time(T, dt, nsteps, &per, &e);
      if (rc != FS_OK || e != cudaSuccess) break;
      if (t == start ? true : per < here * 0.995) {
        here = per;
        pick = t;
      }
    }
    s->tile_level[l] = pick;
    best = here;
  }
  tune_end(T);
  drop_graph(s);
  if (rc != FS_OK) return rc;
  if (e != cudaSuccess) return fail(s, FS_ERR_CUDA, std::string("fs_autotune_tiles: ") + cudaGetErrorString(e));
  *count = nl;
  for (int l = 0; l < nl && l < cap; l++) tiles_out[l] = s->tile_level[l];
  if (ms_out) *ms_out = best;
  return FS_OK;
}

FS_API int fs_profile_step(fs_solver* h, double dt, int nsteps, fs_kernel_time* out, int cap, int* count) {
  SOLVER(h);
  if (nsteps < 0 || cap < 0 || (cap > 0 && !out)) return fail(s, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  CU(s, cudaStreamSynchronize(s->stream));
  s->kstats.clear();
  s->profiling = true;
  int rc = FS_OK;
  for (int k = 0; k < nsteps && rc == FS_OK; k++) rc = step(s, dt);
  s->profiling = false;
  prof_collect(s);
  int m = std::min<int>(cap, (int)s->kstats.size());
  for (int k = 0; k < m; k++) {
    memset(&out[k], 0, sizeof(fs_kernel_time));
    strncpy(out[k].name, s->kstats[k].name.c_str(), sizeof(out[k].name) - 1);
    out[k].launches = s->kstats[k].launches;
    out[k].total_ms = s->kstats[k].ms;
    out[k].bytes = s->kstats[k].bytes;
  }
  if (count) *count = (int)s->kstats.size();
  return rc;
}

FS_API int fs_total_cycles(fs_solver* h, int64_t* cycles) {
  SOLVER(h);
  if (!cycles) return fail(s, FS_ERR_INVALID_ARGUMENT, "cycles is NULL");
  CU(s, cudaStreamSynchronize(s->stream));
  DevState d;
  CU(s, cudaMemcpy(&d, s->dev, sizeof d, cudaMemcpyDeviceToHost));
  *cycles = d.total_cycles;
  return FS_OK;
}

FS_API int fs_convergence_record(fs_solver* h, int64_t* steps, int64_t* failed, double* worst) {
  SOLVER(h);
  CU(s, cudaStreamSynchronize(s->stream));
  DevState d;
  CU(s, cudaMemcpy(&d, s->dev, sizeof d, cudaMemcpyDeviceToHost));
  if (steps) *steps = d.rec_steps + s->host_rec_steps;
  if (failed) *failed = d.rec_failed + s->host_rec_failed;
  if (worst) *worst = std::max(d.rec_worst, s->host_rec_worst);
  return FS_OK;
}

FS_API int64_t fs_launch_count(const fs_solver* h) {
  if (!h) return 0;
  const Solver* s = &h->s;
  int64_t n = s->launches + s->graph_replays * s->graph_launches_fixed;
  if (s->graph_launches_body > 0) {
    // the loop bodies run a device-decided number of times: count them from
    // the device tally (this synchronises)
    DevState d;
    cudaStreamSynchronize(s->stream);
    if (cudaMemcpy(&d, s->dev, sizeof(DevState), cudaMemcpyDeviceToHost) == cudaSuccess)
      n += d.total_cycles * s->graph_launches_body;
  }
  return n;
}

FS_API void* fs_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

FS_API void fs_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"

// ====================================================================== batch
// Many independent simulations, uneven sizes, advanced together: one CUDA
// graph whose branches are the members' captured steps (each with its own
// conditional tolerance loop), launched once per batch step.  Members are
// ordinary solvers whose eager work (uploads, read-backs, statistics) runs on
// the batch's stream, so it is ordered with the batch launches without
// per-step events; while the batch graph is captured each member's step runs
// on its own stream, forked from and joined back to the batch stream, so the
// branches are independent and their kernels overlap on the GPU.
// Members that run the MIXED tolerance loop of the fused multigrid step with the
// same grid and multigrid settings form a size class: their refinement cycles
// run as batched launches inside one conditional loop per class (up to
// kClassMax members per class; a larger group is split).
// chains of size classes that run side by side within one batch step.  With
// the classes' steps batched, running them side by side pays: the 256-member
// benchmark batch (six classes) took 4.47 / 3.97 / 3.76 / 3.56 / 3.29 ms per
// step with 1 / 2 / 3 / 4 / 6 chains.
constexpr int kBatchLanes = 8;

struct BatchClass {
  std::vector<int> idx;  // member indices
  int body_launches = 0;  // launches of one loop iteration
};

struct fs_batch {
  std::vector<fs_solver*> members;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t body_stream = nullptr;        // captures the class loop bodies
  std::vector<cudaStream_t> class_streams;   // one per class, grown as needed
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<cudaEvent_t> class_done;
  std::vector<BatchClass> classes;
  long long* d_iters = nullptr;  // device: loop iterations per class since the last capture
  int iters_cap = 0;
  int64_t launches_done = 0;     // class launches of graphs replaced since
  int64_t fixed_per_replay = 0;  // launches of one replay outside the class loops
  cudaGraphExec_t exec = nullptr;
  std::vector<double> dts;
  int64_t replays = 0;
  int64_t replays_at_build = 0;
  std::string err;
};

namespace fs {

static int bfail(fs_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  g_create_error = m;
  return code;
}

static void batch_free(fs_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (fs_solver* h : b->members) {
    if (!h) continue;
    for (auto& p : h->s.pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    free_all(&h->s);
    delete h;
  }
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  for (cudaEvent_t e : b->class_done) cudaEventDestroy(e);
  for (cudaStream_t c : b->class_streams) cudaStreamDestroy(c);
  if (b->body_stream) cudaStreamDestroy(b->body_stream);
  if (b->d_iters) cudaFree(b->d_iters);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// a class whose members' whole steps can run as batched launches: nothing
// but advection, diffusion and the projection from zero pressure
static bool class_plain(const fs_batch* b, const BatchClass& c) {
  const Solver* r = &b->members[c.idx[0]]->s;
  for (int i : c.idx) {
    const Solver* s = &b->members[i]->s;
    if (s->n_modes > 0 || s->band || s->channel_on || !s->disks.empty() || s->dye || s->guess || s->prm.warm_start ||
        s->prm.advection != r->prm.advection || (s->prm.nu > 0) != (r->prm.nu > 0))
      return false;
  }
  return true;
}

// a member that can run its loop in a size class, and the settings a class shares
static bool class_eligible(const Solver* s) {
  return s->mixed && s->fused && s->prm.pressure_tol > 0 && !s->guess && s->g.nx == s->g.ny &&
         s->prm.mg_first_pre < 0 && s->prm.mg_first_post < 0;
}
static bool same_class(const Solver* a, const Solver* b) {
  const fs_params &p = a->prm, &q = b->prm;
  return a->g.nx == b->g.nx && a->g.ny == b->g.ny && p.mg_pre_smooth == q.mg_pre_smooth &&
         p.mg_post_smooth == q.mg_post_smooth && p.mg_coarse_sweeps == q.mg_coarse_sweeps &&
         p.mg_min_size == q.mg_min_size && p.relax == q.relax && p.max_cycles == q.max_cycles &&
         a->lev.size() == b->lev.size() && std::equal(a->tile_level, a->tile_level + 16, b->tile_level);
}

// the class's conditional loop on cs (already part of the batch capture):
// k_cond_class sets the condition from the members' initial statistics, the
// body is one batched refinement cycle plus k_cond_class's bookkeeping
static int capture_class_loop(fs_batch* b, BatchClass& c, cudaStream_t cs, long long* iters, int init_mode) {
  std::vector<Solver*> ms;
  for (int i : c.idx) ms.push_back(&b->members[i]->s);
  const int count = (int)ms.size();
  cudaStreamCaptureStatus cst;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
  cudaGraphConditionalHandle h = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 0, 0);
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch loop: ") + cudaGetErrorString(e));
  launch_cond_class(ms.data(), count, cs, h, init_mode, iters);
  e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp);
  if (e == cudaSuccess)
    e = cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(b->body_stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch loop: ") + cudaGetErrorString(e));
  c.body_launches = mg_vcycle_class(ms.data(), count, b->body_stream);
  launch_refine_class(ms.data(), count, b->body_stream);
  launch_cond_class(ms.data(), count, b->body_stream, h, 0, iters);
  c.body_launches += 2;
  cudaGraph_t tmp = nullptr;
  cudaError_t e2 = cudaGetLastError();
  e = cudaStreamEndCapture(b->body_stream, &tmp);
  if (e2 != cudaSuccess) e = e2;
  return e == cudaSuccess ? FS_OK : bfail(b, FS_ERR_CUDA, std::string("batch loop: ") + cudaGetErrorString(e));
}

static int batch_build(fs_batch* b, const double* dt) {
  const int n = (int)b->members.size();
  // the class launches of the graph being replaced, before its counters reset
  if (b->exec && b->d_iters && !b->classes.empty()) {
    std::vector<long long> it(b->classes.size());
    if (cudaStreamSynchronize(b->stream) == cudaSuccess &&
        cudaMemcpy(it.data(), b->d_iters, it.size() * sizeof(long long), cudaMemcpyDeviceToHost) == cudaSuccess)
      for (size_t c = 0; c < it.size(); c++) b->launches_done += it[c] * b->classes[c].body_launches;
  }
  b->launches_done += (b->replays - b->replays_at_build) * b->fixed_per_replay;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;

  // size classes
  b->classes.clear();
  std::vector<int> cls(n, -1);
  for (int i = 0; i < n; i++) {
    const Solver* s = &b->members[i]->s;
    if (!class_eligible(s)) continue;
    for (size_t c = 0; c < b->classes.size() && cls[i] < 0; c++) {
      const Solver* r = &b->members[b->classes[c].idx[0]]->s;
      if (same_class(s, r) && (int)b->classes[c].idx.size() < kClassMax) cls[i] = (int)c;
    }
    if (cls[i] < 0) {
      cls[i] = (int)b->classes.size();
      b->classes.emplace_back();
    }
    b->classes[cls[i]].idx.push_back(i);
  }
  const int nc = (int)b->classes.size();
  // streams, events and counters for the classes (outside the capture)
  while ((int)b->class_streams.size() < nc) {
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
      return bfail(b, FS_ERR_CUDA, "batch: stream creation failed");
    b->class_streams.push_back(cs);
    b->class_done.push_back(ev);
  }
  if (nc > b->iters_cap) {
    if (b->d_iters) cudaFree(b->d_iters);
    b->d_iters = nullptr;
    if (cudaMalloc(&b->d_iters, (size_t)nc * sizeof(long long)) != cudaSuccess)
      return bfail(b, FS_ERR_OUT_OF_MEMORY, "batch: counter allocation failed");
    b->iters_cap = nc;
  }
  if (nc > 0 && cudaMemset(b->d_iters, 0, (size_t)nc * sizeof(long long)) != cudaSuccess)
    return bfail(b, FS_ERR_CUDA, "batch: counter reset failed");

  std::vector<int64_t> l0(n);
  std::vector<StepSplit> split(n);
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  e = cudaEventRecord(b->fork, b->stream);
  int rc = e == cudaSuccess ? FS_OK : FS_ERR_CUDA;
  auto member_err = [&](int i) {
    Solver* s = &b->members[i]->s;
    if (!s->err.empty()) b->err = "member " + std::to_string(i) + ": " + s->err;
  };
  // members outside a class: their whole captured step as one branch, joined
  // at the end
  for (int i = 0; i < n && rc == FS_OK; i++) {
    if (cls[i] >= 0) continue;
    Solver* s = &b->members[i]->s;
    std::swap(s->stream, s->own_stream);  // this member's branch
    if (cudaStreamWaitEvent(s->stream, b->fork, 0) != cudaSuccess) rc = FS_ERR_CUDA;
    l0[i] = s->launches;
    if (rc == FS_OK) rc = enqueue_step(s, dt[i], true);
    if (rc == FS_OK && cudaEventRecord(b->joins[i], s->stream) != cudaSuccess) rc = FS_ERR_CUDA;
    std::swap(s->stream, s->own_stream);
    if (rc != FS_OK) member_err(i);
  }
  // The classes run in kBatchLanes chains, each class after the previous one
  // of its lane; a class goes to the lane with the fewest cells so far,
  // largest classes first.  Each class: the members' steps up to their
  // loops, the class loop on the class stream, then the members' remaining
  // steps; the class's completion is recorded on its stream.
  std::vector<int> order(nc), lane_prev(kBatchLanes, -1), prev_class(nc, -1);
  std::vector<double> lane_cells(kBatchLanes, 0.0), class_cells(nc, 0.0);
  for (int c = 0; c < nc; c++) {
    order[c] = c;
    for (int i : b->classes[c].idx) class_cells[c] += (double)b->members[i]->s.n;
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return class_cells[x] > class_cells[y]; });
  for (int c : order) {
    int lane = 0;
    for (int k = 1; k < kBatchLanes; k++)
      if (lane_cells[k] < lane_cells[lane]) lane = k;
    prev_class[c] = lane_prev[lane];
    lane_prev[lane] = c;
    lane_cells[lane] += class_cells[c];
  }
  int64_t class_fixed = 0;  // launches per replay of the batched plain classes
  for (int oc = 0; oc < nc && rc == FS_OK; oc++) {
    const int c = order[oc];
    cudaStream_t cs = b->class_streams[c];
    cudaEvent_t after = prev_class[c] < 0 ? b->fork : b->class_done[prev_class[c]];
    if (cudaStreamWaitEvent(cs, after, 0) != cudaSuccess) rc = FS_ERR_CUDA;
    if (rc == FS_OK && class_plain(b, b->classes[c])) {
      // the whole class step as batched launches on the class stream
      std::vector<Solver*> ms;
      std::vector<const float*> wu, wv;
      std::vector<double> cdt;
      for (int i : b->classes[c].idx) {
        Solver* s = &b->members[i]->s;
        ms.push_back(s);
        const bool diff = s->prm.nu > 0;
        wu.push_back(diff ? s->tu : s->wu);
        wv.push_back(diff ? s->tv : s->wv);
        cdt.push_back(dt[i]);
        s->stats = fs_step_stats{0, 1, -1.0, -1.0};
        s->stats_on_device = true;
        l0[i] = s->launches;
      }
      const int count = (int)ms.size();
      launch_front_advect_class(ms.data(), count, cdt.data(), cs);
      const int nproj = launch_front_project_class(ms.data(), count, wu.data(), wv.data(), cdt.data(), cs);
      rc = capture_class_loop(b, b->classes[c], cs, b->d_iters + c, 2);
      if (rc == FS_OK) launch_back_class(ms.data(), count, wu.data(), wv.data(), cdt.data(), cs);
      class_fixed += (ms[0]->prm.advection == FS_ADVECT_MACCORMACK ? 2 : 1) + (ms[0]->prm.nu > 0 ? 1 : 0) + nproj + 2;
      if (rc == FS_OK && cudaGetLastError() != cudaSuccess) rc = bfail(b, FS_ERR_CUDA, "batch: class launch failed");
      if (rc == FS_OK && cudaEventRecord(b->class_done[c], cs) != cudaSuccess) rc = FS_ERR_CUDA;
      if (rc == FS_OK && cudaStreamWaitEvent(b->stream, b->class_done[c], 0) != cudaSuccess) rc = FS_ERR_CUDA;
      continue;
    }
    for (int i : b->classes[c].idx) {
      if (rc != FS_OK) break;
      Solver* s = &b->members[i]->s;
      std::swap(s->stream, s->own_stream);
      if (cudaStreamWaitEvent(s->stream, after, 0) != cudaSuccess) rc = FS_ERR_CUDA;
      l0[i] = s->launches;
      if (rc == FS_OK) rc = enqueue_step(s, dt[i], true, &split[i]);
      if (rc == FS_OK && cudaEventRecord(b->joins[i], s->stream) != cudaSuccess) rc = FS_ERR_CUDA;
      if (rc == FS_OK && cudaStreamWaitEvent(cs, b->joins[i], 0) != cudaSuccess) rc = FS_ERR_CUDA;
      std::swap(s->stream, s->own_stream);
      if (rc != FS_OK) member_err(i);
    }
    if (rc == FS_OK) rc = capture_class_loop(b, b->classes[c], cs, b->d_iters + c, 1);
    if (rc == FS_OK && cudaEventRecord(b->class_done[c], cs) != cudaSuccess) rc = FS_ERR_CUDA;
    for (int i : b->classes[c].idx) {
      if (rc != FS_OK) break;
      Solver* s = &b->members[i]->s;
      std::swap(s->stream, s->own_stream);
      if (cudaStreamWaitEvent(s->stream, b->class_done[c], 0) != cudaSuccess) rc = FS_ERR_CUDA;
      if (rc == FS_OK) rc = enqueue_step_back(s, dt[i], split[i]);
      if (rc == FS_OK && cudaEventRecord(b->joins[i], s->stream) != cudaSuccess) rc = FS_ERR_CUDA;
      if (rc == FS_OK && cudaStreamWaitEvent(cs, b->joins[i], 0) != cudaSuccess) rc = FS_ERR_CUDA;
      std::swap(s->stream, s->own_stream);
      if (rc != FS_OK) member_err(i);
    }
    if (rc == FS_OK && cudaEventRecord(b->class_done[c], cs) != cudaSuccess) rc = FS_ERR_CUDA;
    if (rc == FS_OK && cudaStreamWaitEvent(b->stream, b->class_done[c], 0) != cudaSuccess) rc = FS_ERR_CUDA;
  }
  for (int i = 0; i < n && rc == FS_OK; i++)
    if (cls[i] < 0 && cudaStreamWaitEvent(b->stream, b->joins[i], 0) != cudaSuccess) rc = FS_ERR_CUDA;
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(b->stream, &g);
  if (rc != FS_OK) {
    if (g) cudaGraphDestroy(g);
    return bfail(b, rc, b->err.empty() ? std::string("batch capture failed") : b->err);
  }
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
  b->fixed_per_replay = nc + class_fixed;  // the class loops' initial condition kernels, batched steps
  for (int i = 0; i < n; i++) {
    Solver* s = &b->members[i]->s;
    int64_t captured = s->launches - l0[i];
    const bool own_loop = cls[i] < 0 && s->prm.pressure_tol > 0;
    s->batch_launches_fixed = captured - (own_loop ? s->graph_launches_body : 0);
    s->in_class = cls[i] >= 0;
    s->launches = l0[i];  // counted when the graph runs
    s->batch_dirty = false;
  }
  b->replays_at_build = b->replays;
  b->dts.assign(dt, dt + n);
  return FS_OK;
}

}  // namespace fs

FS_API int fs_batch_create(const fs_params* params, int32_t count, fs_batch** out) {
  if (!out) return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!params || count < 1 || count > 65536) return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "bad params or count");
  for (int i = 1; i < count; i++)
    if (params[i].device != params[0].device)
      return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "every member must be on the same device");
  fs_batch* b = new (std::nothrow) fs_batch();
  if (!b) return bfail(nullptr, FS_ERR_OUT_OF_MEMORY, "host allocation failed");
  b->device = params[0].device;
  b->members.assign(count, nullptr);
  for (int i = 0; i < count; i++) {
    fs_solver* h = nullptr;
    int rc = fs_create(&params[i], &h);
    if (rc != FS_OK) {
      std::string m = "member " + std::to_string(i) + ": " + g_create_error;
      batch_free(b);
      return bfail(nullptr, rc, m);
    }
    b->members[i] = h;
    if (!h->s.fused) {
      batch_free(b);
      return bfail(nullptr, FS_ERR_UNSUPPORTED,
                   "member " + std::to_string(i) + ": batches need the fused multigrid step (pressure_solver = "
                   "MULTIGRID, kernel_variant = 0, nx == ny)");
    }
  }
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->body_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->joins.assign(count, nullptr);
  for (int i = 0; i < count && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    batch_free(b);
    return bfail(nullptr, FS_ERR_CUDA, std::string("fs_batch_create: ") + cudaGetErrorString(e));
  }
  for (fs_solver* h : b->members) {
    Solver* s = &h->s;
    cudaStreamSynchronize(s->stream);  // creation work is done before the stream changes hands
    s->own_stream = s->stream;
    s->stream = b->stream;
  }
  *out = b;
  return FS_OK;
}

FS_API void fs_batch_destroy(fs_batch* b) { batch_free(b); }

FS_API int32_t fs_batch_size(const fs_batch* b) { return b ? (int32_t)b->members.size() : 0; }

FS_API fs_solver* fs_batch_member(fs_batch* b, int32_t index) {
  if (!b || index < 0 || index >= (int32_t)b->members.size()) return nullptr;
  return b->members[index];
}

FS_API const char* fs_batch_last_error(const fs_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

FS_API int fs_batch_step(fs_batch* b, const double* dt) {
  if (!b) return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (!dt) return bfail(b, FS_ERR_INVALID_ARGUMENT, "dt is NULL");
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, FS_ERR_CUDA, "cudaSetDevice failed");
  const int n = (int)b->members.size();
  bool rebuild = !b->exec;
  for (int i = 0; i < n; i++) {
    if (!std::isfinite(dt[i])) return bfail(b, FS_ERR_INVALID_ARGUMENT, "dt must be finite");
    if (b->members[i]->s.batch_dirty || b->dts.empty() || b->dts[i] != dt[i]) rebuild = true;
  }
  if (rebuild) {
    int rc = batch_build(b, dt);
    if (rc) return rc;
  }
  cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  b->replays++;
  for (int i = 0; i < n; i++) {
    Solver* s = &b->members[i]->s;
    s->stats_on_device = s->prm.pressure_tol > 0;
    if (!s->stats_on_device) s->stats = fs_step_stats{s->prm.pressure_iterations, 1, -1.0, -1.0};
    s->t += dt[i];
    s->steps++;
  }
  return FS_OK;
}

FS_API int fs_batch_sync(fs_batch* b) {
  if (!b) return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "batch is NULL");
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? FS_OK : bfail(b, FS_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e));
}

FS_API int fs_batch_time_steps(fs_batch* b, const double* dt, int32_t nsteps, double* elapsed_ms) {
  if (!b || !elapsed_ms || nsteps < 0) return bfail(b, FS_ERR_INVALID_ARGUMENT, "bad arguments");
  cudaSetDevice(b->device);
  cudaEvent_t a, z;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&z) != cudaSuccess)
    return bfail(b, FS_ERR_CUDA, "cudaEventCreate failed");
  int rc = fs_batch_sync(b);
  if (rc == FS_OK && nsteps > 0 && (!b->exec || b->dts.size() != b->members.size() ||
                                    !std::equal(b->dts.begin(), b->dts.end(), dt))) {
    // capture before the timed region
    rc = batch_build(b, dt);
  }
  cudaEventRecord(a, b->stream);
  for (int k = 0; k < nsteps && rc == FS_OK; k++) rc = fs_batch_step(b, dt);
  cudaEventRecord(z, b->stream);
  cudaEventSynchronize(z);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, z);
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  *elapsed_ms = ms;
  return rc;
}

// kernels launched by the batch's graph replays so far (synchronises)
FS_API int64_t fs_batch_launch_count(fs_batch* b) {
  if (!b) return 0;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  int64_t n = b->launches_done + (b->replays - b->replays_at_build) * b->fixed_per_replay;
  for (fs_solver* h : b->members) {
    const Solver* s = &h->s;
    n += b->replays * s->batch_launches_fixed;
    if (!s->in_class && s->graph_launches_body > 0) {
      DevState d;
      if (cudaMemcpy(&d, s->dev, sizeof(DevState), cudaMemcpyDeviceToHost) == cudaSuccess)
        n += d.total_cycles * s->graph_launches_body;
    }
  }
  if (!b->classes.empty() && b->d_iters) {
    std::vector<long long> it(b->classes.size());
    if (cudaMemcpy(it.data(), b->d_iters, it.size() * sizeof(long long), cudaMemcpyDeviceToHost) == cudaSuccess)
      for (size_t c = 0; c < it.size(); c++) n += it[c] * b->classes[c].body_launches;
  }
  return n;
}

// Settings of the batch's size classes picked by timing whole batch steps, each
// candidate from the same saved state of every member (restored afterwards):
// what & 1, the (pre, post) sweep pair of each class; what & 2, greedy per
// class and tile level, the tile side (64, 32, 16; the tiles give the same
// values whatever their size).
static int batch_autotune(fs_batch* b, const double* dt, int32_t nsteps, int what, double* ms_out) {
  if (!b) return bfail(nullptr, FS_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (!dt || nsteps < 1) return bfail(b, FS_ERR_INVALID_ARGUMENT, "bad dt or nsteps");
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, FS_ERR_CUDA, "cudaSetDevice failed");
  const int n = (int)b->members.size();
  for (int i = 0; i < n; i++)
    if (!std::isfinite(dt[i])) return bfail(b, FS_ERR_INVALID_ARGUMENT, "dt must be finite");
  const int64_t launches_before = fs_batch_launch_count(b);
  const int64_t replays_before = b->replays;
  int rc = batch_build(b, dt);
  if (rc) return rc;
  std::vector<TuneState> T(n);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; i++) e = tune_begin(&b->members[i]->s, T[i]);
  cudaEvent_t ea = nullptr, eb = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&ea);
  if (e == cudaSuccess) e = cudaEventCreate(&eb);
  // ms per batch step of the current settings from the saved state; 1e30 if a member missed its tolerance
  auto time_batch = [&](double* per) -> int {
    for (int i = 0; i < n && e == cudaSuccess; i++) e = tune_copy(T[i], false);
    for (int i = 0; i < n; i++) b->members[i]->s.batch_dirty = true;
    int r = e == cudaSuccess ? fs_batch_step(b, dt) : FS_ERR_CUDA;  // captures outside the timing
    for (int i = 0; i < n && e == cudaSuccess && r == FS_OK; i++) e = tune_copy(T[i], false);
    if (r == FS_OK && e == cudaSuccess) e = cudaEventRecord(ea, b->stream);
    for (int k = 0; k < nsteps && r == FS_OK && e == cudaSuccess; k++) r = fs_batch_step(b, dt);
    if (e == cudaSuccess) e = cudaEventRecord(eb, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(eb);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, ea, eb);
    for (int i = 0; i < n && r == FS_OK && e == cudaSuccess; i++) {
      Solver* s = &b->members[i]->s;
      if (!s->stats_on_device) continue;
      DevState d;
      e = cudaMemcpy(&d, s->dev, sizeof d, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && (!d.converged || d.nonfinite)) ms = 1e30f;
    }
    *per = ms / nsteps;
    return r;
  };
  double best = 1e300;
  if (e == cudaSuccess) rc = time_batch(&best);
  const std::vector<BatchClass> classes = b->classes;
  // sweep pairs per class: a pair must be 1% faster than the current one
  for (const BatchClass& c : classes) {
    if (!(what & 1) || rc != FS_OK || e != cudaSuccess) break;
    Solver* lead = &b->members[c.idx[0]]->s;
    int bp = lead->prm.mg_pre_smooth, bq = lead->prm.mg_post_smooth;
    for (int pre = 1; pre <= 3 && rc == FS_OK && e == cudaSuccess; pre++)
      for (int post = 1; post <= 3 && rc == FS_OK && e == cudaSuccess; post++) {
        if (pre == bp && post == bq) continue;
        const int op = lead->prm.mg_pre_smooth, oq = lead->prm.mg_post_smooth;
        for (int i : c.idx) {
          b->members[i]->s.prm.mg_pre_smooth = pre;
          b->members[i]->s.prm.mg_post_smooth = post;
        }
        double per = 0;
        rc = time_batch(&per);
        if (rc == FS_OK && e == cudaSuccess && per < best * 0.99) {
          best = per;
          bp = pre;
          bq = post;
        }
        for (int i : c.idx) {
          b->members[i]->s.prm.mg_pre_smooth = op;
          b->members[i]->s.prm.mg_post_smooth = oq;
        }
      }
    for (int i : c.idx) {
      b->members[i]->s.prm.mg_pre_smooth = bp;
      b->members[i]->s.prm.mg_post_smooth = bq;
      drop_graph(&b->members[i]->s);
    }
  }
  for (const BatchClass& c : classes) {
    if (!(what & 2) || rc != FS_OK || e != cudaSuccess) break;
    Solver* lead = &b->members[c.idx[0]]->s;
    const int nl = std::min(bottom_first_level(lead), 16);
    // the class's current choice (timed as `best`) stays unless another side
    // is 1% faster: one class level moves a whole batch step only a little,
    // so smaller differences are within the timing noise
    for (int l = 0; l < nl && rc == FS_OK && e == cudaSuccess; l++) {
      const int start = lead->tile_level[l];
      int pick = start;
      for (int t : {64, 32, 16}) {
        for (int i : c.idx) b->members[i]->s.tile_level[l] = t;
        double per = 0;
        rc = time_batch(&per);
        if (rc != FS_OK || e != cudaSuccess) break;
        if (per < best * 0.99) {
          best = per;
          pick = t;
        }
      }
      // the side in use, written out (the class rule when nothing beat it)
      for (int i : c.idx) b->members[i]->s.tile_level[l] = start;
      if (pick == 0) pick = mg_tile_class(lead, l, (int)c.idx.size());
      for (int i : c.idx) b->members[i]->s.tile_level[l] = pick;
    }
  }
  for (int i = 0; i < n; i++) {
    if (T[i].s) tune_end(T[i]);
    b->members[i]->s.batch_dirty = true;
  }
  if (ea) cudaEventDestroy(ea);
  if (eb) cudaEventDestroy(eb);
  // the tuning steps are not part of the batch's history
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  (void)replays_before;
  b->replays = 0;  // launches_before counts every replay so far
  b->replays_at_build = 0;
  b->launches_done = launches_before;
  for (int i = 0; i < n; i++) b->members[i]->s.batch_launches_fixed = 0;
  b->classes.clear();
  if (rc != FS_OK) return rc;
  if (e != cudaSuccess) return bfail(b, FS_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(e));
  if (ms_out) *ms_out = best;
  return FS_OK;
}

FS_API int fs_batch_autotune_tiles(fs_batch* b, const double* dt, int32_t nsteps, double* ms_out) {
  return batch_autotune(b, dt, nsteps, 2, ms_out);
}

FS_API int fs_batch_autotune(fs_batch* b, const double* dt, int32_t nsteps, double* ms_out) {
  return batch_autotune(b, dt, nsteps, 1, ms_out);
}
