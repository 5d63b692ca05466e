// fs_internal.cuh -- shared definitions of libfluidcuda (GB300, sm_103a).
//
// Data layout in HBM: every field is a planar row-major nx*ny array, i fastest
// (the reference packs u and v into one rgba32float texel per cell,
// src/gpu/shaders.js:4-14, and uses only .x of its scalar textures; planar
// arrays move a quarter of the bytes for p, div and the multigrid levels).
#pragma once

#include <cuda.h>  // CUtensorMap (types only; the encoder is looked up at run time)
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/fluid.h"

namespace fs {

// Grid spacing as every kernel sees it.  dx/dy are the f32 values the
// reference uploads in its uniform block (src/gpu/solver.js:249-256); the
// reciprocals replace its per-sample divisions.
struct Grid {
  int nx, ny;
  float dx, dy, idx, idy;
  double dxd, dyd, idxd, idyd;
};

// One multigrid level (src/gpu/multigrid.js:177-197).  Level 0 aliases the
// solver's pressure (or correction) and right-hand side.
struct Level {
  int n;
  float dx;    // (dx * nx) / n, rounded to f32 as multigrid.js:186,220 does
  float h2;    // dx * dx
  float* x;    // solution / correction, in place
  float* x2;   // second buffer for odd n, where red-black needs ping-pong
  float* rhs;
};

// step state kept on the device so that a captured step can run without the host
struct DevState {
  double t;            // simulation time
  double res_initial;  // max|div| entering the last projection
  double res_max;      // max|div| after it
  long long total_cycles;  // cycles run by every projection since creation
  int cycles;          // cycles the last projection ran
  int converged;
  int nonfinite;
  int async_err;  // a bounded wait for an asynchronous (TMA) copy gave up
  // record over every step whose tolerance loop ran on the device (the step
  // finish adds to it; the per-projection fields above are overwritten by the
  // next projection, this is not)
  long long rec_steps;   // projections recorded
  long long rec_failed;  // of those, projections that ended without meeting pressure_tol
  double rec_worst;      // largest max|div u| any of them ended with (+inf for NaN)
  unsigned long long band_step;  // steps the band forcing has run (its random draws' counter)
};

struct KernelStat {
  std::string name;
  int launches = 0;
  double ms = 0;
  double bytes = 0;
};

struct Solver {
  fs_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  Grid g{};
  int64_t n = 0;
  bool mixed = false;
  bool odd = false;  // nx or ny odd: red-black ping-pong semantics
  bool fused = false;  // fused multigrid cycle in use

  // velocity state.  F32: u, v.  MIXED: double-float planes (u, ulo), (v, vlo).
  float* u = nullptr;
  float* v = nullptr;
  float* ulo = nullptr;
  float* vlo = nullptr;
  // working velocity of the step before projection (f32 in both modes)
  float* wu = nullptr;
  float* wv = nullptr;
  float* tu = nullptr;  // ping-pong partner of wu/wv
  float* tv = nullptr;
  float* fu = nullptr;  // MacCormack forward field
  float* fv = nullptr;
  float* mc_bounds = nullptr;  // MacCormack limiter range per face: lo_u, hi_u, lo_v, hi_v planes

  // pressure: F32 -> p32/div32 are the Poisson unknown/rhs.
  //           MIXED -> (ph, pl) and (dh, dl) hold the double-float pressure and
  //           divergence, r32/e32 the f32 residual and correction of one
  //           refinement cycle.
  float* p32 = nullptr;
  float* p32b = nullptr;  // ping-pong (Jacobi, odd red-black, fused cycle)
  float* div32 = nullptr;
  float *ph = nullptr, *pl = nullptr, *pbh = nullptr, *pbl = nullptr;
  float *dh = nullptr, *dl = nullptr;
  float* r32 = nullptr;
  float* e32 = nullptr;
  float* e32b = nullptr;
  float* scratch = nullptr;  // n floats: multigrid residual before restriction
  void* stage = nullptr;     // n doubles: host I/O conversion staging

  std::vector<Level> lev;
  int tile_level[16] = {};  // tile side of each tile level's kernels; 0 = the built-in rule
  // TMA tensor maps of the staged fields (advection, multigrid tiles), by
  // device pointer, plane and box (box_tmap, fs_advect.cu)
  struct Tmap {
    const void* p;
    int nx, ny, bw, bh;
    CUtensorMap m;
  };
  std::vector<Tmap> tmaps;

  // reductions: per-block partials and the final words
  double* red_partials = nullptr;  // 2 * red_cap doubles
  int red_cap = 0;
  double* red_out = nullptr;       // device: [0] max, [1] sum a, [2] sum b
  double* h_red = nullptr;         // pinned host copy

  // band-limited random forcing renewed every step (fs_band.cu), or null
  void* band = nullptr;
  // channel walls and inflow fringe (fs_channel.cu)
  fs_channel channel{};
  bool channel_on = false;
  // forcing (solver.js:370-385)
  float* modes = nullptr;  // kx, ky, phase triplets
  int n_modes = 0;
  double amp = 0, drag = 0, drift = 0;

  // solids
  std::vector<fs_disk> disks;
  fs_guess* guess = nullptr;    // learned initial pressure (fs_set_guess), not owned
  void* diag = nullptr;         // diagnostics buffers (fs_diag.cu), allocated on first use
  void* dye = nullptr;          // RGBA float4 per cell once uploaded (fs_upload_dye)
  void* dye2 = nullptr;         // advection target
  int guess_factor = 2;         // the network runs at 1/guess_factor of the grid
  float* imp = nullptr;         // 3 * n impulse field (x, y, torque)
  double* d_impulse = nullptr;  // 3 * disks
  int imp_cap = 0;
  void* d_disks = nullptr;      // device copy of the disk parameters (set by fs_set_solids)
  int* d_tiles = nullptr;       // 32x8 tiles any disk can reach
  unsigned long long* d_tile_masks = nullptr;  // per listed tile: the disks that can reach it
  int n_tiles = 0;

  // device-side step state: simulation time (read by the forcing kernel) and
  // the statistics of the last projection (written by the tolerance loop)
  DevState* dev = nullptr;

  // CUDA graph of one step (fused multigrid configurations), captured per dt
  cudaGraphExec_t graph_exec = nullptr;
  double graph_dt = 0;
  bool graph_ok = false;        // graph_exec matches the current forcing / solids
  int failed_captures = 0;      // step captures that failed (each leaves its partial graph)
  // the cycle being enqueued when the host knows it (eager loops, fixed cycle
  // counts: 0, 1, ...), -1 inside a captured tolerance loop, where the device's
  // cycle count tells the kernels (fs_params mg_first_pre / mg_first_post)
  int mg_cycle_index = -1;
  bool stats_on_device = false; // the last projection ran inside a graph
  cudaStream_t body_stream = nullptr;  // captures the body of the tolerance loop
  // batch membership: eager work goes to the batch's shared stream; own_stream
  // (the solver's original stream) carries its branch while the batch graph
  // is captured.  batch_dirty: the captured step no longer matches.
  cudaStream_t own_stream = nullptr;
  bool batch_dirty = true;
  int64_t batch_launches_fixed = 0;
  bool in_class = false;  // its batch runs the tolerance loop for its size class
  int64_t graph_launches_fixed = 0;    // kernels per replay outside the loop body
  int64_t graph_launches_body = 0;     // kernels per loop iteration
  int64_t graph_replays = 0;

  double t = 0;
  int64_t steps = 0;
  fs_step_stats stats{0, 1, -1.0, -1.0};
  // the same record for projections whose tolerance loop ran on the host
  int64_t host_rec_steps = 0, host_rec_failed = 0;
  double host_rec_worst = 0;
  std::string err;
  int64_t launches = 0;

  // profiling: an event pair around every launch when enabled
  bool profiling = false;
  struct Pending {
    int stat;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<KernelStat> kstats;
};

// the tolerance as the device-side loop code takes it: the absolute
// pressure_tol, or with pressure_tol_relative its negative, meaning "times
// the max residual the projection started from"
inline double dev_tol(const Solver* s) {
  return s->prm.pressure_tol_relative ? -s->prm.pressure_tol : s->prm.pressure_tol;
}

// ----------------------------------------------------------------- launching
void prof_begin(Solver* s, const char* name, double bytes, int* slot, cudaEvent_t* a);
void prof_end(Solver* s, int slot, cudaEvent_t a);

// Wrap one kernel launch: counts it and, when profiling, brackets it with
// events on the solver's stream.
#define FS_LAUNCH(S, NAME, BYTES, ...)                                   \
  do {                                                                   \
    int _slot = -1;                                                      \
    cudaEvent_t _ev = nullptr;                                           \
    if ((S)->profiling) fs::prof_begin((S), (NAME), (BYTES), &_slot, &_ev); \
    __VA_ARGS__;                                                         \
    (S)->launches++;                                                     \
    if ((S)->profiling) fs::prof_end((S), _slot, _ev);                   \
  } while (0)

inline dim3 grid2d(int nx, int ny, dim3 b) { return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y); }

// failed step captures after which a handle refuses to capture again
constexpr int kMaxFailedCaptures = 4;

// members of one batched launch (a size class of a batch; larger classes are split)
constexpr int kClassMax = 64;

// --------------------------------------------------------- kernel launchers
// fs_advect.cu
template <class TV>
void launch_advect_sl(Solver* s, const TV* u, const TV* v, float* ou, float* ov, float dt);
template <class TV>
void launch_advect_mc(Solver* s, const TV* u, const TV* v, float* fu, float* fv, float* ou,
                      float* ov, float dt);
void launch_diffuse(Solver* s, const float* u, const float* v, float* ou, float* ov, float dt);
void launch_forcing(Solver* s, float* u, float* v, float dt);
int upload_disks(Solver* s);
void launch_solids(Solver* s, float* u, float* v, float dt, bool record_impulse);
void launch_advect_dye(Solver* s, float dt);
// fs_channel.cu
int channel_set(Solver* s, const fs_channel* c);  // null: remove
void launch_channel(Solver* s, float* u, float* v);
// fs_band.cu
int band_set(Solver* s, const fs_band* band);  // null: remove
void band_free(Solver* s);
void launch_band(Solver* s, float* u, float* v, float dt);

// fs_pressure.cu
template <class TV, class TD>
void launch_divergence(Solver* s, const TV* u, const TV* v, TD* d);
void launch_subtract_gradient_f32(Solver* s, const float* wu, const float* wv, const float* p,
                                  float* ou, float* ov);
// double-float (MIXED) variants; lo planes of the input velocity may be nullptr
void launch_div_df(Solver* s, const float* uh, const float* ul, const float* vh, const float* vl, float* dh,
                   float* dl);
void launch_subgrad_df(Solver* s, const float* wuh, const float* wul, const float* wvh, const float* wvl,
                       const float* ph, const float* pl, float* uh, float* ul, float* vh, float* vl);
void launch_d_to_df(Solver* s, const double* x, float* hi, float* lo, int64_t n);
void launch_df_to_d(Solver* s, const float* hi, const float* lo, double* x, int64_t n);
void launch_df_to_f(Solver* s, const float* hi, const float* lo, float* x, int64_t n);
void launch_jacobi(Solver* s, const float* p, const float* d, float* out, float h2, int nx, int ny);
void launch_rb_half(Solver* s, const float* src, const float* d, float* dst, float h2, int colour,
                    int nx, int ny);
void launch_residual(Solver* s, const float* x, const float* rhs, float* out, float h2, int n);
void launch_restrict(Solver* s, const float* fine, float* coarse, int nc);
void launch_prolong_add(Solver* s, const float* coarse, float* fine, int nf);
void launch_fill(Solver* s, float* x, float value, int64_t n);
void launch_fill64(Solver* s, double* x, double value, int64_t n);
// mixed-precision refinement (double-float pressure and divergence)
// cond (a captured tolerance loop's handle): the residual kernel also does
// the loop's step bookkeeping and sets the condition when it can (returns
// true); otherwise the caller launches k_cond
bool launch_refine_init(Solver* s, const float* dh, const float* dl, const float* ph, const float* pl,
                        float* r32, bool zero_p, const cudaGraphConditionalHandle* cond = nullptr);
// TMA tensor map of a row-major f32 plane nx x ny (pitch nx) with a bw x bh
// box, cached per solver; false when TMA cannot copy it (nx % 4 != 0, an
// unaligned base, a box larger than the plane, no encoder in the CUDA driver)
bool box_tmap(Solver* s, const float* f, int nx, int ny, int bw, int bh, CUtensorMap* out);
// divergence + zero-pressure residual + zeroed pressure in one pass (MIXED)
void launch_div_start(Solver* s, const float* wu, const float* wv);
void launch_refine_update(Solver* s, const float* ph, const float* pl, const float* e, const float* dh,
                          const float* dl, float* poh, float* pol, float* r32);
// reductions (results land in s->red_out)
template <class T>
void launch_absmax(Solver* s, const T* x, int64_t n, double* out_word);
void launch_absmax_residual32(Solver* s, const float* p, const float* d);
// tolerance loop state on the device (fs_pressure.cu)
void launch_cond_init(Solver* s, cudaGraphConditionalHandle h, bool graph);
void launch_cond_step(Solver* s, cudaGraphConditionalHandle h, bool graph);
void launch_step_finish(Solver* s, double dt);
void launch_poisson_norms(Solver* s, const float* p, const float* d, float h2f, double h2);
void launch_convert(Solver* s, const void* src, int src_f64, void* dst, int dst_f64, int64_t n);

// multigrid drivers: one pass per reference operation (fs_pressure.cu) and
// the fused cycle (fs_multigrid.cu).  Both leave the result in lev[0].x; the
// fused cycle may swap lev[0].x with lev[0].x2.
void mg_vcycle(Solver* s);
// acc_h/acc_l != nullptr: the level-0 up kernel adds its correction to the
// double-float pressure (acc_h, acc_l) in place instead of writing lev[0].x2
void mg_vcycle_fused(Solver* s, bool first_has_x, float* acc_h = nullptr, float* acc_l = nullptr);
bool mg_fused_supported(const Solver* s);
// tile side of the kernels of level l (an override or the built-in rule)
int mg_tile(const Solver* s, int l);
// tile side of level l of a batch size class of count members led by s0
int mg_tile_class(const Solver* s0, int l, int count);
int bottom_first_level(const Solver* s);
// batched refinement cycle of one size class of a batch (fs_multigrid.cu, fs_pressure.cu)
int mg_vcycle_class(Solver* const* ms, int count, cudaStream_t st);
void launch_refine_class(Solver* const* ms, int count, cudaStream_t st);
void launch_cond_class(Solver* const* ms, int count, cudaStream_t st, cudaGraphConditionalHandle h, int init,
                       long long* iterations);
// the rest of the step of a class whose members are plain (fs_advect.cu, fs_pressure.cu)
void launch_front_advect_class(Solver* const* ms, int count, const double* dts, cudaStream_t st);
int launch_front_project_class(Solver* const* ms, int count, const float* const* wu, const float* const* wv,
                               const double* dts, cudaStream_t st);  // returns its launch count
void launch_back_class(Solver* const* ms, int count, const float* const* wu, const float* const* wv,
                       const double* dts, cudaStream_t st);

// errors (fs_api.cu): message into the handle (or the thread's last error)
int fail_status(Solver* s, int code, const std::string& msg);
void record_error(const std::string& msg);

// learned pressure guess (fs_guess.cu)
bool guess_supported(const Solver* s, int factor);
int guess_prepare(Solver* s, fs_guess* g, int factor);  // buffers for this grid (outside any capture)
int guess_enqueue(Solver* s, fs_guess* g, int factor);  // initial pressure from the divergence
int dump_pair(Solver* s, int factor, float* div, float* mask, float* p);
int dump_pair_device(Solver* s, int factor, float* div, float* mask, float* p);  // enqueued, device outputs

// diagnostics (fs_diag.cu)
void diag_free(Solver* s);
int diagnostics(Solver* s, fs_diagnostics* out, bool with_centres);
int energy_spectrum(Solver* s, double* E, int32_t* counts, int cap, int* kmax_out, double* parseval);
int render(Solver* s, int mode, float exposure, float* host_rgba);

}  // namespace fs
