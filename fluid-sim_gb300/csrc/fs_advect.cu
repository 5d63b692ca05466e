// fs_advect.cu -- advection, explicit diffusion, band forcing and immersed-disk
// direct forcing for GB300 (sm_103a).
//
// Reference: src/gpu/shaders.js ADVECT_VELOCITY (:126-146), ADVECT_FIELD_BY
// (:155-171), MACCORMACK_COMBINE (:187-231), DIFFUSE (:401-425), FORCING
// (:532-566), SOLID_COUPLE (:587-653); the f64 semantics they restate are
// src/cpu/advect.js:46-206, src/cpu/solver.js:52-69 and src/cpu/solid.js:101-233.
//
// Trace arithmetic is done in cell units relative to the destination cell:
// a position is (home cell integer, f32 offset), so the interpolation weights
// keep full f32 precision at any grid size.  The reference forms x = i*dx in
// f32 and divides by dx again, which at n = 2048 quantises the weights to
// ~2e-4 of a cell; the mathematics is otherwise identical.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>

#include <utility>
#include <vector>

#include "fs_internal.cuh"
#include "fs_tc.cuh"

namespace fs {

__device__ __forceinline__ int wrap_idx(int i, int n) {
  if ((unsigned)i < (unsigned)n) return i;
  int r = i % n;
  return r < 0 ? r + n : r;
}

template <class T>
__device__ __forceinline__ float ld(const T* __restrict__ a, int64_t k) {
  return (float)__ldg(a + k);
}

// Bilinear sample at (bi + ox, bj + oy) in the field's own index space
// (src/core/grid.js:147-164 bilerp: top = a + (b-a)fx, bot = c + (d-c)fx).
template <class T>
__device__ __forceinline__ float bilerp(const T* __restrict__ f, int nx, int ny, int bi, int bj,
                                        float ox, float oy) {
  float fo = floorf(ox), go = floorf(oy);
  float fx = ox - fo, fy = oy - go;
  int i0 = wrap_idx(bi + (int)fo, nx), j0 = wrap_idx(bj + (int)go, ny);
  int i1 = i0 + 1 == nx ? 0 : i0 + 1;
  int j1 = j0 + 1 == ny ? 0 : j0 + 1;
  int64_t r0 = (int64_t)j0 * nx, r1 = (int64_t)j1 * nx;
  float a = ld(f, r0 + i0), b = ld(f, r0 + i1), c = ld(f, r1 + i0), d = ld(f, r1 + i1);
  float top = a + (b - a) * fx;
  float bot = c + (d - c) * fx;
  return top + (bot - top) * fy;
}

// Range of the four cells a bilinear sample at (bi+ox, bj+oy) reads
// (src/cpu/advect.js:104-111).
template <class T>
__device__ __forceinline__ void bounds4(const T* __restrict__ f, int nx, int ny, int bi, int bj,
                                        float ox, float oy, float& lo, float& hi) {
  int i0 = wrap_idx(bi + (int)floorf(ox), nx), j0 = wrap_idx(bj + (int)floorf(oy), ny);
  int i1 = i0 + 1 == nx ? 0 : i0 + 1;
  int j1 = j0 + 1 == ny ? 0 : j0 + 1;
  int64_t r0 = (int64_t)j0 * nx, r1 = (int64_t)j1 * nx;
  float a = ld(f, r0 + i0), b = ld(f, r0 + i1), c = ld(f, r1 + i0), d = ld(f, r1 + i1);
  lo = fminf(fminf(a, b), fminf(c, d));
  hi = fmaxf(fmaxf(a, b), fmaxf(c, d));
}

// Sample offsets of the u and v grids relative to a home point.  u lives at
// (i, j+1/2), v at (i+1/2, j) (src/core/grid.js:99-105).  A point at home +
// (dX, dY) cells has u-grid index (hux + dX, huy + dY) etc.
struct Home {
  float ux, uy;  // u-grid offset of the home point
  float vx, vy;  // v-grid offset of the home point
};
__device__ __forceinline__ Home home_u() { return {0.f, 0.f, -0.5f, 0.5f}; }
__device__ __forceinline__ Home home_v() { return {0.5f, -0.5f, 0.f, 0.f}; }

// RK2 midpoint backward trace (src/cpu/advect.js:46-54, shaders.js:117-122),
// in cells: returns the displacement (dX, dY) of the departure point.
template <class TV>
__device__ __forceinline__ void trace(const TV* __restrict__ u, const TV* __restrict__ v, int nx,
                                      int ny, int i, int j, Home h, float cx, float cy, float& dX,
                                      float& dY) {
  float u1 = bilerp(u, nx, ny, i, j, h.ux, h.uy);
  float v1 = bilerp(v, nx, ny, i, j, h.vx, h.vy);
  float mx = -0.5f * cx * u1, my = -0.5f * cy * v1;
  float u2 = bilerp(u, nx, ny, i, j, h.ux + mx, h.uy + my);
  float v2 = bilerp(v, nx, ny, i, j, h.vx + mx, h.vy + my);
  dX = -cx * u2;
  dY = -cy * v2;
}

// ------------------------------------------------------ tiled advection
// The advection kernels are gather-bound: a MacCormack step takes about 20
// bilinear samples per cell.  A CTA stages its 32x16-cell tile of each field
// it samples, plus a halo of 4 cells, in shared memory.  When the largest
// displacement any trace of the tile can reach is at most 3 cells (checked
// once per CTA on the staged velocities, below) every sample lies in the
// staged block and is read from there unchecked; otherwise each sample is
// checked and one whose four cells leave the block falls back to the wrapped
// global read.  The arithmetic of the three ways is the same, so the results
// are too.
constexpr int kTX = 32, kTY = 16, kHalo = 4;
constexpr int kSW = kTX + 2 * kHalo, kSH = kTY + 2 * kHalo;
// largest |u| dt/dx (cells) for which every trace stays in the staged block:
// a sample at home + (h + d), |h| <= 1/2, reads cells floor(h + d) .. +1,
// inside [-kHalo, kTX - 1 + kHalo] while |d| < kHalo - 1/2; the midpoint of
// the RK2 trace moves half as far and interpolates staged values only, so
// its velocity is bounded by the staged maximum too.
constexpr float kFastDisp = 3.0f;

// The two row interpolations of a bilinear sample, top = a + (b - a) fx and
// bot = c + (d - c) fx, as one packed f32x2 subtract and one packed fused
// multiply-add (sm_100 and later): the same two roundings per row as the
// scalar difference and the contracted multiply-add.
__device__ __forceinline__ void lerp_rows(float a, float b, float c, float d, float fx, float& top, float& bot) {
  asm("{\n\t.reg .b64 lo, hi, df, f2, r;\n\t"
      "mov.b64 lo, {%2, %4};\n\t"
      "mov.b64 hi, {%3, %5};\n\t"
      "mov.b64 f2, {%6, %6};\n\t"
      "sub.rn.f32x2 df, hi, lo;\n\t"
      "fma.rn.f32x2 r, df, f2, lo;\n\t"
      "mov.b64 {%0, %1}, r;\n\t}"
      : "=f"(top), "=f"(bot)
      : "f"(a), "f"(b), "f"(c), "f"(d), "f"(fx));
}

template <bool FAST>
struct TileView {
  const float* sm;  // kSH x kSW staged block
  int oi, oj;       // global (unwrapped) index of the block's element (0, 0)
  const float* g;
  int nx, ny;

  // bilinear sample at (bi + ox, bj + oy); with lo/hi also the range of the
  // four cells it read (src/cpu/advect.js:104-111)
  template <bool RANGE = false>
  __device__ __forceinline__ float sample(int bi, int bj, float ox, float oy, float* lo = nullptr,
                                          float* hi = nullptr) const {
    const float fo = floorf(ox), go = floorf(oy);
    const float fx = ox - fo, fy = oy - go;
    const int li = bi + (int)fo - oi, lj = bj + (int)go - oj;
    float a, b, c, d;
    if (FAST || ((unsigned)li < (unsigned)(kSW - 1) && (unsigned)lj < (unsigned)(kSH - 1))) {
      const float* p = sm + lj * kSW + li;
      a = p[0]; b = p[1]; c = p[kSW]; d = p[kSW + 1];
    } else {
      const int i0 = wrap_idx(bi + (int)fo, nx), j0 = wrap_idx(bj + (int)go, ny);
      const int i1 = i0 + 1 == nx ? 0 : i0 + 1;
      const int j1 = j0 + 1 == ny ? 0 : j0 + 1;
      const int64_t r0 = (int64_t)j0 * nx, r1 = (int64_t)j1 * nx;
      a = __ldg(g + r0 + i0); b = __ldg(g + r0 + i1); c = __ldg(g + r1 + i0); d = __ldg(g + r1 + i1);
    }
    if (RANGE) {
      *lo = fminf(fminf(a, b), fminf(c, d));
      *hi = fmaxf(fmaxf(a, b), fmaxf(c, d));
    }
    float top, bot;
    lerp_rows(a, b, c, d, fx, top, bot);
    return top + (bot - top) * fy;
  }
};

// RK2 midpoint backward trace (src/cpu/advect.js:46-54, shaders.js:117-122) in cells
template <bool FAST>
__device__ __forceinline__ void trace_t(const TileView<FAST>& u, const TileView<FAST>& v, int i, int j, Home h,
                                        float cx, float cy, float& dX, float& dY) {
  const float u1 = u.sample(i, j, h.ux, h.uy);
  const float v1 = v.sample(i, j, h.vx, h.vy);
  const float mx = -0.5f * cx * u1, my = -0.5f * cy * v1;
  const float u2 = u.sample(i, j, h.ux + mx, h.uy + my);
  const float v2 = v.sample(i, j, h.vx + mx, h.vy + my);
  dX = -cx * u2;
  dY = -cy * v2;
}

// The same trace from the u-face (UFACE) or the v-face of cell (i, j) for the
// forward pass: the face's own component at the home point sits on a grid
// point (offsets 0, 0), where the bilinear sample equals the stored value for
// every finite field, so it is passed in (own, read from the staged block)
// instead of sampled.  Forward kernel 55.4 -> 53.0 us at 2048^2; in the
// combine kernel the same change measured slower (59.9 -> 63.3 us), which
// keeps trace_t.
template <bool FAST, bool UFACE>
__device__ __forceinline__ void trace_face(const TileView<FAST>& u, const TileView<FAST>& v, int i, int j,
                                           float own, float cx, float cy, float& dX, float& dY) {
  const Home h = UFACE ? home_u() : home_v();
  const float u1 = UFACE ? own : u.sample(i, j, h.ux, h.uy);
  const float v1 = UFACE ? v.sample(i, j, h.vx, h.vy) : own;
  const float mx = -0.5f * cx * u1, my = -0.5f * cy * v1;
  const float u2 = u.sample(i, j, h.ux + mx, h.uy + my);
  const float v2 = v.sample(i, j, h.vx + mx, h.vy + my);
  dX = -cx * u2;
  dY = -cy * v2;
}

// Stage the kSH x kSW blocks of F fields whose (0, 0) is global (oi, oj),
// wrapped, one row per warp at a time; returns max |value| of the first two
// fields (the velocities), NaN counted as infinite.
template <int F>
__device__ __forceinline__ void stage_tiles(float* const (&sm)[F], const float* const (&f)[F], int oi, int oj,
                                            int nx, int ny, float& umax, float& vmax) {
  const int lane = threadIdx.x, warp = threadIdx.y, nwarp = blockDim.y;
  const bool interior = oi >= 0 && oj >= 0 && oi + kSW <= nx && oj + kSH <= ny;
  uint32_t mu = 0, mv = 0;  // bit patterns of non-negative floats order like the floats
  for (int lj = warp; lj < kSH; lj += nwarp) {
    const int gj = interior ? oj + lj : wrap_idx(oj + lj, ny);
    const int64_t row = (int64_t)gj * nx;
    for (int li = lane; li < kSW; li += 32) {
      const int gi = interior ? oi + li : wrap_idx(oi + li, nx);
      const int k = lj * kSW + li;
#pragma unroll
      for (int q = 0; q < F; q++) {
        const float x = __ldg(f[q] + row + gi);
        sm[q][k] = x;
        if (q == 0) mu = max(mu, __float_as_uint(fabsf(x)));
        if (q == 1) mv = max(mv, __float_as_uint(fabsf(x)));
      }
    }
  }
  umax = __uint_as_float(mu);
  vmax = __uint_as_float(mv);
}

// max |value| (NaN counted as infinite) over a staged block, this thread's share
__device__ __forceinline__ uint32_t smem_absmax_bits(const float* sm) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  uint32_t m = 0;
  for (int k = tid; k < kSW * kSH; k += nthr) m = max(m, __float_as_uint(fabsf(sm[k])));
  return m;
}

// TMA staging of F kSH x kSW blocks (tiles whose block lies inside the grid):
// thread 0 arms the barrier and issues the copies, every thread waits (bounded).
// Returns false on every thread if the wait gave up (after waiting once more
// for the copies in flight and raising *err); the caller then skips the tile.
template <int F>
__device__ __forceinline__ bool tma_stage(float* const (&sm)[F], const CUtensorMap* const (&tm)[F], int oi, int oj,
                                          uint64_t* bar, int* err) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar, (uint32_t)(F * kSW * kSH * sizeof(float)));
#pragma unroll
    for (int q = 0; q < F; q++) tc::tma_load_2d(sm[q], tm[q], oi, oj, bar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(bar, 0)) != 0;
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    tc::mbar_wait(bar, 0);
  }
  return ok;
}

// one CTA-wide decision after staging (and the barrier the staging needs)
__device__ __forceinline__ bool fast_tile(float umax, float vmax, float cx, float cy) {
  const bool ok = umax * fabsf(cx) <= kFastDisp && vmax * fabsf(cy) <= kFastDisp;  // false for NaN / inf
  return __syncthreads_and(ok) != 0;
}

// ADVECT_VELOCITY: each component traced from its own face (shaders.js:126-146).
// With bounds != nullptr (the forward pass of MacCormack) the min and max of
// the four cells each sample read -- the limiter's range, src/cpu/advect.js
// :104-111 -- are written too, planes (lo_u, hi_u, lo_v, hi_v), so the combine
// pass does not trace forward again.
template <bool FAST>
__device__ __forceinline__ void advect_rows(const TileView<FAST>& U, const TileView<FAST>& V, float* __restrict__ ou,
                                            float* __restrict__ ov, int nx, int ny, int ti, int tj, float cx,
                                            float cy, float* __restrict__ bounds) {
  const Home hu = home_u(), hv = home_v();
  const int i = ti + threadIdx.x;
  if (i >= nx) return;
  const int64_t n = (int64_t)nx * ny;
  for (int r = threadIdx.y; r < kTY; r += blockDim.y) {
    const int j = tj + r;
    if (j >= ny) break;
    const int64_t c = (int64_t)j * nx + i;
    const int lc = (r + kHalo) * kSW + threadIdx.x + kHalo;  // this cell in the staged block
    float dX, dY, lo, hi;
    trace_face<FAST, true>(U, V, i, j, U.sm[lc], cx, cy, dX, dY);
    if (bounds) {
      ou[c] = U.template sample<true>(i, j, hu.ux + dX, hu.uy + dY, &lo, &hi);
      bounds[c] = lo;
      bounds[n + c] = hi;
    } else {
      ou[c] = U.sample(i, j, hu.ux + dX, hu.uy + dY);
    }
    trace_face<FAST, false>(U, V, i, j, V.sm[lc], cx, cy, dX, dY);
    if (bounds) {
      ov[c] = V.template sample<true>(i, j, hv.vx + dX, hv.vy + dY, &lo, &hi);
      bounds[2 * n + c] = lo;
      bounds[3 * n + c] = hi;
    } else {
      ov[c] = V.sample(i, j, hv.vx + dX, hv.vy + dY);
    }
  }
}

// Tiles whose staged block lies inside the grid are staged by TMA when the
// tensor maps are valid (tma != 0); the others by the wrapped loads.
__global__ void __launch_bounds__(256) k_advect_sl_t(const float* __restrict__ u, const float* __restrict__ v,
                                                     float* __restrict__ ou, float* __restrict__ ov, int nx, int ny,
                                                     float cx, float cy, float* __restrict__ bounds,
                                                     const __grid_constant__ CUtensorMap tm_u,
                                                     const __grid_constant__ CUtensorMap tm_v, int tma, int* err) {
  __shared__ __align__(128) float su[kSW * kSH];
  __shared__ __align__(128) float sv[kSW * kSH];
  __shared__ uint64_t bar;
  const int ti = blockIdx.x * kTX, tj = blockIdx.y * kTY;
  const int oi = ti - kHalo, oj = tj - kHalo;
  float umax, vmax;
  {
    float* const sm[2] = {su, sv};
    if (tma && oi >= 0 && oj >= 0 && oi + kSW <= nx && oj + kSH <= ny) {
      const CUtensorMap* const tm[2] = {&tm_u, &tm_v};
      if (!tma_stage<2>(sm, tm, oi, oj, &bar, err)) return;
      umax = __uint_as_float(smem_absmax_bits(su));
      vmax = __uint_as_float(smem_absmax_bits(sv));
    } else {
      const float* const f[2] = {u, v};
      stage_tiles<2>(sm, f, oi, oj, nx, ny, umax, vmax);
    }
  }
  if (fast_tile(umax, vmax, cx, cy)) {
    const TileView<true> U{su, oi, oj, u, nx, ny}, V{sv, oi, oj, v, nx, ny};
    advect_rows(U, V, ou, ov, nx, ny, ti, tj, cx, cy, bounds);
  } else {
    const TileView<false> U{su, oi, oj, u, nx, ny}, V{sv, oi, oj, v, nx, ny};
    advect_rows(U, V, ou, ov, nx, ny, ti, tj, cx, cy, bounds);
  }
}

// MACCORMACK: the backward pass (ADVECT_FIELD_BY with -dt) is evaluated inside
// the combine kernel at the single point it is needed, then the correction
// limited to the forward pass's range (shaders.js:187-231, src/cpu/advect.js:149-185).
template <bool FAST>
__device__ __forceinline__ void combine_rows(const TileView<FAST>& U, const TileView<FAST>& V,
                                             const TileView<FAST>& FU, const TileView<FAST>& FV,
                                             const float* __restrict__ bounds, float* __restrict__ ou,
                                             float* __restrict__ ov, int nx, int ny, int ti, int tj, float cx,
                                             float cy) {
  const Home hu = home_u(), hv = home_v();
  const int i = ti + threadIdx.x;
  if (i >= nx) return;
  const int64_t n = (int64_t)nx * ny;
  for (int r = threadIdx.y; r < kTY; r += blockDim.y) {
    const int j = tj + r;
    if (j >= ny) break;
    const int64_t c = (int64_t)j * nx + i;
    const int lc = (r + kHalo) * kSW + threadIdx.x + kHalo;  // this cell in the staged block
    const float lou = __ldg(bounds + c), hiu = __ldg(bounds + n + c);
    const float lov = __ldg(bounds + 2 * n + c), hiv = __ldg(bounds + 3 * n + c);
    float dX, dY;
    // u component
    trace_t(U, V, i, j, hu, -cx, -cy, dX, dY);  // backward: trace with -dt
    const float bu = FU.sample(i, j, hu.ux + dX, hu.uy + dY);
    float cu = FU.sm[lc] + 0.5f * (U.sm[lc] - bu);
    cu = cu < lou ? lou : cu > hiu ? hiu : cu;
    // v component
    trace_t(U, V, i, j, hv, -cx, -cy, dX, dY);
    const float bv = FV.sample(i, j, hv.vx + dX, hv.vy + dY);
    float cv = FV.sm[lc] + 0.5f * (V.sm[lc] - bv);
    cv = cv < lov ? lov : cv > hiv ? hiv : cv;
    ou[c] = cu;
    ov[c] = cv;
  }
}

__global__ void __launch_bounds__(256) k_mc_combine_t(const float* __restrict__ u, const float* __restrict__ v,
                                                      const float* __restrict__ fu, const float* __restrict__ fv,
                                                      const float* __restrict__ bounds, float* __restrict__ ou,
                                                      float* __restrict__ ov, int nx, int ny, float cx, float cy,
                                                      const __grid_constant__ CUtensorMap tm_u,
                                                      const __grid_constant__ CUtensorMap tm_v,
                                                      const __grid_constant__ CUtensorMap tm_fu,
                                                      const __grid_constant__ CUtensorMap tm_fv, int tma, int* err) {
  __shared__ __align__(128) float su[kSW * kSH];
  __shared__ __align__(128) float sv[kSW * kSH];
  __shared__ __align__(128) float sfu[kSW * kSH];
  __shared__ __align__(128) float sfv[kSW * kSH];
  __shared__ uint64_t bar;
  const int ti = blockIdx.x * kTX, tj = blockIdx.y * kTY;
  const int oi = ti - kHalo, oj = tj - kHalo;
  float umax, vmax;
  {
    float* const sm[4] = {su, sv, sfu, sfv};
    if (tma && oi >= 0 && oj >= 0 && oi + kSW <= nx && oj + kSH <= ny) {
      const CUtensorMap* const tm[4] = {&tm_u, &tm_v, &tm_fu, &tm_fv};
      if (!tma_stage<4>(sm, tm, oi, oj, &bar, err)) return;
      umax = __uint_as_float(smem_absmax_bits(su));
      vmax = __uint_as_float(smem_absmax_bits(sv));
    } else {
      const float* const f[4] = {u, v, fu, fv};
      stage_tiles<4>(sm, f, oi, oj, nx, ny, umax, vmax);
    }
  }
  if (fast_tile(umax, vmax, cx, cy)) {
    const TileView<true> U{su, oi, oj, u, nx, ny}, V{sv, oi, oj, v, nx, ny};
    const TileView<true> FU{sfu, oi, oj, fu, nx, ny}, FV{sfv, oi, oj, fv, nx, ny};
    combine_rows(U, V, FU, FV, bounds, ou, ov, nx, ny, ti, tj, cx, cy);
  } else {
    const TileView<false> U{su, oi, oj, u, nx, ny}, V{sv, oi, oj, v, nx, ny};
    const TileView<false> FU{sfu, oi, oj, fu, nx, ny}, FV{sfv, oi, oj, fv, nx, ny};
    combine_rows(U, V, FU, FV, bounds, ou, ov, nx, ny, ti, tj, cx, cy);
  }
}

// ------------------------------------------------- batched (one size class)
// The steps of the members of one batch size class (fs_api.cu batch_build),
// one launch per kernel, member = blockIdx.z, pointers and per-member step
// factors in a table passed by value; staging by the wrapped loads (the same
// values the TMA copies deliver).
struct AdvTab {
  struct {
    const float* u;
    const float* v;
    const float* fu;  // combine: the forward field
    const float* fv;
    float* ou;
    float* ov;
    float* bounds;
    float cx, cy;
  } m[kClassMax];
};
struct DiffTab {
  struct {
    const float* u;
    const float* v;
    float* ou;
    float* ov;
    float a, b;
  } m[kClassMax];
};

__global__ void __launch_bounds__(256) k_advect_sl_class(const AdvTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  __shared__ __align__(128) float su[kSW * kSH];
  __shared__ __align__(128) float sv[kSW * kSH];
  const int ti = blockIdx.x * kTX, tj = blockIdx.y * kTY;
  const int oi = ti - kHalo, oj = tj - kHalo;
  float umax, vmax;
  {
    float* const sm[2] = {su, sv};
    const float* const f[2] = {a.u, a.v};
    stage_tiles<2>(sm, f, oi, oj, nx, ny, umax, vmax);
  }
  if (fast_tile(umax, vmax, a.cx, a.cy)) {
    const TileView<true> U{su, oi, oj, a.u, nx, ny}, V{sv, oi, oj, a.v, nx, ny};
    advect_rows(U, V, a.ou, a.ov, nx, ny, ti, tj, a.cx, a.cy, a.bounds);
  } else {
    const TileView<false> U{su, oi, oj, a.u, nx, ny}, V{sv, oi, oj, a.v, nx, ny};
    advect_rows(U, V, a.ou, a.ov, nx, ny, ti, tj, a.cx, a.cy, a.bounds);
  }
}

__global__ void __launch_bounds__(256) k_mc_combine_class(const AdvTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  __shared__ __align__(128) float su[kSW * kSH];
  __shared__ __align__(128) float sv[kSW * kSH];
  __shared__ __align__(128) float sfu[kSW * kSH];
  __shared__ __align__(128) float sfv[kSW * kSH];
  const int ti = blockIdx.x * kTX, tj = blockIdx.y * kTY;
  const int oi = ti - kHalo, oj = tj - kHalo;
  float umax, vmax;
  {
    float* const sm[4] = {su, sv, sfu, sfv};
    const float* const f[4] = {a.u, a.v, a.fu, a.fv};
    stage_tiles<4>(sm, f, oi, oj, nx, ny, umax, vmax);
  }
  if (fast_tile(umax, vmax, a.cx, a.cy)) {
    const TileView<true> U{su, oi, oj, a.u, nx, ny}, V{sv, oi, oj, a.v, nx, ny};
    const TileView<true> FU{sfu, oi, oj, a.fu, nx, ny}, FV{sfv, oi, oj, a.fv, nx, ny};
    combine_rows(U, V, FU, FV, a.bounds, a.ou, a.ov, nx, ny, ti, tj, a.cx, a.cy);
  } else {
    const TileView<false> U{su, oi, oj, a.u, nx, ny}, V{sv, oi, oj, a.v, nx, ny};
    const TileView<false> FU{sfu, oi, oj, a.fu, nx, ny}, FV{sfv, oi, oj, a.fv, nx, ny};
    combine_rows(U, V, FU, FV, a.bounds, a.ou, a.ov, nx, ny, ti, tj, a.cx, a.cy);
  }
}

static const dim3 kBlock(32, 8);

static dim3 tile_grid(const Grid& g) { return dim3((g.nx + kTX - 1) / kTX, (g.ny + kTY - 1) / kTY); }



// Tensor maps of f32 planes for the TMA-staged tiles (the advection tiles'
// kSW x kSH box here, the multigrid tile boxes in fs_multigrid.cu), kept per
// device pointer, plane and box.  TMA needs the row pitch and the box width
// multiples of 16 bytes (nx % 4 == 0) and a 16-byte-aligned base; otherwise,
// or if the CUDA driver lacks the encoder, every tile uses wrapped loads.
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

bool box_tmap(Solver* s, const float* f, int nx, int ny, int bw, int bh, CUtensorMap* out) {
  if (nx % 4 != 0 || bw % 4 != 0 || ((uintptr_t)f & 15) != 0 || nx < bw || ny < bh || bw > 256 || bh > 256)
    return false;
  for (const auto& e : s->tmaps)
    if (e.p == f && e.nx == nx && e.ny == ny && e.bw == bw && e.bh == bh) {
      *out = e.m;
      return true;
    }
  PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
  if (!enc) return false;
  Solver::Tmap e;
  e.p = f;
  e.nx = nx; e.ny = ny; e.bw = bw; e.bh = bh;
  const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  const cuuint64_t pitch[1] = {(cuuint64_t)nx * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
  const cuuint32_t estr[2] = {1, 1};
  if (enc(&e.m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(f), dims, pitch, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  s->tmaps.push_back(e);
  *out = e.m;
  return true;
}

static bool tile_tmap(Solver* s, const float* f, CUtensorMap* out) {
  return box_tmap(s, f, s->g.nx, s->g.ny, kSW, kSH, out);
}

template <>
void launch_advect_sl<float>(Solver* s, const float* u, const float* v, float* ou, float* ov, float dt) {
  const Grid& g = s->g;
  float cx = (float)((double)dt / g.dxd), cy = (float)((double)dt / g.dyd);
  CUtensorMap tu{}, tv{};
  const int tma = tile_tmap(s, u, &tu) && tile_tmap(s, v, &tv) ? 1 : 0;
  FS_LAUNCH(s, "advect_sl", (double)s->n * 16,
            k_advect_sl_t<<<tile_grid(g), kBlock, 0, s->stream>>>(u, v, ou, ov, g.nx, g.ny, cx, cy, nullptr, tu, tv,
                                                                  tma, &s->dev->async_err));
}

template <>
void launch_advect_mc<float>(Solver* s, const float* u, const float* v, float* fu, float* fv, float* ou,
                             float* ov, float dt) {
  const Grid& g = s->g;
  float cx = (float)((double)dt / g.dxd), cy = (float)((double)dt / g.dyd);
  CUtensorMap tu{}, tv{}, tfu{}, tfv{};
  const int tma =
      tile_tmap(s, u, &tu) && tile_tmap(s, v, &tv) && tile_tmap(s, fu, &tfu) && tile_tmap(s, fv, &tfv) ? 1 : 0;
  FS_LAUNCH(s, "advect_sl", (double)s->n * 32,
            k_advect_sl_t<<<tile_grid(g), kBlock, 0, s->stream>>>(u, v, fu, fv, g.nx, g.ny, cx, cy, s->mc_bounds, tu,
                                                                  tv, tma, &s->dev->async_err));
  FS_LAUNCH(s, "mc_combine", (double)s->n * 40,
            k_mc_combine_t<<<tile_grid(g), kBlock, 0, s->stream>>>(u, v, fu, fv, s->mc_bounds, ou, ov, g.nx, g.ny,
                                                                   cx, cy, tu, tv, tfu, tfv, tma,
                                                                   &s->dev->async_err));
}

// DIFFUSE (shaders.js:401-425; src/cpu/solver.js:56-68 operand order)
// c + a (l + r - 2c) + b (bo + t - 2c) with every rounding spelled out, in
// the order of DIFFUSE (shaders.js:420), so that the one-cell and the
// four-cell forms (and the batched kernels) round identically
__device__ __forceinline__ float diffuse_cell(float c, float l, float r, float bo, float t, float a, float b) {
  const float c2 = __fmul_rn(2.f, c);
  return __fadd_rn(__fadd_rn(c, __fmul_rn(a, __fsub_rn(__fadd_rn(l, r), c2))),
                   __fmul_rn(b, __fsub_rn(__fadd_rn(bo, t), c2)));
}

__device__ __forceinline__ void diffuse_body(const float* __restrict__ u, const float* __restrict__ v,
                                             float* __restrict__ ou, float* __restrict__ ov, int nx, int ny, float a,
                                             float b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
  int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
  int64_t r = (int64_t)j * nx, rm = (int64_t)jm * nx, rp = (int64_t)jp * nx;
  ou[r + i] = diffuse_cell(__ldg(u + r + i), __ldg(u + r + im), __ldg(u + r + ip), __ldg(u + rm + i),
                           __ldg(u + rp + i), a, b);
  ov[r + i] = diffuse_cell(__ldg(v + r + i), __ldg(v + r + im), __ldg(v + r + ip), __ldg(v + rm + i),
                           __ldg(v + rp + i), a, b);
}

// Four consecutive cells per thread (nx a multiple of 4): float4 loads of the
// three rows, the group's outer left and right neighbours as scalars.
__device__ __forceinline__ void diffuse4_one(const float* __restrict__ f, float* __restrict__ o, int64_t r,
                                             int64_t rm, int64_t rp, int i0, int il, int ir, float a, float b) {
  const float4 c = __ldg(reinterpret_cast<const float4*>(f + r + i0));
  const float4 bo = __ldg(reinterpret_cast<const float4*>(f + rm + i0));
  const float4 t = __ldg(reinterpret_cast<const float4*>(f + rp + i0));
  const float l = __ldg(f + r + il), rr = __ldg(f + r + ir);
  float4 out;
  out.x = diffuse_cell(c.x, l, c.y, bo.x, t.x, a, b);
  out.y = diffuse_cell(c.y, c.x, c.z, bo.y, t.y, a, b);
  out.z = diffuse_cell(c.z, c.y, c.w, bo.z, t.z, a, b);
  out.w = diffuse_cell(c.w, c.z, rr, bo.w, t.w, a, b);
  *reinterpret_cast<float4*>(o + r + i0) = out;
}

__device__ __forceinline__ void diffuse4_body(const float* __restrict__ u, const float* __restrict__ v,
                                              float* __restrict__ ou, float* __restrict__ ov, int nx, int ny,
                                              float a, float b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (q >= (nx >> 2) || j >= ny) return;
  const int i0 = q << 2, il = i0 == 0 ? nx - 1 : i0 - 1, ir = i0 + 4 == nx ? 0 : i0 + 4;
  const int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
  const int64_t r = (int64_t)j * nx, rm = (int64_t)jm * nx, rp = (int64_t)jp * nx;
  diffuse4_one(u, ou, r, rm, rp, i0, il, ir, a, b);
  diffuse4_one(v, ov, r, rm, rp, i0, il, ir, a, b);
}

__global__ void __launch_bounds__(256) k_diffuse4(const float* __restrict__ u, const float* __restrict__ v,
                                                  float* __restrict__ ou, float* __restrict__ ov,
                                                  int nx, int ny, float a, float b) {
  diffuse4_body(u, v, ou, ov, nx, ny, a, b);
}

__global__ void __launch_bounds__(256) k_diffuse(const float* __restrict__ u, const float* __restrict__ v,
                                                 float* __restrict__ ou, float* __restrict__ ov,
                                                 int nx, int ny, float a, float b) {
  diffuse_body(u, v, ou, ov, nx, ny, a, b);
}

void launch_diffuse(Solver* s, const float* u, const float* v, float* ou, float* ov, float dt) {
  const Grid& g = s->g;
  float a = (float)(s->prm.nu * dt / (g.dxd * g.dxd));
  float b = (float)(s->prm.nu * dt / (g.dyd * g.dyd));
  FS_LAUNCH(s, "diffuse", (double)s->n * 16,
            if (g.nx % 4 == 0) {
              k_diffuse4<<<grid2d(g.nx / 4, g.ny, kBlock), kBlock, 0, s->stream>>>(u, v, ou, ov, g.nx, g.ny, a, b);
            } else {
              k_diffuse<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(u, v, ou, ov, g.nx, g.ny, a, b);
            });
}

__global__ void __launch_bounds__(256) k_diffuse_class(const DiffTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  if ((nx & 3) == 0) diffuse4_body(a.u, a.v, a.ou, a.ov, nx, ny, a.a, a.b);
  else diffuse_body(a.u, a.v, a.ou, a.ov, nx, ny, a.a, a.b);
}

// advection (and diffusion) of every member of a class into (wu, wv), or
// (tu, tv) after the diffusion; the velocity the projection reads
void launch_front_advect_class(Solver* const* ms, int count, const double* dts, cudaStream_t st) {
  Solver* s0 = ms[0];
  const Grid& g = s0->g;
  const bool mc = s0->prm.advection == FS_ADVECT_MACCORMACK;
  AdvTab fwd{}, comb{};
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    const float dt = (float)dts[i];
    const float cx = (float)((double)dt / s->g.dxd), cy = (float)((double)dt / s->g.dyd);
    if (mc) {
      fwd.m[i] = {s->u, s->v, nullptr, nullptr, s->fu, s->fv, s->mc_bounds, cx, cy};
      comb.m[i] = {s->u, s->v, s->fu, s->fv, s->wu, s->wv, s->mc_bounds, cx, cy};
    } else {
      fwd.m[i] = {s->u, s->v, nullptr, nullptr, s->wu, s->wv, nullptr, cx, cy};
    }
  }
  dim3 grid = tile_grid(g);
  grid.z = count;
  k_advect_sl_class<<<grid, kBlock, 0, st>>>(fwd, g.nx, g.ny);
  if (mc) k_mc_combine_class<<<grid, kBlock, 0, st>>>(comb, g.nx, g.ny);
  if (s0->prm.nu > 0) {
    DiffTab dt{};
    for (int i = 0; i < count; i++) {
      Solver* s = ms[i];
      const float a = (float)(s->prm.nu * (float)dts[i] / (s->g.dxd * s->g.dxd));
      const float b = (float)(s->prm.nu * (float)dts[i] / (s->g.dyd * s->g.dyd));
      dt.m[i] = {s->wu, s->wv, s->tu, s->tv, a, b};
    }
    dim3 g2 = grid2d(g.nx % 4 == 0 ? g.nx / 4 : g.nx, g.ny, kBlock);  // four cells per thread when nx % 4 == 0
    g2.z = count;
    k_diffuse_class<<<g2, kBlock, 0, st>>>(dt, g.nx, g.ny);
  }
}

// FORCING + drag, in place (shaders.js:532-566): u <- u*exp(-drag dt) + amp dt/sqrt(M) sum_m
// The phase drift is drift_rate * t with t read from the device step state, so
// a captured step needs no host update per step (solver.js:396 passes
// phaseDrift * t as param_b).
__global__ void __launch_bounds__(256) k_forcing(float* __restrict__ u, float* __restrict__ v,
                                                 const float* __restrict__ modes, int m, int nx,
                                                 int ny, float dx, float dy, float scale, float damp,
                                                 double drift_rate, const DevState* __restrict__ st) {
  __shared__ float s_drift;
  if (threadIdx.x == 0 && threadIdx.y == 0) s_drift = (float)(drift_rate * st->t);
  __syncthreads();
  const float drift = s_drift;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  float pux = i * dx, puy = (j + 0.5f) * dy, pvx = (i + 0.5f) * dx, pvy = j * dy;
  float fu = 0.f, fv = 0.f;
  for (int k = 0; k < m; k++) {
    float kx = __ldg(modes + 3 * k), ky = __ldg(modes + 3 * k + 1), ph = __ldg(modes + 3 * k + 2);
    float kk = sqrtf(kx * kx + ky * ky);
    if (kk < 1e-6f) continue;
    fu += (ky / kk) * cosf(kx * pux + ky * puy + ph + drift);
    fv -= (kx / kk) * cosf(kx * pvx + ky * pvy + ph + drift);
  }
  int64_t c = (int64_t)j * nx + i;
  u[c] = u[c] * damp + scale * fu;
  v[c] = v[c] * damp + scale * fv;
}

void launch_forcing(Solver* s, float* u, float* v, float dt) {
  const Grid& g = s->g;
  float scale = (float)(s->amp * dt / sqrt((double)s->n_modes));
  float damp = (float)exp(-s->drag * dt);
  FS_LAUNCH(s, "forcing", (double)s->n * 16,
            k_forcing<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                u, v, s->modes, s->n_modes, g.nx, g.ny, g.dx, g.dy, scale, damp, s->drift, s->dev));
}

// Direct forcing of immersed disks (src/cpu/solid.js:165-233, shaders.js:587-653):
// chi = 0.5 (1 - tanh((|d| - r)/w)), u += chi (U_s - u), applied where chi >= 1e-6,
// disk after disk at each face.  Impulses are summed per disk on the device.
struct DiskDev {
  float x, y, r, vx, vy, omega, reach2;
};
#define FS_MAX_DISKS 64

// shortest signed separation on a periodic axis (src/cpu/solid.js:38-40), with 1/L precomputed
__device__ __forceinline__ float wrap_delta(float d, float L, float iL) { return d - L * floorf(d * iL + 0.5f); }

// One CTA per 32x8 tile from `tiles` (the tiles some disk can reach, listed
// when the disks are set); cells elsewhere are left untouched.
__global__ void __launch_bounds__(256)
    k_solids(float* __restrict__ u, float* __restrict__ v, const DiskDev* __restrict__ disks, int ndisk,
             const int* __restrict__ tiles, const unsigned long long* __restrict__ masks, int nx, int ny, float dx,
             float dy, float lx, float ly, float width, double dA, float* __restrict__ imp,
             double* __restrict__ dimp) {
  // per-warp impulse sums of every disk, folded per CTA after the loop
  __shared__ float wsum[FS_MAX_DISKS][8][3];
  const int t = __ldg(tiles + blockIdx.x), ntx = (nx + 31) >> 5;
  int i = (t % ntx) * 32 + threadIdx.x, j = (t / ntx) * 8 + threadIdx.y;
  bool in = i < nx && j < ny;
  int64_t c = (int64_t)j * nx + i;
  float pux = i * dx, puy = (j + 0.5f) * dy, pvx = (i + 0.5f) * dx, pvy = j * dy;
  const float ilx = 1.f / lx, ily = 1.f / ly;
  float uu = 0.f, vv = 0.f;
  bool loaded = false;
  float tix = 0.f, tiy = 0.f, tit = 0.f;
  // only the disks that can reach this tile, in order (the others change nothing here)
  const unsigned long long mask = __ldg(masks + blockIdx.x);
  for (unsigned long long rest = mask; rest; rest &= rest - 1) {
    const int k = __ffsll((long long)rest) - 1;
    const DiskDev d = disks[k];
    float fx = 0.f, fy = 0.f, tq = 0.f;
    if (in) {
      float ax = wrap_delta(pux - d.x, lx, ilx), ay = wrap_delta(puy - d.y, ly, ily);
      float bx = wrap_delta(pvx - d.x, lx, ilx), by = wrap_delta(pvy - d.y, ly, ily);
      bool nu_ = ax * ax + ay * ay <= d.reach2, nv_ = bx * bx + by * by <= d.reach2;
      if ((nu_ || nv_) && !loaded) {
        uu = u[c];
        vv = v[c];
        loaded = true;
      }
      if (nu_) {
        float chi = 0.5f * (1.f - tanhf((sqrtf(ax * ax + ay * ay) - d.r) / width));
        if (chi >= 1e-6f) {
          float du = chi * ((d.vx - d.omega * ay) - uu);
          uu += du;
          fx = du;
          tq += -ay * du;
        }
      }
      if (nv_) {
        float chi = 0.5f * (1.f - tanhf((sqrtf(bx * bx + by * by) - d.r) / width));
        if (chi >= 1e-6f) {
          float dv = chi * ((d.vy + d.omega * bx) - vv);
          vv += dv;
          fy = dv;
          tq += bx * dv;
        }
      }
    }
    tix += fx;
    tiy += fy;
    tit += tq;
    // warp sum of this disk's impulse (the shuffles only in warps that
    // touched the disk)
    if (dimp) {
      float sx = 0.f, sy = 0.f, st = 0.f;
      if (__any_sync(0xffffffffu, fx != 0.f || fy != 0.f || tq != 0.f)) {
        sx = fx; sy = fy; st = tq;
        for (int o = 16; o > 0; o >>= 1) {
          sx += __shfl_xor_sync(0xffffffffu, sx, o);
          sy += __shfl_xor_sync(0xffffffffu, sy, o);
          st += __shfl_xor_sync(0xffffffffu, st, o);
        }
      }
      if (threadIdx.x == 0) {
        wsum[k][threadIdx.y][0] = sx;
        wsum[k][threadIdx.y][1] = sy;
        wsum[k][threadIdx.y][2] = st;
      }
    }
  }
  if (in) {
    if (loaded) {
      u[c] = uu;
      v[c] = vv;
    }
    if (imp) {
      imp[c] = tix;
      imp[(int64_t)nx * ny + c] = tiy;
      imp[2 * (int64_t)nx * ny + c] = tit;
    }
  }
  if (!dimp) return;
  // one f64 atomic per CTA, disk and component (a per-warp atomic made the
  // warps of a large disk queue on one address); the order of the atomics is
  // not fixed, so the impulse sums (not the velocity field) may differ in the
  // last bits run to run
  __syncthreads();
  for (int q = threadIdx.y * 32 + threadIdx.x; q < 3 * ndisk; q += 256) {
    const int k = q / 3, comp = q - 3 * k;
    if (!((mask >> k) & 1ull)) continue;  // this tile's warps did not write it
    double sum = 0.0;
#pragma unroll
    for (int w = 0; w < 8; w++) sum += (double)wsum[k][w][comp];
    if (sum != 0.0) atomicAdd(dimp + q, sum * dA);
  }
}

// Disk parameters go to the device once, when they are set; the per-step
// launch then needs nothing from the host (and can be captured in a graph).
int upload_disks(Solver* s) {
  const Grid& g = s->g;
  int nd = (int)s->disks.size();
  if (nd == 0) return 0;
  double width = s->prm.solid_mask_width * g.dxd;
  DiskDev hd[FS_MAX_DISKS];
  for (int k = 0; k < nd; k++) {
    const fs_disk& d = s->disks[k];
    // chi >= 1e-6 needs (|d| - r)/w <= atanh(1 - 2e-6) ~ 6.9; one cell of margin
    double reach = d.r + 7.0 * width + g.dxd + g.dyd;
    hd[k] = {(float)d.x, (float)d.y, (float)d.r, (float)d.vx, (float)d.vy, (float)d.omega,
             (float)(reach * reach)};
  }
  if (!s->d_disks && cudaMalloc(&s->d_disks, sizeof(DiskDev) * FS_MAX_DISKS) != cudaSuccess) return -1;
  if (cudaMemcpy(s->d_disks, hd, sizeof(DiskDev) * nd, cudaMemcpyHostToDevice) != cudaSuccess) return -1;
  // the 32x8 tiles any disk can reach (periodic), as a compact list
  const int ntx = (g.nx + 31) / 32, nty = (g.ny + 7) / 8;
  std::vector<unsigned long long> mark((size_t)ntx * nty, 0);  // per tile: the disks that reach it
  for (int k = 0; k < nd; k++) {
    const fs_disk& d = s->disks[k];
    double reach = d.r + 7.0 * width + g.dxd + g.dyd;
    int i0 = (int)floor((d.x - reach) / g.dxd) - 1, i1 = (int)ceil((d.x + reach) / g.dxd) + 1;
    int j0 = (int)floor((d.y - reach) / g.dyd) - 1, j1 = (int)ceil((d.y + reach) / g.dyd) + 1;
    if (i1 - i0 >= g.nx) { i0 = 0; i1 = g.nx - 1; }
    if (j1 - j0 >= g.ny) { j0 = 0; j1 = g.ny - 1; }
    for (int j = j0; j <= j1; j++)
      for (int i = i0; i <= i1; i++) {
        int wi = ((i % g.nx) + g.nx) % g.nx, wj = ((j % g.ny) + g.ny) % g.ny;
        mark[(size_t)(wj / 8) * ntx + wi / 32] |= 1ull << k;
      }
  }
  std::vector<int> list;
  std::vector<unsigned long long> masks;
  for (size_t t = 0; t < mark.size(); t++)
    if (mark[t]) {
      list.push_back((int)t);
      masks.push_back(mark[t]);
    }
  if (s->d_tiles) cudaFree(s->d_tiles);
  if (s->d_tile_masks) cudaFree(s->d_tile_masks);
  s->d_tiles = nullptr;
  s->d_tile_masks = nullptr;
  s->n_tiles = (int)list.size();
  if (cudaMalloc((void**)&s->d_tiles, sizeof(int) * list.size()) != cudaSuccess) return -1;
  if (cudaMalloc((void**)&s->d_tile_masks, sizeof(unsigned long long) * masks.size()) != cudaSuccess) return -1;
  if (cudaMemcpy(s->d_tiles, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice) != cudaSuccess) return -1;
  if (cudaMemcpy(s->d_tile_masks, masks.data(), sizeof(unsigned long long) * masks.size(),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return -1;
  return 0;
}

void launch_solids(Solver* s, float* u, float* v, float dt, bool record_impulse) {
  (void)dt;
  const Grid& g = s->g;
  int nd = (int)s->disks.size();
  if (nd == 0) return;
  double width = s->prm.solid_mask_width * g.dxd;
  cudaMemsetAsync(s->d_impulse, 0, sizeof(double) * 3 * nd, s->stream);
  // the per-cell impulse field is only written inside the listed tiles
  if (record_impulse) cudaMemsetAsync(s->imp, 0, sizeof(float) * 3 * (size_t)s->n, s->stream);
  FS_LAUNCH(s, "solids", (double)s->n_tiles * 256 * (record_impulse ? 28 : 16),
            k_solids<<<s->n_tiles, kBlock, 0, s->stream>>>(
                u, v, (const DiskDev*)s->d_disks, nd, s->d_tiles, s->d_tile_masks, g.nx, g.ny, g.dx, g.dy,
                (float)(g.nx * g.dxd), (float)(g.ny * g.dyd), (float)width, g.dxd * g.dyd,
                record_impulse ? s->imp : nullptr, s->d_impulse));
}

// ------------------------------------------------------------------- dye
// ADVECT_SCALAR (shaders.js:234-266): RK2 trace from the cell centre through
// the projected velocity, bilinear sample of the RGBA field (centre grid),
// fade, clamp to [0, 1].  The centre (i+1/2, j+1/2) is at u-grid index
// (i+1/2, j) and v-grid index (i, j+1/2).
__device__ __forceinline__ Home home_c() { return {0.5f, 0.f, 0.f, 0.5f}; }

__global__ void __launch_bounds__(256) k_advect_dye(const float* __restrict__ u, const float* __restrict__ v,
                                                    const float4* __restrict__ q, float4* __restrict__ out, int nx,
                                                    int ny, float cx, float cy, float keep) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  float dX, dY;
  trace(u, v, nx, ny, i, j, home_c(), cx, cy, dX, dY);
  float fo = floorf(dX), go = floorf(dY);
  float fx = dX - fo, fy = dY - go;
  int i0 = wrap_idx(i + (int)fo, nx), j0 = wrap_idx(j + (int)go, ny);
  int i1 = i0 + 1 == nx ? 0 : i0 + 1, j1 = j0 + 1 == ny ? 0 : j0 + 1;
  float4 a = q[(int64_t)j0 * nx + i0], b = q[(int64_t)j0 * nx + i1];
  float4 c = q[(int64_t)j1 * nx + i0], d = q[(int64_t)j1 * nx + i1];
  auto lerp2 = [&](float pa, float pb, float pc, float pd) {
    float top = pa + (pb - pa) * fx, bot = pc + (pd - pc) * fx;
    return fminf(fmaxf((top + (bot - top) * fy) * keep, 0.f), 1.f);
  };
  out[(int64_t)j * nx + i] = make_float4(lerp2(a.x, b.x, c.x, d.x), lerp2(a.y, b.y, c.y, d.y),
                                         lerp2(a.z, b.z, c.z, d.z), lerp2(a.w, b.w, c.w, d.w));
}

void launch_advect_dye(Solver* s, float dt) {
  const Grid& g = s->g;
  dim3 b(32, 8);
  FS_LAUNCH(s, "advect_dye", (double)s->n * 40,
            k_advect_dye<<<grid2d(g.nx, g.ny, b), b, 0, s->stream>>>(
                s->u, s->v, static_cast<const float4*>(s->dye), static_cast<float4*>(s->dye2), g.nx, g.ny,
                (float)(dt * g.idxd), (float)(dt * g.idyd), (float)(1.0 - s->prm.dye_fade)));
  // the next step reads s->dye again: copy back (a captured step cannot swap pointers)
  cudaMemcpyAsync(s->dye, s->dye2, (size_t)s->n * 16, cudaMemcpyDeviceToDevice, s->stream);
}

}  // namespace fs
