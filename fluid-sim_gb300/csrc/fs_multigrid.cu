// fs_multigrid.cu -- fused multigrid V-cycle for GB300 (sm_103a).
//
// The V-cycle of src/gpu/multigrid.js:277-330 (RBGS(pre) -> residual ->
// restriction -> ... -> coarse RBGS(40) -> prolongation -> RBGS(post)) costs
// the reference 8 + 5 passes per level plus 80 coarse passes (~184 dispatches
// at 2048^2).  Here one V-cycle is:
//
//   k_mg_down   per level n > 64: a 64x64 tile with a halo of 2*pre+1 cells is
//               staged in shared memory, the pre-smoothing red-black sweeps run
//               there (the valid region shrinks one ring per half-sweep), then
//               the residual and its 2x2 restriction are formed; only the
//               tile's x and the coarse right-hand side go back to HBM;
//   k_mg_bottom one CTA runs every level <= 64 in shared memory: levels >= 32
//               with the whole CTA, levels <= 16 (including the coarse
//               sweeps, 40 by default) with one warp and __syncwarp between
//               half-sweeps;
//   k_mg_up     per level n > 64: prolongation-add of the coarse correction on
//               the tile plus a halo of 2*post, then the post-smoothing sweeps.
//
// The per-cell arithmetic is fs_stencil.cuh, shared with the one-pass-per-
// operation kernels, so the fused cycle reproduces them bit for bit.
//
// Shared-memory layout: the tile region row-major, its rows padded so that a
// tile is staged by one TMA copy per field (cp.async.bulk.tensor.2d,
// completion on an mbarrier); a tile on the periodic edge issues the same
// copy and replaces the zero-filled cells outside the grid by their periodic
// images.  Levels without tensor maps use wrapped 4-byte cp.async copies.
#include <atomic>
#include <string>
#include <utility>

#include "fs_df.cuh"
#include "fs_internal.cuh"
#include "fs_stencil.cuh"
#include "fs_tc.cuh"

namespace fs {

// Fine cells per tile side (even).  The largest levels use 64x64 tiles; the
// smaller levels use 32 or 16 so that they still spread over many CTAs -- a
// level with a handful of CTAs is bound by one CTA's serial latency, not HBM.

__device__ __forceinline__ int wrap_n(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

constexpr int kTileThreads = 256;  // threads of a tile kernel (32 x 8)

// 4-byte asynchronous global -> shared copies (no register round trip, all of
// a thread's copies in flight at once); wait_all before the barrier that
// publishes them.
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"((size_t)__cvta_generic_to_global(gsrc))
               : "memory");
}
// 16-byte form (both addresses 16-byte aligned), L2 only
__device__ __forceinline__ void cp_async16(float* sdst, const float* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"((size_t)__cvta_generic_to_global(gsrc))
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"((size_t)__cvta_generic_to_global(p)));
}

// i in (-n, 2n): one correction wraps it (halo offsets are far below n)
__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ------------------------------------------------------------ tile layout
// A tile kernel works on the R x R region around its T x T tile (halo H),
// row-major in shared memory with pitch W.  Region column 0 sits at box
// column OX = LP - H, so that the box starts LP columns left of the tile, LP
// a multiple of 4: the box's first column is 16-byte aligned in the row and
// one TMA copy of W x R floats (W a multiple of 4) stages a whole field.
template <int T, int H>
struct TileBox {
  static constexpr int R = T + 2 * H;
  static constexpr int LP = (H + 3) & ~3;
  static constexpr int OX = LP - H;
  static constexpr int W = (LP + T + H + 3) & ~3;
  static constexpr int N = W * R;            // floats of one field
  static constexpr int NA = (N + 31) & ~31;  // rounded up to 128 bytes
};

// The coarse block the up kernel's prolongation reads: RC x RC coarse cells
// from (cgi0, cgj0) = ((i0 - H)/2 - 1, (j0 - H)/2 - 1), pitch WC, column 0
// at box column OC (the box again starts on a 16-byte boundary: i0 / 2 is a
// multiple of 8).
template <int T, int H>
struct CoarseBox {
  static constexpr int RC = (T + 2 * H) / 2 + 2;
  static constexpr int LPC = (H / 2 + 1 + 3) & ~3;
  static constexpr int OC = LPC - (H / 2 + 1);
  static constexpr int WC = (OC + RC + 3) & ~3;
  static constexpr int NC = (WC * RC + 31) & ~31;
};

template <int T, int H>
constexpr size_t down_smem_bytes() {
  return 2 * (size_t)TileBox<T, H>::NA * sizeof(float) + 128;
}
template <int T, int H>
constexpr size_t up_smem_bytes() {
  return (2 * (size_t)TileBox<T, H>::NA + CoarseBox<T, H>::NC) * sizeof(float) + 128;
}

// the dynamic shared memory of a tile kernel, from a 128-byte boundary (TMA
// destinations): an offset added to the shared array itself, so that the
// compiler still knows every access is to shared memory
__device__ __forceinline__ float* tile_smem(float* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  return p + (((128u - (a & 127u)) & 127u) >> 2);
}

// wrapped 4-byte copies of the R x R region from (gi0, gj0) of a periodic n x n field
template <int R, int W, int OX>
__device__ __forceinline__ void stage_region(float* dst, const float* __restrict__ src, int gi0, int gj0, int n) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  for (int k = tid; k < R * R; k += nthr) {
    const int lj = k / R, li = k - lj * R;
    cp_async4(&dst[lj * W + OX + li], src + (int64_t)wrap1(gj0 + lj, n) * n + wrap1(gi0 + li, n));
  }
}

// Thread 0 arms the barrier and issues the TMA copies of up to three boxes,
// every thread waits (bounded).  False on every thread if the wait gave up,
// after one more bounded wait for the copies in flight, with *err raised.
struct TmaBox {
  float* dst;
  const CUtensorMap* tm;
  int x, y;
};
__device__ __forceinline__ bool tma_stage_boxes(const TmaBox* b, int count, uint32_t bytes, uint64_t* bar,
                                                int* err) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar, bytes);
    for (int q = 0; q < count; q++) tc::tma_load_2d(b[q].dst, b[q].tm, b[q].x, b[q].y, bar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(bar, 0)) != 0;
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    tc::mbar_wait(bar, 0);
  }
  return ok;
}

// The cells of a TMA box (pitch x rows, origin (bx, by) on an n x n grid)
// that lie outside the grid -- whole rows below / above it, then the columns
// left / right of it in the other rows -- which the copy filled with zeros,
// take their periodic images (one wrap: a tile is at most half the grid and
// the box at most the grid).
struct RingBox {
  float* dst;
  const float* src;
  int pitch, rows, bx, by, n;
};
__device__ __forceinline__ int ring_cells(const RingBox& b) {
  const int cl = max(0, -b.bx), cr = max(0, b.bx + b.pitch - b.n);
  const int rb = max(0, -b.by), rt = max(0, b.by + b.rows - b.n);
  return (rb + rt) * b.pitch + (b.rows - rb - rt) * (cl + cr);
}
// cell k < ring_cells(b): its shared-memory slot and the global value
__device__ __forceinline__ float* ring_cell(const RingBox& b, int k, const float** src) {
  const int cl = max(0, -b.bx), cr = max(0, b.bx + b.pitch - b.n);
  const int rb = max(0, -b.by), rt = max(0, b.by + b.rows - b.n);
  const int nrow = (rb + rt) * b.pitch;
  int r, c;
  if (k < nrow) {
    const int q = k / b.pitch;
    c = k - q * b.pitch;
    r = q < rb ? q : b.rows - rt + (q - rb);
  } else {
    k -= nrow;
    const int nco = cl + cr, q = k / nco, m = k - q * nco;
    r = rb + q;
    c = m < cl ? m : b.pitch - cr + (m - cl);
  }
  *src = b.src + (int64_t)wrap1(b.by + r, b.n) * b.n + wrap1(b.bx + c, b.n);
  return b.dst + r * b.pitch + c;
}

// TMA staging of a tile's boxes where some box crosses the grid's edge: the
// copies are issued, then each thread loads up to RB ring cells into
// registers while they are in flight, and after the (bounded) wait stores
// them over the zero fill; ring cells beyond RB per thread (partial tiles)
// are copied after the wait.  With no ring cell it is tma_stage_boxes.
template <int RB>
__device__ __forceinline__ bool tma_stage_ringed(const TmaBox* b, const RingBox* rg, int count, uint32_t bytes,
                                                 uint64_t* bar, int* err) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar, bytes);
    for (int q = 0; q < count; q++) tc::tma_load_2d(b[q].dst, b[q].tm, b[q].x, b[q].y, bar);
  }
  // the rings of the boxes concatenated (constant indices only: the boxes
  // stay in registers)
  const int c0 = ring_cells(rg[0]), c1 = count > 1 ? ring_cells(rg[1]) : 0, c2 = count > 2 ? ring_cells(rg[2]) : 0;
  const int total = c0 + c1 + c2;
  auto cell = [&](int k, const float** src) -> float* {
    if (k < c0) return ring_cell(rg[0], k, src);
    if (k < c0 + c1) return ring_cell(rg[1], k - c0, src);
    return ring_cell(rg[2], k - c0 - c1, src);
  };
  float rv[RB > 0 ? RB : 1];
  float* rd[RB > 0 ? RB : 1];
#pragma unroll
  for (int u = 0; u < RB; u++) {
    const int k = tid + u * nthr;
    rd[u] = nullptr;
    if (k < total) {
      const float* src;
      rd[u] = cell(k, &src);
      rv[u] = __ldg(src);
    }
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(bar, 0)) != 0;
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    tc::mbar_wait(bar, 0);
    return false;
  }
  if (total > 0) {
#pragma unroll
    for (int u = 0; u < RB; u++)
      if (rd[u]) *rd[u] = rv[u];
    for (int k = tid + RB * nthr; k < total; k += nthr) {
      const float* src;
      float* d = cell(k, &src);
      *d = __ldg(src);
    }
    __syncthreads();
  }
  return true;
}

// One red-black half-sweep of colour c over region cells li, lj in [1, R-2]
// (in place).  Cells whose neighbours are stale give stale values; they lie
// outside the valid region and are never written back.  Each thread walks
// one region column down a chunk of rows, updating every other row: the top
// neighbour of one update (colour 1-c, not written in this half-sweep) is
// the bottom neighbour of the next, so an update loads the cell, its rhs, its
// left and right neighbours and one new vertical neighbour.  Lanes of a warp
// sit in consecutive columns, half of them one row lower; with an even pitch
// the even columns fall on even banks and the odd ones on odd banks.
template <int R, int W, int OX>
__device__ __forceinline__ void rb_half_tile(float* xs, const float* rs, int c, int par0, float h2, float w) {
  constexpr int NI = R - 2;                                 // columns (and rows) swept
  constexpr int NCH = kTileThreads / NI;                    // row chunks
  static_assert(NCH >= 1 && W % 2 == 0, "a tile region of at most 258 columns, even pitch");
  constexpr int CH = ((NI + NCH - 1) / NCH + 1) & ~1;       // rows per chunk, even
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int chunk = tid / NI, m = tid - chunk * NI;
  if (chunk >= NCH) return;
  const int li = 1 + m;
  int lj = 1 + chunk * CH;
  const int lend = min(lj + CH, R - 1);
  lj += (par0 + li + lj + c) & 1;  // first row of colour c in this column
  if (lj >= lend) return;
  float* p = xs + lj * W + OX + li;
  const float* q = rs + lj * W + OX + li;
  float bot = p[-W];
  for (; lj < lend; lj += 2) {
    const float top = p[W];
    *p = gs_update(*p, p[-1], p[1], bot, top, *q, h2, w);
    bot = top;
    p += 2 * W;
    q += 2 * W;
  }
}

// ring cells a thread loads before the TMA wait: the level-0 up kernel of a
// refinement cycle on 64-cell tiles copies its ring after the wait (no
// registers to spare: 62 of the 64 that keep 4 CTAs per SM)
template <int T, bool ACC>
constexpr int ring_regs() {
  return ACC && T == 64 ? 0 : 4;
}

// ------------------------------------------------------------------ down
// H = 2 * pre + 1.  xin == nullptr means the level starts from zero; otherwise
// xin and xout must differ (the halo of a tile is another tile's interior).
// Staging (the up kernel's too), by the level's mode tma: 0 wrapped copies
// everywhere; 1 a TMA copy for the tiles whose box lies inside the grid,
// wrapped copies for the others; 2 a TMA copy for every tile, boxes across
// the grid's edge fixed up (tma_stage_ringed).
template <int T, int H>
__device__ __forceinline__ void mg_down_body(float* smem, const float* __restrict__ rhs,
                                             const float* __restrict__ xin, float* __restrict__ xout,
                                             float* __restrict__ crhs, int n, float h2, int pre, float w,
                                             const CUtensorMap* tm_r, const CUtensorMap* tm_x, int tma,
                                             int* err, bool restrict_only = false) {
  using B = TileBox<T, H>;
  static_assert(H % 2 == 1, "the halo of the down kernel is 2 * pre + 1");
  float* const xs = smem;
  float* const rs = smem + B::NA;
  __shared__ uint64_t bar;
  const int i0 = blockIdx.x * T, j0 = blockIdx.y * T;
  if (restrict_only) {
    // no sweeps from a zero iterate that nothing reads afterwards (the first
    // cycle of a MIXED projection without finest-level sweeps): the residual
    // is the rhs itself (rhs - lap 0 rounds to rhs), restricted straight from
    // global memory by float2 row pairs; no iterate is written
    const int nc = n >> 1, tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    for (int k = tid; k < (T / 2) * (T / 2); k += nthr) {
      const int cj = k / (T / 2), ci = k - cj * (T / 2);
      const int gci = (i0 >> 1) + ci, gcj = (j0 >> 1) + cj;
      if (gci >= nc || gcj >= nc) continue;
      const float* q = rhs + (int64_t)(2 * gcj) * n + 2 * gci;
      const float2 q0 = __ldg(reinterpret_cast<const float2*>(q));
      const float2 q1 = __ldg(reinterpret_cast<const float2*>(q + n));
      crhs[(int64_t)gcj * nc + gci] = restrict4(q0.x, q0.y, q1.x, q1.y);
    }
    return;
  }
  const int gi0 = i0 - H, gj0 = j0 - H;
  const int par0 = (gi0 + gj0) & 1;  // n even: the parity of the wrapped index is the same
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int bx = i0 - B::LP;
  const bool boxed = tma && bx >= 0 && bx + B::W <= n && gj0 >= 0 && gj0 + B::R <= n;
  const bool tile_in = tma && i0 + T <= n && j0 + T <= n;
  if (!xin)
    for (int k = tid; k < B::NA / 4; k += nthr) reinterpret_cast<float4*>(xs)[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (boxed || tma == 2) {
    // the box's x is a multiple of 4 (16 bytes) wherever it lies; a box
    // across the grid's edge (tma == 2) is copied with zero fill and its
    // outer cells replaced by their periodic images
    const TmaBox b[2] = {{rs, tm_r, bx, gj0}, {xs, tm_x, bx, gj0}};
    const uint32_t bytes = (uint32_t)((xin ? 2 : 1) * B::N * sizeof(float));
    if (boxed) {
      if (!tma_stage_boxes(b, xin ? 2 : 1, bytes, &bar, err)) return;
    } else {
      const RingBox rg[2] = {{rs, rhs, B::W, B::R, bx, gj0, n}, {xs, xin, B::W, B::R, bx, gj0, n}};
      if (!tma_stage_ringed<ring_regs<T, false>()>(b, rg, xin ? 2 : 1, bytes, &bar, err)) return;
    }
  } else {
    stage_region<B::R, B::W, B::OX>(rs, rhs, gi0, gj0, n);
    if (xin) stage_region<B::R, B::W, B::OX>(xs, xin, gi0, gj0, n);
    cp_async_wait_all();
    __syncthreads();
  }
  for (int s = 0; s < 2 * pre; s++) {
    rb_half_tile<B::R, B::W, B::OX>(xs, rs, s & 1, par0, h2, w);
    __syncthreads();
  }
  // the tile: region cell (H + x, H + y) is box column LP + x of row H + y
  if (tile_in) {  // inside the grid, n % 4 == 0: float4 rows
    for (int k = tid; k < T * T / 4; k += nthr) {
      const int y = k / (T / 4), x = (k - y * (T / 4)) * 4;
      *reinterpret_cast<float4*>(xout + (int64_t)(j0 + y) * n + i0 + x) =
          *reinterpret_cast<const float4*>(xs + (H + y) * B::W + B::LP + x);
    }
  } else {
    for (int k = tid; k < T * T; k += nthr) {
      const int y = k / T, x = k - y * T;
      const int gi = i0 + x, gj = j0 + y;
      if (gi < n && gj < n) xout[(int64_t)gj * n + gi] = xs[(H + y) * B::W + B::LP + x];
    }
  }
  // residual on each 2x2 block and its restriction (multigrid.js:48-93).  The
  // block at region (H + 2ci, H + 2cj) starts on an even word (LP and W are
  // multiples of 4), so its rows, the rows above and below it and its rhs
  // come as float2 pairs: 10 loads per block instead of 16.
  const int nc = n >> 1;
  const float ih2 = inv_h2(h2);
  for (int k = tid; k < (T / 2) * (T / 2); k += nthr) {
    const int cj = k / (T / 2), ci = k - cj * (T / 2);
    const int off = (H + 2 * cj) * B::W + B::LP + 2 * ci;
    const float* X = xs + off;
    const float* Q = rs + off;
    const float2 x0 = *reinterpret_cast<const float2*>(X);
    const float2 x1 = *reinterpret_cast<const float2*>(X + B::W);
    const float2 xb = *reinterpret_cast<const float2*>(X - B::W);
    const float2 xt = *reinterpret_cast<const float2*>(X + 2 * B::W);
    const float2 q0 = *reinterpret_cast<const float2*>(Q);
    const float2 q1 = *reinterpret_cast<const float2*>(Q + B::W);
    const float r00 = residual_at(x0.x, X[-1], x0.y, xb.x, x1.x, q0.x, ih2);
    const float r10 = residual_at(x0.y, x0.x, X[2], xb.y, x1.y, q0.y, ih2);
    const float r01 = residual_at(x1.x, X[B::W - 1], x1.y, x0.x, xt.x, q1.x, ih2);
    const float r11 = residual_at(x1.y, x1.x, X[B::W + 2], x0.y, xt.y, q1.y, ih2);
    const int gci = (i0 >> 1) + ci, gcj = (j0 >> 1) + cj;
    if (gci < nc && gcj < nc) crhs[(int64_t)gcj * nc + gci] = restrict4(r00, r10, r01, r11);
  }
}

template <int T, int H>
__global__ void __launch_bounds__(256)
    k_mg_down(const float* __restrict__ rhs, const float* __restrict__ xin, float* __restrict__ xout,
              float* __restrict__ crhs, int n, float h2, int pre, float w, const __grid_constant__ CUtensorMap tm_r,
              const __grid_constant__ CUtensorMap tm_x, int tma, int* err, const int* first_cycle, int first_pre,
              int first_x_unused) {
  extern __shared__ float tile_dyn[];
  // the first cycle of a projection may run fewer sweeps on this level
  // (fs_params mg_first_pre, at most pre): first_pre >= 0 applies it, inside
  // a captured loop only while the loop's cycle count is still 0;
  // first_x_unused: that cycle's up kernel on this level runs no sweeps
  // either and does not read the iterate
  const bool first = first_pre >= 0 && (!first_cycle || *first_cycle == 0);
  if (first) pre = first_pre;
  mg_down_body<T, H>(tile_smem(tile_dyn), rhs, xin, xout, crhs, n, h2, pre, w, &tm_r, &tm_x, tma, err,
                     first && pre == 0 && first_x_unused && !xin);
}

// -------------------------------------------------------------------- up
// H = 2 * post.  x += P(coarse) on the region, then the post sweeps.  xin and
// xout must differ: the halo of a tile is another tile's interior.  With ACC
// (level 0 of a MIXED refinement cycle) the tile's correction is added to the
// double-float pressure (ph, pl) in place instead of being written to xout:
// each cell is read and written by its own tile only.
template <int T, int H, bool ACC>
__device__ __forceinline__ void mg_up_body(float* smem, const float* __restrict__ rhs, const float* __restrict__ xin,
                                           float* __restrict__ xout, const float* __restrict__ xc, int n, float h2,
                                           int post, float* __restrict__ ph, float* __restrict__ pl, float w,
                                           const CUtensorMap* tm_r, const CUtensorMap* tm_x,
                                           const CUtensorMap* tm_c, int tma, int* err, bool pfast = false) {
  using B = TileBox<T, H>;
  using C = CoarseBox<T, H>;
  static_assert(T % 16 == 0 && H % 2 == 0, "the up kernel's region starts on an even index");
  float* const xs = smem;
  float* const rs = smem + B::NA;
  float* const cs = smem + 2 * B::NA;
  __shared__ uint64_t bar;
  const int i0 = blockIdx.x * T, j0 = blockIdx.y * T;
  const int gi0 = i0 - H, gj0 = j0 - H;
  const int par0 = (gi0 + gj0) & 1;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int nc = n >> 1;
  // staging: the fine iterate and rhs of the region and the coarse block its
  // prolongation reads.  gi0 is even (T and H are), so fine region column li
  // samples coarse block columns (li + 1) / 2 and (li + 1) / 2 + 1 with weight
  // 1/4 or 3/4 on the second (PROLONG, multigrid.js:99-131: sample at
  // ((i+1/2)/2 - 1/2, (j+1/2)/2 - 1/2)).
  const int cgi0 = (gi0 >> 1) - 1, cgj0 = (gj0 >> 1) - 1;
  const int bx = i0 - B::LP, cbx = cgi0 - C::OC;
  const bool boxed = tma && bx >= 0 && bx + B::W <= n && gj0 >= 0 && gj0 + B::R <= n && cbx >= 0 &&
                     cbx + C::WC <= nc && cgj0 >= 0 && cgj0 + C::RC <= nc;
  const bool tile_in = tma && i0 + T <= n && j0 + T <= n;
  // The tile's double-float pressure, read and written after the sweeps.  A
  // tile inside the grid (n % 4 == 0) loads its hi plane into registers now,
  // PG float4 groups per thread, and prefetches its lo plane into L2; other
  // tiles prefetch both planes (one 128-byte line per thread and array).
  constexpr int G4 = T * T / 4, PG = (G4 + kTileThreads - 1) / kTileThreads;
  float4 hpre[PG];
  if constexpr (ACC) {
    if (tile_in) {
#pragma unroll
      for (int u = 0; u < PG; u++) {
        const int k = tid + u * kTileThreads;
        if (k < G4) {
          const int y = k / (T / 4), x = (k - y * (T / 4)) * 4;
          hpre[u] = *reinterpret_cast<const float4*>(ph + (int64_t)(j0 + y) * n + i0 + x);
        }
      }
    }
    constexpr int LPR = (T + 31) / 32;  // 128-byte lines per tile row
    for (int k = tid; k < T * LPR; k += nthr) {
      const int y = k / LPR, x = (k - y * LPR) * 32;
      const int gi = i0 + x, gj = j0 + y;
      if (gi < n && gj < n) {
        if (!tile_in) prefetch_l2(ph + (int64_t)gj * n + gi);
        prefetch_l2(pl + (int64_t)gj * n + gi);
      }
    }
  }
  // pfast: no sweeps on this level and a zero iterate from the down kernel (the
  // first cycle of a MIXED projection whose finest-level sweeps are skipped on
  // both sides): the correction is the prolongation alone and the rhs is not
  // read, so only the coarse block is staged and the prolongation writes
  // instead of adding (0 + P = P, and a -0 from P gives the same pressure sum
  // as +0).
  if (boxed || tma == 2) {
    // x of every box is a multiple of 4 (16 bytes) wherever it lies; boxes
    // across the grid's edge (tma == 2) are copied with zero fill and their
    // outer cells replaced by their periodic images
    const TmaBox b[3] = {{cs, tm_c, cbx, cgj0}, {xs, tm_x, bx, gj0}, {rs, tm_r, bx, gj0}};
    const int nb = pfast ? 1 : 3;
    const uint32_t bytes = (uint32_t)(((pfast ? 0 : 2 * B::N) + C::WC * C::RC) * sizeof(float));
    if (boxed) {
      if (!tma_stage_boxes(b, nb, bytes, &bar, err)) return;
    } else {
      const RingBox rg[3] = {{cs, xc, C::WC, C::RC, cbx, cgj0, nc}, {xs, xin, B::W, B::R, bx, gj0, n},
                             {rs, rhs, B::W, B::R, bx, gj0, n}};
      if (!tma_stage_ringed<ring_regs<T, ACC>()>(b, rg, nb, bytes, &bar, err)) return;
    }
  } else {
    for (int k = tid; k < C::RC * C::RC; k += nthr) {
      const int lj = k / C::RC, li = k - lj * C::RC;
      cp_async4(&cs[lj * C::WC + C::OC + li], xc + (int64_t)wrap1(cgj0 + lj, nc) * nc + wrap1(cgi0 + li, nc));
    }
    if (!pfast) {
      stage_region<B::R, B::W, B::OX>(xs, xin, gi0, gj0, n);
      stage_region<B::R, B::W, B::OX>(rs, rhs, gi0, gj0, n);
    }
    cp_async_wait_all();
    __syncthreads();
  }
  // prolongation-add by even-aligned 2x2 fine blocks: block (d, e) holds
  // region rows 2d, 2d + 1 and columns 2e, 2e + 1.  Fine column 2e
  // interpolates coarse block columns e, e + 1 (weight 3/4 on e + 1), column
  // 2e + 1 columns e + 1, e + 2 (weight 1/4 on e + 2); likewise the rows.  A
  // thread walks one column of blocks down a chunk of block rows and keeps
  // the two coarse rows it shares with the next block in registers: three
  // coarse loads and two float2 read-modify-writes per block (OX and W are
  // even, so each block row is one aligned float2).
  {
    constexpr int NBC = B::R / 2;                // blocks per region row and column
    constexpr int NCK = kTileThreads / NBC;      // chunks of block rows
    constexpr int CL = (NBC + NCK - 1) / NCK;    // block rows per chunk
    static_assert(NCK >= 1 && B::OX % 2 == 0 && B::W % 2 == 0, "float2 blocks of a region of <= 512 columns");
    const int chunk = tid / NBC, e = tid - chunk * NBC;
    int d = chunk * CL;
    const int dend = min(d + CL, NBC);
    if (chunk < NCK && d < dend) {
      const float* c = cs + d * C::WC + C::OC + e;
      float a0 = c[0], a1 = c[1], a2 = c[2];
      float b0 = c[C::WC], b1 = c[C::WC + 1], b2 = c[C::WC + 2];
      float2* o = reinterpret_cast<float2*>(xs + 2 * d * B::W + B::OX + 2 * e);
      for (; d < dend; d++) {
        c += C::WC;
        const float n0 = c[C::WC], n1 = c[C::WC + 1], n2 = c[C::WC + 2];
        float2 top = pfast ? make_float2(0.f, 0.f) : o[0], bot = pfast ? make_float2(0.f, 0.f) : o[B::W / 2];
        const float pt0 = prolong_val(a0, a1, b0, b1, 0.75f, 0.75f), pt1 = prolong_val(a1, a2, b1, b2, 0.25f, 0.75f);
        const float pb0 = prolong_val(b0, b1, n0, n1, 0.75f, 0.25f), pb1 = prolong_val(b1, b2, n1, n2, 0.25f, 0.25f);
        top.x = pfast ? pt0 : __fadd_rn(top.x, pt0);
        top.y = pfast ? pt1 : __fadd_rn(top.y, pt1);
        bot.x = pfast ? pb0 : __fadd_rn(bot.x, pb0);
        bot.y = pfast ? pb1 : __fadd_rn(bot.y, pb1);
        o[0] = top;
        o[B::W / 2] = bot;
        a0 = b0, a1 = b1, a2 = b2;
        b0 = n0, b1 = n1, b2 = n2;
        o += B::W;  // two fine rows
      }
    }
  }
  __syncthreads();
  for (int s = 0; s < 2 * post; s++) {
    rb_half_tile<B::R, B::W, B::OX>(xs, rs, s & 1, par0, h2, w);
    __syncthreads();
  }
  // the tile: region cell (H + x, H + y) is box column LP + x of row H + y
  if constexpr (ACC) {
    if (tile_in) {
      // float4 groups: the hi plane loaded at the start, every lo load of the
      // thread in flight at once
      float4 lv[PG];
#pragma unroll
      for (int u = 0; u < PG; u++) {
        const int k = tid + u * kTileThreads;
        if (k < G4) {
          const int y = k / (T / 4), x = (k - y * (T / 4)) * 4;
          lv[u] = *reinterpret_cast<const float4*>(pl + (int64_t)(j0 + y) * n + i0 + x);
        }
      }
#pragma unroll
      for (int u = 0; u < PG; u++) {
        const int k = tid + u * kTileThreads;
        if (k < G4) {
          const int y = k / (T / 4), x = (k - y * (T / 4)) * 4;
          const int64_t g = (int64_t)(j0 + y) * n + i0 + x;
          const float4 hv = hpre[u], ev = *reinterpret_cast<const float4*>(xs + (H + y) * B::W + B::LP + x);
          const df p0 = df_add_f(df{hv.x, lv[u].x}, ev.x), p1 = df_add_f(df{hv.y, lv[u].y}, ev.y);
          const df p2 = df_add_f(df{hv.z, lv[u].z}, ev.z), p3 = df_add_f(df{hv.w, lv[u].w}, ev.w);
          *reinterpret_cast<float4*>(ph + g) = make_float4(p0.hi, p1.hi, p2.hi, p3.hi);
          *reinterpret_cast<float4*>(pl + g) = make_float4(p0.lo, p1.lo, p2.lo, p3.lo);
        }
      }
    } else {
      // four cells' double-float pressure loads in flight per thread
      constexpr int V = 4;
      for (int k0 = tid; k0 < T * T; k0 += V * nthr) {
        float hv[V], lv[V], ev[V];
        int64_t gv[V];
#pragma unroll
        for (int u = 0; u < V; u++) {
          const int k = k0 + u * nthr;
          gv[u] = -1;
          if (k < T * T) {
            const int y = k / T, x = k - y * T;
            const int gi = i0 + x, gj = j0 + y;
            if (gi < n && gj < n) {
              gv[u] = (int64_t)gj * n + gi;
              hv[u] = ph[gv[u]];
              lv[u] = pl[gv[u]];
              ev[u] = xs[(H + y) * B::W + B::LP + x];
            }
          }
        }
#pragma unroll
        for (int u = 0; u < V; u++)
          if (gv[u] >= 0) {
            const df p = df_add_f(df{hv[u], lv[u]}, ev[u]);
            ph[gv[u]] = p.hi;
            pl[gv[u]] = p.lo;
          }
      }
    }
  } else if (tile_in) {
    for (int k = tid; k < T * T / 4; k += nthr) {
      const int y = k / (T / 4), x = (k - y * (T / 4)) * 4;
      *reinterpret_cast<float4*>(xout + (int64_t)(j0 + y) * n + i0 + x) =
          *reinterpret_cast<const float4*>(xs + (H + y) * B::W + B::LP + x);
    }
  } else {
    for (int k = tid; k < T * T; k += nthr) {
      const int y = k / T, x = k - y * T;
      const int gi = i0 + x, gj = j0 + y;
      if (gi < n && gj < n) xout[(int64_t)gj * n + gi] = xs[(H + y) * B::W + B::LP + x];
    }
  }
}

template <int T, int H, bool ACC>
__global__ void __launch_bounds__(256)
    k_mg_up(const float* __restrict__ rhs, const float* __restrict__ xin, float* __restrict__ xout,
            const float* __restrict__ xc, int n, float h2, int post, float* __restrict__ ph,
            float* __restrict__ pl, float w, const __grid_constant__ CUtensorMap tm_r,
            const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_c, int tma, int* err,
            const int* first_cycle, int first_post, int first_x_zero) {
  extern __shared__ float tile_dyn[];
  // as k_mg_down; first_x_zero: that cycle's down kernel on this level ran no
  // sweeps, so the iterate is zero
  const bool first = first_post >= 0 && (!first_cycle || *first_cycle == 0);
  if (first) post = first_post;
  const bool pfast = ACC && first && post == 0 && first_x_zero;
  mg_up_body<T, H, ACC>(tile_smem(tile_dyn), rhs, xin, xout, xc, n, h2, post, ph, pl, w, &tm_r, &tm_x, &tm_c, tma,
                        err, pfast);
}

// ---------------------------------------------------------------- bottom
// Levels 0..count-1 of the bottom (each n <= 64), all in shared memory.  Per
// level: x, rhs and, for odd n, a ping-pong partner (red-black on an odd
// periodic grid reads cells of its own colour across the wrap, so the
// reference's ping-pong result is kept).
struct BottomLevels {
  int count;
  int n[8];
  float h2[8];
  int off_x[8], off_x2[8], off_r[8];  // float offsets into dynamic smem (-1: none)
  float w;                            // relaxation factor of every sweep
};

// A thread group: the whole CTA, or warp 0 alone (levels <= 16).
struct Group {
  int tid, nthr;
  bool warp;
  __device__ __forceinline__ void sync() const {
    if (warp) __syncwarp();
    else __syncthreads();
  }
};

__device__ __forceinline__ void bottom_smooth(float* sm, const BottomLevels& L, int l, int sweeps, Group G) {
  const int n = L.n[l];
  const float h2 = L.h2[l];
  float* x = sm + L.off_x[l];
  float* x2 = (n & 1) ? sm + L.off_x2[l] : nullptr;
  const float* r = sm + L.off_r[l];
  for (int s = 0; s < 2 * sweeps; s++) {
    const int c = s & 1;
    if (!(n & 1)) {
      for (int k = G.tid; k < n * n; k += G.nthr) {
        int j = k / n, i = k - j * n;
        if (((i + j) & 1) != c) continue;
        int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
        int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
        x[k] = gs_update(x[k], x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[k], h2, L.w);
      }
    } else {
      for (int k = G.tid; k < n * n; k += G.nthr) {
        int j = k / n, i = k - j * n;
        float cur = x[k];
        if (((i + j) & 1) != c) { x2[k] = cur; continue; }
        int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
        int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
        x2[k] = gs_update(cur, x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[k], h2, L.w);
      }
      G.sync();
      float* t = x; x = x2; x2 = t;  // two swaps per sweep: x is back in off_x at the end
    }
    G.sync();
  }
}

__device__ __forceinline__ void bottom_restrict(float* sm, const BottomLevels& L, int l, Group G) {
  const int n = L.n[l], nc = L.n[l + 1];
  const float ih2 = inv_h2(L.h2[l]);
  const float* x = sm + L.off_x[l];
  const float* r = sm + L.off_r[l];
  float* cr = sm + L.off_r[l + 1];
  float* cx = sm + L.off_x[l + 1];
  for (int k = G.tid; k < nc * nc; k += G.nthr) {
    int cj = k / nc, ci = k - cj * nc;
    float r4[4];
    for (int q = 0; q < 4; q++) {
      int i = 2 * ci + (q & 1), j = 2 * cj + (q >> 1);
      int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
      int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
      r4[q] = residual_at(x[j * n + i], x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[j * n + i], ih2);
    }
    cr[k] = restrict4(r4[0], r4[1], r4[2], r4[3]);
    cx[k] = 0.f;
  }
  G.sync();
}

__device__ __forceinline__ void bottom_prolong(float* sm, const BottomLevels& L, int l, Group G) {
  const int n = L.n[l], nc = L.n[l + 1];
  float* x = sm + L.off_x[l];
  const float* c = sm + L.off_x[l + 1];
  for (int k = G.tid; k < n * n; k += G.nthr) {
    int j = k / n, i = k - j * n;
    int ci0 = (i & 1) ? (i >> 1) : (i >> 1) - 1;
    int cj0 = (j & 1) ? (j >> 1) : (j >> 1) - 1;
    float fx = (i & 1) ? 0.25f : 0.75f, fy = (j & 1) ? 0.25f : 0.75f;
    int x0 = ci0 < 0 ? ci0 + nc : ci0, x1 = ci0 + 1 >= nc ? ci0 + 1 - nc : ci0 + 1;
    int y0 = cj0 < 0 ? cj0 + nc : cj0, y1 = cj0 + 1 >= nc ? cj0 + 1 - nc : cj0 + 1;
    x[k] = __fadd_rn(x[k], prolong_val(c[y0 * nc + x0], c[y0 * nc + x1], c[y1 * nc + x0], c[y1 * nc + x1], fx, fy));
  }
  G.sync();
}

__device__ __forceinline__ void mg_bottom_body(const float* __restrict__ rhs_top, float* __restrict__ x_top,
                                               int has_x, const BottomLevels& L, int pre, int post, int coarse,
                                               float* __restrict__ acc_h, float* __restrict__ acc_l) {
  extern __shared__ float sm[];
  const int tid = threadIdx.x;
  const Group CTA{tid, (int)blockDim.x, false};
  const Group W0{tid, 32, true};
  {
    // the top level's rhs (and iterate) by asynchronous copies, all in flight at once
    const int n = L.n[0];
    for (int k = tid; k < n * n; k += CTA.nthr) {
      cp_async4(&sm[L.off_r[0] + k], rhs_top + k);
      if (has_x) cp_async4(&sm[L.off_x[0] + k], x_top + k);
      else sm[L.off_x[0] + k] = 0.f;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // first level handled by warp 0 alone
  int ls = 0;
  while (ls < L.count && L.n[ls] > 16) ls++;
  if (ls >= L.count) {
    // every bottom level is a CTA level
    for (int l = 0; l < L.count - 1; l++) {
      bottom_smooth(sm, L, l, pre, CTA);
      bottom_restrict(sm, L, l, CTA);
    }
    bottom_smooth(sm, L, L.count - 1, coarse, CTA);
    for (int l = L.count - 2; l >= 0; l--) {
      bottom_prolong(sm, L, l, CTA);
      bottom_smooth(sm, L, l, post, CTA);
    }
  } else {
    for (int l = 0; l < ls; l++) {
      bottom_smooth(sm, L, l, pre, CTA);
      bottom_restrict(sm, L, l, CTA);
    }
    if (tid < 32) {
      for (int l = ls; l < L.count - 1; l++) {
        bottom_smooth(sm, L, l, pre, W0);
        bottom_restrict(sm, L, l, W0);
      }
      bottom_smooth(sm, L, L.count - 1, coarse, W0);
      for (int l = L.count - 2; l >= ls; l--) {
        bottom_prolong(sm, L, l, W0);
        bottom_smooth(sm, L, l, post, W0);
      }
    }
    __syncthreads();
    for (int l = ls - 1; l >= 0; l--) {
      bottom_prolong(sm, L, l, CTA);
      bottom_smooth(sm, L, l, post, CTA);
    }
  }
  {
    const int n = L.n[0];
    for (int k = tid; k < n * n; k += CTA.nthr) {
      float e = sm[L.off_x[0] + k];
      if (acc_h) {  // the whole hierarchy fits here: add the correction to the pressure
        df p = df_add_f(df{acc_h[k], acc_l[k]}, e);
        acc_h[k] = p.hi;
        acc_l[k] = p.lo;
      } else {
        x_top[k] = e;
      }
    }
  }
}

__global__ void __launch_bounds__(1024) k_mg_bottom(const float* __restrict__ rhs_top, float* __restrict__ x_top,
                                                    int has_x, BottomLevels L, int pre, int post, int coarse,
                                                    float* __restrict__ acc_h, float* __restrict__ acc_l) {
  mg_bottom_body(rhs_top, x_top, has_x, L, pre, post, coarse, acc_h, acc_l);
}

// ------------------------------------------------ bottom, compile-time chains
// The common cases: the bottom levels are N0, N0/2, ..., NMIN with every size
// but the coarsest even and N0 <= 64 -- the power-of-two chains down to 8 and
// the 48 -> 24 -> 12 chain of grids of 3 * 2^k cells -- all sizes known at
// compile time, so cell indices use constant divisors.  Levels >= 32 run on
// the whole CTA (256 threads), levels <= 16 -- including the coarse sweeps --
// on warp 0 alone.  Same arithmetic (fs_stencil.cuh) and order as the generic
// kernel above.
struct BottomH2 {
  float h2[4];
  float w;  // relaxation factor of every sweep
};

template <int N>
constexpr int ilog2() {
  return N <= 1 ? 0 : 1 + ilog2<N / 2>();
}
// levels and floats of the chain N0, N0/2, ..., NMIN
template <int N0, int NMIN>
constexpr int chain_levels() {
  return N0 == NMIN ? 1 : 1 + chain_levels<N0 / 2, NMIN>();
}
template <int N0, int NMIN>
constexpr int chain_floats() {
  return N0 == NMIN ? N0 * N0 : N0 * N0 + chain_floats<N0 / 2, NMIN>();
}

constexpr int kBottomThreads = 256;  // threads of the bottom-chain kernels

template <int N, bool WARP>
__device__ __forceinline__ void p2_sync() {
  if (WARP) __syncwarp();
  else __syncthreads();
}

// The chain's loops run a compile-time number of cells per thread (the CTA
// has kBottomThreads threads, warp 0 has 32), fully unrolled, every result of
// a phase computed before any is stored: the cells a phase writes are not
// read in that phase (a colour's cells read only the other colour; restrict
// and prolong write the other level's array, or the cell itself), so the
// loads of a thread's cells are in flight together instead of waiting on the
// stores of the cells before them.  The levels are latency-bound, one phase
// between two barriers after another.
template <int N, bool WARP>
__device__ __forceinline__ void p2_smooth(float* x, const float* r, float h2, int sweeps, float w) {
  constexpr int HALF = N / 2, NT = WARP ? 32 : kBottomThreads;
  constexpr int CELLS = N * HALF, PER = (CELLS + NT - 1) / NT;
  const int tid = WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  // When the threads cover whole rows of a colour (NT a multiple of N/2)
  // and step an even number of rows, a thread's cells share their column and
  // its neighbours' offsets: rows j0, j0 + RS, ...; only the first and last
  // rows of the level wrap vertically.
  constexpr bool ROWS = NT % HALF == 0 && (NT / HALF) % 2 == 0 && CELLS % NT == 0;
  if constexpr (ROWS) {
    constexpr int RS = NT / HALF;
    const int j0 = tid / HALF, m = tid - j0 * HALF;
    for (int s = 0; s < 2 * sweeps; s++) {
      const int i = 2 * m + ((j0 + (s & 1)) & 1);
      const int dl = i == 0 ? N - 1 : -1, dr = i + 1 == N ? 1 - N : 1;
      float nv[PER];
#pragma unroll
      for (int u = 0; u < PER; u++) {
        const int j = j0 + u * RS, k = j * N + i;
        const int db = j == 0 ? (N - 1) * N : -N, dt = j + 1 == N ? -(N - 1) * N : N;
        nv[u] = gs_update(x[k], x[k + dl], x[k + dr], x[k + db], x[k + dt], r[k], h2, w);
      }
#pragma unroll
      for (int u = 0; u < PER; u++) x[(j0 + u * RS) * N + i] = nv[u];
      p2_sync<N, WARP>();
    }
  } else {
    for (int s = 0; s < 2 * sweeps; s++) {
      const int c = s & 1;
      float nv[PER];
      int kk[PER];
#pragma unroll
      for (int u = 0; u < PER; u++) {
        const int idx = tid + u * NT;
        kk[u] = -1;
        if (CELLS % NT == 0 || idx < CELLS) {
          const int j = idx / HALF, m = idx - j * HALF;
          const int i = 2 * m + ((j + c) & 1);
          const int row = j * N, k = row + i;
          const int rm = (j == 0 ? N - 1 : j - 1) * N, rp = (j + 1 == N ? 0 : j + 1) * N;
          const int im = i == 0 ? N - 1 : i - 1, ip = i + 1 == N ? 0 : i + 1;
          kk[u] = k;
          nv[u] = gs_update(x[k], x[row + im], x[row + ip], x[rm + i], x[rp + i], r[k], h2, w);
        }
      }
#pragma unroll
      for (int u = 0; u < PER; u++)
        if (CELLS % NT == 0 || kk[u] >= 0) x[kk[u]] = nv[u];
      p2_sync<N, WARP>();
    }
  }
}

// residual of level N restricted into (cr, cx = 0) of level N/2
template <int N, bool WARP>
__device__ __forceinline__ void p2_restrict(const float* x, const float* r, float h2, float* cr, float* cx) {
  constexpr int NC = N / 2, NT = WARP ? 32 : kBottomThreads, PER = (NC * NC + NT - 1) / NT;
  const int tid = WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  const float ih2 = inv_h2(h2);
  float rv[PER];
  // threads covering whole coarse rows: a thread's blocks share their two
  // fine columns and the columns' neighbour offsets; only the level's first
  // and last fine rows wrap
  constexpr bool ROWS = NT % NC == 0 && (NC * NC) % NT == 0;
  if constexpr (ROWS) {
    constexpr int RS = NT / NC;
    const int cj0 = tid / NC, ci = tid - cj0 * NC;
    const int i0 = 2 * ci;
    const int dl0 = i0 == 0 ? N - 1 : -1, dr1 = i0 + 2 == N ? 1 - N : 1;  // left of column i0, right of i0 + 1
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int j = 2 * (cj0 + u * RS), k0 = j * N + i0, k1 = k0 + N;
      const int db = j == 0 ? (N - 1) * N : -N, dt = j + 2 == N ? -(N - 1) * N : N;  // below row j, above row j + 1
      const float r00 = residual_at(x[k0], x[k0 + dl0], x[k0 + 1], x[k0 + db], x[k1], r[k0], ih2);
      const float r10 = residual_at(x[k0 + 1], x[k0], x[k0 + 1 + dr1], x[k0 + 1 + db], x[k1 + 1], r[k0 + 1], ih2);
      const float r01 = residual_at(x[k1], x[k1 + dl0], x[k1 + 1], x[k0], x[k1 + dt], r[k1], ih2);
      const float r11 = residual_at(x[k1 + 1], x[k1], x[k1 + 1 + dr1], x[k0 + 1], x[k1 + 1 + dt], r[k1 + 1], ih2);
      rv[u] = restrict4(r00, r10, r01, r11);
    }
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int k = (cj0 + u * RS) * NC + ci;
      cr[k] = rv[u];
      cx[k] = 0.f;
    }
  } else {
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int k = tid + u * NT;
      if ((NC * NC) % NT != 0 && k >= NC * NC) break;
      const int cj = k / NC, ci = k - cj * NC;
      float r4[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int i = 2 * ci + (q & 1), j = 2 * cj + (q >> 1);
        const int row = j * N;
        const int rm = (j == 0 ? N - 1 : j - 1) * N, rp = (j + 1 == N ? 0 : j + 1) * N;
        const int im = i == 0 ? N - 1 : i - 1, ip = i + 1 == N ? 0 : i + 1;
        r4[q] = residual_at(x[row + i], x[row + im], x[row + ip], x[rm + i], x[rp + i], r[row + i], ih2);
      }
      rv[u] = restrict4(r4[0], r4[1], r4[2], r4[3]);
    }
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int k = tid + u * NT;
      if ((NC * NC) % NT != 0 && k >= NC * NC) break;
      cr[k] = rv[u];
      cx[k] = 0.f;
    }
  }
  p2_sync<N, WARP>();
}

// x (level N) += bilinear prolongation of c (level N/2)
template <int N, bool WARP>
__device__ __forceinline__ void p2_prolong(float* x, const float* c) {
  constexpr int NC = N / 2, NT = WARP ? 32 : kBottomThreads, PER = (N * N + NT - 1) / NT;
  const int tid = WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  float pv[PER];
  // threads covering whole rows with an even row step: a thread's cells share
  // their column, its coarse columns and both weights; only the first and
  // last rows wrap to the other edge of the coarse level
  constexpr bool ROWS = NT % N == 0 && (NT / N) % 2 == 0 && (N * N) % NT == 0;
  if constexpr (ROWS) {
    constexpr int RS = NT / N;
    const int j0 = tid / N, i = tid - j0 * N;
    const int ci0 = (i & 1) ? (i >> 1) : (i >> 1) - 1;
    const float fx = (i & 1) ? 0.25f : 0.75f, fy = (j0 & 1) ? 0.25f : 0.75f;
    const int x0 = ci0 < 0 ? ci0 + NC : ci0, x1 = ci0 + 1 >= NC ? ci0 + 1 - NC : ci0 + 1;
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int j = j0 + u * RS, k = j * N + i;
      const int cj0 = (j & 1) ? (j >> 1) : (j >> 1) - 1;
      const int y0 = (cj0 < 0 ? cj0 + NC : cj0) * NC, y1 = (cj0 + 1 >= NC ? cj0 + 1 - NC : cj0 + 1) * NC;
      pv[u] = __fadd_rn(x[k], prolong_val(c[y0 + x0], c[y0 + x1], c[y1 + x0], c[y1 + x1], fx, fy));
    }
#pragma unroll
    for (int u = 0; u < PER; u++) x[(j0 + u * RS) * N + i] = pv[u];
  } else {
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int k = tid + u * NT;
      if ((N * N) % NT != 0 && k >= N * N) break;
      const int j = k / N, i = k - j * N;
      const int ci0 = (i & 1) ? (i >> 1) : (i >> 1) - 1;
      const int cj0 = (j & 1) ? (j >> 1) : (j >> 1) - 1;
      const float fx = (i & 1) ? 0.25f : 0.75f, fy = (j & 1) ? 0.25f : 0.75f;
      const int x0 = ci0 < 0 ? ci0 + NC : ci0, x1 = ci0 + 1 >= NC ? ci0 + 1 - NC : ci0 + 1;
      const int y0 = (cj0 < 0 ? cj0 + NC : cj0) * NC, y1 = (cj0 + 1 >= NC ? cj0 + 1 - NC : cj0 + 1) * NC;
      pv[u] = __fadd_rn(x[k], prolong_val(c[y0 + x0], c[y0 + x1], c[y1 + x0], c[y1 + x1], fx, fy));
    }
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int k = tid + u * NT;
      if ((N * N) % NT != 0 && k >= N * N) break;
      x[k] = pv[u];
    }
  }
  p2_sync<N, WARP>();
}

// sub-cycle from level N (chain level LVL, at float offset OFF of the chain's
// x and rhs arrays) down to NMIN and back; levels <= 16 are called by warp 0
// only.  Every level's arrays are the shared arrays plus a compile-time
// offset, so all accesses compile as shared-memory accesses.
template <int N, int NMIN, int LVL, int OFF>
__device__ __forceinline__ void p2_cycle(float* sx, float* sr, const BottomH2& H, int pre, int post, int coarse) {
  constexpr bool W = N <= 16;
  float* const x = sx + OFF;
  float* const r = sr + OFF;
  if constexpr (N == NMIN) {
    p2_smooth<N, W>(x, r, H.h2[LVL], coarse, H.w);
  } else {
    static_assert(N % 2 == 0, "every level above the coarsest is even");
    constexpr int OFFC = OFF + N * N;
    p2_smooth<N, W>(x, r, H.h2[LVL], pre, H.w);
    p2_restrict<N, W>(x, r, H.h2[LVL], sr + OFFC, sx + OFFC);
    if constexpr (!W && N / 2 <= 16) {
      if (threadIdx.x < 32) p2_cycle<N / 2, NMIN, LVL + 1, OFFC>(sx, sr, H, pre, post, coarse);
      __syncthreads();
    } else {
      p2_cycle<N / 2, NMIN, LVL + 1, OFFC>(sx, sr, H, pre, post, coarse);
    }
    p2_prolong<N, W>(x, sx + OFFC);
    p2_smooth<N, W>(x, r, H.h2[LVL], post, H.w);
  }
}

template <int N0, int NMIN>
__device__ __forceinline__ void mg_bottom_chain_body(const float* __restrict__ rhs_top, float* __restrict__ x_top,
                                                     int has_x, const BottomH2& H, int pre, int post, int coarse,
                                                     float* __restrict__ acc_h, float* __restrict__ acc_l) {
  constexpr int L = chain_levels<N0, NMIN>();
  constexpr int SZ = chain_floats<N0, NMIN>();
  static_assert(L <= 4 && NMIN % 2 == 0, "chains of at most four even levels");
  // the chain's levels one after another, level 0 first
  __shared__ __align__(16) float sx[SZ];
  __shared__ __align__(16) float sr[SZ];
  const int tid = threadIdx.x;
  // level 0's rhs (and iterate): 16-byte asynchronous copies, all in flight at
  // once (N0 is even, so N0^2 is a multiple of 4; the level arrays are
  // cudaMalloc'd, 256-byte aligned)
  static_assert((N0 * N0) % 4 == 0, "whole 16-byte groups");
  for (int k = tid; k < N0 * N0 / 4; k += blockDim.x) {
    cp_async16(sr + 4 * k, rhs_top + 4 * k);
    if (has_x) cp_async16(sx + 4 * k, x_top + 4 * k);
    else reinterpret_cast<float4*>(sx)[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  cp_async_wait_all();
  __syncthreads();
  if constexpr (N0 <= 16) {
    if (tid < 32) p2_cycle<N0, NMIN, 0, 0>(sx, sr, H, pre, post, coarse);
    __syncthreads();
  } else {
    p2_cycle<N0, NMIN, 0, 0>(sx, sr, H, pre, post, coarse);
  }
  for (int k = tid; k < N0 * N0; k += blockDim.x) {
    float e = sx[k];
    if (acc_h) {
      df p = df_add_f(df{acc_h[k], acc_l[k]}, e);
      acc_h[k] = p.hi;
      acc_l[k] = p.lo;
    } else {
      x_top[k] = e;
    }
  }
}

template <int N0, int NMIN>
__global__ void __launch_bounds__(kBottomThreads) k_mg_bottom_chain(const float* __restrict__ rhs_top,
                                                         float* __restrict__ x_top, int has_x, BottomH2 H, int pre,
                                                         int post, int coarse, float* __restrict__ acc_h,
                                                         float* __restrict__ acc_l) {
  mg_bottom_chain_body<N0, NMIN>(rhs_top, x_top, has_x, H, pre, post, coarse, acc_h, acc_l);
}

// ------------------------------------------------- batched (one size class)
// The members of a batch with the same grid and multigrid settings run each
// kernel of their refinement cycles as one launch, member = blockIdx.z, with
// their pointers in a table passed by value among the kernel parameters.  A
// member whose tolerance loop has ended (the per-member condition the
// class-wide loop kernel keeps in its DevState) leaves the launch at once, so
// every member runs exactly the cycles it would run alone.
__device__ __forceinline__ bool member_active(const DevState* st, int max_cycles) {
  return !st->converged && !st->nonfinite && st->cycles < max_cycles;
}

// The tile kernels' tables carry each member's TMA tensor maps (tma = 0:
// that member's tiles stage with wrapped copies); the tables are
// __grid_constant__ parameters, so the maps are read in place.  The maps sit
// in their own array (a CUtensorMap is 128-byte aligned): the up table is
// 64 x (3 x 128 + 64) bytes, within the 32,764 bytes of kernel parameters.
struct DownTab {
  CUtensorMap tm[kClassMax];  // rhs
  struct {
    const float* rhs;
    float* xout;
    float* crhs;
    DevState* st;  // loop state; its async_err is the member's TMA error flag
    int tma;
  } m[kClassMax];
};
struct UpTab {
  CUtensorMap tm[kClassMax][3];  // rhs, fine iterate, coarse iterate
  struct {
    const float* rhs;
    const float* xin;
    float* xout;
    const float* xc;
    float* ph;
    float* pl;
    DevState* st;  // loop state; its async_err is the member's TMA error flag
    int tma;
  } m[kClassMax];
};
static_assert(sizeof(UpTab) + 64 <= 32764, "kernel parameter limit");
struct BottomTab {
  struct {
    const float* rhs;
    float* x;
    float* acc_h;
    float* acc_l;
    const DevState* st;
  } m[kClassMax];
};

template <int T, int H>
__global__ void __launch_bounds__(256) k_mg_down_class(const __grid_constant__ DownTab tab, int n, float h2,
                                                       int pre, float w, int max_cycles) {
  extern __shared__ float tile_dyn[];
  const auto& a = tab.m[blockIdx.z];
  if (!member_active(a.st, max_cycles)) return;
  mg_down_body<T, H>(tile_smem(tile_dyn), a.rhs, nullptr, a.xout, a.crhs, n, h2, pre, w, &tab.tm[blockIdx.z],
                     nullptr, a.tma, &a.st->async_err);
}

template <int T, int H, bool ACC>
__global__ void __launch_bounds__(256) k_mg_up_class(const __grid_constant__ UpTab tab, int n, float h2, int post,
                                                     float w, int max_cycles) {
  extern __shared__ float tile_dyn[];
  const auto& a = tab.m[blockIdx.z];
  if (!member_active(a.st, max_cycles)) return;
  const CUtensorMap* tm = tab.tm[blockIdx.z];
  mg_up_body<T, H, ACC>(tile_smem(tile_dyn), a.rhs, a.xin, a.xout, a.xc, n, h2, post, a.ph, a.pl, w, &tm[0], &tm[1],
                        &tm[2], a.tma, &a.st->async_err);
}

template <int N0, int NMIN>
__global__ void __launch_bounds__(kBottomThreads) k_mg_bottom_chain_class(const BottomTab tab, BottomH2 H, int pre, int post,
                                                               int coarse, int max_cycles) {
  const auto& a = tab.m[blockIdx.z];
  if (!member_active(a.st, max_cycles)) return;
  mg_bottom_chain_body<N0, NMIN>(a.rhs, a.x, 0, H, pre, post, coarse, a.acc_h, a.acc_l);
}

__global__ void __launch_bounds__(1024) k_mg_bottom_class(const BottomTab tab, BottomLevels L, int pre, int post,
                                                          int coarse, int max_cycles) {
  const auto& a = tab.m[blockIdx.z];
  if (!member_active(a.st, max_cycles)) return;
  mg_bottom_body(a.rhs, a.x, 0, L, pre, post, coarse, a.acc_h, a.acc_l);
}

// ------------------------------------------------------------------ host
static const dim3 kTileBlock(32, kTileThreads / 32);

// tile side for a level of n cells: 64 where that gives >= 1024 CTAs, else 32
// where that gives >= 256, else 16 (measured at 2048^2: the 1024^2 level runs
// faster as 1024 CTAs of 32 than as 256 of 64, the 512^2 level as 256 of 32
// than as 1024 of 16)
static int tile_for(int n) {
  const int c64 = (n + 63) / 64, c32 = (n + 31) / 32;
  if (c64 * c64 >= 1024) return 64;
  if (c32 * c32 >= 256) return 32;
  return 16;
}

// A side T serves a level of n cells only if T <= n / 2 (16 always: tile
// levels have n > 64).  Then one wrap covers a tile's halo (T + H - 1 < n) and
// its coarse block, which the wrapped staging relies on.
static bool tile_fits(int t, int n) { return t == 16 || 2 * t <= n; }

int mg_tile(const Solver* s, int l) {
  const int n = s->lev[l].n;
  if (l >= 0 && l < 16 && s->tile_level[l] && tile_fits(s->tile_level[l], n)) return s->tile_level[l];
  return tile_for(n);
}

// profile name of a tile kernel: one entry per level ("mg_down_l0", ...)
static std::string level_name(const Solver* s, const Level& L, const char* base) {
  return std::string(base) + "_l" + std::to_string(&L - s->lev.data());
}

// The dynamic shared-memory limit is an attribute of the function on each
// device: by default static + dynamic may not pass 48 KB.  Set once per
// (kernel, device) when the kernel's static shared memory plus the dynamic
// bytes it is launched with pass that.
template <class K>
static void tile_smem_attr(K kernel, size_t bytes, int device, std::atomic<uint64_t>& done) {
  const uint64_t bit = 1ull << (device & 63);
  if (done.load() & bit) return;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return;
  if (fa.sharedSizeBytes + bytes <= 48 * 1024 ||
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
    done.fetch_or(bit);
}

// tensor maps of a level's fields for the tile boxes of TileBox<T, H> (and the
// coarse block); false: every tile stages with wrapped copies
//
// Staging mode of a level with tensor maps: every tile by TMA, the edge
// tiles' ring fixed up (2).  On the 64-cell tiles (>= 1024 CTAs, 4 per SM by
// shared memory: more than one wave) this takes the edge tiles' per-element
// wrapped copies out of the instruction stream the other CTAs share
// (2048^2: level-0 up 32.1 -> 28.7 us, down 23.8 -> 22.7 us).  The smaller
// tiles run in one wave, where the slowest CTA sets the time: there the ring
// loads must be in flight during the copy (tma_stage_ringed's registers); a
// fix-up after the wait made levels 2-4 slower by 1.2-3.2 us per launch.
constexpr int kTileTmaMode = 2;
template <int T, int H>
static bool tile_maps(Solver* s, int n, const float* const* f, CUtensorMap* const* m, int count) {
  using B = TileBox<T, H>;
  for (int q = 0; q < count; q++)
    if (f[q] && !box_tmap(s, f[q], n, n, B::W, B::R, m[q])) return false;
  return true;
}

// first >= 0: the sweeps of this level in the first cycle of a projection;
// cyc: the loop's cycle count on the device that decides (nullptr: the host
// knows this is the first cycle)
template <int T, int H>
static void down_t(Solver* s, Level& L, const Level& C, bool has_x, int first, const int* cyc, bool x_unused) {
  static std::atomic<uint64_t> attr{0};
  constexpr size_t smem = down_smem_bytes<T, H>();
  tile_smem_attr(k_mg_down<T, H>, smem, s->prm.device, attr);
  dim3 grid((L.n + T - 1) / T, (L.n + T - 1) / T);
  double bytes = (double)L.n * L.n * (has_x ? 12.0 : 8.0) + (double)C.n * C.n * 4.0;
  float* out = has_x ? L.x2 : L.x;
  const float* xin = has_x ? L.x : nullptr;
  CUtensorMap tr{}, tx{};
  const float* f[2] = {L.rhs, xin};
  CUtensorMap* m[2] = {&tr, &tx};
  const int tma = tile_maps<T, H>(s, L.n, f, m, 2) ? kTileTmaMode : 0;
  // a first cycle the host knows is profiled under its own name
  const std::string name = level_name(s, L, "mg_down") + (first >= 0 && !cyc ? "_first" : "");
  FS_LAUNCH(s, name.c_str(), bytes,
            k_mg_down<T, H><<<grid, kTileBlock, smem, s->stream>>>(
                L.rhs, xin, out, C.rhs, L.n, L.h2, s->prm.mg_pre_smooth, (float)s->prm.relax, tr, tx, tma,
                &s->dev->async_err, cyc, first < s->prm.mg_pre_smooth ? first : s->prm.mg_pre_smooth,
                x_unused ? 1 : 0));
  if (has_x) std::swap(L.x, L.x2);
}

template <int H>
static void down(Solver* s, Level& L, const Level& C, bool has_x, int first, const int* cyc, bool x_unused) {
  switch (mg_tile(s, (int)(&L - s->lev.data()))) {
    case 64: down_t<64, H>(s, L, C, has_x, first, cyc, x_unused); break;
    case 32: down_t<32, H>(s, L, C, has_x, first, cyc, x_unused); break;
    default: down_t<16, H>(s, L, C, has_x, first, cyc, x_unused); break;
  }
}

template <int T, int H>
static void up_t(Solver* s, Level& L, const Level& C, float* acc_h, float* acc_l, int first, const int* cyc,
                 bool x_zero) {
  using CB = CoarseBox<T, H>;
  dim3 grid((L.n + T - 1) / T, (L.n + T - 1) / T);
  constexpr size_t smem = up_smem_bytes<T, H>();
  CUtensorMap tr{}, tx{}, tc{};
  const float* f[2] = {L.rhs, L.x};
  CUtensorMap* m[2] = {&tr, &tx};
  const int tma =
      tile_maps<T, H>(s, L.n, f, m, 2) && box_tmap(s, C.x, C.n, C.n, CB::WC, CB::RC, &tc) ? kTileTmaMode : 0;
  int* err = &s->dev->async_err;
  if (acc_h) {
    static std::atomic<uint64_t> attr{0};
    tile_smem_attr(k_mg_up<T, H, true>, smem, s->prm.device, attr);
    double bytes = (double)L.n * L.n * 24.0 + (double)C.n * C.n * 4.0;
    FS_LAUNCH(s, first >= 0 && !cyc ? "mg_up_acc_first" : "mg_up_acc", bytes,
              k_mg_up<T, H, true><<<grid, kTileBlock, smem, s->stream>>>(
                  L.rhs, L.x, nullptr, C.x, L.n, L.h2, s->prm.mg_post_smooth, acc_h, acc_l, (float)s->prm.relax, tr,
                  tx, tc, tma, err, cyc, first < s->prm.mg_post_smooth ? first : s->prm.mg_post_smooth,
                  x_zero ? 1 : 0));
    return;
  }
  static std::atomic<uint64_t> attr{0};
  tile_smem_attr(k_mg_up<T, H, false>, smem, s->prm.device, attr);
  double bytes = (double)L.n * L.n * 12.0 + (double)C.n * C.n * 4.0;
  FS_LAUNCH(s, level_name(s, L, "mg_up").c_str(), bytes,
            k_mg_up<T, H, false><<<grid, kTileBlock, smem, s->stream>>>(
                L.rhs, L.x, L.x2, C.x, L.n, L.h2, s->prm.mg_post_smooth, nullptr, nullptr, (float)s->prm.relax, tr,
                tx, tc, tma, err, cyc, first < s->prm.mg_post_smooth ? first : s->prm.mg_post_smooth,
                  x_zero ? 1 : 0));
  std::swap(L.x, L.x2);
}

template <int H>
static void up(Solver* s, Level& L, const Level& C, float* acc_h, float* acc_l, int first, const int* cyc,
               bool x_zero) {
  switch (mg_tile(s, (int)(&L - s->lev.data()))) {
    case 64: up_t<64, H>(s, L, C, acc_h, acc_l, first, cyc, x_zero); break;
    case 32: up_t<32, H>(s, L, C, acc_h, acc_l, first, cyc, x_zero); break;
    default: up_t<16, H>(s, L, C, acc_h, acc_l, first, cyc, x_zero); break;
  }
}

// first level of the bottom solve: every level from there down is <= 64
int bottom_first_level(const Solver* s) {
  int nl = (int)s->lev.size();
  int lb = nl - 1;
  while (lb > 0 && s->lev[lb - 1].n <= 64 && nl - (lb - 1) <= 8) lb--;
  return lb;
}

// the fused cycle needs even tile levels, a bottom of <= 8 levels each <= 64,
// and 1 <= pre, post <= 3
bool mg_fused_supported(const Solver* s) {
  const fs_params& P = s->prm;
  if (P.mg_pre_smooth < 1 || P.mg_pre_smooth > 3 || P.mg_post_smooth < 1 || P.mg_post_smooth > 3) return false;
  int lb = bottom_first_level(s);
  for (int l = 0; l < lb; l++)
    if (s->lev[l].n & 1) return false;
  if ((int)s->lev.size() - lb > 8) return false;
  for (size_t l = lb; l < s->lev.size(); l++)
    if (s->lev[l].n > 64) return false;
  return true;
}

static size_t bottom_layout(const Solver* s, BottomLevels* B) {
  int lb = bottom_first_level(s);
  int nl = (int)s->lev.size();
  B->count = nl - lb;
  B->w = (float)s->prm.relax;
  int off = 0;
  for (int k = 0; k < B->count; k++) {
    const Level& L = s->lev[lb + k];
    int m = L.n * L.n;
    B->n[k] = L.n;
    B->h2[k] = L.h2;
    B->off_x[k] = off; off += m;
    B->off_r[k] = off; off += m;
    if (L.n & 1) { B->off_x2[k] = off; off += m; }
    else B->off_x2[k] = -1;
  }
  // levels <= 64 hold at most 2 * (64^2 + 32^2 + ...) + 15^2 floats < 48 KB
  return (size_t)off * sizeof(float);
}

// The compile-time chain kernel for the bottom levels from lb, identified by
// its first size (64, 32, 16, 8 down to 8; 48, 24, 12 down to 12), or 0 when
// the levels form another chain (odd sizes, other coarsest sizes).
static int bottom_chain(const Solver* s, int lb) {
  const std::vector<Level>& L = s->lev;
  for (size_t k = lb; k + 1 < L.size(); k++)
    if ((L[k].n & 1) || L[k + 1].n * 2 != L[k].n) return 0;
  const int nb = L[lb].n, nmin = L.back().n;
  if (nmin == 8 && (nb == 64 || nb == 32 || nb == 16 || nb == 8)) return nb;
  if (nmin == 12 && (nb == 48 || nb == 24 || nb == 12)) return nb;
  return 0;
}

static BottomH2 bottom_h2(const Solver* s, int lb) {
  BottomH2 H{};
  for (int k = 0; k < (int)s->lev.size() - lb && k < 4; k++) H.h2[k] = s->lev[lb + k].h2;
  H.w = (float)s->prm.relax;
  return H;
}

void mg_vcycle_fused(Solver* s, bool first_has_x, float* acc_h, float* acc_l) {
  std::vector<Level>& L = s->lev;
  const int lb = bottom_first_level(s);
  const fs_params& P = s->prm;
  // the finest level of a MIXED refinement cycle (acc_h: the correction goes
  // into the double-float pressure) may run fewer sweeps in the first cycle of
  // a projection: the host knows which cycle it enqueues (mg_cycle_index >= 0)
  // except inside a captured tolerance loop, where the kernels read the loop's
  // cycle count on the device
  int fpre = -1, fpost = -1;
  const int* cyc = nullptr;
  if (acc_h && s->mg_cycle_index <= 0) {
    fpre = P.mg_first_pre;
    fpost = P.mg_first_post;
    if (s->mg_cycle_index < 0 && (fpre >= 0 || fpost >= 0)) cyc = &s->dev->cycles;
  }
  for (int l = 0; l < lb; l++) {
    bool hx = l == 0 && first_has_x;
    const int f = l == 0 ? fpre : -1;
    const bool xu = l == 0 && fpost == 0;  // the first cycle's up kernel reads no iterate here
    switch (P.mg_pre_smooth) {
      case 1: down<3>(s, L[l], L[l + 1], hx, f, cyc, xu); break;
      case 2: down<5>(s, L[l], L[l + 1], hx, f, cyc, xu); break;
      default: down<7>(s, L[l], L[l + 1], hx, f, cyc, xu); break;
    }
  }
  int nb = L[lb].n;
  bool hx = lb == 0 && first_has_x;
  float* bah = lb == 0 ? acc_h : nullptr;
  float* bal = lb == 0 ? acc_l : nullptr;
  double bytes = (double)nb * nb * (hx ? 12.0 : 8.0);
  // a chain of levels known at compile time: the specialised kernel
  const int chain = bottom_chain(s, lb);
  if (chain) {
    const BottomH2 H = bottom_h2(s, lb);
#define FS_CHAIN(N0, NM)                                                                                     \
  FS_LAUNCH(s, "mg_bottom", bytes,                                                                           \
            k_mg_bottom_chain<N0, NM><<<1, kBottomThreads, 0, s->stream>>>(L[lb].rhs, L[lb].x, hx ? 1 : 0, H,            \
                                                                 P.mg_pre_smooth, P.mg_post_smooth,            \
                                                                 P.mg_coarse_sweeps, bah, bal))
    switch (chain) {
      case 64: FS_CHAIN(64, 8); break;
      case 32: FS_CHAIN(32, 8); break;
      case 16: FS_CHAIN(16, 8); break;
      case 8: FS_CHAIN(8, 8); break;
      case 48: FS_CHAIN(48, 12); break;
      case 24: FS_CHAIN(24, 12); break;
      default: FS_CHAIN(12, 12); break;
    }
#undef FS_CHAIN
  } else {
    BottomLevels B;
    size_t smem = bottom_layout(s, &B);
    int threads = std::min(1024, std::max(32, ((nb * nb / 4 + 31) / 32) * 32));
    FS_LAUNCH(s, "mg_bottom", bytes,
              k_mg_bottom<<<1, threads, smem, s->stream>>>(L[lb].rhs, L[lb].x, hx ? 1 : 0, B, P.mg_pre_smooth,
                                                           P.mg_post_smooth, P.mg_coarse_sweeps, bah, bal));
  }
  for (int l = lb - 1; l >= 0; l--) {
    float* ah = l == 0 ? acc_h : nullptr;
    float* al = l == 0 ? acc_l : nullptr;
    const int f = l == 0 ? fpost : -1;
    const bool xz = l == 0 && fpre == 0;  // the first cycle's down kernel left a zero iterate here
    switch (P.mg_post_smooth) {
      case 1: up<2>(s, L[l], L[l + 1], ah, al, f, cyc, xz); break;
      case 2: up<4>(s, L[l], L[l + 1], ah, al, f, cyc, xz); break;
      default: up<6>(s, L[l], L[l + 1], ah, al, f, cyc, xz); break;
    }
  }
}


// ------------------------------------------------------- batched V-cycle
// mg_vcycle_fused(s, false, ph, pl) of a MIXED refinement cycle for every
// member of one size class (same grid and multigrid settings), one launch per
// level and phase; the level pointers of each member move exactly as in the
// single-solver cycle.  Returns the number of launches it recorded.
template <int T, int H>
static void down_class_t(Solver* const* ms, int count, int l, cudaStream_t st) {
  const Level& L0 = ms[0]->lev[l];
  DownTab tab{};
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    Level& L = s->lev[l];
    auto& m = tab.m[i];
    m.rhs = L.rhs;
    m.xout = L.x;
    m.crhs = s->lev[l + 1].rhs;
    m.st = s->dev;
    const float* f[1] = {L.rhs};
    CUtensorMap* mp[1] = {&tab.tm[i]};
    m.tma = tile_maps<T, H>(s, L.n, f, mp, 1) ? kTileTmaMode : 0;
  }
  static std::atomic<uint64_t> attr{0};
  constexpr size_t smem = down_smem_bytes<T, H>();
  tile_smem_attr(k_mg_down_class<T, H>, smem, ms[0]->prm.device, attr);
  dim3 grid((L0.n + T - 1) / T, (L0.n + T - 1) / T, count);
  k_mg_down_class<T, H><<<grid, kTileBlock, smem, st>>>(tab, L0.n, L0.h2, ms[0]->prm.mg_pre_smooth,
                                                         (float)ms[0]->prm.relax, ms[0]->prm.max_cycles);
}

// tile side for a level of a class: an override of the class's members, else
// like tile_for counting the CTAs of all members (the tiles give the same
// values whatever their size)
static int tile_for_class(const Solver* s0, int l, int count) {
  const int n = s0->lev[l].n;
  if (l < 16 && s0->tile_level[l] && tile_fits(s0->tile_level[l], n)) return s0->tile_level[l];
  for (int t : {64, 32}) {
    int c = (n + t - 1) / t;
    if (tile_fits(t, n) && c * c * count >= 256) return t;
  }
  return 16;
}

int mg_tile_class(const Solver* s0, int l, int count) { return tile_for_class(s0, l, count); }

template <int H>
static void down_class(Solver* const* ms, int count, int l, cudaStream_t st) {
  switch (tile_for_class(ms[0], l, count)) {
    case 64: down_class_t<64, H>(ms, count, l, st); break;
    case 32: down_class_t<32, H>(ms, count, l, st); break;
    default: down_class_t<16, H>(ms, count, l, st); break;
  }
}

template <int T, int H, bool ACC>
static void up_class_t(Solver* const* ms, int count, int l, cudaStream_t st) {
  const Level& L0 = ms[0]->lev[l];
  using CB = CoarseBox<T, H>;
  UpTab tab{};  // 28 KB on the host stack, copied into the launch's parameters
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    Level& L = s->lev[l];
    const Level& C = s->lev[l + 1];
    auto& m = tab.m[i];
    m.rhs = L.rhs;
    m.xin = L.x;
    m.xout = ACC ? nullptr : L.x2;
    m.xc = C.x;
    m.ph = ACC ? s->ph : nullptr;
    m.pl = ACC ? s->pl : nullptr;
    m.st = s->dev;
    const float* f[2] = {L.rhs, L.x};
    CUtensorMap* mp[2] = {&tab.tm[i][0], &tab.tm[i][1]};
    m.tma = tile_maps<T, H>(s, L.n, f, mp, 2) && box_tmap(s, C.x, C.n, C.n, CB::WC, CB::RC, &tab.tm[i][2])
                ? kTileTmaMode
                : 0;
    if (!ACC) std::swap(L.x, L.x2);
  }
  static std::atomic<uint64_t> attr{0};
  constexpr size_t smem = up_smem_bytes<T, H>();
  tile_smem_attr(k_mg_up_class<T, H, ACC>, smem, ms[0]->prm.device, attr);
  dim3 grid((L0.n + T - 1) / T, (L0.n + T - 1) / T, count);
  k_mg_up_class<T, H, ACC><<<grid, kTileBlock, smem, st>>>(tab, L0.n, L0.h2, ms[0]->prm.mg_post_smooth,
                                                            (float)ms[0]->prm.relax, ms[0]->prm.max_cycles);
}

template <int H>
static void up_class(Solver* const* ms, int count, int l, cudaStream_t st) {
  const bool acc = l == 0;
  switch (tile_for_class(ms[0], l, count)) {
    case 64: acc ? up_class_t<64, H, true>(ms, count, l, st) : up_class_t<64, H, false>(ms, count, l, st); break;
    case 32: acc ? up_class_t<32, H, true>(ms, count, l, st) : up_class_t<32, H, false>(ms, count, l, st); break;
    default: acc ? up_class_t<16, H, true>(ms, count, l, st) : up_class_t<16, H, false>(ms, count, l, st); break;
  }
}

int mg_vcycle_class(Solver* const* ms, int count, cudaStream_t st) {
  Solver* s0 = ms[0];
  for (int i = 0; i < count; i++) {  // level 0 is the correction of the refinement cycle
    ms[i]->lev[0].x = ms[i]->e32;
    ms[i]->lev[0].x2 = ms[i]->e32b;
  }
  const std::vector<Level>& L = s0->lev;
  const int lb = bottom_first_level(s0);
  const fs_params& P = s0->prm;
  int launches = 0;
  for (int l = 0; l < lb; l++, launches++) {
    switch (P.mg_pre_smooth) {
      case 1: down_class<3>(ms, count, l, st); break;
      case 2: down_class<5>(ms, count, l, st); break;
      default: down_class<7>(ms, count, l, st); break;
    }
  }
  const int nb = L[lb].n;
  BottomTab tab{};
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    tab.m[i] = {s->lev[lb].rhs, s->lev[lb].x, lb == 0 ? s->ph : nullptr, lb == 0 ? s->pl : nullptr, s->dev};
  }
  const int chain = bottom_chain(s0, lb);
  if (chain) {
    const BottomH2 H = bottom_h2(s0, lb);
    const dim3 grid(1, 1, count);
#define FS_CHAIN(N0, NM)                                                                                        \
  k_mg_bottom_chain_class<N0, NM><<<grid, kBottomThreads, 0, st>>>(tab, H, P.mg_pre_smooth, P.mg_post_smooth,             \
                                                         P.mg_coarse_sweeps, P.max_cycles)
    switch (chain) {
      case 64: FS_CHAIN(64, 8); break;
      case 32: FS_CHAIN(32, 8); break;
      case 16: FS_CHAIN(16, 8); break;
      case 8: FS_CHAIN(8, 8); break;
      case 48: FS_CHAIN(48, 12); break;
      case 24: FS_CHAIN(24, 12); break;
      default: FS_CHAIN(12, 12); break;
    }
#undef FS_CHAIN
  } else {
    BottomLevels B;
    const size_t smem = bottom_layout(s0, &B);
    const int threads = std::min(1024, std::max(32, ((nb * nb / 4 + 31) / 32) * 32));
    k_mg_bottom_class<<<dim3(1, 1, count), threads, smem, st>>>(tab, B, P.mg_pre_smooth, P.mg_post_smooth,
                                                                 P.mg_coarse_sweeps, P.max_cycles);
  }
  launches++;
  for (int l = lb - 1; l >= 0; l--, launches++) {
    switch (P.mg_post_smooth) {
      case 1: up_class<2>(ms, count, l, st); break;
      case 2: up_class<4>(ms, count, l, st); break;
      default: up_class<6>(ms, count, l, st); break;
    }
  }
  return launches;
}
}  // namespace fs
