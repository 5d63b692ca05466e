// fs_pressure.cu -- divergence, Poisson smoothers, multigrid V-cycle, gradient
// subtraction, mixed-precision refinement and reductions for GB300 (sm_103a).
//
// Reference: src/gpu/shaders.js DIVERGENCE (:269-288), JACOBI (:302-325),
// RED_BLACK_GS (:340-372), SUBTRACT_GRADIENT (:375-398); src/gpu/multigrid.js
// RESIDUAL (:48-66), RESTRICT (:72-93), PROLONG (:99-131), CLEAR (:134-141),
// Multigrid._smooth (:256-270) and encodeVCycle (:277-330); the f64 semantics
// are src/core/grid.js:191-218 and src/cpu/projection.js:48-62.
//
// Red-black Gauss-Seidel is done in place, one colour per pass: on an even
// periodic grid the cells of one colour read only the other colour, so this
// equals the reference's ping-pong pass with copy-through
// (shaders.js:353-358) bit for bit.  On an odd grid the wrap pairs cells of
// the same colour, and a ping-pong pass is used to keep the reference result.
#include <math.h>

#include "fs_df.cuh"
#include "fs_internal.cuh"
#include "fs_reduce.cuh"
#include "fs_stencil.cuh"

namespace fs {

static const dim3 kBlock(32, 8);

__device__ __forceinline__ int wrapm(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ------------------------------------------------------------- divergence
// (uR - uL)/dx + (vT - vB)/dy at cell centres (grid.js:191-206)
template <class TV, class TD>
__global__ void __launch_bounds__(256) k_divergence(const TV* __restrict__ u, const TV* __restrict__ v,
                                                    TD* __restrict__ d, int nx, int ny, TD idx, TD idy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int ip = i + 1 == nx ? 0 : i + 1, jp = j + 1 == ny ? 0 : j + 1;
  int64_t c = (int64_t)j * nx + i;
  TD uL = (TD)u[c], uR = (TD)u[(int64_t)j * nx + ip];
  TD vB = (TD)v[c], vT = (TD)v[(int64_t)jp * nx + i];
  d[c] = (uR - uL) * idx + (vT - vB) * idy;
}

template <class TV, class TD>
void launch_divergence(Solver* s, const TV* u, const TV* v, TD* d) {
  const Grid& g = s->g;
  TD ix = sizeof(TD) == 8 ? (TD)g.idxd : (TD)g.idx;
  TD iy = sizeof(TD) == 8 ? (TD)g.idyd : (TD)g.idy;
  FS_LAUNCH(s, "divergence", (double)s->n * (2 * sizeof(TV) + sizeof(TD)),
            k_divergence<TV, TD><<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(u, v, d, g.nx,
                                                                                        g.ny, ix, iy));
}
template void launch_divergence<float, float>(Solver*, const float*, const float*, float*);

// ------------------------------------------------------ gradient subtraction
// u -= (p_i - p_{i-1})/dx, v -= (p_j - p_{j-1})/dy (grid.js:209-218)
__global__ void __launch_bounds__(256)
    k_subgrad_f32(const float* __restrict__ wu, const float* __restrict__ wv, const float* __restrict__ p,
                  float* __restrict__ ou, float* __restrict__ ov, int nx, int ny, float idx, float idy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, jm = j == 0 ? ny - 1 : j - 1;
  int64_t c = (int64_t)j * nx + i;
  float pc = __ldg(p + c);
  ou[c] = __ldg(wu + c) - (pc - __ldg(p + (int64_t)j * nx + im)) * idx;
  ov[c] = __ldg(wv + c) - (pc - __ldg(p + (int64_t)jm * nx + i)) * idy;
}

void launch_subtract_gradient_f32(Solver* s, const float* wu, const float* wv, const float* p,
                                  float* ou, float* ov) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "subtract_gradient", (double)s->n * 20,
            k_subgrad_f32<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(wu, wv, p, ou, ov, g.nx,
                                                                                g.ny, g.idx, g.idy));
}
// ----------------------------------------------------------------- smoothers
// damped Jacobi, relaxation factor w (shaders.js:302-325)
__global__ void __launch_bounds__(256) k_jacobi(const float* __restrict__ p, const float* __restrict__ d,
                                                float* __restrict__ o, int nx, int ny, float h2, float w) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
  int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
  int64_t r = (int64_t)j * nx;
  o[r + i] = gs_update(__ldg(p + r + i), __ldg(p + r + im), __ldg(p + r + ip), __ldg(p + (int64_t)jm * nx + i),
                       __ldg(p + (int64_t)jp * nx + i), __ldg(d + r + i), h2, w);
}

void launch_jacobi(Solver* s, const float* p, const float* d, float* out, float h2, int nx, int ny) {
  FS_LAUNCH(s, "jacobi", (double)nx * ny * 12,
            k_jacobi<<<grid2d(nx, ny, kBlock), kBlock, 0, s->stream>>>(p, d, out, nx, ny, h2,
                                                                        (float)s->prm.relax));
}

// one red-black colour (shaders.js:340-372, relaxation factor w); dst may equal src on even grids
__global__ void __launch_bounds__(256) k_rb_half(const float* src, const float* __restrict__ d, float* dst,
                                                 int nx, int ny, float h2, int colour, float w) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int64_t r = (int64_t)j * nx;
  float cur = src[r + i];
  if (((i + j) & 1) != colour) {
    if (dst != src) dst[r + i] = cur;
    return;
  }
  int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
  int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
  dst[r + i] = gs_update(cur, src[r + im], src[r + ip], src[(int64_t)jm * nx + i], src[(int64_t)jp * nx + i],
                         __ldg(d + r + i), h2, w);
}

void launch_rb_half(Solver* s, const float* src, const float* d, float* dst, float h2, int colour,
                    int nx, int ny) {
  FS_LAUNCH(s, "rb_half", (double)nx * ny * (src == dst ? 6 : 12),
            k_rb_half<<<grid2d(nx, ny, kBlock), kBlock, 0, s->stream>>>(src, d, dst, nx, ny, h2, colour,
                                                                         (float)s->prm.relax));
}

// ------------------------------------------------------- multigrid transfers
// r = rhs - (l + r + b + t - 4c)/h2 (multigrid.js:48-66)
__global__ void __launch_bounds__(256) k_residual(const float* __restrict__ x, const float* __restrict__ rhs,
                                                  float* __restrict__ o, int n, float h2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= n || j >= n) return;
  int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
  int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
  int64_t r = (int64_t)j * n;
  o[r + i] = residual_at(__ldg(x + r + i), __ldg(x + r + im), __ldg(x + r + ip), __ldg(x + (int64_t)jm * n + i),
                         __ldg(x + (int64_t)jp * n + i), __ldg(rhs + r + i), inv_h2(h2));
}

void launch_residual(Solver* s, const float* x, const float* rhs, float* out, float h2, int n) {
  FS_LAUNCH(s, "residual", (double)n * n * 12,
            k_residual<<<grid2d(n, n, kBlock), kBlock, 0, s->stream>>>(x, rhs, out, n, h2));
}

// coarse = 1/4 sum of the 2x2 fine block (multigrid.js:72-93)
__global__ void __launch_bounds__(256) k_restrict(const float* __restrict__ f, float* __restrict__ c, int nc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nc || j >= nc) return;
  int nf = 2 * nc;
  int64_t r0 = (int64_t)(2 * j) * nf, r1 = r0 + nf;
  c[(int64_t)j * nc + i] = restrict4(__ldg(f + r0 + 2 * i), __ldg(f + r0 + 2 * i + 1), __ldg(f + r1 + 2 * i),
                                      __ldg(f + r1 + 2 * i + 1));
}

void launch_restrict(Solver* s, const float* fine, float* coarse, int nc) {
  FS_LAUNCH(s, "restrict", (double)nc * nc * 20,
            k_restrict<<<grid2d(nc, nc, kBlock), kBlock, 0, s->stream>>>(fine, coarse, nc));
}

// fine += bilinear(coarse) at ((i+1/2)/2 - 1/2, (j+1/2)/2 - 1/2) (multigrid.js:99-131)
// The sample point is 1/4 or 3/4 between coarse nodes: weights are exact.
__global__ void __launch_bounds__(256) k_prolong_add(const float* __restrict__ c, float* __restrict__ f, int nf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nf || j >= nf) return;
  int nc = nf >> 1;
  // i even: gx = i/2 - 1/4 -> i0 = i/2 - 1, fx = 3/4 ; i odd: gx = (i-1)/2 + 1/4 -> fx = 1/4
  int i0 = (i & 1) ? (i >> 1) : (i >> 1) - 1;
  int j0 = (j & 1) ? (j >> 1) : (j >> 1) - 1;
  float fx = (i & 1) ? 0.25f : 0.75f, fy = (j & 1) ? 0.25f : 0.75f;
  int x0 = wrapm(i0, nc), x1 = wrapm(i0 + 1, nc), y0 = wrapm(j0, nc), y1 = wrapm(j0 + 1, nc);
  float a = __ldg(c + (int64_t)y0 * nc + x0), b = __ldg(c + (int64_t)y0 * nc + x1);
  float cc = __ldg(c + (int64_t)y1 * nc + x0), d = __ldg(c + (int64_t)y1 * nc + x1);
  int64_t k = (int64_t)j * nf + i;
  f[k] = __fadd_rn(f[k], prolong_val(a, b, cc, d, fx, fy));
}

void launch_prolong_add(Solver* s, const float* coarse, float* fine, int nf) {
  FS_LAUNCH(s, "prolong_add", (double)nf * nf * 9,
            k_prolong_add<<<grid2d(nf, nf, kBlock), kBlock, 0, s->stream>>>(coarse, fine, nf));
}

__global__ void k_fill(float* x, float v, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x[k] = v;
}
__global__ void k_fill64(double* x, double v, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x[k] = v;
}
static int fill_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}
void launch_fill(Solver* s, float* x, float value, int64_t n) {
  FS_LAUNCH(s, "fill", (double)n * 4, k_fill<<<fill_blocks(n), 256, 0, s->stream>>>(x, value, n));
}
void launch_fill64(Solver* s, double* x, double value, int64_t n) {
  FS_LAUNCH(s, "fill", (double)n * 8, k_fill64<<<fill_blocks(n), 256, 0, s->stream>>>(x, value, n));
}

// Reduction kernels walk 32x8-cell tiles with a capped 1-D grid, so the
// last-block fold reads at most kRedGrid partials (a fold over one partial per
// tile of a 2048^2 grid, 16384 of them, was latency-bound at ~40 us).
constexpr int kRedGrid = 152 * 8;
// a 2-D grid over tile columns and rows (no index division in the walk)
static dim3 red_grid2(int nx, int ny) {
  int ntx = (nx + 31) >> 5, nty = (ny + 7) >> 3;
  int gx = ntx < kRedGrid ? ntx : kRedGrid;
  int gy = kRedGrid / gx;
  if (gy > nty) gy = nty;
  return dim3(gx, gy < 1 ? 1 : gy);
}

// 2-D tile walk of the capped reduction grid: tile (tx, ty) of 32x8 cells
#define FOR_RED_TILES(nx, ny)                                                          \
  for (int ty = blockIdx.y, nty_ = ((ny) + 7) >> 3; ty < nty_; ty += gridDim.y)        \
    for (int tx = blockIdx.x, ntx_ = ((nx) + 31) >> 5; tx < ntx_; tx += gridDim.x)

// NaN must not vanish in a max: fmax(x, NaN) = x, so NaN is mapped to +inf.
__device__ __forceinline__ double absnan(double x) { return x != x ? INFINITY : fabs(x); }
__device__ __forceinline__ float absnanf(float x) { return x != x ? INFINITY : fabsf(x); }

template <class T>
__global__ void __launch_bounds__(256) k_absmax(const T* __restrict__ x, int64_t n, RedCtx ctx) {
  float m = 0.f;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, absnanf((float)__ldg(x + k)));
  block_max_finish(m, ctx);
}

static int red_blocks(Solver* s, int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > kRedGrid) b = kRedGrid;
  if (b > s->red_cap) b = s->red_cap;
  return (int)(b < 1 ? 1 : b);
}

template <class T>
void launch_absmax(Solver* s, const T* x, int64_t n, double* out_word) {
  FS_LAUNCH(s, "absmax", (double)n * sizeof(T),
            k_absmax<T><<<red_blocks(s, n), 256, 0, s->stream>>>(x, n, red_ctx(s, out_word)));
}
template void launch_absmax<float>(Solver*, const float*, int64_t, double*);
template void launch_absmax<double>(Solver*, const double*, int64_t, double*);

// ||lap p - d||^2 and ||d||^2 in f64 from f32 fields (poissonResidualAfter,
// solver.js:878-895; h2 = dx*dx in f64 as the host computes it there)
__global__ void __launch_bounds__(256) k_poisson_norms(const float* __restrict__ p, const float* __restrict__ d,
                                                       int nx, int ny, double h2, RedCtx ctx) {
  double num = 0.0, den = 0.0;
  FOR_RED_TILES(nx, ny) {
  int i = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
  if (i < nx && j < ny) {
    int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
    int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t r = (int64_t)j * nx;
    double lap = ((double)p[r + im] + (double)p[r + ip] + (double)p[(int64_t)jm * nx + i] +
                  (double)p[(int64_t)jp * nx + i] - 4.0 * (double)p[r + i]) / h2;
    double dd = (double)d[r + i];
    double rr = lap - dd;
    num += rr * rr;
    den += dd * dd;
  }
  }
  block_sum2_finish(num, den, ctx);
}

void launch_poisson_norms(Solver* s, const float* p, const float* d, float h2f, double h2) {
  (void)h2f;
  const Grid& g = s->g;
  FS_LAUNCH(s, "poisson_norms", (double)s->n * 8,
            k_poisson_norms<<<red_grid2(g.nx, g.ny), kBlock, 0, s->stream>>>(p, d, g.nx, g.ny, h2,
                                                                             red_ctx(s, s->red_out)));
}

// ------------------------------------------------ mixed-precision refinement
// The MIXED mode keeps velocity, divergence and pressure as double-float
// planes (hi, lo) and does this arithmetic on the FP32 pipe (fs_df.cuh).

// divergence of (hi + lo) faces, lo planes optional (nullptr = 0):
// d = (uR - uL)/dx + (vT - vB)/dy with every operation error-free or df
__device__ __forceinline__ void div_df_body(const float* __restrict__ uh, const float* __restrict__ ul,
                                            const float* __restrict__ vh, const float* __restrict__ vl,
                                            float* __restrict__ dh, float* __restrict__ dl, int nx, int ny, df idx,
                                            df idy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int ip = i + 1 == nx ? 0 : i + 1, jp = j + 1 == ny ? 0 : j + 1;
  int64_t c = (int64_t)j * nx + i, cr = (int64_t)j * nx + ip, ct = (int64_t)jp * nx + i;
  df du = two_diff(__ldg(uh + cr), __ldg(uh + c));
  df dv = two_diff(__ldg(vh + ct), __ldg(vh + c));
  if (ul) du = df_add(du, two_diff(__ldg(ul + cr), __ldg(ul + c)));
  if (vl) dv = df_add(dv, two_diff(__ldg(vl + ct), __ldg(vl + c)));
  df d = df_add(df_mul(du, idx), df_mul(dv, idy));
  dh[c] = d.hi;
  dl[c] = d.lo;
}

// the same divergence of f32 faces (no lo planes) from the four face values
__device__ __forceinline__ df div_f32_faces(float uc, float ur, float vc, float vt, df idx, df idy) {
  return df_add(df_mul(two_diff(ur, uc), idx), df_mul(two_diff(vt, vc), idy));
}

// The start of a refinement from zero pressure in one pass over the cells:
// d = div w as double-float (dh, dl), its residual against p = 0 as
// r32 = (float) d, the pressure planes (ph, pl) zeroed and max|r| reduced --
// the work of k_div_df, k_refine_init (zero_p) and two fills, with the same
// arithmetic per cell.  Four consecutive cells per thread (nx a multiple of
// 4), so a thread keeps five 16-byte loads in flight; tiles of 32 quads x 8
// rows walked by the capped reduction grid.
__device__ __forceinline__ void div_start4_body(const float* __restrict__ wu, const float* __restrict__ wv,
                                                float* __restrict__ dh, float* __restrict__ dl,
                                                float* __restrict__ ph, float* __restrict__ pl,
                                                float* __restrict__ r32, int nx, int ny, df idx, df idy,
                                                const RedCtx& ctx) {
  float m = 0.f;
  const int nq = nx >> 2;
  for (int ty = blockIdx.y, nty = (ny + 7) >> 3; ty < nty; ty += gridDim.y)
    for (int tx = blockIdx.x, ntx = (nq + 31) >> 5; tx < ntx; tx += gridDim.x) {
      const int q = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
      if (q >= nq || j >= ny) continue;
      const int i0 = q << 2;
      const int jp = j + 1 == ny ? 0 : j + 1, ir = i0 + 4 == nx ? 0 : i0 + 4;
      const int64_t r = (int64_t)j * nx;
      const float4 u4 = __ldg(reinterpret_cast<const float4*>(wu + r + i0));
      const float4 v4 = __ldg(reinterpret_cast<const float4*>(wv + r + i0));
      const float4 t4 = __ldg(reinterpret_cast<const float4*>(wv + (int64_t)jp * nx + i0));
      const float ur = __ldg(wu + r + ir);
      const df d0 = div_f32_faces(u4.x, u4.y, v4.x, t4.x, idx, idy);
      const df d1 = div_f32_faces(u4.y, u4.z, v4.y, t4.y, idx, idy);
      const df d2 = div_f32_faces(u4.z, u4.w, v4.z, t4.z, idx, idy);
      const df d3 = div_f32_faces(u4.w, ur, v4.w, t4.w, idx, idy);
      const float4 rf = {df_to_f(d0), df_to_f(d1), df_to_f(d2), df_to_f(d3)};
      const float4 zero = {0.f, 0.f, 0.f, 0.f};
      *reinterpret_cast<float4*>(dh + r + i0) = float4{d0.hi, d1.hi, d2.hi, d3.hi};
      *reinterpret_cast<float4*>(dl + r + i0) = float4{d0.lo, d1.lo, d2.lo, d3.lo};
      *reinterpret_cast<float4*>(r32 + r + i0) = rf;
      *reinterpret_cast<float4*>(ph + r + i0) = zero;
      *reinterpret_cast<float4*>(pl + r + i0) = zero;
      m = fmaxf(fmaxf(m, fmaxf(absnanf(rf.x), absnanf(rf.y))), fmaxf(absnanf(rf.z), absnanf(rf.w)));
    }
  block_max_finish(m, ctx);
}

__global__ void __launch_bounds__(256)
    k_div_start4(const float* __restrict__ wu, const float* __restrict__ wv, float* __restrict__ dh,
                 float* __restrict__ dl, float* __restrict__ ph, float* __restrict__ pl, float* __restrict__ r32,
                 int nx, int ny, df idx, df idy, RedCtx ctx) {
  div_start4_body(wu, wv, dh, dl, ph, pl, r32, nx, ny, idx, idy, ctx);
}

__global__ void __launch_bounds__(256)
    k_div_df(const float* __restrict__ uh, const float* __restrict__ ul, const float* __restrict__ vh,
             const float* __restrict__ vl, float* __restrict__ dh, float* __restrict__ dl, int nx, int ny, df idx,
             df idy) {
  div_df_body(uh, ul, vh, vl, dh, dl, nx, ny, idx, idy);
}

void launch_div_df(Solver* s, const float* uh, const float* ul, const float* vh, const float* vl, float* dh,
                   float* dl) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "divergence", (double)s->n * ((ul ? 16 : 8) + 8),
            k_div_df<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                uh, ul, vh, vl, dh, dl, g.nx, g.ny, df_host(g.idxd), df_host(g.idyd)));
}

// u = w - (p_i - p_{i-1})/dx, v = w - (p_j - p_{j-1})/dy in df; w lo planes optional
__device__ __forceinline__ void subgrad_df_body(const float* __restrict__ wuh, const float* __restrict__ wul,
                                                const float* __restrict__ wvh, const float* __restrict__ wvl,
                                                const float* __restrict__ ph, const float* __restrict__ pl,
                                                float* __restrict__ uh, float* __restrict__ ul, float* __restrict__ vh,
                                                float* __restrict__ vl, int nx, int ny, df idx, df idy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, jm = j == 0 ? ny - 1 : j - 1;
  int64_t c = (int64_t)j * nx + i, cl = (int64_t)j * nx + im, cb = (int64_t)jm * nx + i;
  df pc = {__ldg(ph + c), __ldg(pl + c)};
  df gx = df_mul(df_sub(pc, df{__ldg(ph + cl), __ldg(pl + cl)}), idx);
  df gy = df_mul(df_sub(pc, df{__ldg(ph + cb), __ldg(pl + cb)}), idy);
  df wu = {__ldg(wuh + c), wul ? __ldg(wul + c) : 0.f};
  df wv = {__ldg(wvh + c), wvl ? __ldg(wvl + c) : 0.f};
  df u = df_sub(wu, gx), v = df_sub(wv, gy);
  uh[c] = u.hi; ul[c] = u.lo;
  vh[c] = v.hi; vl[c] = v.lo;
}

// the same update for four consecutive cells (nx a multiple of 4): float4
// loads of the pressure rows j and j - 1 and of w, the group's left
// neighbour as a scalar; the same df operations per cell as subgrad_df_body
__device__ __forceinline__ void subgrad4_body(const float* __restrict__ wuh, const float* __restrict__ wul,
                                              const float* __restrict__ wvh, const float* __restrict__ wvl,
                                              const float* __restrict__ ph, const float* __restrict__ pl,
                                              float* __restrict__ uh, float* __restrict__ ul,
                                              float* __restrict__ vh, float* __restrict__ vl, int nx, int ny,
                                              df idx, df idy) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (q >= (nx >> 2) || j >= ny) return;
  const int i0 = q << 2, il = i0 == 0 ? nx - 1 : i0 - 1, jm = j == 0 ? ny - 1 : j - 1;
  const int64_t c = (int64_t)j * nx + i0, cb = (int64_t)jm * nx + i0, cl = (int64_t)j * nx + il;
  const float4 h = __ldg(reinterpret_cast<const float4*>(ph + c));
  const float4 l = __ldg(reinterpret_cast<const float4*>(pl + c));
  const float4 hb = __ldg(reinterpret_cast<const float4*>(ph + cb));
  const float4 lb = __ldg(reinterpret_cast<const float4*>(pl + cb));
  const float4 uw = __ldg(reinterpret_cast<const float4*>(wuh + c));
  const float4 vw = __ldg(reinterpret_cast<const float4*>(wvh + c));
  const float4 z = {0.f, 0.f, 0.f, 0.f};
  const float4 uwl = wul ? __ldg(reinterpret_cast<const float4*>(wul + c)) : z;
  const float4 vwl = wvl ? __ldg(reinterpret_cast<const float4*>(wvl + c)) : z;
  const df pw = {__ldg(ph + cl), __ldg(pl + cl)};
  const df p0 = {h.x, l.x}, p1 = {h.y, l.y}, p2 = {h.z, l.z}, p3 = {h.w, l.w};
  const df u0 = df_sub(df{uw.x, uwl.x}, df_mul(df_sub(p0, pw), idx));
  const df u1 = df_sub(df{uw.y, uwl.y}, df_mul(df_sub(p1, p0), idx));
  const df u2 = df_sub(df{uw.z, uwl.z}, df_mul(df_sub(p2, p1), idx));
  const df u3 = df_sub(df{uw.w, uwl.w}, df_mul(df_sub(p3, p2), idx));
  const df v0 = df_sub(df{vw.x, vwl.x}, df_mul(df_sub(p0, df{hb.x, lb.x}), idy));
  const df v1 = df_sub(df{vw.y, vwl.y}, df_mul(df_sub(p1, df{hb.y, lb.y}), idy));
  const df v2 = df_sub(df{vw.z, vwl.z}, df_mul(df_sub(p2, df{hb.z, lb.z}), idy));
  const df v3 = df_sub(df{vw.w, vwl.w}, df_mul(df_sub(p3, df{hb.w, lb.w}), idy));
  *reinterpret_cast<float4*>(uh + c) = make_float4(u0.hi, u1.hi, u2.hi, u3.hi);
  *reinterpret_cast<float4*>(ul + c) = make_float4(u0.lo, u1.lo, u2.lo, u3.lo);
  *reinterpret_cast<float4*>(vh + c) = make_float4(v0.hi, v1.hi, v2.hi, v3.hi);
  *reinterpret_cast<float4*>(vl + c) = make_float4(v0.lo, v1.lo, v2.lo, v3.lo);
}

__global__ void __launch_bounds__(256)
    k_subgrad4_df(const float* __restrict__ wuh, const float* __restrict__ wul, const float* __restrict__ wvh,
                  const float* __restrict__ wvl, const float* __restrict__ ph, const float* __restrict__ pl,
                  float* __restrict__ uh, float* __restrict__ ul, float* __restrict__ vh, float* __restrict__ vl,
                  int nx, int ny, df idx, df idy) {
  subgrad4_body(wuh, wul, wvh, wvl, ph, pl, uh, ul, vh, vl, nx, ny, idx, idy);
}

__global__ void __launch_bounds__(256)
    k_subgrad_df(const float* __restrict__ wuh, const float* __restrict__ wul, const float* __restrict__ wvh,
                 const float* __restrict__ wvl, const float* __restrict__ ph, const float* __restrict__ pl,
                 float* __restrict__ uh, float* __restrict__ ul, float* __restrict__ vh, float* __restrict__ vl,
                 int nx, int ny, df idx, df idy) {
  subgrad_df_body(wuh, wul, wvh, wvl, ph, pl, uh, ul, vh, vl, nx, ny, idx, idy);
}

void launch_subgrad_df(Solver* s, const float* wuh, const float* wul, const float* wvh, const float* wvl,
                       const float* ph, const float* pl, float* uh, float* ul, float* vh, float* vl) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "subtract_gradient", (double)s->n * ((wul ? 16 : 8) + 8 + 16),
            if (g.nx % 4 == 0) {
              k_subgrad4_df<<<grid2d(g.nx / 4, g.ny, kBlock), kBlock, 0, s->stream>>>(
                  wuh, wul, wvh, wvl, ph, pl, uh, ul, vh, vl, g.nx, g.ny, df_host(g.idxd), df_host(g.idyd));
            } else {
              k_subgrad_df<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                  wuh, wul, wvh, wvl, ph, pl, uh, ul, vh, vl, g.nx, g.ny, df_host(g.idxd), df_host(g.idyd));
            });
}

// df Laplacian of p at (i, j).  Square cells (ih2x == ih2y, the uniform
// branch taken in practice): ((pl + pr) + (pb + pt) - 4 pc) / h^2 with the hi
// parts combined error-free (two_sum, 4*x is exact) and the lo parts, each
// below an ulp of p, summed in f32.  Otherwise the x and y second differences
// are formed and scaled separately.  Both orders of evaluation are fixed, so
// every kernel that calls this rounds alike.
// Scale of the 5-point Laplacian.  mode 0: square cells and 1/dx^2 a power of
// two (the unit domain at power-of-two n), so scaling is one exact multiply;
// mode 1: square cells, df scale; mode 2: dx != dy.
struct LapScale {
  df ih2x, ih2y;
  int mode;
};

static LapScale lap_scale(const Grid& g) {
  double sx = g.idxd * g.idxd, sy = g.idyd * g.idyd;
  LapScale k{df_host(sx), df_host(sy), 2};
  if (sx == sy) {
    int e;
    double m = frexp(sx, &e);
    k.mode = (m == 0.5 && e > -120 && e < 120) ? 0 : 1;
  }
  return k;
}

// (float)(d - lap p) for df d and the df pressures of a cell and its four
// neighbours.  For square cells h^2 lap p = pl + pr + pb + pt - 4 pc is summed
// as in Sum2 of Ogita, Rump & Oishi (SIAM J. Sci. Comput. 26, 2005): a chain
// of error-free two_sums over the hi parts, the lo parts and the rounding
// errors gathered in one f32 term; d - lap then takes one more two_sum.  The
// result is as accurate as a sum in twice the working precision, which is
// what the cancellation between the five terms (and between d and lap p near
// convergence) needs.
__device__ __forceinline__ float residual_df(df d, df pc, df pl, df pr, df pb, df pt, const LapScale& k) {
  if (k.mode == 2) {
    df ax = df_add(df_sub(pl, pc), df_sub(pr, pc));
    df ay = df_add(df_sub(pb, pc), df_sub(pt, pc));
    return df_to_f(df_sub(d, df_add(df_mul(ax, k.ih2x), df_mul(ay, k.ih2y))));
  }
  df a = two_sum(pl.hi, pr.hi);
  df b = two_sum(a.hi, pb.hi);
  df c = two_sum(b.hi, pt.hi);
  df e = two_sum(c.hi, __fmul_rn(-4.f, pc.hi));
  float lo = __fmaf_rn(-4.f, pc.lo, __fadd_rn(__fadd_rn(pl.lo, pr.lo), __fadd_rn(pb.lo, pt.lo)));
  lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(a.lo, b.lo), __fadd_rn(c.lo, e.lo)));
  float lh, ll;  // lap p = lh + ll
  if (k.mode == 0) {
    lh = __fmul_rn(e.hi, k.ih2x.hi);
    ll = __fmul_rn(lo, k.ih2x.hi);
  } else {
    df q = two_prod(e.hi, k.ih2x.hi);
    lh = q.hi;
    ll = __fmaf_rn(e.hi, k.ih2x.lo, __fmaf_rn(lo, k.ih2x.hi, q.lo));
  }
  df r = two_sum(d.hi, -lh);
  return __fadd_rn(r.hi, __fsub_rn(__fadd_rn(r.lo, d.lo), ll));
}

// r = d - lap(p) (or r = d when zero_p); r32 = (float) r; max|r| reduced
__device__ __forceinline__ void refine_init_body(const float* __restrict__ dh, const float* __restrict__ dl,
                                                 const float* __restrict__ ph, const float* __restrict__ pl,
                                                 float* __restrict__ r32, int nx, int ny, const LapScale& ks,
                                                 int zero_p, const RedCtx& ctx) {
  float m = 0.f;
  FOR_RED_TILES(nx, ny) {
    int i = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
    if (i < nx && j < ny) {
      int64_t r = (int64_t)j * nx, c = r + i;
      df d = {__ldg(dh + c), __ldg(dl + c)};
      float rf;
      if (zero_p) {
        rf = df_to_f(d);
      } else {
        int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
        int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
        int64_t cl = r + im, cr = r + ip, cb = (int64_t)jm * nx + i, ct = (int64_t)jp * nx + i;
        rf = residual_df(d, df{__ldg(ph + c), __ldg(pl + c)}, df{__ldg(ph + cl), __ldg(pl + cl)},
                         df{__ldg(ph + cr), __ldg(pl + cr)}, df{__ldg(ph + cb), __ldg(pl + cb)},
                         df{__ldg(ph + ct), __ldg(pl + ct)}, ks);
      }
      r32[c] = rf;
      m = fmaxf(m, absnanf(rf));
    }
  }
  block_max_finish(m, ctx);
}

__global__ void __launch_bounds__(256)
    k_refine_init(const float* __restrict__ dh, const float* __restrict__ dl, const float* __restrict__ ph,
                  const float* __restrict__ pl, float* __restrict__ r32, int nx, int ny, LapScale ks,
                  int zero_p, RedCtx ctx) {
  refine_init_body(dh, dl, ph, pl, r32, nx, ny, ks, zero_p, ctx);
}

// The tolerance loop's bookkeeping after a cycle (init: before the loop) from
// the residual maximum m, and the loop condition "cycle again" -- the work of
// k_cond, also done by the residual kernel's finishing thread when the loop
// folds it in (CondFold).
// tol as the loop code passes it (dev_tol): > 0 absolute, < 0 relative to
// the residual the projection started from
__device__ __forceinline__ double tol_limit(double tol, const DevState* st) {
  return tol < 0 ? -tol * st->res_initial : tol;
}

__device__ __forceinline__ bool cond_apply(DevState* st, double m, double tol, int max_cycles, int init) {
  if (init) {
    st->cycles = 0;
    st->res_initial = m;
  } else {
    st->cycles += 1;
    st->total_cycles += 1;
  }
  st->res_max = m;
  const double lim = tol_limit(tol, st);
  const bool finite = isfinite(m);
  st->nonfinite = finite ? 0 : 1;
  st->converged = (finite && m <= lim) ? 1 : 0;
  return finite && m > lim && st->cycles < max_cycles;
}

struct CondFold {
  cudaGraphConditionalHandle h;
  DevState* st;
  double tol;
  int max_cycles;
  int on;  // 0: the kernel only reduces
};

// The same residual, four consecutive cells per thread (nx a multiple of 4):
// float4 loads of the three pressure rows, the left / right neighbours of the
// group from the adjacent words, so each cell costs ~1/3 of the loads and
// index arithmetic of the one-cell form.  Same arithmetic, same results.
__device__ __forceinline__ void refine_init4_body(const float* __restrict__ dh, const float* __restrict__ dl,
                                                  const float* __restrict__ ph, const float* __restrict__ pl,
                                                  float* __restrict__ r32, int nx, int ny, const LapScale& ks,
                                                  const RedCtx& ctx, const CondFold& cf) {
  float m = 0.f;
  const int nq = nx >> 2;  // quads per row
  // tiles of 32 quads x 8 rows walked by the capped 2-D grid
  for (int ty = blockIdx.y, nty = (ny + 7) >> 3; ty < nty; ty += gridDim.y)
    for (int tx = blockIdx.x, ntx = (nq + 31) >> 5; tx < ntx; tx += gridDim.x) {
      const int q = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
      if (q >= nq || j >= ny) continue;
      const int i0 = q << 2;
      const int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
      const int64_t r = (int64_t)j * nx, rm = (int64_t)jm * nx, rp = (int64_t)jp * nx;
      const int il = i0 == 0 ? nx - 1 : i0 - 1, ir = i0 + 4 == nx ? 0 : i0 + 4;
      const float4 ch = __ldg(reinterpret_cast<const float4*>(ph + r + i0));
      const float4 cl = __ldg(reinterpret_cast<const float4*>(pl + r + i0));
      const float4 bh = __ldg(reinterpret_cast<const float4*>(ph + rm + i0));
      const float4 bl = __ldg(reinterpret_cast<const float4*>(pl + rm + i0));
      const float4 th = __ldg(reinterpret_cast<const float4*>(ph + rp + i0));
      const float4 tl = __ldg(reinterpret_cast<const float4*>(pl + rp + i0));
      const float4 d4h = __ldg(reinterpret_cast<const float4*>(dh + r + i0));
      const float4 d4l = __ldg(reinterpret_cast<const float4*>(dl + r + i0));
      const df lft = {__ldg(ph + r + il), __ldg(pl + r + il)}, rgt = {__ldg(ph + r + ir), __ldg(pl + r + ir)};
      const df c0 = {ch.x, cl.x}, c1 = {ch.y, cl.y}, c2 = {ch.z, cl.z}, c3 = {ch.w, cl.w};
      float4 out;
      out.x = residual_df(df{d4h.x, d4l.x}, c0, lft, c1, df{bh.x, bl.x}, df{th.x, tl.x}, ks);
      out.y = residual_df(df{d4h.y, d4l.y}, c1, c0, c2, df{bh.y, bl.y}, df{th.y, tl.y}, ks);
      out.z = residual_df(df{d4h.z, d4l.z}, c2, c1, c3, df{bh.z, bl.z}, df{th.z, tl.z}, ks);
      out.w = residual_df(df{d4h.w, d4l.w}, c3, c2, rgt, df{bh.w, bl.w}, df{th.w, tl.w}, ks);
      *reinterpret_cast<float4*>(r32 + r + i0) = out;
      m = fmaxf(fmaxf(m, fmaxf(absnanf(out.x), absnanf(out.y))), fmaxf(absnanf(out.z), absnanf(out.w)));
    }
  float f;
  if (block_max_finish_at(m, ctx, &f) && cf.on)
    cudaGraphSetConditional(cf.h, cond_apply(cf.st, (double)f, cf.tol, cf.max_cycles, 0) ? 1u : 0u);
}

__global__ void __launch_bounds__(256, 5)
    k_refine_init4(const float* __restrict__ dh, const float* __restrict__ dl, const float* __restrict__ ph,
                   const float* __restrict__ pl, float* __restrict__ r32, int nx, int ny, LapScale ks, RedCtx ctx,
                   CondFold cf) {
  refine_init4_body(dh, dl, ph, pl, r32, nx, ny, ks, ctx, cf);
}

// p' = p + e; r = d - lap(p') in df; r32 = (float) r; max|r| reduced
__global__ void __launch_bounds__(256)
    k_refine_update(const float* __restrict__ ph, const float* __restrict__ pl, const float* __restrict__ e,
                    const float* __restrict__ dh, const float* __restrict__ dl, float* __restrict__ poh,
                    float* __restrict__ pol, float* __restrict__ r32, int nx, int ny, LapScale ks, RedCtx ctx) {
  float m = 0.f;
  FOR_RED_TILES(nx, ny) {
    int i = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
    if (i < nx && j < ny) {
      int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
      int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
      int64_t r = (int64_t)j * nx, c = r + i;
      int64_t cl = r + im, cr = r + ip, cb = (int64_t)jm * nx + i, ct = (int64_t)jp * nx + i;
      df pc = df_add_f(df{__ldg(ph + c), __ldg(pl + c)}, __ldg(e + c));
      df pL = df_add_f(df{__ldg(ph + cl), __ldg(pl + cl)}, __ldg(e + cl));
      df pR = df_add_f(df{__ldg(ph + cr), __ldg(pl + cr)}, __ldg(e + cr));
      df pB = df_add_f(df{__ldg(ph + cb), __ldg(pl + cb)}, __ldg(e + cb));
      df pT = df_add_f(df{__ldg(ph + ct), __ldg(pl + ct)}, __ldg(e + ct));
      float rf = residual_df(df{__ldg(dh + c), __ldg(dl + c)}, pc, pL, pR, pB, pT, ks);
      poh[c] = pc.hi;
      pol[c] = pc.lo;
      r32[c] = rf;
      m = fmaxf(m, absnanf(rf));
    }
  }
  block_max_finish(m, ctx);
}

// Grid of k_refine_init4: one wave (5 CTAs per SM, the register cap of its
// launch bounds), every block walking the same number of tile rows (6 at
// 2048^2, against two waves of up to 4 with the capped reduction grid).
static dim3 refine4_grid(const Solver* s, int nq, int ny) {
  static int sms[64] = {};
  const int dev = s->prm.device & 63;
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, s->prm.device) != cudaSuccess)
    sms[dev] = 0;
  const int slots = (sms[dev] > 0 ? sms[dev] : 152) * 5;
  const int ntx = (nq + 31) >> 5, nty = (ny + 7) >> 3;
  const int gx = ntx < slots ? ntx : slots;
  int gy = slots / gx;
  if (gy < 1) gy = 1;
  const int per = (nty + gy - 1) / gy;
  gy = (nty + per - 1) / per;
  return dim3(gx, gy);
}

// cond: inside a captured tolerance loop, the residual kernel also does the
// loop's step bookkeeping and sets its condition (four-cell form); returns
// true if it did, else the caller launches k_cond itself
bool launch_refine_init(Solver* s, const float* dh, const float* dl, const float* ph, const float* pl,
                        float* r32, bool zero_p, const cudaGraphConditionalHandle* cond) {
  const Grid& g = s->g;
  const bool quad = !zero_p && g.nx % 4 == 0;
  const CondFold cf = (quad && cond) ? CondFold{*cond, s->dev, dev_tol(s), s->prm.max_cycles, 1}
                                     : CondFold{};
  FS_LAUNCH(s, "refine_init", (double)s->n * (zero_p ? 12 : 20),
            if (quad) {
              k_refine_init4<<<refine4_grid(s, g.nx / 4, g.ny), kBlock, 0, s->stream>>>(
                  dh, dl, ph, pl, r32, g.nx, g.ny, lap_scale(g), red_ctx(s, s->red_out), cf);
            } else {
              k_refine_init<<<red_grid2(g.nx, g.ny), kBlock, 0, s->stream>>>(
                  dh, dl, ph, pl, r32, g.nx, g.ny, lap_scale(g), zero_p ? 1 : 0, red_ctx(s, s->red_out));
            });
  return cf.on != 0;
}

// the start of a MIXED solve from zero pressure (k_div_start4; nx a multiple
// of 4, else the divergence, the zero-pressure residual and two fills)
void launch_div_start(Solver* s, const float* wu, const float* wv) {
  const Grid& g = s->g;
  if (g.nx % 4 != 0) {
    launch_div_df(s, wu, nullptr, wv, nullptr, s->dh, s->dl);
    launch_refine_init(s, s->dh, s->dl, s->ph, s->pl, s->r32, true);
    launch_fill(s, s->ph, 0.f, s->n);
    launch_fill(s, s->pl, 0.f, s->n);
    return;
  }
  FS_LAUNCH(s, "div_start", (double)s->n * 28,
            k_div_start4<<<red_grid2(g.nx / 4, g.ny), kBlock, 0, s->stream>>>(
                wu, wv, s->dh, s->dl, s->ph, s->pl, s->r32, g.nx, g.ny, df_host(g.idxd), df_host(g.idyd),
                red_ctx(s, s->red_out)));
}

void launch_refine_update(Solver* s, const float* ph, const float* pl, const float* e, const float* dh,
                          const float* dl, float* poh, float* pol, float* r32) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "refine_update", (double)s->n * 32,
            k_refine_update<<<red_grid2(g.nx, g.ny), kBlock, 0, s->stream>>>(
                ph, pl, e, dh, dl, poh, pol, r32, g.nx, g.ny, lap_scale(g), red_ctx(s, s->red_out)));
}

// ------------------------------------------------------- df <-> host types
__global__ void k_d_to_df(const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    df v = df_from_d(x[k]);
    hi[k] = v.hi;
    lo[k] = v.lo;
  }
}
__global__ void k_df_to_d(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ x, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x[k] = df_to_d(df{hi[k], lo ? lo[k] : 0.f});
}
__global__ void k_df_to_f(const float* __restrict__ hi, const float* __restrict__ lo, float* __restrict__ x, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    x[k] = df_to_f(df{hi[k], lo[k]});
}
void launch_d_to_df(Solver* s, const double* x, float* hi, float* lo, int64_t n) {
  FS_LAUNCH(s, "convert", (double)n * 16, k_d_to_df<<<fill_blocks(n), 256, 0, s->stream>>>(x, hi, lo, n));
}
void launch_df_to_d(Solver* s, const float* hi, const float* lo, double* x, int64_t n) {
  FS_LAUNCH(s, "convert", (double)n * 16, k_df_to_d<<<fill_blocks(n), 256, 0, s->stream>>>(hi, lo, x, n));
}
void launch_df_to_f(Solver* s, const float* hi, const float* lo, float* x, int64_t n) {
  FS_LAUNCH(s, "convert", (double)n * 12, k_df_to_f<<<fill_blocks(n), 256, 0, s->stream>>>(hi, lo, x, n));
}

// max|d - lap p| over an f32 pair (tolerance loop of the F32 mode)
__global__ void __launch_bounds__(256) k_absmax_res32(const float* __restrict__ p, const float* __restrict__ d,
                                                      int nx, int ny, float ih2x, float ih2y, RedCtx ctx) {
  float m = 0.f;
  FOR_RED_TILES(nx, ny) {
  int i = tx * 32 + threadIdx.x, j = ty * 8 + threadIdx.y;
  if (i < nx && j < ny) {
    int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
    int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t r = (int64_t)j * nx;
    float pc = p[r + i];
    float lap = (p[r + im] - 2.f * pc + p[r + ip]) * ih2x + (p[(int64_t)jm * nx + i] - 2.f * pc + p[(int64_t)jp * nx + i]) * ih2y;
    m = fmaxf(m, absnanf(d[r + i] - lap));
  }
  }
  block_max_finish(m, ctx);
}

void launch_absmax_residual32(Solver* s, const float* p, const float* d) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "absmax_residual", (double)s->n * 8,
            k_absmax_res32<<<red_grid2(g.nx, g.ny), kBlock, 0, s->stream>>>(
                p, d, g.nx, g.ny, g.idx * g.idx, g.idy * g.idy, red_ctx(s, s->red_out)));
}

// ------------------------------------------------- tolerance-loop bookkeeping
// One thread: reads the max residual the last reduction left in red[0], keeps
// the statistics in the device step state and, inside a captured step, sets
// the condition of the WHILE node that repeats the refinement cycle.
__global__ void k_cond(cudaGraphConditionalHandle h, int use_handle, const double* __restrict__ red,
                       DevState* __restrict__ st, double tol, int max_cycles, int init) {
  const bool again = cond_apply(st, red[0], tol, max_cycles, init);
  if (use_handle) cudaGraphSetConditional(h, again ? 1u : 0u);
}

// end of a step: the time, and (track: the step's tolerance loop ran on the
// device) the record of every projection -- how many, how many failed, the
// worst final residual -- that the per-projection statistics overwrite
__device__ __forceinline__ void finish_step(DevState* st, double dt, int track) {
  st->t += dt;
  if (track) {
    st->rec_steps += 1;
    if (!st->converged) st->rec_failed += 1;
    const double m = isfinite(st->res_max) ? st->res_max : INFINITY;
    if (!(m <= st->rec_worst)) st->rec_worst = m;
  }
}

__global__ void k_step_finish(DevState* __restrict__ st, double dt, int track) { finish_step(st, dt, track); }

void launch_cond_init(Solver* s, cudaGraphConditionalHandle h, bool graph) {
  FS_LAUNCH(s, "cond", 0.0,
            k_cond<<<1, 1, 0, s->stream>>>(h, graph ? 1 : 0, s->red_out, s->dev, dev_tol(s),
                                           s->prm.max_cycles, 1));
}
void launch_cond_step(Solver* s, cudaGraphConditionalHandle h, bool graph) {
  FS_LAUNCH(s, "cond", 0.0,
            k_cond<<<1, 1, 0, s->stream>>>(h, graph ? 1 : 0, s->red_out, s->dev, dev_tol(s),
                                           s->prm.max_cycles, 0));
}
void launch_step_finish(Solver* s, double dt) {
  FS_LAUNCH(s, "step_finish", 0.0,
            k_step_finish<<<1, 1, 0, s->stream>>>(s->dev, dt, s->stats_on_device ? 1 : 0));
}

// ------------------------------------------- batched refinement bookkeeping
// One size class of a batch (see fs_multigrid.cu): the refinement residual of
// every member still in its loop as one launch (member = blockIdx.z, each with
// its own reduction), and one kernel that does k_cond's bookkeeping for every
// member and sets the class loop's condition to "any member continues".
__device__ __forceinline__ bool member_in_loop(const DevState* st, int max_cycles) {
  return !st->converged && !st->nonfinite && st->cycles < max_cycles;
}

struct RefineTab {
  struct {
    const float* dh;
    const float* dl;
    const float* ph;
    const float* pl;
    float* r32;
    RedCtx ctx;
    const DevState* st;
  } m[kClassMax];
};

struct CondTab {
  struct {
    const double* red;
    DevState* st;
    double tol;
  } m[kClassMax];
};

__global__ void __launch_bounds__(256, 5) k_refine_class(const RefineTab tab, int nx, int ny, LapScale ks,
                                                      int max_cycles, int quad) {
  const auto& a = tab.m[blockIdx.z];
  if (!member_in_loop(a.st, max_cycles)) return;
  if (quad) refine_init4_body(a.dh, a.dl, a.ph, a.pl, a.r32, nx, ny, ks, a.ctx, CondFold{});
  else refine_init_body(a.dh, a.dl, a.ph, a.pl, a.r32, nx, ny, ks, 0, a.ctx);
}

// one block of kClassMax threads; init = 1 before the loop when the members'
// own k_cond has set their statistics, 2 before the loop doing that here
// (k_cond's init arithmetic), 0 after each cycle
__global__ void __launch_bounds__(kClassMax) k_cond_class(const CondTab tab, int count, int max_cycles,
                                                          cudaGraphConditionalHandle h, int init,
                                                          long long* iterations) {
  const int z = threadIdx.x;
  int again = 0;
  if (z < count) {
    DevState* st = tab.m[z].st;
    if (init == 2) {
      const double m = tab.m[z].red[0];
      st->cycles = 0;
      st->res_initial = m;
      st->res_max = m;
      const bool finite = isfinite(m);
      st->nonfinite = finite ? 0 : 1;
      const double lim = tol_limit(tab.m[z].tol, st);
      st->converged = (finite && m <= lim) ? 1 : 0;
      again = finite && m > lim && 0 < max_cycles;
    } else if (init) {
      again = member_in_loop(st, max_cycles);
    } else if (member_in_loop(st, max_cycles)) {  // this member ran the cycle
      const double m = tab.m[z].red[0];
      st->cycles += 1;
      st->total_cycles += 1;
      st->res_max = m;
      const bool finite = isfinite(m);
      st->nonfinite = finite ? 0 : 1;
      const double lim = tol_limit(tab.m[z].tol, st);
      st->converged = (finite && m <= lim) ? 1 : 0;
      again = finite && m > lim && st->cycles < max_cycles;
    }
  }
  again = __syncthreads_or(again);
  if (threadIdx.x == 0) {
    if (!init) *iterations += 1;
    cudaGraphSetConditional(h, again ? 1u : 0u);
  }
}

void launch_refine_class(Solver* const* ms, int count, cudaStream_t st) {
  Solver* s0 = ms[0];
  const Grid& g = s0->g;
  RefineTab tab{};
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    tab.m[i] = {s->dh, s->dl, s->ph, s->pl, s->r32, red_ctx(s, s->red_out), s->dev};
  }
  const bool quad = g.nx % 4 == 0;
  dim3 grid = quad ? red_grid2(g.nx / 4, g.ny) : red_grid2(g.nx, g.ny);
  grid.z = count;
  k_refine_class<<<grid, kBlock, 0, st>>>(tab, g.nx, g.ny, lap_scale(g), s0->prm.max_cycles, quad ? 1 : 0);
}

void launch_cond_class(Solver* const* ms, int count, cudaStream_t st, cudaGraphConditionalHandle h, int init,
                       long long* iterations) {
  CondTab tab{};
  for (int i = 0; i < count; i++) tab.m[i] = {ms[i]->red_out, ms[i]->dev, dev_tol(ms[i])};
  k_cond_class<<<1, kClassMax, 0, st>>>(tab, count, ms[0]->prm.max_cycles, h, init, iterations);
}

// ---- the rest of a plain class member's step, batched: the divergence of the
// (advected, diffused) velocity, the initial residual from zero pressure, the
// zeroed pressure, and after the loop the gradient subtraction and the step
// finish (k_div_df, k_refine_init with zero_p, launch_fill, k_subgrad_df,
// k_step_finish, one launch each for the whole class)
struct ProjTab {
  struct {
    const float* wu;  // the velocity the projection reads
    const float* wv;
    float* uh;
    float* ul;
    float* vh;
    float* vl;
    float* dh;
    float* dl;
    float* ph;
    float* pl;
    float* r32;
    RedCtx ctx;
    DevState* st;
    df idx, idy;
    double dt;
  } m[kClassMax];
};

__global__ void __launch_bounds__(256) k_div_class(const ProjTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  div_df_body(a.wu, nullptr, a.wv, nullptr, a.dh, a.dl, nx, ny, a.idx, a.idy);
}

__global__ void __launch_bounds__(256) k_refine_zero_class(const ProjTab tab, int nx, int ny, LapScale ks) {
  const auto& a = tab.m[blockIdx.z];
  refine_init_body(a.dh, a.dl, a.ph, a.pl, a.r32, nx, ny, ks, 1, a.ctx);
}

__global__ void k_zero_p_class(const ProjTab tab, int64_t n) {
  const auto& a = tab.m[blockIdx.z];
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    a.ph[k] = 0.f;
    a.pl[k] = 0.f;
  }
}

__global__ void __launch_bounds__(256) k_div_start_class(const ProjTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  div_start4_body(a.wu, a.wv, a.dh, a.dl, a.ph, a.pl, a.r32, nx, ny, a.idx, a.idy, a.ctx);
}

__global__ void __launch_bounds__(256) k_subgrad_class(const ProjTab tab, int nx, int ny) {
  const auto& a = tab.m[blockIdx.z];
  if ((nx & 3) == 0)
    subgrad4_body(a.wu, nullptr, a.wv, nullptr, a.ph, a.pl, a.uh, a.ul, a.vh, a.vl, nx, ny, a.idx, a.idy);
  else
    subgrad_df_body(a.wu, nullptr, a.wv, nullptr, a.ph, a.pl, a.uh, a.ul, a.vh, a.vl, nx, ny, a.idx, a.idy);
}

__global__ void k_finish_class(const ProjTab tab, int count) {
  const int z = threadIdx.x;
  if (z < count) finish_step(tab.m[z].st, tab.m[z].dt, 1);
}

static ProjTab proj_tab(Solver* const* ms, int count, const float* const* wu, const float* const* wv,
                        const double* dts) {
  ProjTab tab{};
  for (int i = 0; i < count; i++) {
    Solver* s = ms[i];
    tab.m[i] = {wu[i],  wv[i],  s->u,  s->ulo, s->v,   s->vlo, s->dh,
                s->dl,  s->ph,  s->pl, s->r32, red_ctx(s, s->red_out), s->dev,
                df_host(s->g.idxd), df_host(s->g.idyd), dts[i]};
  }
  return tab;
}

// before the loop: divergence, initial residual (zero pressure), zeroed pressure
// (returns the number of launches)
int launch_front_project_class(Solver* const* ms, int count, const float* const* wu, const float* const* wv,
                               const double* dts, cudaStream_t st) {
  const Grid& g = ms[0]->g;
  const ProjTab tab = proj_tab(ms, count, wu, wv, dts);
  if (g.nx % 4 == 0) {  // all three in one pass
    dim3 gq = red_grid2(g.nx / 4, g.ny);
    gq.z = count;
    k_div_start_class<<<gq, kBlock, 0, st>>>(tab, g.nx, g.ny);
    return 1;
  }
  dim3 g2 = grid2d(g.nx, g.ny, kBlock);
  g2.z = count;
  k_div_class<<<g2, kBlock, 0, st>>>(tab, g.nx, g.ny);
  dim3 gr = red_grid2(g.nx, g.ny);
  gr.z = count;
  k_refine_zero_class<<<gr, kBlock, 0, st>>>(tab, g.nx, g.ny, lap_scale(g));
  k_zero_p_class<<<dim3(fill_blocks(ms[0]->n), 1, count), 256, 0, st>>>(tab, ms[0]->n);
  return 3;
}

// after the loop: gradient subtraction and the step finish
void launch_back_class(Solver* const* ms, int count, const float* const* wu, const float* const* wv,
                       const double* dts, cudaStream_t st) {
  const Grid& g = ms[0]->g;
  const ProjTab tab = proj_tab(ms, count, wu, wv, dts);
  dim3 g2 = grid2d(g.nx % 4 == 0 ? g.nx / 4 : g.nx, g.ny, kBlock);  // four cells per thread when nx % 4 == 0
  g2.z = count;
  k_subgrad_class<<<g2, kBlock, 0, st>>>(tab, g.nx, g.ny);
  k_finish_class<<<1, kClassMax, 0, st>>>(tab, count);
}


// ---------------------------------------------------------------- conversion
__global__ void k_convert(const void* src, int sf64, void* dst, int df64, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double x = sf64 ? ((const double*)src)[k] : (double)((const float*)src)[k];
    if (df64) ((double*)dst)[k] = x;
    else ((float*)dst)[k] = (float)x;
  }
}
void launch_convert(Solver* s, const void* src, int src_f64, void* dst, int dst_f64, int64_t n) {
  FS_LAUNCH(s, "convert", (double)n * ((src_f64 ? 8 : 4) + (dst_f64 ? 8 : 4)),
            k_convert<<<fill_blocks(n), 256, 0, s->stream>>>(src, src_f64, dst, dst_f64, n));
}

// ------------------------------------------------------------- V-cycle driver
static void mg_smooth(Solver* s, Level& L, int sweeps) {
  bool odd = (L.n & 1) != 0;
  for (int k = 0; k < sweeps; k++)
    for (int colour = 0; colour < 2; colour++) {
      if (!odd) {
        launch_rb_half(s, L.x, L.rhs, L.x, L.h2, colour, L.n, L.n);
      } else {
        launch_rb_half(s, L.x, L.rhs, L.x2, L.h2, colour, L.n, L.n);
        float* t = L.x; L.x = L.x2; L.x2 = t;  // two swaps per sweep: x returns home
      }
    }
}

// encodeVCycle (multigrid.js:277-330): the solution accumulates in lev[0].x
void mg_vcycle(Solver* s) {
  std::vector<Level>& L = s->lev;
  int nl = (int)L.size();
  const fs_params& P = s->prm;
  for (int l = 0; l < nl - 1; l++) {
    mg_smooth(s, L[l], P.mg_pre_smooth);
    launch_residual(s, L[l].x, L[l].rhs, s->scratch, L[l].h2, L[l].n);
    launch_restrict(s, s->scratch, L[l + 1].rhs, L[l + 1].n);
    launch_fill(s, L[l + 1].x, 0.f, (int64_t)L[l + 1].n * L[l + 1].n);
  }
  mg_smooth(s, L[nl - 1], P.mg_coarse_sweeps);
  for (int l = nl - 2; l >= 0; l--) {
    launch_prolong_add(s, L[l + 1].x, L[l].x, L[l].n);
    mg_smooth(s, L[l], P.mg_post_smooth);
  }
}

}  // namespace fs
