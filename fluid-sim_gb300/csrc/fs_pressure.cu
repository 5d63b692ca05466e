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

#include "fs_internal.cuh"

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
template void launch_divergence<float, double>(Solver*, const float*, const float*, double*);
template void launch_divergence<double, double>(Solver*, const double*, const double*, double*);

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

__global__ void __launch_bounds__(256)
    k_subgrad_mixed(const float* __restrict__ wu, const float* __restrict__ wv, const double* __restrict__ p,
                    double* __restrict__ ou, double* __restrict__ ov, int nx, int ny, double idx,
                    double idy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, jm = j == 0 ? ny - 1 : j - 1;
  int64_t c = (int64_t)j * nx + i;
  double pc = __ldg(p + c);
  ou[c] = (double)__ldg(wu + c) - (pc - __ldg(p + (int64_t)j * nx + im)) * idx;
  ov[c] = (double)__ldg(wv + c) - (pc - __ldg(p + (int64_t)jm * nx + i)) * idy;
}

void launch_subtract_gradient_f32(Solver* s, const float* wu, const float* wv, const float* p,
                                  float* ou, float* ov) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "subtract_gradient", (double)s->n * 20,
            k_subgrad_f32<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(wu, wv, p, ou, ov, g.nx,
                                                                                g.ny, g.idx, g.idy));
}
void launch_subtract_gradient_mixed(Solver* s, const float* wu, const float* wv, const double* p,
                                    double* ou, double* ov) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "subtract_gradient", (double)s->n * 32,
            k_subgrad_mixed<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                wu, wv, p, ou, ov, g.nx, g.ny, g.idxd, g.idyd));
}

// ----------------------------------------------------------------- smoothers
// damped Jacobi, omega = 1 (shaders.js:302-325)
__global__ void __launch_bounds__(256) k_jacobi(const float* __restrict__ p, const float* __restrict__ d,
                                                float* __restrict__ o, int nx, int ny, float h2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
  int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
  int64_t r = (int64_t)j * nx;
  float s = __ldg(p + r + im) + __ldg(p + r + ip) + __ldg(p + (int64_t)jm * nx + i) +
            __ldg(p + (int64_t)jp * nx + i);
  float jac = (s - h2 * __ldg(d + r + i)) * 0.25f;
  float cur = __ldg(p + r + i);
  o[r + i] = cur + (jac - cur);
}

void launch_jacobi(Solver* s, const float* p, const float* d, float* out, float h2, int nx, int ny) {
  FS_LAUNCH(s, "jacobi", (double)nx * ny * 12,
            k_jacobi<<<grid2d(nx, ny, kBlock), kBlock, 0, s->stream>>>(p, d, out, nx, ny, h2));
}

// one red-black colour (shaders.js:340-372, omega = 1); dst may equal src on even grids
__global__ void __launch_bounds__(256) k_rb_half(const float* src, const float* __restrict__ d, float* dst,
                                                 int nx, int ny, float h2, int colour) {
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
  float s = src[r + im] + src[r + ip] + src[(int64_t)jm * nx + i] + src[(int64_t)jp * nx + i];
  float gs = (s - h2 * __ldg(d + r + i)) * 0.25f;
  dst[r + i] = cur + (gs - cur);
}

void launch_rb_half(Solver* s, const float* src, const float* d, float* dst, float h2, int colour,
                    int nx, int ny) {
  FS_LAUNCH(s, "rb_half", (double)nx * ny * (src == dst ? 6 : 12),
            k_rb_half<<<grid2d(nx, ny, kBlock), kBlock, 0, s->stream>>>(src, d, dst, nx, ny, h2, colour));
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
  float lap = (__ldg(x + r + im) + __ldg(x + r + ip) + __ldg(x + (int64_t)jm * n + i) +
               __ldg(x + (int64_t)jp * n + i) - 4.f * __ldg(x + r + i)) / h2;
  o[r + i] = __ldg(rhs + r + i) - lap;
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
  float s = 0.f;
  s = s + __ldg(f + r0 + 2 * i);
  s = s + __ldg(f + r0 + 2 * i + 1);
  s = s + __ldg(f + r1 + 2 * i);
  s = s + __ldg(f + r1 + 2 * i + 1);
  c[(int64_t)j * nc + i] = s * 0.25f;
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
  float top = a * (1.f - fx) + b * fx, bot = cc * (1.f - fx) + d * fx;
  int64_t k = (int64_t)j * nf + i;
  f[k] = f[k] + (top * (1.f - fy) + bot * fy);
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

// ------------------------------------------------------------- reductions
// Per-block partials, then the last block to finish folds them in a fixed
// order, so every reduction is deterministic run to run.
struct RedCtx {
  double* partials;  // 2 per block
  unsigned* counter;
  double* out;       // out[0], out[1]
};

template <int OP>  // 0: max of a (b ignored), 1: sums of a and b
__device__ __forceinline__ void block_reduce_finish(double a, double b, RedCtx ctx) {
  __shared__ double sa[32], sb[32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) {
    double oa = __shfl_xor_sync(0xffffffffu, a, o), ob = __shfl_xor_sync(0xffffffffu, b, o);
    if (OP == 0) a = fmax(a, oa); else { a += oa; b += ob; }
  }
  int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int nwarp = (blockDim.x * blockDim.y + 31) >> 5;
  if (lane == 0) { sa[warp] = a; sb[warp] = b; }
  __syncthreads();
  int bid = blockIdx.y * gridDim.x + blockIdx.x, nblk = gridDim.x * gridDim.y;
  if (tid == 0) {
    double ta = sa[0], tb = sb[0];
    for (int w = 1; w < nwarp; w++) {
      if (OP == 0) ta = fmax(ta, sa[w]); else { ta += sa[w]; tb += sb[w]; }
    }
    ctx.partials[2 * bid] = ta;
    ctx.partials[2 * bid + 1] = tb;
    __threadfence();
    unsigned done = atomicAdd(ctx.counter, 1u);
    last = done == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // fold partials: each thread a strided subset in fixed order, then the warps
  double ta = OP == 0 ? 0.0 : 0.0, tb = 0.0;
  int nthr = blockDim.x * blockDim.y;
  for (int k = tid; k < nblk; k += nthr) {
    double pa = ((volatile double*)ctx.partials)[2 * k], pb = ((volatile double*)ctx.partials)[2 * k + 1];
    if (OP == 0) ta = fmax(ta, pa); else { ta += pa; tb += pb; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double oa = __shfl_xor_sync(0xffffffffu, ta, o), ob = __shfl_xor_sync(0xffffffffu, tb, o);
    if (OP == 0) ta = fmax(ta, oa); else { ta += oa; tb += ob; }
  }
  __syncthreads();
  if (lane == 0) { sa[warp] = ta; sb[warp] = tb; }
  __syncthreads();
  if (tid == 0) {
    double fa = sa[0], fb = sb[0];
    for (int w = 1; w < nwarp; w++) {
      if (OP == 0) fa = fmax(fa, sa[w]); else { fa += sa[w]; fb += sb[w]; }
    }
    ctx.out[0] = fa;
    if (OP == 1) ctx.out[1] = fb;
    *ctx.counter = 0;  // ready for the next reduction
  }
}

// NaN must not vanish in a max: fmax(x, NaN) = x, so NaN is mapped to +inf.
__device__ __forceinline__ double absnan(double x) { return x != x ? INFINITY : fabs(x); }

template <class T>
__global__ void __launch_bounds__(256) k_absmax(const T* __restrict__ x, int64_t n, RedCtx ctx) {
  double m = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, absnan((double)__ldg(x + k)));
  block_reduce_finish<0>(m, 0.0, ctx);
}

static RedCtx red_ctx(Solver* s, double* out) {
  return RedCtx{s->red_partials, (unsigned*)(s->red_partials + 2 * s->red_cap), out};
}
static int red_blocks(Solver* s, int64_t n) {
  int64_t b = (n + 255) / 256;
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
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  double num = 0.0, den = 0.0;
  if (i < nx && j < ny) {
    int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
    int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t r = (int64_t)j * nx;
    double lap = ((double)p[r + im] + (double)p[r + ip] + (double)p[(int64_t)jm * nx + i] +
                  (double)p[(int64_t)jp * nx + i] - 4.0 * (double)p[r + i]) / h2;
    double dd = (double)d[r + i];
    double rr = lap - dd;
    num = rr * rr;
    den = dd * dd;
  }
  block_reduce_finish<1>(num, den, ctx);
}

void launch_poisson_norms(Solver* s, const float* p, const float* d, float h2f, double h2) {
  (void)h2f;
  const Grid& g = s->g;
  dim3 grid = grid2d(g.nx, g.ny, kBlock);
  if ((int64_t)grid.x * grid.y > s->red_cap) return;  // partial buffer sized for this grid at create
  FS_LAUNCH(s, "poisson_norms", (double)s->n * 8,
            k_poisson_norms<<<grid, kBlock, 0, s->stream>>>(p, d, g.nx, g.ny, h2, red_ctx(s, s->red_out)));
}

// ------------------------------------------------ mixed-precision refinement
// r = d - lap(p) in f64; r32 = (float) r; max|r| reduced.  With zero_p, r = d.
__global__ void __launch_bounds__(256) k_refine_init(const double* __restrict__ d, const double* __restrict__ p,
                                                     float* __restrict__ r32, int nx, int ny, double ih2x,
                                                     double ih2y, int zero_p, RedCtx ctx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  double m = 0.0;
  if (i < nx && j < ny) {
    int64_t r = (int64_t)j * nx, c = r + i;
    double res = __ldg(d + c);
    if (!zero_p) {
      int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
      int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
      double pc = __ldg(p + c);
      double lap = (__ldg(p + r + im) - 2.0 * pc + __ldg(p + r + ip)) * ih2x +
                   (__ldg(p + (int64_t)jm * nx + i) - 2.0 * pc + __ldg(p + (int64_t)jp * nx + i)) * ih2y;
      res = res - lap;
    }
    r32[c] = (float)res;
    m = absnan(res);
  }
  block_reduce_finish<0>(m, 0.0, ctx);
}

// p' = p + e; r = d - lap(p') in f64; r32 = (float) r; max|r| reduced
__global__ void __launch_bounds__(256)
    k_refine_update(const double* __restrict__ p, const float* __restrict__ e, const double* __restrict__ d,
                    double* __restrict__ po, float* __restrict__ r32, int nx, int ny, double ih2x,
                    double ih2y, RedCtx ctx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  double m = 0.0;
  if (i < nx && j < ny) {
    int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
    int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t r = (int64_t)j * nx, c = r + i;
    int64_t cl = r + im, cr = r + ip, cb = (int64_t)jm * nx + i, ct = (int64_t)jp * nx + i;
    double pc = __ldg(p + c) + (double)__ldg(e + c);
    double pl = __ldg(p + cl) + (double)__ldg(e + cl);
    double pr = __ldg(p + cr) + (double)__ldg(e + cr);
    double pb = __ldg(p + cb) + (double)__ldg(e + cb);
    double pt = __ldg(p + ct) + (double)__ldg(e + ct);
    double lap = (pl - 2.0 * pc + pr) * ih2x + (pb - 2.0 * pc + pt) * ih2y;
    double res = __ldg(d + c) - lap;
    po[c] = pc;
    r32[c] = (float)res;
    m = absnan(res);
  }
  block_reduce_finish<0>(m, 0.0, ctx);
}

void launch_refine_init(Solver* s, const double* d, const double* p, float* r32, bool zero_p) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "refine_init", (double)s->n * (zero_p ? 12 : 20),
            k_refine_init<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                d, p, r32, g.nx, g.ny, g.idxd * g.idxd, g.idyd * g.idyd, zero_p ? 1 : 0,
                red_ctx(s, s->red_out)));
}

void launch_refine_update(Solver* s, const double* p_in, const float* e, const double* d,
                          double* p_out, float* r32) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "refine_update", (double)s->n * 32,
            k_refine_update<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                p_in, e, d, p_out, r32, g.nx, g.ny, g.idxd * g.idxd, g.idyd * g.idyd,
                red_ctx(s, s->red_out)));
}

// max|d - lap p| over an f32 pair (tolerance loop of the F32 mode)
__global__ void __launch_bounds__(256) k_absmax_res32(const float* __restrict__ p, const float* __restrict__ d,
                                                      int nx, int ny, float ih2x, float ih2y, RedCtx ctx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  double m = 0.0;
  if (i < nx && j < ny) {
    int im = i == 0 ? nx - 1 : i - 1, ip = i + 1 == nx ? 0 : i + 1;
    int jm = j == 0 ? ny - 1 : j - 1, jp = j + 1 == ny ? 0 : j + 1;
    int64_t r = (int64_t)j * nx;
    float pc = p[r + i];
    float lap = (p[r + im] - 2.f * pc + p[r + ip]) * ih2x + (p[(int64_t)jm * nx + i] - 2.f * pc + p[(int64_t)jp * nx + i]) * ih2y;
    m = absnan((double)(d[r + i] - lap));
  }
  block_reduce_finish<0>(m, 0.0, ctx);
}

void launch_absmax_residual32(Solver* s, const float* p, const float* d) {
  const Grid& g = s->g;
  FS_LAUNCH(s, "absmax_residual", (double)s->n * 8,
            k_absmax_res32<<<grid2d(g.nx, g.ny, kBlock), kBlock, 0, s->stream>>>(
                p, d, g.nx, g.ny, g.idx * g.idx, g.idy * g.idy, red_ctx(s, s->red_out)));
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
