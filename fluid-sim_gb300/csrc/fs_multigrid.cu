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
//               with the whole CTA, levels <= 16 (including the 40 coarse
//               sweeps) with one warp and __syncwarp between half-sweeps;
//   k_mg_up     per level n > 64: prolongation-add of the coarse correction on
//               the tile plus a halo of 2*post, then the post-smoothing sweeps.
//
// The per-cell arithmetic is fs_stencil.cuh, shared with the one-pass-per-
// operation kernels, so the fused cycle reproduces them bit for bit.
//
// Shared-memory layout: each tile row is split into its even and odd columns
// so that the lanes of a warp, which update cells of one colour in one row
// (stride 2 in the row), hit consecutive words.
#include <utility>

#include "fs_internal.cuh"
#include "fs_stencil.cuh"

namespace fs {

constexpr int kTile = 64;  // fine cells per tile side (even)

__device__ __forceinline__ int wrap_n(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// R x R region with split columns: cell (li, lj) at lj*R + (li&1)*(R/2) + (li>>1)
template <int R>
__device__ __forceinline__ int sidx(int li, int lj) {
  return lj * R + (li & 1) * (R / 2) + (li >> 1);
}

// One red-black half-sweep of colour c over li, lj in [1, R-2] (in place).
// par0 is the parity of the global index of local (0, 0) (n even, so the
// parity survives the periodic wrap).  Cells whose neighbours are stale give
// stale values; they lie outside the valid region and are never written back.
template <int R>
__device__ __forceinline__ void rb_half_smem(float* xs, const float* rs, int c, int par0, float h2) {
  constexpr int W = R - 2;   // rows / columns updated
  constexpr int S = W / 2;   // cells of one colour per row
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  for (int idx = tid; idx < W * S; idx += nthr) {
    int row = idx / S, m = idx - row * S;
    int lj = 1 + row;
    int li = (((par0 + 1 + lj) & 1) == c ? 1 : 2) + 2 * m;
    int k = sidx<R>(li, lj);
    xs[k] = gs_update(xs[k], xs[sidx<R>(li - 1, lj)], xs[sidx<R>(li + 1, lj)], xs[sidx<R>(li, lj - 1)],
                      xs[sidx<R>(li, lj + 1)], rs[k], h2);
  }
}

// ------------------------------------------------------------------ down
// H = 2 * pre + 1.  xin == nullptr means the level starts from zero; otherwise
// xin and xout must differ (the halo of a tile is another tile's interior).
template <int H>
__global__ void __launch_bounds__(256) k_mg_down(const float* __restrict__ rhs, const float* __restrict__ xin,
                                                 float* __restrict__ xout, float* __restrict__ crhs, int n,
                                                 float h2, int pre) {
  constexpr int R = kTile + 2 * H;
  __shared__ float xs[R * R];
  __shared__ float rs[R * R];
  const int i0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
  const int gi0 = i0 - H, gj0 = j0 - H;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  for (int k = tid; k < R * R; k += nthr) {
    int lj = k / R, li = k - lj * R;
    int64_t g = (int64_t)wrap_n(gj0 + lj, n) * n + wrap_n(gi0 + li, n);
    int s = sidx<R>(li, lj);
    rs[s] = __ldg(rhs + g);
    xs[s] = xin ? __ldg(xin + g) : 0.f;
  }
  __syncthreads();
  const int par0 = (gi0 + gj0) & 1;
  for (int s = 0; s < 2 * pre; s++) {
    rb_half_smem<R>(xs, rs, s & 1, par0, h2);
    __syncthreads();
  }
  for (int k = tid; k < kTile * kTile; k += nthr) {
    int y = k / kTile, x = k - y * kTile;
    int gi = i0 + x, gj = j0 + y;
    if (gi < n && gj < n) xout[(int64_t)gj * n + gi] = xs[sidx<R>(H + x, H + y)];
  }
  // residual on each 2x2 block and its restriction (multigrid.js:48-93)
  const int nc = n >> 1;
  for (int k = tid; k < (kTile / 2) * (kTile / 2); k += nthr) {
    int cj = k / (kTile / 2), ci = k - cj * (kTile / 2);
    float r4[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int li = H + 2 * ci + (q & 1), lj = H + 2 * cj + (q >> 1);
      r4[q] = residual_at(xs[sidx<R>(li, lj)], xs[sidx<R>(li - 1, lj)], xs[sidx<R>(li + 1, lj)],
                          xs[sidx<R>(li, lj - 1)], xs[sidx<R>(li, lj + 1)], rs[sidx<R>(li, lj)], h2);
    }
    int gci = (i0 >> 1) + ci, gcj = (j0 >> 1) + cj;
    if (gci < nc && gcj < nc) crhs[(int64_t)gcj * nc + gci] = restrict4(r4[0], r4[1], r4[2], r4[3]);
  }
}

// -------------------------------------------------------------------- up
// H = 2 * post.  x += P(coarse) on the region, then the post sweeps.  xin and
// xout must differ: the halo of a tile is another tile's interior.
template <int H>
__global__ void __launch_bounds__(256) k_mg_up(const float* __restrict__ rhs, const float* __restrict__ xin,
                                               float* __restrict__ xout, const float* __restrict__ xc, int n,
                                               float h2, int post) {
  constexpr int R = kTile + 2 * H;
  __shared__ float xs[R * R];
  __shared__ float rs[R * R];
  const int i0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
  const int gi0 = i0 - H, gj0 = j0 - H;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int nc = n >> 1;
  for (int k = tid; k < R * R; k += nthr) {
    int lj = k / R, li = k - lj * R;
    int gi = wrap_n(gi0 + li, n), gj = wrap_n(gj0 + lj, n);
    int64_t g = (int64_t)gj * n + gi;
    // PROLONG (multigrid.js:99-131): sample at ((i+1/2)/2 - 1/2, (j+1/2)/2 - 1/2)
    int ci0 = (gi & 1) ? (gi >> 1) : (gi >> 1) - 1;
    int cj0 = (gj & 1) ? (gj >> 1) : (gj >> 1) - 1;
    float fx = (gi & 1) ? 0.25f : 0.75f, fy = (gj & 1) ? 0.25f : 0.75f;
    int x0 = ci0 < 0 ? ci0 + nc : ci0, x1 = ci0 + 1 >= nc ? ci0 + 1 - nc : ci0 + 1;
    int y0 = cj0 < 0 ? cj0 + nc : cj0, y1 = cj0 + 1 >= nc ? cj0 + 1 - nc : cj0 + 1;
    float p = prolong_val(__ldg(xc + (int64_t)y0 * nc + x0), __ldg(xc + (int64_t)y0 * nc + x1),
                          __ldg(xc + (int64_t)y1 * nc + x0), __ldg(xc + (int64_t)y1 * nc + x1), fx, fy);
    int s = sidx<R>(li, lj);
    xs[s] = __fadd_rn(__ldg(xin + g), p);
    rs[s] = __ldg(rhs + g);
  }
  __syncthreads();
  const int par0 = (gi0 + gj0) & 1;
  for (int s = 0; s < 2 * post; s++) {
    rb_half_smem<R>(xs, rs, s & 1, par0, h2);
    __syncthreads();
  }
  for (int k = tid; k < kTile * kTile; k += nthr) {
    int y = k / kTile, x = k - y * kTile;
    int gi = i0 + x, gj = j0 + y;
    if (gi < n && gj < n) xout[(int64_t)gj * n + gi] = xs[sidx<R>(H + x, H + y)];
  }
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

__device__ void bottom_smooth(float* sm, const BottomLevels& L, int l, int sweeps, Group G) {
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
        x[k] = gs_update(x[k], x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[k], h2);
      }
    } else {
      for (int k = G.tid; k < n * n; k += G.nthr) {
        int j = k / n, i = k - j * n;
        float cur = x[k];
        if (((i + j) & 1) != c) { x2[k] = cur; continue; }
        int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
        int jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
        x2[k] = gs_update(cur, x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[k], h2);
      }
      G.sync();
      float* t = x; x = x2; x2 = t;  // two swaps per sweep: x is back in off_x at the end
    }
    G.sync();
  }
}

__device__ void bottom_restrict(float* sm, const BottomLevels& L, int l, Group G) {
  const int n = L.n[l], nc = L.n[l + 1];
  const float h2 = L.h2[l];
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
      r4[q] = residual_at(x[j * n + i], x[j * n + im], x[j * n + ip], x[jm * n + i], x[jp * n + i], r[j * n + i], h2);
    }
    cr[k] = restrict4(r4[0], r4[1], r4[2], r4[3]);
    cx[k] = 0.f;
  }
  G.sync();
}

__device__ void bottom_prolong(float* sm, const BottomLevels& L, int l, Group G) {
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

__global__ void __launch_bounds__(1024) k_mg_bottom(const float* __restrict__ rhs_top, float* __restrict__ x_top,
                                                    int has_x, BottomLevels L, int pre, int post, int coarse) {
  extern __shared__ float sm[];
  const int tid = threadIdx.x;
  const Group CTA{tid, (int)blockDim.x, false};
  const Group W0{tid, 32, true};
  {
    const int n = L.n[0];
    for (int k = tid; k < n * n; k += CTA.nthr) {
      sm[L.off_r[0] + k] = __ldg(rhs_top + k);
      sm[L.off_x[0] + k] = has_x ? x_top[k] : 0.f;
    }
  }
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
    for (int k = tid; k < n * n; k += CTA.nthr) x_top[k] = sm[L.off_x[0] + k];
  }
}

// ------------------------------------------------------------------ host
static const dim3 kTileBlock(32, 8);

template <int H>
static void down(Solver* s, Level& L, const Level& C, bool has_x) {
  dim3 grid((L.n + kTile - 1) / kTile, (L.n + kTile - 1) / kTile);
  double bytes = (double)L.n * L.n * (has_x ? 12.0 : 8.0) + (double)C.n * C.n * 4.0;
  float* out = has_x ? L.x2 : L.x;
  FS_LAUNCH(s, "mg_down", bytes,
            k_mg_down<H><<<grid, kTileBlock, 0, s->stream>>>(L.rhs, has_x ? L.x : nullptr, out, C.rhs, L.n,
                                                             L.h2, s->prm.mg_pre_smooth));
  if (has_x) std::swap(L.x, L.x2);
}

template <int H>
static void up(Solver* s, Level& L, const Level& C) {
  dim3 grid((L.n + kTile - 1) / kTile, (L.n + kTile - 1) / kTile);
  double bytes = (double)L.n * L.n * 12.0 + (double)C.n * C.n * 4.0;
  FS_LAUNCH(s, "mg_up", bytes,
            k_mg_up<H><<<grid, kTileBlock, 0, s->stream>>>(L.rhs, L.x, L.x2, C.x, L.n, L.h2,
                                                           s->prm.mg_post_smooth));
  std::swap(L.x, L.x2);
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

void mg_vcycle_fused(Solver* s, bool first_has_x) {
  std::vector<Level>& L = s->lev;
  const int lb = bottom_first_level(s);
  const fs_params& P = s->prm;
  for (int l = 0; l < lb; l++) {
    bool hx = l == 0 && first_has_x;
    switch (P.mg_pre_smooth) {
      case 1: down<3>(s, L[l], L[l + 1], hx); break;
      case 2: down<5>(s, L[l], L[l + 1], hx); break;
      default: down<7>(s, L[l], L[l + 1], hx); break;
    }
  }
  BottomLevels B;
  size_t smem = bottom_layout(s, &B);
  int nb = L[lb].n;
  int threads = std::min(1024, std::max(32, ((nb * nb / 4 + 31) / 32) * 32));
  bool hx = lb == 0 && first_has_x;
  double bytes = (double)nb * nb * (hx ? 12.0 : 8.0);
  FS_LAUNCH(s, "mg_bottom", bytes,
            k_mg_bottom<<<1, threads, smem, s->stream>>>(L[lb].rhs, L[lb].x, hx ? 1 : 0, B, P.mg_pre_smooth,
                                                         P.mg_post_smooth, P.mg_coarse_sweeps));
  for (int l = lb - 1; l >= 0; l--) {
    switch (P.mg_post_smooth) {
      case 1: up<2>(s, L[l], L[l + 1]); break;
      case 2: up<4>(s, L[l], L[l + 1]); break;
      default: up<6>(s, L[l], L[l + 1]); break;
    }
  }
}

}  // namespace fs
