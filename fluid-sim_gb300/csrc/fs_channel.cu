// fs_channel.cu -- a channel with inflow, outflow and no-slip walls on the
// periodic MAC grid.
//
// The reference is periodic only (README.md:139: the FFT projection and the
// periodic wrap of src/core/grid.js:40).  The channel is built the way
// spectral channel codes build inflow and outflow on periodic domains, with
// the reference's own immersed-boundary operator for the walls:
//  * walls: a slab |y - y_w| <= h_w (periodic distance) of solid at rest,
//    coupled by the direct forcing of the reference's disks
//    (src/cpu/solid.js:165-233): chi = 1/2 (1 - tanh((|dy| - h_w) / w)),
//    w = solid_mask_width cells, u += chi (0 - u) where chi >= 1e-6.  The
//    slab's two edges are the channel's no-slip walls;
//  * inflow / outflow: a fringe strip |x - x_f| <= h_f where the same kind of
//    forcing with a tanh ramp of width r_f drives (u, v) to (U_in, 0).  Flow
//    leaves the domain through the strip and enters again on the other side
//    of it as the uniform inflow u = U_in (fringe-region method: Spalart
//    1988; Nordstrom, Nordin & Henningson, SIAM J. Sci. Comput. 20, 1999).
// Fringe first, then the wall, so the wall holds where both reach.  The
// pressure stays periodic, so the multigrid, the advection tiles and every
// other kernel run unchanged.
#include <math.h>

#include "fs_internal.cuh"

namespace fs {

namespace {

// Face positions relative to the strip centres: an integer offset from the
// cell nearest below the centre (jc, ic) times the spacing, plus that cell's
// own offsets (u and v faces) computed in f64 on the host.  Rounding then
// stays ~1e-9 of the domain, far below the mask widths (a few 1e-3), where
// absolute f32 positions would carry ~4e-7.
struct ChannelDev {
  int jc, ic;
  float wyu, wyv;  // (jc + 1/2) dy - wall_y, jc dy - wall_y
  float fxu, fxv;  // ic dx - fringe_x, (ic + 1/2) dx - fringe_x
  float wh, fh, fr, uin;
};

// k - c wrapped into [-n/2, n/2]
__device__ __forceinline__ int wrap_i(int k, int c, int n) {
  int t = k - c;
  if (2 * t > n) t -= n;
  if (2 * t < -n) t += n;
  return t;
}

// chi of a tanh-edged slab of half-width hw around 0, at signed distance d:
// 1/2 (1 - tanh z) written as 1 / (1 + e^{2z}), the same function without
// the cancellation of 1 - tanh z in f32 where chi is small
__device__ __forceinline__ float slab_chi(float d, float hw, float w) {
  return 1.f / (1.f + expf(2.f * (fabsf(d) - hw) / w));
}

// The cells either strip can reach: the rows of the wall band (every column)
// and the columns of the fringe band outside those rows, as one launch of
// 32x8 blocks -- blocks [0, na) cover the rows, the rest the columns.  Bands
// are given by their first index and length, both wrapping.
struct Bands {
  int j0, nw;  // wall rows j0 .. j0 + nw - 1 (mod ny)
  int i0, nf;  // fringe columns i0 .. i0 + nf - 1 (mod nx)
  int gxa, na; // part A: blocks per row band line, blocks in all
  int gxb;     // part B: blocks per column band line
};

__global__ void __launch_bounds__(256)
    k_channel(float* __restrict__ u, float* __restrict__ v, int nx, int ny, float dx, float dy, ChannelDev c,
              float w, Bands b) {
  int i, j;
  const int blk = blockIdx.x;
  if (blk < b.na) {
    const int bx = blk % b.gxa, by = blk / b.gxa;
    i = bx * 32 + threadIdx.x;
    const int t = by * 8 + threadIdx.y;
    if (i >= nx || t >= b.nw) return;
    j = b.j0 + t;
    if (j >= ny) j -= ny;
  } else {
    const int k = blk - b.na, bx = k % b.gxb, by = k / b.gxb;
    const int ti = bx * 32 + threadIdx.x, t = by * 8 + threadIdx.y;
    if (ti >= b.nf || t >= ny - b.nw) return;
    i = b.i0 + ti;
    if (i >= nx) i -= nx;
    j = b.j0 + b.nw + t;
    if (j >= ny) j -= ny;
  }
  // u face (i h, (j+1/2) h), v face ((i+1/2) h, j h), relative to the strips
  const float ty = (float)wrap_i(j, c.jc, ny), tx = (float)wrap_i(i, c.ic, nx);
  const float duy = fmaf(ty, dy, c.wyu), dvy = fmaf(ty, dy, c.wyv);
  const float dux = fmaf(tx, dx, c.fxu), dvx = fmaf(tx, dx, c.fxv);
  const int64_t k = (int64_t)j * nx + i;
  float uu = u[k], vv = v[k];
  const float fu = slab_chi(dux, c.fh, c.fr), fv = slab_chi(dvx, c.fh, c.fr);
  if (fu >= 1e-6f) uu += fu * (c.uin - uu);
  if (fv >= 1e-6f) vv += fv * (0.f - vv);
  const float wu = slab_chi(duy, c.wh, w), wv = slab_chi(dvy, c.wh, w);
  if (wu >= 1e-6f) uu += wu * (0.f - uu);
  if (wv >= 1e-6f) vv += wv * (0.f - vv);
  u[k] = uu;
  v[k] = vv;
}

// the band of indices k (faces at k h and (k + 1/2) h) within reach of a
// strip centred at x0 on a periodic axis of n cells: first index and count,
// one cell of margin each side (the kernel tests every face again)
void band_of(double x0, double reach, double h, int n, int* first, int* count) {
  const int lo = (int)floor((x0 - reach) / h) - 1, hi = (int)ceil((x0 + reach) / h) + 1;
  if (hi - lo + 1 >= n) {
    *first = 0;
    *count = n;
    return;
  }
  *first = ((lo % n) + n) % n;
  *count = hi - lo + 1;
}

}  // namespace

int channel_set(Solver* s, const fs_channel* c) {
  if (!c) {
    s->channel_on = false;
    return FS_OK;
  }
  s->channel = *c;
  s->channel_on = true;
  return FS_OK;
}

void launch_channel(Solver* s, float* u, float* v) {
  const Grid& g = s->g;
  const fs_channel& c = s->channel;
  ChannelDev d{};
  d.jc = (int)floor(c.wall_y / g.dyd);
  d.ic = (int)floor(c.fringe_x / g.dxd);
  d.wyu = (float)((d.jc + 0.5) * g.dyd - c.wall_y);
  d.wyv = (float)(d.jc * g.dyd - c.wall_y);
  d.fxu = (float)(d.ic * g.dxd - c.fringe_x);
  d.fxv = (float)((d.ic + 0.5) * g.dxd - c.fringe_x);
  d.jc = ((d.jc % g.ny) + g.ny) % g.ny;
  d.ic = ((d.ic % g.nx) + g.nx) % g.nx;
  d.wh = (float)c.wall_half;
  d.fh = (float)c.fringe_half;
  d.fr = (float)c.fringe_ramp;
  d.uin = (float)c.inflow_u;
  const double w = s->prm.solid_mask_width * g.dxd;
  // chi >= 1e-6 needs (|d| - half) / width <= atanh(1 - 2e-6) < 7.3; the bands reach 8.5
  // widths (chi down to 4e-8), so f32 rounding of a face position cannot drop one
  Bands b{};
  band_of(c.wall_y, c.wall_half + 8.5 * w, g.dyd, g.ny, &b.j0, &b.nw);
  band_of(c.fringe_x, c.fringe_half + 8.5 * c.fringe_ramp, g.dxd, g.nx, &b.i0, &b.nf);
  b.gxa = (g.nx + 31) / 32;
  b.na = b.gxa * ((b.nw + 7) / 8);
  b.gxb = (b.nf + 31) / 32;
  const int nb = b.gxb * ((g.ny - b.nw + 7) / 8);
  if (b.na + nb == 0) return;
  // algorithmic bytes: u, v read and written on the cells of the two bands
  const double cells = (double)b.nw * g.nx + (double)b.nf * (g.ny - b.nw);
  FS_LAUNCH(s, "channel", 16.0 * cells,
            k_channel<<<b.na + nb, dim3(32, 8), 0, s->stream>>>(u, v, g.nx, g.ny, g.dx, g.dy, d, (float)w, b));
}

}  // namespace fs
