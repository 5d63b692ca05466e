// fs_band.cu -- band-limited random forcing renewed every step, plus linear
// drag (the forced-turbulence driver of the reference: bandForcing and
// linearDrag, src/cpu/solver.js:179-237, called once per step with seed++ by
// validate/longrun-spectrum.js:65-67).
//
// The forcing is a sum of M plane-wave streamfunction modes,
//     psi = sum_m A_m cos(kx_m x + ky_m y + phi_m),
// added to the velocity as its curl (so it is divergence-free),
//     u += s * sum_m A_m ( ky_m/|k_m|) cos(kx_m x_u + ky_m y_u + phi_m),
//     v += s * sum_m A_m (-kx_m/|k_m|) cos(kx_m x_v + ky_m y_v + phi_m),
// s = amp dt / sqrt(M), at the u faces (i h, (j+1/2) h) and v faces
// ((i+1/2) h, j h) (src/core/grid.js uX/uY/vX/vY), then u *= exp(-drag dt).
//
// Two mode generators, both on the device from (seed, step) so a captured
// step renews the forcing with no host work:
//  * FS_BAND_REFERENCE -- bandForcing's own: 24 modes from the reference's
//    32-bit LCG seeded with seed + step, |k| = kf + (r - 1/2) 2 width at a
//    random angle, rounded to integers, random phase, A = 1;
//  * FS_BAND_GAUSSIAN -- every integer (kx, ky) with kf - width <= |k| <=
//    kf + width, each with a complex Gaussian amplitude (sigma 1 per part)
//    from Philox4x32-10 keyed by the seed with counter (step, mode); A e^{i phi}
//    is that amplitude (Box-Muller gives A and phi directly).
//
// Evaluation is separable: cos(kx x + ky y + phi) = Re(e^{i phi} e^{i kx x}
// e^{i ky y}).  A first kernel forms, for every ky value q and column i,
//     G_q(i) = s * sum_{m: ky_m = q} A_m w_m e^{i phi_m} e^{i kx_m x_i}
// (w_m the curl weight), from per-column tables e^{i kx x_i} made once in
// f64 on the host; the second kernel then needs, per cell and field, one
// complex multiply-add per ky value with the per-row table e^{i ky y_j}.
// No per-cell trigonometry, and the cost does not grow with the number of
// modes that share a ky.
#include <math.h>

#include <vector>

#include "fs_internal.cuh"

namespace fs {

namespace {

constexpr int kMaxBandModes = 1024;

struct Band {
  int kind = 0;
  double kf = 0, width = 0, amp = 0, drag = 0;
  uint64_t seed = 0;
  int K = 0;   // tables cover kx, ky in [-K, K]
  int M = 0;   // modes per step
  int2* lattice = nullptr;  // GAUSSIAN: the (kx, ky) of every mode
  float2* ex_u = nullptr;   // [2K+1][nx] e^{i kx i h}
  float2* ex_v = nullptr;   // [2K+1][nx] e^{i kx (i+1/2) h}
  float2* ey_u = nullptr;   // [2K+1][ny] e^{i ky (j+1/2) h}
  float2* ey_v = nullptr;   // [2K+1][ny] e^{i ky j h}
  float2* gu = nullptr;     // [2K+1][nx] per-step column sums for u
  float2* gv = nullptr;     // [2K+1][nx] for v
};

// ------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3"
// (SC'11): ten rounds of two 32x32->64 multiplies with a Weyl key schedule.
struct U4 {
  uint32_t x, y, z, w;
};
__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

struct ModeCoef {
  int kx, ky;
  float2 cu, cv;  // s A w e^{i phi} for u and v
};

// Mode m of this step: wave numbers and the two complex coefficients.  Every
// block of the column kernel regenerates the list (at most kMaxBandModes
// modes), so no block waits for another.
__device__ void band_mode(int kind, int m, uint32_t step, uint64_t seed, double kf, double width, double s,
                          const int2* __restrict__ lattice, ModeCoef* out) {
  double kx, ky, A, phi;
  if (kind == FS_BAND_REFERENCE) {
    // bandForcing (solver.js:180-200): the LCG s = s * 1664525 + 1013904223
    // (mod 2^32), three draws per mode, r = s / 2^32, from seed + step
    uint32_t st = (uint32_t)seed + step;
    double r1 = 0, r2 = 0, r3 = 0;
    for (int n = 0; n <= m; n++) {
      st = st * 1664525u + 1013904223u; r1 = st / 4294967296.0;
      st = st * 1664525u + 1013904223u; r2 = st / 4294967296.0;
      st = st * 1664525u + 1013904223u; r3 = st / 4294967296.0;
    }
    const double theta = 2 * M_PI * r1, kmag = kf + (r2 - 0.5) * 2 * width;
    kx = floor(kmag * cos(theta) + 0.5);  // Math.round
    ky = floor(kmag * sin(theta) + 0.5);
    phi = 2 * M_PI * r3;
    A = (kx == 0 && ky == 0) ? 0.0 : 1.0;
  } else {
    const int2 k = lattice[m];
    kx = k.x;
    ky = k.y;
    const U4 r = philox4x32_10(U4{step, (uint32_t)m, 0u, 0u}, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = ((double)r.x + 0.5) / 4294967296.0, u2 = ((double)r.y + 0.5) / 4294967296.0;
    A = sqrt(-2.0 * log(u1));  // |a + i b| of a Box-Muller pair
    phi = 2 * M_PI * u2;       // its argument
  }
  const double kk = sqrt(kx * kx + ky * ky);
  double sp, cp;
  sincos(phi, &sp, &cp);
  const double wu = kk > 0 ? s * A * (ky / kk) : 0.0, wv = kk > 0 ? s * A * (-kx / kk) : 0.0;
  out->kx = (int)kx;
  out->ky = (int)ky;
  out->cu = make_float2((float)(wu * cp), (float)(wu * sp));
  out->cv = make_float2((float)(wv * cp), (float)(wv * sp));
}

// grid (ceil(nx / 256), 2K+1): column sums G_q(i) for ky = q - K, the modes
// added in the order of their index (deterministic run to run)
__global__ void __launch_bounds__(256)
    k_band_columns(int kind, int M, int K, const DevState* __restrict__ st, uint64_t seed, double kf, double width,
                   double s, const int2* __restrict__ lattice, const float2* __restrict__ ex_u,
                   const float2* __restrict__ ex_v, float2* __restrict__ gu, float2* __restrict__ gv, int nx) {
  __shared__ ModeCoef modes[kMaxBandModes];
  const int q = blockIdx.y - K;
  const uint32_t step = (uint32_t)st->band_step;
  for (int m = threadIdx.x; m < M; m += blockDim.x) band_mode(kind, m, step, seed, kf, width, s, lattice, modes + m);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx) return;
  float2 au = make_float2(0.f, 0.f), av = make_float2(0.f, 0.f);
  for (int m = 0; m < M; m++) {
    const ModeCoef& c = modes[m];
    if (c.ky != q || c.kx < -K || c.kx > K) continue;
    const float2 eu = __ldg(ex_u + (size_t)(c.kx + K) * nx + i), ev = __ldg(ex_v + (size_t)(c.kx + K) * nx + i);
    au.x = fmaf(c.cu.x, eu.x, fmaf(-c.cu.y, eu.y, au.x));
    au.y = fmaf(c.cu.x, eu.y, fmaf(c.cu.y, eu.x, au.y));
    av.x = fmaf(c.cv.x, ev.x, fmaf(-c.cv.y, ev.y, av.x));
    av.y = fmaf(c.cv.x, ev.y, fmaf(c.cv.y, ev.x, av.y));
  }
  gu[(size_t)blockIdx.y * nx + i] = au;
  gv[(size_t)blockIdx.y * nx + i] = av;
}

// u = (u + Re sum_q G_q(i) e^{i q y_j}) * damp, in place; the first thread of
// the grid advances the step counter (no block of this kernel reads it)
__global__ void __launch_bounds__(256)
    k_band_apply(float* __restrict__ u, float* __restrict__ v, int nx, int ny, int K,
                 const float2* __restrict__ gu, const float2* __restrict__ gv, const float2* __restrict__ ey_u,
                 const float2* __restrict__ ey_v, float damp, DevState* __restrict__ st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) st->band_step += 1;
  if (i >= nx || j >= ny) return;
  float fu = 0.f, fv = 0.f;
  const int nq = 2 * K + 1;
  for (int q = 0; q < nq; q++) {
    const float2 a = __ldg(gu + (size_t)q * nx + i), b = __ldg(ey_u + (size_t)q * ny + j);
    const float2 c = __ldg(gv + (size_t)q * nx + i), d = __ldg(ey_v + (size_t)q * ny + j);
    fu = fmaf(a.x, b.x, fmaf(-a.y, b.y, fu));
    fv = fmaf(c.x, d.x, fmaf(-c.y, d.y, fv));
  }
  const int64_t c = (int64_t)j * nx + i;
  u[c] = (u[c] + fu) * damp;
  v[c] = (v[c] + fv) * damp;
}

void free_band(Band* b) {
  auto f = [](void* p) { if (p) cudaFree(p); };
  f(b->lattice); f(b->ex_u); f(b->ex_v); f(b->ey_u); f(b->ey_v); f(b->gu); f(b->gv);
  delete b;
}

// e^{i k (x0 + i h)} for k in [-K, K], i in [0, n): [2K+1][n] float2, in f64
std::vector<float2> phase_table(int K, int n, double h, double x0) {
  std::vector<float2> t((size_t)(2 * K + 1) * n);
  for (int k = -K; k <= K; k++)
    for (int i = 0; i < n; i++) {
      const double a = k * (x0 + i * h);
      t[(size_t)(k + K) * n + i] = make_float2((float)cos(a), (float)sin(a));
    }
  return t;
}

}  // namespace

// the (kx, ky) of the GAUSSIAN kind, in its fixed order: ky ascending, then
// kx ascending, every lattice point with lo^2 <= kx^2 + ky^2 <= hi^2 except 0
std::vector<int2> band_lattice(double kf, double width) {
  std::vector<int2> out;
  const double lo = kf - width, hi = kf + width;
  const int K = (int)ceil(hi);
  for (int ky = -K; ky <= K; ky++)
    for (int kx = -K; kx <= K; kx++) {
      const double kk = (double)kx * kx + (double)ky * ky;
      if (kk == 0 || kk < lo * lo || kk > hi * hi) continue;
      out.push_back(make_int2(kx, ky));
    }
  return out;
}

void band_free(Solver* s) {
  if (s->band) free_band(static_cast<Band*>(s->band));
  s->band = nullptr;
}

int band_set(Solver* s, const fs_band* p) {
  band_free(s);
  if (!p) return FS_OK;
  Band* b = new Band;
  b->kind = p->kind;
  b->kf = p->kf;
  b->width = p->width;
  b->amp = p->amplitude;
  b->drag = p->drag;
  b->seed = p->seed;
  b->K = (int)ceil(p->kf + p->width) + 1;
  std::vector<int2> lat;
  if (p->kind == FS_BAND_GAUSSIAN) {
    lat = band_lattice(p->kf, p->width);
    b->M = (int)lat.size();
  } else {
    b->M = 24;  // bandForcing's mode count (solver.js:190)
  }
  if (b->M == 0 || b->M > kMaxBandModes) {
    free_band(b);
    return fail_status(s, FS_ERR_INVALID_ARGUMENT,
                       "band forcing needs 1.." + std::to_string(kMaxBandModes) + " modes in the band");
  }
  const int nq = 2 * b->K + 1, nx = s->g.nx, ny = s->g.ny;
  auto up = [&](float2** dst, const std::vector<float2>& src) {
    if (cudaMalloc((void**)dst, src.size() * sizeof(float2)) != cudaSuccess) return false;
    return cudaMemcpy(*dst, src.data(), src.size() * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  };
  const double h = s->g.dxd, hy = s->g.dyd;
  bool ok = up(&b->ex_u, phase_table(b->K, nx, h, 0.0)) && up(&b->ex_v, phase_table(b->K, nx, h, 0.5 * h)) &&
            up(&b->ey_u, phase_table(b->K, ny, hy, 0.5 * hy)) && up(&b->ey_v, phase_table(b->K, ny, hy, 0.0)) &&
            cudaMalloc((void**)&b->gu, (size_t)nq * nx * sizeof(float2)) == cudaSuccess &&
            cudaMalloc((void**)&b->gv, (size_t)nq * nx * sizeof(float2)) == cudaSuccess;
  if (ok && !lat.empty()) {
    ok = cudaMalloc((void**)&b->lattice, lat.size() * sizeof(int2)) == cudaSuccess &&
         cudaMemcpy(b->lattice, lat.data(), lat.size() * sizeof(int2), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (!ok) {
    free_band(b);
    cudaGetLastError();
    return fail_status(s, FS_ERR_OUT_OF_MEMORY, "band forcing tables");
  }
  s->band = b;
  return FS_OK;
}

void launch_band(Solver* s, float* u, float* v, float dt) {
  Band* b = static_cast<Band*>(s->band);
  const Grid& g = s->g;
  const double scale = b->amp * (double)dt / sqrt((double)b->M);
  const float damp = b->drag > 0 ? (float)exp(-b->drag * (double)dt) : 1.f;
  const int nq = 2 * b->K + 1;
  FS_LAUNCH(s, "band_columns", (double)nq * g.nx * 32,
            k_band_columns<<<dim3((g.nx + 255) / 256, nq), 256, 0, s->stream>>>(
                b->kind, b->M, b->K, s->dev, b->seed, b->kf, b->width, scale, b->lattice, b->ex_u, b->ex_v, b->gu,
                b->gv, g.nx));
  FS_LAUNCH(s, "band_apply", (double)s->n * 16,
            k_band_apply<<<grid2d(g.nx, g.ny, dim3(32, 8)), dim3(32, 8), 0, s->stream>>>(
                u, v, g.nx, g.ny, b->K, b->gu, b->gv, b->ey_u, b->ey_v, damp, s->dev));
}

}  // namespace fs
