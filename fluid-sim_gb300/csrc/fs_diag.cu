// fs_diag.cu -- diagnostics of the state on the device, replacing the
// read-back + CPU loops of the reference's tools:
//   kinetic energy  1/2 <cu^2 + cv^2>   with (cu, cv) the velocity at cell centres
//                                        (src/core/grid.js:267-295)
//   enstrophy       1/2 <w^2>           w at cell centres = mean of the four corner
//                                        vorticities dv/dx - du/dy (grid.js:221-257, 297-304)
//   max|div u|, sqrt(<div^2>)            (grid.js:306-320)
//   energy spectrum E(k) = sum over the shell round(|k|) = k of 1/2 (|U|^2 + |V|^2) / N^2,
//                   U, V the unnormalised 2-D DFTs of cu, cv (src/core/fft.js:196-254),
//                   with the Parseval check against the kinetic energy (fft.js:240-255).
// Sums are accumulated in double across the grid; per-cell values are f32
// (MIXED: differences of double-float faces are taken hi-hi + lo-lo, which is
// exact for neighbouring values within a factor of two).  The FFT is f32
// radix-2 in shared memory (one CTA per row, then per column); power-of-two
// grids up to 8192.
#include <cuda_runtime.h>
#include <math.h>

#include <string>
#include <vector>

#include "../../include/fluid.h"
#include "fs_internal.cuh"

namespace fs {

struct DiagBuffers {
  double* part = nullptr;  // per-block partials: 3 sums + 1 max
  unsigned* counter = nullptr;
  double* out = nullptr;    // 4 words
  int cap = 0;
  float* cu = nullptr;      // centre velocity for the spectrum
  float* cv = nullptr;
  float2* fu = nullptr;     // transposed row transforms
  float2* fv = nullptr;
  double* E = nullptr;
  int* counts = nullptr;
  float4* rgba = nullptr;   // render target
};

void diag_free(Solver* s) {
  DiagBuffers* d = static_cast<DiagBuffers*>(s->diag);
  if (!d) return;
  void* ptrs[] = {d->part, d->counter, d->out, d->cu, d->cv, d->fu, d->fv, d->E, d->counts, d->rgba};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete d;
  s->diag = nullptr;
}

static constexpr int kDiagBlocks = 152 * 4;

static int diag_alloc(Solver* s, bool spectrum) {
  if (!s->diag) s->diag = new DiagBuffers();
  DiagBuffers* d = static_cast<DiagBuffers*>(s->diag);
  cudaError_t e = cudaSuccess;
  if (!d->part) {
    e = cudaMalloc(&d->part, sizeof(double) * 4 * kDiagBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&d->counter, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&d->out, sizeof(double) * 4);
    if (e == cudaSuccess) e = cudaMemset(d->counter, 0, sizeof(unsigned));
    d->cap = kDiagBlocks;
  }
  if (e == cudaSuccess && spectrum && !d->cu) {
    const int64_t n = s->n;
    const int kmax = std::min(s->g.nx, s->g.ny) / 2;
    e = cudaMalloc(&d->cu, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d->cv, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d->fu, n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d->fv, n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d->E, sizeof(double) * (kmax + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d->counts, sizeof(int) * (kmax + 1));
  }
  if (e != cudaSuccess)
    return fail_status(s, FS_ERR_OUT_OF_MEMORY, std::string("diagnostics buffers: ") + cudaGetErrorString(e));
  return FS_OK;
}

// f32 value and difference of (hi, lo) faces; lo == nullptr for f32 state
struct Face {
  const float* hi;
  const float* lo;
  __device__ __forceinline__ float val(int64_t k) const { return lo ? hi[k] + lo[k] : hi[k]; }
  __device__ __forceinline__ float diff(int64_t a, int64_t b) const {
    return lo ? (hi[a] - hi[b]) + (lo[a] - lo[b]) : hi[a] - hi[b];
  }
};

__global__ void __launch_bounds__(256) k_diag(Face u, Face v, int nx, int ny, float idx, float idy,
                                              double* __restrict__ part, unsigned* __restrict__ counter,
                                              double* __restrict__ out, float* __restrict__ cu,
                                              float* __restrict__ cv) {
  const int n = nx * ny;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  float m = 0.f;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int j = k / nx, i = k - j * nx;
    const int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
    const int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
    const int64_t r = (int64_t)j * nx, rp = (int64_t)jp * nx, rm = (int64_t)jm * nx;
    // centre velocity (grid.js:267-278)
    const float uc = 0.5f * (u.val(r + i) + u.val(r + ip));
    const float vc = 0.5f * (v.val(r + i) + v.val(rp + i));
    s0 += (double)uc * uc + (double)vc * vc;
    if (cu) {
      cu[k] = uc;
      cv[k] = vc;
    }
    // corner vorticity at (i, j), (i+1, j), (i, j+1), (i+1, j+1), then their mean
    const float w00 = v.diff(r + i, r + im) * idx - u.diff(r + i, rm + i) * idy;
    const float w10 = v.diff(r + ip, r + i) * idx - u.diff(r + ip, rm + ip) * idy;
    const float w01 = v.diff(rp + i, rp + im) * idx - u.diff(rp + i, r + i) * idy;
    const float w11 = v.diff(rp + ip, rp + i) * idx - u.diff(rp + ip, r + ip) * idy;
    const float w = 0.25f * (w00 + w10 + w01 + w11);
    s1 += (double)w * w;
    // divergence (grid.js:191-206)
    const float dv = u.diff(r + ip, r + i) * idx + v.diff(rp + i, r + i) * idy;
    s2 += (double)dv * dv;
    m = fmaxf(m, dv != dv ? INFINITY : fabsf(dv));
  }
  // block reduction, then the last block folds the partials in a fixed order
  __shared__ double sh[3][8];
  __shared__ float shm[8];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  if (lane == 0) {
    sh[0][warp] = s0;
    sh[1][warp] = s1;
    sh[2][warp] = s2;
    shm[warp] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0;
    float mm = 0.f;
    for (int w2 = 0; w2 < nw; w2++) {
      a += sh[0][w2];
      b += sh[1][w2];
      c += sh[2][w2];
      mm = fmaxf(mm, shm[w2]);
    }
    double* p = part + 4 * blockIdx.x;
    p[0] = a;
    p[1] = b;
    p[2] = c;
    p[3] = mm;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double a = 0, b = 0, c = 0, mm = 0;
  for (unsigned q = 0; q < gridDim.x; q++) {
    const volatile double* p = part + 4 * q;
    a += p[0];
    b += p[1];
    c += p[2];
    mm = fmax(mm, p[3]);
  }
  out[0] = a;
  out[1] = b;
  out[2] = c;
  out[3] = mm;
  *counter = 0;
}

// ---------------------------------------------------------------- spectrum
__device__ __forceinline__ int bitrev(int x, int logn) { return (int)(__brev((unsigned)x) >> (32 - logn)); }

// in-place radix-2 decimation-in-time FFT of buf[0, n) (bit-reversed input), sign -1
__device__ void fft_smem(float2* buf, int n) {
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1;
    __syncthreads();
    for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
      const int g = t / half, pos = t - g * half;
      const int a = g * len + pos, b = a + half;
      float sn, cs;
      sincospif(-2.f * (float)pos / (float)len, &sn, &cs);
      const float2 x = buf[a], y = buf[b];
      const float2 ty = make_float2(cs * y.x - sn * y.y, cs * y.y + sn * y.x);
      buf[a] = make_float2(x.x + ty.x, x.y + ty.y);
      buf[b] = make_float2(x.x - ty.x, x.y - ty.y);
    }
  }
  __syncthreads();
}

// row j of the real field -> its DFT, written transposed (out[kx][j]) for the column pass
__global__ void k_fft_rows(const float* __restrict__ f, float2* __restrict__ out, int n, int logn) {
  extern __shared__ float2 sb[];
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sb[bitrev(i, logn)] = make_float2(f[(int64_t)j * n + i], 0.f);
  fft_smem(sb, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[(int64_t)i * n + j] = sb[i];
}

__device__ __forceinline__ int freq_of(int i, int n) { return i <= n / 2 ? i : i - n; }

// column kx of both fields: finish the 2-D DFTs and add 1/2 (|U|^2 + |V|^2) / N^2
// of every mode to its shell round(|k|) <= kmax (modes beyond kmax are dropped,
// fft.js:226-233)
__global__ void k_fft_cols_bin(const float2* __restrict__ fu, const float2* __restrict__ fv, int n, int logn,
                               double* __restrict__ E, int* __restrict__ counts) {
  extern __shared__ float2 sb[];
  float2* bu = sb;
  float2* bv = sb + n;
  const int kmax = n / 2;
  double* hist = reinterpret_cast<double*>(sb + 2 * n);
  int* hcnt = reinterpret_cast<int*>(hist + kmax + 1);
  const int c = blockIdx.x;
  for (int k = threadIdx.x; k <= kmax; k += blockDim.x) {
    hist[k] = 0.0;
    hcnt[k] = 0;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    bu[bitrev(i, logn)] = fu[(int64_t)c * n + i];
    bv[bitrev(i, logn)] = fv[(int64_t)c * n + i];
  }
  fft_smem(bu, n);
  fft_smem(bv, n);
  const double NN = (double)n * n * (double)n * n;
  const int kx = freq_of(c, n);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int ky = freq_of(j, n);
    const double pu = (double)bu[j].x * bu[j].x + (double)bu[j].y * bu[j].y;
    const double pv = (double)bv[j].x * bv[j].x + (double)bv[j].y * bv[j].y;
    const double kmag = sqrt((double)kx * kx + (double)ky * ky);
    const int shell = (int)floor(kmag + 0.5);
    if (shell <= kmax) {
      atomicAdd(&hist[shell], 0.5 * (pu + pv) / NN);
      atomicAdd(&hcnt[shell], 1);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= kmax; k += blockDim.x) {
    if (hcnt[k]) {
      atomicAdd(&E[k], hist[k]);
      atomicAdd(&counts[k], hcnt[k]);
    }
  }
}

static void state_faces(Solver* s, Face* u, Face* v) {
  *u = Face{s->u, s->mixed ? s->ulo : nullptr};
  *v = Face{s->v, s->mixed ? s->vlo : nullptr};
}

int diagnostics(Solver* s, fs_diagnostics* out, bool with_centres) {
  int rc = diag_alloc(s, with_centres);
  if (rc) return rc;
  DiagBuffers* d = static_cast<DiagBuffers*>(s->diag);
  Face u, v;
  state_faces(s, &u, &v);
  const int blocks = (int)std::min<int64_t>(kDiagBlocks, (s->n + 255) / 256);
  k_diag<<<blocks, 256, 0, s->stream>>>(u, v, s->g.nx, s->g.ny, (float)s->g.idxd, (float)s->g.idyd, d->part,
                                         d->counter, d->out, with_centres ? d->cu : nullptr,
                                         with_centres ? d->cv : nullptr);
  s->launches++;
  double h[4];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d->out, sizeof h, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("diagnostics: ") + cudaGetErrorString(e));
  const double N = (double)s->n;
  out->kinetic_energy = 0.5 * h[0] / N;
  out->enstrophy = 0.5 * h[1] / N;
  out->l2_divergence = sqrt(h[2] / N);
  out->max_divergence = h[3];
  return FS_OK;
}

int energy_spectrum(Solver* s, double* E, int32_t* counts, int cap, int* kmax_out, double* parseval) {
  const int n = s->g.nx;
  if (s->g.nx != s->g.ny || (n & (n - 1)) || n < 8 || n > 8192)
    return fail_status(s, FS_ERR_UNSUPPORTED, "energy spectrum: square power-of-two grids from 8 to 8192");
  const int kmax = n / 2;
  if (kmax_out) *kmax_out = kmax;
  if (cap < kmax + 1) return fail_status(s, FS_ERR_INVALID_ARGUMENT, "energy spectrum: output shorter than kmax + 1");
  fs_diagnostics dg;
  int rc = diagnostics(s, &dg, true);  // also writes the centre velocity
  if (rc) return rc;
  DiagBuffers* d = static_cast<DiagBuffers*>(s->diag);
  int logn = 0;
  while ((1 << logn) < n) logn++;
  const size_t smem_rows = (size_t)n * sizeof(float2);
  const size_t smem_cols = 2 * (size_t)n * sizeof(float2) + (kmax + 1) * (sizeof(double) + sizeof(int));
  cudaError_t e = cudaFuncSetAttribute(k_fft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_fft_cols_bin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cols);
  if (e == cudaSuccess) e = cudaMemsetAsync(d->E, 0, sizeof(double) * (kmax + 1), s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d->counts, 0, sizeof(int) * (kmax + 1), s->stream);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("energy spectrum: ") + cudaGetErrorString(e));
  k_fft_rows<<<n, 256, smem_rows, s->stream>>>(d->cu, d->fu, n, logn);
  k_fft_rows<<<n, 256, smem_rows, s->stream>>>(d->cv, d->fv, n, logn);
  k_fft_cols_bin<<<n, 256, smem_cols, s->stream>>>(d->fu, d->fv, n, logn, d->E, d->counts);
  s->launches += 3;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(E, d->E, sizeof(double) * (kmax + 1), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(counts, d->counts, sizeof(int) * (kmax + 1), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("energy spectrum: ") + cudaGetErrorString(e));
  if (parseval) {
    double tot = 0.0;
    for (int k = 0; k <= kmax; k++) tot += E[k];
    parseval[0] = tot;
    parseval[1] = dg.kinetic_energy;
  }
  return FS_OK;
}

// ------------------------------------------------------------------ render
// The arithmetic of the reference's RENDER pass (src/gpu/shaders.js:677-768)
// into a device buffer instead of a swapchain texture: centre vorticity from
// the four corner curls, a two-sided neon ramp in tanh(w * exposure) (or in
// speed for mode 1), a white-hot speed term scaled by the same exposure, and
// a dim dye lift.  Colours are linear RGBA f32 (the reference writes
// rgba16float); non-finite colours become black.
__device__ __forceinline__ float smoothstep_f(float e0, float e1, float x) {
  const float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
  return t * t * (3.f - 2.f * t);
}
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) {
  return make_float3(a.x * (1.f - t) + b.x * t, a.y * (1.f - t) + b.y * t, a.z * (1.f - t) + b.z * t);
}
__device__ __forceinline__ float3 scale3(float3 a, float k) { return make_float3(a.x * k, a.y * k, a.z * k); }

__global__ void __launch_bounds__(256) k_render(Face u, Face v, const float4* __restrict__ dye, int nx, int ny,
                                                float idx, float idy, float exposure, int mode,
                                                float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
  const int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
  const int64_t r = (int64_t)j * nx, rp = (int64_t)jp * nx, rm = (int64_t)jm * nx;
  const float w00 = v.diff(r + i, r + im) * idx - u.diff(r + i, rm + i) * idy;
  const float w10 = v.diff(r + ip, r + i) * idx - u.diff(r + ip, rm + ip) * idy;
  const float w01 = v.diff(rp + i, rp + im) * idx - u.diff(rp + i, r + i) * idy;
  const float w11 = v.diff(rp + ip, rp + i) * idx - u.diff(rp + ip, r + ip) * idy;
  const float w = 0.25f * (w00 + w10 + w01 + w11);
  const float cu = u.val(r + i), cv = v.val(r + i);
  const float speed = sqrtf(cu * cu + cv * cv);
  const float3 MAGENTA = make_float3(1.00f, 0.10f, 0.62f), CYAN = make_float3(0.10f, 0.92f, 1.00f);
  const float3 VIOLET = make_float3(0.16f, 0.03f, 0.42f), VOID_ = make_float3(0.004f, 0.003f, 0.016f);
  float3 col;
  if (mode == 0) {
    const float sig = tanhf(fminf(fmaxf(w * exposure, -12.f), 12.f));
    const float mag = fabsf(sig);
    const float3 hue = sig >= 0.f ? MAGENTA : CYAN;
    const float3 ramp = mix3(mix3(VOID_, VIOLET, smoothstep_f(0.f, 0.22f, mag)), hue, smoothstep_f(0.12f, 0.62f, mag));
    col = scale3(ramp, 0.30f + 4.6f * mag * mag);
  } else {
    const float t = tanhf(fminf(fmaxf(speed * exposure, -12.f), 12.f));
    const float3 hue = mix3(VIOLET, CYAN, smoothstep_f(0.15f, 0.95f, t));
    col = scale3(mix3(VOID_, hue, smoothstep_f(0.f, 0.6f, t)), 0.35f + 2.9f * t * t);
  }
  const float sp = tanhf(fminf(fmaxf(speed * exposure * 0.45f, 0.f), 12.f));
  const float sp2 = sp * sp, hot = sp2 * sp2 * sp * 0.85f;
  col = make_float3(col.x + 0.55f * hot, col.y + 0.78f * hot, col.z + 1.0f * hot);
  if (dye) {
    const float4 d = dye[r + i];
    const float lum = d.x * 0.2126f + d.y * 0.7152f + d.z * 0.0722f;
    col = make_float3(col.x + col.x * lum * 1.5f + d.x * 0.20f, col.y + col.y * lum * 1.5f + d.y * 0.20f,
                      col.z + col.z * lum * 1.5f + d.z * 0.20f);
  }
  col = make_float3(col.x == col.x ? col.x : 0.f, col.y == col.y ? col.y : 0.f, col.z == col.z ? col.z : 0.f);
  out[r + i] = make_float4(col.x, col.y, col.z, 1.f);
}

int render(Solver* s, int mode, float exposure, float* host_rgba) {
  if (mode != 0 && mode != 1) return fail_status(s, FS_ERR_INVALID_ARGUMENT, "render: mode is 0 (vorticity) or 1 (speed)");
  int rc = diag_alloc(s, false);
  if (rc) return rc;
  DiagBuffers* d = static_cast<DiagBuffers*>(s->diag);
  cudaError_t e = cudaSuccess;
  if (!d->rgba) e = cudaMalloc(&d->rgba, s->n * 16);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_OUT_OF_MEMORY, "render buffer");
  Face u, v;
  state_faces(s, &u, &v);
  dim3 b(32, 8), g((s->g.nx + 31) / 32, (s->g.ny + 7) / 8);
  k_render<<<g, b, 0, s->stream>>>(u, v, static_cast<const float4*>(s->dye), s->g.nx, s->g.ny, (float)s->g.idxd,
                                   (float)s->g.idyd, exposure, mode, d->rgba);
  s->launches++;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host_rgba, d->rgba, s->n * 16, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
  return FS_OK;
}

}  // namespace fs
