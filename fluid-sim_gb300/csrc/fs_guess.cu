// fs_guess.cu -- the learned pressure guess: a small periodic U-Net that maps
// the divergence (and the solid mask) at half the grid resolution to an
// initial pressure for the multigrid projection, with its forward pass,
// backward pass and Adam update on the GPU.  No counterpart in the reference.
//
// Network (channels 16/32/64/128 over four levels, NHWC bf16 activations,
// f32 accumulation, every convolution 3x3 periodic on the tcgen05 tensor
// cores -- fs_conv.cu):
//   x0 -A-> a0 -B-> a0b -pool-> q1 -C-> a1 -pool-> q2 -D-> a2 -pool-> q3 -E-> a3
//   a3 -F-> f3;  s2 = up(f3) + a2 -G-> g2;  s1 = up(g2) + a1 -H-> h1;
//   s0 = up(h1) + a0b -I-> i0 -J-> out (channel 0, f32)
// ReLU after every convolution but J.  Parameters are kept in f32 (master
// copy, flattened layer by layer as w[co][ci][3][3] then b[co]) and repacked
// to bf16 after every update, once in the forward layout and once transposed
// and flipped, so that the gradient with respect to a layer's input is the
// same tensor-core convolution.  Weight gradients are a tcgen05 GEMM too,
// with the pixels as its K dimension (k_wgrad_tc), and deterministic per-CTA
// partial sums.
//
// Normalisation (the guess is linear-equivariant in the divergence): with
// h the net's grid spacing and sigma = RMS(h^2 d), the input is h^2 d / sigma
// and the output is p / sigma, so the pressure guess is sigma * out.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fluid.h"
#include "fs_df.cuh"
#include "fs_internal.cuh"
#include "fs_reduce.cuh"
#include "fs_tc.cuh"

namespace fs {
namespace conv {
cudaError_t conv3x3(int cin, int cout, int epi, const void* in, const void* w, const float* bias, void* out, int B,
                    int H, int W, int* err, cudaStream_t st);
}
}  // namespace fs

struct fs_guess;

namespace fs {
namespace guess {

typedef __nv_bfloat16 bf;
constexpr int NL = 10;
constexpr int kCI[NL] = {16, 16, 16, 32, 64, 128, 64, 32, 16, 16};
constexpr int kCO[NL] = {16, 16, 32, 64, 128, 64, 32, 16, 16, 16};
constexpr int kRelu[NL] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 0};
enum { LA, LB, LC, LD, LE, LF, LG, LH, LI, LJ };

// activation / gradient buffers: (level, channels)
enum Buf {
  X0, A0, A0B, Q1, A1, Q2, A2, Q3, A3, F3, S2, G2, S1, H1, S0, I0,  // forward
  GJ, DI0, DS0, DH1, DS1, DG2, DS2, DF3, DA3, DQ3, DQ2, DQ1, DA0,   // backward
  NBUF
};
constexpr int kBufLevel[NBUF] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0,
                                 0, 0, 0, 1, 1, 2, 2, 3, 3, 3, 2, 1, 0};
constexpr int kBufCh[NBUF] = {16, 16, 16, 16, 32, 32, 64, 64, 128, 64, 64, 32, 32, 16, 16, 16,
                              16, 16, 16, 16, 32, 32, 64, 64, 128, 64, 32, 16, 16};


struct Net {
  int device = 0;
  cudaStream_t stream = nullptr;  // own stream for the stand-alone entry points
  int64_t off_w[NL], off_b[NL], off_pk[NL];
  int64_t nparam = 0, npk = 0;
  float *theta = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  bf *wpk = nullptr, *wpkT = nullptr;
  float* zero_bias = nullptr;
  int* err = nullptr;
  double* acc = nullptr;  // loss: per-sample mean error [B], loss [B]; guess: sum of squares
  int64_t adam_t = 0;
  double w_p = 1.0, w_r = 0.0;  // loss weights: pressure error, residual (lap of the error)
  int capB = 0, capH = 0, capW = 0;
  bf* buf[NBUF] = {};
  float* out = nullptr;     // [B][H][W]
  float* gin = nullptr;     // solver path: h^2 d at net resolution
  float* gmask = nullptr;   // solver path: mask at net resolution
  float* res = nullptr;     // loss: lap(out - target), [B][H][W]
  float* corr_part = nullptr;
  int64_t corr_cap = 0;
  int64_t launches = 0;
  std::string err_msg;
};

static int64_t level_pixels(const Net* g, int B, int H, int W, int lev) {
  return (int64_t)B * (H >> lev) * (W >> lev);
}

// ------------------------------------------------------------ small kernels
__device__ __forceinline__ void unpack8(uint4 q, float* f) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float2 t = __bfloat1622float2(h[k]);
    f[2 * k] = t.x;
    f[2 * k + 1] = t.y;
  }
}
__device__ __forceinline__ uint4 pack8(const float* f) {
  uint4 q;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&q);
#pragma unroll
  for (int k = 0; k < 4; k++) h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
  return q;
}

#define GRID_STRIDE(k, n) for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < (n); k += (int64_t)gridDim.x * blockDim.x)
// element loops of the network's buffers (all below 2^31 elements, checked on the host)
#define GRID_STRIDE32(k, n) for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < (n); k += gridDim.x * blockDim.x)

// average 2x2 (out dims Ho x Wo); C8 = channels / 8
__global__ void k_pool(const uint4* __restrict__ in, uint4* __restrict__ out, int B, int Ho, int Wo, int C8) {
  const int n = B * Ho * Wo * C8;
  GRID_STRIDE32(k, n) {
    int c = k % C8, r = k / C8;
    int x = r % Wo, t2 = r / Wo, y = t2 % Ho, b = t2 / Ho;
    float s[8] = {}, t[8];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int src = ((b * 2 * Ho + 2 * y + (q >> 1)) * 2 * Wo + 2 * x + (q & 1)) * C8 + c;
      unpack8(in[src], t);
#pragma unroll
      for (int e = 0; e < 8; e++) s[e] += t[e];
    }
#pragma unroll
    for (int e = 0; e < 8; e++) s[e] *= 0.25f;
    out[k] = pack8(s);
  }
}

// out = up(coarse) + skip (fine dims H x W), or, with scale != 0 and out == skip,
// skip += scale * up(coarse)
__global__ void k_upadd(const uint4* __restrict__ coarse, const uint4* skip, uint4* out, int B, int H, int W, int C8,
                        float scale) {
  const int n = B * H * W * C8;
  GRID_STRIDE32(k, n) {
    int c = k % C8, r = k / C8;
    int x = r % W, t2 = r / W, y = t2 % H, b = t2 / H;
    float a[8], s[8];
    unpack8(coarse[((b * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)) * C8 + c], a);
    unpack8(skip[k], s);
#pragma unroll
    for (int e = 0; e < 8; e++) s[e] = __fmaf_rn(scale, a[e], s[e]);
    out[k] = pack8(s);
  }
}

// coarse = sum over each 2x2 block of fine (the adjoint of nearest upsampling)
__global__ void k_poolsum(const uint4* __restrict__ in, uint4* __restrict__ out, int B, int Ho, int Wo, int C8) {
  const int n = B * Ho * Wo * C8;
  GRID_STRIDE32(k, n) {
    int c = k % C8, r = k / C8;
    int x = r % Wo, t2 = r / Wo, y = t2 % Ho, b = t2 / Ho;
    float s[8] = {}, t[8];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int src = ((b * 2 * Ho + 2 * y + (q >> 1)) * 2 * Wo + 2 * x + (q & 1)) * C8 + c;
      unpack8(in[src], t);
#pragma unroll
      for (int e = 0; e < 8; e++) s[e] += t[e];
    }
    out[k] = pack8(s);
  }
}

// g = a > 0 ? g : 0 (the ReLU's derivative, from its output)
__global__ void k_relu_mask(uint4* __restrict__ g, const uint4* __restrict__ a, int n8) {
  GRID_STRIDE32(k, n8) {
    float gv[8], av[8];
    unpack8(g[k], gv);
    unpack8(a[k], av);
#pragma unroll
    for (int e = 0; e < 8; e++) gv[e] = av[e] > 0.f ? gv[e] : 0.f;
    g[k] = pack8(gv);
  }
}

// sigma = RMS from a sum of squares (1 when it is 0), computed by one thread
// of the block: FP64 runs at 1/54 of the FP32 rate on this part, so it is not
// evaluated per element
__device__ __forceinline__ float block_sigma(const double* __restrict__ sumsq, int64_t nnorm) {
  __shared__ float sig;
  if (threadIdx.x == 0) {
    double r = sqrt(sumsq[0] / (double)nnorm);
    sig = r > 0.0 ? (float)r : 1.f;
  }
  __syncthreads();
  return sig;
}

// x0[p] = (div / sigma, mask, 0, ..., 0); sigma = 1 without a sum of squares
__global__ void k_prep(const float* __restrict__ div, const float* __restrict__ mask, uint4* __restrict__ x0,
                       int npix, const double* __restrict__ sumsq, int64_t nnorm) {
  const float inv = sumsq ? 1.f / block_sigma(sumsq, nnorm) : 1.f;
  GRID_STRIDE32(p, npix) {
    float f[8] = {div[p] * inv, mask ? mask[p] : 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float z[8] = {};
    x0[2 * p] = pack8(f);
    x0[2 * p + 1] = pack8(z);
  }
}

// per-sample sum of e = out - target -> acc[b]
__global__ void k_loss_mean(const float* __restrict__ out, const float* __restrict__ tgt, double* __restrict__ acc,
                            int64_t npix) {
  const int b = blockIdx.y;
  double s = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x)
    s += (double)out[b * npix + p] - (double)tgt[b * npix + p];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
    atomicAdd(&acc[b], t);
  }
}

__device__ __forceinline__ int64_t wrap_idx(int b, int y, int x, int H, int W) {
  y = y < 0 ? y + H : (y >= H ? y - H : y);
  x = x < 0 ? x + W : (x >= W ? x - W : x);
  return ((int64_t)b * H + y) * W + x;
}

// res = lap(out - target) (periodic 5-point, unscaled); w_r sum res^2 / (B N) into acc[B]
__global__ void k_loss_res(const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ res,
                           double* __restrict__ acc, int H, int W, int B, double w_r) {
  const int b = blockIdx.y;
  const int64_t npix = (int64_t)H * W;
  double s = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
    const int pi = (int)p, y = pi / W, x = pi - y * W;
    auto e = [&](int yy, int xx) {
      int64_t q = wrap_idx(b, yy, xx, H, W);
      return (double)out[q] - (double)tgt[q];
    };
    double r = e(y, x - 1) + e(y, x + 1) + e(y - 1, x) + e(y + 1, x) - 4.0 * e(y, x);
    res[b * npix + p] = (float)r;
    s += r * r;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
    atomicAdd(&acc[B], w_r * t / ((double)B * npix));
  }
}

// seed gradient dL/dout = (w_p 2 (e - mean_b e) + w_r 2 lap(res)) / (B N) into
// channel 0 of gJ; w_p sum (e - mean)^2 / (B N) into acc[B]
__global__ void k_loss_seed(const float* __restrict__ out, const float* __restrict__ tgt,
                            const float* __restrict__ res, double* __restrict__ acc, uint4* __restrict__ gJ, int H,
                            int W, int B, double w_p, double w_r) {
  const int b = blockIdx.y;
  const int64_t npix = (int64_t)H * W;
  const double mean = acc[b] / (double)npix, scale = 2.0 / ((double)B * npix);
  double s = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = b * npix + p;
    double ec = (double)out[q] - (double)tgt[q] - mean;
    s += ec * ec;
    double g = w_p * ec;
    if (res) {
      const int pi = (int)p, y = pi / W, x = pi - y * W;
      double lr = (double)res[wrap_idx(b, y, x - 1, H, W)] + res[wrap_idx(b, y, x + 1, H, W)] +
                  res[wrap_idx(b, y - 1, x, H, W)] + res[wrap_idx(b, y + 1, x, H, W)] - 4.0 * res[q];
      g += w_r * lr;
    }
    float f[8] = {(float)(scale * g), 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float z[8] = {};
    gJ[2 * q] = pack8(f);
    gJ[2 * q + 1] = pack8(z);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
    atomicAdd(&acc[B], w_p * t / ((double)B * npix));
  }
}

// ------------------------------------------ weight gradients on tcgen05
// dW[co][ci][tap] = sum_p G[p][co] X[p + s_tap][ci] as a GEMM with K = pixels:
// D[m][n] += sum_k A[m][k] B[n][k], rows m = tap * CIN + ci of the shifted
// input X (A), n = co of the output gradient G (B), accumulated in TMEM over
// every pixel a CTA visits.  Rows are packed nine taps deep, so M-blocks of
// 128 rows cover 9 CIN rows (two blocks for 16 input channels, nine for 128);
// a CTA owns NMB consecutive M-blocks (blockIdx.y picks the group) so that
// its accumulators fit the 512 TMEM columns.  Both operands are NHWC bf16 in
// global memory (channels contiguous); the CTA stages them K-major (pixels
// contiguous per row) by transposing blocks of 8 pixels x 8 channels in
// registers, into the no-swizzle core-matrix layout of fs_tc_gemm_check with
// the 8-row groups 272 bytes apart (LBO 128, SBO 272): the 16 bytes of
// padding per group put neighbouring threads' blocks 16 bytes apart modulo
// 128, so the eight threads of one 128-bit store phase write eight different
// bank quads (with SBO 256 every block starts on the same banks).  Per-CTA
// partial sums (and the bias sums of G, by the CTAs of blockIdx.y == 0) go to
// global memory; k_wgrad_reduce adds them in a fixed order, so the gradient
// is deterministic.
constexpr int kWgThreads = 512;  // 16 warps: staging parallelism (one CTA per SM by shared memory)
constexpr int kWgTile = 128;  // pixels per K tile
constexpr int kWgSBO = 272;   // bytes between consecutive 8-row groups of a staged operand

template <int CIN, int COUT, int NMB>
struct WgCfg {
  static constexpr int MROWS = 9 * CIN;                    // rows of D
  static constexpr int MBLK = (MROWS + 127) / 128;         // M-blocks in all
  static constexpr int A_STEP = 16 * kWgSBO;               // one K step (16 pixels) of an M-block
  static constexpr int A_MB = (kWgTile / 16) * A_STEP;      // one M-block
  static constexpr int A_BYTES = NMB * A_MB;                // this CTA's A operand
  static constexpr int B_STEP = (COUT / 8) * kWgSBO;
  static constexpr int B_BYTES = (kWgTile / 16) * B_STEP;
  static constexpr int R_BYTES = 3 * (kWgTile + 2) * (CIN / 8) * 16;  // three input rows of the tile, halo 1
  static constexpr int GR_BYTES = kWgTile * (COUT / 8) * 16;          // the tile's output-gradient row
  static constexpr int SMEM = A_BYTES + B_BYTES + R_BYTES + GR_BYTES + 128;  // + barrier, TMEM slot, flag
  // row groups (tap, chunk) this CTA stages each tile; the rest of its M-blocks are zero padding
  static constexpr int real_groups(int mb0) {
    return 9 * (CIN / 8) - mb0 * 16 < NMB * 16 ? (9 * (CIN / 8) - mb0 * 16 > 0 ? 9 * (CIN / 8) - mb0 * 16 : 0)
                                               : NMB * 16;
  }
  static constexpr int NCOL_USED = NMB * COUT;
  static constexpr int NCOL = NCOL_USED <= 32    ? 32
                              : NCOL_USED <= 64  ? 64
                              : NCOL_USED <= 128 ? 128
                              : NCOL_USED <= 256 ? 256
                                                 : 512;
  static_assert(NCOL_USED <= 512 && COUT % 16 == 0 && CIN % 8 == 0, "TMEM columns, channel counts");
  static_assert(A_BYTES + B_BYTES + 3 * (kWgTile + 2) * (CIN / 8) * 16 + kWgTile * (COUT / 8) * 16 + 128 <= 227 * 1024,
                "shared memory of one CTA");
};

// 8 rows of 8 bf16 (r[i] = pixel i, channels 0..7) -> t[c] = channel c, pixels 0..7
__device__ __forceinline__ void transpose8x8(const uint4* r, uint4* t) {
  const uint32_t* w = reinterpret_cast<const uint32_t*>(r);  // w[4 i + j]: pixel i, channels 2j, 2j+1
  uint32_t* o = reinterpret_cast<uint32_t*>(t);               // o[4 c + j']: channel c, pixels 2j', 2j'+1
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int jp = 0; jp < 4; jp++) {
      const uint32_t a = w[4 * (2 * jp) + j], b = w[4 * (2 * jp + 1) + j];
      o[4 * (2 * j) + jp] = __byte_perm(a, b, 0x5410);
      o[4 * (2 * j + 1) + jp] = __byte_perm(a, b, 0x7632);
    }
}

// byte offset of the 8x8 block (rows 8g.., pixels 8q..) of a staged operand of R rows
__device__ __forceinline__ int kmaj_block(int R, int g, int q) {
  return (q >> 1) * ((R / 8) * kWgSBO) + g * kWgSBO + (q & 1) * 128;
}

// A tile is a segment of up to 128 pixels of one image row; its three input
// rows (y - 1 .. y + 1, x0 - 1 .. x0 + 128, wrapped) are staged once with
// coalesced loads, and the nine taps' shifted operands are transposed out of
// that copy.  The next tile's rows are loaded while the previous tile's MMAs
// run (the row copy is not an MMA operand).
template <int CIN, int COUT, int NMB>
__global__ void __launch_bounds__(kWgThreads) k_wgrad_tc(const uint4* __restrict__ X, const uint4* __restrict__ G,
                                                         int B, int H, int W, float* __restrict__ part,
                                                         float* __restrict__ bpart, int* __restrict__ err) {
  using C = WgCfg<CIN, COUT, NMB>;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* sa = smem;
  unsigned char* sb = smem + C::A_BYTES;
  uint4* xr = reinterpret_cast<uint4*>(smem + C::A_BYTES + C::B_BYTES);  // [3][kWgTile + 2][KC]
  uint4* gr = reinterpret_cast<uint4*>(smem + C::A_BYTES + C::B_BYTES + C::R_BYTES);  // [kWgTile][OC]
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::A_BYTES + C::B_BYTES + C::R_BYTES + C::GR_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  int* failed = reinterpret_cast<int*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mb0 = blockIdx.y * NMB;  // first M-block of this CTA
  const int ntx = (W + kWgTile - 1) / kWgTile;
  const int64_t ntiles = (int64_t)B * H * ntx;
  constexpr int KC = CIN / 8, OC = COUT / 8, RW = kWgTile + 2;
  if (warp == 0) {
    tc::tmem_alloc(tslot, C::NCOL);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
    *failed = 0;
  }
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t sa_s = tc::smem_u32(sa), sb_s = tc::smem_u32(sb);
  constexpr uint32_t IDESC = tc::idesc_bf16(128, COUT);
  float bsum = 0.f;  // bias partial of output channel tid (tid < COUT, blockIdx.y == 0)
  uint32_t phase = 0;
  int issued = 0;
  // the padding row groups of the last M-block are zero for every tile: written once
  const int nreal = C::real_groups(mb0);
  for (int k = tid; k < (kWgTile / 8) * (NMB * 16 - nreal); k += kWgThreads) {
    const int q = k / (NMB * 16 - nreal), gl = nreal + (k - q * (NMB * 16 - nreal));
    uint4* dst = reinterpret_cast<uint4*>(sa + (gl >> 4) * C::A_MB + kmaj_block(128, gl & 15, q));
#pragma unroll
    for (int c = 0; c < 8; c++) dst[c] = make_uint4(0, 0, 0, 0);
  }
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int xt = (int)(t % ntx);
    const int64_t by = t / ntx;  // b * H + y
    const int y = (int)(by % H);
    const int64_t b = by / H;
    const int x0 = xt * kWgTile;
    // the tile's three input rows (the previous tile's transposes, the only
    // readers, finished before the __syncthreads ahead of its MMAs)
    for (int k = tid; k < 3 * RW * KC; k += kWgThreads) {
      const int rc = k / KC, kc = k - rc * KC, r = rc / RW, c = rc - r * RW;
      int gy = y - 1 + r, gx = x0 - 1 + c;
      gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
      gx = ((gx % W) + W) % W;
      xr[k] = X[((b * H + gy) * W + gx) * KC + kc];
    }
    // and its output-gradient row (zero beyond the row's end)
    for (int k = tid; k < kWgTile * OC; k += kWgThreads) {
      const int x = x0 + k / OC;
      gr[k] = x < W ? G[(by * W + x0) * OC + k] : make_uint4(0, 0, 0, 0);
    }
    if (issued) {
      // the MMAs of the previous tile read the operand buffers
      if (tid == 0 && !tc::mbar_wait(bar, phase)) *failed = 1;
      phase ^= 1;
    }
    __syncthreads();
    if (*failed) break;
    // B: G[p][co] -> rows co, K = pixels, from the staged row
    for (int k = tid; k < (kWgTile / 8) * OC; k += kWgThreads) {
      const int q = k / OC, oc = k - q * OC;
      uint4 r[8];
#pragma unroll
      for (int i = 0; i < 8; i++) r[i] = gr[(8 * q + i) * OC + oc];
      uint4 tt[8];
      transpose8x8(r, tt);
      uint4* dst = reinterpret_cast<uint4*>(sb + kmaj_block(COUT, oc, q));
#pragma unroll
      for (int c = 0; c < 8; c++) dst[c] = tt[c];
    }
    // A: for each row group (tap, input chunk) of this CTA's M-blocks, the
    // staged rows at the tap's shift -> rows ci, K = pixels; padding groups zero
    for (int k = tid; k < (kWgTile / 8) * nreal; k += kWgThreads) {
      const int q = k / nreal, gl = k - q * nreal;
      const int gg = mb0 * 16 + gl;  // global row group, < 9 KC
      const int tap = gg / KC, kc = gg - tap * KC;
      const uint4* src = xr + ((tap / 3) * RW + 8 * q + (tap % 3)) * KC + kc;
      uint4 r[8];
#pragma unroll
      for (int i = 0; i < 8; i++) r[i] = src[i * KC];
      uint4 tt[8];
      transpose8x8(r, tt);
      const int blk = gl >> 4, g = gl & 15;  // M-block of this CTA, row group in it
      uint4* dst = reinterpret_cast<uint4*>(sa + blk * C::A_MB + kmaj_block(128, g, q));
#pragma unroll
      for (int c = 0; c < 8; c++) dst[c] = tt[c];
    }
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
#pragma unroll 1
      for (int j = 0; j < NMB; j++)
#pragma unroll
        for (int s = 0; s < kWgTile / 16; s++)
          tc::mma_bf16(taddr + j * COUT, tc::sdesc(sa_s + j * C::A_MB + s * C::A_STEP, 128, kWgSBO),
                       tc::sdesc(sb_s + s * C::B_STEP, 128, kWgSBO), IDESC, (issued || s > 0) ? 1u : 0u);
      tc::mma_commit(bar);
    }
    issued = 1;
    // bias partial: output channel tid sums its staged row (read only, like the MMAs)
    if (blockIdx.y == 0 && tid < COUT) {
#pragma unroll 4
      for (int q = 0; q < kWgTile / 8; q++) {
        const uint4 v = *reinterpret_cast<const uint4*>(sb + kmaj_block(COUT, tid >> 3, q) + (tid & 7) * 16);
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const float2 f = __bfloat1622float2(h[e]);
          bsum += f.x + f.y;
        }
      }
    }
  }
  if (tid == 0 && issued) {
    if (!*failed) {
      if (!tc::mbar_wait(bar, phase)) *failed = 1;
    } else {
      tc::mbar_wait(bar, phase, 1u << 20);  // let what was issued drain before the TMEM is released
    }
  }
  if (tid == 0 && *failed) atomicExch(err, 1);
  __syncthreads();
  tc::fence_after_sync();
  const int64_t cta = blockIdx.x;
  if (!*failed) {
    // warp w reads TMEM lanes 32 (w % 4) ..; the four warp groups share the
    // (M-block, 16-column) chunks
    const int m = 32 * (warp & 3) + lane, grp = warp >> 2;
#pragma unroll 1
    for (int jc = grp; jc < NMB * (COUT / 16); jc += kWgThreads / 128) {
      const int j = jc / (COUT / 16), c0 = (jc - j * (COUT / 16)) * 16;
      const int row = (mb0 + j) * 128 + m;
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(32 * (warp & 3)) << 16) + j * COUT + c0, v);
      if (row < C::MROWS) {
        float* dst = part + (cta * C::MROWS + row) * COUT + c0;
#pragma unroll
        for (int k = 0; k < 16; k++) dst[k] = issued ? v[k] : 0.f;
      }
    }
    if (blockIdx.y == 0 && tid < COUT) bpart[cta * COUT + tid] = bsum;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, C::NCOL);
}

// grad[off_w + OIHW] = sum over the P partials of row tap * cin + ci, column
// co; grad[off_b + co] = sum of the bias partials
__global__ void k_wgrad_reduce(const float* __restrict__ part, const float* __restrict__ bpart, int P, int cin,
                               int cout, float* __restrict__ gw, float* __restrict__ gb) {
  const int64_t mrows = 9 * (int64_t)cin, nw = mrows * cout;
  GRID_STRIDE(e, nw + cout) {
    float s = 0.f;
    if (e < nw) {
      for (int p = 0; p < P; p++) s += part[(int64_t)p * nw + e];
      const int row = (int)(e / cout), co = (int)(e % cout), tap = row / cin, ci = row % cin;
      gw[((int64_t)co * cin + ci) * 9 + tap] = s;
    } else {
      const int co = (int)(e - nw);
      for (int p = 0; p < P; p++) s += bpart[(int64_t)p * cout + co];
      gb[co] = s;
    }
  }
}

// ------------------------------------------------------------ parameters
struct PackTable {
  int64_t off_w[NL], off_pk[NL];
  int ci[NL], co[NL];
};

// f32 master -> bf16 forward pack [t][ci/8][co][ci%8] and the transposed,
// flipped pack [t'][co/8][ci][co%8] with t' = (2-ky)*3 + (2-kx)
__global__ void k_pack(const float* __restrict__ theta, bf* __restrict__ wpk, bf* __restrict__ wpkT, PackTable tab) {
  for (int l = 0; l < NL; l++) {
    const int ci_n = tab.ci[l], co_n = tab.co[l];
    const int64_t n = (int64_t)ci_n * co_n * 9;
    GRID_STRIDE(e, n) {
      int tap = (int)(e % 9);
      int ci = (int)((e / 9) % ci_n), co = (int)(e / (9 * (int64_t)ci_n));
      bf w = __float2bfloat16_rn(theta[tab.off_w[l] + e]);
      int ky = tap / 3, kx = tap % 3;
      wpk[tab.off_pk[l] + (((int64_t)tap * (ci_n / 8) + ci / 8) * co_n + co) * 8 + ci % 8] = w;
      int tt = (2 - ky) * 3 + (2 - kx);
      wpkT[tab.off_pk[l] + (((int64_t)tt * (co_n / 8) + co / 8) * ci_n + ci) * 8 + co % 8] = w;
    }
  }
}

__global__ void k_adam(float* __restrict__ theta, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
  GRID_STRIDE(k, n) {
    float g = grad[k];
    float mk = b1 * m[k] + (1.f - b1) * g;
    float vk = b2 * v[k] + (1.f - b2) * g * g;
    m[k] = mk;
    v[k] = vk;
    theta[k] -= lr * (mk / bc1) / (sqrtf(vk / bc2) + eps);
  }
}

// ------------------------------------------------------------ host side
static int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

struct Ctx {
  Net* g;
  cudaStream_t st;
  Solver* s;  // when run inside a solver step: launches are counted and profiled there
};

#define GL(C, NAME, BYTES, ...)                          \
  do {                                                   \
    if ((C).s) {                                         \
      FS_LAUNCH((C).s, NAME, BYTES, __VA_ARGS__);        \
    } else {                                             \
      __VA_ARGS__;                                       \
      (C).g->launches++;                                 \
    }                                                    \
  } while (0)

static cudaError_t ensure_capacity(Net* g, int B, int H, int W) {
  if (B <= g->capB && H <= g->capH && W <= g->capW) return cudaSuccess;
  int nB = B > g->capB ? B : g->capB, nH = H > g->capH ? H : g->capH, nW = W > g->capW ? W : g->capW;
  for (int k = 0; k < NBUF; k++) {
    if (g->buf[k]) cudaFree(g->buf[k]);
    g->buf[k] = nullptr;
  }
  if (g->out) cudaFree(g->out);
  if (g->gin) cudaFree(g->gin);
  if (g->gmask) cudaFree(g->gmask);
  if (g->res) cudaFree(g->res);
  g->out = g->gin = g->gmask = g->res = nullptr;
  cudaError_t e;
  for (int k = 0; k < NBUF; k++) {
    size_t bytes = (size_t)level_pixels(g, nB, nH, nW, kBufLevel[k]) * kBufCh[k] * 2;
    if ((e = cudaMalloc(&g->buf[k], bytes))) return e;
  }
  size_t npix = (size_t)nB * nH * nW;
  if ((e = cudaMalloc(&g->out, npix * 4))) return e;
  if ((e = cudaMalloc(&g->gin, npix * 4))) return e;
  if ((e = cudaMalloc(&g->gmask, npix * 4))) return e;
  if ((e = cudaMalloc(&g->res, npix * 4))) return e;
  g->capB = nB;
  g->capH = nH;
  g->capW = nW;
  return cudaSuccess;
}

static cudaError_t conv(const Ctx& c, int l, bool transposed, const bf* in, void* out, int B, int H, int W, int epi) {
  Net* g = c.g;
  const int ci = transposed ? kCO[l] : kCI[l], co = transposed ? kCI[l] : kCO[l];
  const bf* w = (transposed ? g->wpkT : g->wpk) + g->off_pk[l];
  const float* bias = transposed ? g->zero_bias : g->theta + g->off_b[l];
  cudaError_t e = cudaSuccess;
  double flops = 2.0 * 9 * ci * co * B * H * W;
  (void)flops;
  const double bytes = (double)(ci + co) * 2 * B * H * W;
  GL(c, "guess_conv", bytes, e = conv::conv3x3(ci, co, epi, in, w, bias, out, B, H, W, g->err, c.st));
  return e;
}

#define CK(expr)                          \
  do {                                    \
    cudaError_t _e = (expr);              \
    if (_e != cudaSuccess) return _e;     \
  } while (0)

static cudaError_t pool(const Ctx& c, Buf in, Buf out, int B, int H, int W, int lev_out) {
  const int C8 = kBufCh[out] / 8, Ho = H >> lev_out, Wo = W >> lev_out;
  int64_t n = (int64_t)B * Ho * Wo * C8;
  GL(c, "guess_pool", n * 80.0,
     k_pool<<<blocks_for(n), 256, 0, c.st>>>((const uint4*)c.g->buf[in], (uint4*)c.g->buf[out], B, Ho, Wo, C8));
  return cudaGetLastError();
}
static cudaError_t poolsum(const Ctx& c, Buf in, Buf out, int B, int H, int W, int lev_out) {
  const int C8 = kBufCh[out] / 8, Ho = H >> lev_out, Wo = W >> lev_out;
  int64_t n = (int64_t)B * Ho * Wo * C8;
  GL(c, "guess_poolsum", n * 80.0,
     k_poolsum<<<blocks_for(n), 256, 0, c.st>>>((const uint4*)c.g->buf[in], (uint4*)c.g->buf[out], B, Ho, Wo, C8));
  return cudaGetLastError();
}
// out = up(coarse) * scale + skip at level lev (fine)
static cudaError_t upadd(const Ctx& c, Buf coarse, Buf skip, Buf out, int B, int H, int W, int lev, float scale) {
  const int C8 = kBufCh[out] / 8, Hf = H >> lev, Wf = W >> lev;
  int64_t n = (int64_t)B * Hf * Wf * C8;
  GL(c, "guess_upadd", n * 52.0,
     k_upadd<<<blocks_for(n), 256, 0, c.st>>>((const uint4*)c.g->buf[coarse], (const uint4*)c.g->buf[skip],
                                              (uint4*)c.g->buf[out], B, Hf, Wf, C8, scale));
  return cudaGetLastError();
}
static cudaError_t relu_mask(const Ctx& c, Buf gbuf, Buf abuf, int B, int H, int W) {
  int n8 = (int)(level_pixels(c.g, B, H, W, kBufLevel[gbuf]) * kBufCh[gbuf] / 8);
  GL(c, "guess_relu_mask", n8 * 48.0,
     k_relu_mask<<<blocks_for(n8), 256, 0, c.st>>>((uint4*)c.g->buf[gbuf], (const uint4*)c.g->buf[abuf], n8));
  return cudaGetLastError();
}

// the network on x0 (already in buf[X0]); result in g->out
static cudaError_t forward(const Ctx& c, int B, int H, int W) {
  Net* g = c.g;
  bf** b = g->buf;
  const int Hl1 = H >> 1, Wl1 = W >> 1, Hl2 = H >> 2, Wl2 = W >> 2, Hl3 = H >> 3, Wl3 = W >> 3;
  CK(conv(c, LA, false, b[X0], b[A0], B, H, W, 1));
  CK(conv(c, LB, false, b[A0], b[A0B], B, H, W, 1));
  CK(pool(c, A0B, Q1, B, H, W, 1));
  CK(conv(c, LC, false, b[Q1], b[A1], B, Hl1, Wl1, 1));
  CK(pool(c, A1, Q2, B, H, W, 2));
  CK(conv(c, LD, false, b[Q2], b[A2], B, Hl2, Wl2, 1));
  CK(pool(c, A2, Q3, B, H, W, 3));
  CK(conv(c, LE, false, b[Q3], b[A3], B, Hl3, Wl3, 1));
  CK(conv(c, LF, false, b[A3], b[F3], B, Hl3, Wl3, 1));
  CK(upadd(c, F3, A2, S2, B, H, W, 2, 1.f));
  CK(conv(c, LG, false, b[S2], b[G2], B, Hl2, Wl2, 1));
  CK(upadd(c, G2, A1, S1, B, H, W, 1, 1.f));
  CK(conv(c, LH, false, b[S1], b[H1], B, Hl1, Wl1, 1));
  CK(upadd(c, H1, A0B, S0, B, H, W, 0, 1.f));
  CK(conv(c, LI, false, b[S0], b[I0], B, H, W, 1));
  CK(conv(c, LJ, false, b[I0], g->out, B, H, W, 2));
  return cudaSuccess;
}

static cudaError_t ensure_corr(Net* g, int64_t floats) {
  if (floats <= g->corr_cap) return cudaSuccess;
  if (g->corr_part) cudaFree(g->corr_part);
  g->corr_part = nullptr;
  CK(cudaMalloc(&g->corr_part, floats * 4));
  g->corr_cap = floats;
  return cudaSuccess;
}

template <int CIN, int COUT, int NMB>
static cudaError_t wgrad_tc(const Ctx& c, int l, Buf xbuf, Buf gbuf, int B, int H, int W) {
  using C = WgCfg<CIN, COUT, NMB>;
  Net* g = c.g;
  static std::atomic<uint64_t> attr{0};
  const uint64_t bit = 1ull << (g->device & 63);
  if (!(attr.load() & bit)) {
    CK(cudaFuncSetAttribute(k_wgrad_tc<CIN, COUT, NMB>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
    attr.fetch_or(bit);
  }
  const int groups = (C::MBLK + NMB - 1) / NMB;
  const int64_t ntiles = (int64_t)B * H * ((W + kWgTile - 1) / kWgTile);
  const int P = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, 4 * 152 / groups));
  const int64_t nw = (int64_t)C::MROWS * COUT;
  CK(ensure_corr(g, (int64_t)P * (nw + COUT)));
  float* part = g->corr_part;
  float* bpart = part + (int64_t)P * nw;
  GL(c, "guess_wgrad", (double)(CIN + COUT) * 2 * B * H * W,
     (k_wgrad_tc<CIN, COUT, NMB><<<dim3(P, groups), kWgThreads, C::SMEM, c.st>>>(
         reinterpret_cast<const uint4*>(g->buf[xbuf]), reinterpret_cast<const uint4*>(g->buf[gbuf]), B, H, W, part,
         bpart, g->err)));
  CK(cudaGetLastError());
  GL(c, "guess_wgrad_reduce", (double)P * (nw + COUT) * 4,
     k_wgrad_reduce<<<blocks_for(nw + COUT), 256, 0, c.st>>>(part, bpart, P, CIN, COUT, g->grad + g->off_w[l],
                                                            g->grad + g->off_b[l]));
  return cudaGetLastError();
}

// the (c_in, c_out) pairs of the network, M-blocks per CTA
static cudaError_t wgrad(const Ctx& c, int l, Buf xbuf, Buf gbuf, int B, int H, int W) {
  const int ci = kCI[l], co = kCO[l];
#define FS_WG(a, b, nmb) \
  if (ci == a && co == b) return wgrad_tc<a, b, nmb>(c, l, xbuf, gbuf, B, H, W);
  FS_WG(16, 16, 2)
  FS_WG(16, 32, 2)
  FS_WG(32, 16, 3)
  FS_WG(32, 64, 3)
  FS_WG(64, 128, 3)
  FS_WG(128, 64, 2)
  FS_WG(64, 32, 3)
#undef FS_WG
  return cudaErrorInvalidValue;
}

// loss against target (f32 [B][H][W]) and the gradient of every parameter into g->grad
static cudaError_t backward(const Ctx& c, const float* target, int B, int H, int W) {
  Net* g = c.g;
  bf** b = g->buf;
  const int64_t npix = (int64_t)H * W;
  const int Hl1 = H >> 1, Wl1 = W >> 1, Hl2 = H >> 2, Wl2 = W >> 2, Hl3 = H >> 3, Wl3 = W >> 3;
  CK(cudaMemsetAsync(g->acc, 0, sizeof(double) * (B + 1), c.st));
  int lb = (int)((npix + 255) / 256);
  if (lb > 256) lb = 256;
  GL(c, "guess_loss", npix * B * 8.0, k_loss_mean<<<dim3(lb, B), 256, 0, c.st>>>(g->out, target, g->acc, npix));
  const bool with_res = g->w_r != 0.0;
  if (with_res)
    GL(c, "guess_loss", npix * B * 12.0,
       k_loss_res<<<dim3(lb, B), 256, 0, c.st>>>(g->out, target, g->res, g->acc, H, W, B, g->w_r));
  GL(c, "guess_loss", npix * B * 40.0,
     k_loss_seed<<<dim3(lb, B), 256, 0, c.st>>>(g->out, target, with_res ? g->res : nullptr, g->acc,
                                                (uint4*)b[GJ], H, W, B, g->w_p, g->w_r));
  CK(cudaGetLastError());
  CK(wgrad(c, LJ, I0, GJ, B, H, W));
  CK(conv(c, LJ, true, b[GJ], b[DI0], B, H, W, 0));
  CK(relu_mask(c, DI0, I0, B, H, W));
  CK(wgrad(c, LI, S0, DI0, B, H, W));
  CK(conv(c, LI, true, b[DI0], b[DS0], B, H, W, 0));
  CK(poolsum(c, DS0, DH1, B, H, W, 1));
  CK(relu_mask(c, DH1, H1, B, H, W));
  CK(wgrad(c, LH, S1, DH1, B, Hl1, Wl1));
  CK(conv(c, LH, true, b[DH1], b[DS1], B, Hl1, Wl1, 0));
  CK(poolsum(c, DS1, DG2, B, H, W, 2));
  CK(relu_mask(c, DG2, G2, B, H, W));
  CK(wgrad(c, LG, S2, DG2, B, Hl2, Wl2));
  CK(conv(c, LG, true, b[DG2], b[DS2], B, Hl2, Wl2, 0));
  CK(poolsum(c, DS2, DF3, B, H, W, 3));
  CK(relu_mask(c, DF3, F3, B, H, W));
  CK(wgrad(c, LF, A3, DF3, B, Hl3, Wl3));
  CK(conv(c, LF, true, b[DF3], b[DA3], B, Hl3, Wl3, 0));
  CK(relu_mask(c, DA3, A3, B, H, W));
  CK(wgrad(c, LE, Q3, DA3, B, Hl3, Wl3));
  CK(conv(c, LE, true, b[DA3], b[DQ3], B, Hl3, Wl3, 0));
  // da2 = ds2 + up(dq3) / 4, masked
  CK(upadd(c, DQ3, DS2, DS2, B, H, W, 2, 0.25f));
  CK(relu_mask(c, DS2, A2, B, H, W));
  CK(wgrad(c, LD, Q2, DS2, B, Hl2, Wl2));
  CK(conv(c, LD, true, b[DS2], b[DQ2], B, Hl2, Wl2, 0));
  CK(upadd(c, DQ2, DS1, DS1, B, H, W, 1, 0.25f));
  CK(relu_mask(c, DS1, A1, B, H, W));
  CK(wgrad(c, LC, Q1, DS1, B, Hl1, Wl1));
  CK(conv(c, LC, true, b[DS1], b[DQ1], B, Hl1, Wl1, 0));
  CK(upadd(c, DQ1, DS0, DS0, B, H, W, 0, 0.25f));
  CK(relu_mask(c, DS0, A0B, B, H, W));
  CK(wgrad(c, LB, A0, DS0, B, H, W));
  CK(conv(c, LB, true, b[DS0], b[DA0], B, H, W, 0));
  CK(relu_mask(c, DA0, A0, B, H, W));
  CK(wgrad(c, LA, X0, DA0, B, H, W));
  return cudaSuccess;
}

static cudaError_t repack(Net* g, cudaStream_t st) {
  PackTable tab;
  for (int l = 0; l < NL; l++) {
    tab.off_w[l] = g->off_w[l];
    tab.off_pk[l] = g->off_pk[l];
    tab.ci[l] = kCI[l];
    tab.co[l] = kCO[l];
  }
  k_pack<<<152 * 4, 256, 0, st>>>(g->theta, g->wpk, g->wpkT, tab);
  g->launches++;
  return cudaGetLastError();
}

// He-normal initial weights (ReLU layers; the output layer scaled by 0.1),
// zero biases; the padded input channels of layer A start (and stay) at zero.
// Gaussian draws: SplitMix64 + Box-Muller.
static void init_params(std::vector<float>& th, const Net* g, uint64_t seed) {
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E5ull;
  auto next = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  for (int l = 0; l < NL; l++) {
    const int ci = kCI[l], co = kCO[l];
    const double fan = 9.0 * (l == LA ? 2 : ci);
    const double sd = sqrt(2.0 / fan) * (kRelu[l] ? 1.0 : 0.1);
    for (int o = 0; o < co; o++)
      for (int i = 0; i < ci; i++)
        for (int t = 0; t < 9; t++) {
          double u1 = unif(), u2 = unif();
          double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
          th[g->off_w[l] + ((int64_t)o * ci + i) * 9 + t] = (l == LA && i >= 2) ? 0.f : (float)(z * sd);
        }
    for (int o = 0; o < co; o++) th[g->off_b[l] + o] = 0.f;
  }
}

}  // namespace guess

// ---------------------------------------------------------- solver hooks
// The network runs at 1/f of the grid resolution (f = 1 or 2).
// h^2 * (d averaged over f x f fine cells) at net resolution, the solid mask
// at the net cell centres, and the sum of squares of the former (for sigma).
__global__ void __launch_bounds__(256)
    k_guess_in(const float* __restrict__ dh, const float* __restrict__ dl, int nx, int ny, int f, float h2,
               float* gin, float* gmask, const float* __restrict__ disks, int ndisk, float dxn, float dyn, float lx,
               float ly, float width, RedCtx ctx) {
  const int Wn = nx / f, Hn = ny / f;
  const int n = Wn * Hn;  // grids are capped at 2^30 cells
  double s2 = 0.0;
  GRID_STRIDE32(k, n) {
    int J = k / Wn, I = k - J * Wn;
    int64_t c = (int64_t)(f * J) * nx + f * I;
    // the divergence is a double-float pair (MIXED) or a plain f32 field (dl == nullptr)
    auto at = [&](int64_t q) { return dl ? __fadd_rn(dh[q], dl[q]) : dh[q]; };
    float d = f == 1 ? at(c) : 0.25f * (at(c) + at(c + 1) + at(c + nx) + at(c + nx + 1));
    float x = h2 * d;
    gin[k] = x;
    s2 += (double)x * x;
    float m = 0.f;
    float px = (I + 0.5f) * dxn, py = (J + 0.5f) * dyn;
    for (int q = 0; q < ndisk; q++) {
      float ax = px - disks[7 * q], ay = py - disks[7 * q + 1];
      ax -= lx * floorf(ax / lx + 0.5f);
      ay -= ly * floorf(ay / ly + 0.5f);
      float chi = 0.5f * (1.f - tanhf(fminf(fmaxf((sqrtf(ax * ax + ay * ay) - disks[7 * q + 2]) / width, -10.f), 10.f)));
      m = fmaxf(m, chi);
    }
    gmask[k] = m;
  }
  block_sum2_finish(s2, 0.0, ctx);
}

// pressure guess = sigma * out at the fine cells: a copy for f = 1, the
// bilinear multigrid prolongation stencil for f = 2; pl = 0
__global__ void __launch_bounds__(256) k_guess_out(const float* __restrict__ out, const double* __restrict__ sumsq,
                                                   int64_t nnorm, float* __restrict__ ph, float* __restrict__ pl,
                                                   int nx, int ny, int f) {
  const int Wn = nx / f, Hn = ny / f;
  const float sig = guess::block_sigma(sumsq, nnorm);
  const int n = nx * ny;  // grids are capped at 2^30 cells
  GRID_STRIDE32(k, n) {
    float v;
    if (f == 1) {
      v = out[k] * sig;
    } else {
      int j = k / nx, i = k - j * nx;
      int ci0 = (i & 1) ? (i >> 1) : (i >> 1) - 1, cj0 = (j & 1) ? (j >> 1) : (j >> 1) - 1;
      float fx = (i & 1) ? 0.25f : 0.75f, fy = (j & 1) ? 0.25f : 0.75f;
      int x0 = ci0 < 0 ? ci0 + Wn : ci0, x1 = ci0 + 1 >= Wn ? ci0 + 1 - Wn : ci0 + 1;
      int y0 = cj0 < 0 ? cj0 + Hn : cj0, y1 = cj0 + 1 >= Hn ? cj0 + 1 - Hn : cj0 + 1;
      float a = out[(int64_t)y0 * Wn + x0], b = out[(int64_t)y0 * Wn + x1];
      float c = out[(int64_t)y1 * Wn + x0], d = out[(int64_t)y1 * Wn + x1];
      v = ((1.f - fy) * ((1.f - fx) * a + fx * b) + fy * ((1.f - fx) * c + fx * d)) * sig;
    }
    ph[k] = v;
    if (pl) pl[k] = 0.f;
  }
}

bool guess_supported(const Solver* s, int f) {
  if (f != 1 && f != 2) return false;
  const int m = 8 * f;
  return s->g.nx % m == 0 && s->g.ny % m == 0;
}

// enqueue the guess into (ph, pl) (MIXED) or p32 (F32) on s->stream
int guess_enqueue(Solver* s, fs_guess* handle, int f) {
  guess::Net* g = reinterpret_cast<guess::Net*>(handle);
  const Grid& gr = s->g;
  const int Wn = gr.nx / f, Hn = gr.ny / f;
  const float h2 = (float)(f * f * gr.dxd * gr.dxd);
  guess::Ctx c{g, s->stream, s};
  double* gsum = g->acc;
  RedCtx ctx = red_ctx(s, gsum);
  const int nd = (int)s->disks.size();
  const float* dsk = static_cast<const float*>(s->d_disks);
  const double width = s->prm.solid_mask_width * gr.dxd;
  int blocks = (int)std::min<int64_t>(((int64_t)Wn * Hn + 255) / 256, 152 * 8);
  if (blocks > s->red_cap) blocks = s->red_cap;
  FS_LAUNCH(s, "guess_in", (double)s->n * 8,
            k_guess_in<<<blocks, 256, 0, s->stream>>>(s->mixed ? s->dh : s->div32, s->mixed ? s->dl : nullptr,
                                                      gr.nx, gr.ny, f, h2, g->gin, g->gmask, dsk, nd,
                                                      (float)(f * gr.dxd), (float)(f * gr.dyd), (float)s->prm.lx,
                                                      (float)s->prm.ly, (float)width, ctx));
  const int64_t npn = (int64_t)Wn * Hn;
  FS_LAUNCH(s, "guess_prep", (double)npn * 40,
            guess::k_prep<<<guess::blocks_for(npn), 256, 0, s->stream>>>(g->gin, g->gmask, (uint4*)g->buf[guess::X0],
                                                                         npn, gsum, npn));
  cudaError_t e = guess::forward(c, 1, Hn, Wn);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("pressure guess: ") + cudaGetErrorString(e));
  FS_LAUNCH(s, "guess_out", (double)s->n * 8,
            k_guess_out<<<guess::blocks_for(s->n), 256, 0, s->stream>>>(
                g->out, gsum, npn, s->mixed ? s->ph : s->p32, s->mixed ? s->pl : nullptr, gr.nx, gr.ny, f));
  return FS_OK;
}

int guess_prepare(Solver* s, fs_guess* handle, int f) {
  guess::Net* g = reinterpret_cast<guess::Net*>(handle);
  cudaError_t e = guess::ensure_capacity(g, 1, s->g.ny / f, s->g.nx / f);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_OUT_OF_MEMORY, std::string("pressure guess buffers: ") + cudaGetErrorString(e));
  return FS_OK;
}

// the divergence, mask and pressure of the last projection at 1/factor of the
// grid resolution (block averages; the mask at the coarse cell centres)
__global__ void k_pair(const float* __restrict__ dh, const float* __restrict__ dl, const float* __restrict__ ph,
                       const float* __restrict__ pl, int nx, int ny, int f, float* div, float* mask, float* p,
                       const float* __restrict__ disks, int ndisk, float dxc, float dyc, float lx, float ly,
                       float width) {
  const int Wc = nx / f, Hc = ny / f;
  const int64_t n = (int64_t)Wc * Hc;
  GRID_STRIDE(k, n) {
    int I = (int)(k % Wc), J = (int)(k / Wc);
    double sd = 0.0, sp = 0.0;
    for (int a = 0; a < f; a++)
      for (int b = 0; b < f; b++) {
        int64_t c = (int64_t)(f * J + a) * nx + f * I + b;
        sd += (double)dh[c] + (dl ? (double)dl[c] : 0.0);
        sp += (double)ph[c] + (pl ? (double)pl[c] : 0.0);
      }
    div[k] = (float)(sd / (f * f));
    p[k] = (float)(sp / (f * f));
    float m = 0.f;
    float px = (I + 0.5f) * dxc, py = (J + 0.5f) * dyc;
    for (int q = 0; q < ndisk; q++) {
      float ax = px - disks[7 * q], ay = py - disks[7 * q + 1];
      ax -= lx * floorf(ax / lx + 0.5f);
      ay -= ly * floorf(ay / ly + 0.5f);
      float chi = 0.5f * (1.f - tanhf(fminf(fmaxf((sqrtf(ax * ax + ay * ay) - disks[7 * q + 2]) / width, -10.f), 10.f)));
      m = fmaxf(m, chi);
    }
    mask[k] = m;
  }
}

int dump_pair(Solver* s, int f, float* div, float* mask, float* p) {
  const Grid& gr = s->g;
  const double width = s->prm.solid_mask_width * gr.dxd;
  const int nd = (int)s->disks.size();
  const int64_t n = (int64_t)(gr.nx / f) * (gr.ny / f);
  float* tmp = nullptr;
  cudaError_t e = cudaMalloc(&tmp, n * 3 * sizeof(float));
  if (e != cudaSuccess) return fail_status(s, FS_ERR_OUT_OF_MEMORY, "fs_dump_pair: cudaMalloc failed");
  k_pair<<<guess::blocks_for(n), 256, 0, s->stream>>>(
      s->mixed ? s->dh : s->div32, s->mixed ? s->dl : nullptr, s->mixed ? s->ph : s->p32, s->mixed ? s->pl : nullptr,
      gr.nx, gr.ny, f, tmp, tmp + n, tmp + 2 * n, static_cast<const float*>(s->d_disks), nd, (float)(f * gr.dxd),
      (float)(f * gr.dyd), (float)s->prm.lx, (float)s->prm.ly, (float)width);
  s->launches++;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(div, tmp, n * 4, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mask, tmp + n, n * 4, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(p, tmp + 2 * n, n * 4, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("fs_dump_pair: ") + cudaGetErrorString(e));
  return FS_OK;
}

// the same pair into caller-owned device buffers, enqueued on the solver's
// stream (no allocation, no synchronisation)
int dump_pair_device(Solver* s, int f, float* div, float* mask, float* p) {
  const Grid& gr = s->g;
  const double width = s->prm.solid_mask_width * gr.dxd;
  const int nd = (int)s->disks.size();
  const int64_t n = (int64_t)(gr.nx / f) * (gr.ny / f);
  k_pair<<<guess::blocks_for(n), 256, 0, s->stream>>>(
      s->mixed ? s->dh : s->div32, s->mixed ? s->dl : nullptr, s->mixed ? s->ph : s->p32, s->mixed ? s->pl : nullptr,
      gr.nx, gr.ny, f, div, mask, p, static_cast<const float*>(s->d_disks), nd, (float)(f * gr.dxd),
      (float)(f * gr.dyd), (float)s->prm.lx, (float)s->prm.ly, (float)width);
  s->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_status(s, FS_ERR_CUDA, std::string("fs_dump_pair_device: ") + cudaGetErrorString(e));
  return FS_OK;
}

}  // namespace fs

// ====================================================================== C ABI
using namespace fs;
using namespace fs::guess;

static thread_local std::string g_guess_err;

static int gfail(Net* g, int code, const std::string& m) {
  if (g) g->err_msg = m;
  record_error(m);
  return code;
}

static int gcuda(Net* g, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return FS_OK;
  return gfail(g, e == cudaErrorMemoryAllocation ? FS_ERR_OUT_OF_MEMORY : FS_ERR_CUDA,
               std::string(where) + ": " + cudaGetErrorString(e));
}

extern "C" FS_API int fs_guess_create(int32_t device, uint64_t seed, fs_guess** out) {
  if (!out) return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_guess_create: NULL out");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return gfail(nullptr, FS_ERR_NO_DEVICE, "fs_guess_create: no CUDA device");
  if (device < 0 || device >= ndev) return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_guess_create: bad device");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return gcuda(nullptr, e, "cudaSetDevice");
  Net* g = new Net();
  g->device = device;
  int64_t k = 0, kp = 0;
  for (int l = 0; l < NL; l++) {
    g->off_w[l] = k;
    k += (int64_t)kCI[l] * kCO[l] * 9;
    g->off_b[l] = k;
    k += kCO[l];
    g->off_pk[l] = kp;
    kp += (int64_t)kCI[l] * kCO[l] * 9;
  }
  g->nparam = k;
  g->npk = kp;
  std::vector<float> th(k);
  init_params(th, g, seed);
#define GA(p, bytes)                                   \
  if ((e = cudaMalloc(&(p), (bytes))) != cudaSuccess) { \
    fs_guess_destroy(reinterpret_cast<fs_guess*>(g));  \
    return gcuda(nullptr, e, "fs_guess_create");        \
  }
  GA(g->theta, k * 4);
  GA(g->grad, k * 4);
  GA(g->m, k * 4);
  GA(g->v, k * 4);
  GA(g->wpk, kp * 2);
  GA(g->wpkT, kp * 2);
  GA(g->zero_bias, 256 * 4);
  GA(g->err, 4);
  GA(g->acc, 4096 * 8);
#undef GA
  if ((e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    fs_guess_destroy(reinterpret_cast<fs_guess*>(g));
    return gcuda(nullptr, e, "cudaStreamCreate");
  }
  cudaMemsetAsync(g->grad, 0, k * 4, g->stream);
  cudaMemsetAsync(g->m, 0, k * 4, g->stream);
  cudaMemsetAsync(g->v, 0, k * 4, g->stream);
  cudaMemsetAsync(g->zero_bias, 0, 256 * 4, g->stream);
  cudaMemsetAsync(g->err, 0, 4, g->stream);
  cudaMemcpyAsync(g->theta, th.data(), k * 4, cudaMemcpyHostToDevice, g->stream);
  repack(g, g->stream);
  e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) {
    fs_guess_destroy(reinterpret_cast<fs_guess*>(g));
    return gcuda(nullptr, e, "fs_guess_create");
  }
  *out = reinterpret_cast<fs_guess*>(g);
  return FS_OK;
}

extern "C" FS_API void fs_guess_destroy(fs_guess* h) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (int k = 0; k < NBUF; k++)
    if (g->buf[k]) cudaFree(g->buf[k]);
  float* fl[] = {g->theta, g->grad, g->m, g->v, g->zero_bias, g->out, g->gin, g->gmask, g->res, g->corr_part};
  for (float* p : fl)
    if (p) cudaFree(p);
  if (g->wpk) cudaFree(g->wpk);
  if (g->wpkT) cudaFree(g->wpkT);
  if (g->err) cudaFree(g->err);
  if (g->acc) cudaFree(g->acc);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

extern "C" FS_API int64_t fs_guess_num_params(const fs_guess* h) {
  const Net* g = reinterpret_cast<const Net*>(h);
  return g ? g->nparam : -1;
}

extern "C" FS_API int fs_guess_get_params(fs_guess* h, float* host, int64_t n) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g || !host) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_get_params: NULL argument");
  if (n != g->nparam) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_get_params: wrong parameter count");
  cudaSetDevice(g->device);
  cudaError_t e = cudaMemcpyAsync(host, g->theta, n * 4, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  return gcuda(g, e, "fs_guess_get_params");
}

extern "C" FS_API int fs_guess_set_params(fs_guess* h, const float* host, int64_t n) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g || !host) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_set_params: NULL argument");
  if (n != g->nparam) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_set_params: wrong parameter count");
  cudaSetDevice(g->device);
  cudaError_t e = cudaMemcpyAsync(g->theta, host, n * 4, cudaMemcpyHostToDevice, g->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->m, 0, n * 4, g->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->v, 0, n * 4, g->stream);
  if (e == cudaSuccess) e = repack(g, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  g->adam_t = 0;
  return gcuda(g, e, "fs_guess_set_params");
}

static int check_shape(Net* g, int B, int H, int W, const char* who) {
  if (B < 1 || H < 8 || W < 8 || H % 8 || W % 8)
    return gfail(g, FS_ERR_INVALID_ARGUMENT, std::string(who) + ": batch >= 1 and H, W multiples of 8 (>= 8)");
  if ((int64_t)B * H * W * 16 >= ((int64_t)1 << 31))
    return gfail(g, FS_ERR_INVALID_ARGUMENT, std::string(who) + ": batch x H x W x 16 must stay below 2^31");
  return FS_OK;
}

static int read_err(Net* g, const char* who) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, g->err, 4, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) return gcuda(g, e, who);
  if (h) {
    cudaMemsetAsync(g->err, 0, 4, g->stream);
    return gfail(g, FS_ERR_CUDA, std::string(who) + ": a tensor-core completion wait timed out");
  }
  return FS_OK;
}

// out = network(div_n, mask): device pointers, f32 [B][H][W]
extern "C" FS_API int fs_guess_predict(fs_guess* h, const float* d_div, const float* d_mask, int32_t B, int32_t H,
                                       int32_t W, float* d_out) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g || !d_div || !d_out) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_predict: NULL argument");
  int rc = check_shape(g, B, H, W, "fs_guess_predict");
  if (rc) return rc;
  cudaSetDevice(g->device);
  cudaError_t e = ensure_capacity(g, B, H, W);
  if (e != cudaSuccess) return gcuda(g, e, "fs_guess_predict");
  Ctx c{g, g->stream, nullptr};
  const int64_t np = (int64_t)B * H * W;
  k_prep<<<blocks_for(np), 256, 0, g->stream>>>(d_div, d_mask, (uint4*)g->buf[X0], np, nullptr, 1);
  g->launches++;
  if ((e = forward(c, B, H, W)) != cudaSuccess) return gcuda(g, e, "fs_guess_predict");
  e = cudaMemcpyAsync(d_out, g->out, np * 4, cudaMemcpyDeviceToDevice, g->stream);
  if (e != cudaSuccess) return gcuda(g, e, "fs_guess_predict");
  return read_err(g, "fs_guess_predict");
}

static int loss_grad_impl(Net* g, const float* d_div, const float* d_mask, const float* d_tgt, int B, int H, int W,
                          double* loss, const char* who) {
  int rc = check_shape(g, B, H, W, who);
  if (rc) return rc;
  if (B > 4000) return gfail(g, FS_ERR_INVALID_ARGUMENT, std::string(who) + ": batch above 4000");
  cudaSetDevice(g->device);
  cudaError_t e = ensure_capacity(g, B, H, W);
  if (e != cudaSuccess) return gcuda(g, e, who);
  Ctx c{g, g->stream, nullptr};
  const int64_t np = (int64_t)B * H * W;
  k_prep<<<blocks_for(np), 256, 0, g->stream>>>(d_div, d_mask, (uint4*)g->buf[X0], np, nullptr, 1);
  g->launches++;
  if ((e = forward(c, B, H, W)) != cudaSuccess) return gcuda(g, e, who);
  if ((e = backward(c, d_tgt, B, H, W)) != cudaSuccess) return gcuda(g, e, who);
  if (loss) {
    e = cudaMemcpyAsync(loss, g->acc + B, 8, cudaMemcpyDeviceToHost, g->stream);
    if (e != cudaSuccess) return gcuda(g, e, who);
  }
  return FS_OK;
}

extern "C" FS_API int fs_guess_loss_grad(fs_guess* h, const float* d_div, const float* d_mask, const float* d_target,
                                         int32_t B, int32_t H, int32_t W, double* loss, float* d_grad) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g || !d_div || !d_target) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_loss_grad: NULL argument");
  int rc = loss_grad_impl(g, d_div, d_mask, d_target, B, H, W, loss, "fs_guess_loss_grad");
  if (rc) return rc;
  if (d_grad) {
    cudaError_t e = cudaMemcpyAsync(d_grad, g->grad, g->nparam * 4, cudaMemcpyDeviceToDevice, g->stream);
    if (e != cudaSuccess) return gcuda(g, e, "fs_guess_loss_grad");
  }
  return read_err(g, "fs_guess_loss_grad");
}

extern "C" FS_API int fs_guess_train_step(fs_guess* h, const float* d_div, const float* d_mask, const float* d_target,
                                          int32_t B, int32_t H, int32_t W, float lr, double* loss) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g || !d_div || !d_target) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_train_step: NULL argument");
  if (!(lr > 0.f)) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_train_step: lr must be positive");
  int rc = loss_grad_impl(g, d_div, d_mask, d_target, B, H, W, loss, "fs_guess_train_step");
  if (rc) return rc;
  g->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = (float)(1.0 - pow(0.9, (double)g->adam_t)), bc2 = (float)(1.0 - pow(0.999, (double)g->adam_t));
  k_adam<<<blocks_for(g->nparam), 256, 0, g->stream>>>(g->theta, g->grad, g->m, g->v, g->nparam, lr, b1, b2, 1e-8f,
                                                      bc1, bc2);
  g->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = repack(g, g->stream);
  if (e != cudaSuccess) return gcuda(g, e, "fs_guess_train_step");
  return loss ? read_err(g, "fs_guess_train_step") : FS_OK;
}

extern "C" FS_API int fs_guess_set_loss(fs_guess* h, double w_pressure, double w_residual) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_set_loss: NULL handle");
  if (!(w_pressure >= 0) || !(w_residual >= 0) || !(w_pressure + w_residual > 0) || !std::isfinite(w_pressure) ||
      !std::isfinite(w_residual))
    return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_set_loss: weights must be finite, >= 0, not both 0");
  g->w_p = w_pressure;
  g->w_r = w_residual;
  return FS_OK;
}

extern "C" FS_API int fs_guess_sync(fs_guess* h) {
  Net* g = reinterpret_cast<Net*>(h);
  if (!g) return gfail(g, FS_ERR_INVALID_ARGUMENT, "fs_guess_sync: NULL handle");
  return read_err(g, "fs_guess_sync");
}

extern "C" FS_API int64_t fs_guess_launch_count(const fs_guess* h) {
  const Net* g = reinterpret_cast<const Net*>(h);
  return g ? g->launches : -1;
}

// ---------------------------------------------------- training-pair files
// "FSPAIR" file: a 40-byte little-endian header then three f32 fields.
//   0  char[8]  magic "FSPAIR\0\1"
//   8  uint32   version (1)
//  12  uint32   nx
//  16  uint32   ny
//  20  uint32   dtype (0 = f32)
//  24  double   dx, the grid spacing of the stored fields
//  32  uint32   nfields (3: div, mask, p)
//  36  uint32   reserved (0)
//  40  div[ny][nx], mask[ny][nx], p[ny][nx]
static const char kPairMagic[8] = {'F', 'S', 'P', 'A', 'I', 'R', 0, 1};

extern "C" FS_API int fs_write_pair_file(const char* path, int32_t nx, int32_t ny, double dx, const float* div,
                                         const float* mask, const float* p) {
  if (!path || !div || !mask || !p || nx < 1 || ny < 1 || !(dx > 0))
    return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_write_pair_file: bad argument");
  FILE* f = fopen(path, "wb");
  if (!f) return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, std::string("fs_write_pair_file: cannot open ") + path);
  unsigned char hdr[40] = {};
  uint32_t u[7] = {1u, (uint32_t)nx, (uint32_t)ny, 0u, 0u, 3u, 0u};
  memcpy(hdr, kPairMagic, 8);
  memcpy(hdr + 8, &u[0], 4);
  memcpy(hdr + 12, &u[1], 4);
  memcpy(hdr + 16, &u[2], 4);
  memcpy(hdr + 20, &u[3], 4);
  memcpy(hdr + 24, &dx, 8);
  memcpy(hdr + 32, &u[5], 4);
  memcpy(hdr + 36, &u[6], 4);
  const size_t n = (size_t)nx * ny;
  bool ok = fwrite(hdr, 1, 40, f) == 40 && fwrite(div, 4, n, f) == n && fwrite(mask, 4, n, f) == n &&
            fwrite(p, 4, n, f) == n;
  ok = (fclose(f) == 0) && ok;
  return ok ? FS_OK : gfail(nullptr, FS_ERR_CUDA, "fs_write_pair_file: write failed");
}

// With div == NULL only the header is read (to size the buffers).
extern "C" FS_API int fs_read_pair_file(const char* path, int32_t* nx, int32_t* ny, double* dx, float* div,
                                        float* mask, float* p) {
  if (!path || !nx || !ny || !dx) return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_read_pair_file: bad argument");
  FILE* f = fopen(path, "rb");
  if (!f) return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, std::string("fs_read_pair_file: cannot open ") + path);
  unsigned char hdr[40];
  uint32_t ver, unx, uny, dtype, nf;
  bool ok = fread(hdr, 1, 40, f) == 40 && memcmp(hdr, kPairMagic, 8) == 0;
  if (ok) {
    memcpy(&ver, hdr + 8, 4);
    memcpy(&unx, hdr + 12, 4);
    memcpy(&uny, hdr + 16, 4);
    memcpy(&dtype, hdr + 20, 4);
    memcpy(dx, hdr + 24, 8);
    memcpy(&nf, hdr + 32, 4);
    ok = ver == 1 && dtype == 0 && nf == 3 && unx > 0 && uny > 0 && unx < (1u << 20) && uny < (1u << 20);
  }
  if (!ok) {
    fclose(f);
    return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_read_pair_file: not a version-1 f32 FSPAIR file");
  }
  *nx = (int32_t)unx;
  *ny = (int32_t)uny;
  if (div) {
    const size_t n = (size_t)unx * uny;
    if (!mask || !p) {
      fclose(f);
      return gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_read_pair_file: NULL field buffer");
    }
    ok = fread(div, 4, n, f) == n && fread(mask, 4, n, f) == n && fread(p, 4, n, f) == n;
  }
  fclose(f);
  return ok ? FS_OK : gfail(nullptr, FS_ERR_INVALID_ARGUMENT, "fs_read_pair_file: truncated file");
}
