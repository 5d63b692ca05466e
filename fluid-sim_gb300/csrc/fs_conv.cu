// fs_conv.cu -- 3x3 periodic convolution of NHWC bf16 images on the tcgen05
// tensor cores (implicit GEMM), the building block of the pressure-guess
// network.  No counterpart in the reference.
//
// out[b, y, x, co] = bias[co] + sum_{ky, kx, ci} w[co, ci, ky, kx] * in[b, y + ky - 1, x + kx - 1, ci]
// with periodic wrap in x and y (the flow domain is periodic), optional ReLU.
//
// GEMM view: M = 128 consecutive pixels of one image row, N = C_out,
// K = 9 taps x C_in.  A CTA (four warps) owns TY rows x 128 pixels.  It stages the input
// halo tile once, as channel-chunk planes [kc][TY + 2][130][8 channels], so
// that 8 consecutive pixels of one chunk form one 128-byte core matrix and
// every tap's A operand is the same tile seen through a descriptor whose start
// address is shifted by (dy, dx) -- no data is rearranged per tap.  Weights
// are packed on the host side of the network as [tap][kc][co][8 ci] (the B
// operand, K-major) and staged one tap at a time into two alternating buffers,
// so the copy of tap t+1 overlaps the MMAs of tap t.  One thread issues the
// MMAs; the accumulators (TY x C_out f32 columns x 128 lanes) live in TMEM and
// the four warps read them back (lane = pixel) for the bias/ReLU/bf16 epilogue.
// Images narrower than 128 pixels are staged wrapped around, so the extra
// lanes compute copies of real pixels and are not stored.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/fluid.h"
#include "fs_tc.cuh"

namespace fs {
void record_error(const std::string& msg);
}

namespace fs {
namespace conv {

constexpr int kThreads = 128;  // four warps: one per TMEM lane quarter
constexpr int kTX = 128;       // pixels per M tile
constexpr int kTW = kTX + 2;   // staged tile width (halo of 1)

__host__ __device__ constexpr int align128(int x) { return (x + 127) & ~127; }

template <int CIN, int COUT, int TY, int NS>
struct Cfg {
  static constexpr int KC = CIN / 8;
  static constexpr int NSPLIT = COUT / NS;                   // CTAs sharing one pixel tile
  // bytes of one chunk plane, padded to 64 mod 128 so that the two chunks of
  // one pixel (stored by neighbouring threads) fall in different banks
  static constexpr int PLANE = ((TY + 2) * kTW * 16 + 63) / 128 * 128 + 64;
  static constexpr int IN_BYTES = align128(KC * PLANE);
  static constexpr int WTAP = KC * NS * 16;                  // bytes of one tap of this CTA's weights
  static constexpr int W_BYTES = align128(WTAP);
  // all nine taps of weights resident (one staging pass, one commit) when small
  static constexpr bool WALL = 9 * WTAP <= 40 * 1024;
  static constexpr int WALL_BYTES = align128(9 * WTAP);
  static constexpr int NCOL_USED = TY * NS;
  static constexpr int NCOL = NCOL_USED <= 32 ? 32 : NCOL_USED <= 64 ? 64 : NCOL_USED <= 128 ? 128 : NCOL_USED <= 256 ? 256 : 512;
  static constexpr int WREGION = WALL ? WALL_BYTES : 2 * W_BYTES;
  static constexpr int SMEM = IN_BYTES + WREGION + 128;  // + barriers and the TMEM slot
  static_assert(CIN % 16 == 0 && NS % 16 == 0 && NS <= 256 && COUT % NS == 0, "channel counts");
  static_assert(NCOL_USED <= 512, "TMEM columns");
};

__device__ __forceinline__ int wrapm(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// EPI: 0 = bias, 1 = bias + ReLU (bf16 NHWC out); 2 = bias, channel 0 only,
// f32 planar out (the network's output layer)
template <int CIN, int COUT, int TY, int NS, int EPI>
__global__ void __launch_bounds__(kThreads) k_conv3x3(const uint4* __restrict__ in, const uint4* __restrict__ wpk,
                                                      const float* __restrict__ bias, void* __restrict__ out,
                                                      int H, int W, int* __restrict__ err) {
  using C = Cfg<CIN, COUT, TY, NS>;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* tile = smem;
  unsigned char* wbuf0 = smem + C::IN_BYTES;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::IN_BYTES + C::WREGION);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
  int* failed = reinterpret_cast<int*>(bar + 3);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * TY;
  const int b = blockIdx.z / C::NSPLIT, n0 = (blockIdx.z % C::NSPLIT) * NS;  // image, first output channel

  if (warp == 0) {
    tc::tmem_alloc(tslot, C::NCOL);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_fence_init();
    *failed = 0;
  }
  // input halo tile, periodic wrap: each thread owns one (column, 8-channel
  // chunk) of the tile and loads its TY + 2 rows, all in flight before the
  // shared-memory stores
  {
    const uint4* img = in + (int64_t)b * H * W * C::KC;
    const bool wide = W >= kTW, tall = H >= TY + 2;  // coordinates wrap at most once
    for (int cc = tid; cc < kTW * C::KC; cc += kThreads) {
      const int xx = cc / C::KC, kc = cc - xx * C::KC;
      int gx = x0 - 1 + xx;
      gx = wide ? (gx < 0 ? gx + W : (gx >= W ? gx - W : gx)) : wrapm(gx, W);
      const uint4* col = img + (int64_t)gx * C::KC + kc;
      uint4 v[TY + 2];
#pragma unroll
      for (int yy = 0; yy < TY + 2; yy++) {
        int gy = y0 - 1 + yy;
        gy = tall ? (gy < 0 ? gy + H : (gy >= H ? gy - H : gy)) : wrapm(gy, H);
        v[yy] = col[(int64_t)gy * W * C::KC];
      }
      unsigned char* dst = tile + kc * C::PLANE + xx * 16;
#pragma unroll
      for (int yy = 0; yy < TY + 2; yy++) *reinterpret_cast<uint4*>(dst + yy * kTW * 16) = v[yy];
    }
  }
  if constexpr (C::WALL) {
    // every tap's weights: global rows [tap][kc][co] of 16 bytes, this CTA's
    // co in [n0, n0 + NS)
    for (int k = tid; k < 9 * C::KC * NS; k += kThreads) {
      const int blk = k / NS, co = k - blk * NS;
      reinterpret_cast<uint4*>(wbuf0)[k] = wpk[(int64_t)blk * COUT + n0 + co];
    }
    tc::fence_async_smem();
  }
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t tile_s = tc::smem_u32(tile), wbuf_s = tc::smem_u32(wbuf0);
  constexpr uint32_t IDESC = tc::idesc_bf16(128, NS);

  if constexpr (C::WALL) {
    // weights and tile are staged: all MMAs back to back and one commit
    if (tid == 0) {
#pragma unroll 1
      for (int t = 0; t < 9; t++) {
        const int dy = t / 3 - 1, dx = t % 3 - 1;
        const uint32_t wb = wbuf_s + t * C::WTAP;
#pragma unroll 1
        for (int r = 0; r < TY; r++) {
#pragma unroll
          for (int j = 0; j < C::KC / 2; j++) {
            uint32_t a = tile_s + 2 * j * C::PLANE + ((r + 1 + dy) * kTW + (1 + dx)) * 16;
            uint32_t bb = wb + 2 * j * NS * 16;
            tc::mma_bf16(taddr + r * NS, tc::sdesc(a, C::PLANE, 128), tc::sdesc(bb, NS * 16, 128), IDESC,
                         (t > 0 || j > 0) ? 1u : 0u);
          }
        }
      }
      tc::mma_commit(&bar[0]);
    }
  } else {
  // Only thread 0 waits on the barriers; the outcome reaches the other
  // threads through *failed after a __syncthreads, so every exit is uniform.
  for (int t = 0; t < 9; t++) {
    const int buf = t & 1;
    if (t >= 2) {
      // the MMAs of tap t-2 must be done with this buffer
      if (tid == 0 && !tc::mbar_wait(&bar[buf], ((t - 2) >> 1) & 1)) *failed = 1;
      __syncthreads();
      if (*failed) break;
    }
    {
      uint4* dst = reinterpret_cast<uint4*>(wbuf0 + buf * C::W_BYTES);
      for (int k = tid; k < C::KC * NS; k += kThreads) {
        const int kc = k / NS, co = k - kc * NS;
        dst[k] = wpk[((int64_t)t * C::KC + kc) * COUT + n0 + co];
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      const uint32_t wb = wbuf_s + buf * C::W_BYTES;
#pragma unroll 1
      for (int r = 0; r < TY; r++) {
#pragma unroll
        for (int j = 0; j < C::KC / 2; j++) {
          uint32_t a = tile_s + 2 * j * C::PLANE + ((r + 1 + dy) * kTW + (1 + dx)) * 16;
          uint32_t bb = wb + 2 * j * NS * 16;
          tc::mma_bf16(taddr + r * NS, tc::sdesc(a, C::PLANE, 128), tc::sdesc(bb, NS * 16, 128), IDESC,
                       (t > 0 || j > 0) ? 1u : 0u);
        }
      }
      tc::mma_commit(&bar[buf]);
    }
  }
  }
  // the last commit went to buffer 0 at parity 0 (tap 8 is the fifth use of
  // buffer 0 in the alternating scheme; the only commit in the resident one)
  // and covers every MMA
  if (tid == 0) {
    if (*failed) {
      // let whatever was issued drain (bounded) before the TMEM is released
      tc::mbar_wait(&bar[0], 0, 1u << 20);
    } else if (!tc::mbar_wait(&bar[0], 0)) {
      *failed = 1;
    }
    if (*failed) atomicExch(err, 1);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (!*failed) {
    constexpr int GROUPS = kThreads / 128;  // warp groups share the rows
    const int q = warp & 3, grp = warp >> 2;
    const int p = 32 * q + lane, x = x0 + p;
    const bool xin = x < W && (x0 > 0 || p < W);
#pragma unroll 1
    for (int c0 = 0; c0 < (EPI == 2 ? 16 : NS); c0 += 16) {
      float bv[16];
#pragma unroll
      for (int k = 0; k < 16; k++) bv[k] = EPI == 2 ? (k == 0 ? bias[0] : 0.f) : bias[n0 + c0 + k];
      for (int r = grp; r < TY; r += GROUPS) {
        const int y = y0 + r;
        const bool valid = xin && y < H;
        float v[16];
        tc::tmem_ld16(taddr + ((uint32_t)(32 * q) << 16) + r * NS + c0, v);
        if (!valid) continue;
        if constexpr (EPI == 2) {
          if (n0 == 0) reinterpret_cast<float*>(out)[((int64_t)b * H + y) * W + x] = v[0] + bv[0];
        } else {
          const int cg = n0 + c0;  // global output channel of v[0]
#pragma unroll
          for (int k = 0; k < 16; k++) {
            v[k] += bv[k];
            if (EPI == 1) v[k] = fmaxf(v[k], 0.f);
          }
          uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) +
                                              (((int64_t)b * H + y) * W + x) * COUT + cg);
          o[0] = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                            pack_bf16(v[6], v[7]));
          o[1] = make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
                            pack_bf16(v[14], v[15]));
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, C::NCOL);
}

// ------------------------------------------------------------ GEMM check
// D[128][N] = A[128][K] B[N][K]^T from row-major bf16 A and B: exercises the
// descriptors, the instruction descriptor and the TMEM read-back on one tile.
// Operands are staged with LBO = 128 and SBO = 256 bytes, so that every
// address either field could produce stays inside the staged block.
template <int N>
__global__ void __launch_bounds__(128) k_gemm_check(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                    float* __restrict__ D, int K, int* __restrict__ err) {
  __shared__ __align__(128) uint16_t sa[128 * 64];  // up to K = 64
  __shared__ __align__(128) uint16_t sb[N * 64];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int NCOL = N < 32 ? 32 : N;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
    tc::fence_before_sync();
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  // element (row m, k) -> K step s = k / 16, chunk c = (k / 8) % 2, group g = m / 8:
  // byte offset s * (rows * 32) + g * 256 + c * 128 + (m % 8) * 16 + (k % 8) * 2
  for (int e = tid; e < 128 * K; e += 128) {
    int m = e / K, k = e % K;
    sa[(k / 16) * (128 * 16) + (m / 8) * 128 + ((k / 8) % 2) * 64 + (m % 8) * 8 + (k % 8)] = A[e];
  }
  for (int e = tid; e < N * K; e += 128) {
    int n = e / K, k = e % K;
    sb[(k / 16) * (N * 16) + (n / 8) * 128 + ((k / 8) % 2) * 64 + (n % 8) * 8 + (k % 8)] = B[e];
  }
  tc::fence_async_smem();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    for (int s = 0; s < K / 16; s++)
      tc::mma_bf16(taddr, tc::sdesc(tc::smem_u32(sa + s * 128 * 16), 128, 256),
                   tc::sdesc(tc::smem_u32(sb + s * N * 16), 128, 256), tc::idesc_bf16(128, N), s > 0 ? 1u : 0u);
    tc::mma_commit(&bar);
  }
  __syncthreads();
  bool ok = tc::mbar_wait(&bar, 0);
  tc::fence_after_sync();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    const int m = 32 * warp + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + c0, v);
      for (int k = 0; k < 16; k++) D[m * N + c0 + k] = v[k];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

// ------------------------------------------------------------------ host
template <int CIN, int COUT, int TY, int NS, int EPI>
static cudaError_t launch_t(const void* in, const void* w, const float* bias, void* out, int B, int H, int W,
                            int* err, cudaStream_t st) {
  using C = Cfg<CIN, COUT, TY, NS>;
  // the dynamic shared-memory limit is an attribute of the function on each device
  static std::atomic<uint64_t> attr_set{0};
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return e0;
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_set.load() & bit)) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3x3<CIN, COUT, TY, NS, EPI>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return e;
    attr_set.fetch_or(bit);
  }
  dim3 grid((W + kTX - 1) / kTX, (H + TY - 1) / TY, B * C::NSPLIT);
  k_conv3x3<CIN, COUT, TY, NS, EPI><<<grid, kThreads, C::SMEM, st>>>(
      static_cast<const uint4*>(in), static_cast<const uint4*>(w), bias, out, H, W, err);
  return cudaGetLastError();
}

template <int EPI>
static cudaError_t dispatch(int cin, int cout, const void* in, const void* w, const float* bias, void* out, int B,
                            int H, int W, int* err, cudaStream_t st) {
// (c_in, c_out, rows per CTA, output channels per CTA)
#define FS_CONV(ci, co, ty, ns) \
  if (cin == ci && cout == co) return launch_t<ci, co, ty, ns, EPI>(in, w, bias, out, B, H, W, err, st);
  FS_CONV(16, 16, 2, 16)
  FS_CONV(16, 32, 4, 32)
  FS_CONV(32, 16, 2, 16)
  FS_CONV(32, 64, 2, 32)
  FS_CONV(64, 32, 4, 32)
  FS_CONV(64, 128, 2, 128)
  FS_CONV(128, 64, 2, 64)
#undef FS_CONV
  return cudaErrorInvalidValue;
}

bool supported(int cin, int cout) {
  return (cin == 16 && (cout == 16 || cout == 32)) || (cin == 32 && (cout == 16 || cout == 64)) ||
         (cin == 64 && (cout == 32 || cout == 128)) || (cin == 128 && cout == 64);
}

cudaError_t conv3x3(int cin, int cout, int epi, const void* in, const void* w, const float* bias, void* out, int B,
                    int H, int W, int* err, cudaStream_t st) {
  if (epi == 0) return dispatch<0>(cin, cout, in, w, bias, out, B, H, W, err, st);
  if (epi == 1) return dispatch<1>(cin, cout, in, w, bias, out, B, H, W, err, st);
  if (cout != 16) return cudaErrorInvalidValue;
  return dispatch<2>(cin, cout, in, w, bias, out, B, H, W, err, st);
}

cudaError_t gemm_check(int n, const void* a, const void* b, float* d, int k, int* err, cudaStream_t st) {
  if (n == 16) k_gemm_check<16><<<1, 128, 0, st>>>((const uint16_t*)a, (const uint16_t*)b, d, k, err);
  else if (n == 64) k_gemm_check<64><<<1, 128, 0, st>>>((const uint16_t*)a, (const uint16_t*)b, d, k, err);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace conv
}  // namespace fs

// ------------------------------------------------------------------ C ABI
using namespace fs;

static int conv_fail(int code, const std::string& m) {
  record_error(m);
  return code;
}

extern "C" FS_API int fs_conv3x3_bf16(const void* d_in, const void* d_wpacked, const float* d_bias, void* d_out,
                                      int32_t batch, int32_t h, int32_t w, int32_t c_in, int32_t c_out,
                                      int32_t epilogue, int32_t* d_err, void* stream) {
  if (!d_in || !d_wpacked || !d_bias || !d_out || !d_err)
    return conv_fail(FS_ERR_INVALID_ARGUMENT, "fs_conv3x3_bf16: NULL pointer");
  if (batch < 1 || batch > 8192 || h < 1 || w < 1 || epilogue < 0 || epilogue > 2)
    return conv_fail(FS_ERR_INVALID_ARGUMENT, "fs_conv3x3_bf16: bad shape or epilogue");
  if (!conv::supported(c_in, c_out) || (epilogue == 2 && c_out != 16))
    return conv_fail(FS_ERR_UNSUPPORTED, "fs_conv3x3_bf16: channel pair " + std::to_string(c_in) + "->" +
                                             std::to_string(c_out) + " not instantiated");
  if (((uintptr_t)d_in | (uintptr_t)d_wpacked | (uintptr_t)d_out) & 15)
    return conv_fail(FS_ERR_INVALID_ARGUMENT, "fs_conv3x3_bf16: buffers must be 16-byte aligned");
  cudaError_t e = conv::conv3x3(c_in, c_out, epilogue, d_in, d_wpacked, d_bias, d_out, batch, h, w, d_err,
                                static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return conv_fail(FS_ERR_CUDA, std::string("fs_conv3x3_bf16: ") + cudaGetErrorString(e));
  return FS_OK;
}

extern "C" FS_API int fs_tc_gemm_check(const void* d_a, const void* d_b, float* d_d, int32_t n, int32_t k,
                                       int32_t* d_err, void* stream) {
  if (!d_a || !d_b || !d_d || !d_err) return conv_fail(FS_ERR_INVALID_ARGUMENT, "fs_tc_gemm_check: NULL pointer");
  if ((n != 16 && n != 64) || k < 16 || k > 64 || k % 16)
    return conv_fail(FS_ERR_INVALID_ARGUMENT, "fs_tc_gemm_check: n must be 16 or 64, k a multiple of 16 <= 64");
  cudaError_t e = conv::gemm_check(n, d_a, d_b, d_d, k, d_err, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return conv_fail(FS_ERR_CUDA, std::string("fs_tc_gemm_check: ") + cudaGetErrorString(e));
  return FS_OK;
}
