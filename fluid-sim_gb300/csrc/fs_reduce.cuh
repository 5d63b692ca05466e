// fs_reduce.cuh -- deterministic block reductions shared by the kernels that
// report a maximum or a sum alongside their main output.
#pragma once

#include <cuda_runtime.h>

#include "fs_internal.cuh"

namespace fs {

// ------------------------------------------------------------- reductions
// Per-block partials, then the last block to finish folds them in a fixed
// order, so every reduction is deterministic run to run.  Max reductions stay
// in f32 end to end (exact for a max, and off the FP64 pipe, which runs at
// 1/54 of the FP32 rate on GB300); the f64 sums serve diagnostics only.
struct RedCtx {
  double* partials;  // 2 per block (sums)
  float* fpartials;  // 1 per block (max)
  unsigned* counter;
  double* out;       // out[0], out[1]
};

__device__ __forceinline__ bool commit_partial_is_last(RedCtx ctx) {
  __shared__ bool last;
  int tid = threadIdx.y * blockDim.x + threadIdx.x;
  int nblk = gridDim.x * gridDim.y;
  if (tid == 0) {
    __threadfence();
    unsigned done = atomicAdd(ctx.counter, 1u);
    last = done == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// every thread passes its value; the block max lands in out[0].  Returns
// true on the one thread that wrote it (thread 0 of the last block to
// finish), with the max in *res.
__device__ __forceinline__ bool block_max_finish_at(float m, RedCtx ctx, float* res) {
  __shared__ float sm[32];
  int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int nthr = blockDim.x * blockDim.y, nwarp = (nthr + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) sm[warp] = m;
  __syncthreads();
  if (tid == 0) {
    float t = sm[0];
    for (int w = 1; w < nwarp; w++) t = fmaxf(t, sm[w]);
    ctx.fpartials[blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
  if (!commit_partial_is_last(ctx)) return false;
  int nblk = gridDim.x * gridDim.y;
  float t = 0.f;
  // L2 reads (the partials of the other blocks), eight in flight per thread
  int k = tid;
  for (; k + 7 * nthr < nblk; k += 8 * nthr) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) v[u] = __ldcg(ctx.fpartials + k + u * nthr);
#pragma unroll
    for (int u = 0; u < 8; u++) t = fmaxf(t, v[u]);
  }
  for (; k < nblk; k += nthr) t = fmaxf(t, __ldcg(ctx.fpartials + k));
  for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
  __syncthreads();
  if (lane == 0) sm[warp] = t;
  __syncthreads();
  if (tid == 0) {
    float f = sm[0];
    for (int w = 1; w < nwarp; w++) f = fmaxf(f, sm[w]);
    ctx.out[0] = (double)f;
    *ctx.counter = 0;  // ready for the next reduction
    *res = f;
    return true;
  }
  return false;
}

__device__ __forceinline__ void block_max_finish(float m, RedCtx ctx) {
  float r;
  (void)block_max_finish_at(m, ctx, &r);
}

// every thread passes (a, b); the block sums land in out[0], out[1] (f64)
__device__ __forceinline__ void block_sum2_finish(double a, double b, RedCtx ctx) {
  __shared__ double sa[32], sb[32];
  int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int nthr = blockDim.x * blockDim.y, nwarp = (nthr + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) { sa[warp] = a; sb[warp] = b; }
  __syncthreads();
  int bid = blockIdx.y * gridDim.x + blockIdx.x;
  if (tid == 0) {
    double ta = sa[0], tb = sb[0];
    for (int w = 1; w < nwarp; w++) { ta += sa[w]; tb += sb[w]; }
    ctx.partials[2 * bid] = ta;
    ctx.partials[2 * bid + 1] = tb;
  }
  if (!commit_partial_is_last(ctx)) return;
  int nblk = gridDim.x * gridDim.y;
  double ta = 0.0, tb = 0.0;
  for (int k = tid; k < nblk; k += nthr) {
    ta += ((volatile double*)ctx.partials)[2 * k];
    tb += ((volatile double*)ctx.partials)[2 * k + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_xor_sync(0xffffffffu, ta, o);
    tb += __shfl_xor_sync(0xffffffffu, tb, o);
  }
  __syncthreads();
  if (lane == 0) { sa[warp] = ta; sb[warp] = tb; }
  __syncthreads();
  if (tid == 0) {
    double fa = sa[0], fb = sb[0];
    for (int w = 1; w < nwarp; w++) { fa += sa[w]; fb += sb[w]; }
    ctx.out[0] = fa;
    ctx.out[1] = fb;
    *ctx.counter = 0;
  }
}


inline RedCtx red_ctx(Solver* s, double* out) {
  // layout of red_partials: [2*cap doubles][cap floats][counter]
  float* fp = (float*)(s->red_partials + 2 * s->red_cap);
  return RedCtx{s->red_partials, fp, (unsigned*)(fp + s->red_cap), out};
}

}  // namespace fs
