// fs_stencil.cuh -- the per-cell arithmetic of the Poisson kernels, with every
// rounding step spelled out.
//
// Both the one-pass-per-operation kernels and the fused multigrid kernels
// call these, so the two paths round identically (nvcc would otherwise be free
// to contract a*b + c*d either way round in different kernels).  The operand
// order is the reference's: src/gpu/shaders.js RED_BLACK_GS / JACOBI
// (l + r + b + t - h^2 d) / 4, multigrid.js RESIDUAL rhs - (l + r + b + t - 4c)/h^2
// and PROLONG mix(mix(a, b, fx), mix(c, d, fx), fy).
#pragma once

#include <cuda_runtime.h>

namespace fs {

__device__ __forceinline__ float sum4(float l, float r, float b, float t) {
  return __fadd_rn(__fadd_rn(__fadd_rn(l, r), b), t);
}

// Gauss-Seidel / Jacobi point update with relaxation factor w (param_a of
// JACOBI / RED_BLACK_GS): cur + w ((sum - h2 d)/4 - cur).  w = 1 multiplies
// exactly, so that case rounds like the plain update the reference runs.
__device__ __forceinline__ float gs_update(float cur, float l, float r, float b, float t, float d, float h2,
                                           float w) {
  float gs = __fmul_rn(__fmaf_rn(-h2, d, sum4(l, r, b, t)), 0.25f);
  return __fadd_rn(cur, __fmul_rn(w, __fsub_rn(gs, cur)));
}

// rhs - (l + r + b + t - 4c) / h2, the division taken as a product with
// ih2 = RN(1/h2) (inv_h2): the reference's WGSL divide is itself not
// correctly rounded (2.5 ulp allowed), and a correctly rounded divide per cell
// costs the tile kernels several instructions where one multiply does
__device__ __forceinline__ float residual_at(float c, float l, float r, float b, float t, float rhs, float ih2) {
  float lap = __fmul_rn(__fmaf_rn(-4.f, c, sum4(l, r, b, t)), ih2);
  return __fsub_rn(rhs, lap);
}

// the reciprocal every residual_at caller passes: RN(1 / h2)
__device__ __forceinline__ float inv_h2(float h2) { return __frcp_rn(h2); }

// a (1 - t) + b t
__device__ __forceinline__ float mix_rn(float a, float b, float t) {
  return __fmaf_rn(b, t, __fmul_rn(a, __fsub_rn(1.f, t)));
}

// bilinear prolongation sample; fx, fy are 1/4 or 3/4
__device__ __forceinline__ float prolong_val(float a, float b, float c, float d, float fx, float fy) {
  return mix_rn(mix_rn(a, b, fx), mix_rn(c, d, fx), fy);
}

// restriction: ((r00 + r10) + r01) + r11, times 1/4
__device__ __forceinline__ float restrict4(float r00, float r10, float r01, float r11) {
  return __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(0.f, r00), r10), r01), r11), 0.25f);
}

}  // namespace fs
