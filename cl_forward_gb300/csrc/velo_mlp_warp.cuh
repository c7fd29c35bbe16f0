// velo_mlp_warp.cuh -- inference of the 10 -> 32 -> 32 -> 2 doublet scorer
// by one warp on the tensor cores: 32 doublets (one per lane) per call.
//
// Each layer is a [16 doublets x K] x [K x N] product per m-tile, issued as
// mma.sync m16n8k16 with FP16 operands and FP32 accumulation (two m-tiles:
// 4 + 8 + 2 MMAs each).  The accumulator fragment of one layer is, after ReLU
// and packing to FP16, the A fragment of the next (the C layout of two
// adjacent n8 tiles is the A layout of one k16 step), so activations never
// leave registers.  A CTA-wide tcgen05 MMA needs M >= 64 rows gathered from
// all warps through shared memory and TMEM between the seeding chunks; the
// warp-level product keeps the 32-doublet batch where the seeding loop
// already holds it.
//
// The weights live in shared memory in fragment order (MlpFrag), converted
// once per CTA from the flat FP32 parameter array: every lane then reads its
// B fragment with one conflict-free 8-byte load per n-tile.
//
// Features, weights and hidden activations are rounded to FP16; the keep
// threshold and window margin are calibrated on this same arithmetic
// (velo_mlp_forward runs this function too).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "velo_internal.h"

namespace velo {

__device__ __forceinline__ uint32_t pack_half2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mma_16816(float* d, const uint32_t* a, MlpPair b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// Weight of the flat FP32 array seen as B = W^T of a layer: B[k][n] = W[n][k],
// zero outside the layer's in x out shape.
__device__ __forceinline__ float mlp_b(const float* w, int layer, int k, int n) {
  if (layer == 0) return (k < kMlpIn && n < kMlpHidden) ? w[kMlpW1 + n * kMlpIn + k] : 0.f;
  if (layer == 1) return w[kMlpW2 + n * kMlpHidden + k];
  return n < kMlpOut ? w[kMlpW3 + n * kMlpHidden + k] : 0.f;
}

// Fills the fragment-ordered copy; all threads of the CTA take part, the
// caller synchronises afterwards.  B fragment of m16n8k16 for lane 4g + t:
// b.x = {B[2t][g], B[2t+1][g]}, b.y = {B[2t+8][g], B[2t+9][g]}.
__device__ inline void stage_mlp_fragments(const float* __restrict__ w, MlpFrag* f) {
  constexpr int n1 = 4 * 32, n2 = 2 * 4 * 32, n3 = 2 * 32;
  for (int i = threadIdx.x; i < n1 + n2 + n3; i += blockDim.x) {
    int layer, kk, j, lane;
    MlpPair* dst;
    if (i < n1) {
      layer = 0; kk = 0; j = i >> 5; lane = i & 31;
      dst = &f->w1[j][lane];
    } else if (i < n1 + n2) {
      const int r = i - n1;
      layer = 1; kk = r >> 7; j = (r >> 5) & 3; lane = r & 31;
      dst = &f->w2[kk][j][lane];
    } else {
      const int r = i - n1 - n2;
      layer = 2; kk = r >> 5; j = 0; lane = r & 31;
      dst = &f->w3[kk][lane];
    }
    const int g = lane >> 2, t = lane & 3, n = 8 * j + g, k0 = 16 * kk + 2 * t;
    dst->x = pack_half2(mlp_b(w, layer, k0, n), mlp_b(w, layer, k0 + 1, n));
    dst->y = pack_half2(mlp_b(w, layer, k0 + 8, n), mlp_b(w, layer, k0 + 9, n));
  }
  for (int i = threadIdx.x; i < 2 * kMlpHidden + 8; i += blockDim.x) {
    if (i < kMlpHidden) f->b1[i] = w[kMlpB1 + i];
    else if (i < 2 * kMlpHidden) f->b2[i - kMlpHidden] = w[kMlpB2 + i - kMlpHidden];
    else f->b3[i - 2 * kMlpHidden] = (i - 2 * kMlpHidden) < kMlpOut ? w[kMlpB3 + i - 2 * kMlpHidden] : 0.f;
  }
}

// Register p (0..3) of four, selected by a lane-varying index.
__device__ __forceinline__ uint32_t pick4(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3, int p) {
  const uint32_t lo = (p & 1) ? v1 : v0, hi = (p & 1) ? v3 : v2;
  return (p & 2) ? hi : lo;
}

// ReLU of the accumulator n-tiles 2kk and 2kk+1, packed as the A fragment of
// k-step kk of the next layer.
__device__ __forceinline__ void relu_pack(const float (*c)[4], int kk, uint32_t* a) {
  a[0] = pack_half2(fmaxf(c[2 * kk][0], 0.f), fmaxf(c[2 * kk][1], 0.f));
  a[1] = pack_half2(fmaxf(c[2 * kk][2], 0.f), fmaxf(c[2 * kk][3], 0.f));
  a[2] = pack_half2(fmaxf(c[2 * kk + 1][0], 0.f), fmaxf(c[2 * kk + 1][1], 0.f));
  a[3] = pack_half2(fmaxf(c[2 * kk + 1][2], 0.f), fmaxf(c[2 * kk + 1][3], 0.f));
}

// All 32 lanes must call it (warp-convergent).  Lane L passes the features of
// doublet L (zeros for an idle lane) and gets back that doublet's logit and
// predicted window half-width.
__device__ __forceinline__ void mlp_eval_warp(const MlpFrag& w, const float* feat, float* logit, float* width) {
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  static_assert(kMlpIn == 10 && kMlpHidden == 32 && kMlpOut == 2, "fragment layout is written for 10-32-32-2");
  // own features as FP16 pairs: pair q = features 2q, 2q+1 (pairs 5..7 are zero)
  uint32_t P[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) P[q] = pack_half2(feat[2 * q], feat[2 * q + 1]);
  float res[2][4];   // per m-tile: the layer-3 accumulators (valid cols 0, 1 at t == 0)
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    // A fragment of layer 1: rows g and g+8 of this m-tile, pairs t and t+4
    uint32_t a[4];
    {
      const int r0 = 16 * m + g, r1 = r0 + 8;
      uint32_t v[4], u[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        v[q] = __shfl_sync(kAll, P[q], r0);
        u[q] = __shfl_sync(kAll, P[q], r1);
      }
      const uint32_t e0 = __shfl_sync(kAll, P[4], r0), e1 = __shfl_sync(kAll, P[4], r1);
      a[0] = pick4(v[0], v[1], v[2], v[3], t);
      a[1] = pick4(u[0], u[1], u[2], u[3], t);
      a[2] = t == 0 ? e0 : 0u;
      a[3] = t == 0 ? e1 : 0u;
    }
    float c[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float2 bias = *reinterpret_cast<const float2*>(&w.b1[8 * j + 2 * t]);
      c[j][0] = bias.x; c[j][1] = bias.y; c[j][2] = bias.x; c[j][3] = bias.y;
      mma_16816(c[j], a, w.w1[j][lane]);
    }
    uint32_t a2[2][4];
    relu_pack(c, 0, a2[0]);
    relu_pack(c, 1, a2[1]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float2 bias = *reinterpret_cast<const float2*>(&w.b2[8 * j + 2 * t]);
      c[j][0] = bias.x; c[j][1] = bias.y; c[j][2] = bias.x; c[j][3] = bias.y;
      mma_16816(c[j], a2[0], w.w2[0][j][lane]);
      mma_16816(c[j], a2[1], w.w2[1][j][lane]);
    }
    relu_pack(c, 0, a2[0]);
    relu_pack(c, 1, a2[1]);
    const float2 bias = *reinterpret_cast<const float2*>(&w.b3[2 * t]);
    res[m][0] = bias.x; res[m][1] = bias.y; res[m][2] = bias.x; res[m][3] = bias.y;
    mma_16816(res[m], a2[0], w.w3[0][lane]);
    mma_16816(res[m], a2[1], w.w3[1][lane]);
  }
  // doublet L sits in m-tile L >> 4, row L & 15: lane 4 (L & 7), register
  // pair 0/1 (rows < 8) or 2/3 (rows >= 8)
  const int src = 4 * (lane & 7), hi_row = (lane >> 3) & 1, mt = lane >> 4;
  const float l00 = __shfl_sync(kAll, res[0][0], src), l01 = __shfl_sync(kAll, res[0][2], src);
  const float l10 = __shfl_sync(kAll, res[1][0], src), l11 = __shfl_sync(kAll, res[1][2], src);
  const float w00 = __shfl_sync(kAll, res[0][1], src), w01 = __shfl_sync(kAll, res[0][3], src);
  const float w10 = __shfl_sync(kAll, res[1][1], src), w11 = __shfl_sync(kAll, res[1][3], src);
  *logit = mt ? (hi_row ? l11 : l10) : (hi_row ? l01 : l00);
  *width = mt ? (hi_row ? w11 : w10) : (hi_row ? w01 : w00);
}

}  // namespace velo
