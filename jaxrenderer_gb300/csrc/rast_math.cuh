// rast_math.cuh -- FP32 arithmetic of the rasterisation path, in the
// reference's operation order.  Every translation unit that includes this is
// compiled with -fmad=false (no multiply-add contraction) and IEEE division
// and square root, so each operation below rounds once, as in
// jaxrenderer's JAX program read operation by operation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rast_gb300.h"

namespace rast {

constexpr float kInf = __builtin_huge_valf();

// lax.dot_general over a length-3 contraction, index order
// (geometry.py:104-108, pipeline.py:190).
__device__ __forceinline__ float dot3(const float* a, const float* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// normalise (geometry.py:39-47): v / sqrt(sum(v*v)).
__device__ __forceinline__ void normalise3(const float* v, float* out) {
  const float n = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  out[0] = v[0] / n;
  out[1] = v[1] / n;
  out[2] = v[2] / n;
}

// Camera.apply (geometry.py:284-315): out[i] = sum_k p[k] * M[i][k].
__device__ __forceinline__ void apply4(const float* m, const float* p, float* out) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
    out[i] = ((p[0] * m[4 * i + 0] + p[1] * m[4 * i + 1]) + p[2] * m[4 * i + 2]) +
             p[3] * m[4 * i + 3];
}

// Camera.to_clip(to_homogeneous(position)) (geometry.py:144-163, 420-438).
__device__ __forceinline__ void to_clip(const float* m, float px, float py, float pz,
                                        float* out) {
  const float p[4] = {px, py, pz, 1.0f};
  apply4(m, p, out);
}

// Camera.apply_vec (geometry.py:352-389).
__device__ __forceinline__ void apply_vec(const float* m, const float* v, float* out) {
  float n[3];
  normalise3(v, n);
  const float h[4] = {n[0], n[1], n[2], 0.0f};
  float t[4];
  apply4(m, h, t);
  normalise3(t, out);
}

// astype(int): saturating, NaN -> 0 (cvt.rzi.s32.f32 semantics).
__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }

// Integer remainder with the sign of the divisor (jnp `%` on ints).
__device__ __forceinline__ int pymod(int a, int b) {
  if (b == 0) return 0;
  int r = a % b;
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}

// Default-mode jnp gather index: negatives wrap once, then clamp.
__device__ __forceinline__ int gather_clamp(int idx, int size) {
  if (idx < 0) idx += size;
  idx = idx < 0 ? 0 : idx;
  return idx > size - 1 ? size - 1 : idx;
}

// Depth -> monotone uint32: NaN first (it wins argmin), -0 == +0.
__device__ __forceinline__ uint32_t depth_order(float z) {
  if (z != z) return 0u;
  if (z == 0.0f) z = 0.0f;
  const uint32_t b = __float_as_uint(z);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Packed chooser key: (ordered depth << 32) | primitive id.  The minimum
// key is the reference's argmin (lowest depth, first index on ties).
__device__ __forceinline__ unsigned long long pack_key(float z, int prim) {
  return (static_cast<unsigned long long>(depth_order(z)) << 32) |
         static_cast<unsigned int>(prim);
}

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr uint32_t kInfOrder = 0xff800000u;  // depth_order(+inf)

// jnp.linalg.det closed form for 3x3 (pipeline.py:91-94), left to right.
__device__ __forceinline__ float det3(const float* a) {
  const float t1 = (a[0] * a[4]) * a[8];
  const float t2 = (a[1] * a[5]) * a[6];
  const float t3 = (a[2] * a[3]) * a[7];
  const float t4 = (a[2] * a[4]) * a[6];
  const float t5 = (a[0] * a[5]) * a[7];
  const float t6 = (a[1] * a[3]) * a[8];
  return ((((t1 + t2) + t3) - t4) - t5) - t6;
}

// jnp.linalg.inv (pipeline.py:105): LU with partial pivoting in reference
// LAPACK getf2 order (pivot = first max |a|, column times the reciprocal of a
// normal pivot, rank-1 update a - l*u), then the permuted identity through a
// unit-lower and an upper triangular solve in reference BLAS trsm order.
__device__ __forceinline__ void inv3(const float* m, float* out) {
  float a[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) a[k] = m[k];
  int perm[3] = {0, 1, 2};
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    int p = j;
    float amax = fabsf(a[3 * j + j]);
#pragma unroll
    for (int r = j + 1; r < 3; ++r) {
      const float v = fabsf(a[3 * r + j]);
      if (v > amax) {
        amax = v;
        p = r;
      }
    }
    if (a[3 * p + j] != 0.0f) {
      if (p != j) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          // select-based swap keeps the arrays in registers
          const float tj = a[3 * j + c];
          const float tp = (p == 1) ? a[3 + c] : a[6 + c];
          a[3 * j + c] = tp;
          if (p == 1) a[3 + c] = tj; else a[6 + c] = tj;
        }
        const int t = perm[j];
        perm[j] = (p == 1) ? perm[1] : perm[2];
        if (p == 1) perm[1] = t; else perm[2] = t;
      }
      const float piv = a[3 * j + j];
      if (fabsf(piv) >= 1.17549435e-38f) {
        const float rcp = 1.0f / piv;
#pragma unroll
        for (int r = j + 1; r < 3; ++r) a[3 * r + j] = a[3 * r + j] * rcp;
      } else {
#pragma unroll
        for (int r = j + 1; r < 3; ++r) a[3 * r + j] = a[3 * r + j] / piv;
      }
    }
#pragma unroll
    for (int r = j + 1; r < 3; ++r)
#pragma unroll
      for (int c = j + 1; c < 3; ++c) a[3 * r + c] = a[3 * r + c] - a[3 * r + j] * a[3 * j + c];
  }
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    float b[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) b[r] = (perm[r] == col) ? 1.0f : 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (b[k] != 0.0f)
#pragma unroll
        for (int i = k + 1; i < 3; ++i) b[i] = b[i] - b[k] * a[3 * i + k];
#pragma unroll
    for (int k = 2; k >= 0; --k)
      if (b[k] != 0.0f) {
        b[k] = b[k] / a[3 * k + k];
#pragma unroll
        for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * a[3 * i + k];
      }
#pragma unroll
    for (int r = 0; r < 3; ++r) out[3 * r + col] = b[r];
  }
}

// min that propagates NaN (PTX min.NaN): min_nan(a, min_nan(b, c)) >= 0 is
// exactly (a >= 0 && b >= 0 && c >= 0), NaN failing as in the reference.
__device__ __forceinline__ float min_nan(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ bool all_nonneg(float a, float b, float c) {
  return min_nan(a, min_nan(b, c)) >= 0.0f;
}

// max(x, 0) of jnp.maximum / lax.max: NaN propagates, -0 -> +0.
__device__ __forceinline__ float max0(float x) {
  return (x != x) ? x : (x > 0.0f ? x : 0.0f);
}

}  // namespace rast
