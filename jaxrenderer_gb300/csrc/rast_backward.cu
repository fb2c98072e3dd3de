// rast_backward.cu -- hand-written reverse mode of the rasterisation path.
//
// Visibility is piecewise constant (as under jax.grad of the reference): the
// forward's winning-primitive buffer is saved, and gradients flow through the
// primitive each kept pixel shows.  The work is split by what it depends on,
// so each part runs once per pixel, per face or per vertex:
//
//   mark_kernel          pixels -> faces they show (visibility flags)
//   face_prep_kernel     per visible face: clip positions, 3x3 inverse m of
//                        [x, y, w] (same operations as the forward set-up);
//                        zero its accumulators; flag its corner vertices
//   vertex_prep_kernel   per flagged vertex: the vertex shader's varyings
//   pixel_kernel         per kept pixel: barycentrics and fragment, then
//                        reverse mode through the fragment shader and the
//                        perspective-correct interpolation; accumulates
//                        dL/dm and dL/dz_clip per face, dL/d(varying) per
//                        vertex, texel gradients; per-scene light terms
//   post_kernel          one launch of two block roles:
//                        face_post, per visible face: dL/dM = -m^T (dL/dm)
//                        m^T, clip rows -> dL/d world_to_clip and dL/d
//                        positions; vertex_post, per flagged vertex: reverse
//                        mode of the vertex shader (normal transform,
//                        Gouraud lighting)
//
// Texel lookups are nearest, so uv gets no gradient (floor); the sampled
// texel and specular exponent do (scatter-add).  The shadow-map comparison is
// a step: no gradient reaches the depth pass.  lax.max's tie derivative (1/2)
// is reproduced.  Per-scene gradients are reduced per block (blocks never
// span scenes) and added once per block.
#include <cuda_runtime.h>

#include <algorithm>

#include "rast_internal.cuh"

namespace rast {
namespace bwd {

constexpr int kThreads = 256;
// Rows (faces or vertices) per block of the per-face and per-vertex kernels:
// few rows of a block are visible, so each block scans kRowsPerThread rows
// per thread and works through the queued ones, paying its job load, queue
// and parameter reduction once per kRows rows.
constexpr int kRowsPerThread = 32;
constexpr int kRows = kThreads * kRowsPerThread;

// Gradient-only arithmetic.  Values that feed gradients alone (checked to a
// relative tolerance) and no branch of the forward's (the texel index, the
// shadow lookup and the barycentrics keep the forward's IEEE operations) use
// the hardware's approximate reciprocal and reciprocal square root, a few
// ulp, instead of IEEE division and square root.
__device__ __forceinline__ float grad_rcp(float x) { return __fdividef(1.0f, x); }

// out = v / |v| with the approximate reciprocal square root; returns |v|.
__device__ __forceinline__ float unit3_grad(const float* v, float* out) {
  const float ss = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
  const float r = rsqrtf(ss);
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = v[k] * r;
  return ss * r;
}

// y = v / |v|;  dv = (dy - y (y . dy)) / |v|  (one reciprocal, three products)
__device__ __forceinline__ void normalise3_bwd(const float* y, float norm, const float* dy, float* dv) {
  const float s = (y[0] * dy[0] + y[1] * dy[1]) + y[2] * dy[2];
  const float r = grad_rcp(norm);
#pragma unroll
  for (int k = 0; k < 3; ++k) dv[k] = (dy[k] - y[k] * s) * r;
}

__device__ __forceinline__ float norm3(const float* v) {
  return sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
}

// d max(x, 0) / dx as lax.max's derivative: 1 above, 0 below, 1/2 at the tie.
__device__ __forceinline__ float dmax0(float x) { return x > 0.0f ? 1.0f : (x == 0.0f ? 0.5f : 0.0f); }

__device__ __forceinline__ void texel_index(const RastJob& J, int u, int w, int64_t* base, int* ch) {
  u = gather_clamp(u, J.tex_w);
  w = gather_clamp(w, J.tex_h);
  *base = J.texture_begin + (static_cast<int64_t>(u) * J.tex_h + w) * J.tex_c;
  *ch = J.tex_c;
}

__device__ __forceinline__ void add_texel_grad(float* g, int64_t base, int ch, const float* d) {
  if (!g) return;
  if (ch == 1) {
    atomicAdd(g + base, (d[0] + d[1]) + d[2]);
  } else {
    atomicAdd(g + base + 0, d[0]);
    atomicAdd(g + base + 1, d[1]);
    atomicAdd(g + base + 2, d[2]);
  }
}

constexpr unsigned kFull = 0xffffffffu;

// Fire-and-forget global float add.  The accumulation targets are read back
// from shared memory as generic pointers, for which atomicAdd would be a
// generic atomic that returns the old value; this is the global reduction.
__device__ __forceinline__ void red_add(float* p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "f"(v) : "memory");
}

// Template values of the shader-specialised kernels: a shader id, kAnyShader
// (any mix, dispatch on each job's shader) or kReflectionShaders (jobs of
// phong_reflection and phong_reflection_shadow only).  may<SH>(x): code for
// shader x is needed.
constexpr int kAnyShader = -1;
constexpr int kReflectionShaders = -2;
template <int SH>
__host__ __device__ constexpr bool may(int x) {
  return SH == x || SH == kAnyShader ||
         (SH == kReflectionShaders && (x == RAST_SHADER_PHONG_REFLECTION || x == RAST_SHADER_PHONG_REFLECTION_SHADOW));
}

// Lanes whose key differs from the next lane's (or lane 31): the last lane
// of each run of equal keys.  Inactive lanes get keys of their own, so each
// stands alone.  Every lane of the warp must call it.
__device__ __forceinline__ unsigned run_tails(long long key, bool active) {
  const int lane = threadIdx.x & 31;
  const long long k = active ? key : -2 - lane;
  const long long next = __shfl_down_sync(kFull, k, 1);
  return __ballot_sync(kFull, lane == 31 || next != k);
}

// Per-pixel contributions of the pixel kernel, summed per run of equal keys
// along the warp's 32 pixels (pixels run along a column, so neighbours
// usually share the face and the texel) with one atomic per run and value.
// Each lane writes its pixel's values as one row of the warp's table
// (columns below) and the target addresses of its pixel; then lane c walks
// column c down the 32 rows, adding, and at the end of each run adds the
// run's sum to its target: 32 shared loads per value instead of a shuffle
// tree per value.  Columns: dL/dm (9) and dL/dz_clip (3) per face; dL/d
// carried varying (3 per corner vertex); dL/dtexel (3); dL/d specular
// exponent (1); with phong_darboux, dL/d Darboux triangle (9, vertex 0's
// row) and dL/d normal-map texel (3).
enum AccTarget { kTgtFace, kTgtVert0, kTgtVert1, kTgtVert2, kTgtTexel, kTgtExponent, kTgtNormalMap, kTgtCount };
template <bool kDarboux>
struct AccLayout {
  static constexpr int kCols = kDarboux ? 37 : 25;
  static constexpr int kRow = kDarboux ? 44 : 28;  // an odd number of float4: conflict-free row stores
  static constexpr int kTargets = kDarboux ? kTgtCount : kTgtNormalMap;
};

// Target (address slot, offset) and key kind of column c.  Key kinds: 0
// face, 1 texel, 2 specular exponent, 3 normal-map texel.
template <bool kDarboux>
__device__ __forceinline__ void acc_column(int c, int tex_channels, int* target, int* offset, int* kind) {
  if (c < 12) {
    *target = kTgtFace, *offset = c, *kind = 0;
  } else if (c < 21) {
    *target = kTgtVert0 + (c - 12) / 3, *offset = (c - 12) % 3, *kind = 0;
  } else if (c < 24) {
    *target = kTgtTexel, *offset = tex_channels == 1 ? 0 : c - 21, *kind = 1;
  } else if (c == 24) {
    *target = kTgtExponent, *offset = 0, *kind = 2;
  } else if (kDarboux && c < 34) {
    *target = kTgtVert0, *offset = 3 + (c - 25), *kind = 0;
  } else {
    *target = kTgtNormalMap, *offset = c - 34, *kind = 3;
  }
}

__host__ __device__ constexpr unsigned long long range_bits(int lo, int n) {
  return ((n >= 64 ? ~0ull : ((1ull << n) - 1ull)) << lo);
}

// Per-scene parameters each kernel can touch (bit k = RAST_GRAD index k).
__host__ __device__ constexpr unsigned long long pixel_bits(int sh) {
  return sh == RAST_SHADER_DEPTH ? 0ull
       : range_bits(RAST_GRAD_BACKGROUND, 3) |  // the over mixer's background
         ((sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) ? 0ull
          : sh == RAST_SHADER_PHONG ? range_bits(RAST_GRAD_LIGHT_DIRECTION, 6)
          : (sh == RAST_SHADER_PHONG_REFLECTION || sh == RAST_SHADER_PHONG_REFLECTION_SHADOW)
              ? range_bits(RAST_GRAD_LIGHT_COLOUR, 18)
          : range_bits(RAST_GRAD_LIGHT_DIRECTION, 21));
}
__host__ __device__ constexpr unsigned long long vertex_bits(int sh) {
  return (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) ? range_bits(RAST_GRAD_LIGHT_DIRECTION, 6)
       : sh == RAST_SHADER_DEPTH ? 0ull
       : sh == kReflectionShaders ? range_bits(RAST_GRAD_WORLD_TO_EYE_NORM, 16)
       : sh < 0 ? range_bits(RAST_GRAD_WORLD_TO_EYE_NORM, 16) | range_bits(RAST_GRAD_LIGHT_DIRECTION, 6) |
                  range_bits(RAST_GRAD_WORLD_TO_CLIP, 16)
       : sh == RAST_SHADER_PHONG_DARBOUX ? range_bits(RAST_GRAD_WORLD_TO_EYE_NORM, 16) | range_bits(RAST_GRAD_WORLD_TO_CLIP, 16)
       : range_bits(RAST_GRAD_WORLD_TO_EYE_NORM, 16);
}
constexpr unsigned long long kClipBits = range_bits(RAST_GRAD_WORLD_TO_CLIP, 16);

struct ParamGrad {
  float v[RAST_NPARAM];
};

struct NoPost {
  static constexpr bool kActive = false;
  __device__ void operator()(float*) const {}
};

// Block reduction of the parameters in BITS, added to this block's scene.
// Every thread of the block must call it.
// `active`: this thread contributed; warps without a contributing thread
// skip their shuffles and add zeros.  `post` (when Post::kActive) maps the
// block's totals, on one thread, before they are added: the linear maps
// every pixel's contribution would go through are applied once per block.
// kTransposed (kernels that reduce once per thread and pixel): the span
// [kLo, kLo + kSpan) of BITS, up to 32 parameters, is summed by a transpose
// through shared memory (each lane stores its values, lane n adds parameter
// kLo + n's 32 values) instead of one shuffle tree per parameter.  Rows of
// 36 floats: the 128-bit row reads of 8 lanes hit distinct banks.  The
// transpose uses the caller's shared scratch `cols` of
// transpose_floats<BITS>() floats (16-byte aligned).
template <unsigned long long BITS>
__host__ __device__ constexpr int param_span() {
  return BITS ? 64 - __builtin_clzll(BITS) - (BITS ? __builtin_ctzll(BITS) : 0) : 0;
}
template <unsigned long long BITS>
__host__ __device__ constexpr int transpose_floats() {
  return (kThreads / 32) * param_span<BITS>() * 36;
}
template <unsigned long long BITS, bool kTransposed = false, class Post = NoPost>
__device__ __forceinline__ void reduce_params(const ParamGrad& pg, float* job_params, bool active, int job,
                                              const Post& post = Post(), float* cols = nullptr) {
  constexpr int kLo = BITS ? __builtin_ctzll(BITS) : 0;
  constexpr int kSpan = param_span<BITS>();
  constexpr bool kTranspose = kTransposed && kSpan > 0 && kSpan <= 32;
  __shared__ float s_red[kThreads / 32][RAST_NPARAM];
  __shared__ float s_tot[Post::kActive ? RAST_NPARAM : 1];
  if (BITS == 0ull || !job_params) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool warp_active = __any_sync(0xffffffffu, active);
  if (kTranspose) {
    if (warp_active) {
      float* col = cols + warp * kSpan * 36;  // this warp's rows: parameter n at col[n * 36 ...]
#pragma unroll
      for (int n = 0; n < kSpan; ++n) col[n * 36 + lane] = ((BITS >> (kLo + n)) & 1ull) ? pg.v[kLo + n] : 0.0f;
      __syncwarp();
      if (lane < kSpan) {
        float a = 0.0f, b = 0.0f, c = 0.0f, d = 0.0f;
        const float4* row = reinterpret_cast<const float4*>(col + lane * 36);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 t = row[q];
          a += t.x;
          b += t.y;
          c += t.z;
          d += t.w;
        }
        s_red[warp][kLo + lane] = (a + b) + (c + d);
      }
    } else if (lane < kSpan) {
      s_red[warp][kLo + lane] = 0.0f;
    }
  } else {
#pragma unroll
    for (int k = 0; k < RAST_NPARAM; ++k) {
      if (!((BITS >> k) & 1ull)) continue;
      float v = 0.0f;
      if (warp_active) {
        v = pg.v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      }
      if (lane == 0) s_red[warp][k] = v;
    }
  }
  __syncthreads();
  const bool mine = threadIdx.x < RAST_NPARAM && ((BITS >> threadIdx.x) & 1ull);
  float v = 0.0f;
  if (mine) {
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) v += s_red[w][threadIdx.x];
  }
  if (Post::kActive) {
    if (threadIdx.x < RAST_NPARAM) s_tot[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x == 0) post(s_tot);
    __syncthreads();
    if (mine) v = s_tot[threadIdx.x];
  }
  if (mine && v != 0.0f) atomicAdd(job_params + static_cast<int64_t>(job) * RAST_NPARAM + threadIdx.x, v);
}

// The scene's light directions normalised (the same operations as the
// fragment shaders'), with their norms: once per job by light_kernel, read by
// every pixel block of the job.
struct LightUnit {
  float dir[3], dir_n;  // light_direction (phong, phong_darboux)
  float eye[3], eye_n;  // light_dir_eye (phong_reflection[_shadow])
};

// Pixels add dL/d(normalised light) to the scene's light-direction slots;
// the block's total goes through normalise's reverse mode once (it is
// linear in the incoming gradient).
struct LightPost {
  static constexpr bool kActive = true;
  const LightUnit* lu;
  int shader;
  __device__ void operator()(float* tot) const {
    const bool eye = shader == RAST_SHADER_PHONG_REFLECTION || shader == RAST_SHADER_PHONG_REFLECTION_SHADOW;
    if (!eye && shader != RAST_SHADER_PHONG && shader != RAST_SHADER_PHONG_DARBOUX) return;
    const int base = eye ? RAST_GRAD_LIGHT_DIR_EYE : RAST_GRAD_LIGHT_DIRECTION;
    const float g[3] = {tot[base], tot[base + 1], tot[base + 2]};
    float d[3];
    normalise3_bwd(eye ? lu->eye : lu->dir, eye ? lu->eye_n : lu->dir_n, g, d);
#pragma unroll
    for (int q = 0; q < 3; ++q) tot[base + q] = d[q];
  }
};

// Workspace views (see layout()).
struct Work {
  unsigned char* fvis;  // per face (setup rows): shown by some pixel
  float4* frec;         // per face: [m0..3] [m4..7] [m8 z0 z1 z2]
  float* facc;          // per face: dL/dm (9), dL/dz_clip (3)
  unsigned char* vvis;  // per vertex (vout rows): corner of a shown face
  float* vvar;          // per vertex: varyings (vstride)
  float* vacc;          // per vertex: dL/d(eye normal or colour varying) (3), then dL/d of the
                        // phong_darboux NDC triangle (9) when that shader is in the batch
  int vstride;
  int vacc_stride;      // 3, or 12 with phong_darboux
  const int2* fmap;     // face block map (kRows faces per block)
  const int2* vmap;     // vertex block map
  unsigned* starts;     // per-job block starts of both maps (2 x (n_jobs + 1))
  LightUnit* light;     // per job: normalised light directions
};

// --------------------------------------------------------------- kernels

// Grids: (pixel blocks of the largest job, n_jobs) for the pixel kernel and
// the mark kernel (whose blocks cover kMarkPixels * kThreads pixels); block
// maps of kRows faces or vertices of one job for the others.

// Pixels per thread of the mark kernel: their winners are loaded together,
// so one block's load latency covers kMarkPixels * kThreads pixels.
constexpr int kMarkPixels = 8;

__global__ void __launch_bounds__(kThreads) mark_kernel(RastBatch B, Work w) {
  const RastJob& J = B.jobs[blockIdx.y];
  const int64_t npx = static_cast<int64_t>(J.width) * J.height;
  const int64_t first = static_cast<int64_t>(blockIdx.x) * kThreads * kMarkPixels;
  if (first >= npx || J.n_faces <= 0) return;  // uniform over the block
  const int layers = job_layers(J, B.max_layers);
  if (layers > 0 && J.mixer == RAST_MIX_OVER && B.pools.layer_prim) {  // every slot the over mixer may blend
    for (int r = 0; r < kMarkPixels; ++r) {
      const int64_t local = first + r * kThreads + threadIdx.x;
      if (local >= npx) break;
      for (int s = 0; s < layers; ++s) {
        const int p = B.pools.layer_prim[s * B.total_pixels + J.pixel_begin + local];
        if (p >= 0) w.fvis[J.setup_begin + p] = 1;
      }
    }
    return;
  }
  int p[kMarkPixels];
#pragma unroll
  for (int r = 0; r < kMarkPixels; ++r) {
    const int64_t local = first + r * kThreads + threadIdx.x;
    p[r] = local < npx ? __ldg(B.pools.prim_id + J.pixel_begin + local) : -1;
  }
  // neighbouring pixels of a warp (along a column) mostly show the same
  // face: one flag store per run of equal winners
#pragma unroll
  for (int r = 0; r < kMarkPixels; ++r) {
    const int prev = __shfl_up_sync(kFull, p[r], 1);
    if (p[r] >= 0 && ((threadIdx.x & 31) == 0 || prev != p[r])) w.fvis[J.setup_begin + p[r]] = 1;
  }
}

// One thread per job: its LightUnit, so that the pixel kernel's blocks load
// it with the job instead of computing it on one thread between two barriers.
__global__ void __launch_bounds__(kThreads) light_kernel(RastBatch B, Work w) {
  const int j = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
  if (j >= B.n_jobs) return;
  const RastJob& J = B.jobs[j];
  LightUnit u;
  u.dir_n = norm3(J.light_direction);
  normalise3(J.light_direction, u.dir);
  u.eye_n = norm3(J.light_dir_eye);
  normalise3(J.light_dir_eye, u.eye);
  w.light[j] = u;
}

// Per visible face: clip rows of its corners, their 3x3 inverse (the forward
// set-up's operations), accumulators zeroed, corner vertices flagged.
__device__ __forceinline__ void face_prep(const RastBatch& B, const Work& w, const RastJob& J, int f) {
  const int64_t row = J.setup_begin + f;
  const int32_t* face = B.pools.faces + (J.face_begin + f) * 3;
  float M[9], zc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int v = gather_clamp(face[k], J.n_verts);
    float p[3], c[4];
    load3(B.pools.position, J.vert_begin + v, p);
    to_clip(J.world_to_clip, p[0], p[1], p[2], c);
    M[3 * k + 0] = c[0];
    M[3 * k + 1] = c[1];
    M[3 * k + 2] = c[3];
    zc[k] = c[2];
    w.vvis[J.vout_begin + v] = 1;
  }
  float m[9];
  inv3(M, m);
  float4* r = w.frec + row * 3;
  r[0] = make_float4(m[0], m[1], m[2], m[3]);
  r[1] = make_float4(m[4], m[5], m[6], m[7]);
  r[2] = make_float4(m[8], zc[0], zc[1], zc[2]);
  float4* a = reinterpret_cast<float4*>(w.facc + row * 12);  // 48-byte rows of a 256-byte aligned array
#pragma unroll
  for (int k = 0; k < 3; ++k) a[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Per flagged vertex: the vertex shader's varyings, accumulators zeroed.
template <int SH>
__device__ __forceinline__ void vertex_prep(const RastBatch& B, const Work& w, const RastJob& J, int v) {
  const int64_t row = J.vout_begin + v;
  const int nv = varying_count(SH >= 0 ? SH : J.shader);
  if (nv > 0) {
    float var[kMaxVarying], clip[4];
    vertex_shader<false, (SH >= 0 ? SH : -1)>(J, B.pools, v, clip, var);
#pragma unroll
    for (int k = 0; k < kMaxVarying; ++k)
      if (k < nv) w.vvar[row * w.vstride + k] = var[k];
  }
  for (int k = 0; k < w.vacc_stride; ++k) w.vacc[row * w.vacc_stride + k] = 0.0f;
}

// The per-face and per-corner kernels cover kRows rows per block: the
// block's visible faces (or flagged corners) are queued in shared memory
// first, so only they occupy lanes.  They are latency-bound gathers: their
// minimum blocks per SM (4 or 5, 48-64 registers) trade a few spills for
// resident warps (vertex_prep 0.55 -> 0.40 ms on the 4096-scene batch).
__global__ void __launch_bounds__(kThreads, 4) face_prep_kernel(RastBatch B, Work w) {
  __shared__ RastJob sJ;
  __shared__ int s_q[kRows];
  __shared__ int s_n;
  const int2 blk = w.fmap[blockIdx.x];
  if (blk.x < 0) return;
  const int nf = __ldg(&B.jobs[blk.x].n_faces);
  load_job_to_shared(B.jobs + blk.x, &sJ);
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const int n = block_queue_rows<kRowsPerThread, kThreads>(
      [&](int r) { return blk.y + r < nf && w.fvis[J.setup_begin + blk.y + r]; }, s_q, &s_n);
  for (int t = threadIdx.x; t < n; t += kThreads) face_prep(B, w, J, blk.y + s_q[t]);
}

// Compiled per shader like the pixel kernel: a single-shader batch's variant
// holds its vertex shader alone (62 registers without spills for
// phong_reflection_shadow, against 64 with spills for the any-shader form:
// 0.397 -> 0.369 ms on the 4096-scene brax-like batch; six blocks per SM at
// 40 registers measured 0.413 ms, two queued vertices per round 0.391 ms).
template <int SH>
__global__ void __launch_bounds__(kThreads, 4) vertex_prep_kernel(RastBatch B, Work w) {
  __shared__ RastJob sJ;
  __shared__ int s_q[kRows];
  __shared__ int s_n;
  const int2 blk = w.vmap[blockIdx.x];
  if (blk.x < 0) return;
  const int nvt = __ldg(&B.jobs[blk.x].n_verts);
  load_job_to_shared(B.jobs + blk.x, &sJ);
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const int n = block_queue_rows<kRowsPerThread, kThreads>(
      [&](int r) { return blk.y + r < nvt && w.vvis[J.vout_begin + blk.y + r]; }, s_q, &s_n);
  for (int t = threadIdx.x; t < n; t += kThreads) vertex_prep<SH>(B, w, J, blk.y + s_q[t]);
}

// Reverse mode of the fragment of shader `sh` at one pixel.  In: the three
// corner varying rows r0..r2, barycentrics b, dL/dcolour.  Out: g_interp
// (dL/d of the interpolated carried varying: eye normal or colour), texel
// gradients (atomics), per-scene light terms into pg.
// Texel-side outputs of one pixel's fragment backward: dL/d texel (gt at
// texture element tb, ch channels) and dL/d specular exponent (gs at sidx);
// keys < 0 mean none.
struct TexGrad {
  int64_t tb = -1;
  int ch = 3;
  float gt[3] = {0.0f, 0.0f, 0.0f};
  int64_t sidx = -1;
  float gs = 0.0f;
  int64_t nb = -1;  // normal-map texel (phong_darboux)
  float gn[3] = {0.0f, 0.0f, 0.0f};
};

template <int SH>
__device__ __forceinline__ void fragment_bwd(const RastJob& J, const RastPools& P, const RastGradPools& G,
                                             const float* r0, const float* r1, const float* r2, const float* b,
                                             const float* gcv, float* g_interp, ParamGrad& pg, TexGrad& tg,
                                             float* gtri, const LightUnit& lu) {
  const int sh = SH >= 0 ? SH : J.shader;
  g_interp[0] = g_interp[1] = g_interp[2] = 0.0f;
  if (may<SH>(RAST_SHADER_GOURAUD) && sh == RAST_SHADER_GOURAUD) {
#pragma unroll
    for (int q = 0; q < 3; ++q) g_interp[q] = gcv[q];
    return;
  }
  if (may<SH>(RAST_SHADER_GOURAUD_TEXTURE) && sh == RAST_SHADER_GOURAUD_TEXTURE) {
    const float u = interp1(b, r0[kVUvG], r1[kVUvG], r2[kVUvG]);
    const float v = interp1(b, r0[kVUvG + 1], r1[kVUvG + 1], r2[kVUvG + 1]);
    const int ui = pymod(f2i(floorf(u)), J.tex_w), wi = pymod(f2i(floorf(v)), J.tex_h);
    float tc[3], lcol[3];
    texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      lcol[q] = interp1(b, r0[kVColour + q], r1[kVColour + q], r2[kVColour + q]);
      g_interp[q] = gcv[q] * tc[q];
      tg.gt[q] = gcv[q] * lcol[q];
    }
    texel_index(J, ui, wi, &tg.tb, &tg.ch);
    return;
  }
  if (sh == RAST_SHADER_DEPTH || sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) return;
  // phong family: n = normalise(sum_k b_k ne_k)
  float nrm[3], n[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) nrm[q] = interp1(b, r0[kVNormal + q], r1[kVNormal + q], r2[kVNormal + q]);
  const float nrmn = unit3_grad(nrm, n);
  float gn[3] = {0.0f, 0.0f, 0.0f};
  if (may<SH>(RAST_SHADER_PHONG_DARBOUX) && sh == RAST_SHADER_PHONG_DARBOUX) {
    // phong_darboux.py:212-293: a Darboux frame from vertex 0's NDC and uv
    // triangles and the interpolated normal, the normal map in that frame,
    // then PhongTextureShader's lighting with the perturbed normal
    const float u = interp1(b, r0[kVUv], r1[kVUv], r2[kVUv]);
    const float v = interp1(b, r0[kVUv + 1], r1[kVUv + 1], r2[kVUv + 1]);
    const int ui = pymod(f2i(floorf(u)), J.tex_w), wi = pymod(f2i(floorf(v)), J.tex_h);
    const float* t = r0 + kVTri;
    const float* tu = r0 + kVTriUv;
    float A[9], AI[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A[c] = t[3 + c] - t[c];
      A[3 + c] = t[6 + c] - t[c];
      A[6 + c] = n[c];
    }
    inv3(A, AI);
    const float bi[3] = {tu[2] - tu[0], tu[4] - tu[0], 0.0f};
    const float bj[3] = {tu[3] - tu[1], tu[5] - tu[1], 0.0f};
    float vi[3], vj[3], ni[3], nj[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      vi[r] = dot3(AI + 3 * r, bi);
      vj[r] = dot3(AI + 3 * r, bj);
    }
    const float vin = unit3_grad(vi, ni), vjn = unit3_grad(vj, nj);
    float nm[3], bn[3], n2[3], tc[3], l[3], lc[3];
    texel3(P.normal_map + J.normal_map_begin, J.nm_w, J.nm_h, 3, ui, wi, nm);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float row[3] = {ni[r], nj[r], n[r]};
      bn[r] = dot3(row, nm);
    }
    const float bnn = unit3_grad(bn, n2);
    texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
    l[0] = lu.dir[0], l[1] = lu.dir[1], l[2] = lu.dir[2];
    const float d = dot3(n2, l);
    bool nonneg = true;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      lc[q] = J.light_colour[q] * d;
      nonneg = nonneg && lc[q] >= 0.0f;
    }
    if (!nonneg) return;
    texel_index(J, ui, wi, &tg.tb, &tg.ch);
    float gd = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      tg.gt[q] = gcv[q] * lc[q];
      const float glc = gcv[q] * tc[q];
      pg.v[RAST_GRAD_LIGHT_COLOUR + q] += glc * d;
      gd += glc * J.light_colour[q];
    }
    float gn2[3], gl[3], gbn[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      gn2[q] = gd * l[q];
      gl[q] = gd * n2[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIRECTION + q] += gl[q];  // normalise's reverse: per block
    normalise3_bwd(n2, bnn, gn2, gbn);
    // bn[r] = ni[r] nm0 + nj[r] nm1 + n[r] nm2
    float gni[3], gnj[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      gni[r] = gbn[r] * nm[0];
      gnj[r] = gbn[r] * nm[1];
      gn[r] += gbn[r] * nm[2];
    }
    const int nu = gather_clamp(ui, J.nm_w), nv = gather_clamp(wi, J.nm_h);
    tg.nb = J.normal_map_begin + (static_cast<int64_t>(nu) * J.nm_h + nv) * 3;
    tg.gn[0] = (gbn[0] * ni[0] + gbn[1] * ni[1]) + gbn[2] * ni[2];
    tg.gn[1] = (gbn[0] * nj[0] + gbn[1] * nj[1]) + gbn[2] * nj[2];
    tg.gn[2] = (gbn[0] * n[0] + gbn[1] * n[1]) + gbn[2] * n[2];
    float gvi[3], gvj[3];
    normalise3_bwd(ni, vin, gni, gvi);
    normalise3_bwd(nj, vjn, gnj, gvj);
    // v = AI b  ->  dL/dAI = gv b^T;  AI = inv(A)  ->  dL/dA = -AI^T dL/dAI AI^T
    float gAI[9], tmp[9], gA[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) gAI[3 * r + k] = gvi[r] * bi[k] + gvj[r] * bj[k];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        tmp[3 * r + k] = (gAI[3 * r + 0] * AI[3 * k + 0] + gAI[3 * r + 1] * AI[3 * k + 1]) + gAI[3 * r + 2] * AI[3 * k + 2];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        gA[3 * r + k] = -((AI[0 * 3 + r] * tmp[0 * 3 + k] + AI[1 * 3 + r] * tmp[1 * 3 + k]) + AI[2 * 3 + r] * tmp[2 * 3 + k]);
    // rows of A: t1 - t0, t2 - t0, n
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gtri[c] = -(gA[c] + gA[3 + c]);
      gtri[3 + c] = gA[c];
      gtri[6 + c] = gA[3 + c];
      gn[c] += gA[6 + c];
    }
  } else if (may<SH>(RAST_SHADER_PHONG) && sh == RAST_SHADER_PHONG) {
    // colour = all(lc >= 0) ? tex * lc : 0,  lc = light_colour * (n . l)
    const float u = interp1(b, r0[kVUv], r1[kVUv], r2[kVUv]);
    const float v = interp1(b, r0[kVUv + 1], r1[kVUv + 1], r2[kVUv + 1]);
    const int ui = pymod(f2i(floorf(u)), J.tex_w), wi = pymod(f2i(floorf(v)), J.tex_h);
    float tc[3], l[3];
    texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
    l[0] = lu.dir[0], l[1] = lu.dir[1], l[2] = lu.dir[2];
    const float d = dot3(n, l);
    bool nonneg = true;
    float lc[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      lc[q] = J.light_colour[q] * d;
      nonneg = nonneg && lc[q] >= 0.0f;
    }
    if (!nonneg) return;
    texel_index(J, ui, wi, &tg.tb, &tg.ch);
    float gd = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      tg.gt[q] = gcv[q] * lc[q];
      const float glc = gcv[q] * tc[q];
      pg.v[RAST_GRAD_LIGHT_COLOUR + q] += glc * d;
      gd += glc * J.light_colour[q];
    }
    float gl[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      gn[q] = gd * l[q];
      gl[q] = gd * n[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIRECTION + q] += gl[q];  // normalise's reverse: per block
  } else {
    // phong_reflection[_shadow] (phong_reflection.py:158-235)
    const bool shadowed = sh == RAST_SHADER_PHONG_REFLECTION_SHADOW;
    float shadow[3] = {1.0f, 1.0f, 1.0f};
    bool lit = true;
    if (shadowed) {
      float scv[4], sc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) scv[q] = interp1(b, r0[kVShadow + q], r1[kVShadow + q], r2[kVShadow + q]);
      apply4(J.shadow_viewport, scv, sc);
      const float sw = sc[3];
#pragma unroll
      for (int q = 0; q < 4; ++q) sc[q] = sc[q] / sw;
      int px = f2i(roundf(sc[0])), py = f2i(roundf(sc[1]));
      if (px < 0) px += J.shadow_w;
      if (py < 0) py += J.shadow_h;
      float depth = kInf;
      if (px >= 0 && px < J.shadow_w && py >= 0 && py < J.shadow_h)
        depth = __ldg(P.shadow_map + J.shadow_begin + static_cast<int64_t>(px) * J.shadow_h + py);
      lit = sc[2] <= depth;
#pragma unroll
      for (int q = 0; q < 3; ++q) shadow[q] = lit ? 1.0f : 1.0f - J.shadow_strength[q];
    }
    const int texidx = __float_as_int(r0[kVTexIdx]);
    const int ti = gather_clamp(texidx, J.n_objects);
    const int32_t* shp = P.texture_shape + (J.texture_shape_begin + ti) * 2;
    float uvr[2];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const float xx = interp1(b, r0[kVUv + a], r1[kVUv + a], r2[kVUv + a]);
      const float whole = (xx >= 0.0f) ? floorf(xx) : ceilf(xx);
      float frac = xx - whole;
      if (frac < 0.0f) frac = frac + 1.0f;
      uvr[a] = frac * static_cast<float>(__ldg(shp + a));
    }
    uvr[0] = uvr[0] + static_cast<float>(texidx * J.texture_offset);
    const int ui = f2i(floorf(uvr[0])), wi = f2i(floorf(uvr[1]));
    float tc[3], l[3];
    texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
    l[0] = lu.eye[0], l[1] = lu.eye[1], l[2] = lu.eye[2];
    const float d = dot3(n, l);
    const float dif = max0(d);
    float r[3], rn[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) r[q] = ((2.0f * d) * n[q]) - l[q];
    const float rnorm = unit3_grad(r, rn);
    const int su = gather_clamp(ui, J.spec_w), sv = gather_clamp(wi, J.spec_h);
    const int64_t sidx = J.specular_begin + static_cast<int64_t>(su) * J.spec_h + sv;
    const float sexp = __ldg(P.specular_map + sidx);
    const float rz = max0(rn[2]);
    const float spec = powf(rz, sexp);
    float gdif = 0.0f, gspec = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float K = J.diffuse[q] * dif + J.specular[q] * spec;
      const float lc = J.light_colour[q];
      tg.gt[q] = gcv[q] * (J.ambient[q] + shadow[q] * K * lc);
      pg.v[RAST_GRAD_AMBIENT + q] += gcv[q] * tc[q];
      const float gK = gcv[q] * shadow[q] * tc[q] * lc;
      pg.v[RAST_GRAD_DIFFUSE + q] += gK * dif;
      pg.v[RAST_GRAD_SPECULAR + q] += gK * spec;
      pg.v[RAST_GRAD_LIGHT_COLOUR + q] += gcv[q] * shadow[q] * K * tc[q];
      if (!lit) pg.v[RAST_GRAD_SHADOW_STRENGTH + q] -= gcv[q] * K * tc[q] * lc;
      gdif += gK * J.diffuse[q];
      gspec += gK * J.specular[q];
    }
    texel_index(J, ui, wi, &tg.tb, &tg.ch);
    // spec = rz ** s: d/dx = s x^(s-1) (0 when s == 0), d/ds = log(x) x^s with log(0) -> 0
    if (rz > 0.0f) {
      tg.sidx = sidx;
      tg.gs = gspec * spec * logf(rz);
    }
    // s x^(s-1) = s x^s / x for x > 0 (no second pow); at x = 0 the pow form
    const float dspec_drz = (sexp == 0.0f) ? 0.0f : (rz > 0.0f ? sexp * (spec * grad_rcp(rz)) : sexp * powf(rz, sexp - 1.0f));
    // through max(rn_z, 0): zero below the kink, without forming 0 * inf
    // (pow's slope at 0 is infinite for exponents below 1)
    const float dmz = dmax0(rn[2]);
    const float grn[3] = {0.0f, 0.0f, dmz == 0.0f ? 0.0f : gspec * dspec_drz * dmz};
    float gr[3];
    normalise3_bwd(rn, rnorm, grn, gr);
    float gd = gdif * dmax0(d);
    float gl[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      gd += 2.0f * gr[q] * n[q];
      gn[q] = 2.0f * d * gr[q];
      gl[q] = -gr[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      gn[q] += gd * l[q];
      gl[q] += gd * n[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIR_EYE + q] += gl[q];  // normalise's reverse: per block
  }
  normalise3_bwd(n, nrmn, gn, g_interp);
}

// Single-shader variants at 4 blocks per SM (64 registers, some spills:
// more resident warps hide the fragment backward's dependency chains
// better); the mixed-shader variants at 3 (80 registers: the mixed 1024-scene
// backward 5.36 -> 4.59 ms, from 2 blocks at 128 registers).
template <int SH>
__host__ __device__ constexpr int pixel_min_blocks() {
  return (SH == RAST_SHADER_PHONG_REFLECTION || SH == RAST_SHADER_PHONG_REFLECTION_SHADOW ||
          SH == RAST_SHADER_PHONG || SH == RAST_SHADER_GOURAUD || SH == RAST_SHADER_GOURAUD_TEXTURE ||
          SH == RAST_SHADER_DEPTH) ? 4 : 3;
}

// dL/dcanvas: read from a gradient image, or formed from the rendered canvas
// and a target for the mean-squared-error loss, (canvas - target) * scale:
// the difference and the product a caller's own elementwise pass would
// round, so both routes hand the kernel the same values.
struct CanvasGrad {
  const float* grad;    // (pixels, 3) or null
  const float* canvas;  // the forward's canvas (with target)
  const float* target;  // (pixels, 3): the MSE route when not null
  float scale;
};

__device__ __forceinline__ float canvas_grad(const CanvasGrad& cg, int64_t k) {
  if (cg.target) return (__ldg(cg.canvas + k) - __ldg(cg.target + k)) * cg.scale;
  return cg.grad ? __ldg(cg.grad + k) : 0.0f;
}

// kLayers: the batch has layered jobs (their over-mixed pixels take one pass
// per slot); without, the pass loop is compiled away.
template <int SH, bool kLayers>
__global__ void __launch_bounds__(kThreads, pixel_min_blocks<SH>())
pixel_kernel(RastBatch B, Work w, CanvasGrad cg, const float* __restrict__ grad_zbuffer, RastGradPools G) {
  __shared__ RastJob sJ;
  __shared__ LightUnit sL;
  constexpr bool kDarboux = may<SH>(RAST_SHADER_PHONG_DARBOUX);
  load_job_to_shared(B.jobs + blockIdx.y, &sJ);
  static_assert(sizeof(LightUnit) == 8 * sizeof(float), "eight floats");
  if (threadIdx.x < 8)
    reinterpret_cast<float*>(&sL)[threadIdx.x] = __ldg(reinterpret_cast<const float*>(w.light + blockIdx.y) + threadIdx.x);
  __syncthreads();
  const RastJob& J = sJ;
  const RastPools& P = B.pools;
  const int sh = SH >= 0 ? SH : J.shader;
  const int64_t npx = static_cast<int64_t>(J.width) * J.height;
  const int64_t local = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  ParamGrad pg;
#pragma unroll
  for (int k = 0; k < RAST_NPARAM; ++k) pg.v[k] = 0.0f;
  const bool in_job = local < npx && J.n_faces > 0;
  const int64_t pix = in_job ? J.pixel_begin + local : 0;
  // The over mixer's pixels take one pass per chooser slot (the slots the
  // forward saved), each kept slot's colour weighted by w = T a of the
  // compositing; every other pixel takes one pass for the primitive it
  // shows.  The pass count is uniform over the block (one job per block).
  const int layers = kLayers ? job_layers(J, B.max_layers) : 0;
  const bool over = kLayers && layers > 0 && J.mixer == RAST_MIX_OVER && P.layer_prim;
  const int passes = over ? layers : 1;
  const bool per_face_alpha = (J.flags & RAST_JOB_FACE_ALPHA) && P.face_alpha;
  // the pixel's output gradients: loaded once up front for layered batches
  // (every pass reads them), at the pass otherwise
  float gz_px = 0.0f, gcv_px[3] = {0.0f, 0.0f, 0.0f};
  auto load_grads = [&]() {
    gz_px = (in_job && grad_zbuffer) ? grad_zbuffer[pix] : 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) gcv_px[q] = in_job ? canvas_grad(cg, pix * 3 + q) : 0.0f;
  };
  if (kLayers) load_grads();
  float transmit = 1.0f;  // the over mixer's T
  bool shown = false;     // a slot of this pixel was kept
  // the warp's table of per-pixel contributions (AccLayout) and their
  // targets; after the passes the same shared memory holds the per-scene
  // parameters' transpose
  using Acc = AccLayout<kDarboux>;
  // the background has a gradient only in layered batches
  constexpr unsigned long long kBits = pixel_bits(SH) & (kLayers ? ~0ull : ~range_bits(RAST_GRAD_BACKGROUND, 3));
  constexpr int kTabFloats = (kThreads / 32) * 32 * Acc::kRow;
  static_assert(transpose_floats<kBits>() <= kTabFloats, "the parameter transpose reuses the table");
  __shared__ __align__(16) float s_tab[kTabFloats];
  __shared__ float* s_tgt[kThreads / 32][32][Acc::kTargets];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* acc_tab = s_tab + warp * 32 * Acc::kRow;
  float** acc_tgt = &s_tgt[warp][0][0];
  const int tex_c = J.tex_c;
  for (int pass = 0; pass < passes; ++pass) {
    int p = -1;
    if (in_job) p = over ? P.layer_prim[pass * B.total_pixels + pix] : P.prim_id[pix];
    // per-pixel contributions, summed per run and added with atomics below
    int64_t frow = -1;
    float fval[12];
    float vval[9];
#pragma unroll
    for (int k = 0; k < 12; ++k) fval[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) vval[k] = 0.0f;
    int64_t vrows[3] = {0, 0, 0};
    TexGrad tg;
    float tval[9];  // dL/d vertex 0's NDC triangle (phong_darboux's Darboux frame)
#pragma unroll
    for (int k = 0; k < 9; ++k) tval[k] = 0.0f;
    if (p >= 0) {
      int i, j;
      pixel_of(local, npx, J.height, &i, &j);
      const float x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
      const float y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
      const int64_t row = J.setup_begin + p;
      const float4* fr = w.frec + row * 3;
      const float4 a = fr[0], bb = fr[1], cz = fr[2];
      const float m[9] = {a.x, a.y, a.z, a.w, bb.x, bb.y, bb.z, bb.w, cz.x};
      const float zc[3] = {cz.y, cz.z, cz.w};
      {
        // corner vertex rows: the same for every pixel of the face (the key of
        // the aggregated vertex accumulation)
        const int32_t* face = P.faces + (J.face_begin + p) * 3;
#pragma unroll
        for (int k = 0; k < 3; ++k) vrows[k] = J.vout_begin + gather_clamp(__ldg(face + k), J.n_verts);
      }
      float c[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) c[k] = (x * m[k] + y * m[3 + k]) + m[6 + k];
      const float wr = (c[0] + c[1]) + c[2];
      const float b[3] = {c[0] / wr, c[1] / wr, c[2] / wr};
      if (!kLayers) load_grads();
      // the corners' varying rows, read where they are used (neighbouring
      // pixels share them, so the reads hit L1) rather than held in registers
      // across the fragment's reverse mode
      const float* r0 = w.vvar + vrows[0] * w.vstride;
      const float* r1 = w.vvar + vrows[1] * w.vstride;
      const float* r2 = w.vvar + vrows[2] * w.vstride;
      float wgt = 1.0f, gz = gz_px;
      bool keep = true;
      if (over) {
        // the slot counts only when its fragment shader keeps it (the
        // Gouraud shaders drop negative interpolated colours)
        if (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) {
#pragma unroll
          for (int q = 0; q < 3; ++q) keep = keep && interp1(b, r0[kVColour + q], r1[kVColour + q], r2[kVColour + q]) >= 0.0f;
        }
        if (keep) {
          const float alpha = per_face_alpha ? __ldg(P.face_alpha + J.face_begin + p) : J.opacity;
          wgt = transmit * alpha;
          transmit = transmit * (1.0f - alpha);
          gz = shown ? 0.0f : gz_px;  // the depth written is the first kept slot's
          shown = true;
        }
      }
      if (keep) {
        float gc[3] = {0.0f, 0.0f, 0.0f};
        float gzc[3] = {0.0f, 0.0f, 0.0f};
        // ---- depth output: z = (sum c_k z_k) * vp22 + vp23
        if (gz != 0.0f) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            gc[k] += gz * J.viewport[10] * zc[k];
            gzc[k] += gz * J.viewport[10] * c[k];
          }
        }
        const float gcv[3] = {wgt * gcv_px[0], wgt * gcv_px[1], wgt * gcv_px[2]};
        if (sh != RAST_SHADER_DEPTH && (gcv[0] != 0.0f || gcv[1] != 0.0f || gcv[2] != 0.0f)) {
          float gi[3];
          fragment_bwd<SH>(J, P, G, r0, r1, r2, b, gcv, gi, pg, tg, tval, sL);
          if (gi[0] != 0.0f || gi[1] != 0.0f || gi[2] != 0.0f) {
            // interpolated = sum_k b_k v_k over the carried varying (offset 0 in
            // both families: eye normal or colour)
            float gb[3];
            gb[0] = (gi[0] * r0[0] + gi[1] * r0[1]) + gi[2] * r0[2];
            gb[1] = (gi[0] * r1[0] + gi[1] * r1[1]) + gi[2] * r1[2];
            gb[2] = (gi[0] * r2[0] + gi[1] * r2[1]) + gi[2] * r2[2];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              vval[3 * k + 0] = b[k] * gi[0];
              vval[3 * k + 1] = b[k] * gi[1];
              vval[3 * k + 2] = b[k] * gi[2];
            }
            // b = c / sum(c)
            const float s = (gb[0] * b[0] + gb[1] * b[1]) + gb[2] * b[2];
            const float rw = grad_rcp(wr);
#pragma unroll
            for (int k = 0; k < 3; ++k) gc[k] += (gb[k] - s) * rw;
          }
        }
        // ---- c_k = x m[k] + y m[3+k] + m[6+k]: dL/dm, dL/dz_clip per face
        frow = row;
        const float xy1[3] = {x, y, 1.0f};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int k = 0; k < 3; ++k) fval[3 * r + k] = xy1[r] * gc[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) fval[9 + k] = gzc[k];
      }
    }
    // ---- per-run sums and atomics (AccLayout): this pixel's row of values
    // and its targets, then lane c sums column c down the warp's rows
    {
      float4* row = reinterpret_cast<float4*>(acc_tab + lane * Acc::kRow);
      row[0] = make_float4(fval[0], fval[1], fval[2], fval[3]);
      row[1] = make_float4(fval[4], fval[5], fval[6], fval[7]);
      row[2] = make_float4(fval[8], fval[9], fval[10], fval[11]);
      row[3] = make_float4(vval[0], vval[1], vval[2], vval[3]);
      row[4] = make_float4(vval[4], vval[5], vval[6], vval[7]);
      row[5] = make_float4(vval[8], tg.gt[0], tg.gt[1], tg.gt[2]);
      if (kDarboux) {
        row[6] = make_float4(tg.gs, tval[0], tval[1], tval[2]);
        row[7] = make_float4(tval[3], tval[4], tval[5], tval[6]);
        row[8] = make_float4(tval[7], tval[8], tg.gn[0], tg.gn[1]);
        row[9] = make_float4(tg.gn[2], 0.0f, 0.0f, 0.0f);
      } else {
        row[6] = make_float4(tg.gs, 0.0f, 0.0f, 0.0f);
      }
      float** tgt = acc_tgt + lane * Acc::kTargets;
      const bool face = frow >= 0;
      tgt[kTgtFace] = face ? w.facc + frow * 12 : nullptr;
#pragma unroll
      for (int k = 0; k < 3; ++k) tgt[kTgtVert0 + k] = face ? w.vacc + vrows[k] * w.vacc_stride : nullptr;
      tgt[kTgtTexel] = (G.texture && tg.tb >= 0) ? G.texture + tg.tb : nullptr;
      tgt[kTgtExponent] = (G.specular_map && tg.sidx >= 0) ? G.specular_map + tg.sidx : nullptr;
      if (kDarboux) tgt[kTgtNormalMap] = (G.normal_map && tg.nb >= 0) ? G.normal_map + tg.nb : nullptr;
      // last pixel of each run, per key kind (face, texel, exponent, normal-map texel)
      const unsigned tails_face = run_tails(frow, face);
      const unsigned tails_texel = run_tails(tg.tb, tg.tb >= 0);
      const unsigned tails_exp = run_tails(tg.sidx, tg.sidx >= 0);
      const unsigned tails_nm = kDarboux ? run_tails(tg.nb, tg.nb >= 0) : 0u;
      __syncwarp();
      for (int c = lane; c < Acc::kCols; c += 32) {  // a second column per lane with phong_darboux
        int target, offset, kind;
        acc_column<kDarboux>(c, tex_c, &target, &offset, &kind);
        const unsigned tails = kind == 0 ? tails_face : kind == 1 ? tails_texel : kind == 2 ? tails_exp : tails_nm;
        float sum = 0.0f;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          sum += acc_tab[q * Acc::kRow + c];
          if ((tails >> q) & 1u) {
            if (sum != 0.0f) {
              float* base = acc_tgt[q * Acc::kTargets + target];
              if (base) red_add(base + offset, sum);
            }
            sum = 0.0f;
          }
        }
      }
      __syncwarp();  // the table is rewritten by the next pass
    }
  }
  // over: the background is seen through what the kept slots let pass
  if (over && shown) {
#pragma unroll
    for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_BACKGROUND + q] += gcv_px[q] * transmit;
  }
  __syncthreads();  // every warp is done with its table before the transpose reuses the memory
  reduce_params<kBits, true>(pg, G.job_params, in_job && (over ? shown : P.prim_id[pix] >= 0), blockIdx.y,
                             LightPost{&sL, sh}, s_tab);
}

// dL/dM = -m^T (dL/dm) m^T for the [x, y, w] rows of the clip positions,
// then clip_k = A [p_k, 1]: dL/dA (per scene, into pg) and dL/dp_k (atomics).
__device__ __forceinline__ void face_post(const RastBatch& B, const Work& w, const RastJob& J,
                                          const RastGradPools& G, int f, ParamGrad& pg) {
  const int64_t row = J.setup_begin + f;
  const float4* fr = w.frec + row * 3;
  const float4 a = fr[0], bb = fr[1], cz = fr[2];
  const float m[9] = {a.x, a.y, a.z, a.w, bb.x, bb.y, bb.z, bb.w, cz.x};
  const float* acc = w.facc + row * 12;
  float gm[9], t[9], gM[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) gm[k] = acc[k];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      t[3 * r + k] = (gm[3 * r + 0] * m[3 * k + 0] + gm[3 * r + 1] * m[3 * k + 1]) + gm[3 * r + 2] * m[3 * k + 2];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      gM[3 * r + k] = -((m[0 * 3 + r] * t[0 * 3 + k] + m[1 * 3 + r] * t[1 * 3 + k]) + m[2 * 3 + r] * t[2 * 3 + k]);
  const int32_t* face = B.pools.faces + (J.face_begin + f) * 3;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float gclip[4] = {gM[3 * k + 0], gM[3 * k + 1], acc[9 + k], gM[3 * k + 2]};
    const int v = gather_clamp(face[k], J.n_verts);
    float p[3];
    load3(B.pools.position, J.vert_begin + v, p);
    const float ph[4] = {p[0], p[1], p[2], 1.0f};
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q) pg.v[RAST_GRAD_WORLD_TO_CLIP + 4 * r + q] += gclip[r] * ph[q];
    if (G.position) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float g = ((gclip[0] * J.world_to_clip[q] + gclip[1] * J.world_to_clip[4 + q]) +
                         gclip[2] * J.world_to_clip[8 + q]) + gclip[3] * J.world_to_clip[12 + q];
        atomicAdd(G.position + (J.vert_begin + v) * 3 + q, g);
      }
    }
  }
}

// One block of face_post work (kRows faces of one job, from the face block
// map); the block's shared job copy and queue are the caller's.
__device__ __forceinline__ void face_post_block(const RastBatch& B, const Work& w, const RastGradPools& G, int2 blk,
                                                RastJob& sJ, int* s_q, int* s_n) {
  if (blk.x < 0) return;  // uniform over the block
  const int nf = __ldg(&B.jobs[blk.x].n_faces);
  load_job_to_shared(B.jobs + blk.x, &sJ);
  if (threadIdx.x == 0) *s_n = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const int n = block_queue_rows<kRowsPerThread, kThreads>(
      [&](int r) { return blk.y + r < nf && w.fvis[J.setup_begin + blk.y + r]; }, s_q, s_n);
  ParamGrad pg;
#pragma unroll
  for (int k = 0; k < 16; ++k) pg.v[RAST_GRAD_WORLD_TO_CLIP + k] = 0.0f;
  for (int t = threadIdx.x; t < n; t += kThreads) face_post(B, w, J, G, blk.y + s_q[t], pg);
  reduce_params<kClipBits>(pg, G.job_params, static_cast<int>(threadIdx.x) < n, blk.x);
}

// Reverse mode of the vertex shader: Gouraud lighting or the eye-space
// normal transform, from the vertex's accumulated dL/d(varying).
template <int SH>
__device__ __forceinline__ void vertex_post(const RastBatch& B, const Work& w, const RastJob& J,
                                            const RastGradPools& G, int v, ParamGrad& pg) {
  const RastPools& P = B.pools;
  const int sh = SH >= 0 ? SH : J.shader;
  const int64_t row = J.vout_begin + v;
  {
    const float* acc = w.vacc + row * w.vacc_stride;
    const float g[3] = {acc[0], acc[1], acc[2]};
    const int64_t vrow = J.vert_begin + v;
    float N[3];
    load3(P.normal, vrow, N);
    const float n1n = norm3(N);
    float n1[3], gN[3];
    normalise3(N, n1);
    if (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) {
      // colour = (C * lc) * (n . l)  or  lc * (n . l)
      float l[3];
      const float ln = norm3(J.light_direction);
      normalise3(J.light_direction, l);
      const float inten = dot3(n1, l);
      float C[3] = {1.0f, 1.0f, 1.0f};
      if (sh == RAST_SHADER_GOURAUD) load3(P.colour, vrow, C);
      float ginten = 0.0f;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float base = (sh == RAST_SHADER_GOURAUD) ? C[q] * J.light_colour[q] : J.light_colour[q];
        ginten += g[q] * base;
        pg.v[RAST_GRAD_LIGHT_COLOUR + q] += g[q] * C[q] * inten;
      }
      if (sh == RAST_SHADER_GOURAUD && G.colour) {
#pragma unroll
        for (int q = 0; q < 3; ++q) atomicAdd(G.colour + vrow * 3 + q, g[q] * J.light_colour[q] * inten);
      }
      float gn[3], gl[3], gL[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        gn[q] = ginten * l[q];
        gl[q] = ginten * n1[q];
      }
      normalise3_bwd(l, ln, gl, gL);
#pragma unroll
      for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIRECTION + q] += gL[q];
      normalise3_bwd(n1, n1n, gn, gN);
    } else {
      // ne = normalise(E[:3, :3] n2), n2 = normalise(n1), n1 = normalise(N)
      const float n2n = norm3(n1);
      float n2[3], h[4], ne[3], gh[3], gn2[3] = {0.0f, 0.0f, 0.0f}, gn1[3];
      normalise3(n1, n2);
      const float hh[4] = {n2[0], n2[1], n2[2], 0.0f};
      apply4(J.world_to_eye_norm, hh, h);
      const float hn = norm3(h);
      normalise3(h, ne);
      normalise3_bwd(ne, hn, g, gh);
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          pg.v[RAST_GRAD_WORLD_TO_EYE_NORM + 4 * r + q] += gh[r] * n2[q];
          gn2[q] += gh[r] * J.world_to_eye_norm[4 * r + q];
        }
      normalise3_bwd(n2, n2n, gn2, gn1);
      normalise3_bwd(n1, n1n, gn1, gN);
    }
    if (G.normal) {
#pragma unroll
      for (int q = 0; q < 3; ++q) atomicAdd(G.normal + vrow * 3 + q, gN[q]);
    }
    if (sh == RAST_SHADER_PHONG_DARBOUX) {
      // the NDC triangle this vertex carried: to_cartesian(world_to_clip [p_k, 1])
      // of its Darboux face's corners (phong_darboux.py:144-148)
      const float* gt = acc + 3;
      const int fid = gather_clamp(P.id_to_face[vrow], J.n_darboux_faces);
      const int32_t* f = P.darboux_faces + (J.darboux_face_begin + fid) * 3;
#pragma unroll 1
      for (int k = 0; k < 3; ++k) {
        const int64_t rk = J.vert_begin + gather_clamp(f[k], J.n_verts);
        float pk[3], tc[4], gclip[4];
        load3(P.position, rk, pk);
        to_clip(J.world_to_clip, pk[0], pk[1], pk[2], tc);
        if (tc[3] == 0.0f) {
          gclip[0] = gt[3 * k + 0];
          gclip[1] = gt[3 * k + 1];
          gclip[2] = gt[3 * k + 2];
          gclip[3] = 0.0f;
        } else {
          const float iw = 1.0f / tc[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) gclip[c] = gt[3 * k + c] * iw;
          gclip[3] = -((gclip[0] * tc[0] + gclip[1] * tc[1]) + gclip[2] * tc[2]) * iw;
        }
        const float ph[4] = {pk[0], pk[1], pk[2], 1.0f};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) pg.v[RAST_GRAD_WORLD_TO_CLIP + 4 * r + q] += gclip[r] * ph[q];
        if (G.position) {
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const float g = ((gclip[0] * J.world_to_clip[q] + gclip[1] * J.world_to_clip[4 + q]) +
                             gclip[2] * J.world_to_clip[8 + q]) + gclip[3] * J.world_to_clip[12 + q];
            atomicAdd(G.position + rk * 3 + q, g);
          }
        }
      }
    }
  }
}

// One block of vertex_post work (kRows vertices of one job, from the
// vertex block map), like face_post_block.
template <int SH>
__device__ __forceinline__ void vertex_post_block(const RastBatch& B, const Work& w, const RastGradPools& G, int2 blk,
                                                  RastJob& sJ, int* s_q, int* s_n) {
  if (blk.x < 0) return;  // uniform over the block
  const int nvt = __ldg(&B.jobs[blk.x].n_verts);
  load_job_to_shared(B.jobs + blk.x, &sJ);
  if (threadIdx.x == 0) *s_n = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const int sh = SH >= 0 ? SH : J.shader;
  const int n = sh == RAST_SHADER_DEPTH ? 0 : block_queue_rows<kRowsPerThread, kThreads>(
      [&](int r) { return blk.y + r < nvt && w.vvis[J.vout_begin + blk.y + r]; }, s_q, s_n);
  ParamGrad pg;
#pragma unroll
  for (int k = 0; k < RAST_NPARAM; ++k) pg.v[k] = 0.0f;
  for (int t = threadIdx.x; t < n; t += kThreads) vertex_post<SH>(B, w, J, G, blk.y + s_q[t], pg);
  reduce_params<vertex_bits(SH)>(pg, G.job_params, static_cast<int>(threadIdx.x) < n, blk.x);
}

// face_post and vertex_post read only what the pixel kernel accumulated and
// add into the gradients with atomics, so one launch runs both, each a
// latency-bound gather over sparse rows: block b takes the face role when
// floor((b + 1) nfb / (nfb + nvb)) > floor(b nfb / (nfb + nvb)) (face block
// floor(b nfb / (nfb + nvb))), the vertex role otherwise (vertex block b
// minus the face blocks before it), so the two kinds are spread evenly over
// the grid and resident together.
template <int SH>
__global__ void __launch_bounds__(kThreads, 4) post_kernel(RastBatch B, Work w, RastGradPools G, unsigned nfb,
                                                            unsigned nvb) {
  __shared__ RastJob sJ;
  __shared__ int s_q[kRows];
  __shared__ int s_n;
  const unsigned long long total = static_cast<unsigned long long>(nfb) + nvb;
  const unsigned long long b = blockIdx.x;
  const unsigned f0 = static_cast<unsigned>(b * nfb / total);
  const unsigned f1 = static_cast<unsigned>((b + 1) * nfb / total);
  if (f1 > f0)
    face_post_block(B, w, G, w.fmap[f0], sJ, s_q, &s_n);
  else
    vertex_post_block<SH>(B, w, G, w.vmap[b - f0], sJ, s_q, &s_n);
}

// ------------------------------------------------------------------ layout

struct Layout {
  size_t fvis_off, frec_off, facc_off, vvis_off, vvar_off, vacc_off, fmap_off, vmap_off, start_off, light_off, total;
  int vacc_stride;
  int vstride;
  unsigned fblocks, vblocks;
};

static Layout layout(const RastBatch& b) {
  Layout L{};
  int vstride = 1;
  for (int s = 0; s < 7; ++s)
    if (b.shader_mask & (1 << s)) vstride = std::max(vstride, varying_count(s));
  L.vstride = vstride;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  const size_t F = static_cast<size_t>(b.total_setup), V = static_cast<size_t>(b.total_vout);
  L.fvis_off = take(F);
  L.frec_off = take(F * 3 * sizeof(float4));
  L.facc_off = take(F * 12 * sizeof(float));
  L.vvis_off = take(V);
  L.vvar_off = take(V * vstride * sizeof(float));
  L.vacc_stride = (b.shader_mask & (1 << RAST_SHADER_PHONG_DARBOUX)) ? 12 : 3;
  L.vacc_off = take(V * L.vacc_stride * sizeof(float));
  L.fblocks = block_map_capacity(b.total_setup, b.n_jobs, kRows);
  L.vblocks = block_map_capacity(b.total_vout, b.n_jobs, kRows);
  L.fmap_off = take(static_cast<size_t>(L.fblocks) * sizeof(int2));
  L.vmap_off = take(static_cast<size_t>(L.vblocks) * sizeof(int2));
  L.start_off = take(2 * block_start_bytes(b.n_jobs));
  L.light_off = take(static_cast<size_t>(b.n_jobs) * sizeof(LightUnit));
  L.total = off;
  return L;
}

template <int SH>
static void launch_all(const RastBatch& b, const Work& w, const Layout& L, const CanvasGrad& gc, const float* gz,
                       const RastGradPools& G, cudaStream_t s, Profiler& prof) {
  const int64_t max_px = static_cast<int64_t>(b.max_width) * b.max_height;
  const dim3 pgrid(static_cast<unsigned>((max_px + kThreads - 1) / kThreads), static_cast<unsigned>(b.n_jobs));
  const unsigned fgrid = L.fblocks, vgrid = L.vblocks;
  build_block_map(b, kMapFaces, kRows, const_cast<int2*>(w.fmap), w.starts, s);
  build_block_map(b, kMapVertices, kRows, const_cast<int2*>(w.vmap), w.starts + b.n_jobs + 1, s);
  const int64_t mark_px = static_cast<int64_t>(kThreads) * kMarkPixels;
  mark_kernel<<<dim3(static_cast<unsigned>((max_px + mark_px - 1) / mark_px), static_cast<unsigned>(b.n_jobs)),
                kThreads, 0, s>>>(b, w);
  light_kernel<<<static_cast<unsigned>((b.n_jobs + kThreads - 1) / kThreads), kThreads, 0, s>>>(b, w);
  prof.mark("backward_mark_kernels");
  face_prep_kernel<<<fgrid, kThreads, 0, s>>>(b, w);
  prof.mark("backward_face_prep_kernel");
  vertex_prep_kernel<SH><<<vgrid, kThreads, 0, s>>>(b, w);
  prof.mark("backward_vertex_prep_kernel");
  if (b.max_layers > 0)
    pixel_kernel<SH, true><<<pgrid, kThreads, 0, s>>>(b, w, gc, gz, G);
  else
    pixel_kernel<SH, false><<<pgrid, kThreads, 0, s>>>(b, w, gc, gz, G);
  prof.mark("backward_pixel_kernel");
  if (fgrid + vgrid > 0) post_kernel<SH><<<fgrid + vgrid, kThreads, 0, s>>>(b, w, G, fgrid, vgrid);
  prof.mark("backward_post_kernel");
}

static int run(const RastBatch* batch, const CanvasGrad& grad_canvas, const float* grad_zbuffer,
               const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream,
               RastProfile* profile) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  if (!grads || !batch->pools.prim_id) return RAST_ERR_INVALID_ARGUMENT;
  if (grad_canvas.target && !grad_canvas.canvas) return RAST_ERR_INVALID_ARGUMENT;
  // the over mixer's gradient needs the slots the forward saved
  if (batch->max_layers > 0 && !batch->pools.layer_prim) return RAST_ERR_INVALID_ARGUMENT;
  const RastBatch& b = *batch;
  const Layout L = layout(b);
  if (workspace_bytes < L.total) return RAST_ERR_WORKSPACE_TOO_SMALL;
  if (L.total > 0 && (workspace == nullptr || (reinterpret_cast<uintptr_t>(workspace) & 255)))
    return RAST_ERR_INVALID_ARGUMENT;
  if (b.total_pixels == 0 || b.total_setup == 0) return RAST_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  Work w{reinterpret_cast<unsigned char*>(ws + L.fvis_off), reinterpret_cast<float4*>(ws + L.frec_off),
         reinterpret_cast<float*>(ws + L.facc_off), reinterpret_cast<unsigned char*>(ws + L.vvis_off),
         reinterpret_cast<float*>(ws + L.vvar_off), reinterpret_cast<float*>(ws + L.vacc_off), L.vstride,
         L.vacc_stride,
         reinterpret_cast<const int2*>(ws + L.fmap_off), reinterpret_cast<const int2*>(ws + L.vmap_off),
         reinterpret_cast<unsigned*>(ws + L.start_off), reinterpret_cast<LightUnit*>(ws + L.light_off)};
  Profiler prof(profile, s, "rast_backward");
  if (cudaMemsetAsync(w.fvis, 0, static_cast<size_t>(b.total_setup), s) != cudaSuccess) return RAST_ERR_CUDA;
  if (cudaMemsetAsync(w.vvis, 0, static_cast<size_t>(b.total_vout), s) != cudaSuccess) return RAST_ERR_CUDA;
  const int mask = b.shader_mask;
  auto only = [&](int sh) { return mask == (1 << sh); };
  if (only(RAST_SHADER_DEPTH)) launch_all<RAST_SHADER_DEPTH>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_GOURAUD)) launch_all<RAST_SHADER_GOURAUD>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_GOURAUD_TEXTURE))
    launch_all<RAST_SHADER_GOURAUD_TEXTURE>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_PHONG)) launch_all<RAST_SHADER_PHONG>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_PHONG_REFLECTION))
    launch_all<RAST_SHADER_PHONG_REFLECTION>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_PHONG_REFLECTION_SHADOW))
    launch_all<RAST_SHADER_PHONG_REFLECTION_SHADOW>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (only(RAST_SHADER_PHONG_DARBOUX))
    launch_all<RAST_SHADER_PHONG_DARBOUX>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else if (mask == ((1 << RAST_SHADER_PHONG_REFLECTION) | (1 << RAST_SHADER_PHONG_REFLECTION_SHADOW)))
    launch_all<kReflectionShaders>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  else
    launch_all<kAnyShader>(b, w, L, grad_canvas, grad_zbuffer, *grads, s, prof);
  if (cudaGetLastError() != cudaSuccess) return RAST_ERR_CUDA;
  return prof.finish();
}

}  // namespace bwd
}  // namespace rast

using namespace rast;

extern "C" size_t rast_backward_workspace_bytes(const RastBatch* batch) {
  if (!batch) return 0;
  return bwd::layout(*batch).total;
}

extern "C" int rast_backward(const RastBatch* batch, const float* grad_canvas, const float* grad_zbuffer,
                             const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream) {
  return bwd::run(batch, bwd::CanvasGrad{grad_canvas, nullptr, nullptr, 0.0f}, grad_zbuffer, grads, workspace,
                  workspace_bytes, stream, nullptr);
}

extern "C" int rast_backward_profiled(const RastBatch* batch, const float* grad_canvas, const float* grad_zbuffer,
                                      const RastGradPools* grads, void* workspace, size_t workspace_bytes,
                                      void* stream, RastProfile* profile) {
  return bwd::run(batch, bwd::CanvasGrad{grad_canvas, nullptr, nullptr, 0.0f}, grad_zbuffer, grads, workspace,
                  workspace_bytes, stream, profile);
}

extern "C" int rast_backward_mse(const RastBatch* batch, const float* target, float scale, const float* grad_zbuffer,
                                 const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream) {
  if (!batch || !target) return RAST_ERR_INVALID_ARGUMENT;
  return bwd::run(batch, bwd::CanvasGrad{nullptr, batch->pools.canvas, target, scale}, grad_zbuffer, grads,
                  workspace, workspace_bytes, stream, nullptr);
}
