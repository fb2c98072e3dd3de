// rast_internal.cuh -- pieces shared by the plain and tiled forms: the
// primitive-setup record, the per-pixel resolve (chooser fallback,
// barycentrics, fragment, mixer) and buffer merge.
#pragma once

#include <nvtx3/nvToolsExt.h>

#include <cstddef>
#include <cstdint>

#include "rast_shaders.cuh"

namespace rast {

constexpr int kTile = 16;         // plain form: 16x16 pixels per CTA
constexpr int kScanThreads = kTile * kTile;
constexpr int kScanChunk = 512;   // primitive setups staged per shared-memory chunk

// Setup record flags (float bits of record[3].y).
constexpr int kKeep = 1;          // |det| > 1e-6 (pipeline.py:98-100)
constexpr int kFront = 2;         // det >= 0 (pipeline.py:232)
constexpr int kCandidate = kKeep | kFront;

inline size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Last job whose *_begin <= row (jobs are laid out in increasing order).
template <typename Get>
__device__ __forceinline__ int find_job(const RastJob* jobs, int n, int64_t row, Get get) {
  int lo = 0, hi = n;  // answer in [lo, hi)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (get(jobs[mid]) <= row) lo = mid; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int find_job_by_vout(const RastJob* jobs, int n, int64_t row) {
  return find_job(jobs, n, row, [](const RastJob& j) { return j.vout_begin; });
}
__device__ __forceinline__ int find_job_by_setup(const RastJob* jobs, int n, int64_t row) {
  return find_job(jobs, n, row, [](const RastJob& j) { return j.setup_begin; });
}

// Job owning rows [row0, row0 + blockDim.x) of a flat per-row launch when
// they all belong to one job (the common case: one binary search per block,
// by thread 0), else -1 (each thread then searches for its own row).  Every
// thread of the block must call it.
template <typename Begin, typename Count>
__device__ __forceinline__ int block_uniform_job(const RastJob* jobs, int n, int64_t row0, int64_t total,
                                                 Begin begin, Count count, int* s_job) {
  if (threadIdx.x == 0) {
    int j = -1;
    if (row0 < total) {
      const int64_t last = min(row0 + static_cast<int64_t>(blockDim.x) - 1, total - 1);
      const int f = find_job(jobs, n, row0, begin);
      if (begin(jobs[f]) + count(jobs[f]) > last) j = f;
    }
    *s_job = j;
  }
  __syncthreads();
  return *s_job;
}

// PerPrimitive.create (pipeline.py:80-113) from the three clip positions.
// Record: [inv0..3] [inv4..7] [inv8 z0 z1 z2] [det flags 0 0].
__device__ __forceinline__ void setup_from_clip(const float4* c, float* inv, float* det_out,
                                                int* flags_out) {
  const float m[9] = {c[0].x, c[0].y, c[0].w, c[1].x, c[1].y, c[1].w, c[2].x, c[2].y, c[2].w};
  const float det = det3(m);
  inv3(m, inv);
  int flags = 0;
  if (fabsf(det) > 1e-6f) flags |= kKeep;
  if (det >= 0.0f) flags |= kFront;
  *det_out = det;
  *flags_out = flags;
}

__device__ __forceinline__ void write_setup(const float4* c, float4* out) {
  float inv[9], det;
  int flags;
  setup_from_clip(c, inv, &det, &flags);
  out[0] = make_float4(inv[0], inv[1], inv[2], inv[3]);
  out[1] = make_float4(inv[4], inv[5], inv[6], inv[7]);
  out[2] = make_float4(inv[8], c[0].z, c[1].z, c[2].z);
  out[3] = make_float4(det, __int_as_float(flags), 0.0f, 0.0f);
}

__device__ __forceinline__ bool is_near_tie(unsigned long long best, uint32_t second) {
  const uint32_t o1 = static_cast<uint32_t>(best >> 32);
  return best != kEmptyKey && o1 != kInfOrder && second != 0xffffffffu && second - o1 <= 1u;
}

// Warp-aggregated count of near ties; every lane of the warp must call it.
__device__ __forceinline__ void count_near_tie(unsigned long long* counter, bool tie) {
  const unsigned m = __ballot_sync(0xffffffffu, tie);
  if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0 && m)
    atomicAdd(counter, static_cast<unsigned long long>(__popc(m)));
}

__device__ __forceinline__ unsigned lanemask_lt() { return (1u << (threadIdx.x & 31)) - 1u; }

// Block-wide compaction: every thread offers `idx` when `flag`; the flagged
// indices land in s_q (order unspecified) and the count is returned.  *s_n
// must be zero and visible to the block on entry; every thread must call.
__device__ __forceinline__ int block_queue(bool flag, int idx, int* s_q, int* s_n) {
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  int base = 0;
  if ((threadIdx.x & 31) == 0 && m) base = atomicAdd(s_n, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (flag) s_q[base + __popc(m & lanemask_lt())] = idx;
  __syncthreads();
  return *s_n;
}

// block_queue over kR rows per thread: row r = threadIdx.x + k * kBlock
// (k < kR) is offered when flag(r); the offered rows land in s_q (order
// unspecified, room for kR * kBlock) and the count is returned.  *s_n must be
// zero and visible to the block on entry; every thread must call.
template <int kR, int kBlock, class Flag>
__device__ __forceinline__ int block_queue_rows(Flag flag, int* s_q, int* s_n) {
#pragma unroll
  for (int k = 0; k < kR; ++k) {
    const int r = static_cast<int>(threadIdx.x) + k * kBlock;
    const bool f = flag(r);
    const unsigned m = __ballot_sync(0xffffffffu, f);
    int base = 0;
    if ((threadIdx.x & 31) == 0 && m) base = atomicAdd(s_n, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (f) s_q[base + __popc(m & lanemask_lt())] = r;
  }
  __syncthreads();
  return *s_n;
}

// ---- block maps: grids over the faces (or vertices) of every job with no
// empty blocks.  Entry b of the map is (job, first item of the block) for
// the b-th block of the concatenated per-job block ranges, (-1, 0) past the
// end.  A batch needs at most floor(total / per_block) + n_jobs blocks.
constexpr int kMapFaces = 0, kMapVertices = 1;

__host__ __device__ inline unsigned block_map_capacity(int64_t total, int n_jobs, int per_block) {
  return static_cast<unsigned>(total / per_block + n_jobs);
}

template <int kField>
__device__ __forceinline__ unsigned blocks_of_job(const RastJob* jobs, int j, int per_block) {
  const int n = kField == kMapFaces ? __ldg(&jobs[j].n_faces) : __ldg(&jobs[j].n_verts);
  return n > 0 ? static_cast<unsigned>((n + per_block - 1) / per_block) : 0u;
}

// Exclusive prefix of per-job block counts -> start[0..n_jobs] (start[n_jobs]
// = total).  One block of 1024 threads; thread t owns a contiguous run of jobs.
template <int kField>
__global__ void __launch_bounds__(1024)
block_prefix_kernel(const RastJob* __restrict__ jobs, int n_jobs, int per_block, unsigned* __restrict__ start) {
  __shared__ unsigned s_sum[1024];
  const int t = threadIdx.x;
  const int per_thread = (n_jobs + 1023) / 1024;
  const int j0 = min(n_jobs, t * per_thread), j1 = min(n_jobs, j0 + per_thread);
  unsigned mine = 0;
  for (int j = j0; j < j1; ++j) mine += blocks_of_job<kField>(jobs, j, per_block);
  s_sum[t] = mine;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const unsigned add = t >= off ? s_sum[t - off] : 0u;
    __syncthreads();
    s_sum[t] += add;
    __syncthreads();
  }
  unsigned at = s_sum[t] - mine;
  for (int j = j0; j < j1; ++j) {
    start[j] = at;
    at += blocks_of_job<kField>(jobs, j, per_block);
  }
  if (t == 1023) start[n_jobs] = s_sum[1023];
}

// One thread per job writes its blocks' entries; the threads past the jobs
// fill the tail of the map (entries >= total) with (-1, 0).
template <int kField>
__global__ void __launch_bounds__(256)
block_fill_kernel(const RastJob* __restrict__ jobs, int n_jobs, int per_block, const unsigned* __restrict__ start,
                  int2* __restrict__ map, unsigned capacity) {
  const int j = blockIdx.x * 256 + threadIdx.x;
  if (j < n_jobs) {
    const unsigned a = start[j], nb = start[j + 1] - a;
    for (unsigned b = 0; b < nb && a + b < capacity; ++b) map[a + b] = make_int2(j, static_cast<int>(b) * per_block);
  }
  const unsigned total = start[n_jobs];
  const unsigned stride = gridDim.x * 256u;
  for (unsigned k = total + static_cast<unsigned>(j); k < capacity; k += stride) map[k] = make_int2(-1, 0);
}

// Builds the map of `field` for batch b on stream s.  `start` holds
// n_jobs + 1 unsigned.
inline cudaError_t build_block_map(const RastBatch& b, int field, int per_block, int2* map, unsigned* start,
                                   cudaStream_t s) {
  const int64_t total = field == kMapFaces ? b.total_setup : b.total_vout;
  const unsigned cap = block_map_capacity(total, b.n_jobs, per_block);
  if (cap == 0 || b.n_jobs <= 0) return cudaSuccess;
  const unsigned grid = static_cast<unsigned>((b.n_jobs + 255) / 256);
  if (field == kMapFaces) {
    block_prefix_kernel<kMapFaces><<<1, 1024, 0, s>>>(b.jobs, b.n_jobs, per_block, start);
    block_fill_kernel<kMapFaces><<<grid, 256, 0, s>>>(b.jobs, b.n_jobs, per_block, start, map, cap);
  } else {
    block_prefix_kernel<kMapVertices><<<1, 1024, 0, s>>>(b.jobs, b.n_jobs, per_block, start);
    block_fill_kernel<kMapVertices><<<grid, 256, 0, s>>>(b.jobs, b.n_jobs, per_block, start, map, cap);
  }
  return cudaGetLastError();
}

// Bytes of the per-job block starts that build_block_map needs.
inline size_t block_start_bytes(int n_jobs) { return (static_cast<size_t>(n_jobs) + 1) * sizeof(unsigned); }

// Pixel (i, j) of a job from its x-major local index i * H + j; 32-bit
// division when the job's pixel count fits (every job in practice).
__device__ __forceinline__ void pixel_of(int64_t local, int64_t npx, int H, int* i, int* j) {
  if (npx <= 0x7fffffff) {
    const int l = static_cast<int>(local);
    *i = l / H;
    *j = l - *i * H;
  } else {
    *i = static_cast<int>(local / H);
    *j = static_cast<int>(local - static_cast<int64_t>(*i) * H);
  }
}

__device__ __forceinline__ void load_job_to_shared(const RastJob* job, RastJob* dst) {
  const int nthreads = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int* src = reinterpret_cast<const int*>(job);
  int* d = reinterpret_cast<int*>(dst);
  for (int k = tid; k < static_cast<int>(sizeof(RastJob) / 4); k += nthreads) d[k] = __ldg(src + k);
}

// Where the vertex varyings of a face come from: the vertex kernel's output
// (plain form) or a recomputation of the vertex shader (tiled form).
struct VaryingSource {
  const float* var;   // per-vertex varyings (plain form), or nullptr
  int vstride;
  int64_t vout_begin;
  const float* fvar = nullptr;  // per-face varyings of visible faces (tiled form): 3 rows of vstride per face
  int64_t setup_begin = 0;
};

struct PixelResult {
  bool keep;
  float z;
  float colour[3];
  int prim;
};

// Interpolation and fragment shader of primitive p at the pixel whose NDC
// coordinates are (x, y) (pipeline.py:283-326): clip coefficients, chooser keep (keep & inside),
// depth, perspective-correct barycentrics, the corner varyings from `src`,
// then the job's fragment shader.
struct Fragment {
  bool chooser_keep;  // keep & inside (the chooser's keeps slice)
  bool keep;          // the fragment shader's keep
  float z;
  float colour[3];
};

// Without xy_given, (x, y) is computed here from the pixel (i, j).
__device__ __forceinline__ void shade_primitive(const RastJob& J, const RastPools& P, const float4* rec_base,
                                                int i, int j, float x, float y, int p, const VaryingSource& src,
                                                Fragment* f, bool xy_given) {
  const float4* rec = rec_base + static_cast<int64_t>(p) * 4;
  const float4 a = rec[0], b = rec[1], cz = rec[2], d = rec[3];
  if (!xy_given) {
    x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
    y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
  }
  const float c[3] = {(x * a.x + y * a.w) + b.z, (x * a.y + y * b.x) + b.w,
                      (x * a.z + y * b.y) + cz.x};
  const bool in_tri = c[0] >= 0.0f && c[1] >= 0.0f && c[2] >= 0.0f;
  const int flags = __float_as_int(d.y);
  f->chooser_keep = (flags & kKeep) && in_tri;
  const bool front = (flags & kFront) != 0;
  const float w_rcp = (c[0] + c[1]) + c[2];
  f->z = ((c[0] * cz.y + c[1] * cz.z) + c[2] * cz.w) * J.viewport[10] + J.viewport[11];
  const float bary[3] = {c[0] / w_rcp, c[1] / w_rcp, c[2] / w_rcp};
  const int32_t* face = P.faces + (J.face_begin + p) * 3;
  const int nv = varying_count(J.shader);
  float v0[kMaxVarying], v1[kMaxVarying], v2[kMaxVarying];
  if (nv > 0) {
    const int i0 = gather_clamp(face[0], J.n_verts);
    const int i1 = gather_clamp(face[1], J.n_verts);
    const int i2 = gather_clamp(face[2], J.n_verts);
    if (src.fvar || src.var) {
      const float *r0, *r1, *r2;
      if (src.fvar) {
        r0 = src.fvar + ((src.setup_begin + p) * 3) * src.vstride;
        r1 = r0 + src.vstride;
        r2 = r1 + src.vstride;
      } else {
        r0 = src.var + (src.vout_begin + i0) * src.vstride;
        r1 = src.var + (src.vout_begin + i1) * src.vstride;
        r2 = src.var + (src.vout_begin + i2) * src.vstride;
      }
      // constant indices keep the three rows in registers
#pragma unroll
      for (int k = 0; k < kMaxVarying; ++k) {
        if (k < nv) {
          v0[k] = __ldg(r0 + k);
          v1[k] = __ldg(r1 + k);
          v2[k] = __ldg(r2 + k);
        }
      }
    } else {
      float clip[4];
      vertex_shader<false>(J, P, i0, clip, v0);
      vertex_shader<false>(J, P, i1, clip, v1);
      vertex_shader<false>(J, P, i2, clip, v2);
    }
  }
  f->colour[0] = f->colour[1] = f->colour[2] = 0.0f;
  f->keep = fragment_shader(J, P, v0, v1, v2, bary, front, f->colour);
}

// One pixel after the scan: `w` is the winning candidate (-1: none, or its
// depth was +inf).  Reproduces the default chooser's fallback to primitive 0
// (shader.py:215-217), then Shader.interpolate / fragment / mix
// (pipeline.py:283-359) for the chosen primitive.
__device__ __forceinline__ void resolve_pixel(const RastJob& J, const RastPools& P,
                                              const float4* rec_base, int i, int j, int w,
                                              const VaryingSource& src, PixelResult* r) {
  r->keep = false;
  r->prim = -1;
  r->z = 0.0f;
  r->colour[0] = r->colour[1] = r->colour[2] = 0.0f;
  if (J.n_faces <= 0) return;
  const int p = w < 0 ? 0 : w;
  Fragment f;
  shade_primitive(J, P, rec_base, i, j, 0.0f, 0.0f, p, src, &f, false);
  r->keep = f.chooser_keep && f.keep;
  r->z = f.z;
  r->prim = r->keep ? p : -1;
#pragma unroll
  for (int k = 0; k < 3; ++k) r->colour[k] = f.colour[k];
}

// Chooser slots of job J: 0 = the default chooser, else the layered
// chooser's slot count (clamped to the batch's max_layers).
__device__ __forceinline__ int job_layers(const RastJob& J, int max_layers) {
  return J.layers <= 0 ? 0 : min(J.layers, max_layers);
}

// One pixel of a layered job (RastJob.layers = L >= 1): slots
// w[0 .. L-1] (stride `wstride`) hold the nearest candidates in ascending
// (depth, id) order, -1 past the last.  Every slot from `first` on runs
// interpolation + fragment; the job's mixer combines the kept ones
// (RastMixer).  first > 0 continues a nearest-mixer pixel whose earlier
// slots were all discarded.
__device__ __forceinline__ void resolve_layers(const RastJob& J, const RastPools& P, const float4* rec_base,
                                               int i, int j, const int32_t* w, int64_t wstride, int L,
                                               const VaryingSource& src, PixelResult* r, int first = 0) {
  r->keep = false;
  r->prim = -1;
  r->z = 0.0f;
  r->colour[0] = r->colour[1] = r->colour[2] = 0.0f;
  const bool over = J.mixer == RAST_MIX_OVER;
  const bool per_face = (J.flags & RAST_JOB_FACE_ALPHA) && P.face_alpha;
  const float x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
  const float y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
  // the slots, loaded up front and shifted down one per step (no indexed
  // register array)
  int w0 = first < 1 ? w[0] : -1, w1 = L > 1 && first < 2 ? w[wstride] : -1;
  int w2 = L > 2 && first < 3 ? w[2 * wstride] : -1, w3 = L > 3 && first < 4 ? w[3 * wstride] : -1;
  static_assert(RAST_MAX_LAYERS == 4, "slot registers w0..w3");
  for (int s = 0; s < first; ++s) w0 = w1, w1 = w2, w2 = w3, w3 = -1;
  float T = 1.0f, C[3] = {0.0f, 0.0f, 0.0f};
  for (int s = first; s < L; ++s) {
    const int p = w0;
    w0 = w1, w1 = w2, w2 = w3, w3 = -1;
    if (p < 0) break;
    Fragment f;
    shade_primitive(J, P, rec_base, i, j, x, y, p, src, &f, true);
    if (!(f.chooser_keep && f.keep)) continue;
    if (!r->keep) {
      r->keep = true;
      r->z = f.z;
      r->prim = p;
      if (!over) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r->colour[k] = f.colour[k];
        return;
      }
    }
    const float alpha = per_face ? __ldg(P.face_alpha + J.face_begin + p) : J.opacity;
    const float wgt = T * alpha;
#pragma unroll
    for (int k = 0; k < 3; ++k) C[k] = C[k] + wgt * f.colour[k];
    T = T * (1.0f - alpha);
  }
  if (r->keep && over) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r->colour[k] = C[k] + T * J.background[k];
  }
}

// Fragments of one warp's pixels under the layered chooser: at most
// RAST_MAX_LAYERS per pixel.
constexpr int kWarpFrags = 32 * RAST_MAX_LAYERS;

// Shared-memory staging of one warp's fragments for resolve_over_warp.
struct WarpFrags {
  float colour[3][kWarpFrags];
  float z[kWarpFrags];
  unsigned char keep[kWarpFrags];
};

// RAST_MIX_OVER pixels of one warp, all 32 lanes calling (inactive lanes
// own no pixel): the warp's (pixel, slot) fragments are numbered in lane
// order, 32 of them shaded per round with one fragment per lane (so pixels
// with fewer layers leave no lane idle while others shade), staged in `wf`,
// then every lane mixes its own pixel's fragments in slot order.  Same
// operations and order as resolve_layers.
__device__ __forceinline__ void resolve_over_warp(const RastJob& J, const RastPools& P, const float4* rec_base,
                                                  bool active, int i, int j, const int32_t* w, int64_t wstride,
                                                  int L, const VaryingSource& src, WarpFrags& wf,
                                                  PixelResult* r) {
  const int lane = threadIdx.x & 31;
  r->keep = false;
  r->prim = -1;
  r->z = 0.0f;
  r->colour[0] = r->colour[1] = r->colour[2] = 0.0f;
  static_assert(RAST_MAX_LAYERS == 4, "slot registers w0..w3");
  int w0 = -1, w1 = -1, w2 = -1, w3 = -1, n = 0;
  float x = 0.0f, y = 0.0f;
  if (active) {
    x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
    y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
    w0 = w[0];
    if (L > 1) w1 = w[wstride];
    if (L > 2) w2 = w[2 * wstride];
    if (L > 3) w3 = w[3 * wstride];
    n = w0 < 0 ? 0 : w1 < 0 ? 1 : w2 < 0 ? 2 : w3 < 0 ? 3 : 4;  // leading filled slots
  }
  int incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  const int excl = incl - n;
  const int total = __shfl_sync(0xffffffffu, incl, 31);  // <= kWarpFrags
  for (int base = 0; base < total; base += 32) {
    const int k = base + lane;
    int owner = 0;  // the lane whose fragments [excl, incl) hold k
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int v = __shfl_sync(0xffffffffu, incl, owner + step - 1);
      if (v <= k) owner += step;
    }
    const int slot = k - __shfl_sync(0xffffffffu, excl, owner);
    const int a0 = __shfl_sync(0xffffffffu, w0, owner), a1 = __shfl_sync(0xffffffffu, w1, owner);
    const int a2 = __shfl_sync(0xffffffffu, w2, owner), a3 = __shfl_sync(0xffffffffu, w3, owner);
    const float ox = __shfl_sync(0xffffffffu, x, owner), oy = __shfl_sync(0xffffffffu, y, owner);
    if (k < total) {
      const int p = slot == 0 ? a0 : slot == 1 ? a1 : slot == 2 ? a2 : a3;
      Fragment f;
      shade_primitive(J, P, rec_base, 0, 0, ox, oy, p, src, &f, true);
#pragma unroll
      for (int c = 0; c < 3; ++c) wf.colour[c][k] = f.colour[c];
      wf.z[k] = f.z;
      wf.keep[k] = f.chooser_keep && f.keep;
    }
  }
  __syncwarp();
  const bool per_face = (J.flags & RAST_JOB_FACE_ALPHA) && P.face_alpha;
  float T = 1.0f, C[3] = {0.0f, 0.0f, 0.0f};
  for (int s = 0; s < n; ++s) {
    const int k = excl + s;
    const int p = w0;
    w0 = w1, w1 = w2, w2 = w3, w3 = -1;
    if (!wf.keep[k]) continue;
    if (!r->keep) {
      r->keep = true;
      r->z = wf.z[k];
      r->prim = p;
    }
    const float alpha = per_face ? __ldg(P.face_alpha + J.face_begin + p) : J.opacity;
    const float wgt = T * alpha;
#pragma unroll
    for (int c = 0; c < 3; ++c) C[c] = C[c] + wgt * wf.colour[c][k];
    T = T * (1.0f - alpha);
  }
  if (r->keep) {
#pragma unroll
    for (int c = 0; c < 3; ++c) r->colour[c] = C[c] + T * J.background[c];
  }
}

// The forward's record of a layered pixel's slots for the backward
// (RastPools.layer_prim, slot-major): slots 0 .. L-1 from the winner planes,
// -1 past them.
__device__ __forceinline__ void save_layers(const RastPools& P, const int32_t* w, int64_t wstride, int64_t pix,
                                            int L) {
  if (!P.layer_prim) return;
#pragma unroll
  for (int s = 0; s < RAST_MAX_LAYERS; ++s) P.layer_prim[s * wstride + pix] = s < L ? w[s * wstride] : -1;
}

// Keeps best[0 .. L-1] the L smallest keys seen, ascending: `key` goes in
// at its rank and the larger ones move down one slot.
template <int L>
__device__ __forceinline__ void insert_key(unsigned long long (&best)[L], unsigned long long key) {
#pragma unroll
  for (int s = L - 1; s > 0; --s)
    if (key < best[s]) best[s] = key < best[s - 1] ? best[s - 1] : key;
  if (key < best[0]) best[0] = key;
}

// merge_buffers (pipeline.py:401-440): overwrite where kept, no depth test;
// then the shadow pass's offset (shadow.py:116) when the job asks for it.
__device__ __forceinline__ void store_pixel(const RastJob& J, const RastPools& P, int64_t pix,
                                            const PixelResult& r) {
  const bool offset = (J.flags & RAST_JOB_APPLY_DEPTH_OFFSET) != 0;
  if (r.keep || offset) {
    float zb = r.keep ? r.z : P.zbuffer[pix];
    if (offset) zb = zb + J.depth_offset;
    P.zbuffer[pix] = zb;
  }
  if (r.keep && J.shader != RAST_SHADER_DEPTH && P.canvas) {
    P.canvas[pix * 3 + 0] = r.colour[0];
    P.canvas[pix * 3 + 1] = r.colour[1];
    P.canvas[pix * 3 + 2] = r.colour[2];
  }
  if (P.prim_id) P.prim_id[pix] = r.prim;
}

// Optional per-kernel event timing of an entry point (RastProfile).
// NVTX range over one entry point's host-side launch sequence (header-only
// NVTX3: without a profiler attached a push / pop is a check of a null hook).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Per-kernel CUDA-event timing of an entry point (the *_profiled entry
// points) and its NVTX annotation: a range named after the entry point and
// one NVTX mark per kernel launched, named after the kernel.
struct Profiler {
  RastProfile* prof;
  cudaStream_t stream;
  cudaEvent_t ev[17];
  int n = 0;
  NvtxRange range;
  Profiler(RastProfile* p, cudaStream_t s, const char* entry) : prof(p), stream(s), range(entry) {
    if (prof) {
      prof->n = 0;
      cudaEventCreate(&ev[0]);
      cudaEventRecord(ev[0], stream);
    }
  }
  void mark(const char* name) {
    nvtxMarkA(name);
    if (!prof || n >= 16) return;
    cudaEventCreate(&ev[n + 1]);
    cudaEventRecord(ev[n + 1], stream);
    prof->names[n] = name;
    ++n;
  }
  int finish() {
    if (!prof) return RAST_OK;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return RAST_ERR_CUDA;
    for (int k = 0; k < n; ++k) cudaEventElapsedTime(&prof->ms[k], ev[k], ev[k + 1]);
    for (int k = 0; k <= n; ++k) cudaEventDestroy(ev[k]);
    prof->n = n;
    return RAST_OK;
  }
};

// Host-side argument checks shared by the entry points.
inline int check_batch(const RastBatch* b) {
  if (!b || !b->jobs) return RAST_ERR_INVALID_ARGUMENT;
  if (b->n_jobs < 1 || b->n_jobs > 65535) return RAST_ERR_INVALID_ARGUMENT;
  if (b->total_vout < 0 || b->total_setup < 0 || b->total_pixels < 0) return RAST_ERR_INVALID_ARGUMENT;
  if (b->max_width < 0 || b->max_height < 0 || b->max_faces < 0 || b->max_verts < 0)
    return RAST_ERR_INVALID_ARGUMENT;
  if ((b->shader_mask & ~0x7f) != 0) return RAST_ERR_INVALID_ARGUMENT;
  if (b->max_layers < 0 || b->max_layers > RAST_MAX_LAYERS) return RAST_ERR_INVALID_ARGUMENT;
  if (b->total_pixels > 0 && !b->pools.zbuffer) return RAST_ERR_INVALID_ARGUMENT;
  if (b->total_setup > 0 && (!b->pools.faces || !b->pools.position)) return RAST_ERR_INVALID_ARGUMENT;
  if (b->total_vout > 0 && !b->pools.position) return RAST_ERR_INVALID_ARGUMENT;
  return RAST_OK;
}

}  // namespace rast
