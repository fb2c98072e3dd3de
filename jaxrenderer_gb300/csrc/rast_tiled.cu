// rast_tiled.cu -- tiled, binned form of the rasteriser for many scenes per
// call.  Same results as the plain form (and the reference): every
// (pixel, candidate primitive) pair whose FP32 edge functions are all >= 0 is
// tested with the same operations; binning only removes pairs that cannot
// pass.
//
//   job_tiles_kernel   per-job tile grid (fixed stride: tiles of the largest job)
//   setup_bin_kernel   one thread per face: clip positions, det/keep/inverse,
//                      conservative tile range of its coverage region, bin counts
//   scan_local_kernel  \  exclusive prefix sum of bin counts -> bin offsets;
//   scan_apply_kernel  /  tiles whose bins exceed the capacity are marked
//   scatter_kernel     one thread per face: face id into every bin it overlaps
//   raster_kernel      persistent warps, one tile each: bin entries staged in
//                      shared memory, per-pixel packed (depth | id) minimum
//   tiled_shade_kernel one thread per pixel: deferred shading of the winner,
//                      vertex varyings recomputed for its three corners only
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "rast_internal.cuh"

namespace rast {
namespace tiled {

constexpr int kSetupThreads = 256;
constexpr int kScanBlock = 1024;       // elements per scan block (256 threads x 4)
constexpr int kRasterWarps = 4;        // warps per CTA of the raster kernel
constexpr int kStage = 32;             // bin entries staged per warp round
constexpr uint32_t kOverflow = 0x80000000u;

// Tile shapes offered to the autotuner.  (tw, th): tw pixels along x
// (axis 0 of the buffers), th along y (contiguous in memory).
struct TileShape {
  int tw, th;
};

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// --------------------------------------------------------- conservative bins

// Clip a convex polygon (n <= 8 vertices) against a*x + b*y + c >= 0.
__device__ __forceinline__ int clip_poly(const float* px, const float* py, int n, float a, float b,
                                         float c, float* ox, float* oy) {
  int m = 0;
  for (int k = 0; k < n; ++k) {
    const int k2 = (k + 1 == n) ? 0 : k + 1;
    const float x0 = px[k], y0 = py[k], x1 = px[k2], y1 = py[k2];
    const float d0 = a * x0 + b * y0 + c;
    const float d1 = a * x1 + b * y1 + c;
    const bool in0 = d0 >= 0.0f, in1 = d1 >= 0.0f;
    if (in0 && m < 8) {
      ox[m] = x0;
      oy[m] = y0;
      ++m;
    }
    if (in0 != in1 && m < 8) {
      const float t = d0 / (d0 - d1);  // no cancellation: d0, d1 of opposite signs
      ox[m] = x0 + t * (x1 - x0);
      oy[m] = y0 + t * (y1 - y0);
      ++m;
    }
  }
  return m;
}

// Pixel range [i0, i1] x [j0, j1] that contains every pixel whose FP32 edge
// functions c_k = (x * inv[k] + y * inv[3 + k]) + inv[6 + k] can all be
// >= 0.  Computed by clipping the job's screen rectangle (one pixel wider on
// every side, in NDC) against c_k >= -eps_k, where eps_k is 64x the rounding
// bound of the three-operation evaluation of c_k, then widening the bounding
// box by one pixel.  Returns false when no pixel can be covered.
__device__ __forceinline__ bool coverage_bbox(const float* inv, const RastJob& J, int* i0, int* i1,
                                              int* j0, int* j1) {
  const int W = J.width, H = J.height;
  const float sx = J.viewport[0], ox = J.viewport[3];
  const float sy = J.viewport[5], oy = J.viewport[7];
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 9; ++k) finite = finite && isfinite(inv[k]);
  if (!finite || !(sx != 0.0f) || !(sy != 0.0f) || !isfinite(sx) || !isfinite(sy)) {
    *i0 = 0;
    *i1 = W - 1;
    *j0 = 0;
    *j1 = H - 1;
    return true;  // cannot bound: every pixel of the job
  }
  // NDC of pixels -1 and W (one pixel outside the screen on each side)
  const float xa = (-1.0f - ox) / sx, xb = (static_cast<float>(W) - ox) / sx;
  const float ya = (-1.0f - oy) / sy, yb = (static_cast<float>(H) - oy) / sy;
  const float xl = fminf(xa, xb), xh = fmaxf(xa, xb), yl = fminf(ya, yb), yh = fmaxf(ya, yb);
  const float X = fmaxf(fabsf(xl), fabsf(xh)), Y = fmaxf(fabsf(yl), fabsf(yh));
  float px[8] = {xl, xh, xh, xl}, py[8] = {yl, yl, yh, yh};
  float qx[8], qy[8];
  int n = 4;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float a = inv[k], b = inv[3 + k], c = inv[6 + k];
    const float eps = 64.0f * 5.9604645e-08f * (X * fabsf(a) + Y * fabsf(b) + fabsf(c));
    if (k == 1) n = clip_poly(qx, qy, n, a, b, c + eps, px, py);
    else n = clip_poly(px, py, n, a, b, c + eps, qx, qy);
    if (n == 0) return false;
  }
  // result is in qx/qy after clips 0 (p->q), 1 (q->p), 2 (p->q)
  float mnx = qx[0], mxx = qx[0], mny = qy[0], mxy = qy[0];
  for (int k = 1; k < n; ++k) {
    mnx = fminf(mnx, qx[k]);
    mxx = fmaxf(mxx, qx[k]);
    mny = fminf(mny, qy[k]);
    mxy = fmaxf(mxy, qy[k]);
  }
  // NDC -> pixel index: i = x * sx + ox (monotone in x with the sign of sx)
  const float pa = mnx * sx + ox, pb = mxx * sx + ox;
  const float qa = mny * sy + oy, qb = mxy * sy + oy;
  const float ilo = floorf(fminf(pa, pb)) - 1.0f, ihi = ceilf(fmaxf(pa, pb)) + 1.0f;
  const float jlo = floorf(fminf(qa, qb)) - 1.0f, jhi = ceilf(fmaxf(qa, qb)) + 1.0f;
  if (!(ihi >= 0.0f) || !(ilo <= static_cast<float>(W - 1)) || !(jhi >= 0.0f) ||
      !(jlo <= static_cast<float>(H - 1)))
    return false;
  *i0 = static_cast<int>(fmaxf(ilo, 0.0f));
  *i1 = static_cast<int>(fminf(ihi, static_cast<float>(W - 1)));
  *j0 = static_cast<int>(fmaxf(jlo, 0.0f));
  *j1 = static_cast<int>(fminf(jhi, static_cast<float>(H - 1)));
  return true;
}

// ------------------------------------------------------------------ kernels

struct Geometry {
  int tw, th;       // tile shape
  int tiles_x;      // tiles along x of the largest job (stride)
  int tiles_y;
  int tiles_per_job;
};

// Vertex positions of face f of job J -> clip space (same operations as the
// vertex shader's gl_Position).
__device__ __forceinline__ void face_clip(const RastJob& J, const RastPools& P, int64_t f,
                                          float4* c) {
  const int32_t* face = P.faces + (J.face_begin + f) * 3;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int v = gather_clamp(__ldg(face + k), J.n_verts);
    const float* p = P.position + (J.vert_begin + v) * 3;
    float out[4];
    to_clip(J.world_to_clip, __ldg(p), __ldg(p + 1), __ldg(p + 2), out);
    c[k] = make_float4(out[0], out[1], out[2], out[3]);
  }
}

// Grid: (ceil(max_faces / kSetupThreads), n_jobs); blockIdx.y is the job.
__global__ void __launch_bounds__(kSetupThreads)
setup_bin_kernel(RastBatch B, Geometry G, float4* __restrict__ setup, ushort4* __restrict__ bbox,
                 uint32_t* __restrict__ counts) {
  __shared__ RastJob sJ;
  const int jid = blockIdx.y;
  const int nf = __ldg(&B.jobs[jid].n_faces);
  if (static_cast<int64_t>(blockIdx.x) * kSetupThreads >= nf) return;
  load_job_to_shared(B.jobs + jid, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const int64_t f0 = static_cast<int64_t>(blockIdx.x) * kSetupThreads + threadIdx.x;
  if (f0 >= nf) return;
  const int64_t row = J.setup_begin + f0;
  const int64_t f = row - J.setup_begin;
  float4 c[3];
  face_clip(J, B.pools, f, c);
  float inv[9], det;
  int flags;
  setup_from_clip(c, inv, &det, &flags);
  float4* out = setup + row * 4;
  // the inverse is read only for candidates (raster) and for face 0 (the
  // chooser's fallback); the flags of every face are kept
  if ((flags & kCandidate) == kCandidate || f == 0) {
    out[0] = make_float4(inv[0], inv[1], inv[2], inv[3]);
    out[1] = make_float4(inv[4], inv[5], inv[6], inv[7]);
    out[2] = make_float4(inv[8], c[0].z, c[1].z, c[2].z);
  }
  out[3] = make_float4(det, __int_as_float(flags), 0.0f, 0.0f);
  int i0, i1, j0, j1;
  ushort4 bb = make_ushort4(1, 1, 0, 0);  // empty: lo > hi
  if ((flags & kCandidate) == kCandidate && coverage_bbox(inv, J, &i0, &i1, &j0, &j1)) {
    const int tx0 = i0 / G.tw, tx1 = i1 / G.tw, ty0 = j0 / G.th, ty1 = j1 / G.th;
    bb = make_ushort4(tx0, ty0, tx1, ty1);
    uint32_t* cnt = counts + static_cast<int64_t>(jid) * G.tiles_per_job;
    for (int ty = ty0; ty <= ty1; ++ty)
      for (int tx = tx0; tx <= tx1; ++tx) atomicAdd(cnt + ty * G.tiles_x + tx, 1u);
  }
  bbox[row] = bb;
}

// Block-local exclusive scan of counts -> offsets, block sums out.
__global__ void __launch_bounds__(256)
scan_local_kernel(const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                  uint32_t* __restrict__ block_sums, int64_t n) {
  __shared__ uint32_t s[256];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x * 4;
  uint32_t v[4], t = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = (base + k < n) ? counts[base + k] : 0u;
    t += v[k];
  }
  s[threadIdx.x] = t;
  __syncthreads();
  for (int off = 1; off < 256; off <<= 1) {
    const uint32_t add = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
    __syncthreads();
    s[threadIdx.x] += add;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - t;  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < n) offsets[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 255) block_sums[blockIdx.x] = s[255];
}

// Adds the prefix of all previous blocks; marks tiles whose bin does not fit
// into `capacity` entries (they are rasterised by a full scan instead).
__global__ void __launch_bounds__(256)
scan_apply_kernel(const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                  const uint32_t* __restrict__ block_sums, int64_t n, uint64_t capacity,
                  unsigned int* __restrict__ status) {
  __shared__ unsigned long long s_prefix;
  __shared__ unsigned long long s_part[256];
  unsigned long long part = 0;
  for (int b = threadIdx.x; b < static_cast<int>(blockIdx.x); b += 256) part += block_sums[b];
  s_part[threadIdx.x] = part;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) s_part[threadIdx.x] += s_part[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) s_prefix = s_part[0];
  __syncthreads();
  const unsigned long long prefix = s_prefix;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x * 4;
  const unsigned long long local_last = (n > 0 && base <= n - 1 && n - 1 < base + 4) ? offsets[n - 1] : 0ull;
  bool over = false;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int64_t i = base + k;
    if (i >= n) break;
    const unsigned long long o = prefix + offsets[i];
    const uint32_t c = counts[i];
    if (o + c > capacity || o >= kOverflow) {
      offsets[i] = kOverflow;
      over = over || c > 0;
    } else {
      offsets[i] = static_cast<uint32_t>(o);
    }
  }
  if (over) atomicOr(status, 1u);
  // total bin entries requested (before capacity), for rast_tiled_stats
  if (n > 0 && base <= n - 1 && n - 1 < base + 4) {
    const unsigned long long total = prefix + local_last + counts[n - 1];
    *reinterpret_cast<unsigned long long*>(status + 1) = total;
  }
}

__global__ void __launch_bounds__(kSetupThreads)
scatter_kernel(RastBatch B, Geometry G, const ushort4* __restrict__ bbox,
               const uint32_t* __restrict__ offsets, uint32_t* __restrict__ cursors,
               int32_t* __restrict__ bins) {
  const int jid = blockIdx.y;
  const int nf = __ldg(&B.jobs[jid].n_faces);
  const int64_t f0 = static_cast<int64_t>(blockIdx.x) * kSetupThreads + threadIdx.x;
  if (f0 >= nf) return;
  const int64_t row = __ldg(&B.jobs[jid].setup_begin) + f0;
  const ushort4 bb = bbox[row];
  if (bb.x > bb.z) return;
  const int32_t fid = static_cast<int32_t>(f0);
  const int64_t tb = static_cast<int64_t>(jid) * G.tiles_per_job;
  for (int ty = bb.y; ty <= bb.w; ++ty)
    for (int tx = bb.x; tx <= bb.z; ++tx) {
      const int64_t t = tb + ty * G.tiles_x + tx;
      const uint32_t o = offsets[t];
      if (o & kOverflow) continue;
      const uint32_t slot = atomicAdd(cursors + t, 1u);
      bins[static_cast<int64_t>(o) + slot] = fid;
    }
}

// Persistent warps: each takes one tile (of any job) at a time.  Lane l owns
// PPL pixels of the tile.  Bin entries are staged 32 at a time in the warp's
// slice of shared memory (one record per lane), then every lane tests its
// pixels against the 32 staged setups.  Tiles whose bin overflowed scan
// every primitive of the job instead.
template <int TW, int TH>
__global__ void __launch_bounds__(32 * kRasterWarps)
raster_kernel(RastBatch B, Geometry G, const float4* __restrict__ setup,
              const uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets,
              const int32_t* __restrict__ bins, int32_t* __restrict__ winner,
              unsigned int* __restrict__ work, int64_t n_tiles, unsigned char* __restrict__ visible) {
  constexpr int PPL = TW * TH / 32;
  __shared__ float4 s_rec[kRasterWarps][kStage][3];
  __shared__ int s_id[kRasterWarps][kStage];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4 (*rec)[3] = s_rec[warp];
  int* ids = s_id[warp];
  unsigned long long tie_count = 0;
  while (true) {
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(work, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= n_tiles) break;
    const int jid = static_cast<int>(t / G.tiles_per_job);
    const int local = static_cast<int>(t % G.tiles_per_job);
    const int tx = local % G.tiles_x, ty = local / G.tiles_x;
    const RastJob& J = B.jobs[jid];
    const int W = J.width, H = J.height;
    if (tx * TW >= W || ty * TH >= H) continue;
    const float sx = J.viewport[0], ox = J.viewport[3], sy = J.viewport[5], oy = J.viewport[7];
    const float vp22 = J.viewport[10], vp23 = J.viewport[11];
    // lane -> one column j of the tile (TH divides 32) and PPL rows i:
    // every pixel of a lane shares y, so y * inv[1][k] is computed once per
    // entry (the same rounded product each pixel would compute).
    constexpr int LPC = 32 / TH;
    const int pj = ty * TH + lane % TH;
    const float y = (static_cast<float>(pj) - oy) / sy;
    float x[PPL], best_z[PPL];
    unsigned long long best[PPL];
    uint32_t second[PPL];
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      x[q] = (static_cast<float>(tx * TW + q * LPC + lane / TH) - ox) / sx;
      best[q] = kEmptyKey;
      best_z[q] = 0.0f;
      second[q] = 0xffffffffu;
    }
    const float4* jrec = setup + J.setup_begin * 4;
    const uint32_t off = offsets[t];
    const bool overflow = (off & kOverflow) != 0;
    const int n = overflow ? J.n_faces : static_cast<int>(counts[t]);
    // entry `e` of the tile's list -> (record, id); ids of non-candidates
    // (only met on the full-scan path) are -1 and their records unused
    auto fetch = [&](int e, float4& r0, float4& r1, float4& r2, int& id) {
      const int fid = overflow ? e : __ldg(bins + static_cast<int64_t>(off) + e);
      const float4* r = jrec + static_cast<int64_t>(fid) * 4;
      id = fid;
      if (overflow && (__float_as_int(__ldg(r + 3).y) & kCandidate) != kCandidate) {
        id = -1;
        r0 = r1 = r2 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
      }
      r0 = __ldg(r);
      r1 = __ldg(r + 1);
      r2 = __ldg(r + 2);
    };
    float4 n0, n1, n2;
    int nid = -1;
    if (lane < n) fetch(lane, n0, n1, n2, nid);
    for (int base = 0; base < n; base += kStage) {
      const int m = min(kStage, n - base);
      if (lane < m) {
        rec[lane][0] = n0;
        rec[lane][1] = n1;
        rec[lane][2] = n2;
        ids[lane] = nid;
      }
      __syncwarp();
      // prefetch the next chunk while this one is tested
      if (base + kStage + lane < n) fetch(base + kStage + lane, n0, n1, n2, nid);
      for (int e = 0; e < m; ++e) {
        const float4 a = rec[e][0], b = rec[e][1], cz = rec[e][2];
        const float y0 = y * a.w, y1 = y * b.x, y2 = y * b.y;
#pragma unroll
        for (int q = 0; q < PPL; ++q) {
          const float c0 = (x[q] * a.x + y0) + b.z;
          const float c1 = (x[q] * a.y + y1) + b.w;
          const float c2 = (x[q] * a.z + y2) + cz.x;
          if (all_nonneg(c0, c1, c2)) {
            const int id = ids[e];
            if (id >= 0) {
              const float z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
              const unsigned long long key = pack_key(z, id);
              if (key < best[q]) {
                second[q] = min(second[q], static_cast<uint32_t>(best[q] >> 32));
                best[q] = key;
                best_z[q] = z;
              } else {
                second[q] = min(second[q], static_cast<uint32_t>(key >> 32));
              }
            }
          }
        }
      }
      __syncwarp();
    }
    const bool depth_only = J.shader == RAST_SHADER_DEPTH;
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int pi = tx * TW + q * LPC + lane / TH;
      if (pi < W && pj < H) {
        const uint32_t o1 = static_cast<uint32_t>(best[q] >> 32);
        const bool found = !(best[q] == kEmptyKey || o1 == kInfOrder);
        const int64_t pix = J.pixel_begin + static_cast<int64_t>(pi) * H + pj;
        if (is_near_tie(best[q], second[q])) ++tie_count;
        if (!depth_only) {
          const int32_t w = found ? static_cast<int32_t>(best[q] & 0xffffffffu) : -1;
          winner[pix] = w;
          // faces whose varyings the shade needs: winners, and face 0 for the
          // chooser's fallback
          if (visible && J.n_faces > 0) visible[J.setup_begin + (w < 0 ? 0 : w)] = 1;
          continue;
        }
        // DepthShader: the fragment keeps everything and writes the default
        // depth, so the pixel resolves here (same operations as
        // resolve_pixel): the winner's depth, or primitive 0's chooser fallback.
        bool keep = found;
        float z = best_z[q];
        int prim = found ? static_cast<int>(best[q] & 0xffffffffu) : 0;
        if (!found && J.n_faces > 0) {
          const float4 a = __ldg(jrec), b = __ldg(jrec + 1), cz = __ldg(jrec + 2), d = __ldg(jrec + 3);
          const float c0 = (x[q] * a.x + y * a.w) + b.z;
          const float c1 = (x[q] * a.y + y * b.x) + b.w;
          const float c2 = (x[q] * a.z + y * b.y) + cz.x;
          keep = (__float_as_int(d.y) & kKeep) && all_nonneg(c0, c1, c2);
          z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
        }
        PixelResult r;
        r.keep = keep;
        r.z = z;
        r.prim = keep ? prim : -1;
        r.colour[0] = r.colour[1] = r.colour[2] = 0.0f;
        store_pixel(J, B.pools, pix, r);
      }
    }
  }
  if (B.near_ties) {
    for (int o = 16; o > 0; o >>= 1) tie_count += __shfl_xor_sync(0xffffffffu, tie_count, o);
    if (lane == 0 && tie_count) atomicAdd(B.near_ties, tie_count);
  }
}

// Vertex varyings of the three corners of every face some pixel needs
// (marked by the raster kernel), stored per face: the shade then reads them
// instead of re-running the vertex shader per pixel.
// Grid: (ceil(max_faces / 128), n_jobs).
__global__ void __launch_bounds__(128)
face_varyings_kernel(RastBatch B, const unsigned char* __restrict__ visible, float* __restrict__ fvar,
                     int vstride) {
  const int jid = blockIdx.y;
  const RastJob& J = B.jobs[jid];
  const int64_t f0 = static_cast<int64_t>(blockIdx.x) * 128 + threadIdx.x;
  if (f0 >= __ldg(&J.n_faces)) return;
  const int64_t row = __ldg(&J.setup_begin) + f0;
  if (!visible[row]) return;
  if (J.shader == RAST_SHADER_DEPTH) return;
  const int32_t* face = B.pools.faces + (J.face_begin + f0) * 3;
  const int nv = varying_count(J.shader);
  float* out = fvar + row * 3 * vstride;
#pragma unroll 1
  for (int k = 0; k < 3; ++k) {
    float var[kMaxVarying], clip[4];
    vertex_shader<false>(J, B.pools, gather_clamp(__ldg(face + k), J.n_verts), clip, var);
    for (int q = 0; q < nv; ++q) out[k * vstride + q] = var[q];
  }
}

// Deferred shading: one thread per pixel of every job, reading the winner's
// corner varyings computed once per visible face.
// Grid: (ceil(max pixels per job / 256), n_jobs).
__global__ void __launch_bounds__(256)
tiled_shade_kernel(RastBatch B, const float4* __restrict__ setup, const int32_t* __restrict__ winner,
                   bool depth_resolved, const float* __restrict__ fvar, int vstride) {
  __shared__ RastJob sJ;
  const int jid = blockIdx.y;
  const int64_t npx = static_cast<int64_t>(__ldg(&B.jobs[jid].width)) * __ldg(&B.jobs[jid].height);
  if (static_cast<int64_t>(blockIdx.x) * 256 >= npx) return;
  if (depth_resolved && __ldg(&B.jobs[jid].shader) == RAST_SHADER_DEPTH) return;  // done by the raster kernel
  load_job_to_shared(B.jobs + jid, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const int64_t local0 = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  if (local0 >= npx) return;
  const int64_t pix = J.pixel_begin + local0;
  const int64_t local = pix - J.pixel_begin;
  const int i = static_cast<int>(local / J.height), j = static_cast<int>(local % J.height);
  PixelResult r;
  VaryingSource src{nullptr, vstride, 0, fvar, J.setup_begin};
  resolve_pixel(J, B.pools, setup + J.setup_begin * 4, i, j, winner[pix], src, &r);
  store_pixel(J, B.pools, pix, r);
}

// ------------------------------------------------------------------ layout

// Bin entries reserved when the caller does not choose: four tiles per face
// on average; tiles beyond the capacity fall back to a full scan (correct,
// slower), so this only trades memory for speed.
inline uint64_t default_bin_capacity(const RastBatch& b) {
  return std::max<uint64_t>(static_cast<uint64_t>(b.total_setup) * 4u, 1u << 16);
}

struct Layout {
  size_t setup_off, bbox_off, counts_off, offsets_off, cursors_off, bsums_off, bins_off, winner_off,
      vis_off, fvar_off, misc_off, total;
  int vstride;
  int64_t n_tiles, n_scan_blocks;
  uint64_t bin_capacity;
  Geometry G;
};

static Layout layout(const RastBatch& b, TileShape ts, uint64_t bin_capacity) {
  Layout L{};
  L.G.tw = ts.tw;
  L.G.th = ts.th;
  L.G.tiles_x = ceil_div(std::max(b.max_width, 1), ts.tw);
  L.G.tiles_y = ceil_div(std::max(b.max_height, 1), ts.th);
  L.G.tiles_per_job = L.G.tiles_x * L.G.tiles_y;
  L.n_tiles = static_cast<int64_t>(b.n_jobs) * L.G.tiles_per_job;
  L.n_scan_blocks = (L.n_tiles + kScanBlock - 1) / kScanBlock;
  L.bin_capacity = bin_capacity;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  L.setup_off = take(static_cast<size_t>(b.total_setup) * 64);
  L.bbox_off = take(static_cast<size_t>(b.total_setup) * sizeof(ushort4));
  L.counts_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.cursors_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.offsets_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.bsums_off = take(static_cast<size_t>(L.n_scan_blocks) * 4);
  L.bins_off = take(static_cast<size_t>(bin_capacity) * 4);
  L.winner_off = take(static_cast<size_t>(b.total_pixels) * 4);
  int vstride = 0;
  for (int sh = 0; sh < 7; ++sh)
    if (b.shader_mask & (1 << sh)) vstride = std::max(vstride, varying_count(sh));
  L.vstride = vstride;
  const bool shading = vstride > 0;
  L.vis_off = take(shading ? static_cast<size_t>(b.total_setup) : 0);
  L.fvar_off = take(shading ? static_cast<size_t>(b.total_setup) * 3 * vstride * sizeof(float) : 0);
  L.misc_off = take(256);
  L.total = off;
  return L;
}

static bool valid_shape(TileShape t) {
  return (t.tw == 8 && t.th == 8) || (t.tw == 16 && t.th == 16) || (t.tw == 32 && t.th == 8) ||
         (t.tw == 8 && t.th == 32) || (t.tw == 16 && t.th == 8);
}

static int render(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                  size_t workspace_bytes, void* stream, RastProfile* profile) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  const RastBatch& b = *batch;
  TileShape ts{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8};
  if (!valid_shape(ts)) return RAST_ERR_INVALID_ARGUMENT;
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : default_bin_capacity(b);
  const Layout L = layout(b, ts, cap);
  if (workspace_bytes < L.total) return RAST_ERR_WORKSPACE_TOO_SMALL;
  if (L.total > 0 && (workspace == nullptr || (reinterpret_cast<uintptr_t>(workspace) & 255)))
    return RAST_ERR_INVALID_ARGUMENT;
  if (b.max_width > 65535 * ts.tw || b.max_height > 65535 * ts.th) return RAST_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  float4* setup = reinterpret_cast<float4*>(ws + L.setup_off);
  ushort4* bbox = reinterpret_cast<ushort4*>(ws + L.bbox_off);
  uint32_t* counts = reinterpret_cast<uint32_t*>(ws + L.counts_off);
  uint32_t* cursors = reinterpret_cast<uint32_t*>(ws + L.cursors_off);
  uint32_t* offsets = reinterpret_cast<uint32_t*>(ws + L.offsets_off);
  uint32_t* bsums = reinterpret_cast<uint32_t*>(ws + L.bsums_off);
  int32_t* bins = reinterpret_cast<int32_t*>(ws + L.bins_off);
  int32_t* winner = reinterpret_cast<int32_t*>(ws + L.winner_off);
  unsigned int* misc = reinterpret_cast<unsigned int*>(ws + L.misc_off);  // [0] work, [1] status
  Profiler prof(profile, s);

  // counts and cursors are adjacent: one memset clears both, plus the counters
  if (cudaMemsetAsync(counts, 0, L.offsets_off - L.counts_off, s) != cudaSuccess) return RAST_ERR_CUDA;
  if (cudaMemsetAsync(misc, 0, 256, s) != cudaSuccess) return RAST_ERR_CUDA;
  unsigned char* vis = L.vstride > 0 ? reinterpret_cast<unsigned char*>(ws + L.vis_off) : nullptr;
  float* fvar = L.vstride > 0 ? reinterpret_cast<float*>(ws + L.fvar_off) : nullptr;
  if (vis && b.total_setup > 0 && cudaMemsetAsync(vis, 0, static_cast<size_t>(b.total_setup), s) != cudaSuccess)
    return RAST_ERR_CUDA;
  prof.mark("memset");
  if (b.total_setup > 0) {
    const dim3 grid(static_cast<unsigned>((b.max_faces + kSetupThreads - 1) / kSetupThreads),
                    static_cast<unsigned>(b.n_jobs));
    setup_bin_kernel<<<grid, kSetupThreads, 0, s>>>(b, L.G, setup, bbox, counts);
    prof.mark("setup_bin_kernel");
    scan_local_kernel<<<static_cast<unsigned>(L.n_scan_blocks), 256, 0, s>>>(counts, offsets, bsums, L.n_tiles);
    scan_apply_kernel<<<static_cast<unsigned>(L.n_scan_blocks), 256, 0, s>>>(counts, offsets, bsums, L.n_tiles,
                                                                              L.bin_capacity, misc + 1);
    prof.mark("scan_kernels");
    scatter_kernel<<<grid, kSetupThreads, 0, s>>>(b, L.G, bbox, offsets, cursors, bins);
    prof.mark("scatter_kernel");
  }
  if (b.total_pixels > 0) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (b.total_setup > 0) {
      const unsigned grid = static_cast<unsigned>(std::max(sms, 1) * 8);
      if (ts.tw == 8 && ts.th == 8)
        raster_kernel<8, 8><<<grid, 32 * kRasterWarps, 0, s>>>(b, L.G, setup, counts, offsets, bins, winner, misc, L.n_tiles, vis);
      else if (ts.tw == 16 && ts.th == 16)
        raster_kernel<16, 16><<<grid, 32 * kRasterWarps, 0, s>>>(b, L.G, setup, counts, offsets, bins, winner, misc, L.n_tiles, vis);
      else if (ts.tw == 32 && ts.th == 8)
        raster_kernel<32, 8><<<grid, 32 * kRasterWarps, 0, s>>>(b, L.G, setup, counts, offsets, bins, winner, misc, L.n_tiles, vis);
      else if (ts.tw == 8 && ts.th == 32)
        raster_kernel<8, 32><<<grid, 32 * kRasterWarps, 0, s>>>(b, L.G, setup, counts, offsets, bins, winner, misc, L.n_tiles, vis);
      else
        raster_kernel<16, 8><<<grid, 32 * kRasterWarps, 0, s>>>(b, L.G, setup, counts, offsets, bins, winner, misc, L.n_tiles, vis);
    } else {
      if (cudaMemsetAsync(winner, 0xff, static_cast<size_t>(b.total_pixels) * 4, s) != cudaSuccess)
        return RAST_ERR_CUDA;
    }
    prof.mark("raster_kernel");
    const int64_t max_px = static_cast<int64_t>(b.max_width) * b.max_height;
    const dim3 sgrid(static_cast<unsigned>((max_px + 255) / 256), static_cast<unsigned>(b.n_jobs));
    if (b.shader_mask != (1 << RAST_SHADER_DEPTH) || b.total_setup == 0) {
      const bool pre = fvar != nullptr && b.total_setup > 0;
      if (pre) {
        const dim3 fgrid(static_cast<unsigned>((b.max_faces + 127) / 128), static_cast<unsigned>(b.n_jobs));
        face_varyings_kernel<<<fgrid, 128, 0, s>>>(b, vis, fvar, L.vstride);
        prof.mark("face_varyings_kernel");
      }
      tiled_shade_kernel<<<sgrid, 256, 0, s>>>(b, setup, winner, b.total_setup > 0, pre ? fvar : nullptr,
                                               L.vstride);
      prof.mark("tiled_shade_kernel");
    }
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return RAST_ERR_CUDA;
  return prof.finish();
}

}  // namespace tiled
}  // namespace rast

using namespace rast;

extern "C" size_t rast_tiled_workspace_bytes(const RastBatch* batch, const RastTiledConfig* cfg) {
  if (!batch) return 0;
  tiled::TileShape ts{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8};
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : tiled::default_bin_capacity(*batch);
  return tiled::layout(*batch, ts, cap).total;
}

extern "C" int rast_tiled_stats(const RastBatch* batch, const RastTiledConfig* cfg, const void* workspace,
                                void* stream, RastTiledStats* out) {
  if (!batch || !workspace || !out) return RAST_ERR_INVALID_ARGUMENT;
  tiled::TileShape ts{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8};
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : tiled::default_bin_capacity(*batch);
  const tiled::Layout L = tiled::layout(*batch, ts, cap);
  unsigned int misc[4] = {0, 0, 0, 0};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(misc, static_cast<const char*>(workspace) + L.misc_off, sizeof(misc),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return RAST_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return RAST_ERR_CUDA;
  out->bin_entries = static_cast<uint64_t>(misc[2]) | (static_cast<uint64_t>(misc[3]) << 32);
  out->overflow = misc[1];
  out->tiles = static_cast<uint64_t>(L.n_tiles);
  out->bin_capacity = L.bin_capacity;
  return RAST_OK;
}

extern "C" int rast_render_tiled(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  return tiled::render(batch, cfg, workspace, workspace_bytes, stream, nullptr);
}

extern "C" int rast_render_tiled_profiled(const RastBatch* batch, const RastTiledConfig* cfg,
                                          void* workspace, size_t workspace_bytes, void* stream,
                                          RastProfile* profile) {
  return tiled::render(batch, cfg, workspace, workspace_bytes, stream, profile);
}

// ------------------------------------------------ allocation-free variant

namespace {

// Workspace of rast_render_tiled_static: one per GPU that loads the library,
// held until process exit.
static __device__ __align__(256) unsigned char g_static_scratch[RAST_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
void* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (host code sees
// only a host-side stand-in for the symbol).  Looked up once per device.
int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RAST_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return RAST_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return RAST_ERR_CUDA;
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return RAST_OK;
}

}  // namespace

extern "C" int rast_render_tiled_static(const RastBatch* batch, const RastTiledConfig* cfg, void* stream) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  const size_t need = rast_tiled_workspace_bytes(batch, cfg);
  if (need > RAST_STATIC_SCRATCH_BYTES) return RAST_ERR_STATIC_SCRATCH_TOO_SMALL;
  void* scratch = nullptr;
  st = static_scratch(&scratch);
  if (st != RAST_OK) return st;
  return tiled::render(batch, cfg, scratch, RAST_STATIC_SCRATCH_BYTES, stream, nullptr);
}
