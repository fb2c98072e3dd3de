// rast_tiled.cu -- tiled, binned form of the rasteriser for many scenes per
// call.  Same results as the plain form (and the reference): every
// (pixel, candidate primitive) pair whose FP32 edge functions are all >= 0 is
// tested with the same operations; binning only removes pairs that cannot
// pass.
//
//   job_tiles_kernel   per-job tile grid (fixed stride: tiles of the largest job)
//   setup_bin_kernel   one thread per face: clip positions, det/keep/inverse;
//                      then one thread per candidate (queued in shared memory):
//                      conservative tile range of its coverage region, bin counts
//   scan_local_kernel  \  exclusive prefix sum of bin counts -> bin offsets;
//   scan_apply_kernel  /  tiles whose bins exceed the capacity are marked
//   scatter_kernel     over the binned faces the set-up listed, one warp per 32:
//                      face id into every bin its rectangle overlaps
//   raster_kernel      persistent warps, one tile each: bin entries staged in
//                      shared memory, per-pixel packed (depth | id) minimum
//   tiled_shade_kernel one thread per pixel: deferred shading of the winner,
//                      vertex varyings recomputed for its three corners only
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rast_internal.cuh"

namespace rast {
namespace tiled {

constexpr int kSetupThreads = 128;    // faces per setup/scatter block (256: 1 % slower, 64: 7 %)
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

// Sutherland-Hodgman clipping in its re-entrant (streaming) form: the
// rectangle's corners pass through three clip stages one at a time and the
// survivors update a bounding box, so no polygon array is kept.  For an edge
// S -> E a stage passes on the crossing point S + t (E - S),
// t = d_S / (d_S - d_E), when the edge crosses its line, then E when
// d_E >= 0; the closing edge (last -> first) is passed at the end.
// Crossing parameter t = d0 / (d0 - d1) of an edge whose ends lie on
// opposite sides (so d0 - d1 != 0).  The fast quotient (2 ulp) moves the
// crossing point by far less than the pixel the box is widened by; outside
// the range where it is accurate the IEEE quotient is used.
__device__ __forceinline__ float clip_t(float d0, float d1) {
  const float den = d0 - d1;
  const float a = fabsf(den);
  return (a > 1e-30f && a < 1e30f) ? __fdividef(d0, den) : d0 / den;
}

struct ClipBox {
  float mnx, mxx, mny, mxy;
  int n;
};

struct ClipStage {
  float a, b, c;                 // the half-plane a x + b y + c >= 0
  float fx, fy, fd, sx, sy, sd;  // first and previous vertex, with their values
  bool any;
};

__device__ __forceinline__ void clip_sink(ClipBox& box, float x, float y) {
  box.mnx = fminf(box.mnx, x);
  box.mxx = fmaxf(box.mxx, x);
  box.mny = fminf(box.mny, y);
  box.mxy = fmaxf(box.mxy, y);
  ++box.n;
}

__device__ __forceinline__ void clip_push2(ClipStage& s, ClipBox& box, float x, float y) {
  const float d = s.a * x + s.b * y + s.c;
  if (s.any) {
    if ((s.sd >= 0.0f) != (d >= 0.0f)) {
      const float t = clip_t(s.sd, d);
      clip_sink(box, s.sx + t * (x - s.sx), s.sy + t * (y - s.sy));
    }
    if (d >= 0.0f) clip_sink(box, x, y);
  } else {
    s.fx = x, s.fy = y, s.fd = d, s.any = true;
  }
  s.sx = x, s.sy = y, s.sd = d;
}

__device__ __forceinline__ void clip_push1(ClipStage& s, ClipStage& s2, ClipBox& box, float x, float y) {
  const float d = s.a * x + s.b * y + s.c;
  if (s.any) {
    if ((s.sd >= 0.0f) != (d >= 0.0f)) {
      const float t = clip_t(s.sd, d);
      clip_push2(s2, box, s.sx + t * (x - s.sx), s.sy + t * (y - s.sy));
    }
    if (d >= 0.0f) clip_push2(s2, box, x, y);
  } else {
    s.fx = x, s.fy = y, s.fd = d, s.any = true;
  }
  s.sx = x, s.sy = y, s.sd = d;
}

__device__ __forceinline__ void clip_push0(ClipStage& s, ClipStage& s1, ClipStage& s2, ClipBox& box, float x,
                                           float y) {
  const float d = s.a * x + s.b * y + s.c;
  if (s.any) {
    if ((s.sd >= 0.0f) != (d >= 0.0f)) {
      const float t = clip_t(s.sd, d);
      clip_push1(s1, s2, box, s.sx + t * (x - s.sx), s.sy + t * (y - s.sy));
    }
    if (d >= 0.0f) clip_push1(s1, s2, box, x, y);
  } else {
    s.fx = x, s.fy = y, s.fd = d, s.any = true;
  }
  s.sx = x, s.sy = y, s.sd = d;
}

// Pixel range [i0, i1] x [j0, j1] that contains every pixel whose FP32 edge
// functions c_k = (x * inv[k] + y * inv[3 + k]) + inv[6 + k] can all be
// >= 0.  Computed by clipping the job's screen rectangle (one pixel wider on
// every side, in NDC) against c_k >= -eps_k, where eps_k is 64x the rounding
// bound of the three-operation evaluation of c_k, then widening the bounding
// box by one pixel.  When those three half-planes bound a triangle whose
// corners are known to a quarter pixel, the clipping is skipped: the
// corners' box, clamped to the screen, contains the clipped box (equals it
// for a triangle inside the rectangle), and half a pixel of margin covers
// the corners' error and the rounding of the pixel <-> NDC maps.  Returns
// false when no pixel can be covered.
// The job's screen rectangle one pixel wider on every side, in NDC (pixels
// -1 and W), computed once per block.
struct ScreenRect {
  float xl, xh, yl, yh, X, Y;
  bool ok;  // finite, non-degenerate viewport
};

__device__ __forceinline__ ScreenRect screen_rect(const RastJob& J) {
  ScreenRect r{};
  const float sx = J.viewport[0], ox = J.viewport[3];
  const float sy = J.viewport[5], oy = J.viewport[7];
  r.ok = (sx != 0.0f) && (sy != 0.0f) && isfinite(sx) && isfinite(sy);
  const float xa = (-1.0f - ox) / sx, xb = (static_cast<float>(J.width) - ox) / sx;
  const float ya = (-1.0f - oy) / sy, yb = (static_cast<float>(J.height) - oy) / sy;
  r.xl = fminf(xa, xb);
  r.xh = fmaxf(xa, xb);
  r.yl = fminf(ya, yb);
  r.yh = fmaxf(ya, yb);
  r.X = fmaxf(fabsf(r.xl), fabsf(r.xh));
  r.Y = fmaxf(fabsf(r.yl), fabsf(r.yh));
  return r;
}

// Corner of the widened half-planes i and j: the solution of
// a_i x + b_i y + c_i = 0 = a_j x + b_j y + c_j by Cramer's rule, with a
// bound on its rounding error: N and D each carry at most 2u times the sum
// of their products' magnitudes, the quotient 2u relative (u = 2^-24); the
// bound below doubles both.  False when the corner's error could exceed a
// quarter pixel (scales psx, psy: pixels per NDC unit) or D's sign is not
// certain.  *d returns D = cross((a_i, b_i), (a_j, b_j)).
__device__ __forceinline__ bool widened_corner(float ai, float bi, float ci, float aj, float bj, float cj, float psx,
                                               float psy, float* x, float* y, float* d) {
  constexpr float u4 = 4.0f * 5.9604645e-08f;
  const float D = ai * bj - aj * bi;
  const float eD = fabsf(ai * bj) + fabsf(aj * bi);
  const float r = 1.0f / D;
  *x = (bi * cj - bj * ci) * r;
  *y = (aj * ci - ai * cj) * r;
  *d = D;
  const float ex = u4 * ((fabsf(bi * cj) + fabsf(bj * ci) + fabsf(*x) * eD) * fabsf(r) + fabsf(*x));
  const float ey = u4 * ((fabsf(aj * ci) + fabsf(ai * cj) + fabsf(*y) * eD) * fabsf(r) + fabsf(*y));
  // written so that NaN or inf anywhere fails
  return fabsf(D) > 2.0f * u4 * eD && ex * psx < 0.25f && ey * psy < 0.25f;
}

// The region where all three widened edge functions are >= 0 is a bounded
// triangle (or empty) when the edge normals (a_k, b_k) wind around the
// origin: D01, D12, D20 of one strict sign.  Then it is the convex hull of
// the three corners (tx, ty), each within a quarter pixel.
__device__ __forceinline__ bool widened_triangle(float a0, float b0, float c0, float a1, float b1, float c1, float a2,
                                                 float b2, float c2, float psx, float psy, float* tx, float* ty) {
  float d01, d12, d20;
  const bool ok = widened_corner(a0, b0, c0, a1, b1, c1, psx, psy, tx + 0, ty + 0, &d01) &
                  widened_corner(a1, b1, c1, a2, b2, c2, psx, psy, tx + 1, ty + 1, &d12) &
                  widened_corner(a2, b2, c2, a0, b0, c0, psx, psy, tx + 2, ty + 2, &d20);
  return ok && ((d01 > 0.0f && d12 > 0.0f && d20 > 0.0f) || (d01 < 0.0f && d12 < 0.0f && d20 < 0.0f));
}

__device__ __forceinline__ bool coverage_bbox(const float* inv, const RastJob& J, const ScreenRect& R, int* i0,
                                              int* i1, int* j0, int* j1) {
  const int W = J.width, H = J.height;
  const float sx = J.viewport[0], ox = J.viewport[3];
  const float sy = J.viewport[5], oy = J.viewport[7];
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 9; ++k) finite = finite && isfinite(inv[k]);
  if (!finite || !R.ok) {
    *i0 = 0;
    *i1 = W - 1;
    *j0 = 0;
    *j1 = H - 1;
    return true;  // cannot bound: every pixel of the job
  }
  const float xl = R.xl, xh = R.xh, yl = R.yl, yh = R.yh, X = R.X, Y = R.Y;
  // edge k: a_k x + b_k y + (c_k + eps_k), kept in scalars (no arrays: the
  // clip stages below capture them)
  bool small = true;  // |c_k| < 1e37 on the rectangle: no overflow below
  auto widened = [&](float a, float b, float c) {
    const float bound = X * fabsf(a) + Y * fabsf(b) + fabsf(c);
    small = small && bound < 1e37f;
    return c + 64.0f * 5.9604645e-08f * bound;
  };
  const float a0 = inv[0], b0 = inv[3], c0 = widened(inv[0], inv[3], inv[6]);
  const float a1 = inv[1], b1 = inv[4], c1 = widened(inv[1], inv[4], inv[7]);
  const float a2 = inv[2], b2 = inv[5], c2 = widened(inv[2], inv[5], inv[8]);
  if (!small) {
    *i0 = 0;
    *i1 = W - 1;
    *j0 = 0;
    *j1 = H - 1;
    return true;  // edge functions too large to evaluate safely: every pixel
  }
  float mnx, mxx, mny, mxy;
  float tx[3], ty[3];
  const float psx = fabsf(sx), psy = fabsf(sy);
  bool tight = false;  // the box is the widened triangle's (corners known to a quarter pixel)
  if (widened_triangle(a0, b0, c0, a1, b1, c1, a2, b2, c2, psx, psy, tx, ty)) {
    // the region lies in the triangle tx, ty: its corners' box (clamped to
    // the screen below) contains the clipped box, and equals it when the
    // triangle is inside the rectangle
    mnx = fminf(tx[0], fminf(tx[1], tx[2]));
    mxx = fmaxf(tx[0], fmaxf(tx[1], tx[2]));
    mny = fminf(ty[0], fminf(ty[1], ty[2]));
    mxy = fmaxf(ty[0], fmaxf(ty[1], ty[2]));
    tight = true;
  } else {
    ClipStage s0{a0, b0, c0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, false};
    ClipStage s1{a1, b1, c1, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, false};
    ClipStage s2{a2, b2, c2, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, false};
    ClipBox box{kInf, -kInf, kInf, -kInf, 0};
#pragma unroll 1
    for (int k = 0; k < 4; ++k) clip_push0(s0, s1, s2, box, (k == 1 || k == 2) ? xh : xl, k >= 2 ? yh : yl);
    // closing edges, stage by stage: re-sending a stage's first vertex closes it
    clip_push0(s0, s1, s2, box, s0.fx, s0.fy);
    if (s1.any) clip_push1(s1, s2, box, s1.fx, s1.fy);
    if (s2.any) clip_push2(s2, box, s2.fx, s2.fy);
    if (box.n == 0) return false;
    mnx = box.mnx, mxx = box.mxx, mny = box.mny, mxy = box.mxy;
  }
  // NDC -> pixel index: i = x * sx + ox (monotone in x with the sign of sx)
  const float pa = mnx * sx + ox, pb = mxx * sx + ox;
  const float qa = mny * sy + oy, qb = mxy * sy + oy;
  float ilo, ihi, jlo, jhi;
  if (tight) {
    // Corners within a quarter pixel: a pixel i whose rounded NDC x lies in
    // the region has i >= min(pa, pb) - 1/4 - e, e the rounding of pa
    // (2u |pa|) and of the pixel's quotient (2u |i - ox| pixels), both below
    // 1/8 pixel for |pa| < 2^20 (beyond that the clamp below decides), so
    // i >= ceil(min - 1/2); likewise i <= floor(max + 1/2).
    ilo = ceilf(fminf(pa, pb) - 0.5f);
    ihi = floorf(fmaxf(pa, pb) + 0.5f);
    jlo = ceilf(fminf(qa, qb) - 0.5f);
    jhi = floorf(fmaxf(qa, qb) + 0.5f);
  } else {
    // the clipped polygon's corners come from fast quotients: one pixel of
    // margin on each side
    ilo = floorf(fminf(pa, pb)) - 1.0f;
    ihi = ceilf(fmaxf(pa, pb)) + 1.0f;
    jlo = floorf(fminf(qa, qb)) - 1.0f;
    jhi = ceilf(fmaxf(qa, qb)) + 1.0f;
  }
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
  int tw, th;       // bin tile shape (powers of two)
  int tws, ths;     // log2 of tw, th: pixel index -> tile index by shifting
  int tiles_x;      // tiles along x of the largest job (stride)
  int tiles_y;
  int tiles_per_job;
  // ceil(2^64 / d) for d = tiles_per_job and tiles_x (0 for d = 1): the
  // raster kernel's per-tile quotients as one high multiply (fast_div)
  unsigned long long tpj_inv, tx_inv;
};

// n / d for n < 2^32 from inv = ceil(2^64 / d): floor(n inv / 2^64) = n / d
// + n e / 2^64 with 0 <= e < 1 floors to floor(n / d), since the fraction of
// n / d is at most 1 - 1/d and n e / 2^64 < 2^-32 <= 1/d.  inv = 0 marks d = 1.
__host__ __device__ inline unsigned long long div_inverse(unsigned d) { return d <= 1u ? 0ull : ~0ull / d + 1ull; }
__device__ __forceinline__ unsigned fast_div(unsigned n, unsigned long long inv) {
  return inv == 0ull ? n : static_cast<unsigned>(__umul64hi(static_cast<unsigned long long>(n), inv));
}

// Per-face coverage rectangle in pixels, [x, z] x [y, w] (ushort4: i0, j0,
// i1, j1); empty (x > z) for faces that are not binned.
constexpr unsigned short kNoRect = 0xffff;
__device__ __forceinline__ ushort4 empty_rect() { return make_ushort4(kNoRect, kNoRect, 0, 0); }

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

// Visits every (lane, tile) pair of the tile rectangles the 32 lanes of a
// warp hold ([tx0, tx1] x [ty0, ty1], empty when tx0 > tx1), 32 pairs per
// round spread over all lanes, so one large face does not serialise on one
// thread.  fn(owner lane, tile index within the job, valid) runs on every
// lane each round; valid is false past the last pair.  All 32 lanes must call.
template <class Fn>
__device__ __forceinline__ void warp_tiles(int tx0, int ty0, int tx1, int ty1, int tiles_x, Fn&& fn) {
  const int lane = threadIdx.x & 31;
  const int w = tx1 - tx0 + 1;
  const int n = (tx0 <= tx1 && ty0 <= ty1) ? w * (ty1 - ty0 + 1) : 0;
  int incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  const int excl = incl - n;
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  for (int base = 0; base < total; base += 32) {
    const int k = base + lane;
    int owner = 0;  // lanes whose pairs all precede pair k
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int v = __shfl_sync(0xffffffffu, incl, owner + step - 1);
      if (v <= k) owner += step;
    }
    const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
    const int o_tx0 = __shfl_sync(0xffffffffu, tx0, owner);
    const int o_ty0 = __shfl_sync(0xffffffffu, ty0, owner);
    const int o_w = __shfl_sync(0xffffffffu, w, owner);
    const bool valid = k < total;
    int tile = 0;
    if (valid) {
      const int local = k - o_excl;
      const int r = local / o_w;
      tile = (o_ty0 + r) * tiles_x + o_tx0 + (local - r * o_w);
    }
    fn(owner, tile, valid);
  }
}

// Phase 1, one thread per face: clip positions, determinant and keep/front
// flags (written for every face).  Candidates (kept, front-facing) and face
// 0 (the chooser's fallback, whose record is read even when it is not a
// candidate) are queued in shared memory with their [x, y, w] clip rows and
// depths.  Phase 2, one thread per queued face, so culled faces leave no idle
// lanes: the LU inverse -> setup record, and for candidates a conservative
// coverage rectangle.  Rectangles of at most kSmallArea pixels (when near
// ties are not counted) go to a second queue; the others are binned: the
// warp adds their tile counts with one atomic per distinct tile per round
// (lanes hitting the same tile merged with __match_any_sync).  Phase 3, one
// warp per queued small face, one lane per pixel of its rectangle: the
// raster kernel's edge tests and depth, folded into the per-pixel minimum of
// the packed (depth | id) keys with a 64-bit atomicMin.
// Grid: one block per kSetupThreads faces of a job (face block map).
constexpr int kRecordOnly = static_cast<int>(0x80000000u);  // queued for its record, not binned
constexpr int kSmallArea = 32;                               // largest small rectangle: one pixel per lane
constexpr int kTableMax = 1024;                              // pixel -> NDC tables kept in shared memory

// 1,536 resident threads per SM without the small path (40 registers): the
// kernel is latency-bound, and more resident warps beat the spills (0.83 /
// 0.90 ms -> 0.73 / 0.76 ms per pass on the 4096-scene brax-like batch at 6
// blocks of 256; 1,280 and 2,048 threads measured slower; 12 blocks of 128,
// 0.71 / 0.74 ms).  The small path's shared arrays allow fewer.
__host__ __device__ constexpr int setup_min_blocks(bool small) { return small ? 0 : 1536 / kSetupThreads; }

template <bool kSmall>
__global__ void __launch_bounds__(kSetupThreads, setup_min_blocks(kSmall))
setup_bin_kernel(RastBatch B, Geometry G, const int2* __restrict__ fmap, float4* __restrict__ setup,
                 ushort4* __restrict__ bbox, uint32_t* __restrict__ counts, unsigned long long* __restrict__ keys,
                 int small_area, int4* __restrict__ binned, unsigned int* __restrict__ n_binned) {
  __shared__ RastJob sJ;
  __shared__ float s_m[12][kSetupThreads];
  __shared__ int s_face[kSetupThreads];
  constexpr int kQ = kSmall ? kSetupThreads : 1;  // small-path arrays only where used
  constexpr int kT = kSmall ? kTableMax : 1;
  __shared__ float s_small[12][kQ];  // inverse (9) and clip depths (3) of small faces
  __shared__ int s_sface[kQ];
  __shared__ int s_srect[kQ][2];     // i0 | i1 << 16, j0 | j1 << 16
  __shared__ float s_xs[kT], s_ys[kT];
  __shared__ int s_qn, s_sn;
  __shared__ ScreenRect s_rect;
  const int2 blk = fmap[blockIdx.x];
  if (blk.x < 0) return;
  const int jid = blk.x;
  const int nf = __ldg(&B.jobs[jid].n_faces);
  load_job_to_shared(B.jobs + jid, &sJ);
  if (threadIdx.x == 0) s_qn = s_sn = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const float sx = J.viewport[0], ox = J.viewport[3], sy = J.viewport[5], oy = J.viewport[7];
  const bool tables = kSmall && J.width <= kTableMax && J.height <= kTableMax;
  if (tables) {  // the same quotients the raster kernel computes per pixel
    for (int i = threadIdx.x; i < J.width; i += kSetupThreads) s_xs[i] = (static_cast<float>(i) - ox) / sx;
    for (int j = threadIdx.x; j < J.height; j += kSetupThreads) s_ys[j] = (static_cast<float>(j) - oy) / sy;
  }
  if (threadIdx.x == 0) s_rect = screen_rect(J);  // read after the queue's barrier
  const int f = blk.y + static_cast<int>(threadIdx.x);
  bool queued = false, cand = false;
  float m[12];
  if (f < nf) {
    const int64_t row = J.setup_begin + f;
    float4 c[3];
    face_clip(J, B.pools, f, c);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      m[3 * k + 0] = c[k].x;
      m[3 * k + 1] = c[k].y;
      m[3 * k + 2] = c[k].w;
      m[9 + k] = c[k].z;
    }
    const float det = det3(m);
    int flags = 0;
    if (fabsf(det) > 1e-6f) flags |= kKeep;
    if (det >= 0.0f) flags |= kFront;
    setup[row * 4 + 3] = make_float4(det, __int_as_float(flags), 0.0f, 0.0f);
    cand = (flags & kCandidate) == kCandidate;
    queued = cand || f == 0;
    if (!cand) bbox[row] = empty_rect();
  }
  const unsigned qm = __ballot_sync(0xffffffffu, queued);
  int base = 0;
  if ((threadIdx.x & 31) == 0 && qm) base = atomicAdd(&s_qn, __popc(qm));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (queued) {
    const int q = base + __popc(qm & lanemask_lt());
    s_face[q] = cand ? f : (f | kRecordOnly);
#pragma unroll
    for (int k = 0; k < 12; ++k) s_m[k][q] = m[k];
  }
  __syncthreads();
  const int qn = s_qn;
  const int q = threadIdx.x;
  if (static_cast<int>(threadIdx.x & ~31u) < qn) {  // warps holding queued faces
    int tx0 = 1, ty0 = 1, tx1 = 0, ty1 = 0;
    bool small = false;
    int fq = 0, i0 = 0, i1 = 0, j0 = 0, j1 = 0;
    float iv[9];
    if (q < qn) {
      const int entry = s_face[q];
      fq = entry & ~kRecordOnly;
      float mq[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) mq[k] = s_m[k][q];
      inv3(mq, iv);
      float4* out = setup + (J.setup_begin + fq) * 4;
      out[0] = make_float4(iv[0], iv[1], iv[2], iv[3]);
      out[1] = make_float4(iv[4], iv[5], iv[6], iv[7]);
      out[2] = make_float4(iv[8], s_m[9][q], s_m[10][q], s_m[11][q]);
      if (!(entry & kRecordOnly)) {
        ushort4 bb = empty_rect();
        if (coverage_bbox(iv, J, s_rect, &i0, &i1, &j0, &j1)) {
          if (kSmall && (i1 - i0 + 1) * (j1 - j0 + 1) <= small_area) {
            small = true;  // rasterised in phase 3, not binned
          } else {
            tx0 = i0 >> G.tws;
            tx1 = i1 >> G.tws;
            ty0 = j0 >> G.ths;
            ty1 = j1 >> G.ths;
            bb = make_ushort4(i0, j0, i1, j1);  // the raster kernel tests only these pixels of each tile
          }
        }
        bbox[J.setup_begin + fq] = bb;
      }
    }
    const unsigned sm = kSmall ? __ballot_sync(0xffffffffu, small) : 0u;
    int sbase = 0;
    if ((threadIdx.x & 31) == 0 && sm) sbase = atomicAdd(&s_sn, __popc(sm));
    if (kSmall) sbase = __shfl_sync(0xffffffffu, sbase, 0);
    if (kSmall && small) {
      const int e = sbase + __popc(sm & lanemask_lt());
      s_sface[e] = fq;
#pragma unroll
      for (int k = 0; k < 9; ++k) s_small[k][e] = iv[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) s_small[9 + k][e] = s_m[9 + k][q];
      s_srect[e][0] = i0 | (i1 << 16);
      s_srect[e][1] = j0 | (j1 << 16);
    }
    // binned faces (those with tiles) join the scatter's list: one atomic per warp
    const bool bin = tx0 <= tx1 && ty0 <= ty1;
    const unsigned bm = __ballot_sync(0xffffffffu, bin);
    unsigned bbase = 0;
    if ((threadIdx.x & 31) == 0 && bm) bbase = atomicAdd(n_binned, static_cast<unsigned>(__popc(bm)));
    bbase = __shfl_sync(0xffffffffu, bbase, 0);
    if (bin)
      binned[bbase + __popc(bm & lanemask_lt())] =
          make_int4(jid, fq, static_cast<int>(static_cast<unsigned>(i0) | (static_cast<unsigned>(j0) << 16)),
                    static_cast<int>(static_cast<unsigned>(i1) | (static_cast<unsigned>(j1) << 16)));
    uint32_t* cnt = counts + static_cast<int64_t>(jid) * G.tiles_per_job;
    warp_tiles(tx0, ty0, tx1, ty1, G.tiles_x, [&](int, int tile, bool valid) {
      const unsigned peers = __match_any_sync(0xffffffffu, valid ? tile : -1);
      if (valid && __popc(peers & lanemask_lt()) == 0) atomicAdd(cnt + tile, static_cast<unsigned>(__popc(peers)));
    });
  }
  if (!kSmall) return;  // no small path: nothing below (no barrier follows)
  __syncthreads();
  const int sn = s_sn;
  const int lane = threadIdx.x & 31;
  const float vp22 = J.viewport[10], vp23 = J.viewport[11];
  for (int e = threadIdx.x >> 5; e < sn; e += kSetupThreads / 32) {
    const int ri = s_srect[e][0], rj = s_srect[e][1];
    const int a0 = ri & 0xffff, b0 = rj & 0xffff;
    const int bw = (ri >> 16) - a0 + 1, bh = (rj >> 16) - b0 + 1;
    if (lane >= bw * bh) continue;
    const int i = a0 + lane % bw, j = b0 + lane / bw;
    const float x = tables ? s_xs[i] : (static_cast<float>(i) - ox) / sx;
    const float y = tables ? s_ys[j] : (static_cast<float>(j) - oy) / sy;
    const float c0 = (x * s_small[0][e] + y * s_small[3][e]) + s_small[6][e];
    const float c1 = (x * s_small[1][e] + y * s_small[4][e]) + s_small[7][e];
    const float c2 = (x * s_small[2][e] + y * s_small[5][e]) + s_small[8][e];
    if (all_nonneg(c0, c1, c2)) {
      const float z = ((c0 * s_small[9][e] + c1 * s_small[10][e]) + c2 * s_small[11][e]) * vp22 + vp23;
      atomicMin(keys + J.pixel_begin + static_cast<int64_t>(i) * J.height + j, pack_key(z, s_sface[e]));
    }
  }
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

// Face ids into the bins of the tiles their rectangles cover, over the list
// of binned faces the set-up kernel appended (job, face, pixel rectangle):
// faces without tiles cost nothing here.  Each warp takes up to 32 listed
// faces, fewer when the list is short (so that every warp of the grid has
// some: a warp's (face, tile) pairs are a chain of dependent loads and
// atomics, and a short list on few warps leaves the GPU waiting on them),
// with the pairs spread over its lanes; lanes writing to the same tile take
// their slots with one atomic (__match_any_sync).  Grid: any number of
// blocks of kSetupThreads threads, striding over the list.
__global__ void __launch_bounds__(kSetupThreads)
scatter_kernel(Geometry G, const int4* __restrict__ binned, const unsigned int* __restrict__ n_binned,
               const uint32_t* __restrict__ offsets, uint32_t* __restrict__ cursors, int32_t* __restrict__ bins) {
  const unsigned n = *n_binned;
  const int lane = threadIdx.x & 31;
  constexpr unsigned kWarps = kSetupThreads / 32;
  const unsigned warps = gridDim.x * kWarps, wid = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const unsigned per_warp = max(1u, min(32u, (n + warps - 1) / warps));  // listed faces per warp
  for (unsigned base = wid * per_warp; base < n; base += warps * per_warp) {
    const unsigned e = base + lane;
    int jid = 0, fq = 0, tx0 = 1, ty0 = 1, tx1 = 0, ty1 = 0;
    if (lane < static_cast<int>(per_warp) && e < n) {
      const int4 b = binned[e];
      const unsigned lo = static_cast<unsigned>(b.z), hi = static_cast<unsigned>(b.w);
      jid = b.x;
      fq = b.y;
      tx0 = static_cast<int>((lo & 0xffffu) >> G.tws);
      ty0 = static_cast<int>((lo >> 16) >> G.ths);
      tx1 = static_cast<int>((hi & 0xffffu) >> G.tws);
      ty1 = static_cast<int>((hi >> 16) >> G.ths);
    }
    warp_tiles(tx0, ty0, tx1, ty1, G.tiles_x, [&](int owner, int tile, bool valid) {
      const int64_t gt = static_cast<int64_t>(__shfl_sync(0xffffffffu, jid, owner)) * G.tiles_per_job + tile;
      const uint32_t o = valid ? offsets[gt] : kOverflow;
      const bool write = !(o & kOverflow);
      const unsigned peers = __match_any_sync(0xffffffffu, write ? gt : -1ll);
      const int leader = __ffs(peers) - 1;
      uint32_t slot = 0;
      if (write && lane == leader) slot = atomicAdd(cursors + gt, static_cast<unsigned>(__popc(peers)));
      slot = __shfl_sync(0xffffffffu, slot, leader) + __popc(peers & lanemask_lt());
      const int fid = __shfl_sync(0xffffffffu, fq, owner);
      if (write) bins[static_cast<int64_t>(o) + slot] = fid;
    });
  }
}

// True when edge function (x ea + y eb) + ec is negative at every pixel of
// the tile [xa, xb] x [ya, yb] (NDC of its first and last pixel centres)
// whatever the rounding of the per-pixel evaluation: its maximum over the
// rectangle, max(xa ea, xb ea) + max(ya eb, yb eb) + ec, plus a margin of
// 16 u (X |ea| + Y |eb| + |ec|) (X, Y: the largest |x|, |y| of the tile;
// u = 2^-24; the per-pixel and the bound's own rounding are each below
// 3.1 u times that sum) is below zero.  NaN anywhere gives false.
__device__ __forceinline__ bool edge_misses_tile(float ea, float eb, float ec, float xa, float xb, float ya, float yb,
                                                 float X, float Y) {
  const float bound = (fmaxf(xa * ea, xb * ea) + fmaxf(ya * eb, yb * eb)) + ec;
  const float margin = 16.0f * 5.9604645e-08f * ((X * fabsf(ea) + Y * fabsf(eb)) + fabsf(ec)) + 1e-30f;
  return bound + margin < 0.0f;
}

// Persistent warps: each takes one tile (of any job) at a time.  Lane l owns
// PPL pixels of the tile.  Bin entries are staged 32 at a time in the warp's
// slice of shared memory (one record per lane), then tested against the
// tile's pixels.  Tiles whose bin overflowed scan every primitive of the job
// instead.  Each pixel keeps its kL smallest keys (kL = 1: the default
// chooser; kL = RAST_MAX_LAYERS for batches with layered jobs), slot s
// written to winner[s * total_pixels + pixel].
//
// Pair path (kL = 1 without near-tie counting): an entry's coverage
// rectangle (from the set-up) cut to the warp's pixels is usually a few
// pixels; entries of at most pair_max() such pixels are not tested against
// every pixel of the tile but as (entry, pixel) pairs spread over the lanes,
// 32 per round (a lane finds its entry by binary search over the warp's
// prefix sums), each folding its key into the pixel's minimum in shared
// memory with a 64-bit atomicMin.  Larger entries take the dense loop (each
// lane its own pixels, keys in registers).  The minimum of packed keys does
// not depend on the order, and both paths evaluate the same operations, so
// the results are those of the dense loop alone.
// Blocks per SM: the pair-path variants of at most 128 pixels take eight
// (64 registers; ten at 48 registers spilled in the pair loop: main 16x8
// 0.58 -> 0.64 ms on the 4096-scene brax-like batch).  The near-tie
// counting one-slot variants take ten (48 registers): more resident warps
// beat their few spills (16x8: 1.02 -> 0.88 ms, 8x8: 1.03 -> 1.01 ms before
// the pair path; 12 and 16 blocks measured slower).  The layered variants
// of at most 64 pixels take eight (64 registers: 1.32 -> 1.18 ms with 4
// layers).  The others keep the compiler's choice (0: no minimum).
template <int TW, int TH, int kL, bool kPairs>
__host__ __device__ constexpr int raster_min_blocks() {
  return kPairs ? (TW * TH <= 128 ? 8 : 0) : (kL == 1 && TW * TH <= 128) ? 10 : (TW * TH <= 64 ? 8 : 0);
}

// Largest (entry, pixel) pair count of an entry on the pair path: about
// where its pairs cost what the dense loop's pass over the warp's pixels does.
template <int TW, int TH>
__host__ __device__ constexpr int pair_max() {
  return TW * TH / 4 + 4;
}

// Inverse of depth_order where it is one to one: false for the keys of NaN
// and of +-0 (whose sign the order drops).
__device__ __forceinline__ bool depth_of_order(uint32_t o, float* z) {
  if (o == 0u || o == 0x80000000u) return false;
  *z = __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
  return true;
}

// kWPT warps per bin tile: the bin tile is TW x (kWPT TH) pixels and a
// work unit u is its rows [(u % kWPT) TH, (u % kWPT + 1) TH), so bins can be
// coarser than the sub-tile each warp rasterises (every warp of a tile
// reads the tile's whole bin and drops the entries that miss its rows).
template <int TW, int TH, bool kKeys, bool kTies, int kL, int kWPT>
__global__ void __launch_bounds__(32 * kRasterWarps, raster_min_blocks<TW, TH, kL, kL == 1 && !kTies>())
raster_kernel(RastBatch B, Geometry G, const float4* __restrict__ setup, const ushort4* __restrict__ rects,
              const uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets,
              const int32_t* __restrict__ bins, int32_t* __restrict__ winner,
              unsigned int* __restrict__ work, int64_t n_units, unsigned char* __restrict__ visible,
              const unsigned long long* __restrict__ keys) {
  constexpr int PPL = TW * TH / 32;
  constexpr bool kPairs = kL == 1 && !kTies;
  constexpr int kPW = kPairs ? kRasterWarps : 1;  // pair-path arrays only where used
  __shared__ float4 s_rec[kRasterWarps][kStage][3];
  __shared__ int s_id[kRasterWarps][kStage];
  __shared__ unsigned long long s_best[kPW][kPairs ? TW * TH : 1];  // pixel (li, lj) at li * TH + lj
  __shared__ float s_x[kPW][kPairs ? TW : 1], s_y[kPW][kPairs ? TH : 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4 (*rec)[3] = s_rec[warp];
  int* ids = s_id[warp];
  unsigned long long* sbest = s_best[kPairs ? warp : 0];
  float* tx_ndc = s_x[kPairs ? warp : 0];
  float* ty_ndc = s_y[kPairs ? warp : 0];
  unsigned long long tie_count = 0;
  unsigned long long tests = 0;  // pixel-triangle pairs this warp tested
  // The next tile is grabbed (one atomic on the shared counter) when this
  // tile's last chunk of bin entries is staged, so the atomic's latency
  // overlaps the end of this tile's tests while a warp never sits on an
  // unstarted tile for long (tiles stay balanced over the warps when each
  // warp gets only a few heavy ones); its bin offset and count are loaded
  // before this tile's epilogue.
  unsigned int next = 0;
  if (lane == 0) next = atomicAdd(work, 1u);
  bool grabbed = true;  // `next` holds a grabbed unit not yet started
  unsigned int unit = 0;
  uint32_t m_off = 0, m_cnt = 0;  // of `unit`
  auto grab = [&]() {
    if (!grabbed && lane == 0) next = atomicAdd(work, 1u);
    grabbed = true;
  };
  auto advance = [&]() {
    grab();
    unit = __shfl_sync(0xffffffffu, next, 0);
    grabbed = false;
    if (unit < n_units) {
      m_off = offsets[unit / kWPT];
      m_cnt = counts[unit / kWPT];
    }
  };
  advance();
  while (unit < n_units) {
    const unsigned int cur = unit;
    const uint32_t off = m_off, t_count = m_cnt;
    const unsigned int t = cur / kWPT;  // bin tile
    const unsigned jq = fast_div(t, G.tpj_inv);
    const int jid = static_cast<int>(jq);
    const int local = static_cast<int>(t - jq * static_cast<unsigned>(G.tiles_per_job));
    const int ty = static_cast<int>(fast_div(static_cast<unsigned>(local), G.tx_inv));
    const int tx = local - ty * G.tiles_x;
    const int y0 = ty * (TH * kWPT) + static_cast<int>(cur % kWPT) * TH;  // first row of this warp's part
    const int x0 = tx * TW;
    const RastJob& J = B.jobs[jid];
    const int W = J.width, H = J.height;
    if (x0 >= W || y0 >= H) {
      advance();
      continue;
    }
    const float4* jrec = setup + J.setup_begin * 4;
    const ushort4* jrect = rects + J.setup_begin;
    const bool overflow = (off & kOverflow) != 0;
    const int n = overflow ? J.n_faces : static_cast<int>(t_count);
    // entry `e` of the tile's list -> (record, id, rectangle); ids of
    // non-candidates (only met on the full-scan path) are -1 and their
    // records unused
    auto fetch = [&](int e, float4& r0, float4& r1, float4& r2, int& id, ushort4& rc) {
      const int fid = overflow ? e : __ldg(bins + static_cast<int64_t>(off) + e);
      const float4* r = jrec + static_cast<int64_t>(fid) * 4;
      id = fid;
      if (kPairs) rc = __ldg(jrect + fid);
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
    ushort4 nrc = empty_rect();
    if (lane < n) fetch(lane, n0, n1, n2, nid, nrc);  // first: its loads overlap the tile's set-up
    const float sx = J.viewport[0], ox = J.viewport[3], sy = J.viewport[5], oy = J.viewport[7];
    const float vp22 = J.viewport[10], vp23 = J.viewport[11];
    // lane -> one column j of the tile (TH divides 32) and PPL rows i:
    // every pixel of a lane shares y, so y * inv[1][k] is computed once per
    // entry (the same rounded product each pixel would compute).
    constexpr int LPC = 32 / TH;
    const int pj = y0 + lane % TH;
    float y;
    float x[PPL], best_z[PPL];
    if (kPairs) {
      // the pixels' NDC quotients, once per tile: tx_ndc[li] for pixel
      // x0 + li, ty_ndc[lj] for y0 + lj
      for (int k = lane; k < TW + TH; k += 32) {
        if (k < TW)
          tx_ndc[k] = (static_cast<float>(x0 + k) - ox) / sx;
        else
          ty_ndc[k - TW] = (static_cast<float>(y0 + k - TW) - oy) / sy;
      }
#pragma unroll
      for (int q = 0; q < PPL; ++q) sbest[q * 32 + lane] = kEmptyKey;
      __syncwarp();
      y = ty_ndc[lane % TH];
#pragma unroll
      for (int q = 0; q < PPL; ++q) x[q] = tx_ndc[q * LPC + lane / TH];
    } else {
      y = (static_cast<float>(pj) - oy) / sy;
#pragma unroll
      for (int q = 0; q < PPL; ++q) x[q] = (static_cast<float>(x0 + q * LPC + lane / TH) - ox) / sx;
    }
    // NDC of the tile's first and last pixel (inside the job) for the
    // per-entry rejection test: the same quotients the pixels compute
    const int lxe = min(TW - 1, W - 1 - x0), lye = min(TH - 1, H - 1 - y0);  // last pixel inside the job
    float xa, xb, ya, yb;
    if (kPairs) {
      xa = tx_ndc[0], xb = tx_ndc[lxe], ya = ty_ndc[0], yb = ty_ndc[lye];
    } else {
      xa = (static_cast<float>(x0) - ox) / sx;
      xb = (static_cast<float>(x0 + lxe) - ox) / sx;
      ya = (static_cast<float>(y0) - oy) / sy;
      yb = (static_cast<float>(y0 + lye) - oy) / sy;
    }
    const float XM = fmaxf(fabsf(xa), fabsf(xb)), YM = fmaxf(fabsf(ya), fabsf(yb));
    unsigned long long best[PPL][kL];
    uint32_t second[PPL];
    unsigned z_known = 0;  // bit q: best_z[q] holds the depth of best[q] (set by this kernel's tests)
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int pi = x0 + q * LPC + lane / TH;
      // the minimum over the faces the setup kernel rasterised itself
      best[q][0] = (kKeys && pi < W && pj < H) ? keys[J.pixel_begin + static_cast<int64_t>(pi) * H + pj] : kEmptyKey;
#pragma unroll
      for (int l = 1; l < kL; ++l) best[q][l] = kEmptyKey;
      best_z[q] = 0.0f;
      second[q] = 0xffffffffu;
    }
    for (int base = 0; base < n; base += kStage) {
      // entries whose triangle misses every pixel of the tile (one edge
      // negative over the whole tile) are dropped; the rest are staged
      // compacted
      bool take = lane < min(kStage, n - base) && nid >= 0;
      int cnt = 0, pinfo = 0;
      float prcp = 0.0f;
      if (kPairs) {
        // the entry's rectangle cut to the warp's pixels (tile-local); on
        // the full-scan path faces without one (small faces of the set-up's
        // own rasterisation, non-candidates) drop out here
        const int lx0 = max(static_cast<int>(nrc.x) - x0, 0), lx1 = min(static_cast<int>(nrc.z) - x0, lxe);
        const int ly0 = max(static_cast<int>(nrc.y) - y0, 0), ly1 = min(static_cast<int>(nrc.w) - y0, lye);
        take = take && lx0 <= lx1 && ly0 <= ly1;
        if (take) {
          const float ra = tx_ndc[lx0], rb = tx_ndc[lx1], sa = ty_ndc[ly0], sb = ty_ndc[ly1];
          const float RX = fmaxf(fabsf(ra), fabsf(rb)), RY = fmaxf(fabsf(sa), fabsf(sb));
          take = !(edge_misses_tile(n0.x, n0.w, n1.z, ra, rb, sa, sb, RX, RY) ||
                   edge_misses_tile(n0.y, n1.x, n1.w, ra, rb, sa, sb, RX, RY) ||
                   edge_misses_tile(n0.z, n1.y, n2.x, ra, rb, sa, sb, RX, RY));
          const int w = lx1 - lx0 + 1;
          cnt = w * (ly1 - ly0 + 1);
          pinfo = lx0 | (ly0 << 8) | (w << 16);
          prcp = __frcp_rn(static_cast<float>(w));
        }
      } else if (take) {
        take = !(edge_misses_tile(n0.x, n0.w, n1.z, xa, xb, ya, yb, XM, YM) ||
                 edge_misses_tile(n0.y, n1.x, n1.w, xa, xb, ya, yb, XM, YM) ||
                 edge_misses_tile(n0.z, n1.y, n2.x, xa, xb, ya, yb, XM, YM));
      }
      const bool pair = kPairs && take && cnt <= pair_max<TW, TH>();
      const bool dense = take && !pair;
      const unsigned keep = __ballot_sync(0xffffffffu, dense);
      const int m = __popc(keep);
      const unsigned pmask = kPairs ? __ballot_sync(0xffffffffu, pair) : 0u;
      if (dense || pair) {
        // dense entries in slots [0, m), pair entries after them, each in
        // lane order
        const int slot = dense ? __popc(keep & lanemask_lt()) : m + __popc(pmask & lanemask_lt());
        rec[slot][0] = n0;
        rec[slot][1] = n1;
        rec[slot][2] = n2;
        ids[slot] = nid;
      }
      // pair path: inclusive prefix sum of the pair counts in lane order
      int pincl = pair ? cnt : 0, ptotal = 0;
      if (kPairs) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, pincl, d);
          if (lane >= d) pincl += v;
        }
        ptotal = __shfl_sync(0xffffffffu, pincl, 31);
      }
      const int pexcl = pincl - (pair ? cnt : 0);
      __syncwarp();
      if (base + kStage >= n) grab();  // the last chunk: the next tile's atomic overlaps its tests
      // prefetch the next chunk while this one is tested
      if (base + kStage + lane < n) fetch(base + kStage + lane, n0, n1, n2, nid, nrc);
      tests += static_cast<unsigned>(m) * static_cast<unsigned>(TW * TH) + static_cast<unsigned>(ptotal);
      for (int e = 0; e < m; ++e) {
        const float4 a = rec[e][0], b = rec[e][1], cz = rec[e][2];
        const float y0p = y * a.w, y1p = y * b.x, y2p = y * b.y;
#pragma unroll
        for (int q = 0; q < PPL; ++q) {
          const float c0 = (x[q] * a.x + y0p) + b.z;
          const float c1 = (x[q] * a.y + y1p) + b.w;
          const float c2 = (x[q] * a.z + y2p) + cz.x;
          if (all_nonneg(c0, c1, c2)) {  // staged entries are candidates (id >= 0)
            const float z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
            const unsigned long long key = pack_key(z, ids[e]);
            if (key < best[q][0]) {
              if (kTies) second[q] = min(second[q], static_cast<uint32_t>(best[q][0] >> 32));
              best_z[q] = z;
              z_known |= 1u << q;
            } else if (kTies) {
              second[q] = min(second[q], static_cast<uint32_t>(key >> 32));
            }
            insert_key<kL>(best[q], key);
          }
        }
      }
      if (kPairs) {
        for (int pb = 0; pb < ptotal; pb += 32) {
          const int pk = pb + lane;
          int owner = 0;  // lanes whose pairs all precede pair pk
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const int v = __shfl_sync(0xffffffffu, pincl, owner + step - 1);
            if (v <= pk) owner += step;
          }
          const int o_excl = __shfl_sync(0xffffffffu, pexcl, owner);
          const int o_info = __shfl_sync(0xffffffffu, pinfo, owner);
          const float o_rcp = __shfl_sync(0xffffffffu, prcp, owner);
          if (pk < ptotal) {
            // pair -> pixel of the owner's rectangle, row-major over its
            // width w (w <= 32 and pk - o_excl < TW * TH: the rounded
            // quotient (k + 1/2) / w stays more than 1/64 from an integer)
            const int k = pk - o_excl;
            const int w = o_info >> 16;
            const int r = __float2int_rz((static_cast<float>(k) + 0.5f) * o_rcp);
            const int li = min((o_info & 0xff) + (k - r * w), TW - 1);
            const int lj = min(((o_info >> 8) & 0xff) + r, TH - 1);
            const int slot = m + __popc(pmask & ((1u << owner) - 1u));
            const float px = tx_ndc[li], py = ty_ndc[lj];
            const float4 a = rec[slot][0], b = rec[slot][1], cz = rec[slot][2];
            const float c0 = (px * a.x + py * a.w) + b.z;
            const float c1 = (px * a.y + py * b.x) + b.w;
            const float c2 = (px * a.z + py * b.y) + cz.x;
            if (all_nonneg(c0, c1, c2)) {
              const float z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
              atomicMin(sbest + li * TH + lj, pack_key(z, ids[slot]));
            }
          }
        }
      }
      __syncwarp();
    }
    advance();  // the next tile's offset and count loads overlap this one's epilogue
    if (kPairs) {
      // the pair path's minima join the lane's own (same pixel layout:
      // pixel q of lane l is li * TH + lj = 32 q + l)
#pragma unroll
      for (int q = 0; q < PPL; ++q) {
        const unsigned long long k = sbest[q * 32 + lane];
        if (k < best[q][0]) {
          best[q][0] = k;
          z_known &= ~(1u << q);
        }
      }
      __syncwarp();  // every lane has read its minima before the next tile's reset
    }
    const bool depth_only = J.shader == RAST_SHADER_DEPTH;
    const int layers = kL > 1 ? job_layers(J, B.max_layers) : 0;
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      const int pi = x0 + q * LPC + lane / TH;
      if (pi < W && pj < H) {
        const uint32_t o1 = static_cast<uint32_t>(best[q][0] >> 32);
        const bool found = !(best[q][0] == kEmptyKey || o1 == kInfOrder);
        const int64_t pix = J.pixel_begin + static_cast<int64_t>(pi) * H + pj;
        if (kTies && is_near_tie(best[q][0], second[q])) ++tie_count;
        if (!depth_only) {
          const int32_t w = found ? static_cast<int32_t>(best[q][0] & 0xffffffffu) : -1;
          winner[pix] = w;
          // faces whose varyings the shade needs: winners, and face 0 for the
          // default chooser's fallback
          if (visible && J.n_faces > 0 && (layers == 0 || w >= 0)) visible[J.setup_begin + (w < 0 ? 0 : w)] = 1;
#pragma unroll
          for (int l = 1; l < kL; ++l) {
            const uint32_t o = static_cast<uint32_t>(best[q][l] >> 32);
            const int32_t wl = (best[q][l] == kEmptyKey || o == kInfOrder) ? -1
                                                                          : static_cast<int32_t>(best[q][l] & 0xffffffffu);
            winner[l * B.total_pixels + pix] = wl;
            if (visible && wl >= 0 && l < layers) visible[J.setup_begin + wl] = 1;
          }
          continue;
        }
        // DepthShader: the fragment keeps everything and writes the default
        // depth, so the pixel resolves here (same operations as
        // resolve_pixel): the winner's depth, or primitive 0's chooser fallback.
        bool keep = found;
        float z = best_z[q];
        int prim = found ? static_cast<int>(best[q][0] & 0xffffffffu) : 0;
        if ((kKeys || kPairs) && found && !(z_known & (1u << q)) && !depth_of_order(o1, &z)) {
          // the winner came from a key alone and its depth is NaN or +-0:
          // its depth again, with the same operations
          const float4* r = jrec + static_cast<int64_t>(prim) * 4;
          const float4 a = __ldg(r), b = __ldg(r + 1), cz = __ldg(r + 2);
          const float c0 = (x[q] * a.x + y * a.w) + b.z;
          const float c1 = (x[q] * a.y + y * b.x) + b.w;
          const float c2 = (x[q] * a.z + y * b.y) + cz.x;
          z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
        }
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
  if (kTies) {
    for (int o = 16; o > 0; o >>= 1) tie_count += __shfl_xor_sync(0xffffffffu, tie_count, o);
    if (lane == 0 && tie_count) atomicAdd(B.near_ties, tie_count);
  }
  // tests is warp-uniform: one add per warp (work + 4: the launch's 64-bit test counter)
  if (lane == 0 && tests) atomicAdd(reinterpret_cast<unsigned long long*>(work + 4), tests);
}

// Vertex varyings of the three corners of every face some pixel needs
// (marked by the raster kernel), stored per face: the shade then reads them
// instead of re-running the vertex shader per pixel.  A block covers
// kVaryRows faces of one job (its own block map): it queues the visible ones
// in shared memory, then one thread per (visible face, corner) runs the
// vertex shader, so faces nobody sees leave no idle lanes and the block's
// job load and queue are paid once per kVaryRows faces.
constexpr int kFaceThreads = 256;
constexpr int kVaryRowsPerThread = 16;
constexpr int kVaryRows = kFaceThreads * kVaryRowsPerThread;

__global__ void __launch_bounds__(kFaceThreads)
face_varyings_kernel(RastBatch B, const int2* __restrict__ vmap, const unsigned char* __restrict__ visible,
                     float* __restrict__ fvar, int vstride) {
  __shared__ RastJob sJ;
  __shared__ int s_face[kVaryRows];
  __shared__ int s_n;
  const int2 blk = vmap[blockIdx.x];
  if (blk.x < 0) return;
  const int jid = blk.x;
  const int nf = __ldg(&B.jobs[jid].n_faces);
  if (__ldg(&B.jobs[jid].shader) == RAST_SHADER_DEPTH) return;
  load_job_to_shared(B.jobs + jid, &sJ);
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const RastJob& J = sJ;
  const int pairs = 3 * block_queue_rows<kVaryRowsPerThread, kFaceThreads>(
                            [&](int r) { return blk.y + r < nf && visible[J.setup_begin + blk.y + r]; }, s_face, &s_n);
  const int nv = varying_count(J.shader);
  for (int t = threadIdx.x; t < pairs; t += kFaceThreads) {
    const int q = t / 3, k = t - 3 * q;
    const int fq = blk.y + s_face[q];
    const int32_t* face = B.pools.faces + (J.face_begin + fq) * 3;
    float var[kMaxVarying], clip[4];
    vertex_shader<false>(J, B.pools, gather_clamp(__ldg(face + k), J.n_verts), clip, var);
    float* out = fvar + ((J.setup_begin + fq) * 3 + k) * vstride;
#pragma unroll
    for (int v = 0; v < kMaxVarying; ++v)
      if (v < nv) out[v] = var[v];
  }
}

// Deferred shading: one thread per pixel of every job, reading the winner's
// corner varyings computed once per visible face.  kLayered: the batch has
// layered jobs.  Their nearest-mixer pixels shade slot 0 with the default
// path's code and look at later slots only when its fragment is discarded;
// their "over" pixels spread the warp's fragments over its lanes
// (resolve_over_warp).
// Grid: (ceil(max pixels per job / 256), n_jobs).
// Eight blocks per SM (32 registers) for the default chooser: more resident
// warps hide the gathers and division chains better than the spills cost
// (1.17 -> 0.95 ms on the 4096-scene brax-like batch; 4, 5 and 6 blocks
// measured slower).  Layered batches take four (64 registers: 2.63 -> 2.56
// ms on the 4096-scene batch with 4 layers, from three).
template <bool kLayered>
__global__ void __launch_bounds__(256, kLayered ? 4 : 8)
tiled_shade_kernel(RastBatch B, const float4* __restrict__ setup, const int32_t* __restrict__ winner,
                   bool depth_resolved, const float* __restrict__ fvar, int vstride) {
  __shared__ RastJob sJ;
  __shared__ WarpFrags s_frags[kLayered ? 8 : 1];  // per warp, layered "over" jobs
  const int jid = blockIdx.y;
  const int64_t npx = static_cast<int64_t>(__ldg(&B.jobs[jid].width)) * __ldg(&B.jobs[jid].height);
  if (static_cast<int64_t>(blockIdx.x) * 256 >= npx) return;
  if (depth_resolved && __ldg(&B.jobs[jid].shader) == RAST_SHADER_DEPTH) return;  // done by the raster kernel
  load_job_to_shared(B.jobs + jid, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const int64_t local0 = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  const int64_t pix = J.pixel_begin + local0;
  const VaryingSource src{nullptr, vstride, 0, fvar, J.setup_begin};
  const float4* rec = setup + J.setup_begin * 4;
  const int L = kLayered ? job_layers(J, B.max_layers) : 0;
  if (kLayered && L > 0 && J.mixer == RAST_MIX_OVER) {  // every lane of the warp takes part
    const bool active = local0 < npx;
    int i = 0, j = 0;
    if (active) pixel_of(local0, npx, J.height, &i, &j);
    PixelResult r;
    resolve_over_warp(J, B.pools, rec, active, i, j, winner + (active ? pix : 0), B.total_pixels, L, src,
                      s_frags[threadIdx.x >> 5], &r);
    if (active) {
      store_pixel(J, B.pools, pix, r);
      save_layers(B.pools, winner + pix, B.total_pixels, pix, L);
    }
    return;
  }
  if (local0 >= npx) return;
  int i, j;
  pixel_of(local0, npx, J.height, &i, &j);
  PixelResult r;
  const int w0 = winner[pix];
  if (kLayered && L > 0) save_layers(B.pools, winner + pix, B.total_pixels, pix, L);
  if (kLayered && L > 0 && w0 < 0) {  // no candidate: the layered chooser keeps nothing
    r.keep = false;
    r.prim = -1;
    r.z = 0.0f;
    store_pixel(J, B.pools, pix, r);
    return;
  }
  resolve_pixel(J, B.pools, rec, i, j, w0, src, &r);  // the winner, or the layered chooser's slot 0
  if (kLayered && L > 1 && !r.keep)  // slot 0 discarded by its fragment shader: the next kept slot
    resolve_layers(J, B.pools, rec, i, j, winner + pix, B.total_pixels, L, src, &r, 1);
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
  size_t setup_off, bbox_off, binned_off, counts_off, offsets_off, cursors_off, bsums_off, bins_off, winner_off,
      vis_off, fvar_off, fmap_off, fstart_off, vmap_off, vstart_off, keys_off, misc_off, total;
  unsigned fmap_blocks, vmap_blocks;  // face block maps: setup/scatter, face varyings
  bool small_path;  // setup kernel rasterises small faces (not when near ties are counted)
  int vstride;
  int winner_layers;  // chooser slots kept per pixel: 1, or RAST_MAX_LAYERS with layered jobs
  int64_t n_tiles, n_scan_blocks;
  uint64_t bin_capacity;
  Geometry G;
};

static Layout layout(const RastBatch& b, TileShape ts, uint64_t bin_capacity, int small_area) {
  Layout L{};
  L.G.tw = ts.tw;
  L.G.th = ts.th;
  L.G.tws = __builtin_ctz(static_cast<unsigned>(ts.tw));
  L.G.ths = __builtin_ctz(static_cast<unsigned>(ts.th));
  L.G.tiles_x = ceil_div(std::max(b.max_width, 1), ts.tw);
  L.G.tiles_y = ceil_div(std::max(b.max_height, 1), ts.th);
  L.G.tiles_per_job = L.G.tiles_x * L.G.tiles_y;
  L.G.tpj_inv = div_inverse(static_cast<unsigned>(L.G.tiles_per_job));
  L.G.tx_inv = div_inverse(static_cast<unsigned>(L.G.tiles_x));
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
  L.binned_off = take(static_cast<size_t>(b.total_setup) * sizeof(int4));
  L.counts_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.cursors_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.offsets_off = take(static_cast<size_t>(L.n_tiles) * 4);
  L.bsums_off = take(static_cast<size_t>(L.n_scan_blocks) * 4);
  L.bins_off = take(static_cast<size_t>(bin_capacity) * 4);
  L.winner_layers = b.max_layers > 0 ? RAST_MAX_LAYERS : 1;  // the raster variant writes every slot
  L.winner_off = take(static_cast<size_t>(b.total_pixels) * 4 * L.winner_layers);
  int vstride = 0;
  for (int sh = 0; sh < 7; ++sh)
    if (b.shader_mask & (1 << sh)) vstride = std::max(vstride, varying_count(sh));
  L.vstride = vstride;
  const bool shading = vstride > 0;
  L.vis_off = take(shading ? static_cast<size_t>(b.total_setup) : 0);
  L.fvar_off = take(shading ? static_cast<size_t>(b.total_setup) * 3 * vstride * sizeof(float) : 0);
  L.fmap_blocks = block_map_capacity(b.total_setup, b.n_jobs, kSetupThreads);
  L.fmap_off = take(static_cast<size_t>(L.fmap_blocks) * sizeof(int2));
  L.fstart_off = take(block_start_bytes(b.n_jobs));
  L.vmap_blocks = shading ? block_map_capacity(b.total_setup, b.n_jobs, kVaryRows) : 0;
  L.vmap_off = take(static_cast<size_t>(L.vmap_blocks) * sizeof(int2));
  L.vstart_off = take(shading ? block_start_bytes(b.n_jobs) : 0);
  L.small_path = b.near_ties == nullptr && small_area > 0 && b.max_layers == 0;
  L.keys_off = take(L.small_path ? static_cast<size_t>(b.total_pixels) * sizeof(unsigned long long) : 0);
  L.misc_off = take(256);
  L.total = off;
  return L;
}

// The small-face threshold of a config (0 = off), clamped to one warp's lanes.
static int small_area_of(const RastTiledConfig* cfg) {
  if (!cfg || cfg->small_area <= 0) return 0;
  return std::min(cfg->small_area, kSmallArea);
}

// Bin tile shapes with a raster kernel: one warp per tile for every shape
// offered to the autotuner; two warps per tile (each rasterising half the
// rows) for the bin tiles whose halves are 8x4, 8x8 or 16x8.
static bool valid_shape(TileShape t, int wpt) {
  if (wpt == 2)
    return (t.tw == 8 && t.th == 8) || (t.tw == 8 && t.th == 16) || (t.tw == 16 && t.th == 16);
  return wpt == 1 &&
         ((t.tw == 8 && t.th == 8) || (t.tw == 16 && t.th == 16) || (t.tw == 32 && t.th == 8) ||
          (t.tw == 8 && t.th == 32) || (t.tw == 16 && t.th == 8) || (t.tw == 8 && t.th == 4) ||
          (t.tw == 4 && t.th == 8));
}

// Shapes with a layered raster variant: at most four pixels per lane, so
// the RAST_MAX_LAYERS keys of every pixel stay in registers (every
// two-warp shape's halves qualify).
static bool valid_layered_shape(TileShape t, int wpt) {
  if (wpt == 2) return valid_shape(t, 2);
  return (t.tw == 8 && t.th == 8) || (t.tw == 16 && t.th == 8) || (t.tw == 8 && t.th == 4) ||
         (t.tw == 4 && t.th == 8);
}

// Warps per tile of a config (0 or absent: one).
static int warps_per_tile_of(const RastTiledConfig* cfg) {
  return cfg && cfg->warps_per_tile > 0 ? cfg->warps_per_tile : 1;
}

// RAST_OK, or the status rast_render_tiled returns for a tile shape it has
// no kernel for.  Checked before any layout arithmetic (which divides by the
// tile's sides).
static int check_shape(const RastBatch& b, TileShape t, int wpt) {
  if (!valid_shape(t, wpt)) return RAST_ERR_INVALID_ARGUMENT;
  if (b.max_layers > 0 && !valid_layered_shape(t, wpt)) return RAST_ERR_UNSUPPORTED;
  return RAST_OK;
}

template <bool kKeys, bool kTies, int kL>
// The raster kernel is persistent: one resident wave of blocks (SMs x the
// blocks of this instance that fit on an SM) takes the work units (bin
// tiles x warps per tile).
static void launch_raster(TileShape ts, int wpt, int sms, cudaStream_t s, const RastBatch& b, const Layout& L,
                          const float4* setup, const ushort4* rects, const uint32_t* counts, const uint32_t* offsets, const int32_t* bins,
                          int32_t* winner, unsigned int* misc, unsigned char* vis,
                          const unsigned long long* keys) {
  const unsigned block = 32 * kRasterWarps;
  auto go = [&](auto kernel) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, static_cast<int>(block), 0) != cudaSuccess ||
        per_sm <= 0)
      per_sm = 8;
    const unsigned grid = static_cast<unsigned>(std::max(sms, 1) * per_sm);
    kernel<<<grid, block, 0, s>>>(b, L.G, setup, rects, counts, offsets, bins, winner, misc, L.n_tiles * wpt, vis,
                                  keys);
  };
  if (wpt == 2) {  // the warp's sub-tile is (tw, th / 2)
    if (ts.tw == 8 && ts.th == 16)
      go(raster_kernel<8, 8, kKeys, kTies, kL, 2>);
    else if (ts.tw == 16 && ts.th == 16)
      go(raster_kernel<16, 8, kKeys, kTies, kL, 2>);
    else
      go(raster_kernel<8, 4, kKeys, kTies, kL, 2>);
    return;
  }
  if (ts.tw == 8 && ts.th == 8)
    go(raster_kernel<8, 8, kKeys, kTies, kL, 1>);
  else if (ts.tw == 8 && ts.th == 4)
    go(raster_kernel<8, 4, kKeys, kTies, kL, 1>);
  else if (ts.tw == 4 && ts.th == 8)
    go(raster_kernel<4, 8, kKeys, kTies, kL, 1>);
  else if (ts.tw == 16 && ts.th == 8)
    go(raster_kernel<16, 8, kKeys, kTies, kL, 1>);
  else if constexpr (kL == 1) {  // eight pixels per lane: default chooser only
    if (ts.tw == 16 && ts.th == 16)
      go(raster_kernel<16, 16, kKeys, kTies, kL, 1>);
    else if (ts.tw == 32 && ts.th == 8)
      go(raster_kernel<32, 8, kKeys, kTies, kL, 1>);
    else
      go(raster_kernel<8, 32, kKeys, kTies, kL, 1>);
  }
}

static int render(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                  size_t workspace_bytes, void* stream, RastProfile* profile,
                  int phase = RAST_PHASE_COVERAGE | RAST_PHASE_SHADE) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  if (phase < 1 || phase > (RAST_PHASE_COVERAGE | RAST_PHASE_SHADE)) return RAST_ERR_INVALID_ARGUMENT;
  const RastBatch& b = *batch;
  TileShape ts{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8};
  const int wpt = warps_per_tile_of(cfg);
  st = check_shape(b, ts, wpt);
  if (st != RAST_OK) return st;
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : default_bin_capacity(b);
  const int small_area = small_area_of(cfg);
  const Layout L = layout(b, ts, cap, small_area);
  if (workspace_bytes < L.total) return RAST_ERR_WORKSPACE_TOO_SMALL;
  if (L.total > 0 && (workspace == nullptr || (reinterpret_cast<uintptr_t>(workspace) & 255)))
    return RAST_ERR_INVALID_ARGUMENT;
  if (b.max_width > 65535 || b.max_height > 65535) return RAST_ERR_UNSUPPORTED;  // pixel rectangles are 16-bit
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
  // [0] raster tile counter, [1] overflow status, [2..3] bin entries, [4..5] raster pixel tests,
  // [6] binned faces
  unsigned int* misc = reinterpret_cast<unsigned int*>(ws + L.misc_off);
  int4* binned = reinterpret_cast<int4*>(ws + L.binned_off);
  Profiler prof(profile, s, "rast_render_tiled");

  const bool cover = (phase & RAST_PHASE_COVERAGE) != 0, shade = (phase & RAST_PHASE_SHADE) != 0;
  unsigned char* vis = L.vstride > 0 ? reinterpret_cast<unsigned char*>(ws + L.vis_off) : nullptr;
  float* fvar = L.vstride > 0 ? reinterpret_cast<float*>(ws + L.fvar_off) : nullptr;
  // shaded jobs resolve in the deferred shade (from the per-face varyings when there are faces)
  const bool shading = b.total_pixels > 0 && (b.shader_mask != (1 << RAST_SHADER_DEPTH) || b.total_setup == 0);
  const bool pre = shading && fvar != nullptr && b.total_setup > 0;
  if (cover) {
    // counts and cursors are adjacent: one memset clears both, plus the counters
    if (cudaMemsetAsync(counts, 0, L.offsets_off - L.counts_off, s) != cudaSuccess) return RAST_ERR_CUDA;
    if (cudaMemsetAsync(misc, 0, 256, s) != cudaSuccess) return RAST_ERR_CUDA;
    unsigned long long* keys = nullptr;
    if (L.small_path && b.total_pixels > 0 && b.total_setup > 0) {
      keys = reinterpret_cast<unsigned long long*>(ws + L.keys_off);
      if (cudaMemsetAsync(keys, 0xff, static_cast<size_t>(b.total_pixels) * sizeof(unsigned long long), s) !=
          cudaSuccess)  // every key starts as kEmptyKey
        return RAST_ERR_CUDA;
    }
    if (vis && b.total_setup > 0 && cudaMemsetAsync(vis, 0, static_cast<size_t>(b.total_setup), s) != cudaSuccess)
      return RAST_ERR_CUDA;
    prof.mark("memset");
    int2* fmap = reinterpret_cast<int2*>(ws + L.fmap_off);
    if (b.total_setup > 0) {
      if (build_block_map(b, kMapFaces, kSetupThreads, fmap, reinterpret_cast<unsigned*>(ws + L.fstart_off), s) !=
          cudaSuccess)
        return RAST_ERR_CUDA;
      prof.mark("block_map_kernel");
      const unsigned grid = L.fmap_blocks;
      if (keys)
        setup_bin_kernel<true><<<grid, kSetupThreads, 0, s>>>(b, L.G, fmap, setup, bbox, counts, keys, small_area,
                                                             binned, misc + 6);
      else
        setup_bin_kernel<false><<<grid, kSetupThreads, 0, s>>>(b, L.G, fmap, setup, bbox, counts, nullptr, 0,
                                                              binned, misc + 6);
      prof.mark("setup_bin_kernel");
      scan_local_kernel<<<static_cast<unsigned>(L.n_scan_blocks), 256, 0, s>>>(counts, offsets, bsums, L.n_tiles);
      scan_apply_kernel<<<static_cast<unsigned>(L.n_scan_blocks), 256, 0, s>>>(counts, offsets, bsums, L.n_tiles,
                                                                                L.bin_capacity, misc + 1);
      prof.mark("scan_kernels");
      {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // the list's length is on the device: a full wave of blocks strides over it
        const unsigned sgrid = static_cast<unsigned>(std::max(sms, 1) * (2048 / kSetupThreads));
        scatter_kernel<<<std::min(sgrid, grid), kSetupThreads, 0, s>>>(L.G, binned, misc + 6, offsets, cursors, bins);
      }
      prof.mark("scatter_kernel");
    }
    if (b.total_pixels > 0) {
      int sms = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (b.total_setup > 0) {
        // the key path exists only when ties are not counted and no job is
        // layered
        if (keys)
          launch_raster<true, false, 1>(ts, wpt, sms, s, b, L, setup, bbox, counts, offsets, bins, winner, misc, vis, keys);
        else if (b.max_layers > 0 && b.near_ties)
          launch_raster<false, true, RAST_MAX_LAYERS>(ts, wpt, sms, s, b, L, setup, bbox, counts, offsets, bins, winner,
                                                      misc, vis, nullptr);
        else if (b.max_layers > 0)
          launch_raster<false, false, RAST_MAX_LAYERS>(ts, wpt, sms, s, b, L, setup, bbox, counts, offsets, bins, winner,
                                                       misc, vis, nullptr);
        else if (b.near_ties)
          launch_raster<false, true, 1>(ts, wpt, sms, s, b, L, setup, bbox, counts, offsets, bins, winner, misc, vis,
                                        nullptr);
        else
          launch_raster<false, false, 1>(ts, wpt, sms, s, b, L, setup, bbox, counts, offsets, bins, winner, misc, vis,
                                         nullptr);
      } else {
        if (cudaMemsetAsync(winner, 0xff, static_cast<size_t>(b.total_pixels) * 4 * L.winner_layers, s) !=
            cudaSuccess)
          return RAST_ERR_CUDA;
      }
      prof.mark("raster_kernel");
      if (pre) {
        int2* vmap = reinterpret_cast<int2*>(ws + L.vmap_off);
        if (build_block_map(b, kMapFaces, kVaryRows, vmap, reinterpret_cast<unsigned*>(ws + L.vstart_off), s) !=
            cudaSuccess)
          return RAST_ERR_CUDA;
        face_varyings_kernel<<<L.vmap_blocks, kFaceThreads, 0, s>>>(b, vmap, vis, fvar, L.vstride);
        prof.mark("face_varyings_kernel");
      }
    }
  }
  if (shade && shading) {
    const int64_t max_px = static_cast<int64_t>(b.max_width) * b.max_height;
    const dim3 sgrid(static_cast<unsigned>((max_px + 255) / 256), static_cast<unsigned>(b.n_jobs));
    const float* fv = pre ? fvar : nullptr;
    if (b.max_layers > 0)
      tiled_shade_kernel<true><<<sgrid, 256, 0, s>>>(b, setup, winner, b.total_setup > 0, fv, L.vstride);
    else
      tiled_shade_kernel<false><<<sgrid, 256, 0, s>>>(b, setup, winner, b.total_setup > 0, fv, L.vstride);
    prof.mark("tiled_shade_kernel");
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
  if (tiled::check_shape(*batch, ts, tiled::warps_per_tile_of(cfg)) != RAST_OK) return 0;
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : tiled::default_bin_capacity(*batch);
  return tiled::layout(*batch, ts, cap, tiled::small_area_of(cfg)).total;
}

extern "C" int rast_tiled_stats(const RastBatch* batch, const RastTiledConfig* cfg, const void* workspace,
                                void* stream, RastTiledStats* out) {
  if (!batch || !workspace || !out) return RAST_ERR_INVALID_ARGUMENT;
  tiled::TileShape ts{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8};
  const int shape_status = tiled::check_shape(*batch, ts, tiled::warps_per_tile_of(cfg));
  if (shape_status != RAST_OK) return shape_status;
  const uint64_t cap = cfg && cfg->bin_capacity > 0 ? cfg->bin_capacity : tiled::default_bin_capacity(*batch);
  const tiled::Layout L = tiled::layout(*batch, ts, cap, tiled::small_area_of(cfg));
  unsigned int misc[7] = {0, 0, 0, 0, 0, 0, 0};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(misc, static_cast<const char*>(workspace) + L.misc_off, sizeof(misc),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return RAST_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return RAST_ERR_CUDA;
  out->bin_entries = static_cast<uint64_t>(misc[2]) | (static_cast<uint64_t>(misc[3]) << 32);
  out->pixel_tests = static_cast<uint64_t>(misc[4]) | (static_cast<uint64_t>(misc[5]) << 32);
  out->overflow = misc[1];
  out->binned_faces = misc[6];
  out->tiles = static_cast<uint64_t>(L.n_tiles);
  out->bin_capacity = L.bin_capacity;
  return RAST_OK;
}

extern "C" int rast_render_tiled(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  return tiled::render(batch, cfg, workspace, workspace_bytes, stream, nullptr);
}

extern "C" int rast_render_tiled_phase(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                                       size_t workspace_bytes, void* stream, int phase) {
  return tiled::render(batch, cfg, workspace, workspace_bytes, stream, nullptr, phase);
}

extern "C" int rast_render_tiled_profiled(const RastBatch* batch, const RastTiledConfig* cfg,
                                          void* workspace, size_t workspace_bytes, void* stream,
                                          RastProfile* profile) {
  return tiled::render(batch, cfg, workspace, workspace_bytes, stream, profile);
}

// ------------------------------------------------------------ autotuning

namespace {

struct TuneCandidate {
  int tw, th, wpt, small;
};

// Every configuration the tiled form has a kernel for.
std::vector<TuneCandidate> tune_candidates(const RastBatch& b) {
  const bool layered = b.max_layers > 0;
  const bool small_ok = !layered && b.near_ties == nullptr;
  std::vector<TuneCandidate> out;
  const int shapes1[7][2] = {{8, 8}, {16, 8}, {16, 16}, {32, 8}, {8, 32}, {8, 4}, {4, 8}};
  const int shapes2[3][2] = {{8, 8}, {8, 16}, {16, 16}};
  for (int small : {0, 32}) {
    if (small && !small_ok) continue;
    for (const auto& sh : shapes1) {
      const tiled::TileShape t{sh[0], sh[1]};
      if (tiled::check_shape(b, t, 1) == RAST_OK) out.push_back({sh[0], sh[1], 1, small});
    }
    for (const auto& sh : shapes2) {
      const tiled::TileShape t{sh[0], sh[1]};
      if (tiled::check_shape(b, t, 2) == RAST_OK) out.push_back({sh[0], sh[1], 2, small});
    }
  }
  return out;
}

// Workload class of a batch: canvas size, faces per job and jobs (powers of
// two), shaders, chooser layers, tie counting, device.
std::string tune_key(const RastBatch& b, int dev) {
  auto bucket = [](double v) { return v < 1.0 ? 0 : static_cast<int>(std::lround(std::log2(v))); };
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  char key[256];
  std::snprintf(key, sizeof(key), "%dx%d|f%d|j%d|m%d|l%d|t%d|d%d|s%d", b.max_width, b.max_height,
                bucket(static_cast<double>(b.total_setup) / std::max(b.n_jobs, 1)), bucket(b.n_jobs), b.shader_mask,
                b.max_layers, b.near_ties != nullptr, dev, sms);
  return key;
}

std::mutex g_tune_mutex;
std::map<std::string, RastTiledConfig> g_tune_cache;

}  // namespace

extern "C" int rast_autotune(const RastBatch* batch, void* stream, RastTiledConfig* out) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  if (!out) return RAST_ERR_INVALID_ARGUMENT;
  const RastBatch& b = *batch;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RAST_ERR_CUDA;
  const std::string key = tune_key(b, dev);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *out = it->second;
      return RAST_OK;
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return RAST_ERR_CUDA;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  float best_ms = 0.0f;
  RastTiledConfig best{};
  bool found = false;
  st = RAST_OK;
  for (const TuneCandidate& c : tune_candidates(b)) {
    RastTiledConfig cfg{c.tw, c.th, 0, c.small, c.wpt};
    // capacity for the timed renders: 1.25 x the entries this shape requests
    for (int round = 0; round < 2 && st == RAST_OK; ++round) {
      const size_t need = rast_tiled_workspace_bytes(&b, &cfg);
      if (need > ws_bytes) {
        if (ws) cudaFreeAsync(ws, s);
        ws = nullptr;
        if (cudaMallocAsync(&ws, need, s) != cudaSuccess) {
          st = RAST_ERR_CUDA;
          break;
        }
        ws_bytes = need;
      }
      if (round == 0) {
        st = rast_render_tiled(&b, &cfg, ws, ws_bytes, s);
        RastTiledStats stats{};
        if (st == RAST_OK) st = rast_tiled_stats(&b, &cfg, ws, s, &stats);
        cfg.bin_capacity = stats.bin_entries + stats.bin_entries / 4 + 4096;
      }
    }
    if (st != RAST_OK) break;
    constexpr int kReps = 3;
    if (cudaEventRecord(e0, s) != cudaSuccess) {
      st = RAST_ERR_CUDA;
      break;
    }
    for (int r = 0; r < kReps && st == RAST_OK; ++r) st = rast_render_tiled(&b, &cfg, ws, ws_bytes, s);
    if (st != RAST_OK) break;
    float ms = 0.0f;
    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      st = RAST_ERR_CUDA;
      break;
    }
    if (!found || ms < best_ms) {
      best_ms = ms;
      best = cfg;
      found = true;
    }
  }
  if (ws) cudaFreeAsync(ws, s);
  cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != RAST_OK) return st;
  if (!found) return RAST_ERR_UNSUPPORTED;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = best;
  }
  *out = best;
  return RAST_OK;
}

// ------------------------------------------------ allocation-free variant

namespace {

// Workspace of rast_render_tiled_static: one per GPU that loads the library,
// held until process exit.
static __device__ __align__(256) unsigned char g_static_scratch[RAST_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;

// Cached device address of g_static_scratch per device, tagged with the id
// of the CUDA context it was looked up in.  A cudaDeviceReset (or a primary
// context reset) loads the module again at a new address in a new context;
// the new context id then triggers a fresh lookup.
struct StaticSlot {
  unsigned long long ctx_id;
  void* ptr;
};
StaticSlot g_static_slot[kMaxDevices] = {};

// cuCtxGetCurrent / cuCtxGetId, resolved through the runtime so the library
// needs no link against the driver library.  Null when the driver lacks
// them: the cache is then keyed by device ordinal alone.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_ctx_fns_resolved = false;

// Id of the current context (0 when it cannot be read).  Caller holds the mutex.
unsigned long long current_ctx_id() {
  if (!g_ctx_fns_resolved) {
    g_ctx_fns_resolved = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
    (void)cudaGetLastError();
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_static_scratch on the current device (host code sees
// only a host-side stand-in for the symbol).  Looked up once per device and
// context, with that device current.
int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RAST_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return RAST_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  StaticSlot& slot = g_static_slot[dev];
  const unsigned long long id = current_ctx_id();
  if (!slot.ptr || (id != 0 && id != slot.ctx_id)) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return RAST_ERR_CUDA;
    slot.ptr = p;
    // the lookup made the device's context current if it was not yet
    slot.ctx_id = id != 0 ? id : current_ctx_id();
  }
  *out = slot.ptr;
  return RAST_OK;
}

}  // namespace

extern "C" int rast_render_tiled_static(const RastBatch* batch, const RastTiledConfig* cfg, void* stream) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  st = tiled::check_shape(*batch, tiled::TileShape{cfg ? cfg->tile_w : 8, cfg ? cfg->tile_h : 8},
                          tiled::warps_per_tile_of(cfg));
  if (st != RAST_OK) return st;
  const size_t need = rast_tiled_workspace_bytes(batch, cfg);
  if (need > RAST_STATIC_SCRATCH_BYTES) return RAST_ERR_STATIC_SCRATCH_TOO_SMALL;
  void* scratch = nullptr;
  st = static_scratch(&scratch);
  if (st != RAST_OK) return st;
  return tiled::render(batch, cfg, scratch, RAST_STATIC_SCRATCH_BYTES, stream, nullptr);
}
