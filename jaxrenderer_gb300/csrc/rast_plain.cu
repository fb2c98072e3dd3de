// rast_plain.cu -- plain form of the rasteriser: the reference's own method
// (pipeline.py:470-537) at GPU speed.
//
//   vertex_kernel  one thread per vertex: gl_Position + varyings
//                  (pipeline.py:497-518)
//   setup_kernel   one thread per face: gather by face index, det, keep,
//                  3x3 LU inverse (PerPrimitive.create, pipeline.py:80-113)
//   scan_kernel    one thread per pixel, every primitive of the job streamed
//                  through shared memory: clip_coef, inside test, depth,
//                  packed (ordered depth | id) minimum = the default
//                  primitive_chooser (shader.py:207-251)
//   shade_kernel   one thread per pixel: chosen primitive -> barycentrics ->
//                  interpolate -> fragment -> mix -> merge
//                  (pipeline.py:283-359, 401-440)
#include <cuda_runtime.h>

#include <algorithm>

#include "rast_internal.cuh"

namespace rast {

// -------------------------------------------------------------- kernels

// Grid: (ceil(max_verts / 256), n_jobs).
__global__ void __launch_bounds__(256)
vertex_kernel(RastBatch B, float4* __restrict__ clip_out, float* __restrict__ var_out, int vstride) {
  __shared__ RastJob sJ;
  const int jid = blockIdx.y;
  const int nv = __ldg(&B.jobs[jid].n_verts);
  if (static_cast<int64_t>(blockIdx.x) * 256 >= nv) return;
  load_job_to_shared(B.jobs + jid, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const int64_t v0 = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  if (v0 >= nv) return;
  const int64_t row = J.vout_begin + v0;
  const int v = static_cast<int>(row - J.vout_begin);
  float clip[4];
  float var[kMaxVarying];
  vertex_shader(J, B.pools, v, clip, var);
  clip_out[row] = make_float4(clip[0], clip[1], clip[2], clip[3]);
  const int nvar = varying_count(J.shader);
  for (int k = 0; k < nvar; ++k) var_out[row * vstride + k] = var[k];
}

// Grid: (ceil(max_faces / 256), n_jobs).
__global__ void __launch_bounds__(256)
setup_kernel(RastBatch B, const float4* __restrict__ clip, float4* __restrict__ setup) {
  const int jid = blockIdx.y;
  const RastJob& J = B.jobs[jid];
  const int64_t f0 = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  if (f0 >= J.n_faces) return;
  const int64_t row = J.setup_begin + f0;
  const int64_t f = row - J.setup_begin;
  const int32_t* face = B.pools.faces + (J.face_begin + f) * 3;
  float4 c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = clip[J.vout_begin + gather_clamp(face[k], J.n_verts)];
  write_setup(c, setup + row * 4);
}

// One CTA = one 16x16 pixel tile of one job; every primitive of the job is
// staged through shared memory in chunks and tested by every pixel.  Each
// pixel keeps the kL smallest packed keys (kL = 1: the default chooser's
// argmin; kL = RAST_MAX_LAYERS when the batch has layered jobs, whose slots
// are the layered chooser's); slot s goes to winner[s * total_pixels + pix].
template <int kL>
__global__ void __launch_bounds__(kScanThreads)
scan_kernel(RastBatch B, const float4* __restrict__ setup, int32_t* __restrict__ winner) {
  __shared__ float4 s_rec[kScanChunk * 3];
  __shared__ int s_flag[kScanChunk];
  const RastJob& J = B.jobs[blockIdx.y];
  const int W = J.width, H = J.height, F = J.n_faces;
  const int tiles_j = (H + kTile - 1) / kTile;
  const int tiles_i = (W + kTile - 1) / kTile;
  if (static_cast<int>(blockIdx.x) >= tiles_i * tiles_j) return;
  const int ti = blockIdx.x / tiles_j, tj = blockIdx.x % tiles_j;
  const int i = ti * kTile + threadIdx.y;
  const int j = tj * kTile + threadIdx.x;
  const int tid = threadIdx.y * kTile + threadIdx.x;
  const float x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
  const float y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
  const float vp22 = J.viewport[10], vp23 = J.viewport[11];
  unsigned long long best[kL];
#pragma unroll
  for (int l = 0; l < kL; ++l) best[l] = kEmptyKey;
  uint32_t second = 0xffffffffu;
  const float4* rec = setup + J.setup_begin * 4;
  for (int base = 0; base < F; base += kScanChunk) {
    const int n = min(kScanChunk, F - base);
    for (int q = tid; q < n * 3; q += kScanThreads)
      s_rec[q] = __ldg(rec + (static_cast<int64_t>(base) + q / 3) * 4 + q % 3);
    for (int q = tid; q < n; q += kScanThreads)
      s_flag[q] = __float_as_int(__ldg(rec + (static_cast<int64_t>(base) + q) * 4 + 3).y);
    __syncthreads();
    for (int p = 0; p < n; ++p) {
      const float4 a = s_rec[3 * p + 0];
      const float4 b = s_rec[3 * p + 1];
      const float4 cz = s_rec[3 * p + 2];
      // clip_coef = [x, y, 1] @ inv (pipeline.py:177-193)
      const float c0 = (x * a.x + y * a.w) + b.z;
      const float c1 = (x * a.y + y * b.x) + b.w;
      const float c2 = (x * a.z + y * b.y) + cz.x;
      if (all_nonneg(c0, c1, c2)) {
        if ((s_flag[p] & kCandidate) == kCandidate) {
          const float z = ((c0 * cz.y + c1 * cz.z) + c2 * cz.w) * vp22 + vp23;
          const unsigned long long key = pack_key(z, base + p);
          const uint32_t o = static_cast<uint32_t>(key >> 32);
          if (key < best[0]) {
            second = min(second, static_cast<uint32_t>(best[0] >> 32));
          } else {
            second = min(second, o);
          }
          insert_key<kL>(best, key);
        }
      }
    }
    __syncthreads();
  }
  const bool valid = i < W && j < H;
  if (valid) {
    const int64_t pix = J.pixel_begin + static_cast<int64_t>(i) * H + j;
#pragma unroll
    for (int l = 0; l < kL; ++l) {
      const uint32_t o = static_cast<uint32_t>(best[l] >> 32);
      winner[l * B.total_pixels + pix] =
          (best[l] == kEmptyKey || o == kInfOrder) ? -1 : static_cast<int32_t>(best[l] & 0xffffffffu);
    }
  }
  if (B.near_ties) count_near_tie(B.near_ties, valid && is_near_tie(best[0], second));
}

// One thread per pixel: the chosen primitive's fragment, mixed and merged
// (kLayered: the batch has layered jobs, whose pixels shade and mix every
// slot).
template <bool kLayered>
__global__ void __launch_bounds__(kScanThreads)
shade_kernel(RastBatch B, const float4* __restrict__ setup, const float* __restrict__ var,
             int vstride, const int32_t* __restrict__ winner) {
  __shared__ RastJob sJ;
  load_job_to_shared(B.jobs + blockIdx.y, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const int W = J.width, H = J.height;
  const int tiles_j = (H + kTile - 1) / kTile;
  const int tiles_i = (W + kTile - 1) / kTile;
  if (static_cast<int>(blockIdx.x) >= tiles_i * tiles_j) return;
  const int ti = blockIdx.x / tiles_j, tj = blockIdx.x % tiles_j;
  const int i = ti * kTile + threadIdx.y;
  const int j = tj * kTile + threadIdx.x;
  if (i >= W || j >= H) return;
  const int64_t pix = J.pixel_begin + static_cast<int64_t>(i) * H + j;
  PixelResult r;
  const VaryingSource src{var, vstride, J.vout_begin};
  const int L = kLayered ? job_layers(J, B.max_layers) : 0;
  if (kLayered && L > 0) {
    resolve_layers(J, B.pools, setup + J.setup_begin * 4, i, j, winner + pix, B.total_pixels, L, src, &r);
    save_layers(B.pools, winner + pix, B.total_pixels, pix, L);
  } else {
    resolve_pixel(J, B.pools, setup + J.setup_begin * 4, i, j, winner[pix], src, &r);
  }
  store_pixel(J, B.pools, pix, r);
}

// ------------------------------------------------------------- launcher

struct PlainLayout {
  size_t clip_off, var_off, setup_off, winner_off, total;
  int vstride;
};

static PlainLayout plain_layout(const RastBatch& b) {
  PlainLayout L{};
  int vstride = 0;
  for (int s = 0; s < 7; ++s)
    if (b.shader_mask & (1 << s)) vstride = std::max(vstride, varying_count(s));
  L.vstride = vstride;
  size_t off = 0;
  L.clip_off = off;
  off = align256(off + static_cast<size_t>(b.total_vout) * sizeof(float4));
  L.var_off = off;
  off = align256(off + static_cast<size_t>(b.total_vout) * vstride * sizeof(float));
  L.setup_off = off;
  off = align256(off + static_cast<size_t>(b.total_setup) * 4 * sizeof(float4));
  L.winner_off = off;
  // one slot per pixel, or RAST_MAX_LAYERS (every slot scan_kernel writes) with layered jobs
  const size_t slots = b.max_layers > 0 ? RAST_MAX_LAYERS : 1;
  off = align256(off + static_cast<size_t>(b.total_pixels) * slots * sizeof(int32_t));
  L.total = off;
  return L;
}

}  // namespace rast

using namespace rast;

extern "C" size_t rast_plain_workspace_bytes(const RastBatch* batch) {
  if (!batch) return 0;
  return plain_layout(*batch).total;
}

static int render_plain(const RastBatch* batch, void* workspace, size_t workspace_bytes,
                        void* stream, RastProfile* profile) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  const RastBatch& b = *batch;
  const PlainLayout L = plain_layout(b);
  if (workspace_bytes < L.total) return RAST_ERR_WORKSPACE_TOO_SMALL;
  if (L.total > 0 && (workspace == nullptr || (reinterpret_cast<uintptr_t>(workspace) & 255)))
    return RAST_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  float4* clip = reinterpret_cast<float4*>(ws + L.clip_off);
  float* var = reinterpret_cast<float*>(ws + L.var_off);
  float4* setup = reinterpret_cast<float4*>(ws + L.setup_off);
  int32_t* winner = reinterpret_cast<int32_t*>(ws + L.winner_off);
  Profiler prof(profile, s, "rast_render_plain");

  if (b.total_vout > 0) {
    const dim3 grid(static_cast<unsigned>((b.max_verts + 255) / 256), static_cast<unsigned>(b.n_jobs));
    vertex_kernel<<<grid, 256, 0, s>>>(b, clip, var, L.vstride);
    prof.mark("vertex_kernel");
  }
  if (b.total_setup > 0) {
    const dim3 grid(static_cast<unsigned>((b.max_faces + 255) / 256), static_cast<unsigned>(b.n_jobs));
    setup_kernel<<<grid, 256, 0, s>>>(b, clip, setup);
    prof.mark("setup_kernel");
  }
  if (b.total_pixels > 0) {
    const int tiles = ((b.max_width + kTile - 1) / kTile) * ((b.max_height + kTile - 1) / kTile);
    const dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(b.n_jobs));
    const dim3 block(kTile, kTile);
    if (b.max_layers > 0)
      scan_kernel<RAST_MAX_LAYERS><<<grid, block, 0, s>>>(b, setup, winner);
    else
      scan_kernel<1><<<grid, block, 0, s>>>(b, setup, winner);
    prof.mark("scan_kernel");
    if (b.max_layers > 0)
      shade_kernel<true><<<grid, block, 0, s>>>(b, setup, var, L.vstride, winner);
    else
      shade_kernel<false><<<grid, block, 0, s>>>(b, setup, var, L.vstride, winner);
    prof.mark("shade_kernel");
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return RAST_ERR_CUDA;
  return prof.finish();
}

extern "C" int rast_render_plain(const RastBatch* batch, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  return render_plain(batch, workspace, workspace_bytes, stream, nullptr);
}

extern "C" int rast_render_plain_profiled(const RastBatch* batch, void* workspace,
                                          size_t workspace_bytes, void* stream,
                                          RastProfile* profile) {
  return render_plain(batch, workspace, workspace_bytes, stream, profile);
}
