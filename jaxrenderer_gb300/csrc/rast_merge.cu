// rast_merge.cu -- merge_objects + per-corner flattening on the device for
// instanced scenes (renderer/model.py:447-555, renderer/renderer.py:277-295).
//
//   mesh_norm_kernel      one warp per mesh: global norm of its normals
//                         (normalise() divides a whole array by one norm)
//   instance_kernel       one warp per instance: its rows of the merged
//                         arrays (world positions, object index per vertex,
//                         normals through the inverse-transpose -- 4x4 LU in
//                         jnp.linalg.inv's order -- and the global norm of the
//                         transformed normals, uvs)
//   corner_kernel         one warp per instance: gathers per face corner
//
// Operation order follows the host merge: apply_pos = to_cartesian(M [p * s,
// 1]) with products summed in index order; apply_vec = normalise(M [n /
// |N|, 0])[:3] over the whole array; gathers wrap negative indices once and
// clamp to the scene's merged array.
#include <cuda_runtime.h>

#include <algorithm>

#include "rast_internal.cuh"

namespace rast {
namespace merge {

constexpr int kThreads = 256;

// jnp.linalg.inv of one N x N matrix: LU with partial pivoting (first index
// of the largest |a|, no swap for a zero pivot column), reciprocal scaling
// for normal pivots, then the two triangular solves per column of the
// permuted identity, skipping zero right-hand sides -- the same sequence as
// geometry.lu_inverse on the host.
template <int N>
__device__ __forceinline__ void inv_lu(const float* m, float* out) {
  float a[N * N];
#pragma unroll
  for (int k = 0; k < N * N; ++k) a[k] = m[k];
  int perm[N];
#pragma unroll
  for (int k = 0; k < N; ++k) perm[k] = k;
#pragma unroll
  for (int j = 0; j < N - 1; ++j) {
    int p = j;
    float best = fabsf(a[N * j + j]);
#pragma unroll
    for (int r = j + 1; r < N; ++r) {
      const float v = fabsf(a[N * r + j]);
      if (v > best) {
        best = v;
        p = r;
      }
    }
    // pivot value after the (conditional) swap, selected without dynamic indexing
    float pv = a[N * j + j];
#pragma unroll
    for (int r = j + 1; r < N; ++r)
      if (p == r) pv = a[N * r + j];
    const bool nz = pv != 0.0f;
    if (nz && p != j) {
#pragma unroll
      for (int r = j + 1; r < N; ++r) {
        if (p == r) {
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const float t = a[N * j + c];
            a[N * j + c] = a[N * r + c];
            a[N * r + c] = t;
          }
          const int t = perm[j];
          perm[j] = perm[r];
          perm[r] = t;
        }
      }
    }
    const float piv = a[N * j + j];
    if (nz) {
      if (fabsf(piv) >= 1.17549435e-38f) {
        const float rcp = 1.0f / piv;
#pragma unroll
        for (int r = j + 1; r < N; ++r) a[N * r + j] = a[N * r + j] * rcp;
      } else {
#pragma unroll
        for (int r = j + 1; r < N; ++r) a[N * r + j] = a[N * r + j] / piv;
      }
    }
#pragma unroll
    for (int r = j + 1; r < N; ++r)
#pragma unroll
      for (int c = j + 1; c < N; ++c) a[N * r + c] = a[N * r + c] - a[N * r + j] * a[N * j + c];
  }
#pragma unroll
  for (int col = 0; col < N; ++col) {
    float b[N];
#pragma unroll
    for (int r = 0; r < N; ++r) b[r] = (perm[r] == col) ? 1.0f : 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (b[k] != 0.0f)
#pragma unroll
        for (int i = k + 1; i < N; ++i) b[i] = b[i] - b[k] * a[N * i + k];
#pragma unroll
    for (int k = N - 1; k >= 0; --k)
      if (b[k] != 0.0f) {
        b[k] = b[k] / a[N * k + k];
#pragma unroll
        for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * a[N * i + k];
      }
#pragma unroll
    for (int r = 0; r < N; ++r) out[N * r + col] = b[r];
  }
}

// gather index semantics of jnp indexing: negative wraps once, then clamp
__device__ __forceinline__ int wrap_clamp(int i, int n) {
  if (i < 0) i += n;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// Sequential (index-order) sum of squares of the `count` floats at v, by one
// warp: every lane squares 4 values of a 128-value round into `stage`
// (128 floats), lane 0 adds the round's squares in index order from
// registers, and the next round's values are loaded while it adds.  The
// running sum starts at +0 and the padding past `count` adds +0: a sum of
// squares is never -0, so neither changes a bit of the index-order sum.
// Every lane gets the total.
__device__ __forceinline__ float warp_sum_sq_sequential(const float* v, int64_t count, float* stage) {
  constexpr int kRound = 128;
  const int lane = threadIdx.x & 31;
  auto load = [&](int64_t base, float* x) {
#pragma unroll
    for (int j = 0; j < kRound / 32; ++j) {
      const int64_t k = base + 32 * j + lane;
      x[j] = k < count ? v[k] : 0.0f;
    }
  };
  float acc = 0.0f;
  float x[kRound / 32];
  load(0, x);
  for (int64_t base = 0; base < count; base += kRound) {
#pragma unroll
    for (int j = 0; j < kRound / 32; ++j) stage[32 * j + lane] = x[j] * x[j];
    __syncwarp();
    if (base + kRound < count) load(base + kRound, x);  // in flight while lane 0 adds
    if (lane == 0) {
      float sq[kRound];
#pragma unroll
      for (int q = 0; q < kRound; ++q) sq[q] = stage[q];
#pragma unroll
      for (int q = 0; q < kRound; ++q) acc = acc + sq[q];
    }
    __syncwarp();
  }
  return __shfl_sync(0xffffffffu, acc, 0);
}

// One warp per mesh: the global norm of its normals (normalise() divides a
// whole array by one norm).  Grid: ceil(n_meshes * 32 / kThreads).
__global__ void __launch_bounds__(kThreads) mesh_norm_kernel(RastMergeBatch B, float* __restrict__ mesh_norm) {
  __shared__ float stage[kThreads / 32][128];
  const int m = static_cast<int>((static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5);
  if (m >= B.n_meshes) return;
  const RastMesh M = B.meshes[m];
  const float acc = warp_sum_sq_sequential(B.mesh_norms + M.norm_begin * 3, static_cast<int64_t>(M.n_norms) * 3,
                                           stage[threadIdx.x >> 5]);
  if ((threadIdx.x & 31) == 0) mesh_norm[m] = sqrtf(acc);
}

// apply_pos: to_cartesian(T [p * s, 1]), products summed in index order
// (x / 1 == x, so the common w == 1 skips the division exactly)
__device__ __forceinline__ void world_position(const float* p, const float* s, const float* T, float* out) {
  const float q0 = p[0] * s[0], q1 = p[1] * s[1], q2 = p[2] * s[2];
  float h[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) h[r] = ((q0 * T[4 * r + 0] + q1 * T[4 * r + 1]) + q2 * T[4 * r + 2]) + 1.0f * T[4 * r + 3];
  if (h[3] == 0.0f || h[3] == 1.0f) {
    out[0] = h[0];
    out[1] = h[1];
    out[2] = h[2];
  } else {
    out[0] = h[0] / h[3];
    out[1] = h[1] / h[3];
    out[2] = h[2] / h[3];
  }
}

// One warp per instance writes its rows of the merged arrays: world
// positions and the object index of every vertex row, apply_vec'd normals
// (inverse-transpose by lane 0, transformed rows by all lanes, the global
// norm summed sequentially by lane 0, then the division), and uvs.
// Grid: ceil(n_instances * 32 / kThreads) blocks.
__global__ void __launch_bounds__(kThreads)
instance_kernel(RastMergeBatch B, const float* __restrict__ mesh_norm, float* __restrict__ mpos,
                int* __restrict__ mobj, float* __restrict__ mnrm, float* __restrict__ muv) {
  __shared__ float stage[kThreads / 32][128];
  const int o = static_cast<int>((static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (o >= B.n_instances) return;  // whole warps
  const RastInstance I = B.instances[o];
  const RastMesh mesh = B.meshes[I.mesh];
  float T[16], sc[3];
#pragma unroll
  for (int k = 0; k < 16; ++k) T[k] = __ldg(B.transforms + static_cast<int64_t>(o) * 16 + k);
#pragma unroll
  for (int k = 0; k < 3; ++k) sc[k] = __ldg(B.local_scaling + static_cast<int64_t>(o) * 3 + k);
  const int64_t vrow = I.vert_row, nrow = I.norm_row, urow = I.uv_row;
  for (int v = lane; v < mesh.n_verts; v += 32) {
    float out[3];
    world_position(B.mesh_verts + (mesh.vert_begin + v) * 3, sc, T, out);
    float* dst = mpos + (vrow + v) * 3;
    dst[0] = out[0];
    dst[1] = out[1];
    dst[2] = out[2];
    mobj[vrow + v] = o - I.scene_first;
  }
  if (muv) {
    for (int u = lane; u < mesh.n_uvs; u += 32) {
      muv[(urow + u) * 2 + 0] = __ldg(B.mesh_uvs + (mesh.uv_begin + u) * 2 + 0);
      muv[(urow + u) * 2 + 1] = __ldg(B.mesh_uvs + (mesh.uv_begin + u) * 2 + 1);
    }
  }
  if (mnrm && mesh.n_norms > 0) {
    float M[16];
    if (lane == 0) {
      float inv[16];
      inv_lu<4>(T, inv);
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) M[4 * r + c] = inv[4 * c + r];
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) M[k] = __shfl_sync(0xffffffffu, M[k], 0);
    const float nn = mesh_norm[I.mesh];
    for (int k = lane; k < mesh.n_norms; k += 32) {
      const float* nv = B.mesh_norms + (mesh.norm_begin + k) * 3;
      const float h0 = nv[0] / nn, h1 = nv[1] / nn, h2 = nv[2] / nn;
      float* dst = mnrm + (nrow + k) * 3;
#pragma unroll
      for (int r = 0; r < 3; ++r)
        dst[r] = ((h0 * M[4 * r + 0] + h1 * M[4 * r + 1]) + h2 * M[4 * r + 2]) + 0.0f * M[4 * r + 3];
    }
    __syncwarp();
    const float on = sqrtf(warp_sum_sq_sequential(mnrm + nrow * 3, static_cast<int64_t>(mesh.n_norms) * 3,
                                                  stage[threadIdx.x >> 5]));
    for (int64_t k = lane; k < static_cast<int64_t>(mesh.n_norms) * 3; k += 32) mnrm[nrow * 3 + k] /= on;
  }
}

// One warp per instance writes the instance's 3 * n_faces corners: merged
// face indices (local + scene offset), gathered from the scene's merged rows
// with wrap-once-then-clamp.  Grid: ceil(n_instances * 32 / kThreads).
__global__ void __launch_bounds__(kThreads)
corner_kernel(RastMergeBatch B, const float* __restrict__ mpos, const int* __restrict__ mobj,
              const float* __restrict__ mnrm, const float* __restrict__ muv) {
  const int o = static_cast<int>((static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (o >= B.n_instances) return;
  const RastInstance I = B.instances[o];
  const RastMesh mesh = B.meshes[I.mesh];
  // the scene's merged arrays start at its first instance's rows
  const RastInstance& F = B.instances[I.scene_first];
  const int64_t vbase = F.vert_row, nbase = F.norm_row, ubase = F.uv_row;
  const int64_t corners = 3 * static_cast<int64_t>(mesh.n_faces);
  const int64_t fsrc = mesh.face_begin * 3;  // faces are (rows, 3): corner c of the mesh is fsrc + c
  float* __restrict__ out_pos = B.position;
  float* __restrict__ out_nrm = B.normal;
  float* __restrict__ out_uv = B.uv;
  int* __restrict__ out_tix = B.texture_index;
  constexpr int kU = 2;  // corners per lane per round: their gathers are in flight together
  for (int64_t base = 0; base < corners; base += 32 * kU) {
    float pv[kU][3], nv[kU][3], uv[kU][2];
    int tix[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int64_t c = base + u * 32 + lane;
      if (c >= corners) continue;
      const int vi = wrap_clamp(I.vert_offset + __ldg(B.mesh_faces + fsrc + c), I.scene_verts);
#pragma unroll
      for (int k = 0; k < 3; ++k) pv[u][k] = mpos[(vbase + vi) * 3 + k];
      if (out_nrm) {
        const int ni = wrap_clamp(I.norm_offset + __ldg(B.mesh_faces_norm + fsrc + c), I.scene_norms);
#pragma unroll
        for (int k = 0; k < 3; ++k) nv[u][k] = mnrm[(nbase + ni) * 3 + k];
      }
      if (out_uv || out_tix) {
        const int fu = __ldg(B.mesh_faces_uv + fsrc + c);
        if (out_uv) {
          const int ui = wrap_clamp(I.uv_offset + fu, I.scene_uvs);
          uv[u][0] = muv[(ubase + ui) * 2 + 0];
          uv[u][1] = muv[(ubase + ui) * 2 + 1];
        }
        // texture_index[faces_uv]: the per-vertex object index gathered
        // with merged uv indices (renderer.py:287-289)
        if (out_tix) tix[u] = mobj[vbase + wrap_clamp(I.uv_offset + fu, I.scene_verts)];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int64_t c = base + u * 32 + lane;
      if (c >= corners) continue;
      const int64_t corner = I.corner_begin + c;
#pragma unroll
      for (int k = 0; k < 3; ++k) out_pos[corner * 3 + k] = pv[u][k];
      if (out_nrm) {
#pragma unroll
        for (int k = 0; k < 3; ++k) out_nrm[corner * 3 + k] = nv[u][k];
      }
      if (out_uv) {
        out_uv[corner * 2 + 0] = uv[u][0];
        out_uv[corner * 2 + 1] = uv[u][1];
      }
      if (out_tix) out_tix[corner] = tix[u];
    }
  }
}

struct Layout {
  size_t norm_off, pos_off, obj_off, nrm_off, uv_off, total;
};

static Layout layout(const RastMergeBatch& b) {
  Layout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  L.norm_off = take(static_cast<size_t>(std::max(b.n_meshes, 0)) * sizeof(float));
  L.pos_off = take(static_cast<size_t>(b.total_verts) * 3 * sizeof(float));
  L.obj_off = take(static_cast<size_t>(b.total_verts) * sizeof(int));
  L.nrm_off = take(b.normal ? static_cast<size_t>(b.total_norms) * 3 * sizeof(float) : 0);
  L.uv_off = take(b.uv ? static_cast<size_t>(b.total_uvs) * 2 * sizeof(float) : 0);
  L.total = off;
  return L;
}

static int check(const RastMergeBatch* b) {
  if (!b) return RAST_ERR_INVALID_ARGUMENT;
  if (b->n_meshes < 0 || b->n_instances < 0 || b->total_faces < 0 || b->total_verts < 0 || b->total_norms < 0 ||
      b->total_uvs < 0)
    return RAST_ERR_INVALID_ARGUMENT;
  if (b->n_instances > 0 && (!b->meshes || !b->instances || !b->transforms || !b->local_scaling ||
                             !b->mesh_verts || !b->mesh_faces || !b->position))
    return RAST_ERR_INVALID_ARGUMENT;
  if (b->normal && (!b->mesh_norms || !b->mesh_faces_norm)) return RAST_ERR_INVALID_ARGUMENT;
  if ((b->uv || b->texture_index) && !b->mesh_faces_uv) return RAST_ERR_INVALID_ARGUMENT;
  if (b->uv && !b->mesh_uvs) return RAST_ERR_INVALID_ARGUMENT;
  return RAST_OK;
}

static int run(const RastMergeBatch* batch, void* workspace, size_t workspace_bytes, void* stream) {
  int st = check(batch);
  if (st != RAST_OK) return st;
  const RastMergeBatch& b = *batch;
  if (b.n_instances == 0) return RAST_OK;
  const Layout L = layout(b);
  if (workspace_bytes < L.total) return RAST_ERR_WORKSPACE_TOO_SMALL;
  if (workspace == nullptr || (reinterpret_cast<uintptr_t>(workspace) & 255)) return RAST_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  float* mesh_norm = reinterpret_cast<float*>(ws + L.norm_off);
  float* mpos = reinterpret_cast<float*>(ws + L.pos_off);
  int* mobj = reinterpret_cast<int*>(ws + L.obj_off);
  float* mnrm = b.normal ? reinterpret_cast<float*>(ws + L.nrm_off) : nullptr;
  float* muv = b.uv ? reinterpret_cast<float*>(ws + L.uv_off) : nullptr;
  const unsigned wg = static_cast<unsigned>((static_cast<int64_t>(b.n_instances) * 32 + kThreads - 1) / kThreads);
  if (b.n_meshes > 0 && b.normal)
    mesh_norm_kernel<<<static_cast<unsigned>((static_cast<int64_t>(b.n_meshes) * 32 + kThreads - 1) / kThreads),
                       kThreads, 0, s>>>(b, mesh_norm);
  instance_kernel<<<wg, kThreads, 0, s>>>(b, mesh_norm, mpos, mobj, mnrm, muv);
  corner_kernel<<<wg, kThreads, 0, s>>>(b, mpos, mobj, mnrm, muv);
  return cudaGetLastError() == cudaSuccess ? RAST_OK : RAST_ERR_CUDA;
}

}  // namespace merge
}  // namespace rast

using namespace rast;

extern "C" size_t rast_merge_workspace_bytes(const RastMergeBatch* batch) {
  if (!batch || merge::check(batch) != RAST_OK) return 0;
  return merge::layout(*batch).total;
}

extern "C" int rast_merge_objects(const RastMergeBatch* batch, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  rast::NvtxRange range("rast_merge_objects");
  return merge::run(batch, workspace, workspace_bytes, stream);
}
