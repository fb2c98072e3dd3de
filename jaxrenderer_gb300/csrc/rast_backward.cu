// rast_backward.cu -- hand-written reverse mode of the rasterisation path.
//
// Visibility is piecewise constant (as under jax.grad of the reference): the
// forward's winning-primitive buffer is saved, and for every pixel whose
// fragment was kept one thread re-runs that pixel's forward for the winning
// face (vertex shader of its three corners, 3x3 inverse, barycentrics,
// fragment) and propagates dL/dcanvas and dL/dzbuffer back through
//   fragment shader -> perspective-correct interpolation -> barycentrics
//   (true_clip_coef = c / sum(c), c = [x, y, 1] @ inv(M)) -> 3x3 inverse
//   -> clip positions -> world_to_clip and vertex positions,
// and through the vertex normal transform (world_to_eye_norm).  Texel
// lookups are nearest, so uv gets no gradient (floor), the sampled texel and
// specular exponent do (scatter-add).  The shadow-map comparison is a step:
// no gradient reaches the depth pass.  Per-vertex, per-texel results are
// accumulated with atomics; per-scene camera and light gradients are
// reduced per block and added once per block.
#include <cuda_runtime.h>

#include "rast_internal.cuh"

namespace rast {
namespace bwd {

constexpr int kThreads = 256;

// y = v / |v|;  dv = (dy - y (y . dy)) / |v|
__device__ __forceinline__ void normalise3_bwd(const float* y, float norm, const float* dy, float* dv) {
  const float s = (y[0] * dy[0] + y[1] * dy[1]) + y[2] * dy[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) dv[k] = (dy[k] - y[k] * s) / norm;
}

__device__ __forceinline__ float norm3(const float* v) {
  return sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
}

// d max(x, 0) / dx as lax.max's derivative: 1 above, 0 below, 1/2 at the tie.
__device__ __forceinline__ float dmax0(float x) { return x > 0.0f ? 1.0f : (x == 0.0f ? 0.5f : 0.0f); }

// Per-pixel accumulator of per-scene parameter gradients (RAST_GRAD_*).
struct ParamGrad {
  float v[RAST_NPARAM];
};

__device__ __forceinline__ void texel_index(const RastJob& J, int u, int w, int64_t* base, int* ch) {
  u = gather_clamp(u, J.tex_w);
  w = gather_clamp(w, J.tex_h);
  *base = J.texture_begin + (static_cast<int64_t>(u) * J.tex_h + w) * J.tex_c;
  *ch = J.tex_c;
}

__device__ __forceinline__ void add_texel_grad(float* g, int64_t base, int ch, const float* d) {
  if (!g) return;
  if (ch == 1) atomicAdd(g + base, (d[0] + d[1]) + d[2]);
  else {
    atomicAdd(g + base + 0, d[0]);
    atomicAdd(g + base + 1, d[1]);
    atomicAdd(g + base + 2, d[2]);
  }
}

// Per-scene parameters a shader's backward can touch (bit k = RAST_GRAD index k).
__host__ __device__ constexpr unsigned long long range_bits(int lo, int n) {
  return ((n >= 64 ? ~0ull : ((1ull << n) - 1ull)) << lo);
}
__host__ __device__ constexpr unsigned long long param_bits(int sh) {
  return sh == RAST_SHADER_DEPTH ? range_bits(RAST_GRAD_WORLD_TO_CLIP, 16)
       : (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE)
           ? range_bits(RAST_GRAD_WORLD_TO_CLIP, 16) | range_bits(RAST_GRAD_LIGHT_DIRECTION, 6)
       : sh == RAST_SHADER_PHONG
           ? range_bits(RAST_GRAD_WORLD_TO_CLIP, 32) | range_bits(RAST_GRAD_LIGHT_DIRECTION, 6)
       : (sh == RAST_SHADER_PHONG_REFLECTION || sh == RAST_SHADER_PHONG_REFLECTION_SHADOW)
           ? range_bits(RAST_GRAD_WORLD_TO_CLIP, 32) | range_bits(RAST_GRAD_LIGHT_COLOUR, 18)
       : range_bits(0, RAST_NPARAM);
}

// SH: the shader of every job of the launch, or -1 for a batch that mixes
// shaders (every path compiled in, selected per job).
template <int SH>
__global__ void __launch_bounds__(kThreads, 2)
backward_kernel(RastBatch B, const float* __restrict__ grad_canvas, const float* __restrict__ grad_zbuffer,
                RastGradPools G) {
  __shared__ RastJob sJ;
  __shared__ float s_red[kThreads / 32][RAST_NPARAM];
  load_job_to_shared(B.jobs + blockIdx.y, &sJ);
  __syncthreads();
  const RastJob& J = sJ;
  const RastPools& P = B.pools;
  const int64_t npix = static_cast<int64_t>(J.width) * J.height;
  const int64_t local = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  ParamGrad pg;
#pragma unroll
  for (int k = 0; k < RAST_NPARAM; ++k) pg.v[k] = 0.0f;
  const int sh = SH >= 0 ? SH : J.shader;
  bool active = local < npix && J.n_faces > 0;
  int p = -1;
  int64_t pix = 0;
  if (active) {
    pix = J.pixel_begin + local;
    p = P.prim_id[pix];
    active = p >= 0;
  }
  if (active) {
    const int i = static_cast<int>(local / J.height), j = static_cast<int>(local % J.height);
    const float x = (static_cast<float>(i) - J.viewport[3]) / J.viewport[0];
    const float y = (static_cast<float>(j) - J.viewport[7]) / J.viewport[5];
    const int32_t* face = P.faces + (J.face_begin + p) * 3;
    int vid[3];
    float pos[3][3], clip[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      vid[k] = gather_clamp(face[k], J.n_verts);
      load3(P.position, J.vert_begin + vid[k], pos[k]);
      to_clip(J.world_to_clip, pos[k][0], pos[k][1], pos[k][2], clip[k]);
    }
    const float M[9] = {clip[0][0], clip[0][1], clip[0][3], clip[1][0], clip[1][1], clip[1][3],
                        clip[2][0], clip[2][1], clip[2][3]};
    float m[9];
    inv3(M, m);
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = (x * m[k] + y * m[3 + k]) + m[6 + k];
    const float w = (c[0] + c[1]) + c[2];
    const float b[3] = {c[0] / w, c[1] / w, c[2] / w};
    float gb[3] = {0.0f, 0.0f, 0.0f};  // dL/d barycentrics
    float gc[3] = {0.0f, 0.0f, 0.0f};  // dL/d clip_coef (direct, from depth)
    float gclip[3][4] = {};            // dL/d clip positions
    float gpos[3][3] = {};             // dL/d world positions (besides the clip path)
    float gnorm[3][3] = {};            // dL/d world normals
    float gcol[3][3] = {};             // dL/d vertex colours (gouraud)

    // ---- depth output: z = (sum c_k z_k) * vp22 + vp23
    const float gz = grad_zbuffer ? grad_zbuffer[pix] : 0.0f;
    if (gz != 0.0f) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gc[k] += gz * J.viewport[10] * clip[k][2];
        gclip[k][2] += gz * J.viewport[10] * c[k];
      }
    }
    const float gcv[3] = {grad_canvas ? grad_canvas[pix * 3 + 0] : 0.0f,
                          grad_canvas ? grad_canvas[pix * 3 + 1] : 0.0f,
                          grad_canvas ? grad_canvas[pix * 3 + 2] : 0.0f};
    const bool has_colour = sh != RAST_SHADER_DEPTH && (gcv[0] != 0.0f || gcv[1] != 0.0f || gcv[2] != 0.0f);

    if (has_colour && (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE)) {
      // vertex: colour_k = (C_k * lc) * (n_k . l), n_k = N_k/|N_k|, l = L/|L|
      float ld[3], l[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) ld[q] = J.light_direction[q];
      const float ln = norm3(ld);
      normalise3(ld, l);
      float n[3][3], nn[3], inten[3], vc[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float N[3];
        load3(P.normal, J.vert_begin + vid[k], N);
        nn[k] = norm3(N);
        normalise3(N, n[k]);
        inten[k] = dot3(n[k], l);
        if (sh == RAST_SHADER_GOURAUD) load3(P.colour, J.vert_begin + vid[k], vc[k]);
      }
      float gvert[3][3];  // dL/d interpolated-varying colour at each corner
      float gtex_out[3] = {0.0f, 0.0f, 0.0f};
      float lcol[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) lcol[q] = interp1(b, (sh == RAST_SHADER_GOURAUD ? (vc[0][q] * J.light_colour[q]) * inten[0] : J.light_colour[q] * inten[0]),
                                                  (sh == RAST_SHADER_GOURAUD ? (vc[1][q] * J.light_colour[q]) * inten[1] : J.light_colour[q] * inten[1]),
                                                  (sh == RAST_SHADER_GOURAUD ? (vc[2][q] * J.light_colour[q]) * inten[2] : J.light_colour[q] * inten[2]));
      float glc[3];  // dL/d interpolated colour
      if (sh == RAST_SHADER_GOURAUD) {
#pragma unroll
        for (int q = 0; q < 3; ++q) glc[q] = gcv[q];
      } else {
        const float u = interp1(b, P.uv[(J.vert_begin + vid[0]) * 2], P.uv[(J.vert_begin + vid[1]) * 2], P.uv[(J.vert_begin + vid[2]) * 2]);
        const float v = interp1(b, P.uv[(J.vert_begin + vid[0]) * 2 + 1], P.uv[(J.vert_begin + vid[1]) * 2 + 1], P.uv[(J.vert_begin + vid[2]) * 2 + 1]);
        const int ui = pymod(f2i(floorf(u)), J.tex_w), wi = pymod(f2i(floorf(v)), J.tex_h);
        int64_t tb;
        int ch;
        texel_index(J, ui, wi, &tb, &ch);
        float tc[3];
        texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          glc[q] = gcv[q] * tc[q];
          gtex_out[q] = gcv[q] * lcol[q];
        }
        add_texel_grad(G.texture, tb, ch, gtex_out);
      }
      // interpolation: value = sum_k b_k v_k
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float vk[3] = {sh == RAST_SHADER_GOURAUD ? (vc[k][0] * J.light_colour[0]) * inten[k] : J.light_colour[0] * inten[k],
                             sh == RAST_SHADER_GOURAUD ? (vc[k][1] * J.light_colour[1]) * inten[k] : J.light_colour[1] * inten[k],
                             sh == RAST_SHADER_GOURAUD ? (vc[k][2] * J.light_colour[2]) * inten[k] : J.light_colour[2] * inten[k]};
        gb[k] += dot3(glc, vk);
#pragma unroll
        for (int q = 0; q < 3; ++q) gvert[k][q] = b[k] * glc[q];
      }
      float gl[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float ginten = 0.0f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const float base = sh == RAST_SHADER_GOURAUD ? vc[k][q] * J.light_colour[q] : J.light_colour[q];
          ginten += gvert[k][q] * base;
          if (sh == RAST_SHADER_GOURAUD) {
            gcol[k][q] += gvert[k][q] * J.light_colour[q] * inten[k];
            pg.v[RAST_GRAD_LIGHT_COLOUR + q] += gvert[k][q] * vc[k][q] * inten[k];
          } else {
            pg.v[RAST_GRAD_LIGHT_COLOUR + q] += gvert[k][q] * inten[k];
          }
        }
        float gn[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          gn[q] = ginten * l[q];
          gl[q] += ginten * n[k][q];
        }
        float N[3], gN[3];
        load3(P.normal, J.vert_begin + vid[k], N);
        normalise3_bwd(n[k], nn[k], gn, gN);
#pragma unroll
        for (int q = 0; q < 3; ++q) gnorm[k][q] += gN[q];
      }
      float gL[3];
      normalise3_bwd(l, ln, gl, gL);
#pragma unroll
      for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIRECTION + q] += gL[q];
    } else if (has_colour) {
      // phong family: per-corner eye-space normals n_k = apply_vec(E, N_k/|N_k|)
      float n1[3][3], n1n[3], n2[3][3], n2n[3], h[3][3], hn[3], ne[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float N[3];
        load3(P.normal, J.vert_begin + vid[k], N);
        n1n[k] = norm3(N);
        normalise3(N, n1[k]);
        n2n[k] = norm3(n1[k]);
        normalise3(n1[k], n2[k]);
        const float hh[4] = {n2[k][0], n2[k][1], n2[k][2], 0.0f};
        float t4[4];
        apply4(J.world_to_eye_norm, hh, t4);
        h[k][0] = t4[0];
        h[k][1] = t4[1];
        h[k][2] = t4[2];
        hn[k] = norm3(h[k]);
        normalise3(h[k], ne[k]);
      }
      float nrm[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) nrm[q] = interp1(b, ne[0][q], ne[1][q], ne[2][q]);
      const float nrmn = norm3(nrm);
      float n[3];
      normalise3(nrm, n);
      float gn[3] = {0.0f, 0.0f, 0.0f};
      if (sh == RAST_SHADER_PHONG) {
        // colour = all(lc >= 0) ? tex * lc : 0,  lc = light_colour * (n . l)
        const float u = interp1(b, P.uv[(J.vert_begin + vid[0]) * 2], P.uv[(J.vert_begin + vid[1]) * 2], P.uv[(J.vert_begin + vid[2]) * 2]);
        const float v = interp1(b, P.uv[(J.vert_begin + vid[0]) * 2 + 1], P.uv[(J.vert_begin + vid[1]) * 2 + 1], P.uv[(J.vert_begin + vid[2]) * 2 + 1]);
        const int ui = pymod(f2i(floorf(u)), J.tex_w), wi = pymod(f2i(floorf(v)), J.tex_h);
        float tc[3], ld[3], l[3];
        texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
#pragma unroll
        for (int q = 0; q < 3; ++q) ld[q] = J.light_direction[q];
        const float ln = norm3(ld);
        normalise3(ld, l);
        const float d = dot3(n, l);
        float lc[3];
        bool nonneg = true;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          lc[q] = J.light_colour[q] * d;
          nonneg = nonneg && lc[q] >= 0.0f;
        }
        if (nonneg) {
          int64_t tb;
          int ch;
          texel_index(J, ui, wi, &tb, &ch);
          float gt[3];
          float gd = 0.0f;
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            gt[q] = gcv[q] * lc[q];
            const float glc = gcv[q] * tc[q];
            pg.v[RAST_GRAD_LIGHT_COLOUR + q] += glc * d;
            gd += glc * J.light_colour[q];
          }
          add_texel_grad(G.texture, tb, ch, gt);
          float gl[3], gL[3];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            gn[q] = gd * l[q];
            gl[q] = gd * n[q];
          }
          normalise3_bwd(l, ln, gl, gL);
#pragma unroll
          for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIRECTION + q] += gL[q];
        }
      } else if (sh == RAST_SHADER_PHONG_REFLECTION || sh == RAST_SHADER_PHONG_REFLECTION_SHADOW) {
        const bool shadowed = sh == RAST_SHADER_PHONG_REFLECTION_SHADOW;
        float v0[kMaxVarying], v1[kMaxVarying], v2[kMaxVarying], dummy[4];
        vertex_shader<false>(J, P, vid[0], dummy, v0);
        vertex_shader<false>(J, P, vid[1], dummy, v1);
        vertex_shader<false>(J, P, vid[2], dummy, v2);
        float shadow[3] = {1.0f, 1.0f, 1.0f};
        bool lit = true;
        if (shadowed) {
          float scv[4], sc[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) scv[q] = interp1(b, v0[kVShadow + q], v1[kVShadow + q], v2[kVShadow + q]);
          apply4(J.shadow_viewport, scv, sc);
          const float sw = sc[3];
#pragma unroll
          for (int q = 0; q < 4; ++q) sc[q] = sc[q] / sw;
          int px = f2i(roundf(sc[0])), py = f2i(roundf(sc[1]));
          if (px < 0) px += J.shadow_w;
          if (py < 0) py += J.shadow_h;
          float depth = kInf;
          if (px >= 0 && px < J.shadow_w && py >= 0 && py < J.shadow_h)
            depth = P.shadow_map[J.shadow_begin + static_cast<int64_t>(px) * J.shadow_h + py];
          lit = sc[2] <= depth;
#pragma unroll
          for (int q = 0; q < 3; ++q) shadow[q] = lit ? 1.0f : 1.0f - J.shadow_strength[q];
        }
        const int texidx = __float_as_int(v0[kVTexIdx]);
        const int ti = gather_clamp(texidx, J.n_objects);
        const int32_t* shp = P.texture_shape + (J.texture_shape_begin + ti) * 2;
        float uvr[2];
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          const float xx = interp1(b, v0[kVUv + a], v1[kVUv + a], v2[kVUv + a]);
          const float whole = (xx >= 0.0f) ? floorf(xx) : ceilf(xx);
          float frac = xx - whole;
          if (frac < 0.0f) frac = frac + 1.0f;
          uvr[a] = frac * static_cast<float>(shp[a]);
        }
        uvr[0] = uvr[0] + static_cast<float>(texidx * J.texture_offset);
        const int ui = f2i(floorf(uvr[0])), wi = f2i(floorf(uvr[1]));
        float tc[3], l[3];
        texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
        const float ln = norm3(J.light_dir_eye);
        normalise3(J.light_dir_eye, l);
        const float d = dot3(n, l);
        const float dif = max0(d);
        float r[3], rn[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) r[q] = ((2.0f * d) * n[q]) - l[q];
        const float rnorm = norm3(r);
        normalise3(r, rn);
        const int su = gather_clamp(ui, J.spec_w), sv = gather_clamp(wi, J.spec_h);
        const int64_t sidx = J.specular_begin + static_cast<int64_t>(su) * J.spec_h + sv;
        const float sexp = P.specular_map[sidx];
        const float rz = max0(rn[2]);
        const float spec = powf(rz, sexp);
        float gdif = 0.0f, gspec = 0.0f, gt[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const float K = J.diffuse[q] * dif + J.specular[q] * spec;
          const float lc = J.light_colour[q];
          // colour = amb*tex + shadow*K*tex*lc (either product order)
          gt[q] = gcv[q] * (J.ambient[q] + shadow[q] * K * lc);
          pg.v[RAST_GRAD_AMBIENT + q] += gcv[q] * tc[q];
          const float gK = gcv[q] * shadow[q] * tc[q] * lc;
          pg.v[RAST_GRAD_DIFFUSE + q] += gK * dif;
          pg.v[RAST_GRAD_SPECULAR + q] += gK * spec;
          pg.v[RAST_GRAD_LIGHT_COLOUR + q] += gcv[q] * shadow[q] * K * tc[q];
          if (!lit) pg.v[RAST_GRAD_SHADOW_STRENGTH + q] -= gcv[q] * K * tc[q] * lc;
          gdif += gK * J.diffuse[q];
          gspec += gK * J.specular[q];
        }
        int64_t tb;
        int ch;
        texel_index(J, ui, wi, &tb, &ch);
        add_texel_grad(G.texture, tb, ch, gt);
        // spec = rz ** s  (jax: d/dx = s x^(s-1) (0 when s == 0), d/ds = log(x) x^s with log(0) -> 0)
        if (G.specular_map && rz > 0.0f) atomicAdd(G.specular_map + sidx, gspec * spec * logf(rz));
        const float dspec_drz = (sexp == 0.0f) ? 0.0f : sexp * powf(rz, sexp - 1.0f);
        float grn[3] = {0.0f, 0.0f, gspec * dspec_drz * dmax0(rn[2])};
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
        float gLe[3];
        normalise3_bwd(l, ln, gl, gLe);
#pragma unroll
        for (int q = 0; q < 3; ++q) pg.v[RAST_GRAD_LIGHT_DIR_EYE + q] += gLe[q];
      }
      // n = normalise(nrm), nrm = sum_k b_k ne_k
      float gnrm[3];
      normalise3_bwd(n, nrmn, gn, gnrm);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gb[k] += dot3(gnrm, ne[k]);
        float gne[3], gh[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) gne[q] = b[k] * gnrm[q];
        normalise3_bwd(ne[k], hn[k], gne, gh);
        // h = E[:3, :3] n2 (+ E[:3, 3] * 0)
        float gn2[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            pg.v[RAST_GRAD_WORLD_TO_EYE_NORM + 4 * r + q] += gh[r] * n2[k][q];
            gn2[q] += gh[r] * J.world_to_eye_norm[4 * r + q];
          }
        float gn1[3], gN[3];
        normalise3_bwd(n2[k], n2n[k], gn2, gn1);
        normalise3_bwd(n1[k], n1n[k], gn1, gN);
#pragma unroll
        for (int q = 0; q < 3; ++q) gnorm[k][q] += gN[q];
      }
    }

    // ---- barycentrics b = c / w, w = sum c
    const float sb_ = (gb[0] * b[0] + gb[1] * b[1]) + gb[2] * b[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) gc[k] += (gb[k] - sb_) / w;
    // ---- c_k = x m[k] + y m[3+k] + m[6+k]  ->  dL/dm
    const float xy1[3] = {x, y, 1.0f};
    float gm[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) gm[3 * r + k] = xy1[r] * gc[k];
    // ---- m = M^-1  ->  dL/dM = -m^T gm m^T
    float t[9], gM[9];
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
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      gclip[k][0] += gM[3 * k + 0];
      gclip[k][1] += gM[3 * k + 1];
      gclip[k][3] += gM[3 * k + 2];
    }
    // ---- clip_k = A [p_k, 1]
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float ph[4] = {pos[k][0], pos[k][1], pos[k][2], 1.0f};
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) pg.v[RAST_GRAD_WORLD_TO_CLIP + 4 * r + q] += gclip[k][r] * ph[q];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        gpos[k][q] += ((gclip[k][0] * J.world_to_clip[q] + gclip[k][1] * J.world_to_clip[4 + q]) +
                       gclip[k][2] * J.world_to_clip[8 + q]) + gclip[k][3] * J.world_to_clip[12 + q];
    }
    // ---- scatter per-vertex gradients
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int64_t row = J.vert_begin + vid[k];
      if (G.position)
#pragma unroll
        for (int q = 0; q < 3; ++q) atomicAdd(G.position + row * 3 + q, gpos[k][q]);
      if (G.normal && sh != RAST_SHADER_DEPTH)
#pragma unroll
        for (int q = 0; q < 3; ++q) atomicAdd(G.normal + row * 3 + q, gnorm[k][q]);
      if (G.colour && sh == RAST_SHADER_GOURAUD)
#pragma unroll
        for (int q = 0; q < 3; ++q) atomicAdd(G.colour + row * 3 + q, gcol[k][q]);
    }
  }
  // ---- per-scene parameter gradients: warp then block reduction
  if (G.job_params) {
    constexpr unsigned long long bits = param_bits(SH);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < RAST_NPARAM; ++k) {
      if (!((bits >> k) & 1ull)) {
        if (lane == 0) s_red[warp][k] = 0.0f;
        continue;
      }
      float v = pg.v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < RAST_NPARAM) {
      float v = 0.0f;
#pragma unroll
      for (int w8 = 0; w8 < kThreads / 32; ++w8) v += s_red[w8][threadIdx.x];
      if (v != 0.0f) atomicAdd(G.job_params + static_cast<int64_t>(blockIdx.y) * RAST_NPARAM + threadIdx.x, v);
    }
  }
}

}  // namespace bwd
}  // namespace rast

using namespace rast;

extern "C" int rast_backward(const RastBatch* batch, const float* grad_canvas, const float* grad_zbuffer,
                             const RastGradPools* grads, void* stream) {
  int st = check_batch(batch);
  if (st != RAST_OK) return st;
  if (!grads || !batch->pools.prim_id) return RAST_ERR_INVALID_ARGUMENT;
  if (batch->shader_mask & (1 << RAST_SHADER_PHONG_DARBOUX)) return RAST_ERR_UNSUPPORTED;
  const RastBatch& b = *batch;
  if (b.total_pixels == 0) return RAST_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t max_px = static_cast<int64_t>(b.max_width) * b.max_height;
  const dim3 grid(static_cast<unsigned>((max_px + bwd::kThreads - 1) / bwd::kThreads), static_cast<unsigned>(b.n_jobs));
  const int mask = b.shader_mask;
  auto only = [&](int sh) { return mask == (1 << sh); };
  if (only(RAST_SHADER_DEPTH))
    bwd::backward_kernel<RAST_SHADER_DEPTH><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else if (only(RAST_SHADER_GOURAUD))
    bwd::backward_kernel<RAST_SHADER_GOURAUD><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else if (only(RAST_SHADER_GOURAUD_TEXTURE))
    bwd::backward_kernel<RAST_SHADER_GOURAUD_TEXTURE><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else if (only(RAST_SHADER_PHONG))
    bwd::backward_kernel<RAST_SHADER_PHONG><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else if (only(RAST_SHADER_PHONG_REFLECTION))
    bwd::backward_kernel<RAST_SHADER_PHONG_REFLECTION><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else if (only(RAST_SHADER_PHONG_REFLECTION_SHADOW))
    bwd::backward_kernel<RAST_SHADER_PHONG_REFLECTION_SHADOW><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  else
    bwd::backward_kernel<-1><<<grid, bwd::kThreads, 0, s>>>(b, grad_canvas, grad_zbuffer, *grads);
  return cudaGetLastError() == cudaSuccess ? RAST_OK : RAST_ERR_CUDA;
}
