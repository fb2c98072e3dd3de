// rast_shaders.cuh -- the seven built-in shaders of jaxrenderer as device
// functions: vertex stage (per-vertex clip position + varyings) and fragment
// stage (interpolated varyings -> keep flag + colour).  Same FP32 operation
// order as the reference files cited at each function.
#pragma once

#include "rast_math.cuh"

namespace rast {

// Varying layout per vertex.  Offsets within one vertex row.
constexpr int kVColour = 0;   // gouraud, gouraud_texture: colour (3)
constexpr int kVUvG = 3;      // gouraud_texture: uv (2)
constexpr int kVNormal = 0;   // phong family: eye-space normal (3)
constexpr int kVUv = 3;       // phong family: uv (2)
constexpr int kVTexIdx = 5;   // phong_reflection*: texture index (int bits)
constexpr int kVShadow = 6;   // phong_reflection_shadow: shadow_coord (4)
constexpr int kVTri = 5;      // phong_darboux: NDC triangle 3x3
constexpr int kVTriUv = 14;   // phong_darboux: uv triangle 3x2
constexpr int kMaxVarying = 20;

__host__ __device__ constexpr int varying_count(int shader) {
  return shader == RAST_SHADER_DEPTH ? 0
       : shader == RAST_SHADER_GOURAUD ? 3
       : shader == RAST_SHADER_GOURAUD_TEXTURE ? 5
       : shader == RAST_SHADER_PHONG ? 5
       : shader == RAST_SHADER_PHONG_DARBOUX ? 20
       : shader == RAST_SHADER_PHONG_REFLECTION ? 6
       : shader == RAST_SHADER_PHONG_REFLECTION_SHADOW ? 10
       : 0;
}

__device__ __forceinline__ void load3(const float* p, int64_t row, float* out) {
  out[0] = p[row * 3 + 0];
  out[1] = p[row * 3 + 1];
  out[2] = p[row * 3 + 2];
}

// Vertex shader of job J for vertex row `v` (0-based within the job).
// Writes gl_Position (clip, 4) and the shader's varyings (var).
// depth.py:47-61, gouraud.py:58-88, gouraud_texture.py:68-101,
// phong.py:78-104, phong_darboux.py:120-170, phong_reflection.py:104-132,
// phong_reflection_shadow.py:115-150.
// kClip = false skips gl_Position (the deferred shading re-run needs only
// the varyings).  SH >= 0: the job's shader, known at compile time (J.shader
// must equal it); otherwise read from the job.
template <bool kClip = true, int SH = -1>
__device__ __forceinline__ void vertex_shader(const RastJob& J, const RastPools& P, int v,
                                              float* clip, float* var) {
  const int64_t row = J.vert_begin + v;
  float pos[3];
  load3(P.position, row, pos);
  if (kClip) to_clip(J.world_to_clip, pos[0], pos[1], pos[2], clip);
  const int sh = SH >= 0 ? SH : J.shader;
  if (sh == RAST_SHADER_GOURAUD || sh == RAST_SHADER_GOURAUD_TEXTURE) {
    float nin[3], n[3], l[3];
    load3(P.normal, row, nin);
    normalise3(nin, n);
    normalise3(J.light_direction, l);
    const float intensity = dot3(n, l);
    if (sh == RAST_SHADER_GOURAUD) {
      float col[3];
      load3(P.colour, row, col);
#pragma unroll
      for (int c = 0; c < 3; ++c) var[kVColour + c] = (col[c] * J.light_colour[c]) * intensity;
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) var[kVColour + c] = J.light_colour[c] * intensity;
      var[kVUvG + 0] = P.uv[row * 2 + 0];
      var[kVUvG + 1] = P.uv[row * 2 + 1];
    }
  } else if (sh != RAST_SHADER_DEPTH) {
    float nin[3], n1[3];
    load3(P.normal, row, nin);
    normalise3(nin, n1);
    apply_vec(J.world_to_eye_norm, n1, var + kVNormal);
    var[kVUv + 0] = P.uv[row * 2 + 0];
    var[kVUv + 1] = P.uv[row * 2 + 1];
    if (sh == RAST_SHADER_PHONG_REFLECTION || sh == RAST_SHADER_PHONG_REFLECTION_SHADOW)
      var[kVTexIdx] = __int_as_float(P.texture_index[row]);
    if (sh == RAST_SHADER_PHONG_REFLECTION_SHADOW) {
      float sc[4];
      to_clip(J.shadow_world_to_clip, pos[0], pos[1], pos[2], sc);
      const float w = sc[3];
#pragma unroll
      for (int c = 0; c < 4; ++c) var[kVShadow + c] = sc[c] / w;
    }
    if (sh == RAST_SHADER_PHONG_DARBOUX) {
      const int fid = gather_clamp(P.id_to_face[row], J.n_darboux_faces);
      const int32_t* f = P.darboux_faces + (J.darboux_face_begin + fid) * 3;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int vk = gather_clamp(f[k], J.n_verts);
        const int64_t rk = J.vert_begin + vk;
        float pk[3], tc[4];
        load3(P.position, rk, pk);
        to_clip(J.world_to_clip, pk[0], pk[1], pk[2], tc);
#pragma unroll
        for (int c = 0; c < 3; ++c)  // to_cartesian (geometry.py:185-202)
          var[kVTri + 3 * k + c] = (tc[3] == 0.0f) ? tc[c] : tc[c] / tc[3];
        var[kVTriUv + 2 * k + 0] = P.uv[rk * 2 + 0];
        var[kVTriUv + 2 * k + 1] = P.uv[rk * 2 + 1];
      }
    }
  }
}

__device__ __forceinline__ float interp1(const float* b, float v0, float v1, float v2) {
  return (b[0] * v0 + b[1] * v1) + b[2] * v2;
}

// Texel of a (w, h, ch) map with default-mode gather indexing.
__device__ __forceinline__ void texel3(const float* tex, int w, int h, int ch, int u, int v,
                                       float* out) {
  u = gather_clamp(u, w);
  v = gather_clamp(v, h);
  const float* t = tex + (static_cast<int64_t>(u) * h + v) * ch;
  if (ch == 1) {
    out[0] = out[1] = out[2] = __ldg(t);
  } else {
    out[0] = __ldg(t + 0);
    out[1] = __ldg(t + 1);
    out[2] = __ldg(t + 2);
  }
}

// Fragment stage of the chosen primitive: Shader.interpolate then
// Shader.fragment.  v0/v1/v2 are the three vertex varying rows, b the
// perspective-correct barycentrics (true_clip_coef, pipeline.py:241).
// Returns the shader's keep (AND-ed by the caller with the chooser's keep).
__device__ __forceinline__ bool fragment_shader(const RastJob& J, const RastPools& P,
                                                const float* v0, const float* v1,
                                                const float* v2, const float* b, bool front,
                                                float* colour) {
  const int sh = J.shader;
  switch (sh) {
    case RAST_SHADER_DEPTH:  // shader.py:333
      return true;
    case RAST_SHADER_GOURAUD: {  // gouraud.py:94-124
      bool ok = front;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        colour[c] = interp1(b, v0[kVColour + c], v1[kVColour + c], v2[kVColour + c]);
        ok = ok && (colour[c] >= 0.0f);
      }
      return ok;
    }
    case RAST_SHADER_GOURAUD_TEXTURE: {  // gouraud_texture.py:107-144
      const float u = interp1(b, v0[kVUvG], v1[kVUvG], v2[kVUvG]);
      const float w = interp1(b, v0[kVUvG + 1], v1[kVUvG + 1], v2[kVUvG + 1]);
      const int ui = pymod(f2i(floorf(u)), J.tex_w);
      const int wi = pymod(f2i(floorf(w)), J.tex_h);
      float tc[3];
      texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
      bool ok = front;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float lc = interp1(b, v0[kVColour + c], v1[kVColour + c], v2[kVColour + c]);
        ok = ok && (lc >= 0.0f);
        colour[c] = tc[c] * lc;
      }
      return ok;
    }
    case RAST_SHADER_PHONG:
    case RAST_SHADER_PHONG_DARBOUX: {  // phong.py:110-164, phong_darboux.py:212-293
      float nrm[3], n[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) nrm[c] = interp1(b, v0[kVNormal + c], v1[kVNormal + c], v2[kVNormal + c]);
      const float u = interp1(b, v0[kVUv], v1[kVUv], v2[kVUv]);
      const float w = interp1(b, v0[kVUv + 1], v1[kVUv + 1], v2[kVUv + 1]);
      const int ui = pymod(f2i(floorf(u)), J.tex_w);
      const int wi = pymod(f2i(floorf(w)), J.tex_h);
      normalise3(nrm, n);
      if (sh == RAST_SHADER_PHONG_DARBOUX) {
        const float* t = v0 + kVTri;     // vertex 0's triangle, not interpolated
        const float* tu = v0 + kVTriUv;
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
        normalise3(vi, ni);
        normalise3(vj, nj);
        float nm[3], bn[3];
        texel3(P.normal_map + J.normal_map_begin, J.nm_w, J.nm_h, 3, ui, wi, nm);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const float row[3] = {ni[r], nj[r], n[r]};
          bn[r] = dot3(row, nm);
        }
        normalise3(bn, n);
      }
      float tc[3], l[3], lc[3];
      texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
      normalise3(J.light_direction, l);
      const float d = dot3(n, l);
      bool nonneg = true;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        lc[c] = J.light_colour[c] * d;
        nonneg = nonneg && (lc[c] >= 0.0f);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) colour[c] = nonneg ? tc[c] * lc[c] : 0.0f;
      return front;
    }
    case RAST_SHADER_PHONG_REFLECTION:
    case RAST_SHADER_PHONG_REFLECTION_SHADOW: {
      // phong_reflection.py:158-235, phong_reflection_shadow.py:178-271
      const bool shadowed = sh == RAST_SHADER_PHONG_REFLECTION_SHADOW;
      float shadow[3] = {1.0f, 1.0f, 1.0f};
      if (shadowed) {
        float scv[4], sc[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) scv[c] = interp1(b, v0[kVShadow + c], v1[kVShadow + c], v2[kVShadow + c]);
        apply4(J.shadow_viewport, scv, sc);
        const float sw = sc[3];
#pragma unroll
        for (int c = 0; c < 4; ++c) sc[c] = sc[c] / sw;
        // Shadow.get (shadow.py:129-153): round half away from zero, wrap
        // negatives once, out of bounds reads +inf.
        int px = f2i(roundf(sc[0]));
        int py = f2i(roundf(sc[1]));
        if (px < 0) px += J.shadow_w;
        if (py < 0) py += J.shadow_h;
        float depth = kInf;
        if (px >= 0 && px < J.shadow_w && py >= 0 && py < J.shadow_h)
          depth = __ldg(P.shadow_map + J.shadow_begin + static_cast<int64_t>(px) * J.shadow_h + py);
        const bool lit = sc[2] <= depth;
#pragma unroll
        for (int c = 0; c < 3; ++c) shadow[c] = lit ? 1.0f : 1.0f - J.shadow_strength[c];
      }
      // MergedModel.uv_repeat (model.py:306-339)
      const int texidx = __float_as_int(v0[kVTexIdx]);
      const int ti = gather_clamp(texidx, J.n_objects);
      const int32_t* shp = P.texture_shape + (J.texture_shape_begin + ti) * 2;
      float uvr[2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const float x = interp1(b, v0[kVUv + a], v1[kVUv + a], v2[kVUv + a]);
        const float whole = (x >= 0.0f) ? floorf(x) : ceilf(x);
        float frac = x - whole;
        if (frac < 0.0f) frac = frac + 1.0f;
        uvr[a] = frac * static_cast<float>(shp[a]);
      }
      uvr[0] = uvr[0] + static_cast<float>(texidx * J.texture_offset);
      const int ui = f2i(floorf(uvr[0]));
      const int wi = f2i(floorf(uvr[1]));
      float tc[3], nrm[3], n[3], l[3], r[3], rn[3];
      texel3(P.texture + J.texture_begin, J.tex_w, J.tex_h, J.tex_c, ui, wi, tc);
#pragma unroll
      for (int c = 0; c < 3; ++c) nrm[c] = interp1(b, v0[kVNormal + c], v1[kVNormal + c], v2[kVNormal + c]);
      normalise3(nrm, n);
      normalise3(J.light_dir_eye, l);
      const float d = dot3(n, l);
      const float dif = max0(d);
#pragma unroll
      for (int c = 0; c < 3; ++c) r[c] = ((2.0f * d) * n[c]) - l[c];
      normalise3(r, rn);
      const int su = gather_clamp(ui, J.spec_w), sv = gather_clamp(wi, J.spec_h);
      const float spec = powf(max0(rn[2]),
                              __ldg(P.specular_map + J.specular_begin + static_cast<int64_t>(su) * J.spec_h + sv));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float a = J.ambient[c] * tc[c];
        const float k = J.diffuse[c] * dif + J.specular[c] * spec;
        const float bb = shadowed ? ((shadow[c] * k) * tc[c]) * J.light_colour[c]
                                  : (k * J.light_colour[c]) * tc[c];
        colour[c] = a + bb;
      }
      return front;
    }
    default:
      return false;
  }
}

}  // namespace rast
