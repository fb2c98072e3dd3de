/*
 * rast_oracle.c -- TEST INFRASTRUCTURE ONLY (see rast_oracle.h).
 *
 * CPU restatement of jaxrenderer's pipeline, compiled with
 * -ffp-contract=off so every multiply and add rounds separately, as the
 * reference's operation order states them.  Compiled twice: OR_DOUBLE=0
 * gives the float checker (suffix _f32), OR_DOUBLE=1 gives the
 * finite-difference twin (suffix _f64).  Citations are file:line in the
 * reference project (JoeyTeng/jaxrenderer v0.3.2).
 */
#include "rast_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef OR_DOUBLE
#define OR_DOUBLE 0
#endif

#if OR_DOUBLE
typedef double real;
#define R_SQRT sqrt
#define R_FLOOR floor
#define R_CEIL ceil
#define R_ROUND round
#define R_POW pow
#define R_FABS fabs
#define R_MIN_NORMAL DBL_MIN
#define R_MAX DBL_MAX
#define SUF(n) n##_f64
#else
typedef float real;
#define R_SQRT sqrtf
#define R_FLOOR floorf
#define R_CEIL ceilf
#define R_ROUND roundf
#define R_POW powf
#define R_FABS fabsf
#define R_MIN_NORMAL FLT_MIN
#define R_MAX FLT_MAX
#define SUF(n) n##_f32
#endif

/* Scene struct with `real` fields; identical layout to OrSceneF32 when real
 * is float. */
typedef struct Scene {
  int shader;
  int width, height;
  int n_threads;
  const real* viewport;
  const real* world_to_clip;
  const real* world_to_eye_norm;
  int n_verts;
  const real* position;
  const real* normal;
  const real* uv;
  const real* colour;
  const int* texture_index;
  const int* id_to_face;
  const int* darboux_faces;
  int n_darboux_faces;
  int n_faces;
  const int* faces;
  real light_direction[3];
  real light_colour[3];
  real light_dir_eye[3];
  real ambient[3];
  real diffuse[3];
  real specular[3];
  const real* texture; int tex_w, tex_h, tex_c;
  const real* specular_map; int spec_w, spec_h;
  const real* normal_map; int nm_w, nm_h;
  const int* texture_shape; int n_objects; int texture_offset;
  const real* shadow_map; int shadow_w, shadow_h;
  const real* shadow_world_to_clip;
  const real* shadow_viewport;
  real shadow_strength[3];
  real* zbuffer;
  real* canvas;
  int* prim_id;
  long long near_ties;
  int layers;
  int mixer;
  real opacity;
  real background[3];
  const real* face_alpha;
  int x_begin, x_end, y_begin, y_end;
  int* branch;
  int* texel;
} Scene;

/* ---------------------------------------------------------------- basics */

/* Sum of products in index order, one rounding per operation:
 * lax.dot_general over a length-3 contraction (geometry.py:104-108). */
static inline real dot3(const real* a, const real* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

/* normalise (geometry.py:39-47): v / jnp.linalg.norm(v). */
static inline void normalise3(const real* v, real* out) {
  real n = R_SQRT((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  out[0] = v[0] / n;
  out[1] = v[1] / n;
  out[2] = v[2] / n;
}

/* Camera.apply (geometry.py:284-315): out[i] = sum_k p[k] * M[i][k]. */
static inline void apply4(const real* m, const real* p, real* out) {
  for (int i = 0; i < 4; ++i)
    out[i] = ((p[0] * m[4 * i + 0] + p[1] * m[4 * i + 1]) + p[2] * m[4 * i + 2]) +
             p[3] * m[4 * i + 3];
}

/* Camera.to_clip of to_homogeneous(position) (geometry.py:144-163, 420-438). */
static inline void to_clip(const real* m, const real* pos3, real* out) {
  real p[4] = {pos3[0], pos3[1], pos3[2], (real)1};
  apply4(m, p, out);
}

/* Camera.apply_vec (geometry.py:352-389): normalise, w=0, transform, drop w,
 * normalise. */
static inline void apply_vec(const real* m, const real* v, real* out) {
  real n[3];
  normalise3(v, n);
  real h[4] = {n[0], n[1], n[2], (real)0};
  real t[4];
  apply4(m, h, t);
  normalise3(t, out);
}

/* float -> int32 conversion (astype(int)): saturating, NaN -> 0. */
static inline int f2i(real x) {
  if (x != x) return 0;
  if (x >= (real)2147483647.0) return 2147483647;
  if (x <= (real)-2147483648.0) return (int)(-2147483647 - 1);
  return (int)x;
}

/* jnp integer remainder: result takes the sign of the divisor. */
static inline int pymod(int a, int b) {
  if (b == 0) return 0;
  int r = a % b;
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}

/* Index normalisation + clamping of a jnp gather in its default mode:
 * negative indices wrap once (index + size), the rest clamps into range. */
static inline int gather_clamp(int idx, int size) {
  if (idx < 0) idx += size;
  if (idx < 0) idx = 0;
  if (idx > size - 1) idx = size - 1;
  return idx;
}

/* Monotone map of a depth to uint32 for the primitive chooser: NaN first,
 * -0 == +0, then increasing order. */
static inline uint32_t depth_order(real z) {
  if (z != z) return 0u;
  float zf = (float)z;
  if (zf == 0.0f) zf = 0.0f;
  uint32_t b;
  memcpy(&b, &zf, 4);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* ---------------------------------------------- 3x3 determinant, inverse */

/* jnp.linalg.det's closed form for 3x3 (used at pipeline.py:91-94):
 * a00 a11 a22 + a01 a12 a20 + a02 a10 a21 - a02 a11 a20 - a00 a12 a21
 * - a01 a10 a22, evaluated left to right. */
static real det3(const real* a) {
  real t1 = (a[0] * a[4]) * a[8];
  real t2 = (a[1] * a[5]) * a[6];
  real t3 = (a[2] * a[3]) * a[7];
  real t4 = (a[2] * a[4]) * a[6];
  real t5 = (a[0] * a[5]) * a[7];
  real t6 = (a[1] * a[3]) * a[8];
  return ((((t1 + t2) + t3) - t4) - t5) - t6;
}

/* jnp.linalg.inv (pipeline.py:105, phong_darboux.py:243): solve(A, I) with
 * an LU factorisation with partial pivoting (reference LAPACK getf2: first
 * index of max |a| as pivot, column scaled by the reciprocal of the pivot
 * when it is a normal number, rank-1 update a - l*u), then the permuted
 * identity solved by a unit-lower and an upper triangular solve in the
 * reference BLAS trsm order (column-oriented, zero entries skipped). */
static void inv3(const real* m, real* out) {
  real a[9];
  memcpy(a, m, sizeof(a));
  int perm[3] = {0, 1, 2};
  for (int j = 0; j < 2; ++j) {
    int p = j;
    real amax = R_FABS(a[3 * j + j]);
    for (int r = j + 1; r < 3; ++r) {
      real v = R_FABS(a[3 * r + j]);
      if (v > amax) {
        amax = v;
        p = r;
      }
    }
    if (a[3 * p + j] != (real)0) {
      if (p != j) {
        for (int c = 0; c < 3; ++c) {
          real t = a[3 * j + c];
          a[3 * j + c] = a[3 * p + c];
          a[3 * p + c] = t;
        }
        int t = perm[j];
        perm[j] = perm[p];
        perm[p] = t;
      }
      real piv = a[3 * j + j];
      if (R_FABS(piv) >= R_MIN_NORMAL) {
        real rcp = (real)1 / piv;
        for (int r = j + 1; r < 3; ++r) a[3 * r + j] = a[3 * r + j] * rcp;
      } else {
        for (int r = j + 1; r < 3; ++r) a[3 * r + j] = a[3 * r + j] / piv;
      }
    }
    for (int r = j + 1; r < 3; ++r)
      for (int c = j + 1; c < 3; ++c) a[3 * r + c] = a[3 * r + c] - a[3 * r + j] * a[3 * j + c];
  }
  for (int col = 0; col < 3; ++col) {
    real b[3];
    for (int r = 0; r < 3; ++r) b[r] = (perm[r] == col) ? (real)1 : (real)0;
    /* unit lower: b_i -= b_k * L_ik for i > k */
    for (int k = 0; k < 3; ++k)
      if (b[k] != (real)0)
        for (int i = k + 1; i < 3; ++i) b[i] = b[i] - b[k] * a[3 * i + k];
    /* upper: b_k /= U_kk, then b_i -= b_k * U_ik for i < k */
    for (int k = 2; k >= 0; --k)
      if (b[k] != (real)0) {
        b[k] = b[k] / a[3 * k + k];
        for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * a[3 * i + k];
      }
    for (int r = 0; r < 3; ++r) out[3 * r + col] = b[r];
  }
}

/* ------------------------------------------------------- vertex shaders */

/* Varying layout per vertex (VAR_* offsets). */
#define NVAR 24
#define V_COLOUR 0  /* gouraud, gouraud_texture */
#define V_UVG 3     /* gouraud_texture uv */
#define V_NORMAL 0  /* phong family */
#define V_UV 3
#define V_TRI 5     /* darboux: 3x3 NDC triangle */
#define V_TRIUV 14  /* darboux: 3x2 uv triangle */
#define V_SHADOW 5  /* reflection_shadow: shadow_coord (4) */

typedef struct VOut {
  real clip[4];
  real var[NVAR];
  int texidx;
} VOut;

static void vertex_shader(const Scene* s, int v, VOut* o) {
  memset(o, 0, sizeof(*o));
  to_clip(s->world_to_clip, s->position + 3 * v, o->clip);
  switch (s->shader) {
    case OR_SHADER_DEPTH: /* depth.py:47-61 */
      break;
    case OR_SHADER_GOURAUD: { /* gouraud.py:58-88 */
      real n[3], l[3];
      normalise3(s->normal + 3 * v, n);
      normalise3(s->light_direction, l);
      real intensity = dot3(n, l);
      for (int c = 0; c < 3; ++c) o->var[V_COLOUR + c] = (s->colour[3 * v + c] * s->light_colour[c]) * intensity;
      break;
    }
    case OR_SHADER_GOURAUD_TEXTURE: { /* gouraud_texture.py:68-101 */
      real n[3], l[3];
      normalise3(s->normal + 3 * v, n);
      normalise3(s->light_direction, l);
      real intensity = dot3(n, l);
      for (int c = 0; c < 3; ++c) o->var[V_COLOUR + c] = s->light_colour[c] * intensity;
      o->var[V_UVG + 0] = s->uv[2 * v + 0];
      o->var[V_UVG + 1] = s->uv[2 * v + 1];
      break;
    }
    case OR_SHADER_PHONG:
    case OR_SHADER_PHONG_REFLECTION:
    case OR_SHADER_PHONG_REFLECTION_SHADOW:
    case OR_SHADER_PHONG_DARBOUX: {
      /* phong.py:78-104, phong_reflection.py:104-132,
       * phong_reflection_shadow.py:115-150, phong_darboux.py:120-170 */
      real n1[3];
      normalise3(s->normal + 3 * v, n1);
      apply_vec(s->world_to_eye_norm, n1, o->var + V_NORMAL);
      o->var[V_UV + 0] = s->uv[2 * v + 0];
      o->var[V_UV + 1] = s->uv[2 * v + 1];
      if (s->shader == OR_SHADER_PHONG_REFLECTION || s->shader == OR_SHADER_PHONG_REFLECTION_SHADOW)
        o->texidx = s->texture_index[v];
      if (s->shader == OR_SHADER_PHONG_REFLECTION_SHADOW) {
        real sc[4];
        to_clip(s->shadow_world_to_clip, s->position + 3 * v, sc);
        for (int c = 0; c < 4; ++c) o->var[V_SHADOW + c] = sc[c] / sc[3];
      }
      if (s->shader == OR_SHADER_PHONG_DARBOUX) {
        const int* f = s->darboux_faces + 3 * s->id_to_face[v];
        for (int k = 0; k < 3; ++k) {
          real tc[4];
          to_clip(s->world_to_clip, s->position + 3 * f[k], tc);
          for (int c = 0; c < 3; ++c) /* to_cartesian (geometry.py:185-202) */
            o->var[V_TRI + 3 * k + c] = (tc[3] == (real)0) ? tc[c] : tc[c] / tc[3];
          o->var[V_TRIUV + 2 * k + 0] = s->uv[2 * f[k] + 0];
          o->var[V_TRIUV + 2 * k + 1] = s->uv[2 * f[k] + 1];
        }
      }
      break;
    }
    default:
      break;
  }
}

/* ----------------------------------------------------- primitive setup */

typedef struct Prim {
  real inv[9];
  real z[3];
  real det;
  int keep;  /* |det| > 1e-6 */
  int front; /* det >= 0 */
} Prim;

/* PerPrimitive.create (pipeline.py:80-113). */
static void setup_prim(const VOut* vo, const int* face, Prim* p) {
  real m[9];
  for (int k = 0; k < 3; ++k) {
    const real* c = vo[face[k]].clip;
    m[3 * k + 0] = c[0];
    m[3 * k + 1] = c[1];
    m[3 * k + 2] = c[3];
    p->z[k] = c[2];
  }
  p->det = det3(m);
  p->keep = R_FABS(p->det) > (real)1e-6f;
  p->front = p->det >= (real)0;
  inv3(m, p->inv);
}

/* _when_keep_primitive (pipeline.py:172-196): clip_coef = [x, y, 1] @ inv. */
static inline void clip_coef(const Prim* p, real x, real y, real* c) {
  for (int k = 0; k < 3; ++k) c[k] = (x * p->inv[k] + y * p->inv[3 + k]) + p->inv[6 + k];
}

/* Window-space depth (pipeline.py:212-219). */
static inline real frag_depth(const Prim* p, const real* c, const real* vp) {
  real z = (c[0] * p->z[0] + c[1] * p->z[1]) + c[2] * p->z[2];
  return z * vp[10] + vp[11];
}

/* ------------------------------------------------------ fragment stage */

static inline void tex3(const real* tex, int w, int h, int ch, int u, int v, real* out) {
  u = gather_clamp(u, w);
  v = gather_clamp(v, h);
  const real* t = tex + ((size_t)u * h + v) * ch;
  for (int c = 0; c < 3; ++c) out[c] = t[ch == 1 ? 0 : c];
}

static inline real interp1(const real* b, real v0, real v1, real v2) {
  return (b[0] * v0 + b[1] * v1) + b[2] * v2;
}

static inline real max0(real x) { return (x != x) ? x : (x > (real)0 ? x : (real)0); }

/* Fragment shader of the chosen primitive.  Returns the shader's keep
 * (AND-ed later with the chooser's keep) and writes the colour. */
/* Branch signature of a fragment (for gradient checks): the sampled texel
 * (u, w) before clamping and the shader's branch bits, hashed into 32 bits.
 * Within one primitive the colour is a smooth function of the inputs
 * wherever this signature does not change. */
static inline int branch_sig(int u, int w, int bits) {
  uint32_t h = ((uint32_t)u * 65599u + (uint32_t)w) * 16u + (uint32_t)bits;
  return (int)(h & 0x7fffffffu);
}

typedef struct FragProbe {
  int branch; /* branch_sig of the fragment */
  int texel;  /* element row (u * tex_h + w, clamped) of the diffuse texel sampled, or -1 */
} FragProbe;

static inline int texel_row(const Scene* s, int u, int w) {
  return gather_clamp(u, s->tex_w) * s->tex_h + gather_clamp(w, s->tex_h);
}

static int fragment(const Scene* s, const VOut* v0, const VOut* v1, const VOut* v2, const real* b,
                    int front, real* colour, FragProbe* probe) {
  FragProbe dummy;
  if (!probe) probe = &dummy;
  int* branch = &probe->branch;
  *branch = 0;
  probe->texel = -1;
  real var[NVAR];
  for (int k = 0; k < NVAR; ++k) var[k] = interp1(b, v0->var[k], v1->var[k], v2->var[k]);
  switch (s->shader) {
    case OR_SHADER_DEPTH: /* shader.py:333 default fragment */
      return 1;
    case OR_SHADER_GOURAUD: { /* gouraud.py:94-124 */
      int ok = front;
      for (int c = 0; c < 3; ++c) {
        colour[c] = var[V_COLOUR + c];
        ok = ok && (var[V_COLOUR + c] >= (real)0);
      }
      *branch = branch_sig(0, 0, ok);
      return ok;
    }
    case OR_SHADER_GOURAUD_TEXTURE: { /* gouraud_texture.py:107-144 */
      int u = pymod(f2i(R_FLOOR(var[V_UVG + 0])), s->tex_w);
      int w = pymod(f2i(R_FLOOR(var[V_UVG + 1])), s->tex_h);
      real tc[3];
      tex3(s->texture, s->tex_w, s->tex_h, s->tex_c, u, w, tc);
      probe->texel = texel_row(s, u, w);
      int ok = front;
      for (int c = 0; c < 3; ++c) {
        ok = ok && (var[V_COLOUR + c] >= (real)0);
        colour[c] = tc[c] * var[V_COLOUR + c];
      }
      *branch = branch_sig(u, w, ok);
      return ok;
    }
    case OR_SHADER_PHONG: { /* phong.py:110-164 */
      int u = pymod(f2i(R_FLOOR(var[V_UV + 0])), s->tex_w);
      int w = pymod(f2i(R_FLOOR(var[V_UV + 1])), s->tex_h);
      real tc[3], n[3], l[3], lc[3];
      tex3(s->texture, s->tex_w, s->tex_h, s->tex_c, u, w, tc);
      probe->texel = texel_row(s, u, w);
      normalise3(var + V_NORMAL, n);
      normalise3(s->light_direction, l);
      real d = dot3(n, l);
      int nonneg = 1;
      for (int c = 0; c < 3; ++c) {
        lc[c] = s->light_colour[c] * d;
        nonneg = nonneg && (lc[c] >= (real)0);
      }
      for (int c = 0; c < 3; ++c) colour[c] = nonneg ? tc[c] * lc[c] : (real)0;
      *branch = branch_sig(u, w, nonneg);
      return front;
    }
    case OR_SHADER_PHONG_DARBOUX: { /* phong_darboux.py:212-293 */
      int u = pymod(f2i(R_FLOOR(var[V_UV + 0])), s->tex_w);
      int w = pymod(f2i(R_FLOOR(var[V_UV + 1])), s->tex_h);
      real n[3];
      normalise3(var + V_NORMAL, n);
      const real* t = v0->var + V_TRI;   /* not interpolated: vertex 0's */
      const real* tu = v0->var + V_TRIUV;
      real A[9], AI[9];
      for (int c = 0; c < 3; ++c) {
        A[c] = t[3 + c] - t[c];
        A[3 + c] = t[6 + c] - t[c];
        A[6 + c] = n[c];
      }
      inv3(A, AI);
      real bi[3] = {tu[2] - tu[0], tu[4] - tu[0], (real)0};
      real bj[3] = {tu[3] - tu[1], tu[5] - tu[1], (real)0};
      real vi[3], vj[3], ni[3], nj[3];
      for (int r = 0; r < 3; ++r) {
        vi[r] = dot3(AI + 3 * r, bi);
        vj[r] = dot3(AI + 3 * r, bj);
      }
      normalise3(vi, ni);
      normalise3(vj, nj);
      real B[9];
      for (int r = 0; r < 3; ++r) {
        B[3 * r + 0] = ni[r];
        B[3 * r + 1] = nj[r];
        B[3 * r + 2] = n[r];
      }
      real nm[3], bn[3], nn[3], l[3], tc[3], lc[3];
      tex3(s->normal_map, s->nm_w, s->nm_h, 3, u, w, nm);
      for (int r = 0; r < 3; ++r) bn[r] = dot3(B + 3 * r, nm);
      normalise3(bn, nn);
      tex3(s->texture, s->tex_w, s->tex_h, s->tex_c, u, w, tc);
      probe->texel = texel_row(s, u, w);
      normalise3(s->light_direction, l);
      real d = dot3(nn, l);
      int nonneg = 1;
      for (int c = 0; c < 3; ++c) {
        lc[c] = s->light_colour[c] * d;
        nonneg = nonneg && (lc[c] >= (real)0);
      }
      for (int c = 0; c < 3; ++c) colour[c] = nonneg ? tc[c] * lc[c] : (real)0;
      *branch = branch_sig(u, w, nonneg);
      return front;
    }
    case OR_SHADER_PHONG_REFLECTION:
    case OR_SHADER_PHONG_REFLECTION_SHADOW: {
      /* phong_reflection.py:158-235, phong_reflection_shadow.py:178-271 */
      int shadowed = s->shader == OR_SHADER_PHONG_REFLECTION_SHADOW;
      int shadow_bit = 0;
      real shadow[3] = {(real)1, (real)1, (real)1};
      if (shadowed) {
        real sc[4];
        apply4(s->shadow_viewport, var + V_SHADOW, sc);
        real sw = sc[3];
        for (int c = 0; c < 4; ++c) sc[c] = sc[c] / sw;
        /* Shadow.get (shadow.py:129-153): round half away from zero, wrap
         * negatives once, out of bounds reads inf. */
        int px = f2i(R_ROUND(sc[0]));
        int py = f2i(R_ROUND(sc[1]));
        if (px < 0) px += s->shadow_w;
        if (py < 0) py += s->shadow_h;
        real depth = (real)INFINITY;
        if (px >= 0 && px < s->shadow_w && py >= 0 && py < s->shadow_h)
          depth = s->shadow_map[(size_t)px * s->shadow_h + py];
        int lit = sc[2] <= depth;
        shadow_bit = lit ? 4 : 0;
        for (int c = 0; c < 3; ++c) shadow[c] = lit ? (real)1 : (real)1 - s->shadow_strength[c];
      }
      /* MergedModel.uv_repeat (model.py:306-339) */
      int ti = gather_clamp(v0->texidx, s->n_objects);
      int shape[2] = {s->texture_shape[2 * ti], s->texture_shape[2 * ti + 1]};
      real uvr[2];
      for (int a = 0; a < 2; ++a) {
        real x = var[V_UV + a];
        real whole = (x >= (real)0) ? R_FLOOR(x) : R_CEIL(x);
        real frac = x - whole;
        if (frac < (real)0) frac = frac + (real)1;
        uvr[a] = frac * (real)shape[a];
      }
      uvr[0] = uvr[0] + (real)(v0->texidx * s->texture_offset);
      int u = f2i(R_FLOOR(uvr[0]));
      int w = f2i(R_FLOOR(uvr[1]));
      real tc[3], n[3], l[3], r[3], rn[3];
      tex3(s->texture, s->tex_w, s->tex_h, s->tex_c, u, w, tc);
      probe->texel = texel_row(s, u, w);
      normalise3(var + V_NORMAL, n);
      normalise3(s->light_dir_eye, l);
      real d = dot3(n, l);
      real dif = max0(d);
      for (int c = 0; c < 3; ++c) r[c] = (((real)2 * d) * n[c]) - l[c];
      normalise3(r, rn);
      int su = gather_clamp(u, s->spec_w), sv = gather_clamp(w, s->spec_h);
      real spec = R_POW(max0(rn[2]), s->specular_map[(size_t)su * s->spec_h + sv]);
      for (int c = 0; c < 3; ++c) {
        real a = s->ambient[c] * tc[c];
        real k = s->diffuse[c] * dif + s->specular[c] * spec;
        real b = shadowed ? ((shadow[c] * k) * tc[c]) * s->light_colour[c]
                          : (k * s->light_colour[c]) * tc[c];
        colour[c] = a + b;
      }
      *branch = branch_sig(u, w, (d > (real)0) | ((rn[2] > (real)0) << 1) | shadow_bit);
      return front;
    }
    default:
      return 0;
  }
}

/* ------------------------------------------------------------- pipeline */

/* Depth order of the choosers: NaN first (argmin's NaN rule), -0 == +0,
 * then ascending; equal depths (both NaN included) are ordered by index. */
static inline int depth_before(real za, int ia, real zb, int ib) {
  int na = za != za, nb = zb != zb;
  if (na || nb) return na && nb ? ia < ib : na;
  if (za < zb) return 1;
  if (zb < za) return 0;
  return ia < ib;
}

/* Interpolation + fragment of primitive `p` at pixel (x, y)
 * (pipeline.py:283-326): keeps `chooser_keep` (keep & inside), depth,
 * colour; returns the fragment shader's keep. */
static int shade_prim(const Scene* s, const VOut* vo, const Prim* pr, int p, real x, real y, int* chooser_keep,
                      real* z, real* colour) {
  const Prim* P = pr + p;
  real c[3];
  clip_coef(P, x, y, c);
  real w_rcp = (c[0] + c[1]) + c[2];
  int in_tri = c[0] >= (real)0 && c[1] >= (real)0 && c[2] >= (real)0;
  *chooser_keep = P->keep && in_tri;
  *z = frag_depth(P, c, s->viewport);
  real b[3] = {c[0] / w_rcp, c[1] / w_rcp, c[2] / w_rcp};
  const int* face = s->faces + 3 * p;
  colour[0] = colour[1] = colour[2] = 0;
  return fragment(s, vo + face[0], vo + face[1], vo + face[2], b, P->front, colour, NULL);
}

/* Layered chooser and its mixers: the compiled primitive_chooser / mix
 * hooks at the override points shader.py:159-251 and :339-396.  The chooser
 * keeps the L nearest candidates (keep & inside & front, depth not +inf) in
 * depth_before order; slots past the last candidate are not kept.  Every
 * kept slot is interpolated and shaded (pipeline.py:337-342).  Mixer 0 takes
 * the first slot the fragment shader keeps (the default mix's argmin over
 * kept depths, shader.py:374-396); mixer 1 composites the kept slots front to
 * back: w = T * a, C = C + w * colour, T = T * (1 - a), then
 * C + T * background.  Depth and primitive id are the first kept slot's. */
#define OR_MAX_LAYERS 4
static int layered_pixel(const Scene* s, const VOut* vo, const Prim* pr, int i, int j, real x, real y) {
  const real* vp = s->viewport;
  const int H = s->height, F = s->n_faces;
  const int L = s->layers > OR_MAX_LAYERS ? OR_MAX_LAYERS : s->layers;
  real sz[OR_MAX_LAYERS];
  int si[OR_MAX_LAYERS];
  int n = 0;
  uint32_t ord1 = 0xFFFFFFFFu, ord2 = 0xFFFFFFFFu; /* two best candidate depths */
  for (int p = 0; p < F; ++p) {
    const Prim* P = pr + p;
    real c[3];
    clip_coef(P, x, y, c);
    int in_tri = c[0] >= (real)0 && c[1] >= (real)0 && c[2] >= (real)0;
    if (!(P->keep && in_tri && P->front)) continue;
    real z = frag_depth(P, c, vp);
    uint32_t o = depth_order(z);
    if (o < ord1) {
      ord2 = ord1;
      ord1 = o;
    } else if (o < ord2) {
      ord2 = o;
    }
    if (z == (real)INFINITY) continue;
    int pos = n;
    while (pos > 0 && depth_before(z, p, sz[pos - 1], si[pos - 1])) --pos;
    if (pos >= L) continue;
    int last = n < L ? n : L - 1;
    for (int k = last; k > pos; --k) {
      sz[k] = sz[k - 1];
      si[k] = si[k - 1];
    }
    sz[pos] = z;
    si[pos] = p;
    if (n < L) ++n;
  }
  int keep = 0, prim = -1;
  real depth = 0, out[3] = {0, 0, 0}, C[3] = {0, 0, 0}, T = 1;
  for (int k = 0; k < n; ++k) {
    int ck;
    real z, col[3];
    int fk = shade_prim(s, vo, pr, si[k], x, y, &ck, &z, col);
    if (!(ck && fk)) continue;
    if (!keep) {
      keep = 1;
      prim = si[k];
      depth = z;
      if (s->mixer == 0) {
        for (int ch = 0; ch < 3; ++ch) out[ch] = col[ch];
        break;
      }
    }
    real a = s->face_alpha ? s->face_alpha[si[k]] : s->opacity;
    real w = T * a;
    for (int ch = 0; ch < 3; ++ch) C[ch] = C[ch] + w * col[ch];
    T = T * ((real)1 - a);
  }
  if (keep && s->mixer == 1)
    for (int ch = 0; ch < 3; ++ch) out[ch] = C[ch] + T * s->background[ch];
  size_t pix = (size_t)i * H + j;
  if (keep) {
    s->zbuffer[pix] = depth;
    if (s->canvas)
      for (int ch = 0; ch < 3; ++ch) s->canvas[pix * 3 + ch] = out[ch];
  }
  if (s->prim_id) s->prim_id[pix] = prim;
  return ord2 != 0xFFFFFFFFu && ord2 - ord1 <= 1u && ord1 != depth_order((real)INFINITY);
}

/* pipeline.render (pipeline.py:470-537) + _postprocessing (:127-459). */
static int render(Scene* s) {
  if (s->n_faces <= 0 || s->width <= 0 || s->height <= 0) {
    s->near_ties = 0;
    return 0;
  }
  VOut* vo = (VOut*)malloc(sizeof(VOut) * (size_t)(s->n_verts > 0 ? s->n_verts : 1));
  Prim* pr = (Prim*)malloc(sizeof(Prim) * (size_t)s->n_faces);
  if (!vo || !pr) {
    free(vo);
    free(pr);
    return -1;
  }
  for (int v = 0; v < s->n_verts; ++v) vertex_shader(s, v, vo + v);
  for (int f = 0; f < s->n_faces; ++f) setup_prim(vo, s->faces + 3 * f, pr + f);

  const real* vp = s->viewport;
  const int W = s->width, H = s->height, F = s->n_faces;
  /* optional pixel window [x_begin, x_end) x [y_begin, y_end): pixels outside
   * it are left untouched (an end of 0 means the whole axis) */
  const int xb = s->x_end > 0 ? (s->x_begin > 0 ? s->x_begin : 0) : 0;
  const int xe = s->x_end > 0 ? (s->x_end < W ? s->x_end : W) : W;
  const int yb = s->y_end > 0 ? (s->y_begin > 0 ? s->y_begin : 0) : 0;
  const int ye = s->y_end > 0 ? (s->y_end < H ? s->y_end : H) : H;
  long long ties = 0;
  int nt = s->n_threads > 0 ? s->n_threads : 1;
  (void)nt;
  (void)W;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : ties) num_threads(nt)
  for (int i = xb; i < xe; ++i) {
    real x = ((real)i - vp[3]) / vp[0];
    for (int j = yb; j < ye; ++j) {
      real y = ((real)j - vp[7]) / vp[5];
      if (s->layers > 0) {
        ties += layered_pixel(s, vo, pr, i, j, x, y);
        continue;
      }
      /* per-primitive preprocess + default primitive_chooser
       * (shader.py:207-217): argmin over where(keep & in & front, z, inf),
       * first index on ties, NaN first. */
      int best = 0;
      real best_z = (real)INFINITY;
      int best_nan = 0;
      uint32_t ord1 = 0xFFFFFFFFu, ord2 = 0xFFFFFFFFu; /* two best candidate depths */
      for (int p = 0; p < F; ++p) {
        const Prim* P = pr + p;
        real c[3];
        clip_coef(P, x, y, c);
        int in_tri = c[0] >= (real)0 && c[1] >= (real)0 && c[2] >= (real)0;
        if (!(P->keep && in_tri && P->front)) continue;
        real z = frag_depth(P, c, vp);
        if (z != z) {
          if (!best_nan) {
            best_nan = 1;
            best = p;
            best_z = z;
          }
        } else if (!best_nan && z < best_z) {
          best = p;
          best_z = z;
        }
        uint32_t o = depth_order(z);
        if (o < ord1) {
          ord2 = ord1;
          ord1 = o;
        } else if (o < ord2) {
          ord2 = o;
        }
      }
      if (ord2 != 0xFFFFFFFFu && ord2 - ord1 <= 1u && ord1 != depth_order((real)INFINITY)) ties += 1;
      /* chosen primitive: recompute its per-pixel values */
      const Prim* P = pr + best;
      real c[3];
      clip_coef(P, x, y, c);
      real w_rcp = (c[0] + c[1]) + c[2];
      int in_tri = c[0] >= (real)0 && c[1] >= (real)0 && c[2] >= (real)0;
      int chooser_keep = P->keep && in_tri;
      real z = frag_depth(P, c, vp);
      real b[3] = {c[0] / w_rcp, c[1] / w_rcp, c[2] / w_rcp};
      const int* face = s->faces + 3 * best;
      real colour[3] = {0, 0, 0};
      FragProbe probe = {0, -1};
      int frag_keep = fragment(s, vo + face[0], vo + face[1], vo + face[2], b, P->front, colour, &probe);
      /* mix (shader.py:374-396) + merge_buffers (pipeline.py:401-440) */
      int keep = chooser_keep && frag_keep;
      size_t pix = (size_t)i * H + j;
      if (keep) {
        s->zbuffer[pix] = z;
        if (s->canvas)
          for (int ch = 0; ch < 3; ++ch) s->canvas[pix * 3 + ch] = colour[ch];
      }
      if (s->prim_id) s->prim_id[pix] = keep ? best : -1;
      if (s->branch) s->branch[pix] = probe.branch;
      if (s->texel) s->texel[pix] = keep ? probe.texel : -1;
    }
  }
  s->near_ties = ties;
  free(vo);
  free(pr);
  return 0;
}

int SUF(or_render)(void* scene) { return render((Scene*)scene); }

#if !OR_DOUBLE
void or_inv3_f32(const float* m, float* out) { inv3(m, out); }
float or_det3_f32(const float* m) { return det3(m); }
unsigned int or_depth_order_f32(float z) { return depth_order(z); }
#endif
