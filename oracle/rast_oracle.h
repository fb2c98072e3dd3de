/*
 * rast_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of jaxrenderer's rasterisation path (vertex shader ->
 * per-pixel scan over every primitive -> primitive chooser -> interpolation
 * -> built-in fragment shaders -> mixer -> buffer merge).  It is the checker
 * for the CUDA kernels in jaxrenderer_gb300/csrc; the product never links it.
 *
 * Parity against the reference's own JAX execution is UNPINNED: JAX/jaxlib
 * (jax 0.4.13 in the reference's poetry.lock) cannot be installed on either
 * machine this project builds on, and the reference ships no golden vectors.
 * The restatement follows the reference's operation order with FMA
 * contraction disabled, and its 3x3 inverse is LU with partial pivoting
 * (reference LAPACK getf2 + BLAS trsm order), which is the algorithm behind
 * jnp.linalg.inv.  The reference's own smoke-test assertions
 * (tests/smoke_test.py) are re-run against it in tests/.
 *
 * Two builds of the same source: *_f32 (float, the parity checker) and
 * *_f64 (double, the finite-difference twin for gradient checks).  The
 * OrScene layout below is written for the f32 build; the f64 build uses the
 * identical layout with every `float` field and pointer replaced by `double`.
 */
#ifndef RAST_ORACLE_H
#define RAST_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Shader ids: same numbering as RastShader in include/rast_gb300.h. */
#define OR_SHADER_DEPTH 0
#define OR_SHADER_GOURAUD 1
#define OR_SHADER_GOURAUD_TEXTURE 2
#define OR_SHADER_PHONG 3
#define OR_SHADER_PHONG_DARBOUX 4
#define OR_SHADER_PHONG_REFLECTION 5
#define OR_SHADER_PHONG_REFLECTION_SHADOW 6

typedef struct OrSceneF32 {
  int shader;
  int width, height;             /* buffers are (width, height[, 3]), x-major */
  int n_threads;                 /* OpenMP threads for the pixel loop (<=0: 1) */
  const float* viewport;         /* 4x4 row-major */
  const float* world_to_clip;    /* 4x4 row-major */
  const float* world_to_eye_norm;/* 4x4 row-major */
  int n_verts;
  const float* position;         /* (V,3) */
  const float* normal;           /* (V,3) */
  const float* uv;               /* (V,2) */
  const float* colour;           /* (V,3) gouraud */
  const int* texture_index;      /* (V)   phong_reflection[_shadow] */
  const int* id_to_face;         /* (V)   phong_darboux */
  const int* darboux_faces;      /* (Fd,3) phong_darboux faces_indices */
  int n_darboux_faces;
  int n_faces;
  const int* faces;              /* (F,3) */
  float light_direction[3];
  float light_colour[3];
  float light_dir_eye[3];
  float ambient[3];
  float diffuse[3];
  float specular[3];
  const float* texture; int tex_w, tex_h, tex_c;     /* (tw,th,tc) */
  const float* specular_map; int spec_w, spec_h;     /* (sw,sh) */
  const float* normal_map; int nm_w, nm_h;           /* (nw,nh,3) */
  const int* texture_shape; int n_objects; int texture_offset;
  const float* shadow_map; int shadow_w, shadow_h;   /* (Ws,Hs) */
  const float* shadow_world_to_clip;                 /* 4x4 */
  const float* shadow_viewport;                      /* 4x4 */
  float shadow_strength[3];
  float* zbuffer;                /* (W,H) in/out */
  float* canvas;                 /* (W,H,3) in/out, NULL for depth */
  int* prim_id;                  /* (W,H) out: written primitive or -1; may be NULL */
  long long near_ties;           /* out: pixels whose two best depths are <= 1 ulp apart */
  /* compiled chooser / mix hooks (RastJob.layers / mixer in rast_gb300.h) */
  int layers;                    /* 0: default chooser; 1..4: layered chooser */
  int mixer;                     /* 0: nearest kept slot; 1: front-to-back over */
  float opacity;                 /* over: every face's opacity (face_alpha NULL) */
  float background[3];           /* over: colour behind the last layer */
  const float* face_alpha;       /* over: (F) per-face opacity, or NULL */
  /* gradient-check helpers (zero = off) */
  int x_begin, x_end;            /* render only pixels x_begin <= i < x_end (x_end 0: all) */
  int y_begin, y_end;            /* and y_begin <= j < y_end (y_end 0: all) */
  int* branch;                   /* (W,H) out, optional: branch signature of the default
                                    chooser's fragment (sampled texel + the shader's
                                    branch bits, hashed); the colour is smooth in the
                                    inputs wherever neither it nor prim_id changes */
  int* texel;                    /* (W,H) out, optional: element row u * tex_h + w of the
                                    diffuse texel the written fragment sampled, or -1 */
} OrSceneF32;

/* Render one scene; `scene` points at an OrSceneF32 (f32 build) or its
 * double twin (f64 build).  Returns 0 on success. */
int or_render_f32(void* scene);
int or_render_f64(void* scene);

/* Unit-test helpers. */
void or_inv3_f32(const float* m, float* out);
float or_det3_f32(const float* m);
unsigned int or_depth_order_f32(float z);

#ifdef __cplusplus
}
#endif
#endif
