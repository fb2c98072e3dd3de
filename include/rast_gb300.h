/*
 * rast_gb300.h -- C ABI of the GB300 (sm_103a) rasteriser.
 *
 * Replaces the hot path of jaxrenderer (JoeyTeng/jaxrenderer v0.3.2):
 *   renderer/pipeline.py:470-537  pipeline.render (vertex stage, per-face
 *                                 gather, PerPrimitive.create :80-113,
 *                                 _postprocessing :127-459)
 *   renderer/shader.py:159-396    default primitive_chooser / interpolate /
 *                                 fragment / mix
 *   renderer/shaders/*.py         the seven built-in shaders
 *   renderer/shadow.py:49-125     the light-space depth pass (+ offset)
 *
 * A call renders a batch of independent "jobs".  A job is one
 * pipeline.render call: one shader, one camera, one vertex range, one face
 * range and one (W, H) target.  Renderer.render with shadows is two jobs
 * (the DEPTH job writing the shadow map, then the PHONG_REFLECTION_SHADOW
 * job reading it) issued as two calls on the same stream.
 *
 * Conventions:
 *  - every pointer inside RastPools and RastBatch.jobs is DEVICE memory the
 *    caller owns; the library allocates nothing except where a function says
 *    so, and keeps no global mutable state;
 *  - buffers are x-major as in the reference (types.py:63-64): pixel (i, j)
 *    of a job lives at pixel_begin + i * height + j; canvas has 3 channels;
 *  - matrices are 4x4 row-major float32;
 *  - calls are ordered on `stream` (a cudaStream_t, NULL = legacy default);
 *  - every function returns RAST_OK (0) or a RastStatus code; nothing throws
 *    across the ABI.  rast_error_string() names a code.
 */
#ifndef RAST_GB300_H
#define RAST_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAST_ABI_VERSION 6  /* 2: chooser / mix hook fields (RastJob.layers ..., RastPools.face_alpha, RastBatch.max_layers);
                                 3: RastTiledStats.pixel_tests; 4: RastTiledConfig.warps_per_tile, rast_autotune;
                                 5: RastTiledStats.binned_faces (was reserved); 6: rast_backward_mse */

/* Built-in shader classes (renderer/shaders/*.py), one kernel path each. */
typedef enum RastShader {
  RAST_SHADER_DEPTH = 0,                   /* shaders/depth.py:38 DepthShader */
  RAST_SHADER_GOURAUD = 1,                 /* shaders/gouraud.py:49 */
  RAST_SHADER_GOURAUD_TEXTURE = 2,         /* shaders/gouraud_texture.py:55 */
  RAST_SHADER_PHONG = 3,                   /* shaders/phong.py:65 PhongTextureShader */
  RAST_SHADER_PHONG_DARBOUX = 4,           /* shaders/phong_darboux.py:106 */
  RAST_SHADER_PHONG_REFLECTION = 5,        /* shaders/phong_reflection.py:91 */
  RAST_SHADER_PHONG_REFLECTION_SHADOW = 6  /* shaders/phong_reflection_shadow.py:99 */
} RastShader;

typedef enum RastStatus {
  RAST_OK = 0,
  RAST_ERR_INVALID_ARGUMENT = 1,   /* bad sizes, NULL pointers, unknown shader */
  RAST_ERR_WORKSPACE_TOO_SMALL = 2,
  RAST_ERR_CUDA = 3,               /* a CUDA runtime call failed */
  RAST_ERR_UNSUPPORTED = 4,
  RAST_ERR_TIMEOUT = 5,            /* a bounded device-side wait ran out */
  RAST_ERR_BIN_OVERFLOW = 6,       /* tiled form: a bin exceeded its capacity */
  RAST_ERR_INDEX_OUT_OF_RANGE = 7, /* validation found a face index outside its vertex range */
  RAST_ERR_STATIC_SCRATCH_TOO_SMALL = 8 /* rast_render_tiled_static: batch needs more than
                                           RAST_STATIC_SCRATCH_BYTES of workspace */
} RastStatus;

/* One pipeline.render call.  Offsets are element rows into RastPools
 * arrays; `*_begin` fields marked (ws) index library workspace and are
 * filled by the caller as running sums of n_verts / n_faces over the jobs. */
typedef struct RastJob {
  int32_t shader;            /* RastShader */
  int32_t width, height;     /* target buffers (W, H) */
  int32_t n_verts;           /* vertices run through the vertex shader (len(extra[0])) */
  int32_t n_faces;           /* faces (F, 3); indices relative to vert_begin */
  int32_t n_darboux_faces;   /* rows of faces_indices (phong_darboux) */
  int32_t n_objects;         /* rows of texture_shape (phong_reflection*) */
  int32_t texture_offset;    /* MergedModel.offset (phong_reflection*) */
  int64_t vert_begin;        /* row of position/normal/uv/colour/texture_index/id_to_face */
  int64_t face_begin;        /* row of faces */
  int64_t darboux_face_begin;/* row of darboux_faces */
  int64_t pixel_begin;       /* pixel of zbuffer / canvas / prim_id */
  int64_t vout_begin;        /* (ws) first vertex-output row: sum of n_verts before */
  int64_t setup_begin;       /* (ws) first primitive-setup row: sum of n_faces before */
  int64_t texture_begin;     /* element of texture pool; (tex_w, tex_h, tex_c) */
  int64_t specular_begin;    /* element of specular pool; (spec_w, spec_h) */
  int64_t normal_map_begin;  /* element of normal-map pool; (nm_w, nm_h, 3) */
  int64_t texture_shape_begin; /* row of texture_shape (int32 pairs) */
  int64_t shadow_begin;      /* element of shadow-map pool; (shadow_w, shadow_h) */
  int32_t tex_w, tex_h, tex_c;
  int32_t spec_w, spec_h;
  int32_t nm_w, nm_h;
  int32_t shadow_w, shadow_h;
  float depth_offset;        /* with RAST_JOB_APPLY_DEPTH_OFFSET: added to every zbuffer
                                pixel after the pass (Shadow offset, shadow.py:116) */
  float viewport[16];        /* Camera.viewport */
  float world_to_clip[16];   /* Camera.world_to_clip */
  float world_to_eye_norm[16]; /* Camera.world_to_eye_norm */
  float shadow_viewport[16];   /* Shadow.camera.viewport */
  float shadow_world_to_clip[16]; /* Shadow.camera.world_to_clip */
  float light_direction[3];  /* LightSource.direction */
  float light_colour[3];     /* LightSource.colour */
  float light_dir_eye[3];    /* PhongReflection*ExtraInput.light_dir_eye */
  float ambient[3], diffuse[3], specular[3];
  float shadow_strength[3];  /* Shadow.strength */
  int32_t flags;             /* RAST_JOB_* bits */
  int32_t layers;            /* primitive_chooser hook: 0 = the default chooser (nearest
                                candidate, shader.py:207-251); 1..RAST_MAX_LAYERS = the
                                layered chooser (that many nearest candidates) */
  int32_t mixer;             /* mix hook (RastMixer); RAST_MIX_NEAREST is the default mix */
  float opacity;             /* RAST_MIX_OVER: opacity of every face (without
                                RAST_JOB_FACE_ALPHA) */
  float background[3];       /* RAST_MIX_OVER: colour seen through the last layer */
  int32_t reserved;
} RastJob;

/* RastJob.flags */
#define RAST_JOB_APPLY_DEPTH_OFFSET 1  /* zbuffer += depth_offset on every pixel after the pass */
#define RAST_JOB_FACE_ALPHA 2          /* RAST_MIX_OVER reads per-face opacity from
                                          RastPools.face_alpha[face_begin + face] */

/* Compiled primitive_chooser / mix hooks (the override points of
 * shader.py:159-251 and :339-396) for multi-candidate transparency.
 *
 * Layered chooser (RastJob.layers = L >= 1): the L candidates (kept,
 * inside, front-facing, depth below +inf) nearest to the camera, in
 * ascending (depth, primitive id) order; slots past the last candidate are
 * not kept.  Each kept slot runs interpolation and the fragment shader.
 *
 * Mixers, over the slots in that order:
 *  RAST_MIX_NEAREST  the first slot the fragment shader keeps (the default
 *                    mix: argmin of depth over kept fragments);
 *  RAST_MIX_OVER     front-to-back "over" compositing: T = 1, C = 0; for
 *                    every kept slot s with opacity a: w = T * a,
 *                    C = C + w * colour_s, T = T * (1 - a); the pixel gets
 *                    C + T * background, the depth of the first kept slot,
 *                    and that slot's primitive id.
 * A pixel with no kept slot is left unchanged (merge_buffers keep = False).
 * The DEPTH shader takes the default chooser only.  Differentiation: the
 * nearest mixer's gradient flows through the primitive each pixel shows
 * (prim_id); the over mixer's through every kept slot, weighted by its w,
 * and to the background (RAST_GRAD_BACKGROUND), with the slots the forward
 * saved in RastPools.layer_prim.  Opacities get no gradient. */
#define RAST_MAX_LAYERS 4
typedef enum RastMixer {
  RAST_MIX_NEAREST = 0,
  RAST_MIX_OVER = 1
} RastMixer;

/* Flat input/output arrays shared by all jobs of a batch (device). */
typedef struct RastPools {
  const float* position;       /* (rows, 3) */
  const float* normal;         /* (rows, 3) */
  const float* uv;             /* (rows, 2) */
  const float* colour;         /* (rows, 3)  gouraud */
  const int32_t* texture_index;/* (rows)     phong_reflection* */
  const int32_t* id_to_face;   /* (rows)     phong_darboux */
  const int32_t* faces;        /* (faces, 3) */
  const int32_t* darboux_faces;/* (rows, 3)  phong_darboux faces_indices */
  const float* texture;        /* diffuse maps, (w, h, c) each */
  const float* specular_map;   /* (w, h) each */
  const float* normal_map;     /* (w, h, 3) each */
  const int32_t* texture_shape;/* (objects, 2) */
  const float* shadow_map;     /* (w, h) each, read by PHONG_REFLECTION_SHADOW */
  float* zbuffer;              /* (pixels)     in/out */
  float* canvas;               /* (pixels, 3)  in/out; unused by DEPTH */
  int32_t* prim_id;            /* (pixels)     out, optional (NULL): primitive written or -1 */
  const float* face_alpha;     /* (faces)      opacity per face, read by RAST_MIX_OVER jobs
                                  with RAST_JOB_FACE_ALPHA; optional (NULL) otherwise */
  int32_t* layer_prim;         /* (RAST_MAX_LAYERS, pixels) out, optional (NULL): the layered
                                  chooser's slots of layered jobs' pixels, slot-major (slot s
                                  of pixel p at s * total_pixels + p), -1 past the last;
                                  rast_backward reads it for batches with layered jobs */
} RastPools;

typedef struct RastBatch {
  const RastJob* jobs;   /* DEVICE array of n_jobs */
  int32_t n_jobs;        /* 1 .. 65535 */
  int32_t max_width;     /* max over jobs of width  */
  int32_t max_height;    /* max over jobs of height */
  int32_t max_verts;     /* max over jobs of n_verts */
  int32_t max_faces;     /* max over jobs of n_faces */
  int32_t shader_mask;   /* OR of (1 << shader) over jobs */
  int64_t total_vout;    /* sum of n_verts   (vertex-output rows) */
  int64_t total_setup;   /* sum of n_faces   (primitive-setup rows) */
  int64_t total_pixels;  /* sum of width*height */
  RastPools pools;
  unsigned long long* near_ties; /* optional device counter (NULL): pixels whose two best
                                    candidate depths are <= 1 ulp apart, accumulated */
  int32_t max_layers;    /* max over jobs of RastJob.layers (0 .. RAST_MAX_LAYERS); a job's
                            layers beyond it are clamped to it */
  int32_t reserved;
} RastBatch;

/* Workspace the caller must pass to rast_render_plain, in bytes, 256-byte
 * aligned base required. */
size_t rast_plain_workspace_bytes(const RastBatch* batch);

/* Plain form: the reference's own method.  Vertex-shader kernel, primitive
 * setup kernel (det, keep, 3x3 LU inverse), per-pixel scan over every
 * primitive of the job (FP32 barycentrics + depth, winner by the packed
 * 64-bit (ordered depth | primitive id) minimum: lowest depth, then lowest
 * primitive id), then interpolation + fragment shader + mixer + merge. */
int rast_render_plain(const RastBatch* batch, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Per-kernel timing of one call, for benchmarks: when passed to a
 * *_profiled entry point, the library records CUDA events around each of its
 * kernels on `stream`, synchronises the stream before returning and fills
 * `ms` / `names` (at most 16 kernels, in launch order). */
typedef struct RastProfile {
  int32_t n;
  float ms[16];
  const char* names[16];
} RastProfile;

/* rast_render_plain with per-kernel timing (synchronises `stream`). */
int rast_render_plain_profiled(const RastBatch* batch, void* workspace, size_t workspace_bytes,
                               void* stream, RastProfile* profile);

/* Tiled form parameters (chosen by the autotuner, rast_autotune).  Zero
 * fields take the defaults: 8x8 tiles, bin capacity of 4 entries per face,
 * no small-face path, one warp per tile. */
typedef struct RastTiledConfig {
  int32_t tile_w;          /* tile (w, h) pixels along x (buffer axis 0) and y (axis 1): */
  int32_t tile_h;          /* 8x8, 16x8, 16x16, 32x8, 8x32, 8x4 or 4x8 */
  uint64_t bin_capacity;   /* total (tile, primitive) bin entries reserved in the workspace */
  int32_t small_area;      /* 0, or 1..32: faces whose conservative pixel rectangle has at most this
                              many pixels are rasterised by the setup kernel (64-bit atomicMin of the
                              packed key per pixel) instead of being binned; ignored while near ties
                              are counted */
  int32_t warps_per_tile;  /* 0 or 1: one warp rasterises a tile; 2: two warps each take half of the
                              tile's rows (bins stay per tile): tile shapes 8x8, 8x16 and 16x16 */
} RastTiledConfig;

/* Workspace bytes rast_render_tiled needs for `batch` under `cfg` (NULL = defaults);
 * 0 for a tile shape rast_render_tiled refuses. */
size_t rast_tiled_workspace_bytes(const RastBatch* batch, const RastTiledConfig* cfg);

/* Tiled form for many scenes per call.  Per face: clip positions, set-up and
 * a conservative pixel rectangle of its coverage (a superset of the pixels
 * whose FP32 edge functions can pass); bin counts, exclusive prefix sum,
 * scatter of primitive ids into the bins of the tiles the rectangle touches;
 * persistent warps rasterise one tile at a time with bin entries staged in
 * shared memory (packed depth|id minimum per pixel; an entry whose rectangle
 * covers few pixels of the tile is tested at those pixels only); deferred
 * shading of the winners.  Identical results to rast_render_plain.  Tiles
 * whose bins exceed bin_capacity are rasterised by a scan over all primitives
 * of their job (same results, slower).  Jobs wider or taller than 65535
 * pixels: RAST_ERR_UNSUPPORTED (the rectangles are 16-bit; the plain form
 * has no such limit).  Launches only kernels and memsets on `stream`:
 * capturable in a CUDA graph. */
int rast_render_tiled(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                      size_t workspace_bytes, void* stream);

/* The two phases of rast_render_tiled, for callers that overlap passes.
 * RAST_PHASE_COVERAGE: set-up, binning, rasterisation (depth-only jobs are
 * complete after it) and the varyings of the faces that won a pixel, left
 * in `workspace`; RAST_PHASE_SHADE: the deferred shading of those winners.
 * A shade call must follow the coverage call of the same batch, config and
 * workspace (stream-ordered); between the two the workspace must not be
 * reused, and the inputs the shading reads (the shadow maps of
 * PHONG_REFLECTION_SHADOW jobs, textures) may still be written, which is
 * what lets a light-space depth pass run beside the main pass's coverage.
 * Both bits = rast_render_tiled.  No counterpart in the reference (it
 * traces one sequential program). */
#define RAST_PHASE_COVERAGE 1
#define RAST_PHASE_SHADE 2
int rast_render_tiled_phase(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                            size_t workspace_bytes, void* stream, int phase);

/* rast_render_tiled with per-kernel timing (synchronises `stream`). */
int rast_render_tiled_profiled(const RastBatch* batch, const RastTiledConfig* cfg, void* workspace,
                               size_t workspace_bytes, void* stream, RastProfile* profile);

/* Tiled form for callers that cannot allocate device memory.
 *
 * No counterpart in the reference.  Some callers cannot call cudaMalloc
 * where they render: code recording into a CUDA graph or running inside a
 * framework callback that forbids allocation, real-time render threads
 * that must not hit the allocator, plugins whose host owns all device
 * memory.  This entry point takes no workspace: it runs rast_render_tiled
 * out of one file-scope __device__ array of RAST_STATIC_SCRATCH_BYTES
 * (64 MiB) that every GPU loading this library holds until the process
 * exits.  It calls no cudaMalloc, cudaFree or allocating library routine.
 *
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current) and caches it; make
 *    that first call before any stream capture on that device.  The cache
 *    is tagged with the CUDA context's id: after a cudaDeviceReset the next
 *    call looks the address up again (and is then again a first call).
 *  - A tile shape without a kernel is refused (RAST_ERR_INVALID_ARGUMENT,
 *    or RAST_ERR_UNSUPPORTED for a layered batch) before any size
 *    arithmetic.
 *  - Batches whose tiled workspace (rast_tiled_workspace_bytes) exceeds
 *    RAST_STATIC_SCRATCH_BYTES are rejected with
 *    RAST_ERR_STATIC_SCRATCH_TOO_SMALL; nothing is launched.
 *  - Every call shares the one array, which keeps the last call's contents
 *    (counters that must start at zero are cleared on `stream` each call).
 *    Calls whose work overlaps on the GPU (different streams, or
 *    different host threads without ordering) race on it: serialise them.
 * Outputs, statuses and results are those of rast_render_tiled. */
#define RAST_STATIC_SCRATCH_BYTES (64u << 20)
int rast_render_tiled_static(const RastBatch* batch, const RastTiledConfig* cfg, void* stream);

/* Autotuner of the tiled form: renders `batch` with every configuration the
 * tiled form has a kernel for (tile shape, small-face path off / on at 32
 * pixels, one or two warps per tile; the layered shapes for batches with
 * layered jobs), each with a bin capacity of 1.25x the entries its shape
 * requests, times three renders of each with CUDA events on `stream` and
 * writes the fastest to *out.  Results are cached in the library per
 * workload class (canvas size, faces per job and jobs rounded to powers of
 * two, shaders, layers, tie counting, device), guarded by a mutex; a cached
 * class returns at once without rendering.  The renders write the batch's
 * output pools: their contents afterwards are unspecified (render again).
 * Allocates its own workspace (cudaMallocAsync / cudaFreeAsync on `stream`)
 * and synchronises `stream`.  No counterpart call exists in the reference
 * (JAX compiles one form). */
int rast_autotune(const RastBatch* batch, void* stream, RastTiledConfig* out);

/* Bin statistics of the last rast_render_tiled call that used `workspace`
 * (synchronises `stream`; for autotuning and diagnostics). */
typedef struct RastTiledStats {
  uint64_t bin_entries;   /* (tile, primitive) pairs requested by the binning */
  uint64_t bin_capacity;  /* entries reserved */
  uint64_t tiles;         /* tile slots (jobs x tiles of the largest job) */
  uint32_t overflow;      /* 1: some tiles exceeded the capacity and were full-scanned */
  uint32_t binned_faces;  /* faces with at least one tile (the scatter's list) */
  uint64_t pixel_tests;   /* pixel-triangle pairs the raster kernel tested, counted per warp: entries
                             tested against every pixel of the warp's part of the tile x its pixels,
                             plus the (entry, pixel) pairs of the pair path (the pixels of an
                             entry's coverage rectangle inside the tile); faces of the small-face
                             path are not included */
} RastTiledStats;

int rast_tiled_stats(const RastBatch* batch, const RastTiledConfig* cfg, const void* workspace,
                     void* stream, RastTiledStats* out);

/* ---------------------------------------------------------------- backward
 * Gradients of a rendered batch, visibility piecewise constant (as under
 * jax.grad of the reference, tests/smoke_test_grad.py:92-128).  The batch
 * must be the one just rendered (same pools) with pools.prim_id holding the
 * forward's winning-primitive buffer; for PHONG_REFLECTION_SHADOW jobs
 * pools.shadow_map holds the forward's shadow maps.  Every gradient array is
 * ACCUMULATED into (the caller zeroes it); NULL arrays are skipped.
 * RastGradPools arrays have the layout of the matching RastPools arrays. */
#define RAST_GRAD_WORLD_TO_CLIP 0       /* 16: d/d Camera.world_to_clip (row-major) */
#define RAST_GRAD_WORLD_TO_EYE_NORM 16  /* 16: d/d Camera.world_to_eye_norm */
#define RAST_GRAD_LIGHT_DIRECTION 32    /* 3: d/d LightSource.direction */
#define RAST_GRAD_LIGHT_COLOUR 35       /* 3: d/d LightSource.colour */
#define RAST_GRAD_LIGHT_DIR_EYE 38      /* 3: d/d light_dir_eye (phong_reflection*) */
#define RAST_GRAD_AMBIENT 41            /* 3 */
#define RAST_GRAD_DIFFUSE 44            /* 3 */
#define RAST_GRAD_SPECULAR 47           /* 3 */
#define RAST_GRAD_SHADOW_STRENGTH 50    /* 3: d/d Shadow.strength */
#define RAST_GRAD_BACKGROUND 53         /* 3: d/d RastJob.background (RAST_MIX_OVER jobs) */
#define RAST_NPARAM 56                  /* per-job stride of job_params */

typedef struct RastGradPools {
  float* position;      /* (rows, 3) d/d vertex positions */
  float* normal;        /* (rows, 3) d/d vertex normals */
  float* colour;        /* (rows, 3) d/d vertex colours (gouraud) */
  float* texture;       /* like RastPools.texture: d/d diffuse texels */
  float* specular_map;  /* like RastPools.specular_map: d/d specular exponents */
  float* job_params;    /* (n_jobs, RAST_NPARAM) per-job camera/light gradients */
  float* normal_map;    /* like RastPools.normal_map: d/d normal-map texels (phong_darboux) */
} RastGradPools;

/* Workspace rast_backward needs for `batch` (256-byte aligned base). */
size_t rast_backward_workspace_bytes(const RastBatch* batch);

/* Reverse mode, split by dependency: per visible face (3x3 inverse of the
 * [x, y, w] clip rows), per corner vertex (vertex shader varyings), per kept
 * pixel (fragment and interpolation backward, accumulating dL/d inverse and
 * dL/d varyings), then per face (inverse and clip transform backward) and
 * per vertex (vertex shader backward).  uv gets no gradient (nearest texel:
 * floor).
 * grad_canvas (pixels, 3) and grad_zbuffer (pixels) may each be NULL. */
int rast_backward(const RastBatch* batch, const float* grad_canvas, const float* grad_zbuffer,
                  const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream);

/* rast_backward with per-kernel timing (synchronises `stream`). */
int rast_backward_profiled(const RastBatch* batch, const float* grad_canvas, const float* grad_zbuffer,
                           const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream,
                           RastProfile* profile);

/* rast_backward for the mean-squared-error image loss
 *   L = (scale / 2) * sum over every canvas value of (canvas - target)^2
 * (scale = 2 / n for the mean over n values): dL/dcanvas =
 * (canvas - target) * scale is formed per pixel inside the backward, from
 * batch->pools.canvas as the last render left it, instead of being read from
 * a gradient image; that spares the caller an elementwise pass over three
 * canvas-sized arrays.  The difference and the product are rounded as an
 * FP32 elementwise pass would round them, so the result is rast_backward's
 * with grad_canvas = (canvas - target) * scale.  target (pixels, 3) like the
 * canvas; grad_zbuffer may be NULL.  NULL target or canvas:
 * RAST_ERR_INVALID_ARGUMENT.  No counterpart in the reference, where the
 * loss is the caller's traced code (tests/smoke_test_grad.py:92-128). */
int rast_backward_mse(const RastBatch* batch, const float* target, float scale, const float* grad_zbuffer,
                      const RastGradPools* grads, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------
 * Device-side merge_objects + per-corner flattening (instanced scenes).
 *
 * Replaces the host work the reference does per frame before rendering:
 * renderer/model.py:447-555 merge_objects (object vertices scaled and
 * transformed with apply_pos, normals with apply_vec by the inverse
 * transpose of the transform, faces offset into the merged arrays) and
 * renderer/renderer.py:277-295 (positions, normals, uvs and texture indices
 * gathered per face corner).  Meshes are uploaded once; per frame only the
 * objects' transforms and local scalings change.  No counterpart entry point
 * exists in the reference (it merges on the host inside the traced call).
 *
 * Scenes are contiguous runs of instances; an instance's rows in its
 * scene's merged vertex / normal / uv arrays start at vert_offset /
 * norm_offset / uv_offset (the sums over the scene's earlier instances),
 * and its 3 * n_faces output corners at corner_begin.  Gathers follow the
 * reference's: indices wrap once if negative, then clamp to the scene's
 * merged array.  Global vector norms (normalise over a whole normal array)
 * are summed sequentially in index order.
 * --------------------------------------------------------------------- */
typedef struct RastMesh {
  int64_t vert_begin;    /* rows into mesh_verts */
  int64_t norm_begin;    /* rows into mesh_norms */
  int64_t uv_begin;      /* rows into mesh_uvs */
  int64_t face_begin;    /* rows into mesh_faces / mesh_faces_norm / mesh_faces_uv */
  int32_t n_verts, n_norms, n_uvs, n_faces;
} RastMesh;

typedef struct RastInstance {
  int32_t mesh;          /* index into the mesh table */
  int32_t scene_first;   /* first instance of this instance's scene */
  int32_t scene_count;   /* instances in the scene */
  int32_t vert_offset;   /* merged-row offsets of this instance in its scene */
  int32_t norm_offset;
  int32_t uv_offset;
  int32_t scene_verts;   /* merged-row totals of the scene */
  int32_t scene_norms;
  int32_t scene_uvs;
  int32_t reserved;
  int64_t corner_begin;  /* first output corner row */
  int64_t vert_row;      /* first row of this instance in the batch's merged */
  int64_t norm_row;      /* vertex / normal / uv arrays (all scenes back to back) */
  int64_t uv_row;
} RastInstance;

typedef struct RastMergeBatch {
  const RastMesh* meshes;          /* device, n_meshes */
  int32_t n_meshes;
  int32_t n_instances;
  const RastInstance* instances;   /* device, n_instances */
  const float* transforms;         /* device (n_instances, 16): ModelObject.transform, row-major */
  const float* local_scaling;      /* device (n_instances, 3) */
  const float* mesh_verts;         /* (rows, 3) */
  const float* mesh_norms;         /* (rows, 3) */
  const float* mesh_uvs;           /* (rows, 2) */
  const int32_t* mesh_faces;       /* (rows, 3) each, local to the mesh */
  const int32_t* mesh_faces_norm;
  const int32_t* mesh_faces_uv;
  int64_t total_faces;             /* sums over instances of their mesh's n_faces, */
  int64_t total_verts;             /* n_verts, n_norms and n_uvs (workspace sizing) */
  int64_t total_norms;
  int64_t total_uvs;
  float* position;                 /* out (corners, 3) */
  float* normal;                   /* out (corners, 3), may be NULL */
  float* uv;                       /* out (corners, 2), may be NULL */
  int32_t* texture_index;          /* out (corners), may be NULL */
} RastMergeBatch;

/* Workspace rast_merge_objects needs (256-byte aligned base): the merged
 * per-scene vertex, normal and uv arrays of the whole batch (36 bytes per
 * merged vertex + normal + uv row) plus per-instance bookkeeping. */
size_t rast_merge_workspace_bytes(const RastMergeBatch* batch);

/* Merge every scene's instances and write the per-corner pools the render
 * entry points read (vert_begin of a scene's job = the corner_begin of its
 * first instance, faces = 3 * arange).  Stream-ordered, graph-capturable. */
int rast_merge_objects(const RastMergeBatch* batch, void* workspace, size_t workspace_bytes, void* stream);

/* Display epilogue of the reference's notebooks: transpose_for_display(
 * (clamp(canvas, 0, 1) * 255).astype(uint8)) (renderer/utils.py:79-96).
 * canvas (n_images, width, height, channels) float, x-major as rendered ->
 * out (n_images, height, width, channels) uint8, row 0 the top when
 * flip_vertical.  Values are clamped with NaN -> 0 and truncated toward
 * zero. */
int rast_display_u8(const float* canvas, int64_t n_images, int32_t width, int32_t height, int32_t channels,
                    int32_t flip_vertical, uint8_t* out, void* stream);

/* Host-side validation of one job against pool sizes (no device access):
 * returns RAST_ERR_INVALID_ARGUMENT for inconsistent sizes. */
int rast_validate_job(const RastJob* job);

const char* rast_error_string(int status);
int rast_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* RAST_GB300_H */
