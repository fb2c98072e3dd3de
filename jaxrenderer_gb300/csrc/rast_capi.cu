// rast_capi.cu -- entry points of the C ABI that are not a render form:
// error names, ABI version, host-side job validation.
#include "rast_internal.cuh"

extern "C" const char* rast_error_string(int status) {
  switch (status) {
    case RAST_OK: return "ok";
    case RAST_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RAST_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case RAST_ERR_CUDA: return "CUDA runtime error";
    case RAST_ERR_UNSUPPORTED: return "unsupported";
    case RAST_ERR_TIMEOUT: return "device-side wait ran out of iterations";
    case RAST_ERR_BIN_OVERFLOW: return "tile bin capacity exceeded";
    case RAST_ERR_INDEX_OUT_OF_RANGE: return "index out of range";
    case RAST_ERR_STATIC_SCRATCH_TOO_SMALL: return "batch exceeds the static scratch of rast_render_tiled_static";
    default: return "unknown status";
  }
}

extern "C" int rast_abi_version(void) { return RAST_ABI_VERSION; }

// Host copy of a job: sizes consistent with what the kernels index.
extern "C" int rast_validate_job(const RastJob* j) {
  if (!j) return RAST_ERR_INVALID_ARGUMENT;
  if (j->shader < 0 || j->shader > RAST_SHADER_PHONG_REFLECTION_SHADOW) return RAST_ERR_INVALID_ARGUMENT;
  if (j->width < 0 || j->height < 0 || j->n_verts < 0 || j->n_faces < 0) return RAST_ERR_INVALID_ARGUMENT;
  if (static_cast<int64_t>(j->width) * j->height > (int64_t{1} << 31)) return RAST_ERR_INVALID_ARGUMENT;
  if (j->n_faces > 0 && j->n_verts <= 0) return RAST_ERR_INVALID_ARGUMENT;
  if (j->vert_begin < 0 || j->face_begin < 0 || j->pixel_begin < 0 || j->vout_begin < 0 ||
      j->setup_begin < 0)
    return RAST_ERR_INVALID_ARGUMENT;
  const int sh = j->shader;
  const bool textured = sh == RAST_SHADER_GOURAUD_TEXTURE || sh == RAST_SHADER_PHONG ||
                        sh == RAST_SHADER_PHONG_DARBOUX || sh == RAST_SHADER_PHONG_REFLECTION ||
                        sh == RAST_SHADER_PHONG_REFLECTION_SHADOW;
  if (textured && (j->tex_w <= 0 || j->tex_h <= 0 || (j->tex_c != 1 && j->tex_c != 3)))
    return RAST_ERR_INVALID_ARGUMENT;
  if ((sh == RAST_SHADER_PHONG_REFLECTION || sh == RAST_SHADER_PHONG_REFLECTION_SHADOW) &&
      (j->n_objects <= 0 || j->spec_w <= 0 || j->spec_h <= 0))
    return RAST_ERR_INVALID_ARGUMENT;
  if (sh == RAST_SHADER_PHONG_DARBOUX && (j->n_darboux_faces <= 0 || j->nm_w <= 0 || j->nm_h <= 0))
    return RAST_ERR_INVALID_ARGUMENT;
  if (sh == RAST_SHADER_PHONG_REFLECTION_SHADOW && (j->shadow_w < 0 || j->shadow_h < 0))
    return RAST_ERR_INVALID_ARGUMENT;
  // chooser / mix hooks: the layered chooser takes 1..RAST_MAX_LAYERS slots,
  // not for the DEPTH shader; the mixer is one of RastMixer
  if (j->layers < 0 || j->layers > RAST_MAX_LAYERS) return RAST_ERR_INVALID_ARGUMENT;
  if (j->layers > 0 && sh == RAST_SHADER_DEPTH) return RAST_ERR_INVALID_ARGUMENT;
  if (j->mixer != RAST_MIX_NEAREST && j->mixer != RAST_MIX_OVER) return RAST_ERR_INVALID_ARGUMENT;
  if (j->mixer == RAST_MIX_OVER && j->layers == 0) return RAST_ERR_INVALID_ARGUMENT;
  return RAST_OK;
}
