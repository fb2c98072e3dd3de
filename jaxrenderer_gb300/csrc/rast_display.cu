// rast_display.cu -- the notebooks' display epilogue on the device:
// transpose_for_display((clamp(canvas, 0, 1) * 255).astype(uint8))
// (renderer/utils.py:79-96).  One thread per output byte quad: reads are
// x-major canvas floats, writes the row-major image.
#include <cuda_runtime.h>

#include "rast_internal.cuh"

namespace rast {
namespace display {

constexpr int kThreads = 256;

// Grid: (ceil(width * height / kThreads), n_images).  Thread t of image n is
// output pixel (row r, column i) = t / width, t % width.
__global__ void __launch_bounds__(kThreads)
display_kernel(const float* __restrict__ canvas, int width, int height, int channels, bool flip,
               uint8_t* __restrict__ out) {
  const int64_t n = blockIdx.y;
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= width * height) return;
  const int r = t / width, i = t - r * width;
  const int j = flip ? height - 1 - r : r;
  const float* src = canvas + ((n * width + i) * height + j) * channels;
  uint8_t* dst = out + ((n * height + r) * width + i) * channels;
  for (int c = 0; c < channels; ++c) {
    const float v = fminf(fmaxf(src[c], 0.0f), 1.0f);  // NaN -> 0
    dst[c] = static_cast<uint8_t>(__float2uint_rz(v * 255.0f));
  }
}

}  // namespace display
}  // namespace rast

extern "C" int rast_display_u8(const float* canvas, int64_t n_images, int32_t width, int32_t height,
                               int32_t channels, int32_t flip_vertical, uint8_t* out, void* stream) {
  using namespace rast;
  NvtxRange range("rast_display_u8");
  if (n_images < 0 || width < 0 || height < 0 || channels <= 0) return RAST_ERR_INVALID_ARGUMENT;
  if (n_images == 0 || width == 0 || height == 0) return RAST_OK;
  if (!canvas || !out) return RAST_ERR_INVALID_ARGUMENT;
  if (n_images > 65535 || static_cast<int64_t>(width) * height > 0x7fffffffll) return RAST_ERR_UNSUPPORTED;
  const dim3 grid(static_cast<unsigned>((static_cast<int64_t>(width) * height + display::kThreads - 1) /
                                        display::kThreads),
                  static_cast<unsigned>(n_images));
  display::display_kernel<<<grid, display::kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      canvas, width, height, channels, flip_vertical != 0, out);
  return cudaGetLastError() == cudaSuccess ? RAST_OK : RAST_ERR_CUDA;
}
