// Image decode for the image files PIV series come in (the image_samples of upstream
// fluidimage: uncompressed grayscale TIFF of 8 or 16 bits in one or many strips, 8-bit
// palette BMP, grayscale PNG of 8 or 16 bits), the step before the PIV path
// (fluidimage.util.imread, util/util.py:46-59, reading through fluiddyn.io.image).
//
// The host parses the container (a few hundred bytes of header) and hands over the
// pixel payload in one piece: a TIFF's strips, a BMP's pixel array, or a PNG's
// inflated and unfiltered scanlines.  k_image_unpack then writes the (height, width)
// image: row r starts at byte row_offsets[r] of the payload (strips, bottom-up BMP
// rows and row padding are all offsets), samples of 1 byte go through an optional
// 256-entry table (BMP palettes) and 2-byte samples are assembled in the file's byte
// order; `invert` maps WhiteIsZero images to BlackIsZero.
//
// PNG's DEFLATE stream and its Average and Paeth row filters are sequential by
// construction (a Huffman bit stream; each predictor needs the reconstructed byte to
// its left), so the scanlines are reconstructed on the host by fi_png_unfilter
// (native code, RFC 2083 section 6) before the copy.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fi_common.cuh"

namespace fi {

__global__ void __launch_bounds__(256)
    k_image_unpack(const uint8_t* __restrict__ raw, int64_t raw_bytes,
                   const int64_t* __restrict__ row_offsets, int height, int width,
                   int bytes_per_sample, int big_endian, const uint8_t* __restrict__ lut,
                   int invert, void* out, int32_t* status) {
  const int64_t row_bytes = (int64_t)width * bytes_per_sample;
  for (int r = blockIdx.y; r < height; r += gridDim.y) {
    const int64_t off = row_offsets[r];
    const bool in = off >= 0 && off <= raw_bytes - row_bytes;
    if (!in && threadIdx.x == 0 && blockIdx.x == 0 && status != nullptr) atomicExch(status, 1);
    const uint8_t* p = raw + (in ? off : 0);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < width; c += gridDim.x * blockDim.x) {
      const int64_t o = (int64_t)r * width + c;
      if (bytes_per_sample == 1) {
        unsigned v = in ? p[c] : 0u;
        if (lut != nullptr) v = lut[v];
        if (invert) v = 255u - v;
        static_cast<uint8_t*>(out)[o] = (uint8_t)v;
      } else {
        unsigned v = 0u;
        if (in) {
          const unsigned b0 = p[2 * c], b1 = p[2 * c + 1];
          v = big_endian ? (b0 << 8) | b1 : (b1 << 8) | b0;
        }
        if (invert) v = 65535u - v;
        static_cast<uint16_t*>(out)[o] = (uint16_t)v;
      }
    }
  }
}

}  // namespace fi

using namespace fi;

extern "C" int fi_image_unpack(const uint8_t* raw, int64_t raw_bytes, const int64_t* row_offsets,
                               int height, int width, int bytes_per_sample, int big_endian,
                               const uint8_t* lut, int invert, void* out, int32_t* status,
                               void* stream) {
  FI_REQUIRE(raw && row_offsets && out, "fi_image_unpack: null pointer");
  FI_REQUIRE(height >= 1 && width >= 1 && raw_bytes >= 1, "fi_image_unpack: empty image");
  FI_REQUIRE(bytes_per_sample == 1 || bytes_per_sample == 2,
             "fi_image_unpack: %d bytes per sample (1 or 2 supported)", bytes_per_sample);
  FI_REQUIRE(lut == nullptr || bytes_per_sample == 1,
             "fi_image_unpack: a sample table applies to 1-byte samples only");
  const int bx = (width + 255) / 256;
  const int by = height < 65535 ? height : 65535;
  k_image_unpack<<<dim3(bx < 64 ? bx : 64, by), 256, 0, (cudaStream_t)stream>>>(
      raw, raw_bytes, row_offsets, height, width, bytes_per_sample, big_endian, lut, invert,
      out, status);
  return check_launch("fi_image_unpack");
}

// PNG scanline reconstruction (RFC 2083 section 6), host memory.  `filtered` holds
// height rows of 1 + row_bytes bytes (the filter type, then the filtered row); the
// reconstructed rows go to `out` (height * row_bytes bytes).  bpp: bytes per complete
// pixel, rounded up to 1 (the left neighbour's distance).
extern "C" int fi_png_unfilter(const uint8_t* filtered, int height, int row_bytes, int bpp,
                               uint8_t* out) {
  FI_REQUIRE(filtered && out && height >= 1 && row_bytes >= 1 && bpp >= 1 && bpp <= 8,
             "fi_png_unfilter: bad arguments");
  for (int r = 0; r < height; ++r) {
    const uint8_t* f = filtered + (int64_t)r * (row_bytes + 1);
    const int type = f[0];
    ++f;
    uint8_t* x = out + (int64_t)r * row_bytes;
    const uint8_t* up = r > 0 ? x - row_bytes : nullptr;  // previous reconstructed row
    switch (type) {
      case 0:  // None
        for (int i = 0; i < row_bytes; ++i) x[i] = f[i];
        break;
      case 1:  // Sub: + the byte bpp to the left
        for (int i = 0; i < row_bytes; ++i)
          x[i] = (uint8_t)(f[i] + (i >= bpp ? x[i - bpp] : 0));
        break;
      case 2:  // Up: + the byte above
        for (int i = 0; i < row_bytes; ++i) x[i] = (uint8_t)(f[i] + (up ? up[i] : 0));
        break;
      case 3:  // Average: + floor((left + above) / 2)
        for (int i = 0; i < row_bytes; ++i) {
          const int a = i >= bpp ? x[i - bpp] : 0, b = up ? up[i] : 0;
          x[i] = (uint8_t)(f[i] + ((a + b) >> 1));
        }
        break;
      case 4:  // Paeth: + whichever of left, above, upper left is nearest a + b - c
        for (int i = 0; i < row_bytes; ++i) {
          const int a = i >= bpp ? x[i - bpp] : 0, b = up ? up[i] : 0;
          const int c = (up && i >= bpp) ? up[i - bpp] : 0;
          const int p = a + b - c;
          const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p,
                    pc = p > c ? p - c : c - p;
          const int pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          x[i] = (uint8_t)(f[i] + pred);
        }
        break;
      default:
        set_error("fi_png_unfilter: row %d has filter type %d (0-4 defined)", r, type);
        return FI_ERR_INVALID;
    }
  }
  return FI_OK;
}
