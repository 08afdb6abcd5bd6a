// Image preprocessing on the device: the scipy.ndimage / numpy tools of
// fluidimage's preprocessing toolbox (works/preproc/_toolbox_py.py:66-155,
// 189-256, 265-289, 332-355).
//
// * rank filters (minimum / maximum / median / percentile) over a box window of a
//   stack of images (nt, ny, nx), with the boundary modes of scipy.ndimage
//   ('reflect', 'mirror', 'nearest', 'wrap', 'constant'), window [i - s//2,
//   i - s//2 + s - 1] along each axis; min and max are separable (one pass per
//   axis), other ranks select the rank-th smallest window value exactly by a
//   radix select on order-preserving integer keys (exact for every dtype);
// * img - weight * filtered with numpy's result type (float64 for integer images
//   and a float weight, float32 for float32 images, wrapping integer arithmetic for
//   an integer weight), optionally clamped at 0;
// * clamping (global_threshold) and the tanh rescaling (rescale_intensity_tanh);
// * the linear rescaling of rescale_intensity (:313-331) and the power law of
//   gamma_correction (:441-470), which upstream takes from scikit-image 0.24
//   (exposure.rescale_intensity with in_range='image' and a numeric out_range;
//   exposure.adjust_gamma), restated from their published definitions.
#include <cstdint>
#include <cstring>

#include "fi_common.cuh"

namespace fi {

// ------------------------------------------------------------------ element access
__device__ __forceinline__ double load_d(const void* p, int dtype, int64_t i) {
  switch (dtype) {
    case FI_PRE_U8: return (double)static_cast<const uint8_t*>(p)[i];
    case FI_PRE_U16: return (double)static_cast<const uint16_t*>(p)[i];
    case FI_PRE_F32: return (double)static_cast<const float*>(p)[i];
    default: return static_cast<const double*>(p)[i];
  }
}

// Order-preserving unsigned key of an element (floats: the sign-magnitude order
// mapped to unsigned order).  NaN has no place in that order: callers reject
// images with NaN.
__device__ __forceinline__ uint64_t key_of(const void* p, int dtype, int64_t i) {
  switch (dtype) {
    case FI_PRE_U8: return static_cast<const uint8_t*>(p)[i];
    case FI_PRE_U16: return static_cast<const uint16_t*>(p)[i];
    case FI_PRE_F32: {
      const uint32_t u = __float_as_uint(static_cast<const float*>(p)[i]);
      return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
    default: {
      const uint64_t u = (uint64_t)__double_as_longlong(static_cast<const double*>(p)[i]);
      return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
    }
  }
}

__device__ __forceinline__ void store_key(void* p, int dtype, int64_t i, uint64_t k) {
  switch (dtype) {
    case FI_PRE_U8: static_cast<uint8_t*>(p)[i] = (uint8_t)k; break;
    case FI_PRE_U16: static_cast<uint16_t*>(p)[i] = (uint16_t)k; break;
    case FI_PRE_F32: {
      const uint32_t u = (uint32_t)k;
      static_cast<float*>(p)[i] = __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
      break;
    }
    default: {
      const uint64_t u = k;
      static_cast<double*>(p)[i] = __longlong_as_double(
          (long long)((u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u));
    }
  }
}

__device__ __forceinline__ int key_bits(int dtype) {
  return dtype == FI_PRE_U8 ? 8 : dtype == FI_PRE_U16 ? 16 : dtype == FI_PRE_F32 ? 32 : 64;
}

// scipy.ndimage boundary extension of index i on an axis of length n; -1 means
// "use cval" (mode 'constant').
__device__ __forceinline__ int64_t extend(int64_t i, int64_t n, int mode) {
  if (i >= 0 && i < n) return i;
  switch (mode) {
    case FI_MODE_NEAREST: return i < 0 ? 0 : n - 1;
    case FI_MODE_WRAP: {
      int64_t r = i % n;
      return r < 0 ? r + n : r;
    }
    case FI_MODE_CONSTANT: return -1;
    case FI_MODE_MIRROR: {
      if (n == 1) return 0;
      const int64_t p = 2 * n - 2;
      int64_t r = i % p;
      if (r < 0) r += p;
      return r < n ? r : p - r;
    }
    default: {  // reflect: d c b a | a b c d | d c b a
      const int64_t p = 2 * n;
      int64_t r = i % p;
      if (r < 0) r += p;
      return r < n ? r : p - 1 - r;
    }
  }
}

// ------------------------------------------------------------------ gaussian
// One axis of scipy.ndimage.gaussian_filter1d (ndimage/_filters.py; the C line
// correlation with a symmetric kernel) over a (nt, ny, nx) stack: the line values as
// float64, out = w_0 x_0, then, from the outermost pair of taps inwards,
// out += (x_-j + x_j) w_j, each product and sum rounded (no contraction); 'reflect'
// extension; the result cast to the image dtype as a C cast (truncation for the
// integer types, round to nearest for float32).
__device__ __forceinline__ void store_cast(void* p, int dtype, int64_t i, double v) {
  switch (dtype) {
    case FI_PRE_U8: static_cast<uint8_t*>(p)[i] = (uint8_t)v; break;
    case FI_PRE_U16: static_cast<uint16_t*>(p)[i] = (uint16_t)v; break;
    case FI_PRE_F32: static_cast<float*>(p)[i] = __double2float_rn(v); break;
    default: static_cast<double*>(p)[i] = v;
  }
}

__global__ void k_gauss_axis(const void* in, void* out, int dtype, int nt, int ny, int nx,
                             int axis, const double* __restrict__ w, int radius) {
  const int64_t count = (int64_t)nt * ny * nx;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < count;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(idx % nx);
    const int y = (int)((idx / nx) % ny);
    const int64_t base = idx - (axis == 1 ? x : (int64_t)y * nx);
    const int64_t n = axis == 1 ? nx : ny;
    const int64_t step = axis == 1 ? 1 : nx;
    const int pos = axis == 1 ? x : y;
    double acc = __dmul_rn(load_d(in, dtype, base + (int64_t)pos * step), w[radius]);
    for (int j = radius; j >= 1; --j) {
      const double a = load_d(in, dtype, base + extend(pos - j, n, FI_MODE_REFLECT) * step);
      const double b = load_d(in, dtype, base + extend(pos + j, n, FI_MODE_REFLECT) * step);
      acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(a, b), w[radius - j]));
    }
    store_cast(out, dtype, idx, acc);
  }
}

// out = blurred + alpha * (blurred - filtered) with numpy's promotions (sharpen,
// _toolbox_py.py:472-490): integer images subtract in their own type (wrapping) and
// give float64; float32 stays float32 (alpha rounded to float32); float64 is float64.
__global__ void k_sharpen_combine(const void* blurred, const void* filtered, int dtype,
                                  int64_t count, double alpha, void* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    switch (dtype) {
      case FI_PRE_U8: {
        const uint8_t b = static_cast<const uint8_t*>(blurred)[i];
        const uint8_t d = (uint8_t)(b - static_cast<const uint8_t*>(filtered)[i]);
        static_cast<double*>(out)[i] = __dadd_rn((double)b, __dmul_rn(alpha, (double)d));
        break;
      }
      case FI_PRE_U16: {
        const uint16_t b = static_cast<const uint16_t*>(blurred)[i];
        const uint16_t d = (uint16_t)(b - static_cast<const uint16_t*>(filtered)[i]);
        static_cast<double*>(out)[i] = __dadd_rn((double)b, __dmul_rn(alpha, (double)d));
        break;
      }
      case FI_PRE_F32: {
        const float b = static_cast<const float*>(blurred)[i];
        const float d = __fsub_rn(b, static_cast<const float*>(filtered)[i]);
        static_cast<float*>(out)[i] = __fadd_rn(b, __fmul_rn(__double2float_rn(alpha), d));
        break;
      }
      default: {
        const double b = static_cast<const double*>(blurred)[i];
        const double d = __dsub_rn(b, static_cast<const double*>(filtered)[i]);
        static_cast<double*>(out)[i] = __dadd_rn(b, __dmul_rn(alpha, d));
      }
    }
  }
}

// ------------------------------------------------------------------ min / max
// One axis of a separable minimum or maximum filter over a (nt, ny, nx) stack.
// Keys compare like the values; cval enters as its key.
__global__ void k_minmax_axis(const void* in, int in_is_key, const uint64_t* kin, int dtype,
                              int64_t nt, int64_t ny, int64_t nx, int axis, int size, int mode,
                              uint64_t ckey, int is_max, uint64_t* kout) {
  const int64_t total = nt * ny * nx;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e % nx, y = (e / nx) % ny, t = e / (nx * ny);
    const int64_t n = axis == 0 ? nt : axis == 1 ? ny : nx;
    const int64_t pos = axis == 0 ? t : axis == 1 ? y : x;
    const int64_t stride = axis == 0 ? ny * nx : axis == 1 ? nx : 1;
    const int64_t base = e - pos * stride;
    uint64_t best = is_max ? 0ull : ~0ull;
    const int64_t s0 = pos - size / 2;
    for (int k = 0; k < size; ++k) {
      const int64_t j = extend(s0 + k, n, mode);
      const uint64_t v = (j < 0) ? ckey : (in_is_key ? kin[base + j * stride]
                                                      : key_of(in, dtype, base + j * stride));
      best = is_max ? (v > best ? v : best) : (v < best ? v : best);
    }
    kout[e] = best;
  }
}

__global__ void k_keys_to_values(const uint64_t* k, int dtype, int64_t count, void* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    store_key(out, dtype, e, k[e]);
}

// ------------------------------------------------------------------ rank select
// The rank-th smallest value of each box window, by a radix select over the keys
// (most significant bit first): per bit, count the window values whose key shares
// the prefix found so far and has a 0 at this bit.
__global__ void k_rank_select(const void* in, int dtype, int64_t nt, int64_t ny, int64_t nx,
                              int st, int sy, int sx, int rank, int mode, uint64_t ckey,
                              void* out) {
  const int64_t total = nt * ny * nx;
  const int bits = key_bits(dtype);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e % nx, y = (e / nx) % ny, t = e / (nx * ny);
    const int64_t t0 = t - st / 2, y0 = y - sy / 2, x0 = x - sx / 2;
    uint64_t prefix = 0;
    int r = rank;
    for (int b = bits - 1; b >= 0; --b) {
      const uint64_t hi_mask = (b == 63) ? 0ull : (~0ull << (b + 1));
      int zeros = 0;
      for (int a = 0; a < st; ++a) {
        const int64_t ta = extend(t0 + a, nt, mode);
        for (int c = 0; c < sy; ++c) {
          const int64_t yc = extend(y0 + c, ny, mode);
          for (int d = 0; d < sx; ++d) {
            const int64_t xd = extend(x0 + d, nx, mode);
            const uint64_t v = (ta < 0 || yc < 0 || xd < 0)
                                   ? ckey
                                   : key_of(in, dtype, (ta * ny + yc) * nx + xd);
            if ((v & hi_mask) == prefix && !((v >> b) & 1ull)) ++zeros;
          }
        }
      }
      if (r >= zeros) {
        r -= zeros;
        prefix |= (1ull << b);
      }
    }
    store_key(out, dtype, e, prefix);
  }
}

// The same for 2-D windows (st == 1) of integer and float32 images, by tiles: a
// block stages its output tile plus the window halo (boundary extension applied
// once per staged element) as 32-bit keys in shared memory, then each thread runs
// the radix select over its window there; the select starts at the highest key bit
// set in the tile (higher bits are zero for every staged value).
constexpr int RS_TX = 32, RS_TY = 16;
constexpr int RS_MAX_SMEM = 96 * 1024;

__global__ void __launch_bounds__(RS_TX * RS_TY)
    k_rank_select_tile(const void* in, int dtype, int64_t ny, int64_t nx, int sy, int sx,
                       int rank, int mode, uint32_t ckey, void* out) {
  extern __shared__ uint32_t patch[];
  __shared__ uint32_t s_or;
  const int pw = RS_TX + sx - 1, ph = RS_TY + sy - 1;
  const int64_t t = blockIdx.z;
  const int64_t x00 = (int64_t)blockIdx.x * RS_TX - sx / 2;
  const int64_t y00 = (int64_t)blockIdx.y * RS_TY - sy / 2;
  const int tid = threadIdx.y * RS_TX + threadIdx.x;
  if (tid == 0) s_or = 0u;
  __syncthreads();
  uint32_t acc_or = 0u;
  for (int e = tid; e < pw * ph; e += RS_TX * RS_TY) {
    const int py = e / pw, px = e - py * pw;
    const int64_t yc = extend(y00 + py, ny, mode), xd = extend(x00 + px, nx, mode);
    const uint32_t v = (yc < 0 || xd < 0) ? ckey
                                          : (uint32_t)key_of(in, dtype, (t * ny + yc) * nx + xd);
    patch[e] = v;
    acc_or |= v;
  }
  for (int o = 16; o > 0; o >>= 1) acc_or |= __shfl_xor_sync(0xffffffffu, acc_or, o);
  if ((tid & 31) == 0) atomicOr(&s_or, acc_or);
  __syncthreads();
  const int64_t x = (int64_t)blockIdx.x * RS_TX + threadIdx.x;
  const int64_t y = (int64_t)blockIdx.y * RS_TY + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const uint32_t all = s_or;
  int top = 31;
  while (top >= 0 && !((all >> top) & 1u)) --top;
  uint32_t prefix = 0u;
  int r = rank;
  for (int b = top; b >= 0; --b) {
    const uint32_t hi_mask = (b == 31) ? 0u : (~0u << (b + 1));
    int zeros = 0;
    for (int c = 0; c < sy; ++c) {
      const uint32_t* row = patch + (threadIdx.y + c) * pw + threadIdx.x;
      for (int d = 0; d < sx; ++d) {
        const uint32_t v = row[d];
        zeros += ((v & hi_mask) == prefix && !((v >> b) & 1u)) ? 1 : 0;
      }
    }
    if (r >= zeros) {
      r -= zeros;
      prefix |= (1u << b);
    }
  }
  store_key(out, dtype, (t * ny + y) * nx + x, prefix);
}

// ------------------------------------------------------------------ arithmetic
// out = img - weight * filt in the numpy result type out_dtype: FI_PRE_F64 /
// FI_PRE_F32 (float arithmetic; float32 for float32 images), or the image's integer
// type (an integer weight: wrapping integer arithmetic); clamp: negatives -> 0.
__global__ void k_subtract_weighted(const void* img, const void* filt, int dtype, int64_t count,
                                    double weight, int out_dtype, int clamp, void* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (out_dtype == FI_PRE_F64) {
      // product rounded before the difference, like numpy (no FMA contraction)
      const double v = __dsub_rn(load_d(img, dtype, e), __dmul_rn(weight, load_d(filt, dtype, e)));
      static_cast<double*>(out)[e] = (clamp && v < 0.0) ? 0.0 : v;
    } else if (out_dtype == FI_PRE_F32) {
      const float w = (float)weight;
      const float v = __fsub_rn((float)load_d(img, dtype, e),
                                __fmul_rn(w, (float)load_d(filt, dtype, e)));
      static_cast<float*>(out)[e] = (clamp && v < 0.f) ? 0.f : v;
    } else {  // integer weight on an integer image: modular arithmetic of the dtype
      const int64_t w = (int64_t)weight;
      const int64_t v = (int64_t)load_d(img, dtype, e) - w * (int64_t)load_d(filt, dtype, e);
      if (out_dtype == FI_PRE_U8) static_cast<uint8_t*>(out)[e] = (uint8_t)v;
      else static_cast<uint16_t*>(out)[e] = (uint16_t)v;
    }
  }
}

// global_threshold: img_out[img_out < lo] = lo; img_out[img_out > hi] = hi (the
// bounds already converted to the image's dtype by the caller).
__global__ void k_clamp(const void* in, int dtype, int64_t count, double lo, double hi, void* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = load_d(in, dtype, e);
    const double w = v < lo ? lo : (v > hi ? hi : v);
    switch (dtype) {
      case FI_PRE_U8: static_cast<uint8_t*>(out)[e] = (uint8_t)w; break;
      case FI_PRE_U16: static_cast<uint16_t*>(out)[e] = (uint16_t)w; break;
      case FI_PRE_F32: static_cast<float*>(out)[e] = (float)w; break;
      default: static_cast<double*>(out)[e] = w;
    }
  }
}

// Per block: sum of img**2 in the image dtype's arithmetic (integer squares wrap
// modulo 2^bits like numpy's img**2) accumulated in float64, and max(img).
__global__ void k_sq_sum_max(const void* in, int dtype, int64_t count, double* part_sum,
                             double* part_max) {
  __shared__ double ss[32], sm[32];
  double s = 0.0, m = -INFINITY;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = load_d(in, dtype, e);
    double q;
    if (dtype == FI_PRE_U8) q = (double)(uint8_t)((uint32_t)v * (uint32_t)v);
    else if (dtype == FI_PRE_U16) q = (double)(uint16_t)((uint32_t)v * (uint32_t)v);
    else if (dtype == FI_PRE_F32) q = (double)__fmul_rn((float)v, (float)v);
    else q = v * v;
    s += q;
    m = fmax(m, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    ss[wid] = s;
    sm[wid] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = -INFINITY;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += ss[w];
      b = fmax(b, sm[w]);
    }
    part_sum[blockIdx.x] = a;
    part_max[blockIdx.x] = b;
  }
}

// rescale_intensity_tanh: out = floor(max(img) / max(tanh(img / thr)) * tanh(img / thr))
// in float64 (tanh is increasing, so max(tanh(img / thr)) = tanh(max(img) / thr)).
__global__ void k_tanh_rescale(const void* in, int dtype, int64_t count, double thr,
                               double scale, double* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = floor(scale * tanh(load_d(in, dtype, e) / thr));
}

// NaN-propagating min / max (numpy's ndarray.min / max).
__device__ __forceinline__ double nan_min(double a, double b) {
  return (a != a || b < a || b != b) ? (a != a ? a : b) : a;
}
__device__ __forceinline__ double nan_max(double a, double b) {
  return (a != a || b > a || b != b) ? (a != a ? a : b) : a;
}

// Per block: min and max of the image (NaN-propagating); part[0..nparts) the minima,
// part[nparts..2 nparts) the maxima.
__global__ void k_min_max_part(const void* in, int dtype, int64_t count, double* part) {
  __shared__ double smn[32], smx[32];
  double mn = INFINITY, mx = -INFINITY;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = load_d(in, dtype, e);
    mn = nan_min(mn, v);
    mx = nan_max(mx, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = nan_min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = nan_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    smn[wid] = mn;
    smx[wid] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mn = nan_min(mn, smn[w]);
      mx = nan_max(mx, smx[w]);
    }
    part[blockIdx.x] = mn;
    part[gridDim.x + blockIdx.x] = mx;
  }
}

// The block's first warp reduces the nparts partial extremes to (imin, imax).
__device__ void reduce_parts(const double* part, int nparts, double* out2) {
  if (threadIdx.x < 32) {
    double mn = INFINITY, mx = -INFINITY;
    for (int i = threadIdx.x; i < nparts; i += 32) {
      mn = nan_min(mn, part[i]);
      mx = nan_max(mx, part[nparts + i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      mn = nan_min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = nan_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (threadIdx.x == 0) {
      out2[0] = mn;
      out2[1] = mx;
    }
  }
  __syncthreads();
}

// rescale_intensity(img, out_range=(omin, omax)), in_range = the image's extremes:
// x clipped to [imin, imax] (a no-op), then (x - imin) / (imax - imin) * (omax - omin)
// + omin, each operation rounded, in float64 for integer and float64 images and in
// float32 for float32 images (the Python-float operands rounded to float32, as
// numpy 2 does with a float32 array); when imin == imax, x clipped to [omin, omax].
__global__ void k_rescale_linear(const void* in, int dtype, int64_t count, const double* part,
                                 int nparts, double omin, double omax, void* out) {
  __shared__ double ext[2];
  reduce_parts(part, nparts, ext);
  const double imin = ext[0], imax = ext[1];
  const bool flat = !(imin != imax);
  const double span_in = imax - imin, span_out = omax - omin;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = load_d(in, dtype, e);
    if (dtype == FI_PRE_F32) {
      const float x = (float)v;
      float r;
      if (flat) {
        const float lo = (float)omin, hi = (float)omax;
        r = fminf(fmaxf(x, lo), hi);
        if (x != x) r = x;
      } else {
        r = __fdiv_rn(__fsub_rn(x, (float)imin), (float)span_in);
        r = __fadd_rn(__fmul_rn(r, (float)span_out), (float)omin);
      }
      static_cast<float*>(out)[e] = r;
    } else {
      double r;
      if (flat) {
        r = fmin(fmax(v, omin), omax);
        if (v != v) r = v;
      } else {
        r = __ddiv_rn(__dsub_rn(v, imin), span_in);
        r = __dadd_rn(__dmul_rn(r, span_out), omin);
      }
      static_cast<double*>(out)[e] = r;
    }
  }
}

// x ** g of a float array as numpy evaluates it: exponents 0, 0.5, 1 and 2 by their
// exact operations (ones, correctly rounded square root, copy, product), others by pow.
__device__ __forceinline__ double np_pow(double x, double g) {
  if (g == 1.0) return x;
  if (g == 2.0) return __dmul_rn(x, x);
  if (g == 0.5) return __dsqrt_rn(x);
  if (g == 0.0) return 1.0;
  return pow(x, g);
}
__device__ __forceinline__ float np_powf(float x, float g) {
  if (g == 1.f) return x;
  if (g == 2.f) return __fmul_rn(x, x);
  if (g == 0.5f) return __fsqrt_rn(x);
  if (g == 0.f) return 1.f;
  return (float)pow((double)x, (double)g);
}

// gamma_correction = adjust_gamma(img, gamma, gain): uint8 through the 256-entry
// table lut; otherwise ((x / scale) ** gamma) * scale * gain cast back to the image
// dtype, scale = the dtype's upper limit (65535 for uint16, 1 for floats), in float64
// for uint16 and float64 images and in float32 for float32 images (gamma and gain
// rounded to float32); the cast to uint16 truncates toward zero and saturates.
__global__ void k_gamma(const void* in, int dtype, int64_t count, double gamma, double gain,
                        const uint8_t* __restrict__ lut, void* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    switch (dtype) {
      case FI_PRE_U8:
        static_cast<uint8_t*>(out)[e] = lut[static_cast<const uint8_t*>(in)[e]];
        break;
      case FI_PRE_U16: {
        const double x = __ddiv_rn((double)static_cast<const uint16_t*>(in)[e], 65535.0);
        const double y = __dmul_rn(__dmul_rn(np_pow(x, gamma), 65535.0), gain);
        const double t = trunc(y);
        static_cast<uint16_t*>(out)[e] = (uint16_t)(t < 0.0 ? 0.0 : (t > 65535.0 ? 65535.0 : t));
        break;
      }
      case FI_PRE_F32: {
        const float x = static_cast<const float*>(in)[e];
        static_cast<float*>(out)[e] = __fmul_rn(np_powf(x, (float)gamma), (float)gain);
        break;
      }
      default: {
        const double x = static_cast<const double*>(in)[e];
        static_cast<double*>(out)[e] = __dmul_rn(np_pow(x, gamma), gain);
      }
    }
  }
}

// ---------------------------------------------------------- histogram equalisation
// equalize_hist_global = skimage.exposure.equalize_hist (scikit-image 0.24): the
// cumulative distribution of the image's histogram, interpolated at every pixel.
// Integer images: one bin per integer value (the histogram of the raw values; the
// bins below the minimum are empty, so the cumulative sums equal those from the
// minimum), out = cdf[x] exactly (np.interp at its nodes).  Float images: numpy's
// uniform histogram of nbins bins over [min, max] — bin index
// ((x - first) / denom) * nbins truncated, then moved by one where x lies below its
// bin's left edge or at or above the next edge (the last bin is closed) — in the
// image's float type, with the edges computed by the caller exactly as numpy does.
__global__ void k_hist_int(const void* in, int dtype, int64_t count, unsigned* hist) {
  __shared__ unsigned sh[256];
  const bool u8 = dtype == FI_PRE_U8;
  if (u8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
  }
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (u8)
      atomicAdd(&sh[static_cast<const uint8_t*>(in)[e]], 1u);
    else
      atomicAdd(&hist[static_cast<const uint16_t*>(in)[e]], 1u);
  }
  if (u8) {
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
  }
}

template <typename T>
__device__ __forceinline__ int np_bin(T x, const T* edges, int nbins, T first, T denom) {
  T f;
  if constexpr (sizeof(T) == 4)
    f = __fmul_rn(__fdiv_rn(__fsub_rn(x, first), denom), (float)nbins);
  else
    f = __dmul_rn(__ddiv_rn(__dsub_rn(x, first), denom), (double)nbins);
  int i = (int)f;
  if (i == nbins) --i;
  if (x < edges[i]) --i;
  if (i != nbins - 1 && x >= edges[i + 1]) ++i;
  return i;
}

// edges: nbins + 1 values in the image's float type (float32 images: float
// values stored as float), first / denom likewise (as doubles, exact).
__global__ void k_hist_float(const void* in, int dtype, int64_t count, const void* edges,
                             int nbins, double first, double denom, unsigned* hist) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    int i;
    if (dtype == FI_PRE_F32) {
      const float x = static_cast<const float*>(in)[e];
      i = np_bin<float>(x, static_cast<const float*>(edges), nbins, (float)first, (float)denom);
    } else {
      const double x = static_cast<const double*>(in)[e];
      i = np_bin<double>(x, static_cast<const double*>(edges), nbins, first, denom);
    }
    atomicAdd(&hist[i], 1u);
  }
}

// One block: cdf[i] = (sum of hist[0..i]) / total (float64), rounded to float32
// and back when round32 (the cdf of float32 images).
__global__ void k_cdf(const unsigned* hist, int nbins, int round32, double* cdf) {
  __shared__ unsigned long long part[1024];
  const int per = (nbins + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  unsigned long long s = 0;
  for (int i = b0; i < b0 + per && i < nbins; ++i) s += hist[i];
  part[threadIdx.x] = s;
  __syncthreads();
  // inclusive scan of the per-thread sums (Hillis-Steele over the block)
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const unsigned long long v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0ull;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const double total = (double)part[blockDim.x - 1];
  unsigned long long run = threadIdx.x ? part[threadIdx.x - 1] : 0ull;
  for (int i = b0; i < b0 + per && i < nbins; ++i) {
    run += hist[i];
    const double c = __ddiv_rn((double)run, total);
    cdf[i] = round32 ? (double)(float)c : c;
  }
}

// Integer images: out = cdf[x] (float64).
__global__ void k_equalize_int(const void* in, int dtype, int64_t count, const double* cdf,
                               double* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int v = dtype == FI_PRE_U8 ? (int)static_cast<const uint8_t*>(in)[e]
                                     : (int)static_cast<const uint16_t*>(in)[e];
    out[e] = cdf[v];
  }
}

// np.interp(x, xp, fp) in float64 (xp increasing, n >= 1): fp[0] below xp[0],
// fp[n-1] from xp[n-1] on, the node value at a node, else the slope form
// slope (x - xp[j]) + fp[j] without contraction (then from the right node if NaN).
// Output in the image's float type.
__global__ void k_interp(const void* in, int dtype, int64_t count, const double* xp,
                         const double* fp, int n, void* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double x = load_d(in, dtype, e);
    double r;
    if (x > xp[n - 1] || x == xp[n - 1]) {
      r = fp[n - 1];
    } else if (x < xp[0]) {
      r = fp[0];
    } else if (x != x) {
      r = x;
    } else {
      int lo = 0, hi = n - 1;  // xp[lo] <= x < xp[hi]
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (xp[mid] <= x) lo = mid; else hi = mid;
      }
      if (xp[lo] == x) {
        r = fp[lo];
      } else {
        const double slope = __ddiv_rn(__dsub_rn(fp[lo + 1], fp[lo]), __dsub_rn(xp[lo + 1], xp[lo]));
        r = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[lo])), fp[lo]);
        if (r != r) {
          r = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[lo + 1])), fp[lo + 1]);
          if (r != r && fp[lo] == fp[lo + 1]) r = fp[lo];
        }
      }
    }
    if (dtype == FI_PRE_F32)
      static_cast<float*>(out)[e] = (float)r;
    else
      static_cast<double*>(out)[e] = r;
  }
}

static int grid_for(int64_t count) {
  const int64_t b = (count + 255) / 256;
  return (int)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

// ------------------------------------------------------------------ CLAHE
// Contrast-limited adaptive histogram equalisation (Zuiderveld, Graphics Gems IV,
// 1994) in the variant of scikit-image 0.24 (equalize_adapthist / _clahe /
// clip_histogram / map_histogram), the core of equalize_hist_adapt
// (_toolbox_py.py:383-409).  Grey levels: 2^14.
constexpr int CLAHE_GREYS = 16384;
constexpr int CLAHE_NT = 256;

// numpy 'reflect' padding index for i >= 0 (mirror without repeating the edge)
__device__ __forceinline__ int reflect_index(int i, int n) {
  if (n == 1) return 0;
  const int period = 2 * (n - 1);
  const int m = i % period;
  return m >= n ? period - m : m;
}

// the grey level of a pixel of the image rescaled to [0, 2^14 - 1]: astype(uint16)
// (truncation), clamped into the table range
__device__ __forceinline__ int clahe_level(const void* y, int dtype, int64_t e) {
  const double v = load_d(y, dtype, e);
  if (!(v >= 0.0)) return 0;
  if (v >= (double)(CLAHE_GREYS - 1)) return CLAHE_GREYS - 1;
  return (int)v;
}

// sum over the block of one int per thread (all threads call it); sh: 33 ints
__device__ __forceinline__ int block_sum_int(int v, int* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[32] = v;
  }
  __syncthreads();
  v = sh[32];
  __syncthreads();
  return v;
}

// One block per contextual region (i, j) of k0 x k1 pixels starting at image pixel
// (i k0, j k1), the image extended at its end by reflection: histogram of the bins
// level / bin_size, clipped at clim with the excess handed out again, and the map
// min(cdf * scale, 2^14 - 1) truncated, stored as uint16 (maps[(i m1 + j) nbins + b]).
// The redistribution: excess // nbins to every bin below clim - that, the bins
// between that and clim filled to it, then one count at a time to the bins below
// clim in strides of max(1, (bins below clim) // excess) from each start bin in turn
// until no excess is left or a full pass hands out nothing (bounded: each pass that
// continues hands out at least one count of an excess of at most k0 k1).
__global__ void __launch_bounds__(CLAHE_NT)
    k_clahe_maps(const void* levels, int dtype, int s0, int s1, int k0, int k1, int m1,
                 int nbins, int bin_size, int clim, double scale, uint16_t* maps) {
  extern __shared__ int hist[];
  __shared__ int red[33];
  const int i = blockIdx.x / m1, j = blockIdx.x % m1;
  for (int b = threadIdx.x; b < nbins; b += CLAHE_NT) hist[b] = 0;
  __syncthreads();
  const int npix = k0 * k1;
  for (int t = threadIdx.x; t < npix; t += CLAHE_NT) {
    const int r = t / k1, c = t - r * k1;
    const int row = reflect_index(i * k0 + r, s0), col = reflect_index(j * k1 + c, s1);
    atomicAdd(&hist[clahe_level(levels, dtype, (int64_t)row * s1 + col) / bin_size], 1);
  }
  __syncthreads();
  // the bins above the limit are cut
  int part = 0;
  for (int b = threadIdx.x; b < nbins; b += CLAHE_NT) {
    const int h = hist[b];
    if (h > clim) {
      part += h - clim;
      hist[b] = clim;
    }
  }
  int excess = block_sum_int(part, red);
  const int incr = excess / nbins, upper = clim - incr;
  part = 0;
  for (int b = threadIdx.x; b < nbins; b += CLAHE_NT) {
    int h = hist[b];
    if (h < upper) {
      h += incr;
      part += incr;
    }
    if (h >= upper && h < clim) {
      part += clim - h;
      h = clim;
    }
    hist[b] = h;
  }
  excess -= block_sum_int(part, red);
  while (excess > 0) {
    const int before = excess;
    for (int start = 0; start < nbins; ++start) {
      int under = 0;
      for (int b = threadIdx.x; b < nbins; b += CLAHE_NT) under += hist[b] < clim;
      under = block_sum_int(under, red);
      const int stride = max(1, under / excess);
      int given = 0;
      for (int p = start + threadIdx.x * stride; p < nbins; p += CLAHE_NT * stride) {
        if (hist[p] < clim) {
          hist[p] += 1;
          ++given;
        }
      }
      excess -= block_sum_int(given, red);
      if (excess <= 0) break;
    }
    if (before == excess) break;
  }
  // cumulative counts (each thread a run of bins) and the grey-level map
  const int per = (nbins + CLAHE_NT - 1) / CLAHE_NT;
  const int b0 = min(nbins, (int)threadIdx.x * per), b1 = min(nbins, b0 + per);
  int local = 0;
  for (int b = b0; b < b1; ++b) local += hist[b];
  // exclusive scan of the per-thread sums
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) red[wid] = incl;
  __syncthreads();
  int before_warp = 0;
  for (int w = 0; w < wid; ++w) before_warp += red[w];
  int run = before_warp + incl - local;
  uint16_t* map = maps + (int64_t)blockIdx.x * nbins;
  for (int b = b0; b < b1; ++b) {
    run += hist[b];
    const double v = fmin(__dmul_rn((double)run, scale), (double)(CLAHE_GREYS - 1));
    map[b] = (uint16_t)(int)v;
  }
}

// Each pixel: the blend of the maps of the four regions around it.  In the image
// shifted by half a region (k0 / 2, k1 / 2), the pixel sits in block (bi, bj) at
// (r, c); the coefficients are r / k0 and c / k1 (float64), the blocks' maps those of
// regions (bi - 1 + e0, bj - 1 + e1) clamped to the grid.  Each term map * weight is
// rounded to float32 and added in float32 in the order (0, 0), (0, 1), (1, 0),
// (1, 1); the sum is truncated to an integer level, written in the image's float type.
__global__ void k_clahe_blend(const void* levels, int dtype, int s0, int s1, int k0, int k1,
                              int m0, int m1, int nbins, int bin_size, const uint16_t* maps,
                              void* out) {
  const int64_t count = (int64_t)s0 * s1;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(e / s1), x = (int)(e - (int64_t)y * s1);
    const int py = y + k0 / 2, px = x + k1 / 2;
    const int bi = py / k0, bj = px / k1;
    const double cy = __ddiv_rn((double)(py - bi * k0), (double)k0);
    const double cx = __ddiv_rn((double)(px - bj * k1), (double)k1);
    const int b = clahe_level(levels, dtype, e) / bin_size;
    float acc = 0.f;
#pragma unroll
    for (int e0 = 0; e0 < 2; ++e0) {
      const int ri = min(max(bi + e0 - 1, 0), m0 - 1);
      const double wy = e0 ? cy : __dsub_rn(1.0, cy);
#pragma unroll
      for (int e1 = 0; e1 < 2; ++e1) {
        const int rj = min(max(bj + e1 - 1, 0), m1 - 1);
        const double wx = e1 ? cx : __dsub_rn(1.0, cx);
        const int mapped = maps[((int64_t)ri * m1 + rj) * nbins + b];
        acc = __fadd_rn(acc, __double2float_rn(__dmul_rn((double)mapped, __dmul_rn(wx, wy))));
      }
    }
    const int level = (int)acc;
    if (dtype == FI_PRE_F32)
      static_cast<float*>(out)[e] = (float)level;
    else
      static_cast<double*>(out)[e] = (double)level;
  }
}

// scikit-image's img_as_ubyte of a float image in [0, 1]: rint(x * 255) in the
// image's float type, clipped to [0, 255] (NaN gives 0).
__global__ void k_to_ubyte(const void* in, int dtype, int64_t count, uint8_t* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    double r;
    if (dtype == FI_PRE_F32)
      r = (double)rintf(__fmul_rn(static_cast<const float*>(in)[e], 255.f));
    else
      r = rint(__dmul_rn(static_cast<const double*>(in)[e], 255.0));
    out[e] = (r >= 0.0) ? (uint8_t)(int)fmin(r, 255.0) : (uint8_t)0;
  }
}

// scikit-image's filters.rank.equalize over disk(radius) of a uint8 image: of the
// disk's pixels inside the image (pop), the count n of values at most the centre's;
// out = (255 n) / pop truncated.  The disk's half-width per row, floor(sqrt(r^2 -
// dy^2)), is found in integers (one per row, in shared memory); rows are scanned as
// runs clipped to the image.
__global__ void k_rank_equalize(const uint8_t* __restrict__ in, int ny, int nx, int radius,
                                uint8_t* __restrict__ out) {
  extern __shared__ int halfw[];
  for (int d = threadIdx.x; d <= 2 * radius; d += blockDim.x) {
    const int dy = d - radius;
    const int q = radius * radius - dy * dy;
    int w = (int)sqrt((double)q);
    while (w > 0 && w * w > q) --w;
    while ((w + 1) * (w + 1) <= q) ++w;
    halfw[d] = w;
  }
  __syncthreads();
  const int64_t count = (int64_t)ny * nx;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(e / nx), x = (int)(e - (int64_t)y * nx);
    const int g = in[e];
    int pop = 0, n = 0;
    const int d0 = max(0, radius - y), d1 = min(2 * radius, radius + ny - 1 - y);
    for (int d = d0; d <= d1; ++d) {
      const int w = halfw[d];
      const int xa = max(0, x - w), xb = min(nx - 1, x + w);
      const uint8_t* row = in + (int64_t)(y + d - radius) * nx;
      pop += xb - xa + 1;
      for (int xx = xa; xx <= xb; ++xx) n += __ldg(row + xx) <= g;
    }
    out[e] = (uint8_t)(int)__ddiv_rn((double)(255 * n), (double)pop);
  }
}

}  // namespace fi

using namespace fi;

extern "C" int fi_rank_filter(const void* in, void* out, int dtype, int nt, int ny, int nx,
                              int st, int sy, int sx, int rank, int mode, double cval,
                              void* scratch, void* stream) {
  FI_REQUIRE(in && out, "fi_rank_filter: null pointer");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_rank_filter: bad dtype %d", dtype);
  FI_REQUIRE(mode >= FI_MODE_REFLECT && mode <= FI_MODE_WRAP, "fi_rank_filter: bad mode %d",
             mode);
  FI_REQUIRE(nt >= 1 && ny >= 1 && nx >= 1 && st >= 1 && sy >= 1 && sx >= 1,
             "fi_rank_filter: bad sizes");
  const int64_t wsize = (int64_t)st * sy * sx;
  FI_REQUIRE(rank >= 0 && rank < wsize, "fi_rank_filter: rank %d not within the window", rank);
  const int64_t count = (int64_t)nt * ny * nx;
  cudaStream_t s = (cudaStream_t)stream;
  // cval as a key of the image's dtype (scipy casts cval to the input type)
  uint64_t ckey = 0;
  {
    double c = cval;
    switch (dtype) {
      case FI_PRE_U8: ckey = (uint8_t)(int64_t)c; break;
      case FI_PRE_U16: ckey = (uint16_t)(int64_t)c; break;
      case FI_PRE_F32: {
        float f = (float)c;
        uint32_t u;
        memcpy(&u, &f, 4);
        ckey = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        break;
      }
      default: {
        uint64_t u;
        memcpy(&u, &c, 8);
        ckey = (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
      }
    }
  }
  const int g = grid_for(count);
  if (rank == 0 || rank == wsize - 1) {
    FI_REQUIRE(scratch, "fi_rank_filter: min/max filters need scratch[2 * count] (uint64)");
    const int is_max = rank == wsize - 1 && wsize > 1;
    uint64_t* k0 = static_cast<uint64_t*>(scratch);
    uint64_t* k1 = k0 + count;
    k_minmax_axis<<<g, 256, 0, s>>>(in, 0, nullptr, dtype, nt, ny, nx, 2, sx, mode, ckey, is_max, k0);
    k_minmax_axis<<<g, 256, 0, s>>>(nullptr, 1, k0, dtype, nt, ny, nx, 1, sy, mode, ckey, is_max, k1);
    k_minmax_axis<<<g, 256, 0, s>>>(nullptr, 1, k1, dtype, nt, ny, nx, 0, st, mode, ckey, is_max, k0);
    k_keys_to_values<<<g, 256, 0, s>>>(k0, dtype, count, out);
    return check_launch("fi_rank_filter", 4);
  }
  const size_t tile_smem = (size_t)(RS_TX + sx - 1) * (RS_TY + sy - 1) * sizeof(uint32_t);
  if (st == 1 && dtype != FI_PRE_F64 && tile_smem <= RS_MAX_SMEM) {
    static SmemLimit limit;
    FI_CUDA_TRY(raise_smem_limit(k_rank_select_tile, tile_smem, limit));
    const dim3 grid((unsigned)((nx + RS_TX - 1) / RS_TX), (unsigned)((ny + RS_TY - 1) / RS_TY),
                    (unsigned)nt);
    k_rank_select_tile<<<grid, dim3(RS_TX, RS_TY), tile_smem, s>>>(
        in, dtype, ny, nx, sy, sx, rank, mode, (uint32_t)ckey, out);
    return check_launch("fi_rank_filter");
  }
  k_rank_select<<<g, 256, 0, s>>>(in, dtype, nt, ny, nx, st, sy, sx, rank, mode, ckey, out);
  return check_launch("fi_rank_filter");
}

extern "C" int fi_subtract_weighted(const void* img, const void* filtered, int dtype,
                                    int64_t count, double weight, int out_dtype, int clamp,
                                    void* out, void* stream) {
  FI_REQUIRE(img && filtered && out && count > 0, "fi_subtract_weighted: bad arguments");
  FI_REQUIRE(out_dtype == FI_PRE_F64 || out_dtype == FI_PRE_F32 ||
                 (out_dtype == dtype && (dtype == FI_PRE_U8 || dtype == FI_PRE_U16)),
             "fi_subtract_weighted: bad output dtype %d", out_dtype);
  k_subtract_weighted<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(
      img, filtered, dtype, count, weight, out_dtype, clamp, out);
  return check_launch("fi_subtract_weighted");
}

extern "C" int fi_clamp(const void* in, int dtype, int64_t count, double lo, double hi, void* out,
                        void* stream) {
  FI_REQUIRE(in && out && count > 0, "fi_clamp: bad arguments");
  k_clamp<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(in, dtype, count, lo, hi, out);
  return check_launch("fi_clamp");
}

extern "C" int fi_sq_sum_max(const void* in, int dtype, int64_t count, double* part_sum,
                             double* part_max, int nparts, void* stream) {
  FI_REQUIRE(in && part_sum && part_max && count > 0 && nparts > 0,
             "fi_sq_sum_max: bad arguments");
  k_sq_sum_max<<<nparts, 256, 0, (cudaStream_t)stream>>>(in, dtype, count, part_sum, part_max);
  return check_launch("fi_sq_sum_max");
}

extern "C" int fi_tanh_rescale(const void* in, int dtype, int64_t count, double threshold,
                               double scale, double* out, void* stream) {
  FI_REQUIRE(in && out && count > 0 && threshold != 0.0, "fi_tanh_rescale: bad arguments");
  k_tanh_rescale<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(in, dtype, count, threshold,
                                                                   scale, out);
  return check_launch("fi_tanh_rescale");
}

extern "C" int fi_gaussian_filter(const void* in, void* out, void* tmp, int dtype, int nt, int ny,
                                  int nx, const double* weights, int radius, void* stream) {
  FI_REQUIRE(in && out && tmp && weights, "fi_gaussian_filter: null pointer");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_gaussian_filter: bad dtype %d",
             dtype);
  FI_REQUIRE(nt > 0 && ny > 0 && nx > 0 && radius >= 0, "fi_gaussian_filter: bad sizes");
  const int64_t count = (int64_t)nt * ny * nx;
  int blocks = (int)((count + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  cudaStream_t s = (cudaStream_t)stream;
  k_gauss_axis<<<blocks, 256, 0, s>>>(in, tmp, dtype, nt, ny, nx, 0, weights, radius);
  k_gauss_axis<<<blocks, 256, 0, s>>>(tmp, out, dtype, nt, ny, nx, 1, weights, radius);
  return check_launch("fi_gaussian_filter", 2);
}

extern "C" int fi_sharpen_combine(const void* blurred, const void* filtered, int dtype,
                                  int64_t count, double alpha, void* out, void* stream) {
  FI_REQUIRE(blurred && filtered && out && count > 0, "fi_sharpen_combine: bad arguments");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_sharpen_combine: bad dtype %d",
             dtype);
  int blocks = (int)((count + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_sharpen_combine<<<blocks, 256, 0, (cudaStream_t)stream>>>(blurred, filtered, dtype, count,
                                                             alpha, out);
  return check_launch("fi_sharpen_combine");
}

extern "C" int fi_min_max(const void* in, int dtype, int64_t count, double* part, int nparts,
                          void* stream) {
  FI_REQUIRE(in && part && count > 0 && nparts > 0 && nparts <= 4096,
             "fi_min_max: bad arguments");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_min_max: bad dtype %d", dtype);
  k_min_max_part<<<nparts, 256, 0, (cudaStream_t)stream>>>(in, dtype, count, part);
  return check_launch("fi_min_max");
}

extern "C" int fi_rescale_intensity(const void* in, int dtype, int64_t count, const double* part,
                                    int nparts, double omin, double omax, void* out,
                                    void* stream) {
  FI_REQUIRE(in && part && out && count > 0 && nparts > 0 && nparts <= 4096,
             "fi_rescale_intensity: bad arguments");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_rescale_intensity: bad dtype %d",
             dtype);
  k_rescale_linear<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(in, dtype, count, part,
                                                                     nparts, omin, omax, out);
  return check_launch("fi_rescale_intensity");
}

extern "C" int fi_gamma(const void* in, int dtype, int64_t count, double gamma, double gain,
                        const uint8_t* lut, void* out, void* stream) {
  FI_REQUIRE(in && out && count > 0, "fi_gamma: bad arguments");
  FI_REQUIRE(dtype >= FI_PRE_U8 && dtype <= FI_PRE_F64, "fi_gamma: bad dtype %d", dtype);
  FI_REQUIRE(dtype != FI_PRE_U8 || lut, "fi_gamma: uint8 images need the table");
  FI_REQUIRE(gamma >= 0.0, "fi_gamma: gamma must be non-negative");
  k_gamma<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(in, dtype, count, gamma, gain, lut,
                                                            out);
  return check_launch("fi_gamma");
}

extern "C" int fi_equalize_hist_int(const void* in, int dtype, int64_t count, unsigned* hist,
                                    double* cdf, double* out, void* stream) {
  FI_REQUIRE(in && hist && cdf && out && count > 0, "fi_equalize_hist_int: bad arguments");
  FI_REQUIRE(dtype == FI_PRE_U8 || dtype == FI_PRE_U16, "fi_equalize_hist_int: bad dtype %d",
             dtype);
  cudaStream_t s = (cudaStream_t)stream;
  const int nbins = dtype == FI_PRE_U8 ? 256 : 65536;
  FI_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * nbins, s));
  k_hist_int<<<grid_for(count), 256, 0, s>>>(in, dtype, count, hist);
  k_cdf<<<1, 1024, 0, s>>>(hist, nbins, 0, cdf);
  k_equalize_int<<<grid_for(count), 256, 0, s>>>(in, dtype, count, cdf, out);
  return check_launch("fi_equalize_hist_int", 3);
}

extern "C" int fi_equalize_hist_float(const void* in, int dtype, int64_t count, const void* edges,
                                      int nbins, double first, double denom,
                                      const double* centers, unsigned* hist, double* cdf,
                                      void* out, void* stream) {
  FI_REQUIRE(in && edges && centers && hist && cdf && out && count > 0 && nbins > 0,
             "fi_equalize_hist_float: bad arguments");
  FI_REQUIRE(dtype == FI_PRE_F32 || dtype == FI_PRE_F64, "fi_equalize_hist_float: bad dtype %d",
             dtype);
  cudaStream_t s = (cudaStream_t)stream;
  FI_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * nbins, s));
  k_hist_float<<<grid_for(count), 256, 0, s>>>(in, dtype, count, edges, nbins, first, denom, hist);
  k_cdf<<<1, 1024, 0, s>>>(hist, nbins, dtype == FI_PRE_F32 ? 1 : 0, cdf);
  k_interp<<<grid_for(count), 256, 0, s>>>(in, dtype, count, centers, cdf, nbins, out);
  return check_launch("fi_equalize_hist_float", 3);
}

extern "C" int fi_clahe(const void* levels, int dtype, int ny, int nx, int k0, int k1,
                        int nbins, double clip_limit, uint16_t* maps, void* out, void* stream) {
  FI_REQUIRE(levels && maps && out, "fi_clahe: null pointer");
  FI_REQUIRE(dtype == FI_PRE_F32 || dtype == FI_PRE_F64, "fi_clahe: bad dtype %d", dtype);
  FI_REQUIRE(ny >= 1 && nx >= 1 && k0 >= 1 && k1 >= 1, "fi_clahe: bad sizes");
  FI_REQUIRE(nbins >= 1 && nbins <= 12000, "fi_clahe: nbins must be in [1, 12000], not %d",
             nbins);
  FI_REQUIRE((int64_t)k0 * k1 <= (1 << 24), "fi_clahe: kernel of %d x %d too large", k0, k1);
  const int m0 = (ny + k0 - 1) / k0, m1 = (nx + k1 - 1) / k1;
  FI_REQUIRE((int64_t)m0 * m1 <= INT32_MAX, "fi_clahe: too many regions");
  const int npix = k0 * k1;
  const double lim = clip_limit * (double)npix;
  const int clim = clip_limit > 0.0 ? (int)(lim > 1.0 ? lim : 1.0) : npix;
  const double scale = (double)(CLAHE_GREYS - 1) / (double)npix;
  const int bin_size = 1 + CLAHE_GREYS / nbins;
  cudaStream_t s = (cudaStream_t)stream;
  k_clahe_maps<<<m0 * m1, CLAHE_NT, sizeof(int) * nbins, s>>>(
      levels, dtype, ny, nx, k0, k1, m1, nbins, bin_size, clim, scale, maps);
  const int64_t count = (int64_t)ny * nx;
  k_clahe_blend<<<grid_for(count), 256, 0, s>>>(levels, dtype, ny, nx, k0, k1, m0, m1, nbins,
                                               bin_size, maps, out);
  return check_launch("fi_clahe", 2);
}

extern "C" int fi_to_ubyte(const void* in, int dtype, int64_t count, uint8_t* out,
                           void* stream) {
  FI_REQUIRE(in && out && count > 0, "fi_to_ubyte: bad arguments");
  FI_REQUIRE(dtype == FI_PRE_F32 || dtype == FI_PRE_F64, "fi_to_ubyte: bad dtype %d", dtype);
  k_to_ubyte<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(in, dtype, count, out);
  return check_launch("fi_to_ubyte");
}

extern "C" int fi_rank_equalize(const uint8_t* in, int ny, int nx, int radius, uint8_t* out,
                                void* stream) {
  FI_REQUIRE(in && out && ny >= 1 && nx >= 1, "fi_rank_equalize: bad arguments");
  FI_REQUIRE(radius >= 0 && radius <= 4096, "fi_rank_equalize: radius %d out of [0, 4096]",
             radius);
  const int64_t count = (int64_t)ny * nx;
  k_rank_equalize<<<grid_for(count), 256, sizeof(int) * (2 * radius + 1),
                    (cudaStream_t)stream>>>(in, ny, nx, radius, out);
  return check_launch("fi_rank_equalize");
}
