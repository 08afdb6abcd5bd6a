// Image deformation by a displacement field given on nodes, and the
// deform-and-correlate chain with its hand-written adjoint.
//
// The reference leaves the deformation of im1 between passes as a to-do
// (works/piv/singlepass.py:736-738: the next pass uses integer window shifts); this
// file provides it and the differentiable correlation used to refine a field.
//
// Field: nodes at sorted coordinates xn[nx], yn[ny] (nx, ny >= 2), values u, v as
// [2][ny][nx] float32; the displacement at a pixel is the bilinear interpolation of
// the four nodes of its cell, constant beyond the outer nodes.
// Warp: imw(x, y) = im sampled bilinearly at (x + s u, y + s v) for a field scale s
// (the central scheme deforms im0 by s = -1/2 and im1 by s = +1/2, so that a
// window's displacement belongs to its centre), border pixels replicated outside
// the image.
// Windows: the non-overlapping 32 x 32 tiles of the image (H / 32 x W / 32 of them);
// per window the normalised circular correlation
//   c(m) = sum_x w0(x) w1(x + m) / (|w0| |w1|),  w = window - its mean
// (the plane of CorrelFFTNumpy.__call__, calcul/correl.py:671-685, divided by its
// norm), read out by a soft-argmax over the lags m in [-15, 15]^2:
//   p = softmax(c / T),  r = sum_m p(m) m   (the window's residual displacement).
// Backward: dL/dr -> dL/dc -> dL/dw1 (correlation adjoint by FFT: the planes are
// recomputed, never stored) -> dL/dim1w -> dL/dnodes (and dL/dim1).
#include "fi_common.cuh"
#include "fi_fft.cuh"

namespace fi {
namespace dc {

constexpr int N = 32;       // window size
constexpr int LD = N + 1;   // transpose buffer row stride (float2)
constexpr int WPB = 4;      // windows (warps) per block

// Cell of coordinate v among sorted nodes (n >= 2): j0 in [0, n - 2], weight t of
// node j0 + 1 in [0, 1].
__device__ __forceinline__ void cell(const float* nodes, int n, float v, int* j0, float* t) {
  int lo = 0, hi = n - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(nodes + mid) <= v) lo = mid; else hi = mid - 1;
  }
  const float a = __ldg(nodes + lo), b = __ldg(nodes + lo + 1);
  *t = fminf(fmaxf((v - a) / (b - a), 0.f), 1.f);
  *j0 = lo;
}

struct Interp {
  int i0, j0;
  float ty, tx;
};

__device__ __forceinline__ Interp interp_at(const float* xn, int nx, const float* yn, int ny,
                                            float x, float y) {
  Interp q;
  cell(xn, nx, x, &q.j0, &q.tx);
  cell(yn, ny, y, &q.i0, &q.ty);
  return q;
}

__device__ __forceinline__ float interp(const float* f, int nx, const Interp& q) {
  const float* a = f + q.i0 * nx + q.j0;
  const float top = (1.f - q.tx) * __ldg(a) + q.tx * __ldg(a + 1);
  const float bot = (1.f - q.tx) * __ldg(a + nx) + q.tx * __ldg(a + nx + 1);
  return (1.f - q.ty) * top + q.ty * bot;
}

// Bilinear sample of an image at (px, py) with replicated borders, and its
// derivatives along x and y (the derivative of the same bilinear formula).
struct Sample {
  float v, gx, gy;
  int xa, xb, ya, yb;
  float fx, fy;
};

__device__ __forceinline__ float pix(const void* im, int dtype, int64_t i) { return load_px(im, dtype, i); }

__device__ __forceinline__ Sample sample(const void* im, int dtype, int H, int W, float px, float py) {
  Sample s;
  px = fminf(fmaxf(px, -1e7f), 1e7f);  // also maps NaN to a finite position
  py = fminf(fmaxf(py, -1e7f), 1e7f);
  const float fpx = floorf(px), fpy = floorf(py);
  const int x0 = (int)fpx, y0 = (int)fpy;
  s.fx = px - fpx;
  s.fy = py - fpy;
  s.xa = min(max(x0, 0), W - 1);
  s.xb = min(max(x0 + 1, 0), W - 1);
  s.ya = min(max(y0, 0), H - 1);
  s.yb = min(max(y0 + 1, 0), H - 1);
  const float v00 = pix(im, dtype, (int64_t)s.ya * W + s.xa);
  const float v01 = pix(im, dtype, (int64_t)s.ya * W + s.xb);
  const float v10 = pix(im, dtype, (int64_t)s.yb * W + s.xa);
  const float v11 = pix(im, dtype, (int64_t)s.yb * W + s.xb);
  const float top = (1.f - s.fx) * v00 + s.fx * v01;
  const float bot = (1.f - s.fx) * v10 + s.fx * v11;
  s.v = (1.f - s.fy) * top + s.fy * bot;
  s.gx = (1.f - s.fy) * (v01 - v00) + s.fy * (v11 - v10);
  s.gy = (1.f - s.fx) * (v10 - v00) + s.fx * (v11 - v01);
  return s;
}

__global__ void k_warp(const float* __restrict__ fld, const float* __restrict__ xn, int nx,
                       const float* __restrict__ yn, int ny, float scale, const void* im1,
                       int dtype, int B, int H, int W, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int b = blockIdx.z;
  if (x >= W || y >= H || b >= B) return;
  const float* f = fld + (int64_t)b * 2 * ny * nx;
  const Interp q = interp_at(xn, nx, yn, ny, (float)x, (float)y);
  const float u = interp(f, nx, q), v = interp(f + ny * nx, nx, q);
  const void* img = (dtype == FI_U8) ? (const void*)((const uint8_t*)im1 + (int64_t)b * H * W)
                    : (dtype == FI_U16) ? (const void*)((const uint16_t*)im1 + (int64_t)b * H * W)
                                        : (const void*)((const float*)im1 + (int64_t)b * H * W);
  out[((int64_t)b * H + y) * W + x] =
      sample(img, dtype, H, W, fmaf(scale, u, (float)x), fmaf(scale, v, (float)y)).v;
}

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float wmax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// lag of plane index m (m = 16, i.e. -16, is left out of the soft-argmax)
__device__ __forceinline__ float lag(int m) { return (float)(m < 16 ? m : m - 32); }

__device__ __forceinline__ void load_row(const float* p, bool vec, float (&a)[N]) {
  if (vec) {
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
      const float4 f = __ldg(reinterpret_cast<const float4*>(p) + q);
      a[4 * q] = f.x;
      a[4 * q + 1] = f.y;
      a[4 * q + 2] = f.z;
      a[4 * q + 3] = f.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < N; ++c) a[c] = __ldg(p + c);
  }
}

// 2-D FFT of the window held row-wise (thread = row) -> column-wise (thread =
// column: x[r] = X(r, lane)); Wb: the warp's transpose buffer.
template <bool INV>
__device__ __forceinline__ void fft2_rows_to_cols(float2 (&x)[N], float2* Wb, int lane) {
  fft_reg<N, INV>(x);
#pragma unroll
  for (int c = 0; c < N; ++c) Wb[lane * LD + c] = x[c];
  __syncwarp();
#pragma unroll
  for (int r = 0; r < N; ++r) x[r] = Wb[r * LD + lane];
  __syncwarp();
  fft_reg<N, INV>(x);
}

// 2-D transform held column-wise -> row-wise (thread = row: x[c] = X(lane, c)).
template <bool INV>
__device__ __forceinline__ void fft2_cols_to_rows(float2 (&x)[N], float2* Wb, int lane) {
  fft_reg<N, INV>(x);
#pragma unroll
  for (int r = 0; r < N; ++r) Wb[r * LD + lane] = x[r];
  __syncwarp();
#pragma unroll
  for (int c = 0; c < N; ++c) x[c] = Wb[lane * LD + c];
  __syncwarp();
  fft_reg<N, INV>(x);
}

// F0 (the spectrum of window 0) at (r, lane) from the packed spectrum Z = F0 + i F1
// stored column-wise in Zb.
__device__ __forceinline__ float2 spec0(const float2* Zb, int r, int lane) {
  const float2 z = Zb[r * LD + lane];
  const float2 zm = Zb[((N - r) & (N - 1)) * LD + ((N - lane) & (N - 1))];
  return make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
}

template <bool BWD>
__global__ void __launch_bounds__(32 * WPB)
    k_windows(const float* __restrict__ im0, const float* __restrict__ im1w, int B, int H, int W,
              float inv_T, float* __restrict__ r_out, float* __restrict__ cz_out,
              float* __restrict__ cpk_out, const float* __restrict__ grad_r,
              float* __restrict__ g_im1w, float* __restrict__ g_im0w) {
  extern __shared__ float2 smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwx = W / N, nwy = H / N;
  const int w = blockIdx.x * WPB + warp;
  if (w >= B * nwx * nwy) return;  // warp-uniform
  float2* Zb = smem + warp * 2 * N * LD;
  float2* Wb = Zb + N * LD;
  const int b = w / (nwx * nwy), rem = w % (nwx * nwy);
  const int y0 = (rem / nwx) * N, x0 = (rem % nwx) * N;
  const int64_t row = ((int64_t)b * H + y0 + lane) * W + x0;
  const bool vec = (W % 4) == 0 && ((reinterpret_cast<uintptr_t>(im0) | reinterpret_cast<uintptr_t>(im1w)) & 15) == 0;
  // ---- windows: means, norms ----
  float2 x[N];
  float mean0, mean1, q0, q1, inv_n;
  {
    float a0[N], a1[N];
    load_row(im0 + row, vec, a0);
    load_row(im1w + row, vec, a1);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      s0 += a0[c];
      s1 += a1[c];
    }
    mean0 = wsum(s0) * (1.f / (N * N));
    mean1 = wsum(s1) * (1.f / (N * N));
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float u0 = a0[c] - mean0, u1 = a1[c] - mean1;
      p0 = fmaf(u0, u0, p0);
      p1 = fmaf(u1, u1, p1);
      x[c] = make_float2(u0, u1);
    }
    q0 = wsum(p0);
    q1 = wsum(p1);
    inv_n = (q0 > 0.f && q1 > 0.f) ? rsqrtf(q0) * rsqrtf(q1) : 0.f;
  }
  // ---- packed spectrum Z = F0 + i F1 (column-wise), kept in Zb ----
  fft2_rows_to_cols<false>(x, Wb, lane);
#pragma unroll
  for (int r = 0; r < N; ++r) Zb[r * LD + lane] = x[r];
  __syncwarp();
  // ---- conj(F0) F1, inverse: the plane u(m) = sum_x w0(x) w1(x + m) (row-wise) ----
  {
    const int lc = (N - lane) & (N - 1);
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const float2 z = x[r];
      const float2 zm = Zb[((N - r) & (N - 1)) * LD + lc];
      const float2 f0 = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
      const float2 f1 = make_float2(0.5f * (z.y + zm.y), 0.5f * (zm.x - z.x));
      x[r] = make_float2(f0.x * f1.x + f0.y * f1.y, f0.x * f1.y - f0.y * f1.x);
    }
  }
  fft2_cols_to_rows<true>(x, Wb, lane);
  // ---- normalised plane c (row m_y = lane, column m_x), soft-argmax ----
  const float scale = inv_n * (1.f / (N * N));
  float cmax = -INFINITY;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    x[c].x *= scale;  // c(m)
    if (c != 16 && lane != 16) cmax = fmaxf(cmax, x[c].x);
  }
  cmax = wmax(cmax);
  float se = 0.f, sx = 0.f, sy = 0.f;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const bool ok = c != 16 && lane != 16;
    const float e = ok ? __expf((x[c].x - cmax) * inv_T) : 0.f;
    x[c].y = e;
    se += e;
    sx = fmaf(e, lag(c), sx);
  }
  sy = se * lag(lane);
  se = wsum(se);
  sx = wsum(sx);
  sy = wsum(sy);
  const float inv_se = 1.f / se;
  const float rx = sx * inv_se, ry = sy * inv_se;
  if constexpr (!BWD) {
    const float cz = __shfl_sync(0xffffffffu, x[0].x, 0);
    if (lane == 0) {
      r_out[2 * w] = rx;
      r_out[2 * w + 1] = ry;
      if (cz_out) cz_out[w] = cz;
      if (cpk_out) cpk_out[w] = cmax;
    }
    return;
  } else {
    // ---- dL/dc(m) = p(m) (a . (m - r)) / T;  S = sum_m dL/dc(m) c(m) ----
    const float ax = __ldg(grad_r + 2 * w), ay = __ldg(grad_r + 2 * w + 1);
    const float ty = ay * (lag(lane) - ry);
    float S = 0.f;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float g = x[c].y * inv_se * (ax * (lag(c) - rx) + ty) * inv_T;
      S = fmaf(g, x[c].x, S);
      x[c] = make_float2(g, 0.f);
    }
    S = wsum(S);
    // ---- conv(y) = sum_m g(m) w0(y - m) = IDFT(G F0)(y) in the real part, and
    // xcor(x) = sum_m g(m) w1(x + m) = IDFT(conj(G) F1)(x) in the imaginary part
    // (both are real: one inverse transform of G F0 + i conj(G) F1)
    fft2_rows_to_cols<false>(x, Wb, lane);
    {
      const int lc = (N - lane) & (N - 1);
#pragma unroll
      for (int r = 0; r < N; ++r) {
        const float2 z = Zb[r * LD + lane];
        const float2 zm = Zb[((N - r) & (N - 1)) * LD + lc];
        const float2 f0 = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
        const float2 f1 = make_float2(0.5f * (z.y + zm.y), 0.5f * (zm.x - z.x));
        const float2 gg = x[r];
        const float2 a0 = make_float2(gg.x * f0.x - gg.y * f0.y, gg.x * f0.y + gg.y * f0.x);
        const float2 a1 = make_float2(gg.x * f1.x + gg.y * f1.y, gg.x * f1.y - gg.y * f1.x);
        x[r] = make_float2(a0.x - a1.y, a0.y + a1.x);  // a0 + i a1
      }
    }
    fft2_cols_to_rows<true>(x, Wb, lane);
    // ---- dL/dw1 = conv / (|w0| |w1|) - S w1 / |w1|^2, then through the mean ----
    float a1[N];
    load_row(im1w + row, vec, a1);
    const float k1 = (q1 > 0.f) ? S / q1 : 0.f;
    const float kc = inv_n * (1.f / (N * N));
    float gs = 0.f;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float gw = x[c].x * kc - k1 * (a1[c] - mean1);
      a1[c] = gw;
      gs += gw;
    }
    const float gmean = wsum(gs) * (1.f / (N * N));
#pragma unroll
    for (int c = 0; c < N; ++c) g_im1w[row + c] = a1[c] - gmean;
    if (g_im0w) {
      // dL/dw0 = xcor / (|w0| |w1|) - S w0 / |w0|^2, then through the mean
      float a0[N];
      load_row(im0 + row, vec, a0);
      const float k0 = (q0 > 0.f) ? S / q0 : 0.f;
      float hs = 0.f;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const float gw = x[c].y * kc - k0 * (a0[c] - mean0);
        a0[c] = gw;
        hs += gw;
      }
      const float hmean = wsum(hs) * (1.f / (N * N));
#pragma unroll
      for (int c = 0; c < N; ++c) g_im0w[row + c] = a0[c] - hmean;
    }
  }
}

// dL/dnodes (and dL/dim1) from dL/dim1w.  Block: 32 x 8 threads over 32-pixel rows;
// the node contributions of a warp's 32 pixels (one row, at most a few cells) are
// reduced per cell by shuffles, then added to global memory by one lane.
__global__ void k_warp_bwd(const float* __restrict__ fld, const float* __restrict__ xn, int nx,
                           const float* __restrict__ yn, int ny, float scale, const void* im1,
                           int dtype, int B, int H, int W, const float* __restrict__ g_out,
                           float* __restrict__ g_fld, float* __restrict__ g_im1) {
  const int lane = threadIdx.x;
  const int x = blockIdx.x * 32 + lane;
  const int b = blockIdx.z;
  const bool in = x < W;
  const float* f = fld + (int64_t)b * 2 * ny * nx;
  float* gf = g_fld + (int64_t)b * 2 * ny * nx;
  const void* img = (dtype == FI_U8) ? (const void*)((const uint8_t*)im1 + (int64_t)b * H * W)
                    : (dtype == FI_U16) ? (const void*)((const uint16_t*)im1 + (int64_t)b * H * W)
                                        : (const void*)((const float*)im1 + (int64_t)b * H * W);
  for (int y = blockIdx.y * blockDim.y + threadIdx.y; y < H; y += gridDim.y * blockDim.y) {
    Interp q{0, 0, 0.f, 0.f};
    float gdx = 0.f, gdy = 0.f;
    int j0 = 0x7fffffff;
    if (in) {
      q = interp_at(xn, nx, yn, ny, (float)x, (float)y);
      const float u = interp(f, nx, q), v = interp(f + ny * nx, nx, q);
      const Sample s = sample(img, dtype, H, W, fmaf(scale, u, (float)x), fmaf(scale, v, (float)y));
      const float g = __ldg(g_out + ((int64_t)b * H + y) * W + x);
      gdx = scale * g * s.gx;
      gdy = scale * g * s.gy;
      j0 = q.j0;
      if (g_im1) {
        float* gi = g_im1 + (int64_t)b * H * W;
        atomicAdd(gi + (int64_t)s.ya * W + s.xa, g * (1.f - s.fy) * (1.f - s.fx));
        atomicAdd(gi + (int64_t)s.ya * W + s.xb, g * (1.f - s.fy) * s.fx);
        atomicAdd(gi + (int64_t)s.yb * W + s.xa, g * s.fy * (1.f - s.fx));
        atomicAdd(gi + (int64_t)s.yb * W + s.xb, g * s.fy * s.fx);
      }
    }
    // cells present in this warp's row (same i0 for every pixel of the row)
    const int i0 = __shfl_sync(0xffffffffu, q.i0, 0);
    int jlo = j0, jhi = in ? j0 : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      jlo = min(jlo, __shfl_xor_sync(0xffffffffu, jlo, o));
      jhi = max(jhi, __shfl_xor_sync(0xffffffffu, jhi, o));
    }
    for (int j = jlo; j <= jhi; ++j) {
      const bool mine = in && j0 == j;
      const float w00 = mine ? (1.f - q.ty) * (1.f - q.tx) : 0.f;
      const float w01 = mine ? (1.f - q.ty) * q.tx : 0.f;
      const float w10 = mine ? q.ty * (1.f - q.tx) : 0.f;
      const float w11 = mine ? q.ty * q.tx : 0.f;
      float c[8] = {gdx * w00, gdx * w01, gdx * w10, gdx * w11,
                    gdy * w00, gdy * w01, gdy * w10, gdy * w11};
#pragma unroll
      for (int k = 0; k < 8; ++k) c[k] = wsum(c[k]);
      if (lane == 0) {
        float* a = gf + i0 * nx + j;
        atomicAdd(a, c[0]);
        atomicAdd(a + 1, c[1]);
        atomicAdd(a + nx, c[2]);
        atomicAdd(a + nx + 1, c[3]);
        float* bb = a + ny * nx;
        atomicAdd(bb, c[4]);
        atomicAdd(bb + 1, c[5]);
        atomicAdd(bb + nx, c[6]);
        atomicAdd(bb + nx + 1, c[7]);
      }
    }
  }
}

static int check_field(const float* nodes, const float* xn, int nx, const float* yn, int ny,
                       const void* im1, int dtype, int B, int H, int W, const char* who) {
  FI_REQUIRE(nodes && xn && yn && im1, "%s: null pointer", who);
  FI_REQUIRE(nx >= 2 && ny >= 2, "%s: the node grid needs at least 2 x 2 nodes", who);
  FI_REQUIRE(B >= 1 && H >= 1 && W >= 1, "%s: empty image", who);
  FI_REQUIRE(dtype == FI_U8 || dtype == FI_U16 || dtype == FI_F32, "%s: bad dtype %d", who,
             dtype);
  FI_REQUIRE(B <= 65535, "%s: at most 65535 images per call", who);
  return FI_OK;
}

}  // namespace dc
}  // namespace fi

using namespace fi;

extern "C" int fi_dc_warp(const float* nodes, const float* xn, int nx, const float* yn, int ny,
                          float scale, const void* im1, int dtype, int batch, int height,
                          int width, float* out, void* stream) {
  if (dc::check_field(nodes, xn, nx, yn, ny, im1, dtype, batch, height, width, "fi_dc_warp") != FI_OK)
    return FI_ERR_INVALID;
  FI_REQUIRE(out, "fi_dc_warp: null output");
  const dim3 block(32, 8), grid((width + 31) / 32, (height + 7) / 8, batch);
  dc::k_warp<<<grid, block, 0, (cudaStream_t)stream>>>(nodes, xn, nx, yn, ny, scale, im1, dtype,
                                                       batch, height, width, out);
  return check_launch("fi_dc_warp");
}

extern "C" int fi_dc_windows(const float* im0, const float* im1w, int batch, int height,
                             int width, float temperature, float* r, float* c_zero,
                             float* c_peak, void* stream) {
  FI_REQUIRE(im0 && im1w && r, "fi_dc_windows: null pointer");
  FI_REQUIRE(batch >= 1 && height >= dc::N && width >= dc::N,
             "fi_dc_windows: images smaller than one 32 x 32 window");
  FI_REQUIRE(temperature > 0.f, "fi_dc_windows: temperature must be positive");
  const int64_t nwin = (int64_t)batch * (height / dc::N) * (width / dc::N);
  FI_REQUIRE(nwin < (1ll << 31), "fi_dc_windows: too many windows");
  const int blocks = (int)((nwin + dc::WPB - 1) / dc::WPB);
  const size_t smem = (size_t)dc::WPB * 2 * dc::N * dc::LD * sizeof(float2);
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(dc::k_windows<false>, smem, limit));
  dc::k_windows<false><<<blocks, 32 * dc::WPB, smem, (cudaStream_t)stream>>>(
      im0, im1w, batch, height, width, 1.f / temperature, r, c_zero, c_peak, nullptr, nullptr,
      nullptr);
  return check_launch("fi_dc_windows");
}

extern "C" int fi_dc_windows_backward(const float* im0, const float* im1w, int batch, int height,
                                      int width, float temperature, const float* grad_r,
                                      float* grad_im1w, float* grad_im0, void* stream) {
  FI_REQUIRE(im0 && im1w && grad_r && grad_im1w, "fi_dc_windows_backward: null pointer");
  FI_REQUIRE(batch >= 1 && height >= dc::N && width >= dc::N,
             "fi_dc_windows_backward: images smaller than one 32 x 32 window");
  FI_REQUIRE(temperature > 0.f, "fi_dc_windows_backward: temperature must be positive");
  const int64_t nwin = (int64_t)batch * (height / dc::N) * (width / dc::N);
  FI_REQUIRE(nwin < (1ll << 31), "fi_dc_windows_backward: too many windows");
  const int blocks = (int)((nwin + dc::WPB - 1) / dc::WPB);
  const size_t smem = (size_t)dc::WPB * 2 * dc::N * dc::LD * sizeof(float2);
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(dc::k_windows<true>, smem, limit));
  dc::k_windows<true><<<blocks, 32 * dc::WPB, smem, (cudaStream_t)stream>>>(
      im0, im1w, batch, height, width, 1.f / temperature, nullptr, nullptr, nullptr, grad_r,
      grad_im1w, grad_im0);
  return check_launch("fi_dc_windows_backward");
}

extern "C" int fi_dc_warp_backward(const float* nodes, const float* xn, int nx, const float* yn,
                                   int ny, float scale, const void* im1, int dtype, int batch,
                                   int height, int width, const float* grad_out,
                                   float* grad_nodes, float* grad_im1, void* stream) {
  if (dc::check_field(nodes, xn, nx, yn, ny, im1, dtype, batch, height, width,
                      "fi_dc_warp_backward") != FI_OK)
    return FI_ERR_INVALID;
  FI_REQUIRE(grad_out && grad_nodes, "fi_dc_warp_backward: null gradient pointer");
  const int rows = 8;
  const int gy = min((height + rows - 1) / rows, 64);
  const dim3 block(32, rows), grid((width + 31) / 32, gy, batch);
  dc::k_warp_bwd<<<grid, block, 0, (cudaStream_t)stream>>>(nodes, xn, nx, yn, ny, scale, im1,
                                                           dtype, batch, height, width, grad_out,
                                                           grad_nodes, grad_im1);
  return check_launch("fi_dc_warp_backward");
}
