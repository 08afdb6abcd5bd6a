// Fused PIV pass: window extraction -> FFT cross-correlation -> peak search ->
// second-chance search -> '2d_gaussian2' subpixel fit, one thread group per window.
//
// Upstream behaviour restated here (fluidimage 0.5.3):
//   window positions   works/piv/singlepass.py:210-260, 787-870
//   padding / crop     works/piv/singlepass.py:196-208, 391-407 (numpy slice rules)
//   correlation        calcul/correl.py:671-685 with calcul/fft.py:254-269
//   plane layout       _like_fftshift, calcul/correl.py:596-636
//   peak search        nan_indices_max, calcul/correl.py:88-164
//   second chance      CorrelBase.compute_displacements_from_correl, correl.py:226-275
//   subpixel           compute_subpix_2d_gaussian2 + SubPix.compute_subpix,
//                      calcul/subpix.py:16-61, 107-218
//
// Data layout: the two images stay in HBM in their own element type; each window
// group stages its two n x n windows in shared memory as one complex array
// (im0 in the real part, im1 in the imaginary part, each scaled by a power of two
// to unit RMS), runs row then column FFTs with one thread per row/column in
// registers, separates the two spectra with the Hermitian symmetry, forms
// conj(F0) F1, runs the inverse FFT and keeps the real part as the correlation
// plane in shared memory.  Window energies are FP64 sums of the staged pixels.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "fi_common.cuh"
#include "fi_fft.cuh"

namespace fi {

static thread_local char g_error[1024] = "";
static std::atomic<long long> g_launches{0};

void add_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

template <int N>
struct Cfg {
  static constexpr int G = (N <= 16) ? 16 : ((N <= 32) ? 32 : 64);  // threads / window
  static constexpr int WPB = (G == 16) ? 16 : ((G == 32) ? 8 : 2);  // windows / block
  static constexpr int THREADS = G * WPB;
  // resident CTAs per SM asked of the register allocator (16-px windows: 3, i.e.
  // 24 warps, at <= 85 registers)
  static constexpr int MIN_BLOCKS = (N <= 16) ? 3 : 1;
  static constexpr int LD = N + 1;   // row stride (float2) of the complex buffer
  static constexpr int LDP = N + 1;  // row stride (float) of the plane
  static constexpr int ZBYTES = N * LD * 8;
  static constexpr int REDBYTES = 256;
  static constexpr int GROUP_BYTES = ZBYTES + REDBYTES;
  static constexpr int SMEM = WPB * GROUP_BYTES;
};

template <int G>
__device__ __forceinline__ unsigned seg_mask() {
  if constexpr (G == 16) return 0xFFFFu << (threadIdx.x & 16);
  return 0xFFFFFFFFu;
}

template <int G>
__device__ __forceinline__ void gsync(int g) {
  if constexpr (G == 16) {
    __syncwarp(seg_mask<16>());
  } else if constexpr (G == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(G) : "memory");
  }
}

// Sum of 4 doubles over the group.
template <int G>
__device__ __forceinline__ void gsum4(double (&v)[4], int g, double* red) {
  constexpr int W = G < 32 ? G : 32;
  const unsigned m = seg_mask<G>();
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += __shfl_xor_sync(m, v[i], o, W);
  if constexpr (G == 64) {
    const int wi = (threadIdx.x >> 5) & 1;
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int i = 0; i < 4; ++i) red[4 * wi + i] = v[i];
    gsync<G>(g);
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = red[i] + red[4 + i];
    gsync<G>(g);
  }
}

// Sum of 4 unsigned 64-bit integers over the group (exact).
template <int G>
__device__ __forceinline__ void gsum4u(unsigned long long (&v)[4], int g, double* red) {
  constexpr int W = G < 32 ? G : 32;
  const unsigned m = seg_mask<G>();
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += __shfl_xor_sync(m, v[i], o, W);
  if constexpr (G == 64) {
    unsigned long long* ru = reinterpret_cast<unsigned long long*>(red);
    const int wi = (threadIdx.x >> 5) & 1;
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int i = 0; i < 4; ++i) ru[4 * wi + i] = v[i];
    gsync<G>(g);
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = ru[i] + ru[4 + i];
    gsync<G>(g);
  }
}

// min/max of 4 floats over the group: v[0], v[1] min; v[2], v[3] max.
template <int G>
__device__ __forceinline__ void gminmax4(float (&v)[4], int g, double* red) {
  constexpr int W = G < 32 ? G : 32;
  const unsigned m = seg_mask<G>();
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) {
    v[0] = fminf(v[0], __shfl_xor_sync(m, v[0], o, W));
    v[1] = fminf(v[1], __shfl_xor_sync(m, v[1], o, W));
    v[2] = fmaxf(v[2], __shfl_xor_sync(m, v[2], o, W));
    v[3] = fmaxf(v[3], __shfl_xor_sync(m, v[3], o, W));
  }
  if constexpr (G == 64) {
    float* rf = reinterpret_cast<float*>(red);
    const int wi = (threadIdx.x >> 5) & 1;
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int i = 0; i < 4; ++i) rf[4 * wi + i] = v[i];
    gsync<G>(g);
    v[0] = fminf(rf[0], rf[4]);
    v[1] = fminf(rf[1], rf[5]);
    v[2] = fmaxf(rf[2], rf[6]);
    v[3] = fmaxf(rf[3], rf[7]);
    gsync<G>(g);
  }
}

// Running "last maximum" (value, flat index) with the second-largest value.
struct Peak {
  float v;   // best value
  int f;     // flat index of the best value (-1: none)
  float v2;  // second-largest value at another position
};

__device__ __forceinline__ void peak_merge(Peak& a, float bv, int bf, float bv2) {
  const bool other = (bv > a.v) || (bv == a.v && bf > a.f);
  if (other) {
    a.v2 = fmaxf(a.v, bv2);
    a.v = bv;
    a.f = bf;
  } else {
    a.v2 = fmaxf(a.v2, bv);
  }
}

template <int G>
__device__ __forceinline__ Peak gpeak(Peak p, int g, double* red) {
  constexpr int W = G < 32 ? G : 32;
  const unsigned m = seg_mask<G>();
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) {
    const float bv = __shfl_xor_sync(m, p.v, o, W);
    const int bf = __shfl_xor_sync(m, p.f, o, W);
    const float bv2 = __shfl_xor_sync(m, p.v2, o, W);
    peak_merge(p, bv, bf, bv2);
  }
  if constexpr (G == 64) {
    float* rf = reinterpret_cast<float*>(red);
    int* ri = reinterpret_cast<int*>(red);
    const int wi = (threadIdx.x >> 5) & 1;
    if ((threadIdx.x & 31) == 0) {
      rf[3 * wi + 0] = p.v;
      ri[3 * wi + 1] = p.f;
      rf[3 * wi + 2] = p.v2;
    }
    gsync<G>(g);
    Peak q{rf[0], ri[1], rf[2]};
    peak_merge(q, rf[3], ri[4], rf[5]);
    p = q;
    gsync<G>(g);
  }
  return p;
}

// Rectangle of virtual NaNs (numpy slice semantics, possibly empty).
struct NanBox {
  int r0, r1, c0, c1;
  __device__ __forceinline__ bool has(int i0, int i1) const {
    return i0 >= r0 && i0 < r1 && i1 >= c0 && i1 < c1;
  }
};

// The NaN boxes written by the peak searches: the second-chance box, then one box
// per secondary search (on upstream's copy of the plane).
struct NanBoxes {
  NanBox b[FI_MAX_PEAKS];
  int n;
  __device__ __forceinline__ bool has(int i0, int i1) const {
    bool h = false;
#pragma unroll
    for (int k = 0; k < FI_MAX_PEAKS; ++k) h |= (k < n) && b[k].has(i0, i1);
    return h;
  }
  __device__ __forceinline__ void add(int i0, int i1, int radius, int N) {
    int r0, r1, c0, c1;
    slice_bounds(i0 - radius, i0 + radius + 1, N, &r0, &r1);
    slice_bounds(i1 - radius, i1 + radius + 1, N, &c0, &c1);
    if (!(r1 > r0 && c1 > c0) || n >= FI_MAX_PEAKS) return;
    const NanBox nb{r0, r1, c0, c1};
#pragma unroll
    for (int k = 0; k < FI_MAX_PEAKS; ++k)  // static indices keep the boxes in registers
      if (k == n) b[k] = nb;
    ++n;
  }
};

template <int N>
__device__ __forceinline__ bool excluded(const float* PL, const uint8_t* mask, const NanBoxes& nb,
                                         int i0, int i1) {
  if (mask && __ldg(mask + i0 * N + i1)) return true;
  if (nb.has(i0, i1)) return true;
  const float v = PL[i0 * Cfg<N>::LDP + i1];
  return v != v;
}

// Raw lag m -> index in the "_like_fftshift" layout: fftshift(a[::-1, ::-1]).
template <int N>
__device__ __forceinline__ int shift_index(int m) {
  return (2 * N - 1 - m + N / 2) % N;
}

struct PeakOut {
  int err;     // FI_VEC_*
  int i0, i1;  // peak indices (valid when err is 0/1/2)
  float cmax;  // correl[i0, i1] / norm
  bool tie;
};

struct SearchBox {
  int i0s, i0e, i1s, i1e;
};

// nan_indices_max + _compute_indices_max on the group's plane (correl.py:88-164).
template <int N>
__device__ PeakOut find_peak(const float* PL, const uint8_t* mask, const SearchBox& box,
                             const NanBoxes& nb, float normf, int t, int g, double* red) {
  using C = Cfg<N>;
  Peak p{-INFINITY, -1, -INFINITY};
  if (t < N && t >= box.i1s && t < box.i1e) {
    for (int i0 = box.i0s; i0 < box.i0e; ++i0) {
      if (excluded<N>(PL, mask, nb, i0, t)) continue;
      const float v = PL[i0 * C::LDP + t];
      if (v >= p.v) {
        p.v2 = p.v;
        p.v = v;
        p.f = i0 * N + t;
      } else if (v > p.v2) {
        p.v2 = v;
      }
    }
  }
  p = gpeak<C::G>(p, g, red);
  PeakOut o;
  if (p.f < 0) {
    o.err = FI_VEC_ALL_NAN;
    o.i0 = o.i1 = 0;
    o.cmax = NAN;
    o.tie = false;
    return o;
  }
  o.i0 = p.f / N;
  o.i1 = p.f % N;
  o.tie = (p.v - p.v2) <= 1e-6f * fabsf(p.v);
  const float val = PL[o.i0 * C::LDP + o.i1];
  o.cmax = (normf == 0.0f) ? 0.0f : __fdiv_rn(val, normf);
  if (o.i0 == 0 || o.i0 == N - 1 || o.i1 == 0 || o.i1 == N - 1) {
    o.err = FI_VEC_PEAK_BOUNDARY;
  } else {
    bool nan = false;
#pragma unroll
    for (int a = -1; a <= 1; ++a)
#pragma unroll
      for (int b = -1; b <= 1; ++b) nan |= excluded<N>(PL, mask, nb, o.i0 + a, o.i1 + b);
    o.err = nan ? FI_VEC_PEAK_NAN : FI_VEC_OK;
  }
  return o;
}

// compute_subpix_2d_gaussian2 (subpix.py:16-61) in float32 with the upstream
// operation order.  False when |depl|^2 > 4.5 (upstream then falls back to the
// centroid).
__device__ bool gauss2_depl(const float (&c)[9], float* deplx_o, float* deply_o,
                            bool* min_tie) {
  float n[9];
  float cmin = c[0];
#pragma unroll
  for (int k = 1; k < 9; ++k) cmin = (c[k] < cmin) ? c[k] : cmin;
#pragma unroll
  for (int k = 0; k < 9; ++k) n[k] = __fsub_rn(c[k], cmin);
  float cmx = n[0];
#pragma unroll
  for (int k = 1; k < 9; ++k) cmx = (n[k] > cmx) ? n[k] : cmx;
  int nlow = 0;  // crop values within 1e-5 of the minimum (relative to the range)
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    n[k] = __fdiv_rn(n[k], cmx);
    nlow += (n[k] < 1e-5f) ? 1 : 0;
    if (n[k] == 0.0f) n[k] = 1e-8f;
  }
  // two or more values at the minimum: the 1e-8 floor makes the fit depend on
  // which of them rounds to exactly zero (a near-tie of the subpixel fit)
  *min_tie = nlow >= 2;
  float c10 = 0.f, c01 = 0.f, c11 = 0.f, c20 = 0.f, c02 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float l = logf(n[3 * a + b]);
      c10 = __fadd_rn(c10, __fmul_rn((float)(b - 1), l));
      c01 = __fadd_rn(c01, __fmul_rn((float)(a - 1), l));
      c11 = __fadd_rn(c11, __fmul_rn((float)((b - 1) * (a - 1)), l));
      c20 = __fadd_rn(c20, __fmul_rn((float)(3 * (b - 1) * (b - 1) - 2), l));
      c02 = __fadd_rn(c02, __fmul_rn((float)(3 * (a - 1) * (a - 1) - 2), l));
    }
  c10 = __fdiv_rn(c10, 6.f);
  c01 = __fdiv_rn(c01, 6.f);
  c11 = __fdiv_rn(c11, 4.f);
  c20 = __fdiv_rn(c20, 6.f);
  c02 = __fdiv_rn(c02, 6.f);
  const float den = __fsub_rn(__fmul_rn(__fmul_rn(4.f, c20), c02), __fmul_rn(c11, c11));
  const float deplx =
      __fdiv_rn(__fsub_rn(__fmul_rn(c11, c01), __fmul_rn(__fmul_rn(2.f, c10), c02)), den);
  const float deply =
      __fdiv_rn(__fsub_rn(__fmul_rn(c11, c10), __fmul_rn(__fmul_rn(2.f, c01), c20)), den);
  *deplx_o = deplx;
  *deply_o = deply;
  const float r2 = __fadd_rn(__fmul_rn(deplx, deplx), __fmul_rn(deply, deply));
  return !(r2 > 4.5f);
}

// '2d_gaussian2' with the centroid fallback on a 3x3 crop (subpix.py:184-216).
// Returns 0 or FI_VEC_WRONG_SUBPIX; (dx, dy) displacement.
__device__ int subpix_gaussian2_vals(const float (&c)[9], int i0, int i1, int ix0, int iy0,
                                     float* dxo, float* dyo, bool* min_tie) {
  float deplx, deply;
  if (gauss2_depl(c, &deplx, &deply, min_tie)) {
    *dxo = __fsub_rn((float)ix0, __fadd_rn(deplx, (float)i1));
    *dyo = __fsub_rn((float)iy0, __fadd_rn(deply, (float)i0));
    return FI_VEC_OK;
  }
  // centroid on the 3x3 crop (float32 sum, float64 moments)
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) s = __fadd_rn(s, c[k]);
  double mx = 0.0, my = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      mx = __dadd_rn(mx, __dmul_rn((double)(b - 1), (double)c[3 * a + b]));
      my = __dadd_rn(my, __dmul_rn((double)(a - 1), (double)c[3 * a + b]));
    }
  const double cx = __ddiv_rn(mx, (double)s);
  const double cy = __ddiv_rn(my, (double)s);
  if (__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)) > 4.5) {
    *dxo = (float)(ix0 - i1);
    *dyo = (float)(iy0 - i0);
    return FI_VEC_WRONG_SUBPIX;
  }
  *dxo = (float)__dsub_rn((double)ix0, __dadd_rn(cx, (double)i1));
  *dyo = (float)__dsub_rn((double)iy0, __dadd_rn(cy, (double)i0));
  return FI_VEC_OK;
}

// Subpixel fit with any method (SubPix.compute_subpix, subpix.py:107-218) at the
// peak (i0, i1) of the plane; cbox: values inside read as NaN (the second-chance
// box that upstream writes into the caller's plane).  Outputs the displacement as
// upstream computes it with Python-int peak indices (d32: float32 for
// '2d_gaussian2', else the float64 value rounded) and with int32 indices (d64:
// float64, the '2d_gaussian2' offset promoted).  Returns 0, FI_VEC_WRONG_SUBPIX or
// FI_VEC_CLOSE_BOUNDARY (then the integer displacement).
struct SubpixOut {
  float dx32, dy32;
  double dx64, dy64;
  bool tie;
};

__device__ int subpix_any(const float* PL, int ld, int N, int i0, int i1, int method, int nsub,
                          const double* minv, const NanBox& cbox, SubpixOut* o) {
  const int ix0 = N / 2 - 1, iy0 = N / 2 - 1;
  const int n = (method == FI_SUBPIX_GAUSSIAN2) ? 1 : nsub;
  o->tie = false;
  auto integer = [&](int err) {
    o->dx32 = (float)(ix0 - i1);
    o->dy32 = (float)(iy0 - i0);
    o->dx64 = (double)(ix0 - i1);
    o->dy64 = (double)(iy0 - i0);
    return err;
  };
  if (i0 - n < 0 || i0 + n + 1 > N || i1 - n < 0 || i1 + n + 1 > N)
    return integer(FI_VEC_CLOSE_BOUNDARY);
  auto val = [&](int r, int c) -> float { return cbox.has(r, c) ? NAN : PL[r * ld + c]; };
  auto from_offsets = [&](double deplx, double deply) {  // float64 offsets
    o->dx64 = __dsub_rn((double)ix0, __dadd_rn(deplx, (double)i1));
    o->dy64 = __dsub_rn((double)iy0, __dadd_rn(deply, (double)i0));
    o->dx32 = (float)o->dx64;
    o->dy32 = (float)o->dy64;
  };
  const double lim = 2.0 * (0.5 + n) * (0.5 + n);
  int m = method;
  if (m == FI_SUBPIX_GAUSSIAN2) {
    float c[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) c[3 * a + b] = val(i0 - 1 + a, i1 - 1 + b);
    float deplx, deply;
    if (gauss2_depl(c, &deplx, &deply, &o->tie)) {
      o->dx32 = __fsub_rn((float)ix0, __fadd_rn(deplx, (float)i1));
      o->dy32 = __fsub_rn((float)iy0, __fadd_rn(deply, (float)i0));
      o->dx64 = __dsub_rn((double)ix0, __dadd_rn((double)deplx, (double)i1));
      o->dy64 = __dsub_rn((double)iy0, __dadd_rn((double)deply, (double)i0));
      return FI_VEC_OK;
    }
    m = FI_SUBPIX_CENTROID;
  }
  if (m == FI_SUBPIX_GAUSSIAN) {
    // coef = pinv(M) . log(crop), float32 logs of the crop with values <= 0 at 1e-6
    const int w = 2 * n + 1, K = w * w;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    for (int j = 0; j < K; ++j) {
      float v = val(i0 - n + j / w, i1 - n + j % w);
      if (v <= 0.0f) v = 1e-6f;
      const double l = (double)logf(v);
      c0 = fma(__ldg(minv + j), l, c0);
      c1 = fma(__ldg(minv + K + j), l, c1);
      c2 = fma(__ldg(minv + 2 * K + j), l, c2);
      c3 = fma(__ldg(minv + 3 * K + j), l, c3);
    }
    if (c0 > 0.0 || c1 > 0.0) {
      m = FI_SUBPIX_CENTROID;
    } else {
      const double sx = 1.0 / sqrt(-2.0 * c0), sy = 1.0 / sqrt(-2.0 * c1);
      const double deplx = c2 * (sx * sx), deply = c3 * (sy * sy);
      if (isnan(deplx) || isnan(deply)) {
        m = FI_SUBPIX_CENTROID;
      } else {
        if (deplx * deplx + deply * deply > lim) return integer(FI_VEC_WRONG_SUBPIX);
        from_offsets(deplx, deply);
        return FI_VEC_OK;
      }
    }
  }
  if (m == FI_SUBPIX_CENTROID) {
    const int w = 2 * n + 1;
    float s = 0.f;
    double mx = 0.0, my = 0.0;
    for (int a = 0; a < w; ++a)
      for (int b = 0; b < w; ++b) {
        const float v = val(i0 - n + a, i1 - n + b);
        s = __fadd_rn(s, v);
        mx = __dadd_rn(mx, __dmul_rn((double)(b - n), (double)v));
        my = __dadd_rn(my, __dmul_rn((double)(a - n), (double)v));
      }
    const double cx = __ddiv_rn(mx, (double)s), cy = __ddiv_rn(my, (double)s);
    if (__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)) > lim)
      return integer(FI_VEC_WRONG_SUBPIX);
    from_offsets(cx, cy);
    return FI_VEC_OK;
  }
  from_offsets(0.0, 0.0);  // 'no_subpix'
  return FI_VEC_OK;
}

// SubPix.compute_subpix at given peak indices on planes in global memory
// (subpix.py:107-218), any method, one thread per plane; "close boundary" when
// the crop leaves the plane.
__global__ void k_subpix_at(const float* planes, int count, int n, const int32_t* pi0,
                            const int32_t* pi1, int method, int nsub, const double* minv,
                            float* dxs, float* dys, uint8_t* errs) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= count) return;
  SubpixOut sp;
  const int e = subpix_any(planes + (int64_t)w * n * n, n, n, pi0[w], pi1[w], method, nsub, minv,
                           NanBox{0, 0, 0, 0}, &sp);
  errs[w] = (uint8_t)e;
  dxs[w] = sp.dx32;
  dys[w] = sp.dy32;
}

// Peak search with the second chance, then subpixel fit; writes the outputs.
// (correl.py:226-275, singlepass.py:318-346)
struct PeakArgs {
  const uint8_t* mask;
  SearchBox box;
  int radius;
  int apply_subpix;
  int subpix_method;
  int nsubpix;
  const double* minv;
  int nb_peaks;
};

// Where the secondary peaks of one window go (fi_piv_pass outputs).
struct SecondaryOut {
  int32_t* count;   // [nvec]
  float* peaks;     // [nvec][nb_peaks-1][FI_PEAK_FIELDS]
  uint8_t* err;     // [nvec][nb_peaks-1]
  int w;
  bool has_in;      // pass >= 1: integer input shift (int32 upstream)
  int dinx, diny;
};

struct VecResult {
  int err;
  float dx, dy, cmax;
  int i0, i1;
  bool tie;        // near-tie of the two largest plane values (either attempt)
  bool subpix_tie; // tied minimum in the 3x3 subpixel crop
  bool sec_tie;    // near-tie in a secondary search
  NanBox nb;
};

template <int N>
__device__ VecResult peak_and_subpix(const float* PL, const PeakArgs& pa, float normf, int t,
                                     int g, double* red, const SecondaryOut* so) {
  const int ix0 = N / 2 - 1, iy0 = N / 2 - 1;
  NanBoxes boxes;
  boxes.n = 0;
  PeakOut p1 = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red);
  VecResult r;
  r.tie = p1.tie;
  r.subpix_tie = false;
  r.sec_tie = false;
  r.nb = NanBox{0, 0, 0, 0};
  PeakOut fin = p1;
  if (p1.err == FI_VEC_PEAK_BOUNDARY || p1.err == FI_VEC_PEAK_NAN) {
    boxes.add(p1.i0, p1.i1, pa.radius, N);
    if (boxes.n) r.nb = boxes.b[0];
    PeakOut p2 = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red);
    r.tie = r.tie || p2.tie;
    if (p2.err == FI_VEC_OK) {
      fin = p2;
    } else {
      fin = p1;
      fin.err = p2.err;
    }
  }
  r.err = fin.err;
  r.i0 = fin.i0;
  r.i1 = fin.i1;
  r.cmax = fin.cmax;
  if (fin.err == FI_VEC_ALL_NAN) {
    r.dx = r.dy = NAN;
  } else {
    r.dx = (float)(ix0 - fin.i1);
    r.dy = (float)(iy0 - fin.i0);
  }
  // upstream's caller plane holds the second-chance box unless the displacement
  // mask made the search work on a copy (CorrelFFTBase, correl.py:561-568)
  const NanBox cbox = (pa.mask == nullptr) ? r.nb : NanBox{0, 0, 0, 0};
  if (fin.err == FI_VEC_OK && pa.apply_subpix && t == 0) {
    SubpixOut sp;
    r.err = subpix_any(PL, Cfg<N>::LDP, N, fin.i0, fin.i1, pa.subpix_method, pa.nsubpix,
                       pa.minv, cbox, &sp);
    r.subpix_tie = sp.tie;
    r.dx = sp.dx32;
    r.dy = sp.dy32;
  }
  // other peaks (correl.py:250-273): NaN box around the last peak, search again
  if (so != nullptr && pa.nb_peaks > 1) {
    if (fin.err != FI_VEC_OK) {
      if (t == 0) so->count[so->w] = -1;
    } else {
      int a0 = fin.i0, a1 = fin.i1, cnt = 0;
      const int K = pa.nb_peaks - 1;
      for (int k = 0; k < K; ++k) {
        boxes.add(a0, a1, pa.radius, N);
        const PeakOut q = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red);
        r.sec_tie = r.sec_tie || q.tie;
        if (q.err != FI_VEC_OK) break;
        a0 = q.i0;
        a1 = q.i1;
        if (t == 0) {
          SubpixOut sp;
          const int e = subpix_any(PL, Cfg<N>::LDP, N, a0, a1, pa.subpix_method, pa.nsubpix,
                                   pa.minv, cbox, &sp);
          float* o = so->peaks + ((int64_t)so->w * K + k) * FI_PEAK_FIELDS;
          o[0] = (float)(ix0 - a1);
          o[1] = (float)(iy0 - a0);
          o[2] = q.cmax;
          // the replacement value of WorkFIX (fix.py:205-211): upstream adds the
          // int32 input shift to the float64 fit, or keeps the first-pass value
          o[3] = so->has_in ? (float)__dadd_rn(sp.dx64, (double)so->dinx) : sp.dx32;
          o[4] = so->has_in ? (float)__dadd_rn(sp.dy64, (double)so->diny) : sp.dy32;
          so->err[(int64_t)so->w * K + k] = (uint8_t)e;
        }
        ++cnt;
      }
      if (t == 0) so->count[so->w] = cnt;
    }
  }
  return r;
}

template <int N, bool FROM_WINDOWS>
__global__ void __launch_bounds__(Cfg<N>::THREADS, Cfg<N>::MIN_BLOCKS)
    k_piv_pass(const fi_piv_pass_args a, const float* __restrict__ win0,
               const float* __restrict__ win1, int nvec, int npad, int do_peaks) {
  using C = Cfg<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = threadIdx.x / C::G;
  const int t = threadIdx.x % C::G;
  const int w = blockIdx.x * C::WPB + g;
  if (w >= nvec) return;
  float2* Z = reinterpret_cast<float2*>(smem_raw + g * C::GROUP_BYTES);
  double* red = reinterpret_cast<double*>(smem_raw + g * C::GROUP_BYTES + C::ZBYTES);
  float* PL = reinterpret_cast<float*>(Z);

  // ---- window positions (pass 0: grid; pass >= 1: shifted windows) ----
  int ixs0 = 0, iys0 = 0, ixs1 = 0, iys1 = 0, dinx = 0, diny = 0;
  bool valid = true;
  int y00 = 0, x00 = 0, y10 = 0, x10 = 0;
  if (!FROM_WINDOWS) {
    const int gx = __ldg(a.ixvecs + (w % a.nx));
    const int gy = __ldg(a.iyvecs + (w / a.nx));
    ixs0 = ixs1 = gx;
    iys0 = iys1 = gy;
    if (a.dxin) {
      dinx = __ldg(a.dxin + w);
      diny = __ldg(a.dyin + w);
      ixs0 = gx - floordiv2(dinx);
      iys0 = gy - floordiv2(diny);
      ixs1 = ixs0 + dinx;
      iys1 = iys0 + diny;
      const int H = a.height, W = a.width;
      const bool out1 = ixs1 > W || iys1 > H || ixs1 < 0 || iys1 < 0;
      const bool out0 = ixs0 > W || iys0 > H || ixs0 < 0 || iys0 < 0;
      if (out1) {
        ixs0 = gx - dinx;
        iys0 = gy - diny;
        ixs1 = gx;
        iys1 = gy;
      } else if (out0) {
        ixs0 = gx;
        iys0 = gy;
        ixs1 = gx + dinx;
        iys1 = gy + diny;
      }
    }
    const int startc = N / 2, stopc = N / 2 + (N % 2);
    const int Ly = a.height + 2 * npad, Lx = a.width + 2 * npad;
    int s0y, e0y, s0x, e0x, s1y, e1y, s1x, e1x;
    slice_bounds(iys0 + npad - startc, iys0 + npad + stopc, Ly, &s0y, &e0y);
    slice_bounds(ixs0 + npad - startc, ixs0 + npad + stopc, Lx, &s0x, &e0x);
    slice_bounds(iys1 + npad - startc, iys1 + npad + stopc, Ly, &s1y, &e1y);
    slice_bounds(ixs1 + npad - startc, ixs1 + npad + stopc, Lx, &s1x, &e1x);
    valid = (e0y - s0y == N) && (e0x - s0x == N) && (e1y - s1y == N) && (e1x - s1x == N);
    y00 = s0y - npad;
    x00 = s0x - npad;
    y10 = s1y - npad;
    x10 = s1x - npad;
  }

  // ---- stage the two windows; exact window sums ----
  // Integer images: exact integer sums of v and v^2 (INT pipe).  Float images and
  // plugin windows: float32 sums with a compensated sum of squares.  FP64 is used
  // only once per window (the FP64 pipe of this GPU is narrow).
  const bool intpath = !FROM_WINDOWS && a.dtype != FI_F32;
  unsigned si0 = 0u, si1 = 0u;
  unsigned long long qi0 = 0ull, qi1 = 0ull;
  float sf0 = 0.f, sf1 = 0.f, qf0 = 0.f, qf1 = 0.f, cf0 = 0.f, cf1 = 0.f;
  float mm[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
  if (t < N) {
    const float min0 = FROM_WINDOWS ? 0.f : __ldg(a.im_min + 0);
    const float min1 = FROM_WINDOWS ? 0.f : __ldg(a.im_min + 1);
    const int mini0 = (int)min0, mini1 = (int)min1;
    const int H = a.height, W = a.width;
#pragma unroll 4
    for (int r = 0; r < N; ++r) {
      float v0 = 0.f, v1 = 0.f;
      if (FROM_WINDOWS) {
        v0 = __ldg(win0 + ((int64_t)w * N + r) * N + t);
        v1 = __ldg(win1 + ((int64_t)w * N + r) * N + t);
      } else if (valid) {
        const int y0 = y00 + r, x0 = x00 + t, y1 = y10 + r, x1 = x10 + t;
        const bool in0 = y0 >= 0 && y0 < H && x0 >= 0 && x0 < W;
        const bool in1 = y1 >= 0 && y1 < H && x1 >= 0 && x1 < W;
        if (intpath) {
          const int i0v = in0 ? load_px_int(a.im0, a.dtype, (int64_t)y0 * W + x0) - mini0 : 0;
          const int i1v = in1 ? load_px_int(a.im1, a.dtype, (int64_t)y1 * W + x1) - mini1 : 0;
          v0 = (float)i0v;
          v1 = (float)i1v;
          si0 += (unsigned)i0v;
          si1 += (unsigned)i1v;
          qi0 += (unsigned long long)((unsigned)i0v * (unsigned)i0v);
          qi1 += (unsigned long long)((unsigned)i1v * (unsigned)i1v);
        } else {
          if (in0) v0 = __fsub_rn(load_px(a.im0, a.dtype, (int64_t)y0 * W + x0), min0);
          if (in1) v1 = __fsub_rn(load_px(a.im1, a.dtype, (int64_t)y1 * W + x1), min1);
        }
      }
      Z[r * C::LD + t] = make_float2(v0, v1);
      if (!intpath) {
        sf0 += v0;
        sf1 += v1;
        // Kahan-compensated sums of squares
        float yk = fmaf(v0, v0, -cf0), tk = qf0 + yk;
        cf0 = (tk - qf0) - yk;
        qf0 = tk;
        yk = fmaf(v1, v1, -cf1);
        tk = qf1 + yk;
        cf1 = (tk - qf1) - yk;
        qf1 = tk;
      }
      mm[0] = fminf(mm[0], v0);
      mm[1] = fminf(mm[1], v1);
      mm[2] = fmaxf(mm[2], v0);
      mm[3] = fmaxf(mm[3], v1);
    }
  }
  double sums[4];
  unsigned long long u[4] = {si0, qi0, si1, qi1};
  if (intpath) {
    gsum4u<C::G>(u, g, red);
  } else {
    sums[0] = (double)sf0;
    sums[1] = (double)qf0 - (double)cf0;
    sums[2] = (double)sf1;
    sums[3] = (double)qf1 - (double)cf1;
    gsum4<C::G>(sums, g, red);
  }
  gminmax4<C::G>(mm, g, red);
  // per-window scalars: one thread computes them and the group reads them back from
  // its scratch.  FP64 is narrow on this GPU (an FP64 instruction costs the whole
  // warp's FP64 issue even with one lane active), so the integer-image,
  // power-of-two-window case uses exact integer sums and float32 only.
  if (t == 0) {
    // a constant window has an exactly zero spectrum (and plane) upstream
    const bool flat0 = mm[0] == mm[2], flat1 = mm[1] == mm[3];
    float* rf = reinterpret_cast<float*>(red + 17);
    int e0 = 0, e1 = 0;
    float normf;
    if constexpr ((N & (N - 1)) == 0) {
      constexpr int L = (N == 16) ? 4 : (N == 32) ? 5 : (N == 64) ? 6 : 3;
      if (intpath) {
        // N^2 S = N^2 sum v^2 - (sum v)^2, exact in 64 bits (v < 2^16: both terms
        // below 2^(4L + 32)); S = (N^2 S) 2^-2L, so frexp(S) has exponent
        // bitlength(N^2 S) - 2L
        const unsigned long long SN0 = flat0 ? 0ull : (u[1] << (2 * L)) - u[0] * u[0];
        const unsigned long long SN1 = flat1 ? 0ull : (u[3] << (2 * L)) - u[2] * u[2];
        if (SN0 != 0ull) e0 = ((64 - __clzll((long long)SN0) - 2 * L) - 2 * L + 1) >> 1;
        if (SN1 != 0ull) e1 = ((64 - __clzll((long long)SN1) - 2 * L) - 2 * L + 1) >> 1;
        // the window sums are below 2^32: the float mean rounds once, like the
        // float64 product rounded to float32
        rf[0] = ldexpf(__uint2float_rn((unsigned)u[0]), -2 * L);
        rf[1] = ldexpf(__uint2float_rn((unsigned)u[2]), -2 * L);
        const float S0f = ldexpf(__ull2float_rn(SN0), -2 * L);
        const float S1f = ldexpf(__ull2float_rn(SN1), -2 * L);
        normf = __fsqrt_rn(__fmul_rn(S0f, S1f));
        // float64 norm only for the caller's norms array
        red[16] = a.norms ? ldexp(sqrt((double)SN0 * (double)SN1), -2 * L) : 0.0;
      } else {
        // N^2 a power of two: the divisions by N^2 are exact products by 2^-2L, and
        // the exponent of sqrt(S / N^2) follows from the one of S (frexp(sqrt(m 2^x))
        // has exponent (x + 1) >> 1)
        constexpr double INN = 1.0 / ((double)N * (double)N);
        const double S0 = flat0 ? 0.0 : fmax(sums[1] - (sums[0] * sums[0]) * INN, 0.0);
        const double S1 = flat1 ? 0.0 : fmax(sums[3] - (sums[2] * sums[2]) * INN, 0.0);
        int x0 = 0, x1 = 0;
        if (S0 > 0.0) {
          frexp(S0, &x0);
          e0 = (x0 - 2 * L + 1) >> 1;
        }
        if (S1 > 0.0) {
          frexp(S1, &x1);
          e1 = (x1 - 2 * L + 1) >> 1;
        }
        rf[0] = (float)(sums[0] * INN);
        rf[1] = (float)(sums[2] * INN);
        red[16] = sqrt(S0 * S1);
        normf = (float)red[16];
      }
      // scale of the inverse FFT: 0.25 / (N^2 sc0 sc1) = 2^(e0 + e1 - 2 - 2L)
      reinterpret_cast<float*>(red + 20)[0] = ldexpf(1.0f, e0 + e1 - 2 - 2 * L);
    } else {
      if (intpath)
        for (int i = 0; i < 4; ++i) sums[i] = (double)u[i];
      const double NN = (double)N * (double)N;
      const double S0 = flat0 ? 0.0 : fmax(sums[1] - sums[0] * sums[0] / NN, 0.0);
      const double S1 = flat1 ? 0.0 : fmax(sums[3] - sums[2] * sums[2] / NN, 0.0);
      if (S0 > 0.0) frexp(sqrt(S0 / NN), &e0);
      if (S1 > 0.0) frexp(sqrt(S1 / NN), &e1);
      rf[0] = (float)(sums[0] / NN);
      rf[1] = (float)(sums[2] / NN);
      // scale of the inverse FFT: 0.25 / (N^2 sc0 sc1), sc0 sc1 a power of two
      reinterpret_cast<float*>(red + 20)[0] =
          (float)(0.25 / (NN * (double)ldexpf(1.0f, -e0) * (double)ldexpf(1.0f, -e1)));
      red[16] = sqrt(S0 * S1);
      normf = (float)red[16];
    }
    rf[2] = ldexpf(1.0f, -e0);
    rf[3] = ldexpf(1.0f, -e1);
    reinterpret_cast<int*>(red + 19)[0] = (flat0 || flat1) ? 1 : 0;
    reinterpret_cast<float*>(red + 20)[1] = normf;
  }
  gsync<C::G>(g);
  const float normf = reinterpret_cast<const float*>(red + 20)[1];
  const double norm_out = red[16];  // the caller's norms array only
  const float mean0 = reinterpret_cast<const float*>(red + 17)[0];
  const float mean1 = reinterpret_cast<const float*>(red + 17)[1];
  const float sc0 = reinterpret_cast<const float*>(red + 17)[2];
  const float sc1 = reinterpret_cast<const float*>(red + 17)[3];
  const bool flat = reinterpret_cast<const int*>(red + 19)[0] != 0;
  const float outscale = reinterpret_cast<const float*>(red + 20)[0];
  gsync<C::G>(g);

  // ---- forward 2-D FFT of z = x0*sc0 + i*x1*sc1 ----
  float2 x[N];
  if (t < N) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float2 v = Z[t * C::LD + c];
      x[c] = make_float2((v.x - mean0) * sc0, (v.y - mean1) * sc1);
    }
    fft_reg<N, false>(x);
#pragma unroll
    for (int c = 0; c < N; ++c) Z[t * C::LD + c] = x[c];
  }
  gsync<C::G>(g);
  if (t < N) {
#pragma unroll
    for (int r = 0; r < N; ++r) x[r] = Z[r * C::LD + t];
    fft_reg<N, false>(x);
#pragma unroll
    for (int r = 0; r < N; ++r) Z[r * C::LD + t] = x[r];
  }
  gsync<C::G>(g);
  // ---- separate the spectra: F0 ~ A + conj(Z[-k]), F1 ~ -i (A - conj(Z[-k])) ----
  if (t < N) {
    const int tc = (N - t) % N;
#pragma unroll
    for (int k0 = 0; k0 < N; ++k0) {
      const float2 A = x[k0];
      const float2 Bc = Z[((N - k0) % N) * C::LD + tc];
      const float2 B = make_float2(Bc.x, -Bc.y);
      const float2 f0 = cadd(A, B);
      const float2 d = csub(A, B);
      const float2 f1 = make_float2(d.y, -d.x);
      float2 p = make_float2(f0.x * f1.x + f0.y * f1.y, f0.x * f1.y - f0.y * f1.x);
      if (flat || (k0 == 0 && t == 0)) p = make_float2(0.f, 0.f);
      x[k0] = p;
    }
  }
  gsync<C::G>(g);
  // ---- inverse 2-D FFT ----
  if (t < N) {
    fft_reg<N, true>(x);
#pragma unroll
    for (int r = 0; r < N; ++r) Z[r * C::LD + t] = x[r];
  }
  gsync<C::G>(g);
  if (t < N) {
#pragma unroll
    for (int c = 0; c < N; ++c) x[c] = Z[t * C::LD + c];
    fft_reg<N, true>(x);
  }
  gsync<C::G>(g);
  if (t < N) {
    const int i0 = shift_index<N>(t);
#pragma unroll
    for (int c = 0; c < N; ++c) PL[i0 * C::LDP + shift_index<N>(c)] = flat ? 0.f : x[c].x * outscale;
  }
  gsync<C::G>(g);

  VecResult res;
  res.nb = NanBox{0, 0, 0, 0};
  if (do_peaks) {
    PeakArgs pa;
    pa.mask = a.mask;
    pa.box = SearchBox{a.box_i0_start, a.box_i0_stop, a.box_i1_start, a.box_i1_stop};
    pa.radius = a.particle_radius;
    pa.apply_subpix = a.apply_subpix;
    pa.subpix_method = a.subpix_method;
    pa.nsubpix = a.nsubpix;
    pa.minv = a.subpix_minv;
    pa.nb_peaks = a.nb_peaks;
    SecondaryOut so{a.peaks_count, a.peaks, a.peaks_err, w, a.dxin != nullptr, dinx, diny};
    res = peak_and_subpix<N>(PL, pa, normf, t, g, red, a.nb_peaks > 1 ? &so : nullptr);
    if (!valid && a.nb_peaks > 1 && t == 0) a.peaks_count[w] = -1;
  }

  // ---- outputs ----
  if (a.planes && t < N) {
    float* out = a.planes + (int64_t)w * N * N;
    const bool write_box = (a.mask == nullptr);
    for (int i0 = 0; i0 < N; ++i0) {
      float v = PL[i0 * C::LDP + t];
      if (!valid || (write_box && res.nb.has(i0, t))) v = NAN;
      out[i0 * N + t] = v;
    }
  }
  if (t == 0) {
    if (a.norms) a.norms[w] = norm_out;
    if (do_peaks) {
      float dxo = res.dx, dyo = res.dy, cm = res.cmax;
      int err = res.err;
      if (!valid) {
        dxo = dyo = cm = NAN;
        err = FI_VEC_BAD_CROP;
      }
      if (a.dxin) {
        // float32 + int32 promotes to float64 upstream, then rounds to float32: the
        // exact sum rounded once, which is the float sum for |shift| < 2^24
        dxo = (abs(dinx) < (1 << 24)) ? __fadd_rn(dxo, (float)dinx) : (float)((double)dxo + (double)dinx);
        dyo = (abs(diny) < (1 << 24)) ? __fadd_rn(dyo, (float)diny) : (float)((double)dyo + (double)diny);
      }
      a.deltaxs[w] = dxo;
      a.deltays[w] = dyo;
      a.correls_max[w] = cm;
      a.errors[w] = (uint8_t)err;
      if (a.flags)
        a.flags[w] = valid ? (uint8_t)((res.tie ? FI_FLAG_NEAR_TIE : 0) |
                                       (res.subpix_tie ? FI_FLAG_SUBPIX_TIE : 0) |
                                       (res.sec_tie ? FI_FLAG_SECONDARY_TIE : 0))
                           : (uint8_t)0;
      if (!FROM_WINDOWS) {
        // midpoints: exact in float32 below 2^24
        const int sx = ixs0 + ixs1, sy = iys0 + iys1;
        a.xs[w] = (abs(sx) < (1 << 24)) ? __fmul_rn((float)sx, 0.5f) : (float)((double)sx * 0.5);
        a.ys[w] = (abs(sy) < (1 << 24)) ? __fmul_rn((float)sy, 0.5f) : (float)((double)sy * 0.5);
      }
    }
  }
}

// Peak search + subpixel fit on planes given in global memory.
template <int N>
__global__ void __launch_bounds__(Cfg<N>::THREADS)
    k_peaks(float* planes, const double* norms, int count, PeakArgs pa, float* dxs, float* dys,
            float* cmaxs, uint8_t* errs, int32_t* pi0, int32_t* pi1, int32_t* pcount,
            float* peaks, uint8_t* perr) {
  using C = Cfg<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = threadIdx.x / C::G;
  const int t = threadIdx.x % C::G;
  const int w = blockIdx.x * C::WPB + g;
  if (w >= count) return;
  float* PL = reinterpret_cast<float*>(smem_raw + g * C::GROUP_BYTES);
  double* red = reinterpret_cast<double*>(smem_raw + g * C::GROUP_BYTES + C::ZBYTES);
  float* in = planes + (int64_t)w * N * N;
  if (t < N)
    for (int i0 = 0; i0 < N; ++i0) PL[i0 * C::LDP + t] = in[i0 * N + t];
  gsync<C::G>(g);
  SecondaryOut so{pcount, peaks, perr, w, false, 0, 0};
  VecResult r =
      peak_and_subpix<N>(PL, pa, (float)norms[w], t, g, red, pa.nb_peaks > 1 ? &so : nullptr);
  if (pa.mask == nullptr && t < N && (r.nb.r1 > r.nb.r0))
    for (int i0 = 0; i0 < N; ++i0)
      if (r.nb.has(i0, t)) in[i0 * N + t] = NAN;
  if (t == 0) {
    dxs[w] = r.dx;
    dys[w] = r.dy;
    cmaxs[w] = r.cmax;
    errs[w] = (uint8_t)r.err;
    if (pi0) pi0[w] = r.i0;
    if (pi1) pi1[w] = r.i1;
  }
}

__global__ void k_min_init(uint32_t* keys) {
  if (threadIdx.x < 2) keys[threadIdx.x] = 0xFFFFFFFFu;
}

// Minimum of 16 bytes of pixels (u8: 16, u16: 8, f32: 4 values).
__device__ __forceinline__ float min16(uint4 v, int dtype) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  if (dtype == FI_F32) {
    return fminf(fminf(__uint_as_float(w[0]), __uint_as_float(w[1])),
                 fminf(__uint_as_float(w[2]), __uint_as_float(w[3])));
  }
  uint32_t m = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (dtype == FI_U16) {
      m = min(m, min(w[k] & 0xffffu, w[k] >> 16));
    } else {
      m = min(m, min(min(w[k] & 0xffu, (w[k] >> 8) & 0xffu),
                     min((w[k] >> 16) & 0xffu, w[k] >> 24)));
    }
  }
  return (float)m;  // exact: below 2^16
}

__global__ void k_images_min(const void* im0, const void* im1, int dtype, int64_t count,
                             uint32_t* keys) {
  float m0 = INFINITY, m1 = INFINITY;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int esize = (dtype == FI_U8) ? 1 : (dtype == FI_U16 ? 2 : 4);
  int64_t vec = 0;  // pixels read by 16-byte loads (both images 16-byte aligned)
  if ((((uintptr_t)im0 | (uintptr_t)im1) & 15) == 0) {
    const int per = 16 / esize;
    const int64_t nv = count / per;
    const uint4* a = reinterpret_cast<const uint4*>(im0);
    const uint4* b = reinterpret_cast<const uint4*>(im1);
    for (int64_t i = tid; i < nv; i += stride) {
      m0 = fminf(m0, min16(__ldg(a + i), dtype));
      m1 = fminf(m1, min16(__ldg(b + i), dtype));
    }
    vec = nv * per;
  }
  for (int64_t i = vec + tid; i < count; i += stride) {
    m0 = fminf(m0, load_px(im0, dtype, i));
    m1 = fminf(m1, load_px(im1, dtype, i));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fminf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fminf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(keys + 0, float_to_key(m0));
    atomicMin(keys + 1, float_to_key(m1));
  }
}

__global__ void k_min_decode(uint32_t* keys) {
  if (threadIdx.x < 2) {
    float* f = reinterpret_cast<float*>(keys);
    f[threadIdx.x] = key_to_float(keys[threadIdx.x]);
  }
}

static int num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

template <int N, bool FW>
static int launch_pass(const fi_piv_pass_args& a, const float* w0, const float* w1, int nvec,
                       int npad, int do_peaks, cudaStream_t s) {
  using C = Cfg<N>;
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(k_piv_pass<N, FW>, C::SMEM, limit));
  const int blocks = (nvec + C::WPB - 1) / C::WPB;
  k_piv_pass<N, FW><<<blocks, C::THREADS, C::SMEM, s>>>(a, w0, w1, nvec, npad, do_peaks);
  return check_launch("k_piv_pass");
}

template <int N>
static int launch_peaks(float* planes, const double* norms, int count, const PeakArgs& pa,
                        float* dxs, float* dys, float* cm, uint8_t* errs, int32_t* pi0,
                        int32_t* pi1, int32_t* pcount, float* peaks, uint8_t* perr,
                        cudaStream_t s) {
  using C = Cfg<N>;
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(k_peaks<N>, C::SMEM, limit));
  const int blocks = (count + C::WPB - 1) / C::WPB;
  k_peaks<N><<<blocks, C::THREADS, C::SMEM, s>>>(planes, norms, count, pa, dxs, dys, cm, errs,
                                                  pi0, pi1, pcount, peaks, perr);
  return check_launch("k_peaks");
}

static bool supported_n(int n) { return n == 16 || n == 24 || n == 32 || n == 48 || n == 64; }

}  // namespace fi

using namespace fi;

extern "C" const char* fi_last_error(void) { return g_error; }

extern "C" const char* fi_version(void) { return "fluidimage_gb300 0.1.0 (sm_103a)"; }

extern "C" long long fi_launch_count(void) { return g_launches.load(); }

extern "C" int fi_abi_sizes(int64_t* out) {
  if (!out) return FI_ERR_INVALID;
  out[0] = (int64_t)sizeof(fi_piv_pass_args);
  out[1] = (int64_t)sizeof(fi_fix_args);
  out[2] = (int64_t)sizeof(fi_tps_plan);
  return FI_OK;
}

extern "C" int fi_memcpy_d2h(void* host_dst, const void* device_src, int64_t nbytes,
                             void* stream) {
  FI_REQUIRE(host_dst && device_src && nbytes >= 0, "fi_memcpy_d2h: bad arguments");
  FI_CUDA_TRY(cudaMemcpyAsync(host_dst, device_src, (size_t)nbytes, cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
  return FI_OK;
}

extern "C" int fi_images_min(const void* im0, const void* im1, int dtype, int64_t count,
                             float* out_min, void* stream) {
  FI_REQUIRE(im0 && im1 && out_min, "fi_images_min: null pointer");
  FI_REQUIRE(dtype == FI_U8 || dtype == FI_U16 || dtype == FI_F32, "fi_images_min: bad dtype %d",
             dtype);
  FI_REQUIRE(count > 0, "fi_images_min: empty image");
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t* keys = reinterpret_cast<uint32_t*>(out_min);
  k_min_init<<<1, 32, 0, s>>>(keys);
  int blocks = (int)((count + 255) / 256);
  const int cap = num_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_images_min<<<blocks, 256, 0, s>>>(im0, im1, dtype, count, keys);
  k_min_decode<<<1, 32, 0, s>>>(keys);
  return check_launch("fi_images_min", 3);
}

extern "C" int fi_piv_pass(const fi_piv_pass_args* args, void* stream) {
  FI_REQUIRE(args, "fi_piv_pass: null args");
  const fi_piv_pass_args& a = *args;
  FI_REQUIRE(supported_n(a.n), "fi_piv_pass: window size %d not supported (16, 24, 32, 48, 64)",
             a.n);
  FI_REQUIRE(a.im0 && a.im1 && a.im_min && a.ixvecs && a.iyvecs, "fi_piv_pass: null input");
  FI_REQUIRE(a.deltaxs && a.deltays && a.correls_max && a.errors && a.xs && a.ys,
             "fi_piv_pass: null output");
  FI_REQUIRE(a.dtype == FI_U8 || a.dtype == FI_U16 || a.dtype == FI_F32,
             "fi_piv_pass: bad dtype %d", a.dtype);
  FI_REQUIRE(a.nx > 0 && a.ny > 0 && a.height > 0 && a.width > 0, "fi_piv_pass: empty grid");
  FI_REQUIRE((a.dxin == nullptr) == (a.dyin == nullptr), "fi_piv_pass: dxin/dyin mismatch");
  FI_REQUIRE(a.box_i0_start >= 0 && a.box_i0_stop <= a.n && a.box_i1_start >= 0 &&
                 a.box_i1_stop <= a.n,
             "fi_piv_pass: bad search box");
  FI_REQUIRE(a.subpix_method >= FI_SUBPIX_GAUSSIAN2 && a.subpix_method <= FI_SUBPIX_NONE,
             "fi_piv_pass: bad subpix_method %d", a.subpix_method);
  FI_REQUIRE(a.subpix_method == FI_SUBPIX_GAUSSIAN2 ||
                 (a.nsubpix >= 1 && a.nsubpix <= FI_MAX_NSUBPIX),
             "fi_piv_pass: nsubpix %d out of 1..%d", a.nsubpix, FI_MAX_NSUBPIX);
  FI_REQUIRE(a.subpix_method != FI_SUBPIX_GAUSSIAN || a.subpix_minv,
             "fi_piv_pass: '2d_gaussian' needs subpix_minv");
  FI_REQUIRE(a.nb_peaks <= FI_MAX_PEAKS, "fi_piv_pass: nb_peaks %d > %d", a.nb_peaks,
             FI_MAX_PEAKS);
  FI_REQUIRE(a.nb_peaks <= 1 || (a.peaks_count && a.peaks && a.peaks_err),
             "fi_piv_pass: secondary peaks need peaks_count, peaks and peaks_err");
  const int64_t nvec64 = (int64_t)a.nx * a.ny;
  FI_REQUIRE(nvec64 < (1ll << 31), "fi_piv_pass: too many vectors");
  const int nvec = (int)nvec64;
  const int npad = a.n / 2 + (a.n % 2);
  cudaStream_t s = (cudaStream_t)stream;
  switch (a.n) {
    case 16: return launch_pass<16, false>(a, nullptr, nullptr, nvec, npad, 1, s);
    case 24: return launch_pass<24, false>(a, nullptr, nullptr, nvec, npad, 1, s);
    case 32: return launch_pass<32, false>(a, nullptr, nullptr, nvec, npad, 1, s);
    case 48: return launch_pass<48, false>(a, nullptr, nullptr, nvec, npad, 1, s);
    default: return launch_pass<64, false>(a, nullptr, nullptr, nvec, npad, 1, s);
  }
}

extern "C" int fi_correl_windows(const float* win0, const float* win1, int count, int n,
                                 float* planes, double* norms, void* stream) {
  FI_REQUIRE(win0 && win1 && planes && norms, "fi_correl_windows: null pointer");
  FI_REQUIRE(supported_n(n), "fi_correl_windows: window size %d not supported", n);
  FI_REQUIRE(count > 0, "fi_correl_windows: no window");
  fi_piv_pass_args a{};
  a.n = n;
  a.planes = planes;
  a.norms = norms;
  cudaStream_t s = (cudaStream_t)stream;
  switch (n) {
    case 16: return launch_pass<16, true>(a, win0, win1, count, 0, 0, s);
    case 24: return launch_pass<24, true>(a, win0, win1, count, 0, 0, s);
    case 32: return launch_pass<32, true>(a, win0, win1, count, 0, 0, s);
    case 48: return launch_pass<48, true>(a, win0, win1, count, 0, 0, s);
    default: return launch_pass<64, true>(a, win0, win1, count, 0, 0, s);
  }
}

extern "C" int fi_subpix_at(const float* planes, int count, int n, const int32_t* peak_i0,
                            const int32_t* peak_i1, int subpix_method, int nsubpix,
                            const double* subpix_minv, float* deltaxs, float* deltays,
                            uint8_t* errors, void* stream) {
  FI_REQUIRE(planes && peak_i0 && peak_i1 && deltaxs && deltays && errors,
             "fi_subpix_at: null pointer");
  FI_REQUIRE(count > 0 && n >= 3, "fi_subpix_at: bad sizes");
  FI_REQUIRE(subpix_method >= FI_SUBPIX_GAUSSIAN2 && subpix_method <= FI_SUBPIX_NONE,
             "fi_subpix_at: bad subpix_method %d", subpix_method);
  FI_REQUIRE(subpix_method == FI_SUBPIX_GAUSSIAN2 || (nsubpix >= 1 && nsubpix <= FI_MAX_NSUBPIX),
             "fi_subpix_at: nsubpix %d out of 1..%d", nsubpix, FI_MAX_NSUBPIX);
  FI_REQUIRE(subpix_method != FI_SUBPIX_GAUSSIAN || subpix_minv,
             "fi_subpix_at: '2d_gaussian' needs subpix_minv");
  k_subpix_at<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
      planes, count, n, peak_i0, peak_i1, subpix_method, nsubpix, subpix_minv, deltaxs, deltays,
      errors);
  return check_launch("fi_subpix_at");
}

extern "C" int fi_peaks_from_planes(float* planes, const double* norms, int count, int n,
                                    const uint8_t* mask, int box_i0_start, int box_i0_stop,
                                    int box_i1_start, int box_i1_stop, int particle_radius,
                                    int apply_subpix, int subpix_method, int nsubpix,
                                    const double* subpix_minv, int nb_peaks, float* deltaxs,
                                    float* deltays, float* correls_max, uint8_t* errors,
                                    int32_t* peak_i0, int32_t* peak_i1, int32_t* peaks_count,
                                    float* peaks, uint8_t* peaks_err, void* stream) {
  FI_REQUIRE(planes && norms && deltaxs && deltays && correls_max && errors,
             "fi_peaks_from_planes: null pointer");
  FI_REQUIRE(supported_n(n), "fi_peaks_from_planes: window size %d not supported", n);
  FI_REQUIRE(count > 0, "fi_peaks_from_planes: no plane");
  FI_REQUIRE(box_i0_start >= 0 && box_i0_stop <= n && box_i1_start >= 0 && box_i1_stop <= n,
             "fi_peaks_from_planes: bad search box");
  FI_REQUIRE(subpix_method >= FI_SUBPIX_GAUSSIAN2 && subpix_method <= FI_SUBPIX_NONE,
             "fi_peaks_from_planes: bad subpix_method %d", subpix_method);
  FI_REQUIRE(subpix_method == FI_SUBPIX_GAUSSIAN2 || (nsubpix >= 1 && nsubpix <= FI_MAX_NSUBPIX),
             "fi_peaks_from_planes: nsubpix %d out of 1..%d", nsubpix, FI_MAX_NSUBPIX);
  FI_REQUIRE(subpix_method != FI_SUBPIX_GAUSSIAN || subpix_minv,
             "fi_peaks_from_planes: '2d_gaussian' needs subpix_minv");
  FI_REQUIRE(nb_peaks >= 1 && nb_peaks <= FI_MAX_PEAKS, "fi_peaks_from_planes: nb_peaks %d",
             nb_peaks);
  FI_REQUIRE(nb_peaks == 1 || (peaks_count && peaks && peaks_err),
             "fi_peaks_from_planes: secondary peaks need peaks_count, peaks and peaks_err");
  PeakArgs pa;
  pa.mask = mask;
  pa.box = SearchBox{box_i0_start, box_i0_stop, box_i1_start, box_i1_stop};
  pa.radius = particle_radius;
  pa.apply_subpix = apply_subpix;
  pa.subpix_method = subpix_method;
  pa.nsubpix = nsubpix;
  pa.minv = subpix_minv;
  pa.nb_peaks = nb_peaks;
  cudaStream_t s = (cudaStream_t)stream;
#define FI_PEAKS_CASE(NN)                                                                     \
  case NN:                                                                                   \
    return launch_peaks<NN>(planes, norms, count, pa, deltaxs, deltays, correls_max, errors, \
                            peak_i0, peak_i1, peaks_count, peaks, peaks_err, s);
  switch (n) {
    FI_PEAKS_CASE(16)
    FI_PEAKS_CASE(24)
    FI_PEAKS_CASE(32)
    FI_PEAKS_CASE(48)
    default:
      return launch_peaks<64>(planes, norms, count, pa, deltaxs, deltays, correls_max, errors,
                              peak_i0, peak_i1, peaks_count, peaks, peaks_err, s);
  }
#undef FI_PEAKS_CASE
}
