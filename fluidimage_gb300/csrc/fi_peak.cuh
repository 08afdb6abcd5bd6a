// Peak search, second-chance search and subpixel fit on a correlation plane held in
// shared memory by a group of G threads (16, 32 or 64), shared by the FP32 FFT
// pass (fi_correl.cu) and the tensor-core DFT pass (fi_correl_tc.cu).
//
// Upstream behaviour restated here (fluidimage 0.5.3):
//   plane layout       _like_fftshift, calcul/correl.py:596-636
//   peak search        nan_indices_max, calcul/correl.py:88-164
//   second chance      CorrelBase.compute_displacements_from_correl, correl.py:226-275
//   subpixel           compute_subpix_2d_gaussian2 + SubPix.compute_subpix,
//                      calcul/subpix.py:16-61, 107-218
//   window positions   works/piv/singlepass.py:210-260, 787-870 (window_positions)
#pragma once

#include <cmath>

#include "fi_common.cuh"

namespace fi {

template <int N>
struct Cfg {
  static constexpr int G = (N <= 16) ? 16 : ((N <= 32) ? 32 : 64);  // threads / window
  static constexpr int WPB = (G == 16) ? 16 : ((G == 32) ? 8 : 2);  // windows / block
  static constexpr int THREADS = G * WPB;
  // resident CTAs per SM asked of the register allocator (16-px windows: 3, i.e.
  // 24 warps, at <= 85 registers; 48-px windows: 4, i.e. 16 warps at 128 registers,
  // 6 % faster than 12 warps at 166 registers despite 72 bytes of spills; 16-px
  // windows at 2 CTAs and 128 registers were 5 % slower)
  static constexpr int MIN_BLOCKS = (N <= 16) ? 3 : ((N == 48) ? 4 : 1);
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
// tie_rel: the two largest values within tie_rel (relative) flag a near-tie.
template <int N>
__device__ PeakOut find_peak(const float* PL, const uint8_t* mask, const SearchBox& box,
                             const NanBoxes& nb, float normf, int t, int g, double* red,
                             float tie_rel) {
  using C = Cfg<N>;
  Peak p{-INFINITY, -1, -INFINITY};
  if (t < N && t >= box.i1s && t < box.i1e) {
    if (mask == nullptr && nb.n == 0) {
      // nothing excluded but NaNs, which never compare greater or equal
#pragma unroll 8
      for (int i0 = box.i0s; i0 < box.i0e; ++i0) {
        const float v = PL[i0 * C::LDP + t];
        if (v >= p.v) {
          p.v2 = p.v;
          p.v = v;
          p.f = i0 * N + t;
        } else if (v > p.v2) {
          p.v2 = v;
        }
      }
    } else {
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
  o.tie = (p.v - p.v2) <= tie_rel * fabsf(p.v);
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
// operation order, in two halves.  First half, for element k of the 3x3 crop:
// (c - min) / (max - min), the 1e-8 floor of zeros and the float32 log; `low`: the
// normalised value lies within 1e-5 of the minimum.
static __device__ __forceinline__ float gauss2_log(const float (&c)[9], int k, bool* low) {
  float cmin = c[0];
#pragma unroll
  for (int q = 1; q < 9; ++q) cmin = (c[q] < cmin) ? c[q] : cmin;
  float n[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) n[q] = __fsub_rn(c[q], cmin);
  float cmx = n[0];
#pragma unroll
  for (int q = 1; q < 9; ++q) cmx = (n[q] > cmx) ? n[q] : cmx;
  float nk = n[0];
#pragma unroll
  for (int q = 1; q < 9; ++q) nk = (q == k) ? n[q] : nk;  // static indices: registers
  float v = __fdiv_rn(nk, cmx);
  *low = v < 1e-5f;
  if (v == 0.0f) v = 1e-8f;
  return logf(v);
}

// Second half: the least-squares coefficients of the nine logs and the offsets.
// False when |depl|^2 > 4.5 (upstream then falls back to the centroid).
static __device__ bool gauss2_fit(const float (&l)[9], float* deplx_o, float* deply_o) {
  float c10 = 0.f, c01 = 0.f, c11 = 0.f, c20 = 0.f, c02 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float lv = l[3 * a + b];
      c10 = __fadd_rn(c10, __fmul_rn((float)(b - 1), lv));
      c01 = __fadd_rn(c01, __fmul_rn((float)(a - 1), lv));
      c11 = __fadd_rn(c11, __fmul_rn((float)((b - 1) * (a - 1)), lv));
      c20 = __fadd_rn(c20, __fmul_rn((float)(3 * (b - 1) * (b - 1) - 2), lv));
      c02 = __fadd_rn(c02, __fmul_rn((float)(3 * (a - 1) * (a - 1) - 2), lv));
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

// Both halves on one thread.  min_tie: two or more crop values at the minimum (the
// 1e-8 floor then makes the fit depend on which of them rounds to exactly zero).
static __device__ bool gauss2_depl(const float (&c)[9], float* deplx_o, float* deply_o,
                                   bool* min_tie) {
  float l[9];
  int nlow = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    bool low;
    l[k] = gauss2_log(c, k, &low);
    nlow += low ? 1 : 0;
  }
  *min_tie = nlow >= 2;
  return gauss2_fit(l, deplx_o, deply_o);
}

// The first half on threads 0..8 of a group of G threads (one crop element each):
// the nine logs into lg[0..8] (shared memory, read by thread 0 after the call) and
// the count of values at the minimum (returned on every thread).
template <int G>
__device__ __forceinline__ int gauss2_logs_group(const float* PL, int ld, int i0, int i1,
                                                 const NanBox& cbox, int t, float* lg) {
  float c[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const int r = i0 - 1 + a, q = i1 - 1 + b;
      c[3 * a + b] = cbox.has(r, q) ? NAN : PL[r * ld + q];
    }
  bool low = false;
  const float l = gauss2_log(c, t < 9 ? t : 0, &low);
  if (t < 9) lg[t] = l;
  const unsigned m = seg_mask<G>();
  const unsigned base = (G == 16) ? (threadIdx.x & 16u) : 0u;
  const unsigned bits = __ballot_sync(m, low && t < 9);
  __syncwarp(m);  // threads 0..8 and thread 0 share a warp
  return __popc((bits >> base) & 0x1FFu);
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

// want64: also the float64 displacement (dx64, dy64) of the '2d_gaussian2' fit and
// of integer results (the other methods compute in float64 anyway).
// logs9 / nlow9: the first half of '2d_gaussian2' computed by gauss2_logs_group.
static __device__ int subpix_any(const float* PL, int ld, int N, int i0, int i1, int method, int nsub,
                          const double* minv, const NanBox& cbox, SubpixOut* o,
                          bool want64 = false, const float* logs9 = nullptr, int nlow9 = 0) {
  const int ix0 = N / 2 - 1, iy0 = N / 2 - 1;
  const int n = (method == FI_SUBPIX_GAUSSIAN2) ? 1 : nsub;
  o->tie = false;
  auto integer = [&](int err) {
    o->dx32 = (float)(ix0 - i1);
    o->dy32 = (float)(iy0 - i0);
    if (want64) {
      o->dx64 = (double)(ix0 - i1);
      o->dy64 = (double)(iy0 - i0);
    }
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
    float deplx, deply;
    bool fit;
    if (logs9) {
      float l[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) l[k] = logs9[k];
      o->tie = nlow9 >= 2;
      fit = gauss2_fit(l, &deplx, &deply);
    } else {
      float c[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) c[3 * a + b] = val(i0 - 1 + a, i1 - 1 + b);
      fit = gauss2_depl(c, &deplx, &deply, &o->tie);
    }
    if (fit) {
      o->dx32 = __fsub_rn((float)ix0, __fadd_rn(deplx, (float)i1));
      o->dy32 = __fsub_rn((float)iy0, __fadd_rn(deply, (float)i0));
      if (want64) {
        o->dx64 = __dsub_rn((double)ix0, __dadd_rn((double)deplx, (double)i1));
        o->dy64 = __dsub_rn((double)iy0, __dadd_rn((double)deply, (double)i0));
      }
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
  float tie_rel;  // near-tie tolerance of the peak searches (1e-6: FP32 planes)
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
  PeakOut p1 = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red, pa.tie_rel);
  VecResult r;
  r.tie = p1.tie;
  r.subpix_tie = false;
  r.sec_tie = false;
  r.nb = NanBox{0, 0, 0, 0};
  PeakOut fin = p1;
  if (p1.err == FI_VEC_PEAK_BOUNDARY || p1.err == FI_VEC_PEAK_NAN) {
    boxes.add(p1.i0, p1.i1, pa.radius, N);
    if (boxes.n) r.nb = boxes.b[0];
    PeakOut p2 = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red, pa.tie_rel);
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
  if (fin.err == FI_VEC_OK && pa.apply_subpix) {
    // '2d_gaussian2': the nine divisions and logs on nine threads (through the
    // group's scratch, past the words the reductions use), the fit on one
    float* lg = reinterpret_cast<float*>(red + 24);
    const bool g2 = pa.subpix_method == FI_SUBPIX_GAUSSIAN2;
    const int nlow = g2 ? gauss2_logs_group<Cfg<N>::G>(PL, Cfg<N>::LDP, fin.i0, fin.i1, cbox, t, lg)
                        : 0;
    if (t == 0) {
      SubpixOut sp;
      r.err = subpix_any(PL, Cfg<N>::LDP, N, fin.i0, fin.i1, pa.subpix_method, pa.nsubpix,
                         pa.minv, cbox, &sp, false, g2 ? lg : nullptr, nlow);
      r.subpix_tie = sp.tie;
      r.dx = sp.dx32;
      r.dy = sp.dy32;
    }
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
        const PeakOut q = find_peak<N>(PL, pa.mask, pa.box, boxes, normf, t, g, red, pa.tie_rel);
        r.sec_tie = r.sec_tie || q.tie;
        if (q.err != FI_VEC_OK) break;
        a0 = q.i0;
        a1 = q.i1;
        if (t == 0) {
          SubpixOut sp;
          const int e = subpix_any(PL, Cfg<N>::LDP, N, a0, a1, pa.subpix_method, pa.nsubpix,
                                   pa.minv, cbox, &sp, so->has_in);
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


// float32 of a float32 displacement plus an int32 input shift, as upstream's
// float64 sum rounded to float32: exact operands and one rounding for shifts below
// 2^24; larger shifts through float64 (kept out of line: never taken in practice).
static __device__ __noinline__ float add_shift_f64(float d, int s) {
  return (float)((double)d + (double)s);
}
__device__ __forceinline__ float add_shift(float d, int s) {
  return (abs(s) < (1 << 24)) ? __fadd_rn(d, (float)s) : add_shift_f64(d, s);
}

// Vector position (i0 + i1) / 2 (singlepass.py:862-863) as float32: float64 / 2 then
// float32 equals rounding the integer sum to float32 then halving (exact).
__device__ __forceinline__ float midpoint(int sum) { return __fmul_rn(__int2float_rn(sum), 0.5f); }

// Window origins of one vector in the unpadded image (pass 0: the grid; pass >= 1:
// windows shifted by the integer input displacement, with upstream's fix-ups of
// windows leaving the image, singlepass.py:210-260, 787-870), and whether both crops
// of the zero-padded images have the full n x n shape (numpy slice rules).
struct WinPos {
  int y0 = 0, x0 = 0, y1 = 0, x1 = 0;          // top-left of window 0 / 1
  int ixs0 = 0, iys0 = 0, ixs1 = 0, iys1 = 0;  // window centres
  int dinx = 0, diny = 0;                      // input shift (passes >= 1)
  bool valid = true;
};

template <int N>
__device__ __forceinline__ WinPos window_positions(const fi_piv_pass_args& a, int w, int npad) {
  WinPos p;
  const int gx = __ldg(a.ixvecs + (w % a.nx));
  const int gy = __ldg(a.iyvecs + (w / a.nx));
  p.ixs0 = p.ixs1 = gx;
  p.iys0 = p.iys1 = gy;
  if (a.dxin) {
    p.dinx = __ldg(a.dxin + w);
    p.diny = __ldg(a.dyin + w);
    p.ixs0 = gx - floordiv2(p.dinx);
    p.iys0 = gy - floordiv2(p.diny);
    p.ixs1 = p.ixs0 + p.dinx;
    p.iys1 = p.iys0 + p.diny;
    const int H = a.height, W = a.width;
    const bool out1 = p.ixs1 > W || p.iys1 > H || p.ixs1 < 0 || p.iys1 < 0;
    const bool out0 = p.ixs0 > W || p.iys0 > H || p.ixs0 < 0 || p.iys0 < 0;
    if (out1) {
      p.ixs0 = gx - p.dinx;
      p.iys0 = gy - p.diny;
      p.ixs1 = gx;
      p.iys1 = gy;
    } else if (out0) {
      p.ixs0 = gx;
      p.iys0 = gy;
      p.ixs1 = gx + p.dinx;
      p.iys1 = gy + p.diny;
    }
  }
  const int startc = N / 2, stopc = N / 2 + (N % 2);
  const int Ly = a.height + 2 * npad, Lx = a.width + 2 * npad;
  int s0y, e0y, s0x, e0x, s1y, e1y, s1x, e1x;
  slice_bounds(p.iys0 + npad - startc, p.iys0 + npad + stopc, Ly, &s0y, &e0y);
  slice_bounds(p.ixs0 + npad - startc, p.ixs0 + npad + stopc, Lx, &s0x, &e0x);
  slice_bounds(p.iys1 + npad - startc, p.iys1 + npad + stopc, Ly, &s1y, &e1y);
  slice_bounds(p.ixs1 + npad - startc, p.ixs1 + npad + stopc, Lx, &s1x, &e1x);
  p.valid = (e0y - s0y == N) && (e0x - s0x == N) && (e1y - s1y == N) && (e1x - s1x == N);
  p.y0 = s0y - npad;
  p.x0 = s0x - npad;
  p.y1 = s1y - npad;
  p.x1 = s1x - npad;
  return p;
}

// Per-window scalars of a window pair from its sums: the means, the power-of-two
// scales 2^-e that bring each window to unit RMS, the norm sqrt(S0 S1) with
// S = sum (v - mean)^2 (upstream's sqrt(4 E0 E1) N, fft.py:107-109, 259-269) in
// float32 and float64, and the scale of the FP32 path's inverse FFT.
// Integer images (intpath): u = {sum v0, sum v0^2, sum v1, sum v1^2}, exact.  Float
// images: sums = the same four as compensated float sums (float64 values).
// FP64 is narrow on this GPU (an FP64 instruction costs the whole warp's FP64 issue
// even with one lane active), so the integer-image, power-of-two-window case uses
// exact integer arithmetic and float32 only.
struct WinScalars {
  float mean0, mean1;
  int e0, e1;
  float normf;
  double norm64;   // computed when want_norm64 (the caller's norms array)
  float outscale;  // 0.25 / (N^2 2^-e0 2^-e1)
};

// Correctly rounded float32 of an unsigned 64-bit integer on the integer pipe: the
// top 32 significant bits with a sticky bit for the rest (the 64-bit conversion
// instruction runs on the narrow FP64 pipe of this GPU).
__device__ __forceinline__ float u64_to_float_rn(unsigned long long v) {
  const unsigned hi = (unsigned)(v >> 32);
  if (hi == 0u) return __uint2float_rn((unsigned)v);
  const int s = 32 - __clz(hi);  // bits beyond the top 32
  const unsigned long long rest = v & ((1ull << s) - 1ull);
  const unsigned m = (unsigned)(v >> s) | (rest != 0ull ? 1u : 0u);
  return __uint2float_rn(m) * __int_as_float((127 + s) << 23);
}

template <int N>
__device__ __forceinline__ WinScalars window_scalars(bool intpath,
                                                     const unsigned long long (&u)[4],
                                                     const double (&sums_in)[4], bool flat0,
                                                     bool flat1, bool want_norm64) {
  WinScalars r;
  int e0 = 0, e1 = 0;
  double sums[4] = {sums_in[0], sums_in[1], sums_in[2], sums_in[3]};
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
      r.mean0 = ldexpf(__uint2float_rn((unsigned)u[0]), -2 * L);
      r.mean1 = ldexpf(__uint2float_rn((unsigned)u[2]), -2 * L);
      const float S0f = ldexpf(u64_to_float_rn(SN0), -2 * L);
      const float S1f = ldexpf(u64_to_float_rn(SN1), -2 * L);
      r.normf = __fsqrt_rn(__fmul_rn(S0f, S1f));
      r.norm64 = want_norm64 ? ldexp(sqrt((double)SN0 * (double)SN1), -2 * L) : 0.0;
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
      r.mean0 = (float)(sums[0] * INN);
      r.mean1 = (float)(sums[2] * INN);
      r.norm64 = sqrt(S0 * S1);
      r.normf = (float)r.norm64;
    }
    // scale of the inverse FFT: 0.25 / (N^2 sc0 sc1) = 2^(e0 + e1 - 2 - 2L)
    r.outscale = ldexpf(1.0f, e0 + e1 - 2 - 2 * L);
  } else if (intpath) {
    // 24 and 48 px windows of integer images: N^2 S exact in 64 bits as above; the
    // scales 2^-e from its bit length (any power of two gives the same planes: the
    // FFT commutes with exact scalings; this one keeps the values near unit RMS); the
    // means, S and the norm in float32 (the DC bin is zeroed, so the mean only
    // centres the values); FP64 only for the caller's norms array
    constexpr unsigned long long NN = (unsigned long long)N * N;
    constexpr int LB = 64 - __builtin_clzll(NN * NN);  // bit length of N^4
    const unsigned long long SN0 = flat0 ? 0ull : NN * u[1] - u[0] * u[0];
    const unsigned long long SN1 = flat1 ? 0ull : NN * u[3] - u[2] * u[2];
    if (SN0 != 0ull) e0 = ((64 - __clzll((long long)SN0)) - LB + 1) >> 1;
    if (SN1 != 0ull) e1 = ((64 - __clzll((long long)SN1)) - LB + 1) >> 1;
    const float nnf = (float)NN;
    r.mean0 = __fdiv_rn(__uint2float_rn((unsigned)u[0]), nnf);
    r.mean1 = __fdiv_rn(__uint2float_rn((unsigned)u[2]), nnf);
    const float S0f = __fdiv_rn(u64_to_float_rn(SN0), nnf);
    const float S1f = __fdiv_rn(u64_to_float_rn(SN1), nnf);
    r.normf = __fsqrt_rn(__fmul_rn(S0f, S1f));
    r.norm64 = want_norm64 ? sqrt((double)SN0 * (double)SN1) / (double)NN : 0.0;
    // scale of the inverse FFT: 0.25 / (N^2 2^-e0 2^-e1)
    r.outscale = ldexpf(__fdiv_rn(0.25f, nnf), e0 + e1);
  } else {
    const double NN = (double)N * (double)N;
    const double S0 = flat0 ? 0.0 : fmax(sums[1] - sums[0] * sums[0] / NN, 0.0);
    const double S1 = flat1 ? 0.0 : fmax(sums[3] - sums[2] * sums[2] / NN, 0.0);
    if (S0 > 0.0) frexp(sqrt(S0 / NN), &e0);
    if (S1 > 0.0) frexp(sqrt(S1 / NN), &e1);
    r.mean0 = (float)(sums[0] / NN);
    r.mean1 = (float)(sums[2] / NN);
    // scale of the inverse FFT: 0.25 / (N^2 sc0 sc1), sc0 sc1 a power of two
    r.outscale = (float)(0.25 / (NN * (double)ldexpf(1.0f, -e0) * (double)ldexpf(1.0f, -e1)));
    r.norm64 = sqrt(S0 * S1);
    r.normf = (float)r.norm64;
  }
  r.e0 = e0;
  r.e1 = e1;
  return r;
}

}  // namespace fi
