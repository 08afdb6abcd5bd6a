// The per-window computation of a PIV pass (staging of the two windows, FFT
// correlation, peak search, subpixel fit, outputs) for one group of threads, shared
// by the single-pass kernels (fi_correl.cu) and the batched kernels (fi_batch.cu).
#pragma once

#include <cstdint>

#include "fi_common.cuh"
#include "fi_fft.cuh"
#include "fi_peak.cuh"

namespace fi {

// Window sizes of the passes (square windows; 2^a 3^b register FFTs).
// window sizes of the single-pass and batched kernels (register FFTs of 2^a 3^b points)
inline bool supported_n(int n) {
  return n == 8 || n == 12 || n == 16 || n == 24 || n == 32 || n == 48 || n == 64;
}
inline bool supported_n_batch(int n) { return supported_n(n); }

// Row `r` of the two windows of an integer image pair (pixels x..x+N-1 of rows y0r
// and y1r, zero outside the image, minus the image minima) staged into Zrow as
// (im0, im1) pairs, with the exact row sums, sums of squares and extremes.  Rows
// inside the image and 16-byte aligned are read by 16-byte loads; others pixel by
// pixel.
struct RowStats {
  unsigned s0 = 0u, s1 = 0u;
  unsigned long long q0 = 0ull, q1 = 0ull;
  int lo0 = 0x7fffffff, lo1 = 0x7fffffff, hi0 = -0x7fffffff, hi1 = -0x7fffffff;
  __device__ __forceinline__ void add(int v0, int v1) {
    s0 += (unsigned)v0;
    s1 += (unsigned)v1;
    q0 += (unsigned long long)((unsigned)v0 * (unsigned)v0);
    q1 += (unsigned long long)((unsigned)v1 * (unsigned)v1);
    lo0 = min(lo0, v0);
    lo1 = min(lo1, v1);
    hi0 = max(hi0, v0);
    hi1 = max(hi1, v1);
  }
};

template <int N>
__device__ __forceinline__ void stage_rows_int(const fi_piv_pass_args& a, int y0r, int x0,
                                               int y1r, int x1, int mini0, int mini1,
                                               float2* Zrow, RowStats& st) {
  const int H = a.height, W = a.width;
  const bool u16 = a.dtype == FI_U16;
  const int esz = u16 ? 2 : 1;
  const unsigned char* p0 = reinterpret_cast<const unsigned char*>(a.im0) +
                            ((int64_t)y0r * W + x0) * esz;
  const unsigned char* p1 = reinterpret_cast<const unsigned char*>(a.im1) +
                            ((int64_t)y1r * W + x1) * esz;
  const bool in0 = y0r >= 0 && y0r < H && x0 >= 0 && x0 + N <= W;
  const bool in1 = y1r >= 0 && y1r < H && x1 >= 0 && x1 + N <= W;
  const bool vec = in0 && in1 && (((reinterpret_cast<uintptr_t>(p0) |
                                     reinterpret_cast<uintptr_t>(p1)) & 15) == 0);
  if (vec && u16 && (N % 8) == 0) {
#pragma unroll
    for (int k = 0; k < N / 8; ++k) {
      const uint4 A = __ldg(reinterpret_cast<const uint4*>(p0) + k);
      const uint4 B = __ldg(reinterpret_cast<const uint4*>(p1) + k);
      const uint32_t wa[4] = {A.x, A.y, A.z, A.w}, wb[4] = {B.x, B.y, B.z, B.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int v0 = (int)((wa[i] >> (16 * h)) & 0xffffu) - mini0;
          const int v1 = (int)((wb[i] >> (16 * h)) & 0xffffu) - mini1;
          Zrow[8 * k + 2 * i + h] = make_float2((float)v0, (float)v1);
          st.add(v0, v1);
        }
    }
    return;
  }
  if (vec && !u16 && (N % 16) == 0) {
#pragma unroll
    for (int k = 0; k < N / 16; ++k) {
      const uint4 A = __ldg(reinterpret_cast<const uint4*>(p0) + k);
      const uint4 B = __ldg(reinterpret_cast<const uint4*>(p1) + k);
      const uint32_t wa[4] = {A.x, A.y, A.z, A.w}, wb[4] = {B.x, B.y, B.z, B.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int v0 = (int)((wa[i] >> (8 * h)) & 0xffu) - mini0;
          const int v1 = (int)((wb[i] >> (8 * h)) & 0xffu) - mini1;
          Zrow[16 * k + 4 * i + h] = make_float2((float)v0, (float)v1);
          st.add(v0, v1);
        }
    }
    return;
  }
  const bool r0 = y0r >= 0 && y0r < H, r1 = y1r >= 0 && y1r < H;
#pragma unroll 4
  for (int c = 0; c < N; ++c) {
    const int xa = x0 + c, xb = x1 + c;
    const int v0 = (r0 && xa >= 0 && xa < W) ? load_px_int(a.im0, a.dtype, (int64_t)y0r * W + xa) - mini0 : 0;
    const int v1 = (r1 && xb >= 0 && xb < W) ? load_px_int(a.im1, a.dtype, (int64_t)y1r * W + xb) - mini1 : 0;
    Zrow[c] = make_float2((float)v0, (float)v1);
    st.add(v0, v1);
  }
}

// One window of a pass, processed by the group g of C::G threads (thread t of it):
// staging, FFT correlation, peak search, subpixel fit, outputs.  gsm: the group's
// shared memory (C::GROUP_BYTES).
template <int N, bool FROM_WINDOWS>
__device__ __forceinline__ void piv_window(const fi_piv_pass_args& a, const float* __restrict__ win0,
                                           const float* __restrict__ win1, int w, int npad,
                                           int do_peaks, int g, int t, unsigned char* gsm) {
  using C = Cfg<N>;
  float2* Z = reinterpret_cast<float2*>(gsm);
  double* red = reinterpret_cast<double*>(gsm + C::ZBYTES);
  float* PL = reinterpret_cast<float*>(Z);

  // ---- window positions (pass 0: grid; pass >= 1: shifted windows) ----
  WinPos wp;
  if (!FROM_WINDOWS) wp = window_positions<N>(a, w, npad);
  const bool valid = wp.valid;
  const int y00 = wp.y0, x00 = wp.x0, y10 = wp.y1, x10 = wp.x1;
  const int dinx = wp.dinx, diny = wp.diny;

  // ---- stage the two windows; exact window sums ----
  // Integer images: exact integer sums of v and v^2 (INT pipe).  Float images and
  // plugin windows: float32 sums with a compensated sum of squares.  FP64 is used
  // only once per window (the FP64 pipe of this GPU is narrow).
  const bool intpath = !FROM_WINDOWS && a.dtype != FI_F32;
  unsigned si0 = 0u, si1 = 0u;
  unsigned long long qi0 = 0ull, qi1 = 0ull;
  float sf0 = 0.f, sf1 = 0.f, qf0 = 0.f, qf1 = 0.f, cf0 = 0.f, cf1 = 0.f;
  float mm[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
  if (intpath) {
    // integer images: with both windows' rows 16-byte aligned (the grid of a first
    // pass), thread t stages row t (16-byte loads); otherwise (shifted windows) thread
    // t stages column t for 32 px windows, so that the warp's loads of a row are
    // coalesced (measured: the shifted 32 px pass of the 2048^2 multipass 0.193 ->
    // 0.168 ms; 16, 24 and 48 px windows were faster row by row)
    const int esz = a.dtype == FI_U16 ? 2 : 1;
    const bool rowwise =
        N != 32 || !valid ||
        ((esz == 2 || N % 16 == 0) && (((x00 | x10) * esz) & 15) == 0 &&
                   ((a.width * esz) & 15) == 0 &&
                   ((reinterpret_cast<uintptr_t>(a.im0) | reinterpret_cast<uintptr_t>(a.im1)) &
                    15) == 0);
    if (t < N && !rowwise) {
      RowStats st;
      const int H = a.height, W = a.width;
      const int mini0 = (int)__ldg(a.im_min + 0), mini1 = (int)__ldg(a.im_min + 1);
#pragma unroll 4
      for (int r = 0; r < N; ++r) {
        const int y0 = y00 + r, xa = x00 + t, y1 = y10 + r, xb = x10 + t;
        const int v0 = (y0 >= 0 && y0 < H && xa >= 0 && xa < W)
                           ? load_px_int(a.im0, a.dtype, (int64_t)y0 * W + xa) - mini0 : 0;
        const int v1 = (y1 >= 0 && y1 < H && xb >= 0 && xb < W)
                           ? load_px_int(a.im1, a.dtype, (int64_t)y1 * W + xb) - mini1 : 0;
        Z[r * C::LD + t] = make_float2((float)v0, (float)v1);
        st.add(v0, v1);
      }
      si0 = st.s0;
      si1 = st.s1;
      qi0 = st.q0;
      qi1 = st.q1;
      mm[0] = (float)st.lo0;
      mm[1] = (float)st.lo1;
      mm[2] = (float)st.hi0;
      mm[3] = (float)st.hi1;
    } else if (t < N) {
      RowStats st;
      if (valid) {
        stage_rows_int<N>(a, y00 + t, x00, y10 + t, x10, (int)__ldg(a.im_min + 0),
                          (int)__ldg(a.im_min + 1), Z + t * C::LD, st);
      } else {
#pragma unroll 4
        for (int c = 0; c < N; ++c) {
          Z[t * C::LD + c] = make_float2(0.f, 0.f);
          st.add(0, 0);
        }
      }
      si0 = st.s0;
      si1 = st.s1;
      qi0 = st.q0;
      qi1 = st.q1;
      mm[0] = (float)st.lo0;
      mm[1] = (float)st.lo1;
      mm[2] = (float)st.hi0;
      mm[3] = (float)st.hi1;
    }
  } else if (t < N) {
    const float min0 = FROM_WINDOWS ? 0.f : __ldg(a.im_min + 0);
    const float min1 = FROM_WINDOWS ? 0.f : __ldg(a.im_min + 1);
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
        if (in0) v0 = __fsub_rn(load_px(a.im0, a.dtype, (int64_t)y0 * W + x0), min0);
        if (in1) v1 = __fsub_rn(load_px(a.im1, a.dtype, (int64_t)y1 * W + x1), min1);
      }
      Z[r * C::LD + t] = make_float2(v0, v1);
      {
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
  double sums[4] = {0.0, 0.0, 0.0, 0.0};
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
  // its scratch
  if (t == 0) {
    // a constant window has an exactly zero spectrum (and plane) upstream
    const bool flat0 = mm[0] == mm[2], flat1 = mm[1] == mm[3];
    const WinScalars ws = window_scalars<N>(intpath, u, sums, flat0, flat1, a.norms != nullptr);
    float* rf = reinterpret_cast<float*>(red + 17);
    rf[0] = ws.mean0;
    rf[1] = ws.mean1;
    rf[2] = ldexpf(1.0f, -ws.e0);
    rf[3] = ldexpf(1.0f, -ws.e1);
    red[16] = ws.norm64;
    reinterpret_cast<int*>(red + 19)[0] = (flat0 || flat1) ? 1 : 0;
    reinterpret_cast<float*>(red + 20)[0] = ws.outscale;
    reinterpret_cast<float*>(red + 20)[1] = ws.normf;
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
    pa.tie_rel = 1e-6f;
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
        dxo = add_shift(dxo, dinx);
        dyo = add_shift(dyo, diny);
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
        const int sx = wp.ixs0 + wp.ixs1, sy = wp.iys0 + wp.iys1;
        a.xs[w] = midpoint(sx);
        a.ys[w] = midpoint(sy);
      }
    }
  }}

}  // namespace fi
