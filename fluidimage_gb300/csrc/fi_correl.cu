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
#include "fi_peak.cuh"

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
  piv_window<N, FROM_WINDOWS>(a, win0, win1, w, npad, do_peaks, g, t,
                              smem_raw + g * C::GROUP_BYTES);
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

// ---- batched passes: one launch per window size over many passes ----
// All passes of one window size n (each its own images, shape, grid and outputs)
// run in one launch of one block per work item: each block takes the next item from
// a device counter (the queue order is the caller's: largest windows first); an item
// is WPB consecutive windows of one pass (WPB groups of Cfg<n>::G threads), items
// numbered pass by pass (item_start).  A block per item, not a persistent loop: the
// loop kept more registers live across items and spilled (a few hundred bytes per
// thread at the single-pass kernels' register budgets).

// resident blocks per SM asked of the register allocator: about 128 / 170 registers
// for 24-32 / 48-64 px windows; for 16 px windows two budgets (128 registers with 16
// windows per block, ~100 with 8) for the tuner to choose from
template <int N, int WPB>
constexpr int batch_min_blocks() {
  return N <= 16 ? (WPB == 16 ? 2 : 5) : (N <= 32 ? 16 / WPB : (N == 48 ? 8 : 6) / WPB);
}

template <int N, int WPB>
__global__ void __launch_bounds__(WPB * Cfg<N>::G, (batch_min_blocks<N, WPB>()))
    k_piv_batch(const fi_piv_pass_args* __restrict__ passes, const int32_t* __restrict__ item_start,
                int npass, int32_t* counter) {
  using C = Cfg<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item, s_pass;
  if (threadIdx.x == 0) {
    const int item = atomicAdd(counter, 1);
    int lo = 0, hi = npass - 1;  // last pass whose first item is <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(item_start + mid) <= item) lo = mid; else hi = mid - 1;
    }
    s_item = item;
    s_pass = lo;
  }
  __syncthreads();
  const int item = s_item, p = s_pass;
  if (item >= __ldg(item_start + npass)) return;
  const int g = threadIdx.x / C::G, t = threadIdx.x % C::G;
  const fi_piv_pass_args& a = passes[p];
  const int w = (item - __ldg(item_start + p)) * WPB + g;
  if (w < a.nx * a.ny)
    piv_window<N, false>(a, nullptr, nullptr, w, N / 2 + (N % 2), 1, g, t,
                         smem_raw + g * C::GROUP_BYTES);
}

static int group_threads(int n) { return n <= 16 ? 16 : (n <= 32 ? 32 : 64); }

static int batch_group_bytes_n(int n) {
  switch (n) {
    case 16: return Cfg<16>::GROUP_BYTES;
    case 24: return Cfg<24>::GROUP_BYTES;
    case 32: return Cfg<32>::GROUP_BYTES;
    case 48: return Cfg<48>::GROUP_BYTES;
    default: return Cfg<64>::GROUP_BYTES;
  }
}

// windows per work item of the batch kernel for each window size: the single-pass
// kernel's windows per block and half of it
static bool batch_wpb_ok(int n, int wpb) {
  switch (n) {
    case 16: return wpb == 16 || wpb == 8;
    case 24: case 32: return wpb == 8 || wpb == 4;
    default: return wpb == 2 || wpb == 1;
  }
}

template <int N, int WPB>
static int launch_batch(const fi_piv_pass_args* passes, const int32_t* item_start, int npass,
                        int blocks, int32_t* counter, cudaStream_t s) {
  using C = Cfg<N>;
  static SmemLimit limit;
  const size_t smem = (size_t)WPB * C::GROUP_BYTES;
  FI_CUDA_TRY(raise_smem_limit(k_piv_batch<N, WPB>, smem, limit));
  k_piv_batch<N, WPB><<<blocks, WPB * C::G, smem, s>>>(passes, item_start, npass, counter);
  return check_launch("k_piv_batch");
}

// Per-pass image minima of a batch: `minblocks` blocks stride over each pass's
// pixels; keys[2 p], keys[2 p + 1] (order-preserving) start at all ones.
__global__ void k_min_batch(const fi_piv_pass_args* __restrict__ passes, int npass, int minblocks,
                            uint32_t* keys) {
  const int p = blockIdx.x / minblocks, b = blockIdx.x % minblocks;
  if (p >= npass) return;
  const fi_piv_pass_args& a = passes[p];
  const int64_t count = (int64_t)a.height * a.width;
  float m0 = INFINITY, m1 = INFINITY;
  const int64_t stride = (int64_t)minblocks * blockDim.x;
  for (int64_t i = (int64_t)b * blockDim.x + threadIdx.x; i < count; i += stride) {
    m0 = fminf(m0, load_px(a.im0, a.dtype, i));
    m1 = fminf(m1, load_px(a.im1, a.dtype, i));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fminf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fminf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(keys + 2 * p, float_to_key(m0));
    atomicMin(keys + 2 * p + 1, float_to_key(m1));
  }
}

// keys -> the float minima each pass reads through its im_min pointer
__global__ void k_min_batch_decode(const fi_piv_pass_args* __restrict__ passes, int npass,
                                   const uint32_t* keys) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npass) return;
  float* out = const_cast<float*>(passes[p].im_min);
  out[0] = key_to_float(keys[2 * p]);
  out[1] = key_to_float(keys[2 * p + 1]);
}

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
  pa.tie_rel = 1e-6f;
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

extern "C" int fi_piv_batch_items(int n, int nvec, int wpb) {
  if (!supported_n(n) || nvec <= 0 || !batch_wpb_ok(n, wpb)) return -1;
  return (nvec + wpb - 1) / wpb;
}

extern "C" int fi_piv_batch_max_blocks(int n, int wpb) {
  if (!supported_n(n) || !batch_wpb_ok(n, wpb)) return -1;
  const int threads = wpb * group_threads(n);
  const int smem = wpb * batch_group_bytes_n(n);
  int per_sm = 0;
  cudaError_t e = cudaErrorInvalidValue;
#define FI_OCC(NN, WW)                                                                         \
  if (n == NN && wpb == WW) {                                                                  \
    static SmemLimit limit;                                                                    \
    e = raise_smem_limit(k_piv_batch<NN, WW>, (size_t)smem, limit);                            \
    if (e == cudaSuccess)                                                                      \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_piv_batch<NN, WW>, threads, \
                                                        (size_t)smem);                         \
  }
  FI_OCC(16, 16) FI_OCC(16, 8) FI_OCC(24, 8) FI_OCC(24, 4) FI_OCC(32, 8) FI_OCC(32, 4)
  FI_OCC(48, 2) FI_OCC(48, 1) FI_OCC(64, 2) FI_OCC(64, 1)
#undef FI_OCC
  if (e != cudaSuccess) {
    set_error("fi_piv_batch_max_blocks: %s", cudaGetErrorString(e));
    return -1;
  }
  return per_sm * num_sms();
}

extern "C" int fi_images_min_batch(const fi_piv_pass_args* pass_args, int npass, uint32_t* keys,
                                   void* stream) {
  FI_REQUIRE(pass_args && keys && npass > 0, "fi_images_min_batch: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  FI_CUDA_TRY(cudaMemsetAsync(keys, 0xFF, (size_t)npass * 2 * sizeof(uint32_t), s));
  const int minblocks = 32;
  k_min_batch<<<npass * minblocks, 256, 0, s>>>(pass_args, npass, minblocks, keys);
  k_min_batch_decode<<<(npass + 127) / 128, 128, 0, s>>>(pass_args, npass, keys);
  return check_launch("fi_images_min_batch", 2);
}

extern "C" int fi_piv_pass_batch(const fi_piv_pass_args* pass_args, const int32_t* item_start,
                                 int npass, int n, int wpb, int items, int32_t* counter,
                                 void* stream) {
  FI_REQUIRE(pass_args && item_start && counter, "fi_piv_pass_batch: null pointer");
  FI_REQUIRE(npass > 0 && items > 0, "fi_piv_pass_batch: empty batch");
  FI_REQUIRE(supported_n(n), "fi_piv_pass_batch: window size %d not supported", n);
  FI_REQUIRE(batch_wpb_ok(n, wpb),
             "fi_piv_pass_batch: %d windows per item not available for %d px windows", wpb, n);
  cudaStream_t s = (cudaStream_t)stream;
  FI_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int32_t), s));
#define FI_BATCH(NN, WW) \
  if (n == NN && wpb == WW) return launch_batch<NN, WW>(pass_args, item_start, npass, items, counter, s);
  FI_BATCH(16, 16) FI_BATCH(16, 8) FI_BATCH(24, 8) FI_BATCH(24, 4) FI_BATCH(32, 8) FI_BATCH(32, 4)
  FI_BATCH(48, 2) FI_BATCH(48, 1) FI_BATCH(64, 2) FI_BATCH(64, 1)
#undef FI_BATCH
  return FI_ERR_INVALID;
}
