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
// plane in shared memory.  Window sums and energies: exact 64-bit integer sums for
// integer images, compensated float32 sums for float images.  The per-window code
// is in fi_window.cuh (shared with the batched kernels of fi_batch.cu).
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "fi_common.cuh"
#include "fi_fft.cuh"
#include "fi_peak.cuh"
#include "fi_window.cuh"

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


// ---- batched passes: one launch per window size over many passes ----
// All passes of one window size n (each its own images, shape, grid and outputs)
// run in one launch of one block per work item: each block takes the next item from
// a device counter (the queue order is the caller's: largest windows first); an item
// is WPB consecutive windows of one pass (WPB groups of Cfg<n>::G threads), items
// numbered pass by pass (item_start).  A block per item, not a persistent loop: the
// loop kept more registers live across items and spilled (a few hundred bytes per
// thread at the single-pass kernels' register budgets).

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
  FI_REQUIRE(supported_n(a.n), "fi_piv_pass: window size %d not supported (8, 12, 16, 24, 32, 48, 64)",
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
    case 8: return launch_pass<8, false>(a, nullptr, nullptr, nvec, npad, 1, s);
    case 12: return launch_pass<12, false>(a, nullptr, nullptr, nvec, npad, 1, s);
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
    case 8: return launch_pass<8, true>(a, win0, win1, count, 0, 0, s);
    case 12: return launch_pass<12, true>(a, win0, win1, count, 0, 0, s);
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
    FI_PEAKS_CASE(8)
    FI_PEAKS_CASE(12)
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
