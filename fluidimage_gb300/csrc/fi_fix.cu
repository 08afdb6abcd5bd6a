// False-vector removal of one pass: WorkFIX.calcul (works/piv/fix.py:66-243) with
// the NaN-aware 8-neighbour mean mean_neighbors_xy (calcul/mean_neighbors.py:5-155).
//
// Stage A (elementwise): vectors with a correlation error, with
// correls_max < correl_min or with |d|^2 > displacement_max^2 become NaN.
// Stage B (3x3 stencil on the vector grid): |d - mean8(d)|^2 > threshold^2 -> NaN.
// Stage C (nb_peaks > 1): replacement by a secondary peak.
// All arithmetic is float32 in the upstream operation order; comparisons use the
// float32-rounded thresholds (numpy 2 scalar promotion).
#include <mutex>

#include "fi_common.cuh"

namespace fi {

// Scratch of fi_fix_static: the stage-A output (x then y) of up to
// FI_FIX_STATIC_MAX_VECTORS vectors.  Every GPU that loads this library holds it
// (2 MiB) until the process exits; all calls on a device share it.
static __device__ __align__(256) float g_fix_scratch[2 * FI_FIX_STATIC_MAX_VECTORS];

// Device address of g_fix_scratch on the current device, looked up once per device.
// (The host-side name g_fix_scratch is only a stand-in and must never be passed to
// a kernel.)
static int fix_scratch_address(float** out) {
  static std::mutex lock;
  static float* addr[64] = {};
  int dev = 0;
  FI_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("fi_fix_static: device index %d out of range", dev);
    return FI_ERR_INVALID;
  }
  std::lock_guard<std::mutex> guard(lock);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    FI_CUDA_TRY(cudaGetSymbolAddress(&p, g_fix_scratch));
    addr[dev] = static_cast<float*>(p);
  }
  *out = addr[dev];
  return FI_OK;
}

// Stage A of vector i.
__device__ __forceinline__ void fix_a_one(const fi_fix_args& a, int i, float cmin, float dmax2,
                                          float* ox, float* oy) {
  float dx = a.deltaxs[i], dy = a.deltays[i];
  bool wrong = a.errors[i] != 0;
  uint8_t flags = 0;
  if (wrong) dx = dy = NAN;
  if (a.correls_max[i] < cmin) {
    flags |= FI_FIX_CORREL_MIN;
    if (!wrong) dx = dy = NAN;
    wrong = true;
  }
  if (a.use_displacement_max) {
    const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 > dmax2) {
      flags |= FI_FIX_DISPLACEMENT;
      if (!wrong) dx = dy = NAN;
      wrong = true;
    }
  }
  ox[i] = dx;
  oy[i] = dy;
  a.fix_flags[i] = flags;
  if (a.diff2) a.diff2[i] = NAN;
}

__global__ void k_fix_a(fi_fix_args a, int nvec, float cmin, float dmax2, float* ox, float* oy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvec) return;
  fix_a_one(a, i, cmin, dmax2, ox, oy);
}

// a[i0][i1] (0 where NaN) and validity b, read from the stage-A output.
struct Grid {
  const float* x;
  const float* y;
  int n0, n1;
  __device__ __forceinline__ bool ok(int i0, int i1) const {
    const int k = i0 * n1 + i1;
    return !(isnan(x[k]) || isnan(y[k]));
  }
  __device__ __forceinline__ float ax(int i0, int i1) const {
    return ok(i0, i1) ? x[i0 * n1 + i1] : 0.0f;
  }
  __device__ __forceinline__ float ay(int i0, int i1) const {
    return ok(i0, i1) ? y[i0 * n1 + i1] : 0.0f;
  }
  __device__ __forceinline__ float b(int i0, int i1) const { return ok(i0, i1) ? 1.0f : 0.0f; }
};

// Sum over the neighbours in the order of _mean_neighbors (mean_neighbors.py:5-125).
template <int C>  // C = 0: x, 1: y, 2: count
__device__ __forceinline__ float nsum(const Grid& g, int i0, int i1) {
  auto v = [&](int r, int c) -> float {
    if (C == 0) return g.ax(r, c);
    if (C == 1) return g.ay(r, c);
    return g.b(r, c);
  };
  const int n0 = g.n0, n1 = g.n1;
  const bool top = i0 == 0, bot = i0 == n0 - 1, lef = i1 == 0, rig = i1 == n1 - 1;
  if ((top || bot) && (lef || rig)) {  // corners
    const int d0 = top ? 1 : -1, d1 = lef ? 1 : -1;
    return __fadd_rn(__fadd_rn(v(i0 + d0, i1), v(i0 + d0, i1 + d1)), v(i0, i1 + d1));
  }
  if (top || bot) {
    const int dn = top ? 1 : -1;
    float s = __fadd_rn(v(i0, i1 - 1), v(i0, i1 + 1));
    s = __fadd_rn(s, v(i0 + dn, i1 + 1));
    s = __fadd_rn(s, v(i0 + dn, i1));
    s = __fadd_rn(s, v(i0 + dn, i1 - 1));
    return s;
  }
  if (lef || rig) {
    const int dn = lef ? 1 : -1;
    float s = __fadd_rn(v(i0 - 1, i1), v(i0 + 1, i1));
    s = __fadd_rn(s, v(i0 - 1, i1 + dn));
    s = __fadd_rn(s, v(i0, i1 + dn));
    s = __fadd_rn(s, v(i0 + 1, i1 + dn));
    return s;
  }
  float s = __fadd_rn(v(i0, i1 - 1), v(i0, i1 + 1));
  s = __fadd_rn(s, __fadd_rn(v(i0 - 1, i1 + 1), v(i0 + 1, i1 + 1)));
  s = __fadd_rn(s, __fadd_rn(v(i0 - 1, i1), v(i0 + 1, i1)));
  s = __fadd_rn(s, __fadd_rn(v(i0 - 1, i1 - 1), v(i0 + 1, i1 - 1)));
  return s;
}

// Stage B of vector i.
__device__ __forceinline__ void fix_b_one(const fi_fix_args& a, int i, const float* ix,
                                          const float* iy, float thr2) {
  Grid g{ix, iy, a.ny, a.nx};
  const int i0 = i / a.nx, i1 = i % a.nx;
  const float dx = ix[i], dy = iy[i];
  float ox = dx, oy = dy;
  if (g.ok(i0, i1)) {
    const float cnt = nsum<2>(g, i0, i1);
    if (cnt != 0.0f) {
      const float mx = __fdiv_rn(nsum<0>(g, i0, i1), cnt);
      const float my = __fdiv_rn(nsum<1>(g, i0, i1), cnt);
      const float ex = __fsub_rn(mx, dx), ey = __fsub_rn(my, dy);
      const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
      if (a.diff2) a.diff2[i] = d2;
      if (d2 > thr2) {
        a.fix_flags[i] |= FI_FIX_NEIGHBOUR;
        ox = oy = NAN;
      }
    }
  }
  a.deltaxs_out[i] = ox;
  a.deltays_out[i] = oy;
}

__global__ void k_fix_b(fi_fix_args a, const float* ix, const float* iy, float thr2) {
  const int nvec = a.nx * a.ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvec) return;
  fix_b_one(a, i, ix, iy, thr2);
}

// Batched stages A and B over the vectors of many passes (vec_start: the first
// vector of each pass, npass + 1 entries).  The squared thresholds are float32
// products of the float32 thresholds, equal to the float64 square rounded to
// float32 (the float64 product of two float32 values is exact).
__device__ __forceinline__ int batch_pass_of(const int32_t* vec_start, int npass, int i) {
  int lo = 0, hi = npass - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(vec_start + mid) <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_fix_batch_a(const fi_fix_args* __restrict__ args,
                              const int32_t* __restrict__ vec_start, int npass) {
  const int total = __ldg(vec_start + npass);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int p = batch_pass_of(vec_start, npass, i);
    const fi_fix_args& a = args[p];
    const int nvec = a.nx * a.ny;
    const float dmax2 = __fmul_rn(a.displacement_max, a.displacement_max);
    float* ox = a.use_threshold ? a.work : a.deltaxs_out;
    float* oy = a.use_threshold ? a.work + nvec : a.deltays_out;
    fix_a_one(a, i - __ldg(vec_start + p), a.correl_min, dmax2, ox, oy);
  }
}

__global__ void k_fix_batch_b(const fi_fix_args* __restrict__ args,
                              const int32_t* __restrict__ vec_start, int npass) {
  const int total = __ldg(vec_start + npass);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int p = batch_pass_of(vec_start, npass, i);
    const fi_fix_args& a = args[p];
    if (!a.use_threshold) continue;
    const int nvec = a.nx * a.ny, j = i - __ldg(vec_start + p);
    if (a.nx < 2 || a.ny < 2) {  // no neighbour stencil (callers reject such passes)
      a.deltaxs_out[j] = a.work[j];
      a.deltays_out[j] = a.work[nvec + j];
      continue;
    }
    fix_b_one(a, j, a.work, a.work + nvec, __fmul_rn(a.threshold, a.threshold));
  }
}

// Stage C (fix.py:135-236): a vector whose secondary peaks (correl ratio > 0.6,
// correl > correl_min, integer displacement + input shift) hold one closer to the
// neighbour mean of the stage-A field than the vector itself is replaced by that
// peak's subpixel value, unless its distance exceeds the threshold, its |d|^2
// exceeds displacement_max (unsquared, as upstream) or its subpixel fit failed.
// Distances in float64 like upstream; ties keep the first (np.argmin).
__global__ void k_fix_c(fi_fix_args a, const float* ix, const float* iy) {
  const int nvec = a.nx * a.ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvec) return;
  const int cnt = a.peaks_count[i];
  if (cnt <= 0) return;
  const int K = a.nb_peaks - 1;
  const float c0 = a.correls_max[i];
  const float* pk = a.peaks + (int64_t)i * K * FI_PEAK_FIELDS;
  const int dxi = a.dxin ? a.dxin[i] : 0, dyi = a.dyin ? a.dyin[i] : 0;
  int good[FI_MAX_PEAKS];
  int ng = 0;
  for (int j = 0; j < cnt && j < K; ++j) {
    const float cm = pk[j * FI_PEAK_FIELDS + 2];
    if (__fdiv_rn(cm, c0) > 0.6f && cm > a.correl_min) good[ng++] = j;
  }
  if (ng == 0) return;
  const float d2 = a.diff2[i];
  if (isnan(d2)) return;  // np.argmin picks the NaN distance of the vector itself
  Grid g{ix, iy, a.ny, a.nx};
  const int i0 = i / a.nx, i1 = i % a.nx;
  const float n = nsum<2>(g, i0, i1);
  const double mx = (double)__fdiv_rn(nsum<0>(g, i0, i1), n);
  const double my = (double)__fdiv_rn(nsum<1>(g, i0, i1), n);
  double best = sqrt((double)d2);
  int am = -1;
  for (int k = 0; k < ng; ++k) {
    const int j = good[k];
    const double ex = mx - (double)((int)pk[j * FI_PEAK_FIELDS] + dxi);
    const double ey = my - (double)((int)pk[j * FI_PEAK_FIELDS + 1] + dyi);
    const double dn = sqrt(ex * ex + ey * ey);
    if (dn < best) {
      best = dn;
      am = j;
    }
  }
  if (am < 0) return;
  if (a.use_threshold && best > a.threshold64) return;
  const double pdx = (double)((int)pk[am * FI_PEAK_FIELDS] + dxi);
  const double pdy = (double)((int)pk[am * FI_PEAK_FIELDS + 1] + dyi);
  if (a.displacement_max64 != 0.0 && pdx * pdx + pdy * pdy > a.displacement_max64) return;
  if (a.peaks_err[(int64_t)i * K + am] != 0) return;
  a.replaced[3 * (int64_t)i] = a.deltaxs[i];
  a.replaced[3 * (int64_t)i + 1] = a.deltays[i];
  a.replaced[3 * (int64_t)i + 2] = c0;
  a.deltaxs_out[i] = pk[am * FI_PEAK_FIELDS + 3];
  a.deltays_out[i] = pk[am * FI_PEAK_FIELDS + 4];
  a.correls_max_out[i] = pk[am * FI_PEAK_FIELDS + 2];
  a.fix_flags[i] |= FI_FIX_REPLACED;
}

// Checks of the secondary-peak inputs; FI_OK when nb_peaks <= 1.
static int check_secondary(const fi_fix_args& a, const char* who) {
  if (a.nb_peaks <= 1) return FI_OK;
  FI_REQUIRE(a.nb_peaks <= FI_MAX_PEAKS, "%s: nb_peaks %d > %d", who, a.nb_peaks, FI_MAX_PEAKS);
  FI_REQUIRE(a.use_threshold,
             "%s: secondary peaks need the neighbour test (threshold_diff_neighbour)", who);
  FI_REQUIRE(a.diff2 && a.peaks_count && a.peaks && a.peaks_err && a.correls_max_out &&
                 a.replaced,
             "%s: secondary peaks need diff2, peaks_count, peaks, peaks_err, "
             "correls_max_out and replaced", who);
  return FI_OK;
}

}  // namespace fi

using namespace fi;

extern "C" int fi_fix(const fi_fix_args* args, void* stream) {
  FI_REQUIRE(args, "fi_fix: null args");
  const fi_fix_args& a = *args;
  FI_REQUIRE(a.nx >= 1 && a.ny >= 1, "fi_fix: empty vector grid");
  FI_REQUIRE(!a.use_threshold || (a.nx >= 2 && a.ny >= 2),
             "fi_fix: the neighbour test needs a vector grid of at least 2 x 2");
  FI_REQUIRE(a.deltaxs && a.deltays && a.correls_max && a.errors && a.deltaxs_out &&
                 a.deltays_out && a.fix_flags,
             "fi_fix: null pointer");
  FI_REQUIRE(!a.use_threshold || a.work, "fi_fix: the neighbour test needs work[2*nvec]");
  if (check_secondary(a, "fi_fix") != FI_OK) return FI_ERR_INVALID;
  const int nvec = a.nx * a.ny;
  cudaStream_t s = (cudaStream_t)stream;
  const float dmax2 = (float)((double)a.displacement_max * (double)a.displacement_max);
  const float thr2 = (float)((double)a.threshold * (double)a.threshold);
  const int threads = 256, blocks = (nvec + threads - 1) / threads;
  int kernels = 1;  // launches counted by check_launch
  if (a.use_threshold) {
    float* wx = a.work;
    float* wy = a.work + nvec;
    k_fix_a<<<blocks, threads, 0, s>>>(a, nvec, a.correl_min, dmax2, wx, wy);
    k_fix_b<<<blocks, threads, 0, s>>>(a, wx, wy, thr2);
    kernels = 2;
    if (a.nb_peaks > 1) {
      k_fix_c<<<blocks, threads, 0, s>>>(a, wx, wy);
      kernels = 3;
    }
  } else {
    k_fix_a<<<blocks, threads, 0, s>>>(a, nvec, a.correl_min, dmax2, a.deltaxs_out,
                                       a.deltays_out);
  }
  return check_launch("fi_fix", kernels);
}

// Allocation-free variant of fi_fix: same kernels, scratch in g_fix_scratch.
extern "C" int fi_fix_static(const fi_fix_args* args, void* stream) {
  FI_REQUIRE(args, "fi_fix_static: null args");
  const fi_fix_args& a = *args;
  FI_REQUIRE(a.nx >= 1 && a.ny >= 1, "fi_fix_static: empty vector grid");
  FI_REQUIRE(!a.use_threshold || (a.nx >= 2 && a.ny >= 2),
             "fi_fix_static: the neighbour test needs a vector grid of at least 2 x 2");
  FI_REQUIRE((int64_t)a.nx * a.ny <= FI_FIX_STATIC_MAX_VECTORS,
             "fi_fix_static: %lld vectors exceed the static scratch limit of %d vectors "
             "(use fi_fix with a caller-provided work buffer)",
             (long long)a.nx * a.ny, FI_FIX_STATIC_MAX_VECTORS);
  FI_REQUIRE(a.deltaxs && a.deltays && a.correls_max && a.errors && a.deltaxs_out &&
                 a.deltays_out && a.fix_flags,
             "fi_fix_static: null pointer");
  if (check_secondary(a, "fi_fix_static") != FI_OK) return FI_ERR_INVALID;
  float* scratch = nullptr;
  const int rc = fix_scratch_address(&scratch);
  if (rc != FI_OK) return rc;
  const int nvec = a.nx * a.ny;
  cudaStream_t s = (cudaStream_t)stream;
  const float dmax2 = (float)((double)a.displacement_max * (double)a.displacement_max);
  const float thr2 = (float)((double)a.threshold * (double)a.threshold);
  const int threads = 256, blocks = (nvec + threads - 1) / threads;
  int kernels = 1;  // launches counted by check_launch
  if (a.use_threshold) {
    // stage A writes every scratch entry it uses before stage B reads it, so
    // nothing left by an earlier call is ever read
    float* wx = scratch;
    float* wy = scratch + nvec;
    k_fix_a<<<blocks, threads, 0, s>>>(a, nvec, a.correl_min, dmax2, wx, wy);
    k_fix_b<<<blocks, threads, 0, s>>>(a, wx, wy, thr2);
    kernels = 2;
    if (a.nb_peaks > 1) {
      k_fix_c<<<blocks, threads, 0, s>>>(a, wx, wy);
      kernels = 3;
    }
  } else {
    k_fix_a<<<blocks, threads, 0, s>>>(a, nvec, a.correl_min, dmax2, a.deltaxs_out,
                                       a.deltays_out);
  }
  return check_launch("fi_fix_static", kernels);
}

extern "C" int fi_fix_batch(const fi_fix_args* fix_args, const int32_t* vec_start, int npass,
                            int total, void* stream) {
  FI_REQUIRE(fix_args && vec_start && npass > 0 && total > 0, "fi_fix_batch: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 256;
  const int blocks = (total + threads - 1) / threads;
  k_fix_batch_a<<<blocks, threads, 0, s>>>(fix_args, vec_start, npass);
  k_fix_batch_b<<<blocks, threads, 0, s>>>(fix_args, vec_start, npass);
  return check_launch("fi_fix_batch", 2);
}
