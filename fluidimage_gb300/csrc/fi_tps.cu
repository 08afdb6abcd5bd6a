// Thin-plate-spline subdomain smoothing/interpolation in FP64:
// ThinPlateSplineSubdom (calcul/interpolate/thin_plate_spline_subdom.py:25-280) with
// compute_tps_weights / compute_tps_matrix (calcul/interpolate/thin_plate_spline.py:
// 108-216), as called by BaseWorkPIV.apply_interp (works/piv/singlepass.py:466-548).
//
// Stages (host-driven, see the C ABI):
//   plan     : ordered selection of the valid vectors, subdomain layout (1 block)
//   members  : per-subdomain ordered membership, counts then CSR indices + norm coefs
//   solve    : per subdomain (one block): build [[K + lambda I, P], [P^T, 0]] in
//              column-major FP64, LU with partial pivoting, then the iterative
//              outlier replacement (threshold_tps, <= 10 re-solves) for x and y
//              reusing the same factors (the matrix depends on the centres only)
//   blend    : smoothed values at the centres, weighted by the subdomain norm coefs
//   eval     : interpolation at new positions, both components per kernel evaluation
//
// Layout arithmetic (linspace, buffers, norm coefs) uses round-to-nearest
// intrinsics so that it reproduces numpy's float64 results bit for bit.
#include <climits>
#include <cmath>

#include "fi_common.cuh"
#include "fi_df.cuh"
#include "fi_lattice.cuh"

namespace fi {

__device__ __forceinline__ double linspace_at(double start, double stop, int num, int j) {
  if (num > 1 && j == num - 1) return stop;
  if (num <= 1) return start;
  const double div = (double)(num - 1);
  const double delta = __dsub_rn(stop, start);
  const double step = __ddiv_rn(delta, div);
  if (step == 0.0) return __dadd_rn(__dmul_rn(__ddiv_rn((double)j, div), delta), start);
  return __dadd_rn(__dmul_rn((double)j, step), start);
}

struct Limits {
  double lminx, lmaxx, lminy, lmaxy;
};

__device__ __forceinline__ Limits subdom_limits(const fi_tps_plan& p, int ix, int iy) {
  Limits L;
  L.lminx = __dsub_rn(linspace_at(p.x_min, p.x_max, p.nb_subdomx + 1, ix), p.buffer_x);
  L.lmaxx = __dadd_rn(linspace_at(p.x_min, p.x_max, p.nb_subdomx + 1, ix + 1), p.buffer_x);
  L.lminy = __dsub_rn(linspace_at(p.y_min, p.y_max, p.nb_subdomy + 1, iy), p.buffer_y);
  L.lmaxy = __dadd_rn(linspace_at(p.y_min, p.y_max, p.nb_subdomy + 1, iy + 1), p.buffer_y);
  return L;
}

__device__ __forceinline__ bool inside(const Limits& L, double x, double y) {
  return x >= L.lminx && x < L.lmaxx && y >= L.lminy && y < L.lmaxy;
}

// _compute_coef_norm (thin_plate_spline_subdom.py:208-222)
__device__ __forceinline__ double coef_norm(const Limits& L, double x, double y) {
  const double xc = __dmul_rn(0.5, __dadd_rn(L.lminx, L.lmaxx));
  const double yc = __dmul_rn(0.5, __dadd_rn(L.lminy, L.lmaxy));
  const double dxm = __dsub_rn(L.lmaxx, xc), dym = __dsub_rn(L.lmaxy, yc);
  const double ddx = __dsub_rn(x, xc), ddy = __dsub_rn(y, yc);
  const double dx2 = __ddiv_rn(__dmul_rn(ddx, ddx), __dmul_rn(dxm, dxm));
  const double dy2 = __ddiv_rn(__dmul_rn(ddy, ddy), __dmul_rn(dym, dym));
  return __dadd_rn(__dmul_rn(__dsub_rn(1.0, dx2), __dsub_rn(1.0, dy2)), 0.001);
}

// r^2 log(r^2) / 2 with r^2 = (y1 - y0)^2 + (x1 - x0)^2 (thin_plate_spline.py:136-145)
__device__ __forceinline__ double tps_phi(double x0, double y0, double x1, double y1) {
  const double dy = __dsub_rn(y1, y0), dx = __dsub_rn(x1, x0);
  const double r2 = __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx));
  if (r2 == 0.0) return 0.0;
  return __ddiv_rn(__dmul_rn(r2, log(r2)), 2.0);
}

// Same value from a table of phi(k / 4) when 4 r^2 is an integer k < tsize (centres
// and grid points on the half-integer lattice); bit-identical to tps_phi.
__device__ __forceinline__ double tps_phi_tab(double x0, double y0, double x1, double y1,
                                              const double* table, int64_t tsize) {
  const double dy = __dsub_rn(y1, y0), dx = __dsub_rn(x1, x0);
  const double r2 = __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx));
  const double q = 4.0 * r2;
  if (table != nullptr && q < (double)tsize) {
    const int64_t k = (int64_t)q;
    if ((double)k == q) return __ldg(table + k);
  }
  if (r2 == 0.0) return 0.0;
  return __ddiv_rn(__dmul_rn(r2, log(r2)), 2.0);
}

// ---------------------------------------------------------------------------
// block-wide ordered compaction helper (blockDim.x multiple of 32, <= 1024)
// returns the exclusive position of this thread's element and the chunk total.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int block_scan_flag(bool flag, int* warp_tot, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned b = __ballot_sync(0xffffffffu, flag);
  const int in_warp = __popc(b & ((1u << lane) - 1u));
  if (lane == 0) warp_tot[wid] = __popc(b);
  __syncthreads();
  if (wid == 0) {
    int v = lane < nw ? warp_tot[lane] : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane < nw) warp_tot[lane] = incl - v;
    if (lane == 31) warp_tot[32] = incl;
  }
  __syncthreads();
  const int pos = warp_tot[wid] + in_warp;
  *total = warp_tot[32];
  __syncthreads();
  return pos;
}

__device__ __forceinline__ double block_reduce_d(double v, double* sh, bool is_max) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : fmin(v, u);
  }
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < nw ? sh[lane] : (is_max ? -INFINITY : INFINITY);
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_xor_sync(0xffffffffu, v, o);
      v = is_max ? fmax(v, u) : fmin(v, u);
    }
    if (lane == 0) sh[32] = v;
  }
  __syncthreads();
  v = sh[32];
  __syncthreads();
  return v;
}

// float -> double, exact, by the IEEE 754 bit layouts on the integer pipe (normal
// numbers; zero, subnormals, infinities and NaN through the hardware conversion)
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}

// The plan header from the count of valid vectors and their extremes
// (ThinPlateSplineSubdom.__init__, thin_plate_spline_subdom.py:38-91).
__device__ fi_tps_plan plan_header(int base, double xmin, double xmax, double ymin, double ymax,
                                   int subdom_size, double smoothing_coef, double pct) {
  fi_tps_plan p{};
  p.num_centers = base;
  if (base == 0) {
    p.status = 1;
    return p;
  }
  p.x_min = xmin;
  p.x_max = xmax;
  p.y_min = ymin;
  p.y_max = ymax;
  const double range_x = __dsub_rn(xmax, xmin), range_y = __dsub_rn(ymax, ymin);
  const double aspect = __ddiv_rn(range_y, range_x);
  const double nb_subdom = __ddiv_rn((double)base, (double)subdom_size);
  const double fx = floor(__dsqrt_rn(__ddiv_rn(nb_subdom, aspect)));
  const double fy = ceil(__dsqrt_rn(__dmul_rn(nb_subdom, aspect)));
  if (!(fx < 1e6) || !(fy < 1e6)) {  // upstream fails (int(inf) / int(nan))
    p.status = 2;
    return p;
  }
  int nbx = (int)fx, nby = (int)fy;
  if (nbx == 0) nbx = 1;
  if (nby == 0) nby = 1;
  p.nb_subdomx = nbx;
  p.nb_subdomy = nby;
  const double x0 = linspace_at(xmin, xmax, nbx + 1, 0), x1 = linspace_at(xmin, xmax, nbx + 1, 1);
  const double y0 = linspace_at(ymin, ymax, nby + 1, 0), y1 = linspace_at(ymin, ymax, nby + 1, 1);
  const double per = __ddiv_rn((double)base, (double)(nbx * nby));
  p.smoothing = __dmul_rn(
      smoothing_coef, __dsqrt_rn(__ddiv_rn(__dmul_rn(__dsub_rn(x1, x0), __dsub_rn(y1, y0)), per)));
  const double coef_buffer = __ddiv_rn(pct, 100.0);
  p.buffer_x = __ddiv_rn(__dmul_rn(coef_buffer, range_x), (double)nbx);
  p.buffer_y = __ddiv_rn(__dmul_rn(coef_buffer, range_y), (double)nby);
  p.status = 0;
  return p;
}

// Compaction of the valid vectors (no NaN component) in index order, limits and
// subdomain layout; one block of 32 warps, each over one contiguous segment of the
// vectors: the warps count their valid vectors, one block scan places the segments,
// then each warp writes its vectors in order (ballots within the warp), with the
// loads of four chunks of 32 issued before they are used.
__global__ void __launch_bounds__(1024)
    k_tps_plan(const float* xs, const float* ys, const float* dx, const float* dy, int nvec,
               int subdom_size, double smoothing_coef, double pct, fi_tps_plan* plan, double* cx,
               double* cy, float* ux, float* uy, int32_t* sel) {
  constexpr int R = 4;
  __shared__ int warp_tot[33];
  __shared__ double red[33];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int seg = (((nvec + nw - 1) / nw) + 31) & ~31;
  const int s0 = min(nvec, wid * seg), s1 = min(nvec, s0 + seg);
  int cnt = 0;
#pragma unroll 4
  for (int i = s0 + lane; i < s1; i += 32) cnt += (isnan(dx[i]) || isnan(dy[i])) ? 0 : 1;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) warp_tot[wid] = cnt;
  __syncthreads();
  if (wid == 0) {
    const int v = lane < nw ? warp_tot[lane] : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane < nw) warp_tot[lane] = incl - v;
    if (lane == 31) warp_tot[32] = incl;
  }
  __syncthreads();
  const int base = warp_tot[32];
  int pos = warp_tot[wid];
  // limits in float32 (exact: the positions are float32); FP64 is narrow on this GPU
  // and one block does all the vectors
  float fxmin = INFINITY, fxmax = -INFINITY, fymin = INFINITY, fymax = -INFINITY;
  for (int c0 = s0; c0 < s1; c0 += R * 32) {
    float vx[R], vy[R], px[R], py[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = c0 + 32 * r + lane;
      const bool in = i < s1;
      vx[r] = in ? dx[i] : NAN;
      vy[r] = in ? dy[i] : NAN;
      px[r] = in ? xs[i] : 0.f;
      py[r] = in ? ys[i] : 0.f;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = c0 + 32 * r + lane;
      const bool ok = !(isnan(vx[r]) || isnan(vy[r]));
      const unsigned b = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        const int at = pos + __popc(b & ((1u << lane) - 1u));
        cx[at] = f2d_exact(px[r]);
        cy[at] = f2d_exact(py[r]);
        ux[at] = vx[r];
        uy[at] = vy[r];
        if (sel) sel[at] = i;
        fxmin = fminf(fxmin, px[r]);
        fxmax = fmaxf(fxmax, px[r]);
        fymin = fminf(fymin, py[r]);
        fymax = fmaxf(fymax, py[r]);
      }
      pos += __popc(b);
    }
  }
  double xmin = fxmin, xmax = fxmax, ymin = fymin, ymax = fymax;
  xmin = block_reduce_d(xmin, red, false);
  xmax = block_reduce_d(xmax, red, true);
  ymin = block_reduce_d(ymin, red, false);
  ymax = block_reduce_d(ymax, red, true);
  if (threadIdx.x != 0) return;
  *plan = plan_header(base, xmin, xmax, ymin, ymax, subdom_size, smoothing_coef, pct);
}

// The same compaction over many blocks (large passes), in three launches with the
// per-block data in the scratch that follows the plan header (FI_TPS_PLAN_BYTES):
// (1) each block counts the valid vectors of its contiguous chunk and their float32
// extremes; (2) one block scans the counts, reduces the extremes and writes the
// header; (3) each block writes its chunk's valid vectors from its offset, in order.
struct PlanScratch {
  int count[FI_TPS_PLAN_MAX_BLOCKS];
  int offset[FI_TPS_PLAN_MAX_BLOCKS];
  float ext[FI_TPS_PLAN_MAX_BLOCKS][4];  // min x, max x, min y, max y
};

__device__ __forceinline__ PlanScratch* plan_scratch(fi_tps_plan* plan) {
  return reinterpret_cast<PlanScratch*>(reinterpret_cast<unsigned char*>(plan) + 256);
}

__device__ __forceinline__ void plan_chunk(int nvec, int& s0, int& s1) {
  const int chunk = (((nvec + gridDim.x - 1) / gridDim.x) + 31) & ~31;
  s0 = min(nvec, (int)blockIdx.x * chunk);
  s1 = min(nvec, s0 + chunk);
}

__global__ void __launch_bounds__(256)
    k_tps_plan_count(const float* xs, const float* ys, const float* dx, const float* dy,
                     int nvec, fi_tps_plan* plan) {
  __shared__ int s_cnt[8];
  __shared__ float s_ext[8][4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int s0, s1;
  plan_chunk(nvec, s0, s1);
  int cnt = 0;
  float e[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
  for (int i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    if (isnan(dx[i]) || isnan(dy[i])) continue;
    ++cnt;
    const float x = xs[i], y = ys[i];
    e[0] = fminf(e[0], x);
    e[1] = fmaxf(e[1], x);
    e[2] = fminf(e[2], y);
    e[3] = fmaxf(e[3], y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    e[0] = fminf(e[0], __shfl_xor_sync(0xffffffffu, e[0], o));
    e[1] = fmaxf(e[1], __shfl_xor_sync(0xffffffffu, e[1], o));
    e[2] = fminf(e[2], __shfl_xor_sync(0xffffffffu, e[2], o));
    e[3] = fmaxf(e[3], __shfl_xor_sync(0xffffffffu, e[3], o));
  }
  if (lane == 0) {
    s_cnt[wid] = cnt;
    for (int k = 0; k < 4; ++k) s_ext[wid][k] = e[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    PlanScratch* sc = plan_scratch(plan);
    int c = 0;
    float f[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      c += s_cnt[w];
      f[0] = fminf(f[0], s_ext[w][0]);
      f[1] = fmaxf(f[1], s_ext[w][1]);
      f[2] = fminf(f[2], s_ext[w][2]);
      f[3] = fmaxf(f[3], s_ext[w][3]);
    }
    sc->count[blockIdx.x] = c;
    for (int k = 0; k < 4; ++k) sc->ext[blockIdx.x][k] = f[k];
  }
}

__global__ void __launch_bounds__(1024)
    k_tps_plan_head(int nblocks, int subdom_size, double smoothing_coef, double pct,
                    fi_tps_plan* plan) {
  __shared__ int s_wsum[32];
  __shared__ float s_ext[32][4];
  PlanScratch* sc = plan_scratch(plan);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int b = threadIdx.x;
  const int v = b < nblocks ? sc->count[b] : 0;
  float e[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
  if (b < nblocks)
    for (int k = 0; k < 4; ++k) e[k] = sc->ext[b][k];
  int incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  for (int o = 16; o > 0; o >>= 1) {
    e[0] = fminf(e[0], __shfl_xor_sync(0xffffffffu, e[0], o));
    e[1] = fmaxf(e[1], __shfl_xor_sync(0xffffffffu, e[1], o));
    e[2] = fminf(e[2], __shfl_xor_sync(0xffffffffu, e[2], o));
    e[3] = fmaxf(e[3], __shfl_xor_sync(0xffffffffu, e[3], o));
  }
  if (lane == 31) s_wsum[wid] = incl;
  if (lane == 0)
    for (int k = 0; k < 4; ++k) s_ext[wid][k] = e[k];
  __syncthreads();
  int before = 0;
  for (int w = 0; w < wid; ++w) before += s_wsum[w];
  if (b < nblocks) sc->offset[b] = before + incl - v;
  if (threadIdx.x == 0) {
    int base = 0;
    float f[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      base += s_wsum[w];
      f[0] = fminf(f[0], s_ext[w][0]);
      f[1] = fmaxf(f[1], s_ext[w][1]);
      f[2] = fminf(f[2], s_ext[w][2]);
      f[3] = fmaxf(f[3], s_ext[w][3]);
    }
    // the float32 extremes are exact in float64 (the positions are float32)
    *plan = plan_header(base, (double)f[0], (double)f[1], (double)f[2], (double)f[3],
                        subdom_size, smoothing_coef, pct);
  }
}

__global__ void __launch_bounds__(256)
    k_tps_plan_write(const float* xs, const float* ys, const float* dx, const float* dy,
                     int nvec, const fi_tps_plan* plan, double* cx, double* cy, float* ux,
                     float* uy, int32_t* sel) {
  constexpr int R = 4;
  __shared__ int warp_off[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int s0, s1;
  plan_chunk(nvec, s0, s1);
  // the block's chunk in one contiguous segment per warp
  const int seg = (((s1 - s0) + nw - 1) / nw + 31) & ~31;
  const int w0 = min(s1, s0 + wid * seg), w1 = min(s1, w0 + seg);
  int cnt = 0;
  for (int i = w0 + lane; i < w1; i += 32) cnt += (isnan(dx[i]) || isnan(dy[i])) ? 0 : 1;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) warp_off[wid] = cnt;
  __syncthreads();
  int pos = reinterpret_cast<const PlanScratch*>(reinterpret_cast<const unsigned char*>(plan) + 256)
                ->offset[blockIdx.x];
  for (int w = 0; w < wid; ++w) pos += warp_off[w];
  for (int c0 = w0; c0 < w1; c0 += R * 32) {
    float vx[R], vy[R], px[R], py[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = c0 + 32 * r + lane;
      const bool in = i < w1;
      vx[r] = in ? dx[i] : NAN;
      vy[r] = in ? dy[i] : NAN;
      px[r] = in ? xs[i] : 0.f;
      py[r] = in ? ys[i] : 0.f;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = c0 + 32 * r + lane;
      const bool ok = !(isnan(vx[r]) || isnan(vy[r]));
      const unsigned bal = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        const int at = pos + __popc(bal & ((1u << lane) - 1u));
        cx[at] = f2d_exact(px[r]);
        cy[at] = f2d_exact(py[r]);
        ux[at] = vx[r];
        uy[at] = vy[r];
        if (sel) sel[at] = i;
      }
      pos += __popc(bal);
    }
  }
}

// Valid centres and subdomains of a plan as the layout kernels read them on the device
// (none when the plan failed), each clamped to the capacity the host sized for.
__device__ __forceinline__ int plan_centers(const fi_tps_plan* p, int cap) {
  return p->status == 0 ? min(cap, p->num_centers) : 0;
}
__device__ __forceinline__ int plan_subdoms(const fi_tps_plan* p, int cap) {
  return p->status == 0 ? min(cap, p->nb_subdomx * p->nb_subdomy) : 0;
}

// count_plan (nullable): the number of points is the plan's centre count (at most npts)
__global__ void k_tps_lattice(const double* px, const double* py, int npts, int32_t* xy2,
                              int32_t* on_lattice, const fi_tps_plan* count_plan) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (count_plan != nullptr) npts = plan_centers(count_plan, npts);
  if (i >= npts) return;
  const double X = 2.0 * px[i], Y = 2.0 * py[i];
  const bool ok = X == rint(X) && Y == rint(Y) && fabs(X) < 1073741824.0 &&
                  fabs(Y) < 1073741824.0;
  xy2[2 * i] = ok ? (int32_t)X : 0;
  xy2[2 * i + 1] = ok ? (int32_t)Y : 0;
  if (!ok) atomicAnd(on_lattice, 0);
}

__global__ void k_set_int(int32_t* p, int32_t v) { *p = v; }

// Index over the points by tiles of YB_TILE: tile_pmax[j] = max of y over tiles
// 0..j, tile_smin[j] = min over tiles j..end.  Both are monotone, so a y band
// [lo, hi) can only hold points of tiles [first j with tile_pmax[j] >= lo, first j
// with tile_smin[j] >= hi).
constexpr int YB_TILE = 256;
// Order-preserving 64-bit keys of doubles (NaN excluded): max / min of doubles as
// integer max / min on the ALU pipe (FP64 is narrow on this GPU).
__device__ __forceinline__ unsigned long long dkey(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) {
  return a < b ? a : b;
}

__global__ void __launch_bounds__(YB_TILE) k_y_tiles(const double* py, int n, double* tmax,
                                                      double* tmin,
                                                      const fi_tps_plan* count_plan) {
  __shared__ unsigned long long smx[YB_TILE / 32], smn[YB_TILE / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // with count_plan, n is the plan's centre count; tiles past it stay neutral
  if (count_plan != nullptr) n = plan_centers(count_plan, n);
  const int i = blockIdx.x * YB_TILE + threadIdx.x;
  const double y = (i < n) ? py[i] : NAN;
  unsigned long long kx = isnan(y) ? dkey(-INFINITY) : dkey(y);
  unsigned long long kn = isnan(y) ? dkey(INFINITY) : dkey(y);
  for (int o = 16; o > 0; o >>= 1) {
    kx = umax64(kx, __shfl_xor_sync(0xffffffffu, kx, o));
    kn = umin64(kn, __shfl_xor_sync(0xffffffffu, kn, o));
  }
  if (lane == 0) {
    smx[wid] = kx;
    smn[wid] = kn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < YB_TILE / 32; ++w) {
      kx = umax64(kx, smx[w]);
      kn = umin64(kn, smn[w]);
    }
    tmax[blockIdx.x] = dkey_inv(kx);
    tmin[blockIdx.x] = dkey_inv(kn);
  }
}

// In place: running max forward, running min backward over the tiles (one block;
// chunks of 1024 tiles, warp shuffle scans on order-preserving integer keys).
__global__ void __launch_bounds__(1024) k_y_tiles_scan(int ntiles, double* tmax, double* tmin) {
  __shared__ unsigned long long wa[32], wb[32];
  __shared__ unsigned long long carry[2];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const unsigned long long kneg = dkey(-INFINITY), kpos = dkey(INFINITY);
  if (t == 0) {
    carry[0] = kneg;
    carry[1] = kpos;
  }
  __syncthreads();
  for (int base = 0; base < ntiles; base += 1024) {
    const int i = base + t;
    const int ir = ntiles - 1 - i;  // backward scan reads from the end
    unsigned long long ka = (i < ntiles) ? dkey(tmax[i]) : kneg;
    unsigned long long kb = (i < ntiles) ? dkey(tmin[ir]) : kpos;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long ua = __shfl_up_sync(0xffffffffu, ka, o);
      const unsigned long long ub = __shfl_up_sync(0xffffffffu, kb, o);
      if (lane >= o) {
        ka = umax64(ka, ua);
        kb = umin64(kb, ub);
      }
    }
    if (lane == 31) {
      wa[wid] = ka;
      wb[wid] = kb;
    }
    __syncthreads();
    if (wid == 0) {
      unsigned long long x = wa[lane], y = wb[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long ux = __shfl_up_sync(0xffffffffu, x, o);
        const unsigned long long uy = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) {
          x = umax64(x, ux);
          y = umin64(y, uy);
        }
      }
      wa[lane] = x;
      wb[lane] = y;
    }
    __syncthreads();
    if (wid > 0) {
      ka = umax64(ka, wa[wid - 1]);
      kb = umin64(kb, wb[wid - 1]);
    }
    ka = umax64(ka, carry[0]);
    kb = umin64(kb, carry[1]);
    if (i < ntiles) {
      tmax[i] = dkey_inv(ka);
      tmin[ir] = dkey_inv(kb);
    }
    __syncthreads();
    if (t == 0) {
      carry[0] = umax64(carry[0], wa[31]);
      carry[1] = umin64(carry[1], wb[31]);
    }
    __syncthreads();
  }
}

// Exclusive prefix sum of v over the block of 1024 threads; *total gets the sum.
__device__ __forceinline__ int64_t block_scan_i64(int64_t v, int64_t* wsum, int64_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const int64_t w = wsum[lane];
    int64_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    wsum[lane] = wi - w;
    if (lane == 31) wsum[32] = wi;
  }
  __syncthreads();
  const int64_t r = wsum[wid] + incl - v;
  *total = wsum[32];
  __syncthreads();
  return r;
}

// subdomain counts up to which fi_tps_offsets ranks the subdomains by size
constexpr int ORDER_MAX = 8192;

// CSR offsets of the centres' and new positions' membership, offsets of the matrix
// slots ((n+3)^2 rounded up to 4 elements) and of the weights (2 (n+3)), the
// summary [total members, total new members, matrix elements, weight elements,
// max members, max new members] and (nullable) the solve order, largest subdomains
// first; one block of 1024 threads.
__global__ void __launch_bounds__(1024)
    k_tps_offsets(const int32_t* counts, const int32_t* ncounts, int nsub, int64_t* off,
                  int64_t* noff, int64_t* moff, int64_t* woff, int64_t* summary,
                  int32_t* order, const fi_tps_plan* count_plan) {
  // with count_plan, nsub is a capacity and the plan gives the subdomains
  if (count_plan != nullptr) nsub = plan_subdoms(count_plan, nsub);
  __shared__ int64_t wsum[33];
  __shared__ int s_max[2];
  if (threadIdx.x == 0) s_max[0] = s_max[1] = 0;
  int64_t carry[4] = {0, 0, 0, 0};
  __syncthreads();
  for (int base = 0; base < nsub; base += 1024) {
    const int i = base + threadIdx.x;
    const int64_t c = (i < nsub) ? counts[i] : 0;
    const int64_t nc = (i < nsub) ? ncounts[i] : 0;
    const int64_t msz = (i < nsub) ? (((c + 3) * (c + 3) + 3) / 4) * 4 : 0;
    const int64_t wsz = (i < nsub) ? 2 * (c + 3) : 0;
    if (i < nsub) {
      atomicMax(&s_max[0], (int)c);
      atomicMax(&s_max[1], (int)nc);
    }
    const int64_t vals[4] = {c, nc, msz, wsz};
    int64_t* outs[4] = {off, noff, moff, woff};
    for (int k = 0; k < 4; ++k) {
      int64_t tot;
      const int64_t ex = block_scan_i64(vals[k], wsum, &tot);
      if (i < nsub) outs[k][i] = carry[k] + ex;
      carry[k] += tot;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; ++k) summary[k] = carry[k];
    summary[4] = s_max[0];
    summary[5] = s_max[1];
  }
  // solve order: members descending, index ascending among equal counts (stable
  // rank by counting, O(nsub^2) / 1024 per thread; identity beyond ORDER_MAX)
  if (order != nullptr) {
    for (int i = threadIdx.x; i < nsub; i += blockDim.x) {
      int rank = i;
      if (nsub <= ORDER_MAX) {
        const int ci = counts[i];
        rank = 0;
        for (int j = 0; j < nsub; ++j) {
          const int cj = counts[j];
          rank += (cj > ci) || (cj == ci && j < i);
        }
      }
      order[rank] = i;
    }
  }
}

// First index q in [0, n) with a[q] >= v for a non-decreasing a (n if none).
__device__ __forceinline__ int lower_bound_ge(const double* a, int n, double v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] >= v) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// First index q in [0, n) with a[q] >= v for a non-decreasing a (n if none), by one
// warp: each round probes 32 evenly spaced entries and keeps the part holding the
// answer (ceil(log32 n) rounds of loads instead of log2 n dependent loads).
__device__ __forceinline__ int warp_lower_bound_ge(const double* a, int n, double v, int lane) {
  int lo = 0, hi = n;  // the answer lies in [lo, hi]
  while (lo < hi) {
    const int step = (hi - lo + 31) / 32;
    const int at = lo + (lane + 1) * step - 1;  // last entry of part `lane`
    const bool ge = at >= hi || a[at] >= v;
    const unsigned b = __ballot_sync(0xffffffffu, ge);
    if (b == 0u) return hi;  // every entry of [lo, hi) is below v
    const int first = __ffs(b) - 1;
    const int nlo = lo + first * step;
    hi = min(hi, lo + (first + 1) * step - 1);
    lo = nlo;
  }
  return lo;
}

// coef_norm with the subdomain's constants c = (xc, yc, dxm^2, dym^2) computed once
// (the same operations in the same order)
__device__ __forceinline__ double coef_norm_hoisted(const double* c, double x, double y) {
  const double ddx = __dsub_rn(x, c[0]), ddy = __dsub_rn(y, c[1]);
  const double dx2 = __ddiv_rn(__dmul_rn(ddx, ddx), c[2]);
  const double dy2 = __ddiv_rn(__dmul_rn(ddy, ddy), c[3]);
  return __dadd_rn(__dmul_rn(__dsub_rn(1.0, dx2), __dsub_rn(1.0, dy2)), 0.001);
}

// Ordered membership of points in subdomain blockIdx.x; mode 0 counts, mode 1 fills.
// With the tile index y_pmax / y_smin of py (k_y_tiles) only the tiles that can hold
// the subdomain's y band are scanned.  subdoms_from_plan: the grid is a capacity,
// blocks past the plan's subdomains return; centres_from_plan: the points are the
// plan's centres (npts a capacity).
__global__ void __launch_bounds__(512)
    k_tps_members(const fi_tps_plan* plan_ptr, const double* px, const double* py, int npts,
                  int mode, int32_t* counts, const int64_t* offsets, int32_t* indices,
                  double* coefs, const int32_t* xy2, const int32_t* on_lattice,
                  const double* y_pmax, const double* y_smin, int subdoms_from_plan,
                  int centres_from_plan) {
  if (subdoms_from_plan && (int)blockIdx.x >= plan_subdoms(plan_ptr, gridDim.x)) return;
  if (centres_from_plan) npts = plan_centers(plan_ptr, npts);
  __shared__ int warp_tot[33];
  __shared__ int s_range[2], s_box[4];
  __shared__ Limits sL;
  __shared__ double s_cn[4];  // coef_norm's subdomain constants: xc, yc, dxm^2, dym^2
  const int i = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the subdomain's limits once per block (FP64 is narrow on this GPU)
  if (threadIdx.x == 0) {
    const fi_tps_plan p = *plan_ptr;
    const int iy = i / p.nb_subdomx, ix = i % p.nb_subdomx;
    const Limits L = subdom_limits(p, ix, iy);
    sL = L;
    // on the lattice, X = 2x is an integer: x >= l <=> X >= ceil(2l), x < l <=> X < ceil(2l)
    const double kmax = 2147483647.0;
    s_box[0] = (int)fmin(ceil(2.0 * L.lminx), kmax);
    s_box[1] = (int)fmin(ceil(2.0 * L.lmaxx), kmax);
    s_box[2] = (int)fmin(ceil(2.0 * L.lminy), kmax);
    s_box[3] = (int)fmin(ceil(2.0 * L.lmaxy), kmax);
    const double xc = __dmul_rn(0.5, __dadd_rn(L.lminx, L.lmaxx));
    const double yc = __dmul_rn(0.5, __dadd_rn(L.lminy, L.lmaxy));
    const double dxm = __dsub_rn(L.lmaxx, xc), dym = __dsub_rn(L.lmaxy, yc);
    s_cn[0] = xc;
    s_cn[1] = yc;
    s_cn[2] = __dmul_rn(dxm, dxm);
    s_cn[3] = __dmul_rn(dym, dym);
    warp_tot[32] = 0;
  }
  __syncthreads();
  const Limits L = sL;
  // the scanned band: tiles that can hold the subdomain's y range (32-ary searches
  // by warp 0 over the non-decreasing tile bounds: two rounds of loads for 8k tiles)
  if (wid == 0) {
    int q0 = 0, q1 = npts;
    if (y_pmax != nullptr && y_smin != nullptr) {
      const int nt = (npts + YB_TILE - 1) / YB_TILE;
      q0 = min(npts, YB_TILE * warp_lower_bound_ge(y_pmax, nt, L.lminy, lane));
      q1 = max(q0, min(npts, YB_TILE * warp_lower_bound_ge(y_smin, nt, L.lmaxy, lane)));
    }
    if (lane == 0) {
      s_range[0] = q0;
      s_range[1] = q1;
    }
  }
  const bool lat = xy2 != nullptr && on_lattice != nullptr && *on_lattice != 0;
  __syncthreads();
  const int X0 = s_box[0], X1 = s_box[1], Y0 = s_box[2], Y1 = s_box[3];
  const int qb = s_range[0], qe = s_range[1];
  if (mode == 0) {  // counts only: per-thread tallies, one block reduction
    int cnt = 0;
    for (int q = qb + threadIdx.x; q < qe; q += blockDim.x) {
      if (lat) {
        const int X = xy2[2 * q], Y = xy2[2 * q + 1];
        cnt += (X >= X0 && X < X1 && Y >= Y0 && Y < Y1) ? 1 : 0;
      } else {
        cnt += inside(L, px[q], py[q]) ? 1 : 0;
      }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&warp_tot[32], cnt);
    __syncthreads();
    if (threadIdx.x == 0) counts[i] = warp_tot[32];
    return;
  }
  // fill: the band in one contiguous segment per warp; the warps count their members,
  // one block scan places the segments, then each warp writes its members in order
  // (ballots within the warp: two barriers in all instead of three per 512 points)
  auto member = [&](int q) -> bool {
    if (lat) {
      const int2 XY = reinterpret_cast<const int2*>(xy2)[q];
      return XY.x >= X0 && XY.x < X1 && XY.y >= Y0 && XY.y < Y1;
    }
    return inside(L, px[q], py[q]);
  };
  const int nw = blockDim.x >> 5;
  const int seg = (((qe - qb) + nw - 1) / nw + 31) & ~31;
  const int s0 = min(qe, qb + wid * seg), s1 = min(qe, s0 + seg);
  int cnt = 0;
#pragma unroll 4
  for (int q = s0 + lane; q < s1; q += 32) cnt += member(q) ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) warp_tot[wid] = cnt;
  __syncthreads();
  if (wid == 0) {
    const int v = lane < nw ? warp_tot[lane] : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane < nw) warp_tot[lane] = incl - v;
  }
  __syncthreads();
  int64_t pos = offsets[i] + warp_tot[wid];
  constexpr int R = 4;  // membership of four chunks of 32 tested (loads issued) first
  for (int c0 = s0; c0 < s1; c0 += R * 32) {
    bool in[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int q = c0 + 32 * r + lane;
      in[r] = q < s1 && member(q);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int q = c0 + 32 * r + lane;
      const unsigned b = __ballot_sync(0xffffffffu, in[r]);
      if (in[r]) {
        const int64_t at = pos + __popc(b & ((1u << lane) - 1u));
        indices[at] = q;
        coefs[at] = coef_norm_hoisted(s_cn, px[q], py[q]);
      }
      pos += __popc(b);
    }
  }
}

// Block argmax of |col[k..n-1]| with the first index on ties (LAPACK idamax).
__device__ __forceinline__ int block_argmax_abs(const double* col, int k, int n, double* shv,
                                                int* shi) {
  double best = -1.0;
  int bi = n;
  for (int r = k + threadIdx.x; r < n; r += blockDim.x) {
    const double v = fabs(col[r]);
    if (v > best) {
      best = v;
      bi = r;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  if (lane == 0) {
    shv[wid] = best;
    shi[wid] = bi;
  }
  __syncthreads();
  if (wid == 0) {
    best = lane < nw ? shv[lane] : -1.0;
    bi = lane < nw ? shi[lane] : n;
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) shi[32] = bi;
  }
  __syncthreads();
  const int r = shi[32];
  __syncthreads();
  return r;
}

// Solve (LU, pivots) x = rhs in place; y in shared memory (n doubles).
__device__ void lu_solve(const double* A, const int32_t* piv, int n, double* y) {
  for (int k = 0; k < n; ++k) {  // row interchanges in order (dgetrs / dlaswp)
    if (threadIdx.x == 0) {
      const int p = piv[k];
      if (p != k) {
        const double t = y[k];
        y[k] = y[p];
        y[p] = t;
      }
    }
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {  // L (unit diagonal), column oriented
    const double yk = y[k];
    const double* col = A + (int64_t)k * n;
    for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) y[r] -= col[r] * yk;
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; --k) {  // U
    const double* col = A + (int64_t)k * n;
    if (threadIdx.x == 0) y[k] = y[k] / col[k];
    __syncthreads();
    const double xk = y[k];
    for (int r = threadIdx.x; r < k; r += blockDim.x) y[r] -= col[r] * xk;
    __syncthreads();
  }
}

// One block per subdomain: build, factorise, iterate the two components.
__global__ void __launch_bounds__(512)
    k_tps_solve(const fi_tps_plan* plan_ptr, const double* cx, const double* cy, const float* ux,
                const float* uy, const int32_t* counts, const int64_t* offsets,
                const int32_t* indices, const int64_t* mat_off, double* matrices, int32_t* pivots,
                double threshold, int use_threshold, const int64_t* w_off, double* weights,
                double* smoothed_x, double* smoothed_y, int32_t* iters, int32_t* nfixed,
                int32_t* singular, double* max_udiff, const int32_t* only_failed) {
  extern __shared__ double sh[];
  __shared__ double shv[33];
  __shared__ int shi[33];
  __shared__ int s_any;
  const fi_tps_plan p = *plan_ptr;
  const int sd = blockIdx.x;
  if (only_failed != nullptr && only_failed[sd] == 0) {  // solved by the mixed-precision path
    if (threadIdx.x == 0) singular[sd] = 0;
    return;
  }
  const int N = counts[sd];
  const int n = N + 3;
  const int64_t off = offsets[sd];
  const int32_t* idx = indices + off;
  double* A = matrices + mat_off[sd];
  int32_t* piv = pivots + (off + 3 * (int64_t)sd);
  double* y = sh;             // n doubles
  float* vals = reinterpret_cast<float*>(sh + n);  // N floats
  const double lam = p.smoothing;

  // ---- build IM = [[K + lam I, P], [P^T, 0]], column-major (symmetric) ----
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = wid; c < n; c += nw) {
    double* col = A + (int64_t)c * n;
    if (c < N) {
      const int b = idx[c];
      const double bx = cx[b], by = cy[b];
      for (int r = lane; r < n; r += 32) {
        double v;
        if (r < N) {
          const int a = idx[r];
          v = (r == c) ? lam : tps_phi(bx, by, cx[a], cy[a]);
        } else {
          v = (r == N) ? 1.0 : ((r == N + 1) ? by : bx);
        }
        col[r] = v;
      }
    } else {
      for (int r = lane; r < n; r += 32) {
        double v = 0.0;
        if (r < N) {
          const int a = idx[r];
          v = (c == N) ? 1.0 : ((c == N + 1) ? cy[a] : cx[a]);
        }
        col[r] = v;
      }
    }
  }
  __syncthreads();

  // ---- LU with partial pivoting (right-looking, column-major) ----
  int sing = 0;
  for (int k = 0; k < n; ++k) {
    double* colk = A + (int64_t)k * n;
    const int pr = block_argmax_abs(colk, k, n, shv, shi);
    const double pv = colk[pr];
    if (pv == 0.0) {
      sing = 1;
      break;
    }
    if (threadIdx.x == 0) piv[k] = pr;
    if (pr != k)
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double* col = A + (int64_t)c * n;
        const double t = col[k];
        col[k] = col[pr];
        col[pr] = t;
      }
    __syncthreads();
    const double d = colk[k];
    for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) colk[r] = colk[r] / d;
    __syncthreads();
    for (int c = k + 1 + wid; c < n; c += nw) {
      double* col = A + (int64_t)c * n;
      const double akc = col[k];
      for (int r = k + 1 + lane; r < n; r += 32) col[r] -= colk[r] * akc;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) singular[sd] = sing;
  if (sing) return;

  // ---- iterative outlier replacement, compute_tps_weights_iter (subdom.py:236-280) ----
  for (int comp = 0; comp < 2; ++comp) {
    const float* u = comp == 0 ? ux : uy;
    double* sm = comp == 0 ? smoothed_x : smoothed_y;
    double* w = weights + w_off[sd] + (int64_t)comp * n;
    for (int r = threadIdx.x; r < N; r += blockDim.x) vals[r] = u[idx[r]];
    __syncthreads();
    int count = 1, fixed = 0;
    while (true) {
      for (int r = threadIdx.x; r < n; r += blockDim.x) y[r] = (r < N) ? (double)vals[r] : 0.0;
      __syncthreads();
      lu_solve(A, piv, n, y);
      // smoothed = EM @ w = values - lam * w (rows < N of IM w = rhs)
      if (threadIdx.x == 0) s_any = 0;
      __syncthreads();
      double mx = 0.0;
      int nbad = 0;
      for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const double s = __dsub_rn((double)vals[r], __dmul_rn(lam, y[r]));
        sm[off + r] = s;
        const double dif = fabs(__dsub_rn(s, (double)vals[r]));
        mx = fmax(mx, dif);
        if (use_threshold && dif > threshold) nbad++;
      }
      mx = block_reduce_d(mx, shv, true);
      if (count == 1 && threadIdx.x == 0) max_udiff[2 * sd + comp] = mx;
      if (nbad) atomicAdd(&s_any, nbad);
      __syncthreads();
      const int bad = s_any;
      if (!use_threshold || bad == 0 || count > 10) break;
      fixed += bad;
      for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const double s = sm[off + r];
        const double dif = fabs(__dsub_rn(s, (double)vals[r]));
        if (dif > threshold) vals[r] = (float)s;
      }
      __syncthreads();
      count++;
    }
    for (int r = threadIdx.x; r < n; r += blockDim.x) w[r] = y[r];
    if (threadIdx.x == 0) {
      iters[2 * sd + comp] = count;
      nfixed[2 * sd + comp] = fixed;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Subdomain bounds along x and y for the blends, computed once per block (FP64 is
// narrow on this GPU): lo[j] = linspace_j - buffer, hi[j] = linspace_{j+1} + buffer,
// and on the half-pixel lattice the integers ceil(2 lo), ceil(2 hi) (for X = 2x an
// integer, x >= l <=> X >= ceil(2l) and x < l <=> X < ceil(2l)).  Both sequences are
// non-decreasing, so the subdomains holding a point form one range per axis.
constexpr int BLEND_AXIS_MAX = 512;
struct AxisBounds {
  double lo[BLEND_AXIS_MAX], hi[BLEND_AXIS_MAX];
  int ilo[BLEND_AXIS_MAX], ihi[BLEND_AXIS_MAX];
  double vmin, vmax, buffer;
  int nb;
};
__device__ __forceinline__ void axis_bound(double vmin, double vmax, int nb, double buffer, int j,
                                           double& lo, double& hi, int& ilo, int& ihi) {
  const double kmax = 2147483647.0;
  lo = __dsub_rn(linspace_at(vmin, vmax, nb + 1, j), buffer);
  hi = __dadd_rn(linspace_at(vmin, vmax, nb + 1, j + 1), buffer);
  ilo = (int)fmax(fmin(ceil(2.0 * lo), kmax), -kmax);
  ihi = (int)fmax(fmin(ceil(2.0 * hi), kmax), -kmax);
}
// the tables when nb <= BLEND_AXIS_MAX (else axis_range computes the bounds it reads)
__device__ void axis_bounds_fill(AxisBounds& b, double vmin, double vmax, int nb, double buffer) {
  if (threadIdx.x == 0) {
    b.vmin = vmin;
    b.vmax = vmax;
    b.buffer = buffer;
    b.nb = nb;
  }
  if (nb > BLEND_AXIS_MAX) return;
  for (int j = threadIdx.x; j < nb; j += blockDim.x)
    axis_bound(vmin, vmax, nb, buffer, j, b.lo[j], b.hi[j], b.ilo[j], b.ihi[j]);
}
// [first, last) of the subdomains along one axis holding v (V = 2v when on the lattice)
__device__ __forceinline__ int2 axis_range(const AxisBounds& b, double v, bool lat, int V) {
  const int nb = b.nb;
  const bool tab = nb <= BLEND_AXIS_MAX;
  auto above = [&](int j) -> bool {  // hi_j > v
    if (tab) return lat ? (b.ihi[j] > V) : (b.hi[j] > v);
    double lo, hi;
    int ilo, ihi;
    axis_bound(b.vmin, b.vmax, nb, b.buffer, j, lo, hi, ilo, ihi);
    return lat ? (ihi > V) : (hi > v);
  };
  auto starts = [&](int j) -> bool {  // lo_j <= v
    if (tab) return lat ? (b.ilo[j] <= V) : (b.lo[j] <= v);
    double lo, hi;
    int ilo, ihi;
    axis_bound(b.vmin, b.vmax, nb, b.buffer, j, lo, hi, ilo, ihi);
    return lat ? (ilo <= V) : (lo <= v);
  };
  int lo = 0, hi = nb;  // first j with hi_j > v
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (above(mid)) hi = mid; else lo = mid + 1;
  }
  int end = lo;
  while (end < nb && starts(end)) ++end;
  return make_int2(lo, end);
}
// V = 2v as an integer when v is on the half-pixel lattice
__device__ __forceinline__ bool on_half_lattice(double v, int& V) {
  const double t = 2.0 * v;
  if (!(fabs(t) < 1e9)) return false;
  V = (int)t;
  return (double)V == t;
}

// Smoothed values at the centres: sum over containing subdomains, in order.
__global__ void k_tps_blend_centers(const fi_tps_plan* plan_ptr, const double* cx,
                                    const double* cy, const int32_t* counts,
                                    const int64_t* offsets, const int32_t* indices,
                                    const double* coefs, const double* smx, const double* smy,
                                    double* outx, double* outy) {
  __shared__ AxisBounds bx, by;
  const fi_tps_plan p = *plan_ptr;
  axis_bounds_fill(bx, p.x_min, p.x_max, p.nb_subdomx, p.buffer_x);
  axis_bounds_fill(by, p.y_min, p.y_max, p.nb_subdomy, p.buffer_y);
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.num_centers) return;
  const double x = cx[q], y = cy[q];
  int X = 0, Y = 0;
  const bool lat = on_half_lattice(x, X) && on_half_lattice(y, Y);
  const int2 rx_ = axis_range(bx, x, lat, X);
  const int2 ry_ = axis_range(by, y, lat, Y);
  double sx = 0.0, sy = 0.0, nrm = 0.0;
  for (int iy = ry_.x; iy < ry_.y; ++iy)
    for (int ix = rx_.x; ix < rx_.y; ++ix) {
      const int sd = iy * p.nb_subdomx + ix;
      const int64_t off = offsets[sd];
      int lo = 0, hi = counts[sd] - 1;
      while (lo < hi) {  // members are sorted: find q
        const int mid = (lo + hi) >> 1;
        if (indices[off + mid] < q) lo = mid + 1; else hi = mid;
      }
      const double c = coefs[off + lo];
      sx = __dadd_rn(sx, __dmul_rn(c, smx[off + lo]));
      sy = __dadd_rn(sy, __dmul_rn(c, smy[off + lo]));
      nrm = __dadd_rn(nrm, c);
    }
  outx[q] = __ddiv_rn(sx, nrm);
  outy[q] = __ddiv_rn(sy, nrm);
}

// Interpolation at the new positions of subdomain blockIdx.y:
// part[k] = coef_k * (sum_j w_j phi(|q_k - c_j|^2) + w_N + w_N+1 y + w_N+2 x).
// Part of each subdomain's TPS at its new positions: coef * (sum_j w_j phi_j + affine)
// (interpolate, thin_plate_spline_subdom.py:224-234).  On the lattice with the
// (hi, lo) table the kernel sum runs in double-float on the FP32 pipe (~1e-14
// relative per term), else in FP64.  When the block's positions and the centres lie
// on one grid of the lattice, or the centres half a pixel off it along an axis (the
// final evaluation, on the grid of the pass's own windows), and the grid's offsets fit
// tab_cap entries (0 when the launch has no room for them), the block reads the
// (hi, lo) values of the grid's offsets from shared memory (the same table entries).
constexpr int EVAL_TABLE = 2048;

__global__ void __launch_bounds__(256)
    k_tps_eval(const int32_t* counts, const int64_t* offsets, const int32_t* indices,
               const int64_t* w_off, const double* weights, const double* cx, const double* cy,
               const int32_t* ncounts, const int64_t* noffsets, const int32_t* nindices,
               const double* ncoefs, const double* px, const double* py, double* partx,
               double* party, const double* table, const float2* table2, int64_t tsize,
               const int32_t* cxy2, const int32_t* c_on_lattice, int max_members,
               int tab_cap) {
  extern __shared__ double sh[];
  const int sd = blockIdx.y;
  const int N = counts[sd], n = N + 3, M = ncounts[sd];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x * blockDim.x >= M) return;
  const int NM = max_members;
  double* scx = sh;
  double* scy = sh + NM;
  double* swx = sh + 2 * NM;
  double* swy = swx + NM + 3;
  int2* sxy2 = reinterpret_cast<int2*>(swy + NM + 3);   // lattice coordinates of the centres
  float2* dwx = reinterpret_cast<float2*>(sxy2 + NM);  // weights as (hi, lo) pairs
  float2* dwy = dwx + NM;
  float2* tab = dwy + NM;  // tab_cap pairs: kernel values of the grid offsets
  __shared__ int s_lat, s_red[6 * 32];
  const int64_t off = offsets[sd];
  const double* w = weights + w_off[sd];
  if (threadIdx.x == 0) s_lat = (cxy2 != nullptr && c_on_lattice != nullptr) ? *c_on_lattice : 0;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const int a = indices[off + j];
    scx[j] = cx[a];
    scy[j] = cy[a];
    if (cxy2 != nullptr) sxy2[j] = make_int2(cxy2[2 * a], cxy2[2 * a + 1]);
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    swx[j] = w[j];
    swy[j] = w[n + j];
    if (table2 != nullptr && j < N) {
      dwx[j] = df_split(w[j]);
      dwy[j] = df_split(w[n + j]);
    }
  }
  __syncthreads();
  const int64_t noff = noffsets[sd];
  const int q = k < M ? nindices[noff + k] : 0;
  const double x = k < M ? px[q] : 0.0, y = k < M ? py[q] : 0.0;
  double vx = 0.0, vy = 0.0;
  const double X2 = 2.0 * x, Y2 = 2.0 * y;
  const bool qlat = k < M && s_lat && table != nullptr && X2 == rint(X2) && Y2 == rint(Y2) &&
                    fabs(X2) < 1073741824.0 && fabs(Y2) < 1073741824.0;
  const int tsz32 = (int)(tsize < (int64_t)INT_MAX ? tsize : (int64_t)INT_MAX);
  // the grid through the centres and the block's lattice positions (origin: the first
  // centre; every lattice coordinate is below 2^30 in magnitude, so offsets fit)
  int tw = 0, jw = 0, QA = 0, QB = 0;
  if (s_lat && table != nullptr && table2 != nullptr) {
    const int2 o = sxy2[0];
    int v[6];
    lat_grid_init(v);
    for (int j = threadIdx.x; j < N; j += blockDim.x) lat_grid_add(v, sxy2[j].x - o.x, sxy2[j].y - o.y);
    if (qlat) lat_grid_add(v, (int)X2 - o.x, (int)Y2 - o.y);
    lat_grid_block(v, s_red);
    const LatTable g = lat_table_of(v, tab_cap, tsz32);
    if (g.ok) {  // centres to grid indices, the table, this position's grid indices
      tw = g.wx;
      const int ax0 = v[2], ay0 = v[4];  // smallest offsets: index 0 of each axis
      for (int j = threadIdx.x; j < N; j += blockDim.x)
        sxy2[j] = make_int2((sxy2[j].x - o.x - ax0) / g.gx, (sxy2[j].y - o.y - ay0) / g.gy);
      for (int e = threadIdx.x; e < g.wx * g.wy; e += blockDim.x) {
        const int b = e / g.wx, a = e - b * g.wx;
        tab[e] = table2[(g.gy * b) * (g.gy * b) + (g.gx * a) * (g.gx * a)];
      }
      if (qlat) {
        QA = ((int)X2 - o.x - ax0) / g.gx;
        QB = ((int)Y2 - o.y - ay0) / g.gy;
      }
      __syncthreads();
    } else {
      // The positions on a grid of steps (gx, gy) >= 4 (origin: the block's first
      // position) and every centre on it or half a pixel (one lattice unit) after it
      // along each axis (the midpoints of odd window shifts): a centre is at
      // o + g A + e (e in {0, 1}), an offset p - c = g k - e, so |p - c| is g |k|, g |k| + 1
      // (e = 1, k <= 0) or g k - 1 (e = 1, k >= 1): the table holds the kernel value of
      // each (|k|, case) pair per axis, row length jw = 3 Kx.
      const int q0 = nindices[noff + (int64_t)blockIdx.x * blockDim.x];
      const double PX2 = 2.0 * px[q0], PY2 = 2.0 * py[q0];
      const bool oklat = PX2 == rint(PX2) && PY2 == rint(PY2) && fabs(PX2) < 1073741824.0 &&
                         fabs(PY2) < 1073741824.0;
      if (oklat) {  // uniform: every thread read the same position
        const int OX = (int)PX2, OY = (int)PY2;
        int vp[6];
        lat_grid_init(vp);
        if (qlat) lat_grid_add(vp, (int)X2 - OX, (int)Y2 - OY);
        lat_grid_block(vp, s_red);
        const int gpx = vp[0], gpy = vp[1];
        // every position of the block is on the lattice when qlat holds for all of
        // them: count the others (in the gcd slot, as 0 / 1) with the centres below
        if (gpx >= 4 && gpy >= 4) {
          int vc[6];
          lat_grid_init(vc);
          vc[0] = (k < M && !qlat) ? 1 : 0;
          for (int j = threadIdx.x; j < N; j += blockDim.x) {
            const int dx = sxy2[j].x - OX, dy = sxy2[j].y - OY;
            const int ax = (dx >= 0) ? dx / gpx : -((-dx + gpx - 1) / gpx);  // floor
            const int ay = (dy >= 0) ? dy / gpy : -((-dy + gpy - 1) / gpy);
            const int ex = dx - ax * gpx, ey = dy - ay * gpy;
            if (ex > 1 || ey > 1) vc[0] = 1;
            vc[2] = min(vc[2], ax);
            vc[3] = max(vc[3], ax);
            vc[4] = min(vc[4], ay);
            vc[5] = max(vc[5], ay);
          }
          lat_grid_block(vc, s_red);
          // grid indices of the positions: offsets / g (exact)
          const int pax0 = vp[2] / gpx, pax1 = vp[3] / gpx, pay0 = vp[4] / gpy,
                    pay1 = vp[5] / gpy;
          const int kx = max(pax1 - vc[2], vc[3] - pax0) + 1;
          const int ky = max(pay1 - vc[4], vc[5] - pay0) + 1;
          const int64_t ex = (int64_t)gpx * kx + 1, ey = (int64_t)gpy * ky + 1;
          if (vc[0] == 0 && vc[2] <= vc[3] && kx > 0 && ky > 0 &&
              (int64_t)9 * kx * ky <= tab_cap && ex <= 32767 && ey <= 32767 &&
              ex * ex + ey * ey < (int64_t)tsz32) {
            jw = 3 * kx;
            for (int j = threadIdx.x; j < N; j += blockDim.x) {
              const int dx = sxy2[j].x - OX, dy = sxy2[j].y - OY;
              const int ax = (dx >= 0) ? dx / gpx : -((-dx + gpx - 1) / gpx);
              const int ay = (dy >= 0) ? dy / gpy : -((-dy + gpy - 1) / gpy);
              sxy2[j] = make_int2(2 * ax + (dx - ax * gpx), 2 * ay + (dy - ay * gpy));
            }
            for (int e = threadIdx.x; e < 9 * kx * ky; e += blockDim.x) {
              const int r = e / jw, c = e - r * jw;
              const int axx = c / 3, sx = c - 3 * axx, ayy = r / 3, sy = r - 3 * ayy;
              const int adx = gpx * axx + (sx == 1 ? 1 : (sx == 2 ? -1 : 0));
              const int ady = gpy * ayy + (sy == 1 ? 1 : (sy == 2 ? -1 : 0));
              tab[e] = (adx < 0 || ady < 0) ? make_float2(0.f, 0.f)
                                            : table2[ady * ady + adx * adx];
            }
            if (qlat) {
              QA = ((int)X2 - OX) / gpx;
              QB = ((int)Y2 - OY) / gpy;
            }
          }
          __syncthreads();
        }
      }
    }
  }
  if (k >= M) return;
  if (qlat && jw > 0) {  // offsets of the jittered grid in the shared table
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
    constexpr int U = 8;
    for (int j0 = 0; j0 < N; j0 += U) {
      float2 f[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int2 c = sxy2[min(j0 + u, N - 1)];
        const int kx = QA - (c.x >> 1), ky = QB - (c.y >> 1);
        const int sx = (c.x & 1) ? (kx <= 0 ? 1 : 2) : 0;
        const int sy = (c.y & 1) ? (ky <= 0 ? 1 : 2) : 0;
        f[u] = tab[(3 * abs(ky) + sy) * jw + 3 * abs(kx) + sx];
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (j0 + u >= N) break;
        df_mac(dwx[j0 + u], f[u], hx, lx);
        df_mac(dwy[j0 + u], f[u], hy, ly);
      }
    }
    vx += (double)hx + (double)lx;
    vy += (double)hy + (double)ly;
  } else if (qlat && tw > 0) {  // grid offsets in the shared table, double-float sums
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
    constexpr int U = 8;
    for (int j0 = 0; j0 < N; j0 += U) {
      float2 f[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int2 c = sxy2[min(j0 + u, N - 1)];
        f[u] = tab[abs(QB - c.y) * tw + abs(QA - c.x)];
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (j0 + u >= N) break;
        df_mac(dwx[j0 + u], f[u], hx, lx);
        df_mac(dwy[j0 + u], f[u], hy, ly);
      }
    }
    vx += (double)hx + (double)lx;
    vy += (double)hy + (double)ly;
  } else if (qlat && table2 != nullptr) {  // 4 r^2 in integers, double-float sums
    const int QX = (int)X2, QY = (int)Y2;
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
    constexpr int U = 8;  // table loads issued ahead of their use
    for (int j0 = 0; j0 < N; j0 += U) {
      float2 f[U];
      bool far[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int j = j0 + u;
        far[u] = false;
        f[u] = make_float2(0.f, 0.f);
        if (j < N) {
          // 32-bit 4 r^2 (lattice coordinates below 2^30; |dx|, |dy| <= 32767 keeps
          // the sum below 2^31, farther pairs are beyond the table)
          const int2 c = sxy2[j];
          const int dx = QX - c.x, dy = QY - c.y;
          const bool near = (unsigned)dx + 32767u <= 65534u && (unsigned)dy + 32767u <= 65534u;
          const int kq = near ? dy * dy + dx * dx : INT_MAX;
          far[u] = kq >= tsz32;
          if (!far[u]) f[u] = __ldg(table2 + kq);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int j = j0 + u;
        if (j >= N) break;
        if (far[u]) {  // beyond the table: float64 kernel value
          const double fd = tps_phi(scx[j], scy[j], x, y);
          vx = fma(swx[j], fd, vx);
          vy = fma(swy[j], fd, vy);
        } else {
          df_mac(dwx[j], f[u], hx, lx);
          df_mac(dwy[j], f[u], hy, ly);
        }
      }
    }
    vx += (double)hx + (double)lx;
    vy += (double)hy + (double)ly;
  } else if (qlat) {  // 4 r^2 in integer arithmetic, table lookup
    const int QX = (int)X2, QY = (int)Y2;
    for (int j = 0; j < N; ++j) {
      const int2 c = sxy2[j];
      const int64_t dx = (int64_t)(QX - c.x), dy = (int64_t)(QY - c.y);
      const int64_t kq = dy * dy + dx * dx;
      const double f = (kq < tsize) ? __ldg(table + kq) : tps_phi(scx[j], scy[j], x, y);
      vx = fma(swx[j], f, vx);
      vy = fma(swy[j], f, vy);
    }
  } else {
    for (int j = 0; j < N; ++j) {
      const double f = tps_phi_tab(scx[j], scy[j], x, y, table, tsize);
      vx = fma(swx[j], f, vx);
      vy = fma(swy[j], f, vy);
    }
  }
  vx = fma(swx[N + 2], x, fma(swx[N + 1], y, __dadd_rn(vx, swx[N])));
  vy = fma(swy[N + 2], x, fma(swy[N + 1], y, __dadd_rn(vy, swy[N])));
  const double c = ncoefs[noff + k];
  partx[noff + k] = __dmul_rn(c, vx);
  party[noff + k] = __dmul_rn(c, vy);
}

__global__ void k_tps_gather(const fi_tps_plan* plan_ptr, const int32_t* ncounts,
                             const int64_t* noffsets, const int32_t* nindices,
                             const double* ncoefs, const double* partx, const double* party,
                             const double* px, const double* py, int npts, double* outx,
                             double* outy, int32_t* rx, int32_t* ry) {
  __shared__ AxisBounds bx, by;
  const fi_tps_plan p = *plan_ptr;
  axis_bounds_fill(bx, p.x_min, p.x_max, p.nb_subdomx, p.buffer_x);
  axis_bounds_fill(by, p.y_min, p.y_max, p.nb_subdomy, p.buffer_y);
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  const double x = px[q], y = py[q];
  int X = 0, Y = 0;
  const bool lat = on_half_lattice(x, X) && on_half_lattice(y, Y);
  const int2 rx_ = axis_range(bx, x, lat, X);
  const int2 ry_ = axis_range(by, y, lat, Y);
  double sx = 0.0, sy = 0.0, nrm = 0.0;
  for (int iy = ry_.x; iy < ry_.y; ++iy)
    for (int ix = rx_.x; ix < rx_.y; ++ix) {
      const int sd = iy * p.nb_subdomx + ix;
      const int64_t off = noffsets[sd];
      int lo = 0, hi = ncounts[sd] - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nindices[off + mid] < q) lo = mid + 1; else hi = mid;
      }
      sx = __dadd_rn(sx, partx[off + lo]);
      sy = __dadd_rn(sy, party[off + lo]);
      nrm = __dadd_rn(nrm, ncoefs[off + lo]);
    }
  const double vx = __ddiv_rn(sx, nrm), vy = __ddiv_rn(sy, nrm);
  outx[q] = vx;
  outy[q] = vy;
  if (rx) rx[q] = (int32_t)rint(vx);
  if (ry) ry[q] = (int32_t)rint(vy);
}

}  // namespace fi

using namespace fi;

extern "C" int fi_tps_plan_make(const float* xs, const float* ys, const float* dx, const float* dy,
                                int nvec, int subdom_size, double smoothing_coef,
                                double percent_buffer_area, fi_tps_plan* plan, double* cx,
                                double* cy, float* ux, float* uy, int32_t* selection,
                                void* stream) {
  FI_REQUIRE(xs && ys && dx && dy && plan && cx && cy && ux && uy, "fi_tps_plan_make: null pointer");
  FI_REQUIRE(nvec > 0 && subdom_size > 0, "fi_tps_plan_make: bad sizes");
  cudaStream_t s = (cudaStream_t)stream;
  // one block for small passes; chunks of about 1024 vectors per block otherwise
  const int nblocks = min(FI_TPS_PLAN_MAX_BLOCKS, (nvec + 1023) / 1024);
  if (nblocks <= 4) {
    k_tps_plan<<<1, 1024, 0, s>>>(xs, ys, dx, dy, nvec, subdom_size, smoothing_coef,
                                  percent_buffer_area, plan, cx, cy, ux, uy, selection);
    return check_launch("fi_tps_plan_make");
  }
  k_tps_plan_count<<<nblocks, 256, 0, s>>>(xs, ys, dx, dy, nvec, plan);
  k_tps_plan_head<<<1, 1024, 0, s>>>(nblocks, subdom_size, smoothing_coef, percent_buffer_area,
                                      plan);
  k_tps_plan_write<<<nblocks, 256, 0, s>>>(xs, ys, dx, dy, nvec, plan, cx, cy, ux, uy,
                                            selection);
  return check_launch("fi_tps_plan_make", 3);
}

extern "C" int fi_tps_lattice(const double* px, const double* py, int npts, int32_t* xy2,
                              int32_t* on_lattice, void* stream) {
  FI_REQUIRE(px && py && xy2 && on_lattice && npts > 0, "fi_tps_lattice: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  k_set_int<<<1, 1, 0, s>>>(on_lattice, 1);
  k_tps_lattice<<<(npts + 255) / 256, 256, 0, s>>>(px, py, npts, xy2, on_lattice, nullptr);
  return check_launch("fi_tps_lattice", 2);
}

extern "C" int fi_tps_y_bounds(const double* py, int npts, double* y_pmax, double* y_smin,
                               void* stream) {
  FI_REQUIRE(py && y_pmax && y_smin && npts > 0, "fi_tps_y_bounds: bad arguments");
  const int nt = (npts + YB_TILE - 1) / YB_TILE;
  k_y_tiles<<<nt, YB_TILE, 0, (cudaStream_t)stream>>>(py, npts, y_pmax, y_smin, nullptr);
  k_y_tiles_scan<<<1, 1024, 0, (cudaStream_t)stream>>>(nt, y_pmax, y_smin);
  return check_launch("fi_tps_y_bounds", 2);
}

extern "C" int fi_tps_offsets(const int32_t* counts, const int32_t* ncounts, int nb_subdom,
                              int64_t* offsets, int64_t* noffsets, int64_t* mat_offsets,
                              int64_t* w_offsets, int64_t* summary, int32_t* order,
                              void* stream) {
  FI_REQUIRE(counts && ncounts && offsets && noffsets && mat_offsets && w_offsets && summary &&
                 nb_subdom > 0,
             "fi_tps_offsets: bad arguments");
  k_tps_offsets<<<1, 1024, 0, (cudaStream_t)stream>>>(counts, ncounts, nb_subdom, offsets,
                                                      noffsets, mat_offsets, w_offsets, summary,
                                                      order, nullptr);
  return check_launch("fi_tps_offsets");
}

extern "C" int fi_tps_members(const fi_tps_plan* plan, int nb_subdom, const double* px,
                              const double* py, int npts, int mode, int32_t* counts,
                              const int64_t* offsets, int32_t* indices, double* coefs,
                              const int32_t* xy2, const int32_t* on_lattice,
                              const double* y_pmax, const double* y_smin, void* stream) {
  FI_REQUIRE(plan && px && py && nb_subdom > 0 && npts > 0, "fi_tps_members: bad arguments");
  FI_REQUIRE(mode == 0 ? counts != nullptr : (offsets && indices && coefs),
             "fi_tps_members: missing outputs");
  FI_REQUIRE(((uintptr_t)xy2 & 7) == 0, "fi_tps_members: xy2 must be 8-byte aligned");
  k_tps_members<<<nb_subdom, 512, 0, (cudaStream_t)stream>>>(plan, px, py, npts, mode, counts,
                                                            offsets, indices, coefs, xy2,
                                                            on_lattice, y_pmax, y_smin, 0, 0);
  return check_launch("fi_tps_members");
}

extern "C" int fi_tps_layout(const fi_tps_plan* plan, int nb_subdom, const double* cx,
                             const double* cy, int num_centers, const double* px,
                             const double* py, int npts, int p_given, int32_t* cxy2,
                             int32_t* clat, int32_t* pxy2, int32_t* plat, double* cbounds,
                             double* pbounds, int32_t* counts, int32_t* ncounts,
                             int64_t* offsets, int32_t* order, void* stream) {
  FI_REQUIRE(plan && cx && cy && px && py && cxy2 && clat && pxy2 && plat && cbounds &&
                 pbounds && counts && ncounts && offsets && nb_subdom > 0 &&
                 num_centers > 0 && npts > 0,
             "fi_tps_layout: bad arguments");
  FI_REQUIRE(((uintptr_t)cxy2 & 7) == 0 && ((uintptr_t)pxy2 & 7) == 0,
             "fi_tps_layout: xy2 must be 8-byte aligned");
  // nb_subdom and num_centers are capacities: the kernels take the plan's counts
  cudaStream_t s = (cudaStream_t)stream;
  const int ctiles = (num_centers + YB_TILE - 1) / YB_TILE;
  const int ptiles = (npts + YB_TILE - 1) / YB_TILE;
  k_set_int<<<1, 1, 0, s>>>(clat, 1);
  k_tps_lattice<<<ctiles, 256, 0, s>>>(cx, cy, num_centers, cxy2, clat, plan);
  int launched = 2;
  if (!p_given) {
    k_set_int<<<1, 1, 0, s>>>(plat, 1);
    k_tps_lattice<<<ptiles, 256, 0, s>>>(px, py, npts, pxy2, plat, nullptr);
    launched += 2;
  }
  k_y_tiles<<<ctiles, YB_TILE, 0, s>>>(cy, num_centers, cbounds, cbounds + ctiles, plan);
  k_y_tiles_scan<<<1, 1024, 0, s>>>(ctiles, cbounds, cbounds + ctiles);
  k_y_tiles<<<ptiles, YB_TILE, 0, s>>>(py, npts, pbounds, pbounds + ptiles, nullptr);
  k_y_tiles_scan<<<1, 1024, 0, s>>>(ptiles, pbounds, pbounds + ptiles);
  k_tps_members<<<nb_subdom, 512, 0, s>>>(plan, cx, cy, num_centers, 0, counts, nullptr, nullptr,
                                          nullptr, cxy2, clat, cbounds, cbounds + ctiles, 1, 1);
  k_tps_members<<<nb_subdom, 512, 0, s>>>(plan, px, py, npts, 0, ncounts, nullptr, nullptr,
                                          nullptr, pxy2, plat, pbounds, pbounds + ptiles, 1, 0);
  k_tps_offsets<<<1, 1024, 0, s>>>(counts, ncounts, nb_subdom, offsets, offsets + nb_subdom,
                                   offsets + 2 * nb_subdom, offsets + 3 * nb_subdom,
                                   offsets + 4 * nb_subdom, order, plan);
  return check_launch("fi_tps_layout", launched + 7);
}

extern "C" int fi_tps_members_fill(const fi_tps_plan* plan, int nb_subdom, const double* cx,
                                   const double* cy, int num_centers, const double* px,
                                   const double* py, int npts, const int32_t* cxy2,
                                   const int32_t* clat, const int32_t* pxy2,
                                   const int32_t* plat, const double* cbounds,
                                   const double* pbounds, const int64_t* offsets,
                                   int32_t* indices, double* coefs, int32_t* nindices,
                                   double* ncoefs, void* stream) {
  FI_REQUIRE(plan && cx && cy && px && py && cbounds && pbounds && offsets && indices &&
                 coefs && nindices && ncoefs && nb_subdom > 0 && num_centers > 0 && npts > 0,
             "fi_tps_members_fill: bad arguments");
  FI_REQUIRE(((uintptr_t)cxy2 & 7) == 0 && ((uintptr_t)pxy2 & 7) == 0,
             "fi_tps_members_fill: xy2 must be 8-byte aligned");
  // the capacities of fi_tps_layout: the kernels take the plan's counts
  cudaStream_t s = (cudaStream_t)stream;
  const int ctiles = (num_centers + YB_TILE - 1) / YB_TILE;
  const int ptiles = (npts + YB_TILE - 1) / YB_TILE;
  k_tps_members<<<nb_subdom, 512, 0, s>>>(plan, cx, cy, num_centers, 1, nullptr, offsets,
                                          indices, coefs, cxy2, clat, cbounds, cbounds + ctiles,
                                          1, 1);
  k_tps_members<<<nb_subdom, 512, 0, s>>>(plan, px, py, npts, 1, nullptr, offsets + nb_subdom,
                                          nindices, ncoefs, pxy2, plat, pbounds,
                                          pbounds + ptiles, 1, 0);
  return check_launch("fi_tps_members_fill", 2);
}

extern "C" int fi_tps_solve(const fi_tps_plan* plan, int nb_subdom, int max_members,
                            const double* cx, const double* cy, const float* ux,
                            const float* uy, const int32_t* counts, const int64_t* offsets,
                            const int32_t* indices, const int64_t* mat_offsets, double* matrices,
                            int32_t* pivots, double threshold, int use_threshold,
                            const int64_t* w_offsets, double* weights, double* smoothed_x,
                            double* smoothed_y, int32_t* iters, int32_t* nfixed,
                            int32_t* singular, double* max_udiff, const int32_t* only_failed,
                            void* stream) {
  FI_REQUIRE(plan && counts && offsets && indices && mat_offsets && matrices && pivots &&
                 w_offsets && weights && smoothed_x && smoothed_y && iters && nfixed &&
                 singular && max_udiff,
             "fi_tps_solve: null pointer");
  FI_REQUIRE(nb_subdom > 0, "fi_tps_solve: no subdomain");
  const size_t smem = (size_t)(max_members + 3) * sizeof(double) + (size_t)max_members * 4 + 16;
  FI_REQUIRE(smem <= 200 * 1024, "fi_tps_solve: subdomain of %d vectors too large", max_members);
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(k_tps_solve, smem, limit));
  k_tps_solve<<<nb_subdom, 512, smem, (cudaStream_t)stream>>>(
      plan, cx, cy, ux, uy, counts, offsets, indices, mat_offsets, matrices, pivots, threshold,
      use_threshold, w_offsets, weights, smoothed_x, smoothed_y, iters, nfixed, singular,
      max_udiff, only_failed);
  return check_launch("fi_tps_solve");
}

extern "C" int fi_tps_blend_centers(const fi_tps_plan* plan, int num_centers, const double* cx,
                                    const double* cy, const int32_t* counts,
                                    const int64_t* offsets, const int32_t* indices,
                                    const double* coefs, const double* smoothed_x,
                                    const double* smoothed_y, double* out_x, double* out_y,
                                    void* stream) {
  FI_REQUIRE(plan && cx && cy && counts && offsets && indices && coefs && out_x && out_y,
             "fi_tps_blend_centers: null pointer");
  if (num_centers <= 0) return FI_OK;
  const int threads = 256;
  k_tps_blend_centers<<<(num_centers + threads - 1) / threads, threads, 0, (cudaStream_t)stream>>>(
      plan, cx, cy, counts, offsets, indices, coefs, smoothed_x, smoothed_y, out_x, out_y);
  return check_launch("fi_tps_blend_centers");
}

// The *_smooth fields of the last pass (singlepass.py:515-529).  First the final grid:
// its positions (px + offx, py + offy rounded to float32) and the interpolated field.
__global__ void k_smooth_grid(const double* __restrict__ px, const double* __restrict__ py,
                              int npts, double offx, double offy,
                              const double* __restrict__ out_x,
                              const double* __restrict__ out_y, float* xs_s, float* ys_s,
                              double* dx_s, double* dy_s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x) {
    xs_s[i] = __double2float_rn(__dadd_rn(px[i], offx));
    ys_s[i] = __double2float_rn(__dadd_rn(py[i], offy));
    dx_s[i] = out_x[i];
    dy_s[i] = out_y[i];
  }
}

// Then, at the selected vectors (sel[k]: their index on the grid), their own positions
// (the pass's xs / ys when vec_xy, else the grid's) and their smoothed values.
__global__ void k_smooth_sel(const int32_t* __restrict__ sel, int n_sel,
                             const double* __restrict__ px, const double* __restrict__ py,
                             const float* __restrict__ xs, const float* __restrict__ ys,
                             int npts, int vec_xy, double offx, double offy,
                             const double* __restrict__ smooth_x,
                             const double* __restrict__ smooth_y, float* xs_s, float* ys_s,
                             double* dx_s, double* dy_s) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_sel; k += gridDim.x * blockDim.x) {
    const int i = sel[k];
    if (i < 0 || i >= npts) continue;
    const double x = vec_xy ? (double)xs[i] : px[i];
    const double y = vec_xy ? (double)ys[i] : py[i];
    xs_s[i] = __double2float_rn(__dadd_rn(x, offx));
    ys_s[i] = __double2float_rn(__dadd_rn(y, offy));
    dx_s[i] = smooth_x[k];
    dy_s[i] = smooth_y[k];
  }
}

extern "C" int fi_tps_smooth_fields(const double* px, const double* py, int npts, const float* xs,
                                    const float* ys, int vec_xy, double offx, double offy,
                                    const int32_t* sel, int n_sel, const double* out_x,
                                    const double* out_y, const double* smooth_x,
                                    const double* smooth_y, float* xs_s, float* ys_s,
                                    double* dx_s, double* dy_s, void* stream) {
  FI_REQUIRE(px && py && out_x && out_y && xs_s && ys_s && dx_s && dy_s && npts > 0,
             "fi_tps_smooth_fields: bad arguments");
  FI_REQUIRE(n_sel >= 0 && (n_sel == 0 || (sel && smooth_x && smooth_y)) &&
                 (!vec_xy || (xs && ys)),
             "fi_tps_smooth_fields: bad selection arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 256;
  const int gb = (npts + threads - 1) / threads;
  k_smooth_grid<<<gb < 1024 ? gb : 1024, threads, 0, s>>>(px, py, npts, offx, offy, out_x, out_y,
                                                          xs_s, ys_s, dx_s, dy_s);
  int launched = 1;
  if (n_sel > 0) {
    const int sb = (n_sel + threads - 1) / threads;
    k_smooth_sel<<<sb < 1024 ? sb : 1024, threads, 0, s>>>(sel, n_sel, px, py, xs, ys, npts,
                                                           vec_xy, offx, offy, smooth_x,
                                                           smooth_y, xs_s, ys_s, dx_s, dy_s);
    ++launched;
  }
  return check_launch("fi_tps_smooth_fields", launched);
}

extern "C" int fi_tps_interpolate(const fi_tps_plan* plan, int nb_subdom, int max_members,
                                  int max_new_members, const double* cx, const double* cy,
                                  const int32_t* counts, const int64_t* offsets,
                                  const int32_t* indices, const int64_t* w_offsets,
                                  const double* weights, const double* px, const double* py,
                                  int npts, const int32_t* ncounts, const int64_t* noffsets,
                                  const int32_t* nindices, const double* ncoefs, double* partx,
                                  double* party, double* out_x, double* out_y, int32_t* out_rx,
                                  int32_t* out_ry, const double* phi_table,
                                  const float* phi_table2, int64_t table_size,
                                  const int32_t* cxy2, const int32_t* c_on_lattice,
                                  int table_entries, void* stream) {
  FI_REQUIRE(plan && cx && cy && counts && offsets && indices && w_offsets && weights && px &&
                 py && ncounts && noffsets && nindices && ncoefs && partx && party && out_x &&
                 out_y,
             "fi_tps_interpolate: null pointer");
  FI_REQUIRE(nb_subdom > 0 && npts > 0, "fi_tps_interpolate: bad sizes");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t base = (size_t)(4 * max_members + 6) * sizeof(double) +
                      (size_t)max_members * sizeof(int2) +
                      (size_t)2 * max_members * sizeof(float2);
  FI_REQUIRE(base <= 200 * 1024, "fi_tps_interpolate: subdomain of %d vectors too large",
             max_members);
  // the grid-offset table (at least EVAL_TABLE entries) where it fits beside the
  // subdomain's centres
  FI_REQUIRE(table_entries >= 0 && table_entries <= 16384,
             "fi_tps_interpolate: table_entries %d out of [0, 16384]", table_entries);
  const int want = table_entries > EVAL_TABLE ? table_entries : EVAL_TABLE;
  const int tab_cap = base + (size_t)want * sizeof(float2) <= 200 * 1024 ? want : 0;
  const size_t smem = base + (size_t)tab_cap * sizeof(float2);
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(k_tps_eval, smem, limit));
  if (max_new_members > 0) {
    const int threads = 256;
    dim3 grid((max_new_members + threads - 1) / threads, nb_subdom);
    k_tps_eval<<<grid, threads, smem, s>>>(
        counts, offsets, indices, w_offsets, weights, cx, cy, ncounts, noffsets, nindices, ncoefs,
        px, py, partx, party, phi_table, reinterpret_cast<const float2*>(phi_table2), table_size,
        cxy2, c_on_lattice, max_members, tab_cap);
    add_launches(1);
  }
  const int threads = 256;
  k_tps_gather<<<(npts + threads - 1) / threads, threads, 0, s>>>(
      plan, ncounts, noffsets, nindices, ncoefs, partx, party, px, py, npts, out_x, out_y, out_rx,
      out_ry);
  return check_launch("fi_tps_interpolate");
}
