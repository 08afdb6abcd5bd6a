// Mixed-precision solver of the smoothed TPS subdomain systems.
//
// Upstream (calcul/interpolate/thin_plate_spline.py:168-216,
// thin_plate_spline_subdom.py:236-280) solves [[K + lam I, P], [P^T, 0]] [w; a] =
// [u; 0] with LAPACK gesv in FP64, for x and y and again after each outlier
// replacement.  That saddle-point matrix has condition numbers ~1e13-1e15, but its
// null-space form is benign: with P = Q [R; 0] (Householder, Q = H1 H2 H3),
// w = Q2 z and
//     B z = Q2^T u,   B = Q2^T (K + lam I) Q2   (SPD, cond ~1e4 for lam > 0),
//     a = R^-1 (Q1^T u - Q1^T (K + lam I) w),   smoothed = u - lam w.
// On this GPU FP32 runs 73x faster than FP64, so B (projected in FP64) is rounded
// to FP32 and factorised there (blocked Cholesky, ~N^3/6 flops), and the solution
// is refined with FP64 residuals t = u - (K + lam I) w (2 N^2 FP64 flops per step
// for both components, a few steps).  Refinement stops when the correction is below
// 1e-10 of the solution (the error then is ~1e-15 relative after the FP32 solve's
// ~1e-5 contraction), or stagnates below 1e-9; a subdomain that does not
// converge (or whose P has rank < 3, or whose Cholesky meets a non-positive pivot)
// is flagged and re-solved by the FP64 LU kernel (k_tps_solve).
//
// K entries come from a table of phi(r^2) = r^2 log(r^2) / 2 indexed by 4 r^2,
// exact for window centres on the half-integer lattice (the integer window shifts
// put every PIV vector there); other distances use log() directly.
#include <cmath>

#include "fi_common.cuh"

namespace fi {

// ------------------------------------------------------------------ phi
__device__ __forceinline__ double phi_direct(double r2) {
  if (r2 == 0.0) return 0.0;
  return __ddiv_rn(__dmul_rn(r2, log(r2)), 2.0);
}

// phi(r^2) for the centre pair (a, b); table lookup when 4 r^2 is an integer in range.
__device__ __forceinline__ double phi_pair(double xa, double ya, double xb, double yb,
                                           const double* table, int64_t tsize) {
  const double dy = __dsub_rn(ya, yb), dx = __dsub_rn(xa, xb);
  const double r2 = __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx));
  const double q = 4.0 * r2;
  if (table != nullptr && q < (double)tsize) {
    const int64_t k = (int64_t)q;
    if ((double)k == q) return __ldg(table + k);
  }
  return phi_direct(r2);
}

__global__ void k_phi_table(double* table, int64_t count) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count;
       k += (int64_t)gridDim.x * blockDim.x)
    table[k] = phi_direct((double)k * 0.25);
}

// ------------------------------------------------------------------ block helpers
template <int NT>
__device__ __forceinline__ double bsum(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < NT / 32 ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[32] = v;
  }
  __syncthreads();
  v = sh[32];
  __syncthreads();
  return v;
}

template <int NT>
__device__ __forceinline__ double2 bsum2(double2 v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  if (lane == 0) {
    sh[2 * wid] = v.x;
    sh[2 * wid + 1] = v.y;
  }
  __syncthreads();
  if (wid == 0) {
    v.x = lane < NT / 32 ? sh[2 * lane] : 0.0;
    v.y = lane < NT / 32 ? sh[2 * lane + 1] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) {
      sh[64] = v.x;
      sh[65] = v.y;
    }
  }
  __syncthreads();
  v.x = sh[64];
  v.y = sh[65];
  __syncthreads();
  return v;
}

template <int NT>
__device__ __forceinline__ double bmax(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < NT / 32 ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[32] = v;
  }
  __syncthreads();
  v = sh[32];
  __syncthreads();
  return v;
}

constexpr int MP_THREADS = 256;

// t = u - A w for two right-hand sides; A (n x n, symmetric, column-major) in FP64.
__device__ void residual2(const double* A, int n, const double* wx, const double* wy,
                          const float* ux, const float* uy, double* tx, double* ty) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = MP_THREADS / 32;
  for (int c = wid; c < n; c += nw) {
    const double* col = A + (int64_t)c * n;  // row c = column c
    double ax = 0.0, ay = 0.0, bx = 0.0, by = 0.0;
    int r = lane;
    for (; r + 96 < n; r += 128) {  // four independent loads in flight per lane
      const double a0 = col[r], a1 = col[r + 32], a2 = col[r + 64], a3 = col[r + 96];
      ax = fma(a0, wx[r], ax);
      ay = fma(a0, wy[r], ay);
      bx = fma(a1, wx[r + 32], bx);
      by = fma(a1, wy[r + 32], by);
      ax = fma(a2, wx[r + 64], ax);
      ay = fma(a2, wy[r + 64], ay);
      bx = fma(a3, wx[r + 96], bx);
      by = fma(a3, wy[r + 96], by);
    }
    for (; r < n; r += 32) {
      const double a = col[r];
      ax = fma(a, wx[r], ax);
      ay = fma(a, wy[r], ay);
    }
    ax += bx;
    ay += by;
    for (int o = 16; o > 0; o >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, o);
      ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    if (lane == 0) {
      tx[c] = (double)ux[c] - ax;
      ty[c] = (double)uy[c] - ay;
    }
  }
  __syncthreads();
}

// Apply H_k = I - tau_k v_k v_k^T (k in order) to the two vectors x, y (length n).
template <bool REVERSE>
__device__ void apply_reflectors2(const double* V, const double* tau, int n, double* x,
                                  double* y, double* sh) {
  for (int kk = 0; kk < 3; ++kk) {
    const int k = REVERSE ? 2 - kk : kk;
    const double* v = V + (int64_t)k * n;
    double2 d = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < n; i += MP_THREADS) {
      d.x += v[i] * x[i];
      d.y += v[i] * y[i];
    }
    d = bsum2<MP_THREADS>(d, sh);
    const double cx = tau[k] * d.x, cy = tau[k] * d.y;
    for (int i = threadIdx.x; i < n; i += MP_THREADS) {
      x[i] -= cx * v[i];
      y[i] -= cy * v[i];
    }
    __syncthreads();
  }
}

// Solve (L L^T) x = r in place for two right-hand sides (float), L lower m x m,
// column-major with leading dimension ld, by tiles of 32: the diagonal tile in one
// warp (shuffles), the off-diagonal tiles by all warps (rows in registers for the
// forward sweep, transposed shared-memory tiles for the backward sweep).
// scratch: (1 + warps) * 32 * 33 floats.
__device__ void chol_solve2(const float* L, int m, int ld, float* rx, float* ry,
                            float* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = MP_THREADS / 32;
  const unsigned full = 0xffffffffu;
  const int T = (m + 31) / 32;
  float* part = scratch;                       // [warp][64] partial sums (backward)
  float* Lt = scratch + 32 * 33 * (1 + wid);   // per warp transposed tile
  // ---- forward: L y = r
  for (int k = 0; k < T; ++k) {
    const int r0 = 32 * k;
    if (wid == 0) {
      float Lrow[32];  // row (r0 + lane) of the diagonal tile
      const int r = r0 + lane;
#pragma unroll
      for (int c = 0; c < 32; ++c)
        Lrow[c] = (r < m && r0 + c < m) ? L[(int64_t)(r0 + c) * ld + r] : ((c == lane) ? 1.f : 0.f);
      float vx = (r < m) ? rx[r] : 0.f, vy = (r < m) ? ry[r] : 0.f;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const float d = __shfl_sync(full, Lrow[j], j);
        const float xj = __shfl_sync(full, vx, j) / d;
        const float yj = __shfl_sync(full, vy, j) / d;
        if (lane == j) {
          vx = xj;
          vy = yj;
        } else if (lane > j) {
          vx = fmaf(-Lrow[j], xj, vx);
          vy = fmaf(-Lrow[j], yj, vy);
        }
      }
      if (r < m) {
        rx[r] = vx;
        ry[r] = vy;
      }
    }
    __syncthreads();
    for (int i = k + 1 + wid; i < T; i += nw) {  // r_i -= L_ik y_k
      const int r = 32 * i + lane;
      if (r < m) {
        float sx = 0.f, sy = 0.f;
#pragma unroll 8
        for (int c = 0; c < 32; ++c) {
          if (r0 + c < m) {
            const float l = L[(int64_t)(r0 + c) * ld + r];
            sx = fmaf(l, rx[r0 + c], sx);
            sy = fmaf(l, ry[r0 + c], sy);
          }
        }
        rx[r] -= sx;
        ry[r] -= sy;
      }
    }
    __syncthreads();
  }
  // ---- backward: L^T x = y
  for (int k = T - 1; k >= 0; --k) {
    const int c0 = 32 * k;
    float px = 0.f, py = 0.f;  // lane t: partial of sum_{i>k} sum_r L_ik[r][t] x_i[r]
    for (int i = k + 1 + wid; i < T; i += nw) {
      const int r = 32 * i + lane;
#pragma unroll
      for (int t = 0; t < 32; ++t)
        Lt[t * 33 + lane] = (r < m && c0 + t < m) ? L[(int64_t)(c0 + t) * ld + r] : 0.f;
      __syncwarp();
#pragma unroll 8
      for (int rr = 0; rr < 32; ++rr) {
        const int ri = 32 * i + rr;
        const float xv = (ri < m) ? rx[ri] : 0.f, yv = (ri < m) ? ry[ri] : 0.f;
        const float l = Lt[lane * 33 + rr];
        px = fmaf(l, xv, px);
        py = fmaf(l, yv, py);
      }
      __syncwarp();
    }
    part[wid * 64 + lane] = px;
    part[wid * 64 + 32 + lane] = py;
    __syncthreads();
    if (wid == 0) {
      const int t = c0 + lane;
      float vx = (t < m) ? rx[t] : 0.f, vy = (t < m) ? ry[t] : 0.f;
      for (int w = 0; w < nw; ++w) {
        vx -= part[w * 64 + lane];
        vy -= part[w * 64 + 32 + lane];
      }
      float Lcol[32];  // column (c0 + lane) of the diagonal tile: Lcol[j] = L[c0 + j][c0 + lane]
#pragma unroll
      for (int j = 0; j < 32; ++j)
        Lcol[j] = (t < m && c0 + j < m) ? L[(int64_t)t * ld + c0 + j] : ((j == lane) ? 1.f : 0.f);
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        const float d = __shfl_sync(full, Lcol[j], j);
        const float xj = __shfl_sync(full, vx, j) / d;
        const float yj = __shfl_sync(full, vy, j) / d;
        if (lane == j) {
          vx = xj;
          vy = yj;
        } else if (lane < j) {
          vx = fmaf(-Lcol[j], xj, vx);
          vy = fmaf(-Lcol[j], yj, vy);
        }
      }
      if (t < m) {
        rx[t] = vx;
        ry[t] = vy;
      }
    }
    __syncthreads();
  }
}

// Tiles of 32 x 32 held in registers, one row per lane (a[c] = element (r, c) of
// the tile, r = lane); rows/columns beyond m read as the identity.
__device__ __forceinline__ void tile_load(const float* B, int m, int ld, int ti, int tj,
                                          float (&a)[32], int lane) {
  const int r = 32 * ti + lane;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const int col = 32 * tj + c;
    a[c] = (r < m && col < m) ? B[(int64_t)col * ld + r] : ((r == col) ? 1.f : 0.f);
  }
}
__device__ __forceinline__ void tile_store(float* B, int m, int ld, int ti, int tj,
                                           const float (&a)[32], int lane, bool lower_only) {
  const int r = 32 * ti + lane;
  if (r >= m) return;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const int col = 32 * tj + c;
    if (col < m && (!lower_only || c <= lane)) B[(int64_t)col * ld + r] = a[c];
  }
}

// Right-looking tiled Cholesky (lower) of the m x m matrix B (column-major, ld), in
// place.  Per tile column k: one warp factorises the diagonal tile in registers
// (shuffles), warps solve the tiles below (one row per lane, L_kk broadcast from
// shared memory), then update the trailing tile pairs (register accumulators,
// the second factor transposed in shared memory and read as broadcasts).
// scratch: (1 + warps) * 32 * 33 floats.  Returns false on a non-positive pivot.
__device__ bool chol_factor(float* B, int m, int ld, float* scratch, int* s_flag) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = MP_THREADS / 32;
  const unsigned full = 0xffffffffu;
  const int T = (m + 31) / 32;
  float* Lkk = scratch;                       // 32 x 33
  float* Lt = scratch + 32 * 33 * (1 + wid);  // per warp, 32 x 33 (transposed tile)
  if (threadIdx.x == 0) *s_flag = 0;
  __syncthreads();
  for (int k = 0; k < T; ++k) {
    if (wid == 0) {  // POTRF of tile (k, k)
      float a[32];
      tile_load(B, m, ld, k, k, a, lane);
      bool bad = false;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        float djj = __shfl_sync(full, a[j], j);
        if (!(djj > 0.f)) {
          bad = true;
          djj = 1.f;
        }
        const float sq = sqrtf(djj);
        const float lrj = (lane > j) ? a[j] / sq : ((lane == j) ? sq : 0.f);
        if (lane >= j) a[j] = lrj;
#pragma unroll
        for (int c = j + 1; c < 32; ++c) {
          const float lcj = __shfl_sync(full, lrj, c);
          if (lane >= c) a[c] = fmaf(-lrj, lcj, a[c]);
        }
      }
      if (bad && lane == 0) *s_flag = 1;
      tile_store(B, m, ld, k, k, a, lane, true);
#pragma unroll
      for (int c = 0; c < 32; ++c) Lkk[lane * 33 + c] = (c <= lane) ? a[c] : 0.f;
    }
    __syncthreads();
    // TRSM: tiles (i, k), i > k: X L_kk^T = A_ik, row by row in each lane
    for (int i = k + 1 + wid; i < T; i += nw) {
      float b[32];
      tile_load(B, m, ld, i, k, b, lane);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        float v = b[j];
#pragma unroll
        for (int c = 0; c < j; ++c) v = fmaf(-b[c], Lkk[j * 33 + c], v);
        b[j] = v / Lkk[j * 33 + j];
      }
      tile_store(B, m, ld, i, k, b, lane, false);
    }
    __syncthreads();
    // trailing update: tiles (i, j), k < j <= i
    const int n = T - k - 1;
    const int npairs = n * (n + 1) / 2;
    for (int pidx = wid; pidx < npairs; pidx += nw) {
      int ii = (int)((sqrtf(8.f * pidx + 1.f) - 1.f) * 0.5f);
      while ((ii + 1) * (ii + 2) / 2 <= pidx) ++ii;
      while (ii * (ii + 1) / 2 > pidx) --ii;
      const int jj = pidx - ii * (ii + 1) / 2;
      const int i = k + 1 + ii, j = k + 1 + jj;
      float l[32];
      tile_load(B, m, ld, j, k, l, lane);  // L_jk rows -> transposed in shared memory
#pragma unroll
      for (int t = 0; t < 32; ++t) Lt[t * 33 + lane] = l[t];
      __syncwarp();
      if (i != j) tile_load(B, m, ld, i, k, l, lane);  // L_ik rows
      float acc[32];
      tile_load(B, m, ld, i, j, acc, lane);
#pragma unroll
      for (int t = 0; t < 32; ++t) {
        const float lr = l[t];
#pragma unroll
        for (int c = 0; c < 32; ++c) acc[c] = fmaf(-lr, Lt[t * 33 + c], acc[c]);
      }
      tile_store(B, m, ld, i, j, acc, lane, i == j);
      __syncwarp();
    }
    __syncthreads();
  }
  return *s_flag == 0;
}

// One block per subdomain.  Status per subdomain: 0 solved here, 1 needs the FP64
// LU fallback (rank-deficient P, Cholesky breakdown or no convergence).
__global__ void __launch_bounds__(MP_THREADS, 2)
    k_tps_solve_mp(const fi_tps_plan* plan_ptr, const double* cx, const double* cy,
                   const float* ux, const float* uy, const int32_t* counts,
                   const int64_t* offsets, const int32_t* indices, const int64_t* mat_off,
                   double* matrices, float* matrices32, const double* phi_table,
                   int64_t table_size, const int32_t* cxy2, const int32_t* c_on_lattice,
                   double threshold, int use_threshold,
                   const int64_t* w_off, double* weights, double* smoothed_x,
                   double* smoothed_y, int32_t* iters, int32_t* nfixed, int32_t* status,
                   double* max_udiff, int max_refine) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sh[80];
  __shared__ double s_tau[3];
  __shared__ double s_R[9];
  __shared__ int s_flag, s_bad[2];
  const fi_tps_plan p = *plan_ptr;
  const int sd = blockIdx.x;
  const int N = counts[sd];
  const int m = N - 3;
  const int64_t off = offsets[sd];
  const int32_t* idx = indices + off;
  const double lam = p.smoothing;
  if (threadIdx.x == 0) status[sd] = 1;
  if (m < 1) return;  // fewer than 4 centres: FP64 LU path

  // shared layout (doubles first)
  double* V = reinterpret_cast<double*>(smraw);  // 3 N
  double* xc = V + 3 * N;                         // N
  double* yc = xc + N;                            // N
  double* wx = yc + N;                            // N  (weights w, then scratch)
  double* wy = wx + N;
  double* tx = wy + N;                            // N  (residual / projections)
  double* ty = tx + N;
  double* zx = ty + N;                            // m (+3 padding)
  double* zy = zx + N;
  float* vx = reinterpret_cast<float*>(zy + N);  // N current values (float32)
  float* vy = vx + N;
  float* rx = vy + N;                             // m correction (float)
  float* ry = rx + N;
  float* panel = ry + N;  // Cholesky / solve scratch: (1 + warps) * 32 * 33 floats

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = MP_THREADS / 32;
  const double* A64 = matrices + mat_off[sd];  // N x N, K + lam I (kept for residuals)
  float* B = matrices32 + mat_off[sd];         // N x N float (lower triangle of B22 used)
  __shared__ int s_lat;
  int2* cxy = reinterpret_cast<int2*>(panel);  // lattice coordinates (panel is free here)

  if (threadIdx.x == 0)
    s_lat = (cxy2 != nullptr && c_on_lattice != nullptr && phi_table != nullptr) ? *c_on_lattice : 0;
  for (int i = threadIdx.x; i < N; i += MP_THREADS) {
    const int a = idx[i];
    xc[i] = cx[a];
    yc[i] = cy[a];
    if (cxy2 != nullptr) cxy[i] = make_int2(cxy2[2 * a], cxy2[2 * a + 1]);
  }
  __syncthreads();
  // ---- Householder QR of P = [1, y, x] (FP64), V rows k hold v_k (zeros above k)
  {
    double* P0 = tx;  // scratch columns
    double* P1 = ty;
    double* P2 = wx;
    for (int i = threadIdx.x; i < N; i += MP_THREADS) {
      P0[i] = 1.0;
      P1[i] = yc[i];
      P2[i] = xc[i];
    }
    __syncthreads();
    double* cols[3] = {P0, P1, P2};
    bool rank_ok = true;
    for (int k = 0; k < 3; ++k) {
      double* x = cols[k];
      double nrm2 = 0.0;
      for (int i = k + threadIdx.x; i < N; i += MP_THREADS) nrm2 += x[i] * x[i];
      nrm2 = bsum<MP_THREADS>(nrm2, sh);
      const double x0 = x[k];
      const double nrm = sqrt(nrm2);
      if (!(nrm > 0.0)) {
        rank_ok = false;
        break;
      }
      const double alpha = (x0 >= 0.0) ? -nrm : nrm;
      double* v = V + (int64_t)k * N;
      for (int i = threadIdx.x; i < N; i += MP_THREADS) v[i] = (i < k) ? 0.0 : x[i];
      __syncthreads();
      if (threadIdx.x == 0) v[k] = x0 - alpha;
      __syncthreads();
      double vv = 0.0;
      for (int i = k + threadIdx.x; i < N; i += MP_THREADS) vv += v[i] * v[i];
      vv = bsum<MP_THREADS>(vv, sh);
      if (!(vv > 0.0)) {
        rank_ok = false;
        break;
      }
      const double tau = 2.0 / vv;
      if (threadIdx.x == 0) {
        s_tau[k] = tau;
        s_R[k * 3 + k] = alpha;
      }
      for (int j = k + 1; j < 3; ++j) {  // apply H_k to the remaining columns
        double* y = cols[j];
        double d = 0.0;
        for (int i = k + threadIdx.x; i < N; i += MP_THREADS) d += v[i] * y[i];
        d = bsum<MP_THREADS>(d, sh);
        for (int i = k + threadIdx.x; i < N; i += MP_THREADS) y[i] -= tau * d * v[i];
        __syncthreads();
        if (threadIdx.x == 0) s_R[k * 3 + j] = y[k];
        __syncthreads();
      }
      if (fabs(alpha) < 1e-9 * sqrt((double)N)) rank_ok = false;  // collinear centres
    }
    __syncthreads();
    if (!rank_ok) return;
  }
  __syncthreads();
  // ---- A = K + lam I in FP64 (column-major; on the lattice 4 r^2 in integers),
  // fused with Y = A V for the projection (A symmetric: row c = column c)
  double* Y0 = tx;
  double* Y1 = ty;
  double* Y2 = wx;
  {
    const double* V0 = V;
    const double* V1 = V + N;
    const double* V2 = V + 2 * (int64_t)N;
    for (int c = wid; c < N; c += nw) {
      const double bx = xc[c], by = yc[c];
      const int2 cb = cxy[c];
      double* col = matrices + mat_off[sd] + (int64_t)c * N;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
      for (int r = lane; r < N; r += 32) {
        double v;
        if (r == c) {
          v = lam;
        } else if (s_lat) {
          const int2 ca = cxy[r];
          const int64_t dx = (int64_t)(ca.x - cb.x), dy = (int64_t)(ca.y - cb.y);
          const int64_t kq = dy * dy + dx * dx;
          v = (kq < table_size) ? __ldg(phi_table + kq)
                                : phi_pair(xc[r], yc[r], bx, by, nullptr, 0);
        } else {
          v = phi_pair(xc[r], yc[r], bx, by, phi_table, table_size);
        }
        col[r] = v;
        a0 = fma(v, V0[r], a0);
        a1 = fma(v, V1[r], a1);
        a2 = fma(v, V2[r], a2);
      }
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      }
      if (lane == 0) {
        Y0[c] = a0;
        Y1[c] = a1;
        Y2[c] = a2;
      }
    }
  }
  __syncthreads();
  // ---- B22 = (Q^T A Q)[3:, 3:] with Q = H0 H1 H2 = I - V T V^T (compact WY):
  // Q^T A Q = A - Z V^T - V Z^T, Y = A V, M = T^T (V^T Y) T, Z = Y T - V M / 2.
  // FP64 (the projection cancels the large affine part of K); only the lower
  // triangle of B22 is formed, directly in FP32.
  {
    __shared__ double s_T[9], s_M[9];
    double* Z0 = wy;
    double* Z1 = zx;
    double* Z2 = zy;
    const double* V0 = V;
    const double* V1 = V + N;
    const double* V2 = V + 2 * (int64_t)N;
    // V^T V (upper) and V^T Y (full), block sums
    const double* Vk[3] = {V0, V1, V2};
    const double* Yk[3] = {Y0, Y1, Y2};
    double vtv[3], vty[9];
    for (int a = 0; a < 3; ++a) {
      vtv[a] = 0.0;
      for (int b = 0; b < 3; ++b) vty[3 * a + b] = 0.0;
    }
    for (int i = threadIdx.x; i < N; i += MP_THREADS) {
      vtv[0] += V0[i] * V1[i];
      vtv[1] += V0[i] * V2[i];
      vtv[2] += V1[i] * V2[i];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) vty[3 * a + b] += Vk[a][i] * Yk[b][i];
    }
    for (int a = 0; a < 3; ++a) vtv[a] = bsum<MP_THREADS>(vtv[a], sh);
    for (int a = 0; a < 9; ++a) vty[a] = bsum<MP_THREADS>(vty[a], sh);
    if (threadIdx.x == 0) {
      double T[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      T[0] = s_tau[0];
      T[4] = s_tau[1];
      T[8] = s_tau[2];
      T[1] = -s_tau[1] * T[0] * vtv[0];                      // T[0][1]
      T[2] = -s_tau[2] * (T[0] * vtv[1] + T[1] * vtv[2]);    // T[0][2]
      T[5] = -s_tau[2] * (T[4] * vtv[2]);                    // T[1][2]
      double G[9];  // (V^T Y) T
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc += vty[3 * a + j] * T[3 * j + b];
          G[3 * a + b] = acc;
        }
      for (int a = 0; a < 3; ++a)  // M = T^T G
        for (int b = 0; b < 3; ++b) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc += T[3 * j + a] * G[3 * j + b];
          s_M[3 * a + b] = acc;
        }
      for (int a = 0; a < 9; ++a) s_T[a] = T[a];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += MP_THREADS) {  // Z = Y T - V M / 2
      const double y[3] = {Y0[i], Y1[i], Y2[i]};
      const double v[3] = {V0[i], V1[i], V2[i]};
      double z[3];
      for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc += y[j] * s_T[3 * j + k] - 0.5 * v[j] * s_M[3 * j + k];
        z[k] = acc;
      }
      Z0[i] = z[0];
      Z1[i] = z[1];
      Z2[i] = z[2];
    }
    __syncthreads();
    for (int c = 3 + wid; c < N; c += nw) {  // lower triangle of B22, rows r >= c
      const double* col = A64 + (int64_t)c * N;
      float* colb = B + (int64_t)c * N;
      const double vc0 = V0[c], vc1 = V1[c], vc2 = V2[c];
      const double zc0 = Z0[c], zc1 = Z1[c], zc2 = Z2[c];
      for (int r = c + lane; r < N; r += 32) {
        double v = col[r];
        v -= Z0[r] * vc0 + V0[r] * zc0;
        v -= Z1[r] * vc1 + V1[r] * zc1;
        v -= Z2[r] * vc2 + V2[r] * zc2;
        colb[r] = (float)v;
      }
    }
    __syncthreads();
  }
  // ---- FP32 Cholesky of B22 = B[3:, 3:]
  float* B22 = B + 3 + 3 * (int64_t)N;
  if (!chol_factor(B22, m, N, panel, &s_flag)) return;

  // ---- outlier iterations with refined solves (x and y in lockstep)
  for (int r = threadIdx.x; r < N; r += MP_THREADS) {
    vx[r] = ux[idx[r]];
    vy[r] = uy[idx[r]];
  }
  for (int r = threadIdx.x; r < N; r += MP_THREADS) zx[r] = zy[r] = 0.0;
  __syncthreads();
  int count[2] = {1, 1}, fixed[2] = {0, 0};
  bool done[2] = {false, false};
  bool converged_all = true;
  bool first_solve = true;
  while (true) {
    // refine z for the current values
    bool conv = false;
    double prev = INFINITY;
    for (int it = 0; it < max_refine; ++it) {
      // w = Q [0; z]
      for (int i = threadIdx.x; i < N; i += MP_THREADS) {
        wx[i] = (i < 3) ? 0.0 : zx[i - 3];
        wy[i] = (i < 3) ? 0.0 : zy[i - 3];
      }
      __syncthreads();
      if (it == 0 && first_solve) {  // z = 0: t = u
        for (int i = threadIdx.x; i < N; i += MP_THREADS) {
          tx[i] = (double)vx[i];
          ty[i] = (double)vy[i];
        }
        __syncthreads();
      } else {
        apply_reflectors2<true>(V, s_tau, N, wx, wy, sh);
        residual2(A64, N, wx, wy, vx, vy, tx, ty);
      }
      // rho = (Q^T t)[3:]
      apply_reflectors2<false>(V, s_tau, N, tx, ty, sh);
      for (int i = threadIdx.x; i < m; i += MP_THREADS) {
        rx[i] = (float)tx[i + 3];
        ry[i] = (float)ty[i + 3];
      }
      __syncthreads();
      chol_solve2(B22, m, N, rx, ry, panel);
      double dmax = 0.0, zmax = 0.0;
      for (int i = threadIdx.x; i < m; i += MP_THREADS) {
        if (!done[0]) zx[i] += (double)rx[i];
        if (!done[1]) zy[i] += (double)ry[i];
        dmax = fmax(dmax, fmax(done[0] ? 0.0 : fabs((double)rx[i]),
                               done[1] ? 0.0 : fabs((double)ry[i])));
        zmax = fmax(zmax, fmax(fabs(zx[i]), fabs(zy[i])));
      }
      dmax = bmax<MP_THREADS>(dmax, sh);
      zmax = bmax<MP_THREADS>(zmax, sh);
      if (dmax == 0.0) {
        conv = true;
        break;
      }
      if (it >= 1) {
        // contraction of the FP32-preconditioned refinement, estimated from the last
        // two corrections; the remaining error is about contraction * dmax
        const double rho = dmax / prev;
        if (rho < 0.1 && rho * dmax <= 1e-13 * zmax) {
          conv = true;
          break;
        }
        if (it >= 2 && rho > 0.5) {  // at the FP64 residual floor
          conv = dmax <= 1e-9 * zmax;
          break;
        }
      }
      prev = dmax;
    }
    first_solve = false;
    if (!conv) {
      converged_all = false;
      break;
    }
    // final w, s = A w is in t before projection: recompute t = u - A w for a
    for (int i = threadIdx.x; i < N; i += MP_THREADS) {
      wx[i] = (i < 3) ? 0.0 : zx[i - 3];
      wy[i] = (i < 3) ? 0.0 : zy[i - 3];
    }
    __syncthreads();
    apply_reflectors2<true>(V, s_tau, N, wx, wy, sh);
    residual2(A64, N, wx, wy, vx, vy, tx, ty);
    // a = R^-1 (Q1^T (u - A w))
    apply_reflectors2<false>(V, s_tau, N, tx, ty, sh);
    double ax3[3], ay3[3];
    for (int k = 2; k >= 0; --k) {
      double sxk = tx[k], syk = ty[k];
      for (int j = k + 1; j < 3; ++j) {
        sxk -= s_R[k * 3 + j] * ax3[j];
        syk -= s_R[k * 3 + j] * ay3[j];
      }
      ax3[k] = sxk / s_R[k * 3 + k];
      ay3[k] = syk / s_R[k * 3 + k];
    }
    // smoothed = u - lam w; outlier test (compute_tps_weights_iter, subdom.py:236-280)
    if (threadIdx.x == 0) s_bad[0] = s_bad[1] = 0;
    __syncthreads();
    double mxx = 0.0, mxy = 0.0;
    int bx = 0, by = 0;
    for (int r = threadIdx.x; r < N; r += MP_THREADS) {
      const double sxv = __dsub_rn((double)vx[r], __dmul_rn(lam, wx[r]));
      const double syv = __dsub_rn((double)vy[r], __dmul_rn(lam, wy[r]));
      const double dfx = fabs(__dsub_rn(sxv, (double)vx[r]));
      const double dfy = fabs(__dsub_rn(syv, (double)vy[r]));
      if (!done[0]) {
        smoothed_x[off + r] = sxv;
        mxx = fmax(mxx, dfx);
        if (use_threshold && dfx > threshold) bx++;
      }
      if (!done[1]) {
        smoothed_y[off + r] = syv;
        mxy = fmax(mxy, dfy);
        if (use_threshold && dfy > threshold) by++;
      }
    }
    mxx = bmax<MP_THREADS>(mxx, sh);
    mxy = bmax<MP_THREADS>(mxy, sh);
    if (bx) atomicAdd(&s_bad[0], bx);
    if (by) atomicAdd(&s_bad[1], by);
    __syncthreads();
    const int nbx = s_bad[0], nby = s_bad[1];
    if (threadIdx.x == 0) {
      if (count[0] == 1 && !done[0]) max_udiff[2 * sd] = mxx;
      if (count[1] == 1 && !done[1]) max_udiff[2 * sd + 1] = mxy;
    }
    // store the weights of the components finishing now
    const int n3 = N + 3;
    double* wxo = weights + w_off[sd];
    double* wyo = wxo + n3;
    bool fin[2];
    fin[0] = !done[0] && (!use_threshold || nbx == 0 || count[0] > 10);
    fin[1] = !done[1] && (!use_threshold || nby == 0 || count[1] > 10);
    for (int r = threadIdx.x; r < N; r += MP_THREADS) {
      if (fin[0]) wxo[r] = wx[r];
      if (fin[1]) wyo[r] = wy[r];
    }
    if (threadIdx.x == 0) {
      if (fin[0])
        for (int k = 0; k < 3; ++k) wxo[N + k] = ax3[k];
      if (fin[1])
        for (int k = 0; k < 3; ++k) wyo[N + k] = ay3[k];
    }
    // replace the erratic values (rounded to float32 like upstream's array)
    for (int r = threadIdx.x; r < N; r += MP_THREADS) {
      if (!done[0] && !fin[0]) {
        const double sv = smoothed_x[off + r];
        if (fabs(__dsub_rn(sv, (double)vx[r])) > threshold) vx[r] = (float)sv;
      }
      if (!done[1] && !fin[1]) {
        const double sv = smoothed_y[off + r];
        if (fabs(__dsub_rn(sv, (double)vy[r])) > threshold) vy[r] = (float)sv;
      }
    }
    for (int c = 0; c < 2; ++c) {
      if (done[c]) continue;
      if (fin[c]) {
        done[c] = true;
      } else {
        fixed[c] += (c == 0) ? nbx : nby;
        count[c]++;
      }
    }
    __syncthreads();
    if (done[0] && done[1]) break;
  }
  if (!converged_all) return;
  if (threadIdx.x == 0) {
    iters[2 * sd] = count[0];
    iters[2 * sd + 1] = count[1];
    nfixed[2 * sd] = fixed[0];
    nfixed[2 * sd + 1] = fixed[1];
    status[sd] = 0;
  }
}

}  // namespace fi

using namespace fi;

extern "C" int fi_tps_phi_table(double* table, int64_t count, void* stream) {
  FI_REQUIRE(table && count > 0, "fi_tps_phi_table: bad arguments");
  k_phi_table<<<1024, 256, 0, (cudaStream_t)stream>>>(table, count);
  return check_launch("fi_tps_phi_table");
}

extern "C" int fi_tps_solve_mp(const fi_tps_plan* plan, int nb_subdom, int max_members,
                               const double* cx, const double* cy, const float* ux,
                               const float* uy, const int32_t* counts, const int64_t* offsets,
                               const int32_t* indices, const int64_t* mat_offsets,
                               double* matrices, float* matrices32, const double* phi_table,
                               int64_t table_size, const int32_t* cxy2,
                               const int32_t* c_on_lattice, double threshold, int use_threshold,
                               const int64_t* w_offsets, double* weights, double* smoothed_x,
                               double* smoothed_y, int32_t* iters, int32_t* nfixed,
                               int32_t* status, double* max_udiff, void* stream) {
  FI_REQUIRE(plan && cx && cy && ux && uy && counts && offsets && indices && mat_offsets &&
                 matrices && matrices32 && w_offsets && weights && smoothed_x &&
                 smoothed_y &&
                 iters && nfixed && status && max_udiff,
             "fi_tps_solve_mp: null pointer");
  FI_REQUIRE(nb_subdom > 0, "fi_tps_solve_mp: no subdomain");
  const int N = max_members > 4 ? max_members : 4;
  const size_t scratch = (size_t)(1 + MP_THREADS / 32) * 32 * 33 * sizeof(float);
  const size_t lat = (size_t)N * sizeof(int2);
  const size_t smem = (size_t)N * 11 * sizeof(double) + (size_t)N * 4 * sizeof(float) +
                      (scratch > lat ? scratch : lat) + 64;
  FI_REQUIRE(smem <= 220 * 1024, "fi_tps_solve_mp: subdomain of %d vectors too large",
             max_members);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    FI_CUDA_TRY(cudaFuncSetAttribute(k_tps_solve_mp,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  k_tps_solve_mp<<<nb_subdom, MP_THREADS, smem, (cudaStream_t)stream>>>(
      plan, cx, cy, ux, uy, counts, offsets, indices, mat_offsets, matrices, matrices32,
      phi_table, table_size, cxy2, c_on_lattice, threshold, use_threshold, w_offsets, weights, smoothed_x,
      smoothed_y, iters, nfixed, status, max_udiff, 60);
  return check_launch("fi_tps_solve_mp");
}
