// Mixed-precision solver of the smoothed TPS subdomain systems.
//
// Upstream (calcul/interpolate/thin_plate_spline.py:168-216,
// thin_plate_spline_subdom.py:236-280) solves [[K + lam I, P], [P^T, 0]] [w; a] =
// [u; 0] with LAPACK gesv in FP64, for x and y and again after each outlier
// replacement.  That saddle-point matrix has condition numbers ~1e13-1e15, but its
// null-space form is benign: with P = Q [R; 0] (Householder, Q = H0 H1 H2),
// w = Q2 z and
//     B z = g = Q2^T u,   B = Q2^T (K + lam I) Q2   (SPD, cond ~1e4 for lam > 0),
//     a = R^-1 (Q1^T u - C z),  C = Q1^T (K + lam I) Q2,   smoothed = u - lam w.
// On this GPU FP32 runs 73x faster than FP64.  B and C are projected once with the
// compact WY form of Q; the projection cancels the large affine part of K, so it
// needs more than FP32: Y = A V and B are computed in double-float (pairs of floats,
// error-free products and sums on the FP32 pipe, ~48 bits), the O(n) parts and C in
// FP64.  B is kept as (hi, lo) pairs and its FP32 rounding is factorised (tiled
// Cholesky).  z is refined in double-float: rho = g - B z on the FP32 pipe
// (error-free products and sums), then an FP32 Cholesky solve for the correction.
// Each sweep contracts the error ~1e3-1e4 times; refinement stops when the
// predicted remaining error is below 1e-10 of z, or when it stagnates (then it must
// be below 1e-9).  A subdomain that does not converge (or whose P has rank < 3, or
// whose Cholesky meets a non-positive pivot) is flagged and re-solved by the FP64
// LU kernel (k_tps_solve).
//
// K entries come from a table of phi(r^2) = r^2 log(r^2) / 2 indexed by 4 r^2,
// exact for window centres on the half-integer lattice (the integer window shifts
// put every PIV vector there); other distances use log() directly.  When a
// subdomain's centres lie on a grid of the lattice, the block keeps the (hi, lo)
// values of every grid offset in shared memory (the same table entries).
#include <cooperative_groups.h>

#include <climits>
#include <cmath>

#include "fi_common.cuh"
#include "fi_df.cuh"
#include "fi_lattice.cuh"

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

// The same values as (hi, lo) float pairs (double-float evaluation).
__global__ void k_phi_table2(float2* table, int64_t count) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count;
       k += (int64_t)gridDim.x * blockDim.x)
    table[k] = df_split(phi_direct((double)k * 0.25));
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

constexpr int TS = 36;  // row stride (floats) of the 32 x 32 shared tiles: float4-aligned rows

// Start moving [p, p + bytes) from memory into L2 without waiting for it (bulk
// prefetch by the copy engine; p 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// rho = g - B z for two right-hand sides, in double-float; B (m x m, symmetric, both
// triangles, column-major, leading dimension ld, a multiple of 4; 32-byte aligned)
// holds (hi, lo) pairs, read with the streaming hint (B is twice the FP32 factor,
// which should stay in L2).  Each warp takes four columns at a time (one row per
// lane), then reduce-scatters its eight sums over the warp.  B is streamed from
// memory: each warp has the copy engine prefetch its next two column groups into L2
// (contiguous, 32 ld bytes per column) while it works on the current one, so that
// its loads wait on L2 rather than on memory.  rho is rounded to float.
template <int NT>
__device__ void residual_df2(const float2* __restrict__ B, int m, int ld, const float2* zx,
                             const float2* zy, const float2* gx, const float2* gy, float* rx,
                             float* ry) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  auto prefetch_group = [&](int c) {
    if (lane == 0 && c < m)
      prefetch_l2(B + (int64_t)c * ld, (unsigned)(min(4, m - c) * ld * sizeof(float2)));
  };
  prefetch_group(4 * wid);
  prefetch_group(4 * wid + 4 * NW);
  for (int c0 = 4 * wid; c0 < m; c0 += 4 * NW) {
    prefetch_group(c0 + 8 * NW);
    // column q: x sums in lane .x, y sums in lane .y of the pairs (packed FP32x2)
    float2 H[4], Lo[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) H[q] = Lo[q] = make_float2(0.f, 0.f);
    const float2* col = B + (int64_t)c0 * ld;
    const int nc = min(4, m - c0);
    // two rows per lane and load (16 bytes: twice the bytes in flight per load); ld
    // is a multiple of 4, so row r + 1 < ld; the padding rows past m are masked
#pragma unroll 2
    for (int r = 2 * lane; r < m; r += 64) {
      const float4 a = *reinterpret_cast<const float4*>(zx + r);
      const float4 b = *reinterpret_cast<const float4*>(zy + r);
      const float2 zh0 = make_float2(a.x, b.x), zl0 = make_float2(a.y, b.y);
      const float2 zh1 = make_float2(a.z, b.z), zl1 = make_float2(a.w, b.w);
      const bool two = r + 1 < m;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (q < nc) v = __ldcs(reinterpret_cast<const float4*>(col + (int64_t)q * ld + r));
        if (!two) v.z = v.w = 0.f;
        df_mac_x2(make_float2(v.x, v.y), zh0, zl0, H[q], Lo[q]);
        df_mac_x2(make_float2(v.z, v.w), zh1, zl1, H[q], Lo[q]);
      }
    }
    float h[8], l[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      h[q] = H[q].x;
      l[q] = Lo[q].x;
      h[4 + q] = H[q].y;
      l[4 + q] = Lo[q].y;
    }
    // reduce-scatter: lane ends with value 4 b4 + 2 b3 + b2 (b_k = bit k of lane)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool up = lane & 16;
      const float sh_ = up ? h[k] : h[k + 4], sl_ = up ? l[k] : l[k + 4];
      const float2 keep = up ? make_float2(h[k + 4], l[k + 4]) : make_float2(h[k], l[k]);
      const float2 got = make_float2(__shfl_xor_sync(full, sh_, 16), __shfl_xor_sync(full, sl_, 16));
      const float2 s = df_add(keep, got);
      h[k] = s.x;
      l[k] = s.y;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const bool up = lane & 8;
      const float sh_ = up ? h[k] : h[k + 2], sl_ = up ? l[k] : l[k + 2];
      const float2 keep = up ? make_float2(h[k + 2], l[k + 2]) : make_float2(h[k], l[k]);
      const float2 got = make_float2(__shfl_xor_sync(full, sh_, 8), __shfl_xor_sync(full, sl_, 8));
      const float2 s = df_add(keep, got);
      h[k] = s.x;
      l[k] = s.y;
    }
    {
      const bool up = lane & 4;
      const float sh_ = up ? h[0] : h[1], sl_ = up ? l[0] : l[1];
      const float2 keep = up ? make_float2(h[1], l[1]) : make_float2(h[0], l[0]);
      const float2 got = make_float2(__shfl_xor_sync(full, sh_, 4), __shfl_xor_sync(full, sl_, 4));
      const float2 s = df_add(keep, got);
      h[0] = s.x;
      l[0] = s.y;
    }
#pragma unroll
    for (int o = 2; o > 0; o >>= 1) {
      const float2 got = make_float2(__shfl_xor_sync(full, h[0], o), __shfl_xor_sync(full, l[0], o));
      const float2 s = df_add(make_float2(h[0], l[0]), got);
      h[0] = s.x;
      l[0] = s.y;
    }
    if ((lane & 3) == 0) {
      const int idx = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
      const int c = c0 + (idx & 3);
      if (c < m) {
        const float2 g = (idx >> 2) ? gy[c] : gx[c];
        const float2 d = df_add(g, make_float2(-h[0], -l[0]));
        ((idx >> 2) ? ry : rx)[c] = __fadd_rn(d.x, d.y);
      }
    }
  }
  __syncthreads();
}

// Apply H_k = I - tau_k v_k v_k^T (k in order) to the two vectors x, y (length n);
// v_k is row k of V (row stride vstride).
template <int NT, bool REVERSE>
__device__ void apply_reflectors2(const double* V, int vstride, const double* tau, int n,
                                  double* x, double* y, double* sh) {
  for (int kk = 0; kk < 3; ++kk) {
    const int k = REVERSE ? 2 - kk : kk;
    const double* v = V + (int64_t)k * vstride;
    double2 d = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < n; i += NT) {
      d.x += v[i] * x[i];
      d.y += v[i] * y[i];
    }
    d = bsum2<NT>(d, sh);
    const double cx = tau[k] * d.x, cy = tau[k] * d.y;
    for (int i = threadIdx.x; i < n; i += NT) {
      x[i] -= cx * v[i];
      y[i] -= cy * v[i];
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

// POTRF of one 32 x 32 tile held in registers (a[c] = element (lane, c)): writes the
// factor's lower triangle to tile (k, k) of B, its rows (zero right of the diagonal)
// and 1 / L_jj (column 32) to Lkk; sets *s_flag on a non-positive pivot.
__device__ __forceinline__ void potrf_tile(float (&a)[32], float* B, int m, int ld, int k,
                                           float* Lkk, int lane, int* s_flag) {
  const unsigned full = 0xffffffffu;
  bool bad = false;
  float dg = 1.f;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    float djj = __shfl_sync(full, a[j], j);
    if (!(djj > 0.f)) {
      bad = true;
      djj = 1.f;
    }
    const float rs = rsqrtf(djj);  // FP32 factor: refinement absorbs its rounding
    const float sq = djj * rs;
    if (lane == j) dg = sq;
    const float lrj = (lane > j) ? a[j] * rs : ((lane == j) ? sq : 0.f);
    if (lane >= j) a[j] = lrj;
    // the row update in chunks of 8 shuffles: the fence keeps the compiler from
    // hoisting all 31 (the row a[] then stays in registers under the cap)
#pragma unroll
    for (int c0 = (j + 1) & ~7; c0 < 32; c0 += 8) {
#pragma unroll
      for (int c = c0; c < c0 + 8; ++c) {
        if (c <= j) continue;
        const float lcj = __shfl_sync(full, lrj, c);
        if (lane >= c) a[c] = fmaf(-lrj, lcj, a[c]);
      }
      __syncwarp();
    }
  }
  if (bad && lane == 0) *s_flag = 1;
  tile_store(B, m, ld, k, k, a, lane, true);
#pragma unroll
  for (int c = 0; c < 32; ++c) Lkk[lane * TS + c] = (c < lane) ? a[c] : 0.f;
  Lkk[lane * TS + 32] = 1.f / dg;
}

// Swizzle of the shared tile column: element (t, r) of a 32 x 32 tile (t the column
// of L_ik, r its row) sits at t * 32 + (r ^ pswz(t)).  The tensor-core fragments read
// rows r = 8a + g (g = lane / 4) of columns t = 8b + q (q = lane % 4): the XOR sends
// the four q to four different groups of eight banks.  An aligned group of four r
// stays contiguous and in order (float4 reads of a row).
__device__ __forceinline__ int pswz(int t) { return (t & 3) << 3; }

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// x = hi + lo with hi and lo TF32 (the split of the 3xTF32 products: Ootomo and
// Yokota, "Recovering single precision accuracy from Tensor Cores while surpassing
// the FP32 theoretical peak performance", IJHPCA 2022)
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Tile (i, j) of B -= L_ik L_jk^T on the tensor cores (warp-level m16n8k8 TF32 MMA),
// FP32-accurate by the 3xTF32 split (hi*hi + hi*lo + lo*hi, FP32 accumulation): the
// factor only preconditions the double-float refinement, which absorbs the ~2^-21
// relative rounding like the FP32 one.  The 32 x 32 tile is 2 x 4 fragments of
// 16 x 8; Pi, Pj: the swizzled shared tiles of L_ik and L_jk.  Entries past m are
// neither read nor written; a diagonal tile keeps its upper triangle.
__device__ __forceinline__ void tile_update_mma(float* B, int m, int ld, int ti, int tj,
                                                const float* Pi, const float* Pj, int lane) {
  const int g = lane >> 2, q = lane & 3;
  float c[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int r = 32 * ti + 16 * mt + g + 8 * (e >> 1);
        const int col = 32 * tj + 8 * nt + 2 * q + (e & 1);
        c[mt][nt][e] = (r < m && col < m) ? B[(int64_t)col * ld + r] : 0.f;
      }
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const int t0 = 8 * ks + q, t1 = t0 + 4;  // both have (t & 3) == q
    const int sw = q << 3;
    uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int r0 = (16 * mt + g) ^ sw, r1 = (16 * mt + g + 8) ^ sw;
      split_tf32(-Pi[t0 * 32 + r0], ah[mt][0], al[mt][0]);
      split_tf32(-Pi[t0 * 32 + r1], ah[mt][1], al[mt][1]);
      split_tf32(-Pi[t1 * 32 + r0], ah[mt][2], al[mt][2]);
      split_tf32(-Pi[t1 * 32 + r1], ah[mt][3], al[mt][3]);
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int rn = (8 * nt + g) ^ sw;
      split_tf32(Pj[t0 * 32 + rn], bh[nt][0], bl[nt][0]);
      split_tf32(Pj[t1 * 32 + rn], bh[nt][1], bl[nt][1]);
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        mma_tf32(c[mt][nt], al[mt], bh[nt]);
        mma_tf32(c[mt][nt], ah[mt], bl[nt]);
        mma_tf32(c[mt][nt], ah[mt], bh[nt]);
      }
  }
  const bool diag = ti == tj;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int rl = 16 * mt + g + 8 * (e >> 1), cl = 8 * nt + 2 * q + (e & 1);
        const int r = 32 * ti + rl, col = 32 * tj + cl;
        if (r < m && col < m && (!diag || cl <= rl)) B[(int64_t)col * ld + r] = c[mt][nt][e];
      }
}

// Shared memory of chol_factor for an m x m matrix: two L_kk tiles (rows of TS
// floats) and the current tile column, transposed (T - 1 tiles of 32 x 32).
__host__ __device__ inline size_t chol_scratch_bytes(int m) {
  const int T = (m + 31) / 32;
  return (size_t)2 * 32 * TS * sizeof(float) + (size_t)(T > 1 ? T - 1 : 0) * 1024 * sizeof(float);
}

// Right-looking tiled Cholesky (lower) of the m x m matrix B (column-major, ld), in
// place (lower triangle).  Per tile column k: warps solve the tiles below the
// diagonal (one row per lane, rows of L_kk read as float4 broadcasts) and keep them,
// transposed and swizzled, in shared memory; then they update the trailing tile
// pairs on the tensor cores (3xTF32 warp MMA, both factors read from the shared tile
// column: the update loads only its own tile).  Lookahead: warp 0 first updates the next
// diagonal tile and factorises it in registers (shuffles) while the other warps
// update the rest; the tiles go to the warps in the order they finish.
// scratch: chol_scratch_bytes(m), 16-byte aligned.  False on a non-positive pivot.
template <int NT>
__device__ bool chol_factor(float* B, int m, int ld, float* scratch, int* s_flag,
                            int* s_next) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  const int T = (m + 31) / 32;
  // two L_kk buffers (step k reads buffer k & 1 while step k + 1's is written); row
  // j: L_kk[j][c] for c < j (0 elsewhere), [32] = 1 / L_jj
  float* Lkk0 = scratch;
  // tile column k: tile i > k at P + (i - k - 1) * 1024, element
  // [t * 32 + (r ^ pswz(t))] = L_ik[r][t]
  float* P = scratch + 2 * 32 * TS;
  if (threadIdx.x == 0) *s_flag = 0;
  __syncthreads();
  if (wid == 0) {
    float a[32];
    tile_load(B, m, ld, 0, 0, a, lane);
    potrf_tile(a, B, m, ld, 0, Lkk0, lane, s_flag);
  }
  __syncthreads();
  for (int k = 0; k < T; ++k) {
    const float* Lkk = Lkk0 + (k & 1) * 32 * TS;
    // TRSM: tiles (i, k), i > k: X L_kk^T = A_ik, row by row in each lane
    for (int i = k + 1 + wid; i < T; i += NW) {
      float b[32];
      tile_load(B, m, ld, i, k, b, lane);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        float v = b[j];
#pragma unroll
        for (int c4 = 0; c4 < (j + 3) / 4; ++c4) {  // entries c >= j of row j are 0
          const float4 q = *reinterpret_cast<const float4*>(Lkk + j * TS + 4 * c4);
          v = fmaf(-b[4 * c4], q.x, v);
          v = fmaf(-b[4 * c4 + 1], q.y, v);
          v = fmaf(-b[4 * c4 + 2], q.z, v);
          v = fmaf(-b[4 * c4 + 3], q.w, v);
        }
        b[j] = v * Lkk[j * TS + 32];
        if ((j & 3) == 3) __syncwarp();  // bounds the broadcasts in flight (registers)
      }
      tile_store(B, m, ld, i, k, b, lane, false);
      float* Pi = P + (i - k - 1) * 1024;
      const bool rin = 32 * i + lane < m;  // rows past m: zero (their updates are unused)
#pragma unroll
      for (int t = 0; t < 32; ++t) Pi[t * 32 + (lane ^ pswz(t))] = rin ? b[t] : 0.f;
    }
    if (threadIdx.x == 0) *s_next = NW;
    __syncthreads();
    if (k + 1 >= T) break;
    // trailing update: tiles (i, j), k < j <= i; pair 0 is tile (k + 1, k + 1)
    const int n = T - k - 1;
    const int npairs = n * (n + 1) / 2;
    int pidx = wid;
    while (pidx < npairs) {
      int ii = (int)((sqrtf(8.f * pidx + 1.f) - 1.f) * 0.5f);
      while ((ii + 1) * (ii + 2) / 2 <= pidx) ++ii;
      while (ii * (ii + 1) / 2 > pidx) --ii;
      const int jj = pidx - ii * (ii + 1) / 2;
      const int i = k + 1 + ii, j = k + 1 + jj;
      const float* Pi = P + ii * 1024;
      const float* Pj = P + jj * 1024;
      if (pidx == 0) {
        // the next diagonal tile in row layout (one row per lane) for its
        // factorisation: acc -= L_ik L_jk^T with L_ik[lane][t] and the row t of L_jk^T
        // from shared memory, packed FP32x2 FMAs
        float acc[32];
        tile_load(B, m, ld, i, j, acc, lane);
#pragma unroll 4
        for (int t = 0; t < 32; ++t) {
          const int sw = pswz(t);
          const float l = -Pi[t * 32 + (lane ^ sw)];
          const float2 lr = make_float2(l, l);
#pragma unroll
          for (int c4 = 0; c4 < 8; ++c4) {
            const float4 q = *reinterpret_cast<const float4*>(Pj + t * 32 + ((4 * c4) ^ sw));
            float2 a01 = make_float2(acc[4 * c4], acc[4 * c4 + 1]);
            float2 a23 = make_float2(acc[4 * c4 + 2], acc[4 * c4 + 3]);
            a01 = __ffma2_rn(lr, make_float2(q.x, q.y), a01);
            a23 = __ffma2_rn(lr, make_float2(q.z, q.w), a23);
            acc[4 * c4] = a01.x;
            acc[4 * c4 + 1] = a01.y;
            acc[4 * c4 + 2] = a23.x;
            acc[4 * c4 + 3] = a23.y;
          }
        }
        potrf_tile(acc, B, m, ld, k + 1, Lkk0 + ((k + 1) & 1) * 32 * TS, lane, s_flag);
      } else {
        tile_update_mma(B, m, ld, i, j, Pi, Pj, lane);
      }
      int nxt = 0;
      if (lane == 0) nxt = atomicAdd(s_next, 1);
      pidx = __shfl_sync(full, nxt, 0);
    }
    __syncthreads();
  }
  return *s_flag == 0;
}

// Inverses of the diagonal tiles of the factor L (lower, column-major, ld), for
// chol_solve2: tile k's inverse (lower triangular) packed by columns at dinv + 528 k,
// column c holding rows c..31 from tri_colstart(c).  Reading row i (fixed column,
// consecutive rows) or column c (rows i >= c: offsets that are triangular numbers
// apart, distinct modulo 32) is free of bank conflicts.  Rows and columns past m are
// the identity's.
__device__ __forceinline__ int tri_colstart(int c) { return 32 * c - (c * (c - 1)) / 2; }
constexpr int TRI_TILE = 528;  // 32 * 33 / 2

template <int NT>
__device__ void chol_diag_inverses(const float* __restrict__ L, int m, int ld, float* dinv) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  const int T = (m + 31) / 32;
  for (int k = wid; k < T; k += NW) {
    float a[32];  // a[j] = L[32 k + lane][32 k + j] (only j <= lane is read below)
    tile_load(L, m, ld, k, k, a, lane);
    float dl = 1.f;  // L[lane][lane] (constant indices keep a[] in registers)
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j == lane) dl = a[j];
    const float rdiag = 1.f / dl;
    // lane i: row i of X = inv(L_kk), right-looking: row j is final once scaled by
    // 1 / L_jj, then every later row i takes off L_ij X_j (independent columns: the
    // dependent chain is 32 steps long, not 528)
    float x[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) x[c] = (c == lane) ? 1.f : 0.f;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float rj = __shfl_sync(full, rdiag, j);
#pragma unroll
      for (int c = 0; c <= j; ++c) {
        const float xjc = __shfl_sync(full, x[c], j) * rj;
        if (lane == j)
          x[c] = xjc;
        else if (lane > j)
          x[c] = fmaf(-a[j], xjc, x[c]);
      }
    }
    float* D = dinv + TRI_TILE * k + lane;
#pragma unroll
    for (int c = 0; c < 32; ++c)
      if (c <= lane) D[tri_colstart(c) - c] = x[c];
  }
  __syncthreads();
}

// Solve (L L^T) x = r in place for two right-hand sides (float).  L: lower m x m,
// column-major, leading dimension ld (a multiple of 4, 16-byte aligned base); only
// its lower triangle is read.  rx, ry: shared, 16-byte aligned, zero from m up to a
// multiple of 32.  dinv: the diagonal tiles' inverses (chol_diag_inverses), so that
// a diagonal step is a triangular product in one warp instead of a chain of 32
// dependent shuffles.  By tiles of 32: the off-diagonal tiles by all warps with
// coalesced (forward) or contiguous float4 (backward) loads, issued before the
// barrier that publishes the diagonal step (their values do not depend on it), and
// float4 broadcasts of x.  part: 64 * warps floats.
template <int NT>
__device__ void chol_solve2(const float* __restrict__ L, int m, int ld, float* rx, float* ry,
                            float* part, const float* dinv) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int T = (m + 31) / 32;
  // ---- forward: L y = r
  for (int k = 0; k < T; ++k) {
    const int r0 = 32 * k;
    // this warp's first off-diagonal tile (k + 1 + wid), loaded ahead
    const int ia = k + 1 + wid;
    const int ra = 32 * ia + lane;
    float la[32];
    if (ia < T && ra < m) {
      const float* Lc = L + (int64_t)r0 * ld + ra;
#pragma unroll
      for (int c = 0; c < 32; ++c) la[c] = Lc[(int64_t)c * ld];
    }
    if (wid == 0) {
      // y_k = inv(L_kk) r_k: lane i sums row i of the inverse
      const float* D = dinv + TRI_TILE * k + lane;
      float vx = 0.f, vy = 0.f;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j <= lane) {
          const float l = D[tri_colstart(j) - j];
          vx = fmaf(l, rx[r0 + j], vx);
          vy = fmaf(l, ry[r0 + j], vy);
        }
      }
      __syncwarp();
      rx[r0 + lane] = vx;
      ry[r0 + lane] = vy;
    }
    __syncthreads();
    // r_i -= L_ik y_k for the tiles i > k (their rows are below m only in full tiles k)
    for (int i = ia; i < T; i += NW) {
      const int r = 32 * i + lane;
      if (r < m) {
        if (i != ia) {
          const float* Lc = L + (int64_t)r0 * ld + r;
#pragma unroll
          for (int c = 0; c < 32; ++c) la[c] = Lc[(int64_t)c * ld];
        }
        float sx = 0.f, sy = 0.f, sx2 = 0.f, sy2 = 0.f;
#pragma unroll
        for (int c4 = 0; c4 < 8; c4 += 2) {
          const float4 yx = *reinterpret_cast<const float4*>(rx + r0 + 4 * c4);
          const float4 yy = *reinterpret_cast<const float4*>(ry + r0 + 4 * c4);
          const float4 yx2 = *reinterpret_cast<const float4*>(rx + r0 + 4 * c4 + 4);
          const float4 yy2 = *reinterpret_cast<const float4*>(ry + r0 + 4 * c4 + 4);
          sx = fmaf(la[4 * c4], yx.x, sx);
          sy = fmaf(la[4 * c4], yy.x, sy);
          sx = fmaf(la[4 * c4 + 1], yx.y, sx);
          sy = fmaf(la[4 * c4 + 1], yy.y, sy);
          sx = fmaf(la[4 * c4 + 2], yx.z, sx);
          sy = fmaf(la[4 * c4 + 2], yy.z, sy);
          sx = fmaf(la[4 * c4 + 3], yx.w, sx);
          sy = fmaf(la[4 * c4 + 3], yy.w, sy);
          sx2 = fmaf(la[4 * c4 + 4], yx2.x, sx2);
          sy2 = fmaf(la[4 * c4 + 4], yy2.x, sy2);
          sx2 = fmaf(la[4 * c4 + 5], yx2.y, sx2);
          sy2 = fmaf(la[4 * c4 + 5], yy2.y, sy2);
          sx2 = fmaf(la[4 * c4 + 6], yx2.z, sx2);
          sy2 = fmaf(la[4 * c4 + 6], yy2.z, sy2);
          sx2 = fmaf(la[4 * c4 + 7], yx2.w, sx2);
          sy2 = fmaf(la[4 * c4 + 7], yy2.w, sy2);
        }
        rx[r] -= sx + sx2;
        ry[r] -= sy + sy2;
      }
    }
    __syncthreads();
  }
  // ---- backward: L^T x = y
  for (int k = T - 1; k >= 0; --k) {
    const int c0 = 32 * k;
    const int t = c0 + lane;  // this lane's column
    float px = 0.f, py = 0.f;
    for (int i = k + 1 + wid; i < T; i += NW) {  // column t is below m here
      const float* Lc = L + (int64_t)t * ld + 32 * i;
      float4 lv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int row = 32 * i + 4 * q;
        lv[q] = (row < ld) ? *reinterpret_cast<const float4*>(Lc + 4 * q)
                           : make_float4(0.f, 0.f, 0.f, 0.f);
        if (row + 0 >= m) lv[q].x = 0.f;
        if (row + 1 >= m) lv[q].y = 0.f;
        if (row + 2 >= m) lv[q].z = 0.f;
        if (row + 3 >= m) lv[q].w = 0.f;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int row = 32 * i + 4 * q;
        const float4 xv = *reinterpret_cast<const float4*>(rx + row);
        const float4 yv = *reinterpret_cast<const float4*>(ry + row);
        px = fmaf(lv[q].x, xv.x, px);
        py = fmaf(lv[q].x, yv.x, py);
        px = fmaf(lv[q].y, xv.y, px);
        py = fmaf(lv[q].y, yv.y, py);
        px = fmaf(lv[q].z, xv.z, px);
        py = fmaf(lv[q].z, yv.z, py);
        px = fmaf(lv[q].w, xv.w, px);
        py = fmaf(lv[q].w, yv.w, py);
      }
    }
    part[wid * 64 + lane] = px;
    part[wid * 64 + 32 + lane] = py;
    __syncthreads();
    if (wid == 0) {
      float vx = rx[t], vy = ry[t];
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        vx -= part[w * 64 + lane];
        vy -= part[w * 64 + 32 + lane];
      }
      rx[t] = vx;
      ry[t] = vy;
      __syncwarp();
      // x_k = inv(L_kk)^T v_k: lane c sums column c of the inverse (rows i >= c)
      const float* D = dinv + TRI_TILE * k + tri_colstart(lane) - lane;
      float sx = 0.f, sy = 0.f;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        if (i >= lane) {
          const float l = D[i];
          sx = fmaf(l, rx[c0 + i], sx);
          sy = fmaf(l, ry[c0 + i], sy);
        }
      }
      __syncwarp();
      rx[t] = sx;
      ry[t] = sy;
    }
    __syncthreads();
  }
}

// Shared-memory layout of k_tps_solve_mp for subdomains of at most n centres.
struct MpLayout {
  int np;        // n rounded up to 32
  size_t d_off;  // doubles: V 3n, xc n, yc n, Y/C 3n, W 4n
  size_t f2_off; // float2: zx, zy, gx, gy (np each)
  size_t f_off;  // float: vx, vy, rx, ry (np each)
  size_t i2_off; // int2: lattice coordinates (np)
  size_t p_off;  // panel: (2 + warps) * 32 * TS floats at least
  size_t bytes;
  __host__ __device__ MpLayout(int n, int warps) {
    np = (n + 31) & ~31;
    d_off = 0;
    f2_off = d_off + (size_t)12 * n * sizeof(double);
    f_off = f2_off + (size_t)4 * np * sizeof(float2);
    i2_off = f_off + (size_t)4 * np * sizeof(float);
    p_off = i2_off + (size_t)np * sizeof(int2);
    // the panel also holds the projection's per-warp tiles and the solves' partial
    // sums; the Cholesky scratch starts at f2_off (the f2, f and i2 regions are free
    // while it runs)
    size_t pbytes = (size_t)(2 + warps) * 32 * TS * sizeof(float);
    // the solves: per-warp partial sums, then the diagonal tiles' inverses
    const size_t sol = ((size_t)64 * warps + (size_t)((n + 31) / 32) * TRI_TILE) * sizeof(float);
    if (pbytes < sol) pbytes = sol;
    const size_t chol = chol_scratch_bytes(n);
    if (f2_off + chol > p_off + pbytes) pbytes = f2_off + chol - p_off;
    bytes = p_off + pbytes;
  }
};

// One block per subdomain.  Status per subdomain: 0 solved here, 1 needs the FP64
// LU fallback (rank-deficient P, Cholesky breakdown or no convergence).
//
// Buffers per subdomain (offset mat_off, a multiple of 4 elements): matrices holds
// B22 = (Q^T A Q)[3:, 3:] as (hi, lo) float pairs, both triangles, leading
// dimension mp = m rounded up to 4; matrices32 holds its FP32 Cholesky factor (lower
// triangle, same layout).
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT)
    k_tps_solve_mp(const fi_tps_plan* plan_ptr, const double* cx, const double* cy,
                   const float* ux, const float* uy, const int32_t* counts,
                   const int64_t* offsets, const int32_t* indices, const int64_t* mat_off,
                   double* matrices, float* matrices32, const double* phi_table,
                   const float2* phi_table2, int64_t table_size, const int32_t* cxy2,
                   const int32_t* c_on_lattice, double threshold, int use_threshold,
                   const int64_t* w_off, double* weights,
                   double* smoothed_x, double* smoothed_y, int32_t* iters, int32_t* nfixed,
                   int32_t* status, double* max_udiff, int32_t* sweeps,
                   const int32_t* order, int max_refine, int n_layout) {
  constexpr int NW = NT / 32;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sh[80];
  __shared__ double s_tau[3];
  __shared__ double s_R[9];
  __shared__ double s_q1[6];
  __shared__ int s_flag, s_next, s_bad[2], s_lat;
  const fi_tps_plan p = *plan_ptr;
  // a cluster of csize CTAs per subdomain (1 without cluster launch): all of them
  // factor P and share the FP64 build and projection, rank 0 then solves alone
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int csize = (int)cluster.num_blocks();
  const int crank = (int)cluster.block_rank();
  const int sd = order != nullptr ? order[blockIdx.x / csize] : (int)(blockIdx.x / csize);
  const int N = counts[sd];
  const int m = N - 3;
  const int64_t off = offsets[sd];
  const int32_t* idx = indices + off;
  const double lam = p.smoothing;
  if (threadIdx.x == 0 && crank == 0) {
    status[sd] = 1;
    if (sweeps != nullptr) sweeps[sd] = 0;
  }
  if (m < 1) return;  // fewer than 4 centres: FP64 LU path
  const int mp = (m + 3) & ~3;

  const MpLayout lay(n_layout, NW);
  const int n = n_layout;
  double* V = reinterpret_cast<double*>(smraw + lay.d_off);  // 3 n (rows k: v_k)
  double* xc = V + 3 * n;
  double* yc = xc + n;
  double* YC = yc + n;  // Y = A V (3 n), then C = (Q^T A Q)[0:3, 3:] (3 n)
  double* W = YC + 3 * n;  // 4 n: QR scratch, Z, then t / w
  float2* zx2 = reinterpret_cast<float2*>(smraw + lay.f2_off);
  float2* zy2 = zx2 + lay.np;
  float2* gx2 = zy2 + lay.np;
  float2* gy2 = gx2 + lay.np;
  float* vx = reinterpret_cast<float*>(smraw + lay.f_off);
  float* vy = vx + lay.np;
  float* rx = vy + lay.np;
  float* ry = rx + lay.np;
  int2* cxy = reinterpret_cast<int2*>(smraw + lay.i2_off);
  float* panel = reinterpret_cast<float*>(smraw + lay.p_off);

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2* B2 = reinterpret_cast<float2*>(matrices + mat_off[sd]);
  float* L32 = matrices32 + mat_off[sd];

  if (threadIdx.x == 0)
    s_lat = (cxy2 != nullptr && c_on_lattice != nullptr && phi_table != nullptr) ? *c_on_lattice : 0;
  for (int i = threadIdx.x; i < N; i += NT) {
    const int a = idx[i];
    xc[i] = cx[a];
    yc[i] = cy[a];
    if (cxy2 != nullptr) cxy[i] = make_int2(cxy2[2 * a], cxy2[2 * a + 1]);
  }
  __syncthreads();
  const bool lat = s_lat != 0;
  // Centres on the lattice: cxy becomes the grid indices ((2x - 2x_0) / gx,
  // (2y - 2y_0) / gy) of the grid of steps (gx, gy) through them, and, when every
  // offset of the grid's extent fits, tab holds the (hi, lo) kernel value of each
  // offset (a, b) at tab[b tw + a] (tw = 0: no table).  The table lives in W's last n
  // doubles, free until the refinement.
  int gx = 1, gy = 1, tw = 0;
  float2* tab = reinterpret_cast<float2*>(W + 3 * n);
  const int tsz32 = (int)(table_size < (int64_t)INT_MAX ? table_size : (int64_t)INT_MAX);
  if (lat) {
    const int2 o = cxy[0];
    int v[6];
    lat_grid_init(v);
    for (int i = threadIdx.x; i < N; i += NT) lat_grid_add(v, cxy[i].x - o.x, cxy[i].y - o.y);
    lat_grid_block(v, reinterpret_cast<int*>(sh));
    const LatTable g = lat_table_of(v, n, tsz32);
    gx = g.gx;
    gy = g.gy;
    for (int i = threadIdx.x; i < N; i += NT)
      cxy[i] = make_int2((cxy[i].x - o.x) / gx, (cxy[i].y - o.y) / gy);
    if (g.ok && phi_table2 != nullptr) {
      tw = g.wx;
      for (int e = threadIdx.x; e < g.wx * g.wy; e += NT) {
        const int b = e / g.wx, a = e - b * g.wx;
        tab[e] = phi_table2[(gy * b) * (gy * b) + (gx * a) * (gx * a)];
      }
    }
    __syncthreads();
  }
  // A = K + lam I, entry (r, c); on the lattice 4 r^2 is an integer table index
  auto a_entry = [&](int r, int c) -> double {
    if (r == c) return lam;
    if (lat) {
      const int2 ca = cxy[r], cb = cxy[c];
      const int64_t dx = (int64_t)gx * (ca.x - cb.x), dy = (int64_t)gy * (ca.y - cb.y);
      const int64_t kq = dy * dy + dx * dx;
      if (kq < table_size) return __ldg(phi_table + kq);
      return phi_pair(xc[r], yc[r], xc[c], yc[c], nullptr, 0);
    }
    return phi_pair(xc[r], yc[r], xc[c], yc[c], phi_table, table_size);
  };
  // the same entry as a (hi, lo) float pair; ci = lattice coordinates of centre i
  const float2 lam2 = df_split(lam);
  auto a_entry_df = [&](int i, int2 ci, int j) -> float2 {
    if (i == j) return lam2;
    if (lat) {
      const int2 cj = cxy[j];
      const int64_t dx = (int64_t)gx * (ci.x - cj.x), dy = (int64_t)gy * (ci.y - cj.y);
      const int64_t kq = dy * dy + dx * dx;
      if (kq < table_size)
        return phi_table2 != nullptr ? phi_table2[kq] : df_split(__ldg(phi_table + kq));
      return df_split(phi_pair(xc[i], yc[i], xc[j], yc[j], nullptr, 0));
    }
    return df_split(phi_pair(xc[i], yc[i], xc[j], yc[j], phi_table, table_size));
  };
  // entries (i, j0 .. j0 + cnt - 1) of A as pairs (0 < cnt <= 8, the rest zero): on the
  // lattice the eight table loads are issued before any is used (the loads, mostly
  // L2 hits, bound these phases), the diagonal and far entries patched afterwards
  auto a_batch_df = [&](int i, int2 ci, int j0, int cnt, float2(&out)[8]) {
    if (lat && tw > 0) {  // every offset in the shared table
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int2 cj = cxy[j0 + min(u, cnt - 1)];
        out[u] = tab[abs(ci.y - cj.y) * tw + abs(ci.x - cj.x)];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (u >= cnt)
          out[u] = make_float2(0.f, 0.f);
        else if (j0 + u == i)
          out[u] = lam2;
      }
    } else if (lat && phi_table2 != nullptr) {
      // 4 r^2 in 32-bit integers: the lattice coordinates are below 2^30 in magnitude,
      // so their differences fit, and |dx|, |dy| <= 32767 keeps dx^2 + dy^2 below
      // 2^31; farther pairs (beyond the table anyway) take the direct kernel value
      int kq[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int2 cj = cxy[j0 + min(u, cnt - 1)];
        const int dx = gx * (ci.x - cj.x), dy = gy * (ci.y - cj.y);
        const bool near = (unsigned)dx + 32767u <= 65534u && (unsigned)dy + 32767u <= 65534u;
        kq[u] = near ? dy * dy + dx * dx : INT_MAX;
        out[u] = phi_table2[kq[u] < tsz32 ? kq[u] : 0];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u;
        if (u >= cnt)
          out[u] = make_float2(0.f, 0.f);
        else if (j == i)
          out[u] = lam2;
        else if (kq[u] >= tsz32)
          out[u] = df_split(phi_pair(xc[i], yc[i], xc[j], yc[j], nullptr, 0));
      }
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u)
        out[u] = (u < cnt) ? a_entry_df(i, ci, j0 + u) : make_float2(0.f, 0.f);
    }
  };

  // ---- Householder QR of P = [1, y, x] (FP64), V rows k hold v_k (zeros above k)
  {
    double* P0 = W;  // scratch columns
    double* P1 = W + n;
    double* P2 = W + 2 * n;
    for (int i = threadIdx.x; i < N; i += NT) {
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
      for (int i = k + threadIdx.x; i < N; i += NT) nrm2 += x[i] * x[i];
      nrm2 = bsum<NT>(nrm2, sh);
      const double x0 = x[k];
      const double nrm = sqrt(nrm2);
      if (!(nrm > 0.0)) {
        rank_ok = false;
        break;
      }
      const double alpha = (x0 >= 0.0) ? -nrm : nrm;
      double* v = V + (int64_t)k * n;
      for (int i = threadIdx.x; i < N; i += NT) v[i] = (i < k) ? 0.0 : x[i];
      __syncthreads();
      if (threadIdx.x == 0) v[k] = x0 - alpha;
      __syncthreads();
      double vv = 0.0;
      for (int i = k + threadIdx.x; i < N; i += NT) vv += v[i] * v[i];
      vv = bsum<NT>(vv, sh);
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
        for (int i = k + threadIdx.x; i < N; i += NT) d += v[i] * y[i];
        d = bsum<NT>(d, sh);
        for (int i = k + threadIdx.x; i < N; i += NT) y[i] -= tau * d * v[i];
        __syncthreads();
        if (threadIdx.x == 0) s_R[k * 3 + j] = y[k];
        __syncthreads();
      }
      if (fabs(alpha) < 1e-9 * sqrt((double)N)) rank_ok = false;  // collinear centres
    }
    __syncthreads();
    if (!rank_ok) return;
  }
  const double* V0 = V;
  const double* V1 = V + n;
  const double* V2 = V + 2 * n;
  double* Y0 = YC;
  double* Y1 = YC + n;
  double* Y2 = YC + 2 * n;
  // V and Z as (hi, lo) float pairs, [3][np] each: the f2 and f regions (6 np pairs)
  // are free until the refinement
  float2* Vd = zx2;
  float2* Zd = zx2 + 3 * lay.np;
  const int np = lay.np;
  for (int i = threadIdx.x; i < np; i += NT) {
    const bool in = i < N;
    Vd[i] = in ? df_split(V0[i]) : make_float2(0.f, 0.f);
    Vd[np + i] = in ? df_split(V1[i]) : make_float2(0.f, 0.f);
    Vd[2 * np + i] = in ? df_split(V2[i]) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // every CTA of the cluster has started (and holds its V) before any CTA writes
  // into a peer's shared memory below
  cluster.sync();
  // ---- Y = A V in double-float on the FP32 pipe.  A is symmetric: lane = column c,
  // the rows r in chunks (jobs = column block x chunk, a multiple of the warp count
  // when the scratch allows); the chunks' partial sums are added in a fixed order.
  // The column blocks are spread over the cluster's CTAs; each Y value is rounded to
  // double and written into every CTA's Y.
  {
    auto write_y = [&](int c, float2 s0, float2 s1, float2 s2) {
      const double y0 = df_to_double(s0), y1 = df_to_double(s1), y2 = df_to_double(s2);
      for (int q = 0; q < csize; ++q) {
        double* Yq = (q == crank) ? YC : cluster.map_shared_rank(YC, q);
        Yq[c] = y0;
        Yq[n + c] = y1;
        Yq[2 * n + c] = y2;
      }
    };
    const int ncb = (N + 31) / 32;
    const int nloc = (crank < ncb) ? (ncb - crank + csize - 1) / csize : 0;
    int rs = 1;
    if (nloc > 0) {
      int a = nloc, b = NW;
      while (b != 0) {
        const int t = a % b;
        a = b;
        b = t;
      }
      rs = NW / a;  // nloc * rs is a multiple of NW
      const int max_jobs = (int)((size_t)(2 + NW) * 32 * TS * sizeof(float) / (96 * sizeof(float2)));
      while (rs > 1 && (nloc * rs > max_jobs || 8 * rs > N)) rs >>= 1;
    }
    float2* part = reinterpret_cast<float2*>(panel);  // [job][3][32]
    for (int j = wid; j < nloc * rs; j += NW) {
      const int l = j / rs, ch = j - l * rs;
      const int c = 32 * (crank + csize * l) + lane;
      const int r0 = (int)((int64_t)N * ch / rs), r1 = (int)((int64_t)N * (ch + 1) / rs);
      // sums of V0 and V1 in the lanes of (h01, l01) (packed FP32x2), V2 in (h2, l2)
      float2 h01 = make_float2(0.f, 0.f), l01 = make_float2(0.f, 0.f);
      float h2 = 0.f, l2 = 0.f;
      if (c < N) {
        const int2 cc = cxy[c];
        for (int rb = r0; rb < r1; rb += 8) {
          const int cnt = min(8, r1 - rb);
          float2 a[8];
          a_batch_df(c, cc, rb, cnt, a);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            if (u < cnt) {
              const int r = rb + u;
              const float2 v0 = Vd[r], v1 = Vd[np + r];
              df_mac_x2(a[u], make_float2(v0.x, v1.x), make_float2(v0.y, v1.y), h01, l01);
              df_mac(a[u], Vd[2 * np + r], h2, l2);
            }
          }
        }
      }
      const float h0 = h01.x, l0 = l01.x, h1 = h01.y, l1 = l01.y;
      if (rs == 1) {
        if (c < N) write_y(c, make_float2(h0, l0), make_float2(h1, l1), make_float2(h2, l2));
      } else {
        part[(3 * j + 0) * 32 + lane] = make_float2(h0, l0);
        part[(3 * j + 1) * 32 + lane] = make_float2(h1, l1);
        part[(3 * j + 2) * 32 + lane] = make_float2(h2, l2);
      }
    }
    if (rs > 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < nloc * 32; t += NT) {
        const int l = t >> 5, ln = t & 31;
        const int c = 32 * (crank + csize * l) + ln;
        if (c >= N) continue;
        const float2* pj = part + (size_t)3 * 32 * (l * rs);
        float2 s0 = pj[ln], s1 = pj[32 + ln], s2 = pj[64 + ln];
        for (int ch = 1; ch < rs; ++ch) {
          pj += 3 * 32;
          s0 = df_add(s0, pj[ln]);
          s1 = df_add(s1, pj[32 + ln]);
          s2 = df_add(s2, pj[64 + ln]);
        }
        write_y(c, s0, s1, s2);
      }
    }
  }
  cluster.sync();
  // ---- Q^T A Q = A - Z V^T - V Z^T (compact WY, Q = H0 H1 H2 = I - V T V^T),
  // Y = A V, M = T^T (V^T Y) T, Z = Y T - V M / 2.  FP64: the projection cancels the
  // large affine part of K.
  double* Z0 = W;
  double* Z1 = W + n;
  double* Z2 = W + 2 * n;
  {
    __shared__ double s_T[9], s_M[9];
    const double* Vk[3] = {V0, V1, V2};
    const double* Yk[3] = {Y0, Y1, Y2};
    double vtv[3], vty[9];
    for (int a = 0; a < 3; ++a) {
      vtv[a] = 0.0;
      for (int b = 0; b < 3; ++b) vty[3 * a + b] = 0.0;
    }
    for (int i = threadIdx.x; i < N; i += NT) {
      vtv[0] += V0[i] * V1[i];
      vtv[1] += V0[i] * V2[i];
      vtv[2] += V1[i] * V2[i];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) vty[3 * a + b] += Vk[a][i] * Yk[b][i];
    }
    for (int a = 0; a < 3; ++a) vtv[a] = bsum<NT>(vtv[a], sh);
    for (int a = 0; a < 9; ++a) vty[a] = bsum<NT>(vty[a], sh);
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
    for (int i = threadIdx.x; i < N; i += NT) {  // Z = Y T - V M / 2
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
    for (int i = N + threadIdx.x; i < np; i += NT) Zd[i] = Zd[np + i] = Zd[2 * np + i] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += NT) {
      Zd[i] = df_split(Z0[i]);
      Zd[np + i] = df_split(Z1[i]);
      Zd[2 * np + i] = df_split(Z2[i]);
    }
    __syncthreads();
  }
  auto proj = [&](int r, int c) -> double {  // (Q^T A Q)[r][c], global indices
    double v = a_entry(r, c);
    v -= Z0[r] * V0[c] + V0[r] * Z0[c];
    v -= Z1[r] * V1[c] + V1[r] * Z1[c];
    v -= Z2[r] * V2[c] + V2[r] * Z2[c];
    return v;
  };
  // C[k][c] = (Q^T A Q)[k][c + 3], k < 3 (Y is no longer needed)
  double* C = YC;
  if (crank == 0) {
    for (int i = threadIdx.x; i < 3 * m; i += NT) {
      const int k = i / m, c = i - k * m;
      C[k * n + c] = proj(k, c + 3);
    }
  }
  // B22 by 32 x 32 tiles (I >= J), half a tile (16 columns) at a time: the lower
  // entries are written by columns, then mirrored through a per-warp shared tile.
  {
    float2* S = reinterpret_cast<float2*>(panel) + wid * 16 * 33;
    const int T = (m + 31) / 32;
    const int npairs = T * (T + 1) / 2;
    for (int pidx = crank * NW + wid; pidx < npairs; pidx += csize * NW) {
      int I = (int)((sqrtf(8.f * pidx + 1.f) - 1.f) * 0.5f);
      while ((I + 1) * (I + 2) / 2 <= pidx) ++I;
      while (I * (I + 1) / 2 > pidx) --I;
      const int J = pidx - I * (I + 1) / 2;
      const int r = 32 * I + lane;
      // the row's -Z_k and -V_k pairs and lattice coordinates
      const int rg = (r < m) ? r + 3 : 3;
      const int2 cr = cxy[rg];
      float2 nz[3], nv[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float2 zv = Zd[k * np + rg], vv = Vd[k * np + rg];
        nz[k] = make_float2(-zv.x, -zv.y);
        nv[k] = make_float2(-vv.x, -vv.y);
      }
      for (int h = 0; h < 2; ++h) {
        for (int qb = 0; qb < 16; qb += 8) {
          const int c0 = 32 * J + 16 * h + qb;
          if (c0 >= m) break;
          const int cnt = min(8, m - c0);
          float2 a[8];
          a_batch_df(rg, cr, c0 + 3, cnt, a);
          // A - Z V^T - V Z^T in double-float: entries of A up to ~1e5 cancel to B
          // entries ~1e2-1e4; the ~2^-48 |A| rounding leaves B within ~1e-11 of its
          // FP64 value, the interpolated field within ~1e-9 px.  Columns c, c + 1 in
          // the lanes of float2 pairs (packed FP32x2 instructions).
#pragma unroll
          for (int u = 0; u < 8; u += 2) {
            const int c = c0 + u;
            const bool in0 = u < cnt && r < m && r >= c;
            const bool in1 = u + 1 < cnt && r < m && r >= c + 1;
            if (in0 || in1) {
              const int cg0 = c + 3, cg1 = min(c + 4, N - 1);
              float2 sh = make_float2(a[u].x, a[u + 1].x), sl = make_float2(a[u].y, a[u + 1].y);
#pragma unroll
              for (int k = 0; k < 3; ++k) {
                const float2 v0 = Vd[k * np + cg0], v1 = Vd[k * np + cg1];
                const float2 z0 = Zd[k * np + cg0], z1 = Zd[k * np + cg1];
                df_mac_x2(nz[k], make_float2(v0.x, v1.x), make_float2(v0.y, v1.y), sh, sl);
                df_mac_x2(nv[k], make_float2(z0.x, z1.x), make_float2(z0.y, z1.y), sh, sl);
              }
              const float2 hi = __fadd2_rn(sh, sl);
              const float2 lo = __fadd2_rn(sl, df_neg2(__fadd2_rn(hi, df_neg2(sh))));
              if (in0) {
                const float2 sv = make_float2(hi.x, lo.x);
                __stcs(B2 + (int64_t)c * mp + r, sv);  // streaming: keeps L2 for the factor
                L32[(int64_t)c * mp + r] = sv.x;
                S[(qb + u) * 33 + lane] = sv;
              }
              if (in1) {
                const float2 sv = make_float2(hi.y, lo.y);
                __stcs(B2 + (int64_t)(c + 1) * mp + r, sv);
                L32[(int64_t)(c + 1) * mp + r] = sv.x;
                S[(qb + u + 1) * 33 + lane] = sv;
              }
            }
          }
        }
        __syncwarp();
#pragma unroll 4
        for (int st = 0; st < 16; ++st) {
          const int rr = 2 * st + (lane >> 4), qq = lane & 15;
          const int r2 = 32 * I + rr, c2 = 32 * J + 16 * h + qq;
          if (r2 < m && c2 < m && r2 > c2) __stcs(B2 + (int64_t)r2 * mp + c2, S[qq * 33 + rr]);
        }
        __syncwarp();
      }
    }
  }
  cluster.sync();  // the cluster's B tiles are in global memory, visible to rank 0
  if (crank != 0) return;
  // ---- FP32 Cholesky of B22
  if (!chol_factor<NT>(L32, m, mp, reinterpret_cast<float*>(smraw + lay.f2_off), &s_flag,
                       &s_next))
    return;

  // the diagonal tiles' inverses, after the per-warp partial sums of the solves
  float* dinv = panel + 64 * NW;
  chol_diag_inverses<NT>(L32, m, mp, dinv);

  // ---- outlier iterations with refined solves (x and y in lockstep)
  double* tx = W;
  double* ty = W + n;
  double* wx = W + 2 * n;
  double* wy = W + 3 * n;
  for (int r = threadIdx.x; r < lay.np; r += NT) {
    vx[r] = (r < N) ? ux[idx[r]] : 0.f;
    vy[r] = (r < N) ? uy[idx[r]] : 0.f;
    zx2[r] = zy2[r] = make_float2(0.f, 0.f);
    rx[r] = ry[r] = 0.f;
  }
  __syncthreads();
  int count[2] = {1, 1}, fixed[2] = {0, 0};
  bool done[2] = {false, false};
  bool converged_all = true;
  bool z_zero = true;
  int nsweeps = 0;
  while (true) {
    // g = Q^T u: rows 3.. as double-float for the refinement, rows 0..2 for a
    for (int i = threadIdx.x; i < N; i += NT) {
      tx[i] = (double)vx[i];
      ty[i] = (double)vy[i];
    }
    __syncthreads();
    apply_reflectors2<NT, false>(V, n, s_tau, N, tx, ty, sh);
    for (int i = threadIdx.x; i < m; i += NT) {
      gx2[i] = df_split(tx[i + 3]);
      gy2[i] = df_split(ty[i + 3]);
    }
    if (threadIdx.x < 3) {
      s_q1[threadIdx.x] = tx[threadIdx.x];
      s_q1[3 + threadIdx.x] = ty[threadIdx.x];
    }
    __syncthreads();
    // refine z (B z = g): FP32 Cholesky solves, double-float residuals
    bool conv = false;
    double prev = INFINITY;
    for (int it = 0; it < max_refine; ++it) {
      if (z_zero) {  // z = 0: rho = g
        for (int i = threadIdx.x; i < m; i += NT) {
          rx[i] = __fadd_rn(gx2[i].x, gx2[i].y);
          ry[i] = __fadd_rn(gy2[i].x, gy2[i].y);
        }
        __syncthreads();
        z_zero = false;
      } else {
        residual_df2<NT>(B2, m, mp, zx2, zy2, gx2, gy2, rx, ry);
      }
      chol_solve2<NT>(L32, m, mp, rx, ry, panel, dinv);
      ++nsweeps;
      double dmax = 0.0, zmax = 0.0;
      for (int i = threadIdx.x; i < m; i += NT) {
        if (!done[0]) zx2[i] = df_add(zx2[i], make_float2(rx[i], 0.f));
        if (!done[1]) zy2[i] = df_add(zy2[i], make_float2(ry[i], 0.f));
        dmax = fmax(dmax, fmax(done[0] ? 0.0 : fabs((double)rx[i]),
                               done[1] ? 0.0 : fabs((double)ry[i])));
        zmax = fmax(zmax, fmax(fabs((double)zx2[i].x), fabs((double)zy2[i].x)));
      }
      dmax = bmax<NT>(dmax, sh);
      zmax = bmax<NT>(zmax, sh);
      if (dmax == 0.0) {
        conv = true;
        break;
      }
      if (it >= 1) {
        // contraction of the FP32-preconditioned refinement, estimated from the last
        // two corrections; the remaining error is about contraction * dmax (1e-10 of
        // z keeps the interpolated displacements within ~1e-8 px)
        const double rho = dmax / prev;
        if (rho < 0.1 && rho * dmax <= 1e-10 * zmax) {
          conv = true;
          break;
        }
        if (it >= 2 && rho > 0.5) {  // at the residual floor
          conv = dmax <= 1e-9 * zmax;
          break;
        }
      }
      prev = dmax;
    }
    if (!conv) {
      converged_all = false;
      break;
    }
    // a = R^-1 (Q1^T u - C z) (R upper triangular); w = Q [0; z]
    double ax3[3], ay3[3];
    {
      double c6[6] = {0, 0, 0, 0, 0, 0};
      for (int i = threadIdx.x; i < m; i += NT) {
        const double zxv = df_to_double(zx2[i]), zyv = df_to_double(zy2[i]);
        for (int k = 0; k < 3; ++k) {
          c6[k] = fma(C[k * n + i], zxv, c6[k]);
          c6[3 + k] = fma(C[k * n + i], zyv, c6[3 + k]);
        }
      }
      for (int k = 0; k < 3; ++k) {
        const double2 s2 = bsum2<NT>(make_double2(c6[k], c6[3 + k]), sh);
        c6[k] = s2.x;
        c6[3 + k] = s2.y;
      }
      for (int k = 2; k >= 0; --k) {
        double sxk = s_q1[k] - c6[k], syk = s_q1[3 + k] - c6[3 + k];
        for (int j = k + 1; j < 3; ++j) {
          sxk -= s_R[k * 3 + j] * ax3[j];
          syk -= s_R[k * 3 + j] * ay3[j];
        }
        ax3[k] = sxk / s_R[k * 3 + k];
        ay3[k] = syk / s_R[k * 3 + k];
      }
      for (int i = threadIdx.x; i < N; i += NT) {
        wx[i] = (i < 3) ? 0.0 : df_to_double(zx2[i - 3]);
        wy[i] = (i < 3) ? 0.0 : df_to_double(zy2[i - 3]);
      }
      __syncthreads();
      apply_reflectors2<NT, true>(V, n, s_tau, N, wx, wy, sh);
    }
    // smoothed = u - lam w; outlier test (compute_tps_weights_iter, subdom.py:236-280)
    if (threadIdx.x == 0) s_bad[0] = s_bad[1] = 0;
    __syncthreads();
    double mxx = 0.0, mxy = 0.0;
    int bx = 0, by = 0;
    for (int r = threadIdx.x; r < N; r += NT) {
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
    mxx = bmax<NT>(mxx, sh);
    mxy = bmax<NT>(mxy, sh);
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
    for (int r = threadIdx.x; r < N; r += NT) {
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
    for (int r = threadIdx.x; r < N; r += NT) {
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
  if (threadIdx.x == 0 && sweeps != nullptr) sweeps[sd] = nsweeps;
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

extern "C" int fi_tps_phi_table2(float* table2, int64_t count, void* stream) {
  FI_REQUIRE(table2 && count > 0 && ((uintptr_t)table2 & 7) == 0,
             "fi_tps_phi_table2: bad arguments");
  k_phi_table2<<<1024, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<float2*>(table2), count);
  return check_launch("fi_tps_phi_table2");
}

// The tail of a launch of narrow blocks: with slots resident blocks per GPU, a solve
// of slots < nb < 2 slots subdomains (in decreasing size) runs the first wave on the
// caller's stream and the last nb - slots subdomains as clusters of two blocks on a
// side stream (fork and join by events), queued behind the first wave: a cluster
// shares a subdomain's build and projection over two blocks, so the small last
// subdomains, which otherwise run alone after the first wave, finish sooner.  One
// side stream and two events per host thread and device, created on first use.
struct TailStreams {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

static cudaError_t tail_streams(int dev, TailStreams** out) {
  static thread_local TailStreams per_dev[FI_SMEM_DEVICES];
  if (dev < 0 || dev >= FI_SMEM_DEVICES) return cudaErrorInvalidDevice;
  TailStreams& t = per_dev[dev];
  if (t.side == nullptr) {
    cudaError_t e = cudaStreamCreateWithFlags(&t.side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      t.side = nullptr;
      return e;
    }
  }
  *out = &t;
  return cudaSuccess;
}

extern "C" int fi_tps_solve_mp(const fi_tps_plan* plan, int nb_subdom, int max_members,
                               const double* cx, const double* cy, const float* ux,
                               const float* uy, const int32_t* counts, const int64_t* offsets,
                               const int32_t* indices, const int64_t* mat_offsets,
                               double* matrices, float* matrices32, const double* phi_table,
                               const float* phi_table2, int64_t table_size, const int32_t* cxy2,
                               const int32_t* c_on_lattice, double threshold, int use_threshold,
                               const int64_t* w_offsets, double* weights, double* smoothed_x,
                               double* smoothed_y, int32_t* iters, int32_t* nfixed,
                               int32_t* status, double* max_udiff, int32_t* sweeps,
                               const int32_t* order, void* stream) {
  FI_REQUIRE(plan && cx && cy && ux && uy && counts && offsets && indices && mat_offsets &&
                 matrices && matrices32 && w_offsets && weights && smoothed_x &&
                 smoothed_y &&
                 iters && nfixed && status && max_udiff,
             "fi_tps_solve_mp: null pointer");
  FI_REQUIRE(nb_subdom > 0, "fi_tps_solve_mp: no subdomain");
  FI_REQUIRE(((uintptr_t)matrices & 15) == 0 && ((uintptr_t)matrices32 & 15) == 0,
             "fi_tps_solve_mp: matrices must be 16-byte aligned");
  FI_REQUIRE(((uintptr_t)phi_table2 & 7) == 0, "fi_tps_solve_mp: phi_table2 must be 8-byte aligned");
  const int N = max_members > 4 ? max_members : 4;
  // 16 warps per subdomain when the subdomains fit in one wave of blocks (shorter
  // latency per subdomain), else two blocks of 8 warps per SM
  int dev = 0, nsm = 0;
  FI_CUDA_TRY(cudaGetDevice(&dev));
  FI_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const bool wide = nb_subdom <= nsm;
  const MpLayout lay(N, wide ? 16 : 8);
  const size_t smem = lay.bytes;
  FI_REQUIRE(smem <= 220 * 1024, "fi_tps_solve_mp: subdomain of %d vectors too large",
             max_members);
  static SmemLimit limit_wide, limit_narrow;
  if (wide)
    FI_CUDA_TRY(raise_smem_limit(k_tps_solve_mp<512>, smem, limit_wide));
  else
    FI_CUDA_TRY(raise_smem_limit(k_tps_solve_mp<256>, smem, limit_narrow));
  if (wide) {
    // clusters of S CTAs per subdomain while the subdomains leave SMs idle
    const int S = (4 * nb_subdom <= nsm) ? 4 : (2 * nb_subdom <= nsm) ? 2 : 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nb_subdom * S));
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)S;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FI_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_tps_solve_mp<512>, plan, cx, cy, ux, uy, counts,
                                   offsets, indices, mat_offsets, matrices, matrices32,
                                   phi_table, reinterpret_cast<const float2*>(phi_table2),
                                   table_size, cxy2, c_on_lattice, threshold,
                                   use_threshold, w_offsets, weights, smoothed_x, smoothed_y,
                                   iters, nfixed, status, max_udiff, sweeps, order, 60, N));
  } else {
    // resident narrow blocks per SM for this shared-memory size (queried once per
    // device and size: the call sits between the host's readback and the launch)
    static size_t occ_smem[FI_SMEM_DEVICES] = {};
    static int occ_blocks[FI_SMEM_DEVICES] = {};
    int per_sm = -1;
    {
      std::lock_guard<std::mutex> lock(smem_limit_mutex());
      if (dev < FI_SMEM_DEVICES && occ_smem[dev] == smem) per_sm = occ_blocks[dev];
    }
    if (per_sm < 0) {
      FI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tps_solve_mp<256>,
                                                                256, smem));
      std::lock_guard<std::mutex> lock(smem_limit_mutex());
      if (dev < FI_SMEM_DEVICES) {
        occ_smem[dev] = smem;
        occ_blocks[dev] = per_sm;
      }
    }
    const int slots = per_sm * nsm;
    const int head = (order != nullptr && slots > 0 && nb_subdom > slots &&
                      nb_subdom < 2 * slots) ? slots : nb_subdom;
    k_tps_solve_mp<256><<<head, 256, smem, (cudaStream_t)stream>>>(
        plan, cx, cy, ux, uy, counts, offsets, indices, mat_offsets, matrices, matrices32,
        phi_table, reinterpret_cast<const float2*>(phi_table2), table_size, cxy2, c_on_lattice,
        threshold, use_threshold, w_offsets, weights,
        smoothed_x, smoothed_y, iters, nfixed, status, max_udiff, sweeps, order, 60, N);
    if (head < nb_subdom) {  // the last subdomains in clusters of two, on the side stream
      FI_CUDA_TRY(cudaGetLastError());
      TailStreams* ts = nullptr;
      FI_CUDA_TRY(tail_streams(dev, &ts));
      FI_CUDA_TRY(cudaEventRecord(ts->fork, (cudaStream_t)stream));
      FI_CUDA_TRY(cudaStreamWaitEvent(ts->side, ts->fork, 0));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)(2 * (nb_subdom - head)));
      cfg.blockDim = dim3(256);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = ts->side;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 2;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      FI_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_tps_solve_mp<256>, plan, cx, cy, ux, uy, counts,
                                     offsets, indices, mat_offsets, matrices, matrices32,
                                     phi_table, reinterpret_cast<const float2*>(phi_table2),
                                     table_size, cxy2, c_on_lattice, threshold,
                                     use_threshold, w_offsets, weights, smoothed_x, smoothed_y,
                                     iters, nfixed, status, max_udiff, sweeps, order + head, 60,
                                     N));
      FI_CUDA_TRY(cudaEventRecord(ts->join, ts->side));
      FI_CUDA_TRY(cudaStreamWaitEvent((cudaStream_t)stream, ts->join, 0));
      return check_launch("fi_tps_solve_mp", 2);
    }
  }
  return check_launch("fi_tps_solve_mp");
}
