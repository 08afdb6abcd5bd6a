// Linear interpolation on the Delaunay triangulation of the PIV vectors, with the
// nearest vector outside their convex hull: the griddata path of apply_interp
// (calcul/interpolate/griddata.py:11-27, works/piv/singlepass.py:498-556), which
// upstream runs through scipy (Qhull Delaunay + barycentric interpolation, then a
// k-d tree for the points outside the hull).
//
// The centres are the valid vectors of a pass: each sits at its window-grid node
// (or half a pixel off it, the midpoint of an odd integer shift), so a node map of
// the grid replaces a spatial index.  For a query point q the Delaunay triangle
// containing q is found among the centres of the grid nodes around q: of the
// triangles of those centres that contain q, the Delaunay one minimises the linear
// interpolant of the lifted heights |p - q|^2 at q (the lower convex hull of the
// lifted points); its circumcircle must then hold no other gathered centre and lie
// inside the gathered window (else the window grows).  All predicates are exact
// integer arithmetic on doubled coordinates (PIV positions are half-integers).
// Where four or more centres are cocircular (a regular grid's cells) several
// triangulations are Delaunay; upstream takes Qhull's, here the triangle with the
// smallest vertex indices, and the query is flagged.
#include "fi_common.cuh"

namespace fi {

namespace {

constexpr int GD_RMAX = 8;                        // window half-width in grid steps
                                                  // (then the whole grid)
constexpr int GD_MAXC = 64;                       // nearest centres of the window kept

struct GdArgs {
  const double* cx;
  const double* cy;
  const float* ux;
  const float* uy;
  int nc;
  const int32_t* ixvecs;
  int nx;
  const int32_t* iyvecs;
  int ny;
  const int32_t* nodemap;   // [ny][nx] centre index or -1
  const int2* cxy;          // doubled centre coordinates (exact: half-integers)
  const int2* hull_left;    // left chain of the hull, increasing Y (doubled coords)
  const int2* hull_right;   // right chain
  const int32_t* hull_n;    // [2]: lengths
  const double* px;
  const double* py;
  int npts;
  double* out_x;
  double* out_y;
  int32_t* rx;
  int32_t* ry;
  uint8_t* flags;
  int32_t* status;
};

__device__ __forceinline__ long long orient2(long long ax, long long ay, long long bx,
                                             long long by, long long cx, long long cy) {
  return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

// doubled coordinates of a centre (exact: positions are half-integers)
__device__ __forceinline__ int2 centre_xy2(const GdArgs& a, int i) { return a.cxy[i]; }

// largest k with 2 * v[k] <= X2 (-1 if none); v increasing
__device__ __forceinline__ int floor_index(const int32_t* v, int n, long long X2) {
  int lo = 0, hi = n;  // first index with 2 v > X2
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (2LL * v[mid] > X2) hi = mid; else lo = mid + 1;
  }
  return lo - 1;
}

// Position of q against the convex hull (chains of the hull, increasing Y): 1
// strictly outside, 2 on a hull edge (*e0, *e1: the chain vertices around q on it),
// 0 inside.
__device__ int hull_position(const GdArgs& a, long long X, long long Y, int2* e0, int2* e1) {
  const int nl = a.hull_n[0], nr = a.hull_n[1];
  const int2* L = a.hull_left;
  const int2* R = a.hull_right;
  if (Y < L[0].y || Y > L[nl - 1].y) return 1;
  // going up, the inside is to the right of the left chain (o <= 0) and to the left
  // of the right chain (o >= 0)
  int res = 0;
  for (int side = 0; side < 2; ++side) {
    const int2* C = side == 0 ? L : R;
    const int n = side == 0 ? nl : nr;
    if (n == 1) {
      if (side == 0 ? (X < C[0].x) : (X > C[0].x)) return 1;
      continue;
    }
    // the segment arriving at the first vertex with y >= Y (its lower end below Y,
    // or the first segment)
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (C[mid].y >= Y) hi = mid; else lo = mid + 1;
    }
    lo = min(max(lo - 1, 0), n - 2);
    if (C[lo].y == C[lo + 1].y) {  // horizontal (bottom or top) edge at Y
      const int xmin = min(C[lo].x, C[lo + 1].x), xmax = max(C[lo].x, C[lo + 1].x);
      if (side == 0 ? (X < xmin) : (X > xmax)) return 1;
      if (Y == C[lo].y && X >= xmin && X <= xmax) {
        *e0 = C[lo];
        *e1 = C[lo + 1];
        res = 2;
      }
      continue;
    }
    const long long o = orient2(C[lo].x, C[lo].y, C[lo + 1].x, C[lo + 1].y, X, Y);
    if (side == 0 ? (o > 0) : (o < 0)) return 1;
    if (o == 0) {
      *e0 = C[lo];
      *e1 = C[lo + 1];
      res = 2;
    }
  }
  return res;
}

__global__ void k_gd_nodemap(const int32_t* sel, const double* cx, const double* cy, int nc,
                             int32_t* nodemap, int2* cxy, int nnodes, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const int w = sel[i];
  const double X = 2.0 * cx[i], Y = 2.0 * cy[i];
  if (w < 0 || w >= nnodes || X != rint(X) || Y != rint(Y) || fabs(X) > 1e9 || fabs(Y) > 1e9) {
    atomicExch(status, w < 0 || w >= nnodes ? 3 : 1);
    cxy[i] = make_int2(0, 0);
    return;
  }
  cxy[i] = make_int2((int)X, (int)Y);
  nodemap[w] = i;
}

// Convex hull of the centres.  Every hull vertex is extreme in its grid row or in
// its grid column (a centre with grid neighbours on both sides in both directions is
// inside them: the half-pixel offsets are below half a grid step), so the chains of
// Andrew's monotone algorithm (increasing Y) are built from those extremes, sorted
// in shared memory (bitonic).  One block.
constexpr int GD_HULL_MAX = 4096;  // row and column extremes (2 (nx + ny))

__global__ void __launch_bounds__(1024) k_gd_hull(GdArgs a, int2* left, int2* right,
                                                  int32_t* hull_n) {
  __shared__ long long key[GD_HULL_MAX];
  const int ny = a.ny, nx = a.nx;
  const int m = 2 * (nx + ny);
  int m2 = 1;
  while (m2 < m) m2 <<= 1;
  const long long NONE = 0x7fffffffffffffffLL;
  auto pack = [](int2 p) { return ((long long)p.y << 32) | (long long)(unsigned)(p.x + 0x40000000); };
  for (int t = threadIdx.x; t < m2; t += blockDim.x) {
    long long k = NONE;
    if (t < 2 * ny) {  // row extremes
      const int r = t >> 1;
      const bool hi = t & 1;
      int2 best = make_int2(0, 0);
      bool any = false;
      for (int c = 0; c < nx; ++c) {
        const int i = a.nodemap[r * nx + c];
        if (i < 0) continue;
        const int2 p = centre_xy2(a, i);
        if (!any || (hi ? (p.x > best.x || (p.x == best.x && p.y > best.y))
                        : (p.x < best.x || (p.x == best.x && p.y < best.y))))
          best = p;
        any = true;
      }
      if (any) k = pack(best);
    } else if (t < m) {  // column extremes
      const int c = (t - 2 * ny) >> 1;
      const bool hi = (t - 2 * ny) & 1;
      int2 best = make_int2(0, 0);
      bool any = false;
      for (int r = 0; r < ny; ++r) {
        const int i = a.nodemap[r * nx + c];
        if (i < 0) continue;
        const int2 p = centre_xy2(a, i);
        if (!any || (hi ? (p.y > best.y || (p.y == best.y && p.x > best.x))
                        : (p.y < best.y || (p.y == best.y && p.x < best.x))))
          best = p;
        any = true;
      }
      if (any) k = pack(best);
    }
    key[t] = k;
  }
  __syncthreads();
  // bitonic sort of the keys (Y, then X)
  for (int size = 2; size <= m2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < m2; t += blockDim.x) {
        const int u = t ^ stride;
        if (u > t) {
          const bool up = (t & size) == 0;
          const long long x = key[t], y = key[u];
          if ((x > y) == up) {
            key[t] = y;
            key[u] = x;
          }
        }
      }
      __syncthreads();
    }
  if (threadIdx.x != 0) return;
  // going up, the left chain turns clockwise (orient < 0) at each vertex and the
  // right chain counter-clockwise: pop the vertices that break the turn
  int nl = 0, nr = 0;
  long long prev = NONE;
  for (int k = 0; k < m2; ++k) {
    const long long kk = key[k];
    if (kk == NONE) break;
    if (kk == prev) continue;
    prev = kk;
    const int2 p = make_int2((int)(kk & 0xffffffffLL) - 0x40000000, (int)(kk >> 32));
    while (nl >= 2 && orient2(left[nl - 2].x, left[nl - 2].y, left[nl - 1].x, left[nl - 1].y,
                              p.x, p.y) >= 0)
      --nl;
    left[nl++] = p;
    while (nr >= 2 && orient2(right[nr - 2].x, right[nr - 2].y, right[nr - 1].x,
                              right[nr - 1].y, p.x, p.y) <= 0)
      --nr;
    right[nr++] = p;
  }
  hull_n[0] = nl;
  hull_n[1] = nr;
}

struct Cand {
  int dx, dy;   // doubled coordinates relative to q
  int idx;      // centre index
  int d2;       // squared distance (doubled units; windows of at most 16 steps)
};

__device__ __forceinline__ Cand make_cand(const GdArgs& a, int i, long long X, long long Y) {
  const int2 p = centre_xy2(a, i);
  Cand c;
  c.dx = (int)(p.x - X);
  c.dy = (int)(p.y - Y);
  c.idx = i;
  c.d2 = (int)min((long long)c.dx * c.dx + (long long)c.dy * c.dy, 0x3fffffffLL);
  return c;
}

// makes (A, B, C) counter-clockwise
__device__ __forceinline__ void orient_ccw(Cand& A, Cand& B, Cand& C) {
  if (orient2(A.dx, A.dy, B.dx, B.dy, C.dx, C.dy) < 0) {
    const Cand t = B;
    B = C;
    C = t;
  }
}

// q (the origin) in the closed triangle: barycentric numerators o (of A, B, C in
// counter-clockwise order as given or after swapping B and C) and their sum *D > 0
__device__ __forceinline__ bool contains_q(const Cand& A0, const Cand& B0, const Cand& C0,
                                           long long (&o)[3], long long* D) {
  Cand A = A0, B = B0, C = C0;
  long long d = orient2(A.dx, A.dy, B.dx, B.dy, C.dx, C.dy);
  if (d == 0) return false;
  if (d < 0) {
    const Cand t = B;
    B = C;
    C = t;
    d = -d;
  }
  const long long oa = orient2(0, 0, B.dx, B.dy, C.dx, C.dy);
  if (oa < 0) return false;
  const long long ob = orient2(A.dx, A.dy, 0, 0, C.dx, C.dy);
  if (ob < 0) return false;
  const long long oc = d - oa - ob;
  if (oc < 0) return false;
  // weights in the order of the arguments
  const bool swapped = orient2(A0.dx, A0.dy, B0.dx, B0.dy, C0.dx, C0.dy) < 0;
  o[0] = oa;
  o[1] = swapped ? oc : ob;
  o[2] = swapped ? ob : oc;
  *D = d;
  return true;
}

// lifted interpolant numerator at q: sum o_i |p_i - q|^2
__device__ __forceinline__ __int128 lifted(const Cand& A, const Cand& B, const Cand& C,
                                           const long long (&o)[3]) {
  return (__int128)o[0] * (long long)A.d2 + (__int128)o[1] * (long long)B.d2 +
         (__int128)o[2] * (long long)C.d2;
}

// incircle(A, B, C, P) > 0 <=> P strictly inside the circle of (A, B, C)
// (counter-clockwise)
// Window coordinates stay below 2^13 (at most 8 grid steps of at most 64 px, doubled),
// so the terms stay below 2^56: exact in 64-bit integers.
__device__ __forceinline__ long long incircle(const Cand& A, const Cand& B, const Cand& C,
                                              const Cand& P) {
  const long long adx = A.dx - P.dx, ady = A.dy - P.dy;
  const long long bdx = B.dx - P.dx, bdy = B.dy - P.dy;
  const long long cdx = C.dx - P.dx, cdy = C.dy - P.dy;
  return (adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) -
         (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady) +
         (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady);
}

__device__ __forceinline__ void sort3(int (&s)[3]) {
  for (int u = 0; u < 2; ++u)
    for (int v = u + 1; v < 3; ++v)
      if (s[v] < s[u]) {
        const int w = s[u];
        s[u] = s[v];
        s[v] = w;
      }
}

// two triangles weight the centres alike (zero weights for the others)
__device__ __forceinline__ bool same_weights(const int (&ti)[3], const long long (&to)[3],
                                             long long tD, const int (&bi)[3],
                                             const long long (&bo)[3], long long bD) {
  for (int u = 0; u < 3; ++u) {
    long long w = 0;
    for (int v = 0; v < 3; ++v)
      if (bi[v] == ti[u]) w = bo[v];
    if ((__int128)to[u] * bD != (__int128)w * tD) return false;
  }
  for (int v = 0; v < 3; ++v) {
    long long w = 0;
    for (int u = 0; u < 3; ++u)
      if (ti[u] == bi[v]) w = to[u];
    if ((__int128)bo[v] * tD != (__int128)w * bD) return false;
  }
  return true;
}

__global__ void __launch_bounds__(128) k_gd_interp(GdArgs a) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.npts) return;
  const double qx2 = 2.0 * a.px[q], qy2 = 2.0 * a.py[q];
  if (qx2 != rint(qx2) || qy2 != rint(qy2) || fabs(qx2) > 1e9 || fabs(qy2) > 1e9) {
    atomicExch(a.status, 1);  // off the half-integer lattice
    return;
  }
  const long long X = (long long)qx2, Y = (long long)qy2;
  int2 e0 = make_int2(0, 0), e1 = make_int2(0, 0);
  const int hpos = hull_position(a, X, Y, &e0, &e1);
  const bool outside = hpos == 1;
  const int i0 = floor_index(a.ixvecs, a.nx, X);
  const int j0 = floor_index(a.iyvecs, a.ny, Y);
  Cand cand[GD_MAXC];
  uint8_t flag = 0;
  int T[3] = {-1, -1, -1};  // a triangle (centre indices) containing q
  for (int r = 1; r <= GD_RMAX + 1; ++r) {
    // nodes of columns [i0 - r + 1, i0 + r] and rows [j0 - r + 1, j0 + r]; past
    // GD_RMAX steps (a large region without vectors) the whole grid
    const bool all = r > GD_RMAX;
    const int c0 = all ? 0 : max(i0 - r + 1, 0), c1 = all ? a.nx - 1 : min(i0 + r, a.nx - 1);
    const int r0 = all ? 0 : max(j0 - r + 1, 0), r1 = all ? a.ny - 1 : min(j0 + r, a.ny - 1);
    int n = 0;
    for (int row = r0; row <= r1; ++row)
      for (int col = c0; col <= c1; ++col) {
        const int i = a.nodemap[row * a.nx + col];
        if (i < 0) continue;
        const int2 p = centre_xy2(a, i);
        Cand c;
        c.dx = (int)(p.x - X);
        c.dy = (int)(p.y - Y);
        c.idx = i;
        const long long d2 = (long long)c.dx * c.dx + (long long)c.dy * c.dy;
        if (d2 > 0x3fffffffLL) continue;  // beyond any window of GD_RMAX steps
        c.d2 = (int)d2;
        // insertion by (d2, idx); the nearest GD_MAXC are kept (the certification
        // below scans the whole window again)
        if (n == GD_MAXC) {
          const Cand& l = cand[GD_MAXC - 1];
          if (l.d2 < c.d2 || (l.d2 == c.d2 && l.idx < c.idx)) continue;
          --n;
        }
        int k = n++;
        while (k > 0 && (cand[k - 1].d2 > c.d2 || (cand[k - 1].d2 == c.d2 && cand[k - 1].idx > c.idx))) {
          cand[k] = cand[k - 1];
          --k;
        }
        cand[k] = c;
      }
    // exclusive bounds of the region the window covers: a centre of column c has
    // 2 ixvecs[c] <= X2 <= 2 ixvecs[c] + 1
    const double xlo = (!all && i0 - r >= 0) ? 2.0 * a.ixvecs[i0 - r] + 1.0 - (double)X : -1e300;
    const double xhi = (!all && i0 + r + 1 < a.nx) ? 2.0 * a.ixvecs[i0 + r + 1] - (double)X : 1e300;
    const double ylo = (!all && j0 - r >= 0) ? 2.0 * a.iyvecs[j0 - r] + 1.0 - (double)Y : -1e300;
    const double yhi = (!all && j0 + r + 1 < a.ny) ? 2.0 * a.iyvecs[j0 + r + 1] - (double)Y : 1e300;
    if (outside) {
      // nearest centre (ties: smallest index), certified when the nearest distance
      // is below the distance to the uncovered region
      if (n == 0) continue;
      const double d = sqrt((double)cand[0].d2);  // the nearest is always kept
      const double margin = fmin(fmin(-xlo, xhi), fmin(-ylo, yhi));
      if (d >= margin * (1.0 - 1e-12)) continue;
      if (n > 1 && cand[1].d2 == cand[0].d2) flag |= 2;
      const int i = cand[0].idx;
      a.out_x[q] = (double)a.ux[i];
      a.out_y[q] = (double)a.uy[i];
      if (a.rx) a.rx[q] = (int32_t)rint((double)a.ux[i]);
      if (a.ry) a.ry[q] = (int32_t)rint((double)a.uy[i]);
      if (a.flags) a.flags[q] = flag;
      return;
    }
    // q on a centre: its value (the weights of every triangle at that vertex)
    if (n > 0 && cand[0].d2 == 0) {
      const int i = cand[0].idx;
      a.out_x[q] = (double)a.ux[i];
      a.out_y[q] = (double)a.uy[i];
      if (a.rx) a.rx[q] = (int32_t)rint((double)a.ux[i]);
      if (a.ry) a.ry[q] = (int32_t)rint((double)a.uy[i]);
      if (a.flags) a.flags[q] = flag;
      return;
    }
    if (hpos == 2) {
      // q on a hull edge: the Delaunay edge containing q joins the nearest centres on
      // that line on either side (the chain vertices e0, e1 unless collinear centres
      // lie between); certified when both lie in the covered region
      const long long ux_ = e1.x - e0.x, uy_ = e1.y - e0.y;
      // positions along the line, relative to q (scaled by |e1 - e0|^2)
      long long t_lo = (e0.x - X) * ux_ + (e0.y - Y) * uy_;  // < 0
      long long t_hi = (e1.x - X) * ux_ + (e1.y - Y) * uy_;  // > 0
      int i_lo = -1, i_hi = -1;
      int2 p_lo = e0, p_hi = e1;
      for (int row = r0; row <= r1; ++row)
        for (int col = c0; col <= c1; ++col) {
          const int i = a.nodemap[row * a.nx + col];
          if (i < 0) continue;
          const int2 p = centre_xy2(a, i);
          const long long px_ = p.x - X, py_ = p.y - Y;  // relative to q
          if ((px_ + X - e0.x) * uy_ - (py_ + Y - e0.y) * ux_ != 0) continue;  // off the line
          const long long t = px_ * ux_ + py_ * uy_;
          if (t < 0 && t >= t_lo) {
            if (t > t_lo || i_lo < 0 || i < i_lo) {
              t_lo = t;
              i_lo = i;
              p_lo = p;
            }
          } else if (t > 0 && t <= t_hi) {
            if (t < t_hi || i_hi < 0 || i < i_hi) {
              t_hi = t;
              i_hi = i;
              p_hi = p;
            }
          }
        }
      auto covered = [&](int2 p) {
        const double dx = (double)(p.x - X), dy = (double)(p.y - Y);
        return dx > xlo && dx < xhi && dy > ylo && dy < yhi;
      };
      if (i_lo < 0 || i_hi < 0 || !covered(p_lo) || !covered(p_hi)) continue;
      const double w = (double)(-t_lo) / (double)(t_hi - t_lo);  // weight of the high end
      const double vx = (1.0 - w) * (double)a.ux[i_lo] + w * (double)a.ux[i_hi];
      const double vy = (1.0 - w) * (double)a.uy[i_lo] + w * (double)a.uy[i_hi];
      a.out_x[q] = vx;
      a.out_y[q] = vy;
      if (a.rx) a.rx[q] = (int32_t)rint(vx);
      if (a.ry) a.ry[q] = (int32_t)rint(vy);
      if (a.flags) a.flags[q] = flag;
      return;
    }
    // a triangle of centres containing q: among the nearest k, the one with the
    // smallest lifted interpolant at q (kept from the previous window when found)
    if (T[0] < 0) {
      for (int kk = 0; kk < 3 && T[0] < 0; ++kk) {
        const int k = min(n, kk == 0 ? 12 : (kk == 1 ? 24 : GD_MAXC));
        if (kk > 0 && k <= (kk == 1 ? 12 : 24)) break;
        __int128 bN = 0;
        long long bD = 1;
        for (int ia = 0; ia < k; ++ia)
          for (int ib = ia + 1; ib < k; ++ib)
            for (int ic = ib + 1; ic < k; ++ic) {
              const Cand &A = cand[ia], &B = cand[ib], &Cc = cand[ic];
              long long o[3];
              long long D;
              if (!contains_q(A, B, Cc, o, &D)) continue;
              const __int128 N = lifted(A, B, Cc, o);
              if (T[0] < 0 || N * bD < bN * D) {
                bN = N;
                bD = D;
                T[0] = A.idx;
                T[1] = B.idx;
                T[2] = Cc.idx;
              }
            }
      }
      if (T[0] < 0) continue;
    }
    // Lawson descent: while a centre of the window lies strictly inside the
    // circumcircle of T (its lifted point is below T's plane), replace T by the
    // triangle of that centre and an edge of T that contains q (its plane at q is
    // lower); ends on a triangle whose circumcircle holds no centre of the window
    bool certified = false;
    for (int it = 0; it < 256; ++it) {
      Cand A = make_cand(a, T[0], X, Y), B = make_cand(a, T[1], X, Y), Cc = make_cand(a, T[2], X, Y);
      orient_ccw(A, B, Cc);
      int inside = -1;
      long long best_det = 0;
      for (int row = r0; row <= r1; ++row)
        for (int col = c0; col <= c1; ++col) {
          const int i = a.nodemap[row * a.nx + col];
          if (i < 0 || i == A.idx || i == B.idx || i == Cc.idx) continue;
          const Cand P = make_cand(a, i, X, Y);
          const long long det = incircle(A, B, Cc, P);
          if (det > best_det || (det > 0 && det == best_det && i < inside)) {
            best_det = det;
            inside = i;
          }
        }
      if (inside < 0) {
        certified = true;
        break;
      }
      const Cand P = make_cand(a, inside, X, Y);
      // of the sub-triangles (P, B, C), (A, P, C), (A, B, P) containing q, the one
      // with the smallest lifted interpolant at q (the lower hull of A, B, C, P over q)
      int nT[3] = {-1, -1, -1};
      __int128 bN = 0;
      long long bD = 1;
      for (int e = 0; e < 3; ++e) {
        const Cand& U = (e == 0) ? P : A;
        const Cand& V = (e == 1) ? P : B;
        const Cand& W = (e == 2) ? P : Cc;
        long long o[3], D;
        if (!contains_q(U, V, W, o, &D)) continue;
        const __int128 N = lifted(U, V, W, o);
        if (nT[0] < 0 || N * bD < bN * D) {
          bN = N;
          bD = D;
          nT[0] = U.idx;
          nT[1] = V.idx;
          nT[2] = W.idx;
        }
      }
      if (nT[0] < 0) break;  // cannot happen for a triangle containing q
      T[0] = nT[0];
      T[1] = nT[1];
      T[2] = nT[2];
    }
    if (!certified) continue;
    // the circumcircle must lie in the covered region (else centres outside the
    // window could be inside it)
    Cand A = make_cand(a, T[0], X, Y), B = make_cand(a, T[1], X, Y), Cc = make_cand(a, T[2], X, Y);
    orient_ccw(A, B, Cc);
    {
      // circumcentre numerators in exact integers, the test in float with a margin
      // far above its rounding (conservative: a rejected circle only grows the window)
      const long long ax = A.dx, ay = A.dy, bx = B.dx, by = B.dy, cx = Cc.dx, cy = Cc.dy;
      const long long dd = 2 * (ax * (by - cy) + bx * (cy - ay) + cx * (ay - by));
      const long long a2 = ax * ax + ay * ay, b2 = bx * bx + by * by, c2 = cx * cx + cy * cy;
      const float ux = (float)(a2 * (by - cy) + b2 * (cy - ay) + c2 * (ay - by)) / (float)dd;
      const float uy = (float)(a2 * (cx - bx) + b2 * (ax - cx) + c2 * (bx - ax)) / (float)dd;
      const float ex = (float)ax - ux, ey = (float)ay - uy;
      const float rad = sqrtf(ex * ex + ey * ey);
      const float mg = 1e-4f * (fabsf(ux) + fabsf(uy) + rad + 1.f);
      if (!(ux - rad - mg > (float)xlo && ux + rad + mg < (float)xhi &&
            uy - rad - mg > (float)ylo && uy + rad + mg < (float)yhi))
        continue;
    }
    // cocircular centres (on the circumcircle): the triangles of that set containing
    // q are all Delaunay; take the smallest sorted index triple, flag the query when
    // their weights differ
    int S[8];
    int ns = 0;
    S[ns++] = A.idx;
    S[ns++] = B.idx;
    S[ns++] = Cc.idx;
    for (int row = r0; row <= r1 && ns < 8; ++row)
      for (int col = c0; col <= c1 && ns < 8; ++col) {
        const int i = a.nodemap[row * a.nx + col];
        if (i < 0 || i == A.idx || i == B.idx || i == Cc.idx) continue;
        if (incircle(A, B, Cc, make_cand(a, i, X, Y)) == 0) S[ns++] = i;
      }
    int best[3] = {T[0], T[1], T[2]};
    sort3(best);
    long long wref_o[3], wref_D;
    int wref_i[3];
    bool tie = false;
    {
      Cand P0 = make_cand(a, best[0], X, Y), P1 = make_cand(a, best[1], X, Y), P2 = make_cand(a, best[2], X, Y);
      contains_q(P0, P1, P2, wref_o, &wref_D);
      wref_i[0] = P0.idx; wref_i[1] = P1.idx; wref_i[2] = P2.idx;
    }
    if (ns > 3) {
      long long o0[3], D0;
      int i0_[3];
      {
        Cand P0 = make_cand(a, best[0], X, Y), P1 = make_cand(a, best[1], X, Y), P2 = make_cand(a, best[2], X, Y);
        contains_q(P0, P1, P2, o0, &D0);
        i0_[0] = P0.idx; i0_[1] = P1.idx; i0_[2] = P2.idx;
      }
      for (int u = 0; u < ns; ++u)
        for (int v = u + 1; v < ns; ++v)
          for (int w = v + 1; w < ns; ++w) {
            Cand P0 = make_cand(a, S[u], X, Y), P1 = make_cand(a, S[v], X, Y), P2 = make_cand(a, S[w], X, Y);
            long long o[3], D;
            if (!contains_q(P0, P1, P2, o, &D)) continue;
            const int ti[3] = {P0.idx, P1.idx, P2.idx};
            if (!same_weights(ti, o, D, i0_, o0, D0)) tie = true;
            int st[3] = {ti[0], ti[1], ti[2]};
            sort3(st);
            if (st[0] < best[0] || (st[0] == best[0] && (st[1] < best[1] || (st[1] == best[1] && st[2] < best[2])))) {
              best[0] = st[0]; best[1] = st[1]; best[2] = st[2];
              for (int z = 0; z < 3; ++z) { wref_o[z] = o[z]; wref_i[z] = ti[z]; }
              wref_D = D;
            }
          }
    }
    if (tie) flag |= 1;
    const double Dd = (double)wref_D;
    double vx = 0.0, vy = 0.0;
    for (int z = 0; z < 3; ++z) {
      const double l = (double)wref_o[z] / Dd;
      vx += l * (double)a.ux[wref_i[z]];
      vy += l * (double)a.uy[wref_i[z]];
    }
    a.out_x[q] = vx;
    a.out_y[q] = vy;
    if (a.rx) a.rx[q] = (int32_t)rint(vx);
    if (a.ry) a.ry[q] = (int32_t)rint(vy);
    if (a.flags) a.flags[q] = flag;
    return;
  }
  atomicExch(a.status, 2);  // no certified triangle (cannot happen with the whole grid)
  a.out_x[q] = a.out_y[q] = NAN;
  if (a.rx) a.rx[q] = 0;
  if (a.ry) a.ry[q] = 0;
}

__global__ void k_gd_fill(int32_t* p, int n, int32_t v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

}  // namespace fi

using namespace fi;

extern "C" int fi_griddata(const double* cx, const double* cy, const float* ux, const float* uy,
                           const int32_t* selection, int num_centers, const int32_t* ixvecs,
                           int nx, const int32_t* iyvecs, int ny, const double* px,
                           const double* py, int npts, int32_t* scratch, double* out_x,
                           double* out_y, int32_t* rx, int32_t* ry, uint8_t* flags,
                           int32_t* status, void* stream) {
  FI_REQUIRE(cx && cy && ux && uy && selection && ixvecs && iyvecs && px && py && scratch &&
                 out_x && out_y && status,
             "fi_griddata: null pointer");
  FI_REQUIRE(num_centers > 0 && nx > 0 && ny > 0 && npts > 0, "fi_griddata: bad sizes");
  FI_REQUIRE(((uintptr_t)scratch & 7) == 0, "fi_griddata: scratch must be 8-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  const int nnodes = nx * ny;
  FI_REQUIRE(2 * (nx + ny) <= GD_HULL_MAX, "fi_griddata: window grid of %d x %d too large",
             nx, ny);
  FI_REQUIRE(num_centers <= nnodes, "fi_griddata: more centres than grid nodes");
  int32_t* nodemap = scratch;
  int2* cxy = reinterpret_cast<int2*>(scratch + ((nnodes + 1) & ~1));
  int2* left = cxy + nnodes;
  int2* right = left + 2 * (nx + ny);
  int32_t* hull_n = reinterpret_cast<int32_t*>(right + 2 * (nx + ny));
  GdArgs a{cx, cy, ux, uy, num_centers, ixvecs, nx, iyvecs, ny, nodemap, cxy, left, right,
           hull_n, px, py, npts, out_x, out_y, rx, ry, flags, status};
  k_gd_fill<<<(nnodes + 255) / 256, 256, 0, s>>>(nodemap, nnodes, -1);
  k_gd_fill<<<1, 32, 0, s>>>(status, 1, 0);
  k_gd_nodemap<<<(num_centers + 255) / 256, 256, 0, s>>>(selection, cx, cy, num_centers,
                                                         nodemap, cxy, nnodes, status);
  k_gd_hull<<<1, 1024, 0, s>>>(a, left, right, hull_n);
  k_gd_interp<<<(npts + 127) / 128, 128, 0, s>>>(a);
  return check_launch("fi_griddata", 5);
}

extern "C" int64_t fi_griddata_scratch_ints(int nx, int ny) {
  return (int64_t)((nx * ny + 1) & ~1) + 2LL * nx * ny + 8LL * (nx + ny) + 2;
}
