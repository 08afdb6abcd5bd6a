// Grids of the half-integer lattice.  Window centres (and the positions a field is
// interpolated at) are lattice points (2x, 2y integers) on regular grids, so the
// distances between two of them take few values: with g the greatest common divisor
// of the offsets from an origin along an axis, every offset is g times a small
// integer, and the kernel value of a pair depends only on the two integer offsets.
// A block finds g and the extent of its points, per axis, with this reduction, and
// keeps the kernel values of every offset of that extent in shared memory instead of
// gathering them from the lattice table in memory, one sector per pair.
#pragma once

#include <cuda_runtime.h>

#include <climits>

namespace fi {

__device__ __forceinline__ unsigned gcd_u32(unsigned a, unsigned b) {
  while (b != 0u) {
    const unsigned t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// Accumulates the lattice offset (dx, dy) into v = {gcd |dx|, gcd |dy|, min dx,
// max dx, min dy, max dy} (start from lat_grid_init).
__device__ __forceinline__ void lat_grid_init(int (&v)[6]) {
  v[0] = v[1] = 0;
  v[2] = v[4] = INT_MAX;
  v[3] = v[5] = INT_MIN;
}

__device__ __forceinline__ void lat_grid_add(int (&v)[6], int dx, int dy) {
  v[0] = (int)gcd_u32((unsigned)v[0], (unsigned)(dx < 0 ? -dx : dx));
  v[1] = (int)gcd_u32((unsigned)v[1], (unsigned)(dy < 0 ? -dy : dy));
  v[2] = min(v[2], dx);
  v[3] = max(v[3], dx);
  v[4] = min(v[4], dy);
  v[5] = max(v[5], dy);
}

__device__ __forceinline__ void lat_grid_merge(int (&v)[6], const int (&w)[6]) {
  v[0] = (int)gcd_u32((unsigned)v[0], (unsigned)w[0]);
  v[1] = (int)gcd_u32((unsigned)v[1], (unsigned)w[1]);
  v[2] = min(v[2], w[2]);
  v[3] = max(v[3], w[3]);
  v[4] = min(v[4], w[4]);
  v[5] = max(v[5], w[5]);
}

// Block-wide merge of every thread's v; every thread returns with the result.
// scratch: 6 ints per warp of the block (at most 32 warps), not otherwise in use
// between the two barriers of this call.
__device__ __forceinline__ void lat_grid_block(int (&v)[6], int* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    int w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = __shfl_xor_sync(0xffffffffu, v[k], o);
    lat_grid_merge(v, w);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) scratch[6 * wid + k] = v[k];
  }
  __syncthreads();
  lat_grid_init(v);
  for (int q = 0; q < nw; ++q) {
    int w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = scratch[6 * q + k];
    lat_grid_merge(v, w);
  }
  __syncthreads();
}

// Table geometry of a reduced grid: step (gx, gy) >= 1 and the numbers of offsets
// wx, wy along each axis (offsets 0 .. w - 1 in steps).  Usable when the table fits
// `capacity` entries and every offset's 4 r^2 = (gx a)^2 + (gy b)^2 stays a 32-bit
// index below `tsize` (then no pair of the grid falls beyond the lattice table).
struct LatTable {
  int gx, gy, wx, wy;
  bool ok;
};

__device__ __forceinline__ LatTable lat_table_of(const int (&v)[6], int64_t capacity,
                                                 int tsize) {
  LatTable t;
  t.gx = v[0] > 0 ? v[0] : 1;
  t.gy = v[1] > 0 ? v[1] : 1;
  t.ok = v[2] <= v[3] && v[4] <= v[5];
  t.wx = t.ok ? (int)(((int64_t)v[3] - v[2]) / t.gx) + 1 : 0;
  t.wy = t.ok ? (int)(((int64_t)v[5] - v[4]) / t.gy) + 1 : 0;
  if (t.ok) {
    const int64_t ex = (int64_t)t.gx * (t.wx - 1), ey = (int64_t)t.gy * (t.wy - 1);
    t.ok = (int64_t)t.wx * t.wy <= capacity && ex <= 32767 && ey <= 32767 &&
           ex * ex + ey * ey < (int64_t)tsize;
  }
  return t;
}

}  // namespace fi
