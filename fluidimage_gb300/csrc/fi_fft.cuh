// Register-resident mixed-radix FFTs for one thread (N <= 64, N = 2^a 3^b).
//
// One thread transforms one row or one column of a window held in registers.
// The decimation-in-time recursion is resolved at compile time: with every loop
// unrolled, array indices and twiddle indices are constants, the "sub-array"
// copies are register renames, and each twiddle is an immediate operand
// (fi_twiddles.cuh).  Quarter-turn twiddles are applied as swaps.
#pragma once

#include <cuda_runtime.h>

#include "fi_twiddles.cuh"

namespace fi {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 cmul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int BASE>
__device__ __forceinline__ float tw_re(int j) {
  if constexpr (BASE == 64) return fi_tw64_re(j); else return fi_tw48_re(j);
}
template <int BASE>
__device__ __forceinline__ float tw_im(int j) {
  if constexpr (BASE == 64) return fi_tw64_im(j); else return fi_tw48_im(j);
}

// a * W_BASE^j (forward) or a * conj(W_BASE^j) (inverse); j known after unrolling.
template <int BASE, bool INV>
__device__ __forceinline__ float2 twiddle(float2 a, int j) {
  j %= BASE;
  if (j == 0) return a;
  if (4 * j == BASE) return cmul_mi<INV>(a);
  if (2 * j == BASE) return make_float2(-a.x, -a.y);
  if (4 * j == 3 * BASE) return cmul_mi<!INV>(a);
  const float wr = tw_re<BASE>(j);
  const float wi = INV ? -tw_im<BASE>(j) : tw_im<BASE>(j);
  return make_float2(a.x * wr - a.y * wi, a.x * wi + a.y * wr);
}

template <int R, bool INV>
__device__ __forceinline__ void small_dft(float2 (&t)[R]) {
  if constexpr (R == 2) {
    const float2 a = t[0], b = t[1];
    t[0] = cadd(a, b);
    t[1] = csub(a, b);
  } else if constexpr (R == 4) {
    const float2 s02 = cadd(t[0], t[2]), d02 = csub(t[0], t[2]);
    const float2 s13 = cadd(t[1], t[3]), d13 = cmul_mi<INV>(csub(t[1], t[3]));
    t[0] = cadd(s02, s13);
    t[2] = csub(s02, s13);
    t[1] = cadd(d02, d13);
    t[3] = csub(d02, d13);
  } else {  // R == 3
    constexpr float kS = 0x1.bb67aep-1f;  // sqrt(3) / 2
    const float2 a = t[0];
    const float2 s = cadd(t[1], t[2]);
    const float2 d = csub(t[1], t[2]);
    const float2 m = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
    // forward: X1 = m - i*kS*d, X2 = m + i*kS*d
    const float2 r = cmul_mi<INV>(make_float2(kS * d.x, kS * d.y));
    t[0] = cadd(a, s);
    t[1] = cadd(m, r);
    t[2] = csub(m, r);
  }
}

template <int N>
struct Radix {
  static constexpr int value = (N % 4 == 0 && N != 8) ? 4 : ((N % 2 == 0) ? 2 : 3);
};

// In-place DFT of x[0..N-1] (natural order in and out), unnormalised.
template <int N, int BASE, bool INV>
struct RegFFT {
  static __device__ __forceinline__ void run(float2* x) {
    if constexpr (N == 1) {
      return;
    } else if constexpr (N == 2 || N == 3 || N == 4) {
      float2 t[N];
#pragma unroll
      for (int i = 0; i < N; ++i) t[i] = x[i];
      small_dft<N, INV>(t);
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = t[i];
    } else {
      constexpr int R = Radix<N>::value;
      constexpr int M = N / R;
      static_assert(BASE % N == 0, "twiddle base must be a multiple of N");
      float2 sub[R][M];
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int m = 0; m < M; ++m) sub[r][m] = x[r + R * m];
#pragma unroll
      for (int r = 0; r < R; ++r) RegFFT<M, BASE, INV>::run(sub[r]);
#pragma unroll
      for (int k = 0; k < M; ++k) {
        float2 t[R];
#pragma unroll
        for (int r = 0; r < R; ++r) t[r] = twiddle<BASE, INV>(sub[r][k], r * k * (BASE / N));
        small_dft<R, INV>(t);
#pragma unroll
        for (int q = 0; q < R; ++q) x[k + M * q] = t[q];
      }
    }
  }
};

template <int N>
struct TwBase {
  static constexpr int value = (64 % N == 0) ? 64 : 48;
};

template <int N, bool INV>
__device__ __forceinline__ void fft_reg(float2* x) {
  RegFFT<N, TwBase<N>::value, INV>::run(x);
}

}  // namespace fi
