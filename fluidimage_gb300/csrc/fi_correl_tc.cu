// Tensor-core PIV pass: the 2-D DFTs of the cross-correlation written as dense
// contractions (F W F^T) on the 5th-generation tensor cores, for 32 x 32 windows.
//
// Upstream operation restated (fluidimage 0.5.3): CorrelFFTNumpy.__call__,
// calcul/correl.py:671-685 with calcul/fft.py:254-269: F = fft2(w), F[0,0] = 0,
// correl = ifft2(conj(F0) F1).real in the _like_fftshift layout (correl.py:596-636),
// norm = sqrt(4 E0 E1) N; then the peak search, second chance and subpixel fit of
// fi_peak.cuh, exactly as the FP32 FFT pass (fi_correl.cu).
//
// One CTA (8 warps) processes tiles of 8 windows, one warp per window, in four
// tcgen05.mma stages with FP32 accumulators in tensor memory (TMEM):
//   1  X = W R          rows (window, r) x packed half spectrum kx   [M 128, N 32, K 32]
//   2  Y = F X          rows (window, kx') x [Re | Im](ky)            [M 128, N 64, K 64]
//   3  Q = conj(F) P    P = conj(Y0) Y1,  rows (window, kx')          [M 128, N 64, K 64]
//   4  c = Q G          rows (window, y) x x, real inverse over kx    [M 128, N 32, K 32]
// R packs the real-input DFT of a row into 32 reals (Re kx = 0..16, Im kx = 1..15);
// the two real columns kx = 0 and 16 share one complex row kx' = 0 in stages 2-3
// (separated by Hermitian symmetry between the stages); G applies the Hermitian
// weights of the inverse.  Between stages the warps read the accumulators
// (tcgen05.ld), split each value into hi + lo 16-bit terms and write the next
// stage's operand to shared memory in the no-swizzle core-matrix layouts
// (K-major or MN-major, whichever the owning thread writes contiguously).
//
// Forms: FI_TC_BF16X1 (one bf16 term), FI_TC_BF16X3 and FI_TC_FP16X3 (3-term split
// products a_hi b_hi + a_hi b_lo + a_lo b_hi).  Every window is scaled by powers of
// two (exact) so that each stage's operand stays inside the FP16 range: the input
// to unit RMS (and its maximum below 2^15), P by 2^-6, Q by 2^-5; the plane is
// scaled back at the end.  Integer pixels split exactly into two terms, so the
// window sums and the DC removal (F[0,0] = 0) are exact.
//
// Synchronisation per stage: writers fence.proxy.async, CTA barrier, one thread
// issues the MMAs and commits them to an mbarrier, every thread waits on it (a
// bounded wait; a timeout sets the status word and ends the CTA's loop).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fi_common.cuh"
#include "fi_peak.cuh"

namespace fi {
namespace tc {

constexpr int N = 32;          // window size
constexpr int WIN = 8;         // windows per tile (one warp each)
constexpr int THREADS = 32 * WIN;
constexpr int TMEM_COLS = 256;
constexpr int LDP = N + 1;     // plane row stride (floats), as Cfg<32>::LDP

// shared memory map (bytes)
constexpr int B1_BYTES = 32 * 32 * 2;  // N 32 x K 32, one term
constexpr int B2_BYTES = 64 * 64 * 2;  // N 64 x K 64
constexpr int B4_BYTES = 32 * 32 * 2;  // N 32 x K 32
constexpr int OFF_B1 = 0;
constexpr int OFF_B2 = OFF_B1 + 2 * B1_BYTES;
constexpr int OFF_B4 = OFF_B2 + 2 * B2_BYTES;
constexpr int OFF_A = OFF_B4 + 2 * B4_BYTES;  // stage operands, then the planes
constexpr int A_BYTES = 64 * 1024;
constexpr int OFF_X = OFF_A + A_BYTES;         // kx' = 0 rows exchanged between warps
constexpr int X_BYTES = WIN * 2 * 64 * 4;
constexpr int OFF_W = OFF_X + X_BYTES;         // per-window scalars
constexpr int W_BYTES = WIN * 64;
constexpr int OFF_RED = OFF_W + W_BYTES;       // per-window peak-search scratch
constexpr int RED_BYTES = WIN * 256;
constexpr int OFF_BAR = OFF_RED + RED_BYTES;   // mbarrier, TMEM base
constexpr int SMEM = OFF_BAR + 64;
static_assert(WIN * N * LDP * 4 <= A_BYTES, "planes must fit the operand region");

// operand sub-regions of the A region
constexpr int A1_PART = 128 * 32 * 2;  // [img][tile][part]: 128 rows x K 32
constexpr int A2_PART = 128 * 64 * 2;  // [img][part]:       128 rows x K 64
constexpr int A3_PART = 128 * 64 * 2;  // [part]
constexpr int A4_PART = 128 * 32 * 2;  // [tile][part]

// per-stage power-of-two scales of the operands (see the header comment)
constexpr int SCALE_P = 6;
constexpr int SCALE_Q = 5;

struct TcWin {
  float dc0, dc1;   // DC removal of X[r, 0]: (sum v) 2^-e / N
  float normf;
  float outscale;   // plane = stage-4 output * outscale
  double norm64;
  int flat;
  int e0, e1;       // input scales 2^-e
  int valid;
};
static_assert(sizeof(TcWin) <= 64, "per-window scalars");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle: start address, leading and stride
// byte offsets between core matrices (8 rows x 16 bytes, stored contiguously).
// K-major: leading = K direction, stride = M/N direction.  MN-major: leading = K
// direction, stride = M/N direction as well (the canonical no-swizzle layouts).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 or f16 operands,
// A K-major or MN-major, B K-major, M = 128.
__device__ __forceinline__ uint32_t idesc(bool f16, bool a_mn, int n) {
  const uint32_t fmt = f16 ? 0u : 1u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((a_mn ? 1u : 0u) << 15) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bounded wait for the mbarrier phase `parity`; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 24) && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}

__device__ __forceinline__ void tmem_ld16(uint32_t addr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(addr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t addr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Two floats -> (hi, lo) 16-bit pairs, packed two per 32-bit word (the first value
// in the low half, as memory order wants).
template <bool F16>
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  if constexpr (F16) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
}

// Eight consecutive values -> one 16-byte store of the hi terms at `hi_ptr` and,
// for the 3-term forms, one of the lo terms at `hi_ptr + lo_off`.
template <bool F16, bool LO>
__device__ __forceinline__ void store8(unsigned char* hi_ptr, int lo_off, const float* v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) split2<F16>(v[2 * i], v[2 * i + 1], h[i], l[i]);
  *reinterpret_cast<uint4*>(hi_ptr) = make_uint4(h[0], h[1], h[2], h[3]);
  if constexpr (LO) *reinterpret_cast<uint4*>(hi_ptr + lo_off) = make_uint4(l[0], l[1], l[2], l[3]);
}

// 2^k as a float (|k| < 127): exact scaling by a product
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// One value -> its hi term at `hi_ptr` and, for the 3-term forms, its lo term at
// `hi_ptr + lo_off` (16-bit stores).
template <bool F16, bool LO>
__device__ __forceinline__ void put2(unsigned char* hi_ptr, int lo_off, float v) {
  if constexpr (F16) {
    const __half h = __float2half_rn(v);
    *reinterpret_cast<__half*>(hi_ptr) = h;
    if constexpr (LO) *reinterpret_cast<__half*>(hi_ptr + lo_off) = __float2half_rn(v - __half2float(h));
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    *reinterpret_cast<__nv_bfloat16*>(hi_ptr) = h;
    if constexpr (LO)
      *reinterpret_cast<__nv_bfloat16*>(hi_ptr + lo_off) = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// cos / sin of 2 pi j / 32
__device__ __forceinline__ float cos32(int j) {
  float s, c;
  sincospif((float)(j & 31) / 16.0f, &s, &c);
  return c;
}
__device__ __forceinline__ float sin32(int j) {
  float s, c;
  sincospif((float)(j & 31) / 16.0f, &s, &c);
  return s;
}

// Byte offset of element (row, k) in a K-major no-swizzle tile with `kcm` core
// matrices along K, and in an MN-major tile with `rcm` core matrices along M/N.
__device__ __forceinline__ int kmaj(int row, int k, int kcm) {
  return (((row >> 3) * kcm + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}
__device__ __forceinline__ int mnmaj(int row, int k, int rcm) {
  return (((k >> 3) * rcm + (row >> 3)) << 7) + ((k & 7) << 4) + ((row & 7) << 1);
}

// The constant operands (hi and lo terms): B1 = R (row DFT, packed), B2 = the
// complex column DFT on [Re | Im], B4 = G (real inverse row DFT, Hermitian weights).
template <bool F16>
__device__ void fill_constants(unsigned char* sm) {
  auto put = [&](int off, int lo_off, float v) {
    if constexpr (F16) {
      const __half h = __float2half_rn(v);
      const __half l = __float2half_rn(v - __half2float(h));
      *reinterpret_cast<__half*>(sm + off) = h;
      *reinterpret_cast<__half*>(sm + off + lo_off) = l;
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
      *reinterpret_cast<__nv_bfloat16*>(sm + off) = h;
      *reinterpret_cast<__nv_bfloat16*>(sm + off + lo_off) = l;
    }
  };
  for (int idx = threadIdx.x; idx < 32 * 32; idx += blockDim.x) {
    const int n = idx >> 5, k = idx & 31;
    // B1[n][x = k]: n <= 16: cos(2 pi n x / 32); n = 16 + j: -sin(2 pi j x / 32)
    const float b1 = (n <= 16) ? cos32(n * k) : -sin32((n - 16) * k);
    put(OFF_B1 + kmaj(n, k, 4), B1_BYTES, b1);
    // B4[x = n][k4 = k]: k4 <= 16: w cos(2 pi k4 x / 32) (w = 1 at 0 and 16, else 2);
    // k4 = 16 + j: -2 sin(2 pi j x / 32)
    float b4;
    if (k <= 16) b4 = ((k == 0 || k == 16) ? 1.0f : 2.0f) * cos32(k * n);
    else b4 = -2.0f * sin32((k - 16) * n);
    put(OFF_B4 + kmaj(n, k, 4), B4_BYTES, b4);
  }
  for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
    const int n = idx >> 6, k = idx & 63;
    const int ky = n & 31, r = k & 31;
    const int j = ky * r;
    float b2;
    if (k < 32) b2 = (n < 32) ? cos32(j) : -sin32(j);
    else b2 = (n < 32) ? sin32(j) : cos32(j);
    put(OFF_B2 + kmaj(n, k, 8), B2_BYTES, b2);
  }
}

// One row of 32 pixels of an image, minus the image minimum, zero outside the
// image (the zero padding of _pad_images); integer values for u8/u16.
__device__ __forceinline__ void load_row_int(const void* im, int dtype, int H, int W, int y,
                                             int x0, int mini, int (&v)[32]) {
  const bool row_in = y >= 0 && y < H;
  if (row_in && x0 >= 0 && x0 + 32 <= W) {
    if (dtype == FI_U16) {
      const uint16_t* p = reinterpret_cast<const uint16_t*>(im) + (int64_t)y * W + x0;
      if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint4 u = __ldg(reinterpret_cast<const uint4*>(p) + q);
          const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            v[8 * q + 2 * i] = (int)(w4[i] & 0xffffu) - mini;
            v[8 * q + 2 * i + 1] = (int)(w4[i] >> 16) - mini;
          }
        }
        return;
      }
    } else {
      const uint8_t* p = reinterpret_cast<const uint8_t*>(im) + (int64_t)y * W + x0;
      if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint2 u = __ldg(reinterpret_cast<const uint2*>(p) + q);
          const uint32_t w2[2] = {u.x, u.y};
#pragma unroll
          for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int b = 0; b < 4; ++b) v[8 * q + 4 * i + b] = (int)((w2[i] >> (8 * b)) & 0xffu) - mini;
        }
        return;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int x = x0 + i;
    v[i] = (row_in && x >= 0 && x < W) ? load_px_int(im, dtype, (int64_t)y * W + x) - mini : 0;
  }
}

__device__ __forceinline__ void load_row_f32(const float* im, int H, int W, int y, int x0,
                                             float minf, float (&v)[32]) {
  const bool row_in = y >= 0 && y < H;
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int x = x0 + i;
    v[i] = (row_in && x >= 0 && x < W) ? __fsub_rn(__ldg(im + (int64_t)y * W + x), minf) : 0.f;
  }
}

template <int FORM>
__global__ void __launch_bounds__(THREADS, 2)
    k_piv_pass_tc(const fi_piv_pass_args a, int nvec, int npad, int ntiles, float tie_rel,
                  int* status) {
  constexpr bool F16 = (FORM == FI_TC_FP16X3);
  constexpr bool LO = (FORM != FI_TC_BF16X1);
  constexpr int NT = LO ? 3 : 1;  // products per K step
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm + OFF_A;
  float* xbuf = reinterpret_cast<float*>(sm + OFF_X);
  TcWin* wins = reinterpret_cast<TcWin*>(sm + OFF_W);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + OFF_BAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  fill_constants<F16>(sm);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;  // this warp's TMEM lanes
  uint32_t phase = 0;
  const float min0 = __ldg(a.im_min + 0), min1 = __ldg(a.im_min + 1);
  const bool intpath = a.dtype != FI_F32;

  // one stage: operands written -> MMAs issued by thread 0 -> bounded wait
  auto run_stage = [&](auto issue) -> bool {
    fence_async_smem();
    fence_before();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      issue();
      mma_commit(bar);
    }
    const bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    fence_after();
    return true;
  };
  // the 1 or 3 products of one K step, accumulating after the first
  auto mma_terms = [&](uint32_t d, uint32_t a_hi, int a_lo_off, uint32_t a_lbo, uint32_t a_sbo,
                       uint32_t b_hi, int b_lo_off, uint32_t b_lbo, uint32_t b_sbo, uint32_t id,
                       bool first) {
#pragma unroll
    for (int term = 0; term < NT; ++term) {
      const uint32_t aa = a_hi + (term == 2 ? a_lo_off : 0);
      const uint32_t bb = b_hi + (term == 1 ? b_lo_off : 0);
      mma(d, sdesc(aa, a_lbo, a_sbo), sdesc(bb, b_lbo, b_sbo), id,
          (first && term == 0) ? 0u : 1u);
    }
  };
  const uint32_t sA_u = smem_u32(sA), sB1 = smem_u32(sm + OFF_B1), sB2 = smem_u32(sm + OFF_B2),
                 sB4 = smem_u32(sm + OFF_B4);
  bool ok = true;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int vec = tile * WIN + warp;  // this warp's window
    const bool active = vec < nvec;
    // ---------------- stage the two windows (warp = window, lane = row) ----------------
    {
      WinPos wp;
      if (active) wp = window_positions<N>(a, vec, npad);
      const bool load = active && wp.valid;
      float f0[32], f1[32];
      unsigned long long u[4] = {0ull, 0ull, 0ull, 0ull};
      double sums[4] = {0.0, 0.0, 0.0, 0.0};
      float mm[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
      if (intpath) {
        int v0[32], v1[32];
        if (load) {
          load_row_int(a.im0, a.dtype, a.height, a.width, wp.y0 + lane, wp.x0, (int)min0, v0);
          load_row_int(a.im1, a.dtype, a.height, a.width, wp.y1 + lane, wp.x1, (int)min1, v1);
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) v0[i] = v1[i] = 0;
        }
        unsigned s0 = 0u, s1 = 0u;
        unsigned long long q0 = 0ull, q1 = 0ull;
        int lo0 = v0[0], hi0 = v0[0], lo1 = v1[0], hi1 = v1[0];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          s0 += (unsigned)v0[i];
          s1 += (unsigned)v1[i];
          q0 += (unsigned long long)((unsigned)v0[i] * (unsigned)v0[i]);
          q1 += (unsigned long long)((unsigned)v1[i] * (unsigned)v1[i]);
          lo0 = min(lo0, v0[i]);
          hi0 = max(hi0, v0[i]);
          lo1 = min(lo1, v1[i]);
          hi1 = max(hi1, v1[i]);
          f0[i] = (float)v0[i];
          f1[i] = (float)v1[i];
        }
        u[0] = s0;
        u[1] = q0;
        u[2] = s1;
        u[3] = q1;
        gsum4u<32>(u, 0, nullptr);
        mm[0] = (float)lo0;
        mm[1] = (float)lo1;
        mm[2] = (float)hi0;
        mm[3] = (float)hi1;
      } else {
        if (load) {
          load_row_f32(reinterpret_cast<const float*>(a.im0), a.height, a.width, wp.y0 + lane,
                       wp.x0, min0, f0);
          load_row_f32(reinterpret_cast<const float*>(a.im1), a.height, a.width, wp.y1 + lane,
                       wp.x1, min1, f1);
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) f0[i] = f1[i] = 0.f;
        }
        float sf0 = 0.f, sf1 = 0.f, qf0 = 0.f, qf1 = 0.f, cf0 = 0.f, cf1 = 0.f;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          sf0 += f0[i];
          sf1 += f1[i];
          float yk = fmaf(f0[i], f0[i], -cf0), tk = qf0 + yk;
          cf0 = (tk - qf0) - yk;
          qf0 = tk;
          yk = fmaf(f1[i], f1[i], -cf1);
          tk = qf1 + yk;
          cf1 = (tk - qf1) - yk;
          qf1 = tk;
          mm[0] = fminf(mm[0], f0[i]);
          mm[1] = fminf(mm[1], f1[i]);
          mm[2] = fmaxf(mm[2], f0[i]);
          mm[3] = fmaxf(mm[3], f1[i]);
        }
        sums[0] = (double)sf0;
        sums[1] = (double)qf0 - (double)cf0;
        sums[2] = (double)sf1;
        sums[3] = (double)qf1 - (double)cf1;
        gsum4<32>(sums, 0, nullptr);
      }
      gminmax4<32>(mm, 0, nullptr);
      if (lane == 0) {
        const bool flat0 = mm[0] == mm[2], flat1 = mm[1] == mm[3];
        const WinScalars ws = window_scalars<N>(intpath, u, sums, flat0, flat1, a.norms != nullptr);
        TcWin tw;
        // input scales: unit RMS, and the maximum below 2^15 (FP16 range)
        int e0 = ws.e0, e1 = ws.e1, x0, x1;
        frexpf(fmaxf(fabsf(mm[2]), fabsf(mm[0])), &x0);
        frexpf(fmaxf(fabsf(mm[3]), fabsf(mm[1])), &x1);
        e0 = max(e0, x0 - 15);
        e1 = max(e1, x1 - 15);
        // (float images only can reach these bounds; pow2f needs |e| < 127)
        e0 = min(max(e0, -100), 100);
        e1 = min(max(e1, -100), 100);
        // (sum v) 2^-e / N: the sum rounded once to float32, then an exact scaling
        const float s0f = intpath ? u64_to_float_rn(u[0]) : (float)sums[0];
        const float s1f = intpath ? u64_to_float_rn(u[2]) : (float)sums[2];
        tw.dc0 = s0f * pow2f(-e0 - 5);
        tw.dc1 = s1f * pow2f(-e1 - 5);
        tw.normf = ws.normf;
        tw.norm64 = ws.norm64;
        tw.flat = (flat0 || flat1) ? 1 : 0;
        tw.e0 = e0;
        tw.e1 = e1;
        // plane = c 2^(e0 + e1 + SCALE_P + SCALE_Q) / N^2
        tw.outscale = ldexpf(1.0f, e0 + e1 + SCALE_P + SCALE_Q - 10);
        tw.valid = load ? 1 : 0;
        wins[warp] = tw;
      }
      __syncwarp();
      const float s0 = pow2f(-wins[warp].e0), s1 = pow2f(-wins[warp].e1);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        f0[i] *= s0;
        f1[i] *= s1;
      }
      // A1[img][tile][part], K-major (K = x): row m = 32 (warp % 4) + lane
      const int t = warp >> 2, m = 32 * (warp & 3) + lane;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        store8<F16, LO>(sA + ((0 * 2 + t) * 2) * A1_PART + kmaj(m, 8 * c, 4), A1_PART, f0 + 8 * c);
        store8<F16, LO>(sA + ((1 * 2 + t) * 2) * A1_PART + kmaj(m, 8 * c, 4), A1_PART, f1 + 8 * c);
      }
    }
    // ---------------- stage 1: X = W R ----------------
    ok = run_stage([&] {
      const uint32_t id = idesc(F16, false, 32);
      for (int img = 0; img < 2; ++img)
        for (int t = 0; t < 2; ++t)
          for (int ks = 0; ks < 2; ++ks)
            mma_terms(tmem + 64 * t + 32 * img, sA_u + ((img * 2 + t) * 2) * A1_PART + ks * 256,
                      A1_PART, 128, 512, sB1 + ks * 256, B1_BYTES, 128, 512, id, ks == 0);
    });
    if (!ok) break;
    // ---------------- epilogue 1: DC removal, pack kx = 0 and 16, operand of stage 2 ----
    {
      const int t = warp >> 2;
      float x0v[32], x1v[32];
      tmem_ld32(tmem + lane_base + 64 * t, x0v);
      tmem_ld32(tmem + lane_base + 64 * t + 32, x1v);
      tmem_wait_ld();
      const TcWin tw = wins[warp];
      x0v[0] -= tw.dc0;
      x1v[0] -= tw.dc1;
      // A2[img][part], MN-major (M = 16 window + kx', K = [Re r | Im r])
#pragma unroll
      for (int img = 0; img < 2; ++img) {
        const float* x = img ? x1v : x0v;
        float re[16], im[16];
        re[0] = x[0];
        im[0] = x[16];
#pragma unroll
        for (int k = 1; k < 16; ++k) {
          re[k] = x[k];
          im[k] = x[16 + k];
        }
        unsigned char* base = sA + (img * 2) * A2_PART;
        const int m = 16 * warp;
        store8<F16, LO>(base + mnmaj(m, lane, 16), A2_PART, re);
        store8<F16, LO>(base + mnmaj(m + 8, lane, 16), A2_PART, re + 8);
        store8<F16, LO>(base + mnmaj(m, 32 + lane, 16), A2_PART, im);
        store8<F16, LO>(base + mnmaj(m + 8, 32 + lane, 16), A2_PART, im + 8);
      }
    }
    // ---------------- stage 2: Y = F X ----------------
    ok = run_stage([&] {
      const uint32_t id = idesc(F16, true, 64);
      for (int img = 0; img < 2; ++img)
        for (int ks = 0; ks < 4; ++ks)
          mma_terms(tmem + 128 + 64 * img, sA_u + (img * 2) * A2_PART + ks * 4096, A2_PART, 2048,
                    128, sB2 + ks * 256, B2_BYTES, 128, 1024, id, ks == 0);
    });
    if (!ok) break;
    // ---------------- epilogue 2: cross spectrum P = conj(F0) F1 ----------------
    {
      const int h = warp >> 2;            // ky half
      const int kxp = lane & 15;          // kx'
      const int wl = 2 * (warp & 3) + (lane >> 4);  // window of this lane
      float y0r[16], y0i[16], y1r[16], y1i[16];
      const uint32_t c0 = tmem + lane_base + 128 + 16 * h;
      tmem_ld16(c0, y0r);
      tmem_ld16(c0 + 32, y0i);
      tmem_ld16(c0 + 64, y1r);
      tmem_ld16(c0 + 96, y1i);
      tmem_wait_ld();
      float* xb = xbuf + (wl * 2 + h) * 64;
      if (kxp == 0) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          xb[j] = y0r[j];
          xb[16 + j] = y0i[j];
          xb[32 + j] = y1r[j];
          xb[48 + j] = y1i[j];
        }
      }
      __syncthreads();
      // rows kx' >= 1: P = conj(F0) F1 (the row kx' = 0 lanes compute a value that is
      // not stored)
      float pr[16], pi[16];
      const float sp = pow2f(-SCALE_P);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        pr[j] = fmaf(y0r[j], y1r[j], y0i[j] * y1i[j]) * sp;
        pi[j] = fmaf(y0r[j], y1i[j], -(y0i[j] * y1r[j])) * sp;
      }
      // A3[part], K-major (row = 16 window + kx' = 32 (warp % 4) + lane,
      // K = [Im P(ky) | Re P(ky)])
      const int m = 32 * (warp & 3) + lane;
      if (kxp != 0) {
        store8<F16, LO>(sA + kmaj(m, 16 * h, 8), A3_PART, pi);
        store8<F16, LO>(sA + kmaj(m, 16 * h + 8, 8), A3_PART, pi + 8);
        store8<F16, LO>(sA + kmaj(m, 32 + 16 * h, 8), A3_PART, pr);
        store8<F16, LO>(sA + kmaj(m, 32 + 16 * h + 8, 8), A3_PART, pr + 8);
      }
      // row kx' = 0 holds Z = F(kx=0) + i F(kx=16): lane j of each half warp separates
      // the two with the mirror -ky for ky = 16 h + j, from the exchanged rows
      {
        const int j = kxp;
        const int ky = 16 * h + j;
        const float* xs = xbuf + (wl * 2 + h) * 64;
        const float* xo = (j == 0) ? xs : xbuf + (wl * 2 + (1 - h)) * 64;
        const int jm = (j == 0) ? 0 : 16 - j;  // index of -ky in its half
        const float z0r = xs[j], z0i = xs[16 + j], z1r = xs[32 + j], z1i = xs[48 + j];
        const float m0r = xo[jm], m0i = xo[16 + jm], m1r = xo[32 + jm], m1i = xo[48 + jm];
        // F(0) = (Z + conj(Zm)) / 2, F(16) = (Z - conj(Zm)) / (2i)
        const float a0r = 0.5f * (z0r + m0r), a0i = 0.5f * (z0i - m0i);
        const float b0r = 0.5f * (z0i + m0i), b0i = 0.5f * (m0r - z0r);
        const float a1r = 0.5f * (z1r + m1r), a1i = 0.5f * (z1i - m1i);
        const float b1r = 0.5f * (z1i + m1i), b1i = 0.5f * (m1r - z1r);
        // P(kx=0) = conj(a0) a1 (zero at ky = 0: F[0,0] = 0), P(kx=16) = conj(b0) b1
        float p0r = fmaf(a0r, a1r, a0i * a1i), p0i = fmaf(a0r, a1i, -(a0i * a1r));
        if (ky == 0) p0r = p0i = 0.f;
        const float p16r = fmaf(b0r, b1r, b0i * b1i), p16i = fmaf(b0r, b1i, -(b0i * b1r));
        // packed row: P(0) + i P(16), written element by element into row 16 wl
        const float vr = (p0r - p16i) * sp, vi = (p0i + p16r) * sp;
        const int m0 = 16 * wl;
        put2<F16, LO>(sA + kmaj(m0, ky, 8), A3_PART, vi);
        put2<F16, LO>(sA + kmaj(m0, 32 + ky, 8), A3_PART, vr);
      }
    }
    // ---------------- stage 3: Q = inverse DFT over ky ----------------
    ok = run_stage([&] {
      const uint32_t id = idesc(F16, false, 64);
      for (int ks = 0; ks < 4; ++ks)
        mma_terms(tmem, sA_u + ks * 256, A3_PART, 128, 1024, sB2 + ks * 256, B2_BYTES, 128, 1024,
                  id, ks == 0);
    });
    if (!ok) break;
    // ---------------- epilogue 3: operand of the real inverse over kx ----------------
    {
      const int h = warp >> 2;  // 0: Im Q (columns 0..31), 1: Re Q (32..63)
      const int kxp = lane & 15;
      const int wl = 2 * (warp & 3) + (lane >> 4);
      float q[32];
      tmem_ld32(tmem + lane_base + 32 * h, q);
      tmem_wait_ld();
      const float sq = pow2f(-SCALE_Q);
#pragma unroll
      for (int i = 0; i < 32; ++i) q[i] *= sq;
      const int k4 = h ? kxp : 16 + kxp;
      // A4[tile][part], MN-major (row = 32 (window % 4) + y, K = k4)
      unsigned char* base = sA + ((wl >> 2) * 2) * A4_PART;
      const int m0 = 32 * (wl & 3);
#pragma unroll
      for (int c = 0; c < 4; ++c) store8<F16, LO>(base + mnmaj(m0 + 8 * c, k4, 16), A4_PART, q + 8 * c);
    }
    // ---------------- stage 4: c = Q G ----------------
    ok = run_stage([&] {
      const uint32_t id = idesc(F16, true, 32);
      for (int t = 0; t < 2; ++t)
        for (int ks = 0; ks < 2; ++ks)
          mma_terms(tmem + 128 + 32 * t, sA_u + (t * 2) * A4_PART + ks * 4096, A4_PART, 2048, 128,
                    sB4 + ks * 256, B4_BYTES, 128, 512, id, ks == 0);
    });
    if (!ok) break;
    // ---------------- epilogue 4: the plane, peak search, subpixel fit ----------------
    {
      const int t = warp >> 2;
      float c[32];
      tmem_ld32(tmem + lane_base + 128 + 32 * t, c);
      tmem_wait_ld();
      const TcWin tw = wins[warp];
      float* PL = reinterpret_cast<float*>(sA) + warp * (N * LDP);
      double* red = reinterpret_cast<double*>(sm + OFF_RED + warp * 256);
      const int i0 = shift_index<N>(lane);
#pragma unroll
      for (int x = 0; x < 32; ++x)
        PL[i0 * LDP + shift_index<N>(x)] = tw.flat ? 0.f : c[x] * tw.outscale;
      __syncwarp();
      if (active) {
        const bool valid = tw.valid != 0;
        WinPos wp = window_positions<N>(a, vec, npad);
        PeakArgs pa;
        pa.mask = a.mask;
        pa.box = SearchBox{a.box_i0_start, a.box_i0_stop, a.box_i1_start, a.box_i1_stop};
        pa.radius = a.particle_radius;
        pa.apply_subpix = a.apply_subpix;
        pa.subpix_method = a.subpix_method;
        pa.nsubpix = a.nsubpix;
        pa.minv = a.subpix_minv;
        pa.nb_peaks = a.nb_peaks;
        pa.tie_rel = tie_rel;
        SecondaryOut so{a.peaks_count, a.peaks, a.peaks_err, vec, a.dxin != nullptr, wp.dinx,
                        wp.diny};
        VecResult res = peak_and_subpix<N>(PL, pa, tw.normf, lane, warp, red,
                                           a.nb_peaks > 1 ? &so : nullptr);
        if (!valid && a.nb_peaks > 1 && lane == 0) a.peaks_count[vec] = -1;
        if (a.planes) {
          float* out = a.planes + (int64_t)vec * N * N;
          const bool write_box = (a.mask == nullptr);
          for (int r = 0; r < N; ++r) {
            float v = PL[r * LDP + lane];
            if (!valid || (write_box && res.nb.has(r, lane))) v = NAN;
            out[r * N + lane] = v;
          }
        }
        if (lane == 0) {
          if (a.norms) a.norms[vec] = tw.norm64;
          float dxo = res.dx, dyo = res.dy, cm = res.cmax;
          int err = res.err;
          if (!valid) {
            dxo = dyo = cm = NAN;
            err = FI_VEC_BAD_CROP;
          }
          if (a.dxin) {
            dxo = add_shift(dxo, wp.dinx);
            dyo = add_shift(dyo, wp.diny);
          }
          a.deltaxs[vec] = dxo;
          a.deltays[vec] = dyo;
          a.correls_max[vec] = cm;
          a.errors[vec] = (uint8_t)err;
          if (a.flags)
            a.flags[vec] = valid ? (uint8_t)((res.tie ? FI_FLAG_NEAR_TIE : 0) |
                                             (res.subpix_tie ? FI_FLAG_SUBPIX_TIE : 0) |
                                             (res.sec_tie ? FI_FLAG_SECONDARY_TIE : 0))
                                 : (uint8_t)0;
          const int sx = wp.ixs0 + wp.ixs1, sy = wp.iys0 + wp.iys1;
          a.xs[vec] = midpoint(sx);
          a.ys[vec] = midpoint(sy);
        }
      }
      // the planes alias the operand region of the next tile
      __syncthreads();
    }
  }
  if (!ok && tid == 0 && status) atomicOr(status, 1);
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

template <int FORM>
static int launch_tc(const fi_piv_pass_args& a, int nvec, int npad, int* status, cudaStream_t s) {
  static SmemLimit limit;
  FI_CUDA_TRY(raise_smem_limit(k_piv_pass_tc<FORM>, SMEM, limit));
  int dev = 0, sms = 0;
  FI_CUDA_TRY(cudaGetDevice(&dev));
  FI_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int ntiles = (nvec + WIN - 1) / WIN;
  const int grid = min(ntiles, 2 * sms);  // two CTAs per SM (shared memory, TMEM)
  // near-tie tolerance of each form (its plane error relative to the peak, with margin)
  const float tie_rel = (FORM == FI_TC_BF16X1) ? 3e-2f : (FORM == FI_TC_BF16X3 ? 1e-4f : 1e-5f);
  k_piv_pass_tc<FORM><<<grid, THREADS, SMEM, s>>>(a, nvec, npad, ntiles, tie_rel, status);
  return check_launch("k_piv_pass_tc");
}

}  // namespace tc
}  // namespace fi

using namespace fi;

extern "C" int fi_piv_pass_tc(const fi_piv_pass_args* args, int form, int* status, void* stream) {
  FI_REQUIRE(args, "fi_piv_pass_tc: null args");
  const fi_piv_pass_args& a = *args;
  FI_REQUIRE(a.n == 32, "fi_piv_pass_tc: window size %d not supported (32)", a.n);
  FI_REQUIRE(form == FI_TC_BF16X1 || form == FI_TC_BF16X3 || form == FI_TC_FP16X3,
             "fi_piv_pass_tc: bad form %d", form);
  FI_REQUIRE(a.im0 && a.im1 && a.im_min && a.ixvecs && a.iyvecs, "fi_piv_pass_tc: null input");
  FI_REQUIRE(a.deltaxs && a.deltays && a.correls_max && a.errors && a.xs && a.ys,
             "fi_piv_pass_tc: null output");
  FI_REQUIRE(a.dtype == FI_U8 || a.dtype == FI_U16 || a.dtype == FI_F32,
             "fi_piv_pass_tc: bad dtype %d", a.dtype);
  FI_REQUIRE(a.nx > 0 && a.ny > 0 && a.height > 0 && a.width > 0, "fi_piv_pass_tc: empty grid");
  FI_REQUIRE((a.dxin == nullptr) == (a.dyin == nullptr), "fi_piv_pass_tc: dxin/dyin mismatch");
  FI_REQUIRE(a.box_i0_start >= 0 && a.box_i0_stop <= a.n && a.box_i1_start >= 0 &&
                 a.box_i1_stop <= a.n,
             "fi_piv_pass_tc: bad search box");
  FI_REQUIRE(a.subpix_method >= FI_SUBPIX_GAUSSIAN2 && a.subpix_method <= FI_SUBPIX_NONE,
             "fi_piv_pass_tc: bad subpix_method %d", a.subpix_method);
  FI_REQUIRE(a.subpix_method == FI_SUBPIX_GAUSSIAN2 ||
                 (a.nsubpix >= 1 && a.nsubpix <= FI_MAX_NSUBPIX),
             "fi_piv_pass_tc: nsubpix %d out of 1..%d", a.nsubpix, FI_MAX_NSUBPIX);
  FI_REQUIRE(a.subpix_method != FI_SUBPIX_GAUSSIAN || a.subpix_minv,
             "fi_piv_pass_tc: '2d_gaussian' needs subpix_minv");
  FI_REQUIRE(a.nb_peaks <= FI_MAX_PEAKS, "fi_piv_pass_tc: nb_peaks %d > %d", a.nb_peaks,
             FI_MAX_PEAKS);
  FI_REQUIRE(a.nb_peaks <= 1 || (a.peaks_count && a.peaks && a.peaks_err),
             "fi_piv_pass_tc: secondary peaks need peaks_count, peaks and peaks_err");
  const int64_t nvec64 = (int64_t)a.nx * a.ny;
  FI_REQUIRE(nvec64 < (1ll << 31), "fi_piv_pass_tc: too many vectors");
  const int nvec = (int)nvec64;
  const int npad = a.n / 2;
  cudaStream_t s = (cudaStream_t)stream;
  switch (form) {
    case FI_TC_BF16X1: return tc::launch_tc<FI_TC_BF16X1>(a, nvec, npad, status, s);
    case FI_TC_BF16X3: return tc::launch_tc<FI_TC_BF16X3>(a, nvec, npad, status, s);
    default: return tc::launch_tc<FI_TC_FP16X3>(a, nvec, npad, status, s);
  }
}
