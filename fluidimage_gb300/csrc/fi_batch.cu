// Batched single-pass PIV over many passes of mixed image sizes, dtypes, window
// sizes and overlaps: one launch per window size whose blocks take work items (WPB
// windows of one pass) from a device counter, the image minima of every couple in
// one launch.  The per-window code is that of the single-pass kernels
// (fi_window.cuh); the parallel executors of a PIV topology (topologies/piv.py:143-151,
// executors/multi_exec_async.py:114-158) are what this replaces for single-pass works.
#include <cstdint>

#include "fi_common.cuh"
#include "fi_fft.cuh"
#include "fi_peak.cuh"
#include "fi_window.cuh"

namespace fi {

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
    case 8: return Cfg<8>::GROUP_BYTES;
    case 12: return Cfg<12>::GROUP_BYTES;
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
    case 8: case 12: case 16: return wpb == 16 || wpb == 8;
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

extern "C" int fi_piv_batch_items(int n, int nvec, int wpb) {
  if (!supported_n_batch(n) || nvec <= 0 || !batch_wpb_ok(n, wpb)) return -1;
  return (nvec + wpb - 1) / wpb;
}

extern "C" int fi_piv_batch_max_blocks(int n, int wpb) {
  if (!supported_n_batch(n) || !batch_wpb_ok(n, wpb)) return -1;
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
  FI_OCC(8, 16) FI_OCC(8, 8) FI_OCC(12, 16) FI_OCC(12, 8)
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
  FI_REQUIRE(supported_n_batch(n), "fi_piv_pass_batch: window size %d not supported", n);
  FI_REQUIRE(batch_wpb_ok(n, wpb),
             "fi_piv_pass_batch: %d windows per item not available for %d px windows", wpb, n);
  cudaStream_t s = (cudaStream_t)stream;
  FI_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int32_t), s));
#define FI_BATCH(NN, WW) \
  if (n == NN && wpb == WW) return launch_batch<NN, WW>(pass_args, item_start, npass, items, counter, s);
  FI_BATCH(8, 16) FI_BATCH(8, 8) FI_BATCH(12, 16) FI_BATCH(12, 8)
  FI_BATCH(16, 16) FI_BATCH(16, 8) FI_BATCH(24, 8) FI_BATCH(24, 4) FI_BATCH(32, 8) FI_BATCH(32, 4)
  FI_BATCH(48, 2) FI_BATCH(48, 1) FI_BATCH(64, 2) FI_BATCH(64, 1)
#undef FI_BATCH
  return FI_ERR_INVALID;
}
