/*
 * fluidimage_gb300 — C ABI of the GB300 (sm_103a) PIV hot path.
 *
 * Every entry point takes plain device pointers and sizes plus a CUDA stream
 * (passed as void*, NULL = legacy default stream), enqueues its kernels on that
 * stream and returns immediately.  The return value is FI_OK (0) or a negative
 * FI_ERR_* code; fi_last_error() gives the message of the calling thread's last
 * failure.  No entry point allocates device memory or synchronises the stream
 * unless stated.  Buffers are owned by the caller.
 *
 * Each entry point cites the upstream fluidimage 0.5.3 interface it replaces
 * (paths inside the fluidimage project).
 */
#ifndef FLUIDIMAGE_GB300_H
#define FLUIDIMAGE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FI_OK 0
#define FI_ERR_INVALID (-1)
#define FI_ERR_CUDA (-2)
#define FI_ERR_UNSUPPORTED (-3)

/* image element types */
#define FI_U8 0
#define FI_U16 1
#define FI_F32 2

/* per-vector error codes written by fi_piv_pass (upstream PIVError strings) */
#define FI_VEC_OK 0
#define FI_VEC_PEAK_BOUNDARY 1 /* "Correlation peak touching boundary." */
#define FI_VEC_PEAK_NAN 2      /* "Correlation peak touching nan."      */
#define FI_VEC_WRONG_SUBPIX 3  /* "wrong subpix" (integer peak kept)     */
#define FI_VEC_BAD_CROP 4      /* "Bad im_crop shape."                   */
#define FI_VEC_ALL_NAN 5       /* plane without finite value (upstream asserts) */
#define FI_VEC_CLOSE_BOUNDARY 6 /* "close boundary" (subpixel crop leaves the plane) */

/* per-vector flag bits written by fi_piv_pass */
#define FI_FLAG_NEAR_TIE 1   /* top two plane values within 1e-6 relative        */
#define FI_FLAG_SUBPIX_TIE 2 /* two 3x3 crop values at the minimum (within 1e-5 of
                                the range): the '2d_gaussian2' 1e-8 floor then
                                depends on float rounding                         */
#define FI_FLAG_SECONDARY_TIE 4 /* near-tie in a secondary peak search          */

/* fix flag bits written by fi_fix */
#define FI_FIX_CORREL_MIN 1     /* "correl < correl_min"        */
#define FI_FIX_DISPLACEMENT 2   /* "delta2 < displacement_max2" */
#define FI_FIX_NEIGHBOUR 4      /* "diff neighbour too large"   */
#define FI_FIX_REPLACED 8       /* replaced by a secondary peak (errors cleared) */

/* Subpixel methods (SubPix.methods, calcul/subpix.py:73) */
#define FI_SUBPIX_GAUSSIAN2 0   /* '2d_gaussian2' (3 x 3, centroid fallback) */
#define FI_SUBPIX_GAUSSIAN 1    /* '2d_gaussian' (least squares, nsubpix)    */
#define FI_SUBPIX_CENTROID 2    /* 'centroid' (nsubpix)                      */
#define FI_SUBPIX_NONE 3        /* 'no_subpix'                               */
#define FI_MAX_NSUBPIX 4        /* crops up to 9 x 9                         */
#define FI_MAX_PEAKS 4          /* nb_peaks_to_search up to 4                */
#define FI_PEAK_FIELDS 5        /* per secondary peak: dx, dy (integer), correl_max,
                                   replacement dx, dy (subpixel fit + input shift) */

const char* fi_last_error(void);

/* Library version string. */
const char* fi_version(void);

/* Number of kernels launched by the library since it was loaded. */
long long fi_launch_count(void);

/* sizeof of fi_piv_pass_args, fi_fix_args and fi_tps_plan (host-only, for bindings). */
int fi_abi_sizes(int64_t* out3);

/*
 * Asynchronous copy of nbytes from device memory to (pinned) host memory on the
 * stream: the few integers the host reads between the TPS stages.
 */
int fi_memcpy_d2h(void* host_dst, const void* device_src, int64_t nbytes, void* stream);

/*
 * Minimum of two images, written as two floats to out_min[0..1] (device).
 * Replaces the "im - im.min()" of BaseWorkPIV._pad_images
 * (works/piv/singlepass.py:196-208).
 */
int fi_images_min(const void* im0, const void* im1, int dtype, int64_t count,
                  float* out_min, void* stream);

/* Arguments of one PIV pass (one window size, all windows of one image pair). */
typedef struct fi_piv_pass_args {
  const void* im0;          /* image 0, row-major height x width (dtype)      */
  const void* im1;          /* image 1, same shape and dtype                  */
  int dtype;                /* FI_U8, FI_U16 or FI_F32                        */
  int height, width;
  const float* im_min;      /* device [2]: minima of im0, im1 (fi_images_min) */
  int n;                    /* window size n x n (16, 24, 32, 48, 64)         */
  const int32_t* ixvecs;    /* grid x centres (nx), device                    */
  int nx;
  const int32_t* iyvecs;    /* grid y centres (ny), device                    */
  int ny;
  const int32_t* dxin;      /* nullable: integer input shift per vector       */
  const int32_t* dyin;      /*   (passes >= 1), device [nx*ny]                */
  const uint8_t* mask;      /* nullable: n*n, 1 where |d| > displacement_max  */
  int box_i0_start, box_i0_stop, box_i1_start, box_i1_stop; /* search box    */
  int particle_radius;      /* second-chance NaN box half width (3)           */
  int apply_subpix;         /* 1: '2d_gaussian2' (+ centroid fallback)        */
  float* deltaxs;           /* out [nvec]                                     */
  float* deltays;           /* out [nvec]                                     */
  float* correls_max;       /* out [nvec]                                     */
  uint8_t* errors;          /* out [nvec] FI_VEC_*                            */
  float* xs;                /* out [nvec] vector x position (midpoint)        */
  float* ys;                /* out [nvec]                                     */
  double* norms;            /* nullable out [nvec]: sqrt(S0 * S1)             */
  float* planes;            /* nullable out [nvec*n*n], fftshift layout       */
  uint8_t* flags;           /* nullable out [nvec] FI_FLAG_*                  */
  int subpix_method;        /* FI_SUBPIX_* (params.piv0.method_subpix)        */
  int nsubpix;              /* crop half width of '2d_gaussian'/'centroid'    */
  const double* subpix_minv;/* '2d_gaussian': pinv of [X^2, Y^2, X, Y, 1],
                               5 x (2 nsubpix + 1)^2 row-major, device        */
  int nb_peaks;             /* params.piv0.nb_peaks_to_search (1..4)          */
  int32_t* peaks_count;     /* out [nvec] if nb_peaks > 1: secondary peaks
                               found, -1 where the peak search raised         */
  float* peaks;             /* out [nvec][nb_peaks-1][FI_PEAK_FIELDS]         */
  uint8_t* peaks_err;       /* out [nvec][nb_peaks-1]: FI_VEC_* of the subpixel
                               fit of each secondary peak                     */
} fi_piv_pass_args;

/*
 * One PIV pass, fused: window extraction (with the integer window shift of
 * passes >= 1), FFT cross-correlation of the mean-removed windows, peak search
 * with the displacement_max mask and the second-chance search, and the
 * '2d_gaussian2' subpixel fit.  One thread group per window, FP32 FFTs in
 * registers, FP64 window energies.
 * Replaces BaseWorkPIV._loop_vectors (works/piv/singlepass.py:262-361) with
 * CorrelFFTNumpy.__call__ (calcul/correl.py:671-685),
 * CorrelBase.compute_displacements_from_correl (calcul/correl.py:226-275),
 * nan_indices_max (calcul/correl.py:88-132) and SubPix.compute_subpix
 * (calcul/subpix.py:107-218), plus the window positions of
 * WorkPIVFromDisplacement (works/piv/singlepass.py:787-870).
 */
int fi_piv_pass(const fi_piv_pass_args* args, void* stream);

/*
 * Batched passes: all passes of window size n of a batch of independent image
 * pairs (each with its own images, shape, dtype, grid, overlap and outputs: one
 * fi_piv_pass_args per pass, in DEVICE memory at pass_args) run in one launch of
 * `items` blocks, each of which takes the next work item (wpb consecutive windows of
 * one pass) from the device counter `counter` (reset by the call).  item_start:
 * device int32 [npass + 1], the first item of each pass (fi_piv_batch_items per
 * pass, accumulated; items = item_start[npass]).  Same per-window computation and
 * outputs as fi_piv_pass (works/piv/singlepass.py:262-361 for each pass); nb_peaks
 * must be 1.  The role of a topology's parallel executors over a series of couples
 * (topologies/piv.py:143-151, executors/multi_exec_async.py:114-158), on one GPU.
 * wpb: 16 or 8 (n = 16), 8 or 4 (n = 24, 32), 2 or 1 (n = 48, 64).
 */
int fi_piv_pass_batch(const fi_piv_pass_args* pass_args, const int32_t* item_start, int npass,
                      int n, int wpb, int items, int32_t* counter, void* stream);
/* Work items of a pass of nvec windows of size n at wpb windows per item (-1: bad). */
int fi_piv_batch_items(int n, int nvec, int wpb);
/* Resident blocks of the batch kernel for (n, wpb) on the current device (-1: bad). */
int fi_piv_batch_max_blocks(int n, int wpb);
/*
 * Image minima of every pass of a batch (the "im - im.min()" of _pad_images,
 * works/piv/singlepass.py:196-208), written through each pass's im_min pointer;
 * keys: device uint32 scratch [2 * npass].
 */
int fi_images_min_batch(const fi_piv_pass_args* pass_args, int npass, uint32_t* keys,
                        void* stream);

/*
 * Image deformation and the differentiable deform-and-correlate chain.  The
 * reference leaves the deformation of im1 between passes as a to-do
 * (works/piv/singlepass.py:736-738); these entry points have no other counterpart.
 *
 * Field: `batch` fields of nodes at sorted coordinates xn[nx], yn[ny] (device
 * float32, nx, ny >= 2), values u, v as [batch][2][ny][nx] device float32; the
 * displacement at a pixel is the bilinear interpolation of its cell's four nodes,
 * constant beyond the outer nodes.
 */
/*
 * out[b][y][x] = im[b] sampled bilinearly at (x + scale u, y + scale v), replicated
 * borders (the central scheme deforms im0 by scale -1/2 and im1 by +1/2).
 */
int fi_dc_warp(const float* nodes, const float* xn, int nx, const float* yn, int ny,
               float scale, const void* im, int dtype, int batch, int height, int width,
               float* out, void* stream);
/*
 * Per non-overlapping 32 x 32 window (batch x height/32 x width/32, row-major): the
 * normalised circular correlation c(m) of (im0, im1w) windows (the plane of
 * CorrelFFTNumpy.__call__, calcul/correl.py:671-685, over its norm) read out by a
 * soft-argmax over the lags m in [-15, 15]^2 at `temperature`:
 * r = sum_m softmax(c / T)(m) m, written as r[w][2] (x, y).  c_zero[w] = c(0),
 * c_peak[w] = max c (both nullable).  float32 images [batch][height][width].
 */
int fi_dc_windows(const float* im0, const float* im1w, int batch, int height, int width,
                  float temperature, float* r, float* c_zero, float* c_peak, void* stream);
/*
 * Adjoint of fi_dc_windows: grad_im1w and, when not NULL, grad_im0 (covered pixels
 * written) from grad_r[w][2].  The correlation planes are recomputed, not stored.
 */
int fi_dc_windows_backward(const float* im0, const float* im1w, int batch, int height,
                           int width, float temperature, const float* grad_r, float* grad_im1w,
                           float* grad_im0, void* stream);
/*
 * Adjoint of fi_dc_warp (same field and scale): grad_nodes (device, accumulated)
 * and, when not NULL, grad_im (float32, accumulated) from
 * grad_out[batch][height][width].
 */
int fi_dc_warp_backward(const float* nodes, const float* xn, int nx, const float* yn, int ny,
                        float scale, const void* im, int dtype, int batch, int height, int width,
                        const float* grad_out, float* grad_nodes, float* grad_im, void* stream);

/* Precision forms of the tensor-core pass (fi_piv_pass_tc). */
#define FI_TC_BF16X1 0 /* one bf16 term per operand                              */
#define FI_TC_BF16X3 1 /* bf16 hi + lo, products hi*hi + hi*lo + lo*hi           */
#define FI_TC_FP16X3 2 /* fp16 hi + lo, 3-term products, power-of-two scaling     */

/*
 * The PIV pass of fi_piv_pass (same arguments, same outputs, same peak search,
 * second chance and subpixel fit) with the correlation planes computed on the
 * tensor cores: the 2-D DFTs of CorrelFFTNumpy.__call__ (calcul/correl.py:671-685
 * with calcul/fft.py:254-269, F[0,0] = 0, _like_fftshift layout) as dense
 * contractions F W F^T in `form` precision (FI_TC_*), accumulated in FP32.
 * 32 x 32 windows.  status: nullable device int, OR-ed with 1 when a wait of the
 * kernel on its tensor-core work timed out (the affected windows are not written).
 * Near-tie flags (FI_FLAG_NEAR_TIE) use the form's plane error as tolerance:
 * 3e-2 (BF16X1), 1e-4 (BF16X3), 1e-5 (FP16X3) relative to the peak.
 */
int fi_piv_pass_tc(const fi_piv_pass_args* args, int form, int* status, void* stream);

/*
 * Per-window plugin contract: correlation planes and norms of `count` window
 * pairs (float32, n x n each, C order), like CorrelFFTNumpy.__call__
 * (calcul/correl.py:671-685) applied to each pair.  planes are written in the
 * "_like_fftshift" layout (calcul/correl.py:596-636).
 */
int fi_correl_windows(const float* win0, const float* win1, int count, int n,
                      float* planes, double* norms, void* stream);

/*
 * Peak search (+ optional subpixel fit) on planes already in device memory,
 * with the semantics of CorrelFFTBase.compute_displacements_from_correl
 * (calcul/correl.py:561-568, 226-275) and CorrelBase.apply_subpix
 * (calcul/correl.py:277-281).  When mask is NULL the second-chance NaN box is
 * written into `planes` in place, as upstream does.  Outputs as fi_piv_pass
 * (integer displacements when apply_subpix == 0), plus the peak indices; with
 * nb_peaks > 1 the other peaks (correl.py:250-273) go to peaks_count / peaks /
 * peaks_err as in fi_piv_pass_args (replacement fields without input shift).
 */
int fi_peaks_from_planes(float* planes, const double* norms, int count, int n,
                         const uint8_t* mask, int box_i0_start, int box_i0_stop,
                         int box_i1_start, int box_i1_stop, int particle_radius,
                         int apply_subpix, int subpix_method, int nsubpix,
                         const double* subpix_minv, int nb_peaks, float* deltaxs,
                         float* deltays, float* correls_max, uint8_t* errors,
                         int32_t* peak_i0, int32_t* peak_i1, int32_t* peaks_count,
                         float* peaks, uint8_t* peaks_err, void* stream);

/*
 * Subpixel fit (FI_SUBPIX_*, nsubpix, subpix_minv as in fi_piv_pass_args) at given
 * peak indices (peak_i0 = row, peak_i1 = column) on planes in device memory: the
 * CorrelBase.apply_subpix / SubPix.compute_subpix pair (calcul/correl.py:277-281,
 * calcul/subpix.py:107-218).  Writes displacements and FI_VEC_* codes
 * (FI_VEC_WRONG_SUBPIX, FI_VEC_CLOSE_BOUNDARY keep the integer displacement).
 */
int fi_subpix_at(const float* planes, int count, int n, const int32_t* peak_i0,
                 const int32_t* peak_i1, int subpix_method, int nsubpix,
                 const double* subpix_minv, float* deltaxs, float* deltays, uint8_t* errors,
                 void* stream);

/* Arguments of the false-vector removal of one pass. */
typedef struct fi_fix_args {
  int nx, ny;                  /* vector grid                                  */
  const float* deltaxs;        /* in [nvec] (pass output)                      */
  const float* deltays;
  const float* correls_max;    /* in [nvec]                                    */
  const uint8_t* errors;       /* in [nvec] FI_VEC_*                           */
  float correl_min;            /* -inf to disable                              */
  int use_displacement_max;
  float displacement_max;      /* fix.displacement_max                         */
  int use_threshold;
  float threshold;             /* fix.threshold_diff_neighbour                 */
  float* deltaxs_out;          /* out [nvec]: NaN where removed                */
  float* deltays_out;
  uint8_t* fix_flags;          /* out [nvec] FI_FIX_*                          */
  float* diff2;                /* out [nvec]: |d - mean8(d)|^2 (float32)       */
  float* work;                 /* scratch [2*nvec] (floats)                    */
  /* secondary peaks (fix.py:135-236); nb_peaks > 1 needs use_threshold,
     diff2 and the outputs below */
  int nb_peaks;                /* fi_piv_pass nb_peaks (1: no replacement)     */
  const int32_t* peaks_count;  /* fi_piv_pass outputs                          */
  const float* peaks;
  const uint8_t* peaks_err;
  const int32_t* dxin;         /* nullable: the pass's integer input shifts    */
  const int32_t* dyin;
  double threshold64;          /* fix.threshold_diff_neighbour (float64)      */
  double displacement_max64;   /* fix.displacement_max (0: none)              */
  float* correls_max_out;      /* out [nvec]: correls_max after replacement (may
                                  alias correls_max)                          */
  float* replaced;             /* out [nvec][3]: old dx, dy, correl_max        */
} fi_fix_args;

/*
 * WorkFIX.calcul (works/piv/fix.py:66-243) with mean_neighbors_xy
 * (calcul/mean_neighbors.py:128-155): errors, correl_min, displacement_max and
 * neighbour tests, then (nb_peaks > 1) the replacement of a vector by the
 * secondary peak closest to the neighbour mean (FI_FIX_REPLACED).
 */
int fi_fix(const fi_fix_args* args, void* stream);

/*
 * WorkFIX stages A and B (works/piv/fix.py:66-133) over the vectors of many passes
 * in two launches: fix_args, device array [npass] (each with its own work buffer
 * when use_threshold); vec_start: device int32 [npass + 1], first vector of each
 * pass; total = vec_start[npass].  Secondary peaks (nb_peaks > 1) are not handled
 * here (fi_fix per pass).  A pass with the neighbour test needs a grid of at least
 * 2 x 2 (its vectors are otherwise passed through untested; fi_fix rejects it).
 */
int fi_fix_batch(const fi_fix_args* fix_args, const int32_t* vec_start, int npass, int total,
                 void* stream);

/*
 * fi_fix without a caller-provided work buffer, for callers that cannot allocate
 * device memory (a host framework that owns a fixed device-memory budget, or a
 * latency-critical loop where cudaMalloc and its implicit device synchronisation
 * are not allowed).  No counterpart in the reference: it is the same WorkFIX
 * computation as fi_fix, with its scratch (args->work is ignored) in a static
 * device array of 2 * FI_FIX_STATIC_MAX_VECTORS floats (2 MiB) that every GPU
 * loading this library holds until the process exits.  Grids of more than
 * FI_FIX_STATIC_MAX_VECTORS vectors are rejected with FI_ERR_INVALID.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture.  It allocates nothing (no cudaMalloc, no cudaFree).  All
 * calls on a device share the array: calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 */
#define FI_FIX_STATIC_MAX_VECTORS 262144
int fi_fix_static(const fi_fix_args* args, void* stream);

/* ---------------------------------------------------------------------------
 * Thin-plate-spline subdomain interpolation (FP64), the apply_interp of
 * works/piv/singlepass.py:409-563 with ThinPlateSplineSubdom
 * (calcul/interpolate/thin_plate_spline_subdom.py:25-280).
 * The host drives the stages; sizes that depend on data (number of valid
 * vectors, subdomain populations) are read back between stages.
 * ------------------------------------------------------------------------- */

/*
 * A TPS plan buffer (device memory) holds the header below at its start and, from
 * byte 256, the scratch of the multi-block compaction: callers of fi_tps_plan_make
 * provide FI_TPS_PLAN_BYTES bytes.
 */
#define FI_TPS_PLAN_MAX_BLOCKS 1024
#define FI_TPS_PLAN_BYTES (256 + 24 * FI_TPS_PLAN_MAX_BLOCKS)

/* Header of a TPS plan (device memory, written by fi_tps_plan). */
typedef struct fi_tps_plan {
  int num_centers;      /* valid (non-NaN) vectors                        */
  int nb_subdomx, nb_subdomy;
  int status;           /* 0, or 1 when there is no valid vector          */
  double smoothing;     /* smoothing_coef normalised by subdomain area     */
  double x_min, x_max, y_min, y_max;
  double buffer_x, buffer_y;
} fi_tps_plan;

/*
 * Select the valid vectors (non-NaN dx and dy, order kept) and compute the
 * subdomain layout (ThinPlateSplineSubdom.__init__, thin_plate_spline_subdom.py:
 * 38-126).  xs, ys, dx, dy: float32 [nvec].  Outputs the centres cx, cy (float64),
 * the values ux, uy (float32) and, if not NULL, the original index of each
 * selected vector.  The header *plan is written in device memory; the host reads
 * num_centers, nb_subdomx, nb_subdomy and status from it before the next stages.
 * plan points to FI_TPS_PLAN_BYTES bytes (header and compaction scratch).
 */
int fi_tps_plan_make(const float* xs, const float* ys, const float* dx, const float* dy,
                     int nvec, int subdom_size, double smoothing_coef,
                     double percent_buffer_area, fi_tps_plan* plan, double* cx, double* cy,
                     float* ux, float* uy, int32_t* selection, void* stream);

/*
 * Half-integer lattice coordinates of npts points: xy2[2i] = 2 px[i],
 * xy2[2i+1] = 2 py[i] as int32, and *on_lattice (device int) = 1 when every point
 * has integral 2x, 2y with |2x|, |2y| < 2^30 (PIV vector positions always do:
 * grid points and midpoints of integer window shifts), else 0.
 */
int fi_tps_lattice(const double* px, const double* py, int npts, int32_t* xy2,
                   int32_t* on_lattice, void* stream);

/*
 * Index over the points for fi_tps_members, by tiles of 256 consecutive points:
 * y_pmax[j] = max of py over tiles 0..j, y_smin[j] = min over tiles j..end
 * (ceil(npts / 256) doubles each).  Both are monotone, so the scan for a
 * subdomain's y band covers only the tiles that can hold members (exact for any
 * point order; a narrow band for row-ordered PIV grids).  No reference counterpart:
 * an index that replaces the all-points scan of np.where in
 * ThinPlateSplineSubdom (thin_plate_spline_subdom.py:107, 179).
 */
int fi_tps_y_bounds(const double* py, int npts, double* y_pmax, double* y_smin, void* stream);

/*
 * Exclusive prefix sums for the buffers of nb_subdom subdomains from the member
 * counts of the centres and of the new positions (fi_tps_members mode 0): CSR
 * offsets of both, matrix slots ((n_i+3)^2 rounded up to 4 elements, as
 * fi_tps_solve_mp wants) and weights (2 (n_i+3)); summary[6] = total members, total
 * new members, matrix elements, weight elements, max members, max new members;
 * order (nullable, [nb_subdom]) = the subdomains by decreasing member count (ties
 * by index; the identity above 8192 subdomains), the block order of
 * fi_tps_solve_mp.  No reference counterpart (the host-side bookkeeping of
 * ThinPlateSplineSubdom).
 */
int fi_tps_offsets(const int32_t* counts, const int32_t* ncounts, int nb_subdom,
                   int64_t* offsets, int64_t* noffsets, int64_t* mat_offsets,
                   int64_t* w_offsets, int64_t* summary, int32_t* order, void* stream);

/*
 * Ordered subdomain membership of npts points (px, py float64).  mode 0 writes
 * counts[nb_subdom]; mode 1 writes, at offsets[i] (exclusive prefix sums of the
 * counts), the point indices and their norm coefficients
 * (_compute_coef_norm, thin_plate_spline_subdom.py:208-222).  With xy2 (8-byte
 * aligned) and on_lattice from fi_tps_lattice (both nullable) the limit tests are
 * exact integer comparisons on the lattice.  y_pmax / y_smin (nullable, fi_tps_y_bounds of py)
 * restrict the scan to the tiles that can hold members.
 */
int fi_tps_members(const fi_tps_plan* plan, int nb_subdom, const double* px, const double* py,
                   int npts, int mode, int32_t* counts, const int64_t* offsets,
                   int32_t* indices, double* coefs, const int32_t* xy2,
                   const int32_t* on_lattice, const double* y_pmax, const double* y_smin,
                   void* stream);

/*
 * The layout stages of one TPS interpolation in one call: fi_tps_lattice of the
 * centres (cx, cy) and, unless p_given, of the new positions (px, py) (else pxy2 /
 * plat are read); fi_tps_y_bounds of both; the member counts of both
 * (fi_tps_members mode 0) and fi_tps_offsets.  nb_subdom and num_centers are
 * capacities (at least the plan's subdomains and valid centres, e.g. nvec for the
 * centres): the kernels read the actual counts from *plan on the device, so that the
 * host needs no copy of the plan before this call and reads the plan header and the
 * summary after it in one synchronisation; with a plan of more subdomains than
 * nb_subdom, only the first nb_subdom are laid out and the caller calls again with
 * the plan's count.  Buffers: cxy2 [2 num_centers], pxy2 [2 npts], clat / plat [1],
 * cbounds / pbounds [2 ceil(n / 256)] (y_pmax then y_smin, n = num_centers / npts),
 * counts / ncounts [nb_subdom], offsets [4 nb_subdom + 6] (offsets, noffsets,
 * mat_offsets, w_offsets, summary), order (nullable, [nb_subdom]) as in
 * fi_tps_offsets.  No reference counterpart (the
 * bookkeeping of ThinPlateSplineSubdom.__init__ / init_with_new_positions,
 * thin_plate_spline_subdom.py:25-127, 160-206).
 */
int fi_tps_layout(const fi_tps_plan* plan, int nb_subdom, const double* cx, const double* cy,
                  int num_centers, const double* px, const double* py, int npts, int p_given,
                  int32_t* cxy2, int32_t* clat, int32_t* pxy2, int32_t* plat, double* cbounds,
                  double* pbounds, int32_t* counts, int32_t* ncounts, int64_t* offsets,
                  int32_t* order, void* stream);

/*
 * Both membership fills (fi_tps_members mode 1) after fi_tps_layout, with the same
 * capacities nb_subdom and num_centers: the centres into indices / coefs at
 * offsets[0:nb_subdom], the new positions into nindices / ncoefs at
 * offsets[nb_subdom:2 nb_subdom]; the other buffers as fi_tps_layout wrote them.
 */
int fi_tps_members_fill(const fi_tps_plan* plan, int nb_subdom, const double* cx,
                        const double* cy, int num_centers, const double* px, const double* py,
                        int npts, const int32_t* cxy2, const int32_t* clat, const int32_t* pxy2,
                        const int32_t* plat, const double* cbounds, const double* pbounds,
                        const int64_t* offsets, int32_t* indices, double* coefs,
                        int32_t* nindices, double* ncoefs, void* stream);

/*
 * Per subdomain: build [[K + smoothing I, P], [P^T, 0]] (compute_tps_weights,
 * thin_plate_spline.py:168-216), LU-factorise it once with partial pivoting and
 * run the iterative outlier replacement of compute_tps_weights_iter
 * (thin_plate_spline_subdom.py:236-280) for both components on the same factors.
 * matrices: scratch, (n_i+3)^2 doubles at mat_offsets[i]; pivots: scratch,
 * n_i+3 ints at offsets[i] + 3 i; weights: 2 (n_i+3) doubles at w_offsets[i]
 * (x then y); smoothed_x/y: n_i doubles at offsets[i].  iters, nfixed,
 * max_udiff: [2 * nb_subdom] (x, y); singular: [nb_subdom] (1 = zero pivot,
 * where upstream raises LinAlgError).  When only_failed is not NULL, subdomains
 * with only_failed[i] == 0 are skipped (already solved by fi_tps_solve_mp).
 */
int fi_tps_solve(const fi_tps_plan* plan, int nb_subdom, int max_members, const double* cx,
                 const double* cy, const float* ux, const float* uy, const int32_t* counts,
                 const int64_t* offsets, const int32_t* indices, const int64_t* mat_offsets,
                 double* matrices, int32_t* pivots, double threshold, int use_threshold,
                 const int64_t* w_offsets, double* weights, double* smoothed_x,
                 double* smoothed_y, int32_t* iters, int32_t* nfixed, int32_t* singular,
                 double* max_udiff, const int32_t* only_failed, void* stream);

/*
 * Table of phi(k / 4) = (k/4) log(k/4) / 2 for k < count (float64): the TPS kernel
 * values on the half-integer lattice of PIV vector positions
 * (compute_tps_matrix, thin_plate_spline.py:136-145).  Built once per device.
 */
int fi_tps_phi_table(double* table, int64_t count, void* stream);

/*
 * The same table as (hi, lo) float pairs (2 * count floats, 8-byte aligned): the
 * double-float evaluation of fi_tps_interpolate.  No reference counterpart.
 */
int fi_tps_phi_table2(float* table2, int64_t count, void* stream);

/*
 * Mixed-precision TPS solve (same inputs and outputs as fi_tps_solve): null-space
 * form B z = Q2^T u with B = Q2^T (K + lam I) Q2 (P = Q R, Householder; B projected
 * in double-float with the compact WY form of Q), factorised in FP32 (blocked Cholesky) and
 * refined with double-float (pairs of floats) residuals g - B z; the affine part is
 * a = R^-1 (Q1^T u - Q1^T A Q2 z).  K comes from the phi table.  The outlier
 * iterations of compute_tps_weights_iter (thin_plate_spline_subdom.py:236-280)
 * warm-start from the previous solution.  mat_offsets[i] must be multiples of 4 and
 * both matrix buffers 16-byte aligned: matrices holds (n_i+3)^2 doubles at
 * mat_offsets[i] (B as float pairs), matrices32 (n_i+3)^2 floats (its Cholesky
 * factor).  cxy2/c_on_lattice (nullable, fi_tps_lattice of the centres) give
 * integer indices into phi_table and phi_table2 (nullable; fi_tps_phi_table2 of the
 * same size, the pairs the double-float projection reads).  status[i] = 0 when solved, 1 when the subdomain must go
 * through fi_tps_solve (pass status as its only_failed argument): rank-deficient P,
 * Cholesky breakdown or no convergence.  sweeps (nullable, [nb_subdom]): refinement
 * sweeps (one FP32 solve each) per subdomain.  order (nullable, fi_tps_offsets):
 * the subdomains in the order the blocks take them (largest first shortens the
 * last wave).  With order, a solve of more subdomains than one wave of resident
 * blocks but fewer than two runs its last subdomains as clusters of two blocks on a
 * side stream of the library (one per host thread and device, created on the first
 * such call), joined back into `stream` by an event before the call returns.
 */
int fi_tps_solve_mp(const fi_tps_plan* plan, int nb_subdom, int max_members, const double* cx,
                    const double* cy, const float* ux, const float* uy, const int32_t* counts,
                    const int64_t* offsets, const int32_t* indices, const int64_t* mat_offsets,
                    double* matrices, float* matrices32, const double* phi_table,
                    const float* phi_table2, int64_t table_size, const int32_t* cxy2,
                    const int32_t* c_on_lattice, double threshold, int use_threshold,
                    const int64_t* w_offsets, double* weights, double* smoothed_x,
                    double* smoothed_y, int32_t* iters, int32_t* nfixed, int32_t* status,
                    double* max_udiff, int32_t* sweeps, const int32_t* order, void* stream);

/*
 * griddata of apply_interp (calcul/interpolate/griddata.py:11-27,
 * works/piv/singlepass.py:498-556): the values (ux, uy) of the num_centers valid
 * vectors of a pass (cx, cy, selection: the compaction of fi_tps_plan_make;
 * selection[i] = index of centre i in the pass's nx x ny window grid, whose node
 * coordinates are ixvecs, iyvecs) interpolated linearly on their Delaunay
 * triangulation at npts points (px, py), and set to the nearest centre's value
 * outside the convex hull.  Positions must be half-integers (PIV vector positions
 * are).  out_x/out_y (float64), rx/ry (nullable, rounded half to even as the next
 * pass's shifts), flags (nullable, uint8): bit 0 = the point lies in a cell of four
 * or more cocircular centres (several Delaunay triangulations exist; the triangle
 * with the smallest centre indices is used), bit 1 = equidistant nearest centres
 * (the smallest index is used).  scratch: fi_griddata_scratch_ints(nx, ny) int32,
 * 8-byte aligned.  *status (device int32) = 0, or 1 (a point off the half-integer
 * lattice), 2 (no certified triangle: not expected), 3 (bad selection).
 */
int fi_griddata(const double* cx, const double* cy, const float* ux, const float* uy,
                const int32_t* selection, int num_centers, const int32_t* ixvecs, int nx,
                const int32_t* iyvecs, int ny, const double* px, const double* py, int npts,
                int32_t* scratch, double* out_x, double* out_y, int32_t* rx, int32_t* ry,
                uint8_t* flags, int32_t* status, void* stream);

/* Scratch size (int32 elements) of fi_griddata for an nx x ny window grid. */
int64_t fi_griddata_scratch_ints(int nx, int ny);

/*
 * Smoothed values at the centres, blended over the subdomains that contain them
 * (compute_tps_weights_subdom, thin_plate_spline_subdom.py:128-159).
 */
int fi_tps_blend_centers(const fi_tps_plan* plan, int num_centers, const double* cx,
                         const double* cy, const int32_t* counts, const int64_t* offsets,
                         const int32_t* indices, const double* coefs, const double* smoothed_x,
                         const double* smoothed_y, double* out_x, double* out_y, void* stream);

/*
 * The *_smooth fields of the last pass (works/piv/singlepass.py:515-529): xs_s/ys_s
 * (float32) = px/py + offx/offy of the final grid, dx_s/dy_s = out_x/out_y, except at
 * the n_sel selected vectors (sel[k], int32: their index on the grid), which take
 * their own positions (xs/ys float32 + offsets when vec_xy, else the grid's) and the
 * smoothed values smooth_x[k]/smooth_y[k].  Sums in float64, rounded to float32.
 */
int fi_tps_smooth_fields(const double* px, const double* py, int npts, const float* xs,
                         const float* ys, int vec_xy, double offx, double offy,
                         const int32_t* sel, int n_sel, const double* out_x,
                         const double* out_y, const double* smooth_x, const double* smooth_y,
                         float* xs_s, float* ys_s, double* dx_s, double* dy_s, void* stream);

/*
 * Interpolation at npts new positions (init_with_new_positions + interpolate,
 * thin_plate_spline_subdom.py:161-234): out_x/out_y float64 and, if not NULL,
 * out_rx/out_ry = round-half-even to int32 (the window shifts of the next pass,
 * works/piv/singlepass.py:752-753).  ncounts/noffsets/nindices/ncoefs: membership
 * of the new positions (fi_tps_members); partx/party: scratch of the same size
 * as nindices.  cxy2/c_on_lattice (nullable, from fi_tps_lattice on the centres)
 * enable integer 4 r^2 table indices; with phi_table2 (nullable, fi_tps_phi_table2)
 * the kernel sums on the lattice run in double-float (~1e-14 relative per term).
 * table_entries (0: 2048, at most 16384): capacity of the per-block shared-memory
 * copy of the kernel values of a grid's offsets, used where the new positions lie on
 * a grid and the centres on it or half a pixel off it (a larger table costs shared
 * memory, and so L1 capacity, on every block of the launch).
 */
int fi_tps_interpolate(const fi_tps_plan* plan, int nb_subdom, int max_members,
                       int max_new_members, const double* cx, const double* cy,
                       const int32_t* counts, const int64_t* offsets, const int32_t* indices,
                       const int64_t* w_offsets, const double* weights, const double* px,
                       const double* py, int npts, const int32_t* ncounts,
                       const int64_t* noffsets, const int32_t* nindices, const double* ncoefs,
                       double* partx, double* party, double* out_x, double* out_y,
                       int32_t* out_rx, int32_t* out_ry, const double* phi_table,
                       const float* phi_table2, int64_t table_size, const int32_t* cxy2,
                       const int32_t* c_on_lattice, int table_entries, void* stream);

/* ---------------------------------------------------------------------------
 * Image preprocessing (works/preproc/_toolbox_py.py)
 * ------------------------------------------------------------------------- */
#define FI_PRE_U8 0
#define FI_PRE_U16 1
#define FI_PRE_F32 2
#define FI_PRE_F64 3
/* scipy.ndimage boundary modes */
#define FI_MODE_REFLECT 0  /* d c b a | a b c d | d c b a */
#define FI_MODE_CONSTANT 1 /* k k k k | a b c d | k k k k (cval) */
#define FI_MODE_NEAREST 2  /* a a a a | a b c d | d d d d */
#define FI_MODE_MIRROR 3   /* d c b | a b c d | c b a */
#define FI_MODE_WRAP 4     /* a b c d | a b c d | a b c d */

/*
 * Rank filter of a stack of nt images ny x nx (FI_PRE_* dtype, C order) over a box
 * window st x sy x sx, output in the input dtype: the rank-th smallest window value
 * (scipy.ndimage.rank_filter semantics: window [i - s//2, i - s//2 + s - 1], the
 * boundary mode and cval); rank 0 / st*sy*sx - 1 are the minimum / maximum filters
 * (separable; scratch: 2 * nt*ny*nx uint64), other ranks an exact radix select.
 * Replaces ndi.minimum_filter / median_filter / percentile_filter in sliding_* and
 * temporal_* (works/preproc/_toolbox_py.py:66-155, 189-256).
 */
int fi_rank_filter(const void* in, void* out, int dtype, int nt, int ny, int nx, int st, int sy,
                   int sx, int rank, int mode, double cval, void* scratch, void* stream);

/*
 * out = img - weight * filtered in numpy's result dtype out_dtype (FI_PRE_F64,
 * FI_PRE_F32, or the image's integer dtype for an integer weight: modular
 * arithmetic), with negatives set to 0 when clamp (sliding_* tools,
 * _toolbox_py.py:88-91).
 */
int fi_subtract_weighted(const void* img, const void* filtered, int dtype, int64_t count,
                         double weight, int out_dtype, int clamp, void* out, void* stream);

/* global_threshold (_toolbox_py.py:265-289): values below lo set to lo, above hi to hi. */
int fi_clamp(const void* in, int dtype, int64_t count, double lo, double hi, void* out,
             void* stream);

/*
 * Partial sums of img**2 (squares in the image dtype, wrapping for integers as
 * numpy does) and partial maxima of img, one per block (nparts blocks), for
 * rescale_intensity_tanh (_toolbox_py.py:332-355).
 */
int fi_sq_sum_max(const void* in, int dtype, int64_t count, double* part_sum, double* part_max,
                  int nparts, void* stream);

/* out = floor(scale * tanh(img / threshold)) in float64 (rescale_intensity_tanh). */
int fi_tanh_rescale(const void* in, int dtype, int64_t count, double threshold, double scale,
                    double* out, void* stream);

/*
 * Partial extremes of img (NaN-propagating like ndarray.min / max), one pair per
 * block: part[0, nparts) the minima, part[nparts, 2 nparts) the maxima; nparts <= 4096.
 */
int fi_min_max(const void* in, int dtype, int64_t count, double* part, int nparts, void* stream);

/*
 * rescale_intensity (_toolbox_py.py:313-331, skimage.exposure.rescale_intensity of
 * scikit-image 0.24 with in_range='image', out_range=(omin, omax)): the image's
 * extremes come from fi_min_max's partials on the device (no host round trip);
 * out = (x - imin) / (imax - imin) * (omax - omin) + omin, float32 for float32 images
 * and float64 otherwise; x clipped to [omin, omax] when imin == imax.
 */
int fi_rescale_intensity(const void* in, int dtype, int64_t count, const double* part, int nparts,
                         double omin, double omax, void* out, void* stream);

/*
 * gamma_correction (_toolbox_py.py:441-470, skimage.exposure.adjust_gamma of
 * scikit-image 0.24): uint8 images through a 256-entry device table lut
 * (rint(255 gain linspace(0, 1, 256) ** gamma), capped at 255); other dtypes
 * ((x / scale) ** gamma) scale gain in the image dtype, scale = 65535 for uint16 and
 * 1 for floats, the uint16 result truncated.  gamma >= 0; the caller rejects
 * negative images (upstream raises ValueError).
 */
int fi_gamma(const void* in, int dtype, int64_t count, double gamma, double gain,
             const uint8_t* lut, void* out, void* stream);

/*
 * equalize_hist_global (_toolbox_py.py:357-379, skimage.exposure.equalize_hist of
 * scikit-image 0.24) of integer images: the histogram of the raw values (hist:
 * 256 / 65536 uint32 scratch), cdf (same length, float64) = cumulative counts /
 * pixels, out (float64) = cdf[x].
 */
int fi_equalize_hist_int(const void* in, int dtype, int64_t count, unsigned* hist, double* cdf,
                         double* out, void* stream);

/*
 * equalize_hist_global of float images: numpy's uniform histogram of nbins bins
 * (edges: nbins + 1 values in the image's float type, first = edges[0], denom =
 * the range, both exactly as numpy computes them), the cumulative distribution
 * (float32 for float32 images), and np.interp of the pixels at the bin centres
 * (centers: nbins float64), out in the image's float type.
 */
int fi_equalize_hist_float(const void* in, int dtype, int64_t count, const void* edges, int nbins,
                           double first, double denom, const double* centers, unsigned* hist,
                           double* cdf, void* out, void* stream);

/*
 * The core of equalize_hist_adapt (_toolbox_py.py:383-409; scikit-image 0.24's
 * exposure.equalize_adapthist, CLAHE): levels = the (ny, nx) image rescaled to
 * [0, 2^14 - 1] (float32 or float64, dtype), truncated to grey levels; contextual
 * regions of k0 x k1 pixels (the image extended at its end by reflection), each
 * region's histogram of nbins bins (1 <= nbins <= 12000) clipped at
 * max(clip_limit k0 k1, 1) with the excess redistributed, its grey-level map (maps:
 * ceil(ny / k0) * ceil(nx / k1) * nbins uint16 scratch), and the bilinear blend of
 * the four maps around each pixel summed in float32 and truncated: out (same dtype
 * as levels) holds the equalised grey levels.
 */
int fi_clahe(const void* levels, int dtype, int ny, int nx, int k0, int k1, int nbins,
             double clip_limit, uint16_t* maps, void* out, void* stream);

/*
 * scikit-image's img_as_ubyte of a float image in [0, 1] (the step before the rank
 * equalisation of equalize_hist_local, _toolbox_py.py:433-435): rint(x * 255) in the
 * image's float type, clipped to [0, 255].
 */
int fi_to_ubyte(const void* in, int dtype, int64_t count, uint8_t* out, void* stream);

/*
 * equalize_hist_local's rank equalisation (_toolbox_py.py:412-438; scikit-image's
 * filters.rank.equalize over morphology.disk(radius)) of a (ny, nx) uint8 image: out
 * = 255 n / pop truncated, pop the disk's pixels inside the image, n those at most
 * the centre pixel.
 */
int fi_rank_equalize(const uint8_t* in, int ny, int nx, int radius, uint8_t* out,
                     void* stream);

/*
 * scipy.ndimage.gaussian_filter of each image of a (nt, ny, nx) stack (axis y then x;
 * the call of sharpen, _toolbox_py.py:486-487): one symmetric 1-D correlation per
 * axis in float64 ('reflect' boundaries; out = w_0 x_0, then the tap pairs from the
 * outermost inwards, no contraction), each pass cast to the image dtype (truncation
 * for the integer types).  weights: device array of 2 radius + 1 float64 (scipy's
 * normalised kernel, _gaussian_kernel1d); tmp: a buffer like out.
 */
int fi_gaussian_filter(const void* in, void* out, void* tmp, int dtype, int nt, int ny, int nx,
                       const double* weights, int radius, void* stream);

/*
 * sharpen's last line (_toolbox_py.py:489): out = blurred + alpha * (blurred -
 * filtered) with numpy's promotions: integer images subtract in their own type
 * (wrapping) and give float64, float32 stays float32, float64 is float64.
 */
int fi_sharpen_combine(const void* blurred, const void* filtered, int dtype, int64_t count,
                       double alpha, void* out, void* stream);

/*
 * Image decode (fluidimage.util.imread, util/util.py:46-59, which reads the image
 * files through fluiddyn.io.image): writes the (height, width) image `out` (uint8 for
 * 1-byte samples, uint16 for 2-byte samples) from a container's pixel payload `raw`
 * (raw_bytes bytes on the device).  Row r starts at byte row_offsets[r] (device,
 * height int64): TIFF strips, bottom-up BMP rows and row padding are offsets.
 * 2-byte samples are big-endian when big_endian is set, else little-endian; lut
 * (device, 256 bytes, nullable) maps 1-byte samples (a BMP palette); invert maps
 * WhiteIsZero images to BlackIsZero (255 - v, 65535 - v).  A row outside the payload
 * is written as zeros and sets *status to 1 (status: device int32, nullable).
 */
int fi_image_unpack(const uint8_t* raw, int64_t raw_bytes, const int64_t* row_offsets,
                    int height, int width, int bytes_per_sample, int big_endian,
                    const uint8_t* lut, int invert, void* out, int32_t* status, void* stream);

/*
 * PNG scanline reconstruction (the PNG files read by fluiddyn.io.image for
 * fluidimage.util.imread; RFC 2083 section 6 filters None, Sub, Up, Average, Paeth).
 * HOST memory, synchronous: `filtered` holds height rows of 1 + row_bytes bytes (the
 * filter type byte, then the row), out receives height * row_bytes bytes; bpp = bytes
 * per complete pixel (at least 1).  FI_ERR_INVALID on an undefined filter type.
 */
int fi_png_unfilter(const uint8_t* filtered, int height, int row_bytes, int bpp, uint8_t* out);

#ifdef __cplusplus
}
#endif

#endif /* FLUIDIMAGE_GB300_H */
