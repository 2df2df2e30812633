/*
 * dic.h -- C ABI of the GB300 2D-DIC engine (FFTCC seed + first-order IC-GN).
 *
 * One engine = one GPU, one host thread, one CUDA stream.  It holds the reference image,
 * its gradients and the per-POI reference data (mean, norms, inverse Hessian) resident
 * on the device across frames, and rebuilds only the target B-spline table per frame.
 *
 * The entry points replace the C++ solver classes of FastICGN / OpenCorr:
 *   ICGN2D1CudaMvp  (src/icgn2d1_cuda_mvp.h:98-143)  and  ICGN2D1  (src/oc_icgn.h:45-77)
 *   FFTCC2DCuda     (src/fftcc2d_cuda.h:85-109)      and  FFTCC2D  (src/oc_fftcc.h:56-100)
 * One engine serves both solvers, so a target frame is uploaded once instead of twice.
 *
 * Conventions: no exceptions cross this boundary.  Every call returns DIC_OK (0) or a
 * negative dic_status and leaves a message for dic_last_error().  Host buffers are
 * caller-owned and are only read/written during the call.  Results follow the CPU
 * OpenCorr rules (src/oc_icgn.cpp:168-387): zncc carries -3 (rejected before or during
 * iteration because the subset left the image or the seed was unusable), -4 (no
 * convergence within max_iteration) or -5 (non-finite result), exactly where the CPU path
 * assigns them.
 */
#ifndef GB300_DIC_H
#define GB300_DIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DIC_ABI_VERSION 2

typedef enum dic_status
{
  DIC_OK = 0,
  DIC_ERR_ARGUMENT = -1,   /* std::invalid_argument in the reference */
  DIC_ERR_STATE = -2,      /* std::logic_error: a required set/prepare step is missing */
  DIC_ERR_RANGE = -3,      /* std::out_of_range: cache index outside the prepared layout */
  DIC_ERR_CUDA = -4,       /* a CUDA runtime call failed */
  DIC_ERR_MEMORY = -5      /* device or pinned allocation failed */
} dic_status;

typedef enum dic_dtype
{
  DIC_U8 = 1,    /* 8-bit grey levels (Image2D Compat8) */
  DIC_U16 = 2,   /* 12- or 16-bit grey levels stored in uint16 */
  DIC_F32 = 3    /* already-converted float grey levels */
} dic_dtype;

/* Solver configuration: ICGN2D1CudaMvp(rx, ry, conv, max_iter, device) and
 * FFTCC2DCuda(rx, ry, device).  FFTCC needs rx == ry (src/oc_fftcc.cpp:162-164). */
typedef struct dic_config
{
  int32_t subset_radius_x;
  int32_t subset_radius_y;
  float conv_criterion;     /* |dp| threshold; OpenCorr CLI default 0.001 */
  int32_t max_iteration;    /* stop_condition; OpenCorr CLI default 10 */
  int32_t device;           /* CUDA device ordinal */
  float input_scale;        /* raw -> float scale applied on upload (cv::Mat::convertTo);
                               0 means 1.  1/16 reads left-aligned 12-bit data. */
} dic_config;

/* One point of interest: opencorr::POI2D (src/oc_poi.h:102-136) reduced to the
 * first-order fields this path reads and writes.  56 bytes. */
typedef struct dic_poi
{
  float x, y;                        /* reference position (px) */
  float u, ux, uy, v, vx, vy;        /* deformation.p[0..2], p[6..8] */
  float u0, v0, zncc, iteration, convergence, feature;   /* result.r[0..5] */
} dic_poi;

/* Frame policy for dic_process_frame (opencorr_cli_cuda_mvp.cpp:3024-3210). */
typedef struct dic_frame_policy
{
  int32_t skip_fftcc;            /* seed from prev_results instead of running FFTCC */
  int32_t poi_fallback;          /* POI-level FFTCC repair of bad POIs */
  float zncc_threshold;          /* bad = zncc < threshold and != -3 (default 0.8) */
  float frame_fallback_ratio;    /* whole-frame FFTCC+IC-GN when bad ratio exceeds this */
  int32_t learned_seed;          /* sequences only (no reference counterpart): seed every frame
                                    with the attached proposal network, IC-GN capped at 6
                                    iterations, FFTCC + IC-GN for POIs below ZNCC 0.9; the
                                    skip/repair fields above are then unused */
  int32_t temporal_extrapolation; /* skip-FFTCC frames with two previous results: seed u, v with
                                    prev + (prev - prev_prev) where both results are finite with
                                    zncc >= zncc_threshold, the step is >= 0.05 px and each
                                    component's step <= the subset radius (:594-616) */
} dic_frame_policy;

typedef struct dic_frame_report
{
  int64_t pois;
  int64_t bad_before_repair;
  int64_t bad_after_repair;
  int64_t repaired_candidates;
  int32_t frame_fallback_used;
  int32_t fftcc_used;
  double iteration_mean;
  int64_t repaired_recovered;   /* repair candidates replaced and no longer bad (:3004-3020) */
  int64_t temporal_seed_count;  /* POIs seeded by temporal extrapolation (:3067) */
} dic_frame_report;

/* Device timings (CUDA events on the engine stream) of the most recent call of each
 * phase, in milliseconds, plus counters. */
typedef struct dic_stats
{
  double ms_prepare_ref;     /* raw -> float reference + Gradient2D4 planes */
  double ms_poi_prepare;     /* per-POI mean, norms, inverse Hessian */
  double ms_prepare_tar;     /* raw -> float target + BicubicBspline table */
  double ms_fftcc;
  double ms_icgn;
  double ms_frame;           /* whole frame of dic_sequence_frame (upload excluded) */
  double ms_proposal;        /* proposal network: input windows + forward + seeds */
  int64_t kernel_launches;   /* kernels launched by this engine since creation */
  int64_t icgn_pois;         /* POIs of the last IC-GN call */
  int64_t icgn_iterations;   /* sum of IC-GN iterations over those POIs */
} dic_stats;

typedef struct dic_engine dic_engine;

const char* dic_version(void);
/* Name, compute capability and CUDA driver / runtime versions of a device, for run
 * metadata (the manifest's engine.cuda block, opencorr_cli_cuda_mvp.cpp:2587-2610). */
int dic_device_info(int32_t device, char* name, int32_t name_capacity, int32_t* cc_major, int32_t* cc_minor,
                    int32_t* driver_version, int32_t* runtime_version);
int32_t dic_abi_version(void);

/* ICGN2D1CudaMvp::ICGN2D1CudaMvp / FFTCC2DCuda::FFTCC2DCuda (src/icgn2d1_cuda_mvp.h:98-100,
 * src/fftcc2d_cuda.h:85). */
int dic_engine_create(const dic_config* config, dic_engine** out);
/* ~ICGN2D1CudaMvp / ~FFTCC2DCuda. */
void dic_engine_destroy(dic_engine* engine);
/* Message of the last failed call on this engine ("" after a success). */
const char* dic_last_error(const dic_engine* engine);
/* The engine's CUDA stream (a cudaStream_t), for callers that order their own work. */
void* dic_stream(dic_engine* engine);

/* setRefImage / setTarImage (src/icgn2d1_cuda_mvp.h:106-107, src/fftcc2d_cuda.h:91-92):
 * copy a host image (row_stride_bytes >= width * element size) to the device.  Setting
 * the reference invalidates the prepared reference state; setting the target invalidates
 * the B-spline table.  Reference and target must have the same size.  A pageable image is
 * copied before the call returns; a page-locked one (dic_host_alloc, cudaMallocHost) is read
 * by DMA on the engine stream, so, as with the reference's images, keep it unchanged until
 * the next call that returns results (or until the engine stream is synchronised). */
int dic_set_ref(dic_engine* engine, const void* pixels, int32_t width, int32_t height,
                int64_t row_stride_bytes, int32_t dtype);
int dic_set_tar(dic_engine* engine, const void* pixels, int32_t width, int32_t height,
                int64_t row_stride_bytes, int32_t dtype);
/* The same from device memory (device-to-device copy on the engine stream). */
int dic_set_ref_device(dic_engine* engine, const void* pixels, int32_t width, int32_t height,
                       int64_t row_stride_bytes, int32_t dtype);
int dic_set_tar_device(dic_engine* engine, const void* pixels, int32_t width, int32_t height,
                       int64_t row_stride_bytes, int32_t dtype);

/* prepareRef(queue) (src/icgn2d1_cuda_mvp.h:121, src/fftcc2d_cuda.h:97): reference
 * float plane, Gradient2D4 planes and the per-POI reference data for this POI layout
 * (keyed by integer x, y), resident until the reference or the layout changes. */
int dic_prepare_ref(dic_engine* engine, const dic_poi* pois, int64_t count);
/* prepareTar (src/icgn2d1_cuda_mvp.h:122): target float plane + B-spline table. */
int dic_prepare_tar(dic_engine* engine);

/* FFTCC2DCuda::compute(queue) / compute(queue, cache_indices)
 * (src/fftcc2d_cuda.h:103-108; src/oc_fftcc.cpp:396-557).  With cache_indices, entry i
 * must name a prepared-layout slot whose integer (x, y) equals that of pois[i]. */
int dic_fftcc(dic_engine* engine, dic_poi* pois, int64_t count, const int64_t* cache_indices);
/* ICGN2D1CudaMvp::compute(queue) (src/icgn2d1_cuda_mvp.h:125; src/oc_icgn.cpp:168-397).
 * Uses the prepared layout when the queue's integer (x, y) match it, else prepares one. */
int dic_icgn(dic_engine* engine, dic_poi* pois, int64_t count);
/* FFTCC seed then IC-GN on one queue with one upload and one download
 * (opencorr_cli_cuda_mvp.cpp:3187-3196, the non-skip branch of processFrame). */
int dic_process_pair(dic_engine* engine, dic_poi* pois, int64_t count);

/* Several GPUs on one pair: the dual-device mode of ICGN2D1CudaMvp (src/icgn2d1_cuda_mvp.cu:
 * 2922-2933 halves the queue between two devices), for any number of engines.  The queue is
 * cut into contiguous bands at row boundaries (dic_split_rows) and each engine solves its band
 * with dic_process_pair from its own host thread; no data moves between devices and the
 * results land in place, in queue order, identical to a single engine's.  Every engine must
 * hold the same reference and target (dic_set_ref / dic_set_tar) and configuration.
 * band_starts (nullable) receives the count + 1 band boundaries.  Returns the first failing
 * engine's status (its dic_last_error holds the message). */
int dic_process_pair_multi(dic_engine* const* engines, int32_t count, dic_poi* pois, int64_t n, int64_t* band_starts);
/* The row-band partition used above: starts[0] = 0 <= starts[1] <= ... <= starts[parts] = n,
 * each inner cut at the first row start (a change of y) at or after k * n / parts.  Host
 * only; no device is touched. */
int dic_split_rows(const dic_poi* pois, int64_t n, int32_t parts, int64_t* starts);

/* processFrame (opencorr_cli_cuda_mvp.cpp:3024-3210): with policy->skip_fftcc and
 * prev_results (count entries) the queue is seeded from the previous frame and solved by
 * IC-GN alone, then repaired per POI or per frame as the policy says; otherwise FFTCC +
 * IC-GN.  pois holds the POI template on entry and the results on return. */
int dic_process_frame(dic_engine* engine, dic_poi* pois, int64_t count, const dic_poi* prev_results,
                      const dic_frame_policy* policy, dic_frame_report* report);
/* processFrame with both histories (:3024-3070): prev_prev_results (count records, the
 * frame before prev_results) feeds the policy's temporal extrapolation; NULL: none. */
int dic_process_frame_history(dic_engine* engine, dic_poi* pois, int64_t count, const dic_poi* prev_results,
                              const dic_poi* prev_prev_results, const dic_frame_policy* policy,
                              dic_frame_report* report);

/* Fixed-reference sequence (runMultiFrame, opencorr_cli_cuda_mvp.cpp:3834-4516).
 * dic_sequence_begin takes the POI template (buildPoiQueue order) and the policy, builds the
 * resident per-POI reference data for it and resets the history; the reference image must
 * be set.  Each dic_sequence_frame uploads one target (host memory, or device memory when
 * pixels_on_device) and solves it: the first frame, and every frame when
 * policy->skip_fftcc is 0, by FFTCC + IC-GN from the template; later frames by IC-GN seeded
 * from the previous frame's results, with POI-level repair and the whole-frame fallback.
 * In a sequence policy->frame_fallback_ratio is the margin added to the first frame's bad
 * ratio (kSkipFftccBadRatioMargin = 0.03 in the reference), as the CLI does
 * (:4275-4279).  The previous results stay on the device; the steady-state frame is one
 * captured CUDA graph (dic_set_graphs(engine, 0) launches kernels one by one instead).
 * results (nullable, count records) receives the frame's results. */
int dic_sequence_begin(dic_engine* engine, const dic_poi* pois, int64_t count, const dic_frame_policy* policy);
int dic_sequence_frame(dic_engine* engine, const void* pixels, int32_t width, int32_t height,
                       int64_t row_stride_bytes, int32_t dtype, int32_t pixels_on_device, dic_poi* results,
                       dic_frame_report* report);
/* No reference counterpart: the results and report of a frame already enqueued, read
 * after the fact: frames_back 0 = the most recent dic_sequence_frame, 1 = the one before
 * (each frame keeps a copy of its results for this until two more frames are enqueued).
 * dic_sequence_frame with results and report NULL only enqueues the frame and returns, so a
 * loop can keep the GPU busy: while frame k runs, stage and enqueue frame k + 1, then fetch
 * frame k (frames_back 1), which reads it on a download stream while frame k + 1 runs.  The
 * fetch waits only for the frame it reads.  DIC_ERR_ARGUMENT for frames_back other than 0
 * or 1; DIC_ERR_STATE for a frame that no successful dic_sequence_frame of the current
 * sequence enqueued. */
int dic_sequence_fetch(dic_engine* engine, int32_t frames_back, dic_poi* results, dic_frame_report* report);
int dic_set_graphs(dic_engine* engine, int32_t enabled);

/* Frame upload on a side stream (no reference counterpart; the reference decodes the next
 * frame on a thread and uploads it inside the next compute call).  dic_stage_frame copies a
 * host frame into one of two pinned buffers and starts its host-to-device copy on the
 * engine's upload stream, then returns; the copy overlaps whatever the engine stream is
 * running (typically the current frame's solve).  A page-locked frame (cudaMallocHost,
 * cudaHostRegister, pinned torch tensors) skips the host copy: it is uploaded directly and
 * the call returns when that copy is done, so the caller may reuse the buffer at once.  dic_sequence_frame with
 * pixels_on_device = DIC_PIXELS_STAGED (pixels NULL) consumes the oldest staged frame: the
 * engine stream waits for its copy, nothing else does.  At most two frames are staged at a
 * time. */
#define DIC_PIXELS_STAGED 2
int dic_stage_frame(dic_engine* engine, const void* pixels, int32_t width, int32_t height, int64_t row_stride_bytes,
                    int32_t dtype);
/* Page-locked host memory for frames and result buffers (no reference counterpart): frames
 * staged from it skip the staging copy, and dic_sequence_fetch / dic_sequence_frame results
 * read into it are direct DMA.  dic_host_alloc returns DIC_ERR_MEMORY when the driver refuses;
 * dic_host_free(NULL) is a no-op. */
int dic_host_alloc(size_t bytes, void** ptr);
void dic_host_free(void* ptr);

/* Uneven batch: several image pairs of different sizes, each with its own subset radius
 * (square, 1..32) and POI queue, solved together (FFTCC seed + IC-GN).  No single call of
 * the reference does this; the CLI loops over pairs.  The pairs' prep and FFTCC chains run
 * side by side on four streams of the engine; all POIs of all pairs then go through one
 * persistent IC-GN launch per subset walk (column walk up to 32 columns, pair walk up to 64
 * -- under pixel sampling one per subset radius, whose windows set the residency -- and the
 * flat walk beyond) whose warps take POIs from a shared atomic counter, so pairs with many
 * POIs or slow-converging POIs do not leave SMs idle.  Results are written back into each
 * job's queue, bit-identical to the job solved alone.  The engine's conv_criterion and
 * max_iteration apply to all jobs. */
typedef struct dic_job
{
  const void* ref;
  const void* tar;
  int32_t width, height;
  int64_t row_stride_bytes;
  int32_t dtype;
  int32_t subset_radius;
  dic_poi* pois;
  int64_t count;
} dic_job;

typedef struct dic_batch_report
{
  int64_t pois;
  int64_t valid;       /* POIs with zncc >= 0 (-1 when the queues are in device memory) */
  int32_t jobs;
  int32_t graph;       /* 1 when the call replayed a captured CUDA graph */
} dic_batch_report;

int dic_batch_process(dic_engine* engine, const dic_job* jobs, int32_t njobs, int32_t pixels_on_device,
                      dic_batch_report* report);

/* Launch-shape autotuner (no reference counterpart).  IC-GN walks a subset in one of three
 * ways: the column walk (up to 32 columns, one warp per POI, lane = column), the pair walk
 * (33 to 64 columns: two interleaved column classes, one or two warps per POI) and the
 * flat walk (wider, one warp per POI).  When enabled, the first IC-GN launch of each kind
 * (per-queue / persistent batch, per walk) with at least 2048 POIs times the candidate
 * shapes -- 2, 4 or 8 warps per CTA; for the pair walk 1 or 2 warps per POI; for a single
 * queue a grid of one CTA per POI group or a persistent work-queue launch at full
 * occupancy; for a batch full or 3/4 occupancy in CTAs per SM -- on a copy of its seeded
 * queue and keeps the fastest for the engine's lifetime.  Results do not depend on the
 * shape.  Enabling (again) clears what was learnt.  Tuning never runs inside a graph
 * capture. */
typedef struct dic_launch_shape
{
  int32_t warps_per_cta;
  int32_t ctas_per_sm;   /* > 0: persistent launch with this many resident CTAs per SM drawing POIs
                            from an atomic counter; 0: one CTA per warps_per_cta POIs */
  int32_t tuned;
  float ms;              /* best candidate's time, when tuned */
  int32_t tile;          /* column-walk IC-GN only: 0 gathers texels from the coefficient table;
                            1 (4 warps, 48x36 texels, 2 CTAs/SM) or 2 (8 warps, 64x40, 1 CTA/SM)
                            stage the block a chunk of consecutive POIs warps onto in shared memory
                            by TMA; warps_per_cta and ctas_per_sm then follow the tile kind */
  int32_t warps_per_poi; /* pair walks (2 and 4): 1 (one warp walks both column classes) or 2
                            (one warp per class, class sums exchanged through shared memory); 1
                            elsewhere (0 is read as 1) */
} dic_launch_shape;

typedef struct dic_tuning
{
  dic_launch_shape icgn[5];    /* [0] flat walk, [1] column walk, [2] pair walk, [3] column walk with
                                  pixel sampling (k_icgn_px, see dic_set_sampling), [4] pair walk
                                  with pixel sampling (k_icgn_pair_px) */
  dic_launch_shape batch[5];   /* [3], [4]: the column and pair walks under pixel sampling
                                  (k_icgn_batch_px, k_icgn_batch_pair_px) */
} dic_tuning;

int dic_set_autotune(dic_engine* engine, int32_t enabled);
int dic_get_tuning(dic_engine* engine, dic_tuning* out);
/* No reference counterpart: fixes the single-queue IC-GN launch shape of one subset walk
 * (walk 1: column walk, subsets at most 32 wide; 2: pair walk, 33 to 64; 0: flat walk,
 * wider; 3 and 4: the column and pair walks under pixel sampling), e.g. to compare the
 * gather and the TMA-staged tile forms, or one and two warps per POI.  warps_per_cta in
 * {2, 4, 8}, ctas_per_sm >= 0, tile in {0, 1, 2} (tile > 0 only with walks 1, 3 and 4; with
 * walks 3 and 4, tile 1 stages each POI's pixel window in shared memory by TMA, 2 by warp
 * copies, and 0 reads the plane in global memory, ctas_per_sm 0 = full occupancy),
 * warps_per_poi in {0, 1, 2} (2 only with walks 2 and 4); tuned and ms are ignored.
 * Results do not depend on the shape.  An enabled autotuner may replace it on the next large
 * queue. */
int dic_set_launch_shape(dic_engine* engine, int32_t walk, const dic_launch_shape* shape);

/* No reference counterpart: how IC-GN reads the target's bicubic interpolant.
 * DIC_SAMPLE_TABLE evaluates BicubicBspline::compute's polynomial from the per-texel
 * coefficient table (src/oc_cubic_bspline.cpp:134-181; 64 B per texel, gathered from L2 per
 * sample).  DIC_SAMPLE_PIXELS (the default) evaluates the same polynomial regrouped by pixel,
 * sum_n wy[n] sum_m wx[m] I(iy-1+n, ix-1+m) with the B-spline weights of the BC matrix, from
 * the 4 x 4 pixels around the texel, each POI's window staged once in shared memory
 * (k_icgn_px, k_icgn_pair_px) and no coefficient table built.  It applies to the column and
 * pair walks (subsets at most 64 columns wide); wider subsets keep the table.  The two differ by float rounding
 * only (both within the parity gate against the CPU; flags agree); samples on the pixel
 * lattice give the pixel itself either way.  Takes effect at the next solve. */
#define DIC_SAMPLE_TABLE 0
#define DIC_SAMPLE_PIXELS 1
int dic_set_sampling(dic_engine* engine, int32_t mode);

/* Device-resident variant: pois points to device memory (count records) and the call only
 * enqueues work on the engine stream (dic_get_stats or a stream sync waits for it).  flags
 * selects the phases, run in this order: DIC_RUN_PREPARE (take this queue's integer (x, y)
 * as the prepared layout; implied when no layout of this size is resident or the reference
 * changed), DIC_RUN_FFTCC, DIC_RUN_ICGN. */
#define DIC_RUN_FFTCC 1
#define DIC_RUN_ICGN 2
#define DIC_RUN_PREPARE 4
#define DIC_RUN_LEARNED 8   /* proposal-network seeds instead of FFTCC (see below) */
int dic_run_device(dic_engine* engine, dic_poi* device_pois, int64_t count, int32_t flags);

/* Copy one resident device plane to host memory (bytes must equal the plane size):
 * DIC_PLANE_REF       W*H float reference grey levels
 * DIC_PLANE_REF_PACK  W*H float4 {ref, gx, gy, 0} (Gradient2D4 planes, src/oc_gradient.cpp)
 * DIC_PLANE_TAR       W*H float target grey levels
 * DIC_PLANE_TAR_COEF  BicubicBspline table (src/oc_cubic_bspline.cpp:84-132) as 2 planes of
 *                     W*H texels x 8 floats; plane j holds coefficient rows 2j and 2j+1,
 *                     c[2j][0..3] then c[2j+1][0..3], of every texel
 * Prepares the plane first if its image changed.  For inspection and tests. */
#define DIC_PLANE_REF 1
#define DIC_PLANE_REF_PACK 2
#define DIC_PLANE_TAR 3
#define DIC_PLANE_TAR_COEF 4
int dic_read_plane(dic_engine* engine, int32_t plane, void* host_dst, int64_t bytes);

/* Proposal network (no counterpart in the reference): a CNN mapping the 31x31 reference and
 * target windows at a POI to (u, v, ux, uy, vx, vy), so IC-GN starts close.  Trained on the
 * GPU by its own BF16 tensor-core forward/backward kernels with FP32 accumulation.
 * Parameters are FP32, dic_cnn_param_count() of them, in the layout of
 * fasticgn_gb300/csrc/dic_cnn.cuh.  Device pointers: x0 is BF16 [n][31][31][2] (NHWC),
 * targets FP32 [n][6] (u, v, ux, uy, vx, vy), outputs FP32 [n][8] (u, v, 100ux, 100uy,
 * 100vx, 100vy, 0, 0), gradients FP32 [param_count]. */
typedef struct dic_cnn dic_cnn;
int64_t dic_cnn_param_count(void);
int dic_cnn_create(int32_t device, dic_cnn** out);
void dic_cnn_destroy(dic_cnn* net);
const char* dic_cnn_last_error(const dic_cnn* net);
int dic_cnn_set_params(dic_cnn* net, const float* host_params, int64_t count);
int dic_cnn_get_params(dic_cnn* net, float* host_params, int64_t count);
int dic_cnn_input(dic_cnn* net, const float* device_ref, const float* device_tar, int32_t width, int32_t height,
                  const dic_poi* device_pois, int64_t count, void* device_x0);
int dic_cnn_forward(dic_cnn* net, const void* device_x0, int64_t count, float* device_out);
/* Fused inference (the whole network per POI tile in shared memory): writes the proposal's
 * (u, ux, uy, v, vx, vy) into device_pois and clears their result fields. */
int dic_cnn_seed(dic_cnn* net, const float* device_ref, const float* device_tar, int32_t width, int32_t height,
                 dic_poi* device_pois, int64_t count);
int dic_cnn_gradient(dic_cnn* net, const void* device_x0, const float* device_target, int64_t count,
                     float* device_grad, float* loss);
int dic_cnn_train_step(dic_cnn* net, const void* device_x0, const float* device_target, int64_t count,
                       float learning_rate, float* loss);

/* Attach (or with NULL detach) a proposal network to an engine on the same device. */
int dic_set_proposal(dic_engine* engine, dic_cnn* net);
/* Learned-seed pair solve: proposal seeds, IC-GN capped at 6 iterations, and FFTCC + IC-GN
 * (the full budget) for every POI that does not converge there or ends with ZNCC < 0.9.
 * report->repaired_candidates counts those fallback POIs. */
int dic_process_pair_learned(dic_engine* engine, dic_poi* pois, int64_t count, dic_frame_report* report);

int dic_get_stats(const dic_engine* engine, dic_stats* out);
/* Turns per-phase CUDA-event timing on (1) or off (0).  On by default. */
int dic_set_timing(dic_engine* engine, int32_t enabled);

/* No reference counterpart: measurement support.  Enqueues on `stream` (a cudaStream_t) one
 * kernel on `device` that reads `bytes` (rounded down to 32) of device memory `repeats` times
 * with the 256-bit non-coherent loads the IC-GN gathers use, four in flight per thread, 8
 * CTAs of 256 threads per SM; device_sink (one float) is written only in a case that never
 * occurs for finite data.  Timed by the caller with events on `stream`: for a buffer that fits
 * in L2 (tens of MB, after one warm-up launch) bytes x repeats / time is the L2-to-SM read
 * bandwidth that bounds the gathers.  device_buf must be 32-byte aligned. */
int dic_read_probe(int32_t device, const void* device_buf, int64_t bytes, int32_t repeats, float* device_sink,
                   void* stream);
/* No reference counterpart: measurement support.  Enqueues on `stream` one kernel on `device`
 * that runs eight independent FP32 FMA chains per thread for `iterations` rounds (8 CTAs of
 * 256 threads per SM); *flop_out receives the FLOP count of the launch (2 per FMA).  Timed by
 * the caller with events on `stream`, it gives the FP32 peak the FFTCC kernels are held to. */
int dic_fma_probe(int32_t device, int32_t iterations, float* device_sink, void* stream, int64_t* flop_out);
/* No reference counterpart: measurement support.  Enqueues on `stream` one kernel on `device`
 * whose warps read 32 consecutive floats of shared memory per load (one conflict-free
 * wavefront), 16 loads per pass, `repeats` passes, 8 CTAs of 256 threads per SM; *bytes_out
 * receives the bytes the launch loads.  Timed by the caller with events on `stream`, it gives
 * the shared-memory load bandwidth the pixel-sampled IC-GN (k_icgn_px) is held to. */
int dic_smem_probe(int32_t device, int32_t repeats, float* device_sink, void* stream, int64_t* bytes_out);

/* Allocation-free pair solve (FFTCC seed + IC-GN).  No counterpart in the reference: its
 * solvers allocate their device buffers themselves.
 *
 * For callers that cannot call cudaMalloc -- a host application that reserves device
 * memory up front and hands its plug-ins only buffers it owns, or an acquisition loop in
 * which an allocation's implicit device synchronisation would stall the camera stream.
 * The caller passes the reference and target images (device memory, dense rows of width
 * pixels of dtype) and the POI queue (device memory, updated in place, same result fields
 * as dic_process_pair); all intermediate planes and per-POI records live in one fixed
 * 32 MiB device array inside this library, held by every GPU that loads it until the
 * process exits.  Limit: 88 bytes per pixel plus 224 bytes per POI (each plane rounded up
 * to 256 bytes) must fit in 32 MiB, e.g. 512x512 with up to 46 811 POIs; larger calls are
 * rejected with DIC_ERR_ARGUMENT and a message in error_text (nullable, error_capacity
 * bytes).  The subset radius must be square, 1..32.
 *
 * The call enqueues its kernels on `stream` (a cudaStream_t, 0 = legacy default stream)
 * and returns without waiting; it makes no cudaMalloc, cudaFree or other allocating call.
 * The first call on a device (the current device) also performs one-time set-up -- it
 * looks up the scratch array's device address and loads the constant tables -- so that
 * first call should come before any stream capture.  Every call shares the one scratch
 * array, which keeps the last call's contents; each call writes every scratch byte it
 * later reads, so nothing needs clearing, but calls that overlap on the GPU (on different
 * streams, or from different threads) race on the scratch and must be serialised by the
 * caller. */
int dic_process_pair_noalloc(const dic_config* config, const void* device_ref, const void* device_tar,
                             int32_t width, int32_t height, int32_t dtype, dic_poi* device_pois,
                             int64_t count, void* stream, char* error_text, int64_t error_capacity);

#ifdef __cplusplus
}
#endif

#endif /* GB300_DIC_H */
