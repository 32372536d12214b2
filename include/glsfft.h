/*
 * glsfft.h -- C ABI of the GB300 FFT / phaseCorrelate path of glsCV.
 *
 * Plain C: opaque handles, int status codes (0 = success), device pointers,
 * and `void *stream` (a cudaStream_t; NULL = the legacy default stream).
 * Every call validates its arguments on the host before any launch and
 * returns a status instead of throwing; the C++ layer in <gls/glsCV.h>
 * turns a non-zero status into a gls::Exception, as the reference's
 * GLS_Assert/CV_Assert throws cv::Exception (glsCV/glsMacro.h:40).
 *
 * Image layout: row-major, continuous, like a continuous cv::Mat.
 * CV_32FC2 = interleaved float (re, im), 8 bytes per pixel, 8-byte aligned;
 * CV_32FC1 = float, 4-byte aligned.  rows and cols are powers of two in
 * [1, GLSFFT_MAX_LEN]; square, rectangular and 1-D (1 x N, N x 1) shapes are
 * all accepted (the reference asserts on non-square 2-D, glsFft.cpp:503-517).
 *
 * Threading: a context may be used from one host thread at a time; calls on
 * one context share its workspace, so issue them on one stream (or
 * synchronise between streams).  Separate contexts are independent.
 */
#ifndef GLSFFT_H_
#define GLSFFT_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GLSFFT_API __attribute__((visibility("default")))
#else
#define GLSFFT_API
#endif

#define GLSFFT_MAX_LEN 4096

/* Flag bits: the reference's values (glsCV/glsFft.h:43-47, OpenCV DFT_*). */
#define GLSFFT_INVERSE 1 /* GLS_FFT_INVERSE = DFT_INVERSE */
#define GLSFFT_SCALE 2   /* GLS_FFT_SCALE = DFT_SCALE: x 1/N per dimension */
#define GLSFFT_SHIFT 64  /* GLS_FFT_SHIFT: quadrant swap of the output */

enum glsfft_status {
    GLSFFT_SUCCESS = 0,
    GLSFFT_ERROR_INVALID_VALUE = 1, /* NULL pointer or handle, unknown flag bit, bad box */
    GLSFFT_ERROR_NOT_POW2 = 2,      /* GLS_Assert(IsPow2(N)), glsFft.cpp:681 */
    GLSFFT_ERROR_SIZE = 3,          /* a dimension outside [1, GLSFFT_MAX_LEN] */
    GLSFFT_ERROR_MISALIGNED = 4,    /* pointer not aligned to its element size */
    GLSFFT_ERROR_CUDA = 5,          /* a CUDA runtime call or launch failed */
    GLSFFT_ERROR_OUT_OF_MEMORY = 6, /* device workspace allocation failed */
    GLSFFT_ERROR_BUDGET = 7,        /* workspace would exceed the context's HBM budget */
    GLSFFT_ERROR_TIMEOUT = 8,       /* a bounded device-side wait expired */
    GLSFFT_ERROR_SHAPE = 9,         /* inputs of different shapes */
    GLSFFT_ERROR_NOALLOC_LIMIT = 10, /* rows*cols above GLSFFT_NOALLOC_MAX_PIXELS */
    GLSFFT_ERROR_IO = 11             /* the plan cache file could not be written */
};

typedef struct glsfft_context_s *glsfft_context;

/* Human-readable text for a status code (never NULL). */
GLSFFT_API const char *glsfft_status_string(int status);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
GLSFFT_API int glsfft_version(void);

/*
 * Create a context on CUDA device `device`: uploads the FP32 twiddle tables
 * (generated in FP64, once) for every length up to GLSFFT_MAX_LEN.
 * Replaces glsCvInit() (glsCV/glsCV.cpp:89-165): no GL context, no window.
 */
GLSFFT_API int glsfft_context_create(glsfft_context *ctx, int device);

/* Free the context and its workspace.  Replaces glsCvTerminate(). */
GLSFFT_API int glsfft_context_destroy(glsfft_context ctx);

/* Cap the workspace the context may hold on the device (bytes; 0 = none). */
GLSFFT_API int glsfft_context_set_budget(glsfft_context ctx, size_t bytes);

/* Bytes of device workspace the context currently holds. */
GLSFFT_API int glsfft_context_workspace(glsfft_context ctx, size_t *bytes);

/* Sticky status of the context's device-side bounded waits outside batch
 * plans and servers (the streamed passes' tile waits): GLSFFT_SUCCESS, or
 * GLSFFT_ERROR_TIMEOUT once a wait expired (that pass's output is then
 * incomplete).  Synchronises with the device; `clear` resets the word.  No
 * reference counterpart. */
GLSFFT_API int glsfft_device_status(glsfft_context ctx, int clear);

/* Host-side fault injection for tests: with wait_limit_ns > 0, every
 * streamed pass launched on this context leaves each block's first tile copy
 * unissued and bounds the wait for it by wait_limit_ns, so the wait runs
 * out: the pass records GLSFFT_ERROR_TIMEOUT (glsfft_device_status) and
 * returns with no copy in flight; the context stays usable.  0 turns the
 * injection off. */
GLSFFT_API int glsfft_context_inject_stall(glsfft_context ctx, long long wait_limit_ns);

/*
 * 2-D complex FFT of a CV_32FC2 rows x cols device image:
 * gls::fft(src, dst, flag), glsCV/glsFft.h:55 / glsFft.cpp:675-708.
 * Rows pass then columns pass, one kernel each.  src == dst is allowed
 * (in-place, as glsPhaseCorrelate.cpp:199 uses it).  Asynchronous on
 * `stream`; uses no workspace.
 */
GLSFFT_API int glsfft_fft2d_c2c(glsfft_context ctx, const void *src, void *dst, int rows,
                                int cols, int flags, void *stream);

/*
 * Same for a CV_32FC1 src promoted to complex with imag = 0
 * (gls::fft's merge step, glsFft.cpp:684-689); dst is CV_32FC2.
 */
GLSFFT_API int glsfft_fft2d_r2c_promote(glsfft_context ctx, const float *src, void *dst,
                                        int rows, int cols, int flags, void *stream);

/*
 * Batched gls::fft: `count` (1..65535) CV_32FC2 rows x cols images stored back
 * to back (image i at byte offset i*rows*cols*8 of src and dst), each
 * transformed as glsfft_fft2d_c2c does, with one launch per pass for the
 * whole batch.  No reference counterpart (glsCV transforms one texture per
 * call); src == dst allowed.
 */
GLSFFT_API int glsfft_fft2d_batched(glsfft_context ctx, const void *src, void *dst, int count,
                                    int rows, int cols, int flags, void *stream);

/*
 * One pass of gls::fft on its own, over `count` back-to-back images: a 1-D
 * FFT of every row (length cols) -- the rows pass, glsFft.cpp:561-605 -- or
 * of every column (length rows) -- the columns pass, glsFft.cpp:607-652.
 * INVERSE conjugates input and output of each line, SCALE multiplies by
 * 1/length, SHIFT swaps the halves of each line.  fft2d(flags) equals
 * fft_rows then fft_cols with the same flags.  One kernel launch each;
 * src == dst allowed.
 */
GLSFFT_API int glsfft_fft_rows(glsfft_context ctx, const void *src, void *dst, int count,
                               int rows, int cols, int flags, void *stream);
GLSFFT_API int glsfft_fft_cols(glsfft_context ctx, const void *src, void *dst, int count,
                               int rows, int cols, int flags, void *stream);

/*
 * Reference-arithmetic mode (verification; no reference counterpart as an
 * entry point): gls::fft over `count` back-to-back images computed with the
 * reference's own FP32 line arithmetic -- algo 0: the radix-2 DIT type1
 * Stockham of UnitTest_glsCV/fft_stockhum.cpp:436-538, algo 1: the radix-4
 * DIT Stockham of :866-1031 (the GLSL shader's algorithm, glsFft.cpp:
 * 203-343) -- with the reference's twiddle table ((float) angle, cosf/sinf)
 * and every product and sum rounded separately, so the result is
 * bit-identical to the reference's CPU routine with gls::fft's flag
 * semantics.  Several times slower than glsfft_fft2d_c2c; uses the context
 * workspace.
 */
GLSFFT_API int glsfft_fft2d_reference(glsfft_context ctx, const void *src, void *dst, int count,
                                      int rows, int cols, int flags, int algo, void *stream);
/* gls::phaseCorrelate (glsPhaseCorrelate.cpp:142-236) on the reference-
 * arithmetic FFT: window product, forward FFTs, phase-only spectrum without
 * epsilon (0/0 -> NaN, as the reference), unscaled inverse with the quadrant
 * shift, real part, first-max location, FP64 centroid; synchronous.  Every
 * step rounds as the reference's CPU code, so dx, dy and response are
 * bit-identical to it on the same inputs.  `algo` is 0 or 1 as above,
 * optionally ORed with GLSFFT_REFERENCE_ZERO_GUARD: a bin whose
 * |F1 conj(F2)| is exactly 0 then gives 0 instead of 0/0 = NaN (the default
 * path's behaviour; smooth inputs such as a blurred field hit such bins, and
 * one NaN poisons the reference's whole surface). */
#define GLSFFT_REFERENCE_ZERO_GUARD 16
GLSFFT_API int glsfft_phase_correlate_reference(glsfft_context ctx, const float *src1,
                                                const float *src2, const float *window, int rows,
                                                int cols, int box, int algo, double *dx,
                                                double *dy, double *response, void *stream);

/*
 * Precision form of the batched 2-D FFT (no reference counterpart): each
 * 1024- or 4096-point line is a four-step FFT (32 x 32 or 64 x 64) whose two
 * DFT stages run as complex matrix products on the tensor cores with FP16
 * hi/lo split operands (hi*hi + hi*lo + lo*hi, FP32 accumulate, power-of-two
 * block scaling), giving FP32-level error.  rows, cols in {1024, 4096};
 * `count` back-to-back images like glsfft_fft2d_batched; same flags.
 */
GLSFFT_API int glsfft_fft2d_tc(glsfft_context ctx, const void *src, void *dst, int count,
                               int rows, int cols, int flags, void *stream);

/*
 * Pass schedules of the plain path (no reference counterpart: glsCV runs
 * one fixed radix-4 schedule, glsFft.cpp:494-671).  The complex row pass and
 * column pass each have schedules 0..6 per line length: 0 the default;
 * 1 half the elements per thread with the radix bound lowered to match;
 * 2 twice the elements per thread; 3 / 4 half / twice the lines or columns
 * per block; 5 = 1 and 3 together; 6 (column pass only) streamed: one
 * persistent block per SM that copies the next 128 KB tile in with the TMA
 * while it transforms the current one (lengths 2048 and 4096; bit-identical
 * to schedule 0; calls whose buffers are not 16-byte aligned run schedule
 * 0).  All compute the
 * same transform (rounding differs with the radix order, within the FP32
 * error bound).  Schedules 1..5 exist for lengths 64..4096 where the block
 * fits the SM.
 */
#define GLSFFT_PASS_SCHEDULES 7
#define GLSFFT_SCHEDULE_STREAMED 6
/* 1 when `schedule` exists for a row pass (along_cols = 0) or column pass
 * (along_cols = 1) of line length `length`, else 0. */
GLSFFT_API int glsfft_schedule_available(int length, int schedule, int along_cols);

/* Pass schedules that glsfft_fft2d_c2c, glsfft_fft2d_batched, the single
 * pass entry points and batch plans' own-launch images use for complex
 * rows x cols images on this context.  Until set or tuned, a size runs its
 * built-in default, measured on GB300: row schedule 2 for 2048- and
 * 4096-point rows, the streamed column pass for 4096-point columns,
 * schedule 0 otherwise. */
GLSFFT_API int glsfft_set_fft_schedule(glsfft_context ctx, int rows, int cols, int row_schedule,
                                       int col_schedule);
GLSFFT_API int glsfft_get_fft_schedule(glsfft_context ctx, int rows, int cols,
                                       int *row_schedule, int *col_schedule);

/*
 * Autotuner of the plain path for one image size: times every available
 * schedule of the row pass and of the column pass over `count` images of
 * rows x cols (median of 7 launches after 2, CUDA events on `stream`) on
 * scratch buffers it allocates and frees, and sets the fastest of each
 * (glsfft_set_fft_schedule) unless the size's default schedule is within
 * 1% of it.  With
 * cache_path set, the choice is looked up in / appended to that plan cache
 * file (one JSON object per line, keyed by device name, SM count, compute
 * capability, driver, runtime and library versions, rows, cols, count); a
 * hit is applied without timing.  result[3] = {row schedule, column
 * schedule, 1 if from the cache}; ms[2] = {chosen, default}: row plus
 * column pass time of one launch each.  Either may be NULL.
 */
GLSFFT_API int glsfft_autotune_fft2d(glsfft_context ctx, int rows, int cols, int count,
                                     const char *cache_path, void *stream, int *result,
                                     double *ms);

/*
 * gls::fft over images in host memory -- the GlsMat upload, transform,
 * download sequence (glsCV/glsMat.cpp:374-417, :493-551 and gls::fft) for
 * `count` rows x cols CV_32FC2 images stored back to back at host_src, each
 * run through n_transforms (1 or 2) transforms with flags[k] (like a batch
 * plan), results to host_dst (may equal host_src).  The images move in
 * chunks of `chunk` images (0: automatic, about 32 MiB and at least four
 * chunks): host -> device, a batch plan, device -> host, on three streams
 * over a ring of three device slots, so the copies in both directions
 * overlap the transforms.  Asynchronous: it runs after the work already
 * queued on `stream`, and `stream` waits for the last result; synchronise it
 * before reading host_dst.  The copies overlap only with page-locked host
 * memory (cudaHostAlloc / cudaHostRegister).  The streams, the 3 x chunk
 * device images and the plans stay in the context (counted against its
 * budget) until the shape, chunk or flags change.  No reference counterpart
 * as one call (glsCV uploads and downloads synchronously).
 */
GLSFFT_API int glsfft_fft2d_host(glsfft_context ctx, const void *host_src, void *host_dst,
                                 int count, int rows, int cols, int n_transforms,
                                 const int *flags, int chunk, void *stream);

/*
 * Spectrum operations on rows x cols device images (any size; the CV_32FC2
 * results may be written in place, the CV_32FC1 ones must not overlap their
 * input), element formulas of the reference shaders with every product, sum
 * and quotient rounded separately:
 *   glsfft_mul_spectrums            gls::mulSpectrums(src0, src1, dst, conj)
 *                                   (glsCV/glsBasicOperation.cpp:320-326): a*b or
 *                                   a*conj(b), CV_32FC2
 *   glsfft_mul_spectrums_phase_only gls::mulSpectrumsPhaseOnly (:329-335):
 *                                   t = a*conj(b), t/|t| (0/0 is NaN, as there)
 *   glsfft_mag_spectrums            gls::magSpectrums (:337-343): |a| as CV_32FC1
 *   glsfft_log_mag_spectrums        gls::logMagSpectrums(src, dst, offset)
 *                                   (:345-351): log(| |a| + offset |) as CV_32FC1
 */
GLSFFT_API int glsfft_mul_spectrums(glsfft_context ctx, const void *src0, const void *src1,
                                    void *dst, int rows, int cols, int conj, void *stream);
GLSFFT_API int glsfft_mul_spectrums_phase_only(glsfft_context ctx, const void *src0,
                                               const void *src1, void *dst, int rows, int cols,
                                               void *stream);
GLSFFT_API int glsfft_mag_spectrums(glsfft_context ctx, const void *src, float *dst, int rows,
                                    int cols, void *stream);
GLSFFT_API int glsfft_log_mag_spectrums(glsfft_context ctx, const void *src, float *dst,
                                        int rows, int cols, float offset, void *stream);

/*
 * gls::minMaxLoc(src, &minVal, &maxVal, &minLoc, &maxLoc) on a CV_32FC1 device
 * image (glsCV/glsMinMaxLoc.cpp:149-200): the first occurrence in row-major
 * order of the smallest and largest values; as in the reference shader only
 * values below (above) its FLT_MAX literal 3.402823e+38 take part and NaN
 * never does, and with none the literal is returned at (0, 0).  Locations are
 * {x, y}; any output may be NULL.  Synchronises `stream`.
 * glsfft_min_max_loc_async leaves the two 64-bit keys in d_keys instead
 * (min, max: order-preserving value bits << 32 | 0xFFFFFFFF - (y*cols + x),
 * 0 = none).
 */
GLSFFT_API int glsfft_min_max_loc(glsfft_context ctx, const float *src, int rows, int cols,
                                  double *min_val, double *max_val, int *min_loc, int *max_loc,
                                  void *stream);
GLSFFT_API int glsfft_min_max_loc_async(glsfft_context ctx, const float *src, int rows,
                                        int cols, unsigned long long *d_keys, void *stream);

/*
 * gls::normalize(src, dst, alpha, beta, NORM_MINMAX) on a CV_32FC1 device
 * image (glsCV/glsNormalize.cpp:52-68): scl = (float)(beta - alpha) /
 * (float)(max - min), dst = (float)(alpha - scl*min) + scl*src; the min / max
 * stay on the device (asynchronous).
 */
GLSFFT_API int glsfft_normalize_minmax(glsfft_context ctx, const float *src, float *dst,
                                       int rows, int cols, double alpha, double beta,
                                       void *stream);

/*
 * glsCam's FFT view as one pipeline on device buffers (glsCam/glsCam.cpp:196-203):
 * window * frame (CV_32FC1; window may be NULL), gls::fft with GLS_FFT_SHIFT,
 * logMagSpectrums(offset), normalize(0, 1, NORM_MINMAX) -> dst (CV_32FC1).
 * The log-magnitude and its min / max are fused into the column FFT; the
 * camera, colour conversion and drawing are left out.  Powers of two;
 * asynchronous.
 */
GLSFFT_API int glsfft_fft_display(glsfft_context ctx, const float *frame, const float *window,
                                  float *dst, int rows, int cols, float offset, void *stream);

typedef struct glsfft_batch_s *glsfft_batch;

/*
 * Batch plan: `count` CV_32FC2 device images of individual sizes (srcs[i] ->
 * dsts[i], rows[i] x cols[i]; src may equal dst), each run through
 * n_transforms (1 or 2) successive gls::fft transforms with flags[k] (e.g.
 * {0, GLSFFT_INVERSE | GLSFFT_SCALE}: forward, then back).  Images with
 * 16 <= rows <= 1024 and 16 <= cols <= 4096 are processed by one persistent
 * launch that pulls (image, pass, tile) items from a work list, each pass of
 * an image waiting (bounded) for that image's previous pass; other shapes get
 * their own pass launches.  Everything is captured once into a CUDA graph.
 * No reference counterpart (glsCV transforms one texture per call).  The
 * plan keeps the pointers: the buffers must outlive it.
 */
GLSFFT_API int glsfft_batch_create(glsfft_context ctx, int count, const void *const *srcs,
                                   void *const *dsts, const int *rows, const int *cols,
                                   int n_transforms, const int *flags, glsfft_batch *plan);

/* Launch the plan's graph on `stream` (asynchronous). */
GLSFFT_API int glsfft_batch_execute(glsfft_batch plan, void *stream);

/*
 * Persistent-kernel schedule of a plan (re-captures its graph):
 * 0 = every thread loads and stores its own operands (2 blocks/SM);
 * 1 = warp-specialised: a producer warp stages tiles with TMA into a 3-stage
 *     shared-memory ring for 8 compute warps and writes the results back
 *     with TMA stores (1 block/SM);
 * 2 = the same at 2 blocks/SM;
 * 3 = the same at 3 blocks/SM with a 2-stage ring (the default).
 */
#define GLSFFT_BATCH_PLAIN 0
#define GLSFFT_BATCH_TMA_WS1 1
#define GLSFFT_BATCH_TMA_WS2 2
#define GLSFFT_BATCH_TMA_WS3 3
GLSFFT_API int glsfft_batch_set_variant(glsfft_batch plan, int variant);

/*
 * Work-queue schedule of a plan (re-captures its graph): items claimed per
 * queue atomic by a warp-specialised block (1..4); claim_ahead 0 = claim the
 * next batch of items after finishing the current one, 1 = before starting
 * it, 2 = deep prefetch (one item per claim; the item three ahead is
 * claimed, two ahead fetched, the next one's image record and dependency
 * counter read while an item is issued); and the item-list lag (items
 * listed between an image's pass and its next pass; 0 keeps the current
 * order).  Defaults: 1, 0, five resident grids.
 */
GLSFFT_API int glsfft_batch_set_schedule(glsfft_batch plan, int claim_chunk, int claim_ahead,
                                         int lag_items);

/*
 * Synchronise `stream` and return the device-side status of the last
 * execution: GLSFFT_SUCCESS, or GLSFFT_ERROR_TIMEOUT when a dependency wait
 * hit its deadline (the launch still ran to completion).
 */
GLSFFT_API int glsfft_batch_status(glsfft_batch plan, void *stream);

/* Images in the persistent launch, work items, and its grid size. */
GLSFFT_API int glsfft_batch_info(glsfft_batch plan, int *persistent_images, int *items,
                                 int *grid);

/*
 * The plan's column-tiled workspace: images of the persistent launch with
 * 1024 rows and 16 <= cols <= 1024 get one image-sized device buffer each
 * (held by the plan, freed by glsfft_batch_destroy) when it fits the
 * context's budget next to the plan's tables.  A rows pass leaves such an image's
 * result there with its columns tiles contiguous, so the warp-specialised
 * schedules read every columns tile as one contiguous copy; without it the
 * columns passes read and write dst in place.  Results are the same either
 * way.  Reports the images that have one and the bytes held.
 */
GLSFFT_API int glsfft_batch_workspace(glsfft_batch plan, int *tiled_images, size_t *bytes);

/*
 * Host-side fault injection for tests: make the last work item wait for one
 * tile more than exists and set the wait deadline to wait_limit_ns, so the
 * next execution reports GLSFFT_ERROR_TIMEOUT instead of finishing cleanly.
 */
GLSFFT_API int glsfft_batch_inject_stall(glsfft_batch plan, long long wait_limit_ns);

/* The plan's current schedule: {variant, claim_chunk, claim_ahead, lag_items}. */
GLSFFT_API int glsfft_batch_get_schedule(glsfft_batch plan, int *schedule4);

/*
 * Autotuner of a batch plan (no reference counterpart).  First the images
 * that get their own pass launches have their per-size pass schedules tuned
 * (glsfft_autotune_fft2d).  Then every persistent-kernel schedule -- variant
 * (GLSFFT_BATCH_*) x item-order lag (2, 3, 4, 5, 6, 8 resident grids) x
 * claim chunk and claim-ahead ((1, 2, 4) x (0, 1), and 1 x 2), 132 in all --
 * is timed, `reps` graph launches
 * each (median, CUDA events on `stream`), on a shadow plan of the same
 * shapes, flags, alignments and aliasing over scratch buffers, so the
 * plan's own images are never read or written.  The six fastest and the
 * default are then timed again in three interleaved rounds (each keeps the
 * median of its three medians); the fastest of those is applied to the plan
 * unless the default schedule is within 1% of it.  With cache_path
 * set, the choice is looked up in / appended to that plan cache file
 * (keyed by device, driver, library version, the plan's size histograms and
 * flags); a hit is applied without timing.
 * result[6] = {variant, claim_chunk, claim_ahead, lag_items, 1 if from the
 * cache, candidates timed}; ms[2] = {chosen, default} per execution.
 * Either may be NULL.
 */
GLSFFT_API int glsfft_batch_autotune(glsfft_batch plan, const char *cache_path, int reps,
                                     void *stream, int *result, double *ms);

/*
 * The last glsfft_batch_autotune search of this plan (timed there, not from
 * the cache): *count candidates; the first `max` are written as
 * sched4[4i..4i+3] = {variant, claim_chunk, claim_ahead, lag in resident
 * grids} and ms[i] = median time per execution.
 */
GLSFFT_API int glsfft_batch_tuning(glsfft_batch plan, int max, int *sched4, double *ms,
                                   int *count);

/*
 * Timing counters of the warp-specialised kernels (no reference
 * counterpart; off by default, re-captures the graph).  While on, every
 * execution adds, summed over blocks, in nanoseconds: [0] producer time in
 * dependency waits, [1] in waits for a stage to be free, [2] in store
 * completion waits before publishing, [3] producer run time, [4] compute
 * warp 0's waits for staged tiles, [5] its run time; [6] items, [7] blocks.
 * glsfft_batch_get_stats synchronises `stream`, returns the sums (8
 * doubles) and resets them.
 */
GLSFFT_API int glsfft_batch_set_stats(glsfft_batch plan, int on);
GLSFFT_API int glsfft_batch_get_stats(glsfft_batch plan, void *stream, double *out8);

GLSFFT_API int glsfft_batch_destroy(glsfft_batch plan);

/*
 * gls::phaseCorrelate(src1, src2, window, &response),
 * glsCV/glsPhaseCorrelate.h:58 / glsPhaseCorrelate.cpp:142-236.
 * src1, src2: CV_32FC1 rows x cols device images; window: same shape or
 * NULL.  box: centroid box edge (the reference uses 5, glsPhaseCorrelate.cpp:219).
 * Writes the shift of src2 relative to src1 and the response
 * (sum over the box / (rows*cols)); dx/dy/response are host pointers
 * (response may be NULL).  Returns once the result is written: every
 * operation issued to `stream` before the call has completed and the call's
 * kernels have finished with the inputs and the workspace (the last one's
 * exit may trail by microseconds); a failed kernel is reported through the
 * stream's synchronisation.  Uses the context workspace
 * (20 * rows * cols bytes).  The three launches are kept as a CUDA graph and
 * replayed while a call repeats the last call's src1, src2, window, shape,
 * box and workspace (the buffers' contents may change); any other call
 * captures them anew.  Not to be called from inside a stream capture.
 */
GLSFFT_API int glsfft_phase_correlate(glsfft_context ctx, const float *src1, const float *src2,
                                      const float *window, int rows, int cols, int box,
                                      double *dx, double *dy, double *response, void *stream);

/*
 * Asynchronous form: writes 5 doubles to device memory `d_result`
 * {dx, dy, response, peak row-major index, peak value}; nothing is copied
 * to the host and nothing synchronises.
 */
GLSFFT_API int glsfft_phase_correlate_async(glsfft_context ctx, const float *src1,
                                            const float *src2, const float *window, int rows,
                                            int cols, int box, double *d_result, void *stream);

/*
 * Copy the real, quadrant-swapped correlation surface of the last
 * phaseCorrelate on this context (the plane the reference downloads for its
 * centroid, glsPhaseCorrelate.cpp:219) into the device buffer `dst` of
 * `count` floats (count must equal rows*cols of that call).  Asynchronous
 * on `stream`.  For tests and debugging.  The surface lives in the context
 * workspace: a later call that uses the workspace (the reference-arithmetic
 * FFT, minMaxLoc / normalize / FFT display with context keys) discards it,
 * and this call then returns GLSFFT_ERROR_SHAPE.
 */
GLSFFT_API int glsfft_phase_correlate_surface(glsfft_context ctx, float *dst, size_t count,
                                              void *stream);

/*
 * phaseCorrelate serving loop (no reference counterpart: glsCam calls
 * gls::phaseCorrelate one frame at a time, glsCam/glsCam.cpp).  A server
 * reserves `hbm_budget` bytes of device memory once and carves resident
 * reference spectra and per-request workspaces (16 * rows * cols bytes + 256)
 * out of it; `slots` streams let up to that many requests run at once.  A
 * native dispatcher admits queued requests in arrival order as a slot frees
 * and their workspace fits (continuous batching; it may admit a request
 * behind one that does not fit yet), and a native poller completes them.
 * Each request computes phaseCorrelate(reference frame, request frame) with
 * the reference's window, using the resident reference spectrum, so only
 * two FFTs run per request.
 */
typedef struct glsfft_server_s *glsfft_server;

GLSFFT_API int glsfft_server_create(glsfft_context ctx, int slots, size_t hbm_budget,
                                    glsfft_server *server);

/*
 * Make a reference resident: its spectrum FFT2(window x frame) is computed
 * once (frame, window: CV_32FC1 device images; window may be NULL) and
 * kept in the server's budget.  Synchronous.  Returns its id in *ref_id.
 * The server reads frame and window on its own stream: work that produces
 * them on another stream must be complete before the call.
 */
GLSFFT_API int glsfft_server_add_reference(glsfft_server server, const float *frame,
                                           const float *window, int rows, int cols, int *ref_id);

/*
 * Queue a request: the shift of host_frame (CV_32FC1, the reference's size,
 * host memory that stays valid until the request completes; page-locked
 * memory keeps the copy asynchronous) relative to reference ref_id.
 * Returns at once with a ticket.  GLSFFT_ERROR_BUDGET when the request could
 * never fit in the budget.
 */
GLSFFT_API int glsfft_server_submit(glsfft_server server, int ref_id, const float *host_frame,
                                    int box, long long *ticket);

/*
 * Wait (at most timeout_s) for a request; fills {dx, dy, response, peak
 * index, peak value} and the latency from arrival to completion, then forgets
 * the ticket.  GLSFFT_ERROR_TIMEOUT when it is still running.
 */
GLSFFT_API int glsfft_server_wait(glsfft_server server, long long ticket, double *result5,
                                  double *latency_s, double timeout_s);

/*
 * Open-loop load: request k arrives offsets_s[k] seconds after the call
 * (submitted by the calling thread on schedule), for reference ref_ids[k]
 * and frame host_frames[k]; blocks until all complete and writes each
 * latency (from its scheduled arrival) and result (5 doubles, may be NULL).
 */
GLSFFT_API int glsfft_server_replay(glsfft_server server, int n, const double *offsets_s,
                                    const int *ref_ids, const float *const *host_frames, int box,
                                    double *latencies_s, double *results5);

/*
 * glsfft_server_replay that also attributes each request's latency (no
 * reference counterpart): phases6[6k .. 6k+3] = seconds from the scheduled
 * arrival to the actual submission (the arrival thread's lateness), queued
 * (waiting for a slot, workspace or a dispatcher), issuing (the frame's
 * copy, the three launches and the events), and device work plus
 * completion polling -- these four sum to latencies_s[k] -- then
 * phases6[6k+4] = the device time between events recorded before the copy
 * and after the last launch (so phase 3 minus it is the completion lag) and
 * phases6[6k+5] = the part of it up to the end of the frame's copy.
 * phases6 may be NULL.
 */
GLSFFT_API int glsfft_server_replay_traced(glsfft_server server, int n, const double *offsets_s,
                                           const int *ref_ids, const float *const *host_frames,
                                           int box, double *latencies_s, double *results5,
                                           double *phases6);

/*
 * How requests bring their frame to the device (no reference counterpart).
 * 1 (the default): the windowed row pass reads the frame from host memory
 * itself, for frames in page-locked memory (cudaHostAlloc /
 * cudaHostRegister; other frames are copied).  0: a copy-engine transfer
 * into the request's workspace, then the row pass.  On GB300 the copy path
 * showed H2D tails of several milliseconds under load with many distinct
 * frames, the direct read did not; the copy path sustains more pairs per
 * second at saturation.  Results are identical.  Applies to requests
 * submitted afterwards.
 */
GLSFFT_API int glsfft_server_set_frame_read(glsfft_server server, int direct);

/* Counters: admitted, completed, failed, peak in flight, peak queue length,
 * budget bytes, peak budget bytes in use, resident references. */
GLSFFT_API int glsfft_server_stats(glsfft_server server, long long *out8);

/* Drop queued requests, finish running ones, free everything. */
GLSFFT_API int glsfft_server_destroy(glsfft_server server);

/* Largest image (rows * cols) glsfft_phase_correlate_noalloc accepts. */
#define GLSFFT_NOALLOC_MAX_PIXELS (512 * 512)

/*
 * phaseCorrelate that allocates no device memory at all.  No counterpart in
 * the reference (glsCV always allocates textures); it exists for callers
 * that may not call cudaMalloc: hosts whose device memory is owned by their
 * own pool or budget (a framework's caching allocator, a plugin host that
 * hands out buffers), where an allocation behind their back escapes that
 * accounting or fails once the pool holds the rest of the device; and
 * per-frame loops, where cudaMalloc/cudaFree synchronise the device and
 * stall the pipeline.  It needs no context.
 *
 * Same computation and result layout as glsfft_phase_correlate_async:
 * src1, src2 (and the optional window) are CV_32FC1 rows x cols device
 * images; 5 doubles {dx, dy, response, peak index, peak value} are written
 * to the device buffer d_result.  Its scratch (two spectra, the correlation
 * surface and the argmax word: 20 * rows * cols bytes) is one statically
 * sized device array of the library, so rows * cols must not exceed
 * GLSFFT_NOALLOC_MAX_PIXELS (GLSFFT_ERROR_NOALLOC_LIMIT otherwise).  That
 * array (5 MiB) and a 256 KiB twiddle table are held on every GPU that loads
 * the library until the process exits.
 *
 * The first call in a CUDA context (the current device's, for runtime-API
 * callers) sets up: it looks up the arrays' device addresses and uploads
 * the twiddle table with a synchronous copy; make that first call before
 * any stream capture.  The set-up is remembered per context, so after a
 * cudaDeviceReset the next call sets up again (and must again come before
 * any capture).  Every call uses the
 * same scratch array, which keeps the previous call's contents (the argmax
 * word is cleared on each call), so calls whose work overlaps on the GPU --
 * on different streams or from different host threads -- race: issue them
 * on one stream.
 */
GLSFFT_API int glsfft_phase_correlate_noalloc(const float *src1, const float *src2,
                                              const float *window, int rows, int cols, int box,
                                              double *d_result, void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GLSFFT_H_ */
