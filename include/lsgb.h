/*
 * lsgb.h -- C ABI of the GB300 Lomb-Scargle engine (liblsgb.so).
 *
 * Plain pointers and sizes only. Every call returns LSGB_OK (0) or a negative
 * status; lsgb_last_error() gives the message of the last failure on the calling
 * thread. Nothing here exits the process.
 *
 * Work model. A batch is n_obj objects whose observations are the rows
 * [offsets[o], offsets[o+1]) of the arrays t, y, dy (the reference's contiguous
 * object runs, source/main.cu:468-510 computeObjectRanges, expressed as offsets).
 * The frequency grid is angular, omega_k = fmin + df * k, k = 0..n_freq-1
 * (source/main.cu:1364, :1609-1611).
 *
 * Each entry point below replaces part of the reference's GPU path:
 *   lsgb_periodogram_device  -> source/main.cu:1006-1280 batchGPULS (and :570-720
 *                               GPULSOneObject for n_obj == 1) without its per-call
 *                               cudaMalloc/cudaFree, host argmax or forced pgram copy;
 *                               kernels source/kernel.cu:368-631 and :76-361.
 *   lsgb_periodogram_host    -> the same behind host buffers, including the copies
 *                               (source/main.cu:1070-1077 H2D, :1100-1110 D2H).
 * The reference-compatible entry point LombScarglePy is declared in lombscargle_py.h.
 */
#ifndef LSGB_H
#define LSGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSGB_API __attribute__((visibility("default")))

/* status codes */
#define LSGB_OK 0
#define LSGB_ERR_INVALID (-1)   /* bad argument: sizes, offsets, enum values */
#define LSGB_ERR_CUDA (-2)      /* a CUDA call failed (message names it) */
#define LSGB_ERR_NOMEM (-3)     /* device or pinned allocation failed */
#define LSGB_ERR_NODEVICE (-4)  /* no CUDA device: the engine never computes on the CPU */

/* bits of a call's status word (lsgb_status_async, lsgb_plan_status_async); the host-buffer
 * calls report them as LSGB_ERR_INVALID / LSGB_ERR_CUDA themselves */
#define LSGB_STATUS_TIMEOUT 1u    /* a bounded pipeline wait of the tensor form ran out */
#define LSGB_STATUS_BAD_INPUT 2u  /* a non-finite t or y, or (LSGB_GENERALIZED) a non-finite
                                     or non-positive dy: no defined periodogram */

/* variant: the reference's ERROR compile flag (source/params.h:12-16) */
#define LSGB_STANDARD 0     /* ERROR=0: standard L-S, source/kernel.cu:484-631 */
#define LSGB_GENERALIZED 1  /* ERROR=1: floating mean + 1/dy^2 weights, source/kernel.cu:368-477 */

/* precision form */
#define LSGB_PLAIN_FP64 0 /* FP64 sincos for every pair, FP64 atan2 tau: the drop-in form */
#define LSGB_MIXED 1      /* FP64 phase anchors + FP32-accurate sums: split-FP16 tensor-core
                             products (default shape) or FP32 recurrences (CUDA-core shapes) */

/* element type of t / y / dy / pgram / best_power */
#define LSGB_F32 0
#define LSGB_F64 1

typedef struct lsgb_engine lsgb_engine;

/* Create an engine bound to a CUDA device. The engine owns grow-only device
 * scratch buffers reused by every call. Calls on one engine must be issued from
 * one host thread at a time and ordered on one stream. */
LSGB_API int lsgb_engine_create(int device, lsgb_engine **out);
LSGB_API void lsgb_engine_destroy(lsgb_engine *eng);
LSGB_API const char *lsgb_last_error(void);
LSGB_API const char *lsgb_version(void);

/* Periodograms of a batch, inputs and outputs in device memory.
 *   t, y, dy     device arrays of offsets_host[n_obj] rows (dtype); dy may be NULL
 *                for LSGB_STANDARD.
 *   offsets_host host array of n_obj+1 non-decreasing row offsets, offsets[0] == 0;
 *                every object must have at least one row.
 *   normalize    LSGB_STANDARD only: multiply by 2/(N*var(y)) as the Python builds do
 *                (source/main.cu:1319-1352, -DNORMALIZEPGRAM=1).
 *   pgram        device [n_obj x n_freq] (dtype) or NULL: full periodogram.
 *   best_idx     device uint32[n_obj] or NULL: first index of the maximum power,
 *                0 when no power is positive (source/main.cu:1545-1563).
 *   best_power   device [n_obj] (dtype) or NULL: that power (0 when none).
 *   stream       cudaStream_t (NULL = legacy default stream).
 * Asynchronous with respect to the host. */
LSGB_API int lsgb_periodogram_device(lsgb_engine *eng, int variant, int precision, int dtype,
                                     const void *t, const void *y, const void *dy,
                                     const uint64_t *offsets_host, uint32_t n_obj, double fmin,
                                     double df, uint32_t n_freq, int normalize, void *pgram,
                                     uint32_t *best_idx, void *best_power, void *stream);

/* What the kernels of the device calls queued on `stream` so far have recorded: queues a
 * copy of the engine's status word into *host_status (host memory, pinned for a truly
 * asynchronous copy) followed by its reset. Once the stream has reached that point,
 * *host_status holds LSGB_STATUS_* bits; nonzero means the results of those calls are
 * invalid. The reference has no counterpart (it exits the process on any CUDA error,
 * source/main.cu:38-46, and never checks its inputs). */
LSGB_API int lsgb_status_async(lsgb_engine *eng, uint32_t *host_status, void *stream);

/* The same with host buffers (pinned or pageable). Copies the inputs in, computes,
 * copies pgram (if non-NULL) and the best index/power (if non-NULL) out, and
 * returns when they are in host memory. A status bit recorded by the call's kernels is
 * returned as LSGB_ERR_INVALID (LSGB_STATUS_BAD_INPUT) or LSGB_ERR_CUDA (timeout). */
LSGB_API int lsgb_periodogram_host(lsgb_engine *eng, int variant, int precision, int dtype,
                                   const void *t, const void *y, const void *dy,
                                   const uint64_t *offsets, uint32_t n_obj, double fmin, double df,
                                   uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                                   void *best_power);

/* The three best frequencies of every object, found on the device in the same kernel
 * pass (no periodogram copy needed). Replaces the reference's PRINTPERIODS==3 host scans
 * over the returned periodogram (source/main.cu:1165-1219, written out by
 * outputPeriodsToFileTopThree :982-995): three scans from (power 0, index 0), each taking
 * the first strictly larger power at an index the earlier scans did not take. So:
 *   top_idx    [n_obj x 3] uint32 (or NULL): per object the indices of its three largest
 *              positive powers, best first, the lowest index first among equal powers;
 *              0 where the object has fewer than three positive powers.
 *   top_power  [n_obj x 3] (dtype, or NULL): those powers (0 where there is none).
 * Other arguments as lsgb_periodogram_device / lsgb_periodogram_host; top_idx[3*o] and
 * top_power[3*o] are exactly what they return as best_idx[o] and best_power[o]. */
LSGB_API int lsgb_periodogram_top3_device(lsgb_engine *eng, int variant, int precision, int dtype,
                                          const void *t, const void *y, const void *dy,
                                          const uint64_t *offsets_host, uint32_t n_obj,
                                          double fmin, double df, uint32_t n_freq, int normalize,
                                          void *pgram, uint32_t *top_idx, void *top_power,
                                          void *stream);
LSGB_API int lsgb_periodogram_top3_host(lsgb_engine *eng, int variant, int precision, int dtype,
                                        const void *t, const void *y, const void *dy,
                                        const uint64_t *offsets, uint32_t n_obj, double fmin,
                                        double df, uint32_t n_freq, int normalize, void *pgram,
                                        uint32_t *top_idx, void *top_power);

/* ---- execution plans: one batch shape, captured once in a CUDA graph ----
 * lsgb_plan_create plans a batch exactly as lsgb_periodogram_device would (same
 * arguments; device pointers are fixed into the plan), uploads its per-object tables
 * once, and captures the kernel sequence (queue reset, statistics, records,
 * periodogram, argmax) in a CUDA graph. lsgb_plan_launch replays it on any stream
 * with one cudaGraphLaunch: the caller may rewrite the contents of t / y / dy
 * between launches, not their sizes or addresses. A plan owns its scratch buffers,
 * so plans and the engine's direct calls do not share state; two launches of one
 * plan must not overlap on the GPU. Takes the engine's current shape and
 * re-anchoring setting. No counterpart in the reference. */
typedef struct lsgb_plan lsgb_plan;
LSGB_API int lsgb_plan_create(lsgb_engine *eng, int variant, int precision, int dtype,
                              const void *t, const void *y, const void *dy,
                              const uint64_t *offsets_host, uint32_t n_obj, double fmin, double df,
                              uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                              void *best_power, lsgb_plan **out);
LSGB_API int lsgb_plan_launch(lsgb_plan *plan, void *stream);
/* Kernels per launch, work units, and the main kernel's time in the last launch
 * (waits for it and then reports a recorded status bit as lsgb_periodogram_host does;
 * pass NULL to skip). */
LSGB_API int lsgb_plan_info(lsgb_plan *plan, uint32_t *kernels, uint64_t *units,
                            float *last_kernel_ms);
/* lsgb_status_async for the launches of a plan. */
LSGB_API int lsgb_plan_status_async(lsgb_plan *plan, uint32_t *host_status, void *stream);
LSGB_API void lsgb_plan_destroy(lsgb_plan *plan);

/* Tuning of the mixed kernel: frequencies per thread (F), threads per CTA, the
 * minimum CTAs per SM the kernel's register budget is compiled for, the inner loop
 * (`packed`: 0 scalar rotation; 1 packed f32x2 rotation over consecutive frequencies;
 * 2 packed f32x2 over frequencies strided by the CTA width, advanced by the
 * second-order recurrence x[p+1] = 2 cos(phi) x[p] - x[p-1] where it is well
 * conditioned; 3 the tensor-core form, with F = coarse steps per unit and 128 threads
 * standing for its 128 fine steps: (64, 128, 1, 3, 0) standard and (32, 128, 1, 3, 0)
 * generalized, the defaults), and two observations per loop iteration (1) or one (0).
 * 0 (-1 for the last two) keeps the current value. Returns LSGB_ERR_INVALID for shapes
 * that are not compiled in. */
LSGB_API int lsgb_set_tuning(lsgb_engine *eng, int variant, int freqs_per_thread,
                             int threads_per_cta, int min_ctas_per_sm, int packed, int unroll);

/* The mixed-form periodogram of lsgb_periodogram_device, with no allocation at all.
 * No counterpart in the reference.
 *
 * For callers that must not allocate device memory while they run: a plugin inside
 * a framework whose own allocator owns the device-memory budget, a latency-critical
 * loop that cannot take the synchronization cudaMalloc/cudaFree may cause, or a
 * service that reserves its whole footprint at start-up. The regular entry points
 * grow engine buffers with cudaMalloc; this one needs no engine and uses one
 * fixed-size scratch array compiled into liblsgb.so (about 8.3 MiB, held on every
 * GPU that loads the library until the process exits).
 *
 * Arguments as lsgb_periodogram_device (mixed form; t, y, dy, pgram, best_idx and
 * best_power are caller-owned device memory; offsets is host memory). Limits of one
 * call: at most 131072 observations, 2048 objects, and 262144 (object x frequency
 * tile) units, a tile being 3072 frequencies for LSGB_STANDARD and 2048 for
 * LSGB_GENERALIZED; larger calls return LSGB_ERR_INVALID with the limit in
 * lsgb_last_error(). The first call on each device looks up the scratch array's
 * device address on that device. All calls share the one array and leave its contents behind, so calls whose GPU
 * work overlaps (different streams or host threads without ordering) race; order
 * them. Host set-up is serialized internally and waits for the stream's earlier
 * work before launching. */
LSGB_API int lsgb_periodogram_noalloc(int variant, int dtype, const void *t, const void *y,
                                      const void *dy, const uint64_t *offsets_host,
                                      uint32_t n_obj, double fmin, double df, uint32_t n_freq,
                                      int normalize, void *pgram, uint32_t *best_idx,
                                      void *best_power, void *stream);

/* ---- continuous-batching request loop (no counterpart in the reference, whose
 * entry point is one synchronous batch per call, source/main.cu:742-941) ----
 * Objects are submitted one at a time. A dispatcher thread packs whatever has
 * arrived into the next free slot (up to max_batch_objects), admits the batch only
 * while the device bytes of all in-flight batches stay under hbm_budget_bytes (a
 * single object larger than the budget runs alone), and launches it on the slot's
 * own stream and engine, so up to `slots` batches overlap on the GPU. Every object
 * gets the best frequency index and power of its periodogram over one shared grid.
 * While a batch is on the GPU the dispatcher polls its completion without sleeping
 * (one host core busy), so that results are published as soon as they are ready; with
 * nothing in flight it blocks until an object is submitted. */
typedef struct lsgb_server lsgb_server;

LSGB_API int lsgb_server_create(int device, int variant, int precision, double fmin, double df,
                                uint32_t n_freq, int normalize, uint32_t slots,
                                uint32_t max_batch_objects, uint64_t hbm_budget_bytes,
                                lsgb_server **out);
/* Copies the object's n observations (host doubles) into the queue; dy is read
 * only for LSGB_GENERALIZED. Thread-safe. */
LSGB_API int lsgb_server_submit(lsgb_server *srv, uint64_t id, const double *t, const double *y,
                                const double *dy, uint32_t n);
/* Up to max completed objects: id, best index, best power, submit and completion
 * times (seconds, lsgb_server_now() clock). Returns the count, or a negative status
 * once the loop has failed. */
LSGB_API int lsgb_server_poll(lsgb_server *srv, uint32_t max, uint64_t *ids, uint32_t *best_idx,
                              double *best_power, double *t_submit, double *t_done);
/* [batches launched, objects completed, largest batch, objects waiting, peak
 * in-flight device bytes] */
LSGB_API int lsgb_server_stats(lsgb_server *srv, uint64_t *out5);
/* [peak in-flight device bytes, peak batches (slots) in flight at once, peak objects
 * waiting for admission, admissions that stopped at the HBM budget] since the server was
 * created. */
LSGB_API int lsgb_server_peaks(lsgb_server *srv, uint64_t *out4);
LSGB_API double lsgb_server_now(void);
/* Finishes every submitted object, then stops the loop and frees it; results not yet
 * taken with lsgb_server_poll are discarded. */
LSGB_API void lsgb_server_destroy(lsgb_server *srv);

/* The compiled mixed-kernel shapes, as out[6*i .. 6*i+5] = (variant, F, threads,
 * min CTAs per SM, packed, unroll), at most max_shapes of them. Returns how many exist. */
LSGB_API int lsgb_mixed_shapes(int *out, int max_shapes);

/* Self-check of the plain form's FP64 sine/cosine (Cody-Waite reduction, table of
 * sin/cos(j pi/64), short polynomials) against CUDA's sincos() on n arguments spread
 * over [-scale, scale]: *max_err receives the largest absolute difference. */
LSGB_API int lsgb_fp64_sincos_check(lsgb_engine *eng, uint32_t n, double scale, double *max_err);

/* Re-anchoring interval R of the CUDA-core mixed form's recurrence (R > 0 runs that
 * form's consecutive-frequency rotation loop whatever the tuned shape). 0 (default): every thread's
 * run of F frequencies starts from an exact anchor, so no frequency is more than F-1
 * recurrence steps from one. R > 0: anchors only at multiples of R, each thread reaching
 * its run by up to R-1 extra FP32 steps -- the error of an R-step recurrence, at extra
 * cost; used to measure precision against R. */
LSGB_API int lsgb_set_reanchor(lsgb_engine *eng, uint32_t interval);

/* The shape the engine uses for a variant, in the same 6-int layout. */
LSGB_API int lsgb_get_tuning(lsgb_engine *eng, int variant, int *out6);

/* Limit, in SM clock cycles, of every bounded pipeline wait of the tensor form (0: the
 * default, 2^32 cycles, about 2 s). For tests and diagnostics: a limit far below a stage's
 * time makes the waits run out, and the call then reports LSGB_STATUS_TIMEOUT. The kernel
 * always waits with the default limit for its own copies and MMAs in flight before it
 * releases its shared memory and TMEM, whatever this limit. Plans keep the limit they were
 * created with. */
LSGB_API int lsgb_set_wait_limit(lsgb_engine *eng, uint64_t cycles);

/* Launch statistics of the last call: kernels launched and the work units the
 * persistent kernel processed. */
LSGB_API int lsgb_last_launch_info(lsgb_engine *eng, uint32_t *kernels_launched,
                                   uint64_t *work_units);

/* Device time (ms) of the last main (periodogram) kernel launch, measured with
 * CUDA events recorded around it on the call's stream; waits for it to finish. */
LSGB_API int lsgb_last_kernel_time(lsgb_engine *eng, float *ms);

#ifdef __cplusplus
}
#endif

#endif /* LSGB_H */
