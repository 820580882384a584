/*
 * Extensions of the GB300 backend beyond the reference C ABI.
 *
 * None of these has a counterpart in the reference binding; they expose what
 * a GPU-resident caller needs (device pointers, streams, arithmetic form) and
 * what the tests and benchmarks need (model parameters, launch counts).
 */
#ifndef AC_GB300_EXT_H
#define AC_GB300_EXT_H

#include <stdint.h>

#include "ac_processor.h"

/* Arithmetic form of the 8->8 convolutions of the luma network. */
enum ACGB300Precision
{
    AC_GB300_FP32 = 0, /* plain FP32 on CUDA cores (the parity form) */
    AC_GB300_FP16 = 1, /* tcgen05 tensor cores, FP16 operands, FP32 accumulation */
    AC_GB300_BF16 = 2  /* tcgen05 tensor cores, BF16 operands, FP32 accumulation */
};

/* A pitched image in device memory (same field meaning as ACImage). */
typedef struct ACGB300DeviceImage
{
    void* ptr;
    int width;
    int height;
    int channels;
    int stride;
    int element_type;
} ACGB300DeviceImage;

/* Selects the arithmetic form of a created processor.  The initial form is
 * AC_GB300_FP32, or the one named by the environment variable
 * AC_GB300_PRECISION ("fp32", "fp16", "bf16") at creation. */
AC_C_API int ac_gb300_set_precision(ACProcessor* processor, int precision);
AC_C_API int ac_gb300_get_precision(const ACProcessor* processor);

/* Output size that ac_processor_process gives for an empty dst. */
AC_C_API int ac_gb300_output_shape(int width, int height, int channels, double factor, int* out_width, int* out_height);

/* Processor::process between device-resident images: src and dst are in HBM
 * (dst preallocated with the output shape), all work is queued on `stream`
 * (a cudaStream_t; NULL = the calling thread's stream of this processor).
 * With sync != 0 the call waits for completion.  Returns AC_SUCCESS or
 * AC_ERROR(AC_EPROCESSOR) / AC_ERROR(AC_EINVAL); details via
 * ac_processor_error(). */
AC_C_API int ac_gb300_process_device(ACProcessor* processor, const ACGB300DeviceImage* src, const ACGB300DeviceImage* dst,
                                     double factor, void* stream, int sync);

/* Processor::process over `count` device images at once, each src/dst pair
 * as for ac_gb300_process_device.  An ACNetLegacy model at factor 2 in the
 * FP16 or BF16 form runs every group of images with one channel count and
 * element type (up to 64 per launch, any mix of sizes) as ONE persistent
 * tensor-core launch over a shared tile queue (the quad kernel, one 46x46
 * tile shape; with AC_GB300_TC_KERNEL=3 the pair kernel, whose tile shape and
 * CTAs per SM come from a measured autotune the first time a batch class is
 * seen); a repeated identical batch (same buffers and shapes) replays a
 * captured CUDA graph.
 * Other models, factors and forms process the images one after another.
 * Returns AC_SUCCESS or AC_ERROR(AC_EPROCESSOR) / AC_ERROR(AC_EINVAL). */
AC_C_API int ac_gb300_process_batch_device(ACProcessor* processor, int count, const ACGB300DeviceImage* src,
                                           const ACGB300DeviceImage* dst, double factor, void* stream, int sync);

/* The persistent tensor-core launch plan of the calling thread's most recent
 * call on this processor: *kernel 4 (the quad kernel, ACNetLegacy), 3 (the
 * pair kernel), 5 (the quad kernel, ACNet<8>) or 0 (no such launch yet);
 * *tile_w x *tile_h its tile shape; *ctas_per_sm the CTAs-per-SM cap;
 * *fusion_depth (may be NULL) the layers one launch runs: 9 for the whole
 * network in one launch, 5 for the network split in two launches at layer 5
 * (the first launch writes a 16-bit activation map, the second runs the
 * rest and the colour epilogue in the reported tiles: 46x57 for
 * ACNetLegacy, 44x60 for ACNet<8> B8, which runs split by default).  The plan is the
 * autotuner's choice for the call's batch class, measured the first time
 * the class was seen, or the one the environment forced (AC_GB300_TC3_SHAPE,
 * AC_GB300_TC3_PER_SM, AC_GB300_FUSION_DEPTH).  Returns AC_SUCCESS or
 * AC_ERROR(AC_EINVAL). */
AC_C_API int ac_gb300_last_plan(ACProcessor* processor, int* kernel, int* tile_w, int* tile_h, int* ctas_per_sm,
                                int* fusion_depth);

/* Host-side fault injection for tests of the failure paths: arms the
 * nth next device allocation of the library's work buffers or serving pool
 * (counted over the whole process) to fail as if the device were out of
 * memory; no allocation is attempted for it.  0 disarms.  The failing call
 * reports AC_ERROR(AC_EPROCESSOR) with a "device allocation" message (a
 * serving job: status -1) and later calls succeed.  No reference
 * counterpart. */
AC_C_API void ac_gb300_debug_fail_alloc(int nth);

/* Number of batched launches this process has run as CUDA graph replays. */
AC_C_API uint64_t ac_gb300_graph_replays(void);

/* The reference CLI's video recipe (cli/src/Main.cpp:183-206) on planar
 * frames in device memory, `frames` frames of `planes` planes each, indexed
 * src[f * planes + p]: plane 0 (Y, one channel) is shifted left by `shift`
 * bits (ac::core::shl, core/src/ImageProcess.cpp:601-608), upscaled by
 * `factor` through the network and shifted back (shr, :609-616) into dst
 * plane 0; every further plane (U and V, or interleaved UV) is resized to its
 * dst plane's size with Catmull-Rom, as ac::core::resize(src, dst, 0, 0).
 * The source planes are not modified.  The Y planes of all frames run as one
 * batch (ac_gb300_process_batch_device; an ACNetLegacy x4 in a tensor-core
 * form as two chained batched x2 passes).  Returns AC_SUCCESS or
 * AC_ERROR(AC_EPROCESSOR) / AC_ERROR(AC_EINVAL). */
AC_C_API int ac_gb300_process_yuv_device(ACProcessor* processor, int frames, int planes, const ACGB300DeviceImage* src,
                                         const ACGB300DeviceImage* dst, double factor, int shift, void* stream, int sync);

/* Allocation-free x2 upscale of `count` device images in ONE persistent
 * tensor-core launch.  No reference counterpart: the reference's processors
 * allocate their work buffers inside each call.  It is for callers that must
 * not allocate device memory once running: a real-time video or rendering
 * pipeline whose device memory is planned up front, or a host application
 * that forbids allocation (and the synchronisation an allocation can imply)
 * on its frame thread.  The call allocates no device memory and, when it
 * succeeds, no host memory.
 *
 * Requirements and limits: an ACNetLegacy processor in the FP16 or BF16 form
 * whose packed weights are already on the device (make one ordinary process
 * call in that form first); 1 to 64 images per call, all with the first
 * image's channel count (1, 3 or 4) and element type; every dst exactly 2x
 * its src.  Anything else is rejected with AC_ERROR(AC_EINVAL) and a message
 * in ac_processor_error().  Scratch: a 256-byte static device array in the
 * library, of which a call uses 8 bytes (the tile-queue counter and a status
 * word, both zeroed on `stream` at the start of every call).
 *
 * The first call on a device does set-up (it looks up the scratch address
 * and configures the kernel): make that first call before any stream
 * capture.  Calls that overlap in time on one device share the scratch and
 * race: serialise them (one stream, or events).  `stream` NULL is the legacy
 * default stream.  With sync != 0 the call waits and reports a timed-out
 * tensor-core wait as AC_ERROR(AC_EPROCESSOR).  With sync == 0 a timeout is
 * not reported: the status word lives in the shared scratch and the next
 * call clears it, so a caller that needs the outcome passes sync != 0. */
AC_C_API int ac_gb300_process_device_noalloc(ACProcessor* processor, int count, const ACGB300DeviceImage* src,
                                             const ACGB300DeviceImage* dst, void* stream, int sync);

/* Kernel timing of the luma network passes: when enabled, the processor
 * records a CUDA event pair on the launching stream around every luma-pass
 * launch of the calling thread; ac_gb300_profile_collect waits for them and
 * returns the summed milliseconds, the launch count and the summed output
 * pixels of those launches, then clears the record. */
AC_C_API int ac_gb300_profile_enable(ACProcessor* processor, int enable);
AC_C_API int ac_gb300_profile_collect(ACProcessor* processor, double* ms, int* launches, double* out_pixels);

/* Diagnostic: one tensor-core tile D[128][16] = A * B^T computed with the
 * same tcgen05 descriptors, tensor-memory layout and completion protocol the
 * kernels use.  A(m, k) = x[(m + (k / 8) * shift) * 8 + k % 8] (x holds px
 * pixels of 8 16-bit values), b is [16][k] with k a multiple of 16 (<= 64),
 * FP16 or (bf16 != 0) BF16 bit patterns; d receives [128][16] floats.
 * Returns 0, 1 if the tensor core did not complete within 2 s, -1 on error. */
AC_C_API int ac_gb300_tc_selftest(const uint16_t* x, int px, const uint16_t* b, int k, int shift, int bf16, float* d);

/* Diagnostic of the failure path: one GPU thread waits, with the kernels'
 * bounded mbarrier wait limited to limit_ms (1..2000), on a phase that nothing
 * completes.  *status receives 1 when the wait gave up (the designed outcome;
 * 2 would mean the phase completed), *elapsed_ms how long it waited.  Returns
 * 0, or -1 on error. */
AC_C_API int ac_gb300_wait_selftest(int limit_ms, int* status, double* elapsed_ms);

/* Number of kernels this library has launched in the process so far. */
AC_C_API uint64_t ac_gb300_launch_count(void);

/* Copies the parameters of `model` (reference NHWC blob layout) into the
 * given arrays when non-NULL and stores the element counts in counts[3]
 * (kernels, biases, alphas).  Returns AC_ERROR(AC_EINVAL) for an unknown
 * model or arrays that are too small. */
AC_C_API int ac_gb300_model_params(const char* model, float* kernels, int kernels_len, float* biases, int biases_len,
                                   float* alphas, int alphas_len, int* counts);

/* ---- Serving loop (no reference counterpart: the reference serves one
 * image per Processor::process call).  A server admits upscale jobs of mixed
 * resolutions, factors, models and formats by an HBM budget, keeps weights
 * and frame buffers resident on the device, batches compatible jobs as they
 * arrive (ACNetLegacy x2 of interleaved images in a tensor-core form: one
 * persistent launch) and overlaps the work of different jobs through
 * `workers` streams.  Jobs with an input of at most 1920x1080 are served on
 * high-priority streams by all but one in eight of the workers; larger jobs
 * run on the others, one or two at a time, their persistent launches at one
 * CTA per SM, so a small job's work finds room on the device at once.  A
 * job's result is the same as ac_processor_process gives for it alone. */
typedef struct ACGB300HostPlane
{
    void* ptr; /* host memory; pinned memory lets the copies overlap */
    int width;
    int height;
    int channels;
    int stride;
    int element_type;
} ACGB300HostPlane;

typedef struct ACGB300ServeJob
{
    const char* model; /* as for ac_processor_create (read during submit) */
    double factor;
    int planes; /* 1: one interleaved image (1, 3 or 4 channels); 2 or 3: planar YUV, Y first */
    int shift;  /* planar YUV: shl / shr bits of Y (ac_gb300_process_yuv_device) */
    ACGB300HostPlane src[3];
    ACGB300HostPlane dst[3]; /* src and dst must stay valid until the job is waited for */
} ACGB300ServeJob;

typedef struct ACGB300ServeResult
{
    int status;        /* 0 done, -1 failed, -2 rejected (malformed, or larger than the budget) */
    double queue_ms;   /* submit -> admitted */
    double device_ms;  /* first copy issued -> result in dst */
    double latency_ms; /* submit -> result in dst */
    double h2d_ms;     /* GPU time of the input copies (CUDA events on the worker's stream) */
    double compute_ms; /* GPU time from the input copies' end to the processing's end */
    double d2h_ms;     /* GPU time of the output copies */
    int batch;         /* jobs that shared this job's launch */
    char error[160];
} ACGB300ServeResult;

typedef struct ACGB300ServeStats
{
    uint64_t submitted, completed, failed, batches, batched_jobs;
    double budget_bytes, in_use_bytes, peak_bytes, pool_bytes;
    uint64_t device_allocs; /* device allocations of the process so far (serving pool and work buffers) */
} ACGB300ServeStats;

typedef struct ACGB300Server ACGB300Server;

/* precision: AC_GB300_FP32 / FP16 / BF16; hbm_budget_bytes caps the device
 * bytes of admitted jobs (frame buffers plus a conservative estimate of their
 * work buffers) and of the buffer pool; at most max_batch (<= 64) jobs share
 * a launch.  Returns NULL only when out of host memory; then check
 * ac_gb300_server_error. */
AC_C_API ACGB300Server* ac_gb300_server_create(int device, int precision, double hbm_budget_bytes, int workers, int max_batch);
/* NULL when the server is usable, else why it is not. */
AC_C_API const char* ac_gb300_server_error(const ACGB300Server* server);
AC_C_API int ac_gb300_server_submit(ACGB300Server* server, const ACGB300ServeJob* job, uint64_t* ticket);
/* AC_SUCCESS once the job finished (its outcome in result->status), 1 when
 * timeout_s passed first, AC_ERROR(AC_EINVAL) for a bad argument. */
AC_C_API int ac_gb300_server_wait(ACGB300Server* server, uint64_t ticket, double timeout_s, ACGB300ServeResult* result);
AC_C_API int ac_gb300_server_stats(ACGB300Server* server, ACGB300ServeStats* stats);
/* Stops the server; jobs not yet run are dropped. */
AC_C_API void ac_gb300_server_destroy(ACGB300Server* server);

#endif
