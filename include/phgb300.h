/*
 * phgb300.h -- C ABI of libphgb300.so, the GB300 (sm_103a) implementation of
 * ParticleHolography.jl's reconstruction hot path.
 *
 * Every entry point replaces the body of one function of the reference
 * (ParticleHolography.jl v0.2.0); the citation above each declaration names
 * it.  A Julia wrapper keeps the reference's exported names and signatures
 * and forwards to these symbols with `ccall`, passing `pointer(A)` of its
 * CuArrays, the array sizes and `CUDA.stream().handle`.
 *
 * Conventions
 *  - All array pointers are DEVICE pointers owned by the caller, unless the
 *    parameter name ends in `_host`.  The library never frees caller memory.
 *  - A Julia array of size (n_fast, n_slow) is column-major; the library
 *    indexes the same buffer as a C-row-major [n_slow][n_fast] array.  A
 *    volume of Julia size (n_fast, n_slow, slices) is [slices][n_slow][n_fast].
 *  - Complex data are interleaved ComplexF32 (8 bytes: re, im).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Every call is
 *    asynchronous on that stream unless its comment says it synchronises.
 *  - Every function returns PH_OK (0) or a PH_ERR_* status; ph_last_error()
 *    gives the message.  Size errors carry the reference's @assert text.
 *  - A ph_ctx owns scratch device memory (allocated with cudaMalloc up to the
 *    HBM budget given at creation), twiddle tables and cached CUDA graphs.
 *    Calls on one context are serialised: a call issued on a different stream
 *    than the previous call first waits for the previous call's work.
 *  - FFT lengths: 2^a up to 8192 and 3*2^a up to 6144, per axis (n_fast and
 *    n_slow independently).  Other lengths return PH_ERR_UNSUPPORTED.
 */
#ifndef PHGB300_H
#define PHGB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PH_API __attribute__((visibility("default")))
#else
#define PH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ph_ctx ph_ctx;

/* status codes */
enum {
    PH_OK = 0,
    PH_ERR_SIZE = 1,        /* mirrors the size @asserts (holofunc.jl:101,185,217,249,301,341) */
    PH_ERR_DTYPE = 2,       /* mirrors the ArgumentError of _ifft_and_abs (holofunc.jl:164) */
    PH_ERR_TOO_LARGE = 3,   /* mirrors ccl.jl:187 (length > 2^32-1) */
    PH_ERR_OOM = 4,         /* scratch would exceed the context's HBM budget, or cudaMalloc failed */
    PH_ERR_CUDA = 5,        /* a CUDA runtime call or kernel launch failed */
    PH_ERR_TIMEOUT = 6,     /* a bounded device-side loop hit its iteration limit */
    PH_ERR_INVALID = 7,     /* null pointer, bad argument */
    PH_ERR_UNSUPPORTED = 8  /* FFT length not supported */
};

/* element types of volumes and label inputs */
enum {
    PH_N0F8 = 0,   /* FixedPointNumbers.N0f8: UInt8 raw, value = raw/255 */
    PH_F16 = 1,
    PH_F32 = 2,
    PH_F64 = 3,
    PH_C64 = 4,    /* ComplexF32 */
    PH_BOOL = 5    /* Bool / UInt8, 0 or nonzero */
};

/* options for ph_set_option */
enum {
    PH_OPT_SLICE_BATCH = 1,   /* slices per reconstruction batch (0 = automatic) */
    PH_OPT_USE_GRAPHS = 2,    /* 1 = replay cached CUDA graphs for repeated shapes (default 1) */
    PH_OPT_LOOP_LIMIT = 3,    /* iteration limit of bounded device loops (CCL root chase) */
    PH_OPT_PROFILE = 4,       /* 1 = time every pass kernel with CUDA events (ph_profile_report) */
    PH_OPT_FORM = 5           /* arithmetic of the projection's row pass: PH_FORM_* (default FP32) */
};

/* forms of the projection's row pass (ph_reconst_xyproj and its range and
 * batch forms, row lengths 1024 and 2048; other lengths and the volume paths
 * stay FP32).  The split forms run the row DFT as two complex DFT GEMMs on the
 * tensor cores with FP32 accumulation, each operand held as a hi + lo pair of
 * 16-bit words: */
enum {
    PH_FORM_FP32 = 0,     /* radix-16 Stockham FFT on the CUDA cores, FP32 */
    PH_FORM_BF16X3 = 1,   /* BF16 pairs, products hi.hi + lo.hi + hi.lo */
    PH_FORM_FP16X3 = 2,   /* FP16 pairs (tiles scaled by powers of two), three products */
    PH_FORM_FP16X2 = 3,   /* FP16 data pairs, DFT matrix in one FP16 word: hi.hi + lo.hi */
    PH_FORM_TUNED = 4     /* the form ph_autotune chose for the shape (FP32 where it chose none) */
};

/* ---- diagnostics ----------------------------------------------------------- */

/* Tensor-core self-test, no counterpart in the reference: d[128][n] (FP32) =
 * a[128][k] . b[n][k]^T for BF16 (fp16 = 0) or FP16 (fp16 = 1) operand bits,
 * computed by one tcgen05 MMA chain with the operand layout, descriptors and
 * tensor-memory path of the split-precision transform passes.  n a multiple of
 * 16 in [16, 128], k 64 or 128; all pointers device memory; *err (device int)
 * is raised if the completion wait times out.  Asynchronous on `stream`. */
PH_API int32_t ph_tc_selftest(float *d, const uint16_t *a, const uint16_t *b, int32_t n, int32_t k, int32_t fp16,
                              int32_t *err, void *stream);

/* ---- context -------------------------------------------------------------- */

/* Creates a context on `device`.  hbm_budget_bytes bounds the scratch memory the
 * context may hold (0 = no bound beyond the device's free memory). */
PH_API int32_t ph_create(int32_t device, size_t hbm_budget_bytes, ph_ctx **out);
PH_API void ph_destroy(ph_ctx *ctx);
PH_API const char *ph_last_error(const ph_ctx *ctx);
PH_API int32_t ph_version(void);
PH_API int32_t ph_set_option(ph_ctx *ctx, int32_t option, int64_t value);
/* Bytes of scratch currently held by the context. */
PH_API size_t ph_scratch_bytes(const ph_ctx *ctx);
/* Pre-allocates the scratch a reconstruction of this shape needs, so that a
 * later call allocates nothing (e.g. inside a CUDA stream capture). */
PH_API int32_t ph_reserve(ph_ctx *ctx, int32_t n_fast, int32_t n_slow, int32_t slices, void *stream);
/* Number of kernels this context has launched since creation. */
PH_API int64_t ph_kernel_launches(const ph_ctx *ctx);
/* With PH_OPT_PROFILE on, every pass kernel is bracketed by CUDA events on the
 * caller's stream.  Writes one line "name,launches,total_ms\n" per kernel
 * name into buf (NUL-terminated, truncated to cap), then clears the records.
 * Synchronises on the recorded events.  Returns the bytes needed. */
PH_API int64_t ph_profile_report(ph_ctx *ctx, char *buf, int64_t cap);

/* The autotuner (no reference counterpart): times the reconstruction of an
 * n_fast x n_slow x slices projection once per candidate -- slices per pass
 * CTA (the built-in rule, 16, 32, 64), the batch of slice intermediates (the
 * built-in rule, 64 slices) and, with allow_forms, the split-precision row-pass
 * forms -- on synthetic inputs, and keeps the fastest for the shape in the
 * context: every later reconstruction of that shape (single calls, batch
 * plans, servers) uses its slice group and batch, and its form under
 * PH_OPT_FORM = PH_FORM_TUNED.  With cache_path, the choice is read from and
 * written to a JSON file keyed by device name and shape (a shape already in
 * the file for the same slice count is not timed again).  choice (nullable,
 * int32[3]) = {form, group cap, batch slices} (0 = built-in rule); *ms_out
 * (nullable) = its time per reconstruction.  Synchronises; not inside a capture. */
PH_API int32_t ph_autotune(ph_ctx *ctx, int32_t n_fast, int32_t n_slow, int32_t slices, int32_t allow_forms,
                           const char *cache_path, int32_t *choice, double *ms_out, void *stream);

/* ---- transfer functions ---------------------------------------------------- */

/* cu_transfer_sqrt_arr (holofunc.jl:30-36; kernel holofunc.jl:8-15).
 * out[y][x] = 1 - ((x+1 - n_fast/2 - 1)*wavlen/n_fast/dx)^2
 *               - ((y+1 - n_slow/2 - 1)*wavlen/n_slow/dx)^2, FP64, stored Float32. */
PH_API int32_t ph_transfer_sqrt(ph_ctx *ctx, float *out, int32_t n_fast, int32_t n_slow,
                         double wavlen, double dx, void *stream);

/* cu_transfer (holofunc.jl:61-67; kernel holofunc.jl:38-45).
 * out = exp(i*2*pi*z0/wavlen*sqrtf(d_sqr)): Float32 sqrt, FP64 phase and
 * sin/cos, stored ComplexF32. */
PH_API int32_t ph_transfer(ph_ctx *ctx, void *out, const float *d_sqr, int32_t n_fast, int32_t n_slow,
                    double z0, double wavlen, void *stream);

/* No reference counterpart: the transfer function with the square-root term
 * kept in FP64 (the exact physics) on the same centred grid as ph_transfer;
 * evanescent frequencies are set to 0. */
PH_API int32_t ph_transfer_fp64(ph_ctx *ctx, void *out, int32_t n_fast, int32_t n_slow,
                         double z, double wavlen, double dx, void *stream);

/* ---- wavefronts ------------------------------------------------------------- */

/* cu_gabor_wavefront (holofunc.jl:80-82): out = sqrtf(holo) + 0i. */
PH_API int32_t ph_gabor_wavefront(ph_ctx *ctx, void *out, const float *holo, int32_t n_fast, int32_t n_slow,
                           void *stream);

/* cu_2d_pad (holofunc.jl:139-149): out (2n x 2n) = mean(in), with `in` placed at
 * rows/cols [n/2, n/2+n).  Square input only, as in the reference. */
PH_API int32_t ph_pad2d(ph_ctx *ctx, void *out, const void *in, int32_t n_fast, int32_t n_slow, void *stream);

/* cu_phase_retrieval_holo (holofunc.jl:100-129): Gerchberg-Saxton, `priter`
 * iterations, returns the wavefront at the plane of holo1 in `out`.
 * residual (nullable, device double): || |u2| - sqrt(I2) ||_2 / ||sqrt(I2)||_2
 * accumulated in FP64 just before the last amplitude replacement at plane 2. */
PH_API int32_t ph_phase_retrieval(ph_ctx *ctx, void *out, const float *holo1, const float *holo2,
                           const void *transfer, const void *invtransfer,
                           int32_t n_fast, int32_t n_slow, int32_t priter,
                           double *residual, void *stream);

/* ---- propagation and reconstruction ----------------------------------------- */

/* cu_asm_prop! (holofunc.jl:383-388): out = ifft(ifftshift(fftshift(fft(in)) .*
 * cu_transfer(zprop, ..., d_sqr))).  `out` may equal `in`. */
PH_API int32_t ph_asm_prop(ph_ctx *ctx, void *out, const void *in, const float *d_sqr, double zprop,
                    int32_t n_fast, int32_t n_slow, double wavlen, void *stream);

/* The propagation primitive shared by holofunc.jl:114,121,386:
 * out = ifft(ifftshift(fftshift(fft(in)) .* tf)) for a caller-built centred
 * transfer function `tf` (ComplexF32).  `out` may equal `in`. */
PH_API int32_t ph_propagate(ph_ctx *ctx, void *out, const void *in, const void *tf, int32_t n_fast, int32_t n_slow,
                            void *stream);

/* cu_apply_low_pass_filter[!] (frequency_filters.jl:88-107):
 * out = ifft(ifftshift(lpf .* fftshift(fft(in)))) for a centred Float32 mask.
 * `out` may equal `in`. */
PH_API int32_t ph_apply_lpf(ph_ctx *ctx, void *out, const void *in, const float *lpf, int32_t n_fast,
                            int32_t n_slow, void *stream);

/* cu_rectangle_filter (frequency_filters.jl:31-38; kernel :5-15): Float32 mask of
 * size imglen^2, 0 where (x - n/2 + 1)^2 + (y - n/2)^2 >= maxi^2 (x the slow
 * axis in this library's view, 1-based), else 1. */
PH_API int32_t ph_lpf_rectangle(ph_ctx *ctx, float *out, int32_t imglen, double prop_dist, double wavlen,
                                double pitch, void *stream);

/* cu_super_gaussian_filter (frequency_filters.jl:66-74; kernel :40-50):
 * exp(-1/2 (tx^2 + ty^2)^3), t = (i - n/2 + 1)/n/pitch/sigma, FP64, stored Float32. */
PH_API int32_t ph_lpf_super_gaussian(ph_ctx *ctx, float *out, int32_t imglen, double prop_dist, double wavlen,
                                     double pitch, void *stream);

/* cu_get_reconst_xyprojection (holofunc.jl:248-266), plus the argmin depth:
 * proj[y][x] = min_k |ifft(ifftshift(X_k))|^2 (unclamped), X_k =
 * fftshift(fft(wf)).*tf_front.*tf_dz^k; argmin (nullable, int32) = the first k
 * attaining the minimum.  The volume is never stored. */
PH_API int32_t ph_reconst_xyproj(ph_ctx *ctx, float *proj, int32_t *argmin, const void *wf,
                          const void *tf_front, const void *tf_dz,
                          int32_t n_fast, int32_t n_slow, int32_t slices, void *stream);

/* One depth shard of cu_get_reconst_xyprojection (holofunc.jl:248-266; its
 * serial slice loop :259-263): slices k in [k0, k1) with their GLOBAL index,
 * X_k = fftshift(fft(wf)).*tf_front.*tf_dz^k, reduced to packed words
 * packed[y][x] = (float bits of min_k |slice_k|^2) << 32 | k, first minimum on
 * ties.  accumulate = 0 first fills packed with PH_PACKED_EMPTY; 1 merges into
 * the words already there (a min per word).  Shards of one frame merged by a
 * per-word minimum (this call with accumulate = 1, or an int64 MIN all-reduce
 * across GPUs: every word, and the identity, is a non-negative int64) give the
 * projection and argmin of one ph_reconst_xyproj over [0, S); unpack them
 * with ph_unpack_projection.  k1 == k0 contributes the identity. */
#define PH_PACKED_EMPTY 0x7fffffffffffffffLL
PH_API int32_t ph_reconst_xyproj_range(ph_ctx *ctx, int64_t *packed, const void *wf, const void *tf_front,
                                       const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t k0, int32_t k1,
                                       int32_t accumulate, void *stream);

/* Packed words -> projection (float bits, nullable) and argmin (slice, nullable):
 * the proj that cu_get_reconst_xyprojection returns (holofunc.jl:265), from
 * the merged shards of ph_reconst_xyproj_range. */
PH_API int32_t ph_unpack_projection(ph_ctx *ctx, float *proj, int32_t *argmin, const int64_t *packed,
                                    int32_t n_fast, int32_t n_slow, void *stream);

/* cu_apply_low_pass_filter (frequency_filters.jl:88-107) followed by
 * cu_get_reconst_xyprojection (holofunc.jl:248-266), with the filter folded
 * into the spectrum: X_k = fftshift(fft(wf)) .* lpf .* tf_front .* tf_dz^k, no
 * inverse/forward FFT pair.  lpf: Float32 centred [n_slow][n_fast] (the
 * reference's CuLowPassFilter). */
PH_API int32_t ph_reconst_xyproj_lpf(ph_ctx *ctx, float *proj, int32_t *argmin, const void *wf,
                                     const void *tf_front, const void *tf_dz, const float *lpf,
                                     int32_t n_fast, int32_t n_slow, int32_t slices, void *stream);

/* cu_get_reconst_vol (holofunc.jl:184-200, vol_dtype N0F8/F16/F32/F64),
 * cu_get_reconst_complex_vol (holofunc.jl:216-232, vol_dtype C64) and
 * cu_get_reconst_vol_and_xyprojection (holofunc.jl:300-321, proj non-null:
 * strict-< minimum over the stored, clamped and converted volume). */
PH_API int32_t ph_reconst_vol(ph_ctx *ctx, void *vol, int32_t vol_dtype, float *proj, const void *wf,
                       const void *tf_front, const void *tf_dz,
                       int32_t n_fast, int32_t n_slow, int32_t slices, void *stream);

/* The binary volume particle_bounding_boxes consumes (particle_detection.jl:58-76):
 * vol[k][y][x] = clamp(|slice_k|^2, 0, 1) <= threshold as Bool (UInt8 0/1),
 * i.e. cu_get_reconst_vol(..., Float32) (holofunc.jl:184-200) .<= threshold in
 * one pass, without storing the Float32 volume.  proj (nullable): the strict-<
 * minimum of the clamped intensities, as ph_reconst_vol with F32. */
PH_API int32_t ph_reconst_binary_vol(ph_ctx *ctx, uint8_t *vol, float threshold, float *proj, const void *wf,
                                     const void *tf_front, const void *tf_dz, int32_t n_fast, int32_t n_slow,
                                     int32_t slices, void *stream);

/* The sub-volumes particle_coordinates / particle_coor_diams cut out of the N0f8
 * volume (particle_detection.jl:146-208), produced without the volume:
 * boxes_host holds `count` records of 6 int64 in the reference's particle_bbs
 * order (x_min, y_min, z_min, x_max, y_max, z_max), 1-based inclusive, x the
 * slow axis (Julia column), y the fast axis (Julia row), z the slice.  Sub-volume
 * i is d_vol[y_min:y_max, x_min:x_max, z_min:z_max] of cu_get_reconst_vol(...,
 * N0f8) (holofunc.jl:184-200), stored [z][x][y] (fast y) at byte
 * offsets_host[i] of `out`; offsets_host[count] = total bytes.  With out NULL
 * only the offsets are written.  Only the slices any box covers are computed. */
PH_API int32_t ph_reconst_subvolumes(ph_ctx *ctx, uint8_t *out, int64_t *offsets_host, const int64_t *boxes_host,
                                     int32_t count, const void *wf, const void *tf_front, const void *tf_dz,
                                     int32_t n_fast, int32_t n_slow, int32_t slices, void *stream);

/* cu_get_reconst_vol_and_xyprojection_padded (holofunc.jl:339-364): wf is
 * n x n, the transfer functions 2n x 2n; vol is N0f8 n x n x slices (the centre
 * crop); return_dtype is the reference's `return_type` (N0F8/F16/F32/F64). */
PH_API int32_t ph_reconst_vol_padded(ph_ctx *ctx, uint8_t *vol, float *proj, const void *wf,
                              const void *tf_front, const void *tf_dz,
                              int32_t n_fast, int32_t n_slow, int32_t slices,
                              int32_t return_dtype, void *stream);

/* ---- batches of reconstructions ------------------------------------------------- */

/* No single reference counterpart: a batch of cu_get_reconst_xyprojection calls
 * (holofunc.jl:248-266), one per hologram, each with its own size, transfer
 * functions and slice count (the reference runs them one after another from
 * its host loop).  One item: */
typedef struct ph_recon_item {
    const float *hologram;   /* Float32 [n_slow][n_fast]: wavefront = sqrt(hologram) + 0i
                                (cu_gabor_wavefront, holofunc.jl:80-82); or NULL */
    const void *wavefront;   /* ComplexF32 [n_slow][n_fast], used when hologram is NULL */
    const void *tf_front;    /* ComplexF32 centred transfer to the first slice */
    const void *tf_dz;       /* ComplexF32 centred transfer between slices */
    float *proj;             /* out: [n_slow][n_fast] minimum over slices of |u|^2 */
    int32_t *argmin;         /* out (nullable): first slice attaining it */
    int32_t n_fast, n_slow, slices;
} ph_recon_item;

typedef struct ph_batch ph_batch;

/* Plans a batch of cu_get_reconst_xyprojection calls (holofunc.jl:248-266):
 * validates every item (the same checks and messages as
 * ph_reconst_xyproj), spreads the items over `lanes` concurrent streams (1-16;
 * longest first, each to the least loaded lane), allocates the lanes' scratch
 * (its own, outside the context's arena) and records the whole batch as one
 * CUDA graph.  The plan keeps the item pointers: the buffers must stay valid
 * until ph_batch_destroy.  Synchronises the context's work. */
PH_API int32_t ph_batch_plan(ph_ctx *ctx, const ph_recon_item *items, int32_t count, int32_t lanes,
                             ph_batch **out);
/* Runs a planned batch on `stream` (one graph launch); the items' outputs are
 * written as by one cu_get_reconst_xyprojection (holofunc.jl:248-266) /
 * ph_reconst_xyproj call each, with identical results.  Asynchronous. */
PH_API int32_t ph_batch_run(ph_batch *batch, void *stream);
/* Bytes of device scratch the plan holds (no reference counterpart). */
PH_API size_t ph_batch_scratch_bytes(const ph_batch *batch);
/* Frees the plan (waits for its launches to finish; no reference counterpart). */
PH_API void ph_batch_destroy(ph_batch *batch);

/* ---- serving --------------------------------------------------------------------- */

/* A request queue in front of cu_get_reconst_xyprojection (holofunc.jl:248-266)
 * for a stream of holograms, with continuous admission under an HBM budget.
 * The server owns one scratch pool (its budget) and `lanes` work slots, each a
 * CUDA stream.  A request needs one block of the pool (its reconstruction
 * scratch, sized for its own shape and slice count) and a free slot; requests
 * are admitted in arrival order as slots and memory free up, and queue until
 * then.  Admitted requests run concurrently on their slots' streams.  A block
 * and its slot return to the server when the request's completion callback has
 * run.  The transfer functions are built as the reference builds them
 * (cu_transfer_sqrt_arr + cu_transfer, holofunc.jl:30-67) for Hf = H(-z0) and
 * Hdz = H(-dz) and kept in an LRU cache keyed by (size, distance, wavelength,
 * pitch), so recurring optics reuse them.  One request: */
typedef struct ph_serve_request {
    const float *hologram;   /* Float32 [n_slow][n_fast]; wavefront = sqrt(hologram) + 0i */
    float *proj;             /* out: minimum over slices of |u|^2 */
    int32_t *argmin;         /* out (nullable): first slice attaining it */
    int32_t n_fast, n_slow, slices;
    double z0, dz;           /* micrometres: first slice at z0, then steps of dz */
    double wavlen, dx;       /* micrometres */
    /* Device ingest (nullable frame; hologram is then ignored): the hologram is
     * made on the device from an 8-bit camera frame, as load_gray2float
     * (utils.jl:23-25), the background removal of the reference's
     * preprocessing docs (img .- bkg .+ offset) and pad_with_mean
     * (utils.jl:319-325) make it on the host.  The frame is row-major
     * [frame_n_fast rows][frame_pitch bytes] (a camera or BMP image: the
     * image's row is the Julia array's first index), frame_channels 1 or 3
     * equal channels (the first is read), rows bottom-up when frame_flip.
     * A frame smaller than n_fast x n_slow is centred and padded with its mean. */
    const uint8_t *frame;
    int32_t frame_n_fast, frame_n_slow, frame_pitch, frame_channels, frame_flip;
    const double *background;   /* nullable: Float64 [frame_n_slow][frame_n_fast] (make_background) */
    double background_offset;   /* added after the subtraction (the docs use 64/255) */
} ph_serve_request;

typedef struct ph_server ph_server;

enum { PH_PENDING = 9 };   /* ph_serve_poll: the request has not finished */

/* Creates a server for requests up to max_n_fast x max_n_slow x max_slices
 * (reconstruction of holofunc.jl:248-266).  scratch_budget_bytes is the pool
 * requests are admitted against (0 = lanes x the largest request's block); it
 * must hold at least one largest request. */
PH_API int32_t ph_serve_create(ph_ctx *ctx, int32_t lanes, int32_t max_n_fast, int32_t max_n_slow,
                               int32_t max_slices, int32_t tf_cache_entries, size_t scratch_budget_bytes,
                               ph_server **out);
/* Queues one cu_get_reconst_xyprojection (holofunc.jl:248-266) request and
 * returns at once with its ticket; it is admitted at once when a slot and its
 * block are free, else when earlier requests finish.  The request runs after
 * the work queued on `stream` before this call (the work that wrote its
 * inputs).  Inputs and outputs must stay valid until it has finished.
 * Thread-safe; one poller per ticket. */
PH_API int32_t ph_serve_submit(ph_server *srv, const ph_serve_request *req, int64_t *ticket, void *stream);
/* PH_OK when the request has finished (the ticket is then released and
 * *latency_ms, if non-NULL, is submission to completion, queueing included),
 * PH_PENDING if not yet (wait = 0), or waits for it (wait = 1), admitting
 * queued requests as earlier ones finish.  No reference counterpart. */
PH_API int32_t ph_serve_poll(ph_server *srv, int64_t ticket, int32_t wait, double *latency_ms);
/* Requests queued and running, pool bytes in use and at peak, the number of
 * requests that had to queue at submission, and the number admitted in shared
 * launches: requests of the same shape, slices and optics queued together are
 * admitted as one group (up to 8) on one slot and one block, and share one
 * launch of each pass (each pointer nullable).  (no reference counterpart) */
PH_API int32_t ph_serve_stats(ph_server *srv, int64_t *queued, int64_t *running, size_t *bytes_in_use,
                              size_t *bytes_peak, int64_t *waited, int64_t *grouped);
/* Runs every queued request to completion, frees the server (no reference counterpart). */
PH_API void ph_serve_destroy(ph_server *srv);

/* ---- preprocessing ------------------------------------------------------------- */

/* cu_make_background_mode (utils.jl:279-317) and make_background(...; mode=:mode)
 * (utils.jl:210-231): the per-pixel most frequent value over `count` UInt8
 * images ([count][n_slow][n_fast], device), the first maximum on ties, written
 * as Float64 value / 255.  count <= 65535 (PH_ERR_TOO_LARGE beyond). */
PH_API int32_t ph_background_mode(ph_ctx *ctx, double *out, const uint8_t *images, int64_t count, int32_t n_fast,
                                  int32_t n_slow, void *stream);
/* make_background(...; mode=:mean) (utils.jl:212-218): the per-pixel mean of
 * the images read as Float32(value / 255), accumulated in Float64 in image order. */
PH_API int32_t ph_background_mean(ph_ctx *ctx, double *out, const uint8_t *images, int64_t count, int32_t n_fast,
                                  int32_t n_slow, void *stream);
/* pad_with_mean (utils.jl:319-325): out (padsize x padsize Float32) = mean(img)
 * (accumulated in Float64), with img (n_slow x n_fast) at fast offset
 * padsize/2 - n_fast/2 and slow offset padsize/2 - n_slow/2.  padsize must
 * exceed both sizes (the reference's @assert). */
PH_API int32_t ph_pad_with_mean(ph_ctx *ctx, float *out, const float *img, int32_t n_fast, int32_t n_slow,
                                int32_t padsize, void *stream);

/* ---- synthetic input ----------------------------------------------------------- */

/* No reference counterpart (the reference ships no generator): the seeded
 * inline hologram of opaque discs described by its docs
 * (whats_inline_holography.md:17-33).  discs_host is [count][4] doubles
 * (x, y, diameter, z) in micrometres.  A unit plane wave starts at the farthest
 * disc; at each disc plane psi *= (1 - A_i); between planes and on to z_sensor
 * psi is propagated by the angular spectrum with FP64-phase transfer
 * functions.  out = (|psi|^2 - min) / (max - min) + noise (noise: device
 * Float32 array or NULL). */
PH_API int32_t ph_synth_hologram(ph_ctx *ctx, float *out, int32_t n_fast, int32_t n_slow, const double *discs_host,
                                 int32_t count, double wavlen, double dx, double z_sensor, const float *noise,
                                 void *stream);

/* ---- connected-component labeling -------------------------------------------- */

/* The thresholding broadcast that feeds the labeling, `img .<= threshold`
 * (runtests.jl:183, particle_detection usage): out[i] = in[i] <= threshold
 * as Bool (UInt8 0/1). */
PH_API int32_t ph_binarize_le(ph_ctx *ctx, uint8_t *out, const float *in, int64_t n, float threshold,
                              void *stream);

/* cu_connected_component_labeling (ccl.jl:186-211).  `img` (F32 or BOOL) is
 * labelled as a C-row-major rows x cols grid: 8-connected components of equal
 * value; pixels with value > 0 get 1 + the minimum linear index of their
 * component, others 0.  The reference's own grid is rows = size(img,1),
 * cols = size(img,2) over the column-major buffer. */
PH_API int32_t ph_ccl(ph_ctx *ctx, uint32_t *labels, const void *img, int32_t img_dtype,
               int64_t rows, int64_t cols, void *stream);

/* The per-slice labeling loop of particle_bounding_boxes (particle_detection.jl:58-76),
 * in one launch set: `img` holds `slices` images of rows x cols (a binary
 * volume); each is labelled on its own exactly as ph_ccl labels one image
 * (labels relative to the image: 1 + the minimum index within the image). */
PH_API int32_t ph_ccl_batch(ph_ctx *ctx, uint32_t *labels, const void *img, int32_t img_dtype, int64_t slices,
                            int64_t rows, int64_t cols, void *stream);

/* get_bounding_rectangles (ccl.jl:240-264) for every component of labels from
 * ph_ccl / ph_ccl_batch, computed on the device: boxes_host gets up to
 * `capacity` records of 5 int64 (global 1-based root index, x_min, y_min,
 * x_max, y_max), x the slow (column) axis and y the fast axis, 1-based, ordered
 * by root; *count_host = the number of components.  Synchronises. */
PH_API int32_t ph_ccl_boxes(ph_ctx *ctx, int64_t *boxes_host, int64_t capacity, int64_t *count_host,
                            const uint32_t *labels, int64_t slices, int64_t rows, int64_t cols, void *stream);

/* count_labels (ccl.jl:213-221) and cu_find_valid_labels (ccl.jl:224-238):
 * writes the sorted 1-based indices i with labels[i] == i into roots_host (up to
 * `capacity` of them, may be NULL when capacity is 0) and their number into
 * *count_host.  Synchronises `stream`. */
PH_API int32_t ph_ccl_roots(ph_ctx *ctx, int64_t *roots_host, int64_t capacity, int64_t *count_host,
                     const uint32_t *labels, int64_t n, void *stream);

/* ---- without device allocation ---------------------------------------------------- */

/* No counterpart in the reference.  The component count of count_labels /
 * ph_ccl_roots for callers that cannot allocate device memory (a real-time
 * acquisition loop that forbids allocation once the camera runs, a host that
 * only lends the library buffers it registered up front): no context, no
 * cudaMalloc.  Its
 * scratch is a fixed 256 KiB device array inside the library, present on every
 * GPU that loads it until the process exits.  count: device int64 output;
 * labels: n UInt32 labels (at most 2^28, larger n returns PH_ERR_TOO_LARGE).
 * Asynchronous on `stream` on the current device.  The first call on a device
 * looks the array's device address up and should come before any stream
 * capture; the address is kept for the process, so calls must not cross a
 * cudaDeviceReset.  All calls share the array: calls that overlap on the GPU
 * race. */
PH_API int32_t ph_ccl_count_noalloc(int64_t *count, const uint32_t *labels, int64_t n, void *stream);
/* Message of the last failed ph_ccl_count_noalloc call of this thread. */
PH_API const char *ph_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PHGB300_H */
