/*
 * scir_gb300.h -- C ABI of the GB300 (sm_103a) batched-filtering library.
 *
 * This is the boundary a SciR build binds over FFI in place of the CUDA
 * module inside crates/scir-gpu.  Two layers are exported:
 *
 *  - Stream-ordered device entry points (scir_fir_batched_f32, ...): every
 *    pointer is a device pointer, every call is asynchronous on the caller's
 *    cudaStream_t (NULL = legacy default stream) and returns a status code.
 *    Buffers are caller-owned, rows are strided by ld_* elements.
 *
 *  - Host-buffer entry points named after the reference's Rust functions
 *    (scir_fir1d_batched_f32_cuda, scir_sosfilt_f64, ...): plain host
 *    pointers in, host pointers out, synchronous, exactly the semantics of
 *    the function they replace.  These are what the Rust FFI crate calls to
 *    keep the scir-gpu / scir-signal signatures.
 *
 * Every function returns SCIR_OK (0) or an scir_status error code; the
 * thread-local detail is available from scir_last_error().  No function falls
 * back to a CPU implementation: when the CUDA device or the compiled kernels
 * are unavailable the call fails with SCIR_ERR_NO_DEVICE / SCIR_ERR_CUDA.
 *
 * Threading: calls may come from any host thread; the library keeps only
 * per-device immutable data and a mutex-protected staging pool for the
 * host-buffer layer.  Device entry points never synchronise the stream.
 */
#ifndef SCIR_GB300_H
#define SCIR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SCIR_API __attribute__((visibility("default")))
#else
#define SCIR_API
#endif

#define SCIR_GB300_ABI_VERSION 1

/* Status codes.  The reference reports GPU failures as
 * GpuError::{BackendUnavailable(String), ShapeMismatch}
 * (crates/scir-gpu/src/lib.rs:58-63); the FFI crate maps SCIR_ERR_SHAPE to
 * ShapeMismatch and every other code to BackendUnavailable(message). */
typedef enum scir_status {
    SCIR_OK = 0,
    SCIR_ERR_INVALID_ARG = 1, /* null pointer, negative size, bad enum      */
    SCIR_ERR_SHAPE = 2,       /* sizes inconsistent (n < k for VALID, ...)  */
    SCIR_ERR_ALIGN = 3,       /* pointer/stride alignment a kernel requires */
    SCIR_ERR_OOM = 4,         /* device or pinned allocation failed         */
    SCIR_ERR_CUDA = 5,        /* CUDA runtime error (message has details)   */
    SCIR_ERR_TIMEOUT = 6,     /* bounded device-side wait gave up           */
    SCIR_ERR_UNSUPPORTED = 7, /* valid request this build does not serve    */
    SCIR_ERR_NO_DEVICE = 8    /* no CUDA device / kernel image for it       */
} scir_status;

/* FIR output conventions.  Every mode is computed as
 *   y[o] = sum_{m<k} c[m] * x[o + s + m],  x = 0 outside [0, n)
 * SCIR_FIR_REF_CORR: the reference fir1d_batched_f32 (crates/scir-gpu/src/
 *   lib.rs:1134-1152): c = taps, s = -(k-1), n outputs, i.e.
 *   y[i] = sum_j taps[k-1-j] * x[i-j]  (= scipy lfilter(taps[::-1], 1, x)).
 * SCIR_FIR_LFILTER: scipy.signal.lfilter(taps, 1, x): c = reversed taps,
 *   s = -(k-1), n outputs.
 * SCIR_FIR_FULL / SCIR_FIR_VALID: numpy.convolve(x, taps, 'full'|'valid'):
 *   n+k-1 outputs / n-k+1 outputs (VALID needs n >= k). */
typedef enum scir_fir_mode {
    SCIR_FIR_REF_CORR = 0,
    SCIR_FIR_LFILTER = 1,
    SCIR_FIR_FULL = 2,
    SCIR_FIR_VALID = 3
} scir_fir_mode;

/* Arithmetic used for a FIR / polyphase contraction.
 * SCIR_PREC_REF_EXACT: FP32 on CUDA cores with the reference's summation
 *   order and separate multiply/add roundings (no FMA): bit-identical to
 *   the reference CPU loop for SCIR_FIR_REF_CORR.
 * SCIR_PREC_FP32: FP32 FMA on CUDA cores ("plain").
 * SCIR_PREC_BF16X3: tensor cores (tcgen05, kind::f16), operands split into
 *   bf16 hi+lo, three products (hi*hi + hi*lo + lo*hi), FP32 accumulate.
 * SCIR_PREC_BF16X6: tensor cores, operands split into three bf16 terms,
 *   six products; FP32-level accuracy.
 * SCIR_PREC_FP16X3: tensor cores, each signal row and the taps scaled by a
 *   power of two (from their largest finite magnitude) and split into fp16
 *   hi+lo (22 significant bits), three products; BF16X6's accuracy at
 *   BF16X3's cost.  FIR entry points only (the polyphase path has no such
 *   form: SCIR_ERR_UNSUPPORTED).
 * SCIR_PREC_AUTO: the library picks (autotuned, accuracy <= 1e-5 normwise;
 *   on the tensor cores the FP16X3 form).
 * On the tensor cores an Inf or NaN sample makes NaN every output whose
 * tile reads it (its channel's outputs within about 8*256 + k samples),
 * since the contraction multiplies it by zero taps too; the CUDA-core forms
 * affect only the outputs whose k-tap support contains it. */
typedef enum scir_precision {
    SCIR_PREC_AUTO = -1,
    SCIR_PREC_REF_EXACT = 0,
    SCIR_PREC_FP32 = 1,
    SCIR_PREC_BF16X3 = 2,
    SCIR_PREC_BF16X6 = 3,
    SCIR_PREC_FP16X3 = 4
} scir_precision;

/* Arithmetic of the second-order-section recursion.
 * SCIR_SOS_FP64_EXACT: FP64 coefficients and state, the reference DF2T
 *   operation order without FMA (crates/scir-iir-filters/src/filter.rs:
 *   50-61): bit-identical to the reference for f64 data.
 * SCIR_SOS_FP64: FP64 coefficients and state with FMA.
 * SCIR_SOS_FP32: coefficients rounded to FP32, FP32 state (DF2T).
 * SCIR_SOS_FP32_COUPLED: FP32 state, each complex-pole section in coupled
 *   (modal) form driven by increments whose coefficients (sigma-1, omega)
 *   were computed in FP64, so poles near the unit circle are not moved by
 *   FP32 rounding; real-pole sections run FP32 DF2T.  States in and out are
 *   DF2T states, as in every other mode. */
typedef enum scir_sos_precision {
    SCIR_SOS_FP64_EXACT = 0,
    SCIR_SOS_FP64 = 1,
    SCIR_SOS_FP32 = 2,
    SCIR_SOS_FP32_COUPLED = 3
} scir_sos_precision;

/* Edge extension for sosfiltfilt (SciPy padtype). */
typedef enum scir_padtype {
    SCIR_PAD_NONE = 0, /* reference filtfilt: no padding, zero state       */
    SCIR_PAD_ODD = 1   /* SciPy default: odd extension + sosfilt_zi state  */
} scir_padtype;

/* ----------------------------------------------------------------------- */
/* Library / device layer                                                  */
/* Replaces the per-call context and module load of the reference's CUDA   */
/* path (crates/scir-gpu/src/lib.rs:589-622, 814-834): kernels are compiled */
/* ahead of time for sm_103a and the primary context of the current device */
/* is used for every call.                                                  */
/* ----------------------------------------------------------------------- */

SCIR_API int scir_abi_version(void);
SCIR_API const char* scir_status_string(int status);
/* Copies the calling thread's last error message (NUL-terminated). */
SCIR_API int scir_last_error(char* buf, size_t len);
/* Initialises per-device state for `device` (SM count, device error word,
 * scratch pool) and makes it current.  Optional: every entry point
 * initialises the current device on first use, but a CUDA-graph capture
 * needs it done before the capture begins.
 * Replaces cuda_available() / CudaCtx::create_default
 * (crates/scir-gpu/src/lib.rs:596-616). */
SCIR_API int scir_init(int device);
SCIR_API int scir_device_count(int* count);
/* Reads and clears the current device's error word: non-zero when a kernel's
 * bounded device-side wait gave up (1) or a kernel rejected its geometry (2)
 * since the last call.  Synchronises with the device.  The reference has no
 * device-side failure reporting (its CUDA path cannot run at all). */
SCIR_API int scir_device_errors(unsigned* code);
/* Measured FMA throughput of the current device's CUDA cores in TFLOP/s
 * (fp64 = 0: FP32 FFMA, 1: FP64 DFMA): independent FMA chains at full
 * occupancy, timed with CUDA events (synchronous, ~0.3 s).  The roofline
 * denominator of FP32- and FP64-pipe-bound kernels.  No reference
 * counterpart. */
SCIR_API int scir_probe_fma_peak(int fp64, double* tflops);
/* Self-test of the bounded-wait failure path on the current device (no
 * reference counterpart: the reference has no device-side failure
 * reporting).  A two-warp pipeline copies n_chunks chunks of 1,024 floats
 * from `in` (device, 16-byte aligned) through a 4-stage shared-memory ring
 * with cp.async.bulk / mbarriers and writes each chunk's sum to out[chunk].
 * The producer issues only the first issue_chunks (<= n_chunks) chunks; if
 * that is fewer, the consumer's wait for the next chunk gives up after
 * wait_limit_cycles SM cycles (1e3 .. 4e9) and the kernel records
 * SCIR_ERR_TIMEOUT's device code (1) in the device error word, as every
 * TMA pipeline of the library does, and returns with no copy in flight;
 * scir_device_errors() then reports it.  Asynchronous on `stream`. */
SCIR_API int scir_selftest_pipeline(const float* in, int64_t n_chunks, int64_t issue_chunks,
                                    long long wait_limit_cycles, float* out, void* stream);
/* Scratch memory (split operands of the tensor-core FIR, filtfilt edge
 * extensions) comes from a per-device stream-ordered pool that keeps freed
 * memory for the next call.  This synchronises the current device and
 * returns the pool's unused memory.  No reference counterpart (the reference
 * allocates and frees device buffers on every call). */
SCIR_API int scir_release_scratch(void);
/* Bytes the current device's scratch pool holds (reserved) and hands out
 * (used) right now; both 0 before the first call that needed scratch.  Does
 * not create the pool.  No reference counterpart. */
SCIR_API int scir_scratch_usage(uint64_t* reserved, uint64_t* used);

/* ----------------------------------------------------------------------- */
/* Batched FIR (device pointers, stream-ordered)                           */
/* Replaces cuda::fir1d_batched_f32_cuda and its PTX kernel                */
/* (crates/scir-gpu/src/lib.rs:1036-1113, 727-811).                        */
/* ----------------------------------------------------------------------- */

/* Output length of `mode` for n samples and k taps (-1 if invalid). */
SCIR_API int64_t scir_fir_out_len(int64_t n, int64_t k, int mode);

/* x: batch rows of n samples, row stride ld_x >= n; taps: k values;
 * y: batch rows of scir_fir_out_len(n, k, mode) samples, stride ld_y. */
SCIR_API int scir_fir_batched_f32(const float* x, int64_t ld_x, int64_t batch,
                                  int64_t n, const float* taps, int64_t k,
                                  int mode, int precision, float* y,
                                  int64_t ld_y, void* stream);

/* ----------------------------------------------------------------------- */
/* Ragged batched FIR: signals of different lengths and tap counts in one  */
/* persistent launch.  No reference counterpart exists (the reference API  */
/* takes one shared tap vector, crates/scir-gpu/src/lib.rs:1134); this is  */
/* the ragged extension of fir1d_batched_f32.                               */
/* ----------------------------------------------------------------------- */

typedef struct scir_ragged_desc {
    int64_t x_off;    /* first input sample of the signal in x            */
    int64_t n;        /* input samples                                    */
    int64_t taps_off; /* first tap of the signal in taps                  */
    int64_t k;        /* taps                                             */
    int64_t y_off;    /* first output sample in y (scir_fir_out_len long) */
} scir_ragged_desc;

typedef struct scir_ragged_plan scir_ragged_plan;

/* Builds a launch plan from a HOST descriptor table: validates every entry,
 * splits signals into work tiles, orders them longest-first and uploads the
 * tile table to the device.  Precision: SCIR_PREC_FP32 / REF_EXACT run every
 * signal on the CUDA cores; SCIR_PREC_AUTO (or FP16X3, BF16X6, BF16X3) sends
 * the signals with at least 512 taps (autotunable) and 16,384 outputs to the
 * tensor cores (split-operand contraction; AUTO: FP16X3) in a second
 * persistent launch, the rest to the CUDA cores in FP32. */
SCIR_API int scir_ragged_plan_create(const scir_ragged_desc* desc, int64_t count,
                                     int mode, int precision,
                                     scir_ragged_plan** plan);
SCIR_API int scir_ragged_plan_destroy(scir_ragged_plan* plan);
/* Number of tiles and algorithmic multiply-adds of the plan. */
SCIR_API int scir_ragged_plan_stats(const scir_ragged_plan* plan,
                                    int64_t* tiles, double* macs,
                                    int64_t* samples_in);
/* The tensor-core bucket of a plan: its tap threshold (0: none) and how
 * many signals it holds. */
SCIR_API int scir_ragged_plan_tensor_cores(const scir_ragged_plan* plan, int* min_taps,
                                           int64_t* signals);
/* One persistent launch over every CUDA-core tile of the plan, preceded by
 * the tensor-core bucket's max pass (FP16X3), operand split and persistent
 * launch when the plan has one (graph-capturable: no allocation, no host
 * synchronisation). */
SCIR_API int scir_fir_ragged_f32(const scir_ragged_plan* plan, const float* x,
                                 const float* taps, float* y, void* stream);

/* ----------------------------------------------------------------------- */
/* Polyphase upfirdn / resample_poly (device pointers, stream-ordered)     */
/* Replaces scir_signal::resample_poly (crates/scir-signal/src/lib.rs:     */
/* 313-362), generalised to any rates as scipy.signal.upfirdn /           */
/* resample_poly.                                                          */
/* ----------------------------------------------------------------------- */

/* scipy.signal.upfirdn output length: ceil(((n-1)*up + kh) / down). */
SCIR_API int64_t scir_upfirdn_out_len(int64_t kh, int64_t n, int up, int down);
/* y[m] = sum_j h[j] * u[m*down - j], u = x zero-stuffed by up. */
SCIR_API int scir_upfirdn_f32(const float* x, int64_t ld_x, int64_t batch,
                              int64_t n, const float* h, int64_t kh, int up,
                              int down, int precision, float* y, int64_t ld_y,
                              void* stream);

/* resample_poly output length: ceil(n*up/down) after gcd reduction. */
SCIR_API int64_t scir_resample_poly_out_len(int64_t n, int up, int down);

/* Default anti-aliasing design for resample_poly, computed on the host in
 * FP64 and already multiplied by the reduced `up`:
 *   design 0 (SciPy): firwin(2*10*max(up,down)+1, 1/max, ('kaiser', 5.0));
 *   design 1 (reference): the reference's baked 31-value 2/3 table, the
 *   same doubles bit for bit (crates/scir-signal/src/lib.rs:315-347); only
 *   up/down = 2/3 (after reduction) is accepted.
 * Writes at most `cap` taps to h (host) and the count to *kh. */
SCIR_API int scir_resample_poly_default_taps(int up, int down, int design,
                                             double* h, int64_t cap,
                                             int64_t* kh);

/* resample_poly with zero-padded edges: after gcd reduction of up/down,
 * y[m] = sum_j h[j] * u[(kh-1)/2 + m*down - j] for m < ceil(n*up/down).
 * h (device, kh taps) must already include the gain `up`; h == NULL selects
 * scir_resample_poly_default_taps(design 0).  up == down: y = x. */
SCIR_API int scir_resample_poly_f32(const float* x, int64_t ld_x, int64_t batch,
                                    int64_t n, int up, int down, const float* h,
                                    int64_t kh, int precision, float* y,
                                    int64_t ld_y, void* stream);

/* ----------------------------------------------------------------------- */
/* DeviceArray operations (device pointers, stream-ordered).  Replace the  */
/* reference's CUDA elementwise kernels add_vec_f32 / add_scalar_f32 /      */
/* mul_scalar_f32 (crates/scir-gpu/src/lib.rs:629-725) and its CPU-only     */
/* resize2d_f32 (lib.rs:394-441).  Results equal the reference's CPU values */
/* bit for bit.                                                             */
/* ----------------------------------------------------------------------- */
enum scir_resize_mode { SCIR_RESIZE_NEAREST = 0, SCIR_RESIZE_BILINEAR = 1 };
SCIR_API int scir_add_vec_f32(const float* a, const float* b, float* out, int64_t n,
                              void* stream);
SCIR_API int scir_add_scalar_f32(const float* a, float alpha, float* out, int64_t n,
                                 void* stream);
SCIR_API int scir_mul_scalar_f32(const float* a, float alpha, float* out, int64_t n,
                                 void* stream);
/* [src_h][src_w] -> [out_h][out_w], half-pixel centres (align_corners = false). */
SCIR_API int scir_resize2d_f32(const float* src, int64_t src_h, int64_t src_w, float* dst,
                               int64_t out_h, int64_t out_w, int mode, void* stream);

/* ----------------------------------------------------------------------- */
/* CUDA-graph capture of library calls (device layer).  No reference       */
/* counterpart.  Everything the library enqueues on `stream` between begin  */
/* and end is recorded and replays with one launch.  Before capturing, call */
/* scir_init() and make one call of each operation with the same shapes     */
/* (per-device state and default taps are created on first use).  The       */
/* capture is thread-local (cudaStreamCaptureModeThreadLocal); the stream   */
/* must not be the legacy default stream.                                   */
/* ----------------------------------------------------------------------- */
typedef struct scir_graph scir_graph;
SCIR_API int scir_graph_capture_begin(void* stream);
SCIR_API int scir_graph_capture_end(void* stream, scir_graph** graph);
SCIR_API int scir_graph_launch(const scir_graph* graph, void* stream);
SCIR_API int scir_graph_destroy(scir_graph* graph);

/* ----------------------------------------------------------------------- */
/* Autotuning.  No reference counterpart (the reference has one kernel     */
/* shape).  Each call times the kernel variants the dispatch can run for    */
/* one problem shape on synthetic data of that shape (buffers from the      */
/* library's scratch pool, a private stream, synchronised) and records the  */
/* fastest for the current device model; later calls with exactly that     */
/* shape use it.  A shape whose inputs and outputs fit in L2 is timed one   */
/* call at a time after a write of twice the L2 size, as it runs on data    */
/* that was just copied in or produced elsewhere (that write needs 2 x L2   */
/* bytes of scratch).  `choice` receives a short description.               */
/* ----------------------------------------------------------------------- */

/* Batched FIR: CUDA-core tiles of 8 or 16 outputs per thread, and for
 * SCIR_PREC_AUTO also the tensor-core FP16X3 form.  precision must be
 * REF_EXACT, FP32 or AUTO (the split-operand modes have one form). */
SCIR_API int scir_autotune_fir(int64_t batch, int64_t n, int64_t k, int mode,
                               int precision, double* best_ms, char* choice,
                               size_t choice_len);
/* resample_poly (kh <= 0: the default design's length): outputs per lane
 * and channels per work item (1, 2 or 4) of the streaming kernel. */
SCIR_API int scir_autotune_resample_poly(int64_t batch, int64_t n, int up,
                                         int down, int64_t kh, double* best_ms,
                                         char* choice, size_t choice_len);
/* Ragged plan: the tap count from which CUDA-core tiles use 16 outputs per
 * thread and, for plans with a tensor-core bucket, the tap count from which
 * signals go to the tensor cores, timed on the caller's buffers; the plan is
 * rebuilt with the fastest (the stream is synchronised first). */
SCIR_API int scir_ragged_plan_autotune(scir_ragged_plan* plan, const float* x,
                                       const float* taps, float* y, void* stream,
                                       int* v16_min_taps, double* best_ms);
/* Forgets every recorded choice. */
SCIR_API int scir_autotune_clear(void);
/* Writes / merges the recorded choices as text (one line per shape). */
SCIR_API int scir_autotune_save(const char* path);
SCIR_API int scir_autotune_load(const char* path);

/* ----------------------------------------------------------------------- */
/* General IIR (device pointers, stream-ordered).  scipy.signal.lfilter     */
/* semantics: transposed direct form II over the whole polynomial, b and a  */
/* divided by a[0], max(na, nb) - 1 <= 32 state values per channel, FP64    */
/* state and arithmetic.  zi / zf: [batch][max(na, nb) - 1] f64 or NULL.     */
/* The reference has no general IIR filter (SciPy is the oracle).           */
/* ----------------------------------------------------------------------- */
SCIR_API int scir_lfilter_f32(const float* x, int64_t ld_x, int64_t batch,
                              int64_t n, const double* b, int nb,
                              const double* a, int na, const double* zi,
                              double* zf, float* y, int64_t ld_y, void* stream);
SCIR_API int scir_lfilter_f64(const double* x, int64_t ld_x, int64_t batch,
                              int64_t n, const double* b, int nb,
                              const double* a, int na, const double* zi,
                              double* zf, double* y, int64_t ld_y, void* stream);
/* scipy.signal.lfilter_zi (host): max(na, nb) - 1 values into zi. */
SCIR_API int scir_lfilter_zi(const double* b, int nb, const double* a, int na,
                             double* zi);

/* ----------------------------------------------------------------------- */
/* IIR design (host, FP64, no device).  Replaces the reference's butter /   */
/* cheby1 / bessel_with_norm -> iirfilter (crates/scir-iir-filters/src/     */
/* filter_design.rs:128-314) and zpk2sos (crates/scir-iir-filters/src/      */
/* sos.rs:154-357), SciPy semantics.  wn holds one edge (low/high-pass) or  */
/* two increasing edges (band-pass/stop) in the units of fs; fs <= 0 means  */
/* the edges are already normalised to Nyquist = 1.  rp (dB, > 0) is read   */
/* for Chebyshev I only.  Bessel orders 1..25 (the reference's range),      */
/* others 0..256.  Complex values are interleaved (re, im) pairs.           */
/* ----------------------------------------------------------------------- */
enum scir_iir_family {
    SCIR_IIR_BUTTER = 0,
    SCIR_IIR_CHEBY1 = 1,
    SCIR_IIR_BESSEL_PHASE = 2, /* BesselNorm::Phase (SciPy's default) */
    SCIR_IIR_BESSEL_DELAY = 3, /* BesselNorm::Delay                   */
    SCIR_IIR_BESSEL_MAG = 4    /* BesselNorm::Mag                     */
};
enum scir_band_type {
    SCIR_BAND_LOWPASS = 0,
    SCIR_BAND_HIGHPASS = 1,
    SCIR_BAND_BANDPASS = 2,
    SCIR_BAND_BANDSTOP = 3
};
/* SosPairing (crates/scir-iir-filters/src/sos.rs:22-35). */
enum scir_sos_pairing {
    SCIR_PAIR_NEAREST = 0,
    SCIR_PAIR_KEEP_ODD = 1,
    SCIR_PAIR_MINIMAL = 2
};
/* Digital zeros, poles and gain.  *nz, *np and *k are always written; z
 * and p ([cap][2] each) only when both are non-NULL (cap >= *nz, *np). */
SCIR_API int scir_iirfilter_zpk(int order, int family, int btype,
                                const double* wn, double rp, double fs,
                                double* z, double* p, int cap, int* nz,
                                int* np, double* k);
/* Sections [nsec][6] (b0 b1 b2 a0 a1 a2) of a zpk system; *nsec is always
 * written, sos only when non-NULL (cap >= *nsec). */
SCIR_API int scir_zpk2sos(const double* z, int nz, const double* p, int np,
                          double k, int pairing, double* sos, int cap,
                          int* nsec);
/* iirfilter(..., output='sos'): scir_iirfilter_zpk then scir_zpk2sos with
 * nearest pairing; ceil(order / 2) sections (order for band filters). */
SCIR_API int scir_iirfilter_sos(int order, int family, int btype,
                                const double* wn, double rp, double fs,
                                double* sos, int cap, int* nsec);

/* FIR design (host, FP64): scipy.signal.firwin(numtaps, cutoff, window,
 * pass_zero, scale, fs) for 1..64 increasing band edges (in the units of fs;
 * fs <= 0: normalised to Nyquist = 1).  The reference bakes its one design
 * as a table (crates/scir-signal/src/lib.rs:315-347); this gives the Rust/C
 * callers the taps of every configuration without SciPy.  beta is read for
 * SCIR_WIN_KAISER only.  A pass band at Nyquist needs odd numtaps. */
enum scir_window {
    SCIR_WIN_HAMMING = 0,
    SCIR_WIN_KAISER = 1,
    SCIR_WIN_HANN = 2,
    SCIR_WIN_BLACKMAN = 3,
    SCIR_WIN_BOXCAR = 4
};
SCIR_API int scir_firwin(int64_t numtaps, const double* cutoff, int ncut,
                         int window, double beta, int pass_zero, int scale,
                         double fs, double* h);

/* ----------------------------------------------------------------------- */
/* Second-order sections (device pointers, stream-ordered)                 */
/* Replaces scir_signal::sosfilt / filtfilt (crates/scir-signal/src/lib.rs:*/
/* 260-291) over DirectForm2Transposed (crates/scir-iir-filters/src/       */
/* filter.rs:50-61).  sos is [nsec][6] = b0 b1 b2 a0 a1 a2, the layout of  */
/* #[repr(C)] SosCoeffs (crates/scir-iir-filters/src/sos.rs:49-66); a0 is  */
/* taken as 1 and not read, as in the reference.                            */
/* ----------------------------------------------------------------------- */

#define SCIR_SOS_MAX_SECTIONS 32

/* x, y: batch rows of n samples (f32, or f64 for the _f64 variant);
 * sos: HOST pointer, [nsec][6] f64 (copied into kernel parameters);
 * zi: optional DEVICE [batch][nsec][2] f64 initial DF2T state (s1, s2);
 * zf: optional DEVICE [batch][nsec][2] f64 final state. */
SCIR_API int scir_sosfilt_f32(const float* x, int64_t ld_x, int64_t batch,
                              int64_t n, const double* sos, int nsec,
                              const double* zi, double* zf, int precision,
                              float* y, int64_t ld_y, void* stream);
SCIR_API int scir_sosfilt_f64(const double* x, int64_t ld_x, int64_t batch,
                              int64_t n, const double* sos, int nsec,
                              const double* zi, double* zf, int precision,
                              double* y, int64_t ld_y, void* stream);

/* SciPy sosfilt_zi for a HOST sos: zi[nsec][2] (host). */
SCIR_API int scir_sosfilt_zi(const double* sos, int nsec, double* zi);
/* SciPy's default filtfilt edge: 3*(2*nsec+1 - min(#b2==0, #a2==0)). */
SCIR_API int64_t scir_sosfiltfilt_default_padlen(const double* sos, int nsec);

/* Forward-backward filtering.  SCIR_PAD_NONE is the reference filtfilt
 * (zero state both ways, crates/scir-signal/src/lib.rs:278-291);
 * SCIR_PAD_ODD is scipy.signal.sosfiltfilt (odd extension of padlen samples
 * each side, padlen < 0 = default, initial states sosfilt_zi * edge value).
 * y may alias x. */
SCIR_API int scir_sosfiltfilt_f32(const float* x, int64_t ld_x, int64_t batch,
                                  int64_t n, const double* sos, int nsec,
                                  int padtype, int64_t padlen, int precision,
                                  float* y, int64_t ld_y, void* stream);
SCIR_API int scir_sosfiltfilt_f64(const double* x, int64_t ld_x, int64_t batch,
                                  int64_t n, const double* sos, int nsec,
                                  int padtype, int64_t padlen, int precision,
                                  double* y, int64_t ld_y, void* stream);

/* scir_sosfiltfilt_f32 without any device allocation, for callers that may
 * not allocate device memory while they filter: a real-time frame loop (an
 * allocation can synchronise the device or stall behind other work and miss
 * the frame), a process whose device memory is reserved up front by another
 * pool, or an FFI host that forbids hidden allocations.  It has no
 * counterpart in the reference.  The edge-extension scratch comes from a
 * fixed file-scope device array of 4 Mi floats (16 MiB, held on every device
 * that loads the library until the process exits); batch * padlen above that
 * is rejected with SCIR_ERR_SHAPE.  The first call on a device looks up the
 * addresses of the array and of the library's device error word (also a
 * file-scope device variable), so make it before any stream capture.  No
 * precision or padtype allocates.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Arguments and results are those of scir_sosfiltfilt_f32. */
SCIR_API int scir_sosfiltfilt_f32_noalloc(const float* x, int64_t ld_x, int64_t batch,
                                          int64_t n, const double* sos, int nsec,
                                          int padtype, int64_t padlen, int precision,
                                          float* y, int64_t ld_y, void* stream);

/* ----------------------------------------------------------------------- */
/* Host-buffer entry points with the reference's signatures (synchronous). */
/* ----------------------------------------------------------------------- */

/* crates/scir-gpu/src/lib.rs:1036 fir1d_batched_f32_cuda(x: &Array2<f32>,
 * taps: &Array1<f32>) -> Result<Array2<f32>, GpuError>; x is b x n
 * row-major, y (b x n) is caller-allocated.  Uses SCIR_PREC_REF_EXACT, so
 * y is bit-identical to scir_gpu::fir1d_batched_f32 (lib.rs:1134). */
SCIR_API int scir_fir1d_batched_f32_cuda(const float* x, size_t b, size_t n,
                                         const float* taps, size_t k, float* y);

/* Generalised host-buffer FIR (any mode/precision), chunked over rows and
 * pipelined H2D / kernel / D2H on library streams. */
SCIR_API int scir_fir_batched_f32_host(const float* x, int64_t batch, int64_t n,
                                       const float* taps, int64_t k, int mode,
                                       int precision, float* y);

/* crates/scir-signal/src/lib.rs:260 sosfilt(sos: &Sos, x: &Array1<f64>)
 * -> Array1<f64>; batch rows allowed.  Uses SCIR_SOS_FP64_EXACT. */
SCIR_API int scir_sosfilt_f64_host(const double* sos, int nsec, const double* x,
                                   size_t batch, size_t n, double* y);
/* crates/scir-signal/src/lib.rs:278 filtfilt(sos, x) (no padding). */
SCIR_API int scir_filtfilt_f64_host(const double* sos, int nsec, const double* x,
                                    size_t batch, size_t n, double* y);
/* crates/scir-signal/src/lib.rs:313 resample_poly(x, up, down) with the
 * reference's design (only 2/3 accepted, as the reference asserts); y holds
 * scir_resample_poly_out_len(n, 2, 3) values per row. */
SCIR_API int scir_resample_poly_f64_host(const double* x, size_t batch,
                                         size_t n, size_t up, size_t down,
                                         double* y);
/* Host-buffer resample_poly on f32 rows with the SciPy design (h == NULL)
 * or explicit host taps, pipelined like scir_fir_batched_f32_host. */
SCIR_API int scir_resample_poly_f32_host(const float* x, int64_t batch,
                                         int64_t n, int up, int down,
                                         const float* h, int64_t kh,
                                         int precision, float* y);

/* How the host-buffer entry points cut a call of `rows` rows (in_row bytes
 * per row in, out_row out) into pipelined chunks: *count receives the number
 * of chunks and the first min(cap, *count) row counts go to sizes.  quantum
 * is the row multiple a chunk is rounded up to (128 for host FIR calls of
 * >= 512 taps whose precision may use the tensor cores, else 1).  Chunks
 * hold about a sixth of the call's bytes within 4 .. 64 MB; with three or
 * more, the first and the last hold half as many rows.  Host arithmetic
 * only: no device is touched. */
SCIR_API int scir_host_chunk_plan(int64_t rows, size_t in_row, size_t out_row, int64_t quantum,
                                  int64_t* sizes, int64_t cap, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* SCIR_GB300_H */
