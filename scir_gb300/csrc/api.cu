// C-ABI entry points: argument validation, precision dispatch and the
// host-buffer layer that keeps the reference's function signatures.
//
// Reference behaviour mirrored here:
//  - fir1d_batched_f32_cuda (crates/scir-gpu/src/lib.rs:1036-1113) copies the
//    host rows to the device, filters, copies back and reports failures as
//    GpuError; it never changes the output shape (b x n).  It creates a CUDA
//    context and loads a module per call; this layer keeps per-device
//    streams and staging buffers alive instead and pipelines row chunks
//    (copy in / filter / copy out on their own streams ordered by events,
//    four chunks in flight).
//  - sosfilt / filtfilt (crates/scir-signal/src/lib.rs:260-291) take f64 and
//    start from a zero state; their host entry points use the exact FP64
//    kernels.
//  - resample_poly (crates/scir-signal/src/lib.rs:313-362) accepts only
//    up=2/down=3 and uses a baked 31-value table; its host entry point keeps
//    that restriction and those doubles, computed in FP64 with the
//    reference's summation order.
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace scir {

int fir_geometry(int64_t n, int64_t k, int mode, int* reverse, int64_t* s, int64_t* n_out) {
    switch (mode) {
    case SCIR_FIR_REF_CORR: *reverse = 0; *s = -(k - 1); *n_out = n; break;
    case SCIR_FIR_LFILTER: *reverse = 1; *s = -(k - 1); *n_out = n; break;
    case SCIR_FIR_FULL: *reverse = 1; *s = -(k - 1); *n_out = n + k - 1; break;
    case SCIR_FIR_VALID:
        if (n < k) return set_error(SCIR_ERR_SHAPE, "VALID needs n >= k (n=%lld, k=%lld)",
                                    (long long)n, (long long)k);
        *reverse = 1; *s = 0; *n_out = n - k + 1; break;
    default: return set_error(SCIR_ERR_INVALID_ARG, "unknown FIR mode %d", mode);
    }
    return SCIR_OK;
}

namespace {

// ---------------------------------------------------------------- f64 polyphase
// Exact FP64 polyphase resample for the reference's f64 signature: products
// and sums rounded separately, contributions added from the oldest input
// sample to the newest, as the reference's full convolution does.
__global__ void __launch_bounds__(256)
poly_exact_f64_kernel(const double* __restrict__ x, int64_t n, const double* __restrict__ h,
                      int64_t kh, int up, int down, int64_t off, double* __restrict__ y,
                      int64_t n_out, int64_t blocks_per_row) {
    const int64_t row = blockIdx.x / blocks_per_row;
    const int64_t m = (blockIdx.x % blocks_per_row) * 256 + threadIdx.x;
    if (m >= n_out) return;
    const double* __restrict__ xr = x + row * n;
    const int64_t t = m * down + off;
    const int64_t ph = t % up, base = t / up;
    const int64_t q_hi = ph < kh ? (kh - 1 - ph) / up : -1;  // largest q with ph + q*up < kh
    double acc = 0.0;
    for (int64_t q = q_hi; q >= 0; --q) {
        const int64_t xi = base - q;
        if (xi < 0 || xi >= n) continue;
        acc = __dadd_rn(acc, __dmul_rn(xr[xi], h[ph + q * up]));
    }
    y[row * n_out + m] = acc;
}

__global__ void fill_zero_rows(float* y, int64_t ld, int64_t batch, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < batch * n) y[(i / n) * ld + (i % n)] = 0.0f;
}

// ---------------------------------------------------------------- default taps
struct TapKey {
    int dev, up, down, design;
    bool operator<(const TapKey& o) const {
        return std::tie(dev, up, down, design) < std::tie(o.dev, o.up, o.down, o.design);
    }
};
struct TapBuf {
    float* d32 = nullptr;
    double* d64 = nullptr;
    int64_t kh = 0;
};
std::mutex g_tap_mutex;
std::map<TapKey, TapBuf> g_taps;

// The reference's baked resample_poly(2, 3) filter, gain 2 included
// (crates/scir-signal/src/lib.rs:315-347).  The values are the reference's
// decimal literals, which C and Rust both round to the nearest double, so
// the taps -- and every output of the exact FP64 path -- are the reference's
// bit for bit.  (A firwin(31, 1/3, 'hamming') * 2 design agrees only to
// ~1e-16 and changes the last bit of most outputs.)
constexpr double kRefResample23[31] = {
    2.074505559623708e-18,  3.538600036880219e-3,   5.068355234374961e-3,
    -4.352628574659906e-18, -1.161274884414711e-2,  -1.705404264360788e-2,
    1.031683205857806e-17,  3.382730607794791e-2,   4.62174845519145e-2,
    -1.768899299634197e-17, -8.47200828101812e-2,   -1.166001508003416e-1,
    2.365319648026013e-17,  2.641261112200551e-1,   5.446004399706618e-1,
    6.652174560128868e-1,   5.446004399706618e-1,   2.641261112200551e-1,
    2.365319648026013e-17,  -1.166001508003416e-1,  -8.472008281018122e-2,
    -1.768899299634197e-17, 4.621748455191452e-2,   3.382730607794793e-2,
    1.031683205857806e-17,  -1.70540426436079e-2,   -1.161274884414712e-2,
    -4.352628574659906e-18, 5.068355234374964e-3,   3.538600036880219e-3,
    2.074505559623708e-18};

int default_taps_host(int up, int down, int design, std::vector<double>& h) {
    const int64_t g = gcd64(up, down);
    up = (int)(up / g);
    down = (int)(down / g);
    if (design == 1) {
        if (up != 2 || down != 3)
            return set_error(SCIR_ERR_UNSUPPORTED,
                             "the reference resample_poly design exists only for up=2, down=3");
        h.assign(kRefResample23, kRefResample23 + 31);
        return SCIR_OK;  // the table already carries the gain
    } else if (design == 0) {
        const int mr = up > down ? up : down;
        const int64_t nt = 2 * 10 * (int64_t)mr + 1;
        h.resize((size_t)nt);
        firwin_lowpass(nt, 1.0 / mr, 1, 5.0, h.data());
    } else {
        return set_error(SCIR_ERR_INVALID_ARG, "unknown resample design %d", design);
    }
    for (double& v : h) v *= up;
    return SCIR_OK;
}

int cached_default_taps(int up, int down, int design, TapBuf* out) {
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    const TapKey key{dev, up, down, design};
    std::lock_guard<std::mutex> lk(g_tap_mutex);
    auto it = g_taps.find(key);
    if (it != g_taps.end()) {
        *out = it->second;
        return SCIR_OK;
    }
    std::vector<double> h;
    int rc = default_taps_host(up, down, design, h);
    if (rc) return rc;
    std::vector<float> hf(h.begin(), h.end());
    TapBuf b;
    b.kh = (int64_t)h.size();
    SCIR_CUDA_TRY(cudaMalloc(&b.d32, hf.size() * sizeof(float)));
    SCIR_CUDA_TRY(cudaMalloc(&b.d64, h.size() * sizeof(double)));
    rc = upload_sync(b.d32, hf.data(), hf.size() * sizeof(float));
    if (rc) return rc;
    rc = upload_sync(b.d64, h.data(), h.size() * sizeof(double));
    if (rc) return rc;
    g_taps[key] = b;
    *out = b;
    return SCIR_OK;
}

int fill_sos(const double* sos, int nsec, bool want_zi, SosCoef* c) {
    SCIR_REQUIRE(sos != nullptr, SCIR_ERR_INVALID_ARG, "sos is NULL");
    SCIR_REQUIRE(nsec >= 1 && nsec <= SCIR_SOS_MAX_SECTIONS, SCIR_ERR_INVALID_ARG,
                 "nsec %d not in [1, %d]", nsec, SCIR_SOS_MAX_SECTIONS);
    if (build_sos_coef(sos, nsec, want_zi, c) != SCIR_OK)
        return set_error(SCIR_ERR_INVALID_ARG, "sosfilt_zi: a section has a pole at z=1 or a0=0");
    return SCIR_OK;
}

// ---------------------------------------------------------------- staging pool
// Per-device streams and grow-only device buffers for the host-buffer layer.
// One stream per copy direction and one kernel stream per buffer carry the
// stages of a row chunk (copy in, filter, copy out), and events order them,
// so the two copy directions and the kernels overlap across kBufs chunks in
// flight: a chunk's upload waits only for the kernel that last read its
// input buffer, its kernel for its upload and for the download that last
// read its output buffer.  Chunks' kernels may run concurrently (a chunk of
// few rows does not fill the GPU).
struct Stager {
    static constexpr int kBufs = 4;              // chunks in flight
    static constexpr int kStreams = 2 + kBufs;   // copy in, copy out, kernels
    std::mutex mu;
    bool ready = false;
    cudaStream_t st[kStreams] = {};
    cudaEvent_t ev_in[kBufs] = {}, ev_k[kBufs] = {}, ev_out[kBufs] = {};
    void* din[kBufs] = {};
    void* dout[kBufs] = {};
    size_t cap_in[kBufs] = {}, cap_out[kBufs] = {};
    void* dtaps = nullptr;
    size_t cap_taps = 0;
};
Stager g_stager[64];

int stager_get(Stager** out) {
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    Stager* s = &g_stager[info->device];
    *out = s;
    return SCIR_OK;
}

int ensure(void** p, size_t* cap, size_t bytes) {
    if (*cap >= bytes) return SCIR_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SCIR_ERR_OOM, "staging allocation of %zu bytes failed: %s", bytes,
                         cudaGetErrorString(e));
    }
    *cap = bytes;
    return SCIR_OK;
}

int stager_init(Stager* s) {
    if (s->ready) return SCIR_OK;
    for (int i = 0; i < Stager::kStreams; ++i)
        SCIR_CUDA_TRY(cudaStreamCreateWithFlags(&s->st[i], cudaStreamNonBlocking));
    for (int i = 0; i < Stager::kBufs; ++i) {
        SCIR_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_in[i], cudaEventDisableTiming));
        SCIR_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_k[i], cudaEventDisableTiming));
        SCIR_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_out[i], cudaEventDisableTiming));
    }
    s->ready = true;
    return SCIR_OK;
}

// The row counts of the chunks a call of `rows` rows (>= 1) is cut into, and
// the largest of them (the staging buffers' row capacity).  Chunks hold a
// sixth of the call's bytes, kept within 4 .. 64 MB (small calls still
// overlap their uploads, kernels and downloads); `quantum` rounds the rows of
// a chunk up to a multiple that fills the body's kernels (the tensor-core FIR
// tiles 128 channels) while a chunk stays within 512 MB.  With three or more
// chunks the first and the last hold half as many rows: the pipeline's first
// upload and last download run alone, so shorter ones shorten the whole call.
std::vector<int64_t> chunk_plan(int64_t rows, size_t in_row, size_t out_row, int64_t quantum,
                                int64_t* max_rows) {
    const size_t row_bytes = in_row + out_row + 1;
    const size_t cap = 512ull << 20;
    const size_t target = std::min<size_t>(64ull << 20,
                                           std::max<size_t>(4ull << 20, (size_t)rows * row_bytes / 6));
    int64_t cr = (int64_t)(target / row_bytes);
    if (cr < 1) cr = 1;
    if (quantum > 1) {
        const int64_t cq = (cr + quantum - 1) / quantum * quantum;
        if ((size_t)cq * row_bytes <= cap) cr = cq;
    }
    if (cr > rows) cr = rows;
    // chunk row counts: cr each, or (with three or more) a half chunk first
    // and last
    std::vector<int64_t> sizes;
    if (rows > 2 * cr && cr >= 2) {
        const int64_t h = cr / 2;
        int64_t left = rows - h;
        sizes.push_back(h);
        while (left > cr + h) {
            sizes.push_back(cr);
            left -= cr;
        }
        if (left > h) sizes.push_back(left - h);
        sizes.push_back(std::min(left, h));
    } else {
        for (int64_t r = 0; r < rows; r += cr) sizes.push_back(std::min(cr, rows - r));
    }
    *max_rows = cr;
    return sizes;
}

// Runs `body(chunk_rows, in_dev, out_dev, stream)` over the chunks of
// chunk_plan with the copies around it: a chunk's rows of `hin` (row bytes
// in_row) go to in_dev, out_dev (row bytes out_row) comes back into `hout`.
template <typename Body>
int pipeline_rows(Stager* s, const void* hin, size_t in_row, void* hout, size_t out_row,
                  int64_t rows, Body body, int64_t quantum = 1) {
    int64_t cr = 0;
    const std::vector<int64_t> sizes = chunk_plan(rows, in_row, out_row, quantum, &cr);
    // every exit, the error ones included, waits for the work in flight: the
    // copies read and write the caller's host arrays (and the tap upload that
    // stage_taps queued on the upload stream reads the caller's taps)
    struct Drain {
        Stager* s;
        ~Drain() {
            for (int j = 0; j < Stager::kStreams; ++j) cudaStreamSynchronize(s->st[j]);
        }
    } drain{s};
    const int64_t nchunks = (int64_t)sizes.size();
    const int used = (int)(nchunks < Stager::kBufs ? nchunks : Stager::kBufs);
    for (int i = 0; i < used; ++i) {
        int rc = ensure(&s->din[i], &s->cap_in[i], (size_t)cr * in_row);
        if (rc) return rc;
        rc = ensure(&s->dout[i], &s->cap_out[i], (size_t)cr * out_row);
        if (rc) return rc;
    }
    cudaStream_t s_in = s->st[0], s_out = s->st[1];
    int64_t r0 = 0;
    for (int64_t c = 0; c < nchunks; r0 += sizes[(size_t)c], ++c) {
        const int i = (int)(c % Stager::kBufs);
        const bool reuse = c >= Stager::kBufs;
        cudaStream_t s_k = s->st[2 + i];
        const int64_t nr = sizes[(size_t)c];
        // input buffer i: last read by the kernel of chunk c - kBufs
        if (reuse) SCIR_CUDA_TRY(cudaStreamWaitEvent(s_in, s->ev_k[i], 0));
        if (in_row)
            SCIR_CUDA_TRY(cudaMemcpyAsync(s->din[i], (const char*)hin + (size_t)r0 * in_row,
                                          (size_t)nr * in_row, cudaMemcpyHostToDevice, s_in));
        SCIR_CUDA_TRY(cudaEventRecord(s->ev_in[i], s_in));
        SCIR_CUDA_TRY(cudaStreamWaitEvent(s_k, s->ev_in[i], 0));
        // output buffer i: last read by the download of chunk c - kBufs
        if (reuse) SCIR_CUDA_TRY(cudaStreamWaitEvent(s_k, s->ev_out[i], 0));
        int rc = body(nr, s->din[i], s->dout[i], s_k);
        if (rc) return rc;
        SCIR_CUDA_TRY(cudaEventRecord(s->ev_k[i], s_k));
        SCIR_CUDA_TRY(cudaStreamWaitEvent(s_out, s->ev_k[i], 0));
        if (out_row)
            SCIR_CUDA_TRY(cudaMemcpyAsync((char*)hout + (size_t)r0 * out_row, s->dout[i],
                                          (size_t)nr * out_row, cudaMemcpyDeviceToHost, s_out));
        SCIR_CUDA_TRY(cudaEventRecord(s->ev_out[i], s_out));
    }
    for (int j = 0; j < Stager::kStreams; ++j) SCIR_CUDA_TRY(cudaStreamSynchronize(s->st[j]));
    SCIR_CUDA_TRY(cudaGetLastError());
    return SCIR_OK;
}

// Queues the upload of `bytes` of host data into the stager's shared tap
// buffer on the upload stream, ahead of the first chunk's upload: every kernel
// of the pipeline waits for a chunk upload recorded after it, so it reads the
// taps whole.  pipeline_rows, which must follow, waits for the copy on every
// exit.  (The previous call drained every stream, so the buffer is free.)
int stage_taps(Stager* s, const void* h, size_t bytes, void** d) {
    int rc = ensure(&s->dtaps, &s->cap_taps, bytes ? bytes : 16);
    if (rc) return rc;
    if (bytes)
        SCIR_CUDA_TRY(cudaMemcpyAsync(s->dtaps, h, bytes, cudaMemcpyHostToDevice, s->st[0]));
    *d = s->dtaps;
    return SCIR_OK;
}

int fir_dispatch(const FirArgs& a, int precision, cudaStream_t st) {
    // a shape the autotuner has timed uses its recorded choice
    const int tuned = (precision == SCIR_PREC_REF_EXACT || precision == SCIR_PREC_FP32 ||
                       precision == SCIR_PREC_AUTO) ? tune_fir_choice(a, precision) : 0;
    if (tuned == 1 || tuned == 2)
        return launch_fir_simt(a, precision == SCIR_PREC_REF_EXACT, st, tuned == 1 ? 8 : 16);
    if (tuned == 3 && precision == SCIR_PREC_AUTO && fir_tc_supported(a))
        return launch_fir_tc(a, kTcFp16x3, st);
    switch (precision) {
    case SCIR_PREC_REF_EXACT: return launch_fir_simt(a, true, st);
    case SCIR_PREC_FP32: return launch_fir_simt(a, false, st);
    case SCIR_PREC_BF16X3:
    case SCIR_PREC_BF16X6:
    case SCIR_PREC_FP16X3:
        if (!fir_tc_supported(a))
            return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR does not serve this shape");
        return launch_fir_tc(a, precision == SCIR_PREC_BF16X3   ? kTcBf16x3
                                : precision == SCIR_PREC_BF16X6 ? kTcBf16x6
                                                                : kTcFp16x3, st);
    case SCIR_PREC_AUTO:
        if (a.k >= 512 && fir_tc_supported(a)) return launch_fir_tc(a, kTcFp16x3, st);
        return launch_fir_simt(a, false, st);
    default: return set_error(SCIR_ERR_INVALID_ARG, "unknown precision %d", precision);
    }
}

int poly_dispatch(const PolyArgs& a, int precision, cudaStream_t st) {
    switch (precision) {
    case SCIR_PREC_FP32:
    case SCIR_PREC_REF_EXACT:
    case SCIR_PREC_AUTO: {
        const int tuned = tune_poly_choice(a);
        return launch_poly_simt(a, st, tuned / 10, tuned % 10);
    }
    case SCIR_PREC_BF16X3:
    case SCIR_PREC_BF16X6:
        if (!poly_tc_supported(a))
            return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase does not serve this shape");
        return launch_poly_tc(a, precision == SCIR_PREC_BF16X3 ? 2 : 3, st);
    case SCIR_PREC_FP16X3:
        return set_error(SCIR_ERR_UNSUPPORTED, "FP16X3 serves the FIR entry points only");
    default: return set_error(SCIR_ERR_INVALID_ARG, "unknown precision %d", precision);
    }
}

int check_rows(const void* x, int64_t ld_x, int64_t batch, int64_t n, const void* y,
               int64_t ld_y, int64_t n_out) {
    SCIR_REQUIRE(batch >= 0 && n >= 0, SCIR_ERR_INVALID_ARG, "negative batch or length");
    SCIR_REQUIRE(ld_x >= n && ld_y >= n_out, SCIR_ERR_SHAPE,
                 "row stride shorter than the row (ld_x=%lld n=%lld ld_y=%lld n_out=%lld)",
                 (long long)ld_x, (long long)n, (long long)ld_y, (long long)n_out);
    if (batch > 0 && n > 0) SCIR_REQUIRE(x != nullptr, SCIR_ERR_INVALID_ARG, "x is NULL");
    if (batch > 0 && n_out > 0) SCIR_REQUIRE(y != nullptr, SCIR_ERR_INVALID_ARG, "y is NULL");
    return SCIR_OK;
}

int resample_geometry(int64_t n, int* up, int* down, int64_t* n_out) {
    SCIR_REQUIRE(*up >= 1 && *down >= 1, SCIR_ERR_INVALID_ARG, "up and down must be >= 1");
    const int64_t g = gcd64(*up, *down);
    *up = (int)(*up / g);
    *down = (int)(*down / g);
    *n_out = ceil_div(n * (int64_t)*up, *down);
    return SCIR_OK;
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" {

SCIR_API int scir_host_chunk_plan(int64_t rows, size_t in_row, size_t out_row, int64_t quantum,
                                  int64_t* sizes, int64_t cap, int64_t* count) {
    clear_error();
    SCIR_REQUIRE(rows >= 1 && quantum >= 1 && count, SCIR_ERR_INVALID_ARG,
                 "rows and quantum must be >= 1 and count non-NULL");
    int64_t cr = 0;
    const std::vector<int64_t> plan = chunk_plan(rows, in_row, out_row, quantum, &cr);
    *count = (int64_t)plan.size();
    SCIR_REQUIRE(sizes || cap == 0, SCIR_ERR_INVALID_ARG, "sizes is NULL");
    for (int64_t i = 0; i < cap && i < (int64_t)plan.size(); ++i) sizes[i] = plan[(size_t)i];
    return SCIR_OK;
}

SCIR_API int64_t scir_fir_out_len(int64_t n, int64_t k, int mode) {
    if (n < 0 || k < 0) return -1;
    switch (mode) {
    case SCIR_FIR_REF_CORR:
    case SCIR_FIR_LFILTER: return n;
    case SCIR_FIR_FULL: return k >= 1 ? n + k - 1 : -1;
    case SCIR_FIR_VALID: return (k >= 1 && n >= k) ? n - k + 1 : -1;
    default: return -1;
    }
}

SCIR_API int scir_fir_batched_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                                  const float* taps, int64_t k, int mode, int precision, float* y,
                                  int64_t ld_y, void* stream) {
    clear_error();
    SCIR_REQUIRE(k >= 0, SCIR_ERR_INVALID_ARG, "negative tap count");
    SCIR_REQUIRE(precision >= SCIR_PREC_AUTO && precision <= SCIR_PREC_FP16X3,
                 SCIR_ERR_INVALID_ARG, "unknown precision %d", precision);
    cudaStream_t st = as_stream(stream);
    FirArgs a;
    int rc;
    if (k == 0) {
        // the reference's empty tap vector gives an all-zero output of length n
        SCIR_REQUIRE(mode == SCIR_FIR_REF_CORR || mode == SCIR_FIR_LFILTER, SCIR_ERR_SHAPE,
                     "FULL/VALID need at least one tap");
        a.n_out = n;
    } else {
        SCIR_REQUIRE(taps != nullptr, SCIR_ERR_INVALID_ARG, "taps is NULL");
        rc = fir_geometry(n, k, mode, &a.reverse, &a.s, &a.n_out);
        if (rc) return rc;
    }
    rc = check_rows(x, ld_x, batch, n, y, ld_y, a.n_out);
    if (rc) return rc;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    if (k == 0) {
        if (batch * n > 0) {
            fill_zero_rows<<<(unsigned)ceil_div(batch * n, 256), 256, 0, st>>>(y, ld_y, batch, n);
            SCIR_LAUNCH_CHECK("fill_zero_rows");
        }
        return SCIR_OK;
    }
    a.x = x; a.ld_x = ld_x; a.batch = batch; a.n = n; a.taps = taps; a.k = k; a.y = y; a.ld_y = ld_y;
    return fir_dispatch(a, precision, st);
}

SCIR_API int64_t scir_upfirdn_out_len(int64_t kh, int64_t n, int up, int down) {
    if (kh < 1 || n < 1 || up < 1 || down < 1) return -1;
    return (((n - 1) * (int64_t)up + kh) - 1) / down + 1;
}

SCIR_API int scir_upfirdn_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                              const float* h, int64_t kh, int up, int down, int precision,
                              float* y, int64_t ld_y, void* stream) {
    clear_error();
    SCIR_REQUIRE(kh >= 1 && h != nullptr, SCIR_ERR_INVALID_ARG, "h must hold at least one tap");
    SCIR_REQUIRE(up >= 1 && down >= 1, SCIR_ERR_INVALID_ARG, "up and down must be >= 1");
    SCIR_REQUIRE(n >= 1, SCIR_ERR_SHAPE, "upfirdn needs at least one input sample");
    PolyArgs a;
    a.n_out = scir_upfirdn_out_len(kh, n, up, down);
    int rc = check_rows(x, ld_x, batch, n, y, ld_y, a.n_out);
    if (rc) return rc;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    a.x = x; a.ld_x = ld_x; a.batch = batch; a.n = n; a.h = h; a.kh = kh;
    a.up = up; a.down = down; a.off = 0; a.y = y; a.ld_y = ld_y;
    return poly_dispatch(a, precision, as_stream(stream));
}

SCIR_API int64_t scir_resample_poly_out_len(int64_t n, int up, int down) {
    if (n < 0 || up < 1 || down < 1) return -1;
    int64_t n_out = 0;
    if (resample_geometry(n, &up, &down, &n_out) != SCIR_OK) return -1;
    return n_out;
}

SCIR_API int scir_resample_poly_default_taps(int up, int down, int design, double* h,
                                             int64_t cap, int64_t* kh) {
    clear_error();
    SCIR_REQUIRE(up >= 1 && down >= 1, SCIR_ERR_INVALID_ARG, "up and down must be >= 1");
    SCIR_REQUIRE(kh != nullptr, SCIR_ERR_INVALID_ARG, "kh is NULL");
    std::vector<double> v;
    int rc = default_taps_host(up, down, design, v);
    if (rc) return rc;
    *kh = (int64_t)v.size();
    if (h) {
        SCIR_REQUIRE(cap >= (int64_t)v.size(), SCIR_ERR_SHAPE, "h holds %lld taps, %zu needed",
                     (long long)cap, v.size());
        memcpy(h, v.data(), v.size() * sizeof(double));
    }
    return SCIR_OK;
}

SCIR_API int scir_resample_poly_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                                    int up, int down, const float* h, int64_t kh, int precision,
                                    float* y, int64_t ld_y, void* stream) {
    clear_error();
    const int up0 = up, down0 = down;
    int64_t n_out = 0;
    int rc = resample_geometry(n, &up, &down, &n_out);
    if (rc) return rc;
    rc = check_rows(x, ld_x, batch, n, y, ld_y, n_out);
    if (rc) return rc;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    cudaStream_t st = as_stream(stream);
    if (batch == 0 || n == 0) return SCIR_OK;
    if (up == 1 && down == 1) {
        SCIR_CUDA_TRY(cudaMemcpy2DAsync(y, ld_y * sizeof(float), x, ld_x * sizeof(float),
                                        n * sizeof(float), batch, cudaMemcpyDeviceToDevice, st));
        return SCIR_OK;
    }
    if (h == nullptr) {
        TapBuf b;
        rc = cached_default_taps(up0, down0, 0, &b);
        if (rc) return rc;
        h = b.d32;
        kh = b.kh;
    }
    SCIR_REQUIRE(kh >= 1, SCIR_ERR_INVALID_ARG, "h must hold at least one tap");
    PolyArgs a;
    a.x = x; a.ld_x = ld_x; a.batch = batch; a.n = n; a.h = h; a.kh = kh;
    a.up = up; a.down = down; a.off = (kh - 1) / 2; a.y = y; a.ld_y = ld_y; a.n_out = n_out;
    return poly_dispatch(a, precision, st);
}

SCIR_API int scir_sosfilt_zi(const double* sos, int nsec, double* zi) {
    clear_error();
    SCIR_REQUIRE(sos && zi, SCIR_ERR_INVALID_ARG, "NULL argument");
    SCIR_REQUIRE(nsec >= 1 && nsec <= SCIR_SOS_MAX_SECTIONS, SCIR_ERR_INVALID_ARG, "bad nsec");
    if (sos_zi_host(sos, nsec, zi) != SCIR_OK)
        return set_error(SCIR_ERR_INVALID_ARG, "a section has a pole at z=1 or a0=0");
    return SCIR_OK;
}

SCIR_API int64_t scir_sosfiltfilt_default_padlen(const double* sos, int nsec) {
    if (!sos || nsec < 1) return -1;
    return sos_default_padlen(sos, nsec);
}

}  // extern "C"

template <typename T>
static int sosfilt_impl(const T* x, int64_t ld_x, int64_t batch, int64_t n, const double* sos,
                        int nsec, const double* zi, double* zf, int precision, T* y, int64_t ld_y,
                        void* stream) {
    clear_error();
    SosCoef c;
    int rc = fill_sos(sos, nsec, false, &c);
    if (rc) return rc;
    rc = check_rows(x, ld_x, batch, n, y, ld_y, n);
    if (rc) return rc;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    // few long channels: the block-parallel time scan
    const bool overlap = (const void*)y < (const void*)(x + batch * ld_x) &&
                         (const void*)x < (const void*)(y + batch * ld_y);
    const int64_t nb = sos_scan_blocks(batch, n, nsec, precision, overlap);
    if (nb > 0)
        return sosfilt_blocked<T>(x, ld_x, batch, n, c, zi, zf, precision, y, ld_y, nb,
                                  as_stream(stream));
    return launch_sosfilt<T>(x, ld_x, batch, n, c, zi, zf, precision, y, ld_y, as_stream(stream));
}

extern "C" {

SCIR_API int scir_sosfilt_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                              const double* sos, int nsec, const double* zi, double* zf,
                              int precision, float* y, int64_t ld_y, void* stream) {
    return sosfilt_impl<float>(x, ld_x, batch, n, sos, nsec, zi, zf, precision, y, ld_y, stream);
}

SCIR_API int scir_sosfilt_f64(const double* x, int64_t ld_x, int64_t batch, int64_t n,
                              const double* sos, int nsec, const double* zi, double* zf,
                              int precision, double* y, int64_t ld_y, void* stream) {
    return sosfilt_impl<double>(x, ld_x, batch, n, sos, nsec, zi, zf, precision, y, ld_y, stream);
}

}  // extern "C"

// Argument checks shared by every sosfiltfilt entry point (the allocating
// ones and scir_sosfiltfilt_f32_noalloc): the padtype, the sections (and
// their sosfilt_zi when padding), the rows, the in-place rule and the edge
// length; then the current device.  Fills *c and the edge length *edge.
int scir::sosfiltfilt_check(const void* x, int64_t ld_x, int64_t batch, int64_t n,
                            const double* sos, int nsec, int padtype, int64_t padlen,
                            const void* y, int64_t ld_y, SosCoef* c, int64_t* edge) {
    SCIR_REQUIRE(padtype == SCIR_PAD_NONE || padtype == SCIR_PAD_ODD, SCIR_ERR_INVALID_ARG,
                 "unknown padtype %d", padtype);
    int rc = fill_sos(sos, nsec, padtype == SCIR_PAD_ODD, c);
    if (rc) return rc;
    rc = check_rows(x, ld_x, batch, n, y, ld_y, n);
    if (rc) return rc;
    SCIR_REQUIRE(y == x ? ld_y == ld_x : true, SCIR_ERR_INVALID_ARG,
                 "in-place sosfiltfilt needs ld_y == ld_x");
    *edge = 0;
    if (padtype == SCIR_PAD_ODD) *edge = padlen < 0 ? sos_default_padlen(sos, nsec) : padlen;
    SCIR_REQUIRE(*edge >= 0, SCIR_ERR_INVALID_ARG, "negative padlen");
    SCIR_REQUIRE(batch == 0 || n > *edge, SCIR_ERR_SHAPE,
                 "the signal must be longer than padlen (n=%lld, padlen=%lld)", (long long)n,
                 (long long)*edge);
    const DeviceInfo* info = nullptr;
    return current_device(&info);
}

template <typename T>
static int sosfiltfilt_impl(const T* x, int64_t ld_x, int64_t batch, int64_t n, const double* sos,
                            int nsec, int padtype, int64_t padlen, int precision, T* y,
                            int64_t ld_y, void* stream) {
    clear_error();
    SosCoef c;
    int64_t edge = 0;
    int rc = sosfiltfilt_check(x, ld_x, batch, n, sos, nsec, padtype, padlen, y, ld_y, &c, &edge);
    if (rc) return rc;
    if (batch == 0 || n == 0) return SCIR_OK;
    cudaStream_t st = as_stream(stream);
    T* tail = nullptr;
    if (edge > 0) {
        rc = scratch_alloc((void**)&tail, sizeof(T) * (size_t)edge * (size_t)batch, st);
        if (rc) return rc;
    }
    rc = launch_sosfiltfilt<T>(x, ld_x, batch, n, c, edge, padtype == SCIR_PAD_ODD, precision, y,
                               ld_y, tail, st);
    scratch_free(tail, st);
    return rc;
}

extern "C" {

SCIR_API int scir_sosfiltfilt_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                                  const double* sos, int nsec, int padtype, int64_t padlen,
                                  int precision, float* y, int64_t ld_y, void* stream) {
    return sosfiltfilt_impl<float>(x, ld_x, batch, n, sos, nsec, padtype, padlen, precision, y,
                                   ld_y, stream);
}

SCIR_API int scir_sosfiltfilt_f64(const double* x, int64_t ld_x, int64_t batch, int64_t n,
                                  const double* sos, int nsec, int padtype, int64_t padlen,
                                  int precision, double* y, int64_t ld_y, void* stream) {
    return sosfiltfilt_impl<double>(x, ld_x, batch, n, sos, nsec, padtype, padlen, precision, y,
                                    ld_y, stream);
}

// ------------------------------------------------------------------ host-buffer layer

SCIR_API int scir_fir_batched_f32_host(const float* x, int64_t batch, int64_t n,
                                       const float* taps, int64_t k, int mode, int precision,
                                       float* y) {
    clear_error();
    SCIR_REQUIRE(batch >= 0 && n >= 0 && k >= 0, SCIR_ERR_INVALID_ARG, "negative size");
    const int64_t n_out = k == 0 ? n : scir_fir_out_len(n, k, mode);
    SCIR_REQUIRE(n_out >= 0, SCIR_ERR_SHAPE, "invalid mode/shape");
    if (batch == 0 || n_out == 0) return SCIR_OK;
    SCIR_REQUIRE(x && y && (k == 0 || taps), SCIR_ERR_INVALID_ARG, "NULL buffer");
    Stager* s = nullptr;
    int rc = stager_get(&s);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    rc = stager_init(s);
    if (rc) return rc;
    void* dt = nullptr;
    rc = stage_taps(s, taps, (size_t)k * sizeof(float), &dt);
    if (rc) return rc;
    return pipeline_rows(s, x, (size_t)n * sizeof(float), y, (size_t)n_out * sizeof(float), batch,
                         [&](int64_t nr, void* din, void* dout, cudaStream_t st) -> int {
                             return scir_fir_batched_f32((const float*)din, n, nr, n,
                                                         (const float*)dt, k, mode, precision,
                                                         (float*)dout, n_out, st);
                         },
                         // whole 128-channel tiles where the tensor cores may run
                         (k >= 512 && precision != SCIR_PREC_FP32 &&
                          precision != SCIR_PREC_REF_EXACT) ? 128 : 1);
}

SCIR_API int scir_fir1d_batched_f32_cuda(const float* x, size_t b, size_t n, const float* taps,
                                         size_t k, float* y) {
    return scir_fir_batched_f32_host(x, (int64_t)b, (int64_t)n, taps, (int64_t)k,
                                     SCIR_FIR_REF_CORR, SCIR_PREC_REF_EXACT, y);
}

SCIR_API int scir_resample_poly_f32_host(const float* x, int64_t batch, int64_t n, int up,
                                         int down, const float* h, int64_t kh, int precision,
                                         float* y) {
    clear_error();
    const int64_t n_out = scir_resample_poly_out_len(n, up, down);
    SCIR_REQUIRE(n_out >= 0 && batch >= 0, SCIR_ERR_INVALID_ARG, "bad sizes or rates");
    if (batch == 0 || n == 0) return SCIR_OK;
    SCIR_REQUIRE(x && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    Stager* s = nullptr;
    int rc = stager_get(&s);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    rc = stager_init(s);
    if (rc) return rc;
    void* dt = nullptr;
    if (h) {
        SCIR_REQUIRE(kh >= 1, SCIR_ERR_INVALID_ARG, "kh must be >= 1");
        rc = stage_taps(s, h, (size_t)kh * sizeof(float), &dt);
        if (rc) return rc;
    }
    return pipeline_rows(s, x, (size_t)n * sizeof(float), y, (size_t)n_out * sizeof(float), batch,
                         [&](int64_t nr, void* din, void* dout, cudaStream_t st) -> int {
                             return scir_resample_poly_f32((const float*)din, n, nr, n, up, down,
                                                           (const float*)dt, kh, precision,
                                                           (float*)dout, n_out, st);
                         });
}

SCIR_API int scir_sosfilt_f64_host(const double* sos, int nsec, const double* x, size_t batch,
                                   size_t n, double* y) {
    clear_error();
    if (batch == 0 || n == 0) return SCIR_OK;
    SCIR_REQUIRE(x && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    Stager* s = nullptr;
    int rc = stager_get(&s);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    rc = stager_init(s);
    if (rc) return rc;
    const size_t row = n * sizeof(double);
    return pipeline_rows(s, x, row, y, row, (int64_t)batch,
                         [&](int64_t nr, void* din, void* dout, cudaStream_t st) -> int {
                             return scir_sosfilt_f64((const double*)din, (int64_t)n, nr,
                                                     (int64_t)n, sos, nsec, nullptr, nullptr,
                                                     SCIR_SOS_FP64_EXACT, (double*)dout,
                                                     (int64_t)n, st);
                         });
}

SCIR_API int scir_filtfilt_f64_host(const double* sos, int nsec, const double* x, size_t batch,
                                    size_t n, double* y) {
    clear_error();
    if (batch == 0 || n == 0) return SCIR_OK;
    SCIR_REQUIRE(x && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    Stager* s = nullptr;
    int rc = stager_get(&s);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    rc = stager_init(s);
    if (rc) return rc;
    const size_t row = n * sizeof(double);
    return pipeline_rows(s, x, row, y, row, (int64_t)batch,
                         [&](int64_t nr, void* din, void* dout, cudaStream_t st) -> int {
                             return scir_sosfiltfilt_f64((const double*)din, (int64_t)n, nr,
                                                         (int64_t)n, sos, nsec, SCIR_PAD_NONE, 0,
                                                         SCIR_SOS_FP64_EXACT, (double*)dout,
                                                         (int64_t)n, st);
                         });
}

SCIR_API int scir_resample_poly_f64_host(const double* x, size_t batch, size_t n, size_t up,
                                         size_t down, double* y) {
    clear_error();
    SCIR_REQUIRE(up >= 1 && down >= 1 && up < (1u << 30) && down < (1u << 30),
                 SCIR_ERR_INVALID_ARG, "bad rates");
    int u = (int)up, d = (int)down;
    std::vector<double> hv;
    int rc = default_taps_host(u, d, 1, hv);  // the reference design: 2/3 only
    if (rc) return rc;
    const int64_t g = gcd64(u, d);
    u /= (int)g;
    d /= (int)g;
    const int64_t n_out = ceil_div((int64_t)n * u, d);
    if (batch == 0 || n == 0) return SCIR_OK;
    SCIR_REQUIRE(x && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    Stager* s = nullptr;
    rc = stager_get(&s);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    rc = stager_init(s);
    if (rc) return rc;
    void* dh = nullptr;
    rc = stage_taps(s, hv.data(), hv.size() * sizeof(double), &dh);
    if (rc) return rc;
    const int64_t kh = (int64_t)hv.size();
    return pipeline_rows(s, x, n * sizeof(double), y, (size_t)n_out * sizeof(double),
                         (int64_t)batch,
                         [&](int64_t nr, void* din, void* dout, cudaStream_t st) -> int {
                             const int64_t bpr = ceil_div(n_out, 256);
                             poly_exact_f64_kernel<<<(unsigned)(bpr * nr), 256, 0, st>>>(
                                 (const double*)din, (int64_t)n, (const double*)dh, kh, u, d,
                                 (kh - 1) / 2, (double*)dout, n_out, bpr);
                             SCIR_LAUNCH_CHECK("poly_exact_f64_kernel");
                             return SCIR_OK;
                         });
}

}  // extern "C"
