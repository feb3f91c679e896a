// Autotuner: picks, per problem shape and device model, among the kernel
// variants the dispatch can run, by timing them on synthetic data of that
// shape.
//
//   FIR (REF_EXACT / FP32 / AUTO precision): CUDA-core tiles of 8 or 16
//     outputs per thread; with AUTO also the tensor-core FP16X3 path (a
//     tensor-core form that holds 1e-5 at three products).  The default without tuning is 16
//     from 128 taps on and the tensor cores from 512 taps on.
//   resample_poly / upfirdn: outputs per lane P (from the minimum that keeps
//     a period within one warp up to 5) and channels per work item (1, 2 or
//     4; four use items of 16 periods).
//   ragged FIR: the tap count from which tiles use 16 outputs per thread
//     (scir_ragged_plan_autotune, in ragged.cu).
//
// The table is keyed by the device model (name and SM count), so a saved
// table applies to every device of that model; scir_autotune_save/load keep
// it in a text file.  Tuning allocates its buffers from the library's scratch
// pool, runs on a private stream and synchronises it.  Shapes whose data fits
// in L2 are timed with L2 flushed before every call (time_calls below).
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace scir {
namespace {

using FirKey = std::tuple<std::string, int64_t, int64_t, int64_t, int64_t, int, int64_t, int>;
// model, batch, n, k, n_out, reverse, s, precision
using PolyKey = std::tuple<std::string, int64_t, int64_t, int64_t, int, int, int64_t>;
// model, batch, n, kh, up, down, off

std::mutex g_mu;
std::map<FirKey, int> g_fir;
std::map<PolyKey, int> g_poly;

int device_model(std::string* out) {
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<int, std::string> names;
    std::lock_guard<std::mutex> lk(mu);
    auto it = names.find(dev);
    if (it == names.end()) {
        cudaDeviceProp prop;
        SCIR_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
        std::string m = prop.name;
        for (char& c : m)
            if (c == ' ') c = '_';
        m += "_sm" + std::to_string(prop.multiProcessorCount);
        it = names.emplace(dev, m).first;
    }
    *out = it->second;
    return SCIR_OK;
}

FirKey fir_key(const std::string& m, const FirArgs& a, int precision) {
    return FirKey{m, a.batch, a.n, a.k, a.n_out, a.reverse, a.s, precision};
}
PolyKey poly_key(const std::string& m, const PolyArgs& a) {
    return PolyKey{m, a.batch, a.n, a.kh, a.up, a.down, a.off};
}

__global__ void fill_uniform_kernel(float* __restrict__ p, int64_t count, uint32_t seed) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 16;
        h *= 2246822519u;
        h ^= h >> 13;
        h *= 3266489917u;
        h ^= h >> 16;
        p[i] = (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;  // U[-1, 1)
    }
}

int fill_uniform(float* p, int64_t count, uint32_t seed, cudaStream_t st) {
    if (count <= 0) return SCIR_OK;
    const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(count, 256), 16384);
    fill_uniform_kernel<<<grid, 256, 0, st>>>(p, count, seed);
    SCIR_LAUNCH_CHECK("fill_uniform_kernel");
    return SCIR_OK;
}

// A buffer of twice the L2 size, written before every timed call when the
// call's data (inputs and outputs) would otherwise stay in L2 from one call
// to the next: a call on data that was just copied in or produced by other
// work finds little of it in L2, and the variants differ in how well they hide
// that latency (at 64 x 65,536 samples and 63 taps the 16-output tile is ahead
// warm, the two tie cold).  Null when the data is larger than L2.
struct L2Flush {
    void* p = nullptr;
    size_t bytes = 0;
};

int l2_flush_for(size_t data_bytes, cudaStream_t st, L2Flush* out) {
    *out = L2Flush{};
    const DeviceInfo* d = nullptr;
    int rc = current_device(&d);
    if (rc) return rc;
    if (d->l2_bytes <= 0 || data_bytes >= (size_t)d->l2_bytes) return SCIR_OK;
    out->bytes = 2 * (size_t)d->l2_bytes;
    rc = scratch_alloc(&out->p, out->bytes, st);
    if (rc) *out = L2Flush{};
    return rc;
}

void l2_flush_free(L2Flush* f, cudaStream_t st) {
    if (f->p) scratch_free(f->p, st);
    *f = L2Flush{};
}

// Time per call of f (CUDA events on st): one warm-up call and one timed call
// that sizes the trials, then trials of max(min_reps, ~2 ms worth, <= 200)
// calls -- three for calls under 5 ms, one above -- and the fastest trial's
// mean (interference from other work on the device only adds time).  With a
// flush buffer every call is timed on its own, after the buffer is written
// (<= 50 calls a trial).
template <typename F>
int time_calls(F&& f, cudaStream_t st, int min_reps, float* ms, const L2Flush& flush) {
    int rc = f();
    if (rc) return rc;
    cudaEvent_t e0, e1;
    SCIR_CUDA_TRY(cudaEventCreate(&e0));
    SCIR_CUDA_TRY(cudaEventCreate(&e1));
    auto timed = [&](int reps, float* t) -> int {
        int r2 = SCIR_OK;
        cudaError_t ce = cudaSuccess;
        if (flush.p) {
            float sum = 0.0f;
            for (int r = 0; r < reps && r2 == SCIR_OK && ce == cudaSuccess; ++r) {
                ce = cudaMemsetAsync(flush.p, r & 0xff, flush.bytes, st);
                if (ce == cudaSuccess) ce = cudaEventRecord(e0, st);
                if (ce == cudaSuccess) r2 = f();
                if (ce == cudaSuccess) ce = cudaEventRecord(e1, st);
                if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
                float one = 0.0f;
                if (ce == cudaSuccess) ce = cudaEventElapsedTime(&one, e0, e1);
                sum += one;
            }
            *t = sum;
        } else {
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && r2 == SCIR_OK; ++r) r2 = f();
            cudaEventRecord(e1, st);
            ce = cudaEventSynchronize(e1);
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(t, e0, e1);
        }
        if (r2) return r2;
        if (ce != cudaSuccess)
            return set_error(SCIR_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(ce));
        *t /= (float)reps;
        return SCIR_OK;
    };
    float one = 0.0f;
    rc = timed(1, &one);
    int reps = min_reps;
    if (!rc && one > 0.0f)
        reps = std::max(min_reps, std::min(flush.p ? 50 : 200, (int)(2.0f / one) + 1));
    const int trials = one < 5.0f ? 3 : 1;
    float best = 0.0f;
    for (int i = 0; i < trials && rc == SCIR_OK; ++i) {
        float t = 0.0f;
        rc = timed(reps, &t);
        if (!rc && (i == 0 || t < best)) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *ms = best;
    return SCIR_OK;
}

// Private tuning stream of the current device.
int tune_stream(cudaStream_t* out) {
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<int, cudaStream_t> streams;
    std::lock_guard<std::mutex> lk(mu);
    auto it = streams.find(dev);
    if (it == streams.end()) {
        cudaStream_t s = nullptr;
        SCIR_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        it = streams.emplace(dev, s).first;
    }
    *out = it->second;
    return SCIR_OK;
}

void put_choice(char* buf, size_t len, const std::string& s) {
    if (!buf || len == 0) return;
    snprintf(buf, len, "%s", s.c_str());
}

const char* fir_choice_name(int c) {
    return c == 1 ? "cuda-cores-v8" : c == 2 ? "cuda-cores-v16" : c == 3 ? "tensor-cores-fp16x3" : "default";
}

}  // namespace

int tune_fir_choice(const FirArgs& a, int precision) {
    std::string m;
    if (device_model(&m)) {
        clear_error();
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_fir.find(fir_key(m, a, precision));
    return it == g_fir.end() ? 0 : it->second;
}

int tune_poly_choice(const PolyArgs& a) {
    std::string m;
    if (device_model(&m)) {
        clear_error();
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_poly.find(poly_key(m, a));
    return it == g_poly.end() ? 0 : it->second;
}

}  // namespace scir

using namespace scir;

extern "C" {

SCIR_API int scir_autotune_fir(int64_t batch, int64_t n, int64_t k, int mode, int precision,
                               double* best_ms, char* choice, size_t choice_len) {
    clear_error();
    SCIR_REQUIRE(batch >= 1 && n >= 1 && k >= 1, SCIR_ERR_INVALID_ARG, "empty problem");
    SCIR_REQUIRE(precision == SCIR_PREC_REF_EXACT || precision == SCIR_PREC_FP32 ||
                     precision == SCIR_PREC_AUTO,
                 SCIR_ERR_UNSUPPORTED, "precision %d has a single kernel form", precision);
    FirArgs a{};
    int rc = fir_geometry(n, k, mode, &a.reverse, &a.s, &a.n_out);
    if (rc) return rc;
    SCIR_REQUIRE(a.n_out >= 1, SCIR_ERR_SHAPE, "empty output");
    std::string model;
    rc = device_model(&model);
    if (rc) return rc;
    cudaStream_t st = nullptr;
    rc = tune_stream(&st);
    if (rc) return rc;
    float *x = nullptr, *taps = nullptr, *y = nullptr;
    rc = scratch_alloc((void**)&x, sizeof(float) * (size_t)(batch * n), st);
    if (!rc) rc = scratch_alloc((void**)&taps, sizeof(float) * (size_t)k, st);
    if (!rc) rc = scratch_alloc((void**)&y, sizeof(float) * (size_t)(batch * a.n_out), st);
    if (!rc) rc = fill_uniform(x, batch * n, 1u, st);
    if (!rc) rc = fill_uniform(taps, k, 2u, st);
    a.x = x;
    a.ld_x = n;
    a.batch = batch;
    a.n = n;
    a.taps = taps;
    a.k = k;
    a.y = y;
    a.ld_y = a.n_out;
    L2Flush flush;
    if (!rc) rc = l2_flush_for(sizeof(float) * (size_t)(batch * (n + a.n_out)), st, &flush);
    const bool exact = precision == SCIR_PREC_REF_EXACT;
    std::vector<int> cand = {1, 2};
    if (precision == SCIR_PREC_AUTO && fir_tc_supported(a)) cand.push_back(3);
    int best = 0;
    float best_t = 0.0f;
    for (int c : cand) {
        if (rc) break;
        float t = 0.0f;
        rc = time_calls(
            [&]() -> int {
                return c == 3 ? launch_fir_tc(a, kTcFp16x3, st) : launch_fir_simt(a, exact, st, c == 1 ? 8 : 16);
            },
            st, 3, &t, flush);
        if (!rc && (best == 0 || t < best_t)) {
            best = c;
            best_t = t;
        }
    }
    l2_flush_free(&flush, st);
    scratch_free(x, st);
    scratch_free(taps, st);
    scratch_free(y, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(SCIR_ERR_CUDA, "autotune: %s", cudaGetErrorString(ce));
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_fir[fir_key(model, a, precision)] = best;
    }
    if (best_ms) *best_ms = best_t;
    put_choice(choice, choice_len, fir_choice_name(best));
    return SCIR_OK;
}

SCIR_API int scir_autotune_resample_poly(int64_t batch, int64_t n, int up, int down,
                                         int64_t kh, double* best_ms, char* choice,
                                         size_t choice_len) {
    clear_error();
    SCIR_REQUIRE(batch >= 1 && n >= 1 && up >= 1 && down >= 1, SCIR_ERR_INVALID_ARG,
                 "empty problem or bad rates");
    const int64_t g = gcd64(up, down);
    const int upr = (int)(up / g), dnr = (int)(down / g);
    SCIR_REQUIRE(upr != dnr, SCIR_ERR_UNSUPPORTED, "up == down is a copy");
    // kh <= 0: SciPy's default design, 2*10*max(up, down) + 1 taps
    const int64_t khr = kh > 0 ? kh : 20 * (int64_t)std::max(upr, dnr) + 1;
    const int64_t n_out = scir_resample_poly_out_len(n, upr, dnr);
    SCIR_REQUIRE(n_out >= 1, SCIR_ERR_SHAPE, "empty output");
    std::string model;
    int rc = device_model(&model);
    if (rc) return rc;
    cudaStream_t st = nullptr;
    rc = tune_stream(&st);
    if (rc) return rc;
    float *x = nullptr, *h = nullptr, *y = nullptr;
    rc = scratch_alloc((void**)&x, sizeof(float) * (size_t)(batch * n), st);
    if (!rc) rc = scratch_alloc((void**)&h, sizeof(float) * (size_t)khr, st);
    if (!rc) rc = scratch_alloc((void**)&y, sizeof(float) * (size_t)(batch * n_out), st);
    if (!rc) rc = fill_uniform(x, batch * n, 3u, st);
    if (!rc) rc = fill_uniform(h, khr, 4u, st);
    PolyArgs a{};
    a.x = x;
    a.ld_x = n;
    a.batch = batch;
    a.n = n;
    a.h = h;
    a.kh = khr;
    a.up = upr;
    a.down = dnr;
    a.off = (khr - 1) / 2;
    a.y = y;
    a.ld_y = n_out;
    a.n_out = n_out;
    L2Flush flush;
    if (!rc) rc = l2_flush_for(sizeof(float) * (size_t)(batch * (n + n_out)), st, &flush);
    const int pmin = (int)std::max<int64_t>(1, ceil_div(upr, 32));
    int best = 0;
    float best_t = 0.0f;
    const int pmax = std::min(5, std::max(pmin, upr));  // more outputs per lane than up idle lanes
    for (int P = pmin; P <= pmax && !rc; ++P) {
        for (int ct = 1; ct <= (batch >= 4 ? 4 : batch >= 2 ? 2 : 1) && !rc; ct *= 2) {
            float t = 0.0f;
            rc = time_calls([&]() -> int { return launch_poly_simt(a, st, P, ct); }, st, 3, &t,
                            flush);
            if (!rc && (best == 0 || t < best_t)) {
                best = P * 10 + ct;
                best_t = t;
            }
        }
    }
    l2_flush_free(&flush, st);
    scratch_free(x, st);
    scratch_free(h, st);
    scratch_free(y, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(SCIR_ERR_CUDA, "autotune: %s", cudaGetErrorString(ce));
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_poly[poly_key(model, a)] = best;
    }
    if (best_ms) *best_ms = best_t;
    put_choice(choice, choice_len,
               "P=" + std::to_string(best / 10) + " channels-per-item=" + std::to_string(best % 10));
    return SCIR_OK;
}

SCIR_API int scir_autotune_clear(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_fir.clear();
    g_poly.clear();
    return SCIR_OK;
}

// Text format, one entry per line after the header:
//   fir  <model> <batch> <n> <k> <n_out> <reverse> <s> <precision> <choice>
//   poly <model> <batch> <n> <kh> <up> <down> <off> <choice>
SCIR_API int scir_autotune_save(const char* path) {
    clear_error();
    SCIR_REQUIRE(path != nullptr, SCIR_ERR_INVALID_ARG, "path is NULL");
    FILE* f = fopen(path, "w");
    SCIR_REQUIRE(f != nullptr, SCIR_ERR_INVALID_ARG, "cannot write %s", path);
    std::lock_guard<std::mutex> lk(g_mu);
    fprintf(f, "scir-autotune 1\n");
    for (const auto& e : g_fir) {
        const FirKey& k = e.first;
        fprintf(f, "fir %s %lld %lld %lld %lld %d %lld %d %d\n", std::get<0>(k).c_str(),
                (long long)std::get<1>(k), (long long)std::get<2>(k), (long long)std::get<3>(k),
                (long long)std::get<4>(k), std::get<5>(k), (long long)std::get<6>(k),
                std::get<7>(k), e.second);
    }
    for (const auto& e : g_poly) {
        const PolyKey& k = e.first;
        fprintf(f, "poly %s %lld %lld %lld %d %d %lld %d\n", std::get<0>(k).c_str(),
                (long long)std::get<1>(k), (long long)std::get<2>(k), (long long)std::get<3>(k),
                std::get<4>(k), std::get<5>(k), (long long)std::get<6>(k), e.second);
    }
    const bool ok = fclose(f) == 0;
    SCIR_REQUIRE(ok, SCIR_ERR_INVALID_ARG, "write to %s failed", path);
    return SCIR_OK;
}

SCIR_API int scir_autotune_load(const char* path) {
    clear_error();
    SCIR_REQUIRE(path != nullptr, SCIR_ERR_INVALID_ARG, "path is NULL");
    FILE* f = fopen(path, "r");
    SCIR_REQUIRE(f != nullptr, SCIR_ERR_INVALID_ARG, "cannot read %s", path);
    char line[512], kind[16], model[256];
    int version = 0, lineno = 0, bad = 0;
    if (!fgets(line, sizeof line, f) || sscanf(line, "scir-autotune %d", &version) != 1 ||
        version != 1)
        bad = 1;
    std::map<FirKey, int> fir;
    std::map<PolyKey, int> poly;
    while (!bad && fgets(line, sizeof line, f)) {
        ++lineno;
        if (line[0] == '\n' || line[0] == '#') continue;
        long long b, n, k, no, s, kh, off;
        int rev, prec, ch, up, dn;
        if (sscanf(line, "%15s", kind) != 1) continue;
        if (!strcmp(kind, "fir") &&
            sscanf(line, "fir %255s %lld %lld %lld %lld %d %lld %d %d", model, &b, &n, &k, &no, &rev,
                   &s, &prec, &ch) == 9 && ch >= 1 && ch <= 3) {
            fir[FirKey{model, b, n, k, no, rev, s, prec}] = ch;
        } else if (!strcmp(kind, "poly") &&
                   sscanf(line, "poly %255s %lld %lld %lld %d %d %lld %d", model, &b, &n, &kh, &up,
                          &dn, &off, &ch) == 8 && ch / 10 >= 1 && ch / 10 <= 5 &&
                   (ch % 10 == 1 || ch % 10 == 2 || ch % 10 == 4)) {
            poly[PolyKey{model, b, n, kh, up, dn, off}] = ch;
        } else {
            bad = lineno + 1;
        }
    }
    fclose(f);
    SCIR_REQUIRE(!bad, SCIR_ERR_INVALID_ARG, "%s: not a scir autotune table (line %d)", path, bad);
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& e : fir) g_fir[e.first] = e.second;
    for (auto& e : poly) g_poly[e.first] = e.second;
    return SCIR_OK;
}

}  // extern "C"
