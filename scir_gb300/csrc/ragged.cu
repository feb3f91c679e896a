// Ragged batched FIR: many signals of different lengths and tap counts in one
// persistent launch.
//
// The reference API takes a single tap vector for a rectangular batch
// (crates/scir-gpu/src/lib.rs:1134); a ragged set would be one call per
// signal.  Here a host-built plan splits every signal into output tiles
// (256*V outputs, V = 8 for short filters, 16 for long ones), orders the
// tiles by cost (outputs x taps, largest first) and uploads the signal and
// tile tables once.  The launch is sized to fill every SM; each CTA takes the
// next tile index from a device counter with one atomicAdd and runs the same
// tile code as the batched kernel (fir_tile.cuh).  There is no device-side
// waiting: a CTA that finds the counter past the last tile exits.  The
// counter is zeroed by a memset node on the launch stream, so a launch can be
// captured into a CUDA graph and replayed.
#include "common.cuh"
#include "fir_tile.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <vector>

struct RaggedSig {
    int64_t x_off, n, taps_off, k, y_off, s, n_out;
    int32_t reverse, chunk8, chunk16, pad_;
};
struct RaggedTile {
    int32_t sig, v16;
    int64_t o0;
};

struct scir_ragged_plan {
    int device = -1, mode = 0, precision = 0;
    // tensor-core bucket: signals with at least tc_min_taps taps (AUTO,
    // FP16X3, BF16X3, BF16X6) run the split-operand tensor-core contraction
    // in its own launch; tc_form is its scir::TcForm (0: no bucket)
    int tc_form = 0, tc_min_taps = 1 << 30;
    std::vector<char> in_tc;          // per signal
    scir::TcRaggedPlan* tc = nullptr;
    int64_t count = 0, ntiles = 0, samples_in = 0;
    double macs = 0.0;
    RaggedSig* d_sigs = nullptr;
    RaggedTile* d_tiles = nullptr;
    unsigned long long* d_counter = nullptr;
    int grid = 0, per_sm = 0;
    size_t smem = 0;
    int v16_min_taps = 128;          // tiles of 16 outputs per thread from this tap count
    std::vector<RaggedSig> h_sigs;   // host copy, for rebuilding the tile list
    size_t tiles_cap = 0;            // RaggedTile slots allocated at d_tiles
};

namespace scir {
namespace {

constexpr int kMaxSmemChunk = kFirMaxChunk;

template <bool EXACT>
__global__ void __launch_bounds__(kFirThreads)
ragged_kernel(const RaggedSig* __restrict__ sigs, const RaggedTile* __restrict__ tiles,
              int64_t ntiles, const float* __restrict__ x, const float* __restrict__ taps,
              float* __restrict__ y, unsigned long long* __restrict__ counter) {
    extern __shared__ __align__(16) float smem[];
    __shared__ long long cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long t = cur;
        __syncthreads();
        if (t >= ntiles) break;
        const RaggedTile tl = tiles[t];
        const RaggedSig sg = sigs[tl.sig];
        if (tl.v16)
            fir_tile<16, EXACT>(smem, x + sg.x_off, sg.n, taps + sg.taps_off, sg.k, sg.reverse,
                                sg.s, y + sg.y_off, sg.n_out, tl.o0, sg.chunk16);
        else
            fir_tile<8, EXACT>(smem, x + sg.x_off, sg.n, taps + sg.taps_off, sg.k, sg.reverse,
                               sg.s, y + sg.y_off, sg.n_out, tl.o0, sg.chunk8);
    }
}

}  // namespace
}  // namespace scir

using namespace scir;

namespace scir {
namespace {

// Cuts every signal into tiles of 256*V outputs (V = 16 from v16_min_taps
// taps on, else 8), orders them largest-cost first (the shared counter then
// hands out work in longest-processing-time order), uploads the list and
// sizes the persistent grid.
int build_tiles(scir_ragged_plan* p, int v16_min_taps) {
    std::vector<RaggedTile> tiles;
    std::vector<double> cost;
    for (size_t i = 0; i < p->h_sigs.size(); ++i) {
        const RaggedSig& s = p->h_sigs[i];
        if (!p->in_tc.empty() && p->in_tc[i]) continue;  // served by the tensor-core bucket
        const int v16 = s.k >= v16_min_taps ? 1 : 0;
        const int64_t tile = (int64_t)kFirThreads * (v16 ? 16 : 8);
        for (int64_t o0 = 0; o0 < s.n_out; o0 += tile) {
            tiles.push_back(RaggedTile{(int32_t)i, v16, o0});
            cost.push_back((double)std::min<int64_t>(tile, s.n_out - o0) * (double)s.k);
        }
    }
    std::vector<size_t> order(tiles.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<RaggedTile> sorted(tiles.size());
    for (size_t i = 0; i < order.size(); ++i) sorted[i] = tiles[order[i]];
    if (sorted.size() > p->tiles_cap || !p->d_tiles) {
        if (p->d_tiles) cudaFree(p->d_tiles);
        p->d_tiles = nullptr;
        p->tiles_cap = 0;
        cudaError_t e = cudaMalloc(&p->d_tiles, std::max<size_t>(1, sorted.size()) * sizeof(RaggedTile));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(SCIR_ERR_OOM, "ragged tile list allocation failed: %s",
                             cudaGetErrorString(e));
        }
        p->tiles_cap = std::max<size_t>(1, sorted.size());
    }
    int rc = upload_sync(p->d_tiles, sorted.data(), sorted.size() * sizeof(RaggedTile));
    if (rc) return rc;
    p->ntiles = (int64_t)sorted.size();
    p->v16_min_taps = v16_min_taps;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    p->grid = (int)std::min<int64_t>((int64_t)p->per_sm * info->sm_count,
                                     std::max<int64_t>(1, p->ntiles));
    return SCIR_OK;
}

// Rebuilds the tensor-core bucket with the signals that have at least
// min_taps taps and 16,384 outputs (fewer outputs leave most of a 128-row
// tile empty), then the CUDA-core tile list for the others.
int build_tc(scir_ragged_plan* p, int min_taps) {
    tc_ragged_destroy(p->tc);
    p->tc = nullptr;
    p->in_tc.assign(p->h_sigs.size(), 0);
    p->tc_min_taps = min_taps;
    if (p->tc_form == 0) return build_tiles(p, p->v16_min_taps);
    std::vector<TcSigIn> in;
    for (size_t i = 0; i < p->h_sigs.size(); ++i) {
        const RaggedSig& s = p->h_sigs[i];
        if (s.k < min_taps || s.n_out < 16384) continue;
        p->in_tc[i] = 1;
        in.push_back(TcSigIn{s.x_off, s.n, s.taps_off, s.k, s.y_off, s.s, s.n_out, s.reverse});
    }
    int rc = tc_ragged_create(in.data(), (int64_t)in.size(), p->tc_form, &p->tc);
    if (rc) return rc;
    return build_tiles(p, p->v16_min_taps);
}

}  // namespace
}  // namespace scir

extern "C" {

SCIR_API int scir_ragged_plan_create(const scir_ragged_desc* desc, int64_t count, int mode,
                                     int precision, scir_ragged_plan** plan) {
    clear_error();
    SCIR_REQUIRE(plan != nullptr, SCIR_ERR_INVALID_ARG, "plan is NULL");
    *plan = nullptr;
    SCIR_REQUIRE(count >= 0 && (count == 0 || desc), SCIR_ERR_INVALID_ARG, "bad descriptor table");
    SCIR_REQUIRE(count < (1LL << 31), SCIR_ERR_UNSUPPORTED, "too many signals");
    // AUTO (FP16X3), FP16X3, BF16X6, BF16X3: long filters on the tensor
    // cores, the rest in FP32 on the CUDA cores
    int tc_form = 0;
    if (precision == SCIR_PREC_AUTO || precision == SCIR_PREC_FP16X3) tc_form = scir::kTcFp16x3;
    if (precision == SCIR_PREC_BF16X6) tc_form = scir::kTcBf16x6;
    if (precision == SCIR_PREC_BF16X3) tc_form = scir::kTcBf16x3;
    if (tc_form) precision = SCIR_PREC_FP32;
    SCIR_REQUIRE(precision == SCIR_PREC_FP32 || precision == SCIR_PREC_REF_EXACT,
                 SCIR_ERR_UNSUPPORTED, "unknown ragged precision");
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;

    auto p = new scir_ragged_plan();
    p->device = info->device;
    p->mode = mode;
    p->precision = precision;
    p->tc_form = tc_form;
    p->count = count;
    std::vector<RaggedSig> sigs((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        const scir_ragged_desc& d = desc[i];
        if (d.n < 0 || d.k < 1 || d.x_off < 0 || d.taps_off < 0 || d.y_off < 0) {
            delete p;
            return set_error(SCIR_ERR_INVALID_ARG, "descriptor %lld: negative size/offset or k < 1",
                             (long long)i);
        }
        RaggedSig& s = sigs[(size_t)i];
        int rev = 0;
        rc = fir_geometry(d.n, d.k, mode, &rev, &s.s, &s.n_out);
        if (rc) {
            delete p;
            return rc;
        }
        s.x_off = d.x_off;
        s.n = d.n;
        s.taps_off = d.taps_off;
        s.k = d.k;
        s.y_off = d.y_off;
        s.reverse = rev;
        const int64_t k8 = (d.k + 7) / 8 * 8, k16 = (d.k + 15) / 16 * 16;
        s.chunk8 = (int)std::min<int64_t>(k8, kMaxSmemChunk);
        s.chunk16 = (int)std::min<int64_t>(k16, kMaxSmemChunk);
        s.pad_ = 0;
        p->samples_in += d.n;
        p->macs += (double)s.n_out * (double)d.k;
    }
    auto fail = [&](int code) {
        scir_ragged_plan_destroy(p);
        return code;
    };
    cudaError_t e = cudaMalloc(&p->d_sigs, std::max<size_t>(1, sigs.size()) * sizeof(RaggedSig));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_counter, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(SCIR_ERR_OOM, "ragged plan allocation failed: %s", cudaGetErrorString(e));
        return fail(SCIR_ERR_OOM);
    }
    rc = upload_sync(p->d_sigs, sigs.data(), sigs.size() * sizeof(RaggedSig));
    if (rc) return fail(rc);
    p->h_sigs = std::move(sigs);
    // tiles of 8 and of 16 outputs per thread share the launch
    p->smem = std::max(fir_tile_smem_bytes(16, kMaxSmemChunk), fir_tile_smem_bytes(8, kMaxSmemChunk));
    auto kern = precision == SCIR_PREC_REF_EXACT ? ragged_kernel<true> : ragged_kernel<false>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem);
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFirThreads, p->smem);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        set_error(SCIR_ERR_CUDA, "ragged kernel occupancy query failed: %s", cudaGetErrorString(e));
        return fail(SCIR_ERR_CUDA);
    }
    p->per_sm = per_sm;
    rc = build_tc(p, tc_form ? 512 : (1 << 30));
    if (rc) return fail(rc);
    *plan = p;
    return SCIR_OK;
}

SCIR_API int scir_ragged_plan_destroy(scir_ragged_plan* plan) {
    if (!plan) return SCIR_OK;
    if (plan->d_sigs) cudaFree(plan->d_sigs);
    if (plan->d_tiles) cudaFree(plan->d_tiles);
    if (plan->d_counter) cudaFree(plan->d_counter);
    scir::tc_ragged_destroy(plan->tc);
    delete plan;
    return SCIR_OK;
}

SCIR_API int scir_ragged_plan_stats(const scir_ragged_plan* plan, int64_t* tiles, double* macs,
                                    int64_t* samples_in) {
    SCIR_REQUIRE(plan != nullptr, SCIR_ERR_INVALID_ARG, "plan is NULL");
    if (tiles) *tiles = plan->ntiles + scir::tc_ragged_tiles(plan->tc);
    if (macs) *macs = plan->macs;
    if (samples_in) *samples_in = plan->samples_in;
    return SCIR_OK;
}

SCIR_API int scir_fir_ragged_f32(const scir_ragged_plan* plan, const float* x, const float* taps,
                                 float* y, void* stream) {
    clear_error();
    SCIR_REQUIRE(plan != nullptr, SCIR_ERR_INVALID_ARG, "plan is NULL");
    if (plan->ntiles == 0 && !plan->tc) return SCIR_OK;
    SCIR_REQUIRE(x && taps && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    int dev = -1;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    SCIR_REQUIRE(dev == plan->device, SCIR_ERR_INVALID_ARG,
                 "plan was built on device %d, current device is %d", plan->device, dev);
    cudaStream_t st = as_stream(stream);
    // the tensor-core bucket first (split kernels + one persistent launch)
    int rc = scir::tc_ragged_run(plan->tc, x, taps, y, st);
    if (rc) return rc;
    if (plan->ntiles == 0) return SCIR_OK;
    SCIR_CUDA_TRY(cudaMemsetAsync(plan->d_counter, 0, sizeof(unsigned long long), st));
    if (plan->precision == SCIR_PREC_REF_EXACT)
        ragged_kernel<true><<<plan->grid, kFirThreads, plan->smem, st>>>(
            plan->d_sigs, plan->d_tiles, plan->ntiles, x, taps, y, plan->d_counter);
    else
        ragged_kernel<false><<<plan->grid, kFirThreads, plan->smem, st>>>(
            plan->d_sigs, plan->d_tiles, plan->ntiles, x, taps, y, plan->d_counter);
    SCIR_LAUNCH_CHECK("ragged_kernel");
    return SCIR_OK;
}

SCIR_API int scir_ragged_plan_autotune(scir_ragged_plan* plan, const float* x, const float* taps,
                                       float* y, void* stream, int* v16_min_taps,
                                       double* best_ms) {
    clear_error();
    SCIR_REQUIRE(plan != nullptr, SCIR_ERR_INVALID_ARG, "plan is NULL");
    if (plan->ntiles == 0 && !plan->tc) return SCIR_OK;
    SCIR_REQUIRE(x && taps && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    cudaStream_t st = as_stream(stream);
    // the tile lists are rebuilt: nothing queued on the stream may still read them
    SCIR_CUDA_TRY(cudaStreamSynchronize(st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SCIR_CUDA_TRY(cudaEventCreate(&e0));
    SCIR_CUDA_TRY(cudaEventCreate(&e1));
    auto time_plan = [&](float* ms) -> int {
        int rc = scir_fir_ragged_f32(plan, x, taps, y, stream);  // warm-up
        if (rc) return rc;
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2 && rc == SCIR_OK; ++r) rc = scir_fir_ragged_f32(plan, x, taps, y, stream);
        cudaEventRecord(e1, st);
        if (rc) return rc;
        cudaError_t ce = cudaEventSynchronize(e1);
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(ms, e0, e1);
        if (ce != cudaSuccess)
            return set_error(SCIR_ERR_CUDA, "ragged autotune timing: %s", cudaGetErrorString(ce));
        *ms *= 0.5f;
        return SCIR_OK;
    };
    // 1. the tap count from which CUDA-core tiles use 16 outputs per thread
    static const int kCand[] = {32, 64, 128, 256, 512, 1 << 30};
    int best = plan->v16_min_taps, rc = SCIR_OK;
    float best_t = 0.0f;
    for (int c : kCand) {
        rc = build_tiles(plan, c);
        float ms = 0.0f;
        if (!rc) rc = time_plan(&ms);
        if (rc) break;
        if (best_t == 0.0f || ms < best_t) {
            best_t = ms;
            best = c;
        }
    }
    if (!rc) rc = build_tiles(plan, best);
    // 2. the tap count from which signals go to the tensor cores
    if (!rc && plan->tc_form) {
        static const int kTc[] = {64, 128, 192, 256, 384, 512, 1024, 2048, 1 << 30};
        int best_tc = plan->tc_min_taps;
        float best_tc_t = 0.0f;
        for (int c : kTc) {
            rc = build_tc(plan, c);
            float ms = 0.0f;
            if (!rc) rc = time_plan(&ms);
            if (rc) break;
            if (best_tc_t == 0.0f || ms < best_tc_t) {
                best_tc_t = ms;
                best_tc = c;
            }
        }
        if (!rc) rc = build_tc(plan, best_tc);
        if (!rc) best_t = best_tc_t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (v16_min_taps) *v16_min_taps = best;
    if (best_ms) *best_ms = best_t;
    return SCIR_OK;
}

SCIR_API int scir_ragged_plan_tensor_cores(const scir_ragged_plan* plan, int* min_taps,
                                           int64_t* signals) {
    clear_error();
    SCIR_REQUIRE(plan != nullptr, SCIR_ERR_INVALID_ARG, "plan is NULL");
    int64_t cnt = 0;
    for (char c : plan->in_tc) cnt += c ? 1 : 0;
    if (min_taps) *min_taps = plan->tc_form ? plan->tc_min_taps : 0;
    if (signals) *signals = cnt;
    return SCIR_OK;
}

}  // extern "C"
