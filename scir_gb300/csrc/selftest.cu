// scir_selftest_pipeline: a small bulk-copy / mbarrier pipeline that checks,
// on the current device, the failure path every TMA pipeline of the library
// relies on.
//
// One CTA of two warps.  Warp 0 (one elected lane) copies chunks of 1,024
// floats from `in` into a 4-stage shared-memory ring with cp.async.bulk
// (completion on the stage's `full` mbarrier); warp 1 waits for each chunk
// with the library's bounded wait (mbar_wait), sums it into out[chunk] and
// releases the stage on its `empty` mbarrier.  The producer issues only the
// first `issue_chunks` of `n_chunks` chunks; when it stops early, the consumer's
// wait for the next chunk waits on a barrier that nothing will complete,
// gives up after `wait_limit_cycles` SM clock cycles, ORs kErrMbarTimeout
// into the device error word and returns -- exactly what a pipeline kernel
// does when a copy never lands.  No copy is in flight when either warp
// returns: the producer waits (bounded) for every chunk it issued before it
// leaves.  The host then reads SCIR_ERR_TIMEOUT from scir_device_errors() and
// the context stays usable.  Nothing in this kernel faults, traps or spins
// without a limit.
#include "common.cuh"
#include "sm100.cuh"

namespace scir {
namespace {

constexpr int kChunk = 1024;   // floats per chunk (4 KB)
constexpr int kRing = 4;       // stages

__global__ void __launch_bounds__(64, 1)
selftest_pipeline_kernel(const float* __restrict__ in, int64_t n_chunks, int64_t issue_chunks,
                         long long limit, float* __restrict__ out, unsigned* __restrict__ err) {
    __shared__ __align__(128) float ring[kRing][kChunk];
    __shared__ __align__(8) uint64_t full[kRing], empty[kRing];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kRing; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 32);
        }
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == 0) {
        if (lane != 0) return;
        int64_t issued = 0;
        bool ok = true;
        for (int64_t i = 0; i < issue_chunks && i < n_chunks; ++i) {
            const int s = (int)(i % kRing);
            // the stage's previous chunk must have been consumed
            if (i >= kRing && !mbar_wait(&empty[s], (uint32_t)(((i / kRing) - 1) & 1), limit)) {
                ok = false;
                break;
            }
            mbar_arrive_expect_tx(&full[s], kChunk * sizeof(float));
            bulk_load(ring[s], in + i * kChunk, kChunk * sizeof(float), &full[s]);
            issued = i + 1;
        }
        // every issued copy has landed before this thread leaves
        for (int64_t i = issued - kRing < 0 ? 0 : issued - kRing; i < issued; ++i)
            if (!mbar_wait(&full[i % kRing], (uint32_t)((i / kRing) & 1), limit)) ok = false;
        if (!ok) atomicOr(err, kErrMbarTimeout);
        return;
    }
    for (int64_t i = 0; i < n_chunks; ++i) {
        const int s = (int)(i % kRing);
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (uint32_t)((i / kRing) & 1), limit))) {
            if (lane == 0) atomicOr(err, kErrMbarTimeout);
            return;
        }
        float acc = 0.0f;
        for (int e = lane; e < kChunk; e += 32) acc += ring[s][e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[i] = acc;
        mbar_arrive(&empty[s]);
    }
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" SCIR_API int scir_selftest_pipeline(const float* in, int64_t n_chunks,
                                               int64_t issue_chunks, long long wait_limit_cycles,
                                               float* out, void* stream) {
    clear_error();
    SCIR_REQUIRE(n_chunks >= 0 && n_chunks <= (1 << 20), SCIR_ERR_INVALID_ARG,
                 "n_chunks %lld not in [0, 2^20]", (long long)n_chunks);
    SCIR_REQUIRE(issue_chunks >= 0 && issue_chunks <= n_chunks, SCIR_ERR_INVALID_ARG,
                 "issue_chunks %lld not in [0, n_chunks]", (long long)issue_chunks);
    SCIR_REQUIRE(wait_limit_cycles >= 1000 && wait_limit_cycles <= 4000000000LL,
                 SCIR_ERR_INVALID_ARG, "wait limit %lld cycles not in [1e3, 4e9]",
                 wait_limit_cycles);
    if (n_chunks > 0) SCIR_REQUIRE(in && out, SCIR_ERR_INVALID_ARG, "NULL buffer");
    SCIR_REQUIRE((reinterpret_cast<uintptr_t>(in) & 15) == 0, SCIR_ERR_ALIGN,
                 "in must be 16-byte aligned");
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    if (n_chunks == 0) return SCIR_OK;
    selftest_pipeline_kernel<<<1, 64, 0, as_stream(stream)>>>(in, n_chunks, issue_chunks,
                                                              wait_limit_cycles, out, err);
    SCIR_LAUNCH_CHECK("selftest_pipeline_kernel");
    return SCIR_OK;
}
