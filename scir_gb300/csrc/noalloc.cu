// scir_sosfiltfilt_f32_noalloc: forward-backward SOS filtering that never
// allocates device memory.
//
// Why it exists: some callers of this library cannot allocate device memory
// at the moment they filter.  A real-time stream (audio, radar, sensor or SDR
// frames every few milliseconds) must not call cudaMalloc/cudaMallocAsync on
// its hot loop, because an allocation can synchronise the device, block
// behind other work or fail under memory pressure and miss the frame
// deadline.  Processes whose device memory is fully reserved up front by
// another framework's pool, and foreign-language hosts that forbid hidden
// allocations behind an FFI call, are in the same position.  This entry
// point does the same work as scir_sosfiltfilt_f32 but takes its scratch (the
// right-edge extension, batch x padlen floats) from a fixed file-scope device
// array instead of the stream-ordered allocator.
//
// Limits and rules:
//  - the array holds kNoallocScratchFloats floats (16 MiB); a call with
//    batch * padlen above that is rejected with SCIR_ERR_SHAPE before any
//    device work;
//  - the array lives in every device that loads the library until the process
//    exits;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current), and
//    the address of the library's device error word, which is a file-scope
//    device variable too; make that first call before any stream capture;
//  - every call shares the one array: calls that overlap on the GPU (other
//    streams, other host threads) race on it and must be serialised by the
//    caller.  Nothing in it needs to start at zero: each call writes every
//    scratch element it reads before reading it.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <mutex>

namespace scir {
namespace {

constexpr size_t kNoallocScratchFloats = size_t(4) << 20;  // 16 MiB

static __device__ __align__(256) float g_noalloc_scratch[kNoallocScratchFloats];

constexpr int kMaxDev = 64;
std::mutex g_noalloc_mutex;
float* g_noalloc_ptr[kMaxDev] = {};

// Device address of the array on the current device, looked up once per
// device with that device current.  The same first call also looks up the
// library's device error word (a file-scope device variable as well, which
// the FP32 pipeline kernels report bounded-wait timeouts to), so after the
// first call nothing on this path touches the CUDA runtime's symbol tables.
int noalloc_scratch(float** out) {
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    SCIR_REQUIRE(dev >= 0 && dev < kMaxDev, SCIR_ERR_NO_DEVICE, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return set_error(SCIR_ERR_CUDA, "cudaGetSymbolAddress(noalloc scratch): %s",
                             cudaGetErrorString(e));
        }
        if (!device_error_word())
            return set_error(SCIR_ERR_CUDA, "device error word unavailable");
        g_noalloc_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return SCIR_OK;
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" SCIR_API int scir_sosfiltfilt_f32_noalloc(const float* x, int64_t ld_x, int64_t batch,
                                                     int64_t n, const double* sos, int nsec,
                                                     int padtype, int64_t padlen, int precision,
                                                     float* y, int64_t ld_y, void* stream) {
    clear_error();
    SosCoef c;  // host memory only
    int64_t edge = 0;
    int rc = sosfiltfilt_check(x, ld_x, batch, n, sos, nsec, padtype, padlen, y, ld_y, &c, &edge);
    if (rc) return rc;
    SCIR_REQUIRE(edge == 0 || batch <= (int64_t)(kNoallocScratchFloats / (size_t)edge),
                 SCIR_ERR_SHAPE,
                 "batch * padlen = %lld * %lld exceeds the fixed scratch of %zu floats",
                 (long long)batch, (long long)edge, kNoallocScratchFloats);
    float* tail = nullptr;
    rc = noalloc_scratch(&tail);
    if (rc) return rc;
    if (batch == 0 || n == 0) return SCIR_OK;
    return launch_sosfiltfilt<float>(x, ld_x, batch, n, c, edge, padtype == SCIR_PAD_ODD,
                                     precision, y, ld_y, edge > 0 ? tail : nullptr,
                                     as_stream(stream));
}
