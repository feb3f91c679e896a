// Shared declarations for the sm_103a batched-filtering library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#include "scir_gb300.h"

namespace scir {

// Records `msg` as the calling thread's last error and returns `status`.
int set_error(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

// Per-device facts the launchers need; filled once per device.
struct DeviceInfo {
    int device = -1;
    int sm_count = 0;
    int max_smem_optin = 0;
    int cc_major = 0, cc_minor = 0;
    int l2_bytes = 0;
};

// Makes sure the current device is initialised and returns its info.
// Fails with SCIR_ERR_NO_DEVICE when no device or no sm_103 image exists.
int current_device(const DeviceInfo** info);

// Copies host -> device and returns only when the bytes are on the device
// (a private stream per device, synchronised), so kernels on any stream may
// read them afterwards.  Not for use inside a stream capture.
int upload_sync(void* dst, const void* src, size_t bytes);

// Stream-ordered scratch allocation (cudaMallocAsync on the caller's stream).
int scratch_alloc(void** p, size_t bytes, cudaStream_t stream);
// The library's stream-ordered scratch pool of the current device.
int scratch_pool(cudaMemPool_t* out);
void scratch_free(void* p, cudaStream_t stream);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace scir

#define SCIR_CUDA_TRY(expr)                                                          \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess)                                                       \
            return ::scir::set_error(SCIR_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, \
                                     cudaGetErrorString(_e), __FILE__, __LINE__);    \
    } while (0)

#define SCIR_LAUNCH_CHECK(name)                                                             \
    do {                                                                                    \
        cudaError_t _e = cudaGetLastError();                                                \
        if (_e != cudaSuccess)                                                              \
            return ::scir::set_error(SCIR_ERR_CUDA, "launch of %s failed: %s", name,        \
                                     cudaGetErrorString(_e));                               \
    } while (0)

#define SCIR_REQUIRE(cond, status, ...)                      \
    do {                                                     \
        if (!(cond)) return ::scir::set_error(status, __VA_ARGS__); \
    } while (0)
