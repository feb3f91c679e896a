// Device and error layer of the library.
//
// The reference creates a CUDA context and JIT-loads its PTX module on every
// call (crates/scir-gpu/src/lib.rs:589-622, 814-834) and reports failures as
// GpuError (lib.rs:58-63).  Here kernels are compiled ahead of time for
// sm_103a, the runtime's primary context of the current device is used, the
// per-device facts are cached once, and errors are status codes plus a
// thread-local message.
#include "common.cuh"
#include "sm100.cuh"

#include <cudaTypedefs.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace scir {

namespace {
thread_local char g_last_error[1024] = {0};

constexpr int kMaxDevices = 64;
std::mutex g_dev_mutex;
DeviceInfo g_dev[kMaxDevices];
bool g_dev_ready[kMaxDevices] = {false};

// A trivial kernel whose presence proves an sm_103 image was loaded.
__global__ void probe_kernel() {}
}  // namespace

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

void clear_error() { g_last_error[0] = 0; }

static int init_device_locked(int dev) {
    DeviceInfo& d = g_dev[dev];
    cudaDeviceProp prop;
    SCIR_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    d.device = dev;
    d.sm_count = prop.multiProcessorCount;
    d.max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    d.cc_major = prop.major;
    d.cc_minor = prop.minor;
    d.l2_bytes = prop.l2CacheSize;
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, probe_kernel);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SCIR_ERR_NO_DEVICE,
                         "device %d (sm_%d%d) has no kernel image in this library "
                         "(built for sm_103a): %s",
                         dev, prop.major, prop.minor, cudaGetErrorString(e));
    }
    g_dev_ready[dev] = true;
    return SCIR_OK;
}

int current_device(const DeviceInfo** info) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SCIR_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(SCIR_ERR_NO_DEVICE, "device ordinal %d out of range", dev);
    if (!g_dev_ready[dev]) {
        std::lock_guard<std::mutex> lk(g_dev_mutex);
        if (!g_dev_ready[dev]) {
            int rc = init_device_locked(dev);
            if (rc != SCIR_OK) return rc;
        }
    }
    *info = &g_dev[dev];
    return SCIR_OK;
}

int upload_sync(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return SCIR_OK;
    static std::mutex mu;
    static cudaStream_t streams[kMaxDevices] = {};
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(SCIR_ERR_NO_DEVICE, "bad device %d", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!streams[dev]) SCIR_CUDA_TRY(cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking));
    SCIR_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, streams[dev]));
    SCIR_CUDA_TRY(cudaStreamSynchronize(streams[dev]));
    return SCIR_OK;
}

// Scratch memory comes from one stream-ordered pool per device that keeps
// freed memory (release threshold = unlimited), so repeated calls of the
// same size reuse it without mapping new pages; scir_release_scratch()
// returns the pool's unused memory to the device.  The pool is separate from
// the device's default pool, so the caller's own cudaMallocAsync settings
// are untouched.
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

int scratch_pool(cudaMemPool_t* out) {
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(SCIR_ERR_NO_DEVICE, "bad device %d", dev);
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        SCIR_CUDA_TRY(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = ~0ull;
        SCIR_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        g_pool[dev] = pool;
    }
    *out = g_pool[dev];
    return SCIR_OK;
}

int scratch_alloc(void** p, size_t bytes, cudaStream_t stream) {
    *p = nullptr;
    if (bytes == 0) return SCIR_OK;
    cudaMemPool_t pool = nullptr;
    int rc = scratch_pool(&pool);
    if (rc) return rc;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? SCIR_ERR_OOM : SCIR_ERR_CUDA,
                         "scratch allocation of %zu bytes failed: %s", bytes,
                         cudaGetErrorString(e));
    }
    return SCIR_OK;
}

void scratch_free(void* p, cudaStream_t stream) {
    if (p) cudaFreeAsync(p, stream);
}

static int tmap_encode(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base,
                       const uint64_t* dims, const uint64_t* strides_bytes, const uint32_t* box,
                       CUtensorMapSwizzle swizzle) {
    static std::mutex mu;
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!encode) {
            void* fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            SCIR_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                           cudaEnableDefault, &q));
            if (!fn || q != cudaDriverEntryPointSuccess)
                return set_error(SCIR_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        }
    }
    if (reinterpret_cast<uintptr_t>(base) & 15)
        return set_error(SCIR_ERR_ALIGN, "TMA needs a 16-byte aligned base address");
    cuuint64_t d[3], st[2];
    cuuint32_t b[3], es[3] = {1, 1, 1};
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
    }
    for (int i = 0; i + 1 < rank; ++i) {
        if (strides_bytes[i] & 15) return set_error(SCIR_ERR_ALIGN, "TMA row stride must be a multiple of 16 bytes");
        st[i] = strides_bytes[i];
    }
    CUresult r = encode(map, dtype, (cuuint32_t)rank, const_cast<void*>(base), d, st, b, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(SCIR_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SCIR_OK;
}

int make_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, const void* base, uint64_t dim0,
                 uint64_t dim1, uint64_t stride1_bytes, uint32_t box0, uint32_t box1,
                 CUtensorMapSwizzle swizzle) {
    const uint64_t dims[2] = {dim0, dim1}, strides[1] = {stride1_bytes};
    const uint32_t box[2] = {box0, box1};
    return tmap_encode(map, dtype, 2, base, dims, strides, box, swizzle);
}

int make_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, const void* base, uint64_t dim0,
                 uint64_t dim1, uint64_t dim2, uint64_t stride1_bytes, uint64_t stride2_bytes,
                 uint32_t box0, uint32_t box1, uint32_t box2, CUtensorMapSwizzle swizzle) {
    const uint64_t dims[3] = {dim0, dim1, dim2}, strides[2] = {stride1_bytes, stride2_bytes};
    const uint32_t box[3] = {box0, box1, box2};
    return tmap_encode(map, dtype, 3, base, dims, strides, box, swizzle);
}

// The error word is a file-scope device variable (zero when the module
// loads), so no entry point ever allocates device memory for it.  Host code
// cannot use the symbol itself as a device address: its address on each
// device is looked up once, with that device current.
namespace {
__device__ unsigned g_device_err_word = 0u;
std::mutex g_err_mutex;
unsigned* g_err_word[kMaxDevices] = {};
}  // namespace

unsigned* device_error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_err_mutex);
    if (!g_err_word[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_err_word) != cudaSuccess || !p) {
            cudaGetLastError();
            return nullptr;
        }
        g_err_word[dev] = static_cast<unsigned*>(p);
    }
    return g_err_word[dev];
}

int device_error_take(unsigned* code) {
    *code = 0;
    unsigned* w = device_error_word();
    if (!w) return set_error(SCIR_ERR_CUDA, "no device error word");
    SCIR_CUDA_TRY(cudaMemcpy(code, w, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (*code) {
        unsigned zero = 0;
        return upload_sync(w, &zero, sizeof(zero));
    }
    return SCIR_OK;
}

}  // namespace scir

extern "C" {

SCIR_API int scir_abi_version(void) { return SCIR_GB300_ABI_VERSION; }

SCIR_API const char* scir_status_string(int status) {
    switch (status) {
    case SCIR_OK: return "ok";
    case SCIR_ERR_INVALID_ARG: return "invalid argument";
    case SCIR_ERR_SHAPE: return "shape mismatch";
    case SCIR_ERR_ALIGN: return "misaligned pointer or stride";
    case SCIR_ERR_OOM: return "out of memory";
    case SCIR_ERR_CUDA: return "CUDA error";
    case SCIR_ERR_TIMEOUT: return "device wait timed out";
    case SCIR_ERR_UNSUPPORTED: return "unsupported";
    case SCIR_ERR_NO_DEVICE: return "no usable CUDA device";
    default: return "unknown status";
    }
}

SCIR_API int scir_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return SCIR_ERR_INVALID_ARG;
    strncpy(buf, scir::g_last_error, len - 1);
    buf[len - 1] = 0;
    return SCIR_OK;
}

SCIR_API int scir_device_count(int* count) {
    if (!count) return scir::set_error(SCIR_ERR_INVALID_ARG, "count is NULL");
    *count = 0;
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
        return scir::set_error(SCIR_ERR_NO_DEVICE, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    }
    return SCIR_OK;
}

SCIR_API int scir_device_errors(unsigned* code) {
    if (!code) return scir::set_error(SCIR_ERR_INVALID_ARG, "code is NULL");
    SCIR_CUDA_TRY(cudaDeviceSynchronize());
    return scir::device_error_take(code);
}

SCIR_API int scir_release_scratch(void) {
    scir::clear_error();
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= scir::kMaxDevices)
        return scir::set_error(SCIR_ERR_NO_DEVICE, "bad device %d", dev);
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lk(scir::g_pool_mu);
        pool = scir::g_pool[dev];
    }
    if (!pool) return SCIR_OK;
    SCIR_CUDA_TRY(cudaDeviceSynchronize());
    SCIR_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
    return SCIR_OK;
}

SCIR_API int scir_scratch_usage(uint64_t* reserved, uint64_t* used) {
    scir::clear_error();
    if (!reserved || !used) return scir::set_error(SCIR_ERR_INVALID_ARG, "NULL output");
    *reserved = *used = 0;
    int dev = 0;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= scir::kMaxDevices)
        return scir::set_error(SCIR_ERR_NO_DEVICE, "bad device %d", dev);
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lk(scir::g_pool_mu);
        pool = scir::g_pool[dev];
    }
    if (!pool) return SCIR_OK;
    cuuint64_t r = 0, u = 0;
    SCIR_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
    SCIR_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
    *reserved = r;
    *used = u;
    return SCIR_OK;
}

SCIR_API int scir_init(int device) {
    int count = 0;
    int rc = scir_device_count(&count);
    if (rc != SCIR_OK) return rc;
    if (device < 0 || device >= count)
        return scir::set_error(SCIR_ERR_INVALID_ARG, "device %d not in [0, %d)", device, count);
    SCIR_CUDA_TRY(cudaSetDevice(device));
    const scir::DeviceInfo* info = nullptr;
    rc = scir::current_device(&info);
    if (rc) return rc;
    // state that entry points would otherwise create on first use (and that
    // must not be created inside a stream capture)
    if (!scir::device_error_word())
        return scir::set_error(SCIR_ERR_CUDA, "device error word unavailable");
    cudaMemPool_t pool = nullptr;
    return scir::scratch_pool(&pool);
}

}  // extern "C"
