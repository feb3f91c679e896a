// Elementwise f32 kernels and 2-D resize behind the reference's DeviceArray
// operations (crates/scir-gpu/src/lib.rs): add_vec_f32 / add_scalar_f32 /
// mul_scalar_f32 (:629-725, out = a + b, a + alpha, a * alpha) and
// resize2d_f32 (:394-441, half-pixel centres, nearest or bilinear).
//
// The elementwise kernels are streaming: 16-byte loads and stores when every
// pointer is 16-byte aligned, grid-strided over a grid of a few waves.  Each
// result is one IEEE operation, so it equals the reference's CPU value bit for
// bit.  resize2d evaluates the reference's expression in its order with
// separately rounded f32 operations (no contraction into FMA), which makes the
// GPU image bit-identical to the CPU loop.
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>

namespace scir {
namespace {

enum ElemOp { kAddVec = 0, kAddScalar = 1, kMulScalar = 2 };

template <int OP>
__device__ __forceinline__ float elem(float a, float b, float alpha) {
    return OP == kAddVec ? __fadd_rn(a, b) : OP == kAddScalar ? __fadd_rn(a, alpha) : __fmul_rn(a, alpha);
}

template <int OP, bool VEC>
__global__ void __launch_bounds__(256)
elementwise_kernel(const float* __restrict__ a, const float* __restrict__ b, float alpha,
                   float* __restrict__ out, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (VEC) {
        const int64_t n4 = n / 4;
        for (int64_t q = i; q < n4; q += stride) {
            const float4 va = reinterpret_cast<const float4*>(a)[q];
            float4 vb = make_float4(0.f, 0.f, 0.f, 0.f);
            if (OP == kAddVec) vb = reinterpret_cast<const float4*>(b)[q];
            float4 r;
            r.x = elem<OP>(va.x, vb.x, alpha);
            r.y = elem<OP>(va.y, vb.y, alpha);
            r.z = elem<OP>(va.z, vb.z, alpha);
            r.w = elem<OP>(va.w, vb.w, alpha);
            reinterpret_cast<float4*>(out)[q] = r;
        }
        i += n4 * 4;  // the last n % 4 elements
        if (i < n) out[i] = elem<OP>(a[i], OP == kAddVec ? b[i] : 0.0f, alpha);
        return;
    }
    for (; i < n; i += stride) out[i] = elem<OP>(a[i], OP == kAddVec ? b[i] : 0.0f, alpha);
}

template <int OP>
int launch_elem(const float* a, const float* b, float alpha, float* out, int64_t n, void* stream) {
    clear_error();
    SCIR_REQUIRE(n >= 0, SCIR_ERR_INVALID_ARG, "negative length");
    if (n == 0) return SCIR_OK;
    SCIR_REQUIRE(a && out && (OP != kAddVec || b), SCIR_ERR_INVALID_ARG, "NULL buffer");
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(out) |
                       (OP == kAddVec ? reinterpret_cast<uintptr_t>(b) : 0)) & 15) == 0;
    const int64_t work = vec ? n / 4 + 1 : n;
    const int64_t grid = std::min<int64_t>(ceil_div(work, 256), (int64_t)info->sm_count * 8);
    cudaStream_t st = as_stream(stream);
    if (vec)
        elementwise_kernel<OP, true><<<(unsigned)grid, 256, 0, st>>>(a, b, alpha, out, n);
    else
        elementwise_kernel<OP, false><<<(unsigned)grid, 256, 0, st>>>(a, b, alpha, out, n);
    SCIR_LAUNCH_CHECK("elementwise_kernel");
    return SCIR_OK;
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// One output pixel per thread.  The source image is read through the
// read-only cache (neighbouring output pixels share source pixels).
template <int MODE>
__global__ void __launch_bounds__(256)
resize2d_kernel(const float* __restrict__ src, int64_t src_h, int64_t src_w,
                float* __restrict__ dst, int64_t out_h, int64_t out_w, float scale_x,
                float scale_y) {
    const int64_t total = out_h * out_w;
    const float mx = (float)src_w - 1.0f, my = (float)src_h - 1.0f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t dy = p / out_w, dx = p - dy * out_w;
        float sx = __fsub_rn(__fmul_rn(__fadd_rn((float)dx, 0.5f), scale_x), 0.5f);
        float sy = __fsub_rn(__fmul_rn(__fadd_rn((float)dy, 0.5f), scale_y), 0.5f);
        sx = sx < 0.0f ? 0.0f : sx;
        sy = sy < 0.0f ? 0.0f : sy;
        float v;
        if (MODE == 0) {
            const float fx = clampf(roundf(sx), 0.0f, mx), fy = clampf(roundf(sy), 0.0f, my);
            v = __ldg(src + (int64_t)fy * src_w + (int64_t)fx);
        } else {
            const float x0 = clampf(floorf(sx), 0.0f, mx), y0 = clampf(floorf(sy), 0.0f, my);
            const float x1 = __fadd_rn(x0, 1.0f) < mx ? __fadd_rn(x0, 1.0f) : mx;
            const float y1 = __fadd_rn(y0, 1.0f) < my ? __fadd_rn(y0, 1.0f) : my;
            const float fx = clampf(__fsub_rn(sx, x0), 0.0f, 1.0f);
            const float fy = clampf(__fsub_rn(sy, y0), 0.0f, 1.0f);
            const int64_t ix0 = (int64_t)x0, iy0 = (int64_t)y0, ix1 = (int64_t)x1, iy1 = (int64_t)y1;
            const float v00 = __ldg(src + iy0 * src_w + ix0), v10 = __ldg(src + iy0 * src_w + ix1);
            const float v01 = __ldg(src + iy1 * src_w + ix0), v11 = __ldg(src + iy1 * src_w + ix1);
            const float top = __fadd_rn(v00, __fmul_rn(__fsub_rn(v10, v00), fx));
            const float bot = __fadd_rn(v01, __fmul_rn(__fsub_rn(v11, v01), fx));
            v = __fadd_rn(top, __fmul_rn(__fsub_rn(bot, top), fy));
        }
        dst[p] = v;
    }
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" {

SCIR_API int scir_add_vec_f32(const float* a, const float* b, float* out, int64_t n, void* stream) {
    return launch_elem<kAddVec>(a, b, 0.0f, out, n, stream);
}

SCIR_API int scir_add_scalar_f32(const float* a, float alpha, float* out, int64_t n,
                                 void* stream) {
    return launch_elem<kAddScalar>(a, nullptr, alpha, out, n, stream);
}

SCIR_API int scir_mul_scalar_f32(const float* a, float alpha, float* out, int64_t n,
                                 void* stream) {
    return launch_elem<kMulScalar>(a, nullptr, alpha, out, n, stream);
}

SCIR_API int scir_resize2d_f32(const float* src, int64_t src_h, int64_t src_w, float* dst,
                               int64_t out_h, int64_t out_w, int mode, void* stream) {
    clear_error();
    SCIR_REQUIRE(mode == SCIR_RESIZE_NEAREST || mode == SCIR_RESIZE_BILINEAR, SCIR_ERR_INVALID_ARG,
                 "unknown resize mode %d", mode);
    SCIR_REQUIRE(src_h >= 1 && src_w >= 1, SCIR_ERR_SHAPE, "empty source image");
    SCIR_REQUIRE(out_h >= 0 && out_w >= 0, SCIR_ERR_INVALID_ARG, "negative output size");
    if (out_h == 0 || out_w == 0) return SCIR_OK;
    SCIR_REQUIRE(src && dst, SCIR_ERR_INVALID_ARG, "NULL buffer");
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    // IEEE single division on the host, as in the reference
    const float scale_x = (float)src_w / (float)out_w;
    const float scale_y = (float)src_h / (float)out_h;
    const int64_t grid = std::min<int64_t>(ceil_div(out_h * out_w, 256), (int64_t)info->sm_count * 8);
    cudaStream_t st = as_stream(stream);
    if (mode == SCIR_RESIZE_NEAREST)
        resize2d_kernel<0><<<(unsigned)grid, 256, 0, st>>>(src, src_h, src_w, dst, out_h, out_w,
                                                           scale_x, scale_y);
    else
        resize2d_kernel<1><<<(unsigned)grid, 256, 0, st>>>(src, src_h, src_w, dst, out_h, out_w,
                                                           scale_x, scale_y);
    SCIR_LAUNCH_CHECK("resize2d_kernel");
    return SCIR_OK;
}

}  // extern "C"
