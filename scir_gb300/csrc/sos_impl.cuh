// Channel-parallel second-order-section filtering (sosfilt / sosfiltfilt):
// the kernels and launchers, instantiated for f32 data in sos.cu and for
// f64 data in sos_f64.cu and sosfiltfilt_f64.cu (translation units that
// compile in parallel).
//
// The recursion is the reference's Direct Form II transposed cascade
// (crates/scir-iir-filters/src/filter.rs:50-61):
//   out = b0*prev + s1;  s1 = b1*prev - a1*out + s2;  s2 = b2*prev - a2*out
// evaluated per sample over every section, a0 taken as 1.
//
// One thread walks one channel.  A warp owns 32 channels; time advances in
// tiles of 32 samples that the warp moves between global memory and a
// [32 channels][33] shared tile with row-contiguous (coalesced) loads and
// stores, so each thread reads its channel's samples from shared memory
// without bank conflicts.  The next tile is prefetched into registers while
// the current one is filtered.
//
// PREC 0 (FP64_EXACT) rounds every product and sum separately in the
// reference's order: for f64 data the result is bit-identical to the
// reference.  PREC 1 uses FP64 FMA.  PREC 2 rounds the coefficients to FP32
// and keeps an FP32 state.  PREC 3 (FP32_COUPLED) runs each complex-pole
// section in coupled (modal) form with FP32 state: the state matrix
// [[sigma, -omega], [omega, sigma]] is applied as an increment with
// coefficients sigma-1 and omega that were computed in FP64, so the poles
// stay where FP64 puts them (a1, a2 rounded to FP32 move a pole 2e-4 from the
// unit circle by ~10 % of that distance); real-pole sections run FP32 DF2T.
// Initial and final states are exchanged in DF2T coordinates.
//
// sosfiltfilt (SciPy semantics with odd padding, or the reference's unpadded
// forward-backward) runs both passes in one thread per channel:
//   1. forward over the left extension 2*x0 - x[edge..1] from zi*ext[0]
//      (its outputs are trimmed, only the state is kept);
//   2. forward over x, writing the intermediate into y;
//   3. forward over the right extension 2*x[n-1] - x[n-2..n-1-edge], whose
//      inputs were saved in a [edge][batch] scratch before step 2 (so y may
//      alias x) and whose outputs overwrite them;
//   4. backward from zi*y1[last] over the right extension (outputs trimmed);
//   5. backward over y in descending tiles, writing the final result.
// The backward pass over the left extension produces only trimmed samples
// and is skipped.
#pragma once
#include "common.cuh"
#include "kernels.cuh"
#include "sos_math.cuh"

#include <type_traits>

namespace scir {
namespace {


// One sample through every section in order.
template <int NS, int PREC, typename A>
__device__ __forceinline__ A sos_step(const SosCoef& sc, A (&s1)[NS], A (&s2)[NS], A in) {
    A out = in;
#pragma unroll
    for (int s = 0; s < NS; ++s) out = sos_sec<PREC>(sc, s, s1[s], s2[s], out);
    return out;
}

template <typename T, int NS, int PREC>
__global__ void __launch_bounds__(32)
sosfilt_kernel(const T* __restrict__ x, int64_t ld_x, int64_t batch, int64_t n,
               const __grid_constant__ SosCoef sc,
               const double* __restrict__ zi, double* __restrict__ zf, T* __restrict__ y,
               int64_t ld_y, int64_t blk_rows, int64_t blk_len) {
    using A = typename AccT<PREC>::type;
    __shared__ T s[kTT][kTT + 1];
    const int lane = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * kTT;
    const int64_t ch = r0 + lane;
    // blocked row view (blk_rows > 0): row r is block r mod blk_rows, of
    // blk_len samples, of channel r div blk_rows; blk_rows is a multiple of
    // 32, so the warp's rows lie in one channel at stride blk_len
    if (blk_rows > 0) {
        x += (r0 / blk_rows) * ld_x + (r0 % blk_rows) * blk_len;
        y += (r0 / blk_rows) * ld_y + (r0 % blk_rows) * blk_len;
        ld_x = ld_y = blk_len;
    } else {
        x += r0 * ld_x;
        y += r0 * ld_y;
    }
    const int64_t rows = batch - r0;  // rows of this warp that exist (may exceed 32)
    A s1[NS], s2[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        s1[k] = A(0);
        s2[k] = A(0);
        if (zi && ch < batch && k < sc.nsec)
            state_in<PREC>(sc, k, zi[(ch * sc.nsec + k) * 2 + 0], zi[(ch * sc.nsec + k) * 2 + 1],
                           s1[k], s2[k]);
    }
    T nxt[kTT];
    tile_fetch(nxt, x, ld_x, 0, rows, n, 0, lane);
    for (int64_t t0 = 0; t0 < n; t0 += kTT) {
#pragma unroll
        for (int i = 0; i < kTT; ++i) s[i][lane] = nxt[i];
        __syncwarp();
        if (t0 + kTT < n) tile_fetch(nxt, x, ld_x, 0, rows, n, t0 + kTT, lane);
        const int tn = (int)((n - t0) < kTT ? (n - t0) : kTT);
        for (int t = 0; t < tn; ++t) {
            const A v = sos_step<NS, PREC>(sc, s1, s2, (A)s[lane][t]);
            s[lane][t] = (T)v;
        }
        __syncwarp();
        tile_store(s, y, ld_y, 0, rows, n, t0, lane);
        __syncwarp();
    }
    if (zf && ch < batch) {
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            if (k < sc.nsec) {
                double o1, o2;
                state_out<PREC>(sc, k, s1[k], s2[k], o1, o2);
                zf[(ch * sc.nsec + k) * 2 + 0] = o1;
                zf[(ch * sc.nsec + k) * 2 + 1] = o2;
            }
        }
    }
}

template <typename T, int NS, int PREC>
__global__ void __launch_bounds__(32)
sosfiltfilt_kernel(const T* __restrict__ x, int64_t ld_x, int64_t batch, int64_t n,
                   const __grid_constant__ SosCoef sc,
                   int64_t edge, int use_zi, T* __restrict__ y, int64_t ld_y,
                   T* __restrict__ tail) {
    using A = typename AccT<PREC>::type;
    __shared__ T s[kTT][kTT + 1];
    const int lane = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * kTT;
    const int64_t ch = r0 + lane;
    const bool live = ch < batch;
    const T* __restrict__ xr = x + (live ? ch : 0) * ld_x;
    A s1[NS], s2[NS];

    // save the right-extension inputs before y (which may alias x) is written
    const A xl = live ? (A)xr[0] : A(0);
    const A xe = live ? (A)xr[n - 1] : A(0);
    if (live) {
        for (int64_t i = 0; i < edge; ++i) tail[i * batch + ch] = (T)(A(2) * xe - (A)xr[n - 2 - i]);
    }
    // 1. left extension: state only
    {
        const A e0 = edge > 0 ? A(2) * xl - (live ? (A)xr[edge] : A(0)) : xl;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const bool on = k < sc.nsec && use_zi;
            const double* z = (PREC == 3 && sc.coupled[k]) ? sc.zc[k] : sc.zi[k];
            s1[k] = on ? (A)(z[0] * (double)e0) : A(0);
            s2[k] = on ? (A)(z[1] * (double)e0) : A(0);
        }
        for (int64_t j = 0; j < edge; ++j) {
            const A e = A(2) * xl - (live ? (A)xr[edge - j] : A(0));
            sos_step<NS, PREC>(sc, s1, s2, e);
        }
    }
    // 2. forward over x into y
    T nxt[kTT];
    tile_fetch(nxt, x, ld_x, r0, batch, n, 0, lane);
    for (int64_t t0 = 0; t0 < n; t0 += kTT) {
#pragma unroll
        for (int i = 0; i < kTT; ++i) s[i][lane] = nxt[i];
        __syncwarp();
        if (t0 + kTT < n) tile_fetch(nxt, x, ld_x, r0, batch, n, t0 + kTT, lane);
        const int tn = (int)((n - t0) < kTT ? (n - t0) : kTT);
        for (int t = 0; t < tn; ++t) s[lane][t] = (T)sos_step<NS, PREC>(sc, s1, s2, (A)s[lane][t]);
        __syncwarp();
        tile_store(s, y, ld_y, r0, batch, n, t0, lane);
        __syncwarp();
    }
    // 3. forward over the right extension
    A ylast = A(0);
    if (edge > 0) {
        for (int64_t i = 0; i < edge; ++i) {
            const A e = live ? (A)tail[i * batch + ch] : A(0);
            const A v = sos_step<NS, PREC>(sc, s1, s2, e);
            if (live) tail[i * batch + ch] = (T)v;
            ylast = v;
        }
    }
    __syncwarp();
    __threadfence_block();
    if (edge == 0) ylast = (live && n > 0) ? (A)y[ch * ld_y + n - 1] : A(0);
    // 4. backward over the right extension from zi * y1[last]
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const bool on = k < sc.nsec && use_zi;
        const double* z = (PREC == 3 && sc.coupled[k]) ? sc.zc[k] : sc.zi[k];
        s1[k] = on ? (A)(z[0] * (double)ylast) : A(0);
        s2[k] = on ? (A)(z[1] * (double)ylast) : A(0);
    }
    for (int64_t i = edge - 1; i >= 0; --i) {
        const A e = live ? (A)tail[i * batch + ch] : A(0);
        sos_step<NS, PREC>(sc, s1, s2, e);
    }
    // 5. backward over y, descending tiles
    if (n > 0) {
        const int64_t last0 = (n - 1) / kTT * kTT;
        tile_fetch(nxt, y, ld_y, r0, batch, n, last0, lane);
        for (int64_t t0 = last0; t0 >= 0; t0 -= kTT) {
#pragma unroll
            for (int i = 0; i < kTT; ++i) s[i][lane] = nxt[i];
            __syncwarp();
            if (t0 - kTT >= 0) tile_fetch(nxt, y, ld_y, r0, batch, n, t0 - kTT, lane);
            const int tn = (int)((n - t0) < kTT ? (n - t0) : kTT);
            for (int t = tn - 1; t >= 0; --t)
                s[lane][t] = (T)sos_step<NS, PREC>(sc, s1, s2, (A)s[lane][t]);
            __syncwarp();
            tile_store(s, y, ld_y, r0, batch, n, t0, lane);
            __syncwarp();
        }
    }
}

template <typename T, int NS, int PREC>
int run_sosfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                const double* zi, double* zf, T* y, int64_t ld_y, cudaStream_t st,
                int64_t blk_rows, int64_t blk_len) {
    const int64_t grid = ceil_div(batch, kTT);
    sosfilt_kernel<T, NS, PREC><<<(unsigned)grid, kTT, 0, st>>>(x, ld_x, batch, n, c, zi, zf, y, ld_y,
                                                               blk_rows, blk_len);
    SCIR_LAUNCH_CHECK("sosfilt_kernel");
    return SCIR_OK;
}

template <typename T, int NS, int PREC>
int run_sosfiltfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                    int64_t edge, int use_zi, T* y, int64_t ld_y, T* tail, cudaStream_t st) {
    const int64_t grid = ceil_div(batch, kTT);
    sosfiltfilt_kernel<T, NS, PREC><<<(unsigned)grid, kTT, 0, st>>>(x, ld_x, batch, n, c, edge,
                                                                      use_zi, y, ld_y, tail);
    SCIR_LAUNCH_CHECK("sosfiltfilt_kernel");
    return SCIR_OK;
}

// Section counts with a compiled kernel; others round up with identity sections.
#define SCIR_SOS_NS_LIST(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(12) X(16) X(24) X(32)

template <typename T, int PREC>
int dispatch_sosfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                     const double* zi, double* zf, T* y, int64_t ld_y, cudaStream_t st,
                     int64_t blk_rows, int64_t blk_len) {
#define SCIR_CASE(NS)                                                                          \
    if (c.nsec <= NS)                                                                          \
        return run_sosfilt<T, NS, PREC>(x, ld_x, batch, n, c, zi, zf, y, ld_y, st, blk_rows, \
                                        blk_len);
    SCIR_SOS_NS_LIST(SCIR_CASE)
#undef SCIR_CASE
    return set_error(SCIR_ERR_UNSUPPORTED, "more than %d sections", SCIR_SOS_MAX_SECTIONS);
}

template <typename T, int PREC>
int dispatch_sosfiltfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                         int64_t edge, int use_zi, T* y, int64_t ld_y, T* tail, cudaStream_t st) {
#define SCIR_CASE(NS)                                                                           \
    if (c.nsec <= NS)                                                                           \
        return run_sosfiltfilt<T, NS, PREC>(x, ld_x, batch, n, c, edge, use_zi, y, ld_y, tail, st);
    SCIR_SOS_NS_LIST(SCIR_CASE)
#undef SCIR_CASE
    return set_error(SCIR_ERR_UNSUPPORTED, "more than %d sections", SCIR_SOS_MAX_SECTIONS);
}

}  // namespace

template <typename T>
int launch_sosfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                   const double* zi, double* zf, int precision, T* y, int64_t ld_y,
                   cudaStream_t st, int64_t blk_rows, int64_t blk_len) {
    if (batch == 0) return SCIR_OK;
    if constexpr (std::is_same<T, float>::value)
        if (precision == SCIR_SOS_FP32 || precision == SCIR_SOS_FP32_COUPLED)
            return launch_sos_pipe(x, ld_x, batch, n, c, zi, zf, false, 0, 0, precision, y, ld_y,
                                   nullptr, st, blk_rows, blk_len);
    const int64_t br = blk_rows, bl = blk_len;
    switch (precision) {
    case SCIR_SOS_FP64_EXACT:
        return dispatch_sosfilt<T, 0>(x, ld_x, batch, n, c, zi, zf, y, ld_y, st, br, bl);
    case SCIR_SOS_FP64: return dispatch_sosfilt<T, 1>(x, ld_x, batch, n, c, zi, zf, y, ld_y, st, br, bl);
    default: break;
    }
    // f32 data with FP32 state went to the pipeline above: these kernels exist
    // for f64 data only
    if constexpr (!std::is_same<T, float>::value) {
        if (precision == SCIR_SOS_FP32)
            return dispatch_sosfilt<T, 2>(x, ld_x, batch, n, c, zi, zf, y, ld_y, st, br, bl);
        if (precision == SCIR_SOS_FP32_COUPLED)
            return dispatch_sosfilt<T, 3>(x, ld_x, batch, n, c, zi, zf, y, ld_y, st, br, bl);
    }
    return set_error(SCIR_ERR_INVALID_ARG, "unknown SOS precision %d", precision);
}

template <typename T>
int launch_sosfiltfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                       int64_t edge, int use_zi, int precision, T* y, int64_t ld_y, T* tail,
                       cudaStream_t st) {
    if (batch == 0 || n == 0) return SCIR_OK;
    if constexpr (std::is_same<T, float>::value)
        if (precision == SCIR_SOS_FP32 || precision == SCIR_SOS_FP32_COUPLED)
            return launch_sos_pipe(x, ld_x, batch, n, c, nullptr, nullptr, true, edge, use_zi,
                                   precision, y, ld_y, tail, st);
    switch (precision) {
    case SCIR_SOS_FP64_EXACT:
        return dispatch_sosfiltfilt<T, 0>(x, ld_x, batch, n, c, edge, use_zi, y, ld_y, tail, st);
    case SCIR_SOS_FP64:
        return dispatch_sosfiltfilt<T, 1>(x, ld_x, batch, n, c, edge, use_zi, y, ld_y, tail, st);
    default: break;
    }
    if constexpr (!std::is_same<T, float>::value) {
        if (precision == SCIR_SOS_FP32)
            return dispatch_sosfiltfilt<T, 2>(x, ld_x, batch, n, c, edge, use_zi, y, ld_y, tail, st);
        if (precision == SCIR_SOS_FP32_COUPLED)
            return dispatch_sosfiltfilt<T, 3>(x, ld_x, batch, n, c, edge, use_zi, y, ld_y, tail, st);
    }
    return set_error(SCIR_ERR_INVALID_ARG, "unknown SOS precision %d", precision);
}

}  // namespace scir
