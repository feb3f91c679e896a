// Channel-parallel SOS filtering with FP32 state (FP32 and FP32_COUPLED),
// the cascade split across the warps of a CTA.
//
// One thread per channel leaves a channel's samples on one warp: with 16,384
// channels that is 512 warps, under one per scheduler, and each warp then
// runs every section of every sample alone (measured on GB300: the time of a
// 2,048-channel launch equals that of a 16,384-channel one).  Here a CTA of
// G warps owns 32 channels and warp w owns sections [w*SPW, (w+1)*SPW): a
// tile of 32 channels x 32 samples moves through the warps in place in a
// shared-memory ring, so the G warps filter G different tiles at once and
// every scheduler gets several warps.
//
// Ring protocol (kRing slots, slot r holds global tile g with g % kRing = r):
//   warp 0 loads tile g + kAhead (cp.async, or computed extension samples)
//   once the last warp has released the slot (tile g + kAhead - kRing),
//   then filters tile g with its sections and arrives on done[0][r];
//   warp w waits on done[w-1][r], filters, arrives on done[w][r];
//   the last warp stores the tile (or its extension outputs) before arriving.
// Every lane arrives (barrier count 32) and every wait is bounded; a timeout
// sets the device error word and the warp stops filtering.
//
// Streams.  sosfilt is one stream x -> y.  sosfiltfilt (SciPy odd padding or
// none) is a forward stream over [left extension, x, right extension] and a
// backward stream over [reversed right-extension outputs, reversed y]:
//   forward:  samples j < edge are 2*x0 - x[edge - j] (outputs dropped),
//             edge <= j < edge+n are x (outputs -> y), the rest are the right
//             extension 2*x[n-1] - x[n-2-i], saved in a [edge][batch] scratch
//             before y (which may alias x) is written (outputs -> the
//             scratch); initial state zi * (first sample);
//   backward: samples j < edge are the right-extension outputs reversed
//             (outputs dropped), the rest are y reversed (outputs -> y);
//             initial state zi * (last forward output).
// The backward pass over the left extension produces only trimmed samples and
// is skipped.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"
#include "sos_math.cuh"

#include <type_traits>

namespace scir {
namespace {

// kTT (32, from sos_math.cuh): channels per CTA = samples per tile
constexpr int kRing = 8;    // tile slots
constexpr int kLd = kTT + 1;

template <int NS>
struct PipeShape {
    static constexpr int G = NS < 4 ? NS : 4;  // warps
    static constexpr int SPW = NS / G;         // sections per warp
    static constexpr int kAhead = kRing - G;   // tiles loaded ahead of warp 0
    static_assert(NS % G == 0, "section count must divide over the warps");
};

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

enum StreamKind { kSos = 0, kFwd = 1, kBwd = 2 };

// The coefficients of a warp's sections (fixed for the launch) live in
// registers as the halves of packed pairs: section 2i in .x, 2i+1 in .y.
// A coupled half holds sigma-1, omega, -omega, C1, C2, b0; a DF2T half
// holds b0, b1, b2, -a1, -a2.  The negated values are exact.
struct PairSec {
    float2 f[6];
};

__device__ __forceinline__ void put_sec(PairSec& p, int half, const SosCoef& sc, int s,
                                        bool coupled) {
    float v[6];
    if (coupled) {
        v[0] = sc.cp[s][0];
        v[1] = sc.cp[s][1];
        v[2] = -sc.cp[s][1];
        v[3] = sc.cp[s][2];
        v[4] = sc.cp[s][3];
        v[5] = sc.cp[s][4];
    } else {
        v[0] = sc.cf[s][0];
        v[1] = sc.cf[s][1];
        v[2] = sc.cf[s][2];
        v[3] = -sc.cf[s][3];
        v[4] = -sc.cf[s][4];
        v[5] = 0.0f;
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        if (half == 0) p.f[j].x = v[j];
        else p.f[j].y = v[j];
    }
}

// The arithmetic of sos_sec (PREC 2 / 3) for one section, on half H of its
// pair.  FORM: 0 = FP32 DF2T, 1 = coupled, 2 = chosen per section (a warp
// whose sections mix real and complex poles).
template <int FORM, int H>
__device__ __forceinline__ float sec_step(const PairSec& r, bool coupled, float& s1, float& s2,
                                          float prev) {
    auto c = [&](int j) { return H == 0 ? r.f[j].x : r.f[j].y; };
    float out;
    if (FORM == 1 || (FORM == 2 && coupled)) {
        const float u = s1, v = s2;
        out = fmaf(c(3), u, fmaf(c(4), v, c(5) * prev));
        s1 = u + fmaf(c(0), u, fmaf(c(2), v, prev));
        s2 = v + fmaf(c(1), u, c(0) * v);
    } else {
        out = fmaf(c(0), prev, s1);
        s1 = fmaf(c(3), out, fmaf(c(1), prev, s2));
        s2 = fmaf(c(4), out, c(2) * prev);
    }
    return out;
}

// Two sections of a warp run one sample apart in one packed (f32x2) step:
// the first section at sample p (x = input) and the second at sample p - 1
// (x = the first section's previous output).  Each half performs exactly the
// operations of sec_step in the same order (fma.rn / mul.rn / add.rn per
// element), so the outputs are bit-identical to the scalar cascade with half
// the instructions.  S1 / S2 hold (s1, s2) of the two sections; FORM 0 or 1.
template <int FORM>
__device__ __forceinline__ float2 pair_step(const PairSec& r, float2& S1, float2& S2, float2 X) {
    float2 Y;
    if (FORM == 1) {
        const float2 U = S1, V = S2;
        Y = __ffma2_rn(r.f[3], U, __ffma2_rn(r.f[4], V, __fmul2_rn(r.f[5], X)));
        S1 = __fadd2_rn(U, __ffma2_rn(r.f[0], U, __ffma2_rn(r.f[2], V, X)));
        S2 = __fadd2_rn(V, __ffma2_rn(r.f[1], U, __fmul2_rn(r.f[0], V)));
    } else {
        Y = __ffma2_rn(r.f[0], X, S1);
        S1 = __ffma2_rn(r.f[3], Y, __ffma2_rn(r.f[1], X, S2));
        S2 = __ffma2_rn(r.f[4], Y, __fmul2_rn(r.f[2], X));
    }
    return Y;
}

struct PipeArgs {
    const float* x;
    int64_t ld_x;
    float* y;
    int64_t ld_y;
    int64_t batch, n, edge;
    const double* zi;  // sosfilt: [batch][nsec][2] or null
    double* zf;        // sosfilt: [batch][nsec][2] or null
    float* tail;       // sosfiltfilt: [edge][batch]
    int use_zi;        // sosfiltfilt: odd padding with sosfilt_zi
    unsigned* err;
};

template <int NS, int PREC, bool FF>
__global__ void __launch_bounds__(32 * PipeShape<NS>::G, 4)
sos_pipe_kernel(const __grid_constant__ SosCoef sc, const PipeArgs a) {
    constexpr int G = PipeShape<NS>::G, SPW = PipeShape<NS>::SPW, kAhead = PipeShape<NS>::kAhead;
    __shared__ float tiles[kRing][kTT][kLd];  // [slot][row = channel][time]
    __shared__ uint64_t done[G][kRing];
    __shared__ float ylast_s[kTT];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * kTT;
    const int64_t ch = r0 + lane;
    const bool live = ch < a.batch;
    const int64_t n = a.n, edge = a.edge;
    const float* __restrict__ xr = a.x + (live ? ch : 0) * a.ld_x;

    if (threadIdx.x == 0) {
        for (int w = 0; w < G; ++w)
            for (int r = 0; r < kRing; ++r) mbar_init(&done[w][r], 32);
        fence_barrier_init();
    }
    // sosfiltfilt: save the right-extension inputs before y (which may alias
    // x) is written, and read the first forward sample
    float first = 0.0f;
    if (FF) {
        if (warp == 0 && live) {
            const float xe = xr[n - 1];
            for (int64_t i = 0; i < edge; ++i) a.tail[i * a.batch + ch] = 2.0f * xe - xr[n - 2 - i];
        }
        if (live) first = edge > 0 ? 2.0f * xr[0] - xr[edge] : xr[0];
        __threadfence_block();
    }
    __syncthreads();

    float s1[SPW], s2[SPW];
    constexpr int NP = (SPW + 1) / 2;  // coefficient pairs of this warp
    PairSec pc[NP];
    bool cpl[SPW];
#pragma unroll
    for (int i = 0; i < SPW; ++i) {
        const int s = warp * SPW + i;
        // the coupled form serves complex-pole sections in FP32_COUPLED only
        cpl[i] = PREC == 3 && sc.coupled[s] != 0;
        put_sec(pc[i / 2], i % 2, sc, s, cpl[i]);
        if (i % 2 == 0 && i + 1 == SPW) put_sec(pc[i / 2], 1, sc, s, cpl[i]);  // unused .y half
        s1[i] = 0.0f;
        s2[i] = 0.0f;
        if (!FF && a.zi && live && s < sc.nsec)
            state_in<PREC>(sc, s, a.zi[(ch * sc.nsec + s) * 2 + 0], a.zi[(ch * sc.nsec + s) * 2 + 1],
                           s1[i], s2[i]);
        if (FF && a.use_zi && s < sc.nsec) {
            const double* z = (PREC == 3 && sc.coupled[s]) ? sc.zc[s] : sc.zi[s];
            s1[i] = (float)(z[0] * (double)first);
            s2[i] = (float)(z[1] * (double)first);
        }
    }

    // this warp's section form, fixed for the launch
    int form = 0;
    if (PREC == 3) {
        int nc = 0;
#pragma unroll
        for (int i = 0; i < SPW; ++i) nc += cpl[i] ? 1 : 0;
        form = nc == SPW ? 1 : nc == 0 ? 0 : 2;
    }
    // section i of the warp on one sample (i is a constant after unrolling)
    auto step_i = [&](auto formc, int i, float v) {
        constexpr int FORM = decltype(formc)::value;
        return (i & 1) ? sec_step<FORM, 1>(pc[i >> 1], cpl[i], s1[i], s2[i], v)
                       : sec_step<FORM, 0>(pc[i >> 1], cpl[i], s1[i], s2[i], v);
    };
    // Filters tn samples of this lane's channel in place through the warp's
    // sections (a full tile fully unrolled, so the shared loads run ahead).
    // Full tiles of an all-coupled warp with 2-4 sections go through its
    // section pairs, one pass over the tile per pair: sample 0 of the first
    // section alone, then 31 packed steps, then sample 31 of the second
    // section alone.  Measured on GB300 (16,384 x 131,072, 8 sections): the
    // coupled cascade 9.65 -> 9.12 ms; the DF2T form, whose two-operation
    // recurrence the lockstep lengthens, 6.17 -> 9.44 ms, so it stays scalar.
    // More sections per warp would spill registers.
    constexpr bool kPaired = SPW >= 2 && SPW <= 4;
    auto filter_tile = [&](auto formc, float(*t)[kLd], int tn) {
        constexpr int FORM = decltype(formc)::value;
        if (FORM == 1 && kPaired && tn == kTT) {
#pragma unroll
            for (int i = 0; i < SPW / 2; ++i) {
                const int sa = 2 * i, sb = 2 * i + 1;
                float2 S1 = make_float2(s1[sa], s1[sb]), S2 = make_float2(s2[sa], s2[sb]);
                float ya = sec_step<FORM, 0>(pc[i], cpl[sa], S1.x, S2.x, t[lane][0]);
#pragma unroll
                for (int p = 1; p < kTT; ++p) {
                    const float2 Y = pair_step<FORM>(pc[i], S1, S2, make_float2(t[lane][p], ya));
                    t[lane][p - 1] = Y.y;
                    ya = Y.x;
                }
                t[lane][kTT - 1] = sec_step<FORM, 1>(pc[i], cpl[sb], S1.y, S2.y, ya);
                s1[sa] = S1.x;
                s1[sb] = S1.y;
                s2[sa] = S2.x;
                s2[sb] = S2.y;
            }
            if (SPW % 2) {
#pragma unroll
                for (int p = 0; p < kTT; ++p)
                    t[lane][p] = sec_step<FORM, 0>(pc[NP - 1], cpl[SPW - 1], s1[SPW - 1],
                                                   s2[SPW - 1], t[lane][p]);
            }
        } else if (tn == kTT) {
#pragma unroll
            for (int p = 0; p < kTT; ++p) {
                float v = t[lane][p];
#pragma unroll
                for (int i = 0; i < SPW; ++i) v = step_i(formc, i, v);
                t[lane][p] = v;
            }
        } else {
            for (int p = 0; p < tn; ++p) {
                float v = t[lane][p];
#pragma unroll
                for (int i = 0; i < SPW; ++i) v = step_i(formc, i, v);
                t[lane][p] = v;
            }
        }
    };

    bool ok = true;
    int64_t gbase = 0;  // global tile index of the stream's first tile

    // Loads stream tile k of stream KIND (length L) into slot `slot` (warp 0).
    // Full tiles inside the copied part of the stream take one cp.async per
    // row along a running row pointer; edge tiles check every element.
    auto load_tile = [&](auto kindc, int64_t L, int64_t k, int slot) {
        constexpr int KIND = decltype(kindc)::value;
        const int64_t j0 = k * kTT, j = j0 + lane;  // this lane's stream position
        float(*t)[kLd] = tiles[slot];
        const bool rows_full = r0 + kTT <= a.batch;
        if (KIND == kSos && rows_full && j0 + kTT <= L) {
            const float* p = a.x + r0 * a.ld_x + j;
#pragma unroll 8
            for (int i = 0; i < kTT; ++i, p += a.ld_x) cp_async4(&t[i][lane], p, true);
        } else if (KIND == kFwd && rows_full && j0 >= edge && j0 + kTT <= edge + n) {
            const float* p = a.x + r0 * a.ld_x + (j - edge);
#pragma unroll 8
            for (int i = 0; i < kTT; ++i, p += a.ld_x) cp_async4(&t[i][lane], p, true);
        } else if (KIND == kBwd && rows_full && j0 >= edge && j0 + kTT <= L) {
            const float* p = a.y + r0 * a.ld_y + (n - 1 - (j - edge));
#pragma unroll 8
            for (int i = 0; i < kTT; ++i, p += a.ld_y) cp_async4(&t[i][lane], p, true);
        } else {
            for (int i = 0; i < kTT; ++i) {
                const int64_t row = r0 + i;
                const bool vr = row < a.batch && j < L;
                const float* rx = a.x + (row < a.batch ? row : 0) * a.ld_x;
                if (KIND == kSos) {
                    cp_async4(&t[i][lane], vr ? rx + j : a.x, vr);
                } else if (KIND == kFwd) {
                    if (j >= edge && j < edge + n) {
                        cp_async4(&t[i][lane], vr ? rx + (j - edge) : a.x, vr);
                    } else {
                        float v = 0.0f;
                        if (vr && j < edge) v = 2.0f * rx[0] - rx[edge - j];
                        else if (vr) v = a.tail[(j - edge - n) * a.batch + row];
                        t[i][lane] = v;
                    }
                } else {
                    if (j >= edge) {
                        const float* ry = a.y + (row < a.batch ? row : 0) * a.ld_y;
                        cp_async4(&t[i][lane], vr ? ry + (n - 1 - (j - edge)) : a.y, vr);
                    } else {
                        t[i][lane] = vr ? a.tail[(edge - 1 - j) * a.batch + row] : 0.0f;
                    }
                }
            }
        }
        cp_async_commit();
    };

    // Writes the outputs of stream tile k (last warp), with the same fast path.
    auto store_tile = [&](auto kindc, int64_t L, int64_t k, int slot) {
        constexpr int KIND = decltype(kindc)::value;
        const int64_t j0 = k * kTT, j = j0 + lane;
        float(*t)[kLd] = tiles[slot];
        const bool rows_full = r0 + kTT <= a.batch;
        float* q = nullptr;
        if (KIND == kSos && rows_full && j0 + kTT <= L) q = a.y + r0 * a.ld_y + j;
        if (KIND == kFwd && rows_full && j0 >= edge && j0 + kTT <= edge + n)
            q = a.y + r0 * a.ld_y + (j - edge);
        if (KIND == kBwd && rows_full && j0 >= edge && j0 + kTT <= L)
            q = a.y + r0 * a.ld_y + (n - 1 - (j - edge));
        if (q) {
#pragma unroll 8
            for (int i = 0; i < kTT; ++i, q += a.ld_y) *q = t[i][lane];
            // the forward stream's last output seeds the backward pass (edge == 0)
            if (KIND == kFwd && j == L - 1)
                for (int i = 0; i < kTT; ++i) ylast_s[i] = t[i][lane];
            return;
        }
        for (int i = 0; i < kTT; ++i) {
            const int64_t row = r0 + i;
            if (row >= a.batch || j >= L) continue;
            const float v = t[i][lane];
            float* ry = a.y + row * a.ld_y;
            if (KIND == kSos) {
                ry[j] = v;
            } else if (KIND == kFwd) {
                if (j >= edge && j < edge + n) ry[j - edge] = v;
                else if (j >= edge + n) a.tail[(j - edge - n) * a.batch + row] = v;
                if (j == L - 1) ylast_s[i] = v;
            } else if (j >= edge) {
                ry[n - 1 - (j - edge)] = v;
            }
        }
    };

    // One stream through the warp pipeline.
    auto run = [&](auto kindc, int64_t L) {
        const int64_t ntiles = (L + kTT - 1) / kTT;
        if (warp == 0)
            for (int64_t k = 0; k < kAhead; ++k) {
                if (k < ntiles) load_tile(kindc, L, k, (int)((gbase + k) % kRing));
                else cp_async_commit();
            }
        for (int64_t k = 0; k < ntiles; ++k) {
            const int64_t g = gbase + k;
            const int slot = (int)(g % kRing);
            const uint32_t par = (uint32_t)((g / kRing) & 1);
            if (warp == 0) {
                cp_async_wait<kAhead - 1>();  // tile k has landed
                __syncwarp();
            } else if (ok) {
                ok = mbar_wait(&done[warp - 1][slot], par);
                if (!ok && lane == 0) atomicOr(a.err, kErrMbarTimeout);
            }
            if (ok) {
                const int tn = (int)((L - k * kTT) < kTT ? (L - k * kTT) : kTT);
                float(*t)[kLd] = tiles[slot];
                if (form == 1) filter_tile(std::integral_constant<int, 1>(), t, tn);
                else if (form == 0) filter_tile(std::integral_constant<int, 0>(), t, tn);
                else filter_tile(std::integral_constant<int, 2>(), t, tn);
                __syncwarp();
                if (warp == G - 1) {
                    store_tile(kindc, L, k, slot);
                    __syncwarp();
                }
            }
            mbar_arrive(&done[warp][slot]);
            if (warp == 0) {
                // refill: tile k + kAhead goes into the slot of tile g + kAhead - kRing
                const int64_t kk = k + kAhead;
                if (kk < ntiles) {
                    const int64_t gp = g + kAhead - kRing;
                    if (ok && gp >= 0) {
                        ok = mbar_wait(&done[G - 1][(int)(gp % kRing)], (uint32_t)((gp / kRing) & 1));
                        if (!ok && lane == 0) atomicOr(a.err, kErrMbarTimeout);
                    }
                    load_tile(kindc, L, kk, (int)((g + kAhead) % kRing));
                } else {
                    cp_async_commit();
                }
            }
        }
        if (warp == 0) cp_async_wait<0>();
        gbase += ntiles;
        __threadfence_block();
        __syncthreads();
    };

    if (!FF) {
        run(std::integral_constant<int, kSos>(), n);
        if (a.zf && live) {
#pragma unroll
            for (int i = 0; i < SPW; ++i) {
                const int s = warp * SPW + i;
                if (s < sc.nsec) {
                    double o1, o2;
                    state_out<PREC>(sc, s, s1[i], s2[i], o1, o2);
                    a.zf[(ch * sc.nsec + s) * 2 + 0] = o1;
                    a.zf[(ch * sc.nsec + s) * 2 + 1] = o2;
                }
            }
        }
        return;
    }
    run(std::integral_constant<int, kFwd>(), n + 2 * edge);
    // backward initial state from the last forward output
    const float yl = ylast_s[lane];
#pragma unroll
    for (int i = 0; i < SPW; ++i) {
        const int s = warp * SPW + i;
        const bool on = a.use_zi && s < sc.nsec;
        const double* z = (PREC == 3 && sc.coupled[s]) ? sc.zc[s] : sc.zi[s];
        s1[i] = on ? (float)(z[0] * (double)yl) : 0.0f;
        s2[i] = on ? (float)(z[1] * (double)yl) : 0.0f;
    }
    run(std::integral_constant<int, kBwd>(), n + edge);
}

// Section counts with a compiled pipeline; others round up with identity
// sections (every count divides over the warps).
#define SCIR_PIPE_NS_LIST(X) X(1) X(2) X(3) X(4) X(8) X(12) X(16) X(24) X(32)

template <int NS, int PREC, bool FF>
int run_pipe(const SosCoef& c, const PipeArgs& a, cudaStream_t st) {
    const int64_t grid = ceil_div(a.batch, kTT);
    // The CTAs are few (one per 32 channels) and each holds a 34 KB ring:
    // with the default carveout only two fit an SM (measured: 16,384 channels
    // ran in two waves), so ask for the largest shared-memory carveout.
    SCIR_CUDA_TRY(cudaFuncSetAttribute(sos_pipe_kernel<NS, PREC, FF>,
                                       cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    sos_pipe_kernel<NS, PREC, FF><<<(unsigned)grid, 32 * PipeShape<NS>::G, 0, st>>>(c, a);
    SCIR_LAUNCH_CHECK("sos_pipe_kernel");
    return SCIR_OK;
}

template <int PREC, bool FF>
int dispatch_pipe(const SosCoef& c, const PipeArgs& a, cudaStream_t st) {
#define SCIR_CASE(NS) \
    if (c.nsec <= NS) return run_pipe<NS, PREC, FF>(c, a, st);
    SCIR_PIPE_NS_LIST(SCIR_CASE)
#undef SCIR_CASE
    return set_error(SCIR_ERR_UNSUPPORTED, "more than %d sections", SCIR_SOS_MAX_SECTIONS);
}

}  // namespace

int launch_sos_pipe(const float* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                    const double* zi, double* zf, bool filtfilt, int64_t edge, int use_zi,
                    int precision, float* y, int64_t ld_y, float* tail, cudaStream_t st) {
    if (batch == 0 || n == 0) return SCIR_OK;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    PipeArgs a{x, ld_x, y, ld_y, batch, n, edge, zi, zf, tail, use_zi, err};
    const bool coupled = precision == SCIR_SOS_FP32_COUPLED;
    if (filtfilt) return coupled ? dispatch_pipe<3, true>(c, a, st) : dispatch_pipe<2, true>(c, a, st);
    return coupled ? dispatch_pipe<3, false>(c, a, st) : dispatch_pipe<2, false>(c, a, st);
}

}  // namespace scir
