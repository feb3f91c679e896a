// Channel-parallel SOS filtering with FP32 state (FP32 and FP32_COUPLED),
// the cascade split across the warps of a CTA.
//
// One thread per channel leaves a channel's samples on one warp: with 16,384
// channels that is 512 warps, under one per scheduler, and each warp then
// runs every section of every sample alone (measured on GB300: the time of a
// 2,048-channel launch equals that of a 16,384-channel one).  Here a CTA of
// G warps owns 64 channels and warp w owns sections [w*SPW, (w+1)*SPW): a
// tile of 64 channels x 32 samples moves through the warps in place in a
// shared-memory ring, so the G warps filter G different tiles at once and
// every scheduler gets several warps.  Lane l carries channels l and l + 32
// as the two halves of packed f32x2 operations: every packed FMA applies one
// section to two independent channels, so each warp has two independent
// recursions per lane to interleave (the coefficients are duplicated in both
// halves of their register pairs).  Each half performs exactly the scalar
// section update's operations in the same order, so the results equal those
// of one thread per channel bit for bit.

// Ring protocol (kRing = G + 4 slots, slot r holds global tile g with g % kRing = r):
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

// kTT (32, from sos_math.cuh): samples per tile = lanes
constexpr int kCH = 2 * kTT;  // channels per CTA: lane l owns rows l and l + 32
constexpr int kLd = kTT + 1;

template <int NS, int PREC, bool FF>
struct PipeShape {
    // warps: up to 4 sections per warp (the duplicated coefficient pairs of
    // 4 sections take 48 registers).  The DF2T sosfilt of 5 - 8 sections
    // runs on 2 warps of 4 sections, 64-thread CTAs (16,384 x 131,072 on
    // GB300: 5.63 ms against 6.41 with 4 warps of 2); the coupled form and
    // sosfiltfilt measured slower that way (8.99 vs 8.64, 21.0 vs 18.8 ms).
    static constexpr int G = NS < 4 ? NS : (NS == 8 && PREC == 2 && !FF) ? 2 : NS <= 12 ? 4 : 8;
    static constexpr int SPW = NS / G;         // sections per warp
    static constexpr int kRing = G + 4;        // tile slots
    static constexpr int kAhead = kRing - G;   // tiles loaded ahead of warp 0
    static_assert(NS % G == 0, "section count must divide over the warps");
    static_assert(SPW <= 4, "at most 4 sections per warp");
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
// registers, each duplicated in both halves of a pair (one section, two
// channels).  A coupled section holds sigma-1, omega, -omega, C1, C2, b0; a
// DF2T section holds b0, b1, b2, -a1, -a2.  The negated values are exact.
struct PackSec {
    float2 f[6];
};

__device__ __forceinline__ void put_sec(PackSec& p, const SosCoef& sc, int s, bool coupled) {
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
    for (int j = 0; j < 6; ++j) p.f[j] = make_float2(v[j], v[j]);
}

// One section on two channels (the halves).  Coupled (COUPLED = true):
//   out = C1*u + C2*v + b0*x;  u += (sigma-1)*u - omega*v + x;  v += omega*u + (sigma-1)*v
// DF2T: out = b0*x + s1;  s1 = b1*x - a1*out + s2;  s2 = b2*x - a2*out.
// Each half rounds exactly like the scalar fmaf / mul / add sequence.
template <bool COUPLED>
__device__ __forceinline__ float2 pack_step(const PackSec& r, float2& S1, float2& S2, float2 X) {
    float2 Y;
    if (COUPLED) {
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
    int64_t blk_rows, blk_len;  // sosfilt: blocked row view (0: plain rows)
};

template <int NS, int PREC, bool FF>
__global__ void __launch_bounds__(32 * PipeShape<NS, PREC, FF>::G, 2)
sos_pipe_kernel(const __grid_constant__ SosCoef sc, const PipeArgs a) {
    constexpr int G = PipeShape<NS, PREC, FF>::G, SPW = PipeShape<NS, PREC, FF>::SPW;
    constexpr int kRing = PipeShape<NS, PREC, FF>::kRing, kAhead = PipeShape<NS, PREC, FF>::kAhead;
    extern __shared__ __align__(16) float smem_tiles[];
    float(*tiles)[kCH][kLd] = reinterpret_cast<float(*)[kCH][kLd]>(smem_tiles);  // [slot][row][time]
    __shared__ uint64_t done[G][kRing];
    __shared__ float ylast_s[kCH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * kCH;
    // the lane's two channels: rows lane and lane + 32 of the CTA
    const int64_t ch[2] = {r0 + lane, r0 + kTT + lane};
    const bool live[2] = {ch[0] < a.batch, ch[1] < a.batch};
    const int64_t n = a.n, edge = a.edge;
    // memory rows of this CTA: row r0 + i at x0 + i * ldx (the blocked view
    // keeps the CTA's 64 rows inside one channel at stride blk_len)
    const int64_t ldx = a.blk_rows ? a.blk_len : a.ld_x, ldy = a.blk_rows ? a.blk_len : a.ld_y;
    const float* const x0 =
        a.x + (a.blk_rows ? (r0 / a.blk_rows) * a.ld_x + (r0 % a.blk_rows) * a.blk_len : r0 * a.ld_x);
    float* const y0 =
        a.y + (a.blk_rows ? (r0 / a.blk_rows) * a.ld_y + (r0 % a.blk_rows) * a.blk_len : r0 * a.ld_y);

    if (threadIdx.x == 0) {
        for (int w = 0; w < G; ++w)
            for (int r = 0; r < kRing; ++r) mbar_init(&done[w][r], 32);
        fence_barrier_init();
    }
    // sosfiltfilt: save the right-extension inputs before y (which may alias
    // x) is written, and read the first forward sample
    float first[2] = {0.0f, 0.0f};
    if (FF) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!live[h]) continue;
            const float* __restrict__ xr = a.x + ch[h] * a.ld_x;
            if (warp == 0) {
                const float xe = xr[n - 1];
                for (int64_t i = 0; i < edge; ++i) a.tail[i * a.batch + ch[h]] = 2.0f * xe - xr[n - 2 - i];
            }
            first[h] = edge > 0 ? 2.0f * xr[0] - xr[edge] : xr[0];
        }
        __threadfence_block();
    }
    __syncthreads();

    // states of this warp's sections for the lane's two channels (.x, .y)
    float2 S1[SPW], S2[SPW];
    PackSec pc[SPW];
    bool cpl[SPW];
#pragma unroll
    for (int i = 0; i < SPW; ++i) {
        const int s = warp * SPW + i;
        // the coupled form serves complex-pole sections in FP32_COUPLED only
        cpl[i] = PREC == 3 && sc.coupled[s] != 0;
        put_sec(pc[i], sc, s, cpl[i]);
        float s1v[2] = {0.0f, 0.0f}, s2v[2] = {0.0f, 0.0f};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!FF && a.zi && live[h] && s < sc.nsec)
                state_in<PREC>(sc, s, a.zi[(ch[h] * sc.nsec + s) * 2 + 0],
                               a.zi[(ch[h] * sc.nsec + s) * 2 + 1], s1v[h], s2v[h]);
            if (FF && a.use_zi && s < sc.nsec) {
                const double* z = (PREC == 3 && sc.coupled[s]) ? sc.zc[s] : sc.zi[s];
                s1v[h] = (float)(z[0] * (double)first[h]);
                s2v[h] = (float)(z[1] * (double)first[h]);
            }
        }
        S1[i] = make_float2(s1v[0], s1v[1]);
        S2[i] = make_float2(s2v[0], s2v[1]);
    }

    // this warp's section form, fixed for the launch
    int form = 0;
    if (PREC == 3) {
        int nc = 0;
#pragma unroll
        for (int i = 0; i < SPW; ++i) nc += cpl[i] ? 1 : 0;
        form = nc == SPW ? 1 : nc == 0 ? 0 : 2;
    }
    // section i of the warp on one sample of both channels
    auto step_i = [&](auto formc, int i, float2 v) {
        constexpr int FORM = decltype(formc)::value;
        if (FORM == 1 || (FORM == 2 && cpl[i])) return pack_step<true>(pc[i], S1[i], S2[i], v);
        return pack_step<false>(pc[i], S1[i], S2[i], v);
    };
    // Filters tn samples of the lane's two channels in place through the
    // warp's sections (a full tile fully unrolled, so the shared loads run
    // ahead and the sections of consecutive samples interleave).
    auto filter_tile = [&](auto formc, float(*t)[kLd], int tn) {
        if (tn == kTT) {
#pragma unroll
            for (int p = 0; p < kTT; ++p) {
                float2 v = make_float2(t[lane][p], t[lane + kTT][p]);
#pragma unroll
                for (int i = 0; i < SPW; ++i) v = step_i(formc, i, v);
                t[lane][p] = v.x;
                t[lane + kTT][p] = v.y;
            }
        } else {
            for (int p = 0; p < tn; ++p) {
                float2 v = make_float2(t[lane][p], t[lane + kTT][p]);
#pragma unroll
                for (int i = 0; i < SPW; ++i) v = step_i(formc, i, v);
                t[lane][p] = v.x;
                t[lane + kTT][p] = v.y;
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
        const bool rows_full = r0 + kCH <= a.batch;
        if (KIND == kSos && rows_full && j0 + kTT <= L) {
            const float* p = x0 + j;
#pragma unroll 8
            for (int i = 0; i < kCH; ++i, p += ldx) cp_async4(&t[i][lane], p, true);
        } else if (KIND == kFwd && rows_full && j0 >= edge && j0 + kTT <= edge + n) {
            const float* p = a.x + r0 * a.ld_x + (j - edge);
#pragma unroll 8
            for (int i = 0; i < kCH; ++i, p += a.ld_x) cp_async4(&t[i][lane], p, true);
        } else if (KIND == kBwd && rows_full && j0 >= edge && j0 + kTT <= L) {
            const float* p = a.y + r0 * a.ld_y + (n - 1 - (j - edge));
#pragma unroll 8
            for (int i = 0; i < kCH; ++i, p += a.ld_y) cp_async4(&t[i][lane], p, true);
        } else {
            for (int i = 0; i < kCH; ++i) {
                const int64_t row = r0 + i;
                const bool vr = row < a.batch && j < L;
                const float* rx = a.x + (row < a.batch ? row : 0) * a.ld_x;
                if (KIND == kSos) {
                    cp_async4(&t[i][lane], vr ? x0 + i * ldx + j : a.x, vr);
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
        const bool rows_full = r0 + kCH <= a.batch;
        float* q = nullptr;
        if (KIND == kSos && rows_full && j0 + kTT <= L) q = y0 + j;
        if (KIND == kFwd && rows_full && j0 >= edge && j0 + kTT <= edge + n)
            q = a.y + r0 * a.ld_y + (j - edge);
        if (KIND == kBwd && rows_full && j0 >= edge && j0 + kTT <= L)
            q = a.y + r0 * a.ld_y + (n - 1 - (j - edge));
        if (q) {
#pragma unroll 8
            for (int i = 0; i < kCH; ++i, q += (KIND == kSos ? ldy : a.ld_y)) *q = t[i][lane];
            // the forward stream's last output seeds the backward pass (edge == 0)
            if (KIND == kFwd && j == L - 1)
                for (int i = 0; i < kCH; ++i) ylast_s[i] = t[i][lane];
            return;
        }
        for (int i = 0; i < kCH; ++i) {
            const int64_t row = r0 + i;
            if (row >= a.batch || j >= L) continue;
            const float v = t[i][lane];
            float* ry = a.y + row * a.ld_y;
            if (KIND == kSos) {
                y0[(row - r0) * ldy + j] = v;
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
        if (a.zf) {
#pragma unroll
            for (int i = 0; i < SPW; ++i) {
                const int s = warp * SPW + i;
                if (s >= sc.nsec) continue;
                const float u1[2] = {S1[i].x, S1[i].y}, u2[2] = {S2[i].x, S2[i].y};
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (!live[h]) continue;
                    double o1, o2;
                    state_out<PREC>(sc, s, u1[h], u2[h], o1, o2);
                    a.zf[(ch[h] * sc.nsec + s) * 2 + 0] = o1;
                    a.zf[(ch[h] * sc.nsec + s) * 2 + 1] = o2;
                }
            }
        }
        return;
    }
    run(std::integral_constant<int, kFwd>(), n + 2 * edge);
    // backward initial state from the last forward output
    const float yl[2] = {ylast_s[lane], ylast_s[lane + kTT]};
#pragma unroll
    for (int i = 0; i < SPW; ++i) {
        const int s = warp * SPW + i;
        const bool on = a.use_zi && s < sc.nsec;
        const double* z = (PREC == 3 && sc.coupled[s]) ? sc.zc[s] : sc.zi[s];
        S1[i] = on ? make_float2((float)(z[0] * (double)yl[0]), (float)(z[0] * (double)yl[1]))
                   : make_float2(0.0f, 0.0f);
        S2[i] = on ? make_float2((float)(z[1] * (double)yl[0]), (float)(z[1] * (double)yl[1]))
                   : make_float2(0.0f, 0.0f);
    }
    run(std::integral_constant<int, kBwd>(), n + edge);
}

// Section counts with a compiled pipeline; others round up with identity
// sections (every count divides over the warps).
#define SCIR_PIPE_NS_LIST(X) X(1) X(2) X(3) X(4) X(8) X(12) X(16) X(24) X(32)

template <int NS, int PREC, bool FF>
int run_pipe(const SosCoef& c, const PipeArgs& a, cudaStream_t st) {
    const int64_t grid = ceil_div(a.batch, kCH);
    // One CTA per 64 channels, each with a (G + 4)-slot ring of 64 x 33
    // floats (68 KB for 4 warps): ask for the largest shared-memory carveout
    // so two CTAs fit an SM.
    const size_t smem = sizeof(float) * (size_t)PipeShape<NS, PREC, FF>::kRing * kCH * kLd;
    auto kern = sos_pipe_kernel<NS, PREC, FF>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    kern<<<(unsigned)grid, 32 * PipeShape<NS, PREC, FF>::G, smem, st>>>(c, a);
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
                    int precision, float* y, int64_t ld_y, float* tail, cudaStream_t st,
                    int64_t blk_rows, int64_t blk_len) {
    if (batch == 0 || n == 0) return SCIR_OK;
    SCIR_REQUIRE(blk_rows == 0 || (!filtfilt && blk_rows % kCH == 0), SCIR_ERR_INVALID_ARG,
                 "blocked rows need sosfilt and a multiple of %d blocks per channel", kCH);
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    PipeArgs a{x, ld_x, y, ld_y, batch, n, edge, zi, zf, tail, use_zi, err, blk_rows, blk_len};
    const bool coupled = precision == SCIR_SOS_FP32_COUPLED;
    if (filtfilt) return coupled ? dispatch_pipe<3, true>(c, a, st) : dispatch_pipe<2, true>(c, a, st);
    return coupled ? dispatch_pipe<3, false>(c, a, st) : dispatch_pipe<2, false>(c, a, st);
}

}  // namespace scir
