// Polyphase upfirdn / resample_poly on the 5th-generation tensor cores
// (tcgen05, kind::f16), split-bf16 operands (BF16X3: x1c1 + x1c2 + x2c1) and
// FP32 accumulation in TMEM.
//
// Contraction.  y[m] = sum_q h[ph + q*up] * x[base - q], t = m*down + off,
// ph = t mod up, base = t div up.  Outputs are cut into segments of 32
// (m0 = 32 s).  A segment reads the 64-sample window x[lo .. lo + 64) with
// lo = base(m0) - (Q - 1) rounded down to a multiple of 8, and is the dense
// product
//   y[b][m0 + n] = sum_k X[b][lo + k] * B[n][k],
//   B[n][k] = h[ph(m0 + n) + (base(m0 + n) - lo - k) * up]   (zero outside),
// one MMA of M = 128 channels x N = 32 outputs x K = 64.  B depends only on
// the segment's place in the tap pattern (s mod S, S = up / gcd(32 down, up))
// and on the window's misalignment r8 = (base(m0) - Q + 1) mod 8, so the
// S*8 variants are built once per call by a small kernel, split into bf16
// hi + lo and stored in the 128-byte-swizzled K-major layout the MMA reads;
// each tile fetches its 8 KB variant with one bulk copy.  Rounding the window
// start down to 8 samples keeps every operand address 16-byte aligned, which
// is what a shifted polyphase window otherwise breaks.  For 160/147 (Q = 21)
// a segment needs 29 + 21 window samples of the 64 (plus up to 7 of
// misalignment); the dense product does 64 x 2 x 3 flops per output, about
// 0.16 ms of tensor time for 256 x 1,048,576 against 0.33 ms of HBM traffic.
// Measured on GB300 (256 x 1,048,576, 160/147): 0.767 ms, slower than the
// FP32 streaming kernel (0.707 ms then, 0.595 ms now), so it runs only when
// BF16X3 is asked for.  The tiles starve on their inputs: each reads 128 rows
// x 256 bytes, the 2.2x overlap of neighbouring windows is only partly caught
// by L2, and three 40 KB stages per SM keep too few bytes in flight (a variant with
// four stages and per-thread output stores measured 1.55 ms: tensor pipe
// 3.6 % busy, long-scoreboard stalls 13 per instruction, DRAM 21 %).
//
// Roles (320 threads, one CTA per SM, persistent over tiles of 128 channels
// x one segment):
//   warp 0     TMA producer: the f32 window (two 128-byte-swizzled boxes of
//              32 samples x 128 rows, zero fill outside the signal) and the
//              tile's tap variant, into a 3-stage ring;
//   warp 1     MMA issuer (one thread): 4 K steps x 3 products into one of
//              two 32-column TMEM accumulators, then commits that free the
//              stage, the operand buffer and hand the accumulator on;
//   warps 2-5  converters: each thread splits one channel row of the window
//              into bf16 hi / lo operand rows (swizzled, conflict-free);
//   warps 6-9  epilogue: tcgen05.ld of the accumulator rows (a thread per
//              channel), staged in swizzled shared memory and written by one
//              TMA tensor store per tile (rows past the batch clipped);
//              output rows without a 16-byte pitch and the last, partial
//              segment of each row are written directly, each thread storing
//              its channel's consecutive outputs.
// Every wait is bounded; a timeout sets the device error word and the CTA
// leaves its loops, waits for its stores, frees TMEM and exits.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace scir {
namespace {

constexpr int kM = 128;           // channels per tile = TMEM lanes
constexpr int kN = 32;            // outputs per segment = MMA N
constexpr int kK = 64;            // window samples = MMA K (one 128-byte bf16 row)
constexpr int kStages = 3;
constexpr int kMaxVariants = 512;
constexpr int kThreads = 320;
constexpr uint32_t kXHalf = kM * 32 * 4;       // one f32 box: 128 rows x 32 samples
constexpr uint32_t kXBytes = 2 * kXHalf;       // 32 KB window tile
constexpr uint32_t kBTerm = kN * kK * 2;       // 4 KB
constexpr uint32_t kBBytes = 2 * kBTerm;       // hi + lo
constexpr uint32_t kATerm = kM * kK * 2;       // 16 KB
constexpr uint32_t kABytes = 2 * kATerm;
constexpr uint32_t kOBytes = kM * kN * 4;      // 16 KB
constexpr uint32_t kSmemBytes =
    kStages * (kXBytes + kBBytes) + 2 * kABytes + 2 * kOBytes + 256 /* barriers */ + 1024 /* align */;

struct PolyTcGeom {
    int up, down, Q, S;  // S = segments per tap-pattern period
    int64_t off, kh, n_out, n_seg, n_groups, n_items;
    float* y;            // output rows for the direct stores (tma_y == 0)
    int64_t ld_y, batch;
    int tma_y;           // output rows are 16-byte aligned: one tensor store per tile
};

// Floor division for a possibly negative numerator and a positive divisor.
__host__ __device__ inline int64_t fdiv(int64_t a, int64_t b) {
    return a >= 0 ? a / b : -((-a + b - 1) / b);
}

// Byte offset of element k (2-byte elements) of row `row` in a K-major tile
// with 128-byte rows and the 128-byte swizzle: 8-row atoms of 1 KB, 16-byte
// unit u of row r stored at unit u ^ (r mod 8).
__host__ __device__ inline uint32_t sw128_off(int row, int k) {
    const int r = row & 7, unit = (k * 2) >> 4;
    return (uint32_t)((row >> 3) * 1024 + r * 128 + ((unit ^ r) << 4) + ((k * 2) & 15));
}

// Tap-operand variants: variant v = (s mod S) * 8 + r8 holds B[n][k] for a
// segment at pattern position s mod S whose window is misaligned by r8, as
// bf16 hi (first 4 KB) and lo (next 4 KB), swizzled.
__global__ void poly_tc_taps_kernel(const float* __restrict__ h, const PolyTcGeom g,
                                    __nv_bfloat16* __restrict__ table, int nvar) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nvar * kN * kK) return;
    const int v = idx / (kN * kK), rem = idx - v * (kN * kK);
    const int n = rem / kK, k = rem - n * kK;
    const int sp = v >> 3, r8 = v & 7;
    const int64_t t0 = (int64_t)(kN * sp) * g.down + g.off;
    const int64_t base0 = fdiv(t0, g.up);
    const int64_t t = t0 + (int64_t)n * g.down;
    const int64_t base = fdiv(t, g.up), ph = t - base * g.up;
    // q = base - lo - k with lo = base0 - (Q - 1) - r8
    const int64_t q = (base - base0) + (g.Q - 1 + r8) - k;
    float c = 0.0f;
    if (q >= 0 && q < g.Q) {
        const int64_t j = ph + q * g.up;
        if (j < g.kh) c = h[j];
    }
    const __nv_bfloat16 hi = __float2bfloat16_rn(c);
    const __nv_bfloat16 lo = __float2bfloat16_rn(c - __bfloat162float(hi));
    const uint32_t e = sw128_off(n, k) / 2;
    table[(size_t)v * (kBBytes / 2) + e] = hi;
    table[(size_t)v * (kBBytes / 2) + kBTerm / 2 + e] = lo;
}

__global__ void __launch_bounds__(kThreads, 1)
poly_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap ymap,
               const __nv_bfloat16* __restrict__ table, const PolyTcGeom g,
               unsigned* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sb = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* xs = sb;                        // kStages x 32 KB f32 windows (two swizzled boxes)
    uint8_t* bs = xs + kStages * kXBytes;    // kStages x 8 KB tap variants (hi, lo)
    uint8_t* as = bs + kStages * kBBytes;    // 2 x 32 KB signal operands (hi, lo)
    uint8_t* os = as + 2 * kABytes;          // 2 x 16 KB output tiles
    uint64_t* full = reinterpret_cast<uint64_t*>(os + 2 * kOBytes);
    uint64_t* empty = full + kStages;
    uint64_t* a_full = empty + kStages;
    uint64_t* a_empty = a_full + 2;
    uint64_t* d_full = a_empty + 2;
    uint64_t* d_empty = d_full + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(d_empty + 2);
    volatile int* abort_epi = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&a_full[b], 4);
            mbar_init(&a_empty[b], 1);
            mbar_init(&d_full[b], 1);
            mbar_init(&d_empty[b], 4);
        }
        *abort_epi = 0;
        fence_barrier_init();
        prefetch_tmap(&xmap);
        prefetch_tmap(&ymap);
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 64);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // tile `item` = (channel group, segment), groups outermost so the CTAs
    // work on neighbouring segments (overlapping windows) at the same time
    auto geom = [&](int64_t item, int64_t& m0, int64_t& row0, int64_t& lo, int& v) {
        const int64_t grp = item / g.n_seg, s = item - grp * g.n_seg;
        row0 = grp * kM;
        m0 = s * kN;
        const int64_t a0 = fdiv(m0 * g.down + g.off, g.up) - (g.Q - 1);
        const int r8 = (int)(a0 - fdiv(a0, 8) * 8);
        lo = a0 - r8;
        v = (int)(s % g.S) * 8 + r8;
    };

    if (warp == 0) {
        // ---------------------------------------------------------- producer
        if (lane == 0) {
            int64_t issued = 0;
            for (int64_t k = 0;; ++k) {
                const int64_t item = blockIdx.x + k * gridDim.x;
                if (item >= g.n_items) break;
                const int s = (int)(k % kStages);
                if (k >= kStages &&
                    !mbar_wait(&empty[s], (uint32_t)(((k - kStages) / kStages) & 1))) {
                    atomicOr(err, kErrMbarTimeout);
                    break;
                }
                int64_t m0, row0, lo;
                int v;
                geom(item, m0, row0, lo, v);
                mbar_arrive_expect_tx(&full[s], kXBytes + kBBytes);
                tma_load_2d(xs + s * kXBytes, &xmap, &full[s], (int32_t)lo, (int32_t)row0);
                tma_load_2d(xs + s * kXBytes + kXHalf, &xmap, &full[s], (int32_t)(lo + 32),
                            (int32_t)row0);
                bulk_load(bs + s * kBBytes, table + (size_t)v * (kBBytes / 2), kBBytes, &full[s]);
                ++issued;
            }
            // copies still in flight (only after a timeout) land before the
            // CTA leaves: the last use of each stage completes its phase
            for (int64_t k = issued > kStages ? issued - kStages : 0; k < issued; ++k)
                mbar_wait(&full[k % kStages], (uint32_t)((k / kStages) & 1));
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32(kM, kN);
            int64_t issued = 0;
            for (int64_t k = 0;; ++k) {
                const int64_t item = blockIdx.x + k * gridDim.x;
                if (item >= g.n_items) break;
                const int s = (int)(k % kStages), b = (int)(k & 1);
                const bool ok = mbar_wait(&a_full[b], (uint32_t)((k >> 1) & 1)) &&
                                mbar_wait(&full[s], (uint32_t)((k / kStages) & 1)) &&
                                (k < 2 || mbar_wait(&d_empty[b], (uint32_t)(((k - 2) >> 1) & 1)));
                if (!ok) {
                    atomicOr(err, kErrMbarTimeout);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * kN);
                const uint32_t ahi = smem_u32(as + b * kABytes), alo = ahi + kATerm;
                const uint32_t bhi = smem_u32(bs + s * kBBytes), blo = bhi + kBTerm;
#pragma unroll
                for (int ks = 0; ks < kK / 16; ++ks) {
                    const uint64_t dah = smem_desc(ahi + ks * 32, 16, 1024, 2);
                    const uint64_t dal = smem_desc(alo + ks * 32, 16, 1024, 2);
                    const uint64_t dbh = smem_desc(bhi + ks * 32, 16, 1024, 2);
                    const uint64_t dbl = smem_desc(blo + ks * 32, 16, 1024, 2);
                    tc_mma_f16(d, dah, dbh, idesc, ks > 0 ? 1u : 0u);
                    tc_mma_f16(d, dah, dbl, idesc, 1u);
                    tc_mma_f16(d, dal, dbh, idesc, 1u);
                }
                tc_commit(&empty[s]);    // window stage and tap variant free
                tc_commit(&a_empty[b]);  // operand buffer free
                tc_commit(&d_full[b]);   // accumulator ready
                ++issued;
            }
            // the last tile's MMAs finish before TMEM is released (they have
            // already, unless a wait timed out)
            if (issued > 0)
                mbar_wait(&d_full[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1));
        }
    } else if (warp < 6) {
        // ---------------------------------------------------------- converters
        const int r = threadIdx.x - 64, rr = r & 7;  // one channel row per thread
        for (int64_t k = 0;; ++k) {
            const int64_t item = blockIdx.x + k * gridDim.x;
            if (item >= g.n_items) break;
            const int s = (int)(k % kStages), b = (int)(k & 1);
            bool ok = mbar_wait(&full[s], (uint32_t)((k / kStages) & 1));
            if (ok && k >= 2) ok = mbar_wait(&a_empty[b], (uint32_t)(((k - 2) >> 1) & 1));
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) atomicOr(err, kErrMbarTimeout);
                break;
            }
            const uint8_t* xw = xs + s * kXBytes;
            uint8_t* ahi = as + b * kABytes;
            uint8_t* alo = ahi + kATerm;
#pragma unroll
            for (int u = 0; u < 8; ++u) {  // window samples 8u .. 8u + 7
                const uint8_t* rowp = xw + (u >> 2) * kXHalf + r * 128;
                const int c0 = (u & 3) * 2;  // 16-byte chunks of the box row (swizzled)
                const float4 f0 = *reinterpret_cast<const float4*>(rowp + ((c0 ^ rr) << 4));
                const float4 f1 = *reinterpret_cast<const float4*>(rowp + (((c0 + 1) ^ rr) << 4));
                const float xv[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const __nv_bfloat162 h2 = __floats2bfloat162_rn(xv[2 * j], xv[2 * j + 1]);
                    const float2 hf = __bfloat1622float2(h2);
                    const __nv_bfloat162 l2 =
                        __floats2bfloat162_rn(xv[2 * j] - hf.x, xv[2 * j + 1] - hf.y);
                    hw[j] = *reinterpret_cast<const uint32_t*>(&h2);
                    lw[j] = *reinterpret_cast<const uint32_t*>(&l2);
                }
                const uint32_t off = (uint32_t)((r >> 3) * 1024 + rr * 128 + ((u ^ rr) << 4));
                *reinterpret_cast<uint4*>(ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4*>(alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            fence_proxy_async_smem();  // generic-proxy writes -> the MMA's async proxy
            __syncwarp();
            if (lane == 0) mbar_arrive(&a_full[b]);
        }
    } else {
        // ---------------------------------------------------------- epilogue
        const int q = warp & 3, r = 32 * q + lane, rr = r & 7;  // TMEM lane quarter of the warp
        const bool leader = warp == 6 && lane == 0;             // issues the tensor stores
        for (int64_t k = 0;; ++k) {
            const int64_t item = blockIdx.x + k * gridDim.x;
            if (item >= g.n_items) break;
            const int b = (int)(k & 1);
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&d_full[b], (uint32_t)((k >> 1) & 1)));
            if (!ok && lane == 0) {
                atomicOr(err, kErrMbarTimeout);
                *abort_epi = 1;
            }
            // the output buffer of this tile was last read by the store of
            // tile k - 2: at most one store (tile k - 1) may still be reading
            if (leader) bulk_wait_read1();
            named_bar_sync(1, 128);
            if (*abort_epi) break;  // the same decision in all four warps
            tc_fence_after();
            float v[32];
            {
                float v0[16], v1[16];
                const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * kN);
                tmem_ld16(ta, v0);
                tmem_ld16(ta + 16, v1);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    v[i] = v0[i];
                    v[16 + i] = v1[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&d_empty[b]);
            int64_t m0, row0, lo;
            int vv;
            geom(item, m0, row0, lo, vv);
            if (!g.tma_y || m0 + kN > g.n_out) {
                // rows whose pitch is not a whole number of 16-byte units, and
                // the last (partial) segment of a row, which a tensor store
                // would clip only at the next 16-byte boundary: each thread
                // writes its channel's consecutive outputs
                const int64_t row = row0 + r;
                if (row < g.batch) {
                    float* __restrict__ yr = g.y + row * g.ld_y + m0;
                    const int64_t nv = g.n_out - m0;
#pragma unroll
                    for (int j = 0; j < kN; ++j)
                        if (j < nv) yr[j] = v[j];
                }
                continue;
            }
            uint8_t* ob = os + b * kOBytes;
#pragma unroll
            for (int c = 0; c < 8; ++c)
                *reinterpret_cast<float4*>(ob + r * 128 + ((c ^ rr) << 4)) =
                    make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
            fence_proxy_async_smem();
            named_bar_sync(1, 128);
            if (leader) {
                tma_store_2d(&ymap, ob, (int32_t)m0, (int32_t)row0);
                bulk_commit();
            }
        }
        if (leader) bulk_wait_all();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 64);
    }
}

// Geometry of a call, or an error status when the shape is not served
// (16-byte rows, an 8-aligned window of 64 covering every segment, at most
// kMaxVariants tap variants, a non-negative delay).
int poly_tc_plan(const PolyArgs& a, PolyTcGeom* g, int* nvar) {
    if ((reinterpret_cast<uintptr_t>(a.x) & 15) || (a.ld_x & 3))
        return set_error(SCIR_ERR_UNSUPPORTED,
                         "tensor-core polyphase needs 16-byte aligned input rows");
    if (a.off < 0 || a.n < 1 || a.kh < 1)
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase: unsupported geometry");
    if (a.n >= (1LL << 31) - 128 || a.n_out >= (1LL << 31) - 128 || a.batch >= (1LL << 31))
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase: rows too long");
    const int64_t Q = ceil_div(a.kh, a.up);
    const int64_t S = a.up / gcd64((int64_t)kN * a.down, a.up);
    if (S * 8 > kMaxVariants)
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase: %lld tap variants",
                         (long long)(S * 8));
    for (int64_t sp = 0; sp < S; ++sp) {
        const int64_t t0 = kN * sp * a.down + a.off;
        const int64_t span = fdiv(t0 + (int64_t)(kN - 1) * a.down, a.up) - fdiv(t0, a.up);
        if (span + Q + 7 > kK)
            return set_error(SCIR_ERR_UNSUPPORTED,
                             "tensor-core polyphase: a 32-output segment spans more than 64 samples");
    }
    g->up = a.up;
    g->down = a.down;
    g->Q = (int)Q;
    g->S = (int)S;
    g->off = a.off;
    g->kh = a.kh;
    g->n_out = a.n_out;
    g->n_seg = ceil_div(a.n_out, kN);
    g->n_groups = ceil_div(a.batch, kM);
    g->n_items = g->n_seg * g->n_groups;
    g->y = a.y;
    g->ld_y = a.ld_y;
    g->batch = a.batch;
    g->tma_y = ((reinterpret_cast<uintptr_t>(a.y) & 15) == 0 && (a.ld_y & 3) == 0) ? 1 : 0;
    *nvar = (int)(S * 8);
    return SCIR_OK;
}

}  // namespace

bool poly_tc_supported(const PolyArgs& a) {
    PolyTcGeom g;
    int nvar = 0;
    const bool ok = poly_tc_plan(a, &g, &nvar) == SCIR_OK;
    if (!ok) clear_error();
    return ok;
}

int launch_poly_tc(const PolyArgs& a, int terms, cudaStream_t st) {
    if (terms != 2)
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase runs BF16X3 only");
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    PolyTcGeom g;
    int nvar = 0;
    int rc = poly_tc_plan(a, &g, &nvar);
    if (rc) return rc;
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    CUtensorMap xmap, ymap;
    rc = make_tmap_2d(&xmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, a.x, (uint64_t)a.n,
                      (uint64_t)a.batch, (uint64_t)a.ld_x * 4, 32, kM, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    if (g.tma_y) {
        rc = make_tmap_2d(&ymap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, a.y, (uint64_t)a.n_out,
                          (uint64_t)a.batch, (uint64_t)a.ld_y * 4, kN, kM,
                          CU_TENSOR_MAP_SWIZZLE_128B);
        if (rc) return rc;
    } else {
        ymap = xmap;  // not used by the direct-store epilogue
    }
    __nv_bfloat16* table = nullptr;
    rc = scratch_alloc((void**)&table, (size_t)nvar * kBBytes, st);
    if (rc) return rc;
    const int total = nvar * kN * kK;
    poly_tc_taps_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, st>>>(a.h, g, table, nvar);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        e = cudaFuncSetAttribute(poly_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSmemBytes);
    }
    if (e == cudaSuccess) {
        const int64_t grid = std::min<int64_t>(g.n_items, info->sm_count);
        poly_tc_kernel<<<(unsigned)grid, kThreads, kSmemBytes, st>>>(xmap, ymap, table, g, err);
        e = cudaGetLastError();
    }
    scratch_free(table, st);
    if (e != cudaSuccess) return set_error(SCIR_ERR_CUDA, "poly_tc_kernel: %s", cudaGetErrorString(e));
    return SCIR_OK;
}

}  // namespace scir
