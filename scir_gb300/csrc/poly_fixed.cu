// Polyphase resample with the rate pair and filter length fixed at compile
// time: 160/147 (48 kHz <-> 44.1 kHz after gcd reduction) with SciPy's
// default 3,201-tap design, the configuration resample_poly(x, 160, 147)
// runs with.
//
// y[m] = sum_q h[ph(m) + 160 q] x[base(m) - q],  t = off + 147 m,
// ph = t mod 160, base = t div 160, off = (kh - 1) / 2 = 1,600.
// A period is 160 outputs for 147 inputs and every output phase appears once
// per period, so with the rates and the filter length constants, output p of
// every period (p < 160) has a fixed phase, a fixed base offset inside the
// period and a fixed tap count -- every index below is a compile-time
// constant.
//
// Work item: one channel x 32 consecutive periods (5,120 outputs).  Lane j
// of every warp takes period j, so all lanes of a warp sit at the same
// output phase and use the same taps; warp w takes output positions
// [20w, 20w + 20) of each period (eight code variants, two per scheduler).
// The taps arrive as kernel parameters, already ordered per warp as they are
// used (warp w, tap q, position i), and are copied once into shared memory;
// a warp reads four of its taps with one broadcast 16-byte load (the same
// address for all lanes), so each output costs its 20 or 21 FMAs plus a
// quarter load per tap.  (Reading them as constant-bank operands was
// measured 25x slower: the 13 KB tap set does not fit the constant cache.)
// The item's 4,724 input samples are staged in shared memory by one bulk
// copy (3-stage ring); lane j reads sample
// 147 j + c, and 147 is odd, so the 32 lanes hit 32 different banks.  Each
// lane keeps the ~40-sample window of its 20 outputs in registers, stores
// its outputs as 16-byte words into a padded output buffer (two, ping-pong),
// and each period's 160 outputs leave by one bulk copy.  Every wait is
// bounded and leaves the CTA together (a timeout ORs the device error word).
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <vector>

namespace scir {
namespace {

constexpr int kUp = 160, kDown = 147, kKh = 3201;
constexpr int kQ = (kKh + kUp - 1) / kUp;         // 21 taps for phase 0, 20 for the rest
constexpr int kOffM = ((kKh - 1) / 2) % kUp;      // off mod up = 0
constexpr int kNW = 8;                            // warps per CTA
constexpr int kPos = kUp / kNW;                   // output positions per warp
constexpr int kPer = 32;                          // periods per item (one per lane)
constexpr int kInSpan = kDown * (kPer - 1) + (kOffM + kDown * (kUp - 1)) / kUp + kQ;  // 4,724
constexpr int kInStage = (kInSpan + 3 + 3) / 4 * 4 + 8;  // samples per stage, 4-aligned start
constexpr int kStages = 3;
constexpr int kRowP = kUp + 4;                    // output buffer row (period) stride, floats
constexpr int kThreads = kNW * 32;

struct FixedTaps {
    float h[kNW * kQ * kPos];  // [warp w][tap q][position i] = h[ph(20w + i) + 160 q], 0 past kh
};

struct FixedGeom {
    int64_t n, ld_x, n_out, ld_y, batch;
    int64_t blocks_per_row, n_items;
    int64_t base0;  // off div up
};

__host__ __device__ constexpr int ph_of(int p) { return (kOffM + kDown * p) % kUp; }
__host__ __device__ constexpr int db_of(int p) { return (kOffM + kDown * p) / kUp; }

// Outputs [20W, 20W + 20) of the lane's period: the lane's window starts at
// stage index `w0` (= delta + 147 j + db(20W)).
template <int W>
__device__ __forceinline__ void compute_positions(const float* __restrict__ taps,
                                                  const float* __restrict__ stage, int w0,
                                                  float* __restrict__ yrow) {
    constexpr int P0 = kPos * W;
    constexpr int D0 = db_of(P0);
    constexpr int WN = db_of(P0 + kPos - 1) - D0 + kQ;
    float win[WN];
#pragma unroll
    for (int k = 0; k < WN; ++k) win[k] = stage[w0 + k];
    float acc[kPos];
#pragma unroll
    for (int i = 0; i < kPos; ++i) acc[i] = 0.0f;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const float4* t4 = reinterpret_cast<const float4*>(taps + (W * kQ + q) * kPos);
#pragma unroll
        for (int i4 = 0; i4 < kPos / 4; ++i4) {
            // a group whose taps are all past kh is skipped at compile time
            if (ph_of(P0 + 4 * i4 + 3) + kUp * q >= kKh && ph_of(P0 + 4 * i4) + kUp * q >= kKh &&
                ph_of(P0 + 4 * i4 + 1) + kUp * q >= kKh && ph_of(P0 + 4 * i4 + 2) + kUp * q >= kKh)
                continue;
            const float4 tv = t4[i4];
            const float t[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int p = P0 + 4 * i4 + e;
                if (ph_of(p) + kUp * q < kKh)
                    acc[4 * i4 + e] = fmaf(t[e], win[db_of(p) - D0 + kQ - 1 - q], acc[4 * i4 + e]);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < kPos; i += 4)
        *reinterpret_cast<float4*>(yrow + P0 + i) = make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
}

__global__ void __launch_bounds__(kThreads, 2)
poly_fixed_kernel(const __grid_constant__ FixedTaps T, const __grid_constant__ FixedGeom g,
                  const float* __restrict__ x, float* __restrict__ y, unsigned* __restrict__ err) {
    extern __shared__ __align__(128) float smem[];
    float* stages = smem;                                  // [kStages][kInStage]
    float* ybuf = stages + kStages * kInStage;             // [2][kPer][kRowP]
    float* taps = ybuf + 2 * kPer * kRowP;                 // [kNW][kQ][kPos]
    uint64_t* full = reinterpret_cast<uint64_t*>(taps + kNW * kQ * kPos);
    __shared__ int delta_s[kStages];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
        fence_barrier_init();
    }
    for (int i = tid; i < kNW * kQ * kPos; i += kThreads) taps[i] = T.h[i];
    __syncthreads();

    // Loads item `item` into stage s (warp 0): samples [s0, s0 + kInStage)
    // with s0 the item's first needed sample rounded down to 4; the valid
    // 16-byte part arrives by one bulk copy, zeros and the last n % 4 samples
    // are written by the lanes.
    auto issue = [&](int s, int64_t item) {
        const int64_t row = item / g.blocks_per_row, blk = item - row * g.blocks_per_row;
        const int64_t first = g.base0 + (int64_t)kDown * kPer * blk - (kQ - 1);
        const int delta = (int)(((first % 4) + 4) % 4);
        const int64_t s0 = first - delta;
        const int64_t len = kInStage;
        const int64_t lo = min(max(s0, (int64_t)0), s0 + len);
        const int64_t hi = max(lo, min(s0 + len, g.n));
        const int64_t hi4 = lo + ((hi - lo) & ~(int64_t)3);
        float* st = stages + s * kInStage;
        const float* xr = x + row * g.ld_x;
        for (int64_t e = lane; e < lo - s0; e += 32) st[e] = 0.0f;
        for (int64_t e = hi4 - s0 + lane; e < len; e += 32) {
            const int64_t src = s0 + e;
            st[e] = src < hi ? __ldg(xr + src) : 0.0f;
        }
        if (lane == 0) delta_s[s] = delta;
        __threadfence_block();
        __syncwarp();
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)((hi4 - lo) * (int64_t)sizeof(float));
            mbar_arrive_expect_tx(&full[s], bytes);
            if (bytes > 0) bulk_load(st + (lo - s0), xr + lo, bytes, &full[s]);
        }
    };

    int64_t issued = 0;  // items issued by this CTA
    if (warp == 0)
        for (int s = 0; s < kStages; ++s) {
            const int64_t item = blockIdx.x + (int64_t)s * gridDim.x;
            if (item < g.n_items) {
                issue(s, item);
                ++issued;
            }
        }
    bool ok = true;
    int64_t consumed = 0;
    for (int64_t k = 0;; ++k, consumed = k) {
        const int64_t item = blockIdx.x + k * gridDim.x;
        if (item >= g.n_items) break;
        const int s = (int)(k % kStages);
        const bool got = mbar_wait(&full[s], (uint32_t)((k / kStages) & 1));
        // every thread leaves together on a timeout
        if (__syncthreads_or(!got)) {
            if (tid == 0) atomicOr(err, kErrMbarTimeout);
            ok = false;
            break;
        }
        const float* st = stages + s * kInStage;
        float* yb = ybuf + (int)(k & 1) * kPer * kRowP;
        const int delta = delta_s[s];
        float* yrow = yb + lane * kRowP;
        const int w0 = delta + kDown * lane;
        switch (warp) {
        case 0: compute_positions<0>(taps, st, w0 + db_of(0 * kPos), yrow); break;
        case 1: compute_positions<1>(taps, st, w0 + db_of(1 * kPos), yrow); break;
        case 2: compute_positions<2>(taps, st, w0 + db_of(2 * kPos), yrow); break;
        case 3: compute_positions<3>(taps, st, w0 + db_of(3 * kPos), yrow); break;
        case 4: compute_positions<4>(taps, st, w0 + db_of(4 * kPos), yrow); break;
        case 5: compute_positions<5>(taps, st, w0 + db_of(5 * kPos), yrow); break;
        case 6: compute_positions<6>(taps, st, w0 + db_of(6 * kPos), yrow); break;
        default: compute_positions<7>(taps, st, w0 + db_of(7 * kPos), yrow); break;
        }
        fence_proxy_async_smem();
        // the output copies of the item before (the other buffer) have
        // finished reading before that buffer is written again
        if (warp == 0) bulk_wait_read0();
        __syncthreads();
        if (warp == 0) {
            // lane j writes period j of the item: outputs [m, m + 160)
            const int64_t row = item / g.blocks_per_row, blk = item - row * g.blocks_per_row;
            const int64_t m = (int64_t)kUp * (kPer * blk + lane);
            const int64_t valid = min((int64_t)kUp, g.n_out - m);
            if (valid > 0) {
                float* yr = y + row * g.ld_y + m;
                const int64_t v4 = valid & ~(int64_t)3;
                if (v4 > 0) bulk_store(yr, yrow, (uint32_t)(v4 * sizeof(float)));
                for (int64_t e = v4; e < valid; ++e) yr[e] = yrow[e];
            }
            bulk_commit();
            // the stage just read is refilled with the item kStages ahead
            const int64_t next = item + (int64_t)kStages * gridDim.x;
            if (next < g.n_items) {
                issue(s, next);
                ++issued;
            }
        }
    }
    if (warp == 0) {
        bulk_wait_all();
        // on a timeout: loads issued but not consumed land before the CTA leaves
        if (!ok && lane == 0) {
            for (int64_t k = consumed; k < issued; ++k) {
                const int s = (int)(k % kStages);
                mbar_wait(&full[s], (uint32_t)((k / kStages) & 1));
            }
        }
    }
}

}  // namespace

bool poly_fixed_supported(const PolyArgs& a) {
    return a.up == kUp && a.down == kDown && a.kh == kKh && a.off == (kKh - 1) / 2 &&
           (reinterpret_cast<uintptr_t>(a.x) & 15) == 0 && a.ld_x % 4 == 0 &&
           (reinterpret_cast<uintptr_t>(a.y) & 15) == 0 && a.ld_y % 4 == 0 &&
           a.n < (1LL << 40);
}

int launch_poly_fixed(const PolyArgs& a, const float* h_host, cudaStream_t st) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    SCIR_REQUIRE(poly_fixed_supported(a) && h_host, SCIR_ERR_UNSUPPORTED,
                 "fixed-rate polyphase kernel does not serve this request");
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    FixedTaps T;
    for (int w = 0; w < kNW; ++w)
        for (int q = 0; q < kQ; ++q)
            for (int i = 0; i < kPos; ++i) {
                const int hi = ph_of(kPos * w + i) + kUp * q;
                T.h[(w * kQ + q) * kPos + i] = hi < kKh ? h_host[hi] : 0.0f;
            }
    FixedGeom g;
    g.n = a.n;
    g.ld_x = a.ld_x;
    g.n_out = a.n_out;
    g.ld_y = a.ld_y;
    g.batch = a.batch;
    g.base0 = a.off / kUp;
    const int64_t periods = ceil_div(a.n_out, kUp);
    g.blocks_per_row = ceil_div(periods, kPer);
    g.n_items = g.blocks_per_row * a.batch;
    const size_t smem = sizeof(float) * ((size_t)kStages * kInStage + 2 * kPer * kRowP +
                                         kNW * kQ * kPos) +
                        kStages * sizeof(uint64_t);
    SCIR_CUDA_TRY(cudaFuncSetAttribute(poly_fixed_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t grid = std::min<int64_t>(g.n_items, 2 * (int64_t)info->sm_count);
    poly_fixed_kernel<<<(unsigned)grid, kThreads, smem, st>>>(T, g, a.x, a.y, err);
    SCIR_LAUNCH_CHECK("poly_fixed_kernel");
    return SCIR_OK;
}

}  // namespace scir
