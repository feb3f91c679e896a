// Polyphase upfirdn / resample_poly on the CUDA cores (FP32).
//
// Computes y[m] = sum_q h[ph + q*up] * x[base - q] with t = m*down + off,
// ph = t mod up, base = t div up -- the non-zero products of the reference's
// zero-stuff-then-convolve resample_poly (crates/scir-signal/src/lib.rs:
// 313-362), which multiplies every zero of the up-sampled signal through the
// whole filter.
//
// Streaming kernel (down <= up, ceil(up/P) <= 32 groups for some P <= 5,
// window fits the register budget): outputs m and m + up share their phase
// and `base` advances by `down` per period.  A period is cut into G groups
// of P consecutive outputs; lane l of every warp owns group l % G of period
// offset l / G.  Each thread builds its P x JWA tap matrix once for the
// whole (persistent) launch: each output's phase taps, shifted to the
// output's place inside the lane's input window and pre-shifted by the
// window's fixed misalignment so the window is read with 16-byte shared
// loads; the products run as packed f32x2 FMAs, each lane keeping the sums
// over even and odd window positions in the two halves of a register pair.
// A work item is CT channels (1, 2 or 4, sharing every lane's tap
// matrix) x IP periods (32, or 16 with four channels); the items' channel
// windows stream into a 4-stage shared-memory ring, one bulk copy per channel
// row clamped to [0, n) with the zero fill written by the lanes (TMA tensor
// boxes for rows that are not 16-byte aligned).  No warp ever waits for
// another: each warp waits only for its stage's data (mbarrier, bounded
// wait), and the last warp to finish with a stage (a shared-memory counter)
// issues that stage's refill for the item four steps ahead.  Which lane takes
// which group is a per-warp permutation chosen on the host to spread the
// lanes' 16-byte window reads over the shared-memory banks.  Each warp stages
// its period's outputs in double-buffered shared memory and writes them back
// with one bulk copy per channel row (per-lane stores when the output rows
// are not 16-byte aligned), lane r issuing row r's copy.
//
// Generic kernel: one thread per output, taps and input through the
// read-only cache (down > up, long phases, misaligned rows).
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

namespace scir {
namespace {

constexpr int kNW = 8;          // warps per CTA
constexpr int kThreads = kNW * 32;
constexpr int kStages = 4;
constexpr int kBox = 256;       // floats per TMA box

struct PolyGeom {
    int up, down, Q, P, G, ppw;   // groups, periods per warp-iteration
    int64_t off;
    int b00;                      // base of rho = 0 inside a period: off div up
    int IP;                       // periods per work item
    int nbox;                     // TMA boxes per channel window
    int win_floats;               // floats per channel window (nbox * kBox)
    int stage_floats;             // CT windows
    int bulk;                     // outputs leave shared memory by bulk copies
    int bulkin;                   // windows arrive by one bulk copy per row
    int64_t n_periods, items_per_row, n_items;
    uint8_t unit[kNW][32];        // work unit (pl * G + gl) of each lane; 255 = idle
};

template <int P, int JWA, int CT>
__global__ void __launch_bounds__(kThreads, 1)
poly_stream_kernel(const __grid_constant__ CUtensorMap xmap, const float* __restrict__ x,
                   int64_t ld_x, int64_t n, const float* __restrict__ h,
                   int64_t kh, const __grid_constant__ PolyGeom g, float* __restrict__ y,
                   int64_t ld_y, int64_t n_out, int64_t g_batch, unsigned* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    float* stages = reinterpret_cast<float*>(smem_raw);
    float* ybuf = stages + kStages * g.stage_floats;  // two output buffers per warp
    uint64_t* full = reinterpret_cast<uint64_t*>(ybuf + 2 * kNW * 32 * P * CT);
    int* done = reinterpret_cast<int*>(full + kStages);  // warps finished with each stage

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t pos_first = (int64_t)g.b00 - (g.Q - 1);  // window start of item 0 (i0 = 0)
    const int shift = (int)(pos_first - (pos_first & ~(int64_t)3));

    // Loads item `item` into stage s (called by a whole warp).  Row windows
    // that start 16-byte aligned come in as one bulk copy per row, clamped
    // to [0, n), lane r copying row r; the lanes write the zeros outside
    // the row and the last n % 4 samples first.  Otherwise lane 0 registers
    // the bytes and the lanes issue the tensor boxes in parallel (zero fill
    // by TMA).
    auto issue_warp = [&](int s, int64_t item) {
        const int64_t row0 = (item / g.items_per_row) * CT;
        const int64_t i0 = (item % g.items_per_row) * g.IP;
        const int64_t pos_a = (i0 * g.down + pos_first) & ~(int64_t)3;
        const int rows = (int)min((int64_t)CT, g_batch - row0);
        if (g.bulkin) {
            const int64_t len = g.win_floats;
            // valid samples [lo, hi) with pos_a <= lo <= hi <= pos_a + len
            const int64_t lo = min(max(pos_a, (int64_t)0), pos_a + len);
            const int64_t hi = max(lo, min(pos_a + len, n));
            const int64_t hi4 = lo + ((hi - lo) & ~(int64_t)3);
            const int nz_lo = (int)(lo - pos_a), nz_hi = (int)(pos_a + len - hi4);
            for (int r = 0; r < rows; ++r) {
                float* w = stages + s * g.stage_floats + r * g.win_floats;
                const float* xr = x + (row0 + r) * ld_x;
                for (int e = lane; e < nz_lo; e += 32) w[e] = 0.0f;
                for (int e = lane; e < nz_hi; e += 32) {
                    const int64_t src = hi4 + e;
                    w[src - pos_a] = src < hi ? __ldg(xr + src) : 0.0f;
                }
            }
            __threadfence_block();
            __syncwarp();
            const uint32_t bytes = (uint32_t)((hi4 - lo) * (int64_t)sizeof(float));
            if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)rows);
            __syncwarp();
            // lane r copies row r
            if (bytes > 0 && lane < rows)
                bulk_load(stages + s * g.stage_floats + lane * g.win_floats + (lo - pos_a),
                          x + (row0 + lane) * ld_x + lo, bytes, &full[s]);
            return;
        }
        if (lane == 0)
            mbar_arrive_expect_tx(&full[s], (uint32_t)(rows * g.nbox * kBox * sizeof(float)));
        __syncwarp();
        for (int e = lane; e < rows * g.nbox; e += 32) {
            const int r = e / g.nbox, b = e - r * g.nbox;
            float* dst = stages + s * g.stage_floats + r * g.win_floats + b * kBox;
            tma_load_2d(dst, &xmap, &full[s], (int32_t)(pos_a + b * kBox), (int32_t)(row0 + r));
        }
    };

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            done[s] = 0;
        }
        fence_barrier_init();
        prefetch_tmap(&xmap);
    }
    __syncthreads();
    if (warp == 0) {
        for (int s = 0; s < kStages; ++s) {
            const int64_t item = blockIdx.x + (int64_t)s * gridDim.x;
            if (item < g.n_items) issue_warp(s, item);
        }
    }

    const int unit = g.unit[warp][lane];
    const bool active = unit < g.G * g.ppw;
    const int gl = active ? unit % g.G : 0, pl = active ? unit / g.G : 0;
    int ybsel = 0;

    // --- the thread's tap matrix, fixed for the whole launch
    const int64_t t0 = (int64_t)(gl * P) * g.down + g.off;
    const int rel0 = (int)(t0 / g.up) - g.b00;  // group window start in a period
    // window start inside the stage for this thread's first period (iteration 0)
    const int L0 = (warp * g.ppw + pl) * g.down + rel0 + shift;
    const int a = L0 & 3;
    // T2[p][j/2] = taps (j, j+1) of output p: register pairs for the packed
    // FMAs below
    float2 T2[P][JWA / 2];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int rho = gl * P + p;
        const int64_t t = (int64_t)rho * g.down + g.off;
        const int ph = (int)(t % g.up);
        const int d = (int)(t / g.up - t0 / g.up);
#pragma unroll
        for (int j = 0; j < JWA; ++j) {
            const int q = d + g.Q - 1 + a - j;
            const int64_t hj = (int64_t)ph + (int64_t)q * g.up;
            const float v = (active && rho < g.up && q >= 0 && q < g.Q && hj < kh) ? __ldg(h + hj) : 0.0f;
            if (j & 1) T2[p][j / 2].y = v;
            else T2[p][j / 2].x = v;
        }
    }

    const int iters = g.IP / g.ppw;  // warp-iterations per item
    for (int64_t k = 0;; ++k) {
        const int64_t item = blockIdx.x + k * gridDim.x;
        if (item >= g.n_items) break;
        const int s = (int)(k % kStages);
        const uint32_t parity = (uint32_t)((k / kStages) & 1);
        // warp-uniform outcome: every lane leaves together on a timeout
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], parity))) {
            if (lane == 0) atomicOr(err, kErrMbarTimeout);
            break;
        }
        const int64_t row0 = (item / g.items_per_row) * CT;
        const int64_t i0 = (item % g.items_per_row) * g.IP;
        const float* win = stages + s * g.stage_floats;
        const int rows = (int)min((int64_t)CT, g_batch - row0);
        const int cnt = g.ppw * g.up;
        for (int it = warp; it < iters; it += kNW) {
            const int po = it * g.ppw + pl;  // period offset inside the item
            const int La = (po * g.down + rel0 + shift) & ~3;
            // acc2 = (sum over even window positions, sum over odd ones): one
            // packed FMA (f32x2) per tap pair halves the FMA instructions
            float2 acc2[CT][P];
#pragma unroll
            for (int r = 0; r < CT; ++r)
#pragma unroll
                for (int p = 0; p < P; ++p) acc2[r][p] = make_float2(0.0f, 0.0f);
            if (active) {
#pragma unroll
                for (int j4 = 0; j4 < JWA / 4; ++j4) {
                    // the same tap matrix serves every channel of the item
                    float2 w[CT][2];
#pragma unroll
                    for (int r = 0; r < CT; ++r) {
                        const float4 v =
                            reinterpret_cast<const float4*>(win + r * g.win_floats + La)[j4];
                        w[r][0] = make_float2(v.x, v.y);
                        w[r][1] = make_float2(v.z, v.w);
                    }
                    // consecutive FMAs update different accumulators
#pragma unroll
                    for (int e = 0; e < 2; ++e)
#pragma unroll
                        for (int r = 0; r < CT; ++r)
#pragma unroll
                            for (int p = 0; p < P; ++p)
                                acc2[r][p] = __ffma2_rn(T2[p][2 * j4 + e], w[r][e], acc2[r][p]);
                }
            }
            float acc[CT][P];
#pragma unroll
            for (int r = 0; r < CT; ++r)
#pragma unroll
                for (int p = 0; p < P; ++p) acc[r][p] = acc2[r][p].x + acc2[r][p].y;
            float* yb = ybuf + (warp * 2 + ybsel) * (32 * P * CT);
            const int64_t m0 = (i0 + (int64_t)it * g.ppw) * g.up;
            if (g.bulk) {
                // the bulk copy issued from this buffer two iterations ago has
                // finished reading it once at most one group is pending
                if (lane < CT) bulk_wait_read1();
                __syncwarp();
            }
            if (active) {
#pragma unroll
                for (int r = 0; r < CT; ++r)
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        if (gl * P + p < g.up) yb[r * cnt + pl * g.up + gl * P + p] = acc[r][p];
            }
            if (g.bulk) {
                // staged outputs -> global by one bulk copy per channel row
                fence_proxy_async_smem();
                __syncwarp();
                if (lane < CT) {
                    // lane r copies row r (its own bulk group): outputs
                    // [m0, m0 + valid); periods past the row end (valid <= 0)
                    // write nothing
                    const int r = lane;
                    const int64_t valid = min((int64_t)cnt, n_out - m0);
                    if (valid > 0 && r < rows) {
                        const int64_t v4 = valid & ~(int64_t)3;
                        float* __restrict__ yr = y + (row0 + r) * ld_y;
                        if (v4 > 0)
                            bulk_store(yr + m0, yb + r * cnt, (uint32_t)(v4 * sizeof(float)));
                        for (int64_t e = v4; e < valid; ++e) yr[m0 + e] = yb[r * cnt + e];
                    }
                    bulk_commit();
                }
                ybsel ^= 1;
            } else {
                __syncwarp();
                for (int r = 0; r < rows; ++r) {
                    float* __restrict__ yr = y + (row0 + r) * ld_y;
                    for (int e = lane; e < cnt; e += 32) {
                        const int64_t m = m0 + e;
                        if (m < n_out) yr[m] = yb[r * cnt + e];
                    }
                }
                __syncwarp();
            }
        }
        // the last warp done with stage s refills it (the fences order every
        // warp's reads of the stage before the refill's writes)
        int last = 0;
        if (lane == 0) {
            __threadfence_block();
            last = atomicAdd(&done[s], 1) == kNW - 1;
            if (last) {
                __threadfence_block();
                done[s] = 0;
            }
        }
        if (__shfl_sync(0xffffffffu, last, 0)) {
            const int64_t next = item + (int64_t)kStages * gridDim.x;
            if (next < g.n_items) issue_warp(s, next);
        }
    }
    if (g.bulk && lane < CT) bulk_wait_all();
}

__global__ void __launch_bounds__(256)
poly_generic_kernel(const float* __restrict__ x, int64_t ld_x, int64_t n,
                    const float* __restrict__ h, int64_t kh, int up, int down, int64_t off,
                    float* __restrict__ y, int64_t ld_y, int64_t n_out, int64_t blocks_per_row) {
    const int64_t row = blockIdx.x / blocks_per_row;
    const int64_t m = (blockIdx.x % blocks_per_row) * 256 + threadIdx.x;
    if (m >= n_out) return;
    const float* __restrict__ xr = x + row * ld_x;
    const int64_t t = m * down + off;
    const int64_t ph = t % up, base = t / up;
    float acc = 0.0f;
    for (int64_t j = ph, q = 0; j < kh; j += up, ++q) {
        const int64_t xi = base - q;
        if (xi < 0) break;
        if (xi < n) acc = fmaf(__ldg(h + j), __ldg(xr + xi), acc);
    }
    y[row * ld_y + m] = acc;
}

template <int P, int JWA, int CT>
int launch_stream(const PolyArgs& a, const PolyGeom& g0, cudaStream_t st) {
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    PolyGeom g = g0;
    g.stage_floats = CT * g.win_floats;
    g.bulk = ((int64_t)g.ppw * g.up % 4 == 0 && (reinterpret_cast<uintptr_t>(a.y) & 15) == 0 &&
              a.ld_y % 4 == 0) ? 1 : 0;
    g.bulkin = ((reinterpret_cast<uintptr_t>(a.x) & 15) == 0 && a.ld_x % 4 == 0) ? 1 : 0;
    g.items_per_row = ceil_div(g.n_periods, g.IP);
    g.n_items = g.items_per_row * ceil_div(a.batch, CT);
    const size_t smem = sizeof(float) * ((size_t)kStages * g.stage_floats + 2 * kNW * 32 * P * CT) +
                        kStages * (sizeof(uint64_t) + sizeof(int));
    if ((int)smem > info->max_smem_optin)
        return set_error(SCIR_ERR_UNSUPPORTED, "polyphase stage needs %zu bytes", smem);
    CUtensorMap map;
    rc = make_tmap_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, a.x, (uint64_t)a.n, (uint64_t)a.batch,
                      (uint64_t)a.ld_x * sizeof(float), kBox, 1, CU_TENSOR_MAP_SWIZZLE_NONE);
    if (rc) return rc;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    auto kern = poly_stream_kernel<P, JWA, CT>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t grid = std::min<int64_t>(g.n_items, (int64_t)info->sm_count);
    kern<<<(unsigned)grid, kThreads, smem, st>>>(map, a.x, a.ld_x, a.n, a.h, a.kh, g, a.y, a.ld_y,
                                                 a.n_out, a.batch, err);
    SCIR_LAUNCH_CHECK("poly_stream_kernel");
    return SCIR_OK;
}

// Window lengths with a compiled kernel (multiples of 4).
int jwa_bucket(int jwa) { return jwa <= 12 ? 12 : jwa <= 20 ? 20 : jwa <= 28 ? 28 : 36; }

// Two channels per work item share each thread's tap matrix when there are
// at least two rows and the doubled accumulators still fit the registers.
template <int P, int JWA>
int launch_ct(const PolyArgs& a, const PolyGeom& g, int ct, cudaStream_t st) {
    // ct: channels per work item, already resolved by try_stream
    if (ct == 4 && P * JWA <= 144) return launch_stream<P, JWA, 4>(a, g, st);
    if (ct >= 2) return launch_stream<P, JWA, 2>(a, g, st);
    return launch_stream<P, JWA, 1>(a, g, st);
}

template <int P>
int dispatch_jwa(const PolyArgs& a, const PolyGeom& g, int jwa_b, int ct, cudaStream_t st) {
    switch (jwa_b) {
    case 12: return launch_ct<P, 12>(a, g, ct, st);
    case 20: return launch_ct<P, 20>(a, g, ct, st);
    case 28: return launch_ct<P, 28>(a, g, ct, st);
    default: return launch_ct<P, 36>(a, g, ct, st);
    }
}

// 16-byte shared wavefronts a warp needs for one window load: lanes are served
// in quarters of 8; two lanes conflict when their 16-byte chunks differ but
// map to the same 4-bank quad (chunk mod 8).
int quarter_wavefronts(const int* chunk) {
    int total = 0;
    for (int q = 0; q < 4; ++q) {
        int worst = 1;
        for (int r = 0; r < 8; ++r) {
            int seen[8], ns = 0;
            for (int l = 8 * q; l < 8 * q + 8; ++l) {
                if (chunk[l] < 0 || (chunk[l] & 7) != r) continue;
                bool dup = false;
                for (int i = 0; i < ns; ++i) dup |= seen[i] == chunk[l];
                if (!dup) seen[ns++] = chunk[l];
            }
            worst = std::max(worst, ns);
        }
        total += worst;
    }
    return total;
}

// Chooses, per warp, which lane takes which (group, period) unit so that the
// lanes' window reads hit distinct bank quads as far as possible (a short
// deterministic local search over lane swaps).
void assign_lanes(PolyGeom& g, int /*maxrel*/) {
    const int64_t pos_first = (int64_t)g.b00 - (g.Q - 1);
    const int shift = (int)(pos_first - (pos_first & ~(int64_t)3));
    const int nunits = g.G * g.ppw;
    uint32_t rng = 12345u;
    for (int w = 0; w < kNW; ++w) {
        int unit[32], chunk[32];
        for (int l = 0; l < 32; ++l) unit[l] = l < nunits ? l : 255;
        auto chunk_of = [&](int u) {
            if (u == 255) return -1;
            const int gl = u % g.G, pl = u / g.G;
            const int64_t t0 = (int64_t)(gl * g.P) * g.down + g.off;
            const int rel0 = (int)(t0 / g.up) - g.b00;
            return (((w * g.ppw + pl) * g.down + rel0 + shift) & ~3) / 4;
        };
        for (int l = 0; l < 32; ++l) chunk[l] = chunk_of(unit[l]);
        int cur = quarter_wavefronts(chunk);
        for (int step = 0; step < 3000 && cur > 4; ++step) {
            rng = rng * 1664525u + 1013904223u;
            const int i = (int)((rng >> 8) & 31);
            rng = rng * 1664525u + 1013904223u;
            const int j = (int)((rng >> 8) & 31);
            if (i / 8 == j / 8) continue;
            std::swap(unit[i], unit[j]);
            std::swap(chunk[i], chunk[j]);
            const int v = quarter_wavefronts(chunk);
            if (v <= cur) {
                cur = v;
            } else {
                std::swap(unit[i], unit[j]);
                std::swap(chunk[i], chunk[j]);
            }
        }
        for (int l = 0; l < 32; ++l) g.unit[w][l] = (uint8_t)unit[l];
    }
}

int try_stream(const PolyArgs& a, int p_force, int ct, cudaStream_t st) {
    if (a.down > a.up) return SCIR_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(a.x) & 15) || (a.ld_x & 3)) return SCIR_ERR_UNSUPPORTED;
    if (a.n >= (1LL << 31) - 4096 || a.batch >= (1LL << 31)) return SCIR_ERR_UNSUPPORTED;
    const int64_t Q = ceil_div(a.kh, a.up);
    // outputs per lane: the fewest that keep a period within 32 lanes, or
    // more when the autotuner found that faster
    int P = (int)ceil_div(a.up, 32);
    if (P < 1) P = 1;
    if (p_force > P) P = p_force;
    if (P > 5) return SCIR_ERR_UNSUPPORTED;
    const int JW = (int)Q + P - 1;
    const int jwa = (JW + 3 + 3) / 4 * 4;
    if (jwa > 36) return SCIR_ERR_UNSUPPORTED;
    const int jwa_b = jwa_bucket(jwa);
    PolyGeom g;
    g.up = a.up;
    g.down = a.down;
    g.Q = (int)Q;
    g.P = P;
    g.G = (int)ceil_div(a.up, P);
    g.ppw = 32 / g.G;
    g.off = a.off;
    g.b00 = (int)(a.off / a.up);
    // channels per work item: by default four when there are four rows and
    // the accumulators fit the registers (measured on 256 x 1,048,576, 160/147:
    // 0.72 ms vs 0.81 with two and 1.10 with one); four use items of 16
    // periods so four channel windows fit the stage ring
    int cte = ct;
    if (cte == 0) cte = (a.batch >= 4 && P * jwa_b <= 144) ? 4 : (a.batch >= 2 && P * jwa_b <= 144) ? 2 : 1;
    if (cte == 4 && (a.batch < 4 || P * jwa_b > 144)) cte = 2;
    if (cte == 2 && a.batch < 2) cte = 1;
    g.IP = (cte == 4 ? 16 : 32) * g.ppw;
    int maxrel = 0;
    for (int gi = 0; gi < g.G; ++gi) {
        const int64_t t0 = (int64_t)(gi * P) * a.down + a.off;
        maxrel = std::max(maxrel, (int)(t0 / a.up) - g.b00);
    }
    const int64_t need = (int64_t)(g.IP - 1) * a.down + maxrel + 3 + jwa_b + 4;
    if (need > 48 * 1024) return SCIR_ERR_UNSUPPORTED;
    g.nbox = (int)ceil_div(need, kBox);
    g.win_floats = g.nbox * kBox;
    g.stage_floats = g.win_floats;
    g.n_periods = ceil_div(a.n_out, a.up);
    g.items_per_row = ceil_div(g.n_periods, g.IP);
    g.n_items = g.items_per_row * a.batch;
    {
        // the lane assignment depends only on the filter geometry: search once
        using Key = std::tuple<int, int, int64_t, int, int>;
        static std::mutex mu;
        static std::map<Key, std::array<uint8_t, kNW * 32>> cache;
        const Key key{a.up, a.down, a.off, g.Q, P};
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it == cache.end()) {
            assign_lanes(g, maxrel);
            std::array<uint8_t, kNW * 32> units;
            memcpy(units.data(), g.unit, sizeof(g.unit));
            cache.emplace(key, units);
        } else {
            memcpy(g.unit, it->second.data(), sizeof(g.unit));
        }
    }
    switch (P) {
    case 1: return dispatch_jwa<1>(a, g, jwa_b, cte, st);
    case 2: return dispatch_jwa<2>(a, g, jwa_b, cte, st);
    case 3: return dispatch_jwa<3>(a, g, jwa_b, cte, st);
    case 4: return dispatch_jwa<4>(a, g, jwa_b, cte, st);
    default: return dispatch_jwa<5>(a, g, jwa_b, cte, st);
    }
}

}  // namespace

int launch_poly_simt(const PolyArgs& a, cudaStream_t st, int p_force, int ct) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    int rc = try_stream(a, p_force, ct, st);
    if (rc != SCIR_ERR_UNSUPPORTED) return rc;
    clear_error();
    const int64_t bpr = ceil_div(a.n_out, 256);
    const int64_t grid = bpr * a.batch;
    SCIR_REQUIRE(grid <= 0x7fffffffLL, SCIR_ERR_UNSUPPORTED, "polyphase grid too large");
    poly_generic_kernel<<<(unsigned)grid, 256, 0, st>>>(a.x, a.ld_x, a.n, a.h, a.kh, a.up, a.down,
                                                        a.off, a.y, a.ld_y, a.n_out, bpr);
    SCIR_LAUNCH_CHECK("poly_generic_kernel");
    return SCIR_OK;
}

}  // namespace scir
