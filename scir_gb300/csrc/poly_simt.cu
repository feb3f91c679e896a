// Polyphase upfirdn / resample_poly on the CUDA cores (FP32).
//
// Computes y[m] = sum_q h[ph + q*up] * x[base - q] with t = m*down + off,
// ph = t mod up, base = t div up -- the non-zero products of the reference's
// zero-stuff-then-convolve resample_poly (crates/scir-signal/src/lib.rs:
// 313-362), which multiplies every zero of the up-sampled signal through the
// whole filter.
//
// Fast kernel (down <= up, ceil(kh/up) <= QM, up <= 256): outputs m and
// m + up share their phase, and base advances by `down` per period.  A warp
// takes one group of P consecutive outputs of the period (same phases in every
// period) and its 32 lanes take 32 consecutive periods.  The group's P x
// (QM+P-1) tap matrix -- each output's phase taps, shifted to the output's
// offset inside a shared input window -- lives in registers, so each period
// costs QM+P-1 shared loads and P*(QM+P-1) FMAs.  The CTA stages CT channels x
// IT periods of input (zero outside [0, n)) and builds every group's tap
// matrix in shared memory once.
//
// Generic kernel: one thread per output, taps and input through the read-only
// cache.  Used for down > up, very long phases or very large up.
#include "common.cuh"
#include "kernels.cuh"

namespace scir {
namespace {

constexpr int kP = 4;         // outputs per thread (consecutive in the period)
constexpr int kCT = 2;        // channels per CTA
constexpr int kIT = 64;       // periods per CTA
constexpr int kThreads = 256; // 8 warps
constexpr int kMaxUp = 256;

__device__ __forceinline__ int padi(int j) { return j + (j >> 5); }

struct PolyGeom {
    int up, down, Q;
    int64_t off;
    int G;            // groups per period
    int span;         // window positions one period of all groups touches
    int WL;           // window length per channel for IT periods
    int b00;          // base offset of rho = 0: off div up (mod the period)
};

template <int QM>
__global__ void __launch_bounds__(kThreads)
poly_fast_kernel(const float* __restrict__ x, int64_t ld_x, int64_t batch, int64_t n,
                 const float* __restrict__ h, int64_t kh, PolyGeom g,
                 float* __restrict__ y, int64_t ld_y, int64_t n_out, int64_t n_periods,
                 int64_t cta_per_row_group) {
    constexpr int JW = QM + kP - 1;
    constexpr int JWP = (JW + 3) / 4 * 4;
    extern __shared__ __align__(16) float smem[];
    float* s_T = smem;                          // [G][P][JWP]
    float* s_x = smem + g.G * kP * JWP;         // [CT][padi(WL)]
    const int WLP = padi(g.WL) + 1;

    const int64_t c0 = (blockIdx.x / cta_per_row_group) * kCT;
    const int64_t i0 = (blockIdx.x % cta_per_row_group) * kIT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // tap matrices of every group
    const int ntab = g.G * kP * JWP;
    for (int e = tid; e < ntab; e += kThreads) {
        const int jj = e % JWP, p = (e / JWP) % kP, gi = e / (JWP * kP);
        const int rho = gi * kP + p;
        float v = 0.0f;
        if (rho < g.up && jj < JW) {
            const int64_t t = (int64_t)rho * g.down + g.off;
            const int64_t t0 = (int64_t)(gi * kP) * g.down + g.off;
            const int ph = (int)(t % g.up);
            const int d = (int)(t / g.up - t0 / g.up);
            const int q = d + QM - 1 - jj;
            const int64_t hj = (int64_t)ph + (int64_t)q * g.up;
            if (q >= 0 && q < g.Q && hj < kh) v = __ldg(h + hj);
        }
        s_T[e] = v;
    }
    // input windows: positions pos_lo .. pos_lo + WL - 1 of each channel
    const int64_t pos_lo = i0 * g.down + g.b00 - (QM - 1);
    for (int c = 0; c < kCT; ++c) {
        const int64_t row = c0 + c;
        float* sx = s_x + c * WLP;
        if (row < batch) {
            const float* __restrict__ xr = x + row * ld_x;
            for (int j = tid; j < g.WL; j += kThreads) {
                const int64_t p = pos_lo + j;
                sx[padi(j)] = (p >= 0 && p < n) ? __ldg(xr + p) : 0.0f;
            }
        }
    }
    __syncthreads();

    for (int gi = warp; gi < g.G; gi += kThreads / 32) {
        float T[kP][JW];
#pragma unroll
        for (int p = 0; p < kP; ++p) {
#pragma unroll
            for (int j = 0; j < JWP; j += 4) {
                const float4 t4 = *reinterpret_cast<const float4*>(s_T + (gi * kP + p) * JWP + j);
                if (j < JW) T[p][j] = t4.x;
                if (j + 1 < JW) T[p][j + 1] = t4.y;
                if (j + 2 < JW) T[p][j + 2] = t4.z;
                if (j + 3 < JW) T[p][j + 3] = t4.w;
            }
        }
        const int rho0 = gi * kP;
        const int64_t t0 = (int64_t)rho0 * g.down + g.off;
        const int rel0 = (int)(t0 / g.up) - g.b00;  // window start of the group inside a period
        for (int c = 0; c < kCT; ++c) {
            const int64_t row = c0 + c;
            if (row >= batch) break;
            const float* sx = s_x + c * WLP;
            float* __restrict__ yr = y + row * ld_y;
            for (int ic = 0; ic < kIT; ic += 32) {
                const int64_t i = i0 + ic + lane;
                if (i >= n_periods) break;
                const int rel = (ic + lane) * g.down + rel0;
                float acc[kP];
#pragma unroll
                for (int p = 0; p < kP; ++p) acc[p] = 0.0f;
#pragma unroll
                for (int j = 0; j < JW; ++j) {
                    const float w = sx[padi(rel + j)];
#pragma unroll
                    for (int p = 0; p < kP; ++p) acc[p] = fmaf(T[p][j], w, acc[p]);
                }
                const int64_t m0 = i * g.up + rho0;
#pragma unroll
                for (int p = 0; p < kP; ++p) {
                    if (rho0 + p < g.up && m0 + p < n_out) yr[m0 + p] = acc[p];
                }
            }
        }
    }
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

template <int QM>
int launch_fast(const PolyArgs& a, int Q, cudaStream_t st) {
    constexpr int JW = QM + kP - 1;
    constexpr int JWP = (JW + 3) / 4 * 4;
    PolyGeom g;
    g.up = a.up;
    g.down = a.down;
    g.Q = Q;
    g.off = a.off;
    g.G = (a.up + kP - 1) / kP;
    g.b00 = (int)((a.off) / a.up);
    int maxrel = 0;
    for (int gi = 0; gi < g.G; ++gi) {
        const int64_t t0 = (int64_t)(gi * kP) * a.down + a.off;
        maxrel = max(maxrel, (int)(t0 / a.up) - g.b00);
    }
    g.span = maxrel + JW;
    g.WL = (kIT - 1) * a.down + g.span;
    const int WLP = g.WL + g.WL / 32 + 1;
    const size_t smem = sizeof(float) * ((size_t)g.G * kP * JWP + (size_t)kCT * WLP);
    const int64_t n_periods = ceil_div(a.n_out, a.up);
    const int64_t per_row_group = ceil_div(n_periods, kIT);
    const int64_t grid = per_row_group * ceil_div(a.batch, kCT);
    SCIR_REQUIRE(grid <= 0x7fffffffLL, SCIR_ERR_UNSUPPORTED, "polyphase grid too large");
    const scir::DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    SCIR_REQUIRE((int)smem <= info->max_smem_optin, SCIR_ERR_UNSUPPORTED,
                 "polyphase tile needs %zu bytes of shared memory", smem);
    auto kern = poly_fast_kernel<QM>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<(unsigned)grid, kThreads, smem, st>>>(a.x, a.ld_x, a.batch, a.n, a.h, a.kh, g, a.y,
                                                 a.ld_y, a.n_out, n_periods, per_row_group);
    SCIR_LAUNCH_CHECK("poly_fast_kernel");
    return SCIR_OK;
}

}  // namespace

int launch_poly_simt(const PolyArgs& a, cudaStream_t st) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    const int64_t Q = ceil_div(a.kh, a.up);
    if (a.down <= a.up && a.up <= kMaxUp && Q <= 32 && a.down * (int64_t)kIT < (1 << 20)) {
        int rc = SCIR_ERR_UNSUPPORTED;
        if (Q <= 4) rc = launch_fast<4>(a, (int)Q, st);
        else if (Q <= 8) rc = launch_fast<8>(a, (int)Q, st);
        else if (Q <= 12) rc = launch_fast<12>(a, (int)Q, st);
        else if (Q <= 16) rc = launch_fast<16>(a, (int)Q, st);
        else if (Q <= 20) rc = launch_fast<20>(a, (int)Q, st);
        else if (Q <= 22) rc = launch_fast<22>(a, (int)Q, st);
        else if (Q <= 24) rc = launch_fast<24>(a, (int)Q, st);
        else if (Q <= 28) rc = launch_fast<28>(a, (int)Q, st);
        else rc = launch_fast<32>(a, (int)Q, st);
        if (rc != SCIR_ERR_UNSUPPORTED) return rc;
        clear_error();
    }
    const int64_t bpr = ceil_div(a.n_out, 256);
    const int64_t grid = bpr * a.batch;
    SCIR_REQUIRE(grid <= 0x7fffffffLL, SCIR_ERR_UNSUPPORTED, "polyphase grid too large");
    poly_generic_kernel<<<(unsigned)grid, 256, 0, st>>>(a.x, a.ld_x, a.n, a.h, a.kh, a.up, a.down,
                                                        a.off, a.y, a.ld_y, a.n_out, bpr);
    SCIR_LAUNCH_CHECK("poly_generic_kernel");
    return SCIR_OK;
}

}  // namespace scir
