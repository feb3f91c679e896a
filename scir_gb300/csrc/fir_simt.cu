// Batched FIR on the CUDA cores (FP32), every output convention.
//
// Replaces the reference's one-thread-per-output PTX kernel
// (crates/scir-gpu/src/lib.rs:727-811, two global loads per tap, no reuse)
// and is the device form of its CPU loop (lib.rs:1134-1152).  One CTA per
// output tile of one row; the tile computation is in fir_tile.cuh.
#include "common.cuh"
#include "fir_tile.cuh"
#include "kernels.cuh"

namespace scir {
namespace {

template <int V, bool EXACT>
__global__ void __launch_bounds__(kFirThreads)
fir_simt_kernel(const float* __restrict__ x, int64_t ld_x, int64_t n,
                const float* __restrict__ taps, int64_t k, int reverse, int64_t s,
                float* __restrict__ y, int64_t ld_y, int64_t n_out,
                int64_t tiles_per_row, int chunk) {
    extern __shared__ __align__(16) float smem[];
    constexpr int TILE = kFirThreads * V;
    // 32-bit tile decode (the launcher keeps the grid below 2^31): a 64-bit
    // division by a runtime value is a long instruction sequence, and at short
    // filters every instruction of a tile's bookkeeping costs FMA issue slots
    const uint32_t tpr = (uint32_t)tiles_per_row;
    const uint32_t rowu = blockIdx.x / tpr;
    const int64_t row = rowu;
    const int64_t o0 = (int64_t)(blockIdx.x - rowu * tpr) * TILE;
    fir_tile<V, EXACT>(smem, x + row * ld_x, n, taps, k, reverse, s, y + row * ld_y, n_out, o0,
                       chunk);
}

template <int V, bool EXACT>
int launch_v(const FirArgs& a, cudaStream_t st) {
    constexpr int TILE = kFirThreads * V;
    const int64_t tiles = ceil_div(a.n_out, TILE);
    const int64_t grid = tiles * a.batch;
    SCIR_REQUIRE(grid <= 0x7fffffffLL, SCIR_ERR_UNSUPPORTED,
                 "FIR grid of %lld tiles exceeds one launch", (long long)grid);
    const int64_t kpad = (a.k + V - 1) / V * V;
    const int chunk = (int)(kpad < kFirMaxChunk ? kpad : kFirMaxChunk);
    const size_t smem = fir_tile_smem_bytes(V, chunk);
    auto kern = fir_simt_kernel<V, EXACT>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<(unsigned)grid, kFirThreads, smem, st>>>(a.x, a.ld_x, a.n, a.taps, a.k, a.reverse, a.s,
                                                    a.y, a.ld_y, a.n_out, tiles, chunk);
    SCIR_LAUNCH_CHECK("fir_simt_kernel");
    return SCIR_OK;
}

}  // namespace

int launch_fir_simt(const FirArgs& a, bool exact, cudaStream_t st, int v) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    // v = 8 or 16 outputs per thread (autotuned), else by tap count
    const bool wide = v == 16 ? true : v == 8 ? false : a.k >= 128;
    if (exact) return wide ? launch_v<16, true>(a, st) : launch_v<8, true>(a, st);
    return wide ? launch_v<16, false>(a, st) : launch_v<8, false>(a, st);
}

}  // namespace scir
