// Batched FIR on the 5th-generation tensor cores (tcgen05, kind::f16) with
// split-bf16 operands and FP32 accumulation in TMEM.
//
// Contraction.  A tile is 128 channels (TMEM lanes) x 8U consecutive outputs
// o0 .. o0+8U-1.  With r = 8u + phi (phi = output phase, u' = U-1-u):
//   y[b][o0 + r] = sum_j X[b][o0 + s + j] * c[j - r]
//                = sum_j A[b][j] * B_phi[u'][j],   B_phi[u'][j] = G_phi[8u' + j],
//   G_phi[i] = c[i - 8(U-1) - phi]  (zero outside [0, k)).
// A (the signal window, K-major) comes straight from a TMA 2-D box with
// 128-byte swizzle.  Each phase operand B_phi is a Hankel matrix whose rows
// shift by 8 bf16 = 16 bytes: exactly the no-swizzle K-major core-matrix
// layout with a 16-byte leading (K) offset and a 128-byte stride (N) offset,
// so every B_phi is a descriptor pointing into a contiguous tap window in
// shared memory -- no im2col, no Toeplitz materialisation.  The 8 phases of
// one tile are 8 MMAs of N = U writing adjacent TMEM column ranges; with
// U = 64 a tile is 512 outputs and fills the 512 TMEM columns.
//
// Precision.  x and c are split into bf16 terms (x = x1 + x2 [+ x3]) by a
// prep pass into scratch memory; BF16X3 accumulates x1c1 + x1c2 + x2c1, BF16X6
// adds x1c3 + x2c2 + x3c1.  The dominant x1c1 and the cross terms are two
// passes of the kernel with their own FP32 accumulators: pass 0 writes x1c1,
// pass 1 adds the cross-term sum to it in the epilogue (measured: mixing
// them in one accumulator doubles to quadruples the error on 4,095-tap
// filters).
//
// Roles (192 threads, one CTA per SM, persistent over tiles):
//   warp 0    TMA producer: signal box(es) + 8 phase tap windows per term and
//             K chunk of 64 into an N-stage ring (full/empty mbarriers);
//   warp 1    one thread issues the MMAs and commits stages and tiles;
//   warps 2-5 epilogue: tcgen05.ld of the accumulator, phase interleave in
//             registers, 16-byte stores (pass 1: load, add, store).
// Every wait is bounded; a timeout sets the device error word, the CTA
// leaves its loops, frees its TMEM and exits.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace scir {
namespace {

constexpr int kM = 128;          // channels per tile = TMEM lanes
constexpr int kKC = 64;          // K per stage: one 128-byte swizzle atom of bf16
constexpr int kPh = 8;           // output phases (Hankel row shift 8 elements)
constexpr int kThreads = 192;
constexpr int kTmemCols = 512;
constexpr uint32_t kABytesTerm = kM * kKC * 2;  // 16 KB

struct TcGeom {
    int nstage, nchunks;
    int64_t padL, nA, s, n_out, batch, LG;
    int64_t blocks_per_cg, n_tiles;
    uint32_t stage_bytes, tx_bytes;
    int vec_store;
};

__global__ void split_signal_kernel(const float* __restrict__ x, int64_t ld_x, int64_t batch,
                                    int64_t n, int64_t padL, int64_t nA, int terms,
                                    __nv_bfloat16* __restrict__ xs) {
    const int64_t plane = batch * nA;
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nA;
             i += (int64_t)gridDim.x * blockDim.x) {
            const int64_t src = i - padL;
            const float v = (src >= 0 && src < n) ? __ldg(x + b * ld_x + src) : 0.0f;
            const __nv_bfloat16 h1 = __float2bfloat16_rn(v);
            const float r1 = v - __bfloat162float(h1);
            const __nv_bfloat16 h2 = __float2bfloat16_rn(r1);
            const int64_t e = b * nA + i;
            xs[e] = h1;
            xs[plane + e] = h2;
            if (terms == 3) xs[2 * plane + e] = __float2bfloat16_rn(r1 - __bfloat162float(h2));
        }
    }
}

__global__ void split_taps_kernel(const float* __restrict__ taps, int64_t k, int reverse, int U,
                                  int64_t LG, int terms, __nv_bfloat16* __restrict__ G) {
    const int64_t total = (int64_t)kPh * LG;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int ph = (int)(e / LG);
        const int64_t i = e % LG;
        const int64_t ci = i - 8 * (int64_t)(U - 1) - ph;
        const float v = (ci >= 0 && ci < k) ? __ldg(taps + (reverse ? k - 1 - ci : ci)) : 0.0f;
        const __nv_bfloat16 h1 = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h1);
        const __nv_bfloat16 h2 = __float2bfloat16_rn(r1);
        G[e] = h1;
        G[total + e] = h2;
        if (terms == 3) G[2 * total + e] = __float2bfloat16_rn(r1 - __bfloat162float(h2));
    }
}

// Products of a pass as (signal term, tap term).  Pass 0 is the dominant
// x1*c1; pass 1 is the cross terms x1c2, x2c1 (BF16X3) and x1c3, x2c2, x3c1
// (BF16X6 adds them).  Each pass accumulates in its own TMEM accumulator;
// pass 1's epilogue adds its sum to pass 0's output in FP32.  Cross terms
// added into the large x1*c1 sum would be rounded against its magnitude;
// kept apart they are rounded against their own, 2^-8 smaller, one.
template <int PASS>
__device__ __forceinline__ int prod_a(int p) {
    return PASS == 0 ? 0 : (p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 0 : p == 3 ? 1 : 2);
}
template <int PASS>
__device__ __forceinline__ int prod_b(int p) {
    return PASS == 0 ? 0 : (p == 0 ? 1 : p == 1 ? 0 : p == 2 ? 2 : p == 3 ? 1 : 0);
}

template <int U, int TA, int TB, int PASS, int NPROD>
__global__ void __launch_bounds__(kThreads, 1)
fir_tc_kernel(const __grid_constant__ CUtensorMap amap, const __nv_bfloat16* __restrict__ G,
              const TcGeom g, float* __restrict__ y, int64_t ld_y, unsigned* __restrict__ err) {
    constexpr int NCOL = kPh * U;                      // accumulator columns per tile
    constexpr int NACC = (kTmemCols / NCOL) >= 2 ? 2 : 1;  // tiles in flight in TMEM
    constexpr int WB = kKC + 8 * U;                    // tap window per phase per chunk
    constexpr uint32_t kABytes = TA * kABytesTerm;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)g.nstage * g.stage_bytes);
    uint64_t* empty = full + g.nstage;
    uint64_t* tfull = empty + g.nstage;
    uint64_t* tempty = tfull + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        if (lane == 0) {
            for (int s = 0; s < g.nstage; ++s) {
                mbar_init(&full[s], 1);
                mbar_init(&empty[s], 1);
            }
            for (int a = 0; a < 2; ++a) {
                mbar_init(&tfull[a], 1);
                mbar_init(&tempty[a], 4 * 32);
            }
            fence_barrier_init();
        }
        __syncwarp();
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            prefetch_tmap(&amap);
            uint32_t it = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < g.n_tiles; tile += gridDim.x) {
                const int64_t cg = tile / g.blocks_per_cg, blk = tile % g.blocks_per_cg;
                const int64_t xc0 = blk * NCOL + g.s + g.padL;
                for (int c = 0; c < g.nchunks; ++c, ++it) {
                    const int st = (int)(it % (uint32_t)g.nstage);
                    const uint32_t ph = (it / (uint32_t)g.nstage) & 1u;
                    if (!mbar_wait(&empty[st], ph ^ 1u)) {
                        atomicOr(err, kErrMbarTimeout);
                        ok = false;
                        break;
                    }
                    uint8_t* sb = base + (size_t)st * g.stage_bytes;
                    mbar_arrive_expect_tx(&full[st], g.tx_bytes);
#pragma unroll
                    for (int t = 0; t < TA; ++t)
                        tma_load_3d(sb + t * kABytesTerm, &amap, &full[st],
                                    (int32_t)(xc0 + (int64_t)c * kKC), (int32_t)(cg * kM), t);
                    uint8_t* bb = sb + kABytes;
#pragma unroll
                    for (int t = 0; t < TB; ++t)
                        for (int phz = 0; phz < kPh; ++phz)
                            bulk_load(bb + (t * kPh + phz) * WB * 2,
                                      G + ((int64_t)(t * kPh + phz) * g.LG + (int64_t)c * kKC),
                                      (uint32_t)(WB * 2), &full[st]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16_f32(kM, U);
            uint32_t it = 0, tcount = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < g.n_tiles; tile += gridDim.x, ++tcount) {
                const int a = (int)(tcount % NACC);
                const uint32_t aph = (tcount / NACC) & 1u;
                if (!mbar_wait(&tempty[a], aph ^ 1u)) {
                    atomicOr(err, kErrMbarTimeout);
                    break;
                }
                tc_fence_after();
                const uint32_t dbase = tmem + (uint32_t)(a * NCOL);
                for (int c = 0; c < g.nchunks; ++c, ++it) {
                    const int st = (int)(it % (uint32_t)g.nstage);
                    const uint32_t ph = (it / (uint32_t)g.nstage) & 1u;
                    if (!mbar_wait(&full[st], ph)) {
                        atomicOr(err, kErrMbarTimeout);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    // base descriptors of the stage; every MMA below reaches its
                    // operands through compile-time offsets (encoded in 16-byte units)
                    const uint32_t sa = smem_u32(base + (size_t)st * g.stage_bytes);
                    const uint64_t ad0 = smem_desc(sa, 16, 1024, 2);
                    const uint64_t bd0 = smem_desc(sa + kABytes, 16, 128, 0);
                    const uint32_t acc_c = c != 0 ? 1u : 0u;
#pragma unroll
                    for (int ks = 0; ks < kKC / 16; ++ks) {
#pragma unroll
                        for (int phz = 0; phz < kPh; ++phz) {
#pragma unroll
                            for (int p = 0; p < NPROD; ++p) {
                                const uint64_t ad = ad0 + (uint64_t)(
                                    (prod_a<PASS>(p) * kABytesTerm + ks * 32) >> 4);
                                const uint64_t bd = bd0 + (uint64_t)(
                                    ((prod_b<PASS>(p) * kPh + phz) * WB * 2 + ks * 32) >> 4);
                                tc_mma_f16(dbase + phz * U, ad, bd, idesc,
                                           (ks == 0 && p == 0) ? acc_c : 1u);
                            }
                        }
                    }
                    tc_commit(&empty[st]);
                }
                if (!ok) break;
                tc_commit(&tfull[a]);
            }
        }
    } else {
        const int q = warp & 3;  // TMEM lane quarter of this warp
        uint32_t tcount = 0;
        for (int64_t tile = blockIdx.x; tile < g.n_tiles; tile += gridDim.x, ++tcount) {
            const int a = (int)(tcount % NACC);
            const uint32_t aph = (tcount / NACC) & 1u;
            const bool ok = mbar_wait(&tfull[a], aph);
            if (!ok) {
                if (lane == 0) atomicOr(err, kErrMbarTimeout);
                break;
            }
            tc_fence_after();
            const int64_t cg = tile / g.blocks_per_cg, blk = tile % g.blocks_per_cg;
            const int64_t row = cg * kM + q * 32 + lane;
            const int64_t o0 = blk * NCOL;
            float* __restrict__ yr = y + row * ld_y;
            const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * NCOL);
#pragma unroll 1
            for (int u0 = 0; u0 < U; u0 += 16) {
                float v[kPh][16];
#pragma unroll
                for (int phz = 0; phz < kPh; ++phz) tmem_ld16(tb + phz * U + u0, v[phz]);
                tmem_wait_ld();
                if (row < g.batch) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int u = U - 1 - (u0 + i);
                        const int64_t o = o0 + 8 * u;
                        if (g.vec_store && o + 8 <= g.n_out) {
                            float4* p4 = reinterpret_cast<float4*>(yr + o);
                            float4 lo = make_float4(v[0][i], v[1][i], v[2][i], v[3][i]);
                            float4 hi = make_float4(v[4][i], v[5][i], v[6][i], v[7][i]);
                            if (PASS == 1) {
                                const float4 plo = p4[0], phi = p4[1];
                                lo.x += plo.x; lo.y += plo.y; lo.z += plo.z; lo.w += plo.w;
                                hi.x += phi.x; hi.y += phi.y; hi.z += phi.z; hi.w += phi.w;
                            }
                            p4[0] = lo;
                            p4[1] = hi;
                        } else {
#pragma unroll
                            for (int phz = 0; phz < kPh; ++phz)
                                if (o + phz < g.n_out)
                                    yr[o + phz] = PASS == 1 ? yr[o + phz] + v[phz][i] : v[phz][i];
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[a]);
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// One pass (PASS 0: x1*c1 into y; PASS 1: the cross terms added into y).
template <int U, int TA, int TB, int PASS, int NPROD>
int launch_pass(const FirArgs& a, const TcGeom& g0, const __nv_bfloat16* xs,
                const __nv_bfloat16* Gs, int terms, const DeviceInfo* info, unsigned* err,
                cudaStream_t st) {
    constexpr int WB = kKC + 8 * U;
    TcGeom g = g0;
    const uint32_t stage = TA * kABytesTerm + TB * kPh * WB * 2;
    g.stage_bytes = (stage + 1023) / 1024 * 1024;
    g.tx_bytes = stage;
    const size_t extra = 1024 + 8 * (2 * 4 + 4) + 16;
    const int nstage =
        (int)std::min<int64_t>(4, (info->max_smem_optin - (int64_t)extra) / g.stage_bytes);
    if (nstage < 2) return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR stage too large");
    g.nstage = nstage;
    const size_t smem = (size_t)nstage * g.stage_bytes + extra;
    CUtensorMap amap;
    int rc = make_tmap_3d(&amap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, xs, (uint64_t)g.nA,
                          (uint64_t)a.batch, (uint64_t)terms, (uint64_t)g.nA * 2,
                          (uint64_t)g.nA * 2 * (uint64_t)a.batch, kKC, kM, 1,
                          CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    auto kern = fir_tc_kernel<U, TA, TB, PASS, NPROD>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t grid = std::min<int64_t>(g.n_tiles, (int64_t)info->sm_count);
    kern<<<(unsigned)grid, kThreads, smem, st>>>(amap, Gs, g, a.y, a.ld_y, err);
    SCIR_LAUNCH_CHECK("fir_tc_kernel");
    return SCIR_OK;
}

template <int U, int TERMS>
int launch_tc(const FirArgs& a, cudaStream_t st) {
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    constexpr int NCOL = kPh * U;
    TcGeom g;
    g.s = a.s;
    g.padL = ((-a.s) % 8 + 8) % 8;
    g.nA = (a.n + g.padL + 7) / 8 * 8;
    g.n_out = a.n_out;
    g.batch = a.batch;
    const int64_t ktot = a.k + NCOL - 1;
    g.nchunks = (int)ceil_div(ktot, kKC);
    g.LG = (int64_t)g.nchunks * kKC + 8 * U;
    g.blocks_per_cg = ceil_div(a.n_out, NCOL);
    g.n_tiles = g.blocks_per_cg * ceil_div(a.batch, kM);
    g.vec_store = ((reinterpret_cast<uintptr_t>(a.y) & 15) == 0 && (a.ld_y & 3) == 0) ? 1 : 0;
    if (a.n + g.padL + 2 * NCOL + ktot >= (1LL << 31) || ceil_div(a.batch, kM) * kM >= (1LL << 31))
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR coordinates exceed 32 bits");
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");

    // split operands into scratch memory
    __nv_bfloat16* xs = nullptr;
    __nv_bfloat16* Gs = nullptr;
    const size_t xs_bytes = sizeof(__nv_bfloat16) * (size_t)TERMS * (size_t)a.batch * (size_t)g.nA;
    const size_t g_bytes = sizeof(__nv_bfloat16) * (size_t)TERMS * kPh * (size_t)g.LG;
    rc = scratch_alloc((void**)&xs, xs_bytes, st);
    if (rc) return rc;
    rc = scratch_alloc((void**)&Gs, g_bytes, st);
    if (rc) {
        scratch_free(xs, st);
        return rc;
    }
    {
        const unsigned gx = (unsigned)std::min<int64_t>(ceil_div(g.nA, 256), 4096);
        const unsigned gy = (unsigned)std::min<int64_t>(a.batch, 65535);
        split_signal_kernel<<<dim3(gx, gy), 256, 0, st>>>(a.x, a.ld_x, a.batch, a.n, g.padL, g.nA,
                                                          TERMS, xs);
        const unsigned gt = (unsigned)std::min<int64_t>(ceil_div((int64_t)kPh * g.LG, 256), 4096);
        split_taps_kernel<<<gt, 256, 0, st>>>(a.taps, a.k, a.reverse, U, g.LG, TERMS, Gs);
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) rc = set_error(SCIR_ERR_CUDA, "split kernels: %s", cudaGetErrorString(le));
    if (rc == SCIR_OK) rc = launch_pass<U, 1, 1, 0, 1>(a, g, xs, Gs, TERMS, info, err, st);
    if (rc == SCIR_OK) {
        if (TERMS == 2) rc = launch_pass<U, 2, 2, 1, 2>(a, g, xs, Gs, TERMS, info, err, st);
        else rc = launch_pass<U, 3, 3, 1, 5>(a, g, xs, Gs, TERMS, info, err, st);
    }
    scratch_free(xs, st);
    scratch_free(Gs, st);
    return rc;
}

}  // namespace

bool fir_tc_supported(const FirArgs& a) {
    return a.k >= 1 && a.n >= 1 && a.batch >= 1 && a.n_out >= 1 && a.n < (1LL << 30);
}

int launch_fir_tc(const FirArgs& a, int terms, cudaStream_t st) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    if (terms == 2) return launch_tc<64, 2>(a, st);
    return launch_tc<64, 3>(a, st);
}

bool poly_tc_supported(const PolyArgs&) { return false; }
int launch_poly_tc(const PolyArgs&, int, cudaStream_t) {
    return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase not built");
}

}  // namespace scir
