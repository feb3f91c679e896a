// Batched FIR on the 5th-generation tensor cores (tcgen05, kind::f16) with
// split-bf16 operands and FP32 accumulation in TMEM.
//
// Contraction.  Outputs are grouped in windows of 1,024 (o0 .. o0+1023) and
// split by output phase phi = r mod 8 (r = o - o0 = 8u + phi, u < 128).  For
// one phase, with u' = 127 - u:
//   y[b][o0 + r] = sum_j X[b][o0 + s + j] * c[j - r]
//                = sum_j A[b][j] * B_phi[u'][j],   B_phi[u'][j] = G_phi[8u' + j],
//   G_phi[i] = c[i - 8*127 - phi]  (zero outside [0, k)).
// A (the signal window of 128 channels, K-major) comes from a TMA box with
// 128-byte swizzle.  B_phi is a Hankel matrix whose rows shift by 8 bf16 =
// 16 bytes: exactly the no-swizzle K-major core-matrix layout with a 16-byte
// leading (K) offset and a 128-byte stride (N) offset, so B_phi is a
// descriptor into a contiguous tap window in shared memory -- no im2col, no
// Toeplitz matrix.  One MMA is M=128 (channels) x N=128 (outputs of one
// phase) x K=16.
//
// Tile shape (measured on GB300, 1,024 ch x 262,144 x 4,095 taps).  Each
// phase operand pads K by the window (k + 8N - 1), and every MMA reads its A
// and B tiles from shared memory, which caps the MMA rate near 120 B/cycle
// of operand reads per SM.  N = 64 is bound by a fixed ~55-cycle cost per
// MMA; N = 256 (two phases per tile) pads K by 2,048 and writes 8 of every
// 32 output bytes per store; N = 128 with four phases per tile (the four
// 128-column accumulators fill TMEM's 512 columns) was fastest.  SCIR_TC_N
// selects 256 at compile time.
//
// Tiles.  A tile is (128 channels, one window, one phase group).  The phase
// groups of a window are consecutive tile indices, so they run on
// neighbouring SMs at the same time: the signal box is shared in L2 and the
// tiles' 16-byte output pieces complete each 32-byte sector in L2.
//
// Precision.  x and c are split into bf16 terms (x = x1 + x2 [+ x3]) by a
// prep pass into scratch memory; BF16X3 accumulates x1c1 + x1c2 + x2c1, BF16X6
// adds x1c3 + x2c2 + x3c1.  The dominant x1c1 and the cross terms are two
// passes of the kernel with their own FP32 accumulators: pass 0 writes x1c1,
// pass 1 adds the cross-term sum to it in the epilogue (measured: mixing
// them in one accumulator doubles to quadruples the error on 4,095-tap
// filters).
//
// Roles (320 threads, one CTA per SM, persistent over tiles):
//   warp 0    TMA producer: signal box(es) + the tile's phase tap windows per term and
//             K chunk of 64 into an N-stage ring (full/empty mbarriers);
//   warp 1    one thread issues the MMAs and commits stages and tiles;
//   warps 2-9 epilogue: tcgen05.ld of the accumulators (two warps per TMEM
//             lane quarter, each half of the columns), one vector store of
//             the tile's adjacent phases per column (pass 1: load, add, store).
// Every wait is bounded; a timeout sets the device error word, the CTA
// leaves its loops, frees its TMEM and exits.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

namespace scir {
namespace {

constexpr int kM = 128;          // channels per tile = TMEM lanes
constexpr int kKC = 64;          // K per stage: one 128-byte swizzle atom of bf16
constexpr int kPh = 8;           // output phases (Hankel row shift 8 elements)
#ifndef SCIR_TC_N
#define SCIR_TC_N 128
#endif
constexpr int kU = SCIR_TC_N;    // rows of a phase operand = MMA N (128 or 256)
constexpr int kPhT = 512 / kU;   // phases per tile: the accumulators fill TMEM
constexpr int kGroups = kPh / kPhT;  // phase groups per window
constexpr int kNCOL = kPh * kU;  // outputs per window
constexpr int kWB = kKC + 8 * kU;  // tap window per phase per chunk (elements)
constexpr uint32_t kBBytesPh = kWB * 2;
constexpr int kEpiWarps = 8;
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kTmemCols = 512;
constexpr uint32_t kABytesTerm = kM * kKC * 2;  // 16 KB

struct TcGeom {
    int nstage, nchunks;
    int64_t padL, nA, s, n_out, batch, LG;
    int64_t blocks_per_cg, n_tiles;  // windows per channel group; tiles in total
    uint32_t stage_bytes, tx_bytes;
    int vec_store;
};

// x -> bf16 term planes xs[t][b][i] = term t of x[b][i - padL] (zero
// outside the row).  Each thread converts 4 consecutive elements: the loads
// are coalesced across the warp and each plane gets one 8-byte store.
__global__ void split_signal_kernel(const float* __restrict__ x, int64_t ld_x, int64_t batch,
                                    int64_t n, int64_t padL, int64_t nA, int terms,
                                    __nv_bfloat16* __restrict__ xs) {
    const int64_t plane = batch * nA;
    const int64_t groups = nA / 4;  // nA is a multiple of 8
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        const float* __restrict__ xr = x + b * ld_x;
        for (int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < groups;
             gi += (int64_t)gridDim.x * blockDim.x) {
            const int64_t i0 = gi * 4;
            __nv_bfloat162 p[3][2];
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                float v[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int64_t src = i0 + j + h - padL;
                    v[h] = (src >= 0 && src < n) ? __ldg(xr + src) : 0.0f;
                }
                const __nv_bfloat162 h1 = __floats2bfloat162_rn(v[0], v[1]);
                const float2 f1 = __bfloat1622float2(h1);
                const float r0 = v[0] - f1.x, r1 = v[1] - f1.y;
                const __nv_bfloat162 h2 = __floats2bfloat162_rn(r0, r1);
                const float2 f2 = __bfloat1622float2(h2);
                p[0][j / 2] = h1;
                p[1][j / 2] = h2;
                p[2][j / 2] = __floats2bfloat162_rn(r0 - f2.x, r1 - f2.y);
            }
            const int64_t e = b * nA + i0;
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                if (t < terms) {
                    uint2 w;
                    w.x = *reinterpret_cast<const uint32_t*>(&p[t][0]);
                    w.y = *reinterpret_cast<const uint32_t*>(&p[t][1]);
                    *reinterpret_cast<uint2*>(xs + t * plane + e) = w;
                }
            }
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

// The kPhT adjacent outputs of one accumulator column set, as one vector.
using VecT = std::conditional<kPhT == 4, float4, float2>::type;
__device__ __forceinline__ void vec_set(float2& r, const float (&v)[2][16], int i) {
    r = make_float2(v[0][i], v[1][i]);
}
__device__ __forceinline__ void vec_add(float2& r, const float (&v)[2][16], int i) {
    r.x += v[0][i];
    r.y += v[1][i];
}
__device__ __forceinline__ void vec_set(float4& r, const float (&v)[4][16], int i) {
    r = make_float4(v[0][i], v[1][i], v[2][i], v[3][i]);
}
__device__ __forceinline__ void vec_add(float4& r, const float (&v)[4][16], int i) {
    r.x += v[0][i];
    r.y += v[1][i];
    r.z += v[2][i];
    r.w += v[3][i];
}

template <int TA, int TB, int PASS, int NPROD>
__global__ void __launch_bounds__(kThreads, 1)
fir_tc_kernel(const __grid_constant__ CUtensorMap amap, const __nv_bfloat16* __restrict__ G,
              const TcGeom g, float* __restrict__ y, int64_t ld_y, unsigned* __restrict__ err) {
    constexpr uint32_t kABytes = TA * kABytesTerm;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)g.nstage * g.stage_bytes);
    uint64_t* empty = full + g.nstage;
    uint64_t* tfull = empty + g.nstage;
    uint64_t* tempty = tfull + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        if (lane == 0) {
            for (int s = 0; s < g.nstage; ++s) {
                mbar_init(&full[s], 1);
                mbar_init(&empty[s], 1);
            }
            mbar_init(tfull, 1);
            mbar_init(tempty, kEpiWarps * 32);
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
                const int pg = (int)(tile % kGroups);
                const int64_t w = tile / kGroups;
                const int64_t cg = w / g.blocks_per_cg, blk = w % g.blocks_per_cg;
                const int64_t xc0 = blk * kNCOL + g.s + g.padL;
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
#pragma unroll
                        for (int l = 0; l < kPhT; ++l)
                            bulk_load(bb + (t * kPhT + l) * kBBytesPh,
                                      G + ((int64_t)(t * kPh + kPhT * pg + l) * g.LG +
                                           (int64_t)c * kKC),
                                      kBBytesPh, &full[st]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16_f32(kM, kU);
            uint32_t it = 0, tcount = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < g.n_tiles; tile += gridDim.x, ++tcount) {
                if (!mbar_wait(tempty, (tcount & 1u) ^ 1u)) {
                    atomicOr(err, kErrMbarTimeout);
                    break;
                }
                tc_fence_after();
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
                        for (int l = 0; l < kPhT; ++l) {
#pragma unroll
                            for (int p = 0; p < NPROD; ++p) {
                                const uint64_t ad = ad0 + (uint64_t)(
                                    (prod_a<PASS>(p) * kABytesTerm + ks * 32) >> 4);
                                const uint64_t bd = bd0 + (uint64_t)(
                                    ((prod_b<PASS>(p) * kPhT + l) * kBBytesPh + ks * 32) >> 4);
                                tc_mma_f16(tmem + l * kU, ad, bd, idesc,
                                           (ks == 0 && p == 0) ? acc_c : 1u);
                            }
                        }
                    }
                    tc_commit(&empty[st]);
                }
                if (!ok) break;
                tc_commit(tfull);
            }
        }
    } else {
        const int q = warp & 3;               // TMEM lane quarter of this warp
        const int half = (warp - 2) >> 2;     // which 128 of the 256 columns
        uint32_t tcount = 0;
        for (int64_t tile = blockIdx.x; tile < g.n_tiles; tile += gridDim.x, ++tcount) {
            if (!mbar_wait(tfull, tcount & 1u)) {
                if (lane == 0) atomicOr(err, kErrMbarTimeout);
                break;
            }
            tc_fence_after();
            const int pg = (int)(tile % kGroups);
            const int64_t w = tile / kGroups;
            const int64_t cg = w / g.blocks_per_cg, blk = w % g.blocks_per_cg;
            const int64_t row = cg * kM + q * 32 + lane;
            const int64_t o0 = blk * kNCOL + kPhT * pg;
            float* __restrict__ yr = y + row * ld_y;
            const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
            for (int u0 = half * (kU / 2); u0 < (half + 1) * (kU / 2); u0 += 16) {
                float v[kPhT][16];
#pragma unroll
                for (int l = 0; l < kPhT; ++l) tmem_ld16(tb + l * kU + u0, v[l]);
                tmem_wait_ld();
                if (row < g.batch) {
                    // column u0 + i holds output ob - 8i (and the next kPhT - 1)
                    const int64_t ob = o0 + 8 * (kU - 1 - u0);
                    if (g.vec_store && ob + kPhT <= g.n_out) {
                        VecT r[16];
                        if (PASS == 1) {
                            // all loads first: 16 independent requests in flight
#pragma unroll
                            for (int i = 0; i < 16; ++i)
                                r[i] = *reinterpret_cast<const VecT*>(yr + ob - 8 * i);
#pragma unroll
                            for (int i = 0; i < 16; ++i) vec_add(r[i], v, i);
                        } else {
#pragma unroll
                            for (int i = 0; i < 16; ++i) vec_set(r[i], v, i);
                        }
#pragma unroll
                        for (int i = 0; i < 16; ++i) *reinterpret_cast<VecT*>(yr + ob - 8 * i) = r[i];
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
#pragma unroll
                            for (int l = 0; l < kPhT; ++l) {
                                const int64_t o = ob - 8 * i + l;
                                if (o < g.n_out) yr[o] = PASS == 1 ? yr[o] + v[l][i] : v[l][i];
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(tempty);
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// One pass (PASS 0: x1*c1 into y; PASS 1: the cross terms added into y).
template <int TA, int TB, int PASS, int NPROD>
int launch_pass(const FirArgs& a, const TcGeom& g0, const __nv_bfloat16* xs,
                const __nv_bfloat16* Gs, int terms, const DeviceInfo* info, unsigned* err,
                cudaStream_t st) {
    TcGeom g = g0;
    const uint32_t stage = TA * kABytesTerm + TB * kPhT * kBBytesPh;
    g.stage_bytes = (stage + 1023) / 1024 * 1024;
    g.tx_bytes = stage;
    const size_t extra = 1024 + 8 * (2 * 8 + 2) + 16;
    const int nstage =
        (int)std::min<int64_t>(8, (info->max_smem_optin - (int64_t)extra) / g.stage_bytes);
    if (nstage < 2) return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR stage too large");
    g.nstage = nstage;
    const size_t smem = (size_t)nstage * g.stage_bytes + extra;
    CUtensorMap amap;
    int rc = make_tmap_3d(&amap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, xs, (uint64_t)g.nA,
                          (uint64_t)a.batch, (uint64_t)terms, (uint64_t)g.nA * 2,
                          (uint64_t)g.nA * 2 * (uint64_t)a.batch, kKC, kM, 1,
                          CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    auto kern = fir_tc_kernel<TA, TB, PASS, NPROD>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t grid = std::min<int64_t>(g.n_tiles, (int64_t)info->sm_count);
    kern<<<(unsigned)grid, kThreads, smem, st>>>(amap, Gs, g, a.y, a.ld_y, err);
    SCIR_LAUNCH_CHECK("fir_tc_kernel");
    return SCIR_OK;
}

template <int TERMS>
int launch_tc(const FirArgs& a, cudaStream_t st) {
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    TcGeom g;
    g.s = a.s;
    g.padL = ((-a.s) % 8 + 8) % 8;
    g.nA = (a.n + g.padL + 7) / 8 * 8;
    g.n_out = a.n_out;
    g.batch = a.batch;
    const int64_t ktot = a.k + kNCOL - 1;
    g.nchunks = (int)ceil_div(ktot, kKC);
    g.LG = (int64_t)g.nchunks * kKC + 8 * kU;
    g.blocks_per_cg = ceil_div(a.n_out, kNCOL);
    g.n_tiles = g.blocks_per_cg * ceil_div(a.batch, kM) * kGroups;
    g.vec_store = ((reinterpret_cast<uintptr_t>(a.y) % (4 * kPhT)) == 0 && (a.ld_y % kPhT) == 0) ? 1 : 0;
    if (a.n + g.padL + 2 * kNCOL + ktot >= (1LL << 31) || ceil_div(a.batch, kM) * kM >= (1LL << 31))
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
        const unsigned gx = (unsigned)std::min<int64_t>(ceil_div(g.nA / 4, 256), 4096);
        const unsigned gy = (unsigned)std::min<int64_t>(a.batch, 65535);
        split_signal_kernel<<<dim3(gx, gy), 256, 0, st>>>(a.x, a.ld_x, a.batch, a.n, g.padL, g.nA,
                                                          TERMS, xs);
        const unsigned gt = (unsigned)std::min<int64_t>(ceil_div((int64_t)kPh * g.LG, 256), 4096);
        split_taps_kernel<<<gt, 256, 0, st>>>(a.taps, a.k, a.reverse, kU, g.LG, TERMS, Gs);
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) rc = set_error(SCIR_ERR_CUDA, "split kernels: %s", cudaGetErrorString(le));
    if (rc == SCIR_OK) rc = launch_pass<1, 1, 0, 1>(a, g, xs, Gs, TERMS, info, err, st);
    if (rc == SCIR_OK) {
        if (TERMS == 2) rc = launch_pass<2, 2, 1, 2>(a, g, xs, Gs, TERMS, info, err, st);
        else rc = launch_pass<3, 3, 1, 5>(a, g, xs, Gs, TERMS, info, err, st);
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
    if (terms == 2) return launch_tc<2>(a, st);
    return launch_tc<3>(a, st);
}

}  // namespace scir
