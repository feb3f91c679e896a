// Batched FIR on the 5th-generation tensor cores (tcgen05, kind::f16) with
// split bf16 or fp16 operands and FP32 accumulation in TMEM, in one pass.
//
// Contraction.  Outputs are grouped in windows of 8U (o0 .. o0 + 8U - 1; U =
// 128 or 256 rows per phase operand) and split by output phase phi = r mod 8
// (r = o - o0 = 8u + phi, u < U).  For one phase, with u' = U - 1 - u and the
// signal window starting at the sample xa = o0 + s - m (m = s mod 8, the
// same for every window, so xa is a multiple of 8 -- 16 bytes of 16-bit
// terms -- as a TMA coordinate must be):
//   y[b][o0 + r] = sum_J X[b][xa + J] * c[J - m - r]
//                = sum_J A[b][J] * B_phi[u'][J],   B_phi[u'][J] = G_phi[8u' + J],
//   G_phi[i] = c[i - 8(U-1) - phi - m]  (zero outside [0, k)).
// A (128 channels x 64 samples per K chunk, K-major, 128-byte swizzle) is a
// TMA box of the signal's term planes, which a split kernel writes once per
// call (x = x1 + x2 [+ x3]).  B_phi is a Hankel matrix whose rows shift by 8
// elements = 16 bytes: exactly the no-swizzle K-major core-matrix layout with
// a 16-byte leading (K) offset and a 128-byte stride (N) offset, so B_phi is
// a descriptor into a contiguous tap window in shared memory -- no im2col,
// no Toeplitz matrix.  One MMA is M=128 (channels) x N<=U (outputs of one
// phase) x K=16.
//
// Precision.  x = x1 + x2 [+ x3] and c = c1 + c2 [+ c3] in bf16 terms;
// BF16X3 forms x1c1 + (x1c2 + x2c1), BF16X6 adds x1c3 + x2c2 + x3c1.
// FP16X3 forms the three products of BF16X3 from two fp16 terms: fp16 keeps
// 11 significant bits to bf16's 8, so x1 + x2 holds 22 bits of x (bf16:
// 16) and the dropped x2c2 is 2^-22 of x1c1 -- BF16X6's accuracy for
// BF16X3's MMAs.  fp16's range is narrow, so every signal row is scaled by
// 2^e before the split (max |x| 2^e < 2^15, from a max pass over the row's
// finite samples) and the taps by their own 2^f; the epilogue multiplies by
// 2^-(e+f), which is exact.  The dominant x1c1 and the sum of the cross terms
// go to two separate FP32 accumulators (cross terms added into the large
// x1c1 sum would be rounded against its magnitude; kept apart they are
// rounded against their own, smaller, one), and the epilogue adds the two.
// A tile's two 256-column accumulators fill TMEM's 512 columns.
//
// Ramps.  In the first and last 2U/16 K chunks of a window only some rows
// of a phase operand meet non-zero taps; the MMAs of such a chunk cover just
// the 16-row groups live at some K step of the chunk in any of the tile's
// phases (N = 16 .. U, B and D offset to the first live group).  The
// accumulators are zeroed by the epilogue after it reads them, so every MMA
// accumulates and columns a ramp MMA skips stay zero.  Measured on 1,024 x
// 262,144 x 4,095 (FP16X3 step, U = 128): live rows per K step 5.50 ms, one
// row range per chunk 4.98 ms -- the single issuing thread, not the tensor
// pipe, was the limit.
//
// Tiles.  A tile is (128 channels, one window, 256/U phases); the 8U/256
// phase groups of a window are consecutive tile indices, so they run on
// neighbouring SMs at the same time and share the signal rows in L2.  Long
// filters take U = 256 (N = 256 MMAs read fewer operand bytes per product),
// shorter ones U = 128 (half the ramp length); the ragged bucket uses 128.
//
// Why planes in memory rather than a split inside this kernel: the MMAs
// read their A and B tiles from shared memory at about the rate shared
// memory delivers, so every other shared-memory access slows them.  A
// variant whose converter warps loaded the f32 rows and stored the bf16
// terms into the A layout themselves was measured at 11.0 ms (BF16X6) /
// 7.3 ms (BF16X3) on 1,024 x 262,144 x 4,095 against 9.5 / 6.0 ms for TMA
// loads of pre-split planes: the loads through L1 and the stores competed
// with the operand reads.
//
// Roles (576 threads, one CTA per SM, persistent over tiles):
//   warp 0     TMA producer: per K chunk the signal box of every term and the
//              tile's tap windows (phases x terms) into an N-stage ring
//              (full barrier with tx count);
//   warp 1     one thread issues the MMAs (per K chunk one row range, N
//              and operand base; every offset within the chunk a
//              constant) and commits stages and tiles;
//   warps 2-17 epilogue: tcgen05.ld of both accumulators (four warps per
//              TMEM lane quarter, U/4 columns each), the sum into registers,
//              TMEM zeroed and released to the MMA thread, then the global
//              stores (U = 128: one 8-byte store of the tile's two adjacent
//              phases per column; U = 256: 4-byte stores).
// Every wait is bounded; a timeout sets the device error word and the CTA
// leaves its loops; the producer first waits (bounded) for its copies in
// flight and the MMA thread for its MMAs, then TMEM is freed.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace scir {
namespace {

constexpr int kM = 128;          // channels per tile = TMEM lanes
constexpr int kKC = 64;          // K per stage: one 128-byte swizzle atom of bf16
constexpr int kPh = 8;           // output phases (Hankel row shift 8 elements)
// Tile geometry for U rows per phase operand (= the MMA's largest N).  U =
// 128 takes two output phases per tile, U = 256 one; either way the tile's
// two FP32 accumulators are 256 columns each and fill TMEM's 512.
template <int U>
struct TcShape {
    static constexpr int kU = U;
    static constexpr int kPhT = 256 / U;        // phases per tile
    static constexpr int kGroups = kPh / kPhT;  // phase groups (tiles) per window
    static constexpr int kNCOL = kPh * U;       // outputs per window
    static constexpr int kWB = kKC + 8 * U;     // tap window per phase per chunk (elements)
    static constexpr uint32_t kBBytesPh = kWB * 2;
};
using RaggedShape = TcShape<128>;  // the ragged bucket's tiles
constexpr int kEpiWarps = 16;      // four per TMEM lane quarter
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr int kTmemCols = 512;
constexpr uint32_t kABytesTerm = kM * kKC * 2;  // 16 KB
constexpr int kCrossCol = 256;                  // first column of the cross accumulators

// One operand element in the term planes: bf16 or fp16, by form.
using op16 = uint16_t;

struct TcGeom {
    int nstage, nchunks, m;
    int64_t xa0, n_out, batch, LG, k;
    int64_t blocks_per_cg, n_tiles;  // windows per channel group; tiles in total
    uint32_t stage_bytes, tx_bytes;
    int vec_store;
};

// Splits 4 floats into 2 or 3 bf16 terms, each packed as 4 bf16 (8 bytes).
__device__ __forceinline__ void split4_any(const float4 v, int terms, uint2 (&out)[3]) {
    const __nv_bfloat162 a1 = __floats2bfloat162_rn(v.x, v.y);
    const __nv_bfloat162 b1 = __floats2bfloat162_rn(v.z, v.w);
    const float2 fa1 = __bfloat1622float2(a1), fb1 = __bfloat1622float2(b1);
    const float ra0 = v.x - fa1.x, ra1 = v.y - fa1.y, rb0 = v.z - fb1.x, rb1 = v.w - fb1.y;
    const __nv_bfloat162 a2 = __floats2bfloat162_rn(ra0, ra1);
    const __nv_bfloat162 b2 = __floats2bfloat162_rn(rb0, rb1);
    out[0].x = *reinterpret_cast<const uint32_t*>(&a1);
    out[0].y = *reinterpret_cast<const uint32_t*>(&b1);
    out[1].x = *reinterpret_cast<const uint32_t*>(&a2);
    out[1].y = *reinterpret_cast<const uint32_t*>(&b2);
    out[2] = make_uint2(0u, 0u);
    if (terms == 3) {
        const float2 fa2 = __bfloat1622float2(a2), fb2 = __bfloat1622float2(b2);
        const __nv_bfloat162 a3 = __floats2bfloat162_rn(ra0 - fa2.x, ra1 - fa2.y);
        const __nv_bfloat162 b3 = __floats2bfloat162_rn(rb0 - fb2.x, rb1 - fb2.y);
        out[2].x = *reinterpret_cast<const uint32_t*>(&a3);
        out[2].y = *reinterpret_cast<const uint32_t*>(&b3);
    }
}

// ---- FP16X3 scaling.  mx holds the bit pattern of max |v| over the finite
// values of a row (0 for none); a row is scaled by 2^f16_shift(mx) so its
// largest magnitude lies in [2^14, 2^15) (fp16 holds up to 65,504), whatever
// the row's range: shifts lie in [-113, 140], applied as two power-of-two
// factors (each within float's exponent range, so every product is exact)
// and the sum of a row's and the taps' shifts is undone by three.
__device__ __forceinline__ int f16_shift(unsigned maxbits) {
    if (maxbits == 0u || maxbits >= 0x7f800000u) return 0;
    const int E = (int)(maxbits >> 23);  // biased exponent: max |v| < 2^(E - 126)
    return 141 - (E > 0 ? E : 1);
}
__device__ __forceinline__ float pow2f(int e) {  // 2^e, e in [-126, 127]
    return __int_as_float((e + 127) << 23);
}
// The two factors of 2^sh, sh in [-113, 140].
struct Scale2 {
    float a, b;
};
__device__ __forceinline__ Scale2 scale2(int sh) { return {pow2f(sh / 2), pow2f(sh - sh / 2)}; }

__device__ __forceinline__ unsigned finite_abs_max(unsigned m, float f) {
    const unsigned b = __float_as_uint(f) & 0x7fffffffu;
    return (b < 0x7f800000u && b > m) ? b : m;
}

// Max |v| over the finite values of v[0, len), folded into *out as bits
// with atomicMax (the order of non-negative floats is the order of their
// bit patterns).  16-byte loads from the first 16-byte boundary on, four in
// flight per thread.
__device__ __forceinline__ void absmax_segment(const float* __restrict__ v, int64_t len,
                                               unsigned* out) {
    unsigned m = 0u;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nt = (int64_t)gridDim.x * blockDim.x;
    int64_t head = (int64_t)(((16u - (unsigned)(reinterpret_cast<uintptr_t>(v) & 15u)) & 15u) / 4u);
    if (head > len) head = len;
    if (t < head) m = finite_abs_max(m, __ldg(v + t));
    const float4* __restrict__ v4 = reinterpret_cast<const float4*>(v + head);
    const int64_t n4 = (len - head) / 4;
    for (int64_t i = t; i < n4; i += 4 * nt) {
        float4 q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            q[u] = i + u * nt < n4 ? __ldg(v4 + i + u * nt) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            m = finite_abs_max(finite_abs_max(m, q[u].x), q[u].y);
            m = finite_abs_max(finite_abs_max(m, q[u].z), q[u].w);
        }
    }
    const int64_t tail = head + 4 * n4 + t;
    if (tail < len) m = finite_abs_max(m, __ldg(v + tail));
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// mx[b] for every signal row b < batch, mx[batch] for the taps (mx zeroed).
__global__ void absmax_rows_kernel(const float* __restrict__ x, int64_t ld_x, int64_t batch,
                                   int64_t n, const float* __restrict__ taps, int64_t k,
                                   unsigned* __restrict__ mx) {
    for (int64_t b = blockIdx.y; b <= batch; b += gridDim.y)
        absmax_segment(b < batch ? x + b * ld_x : taps, b < batch ? n : k, mx + b);
}

// 4 floats times 2^e split into two fp16 terms, packed as 4 fp16 (8 bytes) each.
__device__ __forceinline__ void split4_f16(const float4 v, Scale2 sc, uint2 (&out)[3]) {
    const float s0 = v.x * sc.a * sc.b, s1 = v.y * sc.a * sc.b, s2 = v.z * sc.a * sc.b,
                s3 = v.w * sc.a * sc.b;
    const __half2 a1 = __floats2half2_rn(s0, s1);
    const __half2 b1 = __floats2half2_rn(s2, s3);
    const float2 fa1 = __half22float2(a1), fb1 = __half22float2(b1);
    const __half2 a2 = __floats2half2_rn(s0 - fa1.x, s1 - fa1.y);
    const __half2 b2 = __floats2half2_rn(s2 - fb1.x, s3 - fb1.y);
    out[0].x = *reinterpret_cast<const uint32_t*>(&a1);
    out[0].y = *reinterpret_cast<const uint32_t*>(&b1);
    out[1].x = *reinterpret_cast<const uint32_t*>(&a2);
    out[1].y = *reinterpret_cast<const uint32_t*>(&b2);
    out[2] = make_uint2(0u, 0u);
}

// One tap value as its operand terms (bf16: 2 or 3 terms; fp16: 2 terms of
// v 2^e).
template <bool F16>
__device__ __forceinline__ void split_tap(float v, int terms, Scale2 sc, op16 (&t)[3]) {
    if (F16) {
        const float s = v * sc.a * sc.b;
        const __half h1 = __float2half_rn(s);
        t[0] = __half_as_ushort(h1);
        t[1] = __half_as_ushort(__float2half_rn(s - __half2float(h1)));
        t[2] = 0;
    } else {
        const __nv_bfloat16 h1 = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h1);
        const __nv_bfloat16 h2 = __float2bfloat16_rn(r1);
        t[0] = __bfloat16_as_ushort(h1);
        t[1] = __bfloat16_as_ushort(h2);
        t[2] = terms == 3 ? __bfloat16_as_ushort(__float2bfloat16_rn(r1 - __bfloat162float(h2)))
                          : (op16)0;
    }
}

// x -> term planes xs[t][b][i] = term t of x[b][i] (zero for n <= i < nA);
// FP16X3 scales row b by 2^f16_shift(mx[b]) first.  Each thread converts 8
// consecutive elements (two 16-byte loads where the row allows) and gives
// each plane one 16-byte store; the loads and stores are coalesced across the
// warp.
template <bool F16>
__global__ void split_signal_kernel(const float* __restrict__ x, int64_t ld_x, int64_t batch,
                                    int64_t n, int64_t nA, int terms,
                                    const unsigned* __restrict__ mx, op16* __restrict__ xs) {
    const int64_t plane = batch * nA;
    const int64_t groups = nA / 8;  // nA is a multiple of 8
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        const float* __restrict__ xr = x + b * ld_x;
        const Scale2 scale = scale2(F16 ? f16_shift(mx[b]) : 0);
        const bool al = (reinterpret_cast<uintptr_t>(xr) & 15u) == 0;
        for (int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < groups;
             gi += (int64_t)gridDim.x * blockDim.x) {
            const int64_t i0 = gi * 8;
            float e[8];
            if (al && i0 + 8 <= n) {
                const float4 q0 = __ldg(reinterpret_cast<const float4*>(xr + i0));
                const float4 q1 = __ldg(reinterpret_cast<const float4*>(xr + i0 + 4));
                e[0] = q0.x, e[1] = q0.y, e[2] = q0.z, e[3] = q0.w;
                e[4] = q1.x, e[5] = q1.y, e[6] = q1.z, e[7] = q1.w;
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) e[j] = i0 + j < n ? __ldg(xr + i0 + j) : 0.0f;
            }
            uint2 lo[3], hi[3];
            if (F16) {
                split4_f16(make_float4(e[0], e[1], e[2], e[3]), scale, lo);
                split4_f16(make_float4(e[4], e[5], e[6], e[7]), scale, hi);
            } else {
                split4_any(make_float4(e[0], e[1], e[2], e[3]), terms, lo);
                split4_any(make_float4(e[4], e[5], e[6], e[7]), terms, hi);
            }
            const int64_t o = b * nA + i0;
#pragma unroll
            for (int t = 0; t < 3; ++t)
                if (t < terms)
                    *reinterpret_cast<uint4*>(xs + t * plane + o) =
                        make_uint4(lo[t].x, lo[t].y, hi[t].x, hi[t].y);
        }
    }
}

// Tap operand planes G[t][phi][i] = term t of c[i - 8*(U-1) - phi - m]
// (zero outside [0, k)), c = taps or reversed taps (FP16X3: times
// 2^f16_shift(*mx)).
template <bool F16, int U>
__global__ void split_taps_kernel(const float* __restrict__ taps, int64_t k, int reverse, int m,
                                  int64_t LG, int terms, const unsigned* __restrict__ mx,
                                  op16* __restrict__ G) {
    const int64_t total = (int64_t)kPh * LG;
    const Scale2 scale = scale2(F16 ? f16_shift(*mx) : 0);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int ph = (int)(e / LG);
        const int64_t i = e % LG;
        const int64_t ci = i - 8 * (int64_t)(U - 1) - ph - m;
        const float v = (ci >= 0 && ci < k) ? __ldg(taps + (reverse ? k - 1 - ci : ci)) : 0.0f;
        op16 t[3];
        split_tap<F16>(v, terms, scale, t);
        G[e] = t[0];
        G[total + e] = t[1];
        if (terms == 3) G[2 * total + e] = t[2];
    }
}

// Products as (signal term, tap term); product 0 goes to the x1*c1
// accumulator, the others to the cross-term accumulator.
__host__ __device__ constexpr int prod_a(int p) {
    return p == 0 ? 0 : p == 1 ? 0 : p == 2 ? 1 : p == 3 ? 0 : p == 4 ? 1 : 2;
}
__host__ __device__ constexpr int prod_b(int p) {
    return p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 0 : p == 3 ? 2 : p == 4 ? 1 : 0;
}

// Live 16-row groups [lo, hi) (multiples of 16) of phase operand phi for
// the K step starting at J0: rows u' whose 16 taps G_phi[8u' + J0 ..] meet
// the non-zero range [L0, L0 + k) of G_phi.  32-bit arithmetic: the launch
// checks keep L0 + k and every J0 below 2^31.
template <int U>
__device__ __forceinline__ void live_rows(int J0, int L0, int k, int& lo, int& hi) {
    const int a = L0 - J0 - 15;  // 8u' >= a
    const int b = L0 + k - J0;   // 8u' < b
    const int l = a <= 0 ? 0 : (a + 7) >> 3;
    const int h = b <= 0 ? 0 : min((b + 7) >> 3, U);
    lo = l & ~15;
    hi = min((h + 15) & ~15, U);
}

// What one role needs to know about a tile: the signal box (tensor map and
// coordinates), the filter (tap planes, taps, shift, K chunks), the phase
// group, and where its outputs go.  Batched launches derive it from the
// geometry; ragged launches read it from the plan's tile and signal tables.
struct TileView {
    const CUtensorMap* map;
    const op16* G;
    int64_t LG, k;
    int m, nchunks, pg, vec_store;
    int32_t xc0, row0;   // TMA x coordinate of the first chunk, first row of the box
    int64_t rows;        // rows of the box that exist
    float* y;            // output row row0 (rows ld apart)
    int64_t ld, o0;      // row stride; output index of column 0 of phase 0 inside a row
    int64_t lim0, dlim;  // outputs past (lim0 - r * dlim) of box row r are not stored
    const unsigned* mxr;  // FP16X3: max |x| bits of box row r at mxr[r * mxs]
    int64_t mxs;
    int shc;              // FP16X3: the taps' scale exponent
};

template <bool RAGGED, bool F16, int U>
__device__ __forceinline__ TileView tile_view(int64_t tile, const CUtensorMap* amap,
                                              const op16* G, const TcGeom& g, float* y,
                                              int64_t ld_y, const CUtensorMap* maps,
                                              const TcSig* sigs, const TcTile* tiles,
                                              const unsigned* mx) {
    TileView v;
    v.mxr = nullptr;
    v.mxs = 0;
    v.shc = 0;
    if (RAGGED) {
        const TcTile tt = tiles[tile];
        const TcSig sg = sigs[tt.sig];
        v.map = maps + tt.sig;
        v.G = G + sg.g_off;
        v.LG = sg.LG;
        v.k = sg.k;
        v.m = sg.m;
        v.nchunks = sg.nchunks;
        v.pg = tt.pg;
        v.vec_store = sg.vec_store & g.vec_store;  // the signal's offset and the buffer
        v.xc0 = sg.x0 + tt.blk * TcShape<U>::kNCOL;
        v.row0 = tt.row0;
        v.rows = sg.rows - tt.row0;
        v.ld = sg.seg;
        v.y = y + sg.y_off + (int64_t)tt.row0 * sg.seg;
        v.o0 = (int64_t)tt.blk * TcShape<U>::kNCOL + TcShape<U>::kPhT * tt.pg;
        v.lim0 = sg.n_out - (int64_t)tt.row0 * sg.seg;
        v.dlim = sg.seg;
        if (F16) {  // one signal: every row has its scale
            v.mxr = mx + 2 * (int64_t)tt.sig;
            v.shc = f16_shift(mx[2 * (int64_t)tt.sig + 1]);
        }
    } else {
        const int pg = (int)(tile % TcShape<U>::kGroups);
        const int64_t w = tile / TcShape<U>::kGroups;
        const int64_t cg = w / g.blocks_per_cg, blk = w % g.blocks_per_cg;
        v.map = amap;
        v.G = G;
        v.LG = g.LG;
        v.k = g.k;
        v.m = g.m;
        v.nchunks = g.nchunks;
        v.pg = pg;
        v.vec_store = g.vec_store;
        v.xc0 = (int32_t)(g.xa0 + blk * TcShape<U>::kNCOL);
        v.row0 = (int32_t)(cg * kM);
        v.rows = g.batch - cg * kM;
        v.ld = ld_y;
        v.y = y + cg * kM * ld_y;
        v.o0 = blk * TcShape<U>::kNCOL + TcShape<U>::kPhT * pg;
        v.lim0 = g.n_out;
        v.dlim = 0;
        if (F16) {
            v.mxr = mx + v.row0;
            v.mxs = 1;
            v.shc = f16_shift(mx[g.batch]);
        }
    }
    return v;
}

// T terms per operand: 2 (BF16X3, FP16X3) or 3 (BF16X6); F16: fp16 terms
// of scaled operands (FP16X3), else bf16; U rows per phase operand (128 or
// 256, the MMA's largest N).
template <int T, bool RAGGED, bool F16, int U>
__global__ void __launch_bounds__(kThreads, 1)
fir_tc_kernel(const __grid_constant__ CUtensorMap amap, const op16* __restrict__ G,
              const TcGeom g, float* __restrict__ y, int64_t ld_y, unsigned* __restrict__ err,
              const CUtensorMap* __restrict__ maps, const TcSig* __restrict__ sigs,
              const TcTile* __restrict__ tiles, const unsigned* __restrict__ mx) {
    constexpr int NPROD = T == 2 ? 3 : 6;
    constexpr uint32_t kABytes = T * kABytesTerm;
    constexpr int kU = U, kPhT = TcShape<U>::kPhT;
    constexpr uint32_t kBBytesPh = TcShape<U>::kBBytesPh;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)g.nstage * g.stage_bytes);
    uint64_t* empty = full + g.nstage;
    uint64_t* tfull = empty + g.nstage;
    uint64_t* tempty = tfull + 1;
    uint64_t* mma_done = tempty + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        if (lane == 0) {
            for (int s = 0; s < g.nstage; ++s) {
                mbar_init(&full[s], 1);
                mbar_init(&empty[s], 1);
            }
            mbar_init(tfull, 1);
            mbar_init(tempty, kEpiWarps * 32);
            mbar_init(mma_done, 1);
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
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            if (!RAGGED) prefetch_tmap(&amap);
            uint32_t it = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < g.n_tiles; tile += gridDim.x) {
                const TileView v = tile_view<RAGGED, F16, U>(tile, &amap, G, g, y, ld_y, maps, sigs, tiles, mx);
                for (int c = 0; c < v.nchunks; ++c, ++it) {
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
                    for (int t = 0; t < T; ++t)
                        tma_load_3d(sb + t * kABytesTerm, v.map, &full[st], v.xc0 + c * kKC,
                                    v.row0, t);
                    uint8_t* bb = sb + kABytes;
#pragma unroll
                    for (int t = 0; t < T; ++t)
#pragma unroll
                        for (int l = 0; l < kPhT; ++l)
                            bulk_load(bb + (t * kPhT + l) * kBBytesPh,
                                      v.G + ((int64_t)(t * kPh + kPhT * v.pg + l) * v.LG +
                                             (int64_t)c * kKC),
                                      kBBytesPh, &full[st]);
                }
            }
            // the copies issued last have landed before this thread leaves
            const uint32_t first = it > (uint32_t)g.nstage ? it - (uint32_t)g.nstage : 0u;
            for (uint32_t j = first; j < it; ++j)
                if (!mbar_wait(&full[j % (uint32_t)g.nstage], (j / (uint32_t)g.nstage) & 1u))
                    atomicOr(err, kErrMbarTimeout);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issue
        if (lane == 0) {
            // A and B formats: bf16 (1) or, for FP16X3, f16 (0)
            constexpr uint32_t idesc0 =
                idesc_bf16_f32(kM, 16) & ~(0x3Fu << 17) & (F16 ? ~((1u << 7) | (1u << 10)) : ~0u);
            uint32_t it = 0, tcount = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < g.n_tiles; tile += gridDim.x, ++tcount) {
                const TileView v = tile_view<RAGGED, F16, U>(tile, &amap, G, g, y, ld_y, maps, sigs, tiles, mx);
                // the epilogue has read (and zeroed) the accumulators of the tile before
                if (!mbar_wait(tempty, tcount & 1u)) {
                    atomicOr(err, kErrMbarTimeout);
                    break;
                }
                tc_fence_after();
                // phase 0's first non-zero tap position (phase 1's is one more)
                const int L0 = 8 * (kU - 1) + kPhT * v.pg + v.m, k32 = (int)v.k;
                for (int c = 0; c < v.nchunks; ++c, ++it) {
                    const int st = (int)(it % (uint32_t)g.nstage);
                    const uint32_t ph = (it / (uint32_t)g.nstage) & 1u;
                    if (!mbar_wait(&full[st], ph)) {
                        atomicOr(err, kErrMbarTimeout);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(base + (size_t)st * g.stage_bytes);
                    const uint64_t ad0 = smem_desc(sa, 16, 1024, 2);
                    const uint64_t bd0 = smem_desc(sa + kABytes, 16, 128, 0);
                    // the chunk's live rows: the union over its K steps and both
                    // phases -- the fewest dead rows at its last step in phase 0,
                    // the most live ones at its first step in phase 1 (rows
                    // outside a step's own range meet zero taps) -- so all its
                    // MMAs share one N and constant operand offsets
                    int lo, hi, unused_lo, unused_hi;
                    live_rows<U>(c * kKC + kKC - 16, L0, k32, lo, unused_hi);
                    live_rows<U>(c * kKC, L0 + kPhT - 1, k32, unused_lo, hi);
                    if (hi > lo) {
                        const uint32_t idesc = idesc0 | ((uint32_t)((hi - lo) >> 3) << 17);
                        const uint64_t bdl = bd0 + (uint64_t)lo;  // row lo starts 16 * lo bytes in
                        const uint32_t dl = tmem + (uint32_t)lo;
#pragma unroll
                        for (int ks = 0; ks < kKC / 16; ++ks)
#pragma unroll
                            for (int l = 0; l < kPhT; ++l)
#pragma unroll
                                for (int p = 0; p < NPROD; ++p)
                                    tc_mma_f16(dl + (p == 0 ? 0 : kCrossCol) + l * kU,
                                               ad0 + (uint64_t)((prod_a(p) * kABytesTerm + ks * 32) >> 4),
                                               bdl + (uint64_t)(((prod_b(p) * kPhT + l) * kBBytesPh +
                                                                 ks * 32) >> 4),
                                               idesc, 1u);
                    }
                    tc_commit(&empty[st]);
                }
                if (!ok) break;
                tc_commit(tfull);
            }
            // every MMA issued has completed before TMEM can be freed
            tc_commit(mma_done);
            if (!mbar_wait(mma_done, 0)) atomicOr(err, kErrMbarTimeout);
        }
    } else {
        // ------------------------------------------------ epilogue
        constexpr int kCols = kU / (kEpiWarps / 4);   // columns of a phase per warp
        constexpr int kGrp = kCols / 16;
        const int q = warp & 3;                        // TMEM lane quarter
        const int part = (warp - 2) >> 2;              // which kCols of a phase's U columns
        const int c0 = part * kCols;
        const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16);
        // the accumulators start at zero (every MMA accumulates)
#pragma unroll
        for (int gi = 0; gi < kGrp; ++gi)
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int l = 0; l < kPhT; ++l)
                    tmem_zero16(tq + a * kCrossCol + l * kU + c0 + 16 * gi);
        tmem_wait_st();
        tc_fence_before();
        mbar_arrive(tempty);
        uint32_t tcount = 0;
        for (int64_t tile = blockIdx.x; tile < g.n_tiles; tile += gridDim.x, ++tcount) {
            const TileView v = tile_view<RAGGED, F16, U>(tile, &amap, G, g, y, ld_y, maps, sigs, tiles, mx);
            if (!mbar_wait(tfull, tcount & 1u)) {
                if (lane == 0) atomicOr(err, kErrMbarTimeout);
                break;
            }
            tc_fence_after();
            const int r = q * 32 + lane;  // row of the box
            const int64_t o0 = v.o0;
            const int64_t lim = v.lim0 - (int64_t)r * v.dlim;  // outputs of this row below lim
            float* __restrict__ yr = v.y + (int64_t)r * v.ld;
            // every column of this warp into registers (the two accumulators
            // summed), TMEM zeroed and handed back, then the global stores:
            // the next tile's MMAs run while this tile's outputs are written
            float out[kGrp][kPhT][16];
#pragma unroll
            for (int gi = 0; gi < kGrp; ++gi) {
                const int u0 = c0 + 16 * gi;
#pragma unroll
                for (int l = 0; l < kPhT; ++l) {
                    float vc[16];
                    tmem_ld16(tq + l * kU + u0, out[gi][l]);
                    tmem_ld16(tq + kCrossCol + l * kU + u0, vc);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) out[gi][l][i] += vc[i];
                }
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int l = 0; l < kPhT; ++l) tmem_zero16(tq + a * kCrossCol + l * kU + u0);
            }
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(tempty);
            if (F16 && r < v.rows) {
                // undo the scales 2^(e+f) of the row and the taps: e + f in
                // [-226, 280], three power-of-two factors of one sign (so an
                // intermediate over- or underflows only when the result does)
                const int sh = f16_shift(v.mxr[r * v.mxs]) + v.shc;
                const int q = sh / 3;
                const float f1 = pow2f(-q), f2 = pow2f(-(sh - 2 * q));
#pragma unroll
                for (int gi = 0; gi < kGrp; ++gi)
#pragma unroll
                    for (int l = 0; l < kPhT; ++l)
#pragma unroll
                        for (int i = 0; i < 16; ++i) out[gi][l][i] = out[gi][l][i] * f1 * f1 * f2;
            }
            if (r < v.rows) {
#pragma unroll
                for (int gi = 0; gi < kGrp; ++gi) {
                    // column u0 + i holds output ob - 8i (and the next one)
                    const int64_t ob = o0 + 8 * (kU - 1 - (c0 + 16 * gi));
                    if (kPhT == 2 && v.vec_store && ob + kPhT <= lim) {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            *reinterpret_cast<float2*>(yr + ob - 8 * i) =
                                make_float2(out[gi][0][i], out[gi][kPhT - 1][i]);
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
#pragma unroll
                            for (int l = 0; l < kPhT; ++l) {
                                const int64_t o = ob - 8 * i + l;
                                if (o < lim) yr[o] = out[gi][l][i];
                            }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

template <int T, bool F16, int U>
int launch_tc(const FirArgs& a, cudaStream_t st) {
    using Sh = TcShape<U>;
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    TcGeom g;
    g.m = (int)(((a.s % 8) + 8) % 8);
    g.xa0 = a.s - g.m;
    g.k = a.k;
    g.n_out = a.n_out;
    g.batch = a.batch;
    const int64_t nA = (a.n + 7) / 8 * 8;
    const int64_t ktot = a.k + Sh::kNCOL - 1 + g.m;
    g.nchunks = (int)ceil_div(ktot, kKC);
    g.LG = (int64_t)g.nchunks * kKC + 8 * Sh::kU;
    g.blocks_per_cg = ceil_div(a.n_out, Sh::kNCOL);
    g.n_tiles = g.blocks_per_cg * ceil_div(a.batch, kM) * Sh::kGroups;
    g.vec_store = ((reinterpret_cast<uintptr_t>(a.y) & 7) == 0 && (a.ld_y % 2) == 0) ? 1 : 0;
    // TMA coordinates are 32-bit: the last window's K range and the channel
    // groups must stay below 2^31
    if (nA + 2 * Sh::kNCOL + ktot >= (1LL << 31) || ceil_div(a.batch, kM) * kM >= (1LL << 31))
        return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR coordinates exceed 32 bits");
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");

    const uint32_t stage = T * kABytesTerm + T * Sh::kPhT * Sh::kBBytesPh;
    g.stage_bytes = (stage + 1023) / 1024 * 1024;
    g.tx_bytes = stage;
    const size_t extra = 1024 + 8 * (2 * 8 + 3) + 16;
    const int nstage =
        (int)std::min<int64_t>(8, (info->max_smem_optin - (int64_t)extra) / g.stage_bytes);
    if (nstage < 2) return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR stage too large");
    g.nstage = nstage;
    const size_t smem = (size_t)nstage * g.stage_bytes + extra;

    // the signal's term planes and the tap operand planes into scratch memory
    // (FP16X3: and the max |x| of every row and of the taps)
    op16* xs = nullptr;
    op16* Gs = nullptr;
    unsigned* mx = nullptr;
    const size_t xs_bytes = sizeof(op16) * (size_t)T * (size_t)a.batch * (size_t)nA;
    const size_t g_bytes = sizeof(op16) * (size_t)T * kPh * (size_t)g.LG;
    rc = scratch_alloc((void**)&xs, xs_bytes, st);
    if (!rc) rc = scratch_alloc((void**)&Gs, g_bytes, st);
    if (!rc && F16) rc = scratch_alloc((void**)&mx, sizeof(unsigned) * (size_t)(a.batch + 1), st);
    CUtensorMap amap;
    if (!rc)
        rc = make_tmap_3d(&amap, F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                          xs, (uint64_t)nA, (uint64_t)a.batch, (uint64_t)T, (uint64_t)nA * 2,
                          (uint64_t)nA * 2 * (uint64_t)a.batch, kKC, kM, 1,
                          CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc == SCIR_OK) {
        const unsigned gx = (unsigned)std::min<int64_t>(ceil_div(nA / 8, 256 * 4), 1024);
        const unsigned gy = (unsigned)std::min<int64_t>(a.batch, 65535);
        if (F16) {
            cudaError_t me = cudaMemsetAsync(mx, 0, sizeof(unsigned) * (size_t)(a.batch + 1), st);
            if (me != cudaSuccess) rc = set_error(SCIR_ERR_CUDA, "max reset: %s", cudaGetErrorString(me));
            const unsigned mxg = (unsigned)std::min<int64_t>(ceil_div(a.n, 256 * 64), 64);
            absmax_rows_kernel<<<dim3(mxg, (unsigned)std::min<int64_t>(a.batch + 1, 65535)), 256, 0,
                                 st>>>(a.x, a.ld_x, a.batch, a.n, a.taps, a.k, mx);
        }
        split_signal_kernel<F16><<<dim3(gx, gy), 256, 0, st>>>(a.x, a.ld_x, a.batch, a.n, nA, T,
                                                               mx, xs);
        const unsigned gt = (unsigned)std::min<int64_t>(ceil_div((int64_t)kPh * g.LG, 256), 4096);
        split_taps_kernel<F16, U><<<gt, 256, 0, st>>>(a.taps, a.k, a.reverse, g.m, g.LG, T,
                                                      F16 ? mx + a.batch : nullptr, Gs);
        cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess)
            rc = set_error(SCIR_ERR_CUDA, "split kernels: %s", cudaGetErrorString(le));
    }
    if (rc == SCIR_OK) {
        auto kern = fir_tc_kernel<T, false, F16, U>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = set_error(SCIR_ERR_CUDA, "cudaFuncSetAttribute(fir_tc_kernel): %s",
                           cudaGetErrorString(e));
        } else {
            const int64_t grid = std::min<int64_t>(g.n_tiles, (int64_t)info->sm_count);
            kern<<<(unsigned)grid, kThreads, smem, st>>>(amap, Gs, g, a.y, a.ld_y, err, nullptr,
                                                         nullptr, nullptr, mx);
            cudaError_t le = cudaGetLastError();
            if (le != cudaSuccess)
                rc = set_error(SCIR_ERR_CUDA, "launch of fir_tc_kernel failed: %s",
                               cudaGetErrorString(le));
        }
    }
    scratch_free(xs, st);
    scratch_free(Gs, st);
    scratch_free(mx, st);
    return rc;
}

// Per-signal split parameters of a ragged plan's tensor-core bucket.
struct TcSplit {
    int64_t x_off, n, plane_off, region, pad_front;  // plane elements [plane_off, +region)
    int64_t taps_off, k, LG, g_off;
    int32_t reverse, m;
};

// FP16X3: mx[2i] = max |x_i| bits, mx[2i + 1] = max |taps_i| bits (blockIdx.z
// picks which; mx zeroed).
__global__ void absmax_ragged_kernel(const TcSplit* __restrict__ sp, const float* __restrict__ x,
                                     const float* __restrict__ taps, unsigned* __restrict__ mx) {
    const TcSplit d = sp[blockIdx.y];
    if (blockIdx.z == 0)
        absmax_segment(x + d.x_off, d.n, mx + 2 * (int64_t)blockIdx.y);
    else
        absmax_segment(taps + d.taps_off, d.k, mx + 2 * (int64_t)blockIdx.y + 1);
}

// Signal i's planes: element pad_front + j holds term t of x_i[j] (FP16X3:
// of x_i[j] 2^e_i), zero elsewhere in its region (the history before the
// signal and the tail).
template <bool F16>
__global__ void split_planes_ragged_kernel(const TcSplit* __restrict__ sp, const float* __restrict__ x,
                                           int64_t plane_len, int terms,
                                           const unsigned* __restrict__ mx,
                                           op16* __restrict__ planes) {
    const TcSplit d = sp[blockIdx.y];
    const float* __restrict__ xs = x + d.x_off;
    const Scale2 scale = scale2(F16 ? f16_shift(mx[2 * (int64_t)blockIdx.y]) : 0);
    // 8 elements per thread (regions and plane offsets are multiples of 8):
    // one 16-byte store per plane
    for (int64_t e0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 8; e0 < d.region;
         e0 += (int64_t)gridDim.x * blockDim.x * 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t src = e0 + j - d.pad_front;
            v[j] = (src >= 0 && src < d.n) ? __ldg(xs + src) : 0.0f;
        }
        uint2 lo[3], hi[3];
        if (F16) {
            split4_f16(make_float4(v[0], v[1], v[2], v[3]), scale, lo);
            split4_f16(make_float4(v[4], v[5], v[6], v[7]), scale, hi);
        } else {
            split4_any(make_float4(v[0], v[1], v[2], v[3]), terms, lo);
            split4_any(make_float4(v[4], v[5], v[6], v[7]), terms, hi);
        }
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (t < terms)
                *reinterpret_cast<uint4*>(planes + t * plane_len + d.plane_off + e0) =
                    make_uint4(lo[t].x, lo[t].y, hi[t].x, hi[t].y);
    }
}

// Signal i's tap planes G_i[t][phi][e] = term t of c[e - 8*(U-1) - phi - m]
// (FP16X3: of c 2^f_i).
template <bool F16>
__global__ void split_taps_ragged_kernel(const TcSplit* __restrict__ sp, const float* __restrict__ taps,
                                         int terms, const unsigned* __restrict__ mx,
                                         op16* __restrict__ G) {
    const TcSplit d = sp[blockIdx.y];
    const int64_t total = (int64_t)kPh * d.LG;
    op16* Gi = G + d.g_off;
    const Scale2 scale = scale2(F16 ? f16_shift(mx[2 * (int64_t)blockIdx.y + 1]) : 0);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int ph = (int)(e / d.LG);
        const int64_t i = e % d.LG;
        const int64_t ci = i - 8 * (int64_t)(RaggedShape::kU - 1) - ph - d.m;
        const float v = (ci >= 0 && ci < d.k)
                            ? __ldg(taps + d.taps_off + (d.reverse ? d.k - 1 - ci : ci))
                            : 0.0f;
        op16 t[3];
        split_tap<F16>(v, terms, scale, t);
        Gi[e] = t[0];
        Gi[total + e] = t[1];
        if (terms == 3) Gi[2 * total + e] = t[2];
    }
}

// Stage sizes of the tensor-core kernel for `terms` bf16 terms.
int tc_stages(int terms, const DeviceInfo* info, TcGeom* g, size_t* smem) {
    const uint32_t stage = terms * kABytesTerm + terms * RaggedShape::kPhT * RaggedShape::kBBytesPh;
    g->stage_bytes = (stage + 1023) / 1024 * 1024;
    g->tx_bytes = stage;
    const size_t extra = 1024 + 8 * (2 * 8 + 3) + 16;
    const int nstage =
        (int)std::min<int64_t>(8, (info->max_smem_optin - (int64_t)extra) / g->stage_bytes);
    if (nstage < 2) return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR stage too large");
    g->nstage = nstage;
    *smem = (size_t)nstage * g->stage_bytes + extra;
    return SCIR_OK;
}

}  // namespace

bool fir_tc_supported(const FirArgs& a) {
    return a.k >= 1 && a.n >= 1 && a.batch >= 1 && a.n_out >= 1 && a.n < (1LL << 30);
}

// ------------------------------------------------------------------ ragged bucket

struct TcRaggedPlan {
    int form = kTcBf16x6, terms = 3;
    int64_t nsig = 0, ntiles = 0, plane_len = 0, g_len = 0;
    op16* planes = nullptr;
    op16* G = nullptr;
    unsigned* mx = nullptr;  // FP16X3: max |x_i|, max |taps_i| bits per signal
    CUtensorMap* maps = nullptr;
    TcSig* sigs = nullptr;
    TcTile* tiles = nullptr;
    TcSplit* split = nullptr;
    int64_t max_region = 0, max_g = 0;
};

void tc_ragged_destroy(TcRaggedPlan* p) {
    if (!p) return;
    cudaFree(p->planes);
    cudaFree(p->G);
    cudaFree(p->maps);
    cudaFree(p->sigs);
    cudaFree(p->tiles);
    cudaFree(p->split);
    cudaFree(p->mx);
    delete p;
}

int64_t tc_ragged_tiles(const TcRaggedPlan* p) { return p ? p->ntiles : 0; }

int tc_ragged_create(const TcSigIn* in, int64_t count, int form, TcRaggedPlan** out) {
    *out = nullptr;
    if (count == 0) return SCIR_OK;
    auto p = new TcRaggedPlan();
    const int terms = form == kTcBf16x6 ? 3 : 2;
    p->form = form;
    p->terms = terms;
    p->nsig = count;
    std::vector<TcSig> sig((size_t)count);
    std::vector<TcSplit> sp((size_t)count);
    std::vector<TcTile> tiles;
    std::vector<int> cost;
    int64_t plane_off = 0, g_off = 0;
    for (int64_t i = 0; i < count; ++i) {
        const TcSigIn& d = in[i];
        TcSig& S = sig[(size_t)i];
        TcSplit& P = sp[(size_t)i];
        const int m = (int)(((d.s % 8) + 8) % 8);
        const int64_t xa0 = d.s - m;
        constexpr int kNCOL = RaggedShape::kNCOL;
        const int64_t ktot = d.k + kNCOL - 1 + m;
        const int nchunks = (int)ceil_div(ktot, kKC);
        const int64_t LG = (int64_t)nchunks * kKC + 8 * RaggedShape::kU;
        // windows per segment row: enough that the signal needs <= 128 rows
        const int64_t wpr = std::max<int64_t>(1, ceil_div(d.n_out, (int64_t)kM * kNCOL));
        const int64_t seg = wpr * kNCOL;
        const int64_t rows = ceil_div(d.n_out, seg);
        const int64_t pad_front = (std::max<int64_t>(0, -xa0) + 7) / 8 * 8;
        const int64_t x0 = pad_front + xa0;
        const int64_t X = x0 + (wpr - 1) * kNCOL + (int64_t)nchunks * kKC;  // row extent
        const int64_t region =
            std::max((rows - 1) * seg + X, pad_front + d.n) / 8 * 8 + 8;
        if (X >= (1LL << 31) || seg * 2 >= (1LL << 40)) {
            tc_ragged_destroy(p);
            return set_error(SCIR_ERR_UNSUPPORTED, "ragged tensor-core signal %lld too long",
                             (long long)i);
        }
        S.g_off = g_off;
        S.LG = LG;
        S.k = d.k;
        S.seg = seg;
        S.n_out = d.n_out;
        S.y_off = d.y_off;
        S.m = m;
        S.nchunks = nchunks;
        S.x0 = (int32_t)x0;
        S.rows = (int32_t)rows;
        S.vec_store = (d.y_off % 2 == 0) ? 1 : 0;
        S.pad_ = 0;
        P.x_off = d.x_off;
        P.n = d.n;
        P.plane_off = plane_off;
        P.region = region;
        P.pad_front = pad_front;
        P.taps_off = d.taps_off;
        P.k = d.k;
        P.LG = LG;
        P.g_off = g_off;
        P.reverse = d.reverse;
        P.m = m;
        plane_off += region;
        g_off += (int64_t)terms * kPh * LG;
        p->max_region = std::max(p->max_region, region);
        p->max_g = std::max(p->max_g, (int64_t)kPh * LG);
        for (int64_t blk = 0; blk < wpr; ++blk)
            for (int pg = 0; pg < RaggedShape::kGroups; ++pg) {
                tiles.push_back(TcTile{(int32_t)i, 0, (int32_t)blk, pg});
                cost.push_back(nchunks);
            }
    }
    p->plane_len = (plane_off + 7) / 8 * 8;
    p->g_len = g_off;
    // costliest tiles first: the CTAs take tiles round-robin
    std::vector<size_t> order(tiles.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<TcTile> sorted(tiles.size());
    for (size_t i = 0; i < order.size(); ++i) sorted[i] = tiles[order[i]];
    p->ntiles = (int64_t)sorted.size();
    auto fail = [&](int code) {
        tc_ragged_destroy(p);
        return code;
    };
    cudaError_t e = cudaMalloc(&p->planes, sizeof(op16) * (size_t)terms * (size_t)p->plane_len);
    if (e == cudaSuccess) e = cudaMalloc(&p->G, sizeof(op16) * (size_t)p->g_len);
    if (e == cudaSuccess && form == kTcFp16x3)
        e = cudaMalloc(&p->mx, sizeof(unsigned) * 2 * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&p->maps, sizeof(CUtensorMap) * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&p->sigs, sizeof(TcSig) * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&p->tiles, sizeof(TcTile) * sorted.size());
    if (e == cudaSuccess) e = cudaMalloc(&p->split, sizeof(TcSplit) * (size_t)count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(SCIR_ERR_OOM, "ragged tensor-core plan allocation failed: %s", cudaGetErrorString(e));
        return fail(SCIR_ERR_OOM);
    }
    std::vector<CUtensorMap> maps((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        const TcSig& S = sig[(size_t)i];
        const TcSplit& P = sp[(size_t)i];
        constexpr int kNCOL = RaggedShape::kNCOL;
        const int64_t X = (int64_t)S.x0 + (S.seg / kNCOL - 1) * kNCOL + (int64_t)S.nchunks * kKC;
        const int rc = make_tmap_3d(&maps[(size_t)i],
                                    form == kTcFp16x3 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                      : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                                    p->planes + P.plane_off, (uint64_t)X, (uint64_t)S.rows,
                                    (uint64_t)terms, (uint64_t)S.seg * 2,
                                    (uint64_t)p->plane_len * 2, kKC, kM, 1,
                                    CU_TENSOR_MAP_SWIZZLE_128B);
        if (rc) return fail(rc);
    }
    int rc = upload_sync(p->maps, maps.data(), sizeof(CUtensorMap) * maps.size());
    if (!rc) rc = upload_sync(p->sigs, sig.data(), sizeof(TcSig) * sig.size());
    if (!rc) rc = upload_sync(p->tiles, sorted.data(), sizeof(TcTile) * sorted.size());
    if (!rc) rc = upload_sync(p->split, sp.data(), sizeof(TcSplit) * sp.size());
    if (rc) return fail(rc);
    *out = p;
    return SCIR_OK;
}

template <int T, bool F16>
int tc_ragged_launch(const TcRaggedPlan* p, float* y, const DeviceInfo* info, unsigned* err,
                     cudaStream_t st) {
    TcGeom g{};
    size_t smem = 0;
    int rc = tc_stages(T, info, &g, &smem);
    if (rc) return rc;
    g.n_tiles = p->ntiles;
    g.vec_store = (reinterpret_cast<uintptr_t>(y) & 7) == 0 ? 1 : 0;
    auto kern = fir_tc_kernel<T, true, F16, RaggedShape::kU>;
    SCIR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUtensorMap unused;
    memset(&unused, 0, sizeof(unused));
    const int64_t grid = std::min<int64_t>(p->ntiles, (int64_t)info->sm_count);
    kern<<<(unsigned)grid, kThreads, smem, st>>>(unused, p->G, g, y, 0, err, p->maps, p->sigs,
                                                 p->tiles, p->mx);
    SCIR_LAUNCH_CHECK("fir_tc_kernel (ragged)");
    return SCIR_OK;
}

int tc_ragged_run(const TcRaggedPlan* p, const float* x, const float* taps, float* y,
                  cudaStream_t st) {
    if (!p || p->ntiles == 0) return SCIR_OK;
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    unsigned* err = device_error_word();
    if (!err) return set_error(SCIR_ERR_CUDA, "device error word unavailable");
    SCIR_REQUIRE(p->nsig <= 65535, SCIR_ERR_UNSUPPORTED, "more than 65,535 tensor-core signals");
    const bool f16 = p->form == kTcFp16x3;
    if (f16) {
        SCIR_CUDA_TRY(cudaMemsetAsync(p->mx, 0, sizeof(unsigned) * 2 * (size_t)p->nsig, st));
        const unsigned bm = (unsigned)std::min<int64_t>(ceil_div(p->max_region, 256 * 64), 64);
        absmax_ragged_kernel<<<dim3(bm, (unsigned)p->nsig, 2), 256, 0, st>>>(p->split, x, taps, p->mx);
    }
    const unsigned bx = (unsigned)std::min<int64_t>(ceil_div(p->max_region / 8, 256 * 4), 128);
    const unsigned bt = (unsigned)std::min<int64_t>(ceil_div(p->max_g, 256), 64);
    if (f16) {
        split_planes_ragged_kernel<true><<<dim3(bx, (unsigned)p->nsig), 256, 0, st>>>(
            p->split, x, p->plane_len, p->terms, p->mx, p->planes);
        split_taps_ragged_kernel<true><<<dim3(bt, (unsigned)p->nsig), 256, 0, st>>>(
            p->split, taps, p->terms, p->mx, p->G);
    } else {
        split_planes_ragged_kernel<false><<<dim3(bx, (unsigned)p->nsig), 256, 0, st>>>(
            p->split, x, p->plane_len, p->terms, nullptr, p->planes);
        split_taps_ragged_kernel<false><<<dim3(bt, (unsigned)p->nsig), 256, 0, st>>>(
            p->split, taps, p->terms, nullptr, p->G);
    }
    SCIR_LAUNCH_CHECK("ragged split kernels");
    if (f16) return tc_ragged_launch<2, true>(p, y, info, err, st);
    return p->terms == 2 ? tc_ragged_launch<2, false>(p, y, info, err, st)
                         : tc_ragged_launch<3, false>(p, y, info, err, st);
}

// Filters of at least kWideTaps taps use U = 256 (one phase per tile):
// N = 256 MMAs read fewer operand bytes per product than N = 128 ones, which
// pays for their twice as long ramps only when the filter is long.  Measured
// on 1,024 x 262,144 (FP16X3 step, U = 128 / 256): 4,095 taps 4.99 / 4.79 ms,
// 2,048 taps 3.31 / 3.94 ms, 1,024 taps 2.44 / 3.66 ms.
constexpr int64_t kWideTaps = 3584;

int launch_fir_tc(const FirArgs& a, int form, cudaStream_t st) {
    if (a.batch == 0 || a.n_out == 0) return SCIR_OK;
    const bool wide = a.k >= kWideTaps;
    switch (form) {
    case kTcBf16x3: return wide ? launch_tc<2, false, 256>(a, st) : launch_tc<2, false, 128>(a, st);
    case kTcBf16x6: return wide ? launch_tc<3, false, 256>(a, st) : launch_tc<3, false, 128>(a, st);
    case kTcFp16x3: return wide ? launch_tc<2, true, 256>(a, st) : launch_tc<2, true, 128>(a, st);
    default: return set_error(SCIR_ERR_INVALID_ARG, "unknown tensor-core form %d", form);
    }
}

}  // namespace scir
