// One FIR output tile on the CUDA cores, shared by the batched kernel
// (fir_simt.cu) and the ragged persistent kernel (ragged.cu).
//
// A tile is TILE = 256*V consecutive outputs of one row.  Taps are processed
// in chunks; for each chunk the CTA stages the taps and the input window
// (TILE + chunk samples, zero outside [0, n)) in shared memory with coalesced
// loads.  Thread t computes outputs t*V .. t*V+V-1 of the tile from a sliding
// register window: every block of V taps costs V shared loads of x, V/4
// broadcast loads of taps and V*V FMAs.  The window array has one pad word
// after every V samples, so thread t's window starts at word t(V+1) -- an odd
// stride, bank-conflict free -- and, with the window's misalignment R
// (0..3, the same for the whole CTA) a template parameter, every load in the
// FMA loop is one register plus a compile-time offset.  The window
// is staged from the 16-byte boundary at or below its start (16-byte loads
// where the row is 16-byte aligned and the window inside it), and outputs go
// back through shared memory and out with 16-byte stores where the tile is
// whole and the row aligned: at short filters the staging, not the FMAs,
// took most of the issue slots.
//
// EXACT = true reproduces the reference loop (crates/scir-gpu/src/lib.rs:
// 1134-1152) bit for bit: taps are visited from the newest sample to the
// oldest (m = k-1 .. 0 in correlation order) and each step rounds the product
// and then the sum (no FMA).
#pragma once
#include "common.cuh"

namespace scir {

constexpr int kFirThreads = 256;
constexpr int kFirMaxChunk = 4096;  // taps staged per pass (multiple of 16)

inline size_t fir_tile_smem_bytes(int V, int chunk) {
    const int tile = kFirThreads * V;
    // + 8: the window starts up to 3 samples early and is staged in fours
    return sizeof(float) * (size_t)(chunk + (tile + chunk + 8) + (tile + chunk + 8) / V + 8);
}

// Word of window sample i: one pad word after every V samples.
template <int V>
__device__ __forceinline__ int padv(int i) { return i + i / V; }

template <int V, bool EXACT>
__device__ __forceinline__ void fma_block(float (&acc)[V], const float* __restrict__ s_c, int jb,
                                          const float (&lo)[V], const float (&hi)[V]) {
    float c[V];
#pragma unroll
    for (int j = 0; j < V; j += 4) {
        const float4 t = *reinterpret_cast<const float4*>(s_c + jb + j);
        c[j] = t.x; c[j + 1] = t.y; c[j + 2] = t.z; c[j + 3] = t.w;
    }
    if (EXACT) {
#pragma unroll
        for (int j = V - 1; j >= 0; --j) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const float w = (v + j < V) ? lo[v + j] : hi[v + j - V];
                acc[v] = __fadd_rn(acc[v], __fmul_rn(c[j], w));
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < V; ++j) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const float w = (v + j < V) ? lo[v + j] : hi[v + j - V];
                acc[v] = fmaf(c[j], w, acc[v]);
            }
        }
    }
}

// Window samples seg_start + R + v (v < V) of a thread, seg = padv(seg_start)
// with seg_start a multiple of V: the sample R + v of the segment sits R + v
// words in, one more once it passes the segment's pad word.
template <int V, int R>
__device__ __forceinline__ void load_win(float (&w)[V], const float* __restrict__ s_x, int seg) {
#pragma unroll
    for (int v = 0; v < V; ++v) w[v] = s_x[seg + R + v + (R + v >= V ? 1 : 0)];
}

// The FMA passes over one staged chunk of kcp taps (kcp a multiple of V) for
// a thread whose V outputs start at window sample t V + R.
template <int V, bool EXACT, int R>
__device__ __forceinline__ void fir_chunk(float (&acc)[V], const float* __restrict__ s_c,
                                          const float* __restrict__ s_x, int kcp) {
    const int tseg = threadIdx.x * (V + 1);  // padv(t V)
    constexpr int SEG = V + 1;               // words per V samples
    float wa[V], wb[V];
    if (!EXACT) {
        // ascending blocks; block jb reads window samples tV+R+jb .. +2V-2
        load_win<V, R>(wa, s_x, tseg);
        int jb = 0, sg = tseg;
        for (; jb + 2 * V <= kcp; jb += 2 * V, sg += 2 * SEG) {
            load_win<V, R>(wb, s_x, sg + SEG);
            fma_block<V, false>(acc, s_c, jb, wa, wb);
            load_win<V, R>(wa, s_x, sg + 2 * SEG);
            fma_block<V, false>(acc, s_c, jb + V, wb, wa);
        }
        if (jb < kcp) {
            load_win<V, R>(wb, s_x, sg + SEG);
            fma_block<V, false>(acc, s_c, jb, wa, wb);
        }
    } else {
        // descending blocks and taps: newest sample first, as the reference
        int jb = kcp - V, sg = tseg + (kcp / V - 1) * SEG;
        load_win<V, R>(wb, s_x, sg + SEG);
        for (; jb - V >= 0; jb -= 2 * V, sg -= 2 * SEG) {
            load_win<V, R>(wa, s_x, sg);
            fma_block<V, true>(acc, s_c, jb, wa, wb);
            load_win<V, R>(wb, s_x, sg - SEG);
            fma_block<V, true>(acc, s_c, jb - V, wb, wa);
        }
        if (jb >= 0) {
            load_win<V, R>(wa, s_x, sg);
            fma_block<V, true>(acc, s_c, jb, wa, wb);
        }
    }
}

// Computes outputs [o0, o0 + TILE) of one row (TILE = kFirThreads * V) into
// yr; smem must hold fir_tile_smem_bytes(V, chunk).
template <int V, bool EXACT>
__device__ __forceinline__ void fir_tile(float* smem, const float* __restrict__ xr, int64_t n,
                                         const float* __restrict__ taps, int64_t k, int reverse,
                                         int64_t s, float* __restrict__ yr, int64_t n_out,
                                         int64_t o0, int chunk) {
    constexpr int TILE = kFirThreads * V;
    float* s_c = smem;          // `chunk` taps of the current pass
    float* s_x = smem + chunk;  // padded input window
    const int tid = threadIdx.x;
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.0f;

    const int base0 = tid * V;
    // one pass for filters that fit a chunk, without a 64-bit division
    const int nchunks = k <= 0 ? 0 : k <= chunk ? 1 : (int)((k + chunk - 1) / chunk);
    for (int ci = 0; ci < nchunks; ++ci) {
        const int cidx = EXACT ? (nchunks - 1 - ci) : ci;
        const int64_t m0 = (int64_t)cidx * chunk;
        const int kc = (int)((k - m0) < (int64_t)chunk ? (k - m0) : (int64_t)chunk);
        const int kcp = (kc + V - 1) / V * V;
        __syncthreads();  // the previous pass is done reading shared memory
        for (int j = tid; j < kcp; j += kFirThreads) {
            float c = 0.0f;
            if (j < kc) {
                const int64_t m = m0 + j;
                c = __ldg(taps + (reverse ? (k - 1 - m) : m));
            }
            s_c[j] = c;
        }
        // s_x[padi(i)] = x[w0 + i], w0 = the window start rounded down to a
        // multiple of 4 (r = ws - w0 is added to every window position below)
        const int64_t ws = o0 + s + m0;
        const int64_t w0 = ws - (((ws % 4) + 4) % 4);
        const int r = (int)(ws - w0);
        const int W4 = (TILE + kcp + r + 3) / 4;  // float4 groups staged
        if ((reinterpret_cast<uintptr_t>(xr) & 15) == 0 && w0 >= 0 && w0 + 4 * (int64_t)W4 <= n) {
            const float4* __restrict__ x4 = reinterpret_cast<const float4*>(xr + w0);
            for (int j4 = tid; j4 < W4; j4 += kFirThreads) {
                const float4 q = __ldg(x4 + j4);
                const int i = 4 * j4;
                // four samples inside one V-segment (V and i multiples of 4)
                float* d = s_x + padv<V>(i);
                d[0] = q.x;
                d[1] = q.y;
                d[2] = q.z;
                d[3] = q.w;
            }
        } else {
            for (int i = tid; i < 4 * W4; i += kFirThreads) {
                const int64_t p = w0 + i;
                s_x[padv<V>(i)] = (p >= 0 && p < n) ? __ldg(xr + p) : 0.0f;
            }
        }
        __syncthreads();

        switch (r) {
        case 0: fir_chunk<V, EXACT, 0>(acc, s_c, s_x, kcp); break;
        case 1: fir_chunk<V, EXACT, 1>(acc, s_c, s_x, kcp); break;
        case 2: fir_chunk<V, EXACT, 2>(acc, s_c, s_x, kcp); break;
        default: fir_chunk<V, EXACT, 3>(acc, s_c, s_x, kcp); break;
        }
    }

    __syncthreads();
#pragma unroll
    for (int v = 0; v < V; ++v) s_x[padv<V>(base0 + v)] = acc[v];
    __syncthreads();
    if ((reinterpret_cast<uintptr_t>(yr + o0) & 15) == 0 && o0 + TILE <= n_out) {
        float4* __restrict__ y4 = reinterpret_cast<float4*>(yr + o0);
        for (int j4 = tid; j4 < TILE / 4; j4 += kFirThreads) {
            const int i = 4 * j4;
            const float* q = s_x + padv<V>(i);
            y4[j4] = make_float4(q[0], q[1], q[2], q[3]);
        }
    } else {
        for (int j = tid; j < TILE; j += kFirThreads) {
            const int64_t o = o0 + j;
            if (o < n_out) yr[o] = s_x[padv<V>(j)];
        }
    }
}


}  // namespace scir
