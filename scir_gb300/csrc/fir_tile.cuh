// One FIR output tile on the CUDA cores, shared by the batched kernel
// (fir_simt.cu) and the ragged persistent kernel (ragged.cu).
//
// A tile is TILE = 256*V consecutive outputs of one row.  Taps are processed
// in chunks; for each chunk the CTA stages the taps and the input window
// (TILE + chunk samples, zero outside [0, n)) in shared memory with coalesced
// loads.  Thread t computes outputs t*V .. t*V+V-1 of the tile from a sliding
// register window: every block of V taps costs V shared loads of x, V/4
// broadcast loads of taps and V*V FMAs.  The window array is padded by one
// word per 32 so the stride-V lane pattern is bank-conflict free.  The window
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
    return sizeof(float) * (size_t)(chunk + (tile + chunk) + (tile + chunk + 8) / 32 + 8);
}

__device__ __forceinline__ int fir_padi(int j) { return j + (j >> 5); }

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

template <int V>
__device__ __forceinline__ void load_win(float (&w)[V], const float* __restrict__ s_x, int pos) {
#pragma unroll
    for (int v = 0; v < V; ++v) w[v] = s_x[fir_padi(pos + v)];
}

// Computes outputs [o0, o0 + TILE) of one row (TILE = kFirThreads * V) into
// yr; smem must hold chunk + (TILE + chunk) * 33/32 + 4 floats.
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
    int r = 0;  // window misalignment of the current pass
    const int nchunks = (int)((k + chunk - 1) / chunk);
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
        r = (int)(ws - w0);
        const int W4 = (TILE + kcp + r + 3) / 4;  // float4 groups staged
        if ((reinterpret_cast<uintptr_t>(xr) & 15) == 0 && w0 >= 0 && w0 + 4 * (int64_t)W4 <= n) {
            const float4* __restrict__ x4 = reinterpret_cast<const float4*>(xr + w0);
            for (int j4 = tid; j4 < W4; j4 += kFirThreads) {
                const float4 q = __ldg(x4 + j4);
                const int i = 4 * j4;
                s_x[fir_padi(i)] = q.x;
                s_x[fir_padi(i + 1)] = q.y;
                s_x[fir_padi(i + 2)] = q.z;
                s_x[fir_padi(i + 3)] = q.w;
            }
        } else {
            for (int i = tid; i < 4 * W4; i += kFirThreads) {
                const int64_t p = w0 + i;
                s_x[fir_padi(i)] = (p >= 0 && p < n) ? __ldg(xr + p) : 0.0f;
            }
        }
        __syncthreads();

        const int base = base0 + r;
        float wa[V], wb[V];
        if (!EXACT) {
            // ascending blocks; block jb reads window positions base+jb .. base+jb+2V-2
            load_win<V>(wa, s_x, base);
            int jb = 0;
            for (; jb + 2 * V <= kcp; jb += 2 * V) {
                load_win<V>(wb, s_x, base + jb + V);
                fma_block<V, false>(acc, s_c, jb, wa, wb);
                load_win<V>(wa, s_x, base + jb + 2 * V);
                fma_block<V, false>(acc, s_c, jb + V, wb, wa);
            }
            if (jb < kcp) {
                load_win<V>(wb, s_x, base + jb + V);
                fma_block<V, false>(acc, s_c, jb, wa, wb);
            }
        } else {
            // descending blocks and taps: newest sample first, as the reference
            int jb = kcp - V;
            load_win<V>(wb, s_x, base + jb + V);
            for (; jb - V >= 0; jb -= 2 * V) {
                load_win<V>(wa, s_x, base + jb);
                fma_block<V, true>(acc, s_c, jb, wa, wb);
                load_win<V>(wb, s_x, base + jb - V);
                fma_block<V, true>(acc, s_c, jb - V, wb, wa);
            }
            if (jb >= 0) {
                load_win<V>(wa, s_x, base + jb);
                fma_block<V, true>(acc, s_c, jb, wa, wb);
            }
        }
    }

    __syncthreads();
#pragma unroll
    for (int v = 0; v < V; ++v) s_x[fir_padi(base0 + v)] = acc[v];
    __syncthreads();
    if ((reinterpret_cast<uintptr_t>(yr + o0) & 15) == 0 && o0 + TILE <= n_out) {
        float4* __restrict__ y4 = reinterpret_cast<float4*>(yr + o0);
        for (int j4 = tid; j4 < TILE / 4; j4 += kFirThreads) {
            const int i = 4 * j4;
            y4[j4] = make_float4(s_x[fir_padi(i)], s_x[fir_padi(i + 1)], s_x[fir_padi(i + 2)],
                                 s_x[fir_padi(i + 3)]);
        }
    } else {
        for (int j = tid; j < TILE; j += kFirThreads) {
            const int64_t o = o0 + j;
            if (o < n_out) yr[o] = s_x[fir_padi(j)];
        }
    }
}


}  // namespace scir
