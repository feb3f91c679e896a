// Arithmetic shared by the SOS and IIR kernels: one section update in each
// state precision, the exchange of section states with the DF2T coordinates
// of the API (zi / zf), and the 32 x 32 row tiles of the one-thread-per-
// channel kernels.
//
// The recursion is the reference's Direct Form II transposed cascade
// (crates/scir-iir-filters/src/filter.rs:50-61):
//   out = b0*prev + s1;  s1 = b1*prev - a1*out + s2;  s2 = b2*prev - a2*out
// with a0 taken as 1.  PREC 0 (FP64_EXACT) rounds every product and sum
// separately in the reference's order; PREC 1 uses FP64 FMA; PREC 2 keeps
// FP32 state and FP32 coefficients; PREC 3 (FP32_COUPLED) runs each
// complex-pole section in coupled (modal) form with FP32 state and
// increments sigma - 1, omega computed in FP64 (real-pole sections: FP32
// DF2T).
#pragma once
#include "kernels.cuh"

namespace scir {

template <int PREC>
struct AccT { using type = double; };
template <>
struct AccT<2> { using type = float; };
template <>
struct AccT<3> { using type = float; };

// One section update (s is a compile-time constant after unrolling).
// Coefficients are read from the kernel-parameter bank (sc is a __grid_constant__
// parameter), so they cost no registers; sections past nsec hold b0 = 1.
template <int PREC, typename A>
__device__ __forceinline__ A sos_sec(const SosCoef& sc, int s, A& s1, A& s2, A prev) {
    A out;
    if constexpr (PREC == 0) {
        const double* c = sc.c[s];
        out = __dadd_rn(__dmul_rn(c[0], prev), s1);
        s1 = __dadd_rn(__dsub_rn(__dmul_rn(c[1], prev), __dmul_rn(c[3], out)), s2);
        s2 = __dsub_rn(__dmul_rn(c[2], prev), __dmul_rn(c[4], out));
    } else if constexpr (PREC == 1) {
        const double* c = sc.c[s];
        out = fma(c[0], prev, s1);
        s1 = fma(-c[3], out, fma(c[1], prev, s2));
        s2 = fma(-c[4], out, c[2] * prev);
    } else if constexpr (PREC == 2) {
        const float* c = sc.cf[s];
        out = fmaf(c[0], prev, s1);
        s1 = fmaf(-c[3], out, fmaf(c[1], prev, s2));
        s2 = fmaf(-c[4], out, c[2] * prev);
    } else {
        if (sc.coupled[s]) {
            const float* k = sc.cp[s];
            const float u = s1, v = s2;
            out = fmaf(k[2], u, fmaf(k[3], v, k[4] * prev));
            s1 = u + fmaf(k[0], u, fmaf(-k[1], v, prev));
            s2 = v + fmaf(k[1], u, k[0] * v);
        } else {
            const float* c = sc.cf[s];
            out = fmaf(c[0], prev, s1);
            s1 = fmaf(-c[3], out, fmaf(c[1], prev, s2));
            s2 = fmaf(-c[4], out, c[2] * prev);
        }
    }
    return out;
}

// DF2T state (s1, s2) of section s in the kernel's own coordinates.
template <int PREC, typename A>
__device__ __forceinline__ void state_in(const SosCoef& sc, int s, double s1, double s2, A& o1,
                                         A& o2) {
    if (PREC == 3 && sc.coupled[s]) {
        const double* m = sc.to_cp[s];
        o1 = (A)(m[0] * s1 + m[1] * s2);
        o2 = (A)(m[2] * s1 + m[3] * s2);
    } else {
        o1 = (A)s1;
        o2 = (A)s2;
    }
}

template <int PREC, typename A>
__device__ __forceinline__ void state_out(const SosCoef& sc, int s, A i1, A i2, double& s1,
                                          double& s2) {
    if (PREC == 3 && sc.coupled[s]) {
        const double* m = sc.from_cp[s];
        s1 = m[0] * (double)i1 + m[1] * (double)i2;
        s2 = m[2] * (double)i1 + m[3] * (double)i2;
    } else {
        s1 = (double)i1;
        s2 = (double)i2;
    }
}

// Row tiles of 32 channels x 32 samples for one-thread-per-channel
// recursions: a warp loads a tile row by row (coalesced) into registers,
// transposes it through a [32][33] shared tile, and stores it back row by row.
constexpr int kTT = 32;  // samples per tile

// Loads tile [t0, t0+32) of 32 rows starting at row r0 into registers
// (lane = time); rows past `batch` and samples past n read as zero.
template <typename T>
__device__ __forceinline__ void tile_fetch(T (&r)[kTT], const T* __restrict__ x, int64_t ld,
                                           int64_t r0, int64_t batch, int64_t n, int64_t t0,
                                           int lane) {
    const int64_t t = t0 + lane;
#pragma unroll
    for (int i = 0; i < kTT; ++i) {
        const int64_t row = r0 + i;
        r[i] = (row < batch && t < n && t >= 0) ? x[row * ld + t] : T(0);
    }
}

template <typename T>
__device__ __forceinline__ void tile_store(T (*s)[kTT + 1], T* __restrict__ y, int64_t ld,
                                           int64_t r0, int64_t batch, int64_t n, int64_t t0,
                                           int lane) {
    const int64_t t = t0 + lane;
#pragma unroll 4
    for (int i = 0; i < kTT; ++i) {
        const int64_t row = r0 + i;
        if (row < batch && t < n) y[row * ld + t] = s[i][lane];
    }
}

}  // namespace scir
