// Block-parallel time scan for sosfilt on few, long channels.
//
// The channel-parallel kernels give one channel's whole recursion to one
// lane, so a handful of channels -- one long recording, a few sensors --
// leaves almost all of the GPU idle (a single channel of 100 M samples runs
// on one warp).  The cascade is linear and time-invariant, so each channel is
// cut into blocks of L samples that are filtered at the same time:
//
//   1. every block is filtered from zero state, as if it were a separate
//      channel (the same kernels, blocks as rows with row stride L); each
//      block's final state f_b (the 2 x nsec DF2T states) goes to scratch;
//   2. the true state entering block b follows from the scan
//        S_0 = zi,  S_{b+1} = Phi S_b + f_b,  Phi = A^L,
//      A the one-sample state transition of the cascade with zero input (in
//      the DF2T coordinates the API exchanges states in), Phi formed on the
//      host in FP64 by repeated squaring; one warp runs a scan in FP64 (lane
//      i holds state component i).  With many blocks the scan has two
//      levels, so its sequential depth is ~3 sqrt(nb) steps, not nb: groups
//      of m blocks are scanned from zero state at the same time (their end
//      states F_g), the group entry states follow from G_{g+1} = Phi^m G_g +
//      F_g, and every group is scanned again from G_g;
//   3. every block is filtered again from S_b, which gives the outputs of
//      the sequential recursion; the samples past the last whole block are
//      filtered from S_nb, and the final state goes to zf.
//
// The DF2T cascade coordinates are ill-conditioned for poles near the unit
// circle (|Phi| reaches ~1e18 for an order-8 band-pass 2e-4 from the circle),
// so the scan costs accuracy: in an FP64 model of that filter the block
// result differs from the sequential one by 6e-9 (L = 1,024 .. 4,096) to
// 4e-12 (L = 65,536) normwise.  That is far below the FP32-state modes' own error,
// so those modes (FP32, FP32_COUPLED) take this path when it pays; FP64
// takes it only for L >= 65,536 (stated bound 1e-9), and FP64_EXACT -- the
// reference's sequential operation order -- never does.
#include "common.cuh"
#include "kernels.cuh"

#include <cstring>
#include <vector>

namespace scir {
namespace {

constexpr int kMaxScanStates = 32;  // 2 x 16 sections

// S_{b+1} = Phi S_b + f_b for one channel per CTA (one warp, lane i holds
// state component i; S states): f [ch][nb][S] final states of the
// zero-state blocks, zi [ch][S] or null; writes the states entering every
// block, sin [ch][nb][S], and the state after the last block, fin [ch][S]
// (either output may be null).
// The f values of the next 32 blocks are loaded together, so a step waits
// only for the shuffles and FMAs of the recurrence itself.
template <int S>
__global__ void __launch_bounds__(32)
sos_block_scan_kernel(const double* __restrict__ phi, const double* __restrict__ f,
                      const double* __restrict__ zi, int64_t nb, double* __restrict__ sin,
                      double* __restrict__ fin) {
    const int64_t ch = blockIdx.x;
    const int i = threadIdx.x;
    const bool on = i < S;
    double prow[S];
#pragma unroll
    for (int j = 0; j < S; ++j) prow[j] = on ? phi[i * S + j] : 0.0;
    double s = (on && zi) ? zi[ch * S + i] : 0.0;
    const double* fc = f + ch * nb * S;
    double* sc = sin ? sin + ch * nb * S : nullptr;
    for (int64_t b0 = 0; b0 < nb; b0 += 32) {
        double fb[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) fb[j] = (on && b0 + j < nb) ? fc[(b0 + j) * S + i] : 0.0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (b0 + j >= nb) break;
            if (on && sin) sc[(b0 + j) * S + i] = s;
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int q = 0; q < S; ++q)
                acc[q & 3] = fma(prow[q], __shfl_sync(0xffffffffu, s, q), acc[q & 3]);
            s = (acc[0] + acc[1]) + (acc[2] + acc[3]) + fb[j];
        }
    }
    if (on && fin) fin[ch * S + i] = s;
}

template <int S>
int launch_scan(const double* phi, const double* f, const double* zi, int64_t batch, int64_t nb,
                double* sin, double* fin, cudaStream_t st) {
    sos_block_scan_kernel<S><<<(unsigned)batch, 32, 0, st>>>(phi, f, zi, nb, sin, fin);
    SCIR_LAUNCH_CHECK("sos_block_scan_kernel");
    return SCIR_OK;
}

int scan_dispatch(int S, const double* phi, const double* f, const double* zi, int64_t batch,
                  int64_t nb, double* sin, double* fin, cudaStream_t st) {
    switch (S) {
#define SCIR_SCAN_CASE(N) \
    case N: return launch_scan<N>(phi, f, zi, batch, nb, sin, fin, st);
        SCIR_SCAN_CASE(2) SCIR_SCAN_CASE(4) SCIR_SCAN_CASE(6) SCIR_SCAN_CASE(8) SCIR_SCAN_CASE(10)
        SCIR_SCAN_CASE(12) SCIR_SCAN_CASE(14) SCIR_SCAN_CASE(16) SCIR_SCAN_CASE(18)
        SCIR_SCAN_CASE(20) SCIR_SCAN_CASE(22) SCIR_SCAN_CASE(24) SCIR_SCAN_CASE(26)
        SCIR_SCAN_CASE(28) SCIR_SCAN_CASE(30) SCIR_SCAN_CASE(32)
#undef SCIR_SCAN_CASE
    default: return set_error(SCIR_ERR_UNSUPPORTED, "block scan with %d states", S);
    }
}

// Phi = A^L for the cascade c (DF2T state coordinates, zero input), FP64.
void cascade_phi(const SosCoef& c, int64_t L, std::vector<double>& phi) {
    const int ns = c.nsec, S = 2 * ns;
    std::vector<double> A((size_t)S * S, 0.0), P((size_t)S * S, 0.0), T((size_t)S * S);
    for (int col = 0; col < S; ++col) {
        double st[kMaxScanStates] = {0.0};
        st[col] = 1.0;
        double u = 0.0;
        for (int s = 0; s < ns; ++s) {
            const double* k = c.c[s];  // b0 b1 b2 a1 a2
            const double s1 = st[2 * s], s2 = st[2 * s + 1];
            const double yv = k[0] * u + s1;
            st[2 * s] = k[1] * u - k[3] * yv + s2;
            st[2 * s + 1] = k[2] * u - k[4] * yv;
            u = yv;
        }
        for (int r = 0; r < S; ++r) A[(size_t)r * S + col] = st[r];
    }
    for (int r = 0; r < S; ++r) P[(size_t)r * S + r] = 1.0;
    auto mul = [&](const std::vector<double>& X, const std::vector<double>& Y,
                   std::vector<double>& Z) {
        for (int r = 0; r < S; ++r)
            for (int q = 0; q < S; ++q) {
                double acc = 0.0;
                for (int j = 0; j < S; ++j) acc += X[(size_t)r * S + j] * Y[(size_t)j * S + q];
                Z[(size_t)r * S + q] = acc;
            }
    };
    std::vector<double> B = A;
    for (int64_t e = L; e > 0; e >>= 1) {
        if (e & 1) {
            mul(B, P, T);
            P.swap(T);
        }
        if (e > 1) {
            mul(B, B, T);
            B.swap(T);
        }
    }
    phi.swap(P);
}

}  // namespace

int64_t sos_scan_blocks(int64_t batch, int64_t n, int nsec, int precision, bool in_place) {
    if (in_place || nsec > kMaxScanStates / 2 || batch < 1 || batch > 64) return 0;
    if (precision != SCIR_SOS_FP32 && precision != SCIR_SOS_FP32_COUPLED &&
        precision != SCIR_SOS_FP64)
        return 0;
    // FP32 state: the longest blocks (1,024 .. 65,536 samples) that still
    // give ~19,456 block rows (two 64-row CTAs per SM); FP64 state: 65,536
    // for its stated bound
    int64_t L = 65536;
    if (precision != SCIR_SOS_FP64)
        while (L > 1024 && batch * (n / L) < 19456) L /= 2;
    // blocks per channel: a multiple of 64, so a CTA's rows share a channel
    const int64_t nb = (n / L) / 64 * 64;
    return nb >= 64 ? nb : 0;
}

// Blocks per group of the two-level scan (0: one level): about sqrt(nb),
// a power of two >= 64 that divides nb, from 256 blocks up.
static int64_t scan_group(int64_t nb) {
    if (nb < 256) return 0;
    int64_t m = 64;
    while (nb % (2 * m) == 0 && 4 * m * m <= nb) m *= 2;
    return m;
}

template <typename T>
int sosfilt_blocked(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                    const double* zi, double* zf, int precision, T* y, int64_t ld_y, int64_t nb,
                    cudaStream_t st) {
    const int S = 2 * c.nsec;
    const int64_t L = n / nb, tail = n - nb * L;
    const int64_t m = scan_group(nb), ng = m ? nb / m : 0;
    // Phi = A^L, then (two levels) Phi^m = A^(L m), in one upload
    std::vector<double> phi, phim;
    cascade_phi(c, L, phi);
    if (m) {
        cascade_phi(c, L * m, phim);
        phi.insert(phi.end(), phim.begin(), phim.end());
    }
    double* d_phi = nullptr;
    double* f = nullptr;
    double* sin = nullptr;
    double* fin = nullptr;
    double* grp = nullptr;  // two levels: F_g, then G_g, [ch][ng][S] each
    int rc = scratch_alloc((void**)&d_phi, sizeof(double) * phi.size(), st);
    if (!rc) rc = scratch_alloc((void**)&f, sizeof(double) * (size_t)(batch * nb * S), st);
    if (!rc) rc = scratch_alloc((void**)&sin, sizeof(double) * (size_t)(batch * nb * S), st);
    if (!rc) rc = scratch_alloc((void**)&fin, sizeof(double) * (size_t)(batch * S), st);
    if (!rc && m)
        rc = scratch_alloc((void**)&grp, sizeof(double) * (size_t)(2 * batch * ng * S), st);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(d_phi, phi.data(), sizeof(double) * phi.size(),
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) rc = set_error(SCIR_ERR_CUDA, "Phi upload: %s", cudaGetErrorString(e));
    }
    // 1. every block from zero state (blocks as rows); final states into f
    if (!rc)
        rc = launch_sosfilt<T>(x, ld_x, batch * nb, L, c, nullptr, f, precision, y, ld_y, st, nb, L);
    // 2. the states entering every block
    if (!rc && !m) rc = scan_dispatch(S, d_phi, f, zi, batch, nb, sin, fin, st);
    if (!rc && m) {
        double* F = grp;
        double* G = grp + batch * ng * S;
        const double* d_phim = d_phi + (size_t)S * S;
        // groups of m blocks from zero state (each group a channel of the
        // one-level scan): their end states F
        rc = scan_dispatch(S, d_phi, f, nullptr, batch * ng, m, nullptr, F, st);
        // the group entry states G and the state after the last group
        if (!rc) rc = scan_dispatch(S, d_phim, F, zi, batch, ng, G, fin, st);
        // every group again from its entry state: the states entering every block
        if (!rc) rc = scan_dispatch(S, d_phi, f, G, batch * ng, m, sin, nullptr, st);
    }
    // 3. every block again from its true state; the samples past the last
    //    block from the state after it; the final state
    if (!rc)
        rc = launch_sosfilt<T>(x, ld_x, batch * nb, L, c, sin, nullptr, precision, y, ld_y, st, nb, L);
    if (!rc && tail > 0)
        rc = launch_sosfilt<T>(x + nb * L, ld_x, batch, tail, c, fin, zf, precision, y + nb * L,
                               ld_y, st);
    if (!rc && tail == 0 && zf) {
        cudaError_t e = cudaMemcpyAsync(zf, fin, sizeof(double) * (size_t)(batch * S),
                                        cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) rc = set_error(SCIR_ERR_CUDA, "zf copy: %s", cudaGetErrorString(e));
    }
    scratch_free(d_phi, st);
    scratch_free(f, st);
    scratch_free(sin, st);
    scratch_free(fin, st);
    scratch_free(grp, st);
    return rc;
}
template int sosfilt_blocked<float>(const float*, int64_t, int64_t, int64_t, const SosCoef&,
                                    const double*, double*, int, float*, int64_t, int64_t,
                                    cudaStream_t);
template int sosfilt_blocked<double>(const double*, int64_t, int64_t, int64_t, const SosCoef&,
                                     const double*, double*, int, double*, int64_t, int64_t,
                                     cudaStream_t);

}  // namespace scir
