// Launcher interfaces shared between the C-ABI layer and the kernel files.
#pragma once

#include "common.cuh"

namespace scir {

// A batched FIR request in correlation form:
//   y[row][o] = sum_{m<k} c[m] * x[row][o + s + m],  x = 0 outside [0, n),
// with c[m] = taps[reverse ? k-1-m : m] and o in [0, n_out).
struct FirArgs {
    const float* x;
    int64_t ld_x, batch, n;
    const float* taps;
    int64_t k;
    int reverse;
    int64_t s;
    float* y;
    int64_t ld_y, n_out;
};

// Fills reverse / s / n_out from a scir_fir_mode; returns a status.
int fir_geometry(int64_t n, int64_t k, int mode, int* reverse, int64_t* s, int64_t* n_out);

// v: outputs per thread (8 or 16), 0 = by tap count.
int launch_fir_simt(const FirArgs& a, bool exact, cudaStream_t st, int v = 0);
// Tensor-core (tcgen05) FIR with split-bf16 operands; terms = 2 (BF16X3) or 3 (BF16X6).
// Operand forms of the tensor-core FIR: two or three bf16 terms, or two fp16
// terms of power-of-two scaled operands.
enum TcForm : int { kTcBf16x3 = 2, kTcBf16x6 = 3, kTcFp16x3 = 4 };
int launch_fir_tc(const FirArgs& a, int form, cudaStream_t st);
bool fir_tc_supported(const FirArgs& a);

// Tensor-core bucket of a ragged plan (fir_tc.cu).  Each signal is tiled as
// up to 128 segment rows (row r = outputs [r * seg, (r + 1) * seg), seg a
// multiple of 1,024) over one bf16 plane per term that holds the signal
// after a zero pad of its filter history; a TMA map per signal reads the
// rows with stride seg (overlapping).  Tiles are (signal, window of a row,
// phase group).
struct TcSig {
    int64_t g_off;     // first element of the signal's tap planes [terms][8][LG]
    int64_t LG, k;
    int64_t seg;       // outputs per segment row
    int64_t n_out, y_off;
    int32_t m, nchunks, x0, rows, vec_store, pad_;
};
struct TcTile {
    int32_t sig, row0, blk, pg;
};
struct TcSigIn {       // one signal as the ragged plan describes it
    int64_t x_off, n, taps_off, k, y_off, s, n_out;
    int reverse;
};
struct TcRaggedPlan;
int tc_ragged_create(const TcSigIn* sigs, int64_t count, int form, TcRaggedPlan** out);
void tc_ragged_destroy(TcRaggedPlan* p);
int64_t tc_ragged_tiles(const TcRaggedPlan* p);
int tc_ragged_run(const TcRaggedPlan* p, const float* x, const float* taps, float* y,
                  cudaStream_t st);

// Polyphase FIR: y[m] = sum_q h[ph + q*up] * x[base - q],
// t = m*down + off, ph = t mod up, base = t div up, m in [0, n_out).
struct PolyArgs {
    const float* x;
    int64_t ld_x, batch, n;
    const float* h;
    int64_t kh;
    int up, down;
    int64_t off;
    float* y;
    int64_t ld_y, n_out;
};
// p_force: outputs per lane (at least the minimum for the rate), ct: channels
// per work item (1, 2 or 4); 0 = defaults.
int launch_poly_simt(const PolyArgs& a, cudaStream_t st, int p_force = 0, int ct = 0);

// Autotuning table (tune.cu): the recorded choice for a problem shape on the
// current device model, or 0 when the shape was never tuned.
// FIR choice: 1 = CUDA cores, 8 outputs per thread; 2 = CUDA cores, 16;
// 3 = tensor cores (BF16X6, AUTO precision only).
int tune_fir_choice(const FirArgs& a, int precision);
// polyphase choice: P * 10 + CT (0 = untuned).
int tune_poly_choice(const PolyArgs& a);
int launch_poly_tc(const PolyArgs& a, int terms, cudaStream_t st);
bool poly_tc_supported(const PolyArgs& a);

// Second-order sections.
struct SosCoef {
    double c[SCIR_SOS_MAX_SECTIONS][5];  // b0 b1 b2 a1 a2 (a0 taken as 1); unused = identity
    float cf[SCIR_SOS_MAX_SECTIONS][5];  // the same rounded to FP32
    double zi[SCIR_SOS_MAX_SECTIONS][2]; // sosfilt_zi (filtfilt with padding)
    // Coupled (modal) form of complex-pole sections, all from FP64 on the host:
    //   y = c1*u + c2*v + d*x;  u += (sigma-1)*u - omega*v + x;  v += omega*u + (sigma-1)*v
    float cp[SCIR_SOS_MAX_SECTIONS][5];  // sigma-1, omega, c1, c2, d
    int coupled[SCIR_SOS_MAX_SECTIONS];  // 0: real poles, the section runs DF2T in FP32
    double to_cp[SCIR_SOS_MAX_SECTIONS][4];   // DF2T state (s1, s2) -> coupled (u, v), row-major
    double from_cp[SCIR_SOS_MAX_SECTIONS][4]; // coupled (u, v) -> DF2T state (s1, s2)
    double zc[SCIR_SOS_MAX_SECTIONS][2];      // zi in coupled coordinates
    int nsec;
};

// Fills every field of SosCoef from a host [nsec][6] SOS matrix.
int build_sos_coef(const double* sos, int nsec, bool want_zi, SosCoef* c);
// FP32-state SOS (FP32, FP32_COUPLED) on f32 data: the cascade split over
// the warps of a CTA (sos_pipe.cu).
// blk_rows > 0 (sosfilt only) selects a blocked row view: row r is block
// r mod blk_rows, of blk_len samples at stride blk_len, of channel
// r div blk_rows (x and y rows ld_x / ld_y apart); blk_rows must be a
// multiple of 64.
int launch_sos_pipe(const float* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                    const double* zi, double* zf, bool filtfilt, int64_t edge, int use_zi,
                    int precision, float* y, int64_t ld_y, float* tail, cudaStream_t st,
                    int64_t blk_rows = 0, int64_t blk_len = 0);

template <typename T>
int launch_sosfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                   const double* zi, double* zf, int precision, T* y, int64_t ld_y,
                   cudaStream_t st, int64_t blk_rows = 0, int64_t blk_len = 0);
// Block-parallel time scan for few long channels (sos_scan.cu): the blocks
// per channel to cut the signal into (a multiple of 64), or 0 when the
// request should take the channel-parallel kernels as it is.
int64_t sos_scan_blocks(int64_t batch, int64_t n, int nsec, int precision, bool in_place);
template <typename T>
int sosfilt_blocked(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                    const double* zi, double* zf, int precision, T* y, int64_t ld_y, int64_t nb,
                    cudaStream_t st);
template <typename T>
int launch_sosfiltfilt(const T* x, int64_t ld_x, int64_t batch, int64_t n, const SosCoef& c,
                       int64_t edge, int use_zi, int precision, T* y, int64_t ld_y,
                       T* tail_scratch, cudaStream_t st);

// Argument checks of the sosfiltfilt entry points (api.cu): fills *c and the
// edge-extension length *edge, and initialises the current device.
int sosfiltfilt_check(const void* x, int64_t ld_x, int64_t batch, int64_t n, const double* sos,
                      int nsec, int padtype, int64_t padlen, const void* y, int64_t ld_y,
                      SosCoef* c, int64_t* edge);

// Host-side FP64 design helpers (design.cpp).
int sos_zi_host(const double* sos, int nsec, double* zi);
int64_t sos_default_padlen(const double* sos, int nsec);
int64_t gcd64(int64_t a, int64_t b);
// firwin low-pass, window 0 = Hamming, 1 = Kaiser(beta); unit DC gain.
void firwin_lowpass(int64_t numtaps, double cutoff, int window, double beta, double* h);

}  // namespace scir
