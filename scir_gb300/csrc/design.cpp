// Host-side FP64 filter-design helpers used by the entry points.
//
// - firwin_lowpass: windowed-sinc low-pass with unit DC gain, the
//   construction of scipy.signal.firwin(numtaps, cutoff, window) for a
//   single pass band starting at 0.  The reference's baked resample table
//   (crates/scir-signal/src/lib.rs:315-347) is firwin(31, 1/3, 'hamming')*2,
//   and SciPy's resample_poly default is firwin(20*max+1, 1/max,
//   ('kaiser', 5.0))*up; both are produced here instead of being stored.
// - sos_zi_host: scipy.signal.sosfilt_zi (per-section lfilter_zi in closed
//   form, scaled by the DC gain of the preceding sections).
// - sos_default_padlen: SciPy's filtfilt edge for an SOS cascade.
// - build_sos_coef: the kernel-parameter block of an SOS cascade, including
//   the coupled (modal) form of every complex-pole section and the maps
//   between its state and the DF2T state, all computed in FP64.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "kernels.cuh"
#include "scir_gb300.h"

namespace scir {

int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        const int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Modified Bessel function of the first kind, order 0, from its power series
// sum_k ((x/2)^k / k!)^2; terms are added until they stop changing the sum.
static double bessel_i0(double x) {
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= q / ((double)k * (double)k);
        const double next = sum + term;
        if (next == sum) break;
        sum = next;
    }
    return sum;
}

static double sinc(double x) {
    if (x == 0.0) return 1.0;
    const double px = M_PI * x;
    return std::sin(px) / px;
}

// window 0: symmetric Hamming 0.54 - 0.46 cos(2 pi n / (M-1));
// window 1: symmetric Kaiser I0(beta sqrt(1 - ((n - a)/a)^2)) / I0(beta), a = (M-1)/2.
void firwin_lowpass(int64_t numtaps, double cutoff, int window, double beta, double* h) {
    const double alpha = 0.5 * (double)(numtaps - 1);
    double sum = 0.0;
    const double i0b = window == 1 ? bessel_i0(beta) : 1.0;
    for (int64_t i = 0; i < numtaps; ++i) {
        const double m = (double)i - alpha;
        double w = 1.0;
        if (numtaps > 1) {
            if (window == 0) {
                const double fac = -M_PI + 2.0 * M_PI * (double)i / (double)(numtaps - 1);
                w = 0.54 + 0.46 * std::cos(fac);
            } else {
                const double r = m / alpha;
                const double arg = 1.0 - r * r;
                w = bessel_i0(beta * std::sqrt(arg > 0.0 ? arg : 0.0)) / i0b;
            }
        }
        h[i] = cutoff * sinc(cutoff * m) * w;
        sum += h[i];
    }
    for (int64_t i = 0; i < numtaps; ++i) h[i] /= sum;
}

int sos_zi_host(const double* sos, int nsec, double* zi) {
    double scale = 1.0;
    for (int s = 0; s < nsec; ++s) {
        const double* c = sos + 6 * s;
        double b0 = c[0], b1 = c[1], b2 = c[2], a0 = c[3], a1 = c[4], a2 = c[5];
        if (a0 == 0.0) return SCIR_ERR_INVALID_ARG;
        if (a0 != 1.0) {
            b0 /= a0; b1 /= a0; b2 /= a0; a1 /= a0; a2 /= a0; a0 = 1.0;
        }
        const double suma = a0 + a1 + a2;
        if (suma == 0.0) return SCIR_ERR_INVALID_ARG;
        const double yinf = (b0 + b1 + b2) / suma;
        const double d1 = b1 - yinf * a1, d2 = b2 - yinf * a2;
        zi[2 * s + 0] = scale * (d1 + d2);
        zi[2 * s + 1] = scale * d2;
        scale *= (c[0] + c[1] + c[2]) / (c[3] + c[4] + c[5]);
    }
    return SCIR_OK;
}

int64_t sos_default_padlen(const double* sos, int nsec) {
    int zb = 0, za = 0;
    for (int s = 0; s < nsec; ++s) {
        if (sos[6 * s + 2] == 0.0) ++zb;
        if (sos[6 * s + 5] == 0.0) ++za;
    }
    return 3 * (int64_t)(2 * nsec + 1 - (zb < za ? zb : za));
}

}  // namespace scir

namespace scir {

// Coupled form of H(z) = (b0 + b1 z^-1 + b2 z^-2) / (1 + a1 z^-1 + a2 z^-2)
// with complex poles sigma +- i omega:
//   state s = (u, v), s' = A s + [1, 0]^T x, A = [[sigma, -omega], [omega, sigma]],
//   y = C s + b0 x,  C = (b1 - a1 b0, (b2 - a2 b0 + C1 sigma) / omega),
// which has the same transfer function (the denominator of C (zI - A)^-1 B
// is z^2 + a1 z + a2).  Zero-input responses match DF2T when
// [C; CA] s = (s1, s2 - a1 s1), which gives the two state maps.
int build_sos_coef(const double* sos, int nsec, bool want_zi, SosCoef* c) {
    memset(c, 0, sizeof(*c));
    c->nsec = nsec;
    for (int s = 0; s < SCIR_SOS_MAX_SECTIONS; ++s) {
        if (s < nsec) {
            const double* r = sos + 6 * s;
            c->c[s][0] = r[0];
            c->c[s][1] = r[1];
            c->c[s][2] = r[2];
            c->c[s][3] = r[4];
            c->c[s][4] = r[5];
        } else {
            c->c[s][0] = 1.0;  // identity section: out = prev
        }
        for (int j = 0; j < 5; ++j) c->cf[s][j] = (float)c->c[s][j];
        if (s >= nsec) continue;
        const double b0 = c->c[s][0], b1 = c->c[s][1], b2 = c->c[s][2];
        const double a1 = c->c[s][3], a2 = c->c[s][4];
        const double disc = a1 * a1 - 4.0 * a2;
        if (!(disc < 0.0)) continue;  // real poles: DF2T
        const double sigma = -0.5 * a1, omega = 0.5 * std::sqrt(-disc);
        const double C1 = b1 - a1 * b0;
        const double C2 = (b2 - a2 * b0 + C1 * sigma) / omega;
        const double o00 = C1, o01 = C2;
        const double o10 = C1 * sigma + C2 * omega, o11 = -C1 * omega + C2 * sigma;
        const double det = o00 * o11 - o01 * o10;
        const double scale = std::fabs(o00 * o11) + std::fabs(o01 * o10);
        if (!(std::fabs(det) > 1e-12 * scale) || !std::isfinite(det)) continue;
        const double i00 = o11 / det, i01 = -o01 / det, i10 = -o10 / det, i11 = o00 / det;
        // (u, v) = O^-1 (s1, s2 - a1 s1)
        c->to_cp[s][0] = i00 - a1 * i01;
        c->to_cp[s][1] = i01;
        c->to_cp[s][2] = i10 - a1 * i11;
        c->to_cp[s][3] = i11;
        // (s1, s2) = (O0 s, O1 s + a1 O0 s)
        c->from_cp[s][0] = o00;
        c->from_cp[s][1] = o01;
        c->from_cp[s][2] = o10 + a1 * o00;
        c->from_cp[s][3] = o11 + a1 * o01;
        c->cp[s][0] = (float)(-0.5 * a1 - 1.0);  // sigma - 1, exact in FP64
        c->cp[s][1] = (float)omega;
        c->cp[s][2] = (float)C1;
        c->cp[s][3] = (float)C2;
        c->cp[s][4] = (float)b0;
        c->coupled[s] = 1;
    }
    if (want_zi) {
        double zi[2 * SCIR_SOS_MAX_SECTIONS];
        if (sos_zi_host(sos, nsec, zi) != SCIR_OK) return SCIR_ERR_INVALID_ARG;
        for (int s = 0; s < nsec; ++s) {
            c->zi[s][0] = zi[2 * s];
            c->zi[s][1] = zi[2 * s + 1];
            const double* m = c->to_cp[s];
            c->zc[s][0] = m[0] * zi[2 * s] + m[1] * zi[2 * s + 1];
            c->zc[s][1] = m[2] * zi[2 * s] + m[3] * zi[2 * s + 1];
        }
    }
    return SCIR_OK;
}

}  // namespace scir

// ------------------------------------------------------------------ firwin
// scipy.signal.firwin(numtaps, cutoff, window, pass_zero, scale, fs): the
// published windowed-sinc construction for any set of band edges.  Edges are
// normalised to Nyquist = 1; the pass bands are the intervals between
// consecutive entries of [0 if pass_zero] + cutoff + [1 if the last band
// reaches Nyquist]; h[i] = sum over bands of r sinc(r m) - l sinc(l m),
// m = i - (numtaps - 1)/2, times a symmetric window; with `scale` the
// response is set to 1 at the centre of the first pass band (0 if it starts
// at DC, Nyquist if it ends there).
namespace scir {
namespace {

double fir_window(int window, double beta, int64_t i, int64_t M) {
    if (M == 1) return 1.0;
    const double fac = -M_PI + (double)i * (2.0 * M_PI / (double)(M - 1));  // linspace(-pi, pi, M)
    switch (window) {
    case SCIR_WIN_HAMMING: return 0.54 + 0.46 * std::cos(fac);
    case SCIR_WIN_HANN: return 0.5 + 0.5 * std::cos(fac);
    case SCIR_WIN_BLACKMAN: return 0.42 + 0.5 * std::cos(fac) + 0.08 * std::cos(2.0 * fac);
    case SCIR_WIN_BOXCAR: return 1.0;
    default: {  // Kaiser: I0(beta sqrt(1 - (2i/(M-1) - 1)^2)) / I0(beta)
        const double r = 2.0 * (double)i / (double)(M - 1) - 1.0;
        const double arg = 1.0 - r * r;
        return bessel_i0(beta * std::sqrt(arg > 0.0 ? arg : 0.0)) / bessel_i0(beta);
    }
    }
}

}  // namespace

}  // namespace scir

extern "C" SCIR_API int scir_firwin(int64_t numtaps, const double* cutoff, int ncut, int window,
                                    double beta, int pass_zero, int scale, double fs,
                                    double* h) {
    using namespace scir;
    clear_error();
    SCIR_REQUIRE(numtaps >= 1, SCIR_ERR_INVALID_ARG, "numtaps must be >= 1");
    SCIR_REQUIRE(cutoff && ncut >= 1 && ncut <= 64 && h, SCIR_ERR_INVALID_ARG,
                 "need 1..64 cutoff frequencies and an output buffer");
    SCIR_REQUIRE(window >= SCIR_WIN_HAMMING && window <= SCIR_WIN_BOXCAR, SCIR_ERR_INVALID_ARG,
                 "unknown window %d", window);
    const double nyq = fs > 0.0 ? 0.5 * fs : 1.0;
    double edges[66];
    int ne = 0;
    if (pass_zero) edges[ne++] = 0.0;
    for (int i = 0; i < ncut; ++i) {
        const double c = cutoff[i] / nyq;
        SCIR_REQUIRE(c > 0.0 && c < 1.0, SCIR_ERR_INVALID_ARG,
                     "cutoff frequencies must be strictly between 0 and fs/2");
        SCIR_REQUIRE(i == 0 || c > edges[ne - 1], SCIR_ERR_INVALID_ARG,
                     "cutoff frequencies must increase");
        edges[ne++] = c;
    }
    // the last band reaches Nyquist when the count of edges so far is odd
    const bool pass_nyquist = (ne % 2) == 1;
    SCIR_REQUIRE(!(pass_nyquist && numtaps % 2 == 0), SCIR_ERR_INVALID_ARG,
                 "a filter with a pass band at Nyquist needs an odd number of taps");
    if (pass_nyquist) edges[ne++] = 1.0;
    const double alpha = 0.5 * (double)(numtaps - 1);
    for (int64_t i = 0; i < numtaps; ++i) {
        const double m = (double)i - alpha;
        double v = 0.0;
        for (int b = 0; b + 1 < ne; b += 2) {
            const double l = edges[b], r = edges[b + 1];
            v += r * sinc(r * m) - l * sinc(l * m);
        }
        h[i] = v * fir_window(window, beta, i, numtaps);
    }
    if (scale) {
        const double l = edges[0], r = edges[1];
        const double f = l == 0.0 ? 0.0 : r == 1.0 ? 1.0 : 0.5 * (l + r);
        double s = 0.0;
        for (int64_t i = 0; i < numtaps; ++i) s += h[i] * std::cos(M_PI * ((double)i - alpha) * f);
        SCIR_REQUIRE(s != 0.0, SCIR_ERR_INVALID_ARG, "zero response at the scaling frequency");
        for (int64_t i = 0; i < numtaps; ++i) h[i] /= s;
    }
    return SCIR_OK;
}
