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
#include <cmath>
#include <cstdint>

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
