// Host-side IIR design in FP64, so C and Rust callers get zeros/poles/gain
// and second-order sections without SciPy: the reference's iirfilter
// (crates/scir-iir-filters/src/filter_design.rs:216-314) with its
// prototypes (:322-445) and zpk2sos (crates/scir-iir-filters/src/sos.rs:
// 154-357), both following scipy.signal.iirfilter / zpk2sos.
//
//   1. analog low-pass prototype (zeros, poles, gain):
//      Butterworth  poles -exp(i*pi*m/(2N)), m = -N+1, -N+3, ..., N-1;
//      Chebyshev I  poles -sinh(mu + i*pi*m/(2N)), mu = asinh(1/eps)/N,
//                   eps = sqrt(10^(rp/10) - 1), gain prod(-p) (divided by
//                   sqrt(1 + eps^2) for even N);
//      Bessel       poles = roots of the reverse Bessel polynomial
//                   theta_N(s) = sum_k (2N-k)! / (2^(N-k) k! (N-k)!) s^k,
//                   found by Aberth-Ehrlich iteration in extended precision
//                   and scaled per normalisation: "delay" (the roots, gain
//                   theta_N(0)), "phase" (roots / theta_N(0)^(1/N), gain 1)
//                   or "mag" (phase poles / w3, w3 the -3 dB frequency,
//                   found by bisection; gain prod(-p));
//   2. frequency transform on the prewarped edges 4*tan(pi*Wn/2):
//      low-pass scaling, low-to-high inversion, low-to-band-pass and
//      low-to-band-stop substitutions (zeros at the origin or at +-i*wo for
//      the degree difference);
//   3. bilinear transform z = (4 + s) / (4 - s), extra zeros at -1;
//   4. zpk2sos: poles and zeros are reduced to one member per conjugate pair
//      (sorted by real part, then |imag|); "nearest" pads an odd count with
//      a pole and a zero at 0, "keep_odd" does not, "minimal" adds nothing
//      and may leave a first-order section; sections are filled from the
//      last to the first, each taking the remaining pole closest to the unit
//      circle (with its conjugate, or the next real pole closest to the
//      circle) and the zeros nearest to it, with two special cases (the last
//      real pole takes one real zero, plus a zero and a pole at 0 unless
//      "minimal"; a complex pole that would leave one real pole and one real
//      zero must take a complex zero); the gain goes into the first
//      section's numerator.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "scir_gb300.h"

namespace scir {
namespace {

using cplx = std::complex<double>;
using cvec = std::vector<cplx>;
using xreal = long double;
using xcplx = std::complex<long double>;

constexpr int kMaxDesignOrder = 256;
constexpr int kMaxBesselOrder = 25;

struct Zpk {
    cvec z, p;
    double k = 1.0;
};

Zpk buttap(int N) {
    Zpk r;
    for (int m = -N + 1; m <= N - 1; m += 2)
        r.p.push_back(-std::exp(cplx(0.0, M_PI * m / (2.0 * N))));
    return r;
}

Zpk cheb1ap(int N, double rp) {
    Zpk r;
    if (N == 0) {
        r.k = std::pow(10.0, -rp / 20.0);
        return r;
    }
    const double eps = std::sqrt(std::pow(10.0, 0.1 * rp) - 1.0);
    const double mu = std::asinh(1.0 / eps) / N;
    cplx prod(1.0, 0.0);
    for (int m = -N + 1; m <= N - 1; m += 2) {
        const cplx p = -std::sinh(cplx(mu, M_PI * m / (2.0 * N)));
        r.p.push_back(p);
        prod *= -p;
    }
    r.k = prod.real();
    if (N % 2 == 0) r.k /= std::sqrt(1.0 + eps * eps);
    return r;
}

// Roots of sum_k c[k] u^k (c[deg] = 1, real coefficients) by Aberth-Ehrlich
// iteration from conjugate-symmetric starting points on a circle of radius
// r0 in the left half-plane, then two Newton steps per root.
std::vector<xcplx> aberth_roots(const std::vector<xreal>& c, xreal r0) {
    const int deg = (int)c.size() - 1;
    std::vector<xcplx> u(deg);
    for (int j = 0; j < deg; ++j) {
        const xreal ang = (xreal)M_PI / 2 + (xreal)M_PI * (2 * j + 1) / (2 * deg);
        u[j] = xcplx(r0 * std::cos(ang), r0 * std::sin(ang));
        if (deg % 2 == 1 && j == deg / 2) u[j] = xcplx(-r0, 0);  // exactly real
    }
    auto eval = [&](const xcplx& x, xcplx* f, xcplx* df) {
        xcplx a = c[deg], d = 0;
        for (int k = deg - 1; k >= 0; --k) {
            d = d * x + a;
            a = a * x + c[k];
        }
        *f = a;
        *df = d;
    };
    const xreal tol = 8 * std::numeric_limits<xreal>::epsilon();
    for (int it = 0; it < 500; ++it) {
        xreal worst = 0;
        for (int j = 0; j < deg; ++j) {
            xcplx f, df;
            eval(u[j], &f, &df);
            if (f == xcplx(0)) continue;
            const xcplx w = f / df;
            xcplx s = 0;
            for (int q = 0; q < deg; ++q)
                if (q != j) s += xcplx(1) / (u[j] - u[q]);
            const xcplx step = w / (xcplx(1) - w * s);
            u[j] -= step;
            worst = std::max(worst, std::abs(step) / std::max(std::abs(u[j]), (xreal)1e-30));
        }
        if (worst < tol) break;
    }
    for (int j = 0; j < deg; ++j) {
        for (int it = 0; it < 2; ++it) {
            xcplx f, df;
            eval(u[j], &f, &df);
            if (df != xcplx(0)) u[j] -= f / df;
        }
    }
    return u;
}

// Double-double arithmetic (Dekker / Knuth error-free transformations:
// a value is hi + lo with |lo| <= ulp(hi)/2, about 106 significant bits).
// The roots of theta_N are ill-conditioned in the monomial basis (relative
// sensitivity ~1e12 at N = 25), so extended precision alone leaves ~1e-7;
// Newton steps in double-double bring them to double accuracy.
struct dd {
    double hi, lo;
};

dd two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
dd quick_two_sum(double a, double b) {
    const double s = a + b;
    return {s, b - (s - a)};
}
dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    const dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}
dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
dd dd_mul(dd a, dd b) {
    const double p = a.hi * b.hi;
    const double e = std::fma(a.hi, b.hi, -p);
    return quick_two_sum(p, e + (a.hi * b.lo + a.lo * b.hi));
}
dd dd_div(dd a, dd b) {
    const double q1 = a.hi / b.hi;
    dd r = dd_add(a, dd_neg(dd_mul(b, {q1, 0.0})));
    const double q2 = r.hi / b.hi;
    r = dd_add(r, dd_neg(dd_mul(b, {q2, 0.0})));
    const double q3 = r.hi / b.hi;
    return dd_add(quick_two_sum(q1, q2), {q3, 0.0});
}
dd dd_from(xreal v) {
    const double hi = (double)v;
    return {hi, (double)(v - (xreal)hi)};
}
xreal dd_to(dd a) { return (xreal)a.hi + (xreal)a.lo; }

struct cdd {
    dd re, im;
};
cdd c_add(cdd a, cdd b) { return {dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
cdd c_mul(cdd a, cdd b) {
    return {dd_add(dd_mul(a.re, b.re), dd_neg(dd_mul(a.im, b.im))),
            dd_add(dd_mul(a.re, b.im), dd_mul(a.im, b.re))};
}
cdd c_div(cdd a, cdd b) {
    const dd den = dd_add(dd_mul(b.re, b.re), dd_mul(b.im, b.im));
    const cdd num = c_mul(a, {b.re, dd_neg(b.im)});
    return {dd_div(num.re, den), dd_div(num.im, den)};
}

// Newton steps on theta_N (coefficients a, a[N] = 1) at the root r,
// evaluated by Horner's rule in double-double.
xcplx polish_dd(const std::vector<dd>& a, xcplx r) {
    const int N = (int)a.size() - 1;
    cdd x{dd_from(r.real()), dd_from(r.imag())};
    for (int it = 0; it < 6; ++it) {
        cdd f{a[N], {0.0, 0.0}}, d{{0.0, 0.0}, {0.0, 0.0}};
        for (int k = N - 1; k >= 0; --k) {
            d = c_add(c_mul(d, x), f);
            f = c_add(c_mul(f, x), {a[k], {0.0, 0.0}});
        }
        if (d.re.hi == 0.0 && d.im.hi == 0.0) break;
        const cdd step = c_div(f, d);
        x = {dd_add(x.re, dd_neg(step.re)), dd_add(x.im, dd_neg(step.im))};
    }
    return xcplx(dd_to(x.re), dd_to(x.im));
}

// norm: 0 phase, 1 delay, 2 mag.
Zpk besselap(int N, int norm) {
    Zpk r;
    if (N == 0) return r;
    // a[k] of theta_N with a[N] = 1: a[k] / a[k+1] = (2N-k)(k+1) / (2(N-k))
    std::vector<xreal> a(N + 1);
    a[N] = 1;
    for (int k = N - 1; k >= 0; --k) a[k] = a[k + 1] * (xreal)(2 * N - k) * (k + 1) / (2 * (N - k));
    // phase-normalised polynomial q(u) = theta_N(c u) / a[0], c = a[0]^(1/N):
    // coefficients a[k] c^k / a[0], both ends 1
    const xreal cn = std::pow(a[0], (xreal)1 / N);
    std::vector<xreal> q(N + 1);
    xreal ck = 1;
    for (int k = 0; k <= N; ++k) {
        q[k] = a[k] * ck / a[0];
        ck *= cn;
    }
    q[N] = 1;
    std::vector<xcplx> u = aberth_roots(q, 1.2L);
    // polish the delay-normalised roots (theta_N's integer coefficients are
    // exact in double-double) and scale back
    std::vector<dd> ad(N + 1);
    ad[N] = {1.0, 0.0};
    for (int k = N - 1; k >= 0; --k)
        ad[k] = dd_div(dd_mul(ad[k + 1], {(double)(2 * N - k) * (k + 1), 0.0}), {2.0 * (N - k), 0.0});
    for (xcplx& x : u) x = polish_dd(ad, x * cn) / cn;
    // conjugate-symmetric clean-up: exact reals, exact conjugate pairs
    std::sort(u.begin(), u.end(), [](const xcplx& x, const xcplx& y) {
        if (x.real() != y.real()) return x.real() < y.real();
        return x.imag() < y.imag();
    });
    std::vector<xcplx> clean;
    std::vector<bool> used(u.size(), false);
    for (size_t i = 0; i < u.size(); ++i) {
        if (used[i]) continue;
        used[i] = true;
        if (std::fabs(u[i].imag()) <= 1e-12L * std::abs(u[i])) {
            clean.push_back(xcplx(u[i].real(), 0));
            continue;
        }
        size_t best = i;
        xreal bd = std::numeric_limits<xreal>::max();
        for (size_t j = 0; j < u.size(); ++j) {
            if (used[j]) continue;
            const xreal d = std::abs(u[j] - std::conj(u[i]));
            if (d < bd) {
                bd = d;
                best = j;
            }
        }
        used[best] = true;
        const xcplx m = (u[i] + std::conj(u[best])) / (xreal)2;
        clean.push_back(m);
        clean.push_back(std::conj(m));
    }
    xreal scale = 1;  // divisor applied to the phase-normalised poles
    if (norm == 1) {
        scale = 1 / cn;
    } else if (norm == 2) {
        // |H(jw)|^2 = 1 / prod |jw - p|^2 for the phase form (prod(-p) = 1)
        auto excess = [&](xreal w) {
            xreal s = 0;
            for (const xcplx& p : clean) s += std::log(std::norm(xcplx(0, w) - p));
            return s - std::log((xreal)2);
        };
        xreal lo = 0, hi = 1;
        while (excess(hi) < 0) hi *= 2;
        for (int it = 0; it < 200 && hi - lo > 4 * std::numeric_limits<xreal>::epsilon() * hi; ++it) {
            const xreal mid = (lo + hi) / 2;
            (excess(mid) < 0 ? lo : hi) = mid;
        }
        scale = (lo + hi) / 2;
    }
    xcplx prod = 1;
    for (const xcplx& p : clean) {
        const xcplx ps = p / scale;
        r.p.push_back(cplx((double)ps.real(), (double)ps.imag()));
        prod *= -ps;
    }
    r.k = norm == 0 ? 1.0 : norm == 1 ? (double)a[0] : (double)prod.real();
    return r;
}

cplx prod_neg(const cvec& v) {
    cplx r(1.0, 0.0);
    for (const cplx& x : v) r *= -x;
    return r;
}

Zpk lp2lp(const Zpk& a, double wo) {
    Zpk r = a;
    for (cplx& x : r.z) x *= wo;
    for (cplx& x : r.p) x *= wo;
    r.k = a.k * std::pow(wo, (double)((int)a.p.size() - (int)a.z.size()));
    return r;
}

Zpk lp2hp(const Zpk& a, double wo) {
    Zpk r;
    const int degree = (int)a.p.size() - (int)a.z.size();
    for (const cplx& x : a.z) r.z.push_back(wo / x);
    for (const cplx& x : a.p) r.p.push_back(wo / x);
    for (int i = 0; i < degree; ++i) r.z.push_back(0.0);
    r.k = a.k * (prod_neg(a.z) / prod_neg(a.p)).real();
    return r;
}

void shift_pairs(const cvec& in, double wo, cvec* out) {
    for (const cplx& x : in) out->push_back(x + std::sqrt(x * x - wo * wo));
    for (const cplx& x : in) out->push_back(x - std::sqrt(x * x - wo * wo));
}

Zpk lp2bp(const Zpk& a, double wo, double bw) {
    Zpk r;
    const int degree = (int)a.p.size() - (int)a.z.size();
    cvec zl, pl;
    for (const cplx& x : a.z) zl.push_back(x * bw / 2.0);
    for (const cplx& x : a.p) pl.push_back(x * bw / 2.0);
    shift_pairs(zl, wo, &r.z);
    shift_pairs(pl, wo, &r.p);
    for (int i = 0; i < degree; ++i) r.z.push_back(0.0);
    r.k = a.k * std::pow(bw, (double)degree);
    return r;
}

Zpk lp2bs(const Zpk& a, double wo, double bw) {
    Zpk r;
    const int degree = (int)a.p.size() - (int)a.z.size();
    cvec zh, ph;
    for (const cplx& x : a.z) zh.push_back((bw / 2.0) / x);
    for (const cplx& x : a.p) ph.push_back((bw / 2.0) / x);
    shift_pairs(zh, wo, &r.z);
    shift_pairs(ph, wo, &r.p);
    for (int i = 0; i < degree; ++i) r.z.push_back(cplx(0.0, wo));
    for (int i = 0; i < degree; ++i) r.z.push_back(cplx(0.0, -wo));
    r.k = a.k * (prod_neg(a.z) / prod_neg(a.p)).real();
    return r;
}

Zpk bilinear(const Zpk& a, double fs) {
    Zpk r;
    const double fs2 = 2.0 * fs;
    const int degree = (int)a.p.size() - (int)a.z.size();
    cplx num(1.0, 0.0), den(1.0, 0.0);
    for (const cplx& x : a.z) {
        r.z.push_back((fs2 + x) / (fs2 - x));
        num *= fs2 - x;
    }
    for (const cplx& x : a.p) {
        r.p.push_back((fs2 + x) / (fs2 - x));
        den *= fs2 - x;
    }
    for (int i = 0; i < degree; ++i) r.z.push_back(-1.0);
    r.k = a.k * (num / den).real();
    return r;
}

// One member of each conjugate pair (positive imaginary part, the pair
// averaged) followed by the real values, each group sorted by real part and
// then |imag|; false if a complex value has no conjugate.
bool cplxreal(const cvec& in, cvec* out) {
    const double tol = 100.0 * std::numeric_limits<double>::epsilon();
    cvec z = in;
    std::stable_sort(z.begin(), z.end(), [](const cplx& a, const cplx& b) {
        if (a.real() != b.real()) return a.real() < b.real();
        return std::fabs(a.imag()) < std::fabs(b.imag());
    });
    cvec zr, zp, zn;
    for (const cplx& x : z) {
        if (std::fabs(x.imag()) <= tol * std::abs(x)) zr.push_back(cplx(x.real(), 0.0));
        else if (x.imag() > 0) zp.push_back(x);
        else zn.push_back(x);
    }
    if (zp.size() != zn.size()) return false;
    // runs of (approximately) equal real part are ordered by |imag|
    auto by_imag = [](const cplx& a, const cplx& b) { return std::fabs(a.imag()) < std::fabs(b.imag()); };
    size_t i = 0;
    while (i < zp.size()) {
        size_t j = i + 1;
        while (j < zp.size() && zp[j].real() - zp[j - 1].real() <= tol * std::abs(zp[j - 1])) ++j;
        std::stable_sort(zp.begin() + (long)i, zp.begin() + (long)j, by_imag);
        std::stable_sort(zn.begin() + (long)i, zn.begin() + (long)j, by_imag);
        i = j;
    }
    out->clear();
    for (size_t q = 0; q < zp.size(); ++q) {
        if (std::abs(zp[q] - std::conj(zn[q])) > tol * std::abs(zn[q])) return false;
        out->push_back((zp[q] + std::conj(zn[q])) / 2.0);
    }
    for (const cplx& x : zr) out->push_back(x);
    return true;
}

bool is_real(const cplx& x) { return x.imag() == 0.0; }

// First index of the value closest to the unit circle among `p` (only the
// real ones when real_only); SIZE_MAX if there is none.
size_t idx_worst(const cvec& p, bool real_only) {
    size_t best = (size_t)-1;
    double bd = std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < p.size(); ++i) {
        if (real_only && !is_real(p[i])) continue;
        const double d = std::fabs(1.0 - std::abs(p[i]));
        if (d < bd) {
            bd = d;
            best = i;
        }
    }
    return best;
}

// First index of the value of `fro` nearest to `to` among the real
// (which = 1), complex (2) or all (0) values; SIZE_MAX if there is none.
size_t nearest(const cvec& fro, const cplx& to, int which) {
    size_t best = (size_t)-1;
    double bd = std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < fro.size(); ++i) {
        if ((which == 1 && !is_real(fro[i])) || (which == 2 && is_real(fro[i]))) continue;
        const double d = std::abs(fro[i] - to);
        if (d < bd) {
            bd = d;
            best = i;
        }
    }
    return best;
}

// Real coefficients of prod (x - r_i), highest power first.
std::vector<double> poly_real(const cvec& roots) {
    cvec c(1, cplx(1.0, 0.0));
    for (const cplx& r : roots) {
        cvec n(c.size() + 1, cplx(0.0, 0.0));
        for (size_t i = 0; i < c.size(); ++i) {
            n[i] += c[i];
            n[i + 1] -= c[i] * r;
        }
        c = n;
    }
    std::vector<double> out(c.size());
    for (size_t i = 0; i < c.size(); ++i) out[i] = c[i].real();
    return out;
}

// Numerator right-aligned in row[0..2], denominator in row[3..5].
void single_sos(const cvec& z, const cvec& p, double* row) {
    for (int i = 0; i < 6; ++i) row[i] = 0.0;
    const std::vector<double> b = poly_real(z), a = poly_real(p);
    for (size_t i = 0; i < b.size(); ++i) row[3 - b.size() + i] = b[i];
    for (size_t i = 0; i < a.size(); ++i) row[6 - a.size() + i] = a[i];
}

bool take(cvec& v, size_t i, cplx* out) {
    if (i >= v.size()) return false;
    *out = v[i];
    v.erase(v.begin() + (long)i);
    return true;
}

int zpk2sos(const Zpk& f, int pairing, std::vector<double>* sos) {
    cvec z = f.z, p = f.p;
    if (z.empty() && p.empty()) {
        *sos = {f.k, 0.0, 0.0, 1.0, 0.0, 0.0};
        return SCIR_OK;
    }
    size_t nsec;
    if (pairing == SCIR_PAIR_MINIMAL) {
        SCIR_REQUIRE(p.size() >= z.size(), SCIR_ERR_INVALID_ARG,
                     "minimal pairing needs at least as many poles as zeros");
        nsec = (p.size() + 1) / 2;
    } else {
        while (p.size() < z.size()) p.push_back(0.0);
        while (z.size() < p.size()) z.push_back(0.0);
        nsec = (p.size() + 1) / 2;
        if (p.size() % 2 == 1 && pairing == SCIR_PAIR_NEAREST) {
            p.push_back(0.0);
            z.push_back(0.0);
        }
    }
    cvec zc, pc;
    SCIR_REQUIRE(cplxreal(z, &zc) && cplxreal(p, &pc), SCIR_ERR_INVALID_ARG,
                 "zpk2sos: a complex zero or pole has no conjugate");
    z = zc;
    p = pc;
    const char* lost = "zpk2sos: zeros and poles cannot be paired";
    sos->assign(nsec * 6, 0.0);
    for (size_t si = nsec; si-- > 0;) {
        double* row = sos->data() + si * 6;
        cplx p1, p2, z1, z2;
        SCIR_REQUIRE(take(p, idx_worst(p, false), &p1), SCIR_ERR_INVALID_ARG, "%s", lost);
        const long nreal_p = std::count_if(p.begin(), p.end(), is_real);
        const long nreal_z = std::count_if(z.begin(), z.end(), is_real);
        if (is_real(p1) && nreal_p == 0) {
            // the last real pole
            if (pairing != SCIR_PAIR_MINIMAL) {
                SCIR_REQUIRE(take(z, nearest(z, p1, 1), &z1), SCIR_ERR_INVALID_ARG, "%s", lost);
                single_sos({z1, 0.0}, {p1, 0.0}, row);
            } else if (!z.empty()) {
                SCIR_REQUIRE(take(z, nearest(z, p1, 1), &z1), SCIR_ERR_INVALID_ARG, "%s", lost);
                single_sos({z1}, {p1}, row);
            } else {
                single_sos({}, {p1}, row);
            }
        } else if (p.size() + 1 == z.size() && !is_real(p1) && nreal_p == 1 && nreal_z == 1) {
            // one real pole and one real zero would be left: take a complex zero
            SCIR_REQUIRE(take(z, nearest(z, p1, 2), &z1), SCIR_ERR_INVALID_ARG, "%s", lost);
            single_sos({z1, std::conj(z1)}, {p1, std::conj(p1)}, row);
        } else {
            if (is_real(p1)) {
                SCIR_REQUIRE(take(p, idx_worst(p, true), &p2), SCIR_ERR_INVALID_ARG, "%s", lost);
            } else {
                p2 = std::conj(p1);
            }
            if (z.empty()) {
                single_sos({}, {p1, p2}, row);
            } else {
                take(z, nearest(z, p1, 0), &z1);
                if (!is_real(z1)) {
                    single_sos({z1, std::conj(z1)}, {p1, p2}, row);
                } else if (!z.empty()) {
                    SCIR_REQUIRE(take(z, nearest(z, p1, 1), &z2), SCIR_ERR_INVALID_ARG, "%s", lost);
                    single_sos({z1, z2}, {p1, p2}, row);
                } else {
                    single_sos({z1}, {p1, p2}, row);
                }
            }
        }
    }
    SCIR_REQUIRE(z.empty() && p.empty(), SCIR_ERR_INVALID_ARG, "%s", lost);
    for (int i = 0; i < 3; ++i) (*sos)[i] *= f.k;
    return SCIR_OK;
}

int design_zpk(int order, int family, int btype, const double* wn, double rp, double fs, Zpk* out) {
    SCIR_REQUIRE(order >= 0 && order <= kMaxDesignOrder, SCIR_ERR_INVALID_ARG,
                 "order %d not in [0, %d]", order, kMaxDesignOrder);
    SCIR_REQUIRE(family >= SCIR_IIR_BUTTER && family <= SCIR_IIR_BESSEL_MAG, SCIR_ERR_INVALID_ARG,
                 "unknown filter family %d", family);
    SCIR_REQUIRE(btype >= SCIR_BAND_LOWPASS && btype <= SCIR_BAND_BANDSTOP, SCIR_ERR_INVALID_ARG,
                 "unknown band type %d", btype);
    SCIR_REQUIRE(wn != nullptr, SCIR_ERR_INVALID_ARG, "Wn is NULL");
    SCIR_REQUIRE(family != SCIR_IIR_CHEBY1 || rp > 0.0, SCIR_ERR_INVALID_ARG,
                 "pass-band ripple rp (dB) must be > 0");
    SCIR_REQUIRE(family < SCIR_IIR_BESSEL_PHASE || order <= kMaxBesselOrder, SCIR_ERR_INVALID_ARG,
                 "Bessel order %d above %d", order, kMaxBesselOrder);
    const int nw = btype >= SCIR_BAND_BANDPASS ? 2 : 1;
    double w[2];
    for (int i = 0; i < nw; ++i) {
        SCIR_REQUIRE(wn[i] > 0.0, SCIR_ERR_INVALID_ARG, "frequencies Wn must be > 0");
        w[i] = fs > 0.0 ? 2.0 * wn[i] / fs : wn[i];
        SCIR_REQUIRE(w[i] > 0.0 && w[i] < 1.0, SCIR_ERR_INVALID_ARG,
                     "digital critical frequencies must be 0 < Wn < fs/2");
    }
    if (nw == 2) SCIR_REQUIRE(w[0] < w[1], SCIR_ERR_INVALID_ARG, "band edges must increase");
    Zpk f = family == SCIR_IIR_BUTTER   ? buttap(order)
            : family == SCIR_IIR_CHEBY1 ? cheb1ap(order, rp)
                                        : besselap(order, family == SCIR_IIR_BESSEL_PHASE   ? 0
                                                          : family == SCIR_IIR_BESSEL_DELAY ? 1
                                                                                            : 2);
    const double fsd = 2.0;
    double warped[2];
    for (int i = 0; i < nw; ++i) warped[i] = 2.0 * fsd * std::tan(M_PI * w[i] / fsd);
    if (btype == SCIR_BAND_LOWPASS) f = lp2lp(f, warped[0]);
    else if (btype == SCIR_BAND_HIGHPASS) f = lp2hp(f, warped[0]);
    else if (btype == SCIR_BAND_BANDPASS) f = lp2bp(f, std::sqrt(warped[0] * warped[1]), warped[1] - warped[0]);
    else f = lp2bs(f, std::sqrt(warped[0] * warped[1]), warped[1] - warped[0]);
    *out = bilinear(f, fsd);
    return SCIR_OK;
}

int write_sos(const std::vector<double>& s, double* sos, int cap, int* nsec) {
    const int n = (int)(s.size() / 6);
    *nsec = n;
    if (sos) {
        SCIR_REQUIRE(cap >= n, SCIR_ERR_SHAPE, "%d sections, room for %d", n, cap);
        memcpy(sos, s.data(), s.size() * sizeof(double));
    }
    return SCIR_OK;
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" {

SCIR_API int scir_iirfilter_zpk(int order, int family, int btype, const double* wn, double rp,
                                double fs, double* z, double* p, int cap, int* nz, int* np,
                                double* k) {
    clear_error();
    SCIR_REQUIRE(nz && np && k, SCIR_ERR_INVALID_ARG, "NULL count or gain pointer");
    Zpk f;
    int rc = design_zpk(order, family, btype, wn, rp, fs, &f);
    if (rc) return rc;
    *nz = (int)f.z.size();
    *np = (int)f.p.size();
    *k = f.k;
    if (z || p) {
        SCIR_REQUIRE(z && p, SCIR_ERR_INVALID_ARG, "z and p must both be given or both NULL");
        SCIR_REQUIRE(cap >= *nz && cap >= *np, SCIR_ERR_SHAPE, "%d zeros / %d poles, room for %d",
                     *nz, *np, cap);
        for (size_t i = 0; i < f.z.size(); ++i) {
            z[2 * i] = f.z[i].real();
            z[2 * i + 1] = f.z[i].imag();
        }
        for (size_t i = 0; i < f.p.size(); ++i) {
            p[2 * i] = f.p[i].real();
            p[2 * i + 1] = f.p[i].imag();
        }
    }
    return SCIR_OK;
}

SCIR_API int scir_zpk2sos(const double* z, int nz, const double* p, int np, double k,
                          int pairing, double* sos, int cap, int* nsec) {
    clear_error();
    SCIR_REQUIRE(nz >= 0 && np >= 0 && nsec, SCIR_ERR_INVALID_ARG, "bad counts or NULL nsec");
    SCIR_REQUIRE((nz == 0 || z) && (np == 0 || p), SCIR_ERR_INVALID_ARG, "NULL zeros or poles");
    SCIR_REQUIRE(pairing >= SCIR_PAIR_NEAREST && pairing <= SCIR_PAIR_MINIMAL, SCIR_ERR_INVALID_ARG,
                 "unknown pairing %d", pairing);
    Zpk f;
    for (int i = 0; i < nz; ++i) f.z.push_back(cplx(z[2 * i], z[2 * i + 1]));
    for (int i = 0; i < np; ++i) f.p.push_back(cplx(p[2 * i], p[2 * i + 1]));
    f.k = k;
    std::vector<double> s;
    int rc = zpk2sos(f, pairing, &s);
    if (rc) return rc;
    return write_sos(s, sos, cap, nsec);
}

SCIR_API int scir_iirfilter_sos(int order, int family, int btype, const double* wn, double rp,
                                double fs, double* sos, int cap, int* nsec) {
    clear_error();
    SCIR_REQUIRE(nsec != nullptr, SCIR_ERR_INVALID_ARG, "nsec is NULL");
    Zpk f;
    int rc = design_zpk(order, family, btype, wn, rp, fs, &f);
    if (rc) return rc;
    std::vector<double> s;
    rc = zpk2sos(f, SCIR_PAIR_NEAREST, &s);
    if (rc) return rc;
    return write_sos(s, sos, cap, nsec);
}

}  // extern "C"
