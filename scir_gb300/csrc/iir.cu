// General IIR filtering y = lfilter(b, a, x) along the rows of a batch, and
// lfilter_zi, with scipy.signal.lfilter's semantics: a transposed direct
// form II over the whole polynomial (coefficients divided by a[0]),
//   y[i] = b0 x[i] + z0,   z_j = b_{j+1} x[i] - a_{j+1} y[i] + z_{j+1},
//   z_{N-1} = b_N x[i] - a_N y[i],
// with N = max(len(a), len(b)) - 1 state values per channel.  The state and
// the arithmetic are FP64 (a direct-form polynomial of high order loses its
// poles in FP32); f32 data are widened on load and rounded on store.  One
// thread walks one channel through 32 x 32 row tiles, like the SOS kernel.
// The reference has no general IIR on any device; SciPy's lfilter is the
// oracle.
#include "common.cuh"
#include "kernels.cuh"
#include "sos_math.cuh"

#include <cmath>
#include <cstring>
#include <utility>

namespace scir {
namespace {

constexpr int kMaxOrder = 32;

struct IirCoef {
    double b[kMaxOrder + 1];
    double a[kMaxOrder + 1];  // a[0] = 1
    int order;   // compiled recursion order (>= 1)
    int nstate;  // state values per channel in zi / zf: max(na, nb) - 1 (may be 0)
};

template <typename T, int ORD>
__global__ void __launch_bounds__(32)
lfilter_kernel(const T* __restrict__ x, int64_t ld_x, int64_t batch, int64_t n,
               const __grid_constant__ IirCoef c, const double* __restrict__ zi,
               double* __restrict__ zf, T* __restrict__ y, int64_t ld_y) {
    __shared__ T s[kTT][kTT + 1];
    const int lane = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * kTT;
    const int64_t ch = r0 + lane;
    const bool live = ch < batch;
    double z[ORD];
#pragma unroll
    for (int j = 0; j < ORD; ++j) z[j] = (zi && live && j < c.nstate) ? zi[ch * c.nstate + j] : 0.0;
    T nxt[kTT];
    tile_fetch(nxt, x, ld_x, r0, batch, n, 0, lane);
    for (int64_t t0 = 0; t0 < n; t0 += kTT) {
#pragma unroll
        for (int i = 0; i < kTT; ++i) s[i][lane] = nxt[i];
        __syncwarp();
        if (t0 + kTT < n) tile_fetch(nxt, x, ld_x, r0, batch, n, t0 + kTT, lane);
        const int tn = (int)((n - t0) < kTT ? (n - t0) : kTT);
        for (int t = 0; t < tn; ++t) {
            const double xi = (double)s[lane][t];
            const double yi = fma(c.b[0], xi, z[0]);
#pragma unroll
            for (int j = 0; j < ORD - 1; ++j)
                z[j] = fma(-c.a[j + 1], yi, fma(c.b[j + 1], xi, z[j + 1]));
            z[ORD - 1] = fma(-c.a[ORD], yi, c.b[ORD] * xi);
            s[lane][t] = (T)yi;
        }
        __syncwarp();
        tile_store(s, y, ld_y, r0, batch, n, t0, lane);
        __syncwarp();
    }
    if (zf && live)
        for (int j = 0; j < c.nstate; ++j) zf[ch * c.nstate + j] = z[j];
}

// Coefficients past the filter's order are zero, so a kernel of a larger
// compiled order computes the same recursion (its extra states stay zero).
#define SCIR_IIR_ORDERS(X) X(1) X(2) X(4) X(8) X(16) X(32)

template <typename T>
int launch_lfilter(const T* x, int64_t ld_x, int64_t batch, int64_t n, const IirCoef& c,
                   const double* zi, double* zf, T* y, int64_t ld_y, cudaStream_t st) {
    if (batch == 0) return SCIR_OK;
    const unsigned grid = (unsigned)ceil_div(batch, kTT);
#define SCIR_CASE(O)                                                                       \
    if (c.order <= O) {                                                                    \
        lfilter_kernel<T, O><<<grid, kTT, 0, st>>>(x, ld_x, batch, n, c, zi, zf, y, ld_y); \
        SCIR_LAUNCH_CHECK("lfilter_kernel");                                               \
        return SCIR_OK;                                                                    \
    }
    SCIR_IIR_ORDERS(SCIR_CASE)
#undef SCIR_CASE
    return set_error(SCIR_ERR_UNSUPPORTED, "IIR order above %d", kMaxOrder);
}

// Normalised coefficients (divided by a[0]) padded to the common order.
int make_coef(const double* b, int nb, const double* a, int na, IirCoef* c) {
    SCIR_REQUIRE(b && a && nb >= 1 && na >= 1, SCIR_ERR_INVALID_ARG, "empty b or a");
    SCIR_REQUIRE(a[0] != 0.0, SCIR_ERR_INVALID_ARG, "a[0] must be non-zero");
    const int order = (nb > na ? nb : na) - 1;
    SCIR_REQUIRE(order <= kMaxOrder, SCIR_ERR_UNSUPPORTED, "IIR order %d above %d", order,
                 kMaxOrder);
    memset(c, 0, sizeof(*c));
    for (int i = 0; i < nb; ++i) c->b[i] = b[i] / a[0];
    for (int i = 0; i < na; ++i) c->a[i] = a[i] / a[0];
    c->a[0] = 1.0;
    c->order = order < 1 ? 1 : order;
    c->nstate = order;
    return SCIR_OK;
}

template <typename T>
int lfilter_impl(const T* x, int64_t ld_x, int64_t batch, int64_t n, const double* b, int nb,
                 const double* a, int na, const double* zi, double* zf, T* y, int64_t ld_y,
                 void* stream) {
    clear_error();
    IirCoef c;
    int rc = make_coef(b, nb, a, na, &c);
    if (rc) return rc;
    SCIR_REQUIRE(batch >= 0 && n >= 0, SCIR_ERR_INVALID_ARG, "negative batch or length");
    SCIR_REQUIRE(ld_x >= n && ld_y >= n, SCIR_ERR_SHAPE, "row stride shorter than the row");
    if (batch > 0 && n > 0) SCIR_REQUIRE(x && y, SCIR_ERR_INVALID_ARG, "NULL buffer");
    SCIR_REQUIRE(y == x ? ld_y == ld_x : true, SCIR_ERR_INVALID_ARG,
                 "in-place lfilter needs ld_y == ld_x");
    SCIR_REQUIRE(ceil_div(batch, kTT) < (1LL << 31), SCIR_ERR_UNSUPPORTED, "batch too large");
    const DeviceInfo* info = nullptr;
    rc = current_device(&info);
    if (rc) return rc;
    if (batch == 0) return SCIR_OK;
    return launch_lfilter<T>(x, ld_x, batch, n, c, zi, zf, y, ld_y, as_stream(stream));
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" {

SCIR_API int scir_lfilter_f32(const float* x, int64_t ld_x, int64_t batch, int64_t n,
                              const double* b, int nb, const double* a, int na, const double* zi,
                              double* zf, float* y, int64_t ld_y, void* stream) {
    return lfilter_impl<float>(x, ld_x, batch, n, b, nb, a, na, zi, zf, y, ld_y, stream);
}

SCIR_API int scir_lfilter_f64(const double* x, int64_t ld_x, int64_t batch, int64_t n,
                              const double* b, int nb, const double* a, int na, const double* zi,
                              double* zf, double* y, int64_t ld_y, void* stream) {
    return lfilter_impl<double>(x, ld_x, batch, n, b, nb, a, na, zi, zf, y, ld_y, stream);
}

// scipy.signal.lfilter_zi: the steady state of the transposed direct form
// above under a unit step, z = A z + B with A = companion(a)^T (first column
// -a[1:], ones on the super-diagonal) and B = b[1:] - a[1:] * b[0]; the
// system (I - A) z = B is solved by Gaussian elimination with partial
// pivoting (order <= 32).
SCIR_API int scir_lfilter_zi(const double* b, int nb, const double* a, int na, double* zi) {
    clear_error();
    IirCoef c;
    int rc = make_coef(b, nb, a, na, &c);
    if (rc) return rc;
    SCIR_REQUIRE(zi != nullptr, SCIR_ERR_INVALID_ARG, "zi is NULL");
    const int N = (nb > na ? nb : na) - 1;
    if (N < 1) return SCIR_OK;
    // M = I - A, A[j][0] = -a[j+1], A[j][j+1] = 1
    double M[kMaxOrder][kMaxOrder + 1];
    for (int r = 0; r < N; ++r) {
        for (int col = 0; col < N; ++col) M[r][col] = (r == col) ? 1.0 : 0.0;
        M[r][0] += c.a[r + 1];
        if (r + 1 < N) M[r][r + 1] -= 1.0;
        M[r][N] = c.b[r + 1] - c.a[r + 1] * c.b[0];
    }
    for (int col = 0; col < N; ++col) {
        int piv = col;
        for (int r = col + 1; r < N; ++r)
            if (std::fabs(M[r][col]) > std::fabs(M[piv][col])) piv = r;
        SCIR_REQUIRE(M[piv][col] != 0.0, SCIR_ERR_INVALID_ARG,
                     "lfilter_zi: singular system (a pole at z = 1)");
        if (piv != col)
            for (int k = col; k <= N; ++k) std::swap(M[col][k], M[piv][k]);
        for (int r = col + 1; r < N; ++r) {
            const double f = M[r][col] / M[col][col];
            if (f == 0.0) continue;
            for (int k = col; k <= N; ++k) M[r][k] -= f * M[col][k];
        }
    }
    for (int r = N - 1; r >= 0; --r) {
        double v = M[r][N];
        for (int k = r + 1; k < N; ++k) v -= M[r][k] * zi[k];
        zi[r] = v / M[r][r];
    }
    return SCIR_OK;
}

}  // extern "C"
