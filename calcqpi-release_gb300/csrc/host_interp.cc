// host_interp.cc -- one-dimensional interpolation for the orbital-file tool (CPU only).
//
// mkwavefunctions interpolates a set of orbital files pixel by pixel between parameter values
// (interpolate(), src/mkwavefunctions.cc:39-70) with GSL's gsl_interp (GSL 2.x, a dependency
// that is not part of the reference's sources).  The methods are restated from their
// published definitions:
//   linear            piecewise linear;
//   polynomial        the single polynomial through all points (Newton form);
//   cspline           cubic spline with natural ends (second derivative zero);
//   cspline_periodic  cubic spline whose first and second derivatives wrap around;
//   akima             Akima (1970): the slope at x_i weights the neighbouring interval slopes
//                     m_{i-1}, m_i by |m_{i+1} - m_i| and |m_{i-1} - m_{i-2}|; the two missing
//                     interval slopes at each end continue linearly (m_{-1} = 2 m_0 - m_1,
//                     m_{-2} = 3 m_0 - 2 m_1, likewise at the right end); where both weights
//                     vanish the interval is kept straight (the non-rounded corner);
//   akima_periodic    the same with the interval slopes continued periodically;
//   steffen           Steffen (1990, A&A 239, 443): monotone cubic Hermite slopes
//                     (sign(m_{i-1}) + sign(m_i)) min(|m_{i-1}|, |m_i|, |p_i| / 2), p_i the
//                     slope of the parabola through the three points; end slopes from the
//                     one-sided parabola, zero when it turns against the end interval and at
//                     most twice that interval's slope.
// A point outside [xa[0], xa[n-1]], x values that do not strictly increase, or fewer points
// than the method needs (2 linear / cspline_periodic, 3 polynomial / cspline / steffen,
// 5 akima) return CQPI_ERR_ARG.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "cqpi.h"
#include "cqpi_host.h"

namespace {

enum Method { LINEAR, POLYNOMIAL, CSPLINE, CSPLINE_PERIODIC, AKIMA, AKIMA_PERIODIC, STEFFEN };

struct MethodInfo {
    const char *name;
    Method m;
    int min_points;
};

const MethodInfo kMethods[] = {{"linear", LINEAR, 2},     {"polynomial", POLYNOMIAL, 3},
                               {"cspline", CSPLINE, 3},   {"cspline_periodic", CSPLINE_PERIODIC, 2},
                               {"akima", AKIMA, 5},       {"akima_periodic", AKIMA_PERIODIC, 5},
                               {"steffen", STEFFEN, 3}};

// Solve a (possibly cyclic) tridiagonal system densely: n stays small (one value per file).
bool solve_dense(std::vector<double> &A, std::vector<double> &r, int n)
{
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int q = c + 1; q < n; q++)
            if (std::fabs(A[q * n + c]) > std::fabs(A[p * n + c])) p = q;
        if (A[p * n + c] == 0.0) return false;
        if (p != c) {
            for (int q = 0; q < n; q++) std::swap(A[c * n + q], A[p * n + q]);
            std::swap(r[c], r[p]);
        }
        for (int q = c + 1; q < n; q++) {
            const double f = A[q * n + c] / A[c * n + c];
            if (f == 0.0) continue;
            for (int e = c; e < n; e++) A[q * n + e] -= f * A[c * n + e];
            r[q] -= f * r[c];
        }
    }
    for (int c = n - 1; c >= 0; c--) {
        double v = r[c];
        for (int e = c + 1; e < n; e++) v -= A[c * n + e] * r[e];
        r[c] = v / A[c * n + c];
    }
    return true;
}

// Second derivatives of the natural (periodic = false) or periodic cubic spline.
bool spline_second(const double *xa, const double *ya, int n, bool periodic, std::vector<double> &M)
{
    M.assign(n, 0.0);
    const int ni = n - 1;
    std::vector<double> h(ni), m(ni);
    for (int i = 0; i < ni; i++) {
        h[i] = xa[i + 1] - xa[i];
        m[i] = (ya[i + 1] - ya[i]) / h[i];
    }
    if (!periodic) {
        // interior points 1..n-2: h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1} = 6 (m_i - m_{i-1})
        const int k = n - 2;
        std::vector<double> A((size_t)k * k, 0.0), r(k);
        for (int j = 0; j < k; j++) {
            const int i = j + 1;
            if (j > 0) A[j * k + j - 1] = h[i - 1];
            A[j * k + j] = 2.0 * (h[i - 1] + h[i]);
            if (j + 1 < k) A[j * k + j + 1] = h[i];
            r[j] = 6.0 * (m[i] - m[i - 1]);
        }
        if (!solve_dense(A, r, k)) return false;
        for (int j = 0; j < k; j++) M[j + 1] = r[j];
        return true;
    }
    if (ni < 2) return true;   // two points: a straight line
    // points 0..ni-1 on a circle (point ni is point 0)
    std::vector<double> A((size_t)ni * ni, 0.0), r(ni);
    for (int i = 0; i < ni; i++) {
        const int il = (i + ni - 1) % ni, ir = (i + 1) % ni;
        A[i * ni + il] += h[il];
        A[i * ni + i] += 2.0 * (h[il] + h[i]);
        A[i * ni + ir] += h[i];
        r[i] = 6.0 * (m[i] - m[il]);
    }
    if (!solve_dense(A, r, ni)) return false;
    for (int i = 0; i < ni; i++) M[i] = r[i];
    M[ni] = M[0];
    return true;
}

double hermite(double x0, double x1, double y0, double y1, double s0, double s1, double x)
{
    const double h = x1 - x0, t = x - x0, m = (y1 - y0) / h;
    const double c = (3.0 * m - 2.0 * s0 - s1) / h, d = (s0 + s1 - 2.0 * m) / (h * h);
    return y0 + t * (s0 + t * (c + t * d));
}

double sgn_nonzero(double v) { return std::signbit(v) ? -1.0 : 1.0; }

}  // namespace

extern "C" {

int cqpi_interp_known(const char *method)
{
    if (!method) return 0;
    for (const MethodInfo &mi : kMethods)
        if (!strcmp(method, mi.name)) return 1;
    return 0;
}

int cqpi_interp_eval(const char *method, int32_t n, const double *xa, const double *ya, int32_t count,
                     const double *x, double *y)
{
    const MethodInfo *mi = nullptr;
    if (method)
        for (const MethodInfo &k : kMethods)
            if (!strcmp(method, k.name)) mi = &k;
    if (!mi) return CQPI_ERR_ARG;
    if (!xa || !ya || !x || !y || count < 0 || n < mi->min_points) return CQPI_ERR_ARG;
    for (int i = 0; i + 1 < n; i++)
        if (!(xa[i] < xa[i + 1])) return CQPI_ERR_ARG;
    for (int q = 0; q < count; q++)
        if (!(x[q] >= xa[0] && x[q] <= xa[n - 1])) return CQPI_ERR_ARG;
    const int ni = n - 1;
    std::vector<double> h(ni), m(ni);
    for (int i = 0; i < ni; i++) {
        h[i] = xa[i + 1] - xa[i];
        m[i] = (ya[i + 1] - ya[i]) / h[i];
    }
    auto interval = [&](double v) {
        int lo = 0, hi = n - 1;   // xa[lo] <= v < xa[hi]; v = xa[n-1] falls in the last interval
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (xa[mid] > v) hi = mid;
            else lo = mid;
        }
        return lo;
    };
    switch (mi->m) {
    case LINEAR:
        for (int q = 0; q < count; q++) {
            const int i = interval(x[q]);
            y[q] = ya[i] + (x[q] - xa[i]) * m[i];
        }
        break;
    case POLYNOMIAL: {
        std::vector<double> c(ya, ya + n);   // divided differences, in place
        for (int k = 1; k < n; k++)
            for (int i = n - 1; i >= k; i--) c[i] = (c[i] - c[i - 1]) / (xa[i] - xa[i - k]);
        for (int q = 0; q < count; q++) {
            double v = c[n - 1];
            for (int k = n - 2; k >= 0; k--) v = v * (x[q] - xa[k]) + c[k];
            y[q] = v;
        }
        break;
    }
    case CSPLINE:
    case CSPLINE_PERIODIC: {
        std::vector<double> M;
        if (!spline_second(xa, ya, n, mi->m == CSPLINE_PERIODIC, M)) return CQPI_ERR_ARG;
        for (int q = 0; q < count; q++) {
            const int i = interval(x[q]);
            const double t = x[q] - xa[i];
            const double b = m[i] - h[i] * (2.0 * M[i] + M[i + 1]) / 6.0;
            y[q] = ya[i] + t * (b + t * (M[i] / 2.0 + t * (M[i + 1] - M[i]) / (6.0 * h[i])));
        }
        break;
    }
    case AKIMA:
    case AKIMA_PERIODIC: {
        // slope of interval j at ms[j + 2], two extra slopes on either side
        std::vector<double> ms(ni + 4);
        for (int i = 0; i < ni; i++) ms[i + 2] = m[i];
        if (mi->m == AKIMA) {
            ms[1] = 2.0 * m[0] - m[1];
            ms[0] = 3.0 * m[0] - 2.0 * m[1];
            ms[ni + 2] = 2.0 * m[ni - 1] - m[ni - 2];
            ms[ni + 3] = 3.0 * m[ni - 1] - 2.0 * m[ni - 2];
        } else {
            ms[1] = m[ni - 1];
            ms[0] = m[ni - 2];
            ms[ni + 2] = m[0];
            ms[ni + 3] = m[1];
        }
        // Akima slope at point i (interval slopes m_{i-2}..m_{i+1} = ms[i..i+3]); flag when
        // both weights vanish
        auto slope = [&](int i, bool &flat) {
            const double w1 = std::fabs(ms[i + 3] - ms[i + 2]), w2 = std::fabs(ms[i + 1] - ms[i]);
            flat = (w1 + w2 == 0.0);
            return flat ? 0.0 : (w1 * ms[i + 1] + w2 * ms[i + 2]) / (w1 + w2);
        };
        for (int q = 0; q < count; q++) {
            const int i = interval(x[q]);
            bool fl, fr;
            const double sl = slope(i, fl);
            double sr = slope(i + 1, fr);
            if (fl) {
                y[q] = ya[i] + (x[q] - xa[i]) * m[i];
                continue;
            }
            if (fr) sr = m[i];
            y[q] = hermite(xa[i], xa[i + 1], ya[i], ya[i + 1], sl, sr, x[q]);
        }
        break;
    }
    case STEFFEN: {
        std::vector<double> s(n);
        for (int i = 1; i < ni; i++) {
            const double p = (m[i - 1] * h[i] + m[i] * h[i - 1]) / (h[i - 1] + h[i]);
            const double a = std::fmin(std::fmin(std::fabs(m[i - 1]), std::fabs(m[i])), 0.5 * std::fabs(p));
            s[i] = (sgn_nonzero(m[i - 1]) + sgn_nonzero(m[i])) * a;
        }
        auto end_slope = [](double m0, double m1, double h0, double h1) {
            const double p = m0 * (1.0 + h0 / (h0 + h1)) - m1 * h0 / (h0 + h1);
            if (p * m0 <= 0.0) return 0.0;
            if (std::fabs(p) > 2.0 * std::fabs(m0)) return 2.0 * m0;
            return p;
        };
        s[0] = end_slope(m[0], m[1], h[0], h[1]);
        s[n - 1] = end_slope(m[ni - 1], m[ni - 2], h[ni - 1], h[ni - 2]);
        for (int q = 0; q < count; q++) {
            const int i = interval(x[q]);
            y[q] = hermite(xa[i], xa[i + 1], ya[i], ya[i + 1], s[i], s[i + 1], x[q]);
        }
        break;
    }
    }
    return CQPI_OK;
}

}  // extern "C"
