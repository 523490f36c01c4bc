/*
 * gsl_interp.h -- project-written subset of the GSL 2.x one-dimensional interpolation API
 * ("Interpolation" chapter of the GSL reference manual): gsl_interp_{linear, polynomial,
 * cspline, cspline_periodic, akima, akima_periodic, steffen}, gsl_interp_alloc / init /
 * eval / free / name and the accelerator calls.
 *
 * TEST INFRASTRUCTURE ONLY: it lets oracle/build_ref.sh compile the reference's unmodified
 * src/mkwavefunctions.cc (its interpolate(), :39-70).  GSL itself is not installed here and
 * no GSL source was used; every method is written from its published description:
 *   linear            piecewise linear;
 *   polynomial        the interpolating polynomial through all points (Newton divided
 *                     differences);
 *   cspline           cubic spline, natural ends (zero second derivative);
 *   cspline_periodic  cubic spline with periodic first and second derivatives;
 *   akima             Akima (1970) slopes, the two missing end slopes on each side
 *                     extrapolated linearly from the first / last two interval slopes,
 *                     and a straight interval where the Akima weights vanish
 *                     ("non-rounded corner");
 *   akima_periodic    the same with the interval slopes continued periodically;
 *   steffen           Steffen (1990) monotone cubic Hermite slopes, one-sided parabola
 *                     slopes at the ends limited as in the paper.
 * Outside [xa[0], xa[n-1]] gsl_interp_eval reports through the GSL error handler, which
 * aborts the program by default; this shim does the same.
 */
#ifndef CQPI_COMPAT_GSL_INTERP_H
#define CQPI_COMPAT_GSL_INTERP_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <vector>

typedef struct {
    const char *name;
    unsigned int min_size;
    int kind;
} gsl_interp_type;

enum { CQPI_GI_LINEAR, CQPI_GI_POLY, CQPI_GI_CSPLINE, CQPI_GI_CSPLINE_P, CQPI_GI_AKIMA, CQPI_GI_AKIMA_P, CQPI_GI_STEFFEN };

static const gsl_interp_type cqpi_gi_types[7] = {
    {"linear", 2, CQPI_GI_LINEAR},   {"polynomial", 3, CQPI_GI_POLY},       {"cspline", 3, CQPI_GI_CSPLINE},
    {"cspline-periodic", 2, CQPI_GI_CSPLINE_P}, {"akima", 5, CQPI_GI_AKIMA}, {"akima-periodic", 5, CQPI_GI_AKIMA_P},
    {"steffen", 3, CQPI_GI_STEFFEN}};
static const gsl_interp_type *gsl_interp_linear = &cqpi_gi_types[0];
static const gsl_interp_type *gsl_interp_polynomial = &cqpi_gi_types[1];
static const gsl_interp_type *gsl_interp_cspline = &cqpi_gi_types[2];
static const gsl_interp_type *gsl_interp_cspline_periodic = &cqpi_gi_types[3];
static const gsl_interp_type *gsl_interp_akima = &cqpi_gi_types[4];
static const gsl_interp_type *gsl_interp_akima_periodic = &cqpi_gi_types[5];
static const gsl_interp_type *gsl_interp_steffen = &cqpi_gi_types[6];

typedef struct {
    const gsl_interp_type *type;
    size_t size;
    std::vector<double> xa, ya;
    std::vector<double> b, c, d;   // per interval: y = y_i + b t + c t^2 + d t^3, t = x - x_i
    std::vector<double> dd;        // Newton coefficients (polynomial)
} gsl_interp;

typedef struct { size_t cache; } gsl_interp_accel;

static inline void cqpi_gi_fail(const char *why)
{
    fprintf(stderr, "gsl: interpolation error: %s\n", why);
    abort();
}

static inline gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n)
{
    if (n < T->min_size) cqpi_gi_fail("insufficient number of points for interpolation type");
    gsl_interp *g = new gsl_interp;
    g->type = T;
    g->size = n;
    return g;
}
static inline void gsl_interp_free(gsl_interp *g) { delete g; }
static inline const char *gsl_interp_name(const gsl_interp *g) { return g->type->name; }
static inline gsl_interp_accel *gsl_interp_accel_alloc(void) { return new gsl_interp_accel{0}; }
static inline void gsl_interp_accel_free(gsl_interp_accel *a) { delete a; }

// Hermite interval coefficients from the end slopes s0, s1
static inline void cqpi_gi_hermite(gsl_interp *g, size_t i, double s0, double s1)
{
    const double h = g->xa[i + 1] - g->xa[i], m = (g->ya[i + 1] - g->ya[i]) / h;
    g->b[i] = s0;
    g->c[i] = (3.0 * m - 2.0 * s0 - s1) / h;
    g->d[i] = (s0 + s1 - 2.0 * m) / (h * h);
}

// cubic spline coefficients from the second derivatives M (size n)
static inline void cqpi_gi_from_second(gsl_interp *g, const std::vector<double> &M)
{
    for (size_t i = 0; i + 1 < g->size; i++) {
        const double h = g->xa[i + 1] - g->xa[i];
        g->b[i] = (g->ya[i + 1] - g->ya[i]) / h - h * (2.0 * M[i] + M[i + 1]) / 6.0;
        g->c[i] = M[i] / 2.0;
        g->d[i] = (M[i + 1] - M[i]) / (6.0 * h);
    }
}

static inline int gsl_interp_init(gsl_interp *g, const double *xa, const double *ya, size_t n)
{
    if (n != g->size) cqpi_gi_fail("data must match size of interpolation object");
    for (size_t i = 0; i + 1 < n; i++)
        if (!(xa[i] < xa[i + 1])) cqpi_gi_fail("x values must be strictly increasing");
    g->xa.assign(xa, xa + n);
    g->ya.assign(ya, ya + n);
    const size_t ni = n - 1;
    g->b.assign(ni, 0.0);
    g->c.assign(ni, 0.0);
    g->d.assign(ni, 0.0);
    std::vector<double> h(ni), m(ni);
    for (size_t i = 0; i < ni; i++) {
        h[i] = xa[i + 1] - xa[i];
        m[i] = (ya[i + 1] - ya[i]) / h[i];
    }
    switch (g->type->kind) {
    case CQPI_GI_LINEAR:
        for (size_t i = 0; i < ni; i++) g->b[i] = m[i];
        break;
    case CQPI_GI_POLY: {
        g->dd.assign(ya, ya + n);
        for (size_t k = 1; k < n; k++)
            for (size_t i = n - 1; i >= k; i--) g->dd[i] = (g->dd[i] - g->dd[i - 1]) / (xa[i] - xa[i - k]);
        break;
    }
    case CQPI_GI_CSPLINE: {
        // natural spline: M_0 = M_{n-1} = 0, tridiagonal system for the interior M (Thomas)
        std::vector<double> M(n, 0.0);
        const size_t k = n - 2;
        std::vector<double> diag(k), up(k), rhs(k);
        for (size_t j = 0; j < k; j++) {
            diag[j] = 2.0 * (h[j] + h[j + 1]);
            up[j] = h[j + 1];
            rhs[j] = 6.0 * (m[j + 1] - m[j]);
        }
        for (size_t j = 1; j < k; j++) {
            const double f = h[j] / diag[j - 1];
            diag[j] -= f * up[j - 1];
            rhs[j] -= f * rhs[j - 1];
        }
        for (size_t j = k; j-- > 0;) M[j + 1] = (rhs[j] - (j + 1 < k ? up[j] * M[j + 2] : 0.0)) / diag[j];
        cqpi_gi_from_second(g, M);
        break;
    }
    case CQPI_GI_CSPLINE_P: {
        // periodic spline on the ni unique points: cyclic tridiagonal system, solved densely
        std::vector<double> M(n, 0.0);
        if (ni >= 2) {
            std::vector<double> A(ni * ni, 0.0), r(ni);
            for (size_t j = 0; j < ni; j++) {
                const size_t jm = (j + ni - 1) % ni;   // interval before point j
                A[j * ni + jm] += h[jm];
                A[j * ni + j] += 2.0 * (h[jm] + h[j]);
                A[j * ni + (j + 1) % ni] += h[j];
                r[j] = 6.0 * (m[j] - m[jm]);
            }
            for (size_t c = 0; c < ni; c++) {
                size_t p = c;
                for (size_t q = c + 1; q < ni; q++)
                    if (fabs(A[q * ni + c]) > fabs(A[p * ni + c])) p = q;
                for (size_t q = 0; q < ni; q++) { double t = A[c * ni + q]; A[c * ni + q] = A[p * ni + q]; A[p * ni + q] = t; }
                { double t = r[c]; r[c] = r[p]; r[p] = t; }
                for (size_t q = c + 1; q < ni; q++) {
                    const double f = A[q * ni + c] / A[c * ni + c];
                    for (size_t e = c; e < ni; e++) A[q * ni + e] -= f * A[c * ni + e];
                    r[q] -= f * r[c];
                }
            }
            for (size_t c = ni; c-- > 0;) {
                double v = r[c];
                for (size_t e = c + 1; e < ni; e++) v -= A[c * ni + e] * M[e];
                M[c] = v / A[c * ni + c];
            }
            M[ni] = M[0];
        }
        cqpi_gi_from_second(g, M);
        break;
    }
    case CQPI_GI_AKIMA:
    case CQPI_GI_AKIMA_P: {
        // interval slopes with two extra on each side: e[j + 2] = slope of interval j
        std::vector<double> e(ni + 4);
        for (size_t i = 0; i < ni; i++) e[i + 2] = m[i];
        if (g->type->kind == CQPI_GI_AKIMA) {
            e[1] = 2.0 * m[0] - m[1];
            e[0] = 3.0 * m[0] - 2.0 * m[1];
            e[ni + 2] = 2.0 * m[ni - 1] - m[ni - 2];
            e[ni + 3] = 3.0 * m[ni - 1] - 2.0 * m[ni - 2];
        } else {
            e[1] = m[ni - 1];
            e[0] = m[ni - 2];
            e[ni + 2] = m[0];
            e[ni + 3] = m[1];
        }
        // weights at point i: w1 = |m_{i+1} - m_i|, w2 = |m_{i-1} - m_{i-2}|
        for (size_t i = 0; i < ni; i++) {
            const double wl1 = fabs(e[i + 3] - e[i + 2]), wl2 = fabs(e[i + 1] - e[i]);
            if (wl1 + wl2 == 0.0) {
                // straight interval
                g->b[i] = m[i];
                continue;
            }
            const double sl = (wl1 * e[i + 1] + wl2 * e[i + 2]) / (wl1 + wl2);
            const double wr1 = fabs(e[i + 4] - e[i + 3]), wr2 = fabs(e[i + 2] - e[i + 1]);
            const double sr = (wr1 + wr2 == 0.0) ? m[i] : (wr1 * e[i + 2] + wr2 * e[i + 3]) / (wr1 + wr2);
            cqpi_gi_hermite(g, i, sl, sr);
        }
        break;
    }
    case CQPI_GI_STEFFEN: {
        std::vector<double> s(n);
        for (size_t i = 1; i < ni; i++) {
            const double p = (m[i - 1] * h[i] + m[i] * h[i - 1]) / (h[i - 1] + h[i]);
            const double sg = copysign(1.0, m[i - 1]) + copysign(1.0, m[i]);
            double a = fabs(m[i - 1]);
            if (fabs(m[i]) < a) a = fabs(m[i]);
            if (0.5 * fabs(p) < a) a = 0.5 * fabs(p);
            s[i] = sg * a;
        }
        // ends: slope of the parabola through the first / last three points, limited
        {
            const double p0 = m[0] * (1.0 + h[0] / (h[0] + h[1])) - m[1] * h[0] / (h[0] + h[1]);
            s[0] = (p0 * m[0] <= 0.0) ? 0.0 : (fabs(p0) > 2.0 * fabs(m[0]) ? 2.0 * m[0] : p0);
            const size_t L = ni - 1;
            const double pn = m[L] * (1.0 + h[L] / (h[L] + h[L - 1])) - m[L - 1] * h[L] / (h[L] + h[L - 1]);
            s[n - 1] = (pn * m[L] <= 0.0) ? 0.0 : (fabs(pn) > 2.0 * fabs(m[L]) ? 2.0 * m[L] : pn);
        }
        for (size_t i = 0; i < ni; i++) cqpi_gi_hermite(g, i, s[i], s[i + 1]);
        break;
    }
    }
    return 0;
}

static inline double gsl_interp_eval(const gsl_interp *g, const double *xa, const double *ya, double x,
                                     gsl_interp_accel *acc)
{
    (void)xa;
    (void)ya;
    (void)acc;
    const size_t n = g->size;
    if (x < g->xa[0] || x > g->xa[n - 1]) cqpi_gi_fail("interpolation error (x outside the data range)");
    if (g->type->kind == CQPI_GI_POLY) {
        double v = g->dd[n - 1];
        for (size_t k = n - 1; k-- > 0;) v = v * (x - g->xa[k]) + g->dd[k];
        return v;
    }
    size_t lo = 0, hi = n - 1;   // interval i with xa[i] <= x < xa[i+1] (the last one includes xa[n-1])
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        if (g->xa[mid] > x) hi = mid;
        else lo = mid;
    }
    const double t = x - g->xa[lo];
    return g->ya[lo] + t * (g->b[lo] + t * (g->c[lo] + t * g->d[lo]));
}

#endif
