/*
 * fftw3.h -- a small, project-written implementation of the subset of the FFTW3
 * C API (public documentation: "Complex DFTs", "Real-data DFTs", "Multi-threaded
 * FFTW") that the reference's continuum-LDOS sources call.
 *
 * TEST INFRASTRUCTURE ONLY: it lets oracle/build_ref.sh compile the reference's
 * unmodified sources into oracle/_ref/.  Semantics follow the documentation:
 * unnormalised transforms, sign -1 (FFTW_FORWARD) or +1 (FFTW_BACKWARD),
 * row-major multi-dimensional arrays, in-place allowed.  Power-of-two lengths
 * use an iterative radix-2 transform, other lengths a direct DFT.
 */
#ifndef CQPI_COMPAT_FFTW3_H
#define CQPI_COMPAT_FFTW3_H

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <complex>
#include <vector>

typedef double fftw_complex[2];
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

struct cqpi_fftw_plan_s {
    int kind; /* 0 = complex, 1 = r2c, 2 = c2r */
    int n0, n1, sign;
    void *in, *out;
};
typedef struct cqpi_fftw_plan_s *fftw_plan;

static inline void cqpi_dft1d(std::complex<double> *x, int N, int sign)
{
    std::vector<std::complex<double> > tw(N);
    for (int k = 0; k < N; k++) tw[k] = std::complex<double>(cos(2.0 * M_PI * k / N), sign * sin(2.0 * M_PI * k / N));
    if (N > 0 && (N & (N - 1)) == 0) {
        for (int i = 1, j = 0; i < N; i++) {
            int bit = N >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) std::swap(x[i], x[j]);
        }
        for (int len = 2; len <= N; len <<= 1) {
            int step = N / len;
            for (int s = 0; s < N; s += len)
                for (int k = 0; k < len / 2; k++) {
                    std::complex<double> u = x[s + k], v = x[s + k + len / 2] * tw[k * step];
                    x[s + k] = u + v;
                    x[s + k + len / 2] = u - v;
                }
        }
    } else {
        std::vector<std::complex<double> > y(N);
        for (int k = 0; k < N; k++) {
            std::complex<double> s = 0.0;
            for (int i = 0; i < N; i++) s += x[i] * tw[(int)(((long long)i * k) % N)];
            y[k] = s;
        }
        for (int k = 0; k < N; k++) x[k] = y[k];
    }
}

/* in-place 2D complex DFT of a row-major n0 x n1 array */
static inline void cqpi_dft2d(std::complex<double> *a, int n0, int n1, int sign)
{
#pragma omp parallel
    {
        std::vector<std::complex<double> > col(n0 > n1 ? n0 : n1);
#pragma omp for
        for (int r = 0; r < n0; r++) cqpi_dft1d(a + (size_t)r * n1, n1, sign);
#pragma omp for
        for (int c = 0; c < n1; c++) {
            for (int r = 0; r < n0; r++) col[r] = a[(size_t)r * n1 + c];
            cqpi_dft1d(col.data(), n0, sign);
            for (int r = 0; r < n0; r++) a[(size_t)r * n1 + c] = col[r];
        }
    }
}

static inline fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned)
{
    fftw_plan p = (fftw_plan)malloc(sizeof(struct cqpi_fftw_plan_s));
    p->kind = 0; p->n0 = n0; p->n1 = n1; p->sign = sign; p->in = in; p->out = out;
    return p;
}
static inline fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned)
{
    fftw_plan p = (fftw_plan)malloc(sizeof(struct cqpi_fftw_plan_s));
    p->kind = 1; p->n0 = n0; p->n1 = n1; p->sign = FFTW_FORWARD; p->in = in; p->out = out;
    return p;
}
static inline fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned)
{
    fftw_plan p = (fftw_plan)malloc(sizeof(struct cqpi_fftw_plan_s));
    p->kind = 2; p->n0 = n0; p->n1 = n1; p->sign = FFTW_BACKWARD; p->in = in; p->out = out;
    return p;
}

static inline void fftw_execute(const fftw_plan p)
{
    size_t n0 = (size_t)p->n0, n1 = (size_t)p->n1, nh = n1 / 2 + 1;
    if (p->kind == 0) {
        std::vector<std::complex<double> > a(n0 * n1);
        memcpy((void *)a.data(), p->in, sizeof(double) * 2 * n0 * n1);
        cqpi_dft2d(a.data(), (int)n0, (int)n1, p->sign);
        memcpy(p->out, (void *)a.data(), sizeof(double) * 2 * n0 * n1);
    } else if (p->kind == 1) {
        /* real input n0 x n1 (in-place: row stride 2*nh doubles), output n0 x nh */
        const double *in = (const double *)p->in;
        size_t rs = (p->in == p->out) ? 2 * nh : n1;
        std::vector<std::complex<double> > a(n0 * n1);
        for (size_t r = 0; r < n0; r++)
            for (size_t c = 0; c < n1; c++) a[r * n1 + c] = in[r * rs + c];
        cqpi_dft2d(a.data(), (int)n0, (int)n1, FFTW_FORWARD);
        double *out = (double *)p->out;
        for (size_t r = 0; r < n0; r++)
            for (size_t c = 0; c < nh; c++) {
                out[2 * (r * nh + c)] = a[r * n1 + c].real();
                out[2 * (r * nh + c) + 1] = a[r * n1 + c].imag();
            }
    } else {
        /* Hermitian input n0 x nh -> real output n0 x n1 */
        const double *in = (const double *)p->in;
        std::vector<std::complex<double> > a(n0 * n1);
        for (size_t r = 0; r < n0; r++)
            for (size_t c = 0; c < n1; c++) {
                if (c < nh) a[r * n1 + c] = std::complex<double>(in[2 * (r * nh + c)], in[2 * (r * nh + c) + 1]);
                else {
                    size_t rr = (n0 - r) % n0, cc = n1 - c;
                    a[r * n1 + c] = std::conj(std::complex<double>(in[2 * (rr * nh + cc)], in[2 * (rr * nh + cc) + 1]));
                }
            }
        cqpi_dft2d(a.data(), (int)n0, (int)n1, FFTW_BACKWARD);
        double *out = (double *)p->out;
        size_t rs = (p->in == p->out) ? 2 * nh : n1;
        for (size_t r = 0; r < n0; r++)
            for (size_t c = 0; c < n1; c++) out[r * rs + c] = a[r * n1 + c].real();
    }
}

static inline void fftw_destroy_plan(fftw_plan p) { free(p); }
static inline int fftw_init_threads(void) { return 1; }
static inline void fftw_plan_with_nthreads(int) {}
static inline void fftw_cleanup_threads(void) {}
static inline void fftw_cleanup(void) {}

#endif
