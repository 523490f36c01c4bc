/*
 * compat_gsl.h -- a small, project-written implementation of the subset of the
 * GSL C API (GNU Scientific Library, public documentation: "Complex Numbers",
 * "Vectors and Matrices", "Permutations", "BLAS Support", "Linear Algebra",
 * "Eigensystems") that the reference's continuum-LDOS sources call.
 *
 * TEST INFRASTRUCTURE ONLY: it exists so oracle/build_ref.sh can compile the
 * reference's unmodified src/*.cc into oracle/_ref/ (GSL itself is not
 * installed here).  No GSL source was available or used; every routine is
 * written from the documented semantics.  The Hermitian eigensolver is a cyclic
 * complex Jacobi method (any correct eigensolver yields the same Green's
 * function G0(k) = sum_n U_n U_n^H / (w - e_n + i eta) up to rounding).
 */
#ifndef CQPI_COMPAT_GSL_H
#define CQPI_COMPAT_GSL_H

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <complex>

#define GSL_MAJOR_VERSION 2
#define GSL_MINOR_VERSION 7

/* ------------------------------------------------------------- complex */
typedef struct { double dat[2]; } gsl_complex;
#define GSL_REAL(z) ((z).dat[0])
#define GSL_IMAG(z) ((z).dat[1])
#define GSL_SET_COMPLEX(zp, x, y) do { (zp)->dat[0] = (x); (zp)->dat[1] = (y); } while (0)

static inline gsl_complex gsl_complex_rect(double x, double y) { gsl_complex z; z.dat[0] = x; z.dat[1] = y; return z; }
static inline gsl_complex cqpi_from_std(std::complex<double> c) { return gsl_complex_rect(c.real(), c.imag()); }
static inline std::complex<double> cqpi_to_std(gsl_complex z) { return std::complex<double>(z.dat[0], z.dat[1]); }
#define GSL_COMPLEX_ONE (gsl_complex_rect(1.0, 0.0))
#define GSL_COMPLEX_ZERO (gsl_complex_rect(0.0, 0.0))
#define GSL_COMPLEX_NEGONE (gsl_complex_rect(-1.0, 0.0))

static inline gsl_complex gsl_complex_add(gsl_complex a, gsl_complex b) { return gsl_complex_rect(a.dat[0] + b.dat[0], a.dat[1] + b.dat[1]); }
static inline gsl_complex gsl_complex_sub(gsl_complex a, gsl_complex b) { return gsl_complex_rect(a.dat[0] - b.dat[0], a.dat[1] - b.dat[1]); }
static inline gsl_complex gsl_complex_mul(gsl_complex a, gsl_complex b)
{
    return gsl_complex_rect(a.dat[0] * b.dat[0] - a.dat[1] * b.dat[1], a.dat[0] * b.dat[1] + a.dat[1] * b.dat[0]);
}
static inline gsl_complex gsl_complex_mul_real(gsl_complex a, double x) { return gsl_complex_rect(a.dat[0] * x, a.dat[1] * x); }
static inline gsl_complex gsl_complex_sub_real(gsl_complex a, double x) { return gsl_complex_rect(a.dat[0] - x, a.dat[1]); }
static inline gsl_complex gsl_complex_conjugate(gsl_complex a) { return gsl_complex_rect(a.dat[0], -a.dat[1]); }
static inline double gsl_complex_abs2(gsl_complex a) { return a.dat[0] * a.dat[0] + a.dat[1] * a.dat[1]; }
static inline double gsl_complex_abs(gsl_complex a) { return hypot(a.dat[0], a.dat[1]); }
static inline double gsl_complex_arg(gsl_complex a) { return atan2(a.dat[1], a.dat[0]); }
static inline gsl_complex gsl_complex_inverse(gsl_complex a)
{
    double s = 1.0 / gsl_complex_abs(a);
    return gsl_complex_rect((a.dat[0] * s) * s, -(a.dat[1] * s) * s);
}
static inline gsl_complex gsl_complex_div(gsl_complex a, gsl_complex b) { return gsl_complex_mul(a, gsl_complex_inverse(b)); }
static inline gsl_complex gsl_complex_exp(gsl_complex a)
{
    double r = exp(a.dat[0]);
    return gsl_complex_rect(r * cos(a.dat[1]), r * sin(a.dat[1]));
}
static inline gsl_complex gsl_complex_sqrt(gsl_complex a) { return cqpi_from_std(std::sqrt(cqpi_to_std(a))); }
static inline gsl_complex gsl_complex_polar(double r, double th) { return gsl_complex_rect(r * cos(th), r * sin(th)); }

/* ------------------------------------------------------------- vectors */
typedef struct { size_t size, stride; double *data; void *block; int owner; } gsl_vector;
typedef struct { size_t size, stride; double *data; void *block; int owner; } gsl_vector_complex;
typedef struct { gsl_vector_complex vector; } gsl_vector_complex_view;
typedef struct { gsl_vector vector; } gsl_vector_view;

static inline gsl_vector *gsl_vector_alloc(size_t n)
{
    gsl_vector *v = (gsl_vector *)malloc(sizeof(gsl_vector));
    v->size = n; v->stride = 1; v->data = (double *)calloc(n ? n : 1, sizeof(double)); v->block = 0; v->owner = 1;
    return v;
}
static inline gsl_vector *gsl_vector_calloc(size_t n) { return gsl_vector_alloc(n); }
static inline void gsl_vector_free(gsl_vector *v) { if (!v) return; if (v->owner) free(v->data); free(v); }
static inline double gsl_vector_get(const gsl_vector *v, size_t i) { return v->data[i * v->stride]; }
static inline void gsl_vector_set(gsl_vector *v, size_t i, double x) { v->data[i * v->stride] = x; }
static inline void gsl_vector_set_zero(gsl_vector *v) { for (size_t i = 0; i < v->size; i++) v->data[i * v->stride] = 0.0; }

static inline gsl_vector_complex *gsl_vector_complex_alloc(size_t n)
{
    gsl_vector_complex *v = (gsl_vector_complex *)malloc(sizeof(gsl_vector_complex));
    v->size = n; v->stride = 1; v->data = (double *)calloc(2 * (n ? n : 1), sizeof(double)); v->block = 0; v->owner = 1;
    return v;
}
static inline void gsl_vector_complex_free(gsl_vector_complex *v) { if (!v) return; if (v->owner) free(v->data); free(v); }
static inline gsl_complex gsl_vector_complex_get(const gsl_vector_complex *v, size_t i)
{
    return gsl_complex_rect(v->data[2 * i * v->stride], v->data[2 * i * v->stride + 1]);
}
static inline void gsl_vector_complex_set(gsl_vector_complex *v, size_t i, gsl_complex z)
{
    v->data[2 * i * v->stride] = z.dat[0]; v->data[2 * i * v->stride + 1] = z.dat[1];
}
static inline void gsl_vector_complex_set_zero(gsl_vector_complex *v) { for (size_t i = 0; i < v->size; i++) gsl_vector_complex_set(v, i, GSL_COMPLEX_ZERO); }
static inline int gsl_vector_complex_memcpy(gsl_vector_complex *d, const gsl_vector_complex *s)
{
    for (size_t i = 0; i < d->size; i++) gsl_vector_complex_set(d, i, gsl_vector_complex_get(s, i));
    return 0;
}
static inline int gsl_vector_complex_scale(gsl_vector_complex *v, gsl_complex a)
{
    for (size_t i = 0; i < v->size; i++) gsl_vector_complex_set(v, i, gsl_complex_mul(gsl_vector_complex_get(v, i), a));
    return 0;
}
static inline int gsl_vector_complex_add(gsl_vector_complex *a, const gsl_vector_complex *b)
{
    for (size_t i = 0; i < a->size; i++) gsl_vector_complex_set(a, i, gsl_complex_add(gsl_vector_complex_get(a, i), gsl_vector_complex_get(b, i)));
    return 0;
}

/* ------------------------------------------------------------- matrices */
typedef struct { size_t size1, size2, tda; double *data; void *block; int owner; } gsl_matrix;
typedef struct { size_t size1, size2, tda; double *data; void *block; int owner; } gsl_matrix_complex;

static inline gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2)
{
    gsl_matrix *m = (gsl_matrix *)malloc(sizeof(gsl_matrix));
    m->size1 = n1; m->size2 = n2; m->tda = n2; m->data = (double *)calloc(n1 * n2 ? n1 * n2 : 1, sizeof(double));
    m->block = 0; m->owner = 1;
    return m;
}
static inline void gsl_matrix_free(gsl_matrix *m) { if (!m) return; if (m->owner) free(m->data); free(m); }
static inline double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j) { return m->data[i * m->tda + j]; }
static inline void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x) { m->data[i * m->tda + j] = x; }

static inline gsl_matrix_complex *gsl_matrix_complex_alloc(size_t n1, size_t n2)
{
    gsl_matrix_complex *m = (gsl_matrix_complex *)malloc(sizeof(gsl_matrix_complex));
    m->size1 = n1; m->size2 = n2; m->tda = n2; m->data = (double *)calloc(2 * (n1 * n2 ? n1 * n2 : 1), sizeof(double));
    m->block = 0; m->owner = 1;
    return m;
}
static inline gsl_matrix_complex *gsl_matrix_complex_calloc(size_t n1, size_t n2) { return gsl_matrix_complex_alloc(n1, n2); }
static inline void gsl_matrix_complex_free(gsl_matrix_complex *m) { if (!m) return; if (m->owner) free(m->data); free(m); }
static inline gsl_complex gsl_matrix_complex_get(const gsl_matrix_complex *m, size_t i, size_t j)
{
    const double *p = m->data + 2 * (i * m->tda + j);
    return gsl_complex_rect(p[0], p[1]);
}
static inline void gsl_matrix_complex_set(gsl_matrix_complex *m, size_t i, size_t j, gsl_complex z)
{
    double *p = m->data + 2 * (i * m->tda + j);
    p[0] = z.dat[0]; p[1] = z.dat[1];
}
static inline void gsl_matrix_complex_set_zero(gsl_matrix_complex *m)
{
    for (size_t i = 0; i < m->size1; i++)
        for (size_t j = 0; j < m->size2; j++) gsl_matrix_complex_set(m, i, j, GSL_COMPLEX_ZERO);
}
static inline void gsl_matrix_complex_set_identity(gsl_matrix_complex *m)
{
    for (size_t i = 0; i < m->size1; i++)
        for (size_t j = 0; j < m->size2; j++) gsl_matrix_complex_set(m, i, j, i == j ? GSL_COMPLEX_ONE : GSL_COMPLEX_ZERO);
}
static inline int gsl_matrix_complex_memcpy(gsl_matrix_complex *d, const gsl_matrix_complex *s)
{
    for (size_t i = 0; i < d->size1; i++)
        for (size_t j = 0; j < d->size2; j++) gsl_matrix_complex_set(d, i, j, gsl_matrix_complex_get(s, i, j));
    return 0;
}
static inline int gsl_matrix_complex_conjtrans_memcpy(gsl_matrix_complex *d, const gsl_matrix_complex *s)
{
    for (size_t i = 0; i < d->size1; i++)
        for (size_t j = 0; j < d->size2; j++) gsl_matrix_complex_set(d, i, j, gsl_complex_conjugate(gsl_matrix_complex_get(s, j, i)));
    return 0;
}
static inline int gsl_matrix_complex_add(gsl_matrix_complex *a, const gsl_matrix_complex *b)
{
    for (size_t i = 0; i < a->size1; i++)
        for (size_t j = 0; j < a->size2; j++) gsl_matrix_complex_set(a, i, j, gsl_complex_add(gsl_matrix_complex_get(a, i, j), gsl_matrix_complex_get(b, i, j)));
    return 0;
}
static inline int gsl_matrix_complex_sub(gsl_matrix_complex *a, const gsl_matrix_complex *b)
{
    for (size_t i = 0; i < a->size1; i++)
        for (size_t j = 0; j < a->size2; j++) gsl_matrix_complex_set(a, i, j, gsl_complex_sub(gsl_matrix_complex_get(a, i, j), gsl_matrix_complex_get(b, i, j)));
    return 0;
}
static inline int gsl_matrix_complex_scale(gsl_matrix_complex *a, gsl_complex x)
{
    for (size_t i = 0; i < a->size1; i++)
        for (size_t j = 0; j < a->size2; j++) gsl_matrix_complex_set(a, i, j, gsl_complex_mul(gsl_matrix_complex_get(a, i, j), x));
    return 0;
}
static inline gsl_vector_complex_view gsl_matrix_complex_column(gsl_matrix_complex *m, size_t j)
{
    gsl_vector_complex_view v;
    v.vector.size = m->size1; v.vector.stride = m->tda; v.vector.data = m->data + 2 * j; v.vector.block = 0; v.vector.owner = 0;
    return v;
}
static inline gsl_vector_complex_view gsl_matrix_complex_row(gsl_matrix_complex *m, size_t i)
{
    gsl_vector_complex_view v;
    v.vector.size = m->size2; v.vector.stride = 1; v.vector.data = m->data + 2 * i * m->tda; v.vector.block = 0; v.vector.owner = 0;
    return v;
}

/* ------------------------------------------------------------- permutations */
typedef struct { size_t size; size_t *data; } gsl_permutation;
static inline gsl_permutation *gsl_permutation_alloc(size_t n)
{
    gsl_permutation *p = (gsl_permutation *)malloc(sizeof(gsl_permutation));
    p->size = n; p->data = (size_t *)malloc(sizeof(size_t) * (n ? n : 1));
    for (size_t i = 0; i < n; i++) p->data[i] = i;
    return p;
}
static inline void gsl_permutation_free(gsl_permutation *p) { if (!p) return; free(p->data); free(p); }

/* ------------------------------------------------------------- BLAS */
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE_t;

static inline gsl_complex cqpi_op_get(CBLAS_TRANSPOSE_t t, const gsl_matrix_complex *m, size_t i, size_t j)
{
    if (t == CblasNoTrans) return gsl_matrix_complex_get(m, i, j);
    if (t == CblasTrans) return gsl_matrix_complex_get(m, j, i);
    return gsl_complex_conjugate(gsl_matrix_complex_get(m, j, i));
}

/* C = alpha op(A) op(B) + beta C */
static inline int gsl_blas_zgemm(CBLAS_TRANSPOSE_t ta, CBLAS_TRANSPOSE_t tb, const gsl_complex alpha,
                                 const gsl_matrix_complex *A, const gsl_matrix_complex *B, const gsl_complex beta,
                                 gsl_matrix_complex *C)
{
    size_t M = C->size1, N = C->size2, K = (ta == CblasNoTrans) ? A->size2 : A->size1;
    std::complex<double> al = cqpi_to_std(alpha), be = cqpi_to_std(beta);
    std::complex<double> *tmp = new std::complex<double>[M * N];
    for (size_t i = 0; i < M; i++)
        for (size_t j = 0; j < N; j++) {
            std::complex<double> s = 0.0;
            for (size_t k = 0; k < K; k++) s += cqpi_to_std(cqpi_op_get(ta, A, i, k)) * cqpi_to_std(cqpi_op_get(tb, B, k, j));
            tmp[i * N + j] = s;
        }
    for (size_t i = 0; i < M; i++)
        for (size_t j = 0; j < N; j++) {
            std::complex<double> c = (be == std::complex<double>(0.0, 0.0)) ? std::complex<double>(0.0, 0.0)
                                                                             : be * cqpi_to_std(gsl_matrix_complex_get(C, i, j));
            gsl_matrix_complex_set(C, i, j, cqpi_from_std(al * tmp[i * N + j] + c));
        }
    delete[] tmp;
    return 0;
}

/* y = alpha op(A) x + beta y */
static inline int gsl_blas_zgemv(CBLAS_TRANSPOSE_t ta, const gsl_complex alpha, const gsl_matrix_complex *A,
                                 const gsl_vector_complex *x, const gsl_complex beta, gsl_vector_complex *y)
{
    size_t M = (ta == CblasNoTrans) ? A->size1 : A->size2, K = (ta == CblasNoTrans) ? A->size2 : A->size1;
    std::complex<double> al = cqpi_to_std(alpha), be = cqpi_to_std(beta);
    std::complex<double> *tmp = new std::complex<double>[M];
    for (size_t i = 0; i < M; i++) {
        std::complex<double> s = 0.0;
        for (size_t k = 0; k < K; k++) s += cqpi_to_std(cqpi_op_get(ta, A, i, k)) * cqpi_to_std(gsl_vector_complex_get(x, k));
        tmp[i] = s;
    }
    for (size_t i = 0; i < M; i++) {
        std::complex<double> c = (be == std::complex<double>(0.0, 0.0)) ? std::complex<double>(0.0, 0.0)
                                                                         : be * cqpi_to_std(gsl_vector_complex_get(y, i));
        gsl_vector_complex_set(y, i, cqpi_from_std(al * tmp[i] + c));
    }
    delete[] tmp;
    return 0;
}

/* dotc = x^H y */
static inline int gsl_blas_zdotc(const gsl_vector_complex *x, const gsl_vector_complex *y, gsl_complex *dotc)
{
    std::complex<double> s = 0.0;
    for (size_t i = 0; i < x->size; i++) s += std::conj(cqpi_to_std(gsl_vector_complex_get(x, i))) * cqpi_to_std(gsl_vector_complex_get(y, i));
    *dotc = cqpi_from_std(s);
    return 0;
}

/* A = alpha x y^H + A */
static inline int gsl_blas_zgerc(const gsl_complex alpha, const gsl_vector_complex *x, const gsl_vector_complex *y,
                                 gsl_matrix_complex *A)
{
    std::complex<double> al = cqpi_to_std(alpha);
    for (size_t i = 0; i < A->size1; i++) {
        std::complex<double> xi = al * cqpi_to_std(gsl_vector_complex_get(x, i));
        for (size_t j = 0; j < A->size2; j++)
            gsl_matrix_complex_set(A, i, j, cqpi_from_std(cqpi_to_std(gsl_matrix_complex_get(A, i, j)) +
                                                          xi * std::conj(cqpi_to_std(gsl_vector_complex_get(y, j)))));
    }
    return 0;
}

/* ------------------------------------------------------------- LU */
static inline int gsl_linalg_complex_LU_decomp(gsl_matrix_complex *A, gsl_permutation *p, int *signum)
{
    size_t n = A->size1;
    *signum = 1;
    for (size_t i = 0; i < n; i++) p->data[i] = i;
    for (size_t j = 0; j < n; j++) {
        size_t piv = j; double best = gsl_complex_abs(gsl_matrix_complex_get(A, j, j));
        for (size_t i = j + 1; i < n; i++) {
            double a = gsl_complex_abs(gsl_matrix_complex_get(A, i, j));
            if (a > best) { best = a; piv = i; }
        }
        if (piv != j) {
            for (size_t k = 0; k < n; k++) {
                gsl_complex t = gsl_matrix_complex_get(A, j, k);
                gsl_matrix_complex_set(A, j, k, gsl_matrix_complex_get(A, piv, k));
                gsl_matrix_complex_set(A, piv, k, t);
            }
            size_t t = p->data[j]; p->data[j] = p->data[piv]; p->data[piv] = t;
            *signum = -*signum;
        }
        std::complex<double> d = cqpi_to_std(gsl_matrix_complex_get(A, j, j));
        if (d != std::complex<double>(0.0, 0.0))
            for (size_t i = j + 1; i < n; i++) {
                std::complex<double> l = cqpi_to_std(gsl_matrix_complex_get(A, i, j)) / d;
                gsl_matrix_complex_set(A, i, j, cqpi_from_std(l));
                for (size_t k = j + 1; k < n; k++)
                    gsl_matrix_complex_set(A, i, k, cqpi_from_std(cqpi_to_std(gsl_matrix_complex_get(A, i, k)) -
                                                                  l * cqpi_to_std(gsl_matrix_complex_get(A, j, k))));
            }
    }
    return 0;
}

static inline int gsl_linalg_complex_LU_invert(const gsl_matrix_complex *LU, const gsl_permutation *p, gsl_matrix_complex *inv)
{
    size_t n = LU->size1;
    std::complex<double> *col = new std::complex<double>[n];
    for (size_t c = 0; c < n; c++) {
        /* solve LU x = P e_c */
        for (size_t i = 0; i < n; i++) col[i] = (p->data[i] == c) ? 1.0 : 0.0;
        for (size_t i = 0; i < n; i++)
            for (size_t k = 0; k < i; k++) col[i] -= cqpi_to_std(gsl_matrix_complex_get(LU, i, k)) * col[k];
        for (size_t ii = n; ii-- > 0;) {
            for (size_t k = ii + 1; k < n; k++) col[ii] -= cqpi_to_std(gsl_matrix_complex_get(LU, ii, k)) * col[k];
            col[ii] /= cqpi_to_std(gsl_matrix_complex_get(LU, ii, ii));
        }
        for (size_t i = 0; i < n; i++) gsl_matrix_complex_set(inv, i, c, cqpi_from_std(col[i]));
    }
    delete[] col;
    return 0;
}

static inline int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum)
{
    size_t n = A->size1;
    *signum = 1;
    for (size_t i = 0; i < n; i++) p->data[i] = i;
    for (size_t j = 0; j < n; j++) {
        size_t piv = j; double best = fabs(gsl_matrix_get(A, j, j));
        for (size_t i = j + 1; i < n; i++)
            if (fabs(gsl_matrix_get(A, i, j)) > best) { best = fabs(gsl_matrix_get(A, i, j)); piv = i; }
        if (piv != j) {
            for (size_t k = 0; k < n; k++) {
                double t = gsl_matrix_get(A, j, k);
                gsl_matrix_set(A, j, k, gsl_matrix_get(A, piv, k));
                gsl_matrix_set(A, piv, k, t);
            }
            size_t t = p->data[j]; p->data[j] = p->data[piv]; p->data[piv] = t;
            *signum = -*signum;
        }
        double d = gsl_matrix_get(A, j, j);
        if (d != 0.0)
            for (size_t i = j + 1; i < n; i++) {
                double l = gsl_matrix_get(A, i, j) / d;
                gsl_matrix_set(A, i, j, l);
                for (size_t k = j + 1; k < n; k++) gsl_matrix_set(A, i, k, gsl_matrix_get(A, i, k) - l * gsl_matrix_get(A, j, k));
            }
    }
    return 0;
}

static inline int gsl_linalg_LU_solve(const gsl_matrix *LU, const gsl_permutation *p, const gsl_vector *b, gsl_vector *x)
{
    size_t n = LU->size1;
    for (size_t i = 0; i < n; i++) gsl_vector_set(x, i, gsl_vector_get(b, p->data[i]));
    for (size_t i = 0; i < n; i++)
        for (size_t k = 0; k < i; k++) gsl_vector_set(x, i, gsl_vector_get(x, i) - gsl_matrix_get(LU, i, k) * gsl_vector_get(x, k));
    for (size_t ii = n; ii-- > 0;) {
        double s = gsl_vector_get(x, ii);
        for (size_t k = ii + 1; k < n; k++) s -= gsl_matrix_get(LU, ii, k) * gsl_vector_get(x, k);
        gsl_vector_set(x, ii, s / gsl_matrix_get(LU, ii, ii));
    }
    return 0;
}

/* ------------------------------------------------------------- Hermitian eigensystem */
typedef struct { size_t size; } gsl_eigen_hermv_workspace;
typedef enum { GSL_EIGEN_SORT_VAL_ASC, GSL_EIGEN_SORT_VAL_DESC, GSL_EIGEN_SORT_ABS_ASC, GSL_EIGEN_SORT_ABS_DESC } gsl_eigen_sort_t;

static inline gsl_eigen_hermv_workspace *gsl_eigen_hermv_alloc(size_t n)
{
    gsl_eigen_hermv_workspace *w = (gsl_eigen_hermv_workspace *)malloc(sizeof(gsl_eigen_hermv_workspace));
    w->size = n;
    return w;
}
static inline void gsl_eigen_hermv_free(gsl_eigen_hermv_workspace *w) { free(w); }

/* Cyclic complex Jacobi: A is destroyed (as in GSL), evec gets eigenvectors in columns. */
static inline int gsl_eigen_hermv(gsl_matrix_complex *Am, gsl_vector *eval, gsl_matrix_complex *evec, gsl_eigen_hermv_workspace *)
{
    size_t b = Am->size1;
    std::complex<double> *A = new std::complex<double>[b * b], *V = new std::complex<double>[b * b];
    for (size_t i = 0; i < b; i++)
        for (size_t j = 0; j < b; j++) {
            A[i * b + j] = cqpi_to_std(gsl_matrix_complex_get(Am, i, j));
            V[i * b + j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, diag = 0.0;
        for (size_t p = 0; p < b; p++)
            for (size_t q = 0; q < b; q++) (p == q ? diag : off) += std::norm(A[p * b + q]);
        if (off == 0.0 || off <= 1e-32 * diag) break;
        for (size_t p = 0; p + 1 < b; p++)
            for (size_t q = p + 1; q < b; q++) {
                double c = std::abs(A[p * b + q]);
                if (c == 0.0) continue;
                std::complex<double> e = A[p * b + q] / c;
                double tau = (A[q * b + q].real() - A[p * b + p].real()) / (2.0 * c);
                double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                double cs = 1.0 / sqrt(1.0 + t * t), sn = t * cs;
                for (size_t r = 0; r < b; r++) {
                    std::complex<double> xp = A[r * b + p], xq = A[r * b + q] * std::conj(e);
                    A[r * b + p] = cs * xp - sn * xq; A[r * b + q] = sn * xp + cs * xq;
                    std::complex<double> vp = V[r * b + p], vq = V[r * b + q] * std::conj(e);
                    V[r * b + p] = cs * vp - sn * vq; V[r * b + q] = sn * vp + cs * vq;
                }
                for (size_t k = 0; k < b; k++) {
                    std::complex<double> xp = A[p * b + k], xq = A[q * b + k] * e;
                    A[p * b + k] = cs * xp - sn * xq; A[q * b + k] = sn * xp + cs * xq;
                }
                A[p * b + q] = A[q * b + p] = 0.0;
                A[p * b + p] = A[p * b + p].real(); A[q * b + q] = A[q * b + q].real();
            }
    }
    for (size_t i = 0; i < b; i++) {
        gsl_vector_set(eval, i, A[i * b + i].real());
        for (size_t j = 0; j < b; j++) gsl_matrix_complex_set(evec, i, j, cqpi_from_std(V[i * b + j]));
    }
    delete[] A; delete[] V;
    return 0;
}

static inline int gsl_eigen_hermv_sort(gsl_vector *eval, gsl_matrix_complex *evec, gsl_eigen_sort_t t)
{
    size_t n = eval->size;
    for (size_t i = 0; i < n; i++) {
        size_t k = i;
        for (size_t j = i + 1; j < n; j++) {
            double a = gsl_vector_get(eval, j), c = gsl_vector_get(eval, k);
            bool better = false;
            switch (t) {
            case GSL_EIGEN_SORT_VAL_ASC: better = a < c; break;
            case GSL_EIGEN_SORT_VAL_DESC: better = a > c; break;
            case GSL_EIGEN_SORT_ABS_ASC: better = fabs(a) < fabs(c); break;
            case GSL_EIGEN_SORT_ABS_DESC: better = fabs(a) > fabs(c); break;
            }
            if (better) k = j;
        }
        if (k != i) {
            double tv = gsl_vector_get(eval, i); gsl_vector_set(eval, i, gsl_vector_get(eval, k)); gsl_vector_set(eval, k, tv);
            for (size_t r = 0; r < evec->size1; r++) {
                gsl_complex z = gsl_matrix_complex_get(evec, r, i);
                gsl_matrix_complex_set(evec, r, i, gsl_matrix_complex_get(evec, r, k));
                gsl_matrix_complex_set(evec, r, k, z);
            }
        }
    }
    return 0;
}

#endif
