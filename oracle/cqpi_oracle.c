/*
 * cqpi_oracle.c -- CPU restatement of the CalcQPI continuum-LDOS path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference arm of
 * bench.py may load it, as the checker or as the timed CPU baseline.  No
 * product code links it or calls it.
 *
 * Parity pin: the functions below are checked against golden outputs of the
 * reference's own sources (oracle/build_ref.sh builds them against a
 * project-written GSL/FFTW API subset, tests/golden/make_golden.py records
 * the outputs as fixtures).
 *
 * Every function restates one step of the reference, cited by file:line
 * (paths within gpwahl/calcqpi-release).  Complex numbers are interleaved
 * (re, im) doubles.  Array conventions shared with the engine:
 *   hoppings   R[h][3] int32, orb[h][2] int32 (0-based), t[h][2], anti[h]
 *   k index    ik = i*kp + j, i = x index, j = y index   (qpi.cc:457-468)
 *   eigen      eval[ik][b], evec[ik][o][n] = component o of eigenvector n
 *   G0 grids   g0[X][Y][o][a] (b x b row-major per point)
 *   orbitals   wf[o][ix][iy], side = (2w+1)*os           (wannierfunctions.cc:433-442)
 *   LDOS       ldos[x][y], x = i*os+ii  (the reference's tmatrix::ldos)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RE(p, i) ((p)[2 * (i)])
#define IM(p, i) ((p)[2 * (i) + 1])

/* ---- H(k):  tightbinding.cc:210-219, hoppingterm::addhop tightbinding.h:128-135 ---- */
void orc_hk(int b, int64_t nhops, const int32_t *R, const int32_t *orb,
            const double *t, const uint8_t *anti, double efermi, int scmax,
            double kx, double ky, double *H)
{
    memset(H, 0, sizeof(double) * 2 * b * b);
    for (int i = 0; i < b; i++) RE(H, i * b + i) = (i < scmax) ? -efermi : efermi;
    for (int64_t h = 0; h < nhops; h++) {
        /* kz = 0 in the 2D k-grid (qpi.cc:465-468: kvector[2] stays 0) */
        double ph = 2.0 * M_PI * (R[3 * h] * kx + R[3 * h + 1] * ky + R[3 * h + 2] * 0.0);
        if (anti[h]) ph = -ph;
        double c = cos(ph), s = sin(ph);
        double tr = t[2 * h], ti = t[2 * h + 1];
        int e = orb[2 * h] * b + orb[2 * h + 1];
        RE(H, e) += tr * c - ti * s;
        IM(H, e) += tr * s + ti * c;
    }
}

/* ---- Hermitian eigen-solve (gsl_eigen_hermv stand-in, qpi.cc:470) ----
 * Cyclic complex Jacobi.  G0(k) is invariant under eigenvector phase and
 * ordering, so any correct Hermitian eigensolver gives the same G0 to
 * rounding.  A is overwritten; V receives eigenvectors as columns. */
void orc_hermitian_jacobi(int b, double *A, double *V, double *ev)
{
    memset(V, 0, sizeof(double) * 2 * b * b);
    for (int i = 0; i < b; i++) RE(V, i * b + i) = 1.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < b; p++)
            for (int q = 0; q < b; q++) {
                double a2 = RE(A, p * b + q) * RE(A, p * b + q) + IM(A, p * b + q) * IM(A, p * b + q);
                if (p == q) diag += a2; else off += a2;
            }
        if (off <= 1e-32 * diag || off == 0.0) break;
        for (int p = 0; p < b - 1; p++)
            for (int q = p + 1; q < b; q++) {
                double apr = RE(A, p * b + q), api = IM(A, p * b + q);
                double c_abs = hypot(apr, api);
                if (c_abs == 0.0) continue;
                double app = RE(A, p * b + p), aqq = RE(A, q * b + q);
                /* e^{i alpha} = A_pq / |A_pq| */
                double er = apr / c_abs, ei = api / c_abs;
                double tau = (aqq - app) / (2.0 * c_abs);
                double tt = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                double cs = 1.0 / sqrt(1.0 + tt * tt), sn = tt * cs;
                /* G = [[cs, sn], [-sn e^{-ia}, cs e^{-ia}]] ; A <- G^H A G ; V <- V G */
                for (int r = 0; r < b; r++) {       /* columns: X = A G */
                    double xpr = RE(A, r * b + p), xpi = IM(A, r * b + p);
                    double xqr = RE(A, r * b + q), xqi = IM(A, r * b + q);
                    /* xq * e^{-ia} */
                    double yr = xqr * er + xqi * ei, yi = xqi * er - xqr * ei;
                    RE(A, r * b + p) = cs * xpr - sn * yr;  IM(A, r * b + p) = cs * xpi - sn * yi;
                    RE(A, r * b + q) = sn * xpr + cs * yr;  IM(A, r * b + q) = sn * xpi + cs * yi;
                    double vpr = RE(V, r * b + p), vpi = IM(V, r * b + p);
                    double vqr = RE(V, r * b + q), vqi = IM(V, r * b + q);
                    double wr = vqr * er + vqi * ei, wi = vqi * er - vqr * ei;
                    RE(V, r * b + p) = cs * vpr - sn * wr;  IM(V, r * b + p) = cs * vpi - sn * wi;
                    RE(V, r * b + q) = sn * vpr + cs * wr;  IM(V, r * b + q) = sn * vpi + cs * wi;
                }
                for (int cidx = 0; cidx < b; cidx++) { /* rows: A <- G^H X */
                    double xpr = RE(A, p * b + cidx), xpi = IM(A, p * b + cidx);
                    double xqr = RE(A, q * b + cidx), xqi = IM(A, q * b + cidx);
                    /* xq * e^{+ia} */
                    double yr = xqr * er - xqi * ei, yi = xqi * er + xqr * ei;
                    RE(A, p * b + cidx) = cs * xpr - sn * yr;  IM(A, p * b + cidx) = cs * xpi - sn * yi;
                    RE(A, q * b + cidx) = sn * xpr + cs * yr;  IM(A, q * b + cidx) = sn * xpi + cs * yi;
                }
                RE(A, p * b + q) = IM(A, p * b + q) = 0.0;
                RE(A, q * b + p) = IM(A, q * b + p) = 0.0;
                IM(A, p * b + p) = 0.0;
                IM(A, q * b + q) = 0.0;
            }
    }
    for (int i = 0; i < b; i++) ev[i] = RE(A, i * b + i);
}

/* ---- tmatrix::calchamiltonian, qpi.cc:454-475 (non-MPI form 457-475) ---- */
void orc_bands(int b, int64_t nhops, const int32_t *R, const int32_t *orb,
               const double *t, const uint8_t *anti, double efermi, int scmax,
               int kp, double *eval, double *evec)
{
    size_t cut = (size_t)(kp >> 1);
#pragma omp parallel
    {
        double *H = (double *)malloc(sizeof(double) * 2 * b * b);
#pragma omp for schedule(static)
        for (int i = 0; i < kp; i++)
            for (int j = 0; j < kp; j++) {
                double x = ((size_t)i > cut) ? ((double)i - kp) / kp : ((double)i / kp);
                double y = ((size_t)j > cut) ? ((double)j - kp) / kp : ((double)j / kp);
                size_t ik = (size_t)i * kp + j;
                orc_hk(b, nhops, R, orb, t, anti, efermi, scmax, x, y, H);
                orc_hermitian_jacobi(b, H, evec + ik * 2 * b * b, eval + ik * b);
            }
        free(H);
    }
}

/* ---- G0(k) = sum_n U_n U_n^H / (omega - e_n + i eta)
 *      tightbinding.cc:282-289 (gsl_blas_zgerc), loop qpi.cc:478-486 ---- */
void orc_greens_k(int b, int kp, const double *eval, const double *evec,
                  double omega, double eta, double *g0)
{
    size_t nk = (size_t)kp * kp;
#pragma omp parallel for schedule(static)
    for (long long ik = 0; ik < (long long)nk; ik++) {
        const double *U = evec + (size_t)ik * 2 * b * b;
        double *G = g0 + (size_t)ik * 2 * b * b;
        memset(G, 0, sizeof(double) * 2 * b * b);
        for (int n = 0; n < b; n++) {
            /* factor = 1 / (omega - e_n + i eta)  (gsl_complex_inverse) */
            double dr = omega - eval[(size_t)ik * b + n], di = eta;
            double den = dr * dr + di * di;
            double fr = dr / den, fi = -di / den;
            for (int o = 0; o < b; o++) {
                double ur = RE(U, o * b + n), ui = IM(U, o * b + n);
                double xr = fr * ur - fi * ui, xi = fr * ui + fi * ur;
                for (int a = 0; a < b; a++) {
                    /* conj(U[a][n]) */
                    double vr = RE(U, a * b + n), vi = -IM(U, a * b + n);
                    RE(G, o * b + a) += xr * vr - xi * vi;
                    IM(G, o * b + a) += xr * vi + xi * vr;
                }
            }
        }
    }
}

/* ---- 1D DFT with sign +1 (FFTW_BACKWARD), unnormalised ---- */
static void dft_backward_1d(int N, double *x, int stride, double *tmp, const double *tw)
{
    /* tw[2k] = cos(2 pi k / N), tw[2k+1] = sin(2 pi k / N) */
    for (int i = 0; i < N; i++) { tmp[2 * i] = x[2 * (size_t)i * stride]; tmp[2 * i + 1] = x[2 * (size_t)i * stride + 1]; }
    if ((N & (N - 1)) == 0) {
        /* iterative radix-2, bit-reversed input */
        for (int i = 1, j = 0; i < N; i++) {
            int bit = N >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) {
                double a = tmp[2 * i], c = tmp[2 * i + 1];
                tmp[2 * i] = tmp[2 * j]; tmp[2 * i + 1] = tmp[2 * j + 1];
                tmp[2 * j] = a; tmp[2 * j + 1] = c;
            }
        }
        for (int len = 2; len <= N; len <<= 1) {
            int step = N / len;
            for (int s = 0; s < N; s += len)
                for (int k = 0; k < len / 2; k++) {
                    double wr = tw[2 * (k * step)], wi = tw[2 * (k * step) + 1];
                    double *u = tmp + 2 * (s + k), *v = tmp + 2 * (s + k + len / 2);
                    double vr = v[0] * wr - v[1] * wi, vi = v[0] * wi + v[1] * wr;
                    v[0] = u[0] - vr; v[1] = u[1] - vi;
                    u[0] += vr; u[1] += vi;
                }
        }
        for (int i = 0; i < N; i++) { x[2 * (size_t)i * stride] = tmp[2 * i]; x[2 * (size_t)i * stride + 1] = tmp[2 * i + 1]; }
    } else {
        for (int k = 0; k < N; k++) {
            double sr = 0.0, si = 0.0;
            for (int i = 0; i < N; i++) {
                int idx = (int)(((long long)i * k) % N);
                double wr = tw[2 * idx], wi = tw[2 * idx + 1];
                sr += tmp[2 * i] * wr - tmp[2 * i + 1] * wi;
                si += tmp[2 * i] * wi + tmp[2 * i + 1] * wr;
            }
            x[2 * (size_t)k * stride] = sr; x[2 * (size_t)k * stride + 1] = si;
        }
    }
}

/* ---- tmatrix::calcrealspacegreensfunction, qpi.cc:557-578 ----
 * For each orbital pair: divide by kp^2, 2D backward DFT (plan qpi.h:105),
 * in place.  g0 holds G0(k) on entry and G0(R) on exit, [X][Y][o][a]. */
void orc_fft_backward_2d(int kp, int b, double *g0)
{
    double *tw = (double *)malloc(sizeof(double) * 2 * kp);
    for (int k = 0; k < kp; k++) { tw[2 * k] = cos(2.0 * M_PI * k / kp); tw[2 * k + 1] = sin(2.0 * M_PI * k / kp); }
    double norm = (double)kp * kp;
    size_t nk = (size_t)kp * kp, bb = (size_t)b * b;
    for (size_t e = 0; e < bb; e++) {
#pragma omp parallel for schedule(static)
        for (long long ik = 0; ik < (long long)nk; ik++) {
            g0[2 * (ik * bb + e)] /= norm;
            g0[2 * (ik * bb + e) + 1] /= norm;
        }
#pragma omp parallel
        {
            double *tmp = (double *)malloc(sizeof(double) * 2 * kp);
#pragma omp for schedule(static)
            for (int i = 0; i < kp; i++)      /* transform along Y for each X */
                dft_backward_1d(kp, g0 + 2 * ((size_t)i * kp * bb + e), (int)bb, tmp, tw);
#pragma omp for schedule(static)
            for (int j = 0; j < kp; j++)      /* transform along X for each Y */
                dft_backward_1d(kp, g0 + 2 * ((size_t)j * bb + e), (int)(kp * bb), tmp, tw);
            free(tmp);
        }
    }
    free(tw);
}

/* ---- tmatrix::setscatteringmatrix, qpi.cc:833-854 ----
 * T = (1 - V G0(R=0))^{-1} V with V = diag(vscat).  LU with partial
 * pivoting on |.| (gsl_linalg_complex_LU_decomp) then invert. */
int orc_tmatrix(int b, const double *vscat, const double *g00, double *T)
{
    double *M = (double *)calloc(2 * b * b, sizeof(double));
    double *inv = (double *)calloc(2 * b * b, sizeof(double));
    for (int i = 0; i < b; i++)
        for (int j = 0; j < b; j++) {
            /* (V G0)_{ij} = v_i G0_{ij} */
            double vr = vscat[2 * i], vi = vscat[2 * i + 1];
            double gr = RE(g00, i * b + j), gi = IM(g00, i * b + j);
            RE(M, i * b + j) = (i == j ? 1.0 : 0.0) - (vr * gr - vi * gi);
            IM(M, i * b + j) = -(vr * gi + vi * gr);
        }
    for (int i = 0; i < b; i++) RE(inv, i * b + i) = 1.0;
    int rc = 0;
    for (int c = 0; c < b; c++) {
        int piv = c; double best = -1.0;
        for (int r = c; r < b; r++) {
            double a = hypot(RE(M, r * b + c), IM(M, r * b + c));
            if (a > best) { best = a; piv = r; }
        }
        if (best == 0.0) { rc = -1; break; }
        if (piv != c)
            for (int k = 0; k < b; k++) {
                double t0 = RE(M, c * b + k), t1 = IM(M, c * b + k);
                RE(M, c * b + k) = RE(M, piv * b + k); IM(M, c * b + k) = IM(M, piv * b + k);
                RE(M, piv * b + k) = t0; IM(M, piv * b + k) = t1;
                t0 = RE(inv, c * b + k); t1 = IM(inv, c * b + k);
                RE(inv, c * b + k) = RE(inv, piv * b + k); IM(inv, c * b + k) = IM(inv, piv * b + k);
                RE(inv, piv * b + k) = t0; IM(inv, piv * b + k) = t1;
            }
        double pr = RE(M, c * b + c), pi = IM(M, c * b + c), pd = pr * pr + pi * pi;
        for (int r = 0; r < b; r++) {
            if (r == c) continue;
            double mr = RE(M, r * b + c), mi = IM(M, r * b + c);
            double fr = (mr * pr + mi * pi) / pd, fi = (mi * pr - mr * pi) / pd;
            for (int k = 0; k < b; k++) {
                double xr = RE(M, c * b + k), xi = IM(M, c * b + k);
                RE(M, r * b + k) -= fr * xr - fi * xi; IM(M, r * b + k) -= fr * xi + fi * xr;
                xr = RE(inv, c * b + k); xi = IM(inv, c * b + k);
                RE(inv, r * b + k) -= fr * xr - fi * xi; IM(inv, r * b + k) -= fr * xi + fi * xr;
            }
        }
    }
    if (rc == 0)
        for (int r = 0; r < b; r++) {
            double pr = RE(M, r * b + r), pi = IM(M, r * b + r), pd = pr * pr + pi * pi;
            for (int k = 0; k < b; k++) {
                double xr = RE(inv, r * b + k), xi = IM(inv, r * b + k);
                RE(inv, r * b + k) = (xr * pr + xi * pi) / pd;
                IM(inv, r * b + k) = (xi * pr - xr * pi) / pd;
            }
        }
    /* T = inv * V : column j scaled by v_j */
    for (int i = 0; i < b; i++)
        for (int j = 0; j < b; j++) {
            double xr = RE(inv, i * b + j), xi = IM(inv, i * b + j);
            double vr = vscat[2 * j], vi = vscat[2 * j + 1];
            RE(T, i * b + j) = xr * vr - xi * vi;
            IM(T, i * b + j) = xr * vi + xi * vr;
        }
    free(M); free(inv);
    return rc;
}

static void zmul(int b, const double *A, const double *B, double *C)
{
    for (int i = 0; i < b; i++)
        for (int j = 0; j < b; j++) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < b; k++) {
                double ar = RE(A, i * b + k), ai = IM(A, i * b + k);
                double br = RE(B, k * b + j), bi = IM(B, k * b + j);
                sr += ar * br - ai * bi; si += ar * bi + ai * br;
            }
            RE(C, i * b + j) = sr; IM(C, i * b + j) = si;
        }
}

/* ---- tmatrix::calcwannierldos (CPU), qpi.cc:876-950 ----
 * Direct form of the reference: per site, W products T*G0(-(p+d1)) and W^2
 * products G0(p+d2)*buffer, then the sub-pixel / orbital accumulation.
 * The G0 index formulas keep the reference's unsigned arithmetic
 * (size_t kpoints + int offsets, qpi.cc:901,907,921).
 * Rows [row_begin, row_end) of sites i are computed (all when row_end<=0);
 * ldos[x][y] for those rows is overwritten. */
void orc_wannier_ldos(int n, int kp, int b, int os, int w, int m, int spin,
                      const double *T, const double *g0r, const double *wf,
                      const uint8_t *wf_zero, double *ldos, int row_begin, int row_end)
{
    size_t wn = (size_t)os * n, side = (size_t)(2 * w + 1) * os, bb = (size_t)b * b;
    size_t kpoints = (size_t)kp, n2 = (size_t)(n >> 1), spinbands = (size_t)(m >> 1);
    if (row_end <= 0 || row_end > n) row_end = n;
    for (int i = row_begin; i < row_end; i++)
        for (size_t ii = 0; ii < (size_t)os; ii++)
            for (size_t y = 0; y < wn; y++) ldos[((size_t)i * os + ii) * wn + y] = 0.0;
#define G0AT(X, Y) (g0r + 2 * (((size_t)(X) * kpoints + (size_t)(Y)) * bb))
#define WF(o, X, Y) (wf[((size_t)(o) * side + (size_t)(X)) * side + (size_t)(Y)])
#pragma omp parallel
    {
        double *buffer = (double *)malloc(sizeof(double) * 2 * bb);
        double *cldos = (double *)malloc(sizeof(double) * 2 * bb);
#pragma omp for collapse(2) schedule(dynamic, 4)
        for (int i = row_begin; i < row_end; i++)
            for (int j = 0; j < n; j++) {
                int ipos = i - (int)n2, jpos = j - (int)n2;
                for (int nni1 = -w; nni1 <= w; nni1++)
                    for (int nnj1 = -w; nnj1 <= w; nnj1++) {
                        zmul(b, T, G0AT((kpoints + kpoints - (size_t)(ipos + nni1)) % kpoints,
                                        (kpoints + kpoints - (size_t)(jpos + nnj1)) % kpoints), buffer);
                        for (int nni2 = -w; nni2 <= w; nni2++)
                            for (int nnj2 = -w; nnj2 <= w; nnj2++) {
                                zmul(b, G0AT((kpoints + (size_t)(ipos + nni2)) % kpoints,
                                             (kpoints + (size_t)(jpos + nnj2)) % kpoints), buffer, cldos);
                                const double *gd = G0AT((kpoints - (size_t)nni1 + (size_t)nni2) % kpoints,
                                                        (kpoints - (size_t)nnj1 + (size_t)nnj2) % kpoints);
                                for (size_t ii = 0; ii < (size_t)os; ii++)
                                    for (size_t jj = 0; jj < (size_t)os; jj++) {
                                        size_t x = ii + (size_t)w * os, y = jj + (size_t)w * os;
                                        size_t x1 = x - (size_t)((long)nni1 * os), y1 = y - (size_t)((long)nnj1 * os);
                                        size_t x2 = x - (size_t)((long)nni2 * os), y2 = y - (size_t)((long)nnj2 * os);
                                        double *out = &ldos[((size_t)i * os + ii) % wn * wn + ((size_t)j * os + jj) % wn];
                                        if (!spin) {
                                            for (size_t o1 = 0; o1 < (size_t)m; o1++) {
                                                if (wf_zero[o1]) continue;
                                                for (size_t o2 = 0; o2 < (size_t)m; o2++) {
                                                    if (wf_zero[o2]) continue;
                                                    double f = WF(o1, x1, y1) * WF(o2, x2, y2);
                                                    *out -= IM(cldos, o2 * b + o1) * f;
                                                    *out -= IM(gd, o2 * b + o1) * f;
                                                }
                                            }
                                        } else {
                                            for (size_t o1 = 0; o1 < spinbands; o1++) {
                                                if (!wf_zero[o1])
                                                    for (size_t o2 = 0; o2 < spinbands; o2++) {
                                                        if (wf_zero[o2]) continue;
                                                        double f = WF(o1, x1, y1) * WF(o2, x2, y2);
                                                        *out -= IM(cldos, o2 * b + o1) * f;
                                                        *out -= IM(gd, o2 * b + o1) * f;
                                                    }
                                                size_t s1 = spinbands + o1;
                                                if (!wf_zero[s1])
                                                    for (size_t o2 = 0; o2 < spinbands; o2++) {
                                                        size_t s2 = spinbands + o2;
                                                        if (wf_zero[s2]) continue;
                                                        double f = WF(s1, x1, y1) * WF(s2, x2, y2);
                                                        *out -= IM(cldos, s2 * b + s1) * f;
                                                        *out -= IM(gd, s2 * b + s1) * f;
                                                    }
                                            }
                                        }
                                    }
                            }
                    }
            }
        free(buffer); free(cldos);
    }
#undef G0AT
#undef WF
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int nt)
{
#ifdef _OPENMP
    if (nt > 0) omp_set_num_threads(nt);
#else
    (void)nt;
#endif
}

/* ---- tmatrix::calcwannierjosephson (CPU), qpi.cc:953-1033 ----
 * The same double window sum as orc_wannier_ldos with three differences of the
 * reference's Josephson mode: the orbital count is the particle block bands>>1
 * (qpi.cc:956), the column of cldos and G0 is shifted into the hole block
 * (o1 + maxband, qpi.cc:986-987,1000-1001,1009-1010), and the sum of the two
 * terms is multiplied by the tip factor before its imaginary part is taken
 * (qpi.cc:988-989).  tip = (tip_re, tip_im) is the driver's per-energy factor
 * (orc_josephson_tip, calcqpi.cc:706-708). */
void orc_wannier_josephson(int n, int kp, int b, int os, int w, int spin,
                           const double *T, const double *g0r, const double *wf,
                           const uint8_t *wf_zero, double tip_re, double tip_im, double *ldos,
                           int row_begin, int row_end)
{
    size_t wn = (size_t)os * n, side = (size_t)(2 * w + 1) * os, bb = (size_t)b * b;
    size_t kpoints = (size_t)kp, n2 = (size_t)(n >> 1);
    size_t maxband = (size_t)(b >> 1), spinbands = maxband >> 1;
    if (row_end <= 0 || row_end > n) row_end = n;
    for (int i = row_begin; i < row_end; i++)
        for (size_t ii = 0; ii < (size_t)os; ii++)
            for (size_t y = 0; y < wn; y++) ldos[((size_t)i * os + ii) * wn + y] = 0.0;
#define G0AT(X, Y) (g0r + 2 * (((size_t)(X) * kpoints + (size_t)(Y)) * bb))
#define WF(o, X, Y) (wf[((size_t)(o) * side + (size_t)(X)) * side + (size_t)(Y)])
/* ldos -= Im(tip * (cldos + g0)[r][c]) * f */
#define JACC(r, c, f)                                                                       \
    do {                                                                                    \
        double vr = RE(cldos, (r) * b + (c)) + RE(gd, (r) * b + (c));                       \
        double vi = IM(cldos, (r) * b + (c)) + IM(gd, (r) * b + (c));                       \
        *out -= (vr * tip_im + vi * tip_re) * (f);                                          \
    } while (0)
#pragma omp parallel
    {
        double *buffer = (double *)malloc(sizeof(double) * 2 * bb);
        double *cldos = (double *)malloc(sizeof(double) * 2 * bb);
#pragma omp for collapse(2) schedule(dynamic, 4)
        for (int i = row_begin; i < row_end; i++)
            for (int j = 0; j < n; j++) {
                int ipos = i - (int)n2, jpos = j - (int)n2;
                for (int nni1 = -w; nni1 <= w; nni1++)
                    for (int nnj1 = -w; nnj1 <= w; nnj1++) {
                        zmul(b, T, G0AT((kpoints + kpoints - (size_t)(ipos + nni1)) % kpoints,
                                        (kpoints + kpoints - (size_t)(jpos + nnj1)) % kpoints), buffer);
                        for (int nni2 = -w; nni2 <= w; nni2++)
                            for (int nnj2 = -w; nnj2 <= w; nnj2++) {
                                zmul(b, G0AT((kpoints + (size_t)(ipos + nni2)) % kpoints,
                                             (kpoints + (size_t)(jpos + nnj2)) % kpoints), buffer, cldos);
                                const double *gd = G0AT((kpoints - (size_t)nni1 + (size_t)nni2) % kpoints,
                                                        (kpoints - (size_t)nnj1 + (size_t)nnj2) % kpoints);
                                for (size_t ii = 0; ii < (size_t)os; ii++)
                                    for (size_t jj = 0; jj < (size_t)os; jj++) {
                                        size_t x = ii + (size_t)w * os, y = jj + (size_t)w * os;
                                        size_t x1 = x - (size_t)((long)nni1 * os), y1 = y - (size_t)((long)nnj1 * os);
                                        size_t x2 = x - (size_t)((long)nni2 * os), y2 = y - (size_t)((long)nnj2 * os);
                                        double *out = &ldos[((size_t)i * os + ii) % wn * wn + ((size_t)j * os + jj) % wn];
                                        if (!spin) {
                                            for (size_t o1 = 0; o1 < maxband; o1++) {
                                                if (wf_zero[o1]) continue;
                                                for (size_t o2 = 0; o2 < maxband; o2++) {
                                                    if (wf_zero[o2]) continue;
                                                    JACC(o2, o1 + maxband, WF(o1, x1, y1) * WF(o2, x2, y2));
                                                }
                                            }
                                        } else {
                                            for (size_t o1 = 0; o1 < spinbands; o1++) {
                                                if (!wf_zero[o1])
                                                    for (size_t o2 = 0; o2 < spinbands; o2++) {
                                                        if (wf_zero[o2]) continue;
                                                        JACC(o2, o1 + maxband, WF(o1, x1, y1) * WF(o2, x2, y2));
                                                    }
                                                size_t s1 = spinbands + o1;
                                                if (!wf_zero[s1])
                                                    for (size_t o2 = 0; o2 < spinbands; o2++) {
                                                        size_t s2 = spinbands + o2;
                                                        if (wf_zero[s2]) continue;
                                                        JACC(s2, s1 + maxband, WF(s1, x1, y1) * WF(s2, x2, y2));
                                                    }
                                            }
                                        }
                                    }
                            }
                    }
            }
        free(buffer); free(cldos);
    }
#undef JACC
#undef G0AT
#undef WF
}

/* ---- the Josephson tip factor of the driver, calcqpi.cc:705-708 ----
 * tip = (0, -sign(E) pi deltat) / sqrt((E + i etat)^2 - deltat^2), principal root,
 * sign(E) = copysign(1, E).  The square root is the textbook careful form
 * (t = sqrt((|x| + |z|)/2), the other part y/(2t)). */
void orc_josephson_tip(double energy, double deltat, double etat, double *tip)
{
    double zr = energy * energy - etat * etat - deltat * deltat, zi = 2.0 * energy * etat;
    double sr = 0.0, si = 0.0;
    if (zr != 0.0 || zi != 0.0) {
        double t = sqrt(0.5 * (fabs(zr) + hypot(zr, zi)));
        if (zr >= 0.0) { sr = t; si = zi / (2.0 * t); }
        else { sr = fabs(zi) / (2.0 * t); si = copysign(t, zi); }
    }
    double num = -copysign(1.0, energy) * M_PI * deltat;   /* numerator (0, num) */
    double d = sr * sr + si * si;
    tip[0] = num * si / d;
    tip[1] = num * sr / d;
}

/* ---- mkthresholdlist, qpi.cc:139-211 (maxband / spin form) and :213-253 (spinarr form) ----
 * Entries (list, i, j, o1, o2, factor) of the proximity list: factor = wf_o1(x - xn1 os,
 * y - yn1 os) wf_o2(x - xn2 os, y - yn2 os), x = i + 2w os, kept when |factor| >
 * threshold * max_l,x,y wf_l^2.  list = ((xn1 wins + yn1) wins + xn2) wins + yn2 with
 * wins = 2w+1 (the reference's flags[xn1][yn1][xn2][yn2]); entries come in the
 * reference's push order, so each list is contiguous.  spinarr (NULL for the maxband form)
 * has norb entries.  Writes at most cap entries (ent[k][5] int32, fac[k]) and returns the
 * count.  wf[o][ix][iy] of side (2w+1) os, norb orbitals. */
int64_t orc_threshold_list(int w, int os, int norb, const double *wf, double threshold, int maxband, int spin,
                           const int32_t *spinarr, int32_t *ent, double *fac, int64_t cap)
{
    size_t wins = (size_t)(2 * w + 1), xs = (size_t)os * wins;
    double maxval = 0.0;
    int64_t count = 0;
#define WFC(o, X, Y) (wf[((size_t)(o) * xs + (size_t)(X)) * xs + (size_t)(Y)])
    for (int l = 0; l < norb; l++)
        for (size_t i = 0; i < xs; i++)
            for (size_t j = 0; j < xs; j++) {
                double v = WFC(l, i, j) * WFC(l, i, j);
                if (v > maxval) maxval = v;
            }
    if (!maxband) maxband = norb;
    size_t spinbands = (size_t)(maxband >> 1);
#define PUSH(L, I, J, O1, O2, F)                                                            \
    do {                                                                                    \
        if (count < cap) {                                                                  \
            int32_t *e_ = ent + 5 * count;                                                  \
            e_[0] = (int32_t)(L); e_[1] = (int32_t)(I); e_[2] = (int32_t)(J);               \
            e_[3] = (int32_t)(O1); e_[4] = (int32_t)(O2); fac[count] = (F);                  \
        }                                                                                   \
        count++;                                                                            \
    } while (0)
    for (size_t xn1 = 0; xn1 < wins; xn1++)
        for (size_t yn1 = 0; yn1 < wins; yn1++)
            for (size_t xn2 = 0; xn2 < wins; xn2++)
                for (size_t yn2 = 0; yn2 < wins; yn2++) {
                    size_t L = ((xn1 * wins + yn1) * wins + xn2) * wins + yn2;
                    if (spinarr) {
                        for (int o1 = 0; o1 < norb; o1++) {
                            if (!spinarr[o1]) continue;
                            for (int o2 = 0; o2 < norb; o2++) {
                                if (spinarr[o1] != spinarr[o2]) continue;
                                for (size_t i = 0; i < (size_t)os; i++)
                                    for (size_t j = 0; j < (size_t)os; j++) {
                                        size_t x = i + (wins - 1) * os, y = j + (wins - 1) * os;
                                        double f = WFC(o1, x - xn1 * os, y - yn1 * os) * WFC(o2, x - xn2 * os, y - yn2 * os);
                                        if (fabs(f) > threshold * maxval) PUSH(L, i, j, o1, o2, f);
                                    }
                            }
                        }
                    } else if (spin) {
                        for (size_t o1 = 0; o1 < spinbands; o1++)
                            for (size_t o2 = 0; o2 < spinbands; o2++)
                                for (size_t i = 0; i < (size_t)os; i++)
                                    for (size_t j = 0; j < (size_t)os; j++) {
                                        size_t x = i + (wins - 1) * os, y = j + (wins - 1) * os;
                                        double f = WFC(o1, x - xn1 * os, y - yn1 * os) * WFC(o2, x - xn2 * os, y - yn2 * os);
                                        if (fabs(f) > threshold * maxval) PUSH(L, i, j, o1, o2, f);
                                        size_t s1 = spinbands + o1, s2 = spinbands + o2;
                                        f = WFC(s1, x - xn1 * os, y - yn1 * os) * WFC(s2, x - xn2 * os, y - yn2 * os);
                                        if (fabs(f) > threshold * maxval) PUSH(L, i, j, s1, s2, f);
                                    }
                    } else {
                        for (size_t o1 = 0; o1 < (size_t)maxband; o1++)
                            for (size_t o2 = 0; o2 < (size_t)maxband; o2++)
                                for (size_t i = 0; i < (size_t)os; i++)
                                    for (size_t j = 0; j < (size_t)os; j++) {
                                        size_t x = i + (wins - 1) * os, y = j + (wins - 1) * os;
                                        double f = WFC(o1, x - xn1 * os, y - yn1 * os) * WFC(o2, x - xn2 * os, y - yn2 * os);
                                        if (fabs(f) > threshold * maxval) PUSH(L, i, j, o1, o2, f);
                                    }
                    }
                }
#undef PUSH
#undef WFC
    return count;
}

/* ---- tmatrix::calcwannierldos(os, w, flaglist) (CPU), qpi.cc:1085-1134 ----
 * The double window sum of orc_wannier_ldos with the proximity list in place of the
 * orbital / sub-pixel loops: per (d1, d2) only the entries of list (d1, d2) are
 * accumulated.  ent/fac/nent as written by orc_threshold_list (lists contiguous, in list
 * order). */
void orc_wannier_ldos_list(int n, int kp, int b, int os, int w, const double *T, const double *g0r,
                           int64_t nent, const int32_t *ent, const double *fac, double *ldos,
                           int row_begin, int row_end)
{
    size_t wn = (size_t)os * n, bb = (size_t)b * b, wins = (size_t)(2 * w + 1);
    size_t nlist = wins * wins * wins * wins;
    size_t kpoints = (size_t)kp, n2 = (size_t)(n >> 1);
    int64_t *off = (int64_t *)calloc(nlist + 1, sizeof(int64_t));
    for (int64_t k = 0; k < nent; k++) off[ent[5 * k] + 1]++;
    for (size_t l = 0; l < nlist; l++) off[l + 1] += off[l];
    if (row_end <= 0 || row_end > n) row_end = n;
    for (int i = row_begin; i < row_end; i++)
        for (size_t ii = 0; ii < (size_t)os; ii++)
            for (size_t y = 0; y < wn; y++) ldos[((size_t)i * os + ii) * wn + y] = 0.0;
#define G0AT(X, Y) (g0r + 2 * (((size_t)(X) * kpoints + (size_t)(Y)) * bb))
#pragma omp parallel
    {
        double *buffer = (double *)malloc(sizeof(double) * 2 * bb);
        double *cldos = (double *)malloc(sizeof(double) * 2 * bb);
#pragma omp for collapse(2) schedule(dynamic, 4)
        for (int i = row_begin; i < row_end; i++)
            for (int j = 0; j < n; j++) {
                int ipos = i - (int)n2, jpos = j - (int)n2;
                for (int nni1 = -w; nni1 <= w; nni1++)
                    for (int nnj1 = -w; nnj1 <= w; nnj1++) {
                        zmul(b, T, G0AT((kpoints + kpoints - (size_t)(ipos + nni1)) % kpoints,
                                        (kpoints + kpoints - (size_t)(jpos + nnj1)) % kpoints), buffer);
                        for (int nni2 = -w; nni2 <= w; nni2++)
                            for (int nnj2 = -w; nnj2 <= w; nnj2++) {
                                zmul(b, G0AT((kpoints + (size_t)(ipos + nni2)) % kpoints,
                                             (kpoints + (size_t)(jpos + nnj2)) % kpoints), buffer, cldos);
                                const double *gd = G0AT((kpoints - (size_t)nni1 + (size_t)nni2) % kpoints,
                                                        (kpoints - (size_t)nnj1 + (size_t)nnj2) % kpoints);
                                size_t L = (((size_t)(nni1 + w) * wins + (size_t)(nnj1 + w)) * wins + (size_t)(nni2 + w)) * wins
                                           + (size_t)(nnj2 + w);
                                for (int64_t k = off[L]; k < off[L + 1]; k++) {
                                    const int32_t *e = ent + 5 * k;
                                    size_t ii = (size_t)e[1], jj = (size_t)e[2], o1 = (size_t)e[3], o2 = (size_t)e[4];
                                    double *out = &ldos[((size_t)i * os + ii) % wn * wn + ((size_t)j * os + jj) % wn];
                                    *out -= IM(cldos, o2 * b + o1) * fac[k];
                                    *out -= IM(gd, o2 * b + o1) * fac[k];
                                }
                            }
                    }
            }
        free(buffer); free(cldos);
    }
#undef G0AT
    free(off);
}

/* complex b x b inverse by Gauss-Jordan with partial pivoting (the role of
 * gsl_linalg_complex_LU_decomp + LU_invert in calcgreensfunctioninv); A is destroyed */
static void zinv(int b, double *A, double *inv)
{
    memset(inv, 0, sizeof(double) * 2 * b * b);
    for (int i = 0; i < b; i++) RE(inv, i * b + i) = 1.0;
    for (int c = 0; c < b; c++) {
        int piv = c; double best = -1.0;
        for (int r = c; r < b; r++) {
            double a = hypot(RE(A, r * b + c), IM(A, r * b + c));
            if (a > best) { best = a; piv = r; }
        }
        if (piv != c)
            for (int k = 0; k < b; k++) {
                double t0 = RE(A, c * b + k), t1 = IM(A, c * b + k);
                RE(A, c * b + k) = RE(A, piv * b + k); IM(A, c * b + k) = IM(A, piv * b + k);
                RE(A, piv * b + k) = t0; IM(A, piv * b + k) = t1;
                t0 = RE(inv, c * b + k); t1 = IM(inv, c * b + k);
                RE(inv, c * b + k) = RE(inv, piv * b + k); IM(inv, c * b + k) = IM(inv, piv * b + k);
                RE(inv, piv * b + k) = t0; IM(inv, piv * b + k) = t1;
            }
        double pr = RE(A, c * b + c), pi = IM(A, c * b + c), pd = pr * pr + pi * pi;
        for (int r = 0; r < b; r++) {
            if (r == c) continue;
            double mr = RE(A, r * b + c), mi = IM(A, r * b + c);
            double fr = (mr * pr + mi * pi) / pd, fi = (mi * pr - mr * pi) / pd;
            for (int k = 0; k < b; k++) {
                double xr = RE(A, c * b + k), xi = IM(A, c * b + k);
                RE(A, r * b + k) -= fr * xr - fi * xi; IM(A, r * b + k) -= fr * xi + fi * xr;
                xr = RE(inv, c * b + k); xi = IM(inv, c * b + k);
                RE(inv, r * b + k) -= fr * xr - fi * xi; IM(inv, r * b + k) -= fr * xi + fi * xr;
            }
        }
    }
    for (int r = 0; r < b; r++) {
        double pr = RE(A, r * b + r), pi = IM(A, r * b + r), pd = pr * pr + pi * pi;
        for (int k = 0; k < b; k++) {
            double xr = RE(inv, r * b + k), xi = IM(inv, r * b + k);
            RE(inv, r * b + k) = (xr * pr + xi * pi) / pd;
            IM(inv, r * b + k) = (xi * pr - xr * pi) / pd;
        }
    }
}

/* (omega + i eta - H)^-1: tightbindingcontext::calcgreensfunctioninv, tightbinding.h:75-85 */
static void resolvent(int b, const double *H, double omega, double eta, double *work, double *g)
{
    for (int i = 0; i < b * b; i++) { RE(work, i) = -RE(H, i); IM(work, i) = -IM(H, i); }
    for (int i = 0; i < b; i++) { RE(work, i * b + i) += omega; IM(work, i * b + i) += eta; }
    zinv(b, work, g);
}

static double matnorm(int b, const double *A)   /* qpi.cc:55-61 */
{
    double v = 0.0;
    for (int i = 0; i < b * b; i++) v += RE(A, i) * RE(A, i) + IM(A, i) * IM(A, i);
    return sqrt(v);
}

/* ---- tmatrix::calcsurfacegreensfunction, qpi.cc:488-554 ----
 * Per k-point: eps_s = in-plane H of the surface model (or the bulk model), eps_b = in-plane
 * H of the bulk model (hoppings with R_z = 0, tightbinding.cc:184-207), alpha = the bulk
 * hoppings with R_z < 0 (no diagonal), beta = alpha^H; renormalise
 *   g = (w + i eta - eps_b)^-1,  eps_s += a g b,  eps_b += a g b + b g a,
 *   a = a g a,  b = b g b
 * until |a|_F <= epserr and |b|_F <= epserr; then G0(k) = (w + i eta - eps_s|eps_b)^-1.
 * Hopping sets are passed already split (R_z = 0 and R_z < 0); ns < 0 uses the bulk set
 * for the surface.  max_iter bounds the loop (the reference has no bound); returns the
 * number of k-points that did not converge.  g0[kp][kp][b][b] as orc_greens_k. */
int64_t orc_surface_greens_k(int b, int kp,
                             int64_t nb_, const int32_t *Rb, const int32_t *ob, const double *tb, const uint8_t *ab,
                             int64_t no, const int32_t *Ro, const int32_t *oo, const double *to, const uint8_t *ao,
                             int64_t ns, const int32_t *Rs, const int32_t *os_, const double *ts, const uint8_t *as,
                             double efermi, int scmax, double omega, double eta, double epserr, int surface,
                             int max_iter, double *g0)
{
    size_t cut = (size_t)(kp >> 1), bb = (size_t)b * b;
    int64_t bad = 0;
#pragma omp parallel reduction(+ : bad)
    {
        double *es = (double *)malloc(sizeof(double) * 2 * bb), *eb = (double *)malloc(sizeof(double) * 2 * bb);
        double *al = (double *)malloc(sizeof(double) * 2 * bb), *be = (double *)malloc(sizeof(double) * 2 * bb);
        double *g = (double *)malloc(sizeof(double) * 2 * bb), *w = (double *)malloc(sizeof(double) * 2 * bb);
        double *b1 = (double *)malloc(sizeof(double) * 2 * bb), *b2 = (double *)malloc(sizeof(double) * 2 * bb);
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < kp; i++)
            for (int j = 0; j < kp; j++) {
                double x = ((size_t)i > cut) ? ((double)i - kp) / kp : (double)i / kp;
                double y = ((size_t)j > cut) ? ((double)j - kp) / kp : (double)j / kp;
                if (ns >= 0) orc_hk(b, ns, Rs, os_, ts, as, efermi, scmax, x, y, es);
                else orc_hk(b, nb_, Rb, ob, tb, ab, efermi, scmax, x, y, es);
                orc_hk(b, nb_, Rb, ob, tb, ab, efermi, scmax, x, y, eb);
                orc_hk(b, no, Ro, oo, to, ao, 0.0, scmax, x, y, al);   /* no diagonal */
                for (int r = 0; r < b; r++)
                    for (int c = 0; c < b; c++) {
                        RE(be, r * b + c) = RE(al, c * b + r);
                        IM(be, r * b + c) = -IM(al, c * b + r);
                    }
                int it = 0;
                do {
                    resolvent(b, eb, omega, eta, w, g);
                    zmul(b, g, be, b1);
                    zmul(b, al, b1, b2);              /* a g b */
                    for (size_t e = 0; e < 2 * bb; e++) { es[e] += b2[e]; eb[e] += b2[e]; }
                    zmul(b, g, al, b1);
                    zmul(b, be, b1, b2);              /* b g a */
                    for (size_t e = 0; e < 2 * bb; e++) eb[e] += b2[e];
                    zmul(b, g, al, b1);
                    zmul(b, al, b1, b2);
                    memcpy(al, b2, sizeof(double) * 2 * bb);
                    zmul(b, g, be, b1);
                    zmul(b, be, b1, b2);
                    memcpy(be, b2, sizeof(double) * 2 * bb);
                    it++;
                } while ((matnorm(b, al) > epserr || matnorm(b, be) > epserr) && it < max_iter);
                if (matnorm(b, al) > epserr || matnorm(b, be) > epserr) bad++;
                resolvent(b, surface ? es : eb, omega, eta, w, g0 + 2 * (((size_t)i * kp + j) * bb));
            }
        free(es); free(eb); free(al); free(be); free(g); free(w); free(b1); free(b2);
    }
    return bad;
}
