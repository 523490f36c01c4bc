// bands.cu -- H(k) build and batched FP64 Hermitian eigen-solve of every k-point.
//
// Replaces tmatrix::calchamiltonian (src/qpi.cc:454-475), which calls
// tightbind::setmatrix (src/tightbinding.cc:210-219) and gsl_eigen_hermv per
// k-point.  One thread owns one k-point; the b x b matrix and its eigenvectors
// live in registers (b is a template parameter padded up to B).  The solver is
// cyclic complex Jacobi in FP64: G0(k) is invariant under eigenvector phase and
// ordering, so it matches any exact Hermitian eigensolver to rounding.
//
// Roofline: FP64-FLOP bound (GB300 FP64 is ~1/64 of FP32); once per run.
#include "cqpi_internal.h"

namespace cqpi {

// tr: all hoppings are real, so H(-k) = conj(H(k)): threads cover the k_x rows
// 0 .. kp/2 only and each writes its k-point and the point reflection -k (same
// eigenvalues, conjugated eigenvectors); on the self-reflected rows 0 and kp/2 the
// thread with the larger j' = -j mod kp leaves the pair to its partner.
template <int B>
__global__ void __launch_bounds__(128) bands_kernel(int b, int kp, int tr, int scmax, double efermi, int nR,
                                                    const int32_t *__restrict__ R, const double2 *__restrict__ tn,
                                                    const double2 *__restrict__ ta, double *__restrict__ eval,
                                                    double2 *__restrict__ evec, float2 *__restrict__ evec32,
                                                    float2 *__restrict__ eval32, const double2 *__restrict__ tw)
{
    const long long nk = (long long)kp * kp;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nthr = tr ? (long long)(kp / 2 + 1) * kp : nk;
    if (k >= nthr) return;
    const int i = (int)(k / kp), j = (int)(k % kp);
    const int ir = (kp - i) % kp, jr = (kp - j) % kp;
    if (tr && ir == i && jr < j) return;
    const long long kr = (long long)ir * kp + jr;    // -k
    const bool pair = tr && kr != k;
    const int bb = b * b;

    double ar[B][B], ai[B][B], vr[B][B], vi[B][B];
#pragma unroll
    for (int p = 0; p < B; p++)
#pragma unroll
        for (int q = 0; q < B; q++) {
            ar[p][q] = 0.0; ai[p][q] = 0.0;
            vr[p][q] = (p == q) ? 1.0 : 0.0; vi[p][q] = 0.0;
        }
#pragma unroll
    for (int p = 0; p < B; p++)
        if (p < b) ar[p][p] = (p < scmax) ? -efermi : efermi;

    // H(k) = diag + sum_R tn(R) e^{+i th} + ta(R) e^{-i th},  th = 2 pi (Rx x_i + Ry y_j).
    // The phase is reduced exactly, (Rx i + Ry j) mod kp (x_i and i/kp differ by an
    // integer), and read from the FP64 table tw[t] = e^{+2 pi i t / kp}.
    for (int r = 0; r < nR; r++) {
        long long mm = ((long long)R[2 * r] * i + (long long)R[2 * r + 1] * j) % kp;
        if (mm < 0) mm += kp;
        const double2 ph = __ldg(tw + mm);
        const double c = ph.x, s = ph.y;
        const double2 *tnr = tn + (size_t)r * bb, *tar = ta + (size_t)r * bb;
#pragma unroll
        for (int p = 0; p < B; p++)
#pragma unroll
            for (int q = 0; q < B; q++) {
                if (p < b && q < b) {
                    double2 x = __ldg(tnr + p * b + q), y = __ldg(tar + p * b + q);
                    ar[p][q] += (x.x + y.x) * c - (x.y - y.y) * s;
                    ai[p][q] += (x.y + y.y) * c + (x.x - y.x) * s;
                }
            }
    }

    // cyclic Jacobi sweeps
    for (int sweep = 0; sweep < 40; sweep++) {
        double off = 0.0, dg = 0.0;
#pragma unroll
        for (int p = 0; p < B; p++)
#pragma unroll
            for (int q = 0; q < B; q++) {
                double a2 = ar[p][q] * ar[p][q] + ai[p][q] * ai[p][q];
                if (p == q) dg += a2; else off += a2;
            }
        if (off == 0.0 || off <= 1e-32 * dg) break;
#pragma unroll
        for (int p = 0; p < B - 1; p++)
#pragma unroll
            for (int q = p + 1; q < B; q++) {
                const double c2 = ar[p][q] * ar[p][q] + ai[p][q] * ai[p][q];
                if (c2 == 0.0) continue;
                const double rc = rsqrt(c2), cab = c2 * rc;
                const double er = ar[p][q] * rc, ei = ai[p][q] * rc;
                const double tau = (ar[q][q] - ar[p][p]) * (0.5 * rc);
                const double tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const double cs = rsqrt(1.0 + tt * tt), sn = tt * cs;
                // columns: X = A G, V = V G with G = [[cs, sn], [-sn e^{-ia}, cs e^{-ia}]]
#pragma unroll
                for (int r = 0; r < B; r++) {
                    double xpr = ar[r][p], xpi = ai[r][p];
                    double yr = ar[r][q] * er + ai[r][q] * ei, yi = ai[r][q] * er - ar[r][q] * ei;
                    ar[r][p] = cs * xpr - sn * yr; ai[r][p] = cs * xpi - sn * yi;
                    ar[r][q] = sn * xpr + cs * yr; ai[r][q] = sn * xpi + cs * yi;
                    double vpr = vr[r][p], vpi = vi[r][p];
                    double wr = vr[r][q] * er + vi[r][q] * ei, wi = vi[r][q] * er - vr[r][q] * ei;
                    vr[r][p] = cs * vpr - sn * wr; vi[r][p] = cs * vpi - sn * wi;
                    vr[r][q] = sn * vpr + cs * wr; vi[r][q] = sn * vpi + cs * wi;
                }
                // rows: A = G^H X
#pragma unroll
                for (int cc = 0; cc < B; cc++) {
                    double xpr = ar[p][cc], xpi = ai[p][cc];
                    double yr = ar[q][cc] * er - ai[q][cc] * ei, yi = ai[q][cc] * er + ar[q][cc] * ei;
                    ar[p][cc] = cs * xpr - sn * yr; ai[p][cc] = cs * xpi - sn * yi;
                    ar[q][cc] = sn * xpr + cs * yr; ai[q][cc] = sn * xpi + cs * yi;
                }
                ar[p][q] = ai[p][q] = ar[q][p] = ai[q][p] = 0.0;
                ai[p][p] = 0.0; ai[q][q] = 0.0;
            }
    }

#pragma unroll
    for (int n = 0; n < B; n++)
        if (n < b) {
            eval[(size_t)n * nk + k] = ar[n][n];
            if (pair) eval[(size_t)n * nk + kr] = ar[n][n];
            if (eval32) {
                // eigenvalue as an unevaluated float pair hi + lo (for FP32 energy differences)
                const float hi = (float)ar[n][n];
                const float2 e2 = make_float2(hi, (float)(ar[n][n] - (double)hi));
                eval32[(size_t)n * nk + k] = e2;
                if (pair) eval32[(size_t)n * nk + kr] = e2;
            }
        }
#pragma unroll
    for (int o = 0; o < B; o++)
#pragma unroll
        for (int n = 0; n < B; n++)
            if (o < b && n < b) {
                evec[(size_t)(o * b + n) * nk + k] = make_double2(vr[o][n], vi[o][n]);
                if (pair) evec[(size_t)(o * b + n) * nk + kr] = make_double2(vr[o][n], -vi[o][n]);
                if (evec32) {
                    evec32[(size_t)(o * b + n) * nk + k] = make_float2((float)vr[o][n], (float)vi[o][n]);
                    if (pair) evec32[(size_t)(o * b + n) * nk + kr] = make_float2((float)vr[o][n], -(float)vi[o][n]);
                }
            }
}

template <int B>
static void launch_bands_t(cqpi_handle *h)
{
    const long long nk = (long long)h->kp * h->kp;
    const long long nthr = h->time_reversal ? (long long)(h->kp / 2 + 1) * h->kp : nk;
    bands_kernel<B><<<cdiv(nthr, 128), 128, 0, h->stream>>>(h->b, h->kp, h->time_reversal ? 1 : 0, h->scmax,
                                                            h->efermi, h->nR, h->d_R,
                                                          (const double2 *)h->d_tn, (const double2 *)h->d_ta,
                                                          h->d_eval, h->d_evec, h->d_evec32, h->d_eval32, h->d_tw);
    h->launches++;
}

void launch_bands(cqpi_handle *h)
{
    const int b = h->b;
    if (b <= 1) launch_bands_t<1>(h);
    else if (b <= 2) launch_bands_t<2>(h);
    else if (b <= 3) launch_bands_t<3>(h);
    else if (b <= 4) launch_bands_t<4>(h);
    else if (b <= 6) launch_bands_t<6>(h);
    else if (b <= 8) launch_bands_t<8>(h);
    else if (b <= 10) launch_bands_t<10>(h);
    else if (b <= 12) launch_bands_t<12>(h);
    else launch_bands_t<16>(h);
}

}  // namespace cqpi
