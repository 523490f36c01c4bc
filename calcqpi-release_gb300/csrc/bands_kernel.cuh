// bands_kernel.cuh -- the body of the per-k eigen-solve kernel, included twice by bands.cu:
// as bands_kernel with full unrolling of its b x b loop nests (band counts up to 5, whose
// matrices stay in registers) and as bands_kernel_wide with the loops kept (6 to 16 bands,
// whose matrices live in local memory either way; unrolled, the 6-band copy spilled 7 KB per
// thread and the larger b^3 .. b^4 nests only made the compiler run for minutes).  The includer defines CQPI_BANDS_KERNEL (the kernel's name)
// and CQPI_BANDS_UNROLL (the loop pragma).
// tr: all hoppings are real, so H(-k) = conj(H(k)): threads cover the k_x rows
// 0 .. kp/2 only and each writes its k-point and the point reflection -k (same
// eigenvalues, conjugated eigenvectors); on the self-reflected rows 0 and kp/2 the
// thread with the larger j' = -j mod kp leaves the pair to its partner.
template <int B>
__global__ void __launch_bounds__(128) CQPI_BANDS_KERNEL(int b, int kp, int tr, int scmax, double efermi, int npr,
                                                    const int32_t *__restrict__ pR, const double2 *__restrict__ pPQ,
                                                    double *__restrict__ eval,
                                                    double2 *__restrict__ evec, float2 *__restrict__ evec32,
                                                    float2 *__restrict__ eval32, const double2 *__restrict__ tw,
                                                    int mixed)
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
CQPI_BANDS_UNROLL
    for (int p = 0; p < B; p++)
CQPI_BANDS_UNROLL
        for (int q = 0; q < B; q++) {
            ar[p][q] = 0.0; ai[p][q] = 0.0;
            vr[p][q] = (p == q) ? 1.0 : 0.0; vi[p][q] = 0.0;
        }
CQPI_BANDS_UNROLL
    for (int p = 0; p < B; p++)
        if (p < b) ar[p][p] = (p < scmax) ? -efermi : efermi;

    // H(k) = diag + sum over {R, -R} pairs of P cos th + Q sin th, th = 2 pi (Rx x_i + Ry y_j)
    // (P, Q built on the host from the normal and conjugated terms).  Only the lower triangle
    // is accumulated and then mirrored: the matrix is taken as Hermitian, from its lower
    // triangle and real diagonal, as gsl_eigen_hermv takes it (src/qpi.cc:470).  The phase is
    // reduced exactly, (Rx i + Ry j) mod kp (x_i and i/kp differ by an integer), and read from
    // the FP64 table tw[t] = e^{+2 pi i t / kp}.
    for (int r = 0; r < npr; r++) {
        long long mm = ((long long)pR[2 * r] * i + (long long)pR[2 * r + 1] * j) % kp;
        if (mm < 0) mm += kp;
        const double2 ph = __ldg(tw + mm);
        const double c = ph.x, s = ph.y;
        const double2 *P = pPQ + (size_t)r * 2 * bb, *Q = P + bb;
CQPI_BANDS_UNROLL
        for (int p = 0; p < B; p++)
CQPI_BANDS_UNROLL
            for (int q = 0; q <= p; q++) {
                if (p < b) {
                    const double2 x = __ldg(P + p * b + q), y = __ldg(Q + p * b + q);
                    ar[p][q] += x.x * c + y.x * s;
                    ai[p][q] += x.y * c + y.y * s;
                }
            }
    }
CQPI_BANDS_UNROLL
    for (int p = 0; p < B; p++) {
        ai[p][p] = 0.0;
CQPI_BANDS_UNROLL
        for (int q = p + 1; q < B; q++) { ar[p][q] = ar[q][p]; ai[p][q] = -ai[q][p]; }
    }

    // Mixed precision: cyclic Jacobi in FP32 on a copy of H gives eigenvectors to ~1e-7; they
    // are orthonormalised in FP64 (modified Gram-Schmidt), H is rotated into that basis in FP64
    // (A = V^H H V, off-diagonal ~1e-7 of the diagonal) and the FP64 Jacobi below converges in
    // one or two sweeps instead of five to eight (FP64 runs at 1/64 of the FP32 rate here).
    if (mixed) {
        float fr[B][B], fi[B][B], ur[B][B], ui[B][B];
CQPI_BANDS_UNROLL
        for (int p = 0; p < B; p++)
CQPI_BANDS_UNROLL
            for (int q = 0; q < B; q++) {
                fr[p][q] = (float)ar[p][q]; fi[p][q] = (float)ai[p][q];
                ur[p][q] = (p == q) ? 1.f : 0.f; ui[p][q] = 0.f;
            }
        for (int sweep = 0; sweep < 12; sweep++) {
            float off = 0.f, dg = 0.f;
CQPI_BANDS_UNROLL
            for (int p = 0; p < B; p++)
CQPI_BANDS_UNROLL
                for (int q = 0; q < B; q++) {
                    const float a2 = fr[p][q] * fr[p][q] + fi[p][q] * fi[p][q];
                    if (p == q) dg += a2; else off += a2;
                }
            if (off == 0.f || off <= 1e-13f * dg) break;
CQPI_BANDS_UNROLL
            for (int p = 0; p < B - 1; p++)
CQPI_BANDS_UNROLL
                for (int q = p + 1; q < B; q++) {
                    const float c2 = fr[p][q] * fr[p][q] + fi[p][q] * fi[p][q];
                    if (c2 == 0.f) continue;
                    const float rc = rsqrtf(c2);
                    const float er = fr[p][q] * rc, ei = fi[p][q] * rc;
                    const float tau = (fr[q][q] - fr[p][p]) * (0.5f * rc);
                    const float tt = (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
                    const float cs = rsqrtf(1.f + tt * tt), sn = tt * cs;
CQPI_BANDS_UNROLL
                    for (int r = 0; r < B; r++) {
                        const float xpr = fr[r][p], xpi = fi[r][p];
                        const float yr = fr[r][q] * er + fi[r][q] * ei, yi = fi[r][q] * er - fr[r][q] * ei;
                        fr[r][p] = cs * xpr - sn * yr; fi[r][p] = cs * xpi - sn * yi;
                        fr[r][q] = sn * xpr + cs * yr; fi[r][q] = sn * xpi + cs * yi;
                        const float vpr = ur[r][p], vpi = ui[r][p];
                        const float wr = ur[r][q] * er + ui[r][q] * ei, wi = ui[r][q] * er - ur[r][q] * ei;
                        ur[r][p] = cs * vpr - sn * wr; ui[r][p] = cs * vpi - sn * wi;
                        ur[r][q] = sn * vpr + cs * wr; ui[r][q] = sn * vpi + cs * wi;
                    }
CQPI_BANDS_UNROLL
                    for (int cc = 0; cc < B; cc++) {
                        const float xpr = fr[p][cc], xpi = fi[p][cc];
                        const float yr = fr[q][cc] * er - fi[q][cc] * ei, yi = fi[q][cc] * er + fr[q][cc] * ei;
                        fr[p][cc] = cs * xpr - sn * yr; fi[p][cc] = cs * xpi - sn * yi;
                        fr[q][cc] = sn * xpr + cs * yr; fi[q][cc] = sn * xpi + cs * yi;
                    }
                    fr[p][q] = fi[p][q] = fr[q][p] = fi[q][p] = 0.f;
                    fi[p][p] = 0.f; fi[q][q] = 0.f;
                }
        }
        // V = orthonormalised U (FP64 modified Gram-Schmidt over the b columns)
CQPI_BANDS_UNROLL
        for (int c = 0; c < B; c++) {
CQPI_BANDS_UNROLL
            for (int r = 0; r < B; r++) { vr[r][c] = (double)ur[r][c]; vi[r][c] = (double)ui[r][c]; }
CQPI_BANDS_UNROLL
            for (int c2 = 0; c2 < B; c2++) {
                if (c2 >= c || c2 >= b) continue;
                double pr = 0.0, pi = 0.0;   // v_c2^H v_c
CQPI_BANDS_UNROLL
                for (int r = 0; r < B; r++) {
                    pr += vr[r][c2] * vr[r][c] + vi[r][c2] * vi[r][c];
                    pi += vr[r][c2] * vi[r][c] - vi[r][c2] * vr[r][c];
                }
CQPI_BANDS_UNROLL
                for (int r = 0; r < B; r++) {
                    vr[r][c] -= pr * vr[r][c2] - pi * vi[r][c2];
                    vi[r][c] -= pr * vi[r][c2] + pi * vr[r][c2];
                }
            }
            if (c < b) {
                double nn = 0.0;
CQPI_BANDS_UNROLL
                for (int r = 0; r < B; r++) nn += vr[r][c] * vr[r][c] + vi[r][c] * vi[r][c];
                const double inv = rsqrt(nn);
CQPI_BANDS_UNROLL
                for (int r = 0; r < B; r++) { vr[r][c] *= inv; vi[r][c] *= inv; }
            }
        }
        // A = V^H (H V): rows of H V overwrite the rows of H, then columns of V^H T the columns
CQPI_BANDS_UNROLL
        for (int r = 0; r < B; r++) {
            double tr_[B], ti_[B];
CQPI_BANDS_UNROLL
            for (int c = 0; c < B; c++) {
                double sr = 0.0, si = 0.0;
CQPI_BANDS_UNROLL
                for (int k2 = 0; k2 < B; k2++) {
                    sr += ar[r][k2] * vr[k2][c] - ai[r][k2] * vi[k2][c];
                    si += ar[r][k2] * vi[k2][c] + ai[r][k2] * vr[k2][c];
                }
                tr_[c] = sr; ti_[c] = si;
            }
CQPI_BANDS_UNROLL
            for (int c = 0; c < B; c++) { ar[r][c] = tr_[c]; ai[r][c] = ti_[c]; }
        }
CQPI_BANDS_UNROLL
        for (int c = 0; c < B; c++) {
            double tr_[B], ti_[B];
CQPI_BANDS_UNROLL
            for (int r = 0; r < B; r++) {
                double sr = 0.0, si = 0.0;
CQPI_BANDS_UNROLL
                for (int k2 = 0; k2 < B; k2++) {   // conj(V[k2][r]) T[k2][c]
                    sr += vr[k2][r] * ar[k2][c] + vi[k2][r] * ai[k2][c];
                    si += vr[k2][r] * ai[k2][c] - vi[k2][r] * ar[k2][c];
                }
                tr_[r] = sr; ti_[r] = si;
            }
CQPI_BANDS_UNROLL
            for (int r = 0; r < B; r++) { ar[r][c] = tr_[r]; ai[r][c] = ti_[r]; }
        }
    }

    // cyclic Jacobi sweeps (FP64), from V = identity or from the FP32 eigenvectors
    for (int sweep = 0; sweep < 40; sweep++) {
        double off = 0.0, dg = 0.0;
CQPI_BANDS_UNROLL
        for (int p = 0; p < B; p++)
CQPI_BANDS_UNROLL
            for (int q = 0; q < B; q++) {
                double a2 = ar[p][q] * ar[p][q] + ai[p][q] * ai[p][q];
                if (p == q) dg += a2; else off += a2;
            }
        if (off == 0.0 || off <= 1e-32 * dg) break;
CQPI_BANDS_UNROLL
        for (int p = 0; p < B - 1; p++)
CQPI_BANDS_UNROLL
            for (int q = p + 1; q < B; q++) {
                const double c2 = ar[p][q] * ar[p][q] + ai[p][q] * ai[p][q];
                if (c2 == 0.0) continue;
                const double rc = rsqrt(c2);
                const double er = ar[p][q] * rc, ei = ai[p][q] * rc;
                const double tau = (ar[q][q] - ar[p][p]) * (0.5 * rc);
                const double tt = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const double cs = rsqrt(1.0 + tt * tt), sn = tt * cs;
                // columns: X = A G, V = V G with G = [[cs, sn], [-sn e^{-ia}, cs e^{-ia}]]
CQPI_BANDS_UNROLL
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
CQPI_BANDS_UNROLL
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

CQPI_BANDS_UNROLL
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
CQPI_BANDS_UNROLL
    for (int o = 0; o < B; o++)
CQPI_BANDS_UNROLL
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

