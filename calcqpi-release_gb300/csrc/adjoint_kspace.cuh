// adjoint_kspace.cuh -- the per-k kernels of the adjoint's step 5 (the resolvent bracket
// C(k) and Hbar(k) = U C(k) U^H), included twice by adjoint.cu: with full unrolling of their
// b x b loop nests for up to 6 bands (adj_kacc_kernel, adj_hbar_kernel) and with the loops kept
// for 8 to 16 bands (adj_kacc_kernel_wide, adj_hbar_kernel_wide), whose matrices live in local
// memory either way.  The includer defines CQPI_ADJ_KACC, CQPI_ADJ_HBAR (the kernels' names)
// and CQPI_ADJ_UNROLL (the loop pragma).
// C(k) += sum_e F_e* (U^H Gbar_e(k) U) F_e*, F_e = diag(1/(omega_e + i eta - eps_n)), over the ne
// energies of a batch (Gbar_e(k) at gk + e * b*b*nk); one thread per k.  Up to 3 bands the
// energy sum is held in FP64 registers and C(k) is read and written once per batch; more bands
// add each energy's bracket to C(k) in memory.
// C: the working precision.  double2: FP64 throughout.  float2 (the mixed handle): eigenvectors
// and Gbar(k) in FP32, the pole distances omega - eps from the eigenvalues' float pairs
// (hi, lo) as the forward builds G0 (exact near a pole by Sterbenz), the energy sum of a batch
// in FP32 with compensated (Kahan) addition, added to the FP64 C(k) once per batch.
template <int B, class C>
__global__ void __launch_bounds__(128) CQPI_ADJ_KACC(int b, long long nk, int ne, const double *__restrict__ omegas,
                                                       double eta, const typename KaccEv<C>::T *__restrict__ eval,
                                                       const C *__restrict__ evec, const C *__restrict__ gk,
                                                       double2 *__restrict__ Cacc)
{
    constexpr bool REG = B <= 3;
    constexpr bool F32 = std::is_same<C, float2>::value;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    C U[B][B], G[B][B], X[B][B], f[B];
    typename KaccEv<C>::T ev[B];
    using A = typename std::conditional<F32, float2, double2>::type;   // the batch sum
    A acc[REG ? B : 1][REG ? B : 1], cmp[REG && F32 ? B : 1][REG && F32 ? B : 1];
CQPI_ADJ_UNROLL
    for (int n = 0; n < B; n++)
        if (n < b) ev[n] = eval[(size_t)n * nk + k];
CQPI_ADJ_UNROLL
    for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++)
            if (o < b && n < b) U[o][n] = evec[(size_t)(o * b + n) * nk + k];
    if constexpr (REG) {
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++)
CQPI_ADJ_UNROLL
            for (int m = 0; m < B; m++) {
                acc[n][m] = cmake<A>(0.0, 0.0);
                if constexpr (F32) cmp[n][m] = make_float2(0.f, 0.f);
            }
    }
    const size_t plane = (size_t)b * b * nk;
    for (int e = 0; e < ne; e++) {
        const double omega = omegas[e];
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++) {
            if (n < b) {
                // conj(1/(dr + i eta))
                if constexpr (F32) {
                    const float om_hi = (float)omega, om_lo = (float)(omega - (double)om_hi);
                    const float dr = (om_hi - ev[n].x) + (om_lo - ev[n].y);
                    const float et = (float)eta;
                    const float inv = 1.f / (dr * dr + et * et);
                    f[n] = make_float2(dr * inv, et * inv);
                } else {
                    const double dr = omega - ev[n];
                    const double inv = 1.0 / (dr * dr + eta * eta);
                    f[n] = make_double2(dr * inv, eta * inv);
                }
            }
        }
CQPI_ADJ_UNROLL
        for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
            for (int n = 0; n < B; n++)
                if (o < b && n < b) G[o][n] = gk[e * plane + (size_t)(o * b + n) * nk + k];
        // X = Gbar U
CQPI_ADJ_UNROLL
        for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
            for (int m = 0; m < B; m++) {
                if (o >= b || m >= b) continue;
                C s = cmake<C>(0.0, 0.0);
CQPI_ADJ_UNROLL
                for (int a = 0; a < B; a++)
                    if (a < b) s = cadd(s, cmul(G[o][a], U[a][m]));
                X[o][m] = s;
            }
        // C += f*_n (U^H X)_nm f*_m
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++)
CQPI_ADJ_UNROLL
            for (int m = 0; m < B; m++) {
                if (n >= b || m >= b) continue;
                C s = cmake<C>(0.0, 0.0);
CQPI_ADJ_UNROLL
                for (int o = 0; o < B; o++)
                    if (o < b) {
                        C un = U[o][n];
                        un.y = -un.y;
                        s = cadd(s, cmul(un, X[o][m]));
                    }
                s = cmul(cmul(f[n], s), f[m]);
                if constexpr (REG && F32) {
                    // compensated: cmp holds the rounding error of the running sum
                    const float2 y = make_float2(s.x - cmp[n][m].x, s.y - cmp[n][m].y);
                    const float2 t = make_float2(acc[n][m].x + y.x, acc[n][m].y + y.y);
                    cmp[n][m] = make_float2((t.x - acc[n][m].x) - y.x, (t.y - acc[n][m].y) - y.y);
                    acc[n][m] = t;
                } else if constexpr (REG) {
                    acc[n][m] = cadd(acc[n][m], to_d2(s));
                } else {
                    double2 *c = Cacc + (size_t)(n * b + m) * nk + k;
                    *c = cadd(*c, to_d2(s));
                }
            }
    }
    if constexpr (REG) {
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++)
CQPI_ADJ_UNROLL
            for (int m = 0; m < B; m++) {
                if (n >= b || m >= b) continue;
                double2 *c = Cacc + (size_t)(n * b + m) * nk + k;
                if constexpr (F32)
                    *c = make_double2(c->x + ((double)acc[n][m].x - (double)cmp[n][m].x),
                                      c->y + ((double)acc[n][m].y - (double)cmp[n][m].y));
                else
                    *c = cadd(*c, acc[n][m]);
            }
    }
}

// Hbar(k) = U C(k) U^H, written over gk in the working precision C (the mixed handle: the FP32
// eigenvectors, C(k) rounded to FP32)
template <int B, class C>
__global__ void __launch_bounds__(128) CQPI_ADJ_HBAR(int b, long long nk, const C *__restrict__ evec,
                                                       const double2 *__restrict__ Cacc, C *__restrict__ hbar)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    C U[B][B], X[B][B];
CQPI_ADJ_UNROLL
    for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
        for (int n = 0; n < B; n++)
            if (o < b && n < b) U[o][n] = evec[(size_t)(o * b + n) * nk + k];
    // X = U C
CQPI_ADJ_UNROLL
    for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
        for (int m = 0; m < B; m++) {
            if (o >= b || m >= b) continue;
            C s = cmake<C>(0.0, 0.0);
CQPI_ADJ_UNROLL
            for (int n = 0; n < B; n++)
                if (n < b) {
                    const double2 c = Cacc[(size_t)(n * b + m) * nk + k];
                    s = cadd(s, cmul(U[o][n], cmake<C>(c.x, c.y)));
                }
            X[o][m] = s;
        }
CQPI_ADJ_UNROLL
    for (int o = 0; o < B; o++)
CQPI_ADJ_UNROLL
        for (int a = 0; a < B; a++) {
            if (o >= b || a >= b) continue;
            C s = cmake<C>(0.0, 0.0);
CQPI_ADJ_UNROLL
            for (int m = 0; m < B; m++)
                if (m < b) s = cadd(s, cmul(X[o][m], cconj(U[a][m])));
            hbar[(size_t)(o * b + a) * nk + k] = s;
        }
}

