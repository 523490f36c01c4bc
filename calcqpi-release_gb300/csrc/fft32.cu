// fft32.cu -- mixed-path Green's function: fused G0(k,w) assembly + pruned 2D FFT in FP32
// for power-of-two k-grids.
//
// Replaces, per energy, tmatrix::setgreensfunction (src/qpi.cc:478-486) and
// tmatrix::calcrealspacegreensfunction (src/qpi.cc:557-578), which transform all b^2
// kp x kp planes in FP64 with FFTW and keep every R.  Here only the box
// R in [-Rb, Rb]^2 that the contraction reads is produced:
//
//   pass 1 (g0_rowfft): one CTA per k-row i.  For every energy of the batch it builds
//     G0(k_i, k_j) = sum_n U_n U_n^H / (w - e_n + i eta) for all j and all b^2 planes
//     directly in shared memory (w - e_n in FP64, the rest in FP32; the eigen data of the
//     row is re-read from L1/L2 for each energy), runs radix-2 transforms along j on all
//     planes with one barrier per stage, and stores the NB pruned outputs Y = yb - Rb.
//     No G0(k) array ever reaches HBM.
//   pass 2 (colfft): NC adjacent columns yb per CTA, transforms along i, keeps
//     X = xb - Rb, scales by kp^-2 and records max|Re|,|Im| per energy (the operand
//     scale of the tensor-core contraction).
//
// Shared-memory rows are padded by one element per 32 (index p + p/32) so that the
// bit-reversed stores and the short-stride butterflies do not collide on banks.
// Roofline: pass 1 reads the eigen cache (96 B per k-point for 3 bands) and writes
// b^2 * kp * NB complex values; both passes are shared-memory / issue bound at
// kp = 1024 (0.6 GFLOP per energy), see profiles/.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "cplx.h"
#include "cqpi_internal.h"
#include "fft_reg.cuh"

namespace cqpi {

__device__ __forceinline__ int brev_bits(int x, int bits) { return bits == 0 ? 0 : (int)(__brev((unsigned)x) >> (32 - bits)); }
__device__ __forceinline__ int pmod(int a, int m) { int r = a % m; return r < 0 ? r + m : r; }

// Planes of the upper triangle o <= a in row-major order (reciprocity: with real hoppings
// H(-k) = conj H(k), so G0(-k) = G0(k)^T and G0(R)[a][o] = G0(-R)[o][a]: only these planes are
// transformed and the lower ones are filled by the point reflection of R).
__device__ __forceinline__ void tri_plane(int b, int idx, int &o, int &a)
{
    o = 0;
    while (idx >= b - o) { idx -= b - o; o++; }
    a = o + idx;
}
__device__ __forceinline__ int tri_index(int b, int o, int a) { return o * b - (o * (o - 1)) / 2 + (a - o); }

template <int B>
__global__ void __launch_bounds__(256) g0_rowfft_kernel(int b, int kp, int logkp, int NB, int Rb, int pg, double eta,
                                                        const double *__restrict__ energies, int ne,
                                                        const double *__restrict__ eval, const float2 *__restrict__ evec,
                                                        const float2 *__restrict__ tw, float2 *__restrict__ half)
{
    extern __shared__ __align__(16) float2 sm[];
    const int bb = b * b;
    const long long nk = (long long)kp * kp;
    const int i = blockIdx.x;
    const int plen = pad32(kp) + 1;
    float2 *tws = sm + (size_t)pg * plen;
    const int hk = kp >> 1;
    for (int t = threadIdx.x; t < hk; t += blockDim.x) tws[t] = tw[t];
    const float et = (float)eta;

    for (int e = 0; e < ne; e++) {
        const double om = energies[e];
        for (int pl0 = 0; pl0 < bb; pl0 += pg) {
            const int npl = min(pg, bb - pl0);
            __syncthreads();   // previous users of the plane buffers are done
            // ---- G0(k) of this row for planes [pl0, pl0+npl), bit-reversed positions
            for (int j = threadIdx.x; j < kp; j += blockDim.x) {
                const long long k = (long long)i * kp + j;
                float2 f[B];
#pragma unroll
                for (int n = 0; n < B; n++) {
                    if (n < b) {
                        const float dr = (float)(om - eval[(size_t)n * nk + k]);
                        const float den = dr * dr + et * et;
                        f[n] = make_float2(dr / den, -et / den);
                    }
                }
                const int pos = pad32(brev_bits(j, logkp));
                if (B <= 6 && npl == bb) {
                    // all planes at once: eigenvectors of this k-point in registers
                    float2 U[B][B];
#pragma unroll
                    for (int o = 0; o < B; o++)
#pragma unroll
                        for (int n = 0; n < B; n++)
                            if (o < b && n < b) U[o][n] = evec[(size_t)(o * b + n) * nk + k];
#pragma unroll
                    for (int o = 0; o < B; o++) {
                        if (o >= b) continue;
                        float2 x[B];
#pragma unroll
                        for (int n = 0; n < B; n++)
                            if (n < b) x[n] = cmul(U[o][n], f[n]);
#pragma unroll
                        for (int a = 0; a < B; a++) {
                            if (a >= b) continue;
                            float2 s = make_float2(0.f, 0.f);
#pragma unroll
                            for (int n = 0; n < B; n++) {
                                if (n < b) {
                                    s.x += x[n].x * U[a][n].x + x[n].y * U[a][n].y;   // x * conj(U[a][n])
                                    s.y += x[n].y * U[a][n].x - x[n].x * U[a][n].y;
                                }
                            }
                            sm[(size_t)(o * b + a) * plen + pos] = s;
                        }
                    }
                } else {
                    for (int q = 0; q < npl; q++) {
                        const int pl = pl0 + q, o = pl / b, a = pl - o * b;
                        float2 s = make_float2(0.f, 0.f);
#pragma unroll
                        for (int n = 0; n < B; n++) {
                            if (n < b) {
                                const float2 uo = evec[(size_t)(o * b + n) * nk + k];
                                const float2 ua = evec[(size_t)(a * b + n) * nk + k];
                                const float2 x = cmul(uo, f[n]);
                                s.x += x.x * ua.x + x.y * ua.y;   // x * conj(ua)
                                s.y += x.y * ua.x - x.x * ua.y;
                            }
                        }
                        sm[(size_t)q * plen + pos] = s;
                    }
                }
            }
            __syncthreads();
            // ---- radix-2 decimation in time over all planes of the group
            const int nbf = npl * hk;
            for (int s = 0; s < logkp; s++) {
                const int hl = 1 << s, tsh = logkp - 1 - s;
                for (int t = threadIdx.x; t < nbf; t += blockDim.x) {
                    const int q = t >> (logkp - 1), tt = t & (hk - 1);
                    const int kk = tt & (hl - 1);
                    const int idx = ((tt >> s) << (s + 1)) | kk;
                    float2 *a = sm + (size_t)q * plen;
                    const float2 w = tws[kk << tsh];
                    const float2 u = a[pad32(idx)], v = cmul(a[pad32(idx + hl)], w);
                    a[pad32(idx)] = cadd(u, v);
                    a[pad32(idx + hl)] = csub(u, v);
                }
                __syncthreads();
            }
            // ---- pruned outputs
            for (int q = 0; q < npl; q++) {
                float2 *dst = half + (((size_t)e * bb + pl0 + q) * kp + i) * NB;
                const float2 *a = sm + (size_t)q * plen;
                for (int yb = threadIdx.x; yb < NB; yb += blockDim.x) dst[yb] = a[pad32(pmod(yb - Rb, kp))];
            }
        }
    }
}


// ------------------------------------------------------------------ register four-step row transform
// Pass 1 with the transform along j done as kp = N1 x N2: for each n1 a length-N2 FFT over
// n2 of x[n1 + N1 n2] (registers), twiddle e^{+2 pi i n1 k2 / kp}, then for each k2 a
// length-N1 FFT over n1 (registers) giving X[k2 + N2 k1].  One shared-memory exchange
// between the two passes instead of log2(kp) butterfly rounds.  BM: largest band count
// whose eigenvectors are kept in registers during the G0 build.  MAXT: largest block size
// the kernel is launched with (one thread per transform of a plane group where possible).
template <int N1, int N2, int BM = 4, int MAXT = 256>
__global__ void __launch_bounds__(MAXT) g0_rowfft_reg_kernel(int b, int NB, int Rb, int pg, int eig_smem, int tr,
                                                            double eta,
                                                            const double *__restrict__ energies, int ne,
                                                            const float2 *__restrict__ eval_g,
                                                            const float2 *__restrict__ evec_g,
                                                            const float2 *__restrict__ tw, float2 *__restrict__ half)
{
    constexpr int KP = N1 * N2;
    extern __shared__ __align__(16) float2 sm[];
    const int bb = b * b;
    const int np = tr ? (b * (b + 1)) / 2 : bb;   // planes transformed (tr: upper triangle)
    const long long nk = (long long)KP * KP;
    const int i = blockIdx.x;
    constexpr int PLEN = KP + KP / 32 + 1;
    float2 *tws = sm + (size_t)pg * PLEN;        // e^{+2 pi i t / kp}, t < kp
    for (int t = threadIdx.x; t < KP; t += blockDim.x) tws[t] = tw[t];
    const float et = (float)eta;
    // eigen cache of this k_x row: kept in shared memory for all energies when it fits
    // ([band][j] eigenvalues, [o*b+n][j] eigenvectors), else read from global memory
    const float2 *eval = eval_g + (size_t)i * KP;
    const float2 *evec = evec_g + (size_t)i * KP;
    long long estride = nk;
    if (eig_smem) {
        float2 *se = tws + KP;
        float2 *sv = se + (size_t)b * KP;
        for (int t = threadIdx.x; t < b * KP; t += blockDim.x) se[t] = eval[(size_t)(t / KP) * nk + (t % KP)];
        for (int t = threadIdx.x; t < bb * KP; t += blockDim.x) sv[t] = evec[(size_t)(t / KP) * nk + (t % KP)];
        eval = se;
        evec = sv;
        estride = KP;
    }

    for (int e = 0; e < ne; e++) {
        const double om = energies[e];
        // omega - eps in FP32 from float pairs: (om_hi - e_hi) is exact when the two are
        // within a factor of two (Sterbenz), so the difference keeps its accuracy near poles
        const float om_hi = (float)om, om_lo = (float)(om - (double)om_hi);
        for (int pl0 = 0; pl0 < np; pl0 += pg) {
            const int npl = min(pg, np - pl0);
            __syncthreads();
            // ---- G0(k) for planes [pl0, pl0+npl), natural order j (padded)
            for (int j = threadIdx.x; j < KP; j += blockDim.x) {
                const int pos = pad32(j);
                if (b <= BM && npl == np) {
                    float2 f[BM], U[BM][BM];
#pragma unroll
                    for (int n = 0; n < BM; n++) {
                        if (n < b) {
                            const float2 ev = eval[(size_t)n * estride + j];
                            const float dr = (om_hi - ev.x) + (om_lo - ev.y);
                            const float inv = __frcp_rn(dr * dr + et * et);
                            f[n] = make_float2(dr * inv, -et * inv);
                        }
                    }
#pragma unroll
                    for (int o = 0; o < BM; o++)
#pragma unroll
                        for (int n = 0; n < BM; n++)
                            if (o < b && n < b) U[o][n] = evec[(size_t)(o * b + n) * estride + j];
#pragma unroll
                    for (int o = 0; o < BM; o++) {
                        if (o >= b) continue;
                        float2 x[BM];
#pragma unroll
                        for (int n = 0; n < BM; n++)
                            if (n < b) x[n] = cmul(U[o][n], f[n]);
#pragma unroll
                        for (int a = 0; a < BM; a++) {
                            if (a >= b || (tr && a < o)) continue;
                            float2 s = make_float2(0.f, 0.f);
#pragma unroll
                            for (int n = 0; n < BM; n++) {
                                if (n < b) {
                                    s.x += x[n].x * U[a][n].x + x[n].y * U[a][n].y;
                                    s.y += x[n].y * U[a][n].x - x[n].x * U[a][n].y;
                                }
                            }
                            sm[(size_t)(tr ? tri_index(b, o, a) : o * b + a) * PLEN + pos] = s;
                        }
                    }
                } else {
                    for (int q = 0; q < npl; q++) {
                        const int pl = pl0 + q;
                        int o = pl / b, a = pl - o * b;
                        if (tr) tri_plane(b, pl, o, a);
                        float2 s = make_float2(0.f, 0.f);
                        for (int n = 0; n < b; n++) {
                            const float2 ev = eval[(size_t)n * estride + j];
                            const float dr = (om_hi - ev.x) + (om_lo - ev.y);
                            const float inv = __frcp_rn(dr * dr + et * et);
                            const float2 f = make_float2(dr * inv, -et * inv);
                            const float2 x = cmul(evec[(size_t)(o * b + n) * estride + j], f);
                            const float2 ua = evec[(size_t)(a * b + n) * estride + j];
                            s.x += x.x * ua.x + x.y * ua.y;
                            s.y += x.y * ua.x - x.x * ua.y;
                        }
                        sm[(size_t)q * PLEN + pos] = s;
                    }
                }
            }
            __syncthreads();
            // ---- pass A: (plane, n1) tasks, length-N2 transforms over n2, twiddle
            for (int task = threadIdx.x; task < npl * N1; task += blockDim.x) {
                const int q = task / N1, n1 = task - q * N1;
                float2 *a = sm + (size_t)q * PLEN;
                float2 x[N2];
#pragma unroll
                for (int n2 = 0; n2 < N2; n2++) x[n2] = a[pad32(n1 + N1 * n2)];
                fft_reg<N2>(x);
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) a[pad32(n1 + N1 * k2)] = cmul(x[k2], tws[(n1 * k2) & (KP - 1)]);
            }
            __syncthreads();
            // ---- pass B: (plane, k2) tasks, length-N1 transforms over n1, pruned stores
            for (int task = threadIdx.x; task < npl * N2; task += blockDim.x) {
                const int q = task / N2, k2 = task - q * N2;
                const float2 *a = sm + (size_t)q * PLEN;
                float2 x[N1];
#pragma unroll
                for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
                fft_reg<N1>(x);
                float2 *dst = half + (((size_t)e * np + pl0 + q) * KP + i) * NB;
#pragma unroll
                for (int k1 = 0; k1 < N1; k1++) {
                    // output Y in [0, kp) is R = Y mod kp; with NB <= kp exactly one box slot or none
                    const int yb = (k2 + N2 * k1 + Rb) & (KP - 1);
                    if (yb < NB) dst[yb] = x[k1];
                }
            }
        }
    }
}

// Persistent form of the fused G0 build + four-step row transform for up to 3 bands, where
// every plane of a k_x row fits one shared-memory group (np = b^2, or the b(b+1)/2 upper
// planes under reciprocity; one thread per (plane, n1) / (plane, k2) task).  The grid is the
// number of blocks resident on the device; block c takes the (row i, energy e) items
// [c * items / grid, (c + 1) * items / grid) in row-major order, so there is no partial last
// wave and the blocks running at one time read the eigen data of a few neighbouring rows
// (L1 / L2 hits).  Band count B as a template parameter keeps the G0 build's matrices in the
// registers they need, so three blocks fit per SM.  The first pass's twiddles are stored as
// [k2][n1] (a warp, consecutive n1, reads consecutive entries).
template <int N1, int N2, int B>
__global__ void __launch_bounds__(B * B * (N1 > N2 ? N1 : N2), (B == 3 ? 2 : 1))
g0_rowfft_pk_kernel(int NB, int Rb, int tr, double eta, const double *__restrict__ energies, int ne,
                    const float2 *__restrict__ eval_g, const float2 *__restrict__ evec_g,
                    const float2 *__restrict__ tw, float2 *__restrict__ half)
{
    constexpr int KP = N1 * N2;
    constexpr int PLEN = KP + KP / 32 + 1;
    extern __shared__ __align__(16) float2 sm[];
    const int np = tr ? (B * (B + 1)) / 2 : B * B;
    float2 *tw2 = sm + (size_t)np * PLEN;        // [k2][n1] = e^{+2 pi i n1 k2 / kp}
    for (int t = threadIdx.x; t < KP; t += blockDim.x) {
        const int k2 = t / N1, n1 = t - k2 * N1;
        tw2[t] = tw[(n1 * k2) & (KP - 1)];
    }
    const long long nk = (long long)KP * KP;
    const long long items = (long long)KP * ne;
    const long long t0 = items * blockIdx.x / gridDim.x, t1 = items * (blockIdx.x + 1) / gridDim.x;
    const float et = (float)eta;
    for (long long t = t0; t < t1; t++) {
        const int i = (int)(t / ne), e = (int)(t - (long long)i * ne);
        const float2 *eval = eval_g + (size_t)i * KP;
        const float2 *evec = evec_g + (size_t)i * KP;
        const double om = energies[e];
        // omega - eps in FP32 from float pairs (see g0_rowfft_reg_kernel)
        const float om_hi = (float)om, om_lo = (float)(om - (double)om_hi);
        __syncthreads();   // the previous item's second pass has read the planes (and tw2 is set)
#pragma unroll 2
        for (int j = threadIdx.x; j < KP; j += blockDim.x) {
            const int pos = pad32(j);
            float2 f[B], U[B][B];
#pragma unroll
            for (int n = 0; n < B; n++) {
                const float2 ev = eval[(size_t)n * nk + j];
                const float dr = (om_hi - ev.x) + (om_lo - ev.y);
                const float inv = __frcp_rn(dr * dr + et * et);
                f[n] = make_float2(dr * inv, -et * inv);
            }
#pragma unroll
            for (int o = 0; o < B; o++)
#pragma unroll
                for (int n = 0; n < B; n++) U[o][n] = evec[(size_t)(o * B + n) * nk + j];
#pragma unroll
            for (int o = 0; o < B; o++) {
                float2 x[B];
#pragma unroll
                for (int n = 0; n < B; n++) x[n] = cmul(U[o][n], f[n]);
#pragma unroll
                for (int a = 0; a < B; a++) {
                    if (tr && a < o) continue;
                    float2 s = make_float2(0.f, 0.f);
#pragma unroll
                    for (int n = 0; n < B; n++) {
                        s.x += x[n].x * U[a][n].x + x[n].y * U[a][n].y;
                        s.y += x[n].y * U[a][n].x - x[n].x * U[a][n].y;
                    }
                    sm[(size_t)(tr ? tri_index(B, o, a) : o * B + a) * PLEN + pos] = s;
                }
            }
        }
        __syncthreads();
        // first pass: (plane, n1) tasks, length-N2 transforms over n2, twiddle
        for (int task = threadIdx.x; task < np * N1; task += blockDim.x) {
            const int q = task / N1, n1 = task - q * N1;
            float2 *a = sm + (size_t)q * PLEN;
            float2 x[N2];
#pragma unroll
            for (int n2 = 0; n2 < N2; n2++) x[n2] = a[pad32(n1 + N1 * n2)];
            fft_reg<N2>(x);
#pragma unroll
            for (int k2 = 0; k2 < N2; k2++) a[pad32(n1 + N1 * k2)] = cmul(x[k2], tw2[k2 * N1 + n1]);
        }
        __syncthreads();
        // second pass: (plane, k2) tasks, length-N1 transforms over n1, pruned stores
        for (int task = threadIdx.x; task < np * N2; task += blockDim.x) {
            const int q = task / N2, k2 = task - q * N2;
            const float2 *a = sm + (size_t)q * PLEN;
            float2 x[N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
            fft_reg<N1>(x);
            float2 *dst = half + (((size_t)e * np + q) * KP + i) * NB;
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) {
                const int yb = (k2 + N2 * k1 + Rb) & (KP - 1);
                if (yb < NB) dst[yb] = x[k1];
            }
        }
    }
}

// Pass 1 of the unfused mixed path (more than 4 bands: G0(k) planes already in HBM, written
// by greens_k_kernel): RPC rows r = (energy * b^2 + plane) * kp + i per CTA, loaded with
// coalesced row reads, then the four-step register transform along j and the pruned stores
// of g0_rowfft_reg_kernel.  HBM-bound: one read of the G0(k) planes, NB / kp of it written.
// rows per CTA: 256 / min(N1, N2), so that the first register pass (RPC x N1 tasks) keeps
// all 256 threads busy when N1 < N2 (kp = 2048: 8 rows, 151 KB of shared memory)
template <int N1, int N2>
__host__ __device__ constexpr int rowfft_g0k_rpc() { return 256 / (N1 < N2 ? N1 : N2); }

template <int N1, int N2>
__global__ void __launch_bounds__(256) rowfft_reg_g0k_kernel(int NB, int Rb, long long nrows,
                                                             const float2 *__restrict__ g0k,
                                                             const float2 *__restrict__ tw, float2 *__restrict__ half)
{
    constexpr int KP = N1 * N2;
    constexpr int RPC = rowfft_g0k_rpc<N1, N2>();
    constexpr int PLEN = KP + KP / 32 + 1;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tws = sm + (size_t)RPC * PLEN;
    for (int t = threadIdx.x; t < KP; t += blockDim.x) {   // [k2][n1], as in colfft_reg_kernel
        const int k2 = t / N1, n1 = t - k2 * N1;
        tws[t] = tw[(n1 * k2) & (KP - 1)];
    }
    const long long r0 = (long long)blockIdx.x * RPC;
    for (int idx = threadIdx.x; idx < RPC * KP; idx += blockDim.x) {
        const int rr = idx / KP, j = idx - rr * KP;
        if (r0 + rr < nrows) sm[(size_t)rr * PLEN + pad32(j)] = g0k[(size_t)(r0 + rr) * KP + j];
    }
    __syncthreads();
    for (int task = threadIdx.x; task < RPC * N1; task += blockDim.x) {
        const int q = task / N1, n1 = task - q * N1;
        float2 *a = sm + (size_t)q * PLEN;
        float2 x[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; n2++) x[n2] = a[pad32(n1 + N1 * n2)];
        fft_reg<N2>(x);
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) a[pad32(n1 + N1 * k2)] = cmul(x[k2], tws[k2 * N1 + n1]);
    }
    __syncthreads();
    for (int task = threadIdx.x; task < RPC * N2; task += blockDim.x) {
        const int q = task / N2, k2 = task - q * N2;
        if (r0 + q >= nrows) continue;
        const float2 *a = sm + (size_t)q * PLEN;
        float2 x[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
        fft_reg<N1>(x);
        float2 *dst = half + (size_t)(r0 + q) * NB;
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) {
            const int yb = (k2 + N2 * k1 + Rb) & (KP - 1);
            if (yb < NB) dst[yb] = x[k1];
        }
    }
}

// Pass 2 as a four-step register transform (kp = N1 x N2, box no wider than kp): a block
// takes NC = 256/N1 adjacent columns yb of one (plane, energy), transforms along i with the
// same two register passes as the row transform, scales by kp^-2 and writes the box rows
// xb = (X + Rb) mod kp < NB, tracking max|G0| of the energy for the split scale.
template <int N1, int N2>
__global__ void __launch_bounds__(256) colfft_reg_kernel(int NB, int Rb, int b, int np, int tr, float scale,
                                                         const float2 *__restrict__ half, const float2 *__restrict__ tw,
                                                         float2 *__restrict__ box, unsigned *__restrict__ gmax)
{
    constexpr int KP = N1 * N2;
    constexpr int NC = 256 / N1;
    constexpr int PLEN = KP + KP / 32 + 1;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tws = sm + (size_t)NC * PLEN;
    const int yb0 = blockIdx.x * NC, pl = blockIdx.y, e = blockIdx.z;
    const int bb = b * b;
    int po = pl / b, pa = pl - po * b;          // the plane's orbitals (o, a)
    if (tr) tri_plane(b, pl, po, pa);
    // first-pass twiddles as [k2][n1] = e^{+2 pi i n1 k2 / kp}: a warp (consecutive n1) reads
    // consecutive entries
    for (int t = threadIdx.x; t < KP; t += blockDim.x) {
        const int k2 = t / N1, n1 = t - k2 * N1;
        tws[t] = tw[(n1 * k2) & (KP - 1)];
    }
    const float2 *src = half + ((size_t)e * np + pl) * (size_t)KP * NB;
    // every load of the block in flight at once (cp.async, zero-filled past the box)
    for (int idx = threadIdx.x; idx < KP * NC; idx += blockDim.x) {
        const int i = idx / NC, c = idx - i * NC, yb = yb0 + c;
        const bool in = yb < NB;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sm + (size_t)c * PLEN + pad32(i));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(in ? src + (size_t)i * NB + yb : src),
                     "r"(in ? 8u : 0u) : "memory");
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    for (int task = threadIdx.x; task < NC * N1; task += blockDim.x) {
        const int c = task / N1, n1 = task - c * N1;
        float2 *a = sm + (size_t)c * PLEN;
        float2 x[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; n2++) x[n2] = a[pad32(n1 + N1 * n2)];
        fft_reg<N2>(x);
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) a[pad32(n1 + N1 * k2)] = cmul(x[k2], tws[k2 * N1 + n1]);
    }
    __syncthreads();
    float mx = 0.0f;
    float2 *dst = box + (size_t)e * NB * NB * bb;
    for (int task = threadIdx.x; task < NC * N2; task += blockDim.x) {
        const int c = task / N2, k2 = task - c * N2, yb = yb0 + c;
        const float2 *a = sm + (size_t)c * PLEN;
        float2 x[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
        fft_reg<N1>(x);
        if (yb < NB) {
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) {
                const int xb = (k2 + N2 * k1 + Rb) & (KP - 1);
                if (xb < NB) {
                    const float2 v = cscale(x[k1], scale);
                    dst[((size_t)xb * NB + yb) * bb + po * b + pa] = v;
                    // reciprocity: G0(-R)[a][o] = G0(R)[o][a]
                    if (tr && po != pa) dst[((size_t)(2 * Rb - xb) * NB + (2 * Rb - yb)) * bb + pa * b + po] = v;
                    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(gmax + e, __float_as_uint(mx));
}

// Pass 2: NC = 2^lnc adjacent columns (fixed plane, energy), transform along i.
__global__ void __launch_bounds__(256) colfft_kernel(int kp, int logkp, int NB, int Rb, int bb, int lnc, float scale,
                                                     const float2 *__restrict__ half, const float2 *__restrict__ tw,
                                                     float2 *__restrict__ box, unsigned *__restrict__ gmax)
{
    extern __shared__ __align__(16) float2 sm[];
    const int NC = 1 << lnc;
    const int yb0 = blockIdx.x * NC, pl = blockIdx.y, e = blockIdx.z;
    const int hk = kp >> 1;
    float2 *tws = sm + (size_t)kp * NC;
    for (int t = threadIdx.x; t < hk; t += blockDim.x) tws[t] = tw[t];
    const float2 *src = half + ((size_t)e * bb + pl) * (size_t)kp * NB;
    for (int idx = threadIdx.x; idx < kp * NC; idx += blockDim.x) {
        const int ii = idx >> lnc, c = idx & (NC - 1), yb = yb0 + c;
        sm[(brev_bits(ii, logkp) << lnc) + c] = (yb < NB) ? src[(size_t)ii * NB + yb] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int s = 0; s < logkp; s++) {
        const int hl = 1 << s, tsh = logkp - 1 - s;
        for (int t = threadIdx.x; t < hk * NC; t += blockDim.x) {
            const int c = t & (NC - 1), bt = t >> lnc;
            const int kk = bt & (hl - 1);
            const int idx = ((bt >> s) << (s + 1)) | kk;
            const float2 w = tws[kk << tsh];
            const float2 u = sm[(idx << lnc) + c], v = cmul(sm[((idx + hl) << lnc) + c], w);
            sm[(idx << lnc) + c] = cadd(u, v);
            sm[((idx + hl) << lnc) + c] = csub(u, v);
        }
        __syncthreads();
    }
    float2 *dst = box + (size_t)e * NB * NB * bb;
    float mx = 0.0f;
    const int tot = NB * NC;
    const int lim = ((tot + (int)blockDim.x - 1) / (int)blockDim.x) * (int)blockDim.x;
    for (int idx = threadIdx.x; idx < lim; idx += blockDim.x) {
        const int xb = idx >> lnc, c = idx & (NC - 1), yb = yb0 + c;
        if (idx < tot && yb < NB) {
            const float2 v = cscale(sm[(pmod(xb - Rb, kp) << lnc) + c], scale);
            dst[((size_t)xb * NB + yb) * bb + pl] = v;
            mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(gmax + e, __float_as_uint(mx));
}

static int ilog2i(int v)
{
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

// planes per pass-1 CTA: shared memory <= 96 KiB
static int rowfft_plane_group(const cqpi_handle *h)
{
    const size_t plen = (size_t)h->kp + (h->kp >> 5) + 1;
    int pg = (int)((96 * 1024 - 4 * (size_t)h->kp) / (8 * plen));
    return std::max(1, std::min(pg, h->b * h->b));
}

static int colfft_lnc(int kp)
{
    int lnc = 4;   // 16 columns
    while (lnc > 0 && (size_t)8 * kp * (1 << lnc) + 4 * (size_t)kp > 120 * 1024) lnc--;
    return lnc;
}

static bool rowfft_reg_ok(const cqpi_handle *h);
static cudaError_t configure_rowfft_reg(cqpi_handle *h);
static cudaError_t configure_rowfft_g0k(cqpi_handle *h);
static cudaError_t configure_colfft_reg(cqpi_handle *h);
static void launch_colfft_reg(cqpi_handle *h, int ne, int tr);

bool fft32_supported(const cqpi_handle *h) { return h->kp >= 2 && (h->kp & (h->kp - 1)) == 0 && h->kp <= 8192; }

cudaError_t configure_fft32(cqpi_handle *h)
{
    if (!fft32_supported(h)) return cudaSuccess;
    const int pg = rowfft_plane_group(h);
    const size_t s1 = 8 * ((size_t)pg * (h->kp + (h->kp >> 5) + 1) + h->kp / 2);
    const size_t s2 = 8 * ((size_t)h->kp * (1 << colfft_lnc(h->kp)) + h->kp / 2);
    cudaError_t e;
#define CQPI_SETSMEM(K) e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1); if (e != cudaSuccess) return e;
    CQPI_SETSMEM(g0_rowfft_kernel<1>) CQPI_SETSMEM(g0_rowfft_kernel<2>) CQPI_SETSMEM(g0_rowfft_kernel<3>)
    CQPI_SETSMEM(g0_rowfft_kernel<4>) CQPI_SETSMEM(g0_rowfft_kernel<6>) CQPI_SETSMEM(g0_rowfft_kernel<8>)
    CQPI_SETSMEM(g0_rowfft_kernel<10>) CQPI_SETSMEM(g0_rowfft_kernel<12>) CQPI_SETSMEM(g0_rowfft_kernel<16>)
#undef CQPI_SETSMEM
    e = cudaFuncSetAttribute(colfft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
    if (e != cudaSuccess) return e;
    if (!rowfft_reg_ok(h)) return cudaSuccess;
    e = configure_rowfft_reg(h);
    if (e != cudaSuccess) return e;
    e = configure_rowfft_g0k(h);
    if (e != cudaSuccess) return e;
    return configure_colfft_reg(h);
}

template <int B>
static void launch_rowfft(cqpi_handle *h, int ne, const double *d_energies, int pg, size_t smem)
{
    g0_rowfft_kernel<B><<<h->kp, 256, smem, h->stream>>>(h->b, h->kp, ilog2i(h->kp), h->NB, h->Rb, pg, h->eta,
                                                         d_energies, ne, h->d_eval, h->d_evec32, h->d_tw32,
                                                         h->ws.half32);
}

// register four-step variant: kp = N1 x N2 in {64 ... 4096} and a box no wider than kp
static bool rowfft_reg_ok(const cqpi_handle *h) { return h->kp >= 64 && h->kp <= 4096 && h->NB <= h->kp; }

// planes the fused row transform carries: the upper triangle under reciprocity (real hoppings,
// CQPI_RECIPROCITY=0 disables), else all b^2
// (both transforms must be the register kernels: the radix-2 ones carry every plane)
static int rowfft_planes(const cqpi_handle *h)
{
    const char *f = getenv("CQPI_RECIPROCITY");
    const char *fr = getenv("CQPI_ROWFFT");
    const char *fc = getenv("CQPI_COLFFT");
    const bool tr = h->time_reversal && !(f && !strcmp(f, "0")) && !(fr && !strcmp(fr, "radix2")) &&
                    !(fc && !strcmp(fc, "radix2"));
    return tr ? h->b * (h->b + 1) / 2 : h->b * h->b;
}

// all = true: the largest group any hopping set can need (for the shared-memory limit)
static int rowfft_reg_plane_group(const cqpi_handle *h, bool all = false)
{
    const size_t plen = (size_t)h->kp + (h->kp >> 5) + 1;
    int pg = (int)((96 * 1024 - 8 * (size_t)h->kp) / (8 * plen));
    return std::max(1, std::min(pg, all ? h->b * h->b : rowfft_planes(h)));
}

// bytes of one k_x row of the eigen cache (FP64 eigenvalues, FP32 eigenvectors)
static size_t rowfft_eig_bytes(const cqpi_handle *h) { return (size_t)h->kp * (8 * h->b + 8 * h->b * h->b); }   // float2 pairs

// shared memory of the register row transform: pg planes, the twiddles and, when it fits
// in 227 KiB, the row's eigen cache
static size_t rowfft_reg_smem(const cqpi_handle *h, bool *eig_smem, bool all = false)
{
    const int pg = rowfft_reg_plane_group(h, all);
    const size_t base = 8 * ((size_t)pg * (h->kp + h->kp / 32 + 1) + h->kp);
    const bool fits = base + rowfft_eig_bytes(h) <= 227 * 1024;
    if (eig_smem) *eig_smem = fits;
    return fits ? base + rowfft_eig_bytes(h) : base;
}

// block size: one thread per (plane, n1) / (plane, k2) transform of a plane group, so that
// both passes run in one round (e.g. 9 planes x 32 = 288 for three bands and kp = 1024)
template <int N1, int N2, int MAXT>
static int rowfft_reg_threads(const cqpi_handle *h)
{
    const int pg = rowfft_reg_plane_group(h);
    const int t = ((pg * std::max(N1, N2) + 31) / 32) * 32;
    return std::max(64, std::min(MAXT, t));
}

template <int N1, int N2, int MAXT = 256>
static void launch_rowfft_reg_t(cqpi_handle *h, int ne, const double *d_energies)
{
    const int pg = rowfft_reg_plane_group(h);
    bool eig = false;
    size_t smem = rowfft_reg_smem(h, &eig);
    // a small block (up to 6 warps: the 6 reciprocity planes of 3 bands) runs faster as two
    // blocks per SM reading the row's eigen data through L2 than as one block with it in
    // shared memory (measured: C2 G0 + transforms 7.1 -> 6.0 ms per job)
    const int threads = rowfft_reg_threads<N1, N2, MAXT>(h);
    const size_t base = eig ? smem - rowfft_eig_bytes(h) : smem;
    const bool two = threads <= 192 && 2 * base <= 227 * 1024;
    const char *f = getenv("CQPI_ROWFFT_EIG");
    if (eig && (two || (f && !strcmp(f, "global"))) && !(f && !strcmp(f, "smem"))) {
        eig = false;
        smem = base;
    }
    const int tr = rowfft_planes(h) != h->b * h->b ? 1 : 0;
    g0_rowfft_reg_kernel<N1, N2, 4, MAXT><<<h->kp, threads, smem, h->stream>>>(
        h->b, h->NB, h->Rb, pg, eig ? 1 : 0, tr, h->eta, d_energies, ne, h->d_eval32, h->d_evec32, h->d_tw32,
        h->ws.half32);
}

// shared memory of the persistent row transform at kp = 1024: np planes and the twiddles
static size_t rowfft_pk_smem(int np) { return 8 * ((size_t)np * (1024 + 1024 / 32 + 1) + 1024); }

// the persistent row transform (kp = 1024, up to 3 bands); CQPI_ROWFFT=classic keeps the
// one-block-per-row kernel
static bool rowfft_pk_ok(const cqpi_handle *h)
{
    const char *f = getenv("CQPI_ROWFFT");
    return h->kp == 1024 && h->b <= 3 && h->NB <= h->kp && !(f && !strcmp(f, "classic"));
}

template <int B>
static void launch_rowfft_pk(cqpi_handle *h, int ne, const double *d_energies)
{
    const int np = rowfft_planes(h);
    const int tr = np != B * B ? 1 : 0;
    const int threads = np * 32;
    const size_t smem = rowfft_pk_smem(np);
    // resident blocks per SM for this block size and shared memory (same on every GB300)
    static int per_sm[2][4] = {};
    int &r = per_sm[tr][B];
    if (r == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, g0_rowfft_pk_kernel<32, 32, B>, threads, smem) !=
                       cudaSuccess || r < 1))
        r = 1;
    const long long items = 1024LL * ne;
    const int grid = (int)std::min<long long>(items, (long long)h->num_sms * r);
    g0_rowfft_pk_kernel<32, 32, B><<<grid, threads, smem, h->stream>>>(h->NB, h->Rb, tr, h->eta, d_energies, ne,
                                                                       h->d_eval32, h->d_evec32, h->d_tw32,
                                                                       h->ws.half32);
}

static cudaError_t configure_rowfft_reg(cqpi_handle *h)
{
    // the largest launch: every plane, or the reciprocity planes with the eigen cache
    const int smem = (int)std::max(rowfft_reg_smem(h, nullptr, true), rowfft_reg_smem(h, nullptr, false));
    switch (h->kp) {
    case 64: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 128: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<8, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 256: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<16, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 512: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<16, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 1024: {
        // the persistent kernel (up to 3 bands): every plane (at most 9) plus the twiddles
        if (h->b <= 3) {
            const int pk = (int)rowfft_pk_smem(9);
            cudaError_t e = cudaFuncSetAttribute(g0_rowfft_pk_kernel<32, 32, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, pk);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(g0_rowfft_pk_kernel<32, 32, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, pk);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(g0_rowfft_pk_kernel<32, 32, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, pk);
            if (e != cudaSuccess) return e;
        }
        return cudaFuncSetAttribute(g0_rowfft_reg_kernel<32, 32, 4, 288>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }
    case 2048: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<32, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 4096: return cudaFuncSetAttribute(g0_rowfft_reg_kernel<64, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }
    return cudaSuccess;
}

template <int N1, int N2>
static size_t colfft_reg_smem()
{
    return 8 * ((size_t)(256 / N1) * (N1 * N2 + (N1 * N2) / 32 + 1) + N1 * N2);
}

template <int N1, int N2>
static cudaError_t configure_colfft_reg_t()
{
    return cudaFuncSetAttribute(colfft_reg_kernel<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)colfft_reg_smem<N1, N2>());
}

template <int N1, int N2>
static void launch_colfft_reg_t(cqpi_handle *h, int ne, int tr)
{
    constexpr int NC = 256 / N1;
    const int np = tr ? h->b * (h->b + 1) / 2 : h->b * h->b;
    dim3 grid(cdiv(h->NB, NC), np, ne);
    colfft_reg_kernel<N1, N2><<<grid, 256, colfft_reg_smem<N1, N2>(), h->stream>>>(
        h->NB, h->Rb, h->b, np, tr, (float)(1.0 / ((double)h->kp * h->kp)), h->ws.half32, h->d_tw32, h->ws.box32,
        h->ws.gmax);
}

static cudaError_t configure_colfft_reg(cqpi_handle *h)
{
    switch (h->kp) {
    case 64: return configure_colfft_reg_t<8, 8>();
    case 128: return configure_colfft_reg_t<8, 16>();
    case 256: return configure_colfft_reg_t<16, 16>();
    case 512: return configure_colfft_reg_t<16, 32>();
    case 1024: return configure_colfft_reg_t<32, 32>();
    case 2048: return configure_colfft_reg_t<32, 64>();
    case 4096: return configure_colfft_reg_t<64, 64>();
    }
    return cudaSuccess;
}

template <int N1, int N2>
static size_t rowfft_g0k_smem()
{
    constexpr int RPC = rowfft_g0k_rpc<N1, N2>();
    return 8 * ((size_t)RPC * (N1 * N2 + (N1 * N2) / 32 + 1) + N1 * N2);
}

template <int N1, int N2>
static cudaError_t configure_rowfft_g0k_t()
{
    return cudaFuncSetAttribute(rowfft_reg_g0k_kernel<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)rowfft_g0k_smem<N1, N2>());
}

static cudaError_t configure_rowfft_g0k(cqpi_handle *h)
{
    switch (h->kp) {
    case 64: return configure_rowfft_g0k_t<8, 8>();
    case 128: return configure_rowfft_g0k_t<8, 16>();
    case 256: return configure_rowfft_g0k_t<16, 16>();
    case 512: return configure_rowfft_g0k_t<16, 32>();
    case 1024: return configure_rowfft_g0k_t<32, 32>();
    case 2048: return configure_rowfft_g0k_t<32, 64>();
    case 4096: return configure_rowfft_g0k_t<64, 64>();
    }
    return cudaSuccess;
}

template <int N1, int N2>
static void launch_rowfft_g0k_t(cqpi_handle *h, int ne, int np)
{
    constexpr int RPC = rowfft_g0k_rpc<N1, N2>();
    const long long nrows = (long long)ne * np * h->kp;
    rowfft_reg_g0k_kernel<N1, N2><<<(unsigned)((nrows + RPC - 1) / RPC), 256, rowfft_g0k_smem<N1, N2>(), h->stream>>>(
        h->NB, h->Rb, nrows, h->ws.g0k32, h->d_tw32, h->ws.half32);
}

static void launch_colfft_reg(cqpi_handle *h, int ne, int tr)
{
    switch (h->kp) {
    case 64: launch_colfft_reg_t<8, 8>(h, ne, tr); break;
    case 128: launch_colfft_reg_t<8, 16>(h, ne, tr); break;
    case 256: launch_colfft_reg_t<16, 16>(h, ne, tr); break;
    case 512: launch_colfft_reg_t<16, 32>(h, ne, tr); break;
    case 1024: launch_colfft_reg_t<32, 32>(h, ne, tr); break;
    case 2048: launch_colfft_reg_t<32, 64>(h, ne, tr); break;
    case 4096: launch_colfft_reg_t<64, 64>(h, ne, tr); break;
    }
}

static void launch_rowfft_reg(cqpi_handle *h, int ne, const double *d_energies)
{
    switch (h->kp) {
    case 64: launch_rowfft_reg_t<8, 8>(h, ne, d_energies); break;
    case 128: launch_rowfft_reg_t<8, 16>(h, ne, d_energies); break;
    case 256: launch_rowfft_reg_t<16, 16>(h, ne, d_energies); break;
    case 512: launch_rowfft_reg_t<16, 32>(h, ne, d_energies); break;
    case 1024:
        if (rowfft_pk_ok(h)) {
            if (h->b == 1) launch_rowfft_pk<1>(h, ne, d_energies);
            else if (h->b == 2) launch_rowfft_pk<2>(h, ne, d_energies);
            else launch_rowfft_pk<3>(h, ne, d_energies);
        } else {
            launch_rowfft_reg_t<32, 32, 288>(h, ne, d_energies);
        }
        break;
    case 2048: launch_rowfft_reg_t<32, 64>(h, ne, d_energies); break;
    case 4096: launch_rowfft_reg_t<64, 64>(h, ne, d_energies); break;
    }
}

void launch_greens_fft32(cqpi_handle *h, int ne, const double *d_energies)
{
    const int pg = rowfft_plane_group(h);
    const size_t s1 = 8 * ((size_t)pg * (h->kp + (h->kp >> 5) + 1) + h->kp / 2);
    const int b = h->b;
    const char *force = getenv("CQPI_ROWFFT");
    if (rowfft_reg_ok(h) && !(force && !strcmp(force, "radix2"))) launch_rowfft_reg(h, ne, d_energies);
    else if (b <= 1) launch_rowfft<1>(h, ne, d_energies, pg, s1);
    else if (b <= 2) launch_rowfft<2>(h, ne, d_energies, pg, s1);
    else if (b <= 3) launch_rowfft<3>(h, ne, d_energies, pg, s1);
    else if (b <= 4) launch_rowfft<4>(h, ne, d_energies, pg, s1);
    else if (b <= 6) launch_rowfft<6>(h, ne, d_energies, pg, s1);
    else if (b <= 8) launch_rowfft<8>(h, ne, d_energies, pg, s1);
    else if (b <= 10) launch_rowfft<10>(h, ne, d_energies, pg, s1);
    else if (b <= 12) launch_rowfft<12>(h, ne, d_energies, pg, s1);
    else launch_rowfft<16>(h, ne, d_energies, pg, s1);
    h->launches++;
    const char *fc = getenv("CQPI_COLFFT");
    if (rowfft_reg_ok(h) && !(fc && !strcmp(fc, "radix2"))) {
        launch_colfft_reg(h, ne, rowfft_planes(h) != b * b ? 1 : 0);
    } else {
        const int lnc = colfft_lnc(h->kp), NC = 1 << lnc;
        const size_t s2 = 8 * ((size_t)h->kp * NC + h->kp / 2);
        dim3 grid(cdiv(h->NB, NC), h->b * h->b, ne);
        colfft_kernel<<<grid, 256, s2, h->stream>>>(h->kp, ilog2i(h->kp), h->NB, h->Rb, h->b * h->b, lnc,
                                                    (float)(1.0 / ((double)h->kp * h->kp)), h->ws.half32, h->d_tw32,
                                                    h->ws.box32, h->ws.gmax);
    }
    h->launches++;
}

static bool fft32_planes_ok(const cqpi_handle *h)
{
    const char *force = getenv("CQPI_ROWFFT");
    return fft32_supported(h) && rowfft_reg_ok(h) && !(force && !strcmp(force, "radix2"));
}

// The unfused mixed path of the normal Green's function transforms only the b(b+1)/2
// reciprocity planes when the hoppings are real (greens_k_kernel then writes those planes, in
// the upper-triangle order, and the column kernel fills the rest of the box by reflection).
bool g0k_reciprocity(const cqpi_handle *h)
{
    return h->precision == CQPI_PREC_MIXED && h->gmode == CQPI_GREEN_NORMAL && fft32_planes_ok(h) &&
           rowfft_planes(h) != h->b * h->b;
}

// Transforms of the unfused mixed path (G0(k) planes in ws.g0k32) with the register
// four-step kernels; false when the k-grid is outside their range (the radix-2 kernels of
// greens.cu run instead).
bool launch_fft32_planes(cqpi_handle *h, int ne)
{
    if (!fft32_planes_ok(h)) return false;
    const bool tr = g0k_reciprocity(h);
    const int np = tr ? rowfft_planes(h) : h->b * h->b;
    switch (h->kp) {
    case 64: launch_rowfft_g0k_t<8, 8>(h, ne, np); break;
    case 128: launch_rowfft_g0k_t<8, 16>(h, ne, np); break;
    case 256: launch_rowfft_g0k_t<16, 16>(h, ne, np); break;
    case 512: launch_rowfft_g0k_t<16, 32>(h, ne, np); break;
    case 1024: launch_rowfft_g0k_t<32, 32>(h, ne, np); break;
    case 2048: launch_rowfft_g0k_t<32, 64>(h, ne, np); break;
    case 4096: launch_rowfft_g0k_t<64, 64>(h, ne, np); break;
    }
    h->launches++;
    launch_colfft_reg(h, ne, tr ? 1 : 0);
    h->launches++;
    return true;
}

}  // namespace cqpi
