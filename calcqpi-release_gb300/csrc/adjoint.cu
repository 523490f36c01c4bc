// adjoint.cu -- reverse-mode derivative of the continuum-LDOS pipeline: given
// W = dL/drho for every map of a run, the gradient of L with respect to the model's
// hopping amplitudes t and every impurity matrix V.
//
// Forward chain (one spin block):
//   H(k) = D + sum_R tn(R) e^{+i th} + ta(R) e^{-i th}            (bands.cu)
//   G(k) = (z - H(k))^{-1} = U diag(f) U^H,  f_n = 1/(omega + i eta - eps_n)
//   G(R) = kp^-2 sum_k e^{+2 pi i k.R / kp} G(k)                    (greens.cu / fft32.cu)
//   T    = (1 - V g)^{-1} V,  g = G(0)                               (tmatrix_kernel)
//   u_a  = sum_{d,o} phi_o(q,d) G(p+d)[o][a],  s_c = sum_{d,o} G(-p-d)[c][o] phi_o(q,d)
//   rho  = -term1(q) - Im(sum_ac u_a T_ac s_c),
//   term1(q) = sum_{d1,d2,o1,o2} phi_o1(q,d1) phi_o2(q,d2) Im G(d2-d1)[o2][o1]
// (src/qpi.cc:454-486, 557-578, 833-854, 876-950).  Gradients of real L with respect to a
// complex z are written zbar = dL/dRe z + i dL/dIm z; for L = -W Im(c z) this is
// zbar = -i W conj(c), and a holomorphic linear map z -> y = P z Q pulls back as
// zbar = P^H ybar Q^H.  The adjoint recomputes G(R) and T per energy (nothing of the
// forward run is stored) and goes back through:
//   1. adj_contract_kernel: u, s per pixel; ubar = -i W conj(T s), sbar = -i W conj(u T);
//      per site the window gradients phi^T ubar / phi^T sbar (one value per window entry,
//      stored) and the site's part of M = sum W u s^T (-> Tbar = -i conj M);
//      adj_gather_kernel sums the window gradients of the sites whose windows cover a box
//      point into the G(R) box gradient (no atomics), adj_mreduce_kernel the M parts, and
//      adj_wsum_kernel forms sum_p W per sub-pixel for the term1 part.
//   2. adj_term1_kernel: term1 part of the box gradient.
//   3. adj_tv_kernel: gbar(0) += T^H Tbar T^H, Vbar += A^-H Tbar (1 + g T)^H, A = 1 - V g.
//   4. adj_cols_kernel / adj_rows_kernel: Gbar(k) = kp^-2 sum_R e^{-2 pi i k.R/kp} Gbar(R)
//      (the forward's pruned transform read backwards: box -> full k-grid, FP64).
//   5. adj_kacc_kernel: Hbar(k) = G^H Gbar G^H = U [F* (U^H Gbar U) F*] U^H; the bracket
//      is accumulated over energies per k in FP64, U [..] U^H is applied once at the end
//      (adj_hbar_kernel).
//   6. adj_hop_kernel: tbar for every unique R, normal and conjugated terms:
//      sum_k e^{-/+ i th(k)} Hbar(k)[p][q] (FP64 sums over the k-grid).
// The contraction adjoint computes in the handle's precision (FP32 with the mixed box,
// FP64 with the FP64 box) and accumulates in FP64; steps 4-5 follow the handle's precision
// too (FP32 transform and per-k rotation for the mixed handle, the energy sum of C(k) in
// FP64); steps 2, 3 and 6 are FP64.
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "cplx.h"
#include "cqpi_internal.h"
#include "fft_reg.cuh"

namespace cqpi {

namespace {

__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ void atomic_add2(double2 *p, double2 v)
{
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}

}  // namespace

// ------------------------------------------------------------------ 1. contraction adjoint
// grid (n*n sites, ne*nimp maps), block: one thread per sub-pixel q (Q <= 128).
// Outputs of site p and map ei (nsite = n*n, t = d*mb + o a window entry, Wmb = W*mb):
//   Ub[((ei*Wmb + t)*b + a)*nsite + p] = sum_q phi_o(q,d) ubar_a(p,q)   (-> Gbar(p+d)[o][a])
//   Sb[((ei*Wmb + t)*b + c)*nsite + p] = sum_q phi_o(q,d) sbar_c(p,q)   (-> Gbar(-p-d)[c][o])
//   Mp[(ei*nsite + p)*b*b + a*b + c]  = sum_q W u_a s_c
template <int B, class C>
__global__ void __launch_bounds__(128) adj_contract_kernel(int b, int n, int os, int w, int Rb, int NB, int Q, int W, int nimp,
                                                           int mb, int bs0, const typename real_of<C>::type *__restrict__ phi,
                                                           const C *__restrict__ box, const double2 *__restrict__ T,
                                                           const float *__restrict__ wmap, C *__restrict__ Ub,
                                                           C *__restrict__ Sb, double2 *__restrict__ Mp)
{
    using Rl = typename real_of<C>::type;
    extern __shared__ __align__(16) unsigned char adj_sm[];
    Rl *ubr = reinterpret_cast<Rl *>(adj_sm);               // [128][b] each: ubar, sbar (re, im)
    Rl *ubi = ubr + 128 * b, *sbr = ubi + 128 * b, *sbi = sbr + 128 * b;
    double2 *mred = reinterpret_cast<double2 *>(sbi + 128 * b);   // [4 warps][b*b]
    const int site = blockIdx.x, ei = blockIdx.y;
    const int e = ei / nimp;
    const int nsite = n * n;
    const int i = site / n, j = site % n;
    const int n2 = n >> 1, px = i - n2, py = j - n2;
    const int wn = n * os, bb = b * b, side = 2 * w + 1;
    const int q = threadIdx.x;
    const bool qv = q < Q;
    const int qx = qv ? q / os : 0, qy = qv ? q % os : 0;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    const double2 *Te = T + (size_t)ei * bb;
    const Rl *ph = phi + (size_t)q * W * mb;

    Rl W_ = 0;
    Rl ur[B], ui[B], sr[B], si[B];
#pragma unroll
    for (int a = 0; a < B; a++) { ur[a] = 0; ui[a] = 0; sr[a] = 0; si[a] = 0; }
    if (qv) {
        W_ = (Rl)wmap[((size_t)ei * wn + (size_t)j * os + qy) * wn + (size_t)i * os + qx];
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            const C *gs = boxe + ((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb;
            const C *gu = boxe + ((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb;
            for (int ol = 0; ol < mb; ol++) {
                const Rl f = ph[d * mb + ol];
                if (f == (Rl)0) continue;
                const int o = bs0 + ol;
#pragma unroll
                for (int a = 0; a < B; a++) {
                    if (a < b) {
                        const C vs = gs[a * b + o], vu = gu[o * b + a];
                        sr[a] += vs.x * f; si[a] += vs.y * f;
                        ur[a] += vu.x * f; ui[a] += vu.y * f;
                    }
                }
            }
        }
    }
    // ts = T s, ut = u^T T; ubar = -i W conj(ts), sbar = -i W conj(ut)
#pragma unroll
    for (int a = 0; a < B; a++) {
        Rl tsr = 0, tsi = 0, utr = 0, uti = 0;
        if (a < b) {
#pragma unroll
            for (int c = 0; c < B; c++) {
                if (c < b) {
                    const double2 t = Te[a * b + c];      // T_ac
                    tsr += (Rl)t.x * sr[c] - (Rl)t.y * si[c];
                    tsi += (Rl)t.x * si[c] + (Rl)t.y * sr[c];
                    const double2 t2 = Te[c * b + a];     // T_ca
                    utr += ur[c] * (Rl)t2.x - ui[c] * (Rl)t2.y;
                    uti += ur[c] * (Rl)t2.y + ui[c] * (Rl)t2.x;
                }
            }
        }
        if (a < b) {
            ubr[q * b + a] = -W_ * tsi; ubi[q * b + a] = -W_ * tsr;
            sbr[q * b + a] = -W_ * uti; sbi[q * b + a] = -W_ * utr;
        }
    }
    // M_ac = sum_q W u_a s_c: warp sums, then the four warps' sums in shared memory
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
        for (int c = 0; c < B; c++) {
            if (a >= b || c >= b) continue;
            double mr = qv ? (double)W_ * ((double)ur[a] * sr[c] - (double)ui[a] * si[c]) : 0.0;
            double mi = qv ? (double)W_ * ((double)ur[a] * si[c] + (double)ui[a] * sr[c]) : 0.0;
            for (int o = 16; o > 0; o >>= 1) {
                mr += __shfl_xor_sync(0xffffffffu, mr, o);
                mi += __shfl_xor_sync(0xffffffffu, mi, o);
            }
            if (lane == 0) mred[warp * bb + a * b + c] = make_double2(mr, mi);
        }
    __syncthreads();
    for (int k = threadIdx.x; k < bb; k += blockDim.x) {
        double2 m = make_double2(0.0, 0.0);
        for (int wv = 0; wv < (int)(blockDim.x >> 5); wv++) m = cadd(m, mred[wv * bb + k]);
        Mp[((size_t)ei * nsite + site) * bb + k] = m;
    }
    // window gradients of this site: entry (d, o) of phi^T ubar and of phi^T sbar
    const int Wmb = W * mb;
    for (int t = threadIdx.x; t < Wmb; t += blockDim.x) {
        const int d = t / mb, ol = t - d * mb;
        Rl gur[B], gui[B], gsr[B], gsi[B];
#pragma unroll
        for (int a = 0; a < B; a++) { gur[a] = 0; gui[a] = 0; gsr[a] = 0; gsi[a] = 0; }
        for (int qq = 0; qq < Q; qq++) {
            const Rl f = phi[((size_t)qq * W + d) * mb + ol];
            if (f == (Rl)0) continue;
#pragma unroll
            for (int a = 0; a < B; a++) {
                if (a < b) {
                    gur[a] += f * ubr[qq * b + a]; gui[a] += f * ubi[qq * b + a];
                    gsr[a] += f * sbr[qq * b + a]; gsi[a] += f * sbi[qq * b + a];
                }
            }
        }
#pragma unroll
        for (int a = 0; a < B; a++) {
            if (a < b) {
                const size_t idx = (((size_t)ei * Wmb + t) * b + a) * nsite + site;
                Ub[idx] = cmake<C>(gur[a], gui[a]);
                Sb[idx] = cmake<C>(gsr[a], gsi[a]);
            }
        }
    }
}

// The same outputs with one warp per site (up to 4 bands): the orbital table phi is staged in
// shared memory as [entry t][q] (row stride QP = 129 words, zero past Q), lane l handles the
// pixels q = l + 32k (k < 4) in the forward part, so every window value G(R)[o][a] loaded for a
// site feeds 4 pixels, and the entries t = l + 32m in the window-gradient part, so every
// ubar / sbar row read feeds 3 entries.  grid (ceil(n*n / wpb), ne*nimp), wpb warps: the orbital
// table is shared by the block's sites, and 10 FP32 warps (two blocks of 100 KB per SM for the
// C2 orbitals) keep 20 warps resident instead of the 12 of three 4-warp blocks.
constexpr int ADJ_QP = 129;
// warps (sites) per block: 10 for the FP32 working type; the FP64 one keeps 4 warps per block,
// whose larger register budget it needs
template <class C> struct AdjWpb { static constexpr int value = 10, blocks = 2; };
template <> struct AdjWpb<double2> { static constexpr int value = 4, blocks = 1; };
template <int B, class C>
__global__ void __launch_bounds__(32 * AdjWpb<C>::value, AdjWpb<C>::blocks) adj_contract_warp_kernel(int b, int n, int os, int w, int Rb, int NB, int Q, int W,
                                                                int nimp, int mb, int bs0,
                                                                const typename real_of<C>::type *__restrict__ phi,
                                                                const C *__restrict__ box, const double2 *__restrict__ T,
                                                                const float *__restrict__ wmap, C *__restrict__ Ub,
                                                                C *__restrict__ Sb, double2 *__restrict__ Mp)
{
    using Rl = typename real_of<C>::type;
    extern __shared__ __align__(16) unsigned char adj_sm[];
    const int Wmb = W * mb;
    Rl *phT = reinterpret_cast<Rl *>(adj_sm);                     // [Wmb][ADJ_QP]
    Rl *ubs = phT + (size_t)Wmb * ADJ_QP;                          // [warp][128 q][b][4]: ubar re, im, sbar re, im
    for (int i = threadIdx.x; i < Wmb * ADJ_QP; i += blockDim.x) {
        const int t = i / ADJ_QP, q = i - t * ADJ_QP;
        phT[i] = q < Q ? phi[(size_t)q * Wmb + t] : (Rl)0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nsite = n * n, site = blockIdx.x * AdjWpb<C>::value + warp;
    if (site >= nsite) return;
    const int ei = blockIdx.y, e = ei / nimp;
    const int i = site / n, j = site % n;
    const int n2 = n >> 1, px = i - n2, py = j - n2;
    const int wn = n * os, bb = b * b, side = 2 * w + 1;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    const double2 *Te = T + (size_t)ei * bb;
    // forward part: u_a(q), s_a(q) for the 4 pixel slots of this lane
    Rl ur[4][B], ui[4][B], sr[4][B], si[4][B];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int a = 0; a < B; a++) { ur[k][a] = 0; ui[k][a] = 0; sr[k][a] = 0; si[k][a] = 0; }
    // the site's window values G(p+d)[o][a] and G(-p-d)[a][o], staged by the warp in its ubar /
    // sbar region (free until the forward part is done) when they fit: [u/s][t][a] complex
    Rl *ub = ubs + (size_t)warp * 128 * b * 4;
    const bool staged = Wmb <= 128;
    if (staged) {
        for (int idx = lane; idx < 2 * Wmb * b; idx += 32) {
            const int op = idx / (Wmb * b), rest = idx - op * Wmb * b;
            const int t = rest / b, a = rest - t * b;
            const int d = t / mb, o = bs0 + (t - d * mb);
            const int dx = d / side - w, dy = d % side - w;
            const C v = op == 0 ? boxe[((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb + o * b + a]
                                : boxe[((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb + a * b + o];
            ub[2 * idx] = v.x;
            ub[2 * idx + 1] = v.y;
        }
        __syncwarp();
    }
    for (int d = 0; d < W; d++) {
        const int dx = d / side - w, dy = d % side - w;
        const C *gs = boxe + ((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb;
        const C *gu = boxe + ((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb;
#pragma unroll 3
        for (int ol = 0; ol < mb; ol++) {
            const int o = bs0 + ol, t = d * mb + ol;
            C vu[B], vs[B];
            if (staged) {
                const Rl *wu = ub + 2 * (t * b), *ws = ub + 2 * ((Wmb + t) * b);
#pragma unroll
                for (int a = 0; a < B; a++)
                    if (a < b) { vu[a] = cmake<C>(wu[2 * a], wu[2 * a + 1]); vs[a] = cmake<C>(ws[2 * a], ws[2 * a + 1]); }
            } else {
#pragma unroll
                for (int a = 0; a < B; a++)
                    if (a < b) { vu[a] = gu[o * b + a]; vs[a] = gs[a * b + o]; }
            }
            const Rl *pt = phT + (size_t)t * ADJ_QP + lane;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const Rl f = pt[32 * k];
#pragma unroll
                for (int a = 0; a < B; a++)
                    if (a < b) {
                        ur[k][a] += vu[a].x * f; ui[k][a] += vu[a].y * f;
                        sr[k][a] += vs[a].x * f; si[k][a] += vs[a].y * f;
                    }
            }
        }
    }
    // ubar = -i W conj(T s), sbar = -i W conj(u^T T); M_ac = sum_q W u_a s_c (the staged windows
    // are read by every lane before the region is overwritten)
    __syncwarp();
    // M partials of the lane's pixels in the working precision; the warp and site sums in FP64
    Rl mr[B][B], mi[B][B];
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
        for (int c = 0; c < B; c++) { mr[a][c] = 0; mi[a][c] = 0; }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int q = lane + 32 * k;
        const bool qv = q < Q;
        const int qx = qv ? q / os : 0, qy = qv ? q % os : 0;
        const Rl W_ = qv ? (Rl)wmap[((size_t)ei * wn + (size_t)j * os + qy) * wn + (size_t)i * os + qx] : (Rl)0;
#pragma unroll
        for (int a = 0; a < B; a++) {
            if (a >= b) continue;
            Rl tsr = 0, tsi = 0, utr = 0, uti = 0;
#pragma unroll
            for (int c = 0; c < B; c++) {
                if (c >= b) continue;
                const double2 t = Te[a * b + c];      // T_ac
                tsr += (Rl)t.x * sr[k][c] - (Rl)t.y * si[k][c];
                tsi += (Rl)t.x * si[k][c] + (Rl)t.y * sr[k][c];
                const double2 t2 = Te[c * b + a];     // T_ca
                utr += ur[k][c] * (Rl)t2.x - ui[k][c] * (Rl)t2.y;
                uti += ur[k][c] * (Rl)t2.y + ui[k][c] * (Rl)t2.x;
                mr[a][c] += W_ * (ur[k][a] * sr[k][c] - ui[k][a] * si[k][c]);
                mi[a][c] += W_ * (ur[k][a] * si[k][c] + ui[k][a] * sr[k][c]);
            }
            Rl *u4 = ub + ((size_t)q * b + a) * 4;
            u4[0] = -W_ * tsi; u4[1] = -W_ * tsr; u4[2] = -W_ * uti; u4[3] = -W_ * utr;
        }
    }
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
        for (int c = 0; c < B; c++) {
            if (a >= b || c >= b) continue;
            double x = (double)mr[a][c], y = (double)mi[a][c];
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                y += __shfl_xor_sync(0xffffffffu, y, o);
            }
            if (lane == 0) Mp[((size_t)ei * nsite + site) * bb + a * b + c] = make_double2(x, y);
        }
    __syncwarp();
    // window gradients: entries t = t0 + lane + 32 m, 3 per lane per round
    for (int t0 = 0; t0 < Wmb; t0 += 96) {
        Rl gur[3][B], gui[3][B], gsr[3][B], gsi[3][B];
#pragma unroll
        for (int m = 0; m < 3; m++)
#pragma unroll
            for (int a = 0; a < B; a++) { gur[m][a] = 0; gui[m][a] = 0; gsr[m][a] = 0; gsi[m][a] = 0; }
        for (int q = 0; q < Q; q++) {
            Rl f[3];
#pragma unroll
            for (int m = 0; m < 3; m++) {
                const int t = t0 + lane + 32 * m;
                f[m] = t < Wmb ? phT[(size_t)t * ADJ_QP + q] : (Rl)0;
            }
#pragma unroll
            for (int a = 0; a < B; a++) {
                if (a >= b) continue;
                const Rl *u4 = ub + ((size_t)q * b + a) * 4;
                const Rl x0 = u4[0], x1 = u4[1], x2 = u4[2], x3 = u4[3];
#pragma unroll
                for (int m = 0; m < 3; m++) {
                    gur[m][a] += f[m] * x0; gui[m][a] += f[m] * x1;
                    gsr[m][a] += f[m] * x2; gsi[m][a] += f[m] * x3;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const int t = t0 + lane + 32 * m;
            if (t >= Wmb) continue;
#pragma unroll
            for (int a = 0; a < B; a++) {
                if (a >= b) continue;
                const size_t idx = (((size_t)ei * Wmb + t) * b + a) * nsite + site;
                Ub[idx] = cmake<C>(gur[m][a], gui[m][a]);
                Sb[idx] = cmake<C>(gsr[m][a], gsi[m][a]);
            }
        }
    }
}

// Box gradient from the stored window gradients: for box point R and element (r1, r2),
//   Gbar(R)[r1][r2] += sum_{imp, d} Ub[(d, r1-bs0)][r2] of site R - d      (r1 in the block)
//                    + sum_{imp, d} Sb[(d, r2-bs0)][r1] of site -R - d     (r2 in the block)
// over the sites inside the field of view.  grid (ceil(NB/128), NB, ne*b*b); thread = Y.
template <class C>
__global__ void __launch_bounds__(128) adj_gather_kernel(int b, int n, int w, int Rb, int NB, int W, int mb, int bs0, int nimp,
                                                         const C *__restrict__ Ub, const C *__restrict__ Sb,
                                                         double2 *__restrict__ gbox)
{
    const int yb = blockIdx.x * blockDim.x + threadIdx.x, xb = blockIdx.y;
    const int bb = b * b;
    const int e = blockIdx.z / bb, el = blockIdx.z - e * bb, r1 = el / b, r2 = el - r1 * b;
    if (yb >= NB) return;
    const int n2 = n >> 1, side = 2 * w + 1, nsite = n * n, Wmb = W * mb;
    const int X = xb - Rb, Y = yb - Rb;
    const int ou = r1 - bs0, os_ = r2 - bs0;
    // FP64 sums for the FP64 working type; FP32 with compensation (Kahan) for the mixed
    // handle's FP32 window gradients (FP64 adds run at 1/64 of the FP32 rate here)
    constexpr bool F32 = std::is_same<C, float2>::value;
    double sx = 0.0, sy = 0.0;
    float fx = 0.f, fy = 0.f, cx = 0.f, cy = 0.f;
    auto add = [&](C v) {
        if constexpr (F32) {
            const float yx = (float)v.x - cx, tx = fx + yx;
            cx = (tx - fx) - yx;
            fx = tx;
            const float yy = (float)v.y - cy, ty = fy + yy;
            cy = (ty - fy) - yy;
            fy = ty;
        } else {
            sx += (double)v.x;
            sy += (double)v.y;
        }
    };
    for (int imp = 0; imp < nimp; imp++) {
        const int ei = e * nimp + imp;
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            if (ou >= 0 && ou < mb) {
                const int i = X - dx + n2, j = Y - dy + n2;    // site R - d
                if (i >= 0 && i < n && j >= 0 && j < n) {
                    add(Ub[(((size_t)ei * Wmb + d * mb + ou) * b + r2) * nsite + (size_t)i * n + j]);
                }
            }
            if (os_ >= 0 && os_ < mb) {
                const int i = -X - dx + n2, j = -Y - dy + n2;  // site -R - d
                if (i >= 0 && i < n && j >= 0 && j < n) {
                    add(Sb[(((size_t)ei * Wmb + d * mb + os_) * b + r1) * nsite + (size_t)i * n + j]);
                }
            }
        }
    }
    if constexpr (F32) {
        sx = (double)fx - (double)cx;
        sy = (double)fy - (double)cy;
    }
    double2 *g = gbox + (((size_t)e * NB + xb) * NB + yb) * bb + el;
    *g = make_double2(g->x + sx, g->y + sy);
}

// M[ei] = sum over sites of the per-site parts; one block per map
__global__ void __launch_bounds__(256) adj_mreduce_kernel(int nsite, int bb, const double2 *__restrict__ Mp,
                                                          double2 *__restrict__ M)
{
    // the threads in use are a multiple of bb, so thread t reads the contiguous parts array
    // at stride nt (coalesced) and always the element t % bb; then a fixed-order sum per element
    __shared__ double2 red[256];
    const int ei = blockIdx.x, t = threadIdx.x;
    const int nt = ((int)blockDim.x / bb) * bb;
    double2 sum = make_double2(0.0, 0.0);
    if (t < nt) {
        const double2 *src = Mp + (size_t)ei * nsite * bb;
        const size_t n = (size_t)nsite * bb;
        for (size_t i = t; i < n; i += nt) sum = cadd(sum, src[i]);
    }
    red[t] = sum;
    __syncthreads();
    if (t < bb) {
        double2 u = make_double2(0.0, 0.0);
        for (int v = t; v < nt; v += bb) u = cadd(u, red[v]);
        M[(size_t)ei * bb + t] = u;
    }
}

// The same sum over FP32 per-site parts (the tensor-core contraction adjoint's): per-thread
// sums in FP32 with compensation (Kahan), the fixed-order per-element sum in FP64
__global__ void __launch_bounds__(256) adj_mreduce32_kernel(int nsite, int bb, const float2 *__restrict__ Mp,
                                                            double2 *__restrict__ M)
{
    __shared__ double2 red[256];
    const int ei = blockIdx.x, t = threadIdx.x;
    const int nt = ((int)blockDim.x / bb) * bb;
    float sx = 0.f, sy = 0.f, cx = 0.f, cy = 0.f;
    if (t < nt) {
        const float2 *src = Mp + (size_t)ei * nsite * bb;
        const size_t n = (size_t)nsite * bb;
        for (size_t i = t; i < n; i += nt) {
            const float2 v = src[i];
            const float yx = v.x - cx, tx = sx + yx;
            cx = (tx - sx) - yx;
            sx = tx;
            const float yy = v.y - cy, ty = sy + yy;
            cy = (ty - sy) - yy;
            sy = ty;
        }
    }
    red[t] = make_double2((double)sx - (double)cx, (double)sy - (double)cy);
    __syncthreads();
    if (t < bb) {
        double2 u = make_double2(0.0, 0.0);
        for (int v = t; v < nt; v += bb) u = cadd(u, red[v]);
        M[(size_t)ei * bb + t] = u;
    }
}

// wsum[e][q] = sum over the impurities' maps and the sites of W at sub-pixel q = qx*os + qy.
// One block per (qy, energy of the batch): it reads the map rows y = j*os + qy of every
// impurity, contiguous in x; the threads in use are a multiple of os, so thread t sums the one
// sub-pixel column qx = t % os in a register, and the per-qx partial sums are added in shared
// memory in a fixed order (no atomics; the result does not depend on scheduling).
__global__ void __launch_bounds__(256) adj_wsum_kernel(int wn, int os, int Q, int nimp, const float *__restrict__ wmap,
                                                       double *__restrict__ wsum)
{
    __shared__ double part[256];
    const int qy = blockIdx.x, e = blockIdx.y, t = threadIdx.x;
    const int nt = ((int)blockDim.x / os) * os;
    double acc = 0.0;
    if (t < nt)
        for (int imp = 0; imp < nimp; imp++)
            for (int y = qy; y < wn; y += os) {
                const float *row = wmap + (((size_t)e * nimp + imp) * wn + y) * wn;
                float r = 0.f;
                for (int x = t; x < wn; x += nt) r += row[x];
                acc += (double)r;
            }
    part[t] = acc;
    __syncthreads();
    if (t < os) {
        double sum = 0.0;
        for (int u = t; u < nt; u += os) sum += part[u];
        wsum[(size_t)e * Q + t * os + qy] = sum;
    }
}

// ------------------------------------------------------------------ 2. term1
// rho has -term1, so Gbar(Delta)[o2][o1] += -i sum_q wsum(q) K(q, Delta, o1, o2) with the
// energy-independent K = sum_{d1} phi_o1(q,d1) phi_o2(q,d1+Delta), tabulated once per call:
// Kt[(Delta * mb*mb + o2*mb + o1) * Q + q]; grid (4w+1)^2 offsets Delta, threads over q.
__global__ void __launch_bounds__(128) adj_kt_kernel(int w, int Q, int W, int mb, const double *__restrict__ phi,
                                                     double *__restrict__ Kt)
{
    const int span = 4 * w + 1, side = 2 * w + 1;
    const int rx = blockIdx.x / span - 2 * w, ry = blockIdx.x % span - 2 * w;
    for (int q = threadIdx.x; q < Q; q += blockDim.x)
        for (int o2 = 0; o2 < mb; o2++)
            for (int o1 = 0; o1 < mb; o1++) {
                double k = 0.0;
                for (int d1 = 0; d1 < W; d1++) {
                    const int x2 = d1 / side + rx, y2 = d1 % side + ry;   // window position of d2 = d1 + Delta
                    if (x2 < 0 || x2 >= side || y2 < 0 || y2 >= side) continue;
                    k += phi[((size_t)q * W + d1) * mb + o1] * phi[((size_t)q * W + x2 * side + y2) * mb + o2];
                }
                Kt[(((size_t)blockIdx.x * mb + o2) * mb + o1) * Q + q] = k;
            }
}

// grid ((4w+1)^2 offsets Delta, ne); one thread per orbital pair
__global__ void __launch_bounds__(128) adj_term1_kernel(int b, int w, int Rb, int NB, int Q, int mb, int bs0,
                                                        const double *__restrict__ Kt, const double *__restrict__ wsum,
                                                        double2 *__restrict__ gbox)
{
    const int e = blockIdx.y;
    const int span = 4 * w + 1;
    const int rx = blockIdx.x / span - 2 * w, ry = blockIdx.x % span - 2 * w;
    const int bb = b * b;
    double2 *g = gbox + ((size_t)e * NB * NB + (size_t)(rx + Rb) * NB + (ry + Rb)) * bb;
    for (int t = threadIdx.x; t < mb * mb; t += blockDim.x) {
        const int o2 = t / mb, o1 = t % mb;
        const double *k = Kt + ((size_t)blockIdx.x * mb * mb + t) * Q;
        const double *ws = wsum + (size_t)e * Q;
        double acc = 0.0;
        for (int q = 0; q < Q; q++) acc += ws[q] * k[q];
        if (acc != 0.0) atomicAdd(&g[(bs0 + o2) * b + (bs0 + o1)].y, -acc);
    }
}

// ------------------------------------------------------------------ 3. T-matrix and V
// one thread per (energy, impurity)
template <class C>
__global__ void adj_tv_kernel(int b, int NB, int Rb, int nimp, int ne, const C *__restrict__ box,
                              const double2 *__restrict__ V, const double2 *__restrict__ T,
                              const double2 *__restrict__ Mbuf, double2 *__restrict__ gbox, double2 *__restrict__ gV)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ne * nimp) return;
    const int e = id / nimp, imp = id % nimp;
    const int bb = b * b;
    constexpr int MB = CQPI_MAX_BANDS * CQPI_MAX_BANDS;
    double2 g[MB], A[MB], Ai[MB], Tb[MB], X[MB];
    const C *g0 = box + (((size_t)e * NB + Rb) * NB + Rb) * bb;
    const double2 *v = V + (size_t)imp * bb, *Te = T + (size_t)id * bb, *M = Mbuf + (size_t)id * bb;
    for (int k = 0; k < bb; k++) {
        g[k] = to_d2(g0[k]);
        Tb[k] = make_double2(-M[k].y, -M[k].x);   // Tbar = -i conj(M)
    }
    // A = 1 - V g, Ai = A^-1 (Gauss-Jordan with partial pivoting)
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(v[r * b + k], g[k * b + c]));
            A[r * b + c] = make_double2((r == c ? 1.0 : 0.0) - s.x, -s.y);
            Ai[r * b + c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
        }
    for (int c = 0; c < b; c++) {
        int piv = c;
        double best = -1.0;
        for (int r = c; r < b; r++) {
            const double a = hypot(A[r * b + c].x, A[r * b + c].y);
            if (a > best) { best = a; piv = r; }
        }
        if (!(best > 0.0)) return;   // singular: the forward run reported it
        if (piv != c)
            for (int k = 0; k < b; k++) {
                double2 t0 = A[c * b + k]; A[c * b + k] = A[piv * b + k]; A[piv * b + k] = t0;
                t0 = Ai[c * b + k]; Ai[c * b + k] = Ai[piv * b + k]; Ai[piv * b + k] = t0;
            }
        const double2 p = A[c * b + c];
        const double pd = p.x * p.x + p.y * p.y;
        const double2 pinv = make_double2(p.x / pd, -p.y / pd);
        for (int k = 0; k < b; k++) {
            A[c * b + k] = cmul(A[c * b + k], pinv);
            Ai[c * b + k] = cmul(Ai[c * b + k], pinv);
        }
        for (int r = 0; r < b; r++) {
            if (r == c) continue;
            const double2 f = A[r * b + c];
            for (int k = 0; k < b; k++) {
                A[r * b + k] = csub(A[r * b + k], cmul(f, A[c * b + k]));
                Ai[r * b + k] = csub(Ai[r * b + k], cmul(f, Ai[c * b + k]));
            }
        }
    }
    // gbar(0) += T^H Tbar T^H
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(Tb[r * b + k], cconj(Te[c * b + k])));   // (Tbar T^H)_rc
            X[r * b + c] = s;
        }
    double2 *gz = gbox + (((size_t)e * NB + Rb) * NB + Rb) * bb;
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(cconj(Te[k * b + r]), X[k * b + c]));     // (T^H X)_rc
            atomic_add2(gz + r * b + c, s);
        }
    // Vbar += A^-H Tbar (1 + g T)^H
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(r == c ? 1.0 : 0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(g[r * b + k], Te[k * b + c]));        // (1 + g T)_rc
            A[r * b + c] = s;
        }
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(Tb[r * b + k], cconj(A[c * b + k])));    // (Tbar (1+gT)^H)_rc
            X[r * b + c] = s;
        }
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(cconj(Ai[k * b + r]), X[k * b + c]));    // (A^-H X)_rc
            atomic_add2(gV + (size_t)imp * bb + r * b + c, s);
        }
}

// ------------------------------------------------------------------ 4. box -> k-grid
// In-place radix-2 transform of x[0..kp) (natural order in and out) with e^{-2 pi i t/kp}
// twiddles from tw (e^{+2 pi i t/kp}).
template <class C>
__device__ void fft_minus(C *x, int kp, int logkp, const C *__restrict__ tw)
{
    for (int t = threadIdx.x; t < kp; t += blockDim.x) {
        const int r = logkp ? (int)(__brev((unsigned)t) >> (32 - logkp)) : 0;
        if (r > t) { const C a = x[t]; x[t] = x[r]; x[r] = a; }
    }
    __syncthreads();
    for (int l = 1; l <= logkp; l++) {
        const int len = 1 << l, hl = len >> 1, lstep = logkp - l;   // step = kp / len
        for (int t = threadIdx.x; t < (kp >> 1); t += blockDim.x) {
            const int kk = t & (hl - 1), idx = ((t >> (l - 1)) << l) + kk;
            C wv = __ldg(tw + (kk << lstep));
            wv.y = -wv.y;
            const C u = x[idx], v = cmul(x[idx + hl], wv);
            x[idx] = cadd(u, v);
            x[idx + hl] = csub(u, v);
        }
        __syncthreads();
    }
}

// A[pl][yb][kx] = sum_{X in box} e^{-2 pi i kx X/kp} Gbar(X, Y=yb-Rb)[pl]; grid (NB, bb)
// C: double2 (FP64 handle) or float2 (mixed handle: the k-space steps in FP32, the energy
// sum of C(k) in FP64)
template <class C>
__global__ void __launch_bounds__(256) adj_cols_kernel(int kp, int logkp, int NB, int Rb, int bb, const double2 *__restrict__ gbox,
                                                       const C *__restrict__ tw, C *__restrict__ A)
{
    extern __shared__ __align__(16) unsigned char adj_xs_raw[];
    C *xs = reinterpret_cast<C *>(adj_xs_raw);
    const int yb = blockIdx.x, pl = blockIdx.y;
    for (int pos = threadIdx.x; pos < kp; pos += blockDim.x) {
        double2 s = make_double2(0.0, 0.0);
        // box columns X = xb - Rb with X == pos (mod kp)
        int xb = ((pos + Rb) % kp);
        for (; xb < NB; xb += kp) s = cadd(s, gbox[((size_t)xb * NB + yb) * bb + pl]);
        xs[pos] = cmake<C>(s.x, s.y);
    }
    __syncthreads();
    fft_minus<C>(xs, kp, logkp, tw);
    C *dst = A + ((size_t)pl * NB + yb) * kp;
    for (int t = threadIdx.x; t < kp; t += blockDim.x) dst[t] = xs[t];
}

// Gbar(kx, ky)[pl] = kp^-2 sum_{Y in box} e^{-2 pi i ky Y/kp} A[pl][Y+Rb][kx]; grid (kp, bb)
template <class C>
__global__ void __launch_bounds__(256) adj_rows_kernel(int kp, int logkp, int NB, int Rb, int bb, double scale,
                                                       const C *__restrict__ A, const C *__restrict__ tw,
                                                       C *__restrict__ gk)
{
    extern __shared__ __align__(16) unsigned char adj_xs_raw[];
    C *xs = reinterpret_cast<C *>(adj_xs_raw);
    const int kx = blockIdx.x, pl = blockIdx.y;
    const C *src = A + (size_t)pl * NB * kp + kx;
    for (int pos = threadIdx.x; pos < kp; pos += blockDim.x) {
        C s = cmake<C>(0.0, 0.0);
        int yb = ((pos + Rb) % kp);
        for (; yb < NB; yb += kp) s = cadd(s, src[(size_t)yb * kp]);
        xs[pos] = s;
    }
    __syncthreads();
    fft_minus<C>(xs, kp, logkp, tw);
    const size_t nk = (size_t)kp * kp;
    C *dst = gk + (size_t)pl * nk + (size_t)kx * kp;
    for (int t = threadIdx.x; t < kp; t += blockDim.x) dst[t] = cscale(xs[t], (typename real_of<C>::type)scale);
}

// ------------------------------------------------------------------ 5. per-k resolvent
// eigenvalue storage read by the resolvent bracket: FP64, or the float pairs of the mixed handle
template <class C> struct KaccEv { using T = double; };
template <> struct KaccEv<float2> { using T = float2; };
#define CQPI_ADJ_KACC adj_kacc_kernel
#define CQPI_ADJ_HBAR adj_hbar_kernel
#define CQPI_ADJ_UNROLL _Pragma("unroll")
#include "adjoint_kspace.cuh"
#undef CQPI_ADJ_KACC
#undef CQPI_ADJ_HBAR
#undef CQPI_ADJ_UNROLL
#define CQPI_ADJ_KACC adj_kacc_kernel_wide
#define CQPI_ADJ_HBAR adj_hbar_kernel_wide
#define CQPI_ADJ_UNROLL _Pragma("unroll 1")
#include "adjoint_kspace.cuh"
#undef CQPI_ADJ_KACC
#undef CQPI_ADJ_HBAR
#undef CQPI_ADJ_UNROLL

// ------------------------------------------------------------------ 6. hoppings
// grid (nR, chunks); out[r][0][pq] = sum_k e^{-i th_r(k)} Hbar(k)[pq] (normal terms),
// out[r][1][pq] = sum_k e^{+i th_r(k)} Hbar(k)[pq] (conjugated terms), th = 2 pi (Rx i + Ry j)/kp
__global__ void __launch_bounds__(256) adj_hop_kernel(int b, int kp, int logkp, const int32_t *__restrict__ R,
                                                      const double2 *__restrict__ tw, const double2 *__restrict__ hbar,
                                                      double2 *__restrict__ out)
{
    const int r = blockIdx.x;
    const int bb = b * b;
    const long long nk = (long long)kp * kp;
    const long long Rx = R[2 * r], Ry = R[2 * r + 1];
    __shared__ double2 red[2][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int pq = 0; pq < bb; pq++) {
        double2 sn = make_double2(0.0, 0.0), sa = make_double2(0.0, 0.0);
        for (long long k = (long long)blockIdx.y * blockDim.x + threadIdx.x; k < nk; k += (long long)gridDim.y * blockDim.x) {
            // kp is a power of two: k = i*kp + j, and the phase index (Rx i + Ry j) mod kp is
            // the low bits of the product (two's complement)
            const long long i = k >> logkp, j = k & (kp - 1);
            const long long mm = (Rx * i + Ry * j) & (long long)(kp - 1);
            const double2 ph = __ldg(tw + mm);
            const double2 h = hbar[(size_t)pq * nk + k];
            sn = cadd(sn, cmul(cconj(ph), h));
            sa = cadd(sa, cmul(ph, h));
        }
        for (int o = 16; o > 0; o >>= 1) {
            sn.x += __shfl_xor_sync(0xffffffffu, sn.x, o);
            sn.y += __shfl_xor_sync(0xffffffffu, sn.y, o);
            sa.x += __shfl_xor_sync(0xffffffffu, sa.x, o);
            sa.y += __shfl_xor_sync(0xffffffffu, sa.y, o);
        }
        if (lane == 0) { red[0][warp] = sn; red[1][warp] = sa; }
        __syncthreads();
        if (threadIdx.x < 2) {
            double2 s = make_double2(0.0, 0.0);
            for (int wv = 0; wv < (int)(blockDim.x >> 5); wv++) s = cadd(s, red[threadIdx.x][wv]);
            atomic_add2(out + ((size_t)r * 2 + threadIdx.x) * bb + pq, s);
        }
        __syncthreads();
    }
}

// The mixed handle's form of adj_hop_kernel: Hbar(k) and the phases in FP32, RG unique R per
// block so that every Hbar(k) value loaded feeds RG of them, each thread's sums over its
// k-points compensated (Kahan) in FP32, the warp and block sums in FP64.
constexpr int HOP_RG = 4;
__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    const float y = x - c, t = s + y;
    c = (t - s) - y;
    s = t;
}
__global__ void __launch_bounds__(256) adj_hop32_kernel(int b, int nR, int kp, int logkp, const int32_t *__restrict__ R,
                                                        const float2 *__restrict__ tw, const float2 *__restrict__ hbar,
                                                        double2 *__restrict__ out)
{
    const int r0 = blockIdx.x * HOP_RG;
    const int bb = b * b;
    const long long nk = (long long)kp * kp;
    long long Rx[HOP_RG], Ry[HOP_RG];
#pragma unroll
    for (int g = 0; g < HOP_RG; g++) {
        const int r = min(r0 + g, nR - 1);
        Rx[g] = R[2 * r];
        Ry[g] = R[2 * r + 1];
    }
    __shared__ double red[8][HOP_RG][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int pq = 0; pq < bb; pq++) {
        // [g][0..3] = normal re, im, conjugated re, im: sums and compensations
        float sm[HOP_RG][4], cm[HOP_RG][4];
#pragma unroll
        for (int g = 0; g < HOP_RG; g++)
#pragma unroll
            for (int c = 0; c < 4; c++) { sm[g][c] = 0.f; cm[g][c] = 0.f; }
        for (long long k = (long long)blockIdx.y * blockDim.x + threadIdx.x; k < nk; k += (long long)gridDim.y * blockDim.x) {
            const long long i = k >> logkp, j = k & (kp - 1);
            const float2 h = hbar[(size_t)pq * nk + k];
#pragma unroll
            for (int g = 0; g < HOP_RG; g++) {
                const float2 ph = __ldg(tw + ((Rx[g] * i + Ry[g] * j) & (long long)(kp - 1)));
                // conj(ph) h and ph h
                kahan_add(sm[g][0], cm[g][0], ph.x * h.x + ph.y * h.y);
                kahan_add(sm[g][1], cm[g][1], ph.x * h.y - ph.y * h.x);
                kahan_add(sm[g][2], cm[g][2], ph.x * h.x - ph.y * h.y);
                kahan_add(sm[g][3], cm[g][3], ph.x * h.y + ph.y * h.x);
            }
        }
#pragma unroll
        for (int g = 0; g < HOP_RG; g++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                double v = (double)sm[g][c] - (double)cm[g][c];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) red[warp][g][c] = v;
            }
        __syncthreads();
        if (threadIdx.x < 2 * HOP_RG) {
            const int g = threadIdx.x >> 1, na = threadIdx.x & 1;
            double2 t = make_double2(0.0, 0.0);
            for (int wv = 0; wv < (int)(blockDim.x >> 5); wv++) {
                t.x += red[wv][g][2 * na];
                t.y += red[wv][g][2 * na + 1];
            }
            if (r0 + g < nR) atomic_add2(out + ((size_t)(r0 + g) * 2 + na) * bb + pq, t);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ launchers
template <int B, class C>
static void launch_contract_t(cqpi_handle *h, int ne, const typename real_of<C>::type *phi, const C *box,
                              const float *wmap, AdjWorkspace &aw)
{
    const int nsite = h->n * h->n, bb = h->b * h->b;
    dim3 grid((unsigned)nsite, (unsigned)(ne * h->nimp));
    const size_t smem = 4 * 128 * (size_t)h->b * sizeof(typename real_of<C>::type) + 4 * sizeof(double2) * bb;
    C *Ub = reinterpret_cast<C *>(aw.win);
    C *Sb = Ub + (size_t)ne * h->nimp * h->W * h->mb * h->b * nsite;
    using Rl = typename real_of<C>::type;
    constexpr int wpb = AdjWpb<C>::value;
    const size_t wsm = sizeof(Rl) * ((size_t)h->W * h->mb * ADJ_QP + wpb * 128 * (size_t)h->b * 4);
    bool warp_form = false, mma = false;
    if constexpr (B <= 4 && std::is_same<C, float2>::value) {
        // the mixed handle: the two products on the tensor cores (adjoint_mma.cu)
        warp_form = mma = launch_adj_contract_mma(h, ne, phi, box, wmap, Ub, Sb, reinterpret_cast<float2 *>(aw.Mp));
    }
    if constexpr (B <= 4) {
        // one warp per site when the orbital table and the warps' ubar / sbar rows fit
        if (!warp_form && wsm <= 200 * 1024 &&
            cudaFuncSetAttribute(adj_contract_warp_kernel<B, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm) ==
                cudaSuccess) {
            adj_contract_warp_kernel<B, C><<<dim3(cdiv(nsite, wpb), (unsigned)(ne * h->nimp)), 32 * wpb, wsm,
                                             h->stream>>>(
                h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp, h->mb, h->blk_start[0], phi, box, h->ws.T, wmap,
                Ub, Sb, aw.Mp);
            warp_form = true;
        }
    }
    if (!warp_form)
        adj_contract_kernel<B, C><<<grid, 128, smem, h->stream>>>(h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp,
                                                               h->mb, h->blk_start[0], phi, box, h->ws.T, wmap, Ub, Sb, aw.Mp);
    adj_gather_kernel<C><<<dim3(cdiv(h->NB, 128), (unsigned)h->NB, (unsigned)(ne * bb)), 128, 0, h->stream>>>(
        h->b, h->n, h->w, h->Rb, h->NB, h->W, h->mb, h->blk_start[0], h->nimp, Ub, Sb, aw.gbox);
    if (mma)
        adj_mreduce32_kernel<<<(unsigned)(ne * h->nimp), 256, 0, h->stream>>>(
            nsite, bb, reinterpret_cast<const float2 *>(aw.Mp), aw.M);
    else
        adj_mreduce_kernel<<<(unsigned)(ne * h->nimp), 256, 0, h->stream>>>(nsite, bb, aw.Mp, aw.M);
    adj_wsum_kernel<<<dim3((unsigned)h->os, (unsigned)ne), 256, 0, h->stream>>>(h->wn, h->os, h->Q, h->nimp, wmap,
                                                                               aw.wsum);
    h->launches += 4;
}

template <class C>
static void dispatch_contract(cqpi_handle *h, int ne, const typename real_of<C>::type *phi, const C *box,
                              const float *wmap, AdjWorkspace &aw)
{
    const int b = h->b;
    if (b <= 1) launch_contract_t<1, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 2) launch_contract_t<2, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 3) launch_contract_t<3, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 4) launch_contract_t<4, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 6) launch_contract_t<6, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 8) launch_contract_t<8, C>(h, ne, phi, box, wmap, aw);
    else if (b <= 12) launch_contract_t<12, C>(h, ne, phi, box, wmap, aw);
    else launch_contract_t<16, C>(h, ne, phi, box, wmap, aw);
}

void launch_adj_energy_batch(cqpi_handle *h, int ne, const float *wmap, AdjWorkspace &aw)
{
    if (h->precision == CQPI_PREC_FP64) dispatch_contract<double2>(h, ne, h->d_phi, h->ws.box, wmap, aw);
    else dispatch_contract<float2>(h, ne, h->d_phi32, h->ws.box32, wmap, aw);
    const int span = 4 * h->w + 1;
    adj_kt_kernel<<<span * span, 128, 0, h->stream>>>(h->w, h->Q, h->W, h->mb, h->d_phi, aw.kt);
    adj_term1_kernel<<<dim3(span * span, ne), 128, 0, h->stream>>>(h->b, h->w, h->Rb, h->NB, h->Q, h->mb,
                                                                   h->blk_start[0], aw.kt, aw.wsum, aw.gbox);
    h->launches += 2;
    const int nt = ne * h->nimp;
    if (h->precision == CQPI_PREC_FP64)
        adj_tv_kernel<double2><<<cdiv(nt, 64), 64, 0, h->stream>>>(h->b, h->NB, h->Rb, h->nimp, ne, h->ws.box, h->d_V,
                                                                   h->ws.T, aw.M, aw.gbox, aw.gV);
    else
        adj_tv_kernel<float2><<<cdiv(nt, 64), 64, 0, h->stream>>>(h->b, h->NB, h->Rb, h->nimp, ne, h->ws.box32, h->d_V,
                                                                  h->ws.T, aw.M, aw.gbox, aw.gV);
    h->launches++;
}

static int ilog2_exact(int v)
{
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

template <int B>
static void launch_kacc_t(cqpi_handle *h, int ne, const double *omegas, AdjWorkspace &aw)
{
    const long long nk = (long long)h->kp * h->kp;
    const unsigned grid = (unsigned)cdiv(nk, 128);
    const float2 *gk32 = reinterpret_cast<const float2 *>(aw.gk);
    if constexpr (B <= 6) {
        if (h->precision == CQPI_PREC_FP64)
            adj_kacc_kernel<B, double2><<<grid, 128, 0, h->stream>>>(h->b, nk, ne, omegas, h->eta, h->d_eval, h->d_evec,
                                                                     aw.gk, aw.C);
        else
            adj_kacc_kernel<B, float2><<<grid, 128, 0, h->stream>>>(h->b, nk, ne, omegas, h->eta, h->d_eval32,
                                                                    h->d_evec32, gk32, aw.C);
    } else {
        if (h->precision == CQPI_PREC_FP64)
            adj_kacc_kernel_wide<B, double2><<<grid, 128, 0, h->stream>>>(h->b, nk, ne, omegas, h->eta, h->d_eval,
                                                                          h->d_evec, aw.gk, aw.C);
        else
            adj_kacc_kernel_wide<B, float2><<<grid, 128, 0, h->stream>>>(h->b, nk, ne, omegas, h->eta, h->d_eval32,
                                                                         h->d_evec32, gk32, aw.C);
    }
    h->launches++;
}

// Rows of the box -> k-grid transform for the mixed handle on power-of-two k-grids of 64 ...
// 4096 points with the box no wider than the grid: NC = 256 / max(N1, N2) k_x columns of one
// plane per block.  The block reads the NB box rows of its columns (NC contiguous values per
// row), puts row yb at k_y position (yb - Rb) mod kp (zero elsewhere), and runs the four-step
// register transform of the forward rows with sign -1, as conj(F+(conj x)); each warp of the
// second pass writes 32 consecutive k_y of one column.  (adj_rows_kernel: one block per
// column, radix-2 with a barrier per stage, and a column read at stride kp.)
template <int N1, int N2>
__global__ void __launch_bounds__(256) adj_rows_reg_kernel(int NB, int Rb, float scale, const float2 *__restrict__ A,
                                                           const float2 *__restrict__ tw, float2 *__restrict__ gk)
{
    constexpr int KP = N1 * N2;
    constexpr int NC = 256 / (N1 > N2 ? N1 : N2);
    constexpr int PLEN = KP + KP / 32 + 1;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tws = sm + (size_t)NC * PLEN;       // [k2][n1] = e^{+2 pi i n1 k2 / kp}
    const int kx0 = blockIdx.x * NC, pl = blockIdx.y;
    for (int t = threadIdx.x; t < KP; t += blockDim.x) {
        const int k2 = t / N1, n1 = t - k2 * N1;
        tws[t] = tw[(n1 * k2) & (KP - 1)];
    }
    for (int t = threadIdx.x; t < NC * PLEN; t += blockDim.x) sm[t] = make_float2(0.f, 0.f);
    __syncthreads();
    const float2 *src = A + (size_t)pl * NB * KP + kx0;
    for (int idx = threadIdx.x; idx < NB * NC; idx += blockDim.x) {
        const int yb = idx / NC, c = idx - yb * NC;
        const float2 v = src[(size_t)yb * KP + c];
        const int pos = (yb - Rb + KP) & (KP - 1);
        sm[(size_t)c * PLEN + pad32(pos)] = make_float2(v.x, -v.y);
    }
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
    const size_t nk = (size_t)KP * KP;
    for (int task = threadIdx.x; task < NC * N2; task += blockDim.x) {
        const int c = task / N2, k2 = task - c * N2;
        const float2 *a = sm + (size_t)c * PLEN;
        float2 x[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
        fft_reg<N1>(x);
        float2 *dst = gk + (size_t)pl * nk + (size_t)(kx0 + c) * KP;
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) dst[k2 + N2 * k1] = make_float2(x[k1].x * scale, -x[k1].y * scale);
    }
}

// Columns of the same transform for the mixed handle: NC box columns yb of one plane per
// block; the block gathers the plane's FP64 gradients of its columns from the box (NC values
// of one X at a time), puts X at position (X - Rb) mod kp, and writes the transformed columns
// A[plane][yb][kx] in FP32 (unscaled; the rows apply kp^-2).
template <int N1, int N2>
__global__ void __launch_bounds__(256) adj_cols_reg_kernel(int NB, int Rb, int bb, const double2 *__restrict__ gbox,
                                                           const float2 *__restrict__ tw, float2 *__restrict__ A)
{
    constexpr int KP = N1 * N2;
    constexpr int NC = 256 / (N1 > N2 ? N1 : N2);
    constexpr int PLEN = KP + KP / 32 + 1;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tws = sm + (size_t)NC * PLEN;
    const int yb0 = blockIdx.x * NC, pl = blockIdx.y;
    for (int t = threadIdx.x; t < KP; t += blockDim.x) {
        const int k2 = t / N1, n1 = t - k2 * N1;
        tws[t] = tw[(n1 * k2) & (KP - 1)];
    }
    for (int t = threadIdx.x; t < NC * PLEN; t += blockDim.x) sm[t] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int idx = threadIdx.x; idx < NB * NC; idx += blockDim.x) {
        const int xb = idx / NC, c = idx - xb * NC, yb = yb0 + c;
        if (yb >= NB) continue;
        const double2 v = gbox[((size_t)xb * NB + yb) * bb + pl];
        const int pos = (xb - Rb + KP) & (KP - 1);
        sm[(size_t)c * PLEN + pad32(pos)] = make_float2((float)v.x, -(float)v.y);
    }
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
    for (int task = threadIdx.x; task < NC * N2; task += blockDim.x) {
        const int c = task / N2, k2 = task - c * N2, yb = yb0 + c;
        if (yb >= NB) continue;
        const float2 *a = sm + (size_t)c * PLEN;
        float2 x[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) x[n1] = a[pad32(n1 + N1 * k2)];
        fft_reg<N1>(x);
        float2 *dst = A + ((size_t)pl * NB + yb) * KP;
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) dst[k2 + N2 * k1] = make_float2(x[k1].x, -x[k1].y);
    }
}

template <int N1, int N2>
static void launch_adj_cols_reg(cqpi_handle *h, const double2 *gbe, float2 *A)
{
    constexpr int KP = N1 * N2, NC = 256 / (N1 > N2 ? N1 : N2);
    const size_t smem = 8 * ((size_t)NC * (KP + KP / 32 + 1) + KP);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(adj_cols_reg_kernel<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    adj_cols_reg_kernel<N1, N2><<<dim3(cdiv(h->NB, NC), h->b * h->b), 256, smem, h->stream>>>(
        h->NB, h->Rb, h->b * h->b, gbe, h->d_tw32, A);
}

// the register columns transform of the mixed handle (CQPI_ADJ_ROWS=radix2 keeps adj_cols_kernel)
static bool adj_cols_reg(cqpi_handle *h, const double2 *gbe, float2 *A)
{
    const char *f = getenv("CQPI_ADJ_ROWS");
    if (h->NB > h->kp || (f && !strcmp(f, "radix2"))) return false;
    switch (h->kp) {
    case 64: launch_adj_cols_reg<8, 8>(h, gbe, A); return true;
    case 128: launch_adj_cols_reg<8, 16>(h, gbe, A); return true;
    case 256: launch_adj_cols_reg<16, 16>(h, gbe, A); return true;
    case 512: launch_adj_cols_reg<16, 32>(h, gbe, A); return true;
    case 1024: launch_adj_cols_reg<32, 32>(h, gbe, A); return true;
    case 2048: launch_adj_cols_reg<32, 64>(h, gbe, A); return true;
    case 4096: launch_adj_cols_reg<64, 64>(h, gbe, A); return true;
    }
    return false;
}

template <int N1, int N2>
static void launch_adj_rows_reg(cqpi_handle *h, const float2 *A, float2 *gk)
{
    constexpr int KP = N1 * N2, NC = 256 / (N1 > N2 ? N1 : N2);
    const size_t smem = 8 * ((size_t)NC * (KP + KP / 32 + 1) + KP);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(adj_rows_reg_kernel<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    adj_rows_reg_kernel<N1, N2><<<dim3(KP / NC, h->b * h->b), 256, smem, h->stream>>>(
        h->NB, h->Rb, (float)(1.0 / ((double)KP * KP)), A, h->d_tw32, gk);
}

// the register rows transform of the mixed handle (CQPI_ADJ_ROWS=radix2 keeps adj_rows_kernel)
static bool adj_rows_reg(cqpi_handle *h, const float2 *A, float2 *gk)
{
    const char *f = getenv("CQPI_ADJ_ROWS");
    if (h->NB > h->kp || (f && !strcmp(f, "radix2"))) return false;
    switch (h->kp) {
    case 64: launch_adj_rows_reg<8, 8>(h, A, gk); return true;
    case 128: launch_adj_rows_reg<8, 16>(h, A, gk); return true;
    case 256: launch_adj_rows_reg<16, 16>(h, A, gk); return true;
    case 512: launch_adj_rows_reg<16, 32>(h, A, gk); return true;
    case 1024: launch_adj_rows_reg<32, 32>(h, A, gk); return true;
    case 2048: launch_adj_rows_reg<32, 64>(h, A, gk); return true;
    case 4096: launch_adj_rows_reg<64, 64>(h, A, gk); return true;
    }
    return false;
}

// Gbar(k) of energy e of the batch (box -> k-grid transform) into slot e of aw.gk
void launch_adj_kspace(cqpi_handle *h, int e, AdjWorkspace &aw)
{
    const int kp = h->kp, logkp = ilog2_exact(kp), bb = h->b * h->b;
    const size_t nk = (size_t)kp * kp;
    const double2 *gbe = aw.gbox + (size_t)e * h->NB * h->NB * bb;
    if (h->precision == CQPI_PREC_FP64) {
        const size_t smem = sizeof(double2) * kp;
        adj_cols_kernel<double2><<<dim3(h->NB, bb), 256, smem, h->stream>>>(kp, logkp, h->NB, h->Rb, bb, gbe, h->d_tw,
                                                                            aw.A);
        adj_rows_kernel<double2><<<dim3(kp, bb), 256, smem, h->stream>>>(kp, logkp, h->NB, h->Rb, bb,
                                                                         1.0 / ((double)kp * kp), aw.A, h->d_tw,
                                                                         aw.gk + (size_t)e * bb * nk);
    } else {
        // the mixed handle: the transform and the per-k rotation in FP32, in the same buffers
        const size_t smem = sizeof(float2) * kp;
        float2 *A32 = reinterpret_cast<float2 *>(aw.A), *gk32 = reinterpret_cast<float2 *>(aw.gk);
        if (!adj_cols_reg(h, gbe, A32))
            adj_cols_kernel<float2><<<dim3(h->NB, bb), 256, smem, h->stream>>>(kp, logkp, h->NB, h->Rb, bb, gbe,
                                                                               h->d_tw32, A32);
        if (!adj_rows_reg(h, A32, gk32 + (size_t)e * bb * nk))
            adj_rows_kernel<float2><<<dim3(kp, bb), 256, smem, h->stream>>>(kp, logkp, h->NB, h->Rb, bb,
                                                                            1.0 / ((double)kp * kp), A32, h->d_tw32,
                                                                            gk32 + (size_t)e * bb * nk);
    }
    h->launches += 2;
}

// C(k) += the resolvent brackets of the ne energies whose Gbar(k) fill the slots of aw.gk
void launch_adj_kacc(cqpi_handle *h, int ne, const double *omegas, AdjWorkspace &aw)
{
    const int b = h->b;
    if (b <= 1) launch_kacc_t<1>(h, ne, omegas, aw);
    else if (b <= 2) launch_kacc_t<2>(h, ne, omegas, aw);
    else if (b <= 3) launch_kacc_t<3>(h, ne, omegas, aw);
    else if (b <= 4) launch_kacc_t<4>(h, ne, omegas, aw);
    else if (b <= 6) launch_kacc_t<6>(h, ne, omegas, aw);
    else if (b <= 8) launch_kacc_t<8>(h, ne, omegas, aw);
    else if (b <= 12) launch_kacc_t<12>(h, ne, omegas, aw);
    else launch_kacc_t<16>(h, ne, omegas, aw);
}

template <int B>
static void launch_hbar_t(cqpi_handle *h, AdjWorkspace &aw)
{
    const long long nk = (long long)h->kp * h->kp;
    float2 *hb32 = reinterpret_cast<float2 *>(aw.gk);
    if (h->precision == CQPI_PREC_FP64) {
        if constexpr (B <= 6)
            adj_hbar_kernel<B, double2><<<cdiv(nk, 128), 128, 0, h->stream>>>(h->b, nk, h->d_evec, aw.C, aw.gk);
        else
            adj_hbar_kernel_wide<B, double2><<<cdiv(nk, 128), 128, 0, h->stream>>>(h->b, nk, h->d_evec, aw.C, aw.gk);
    } else {
        if constexpr (B <= 6)
            adj_hbar_kernel<B, float2><<<cdiv(nk, 128), 128, 0, h->stream>>>(h->b, nk, h->d_evec32, aw.C, hb32);
        else
            adj_hbar_kernel_wide<B, float2><<<cdiv(nk, 128), 128, 0, h->stream>>>(h->b, nk, h->d_evec32, aw.C, hb32);
    }
    h->launches++;
}

void launch_adj_hoppings(cqpi_handle *h, AdjWorkspace &aw)
{
    const int b = h->b;
    if (b <= 1) launch_hbar_t<1>(h, aw);
    else if (b <= 2) launch_hbar_t<2>(h, aw);
    else if (b <= 3) launch_hbar_t<3>(h, aw);
    else if (b <= 4) launch_hbar_t<4>(h, aw);
    else if (b <= 6) launch_hbar_t<6>(h, aw);
    else if (b <= 8) launch_hbar_t<8>(h, aw);
    else if (b <= 12) launch_hbar_t<12>(h, aw);
    else launch_hbar_t<16>(h, aw);
    if (h->nR > 0) {
        const int chunks = std::max(1, std::min(64, (int)(((long long)h->kp * h->kp) / (256 * 64))));
        if (h->precision == CQPI_PREC_FP64)
            adj_hop_kernel<<<dim3(h->nR, chunks), 256, 0, h->stream>>>(b, h->kp, ilog2_exact(h->kp), h->d_R, h->d_tw, aw.gk,
                                                                       aw.gR);
        else
            adj_hop32_kernel<<<dim3(cdiv(h->nR, HOP_RG), chunks), 256, 0, h->stream>>>(
                b, h->nR, h->kp, ilog2_exact(h->kp), h->d_R, h->d_tw32, reinterpret_cast<const float2 *>(aw.gk), aw.gR);
        h->launches++;
    }
}

}  // namespace cqpi
