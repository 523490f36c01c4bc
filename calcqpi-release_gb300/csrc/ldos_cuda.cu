// ldos_cuda.cu -- continuum LDOS contraction on CUDA cores: the all-FP64 path
// (double2) and the FP32 variant of the mixed path (float2 G0(R), FP64 term1).
//
// Replaces tmatrix::calcwannierldos (src/qpi.cc:876-950) and the reference GPU
// kernels gpucalcwannierldos / gpucalcwannierldosspin (src/qpicudakernel.cu:60-158).
// The reference sums over both window offsets d1, d2 (W^2 b x b products per site);
// here the double sum is factorised (phi is real, so Im commutes with the sums):
//
//   s_c(p,q)  = sum_{d,o in blk} G0(-(p+d))[c][o] phi_o(q,d)
//   ts        = T s
//   term2     = sum_{d,o in blk} phi_o(q,d) sum_a G0(p+d)[o][a] ts_a
//   rho(p,q)  = -term1(q) - Im(term2)            (summed over spin blocks)
//
// which is the reference's sum over cldos[o2][o1] = (G0(p+d2) T G0(-(p+d1)))[o2][o1]
// regrouped.  One thread per output pixel; x = site_i*os + q_x is the fastest
// index so map stores coalesce.  Roofline: FP64- resp. FP32-FLOP bound.
//
// Josephson mode (JOS, tmatrix::calcwannierjosephson, src/qpi.cc:953-1033): the s side
// reads the hole-block column o + coff (coff = bands/2), term2 is kept complex and
//   rho(p,q) = -term1_J(q) - Im(tip * term2)
// with the per-energy tip factor (term1_J already holds Im(tip * sum phi phi G0)).
#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

template <int B, class C, bool JOS>
__global__ void __launch_bounds__(128) ldos_cuda_kernel(int b, int n, int os, int w, int Rb, int NB, int Q, int W, int nimp,
                                                        int nblk, int mb, int bs0, int bs1, int coff,
                                                        const double2 *__restrict__ tip,
                                                        const typename real_of<C>::type *__restrict__ phi,
                                                        const C *__restrict__ box, const C *__restrict__ T,
                                                        const double *__restrict__ term1, double scale,
                                                        float *__restrict__ out32, double *__restrict__ out64)
{
    using Rl = typename real_of<C>::type;
    const int wn = n * os;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= wn || y >= wn) return;
    const int ei = blockIdx.z;            // energy * nimp + impurity
    const int e = ei / nimp;
    const int bb = b * b, side = 2 * w + 1;
    const int i = x / os, qx = x % os, j = y / os, qy = y % os, q = qx * os + qy;
    const int n2 = n >> 1;
    const int px = i - n2, py = j - n2;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    const C *Te = T + (size_t)ei * bb;

    Rl term2 = 0, term2r = 0;
    for (int blk = 0; blk < nblk; blk++) {
        const int bs = blk ? bs1 : bs0;
        const Rl *ph = phi + ((size_t)blk * Q + q) * W * mb;
        Rl sr[B], si[B];
#pragma unroll
        for (int c = 0; c < B; c++) { sr[c] = 0; si[c] = 0; }
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            const C *g = boxe + ((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb;
            for (int ol = 0; ol < mb; ol++) {
                const Rl f = __ldg(ph + d * mb + ol);
                if (f == (Rl)0) continue;
                const int o = bs + ol;
#pragma unroll
                for (int c = 0; c < B; c++) {
                    if (c < b) {
                        const C v = __ldg(g + c * b + o + coff);
                        sr[c] += v.x * f;
                        si[c] += v.y * f;
                    }
                }
            }
        }
        Rl tr[B], ti[B];
#pragma unroll
        for (int a = 0; a < B; a++) {
            tr[a] = 0; ti[a] = 0;
            if (a < b) {
#pragma unroll
                for (int c = 0; c < B; c++) {
                    if (c < b) {
                        const C t = __ldg(Te + a * b + c);
                        tr[a] += t.x * sr[c] - t.y * si[c];
                        ti[a] += t.x * si[c] + t.y * sr[c];
                    }
                }
            }
        }
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            const C *g = boxe + ((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb;
            for (int ol = 0; ol < mb; ol++) {
                const Rl f = __ldg(ph + d * mb + ol);
                if (f == (Rl)0) continue;
                const int o = bs + ol;
                Rl im = 0, re = 0;
#pragma unroll
                for (int a = 0; a < B; a++) {
                    if (a < b) {
                        const C v = __ldg(g + o * b + a);
                        im += v.x * ti[a] + v.y * tr[a];
                        if (JOS) re += v.x * tr[a] - v.y * ti[a];
                    }
                }
                term2 += f * im;
                if (JOS) term2r += f * re;
            }
        }
    }
    double t2 = (double)term2;
    if (JOS) {
        const double2 tp = tip[e];
        t2 = tp.x * (double)term2 + tp.y * (double)term2r;
    }
    const double rho = (-term1[(size_t)e * Q + q] - t2) * scale;
    const size_t oi = ((size_t)ei * wn + y) * wn + x;
    if (out64) out64[oi] = rho;
    if (out32) out32[oi] = (float)rho;
}

template <int B, class C>
static void launch_t(cqpi_handle *h, int ne, const typename real_of<C>::type *phi, const C *box, const C *T,
                     const double *term1, float *o32, double *o64)
{
    dim3 blk(32, 4);
    dim3 grid(cdiv(h->wn, 32), cdiv(h->wn, 4), ne * h->nimp);
    const double2 *tip = h->jos_tip;
    if (tip)
        ldos_cuda_kernel<B, C, true><<<grid, blk, 0, h->stream>>>(h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W,
                                                                  h->nimp, h->nblk, h->mb, h->blk_start[0],
                                                                  h->blk_start[1], h->b >> 1, tip, phi, box, T, term1,
                                                                  (double)h->out_scale, o32, o64);
    else
        ldos_cuda_kernel<B, C, false><<<grid, blk, 0, h->stream>>>(h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W,
                                                                   h->nimp, h->nblk, h->mb, h->blk_start[0],
                                                                   h->blk_start[1], 0, nullptr, phi, box, T, term1,
                                                                   (double)h->out_scale, o32, o64);
    h->launches++;
}

template <class C>
static void dispatch(cqpi_handle *h, int ne, const typename real_of<C>::type *phi, const C *box, const C *T,
                     const double *term1, float *o32, double *o64)
{
    const int b = h->b;
    if (b <= 1) launch_t<1, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 2) launch_t<2, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 3) launch_t<3, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 4) launch_t<4, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 6) launch_t<6, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 8) launch_t<8, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 10) launch_t<10, C>(h, ne, phi, box, T, term1, o32, o64);
    else if (b <= 12) launch_t<12, C>(h, ne, phi, box, T, term1, o32, o64);
    else launch_t<16, C>(h, ne, phi, box, T, term1, o32, o64);
}

void launch_ldos_fp64(cqpi_handle *h, int ne, const double2 *box, const double2 *T, const double *term1, float *out32,
                      double *out64)
{
    dispatch<double2>(h, ne, h->d_phi, box, T, term1, out32, out64);
}

void launch_ldos_fp32(cqpi_handle *h, int ne, const float2 *box, const float2 *T, const double *term1, float *out32,
                      double *out64)
{
    dispatch<float2>(h, ne, h->d_phi32, box, T, term1, out32, out64);
}

}  // namespace cqpi
