// ldos_fp64.cu -- continuum LDOS contraction, all-FP64 path (CUDA cores).
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
// index so map stores coalesce.  Roofline: FP64-FLOP bound.
#include "cqpi_internal.h"

namespace cqpi {

template <int B>
__global__ void __launch_bounds__(128) ldos_fp64_kernel(int b, int n, int os, int w, int Rb, int NB, int Q, int W, int nimp,
                                                        int nblk, int mb, int bs0, int bs1, const double *__restrict__ phi,
                                                        const double2 *__restrict__ box, const double2 *__restrict__ T,
                                                        const double *__restrict__ term1, float *__restrict__ out32,
                                                        double *__restrict__ out64)
{
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
    const double2 *boxe = box + (size_t)e * NB * NB * bb;
    const double2 *Te = T + (size_t)ei * bb;

    double term2 = 0.0;
    for (int blk = 0; blk < nblk; blk++) {
        const int bs = blk ? bs1 : bs0;
        const double *ph = phi + ((size_t)blk * Q + q) * W * mb;
        double sr[B], si[B];
#pragma unroll
        for (int c = 0; c < B; c++) { sr[c] = 0.0; si[c] = 0.0; }
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            const double2 *g = boxe + ((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb;
            for (int ol = 0; ol < mb; ol++) {
                const double f = __ldg(ph + d * mb + ol);
                if (f == 0.0) continue;
                const int o = bs + ol;
#pragma unroll
                for (int c = 0; c < B; c++) {
                    if (c < b) {
                        const double2 v = __ldg(g + c * b + o);
                        sr[c] += v.x * f;
                        si[c] += v.y * f;
                    }
                }
            }
        }
        double tr[B], ti[B];
#pragma unroll
        for (int a = 0; a < B; a++) {
            tr[a] = 0.0; ti[a] = 0.0;
            if (a < b) {
#pragma unroll
                for (int c = 0; c < B; c++) {
                    if (c < b) {
                        const double2 t = __ldg(Te + a * b + c);
                        tr[a] += t.x * sr[c] - t.y * si[c];
                        ti[a] += t.x * si[c] + t.y * sr[c];
                    }
                }
            }
        }
        for (int d = 0; d < W; d++) {
            const int dx = d / side - w, dy = d % side - w;
            const double2 *g = boxe + ((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb;
            for (int ol = 0; ol < mb; ol++) {
                const double f = __ldg(ph + d * mb + ol);
                if (f == 0.0) continue;
                const int o = bs + ol;
                double im = 0.0;
#pragma unroll
                for (int a = 0; a < B; a++) {
                    if (a < b) {
                        const double2 v = __ldg(g + o * b + a);
                        im += v.x * ti[a] + v.y * tr[a];
                    }
                }
                term2 += f * im;
            }
        }
    }
    const double rho = -term1[(size_t)e * Q + q] - term2;
    const size_t oi = ((size_t)ei * wn + y) * wn + x;
    if (out64) out64[oi] = rho;
    if (out32) out32[oi] = (float)rho;
}

template <int B>
static void launch_t(cqpi_handle *h, int ne, const double2 *box, const double2 *T, const double *term1, float *o32, double *o64)
{
    dim3 blk(32, 4);
    dim3 grid(cdiv(h->wn, 32), cdiv(h->wn, 4), ne * h->nimp);
    ldos_fp64_kernel<B><<<grid, blk, 0, h->stream>>>(h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp, h->nblk,
                                                     h->mb, h->blk_start[0], h->blk_start[1], h->d_phi, box, T, term1,
                                                     o32, o64);
    h->launches++;
}

void launch_ldos_fp64(cqpi_handle *h, int ne, const double2 *box, const double2 *T, const double *term1, float *out32,
                      double *out64)
{
    const int b = h->b;
    if (b <= 1) launch_t<1>(h, ne, box, T, term1, out32, out64);
    else if (b <= 2) launch_t<2>(h, ne, box, T, term1, out32, out64);
    else if (b <= 3) launch_t<3>(h, ne, box, T, term1, out32, out64);
    else if (b <= 4) launch_t<4>(h, ne, box, T, term1, out32, out64);
    else if (b <= 6) launch_t<6>(h, ne, box, T, term1, out32, out64);
    else if (b <= 8) launch_t<8>(h, ne, box, T, term1, out32, out64);
    else if (b <= 10) launch_t<10>(h, ne, box, T, term1, out32, out64);
    else if (b <= 12) launch_t<12>(h, ne, box, T, term1, out32, out64);
    else launch_t<16>(h, ne, box, T, term1, out32, out64);
}

}  // namespace cqpi
