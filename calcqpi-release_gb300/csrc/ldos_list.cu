// ldos_list.cu -- the proximity-list form of the continuum LDOS (threshold keyword).
//
// Replaces tmatrix::calcwannierldos(os, w, flaglist) (src/qpi.cc:1085-1134) and the
// reference GPU kernel gpucalcwannierldoslist (src/qpicudakernel.cu:273-315).  The list
// (mkthresholdlist, src/qpi.cc:139-253) keeps the (q, d1, d2, o1, o2) terms of the double
// window sum whose orbital factor f = phi_o1(q,d1) phi_o2(q,d2) is above threshold * max
// phi^2; the mask does not factorise, so the sum is regrouped per site p instead:
//
//   V(d1)        = T G0(-(p+d1))                                   (W b x b products)
//   C(d1,d2,pr)  = Im sum_a G0(p+d2)[o2][a] V(d1)[a][o1]            for the pairs pr = (o1,o2)
//                                                                   the list uses
//   rho(p,q)     = -term1_L(q) - sum_{entries (d1,q)} f C(d1,d2,pr)
//   term1_L(q)   = sum_{entries of q} f Im G0(d2-d1)[o2][o1]        (site independent)
//
// Entries are stored CSR by (d1, q) with u = d2 * npair + pair index, so one block per site
// computes C(d1, .) for one d1 at a time in shared memory and every thread accumulates the
// entries of its own sub-pixels q (no atomics).  FP64 for the FP64 path; FP32 G0(R), T and
// accumulation (FP64 term1_L) for the mixed path.  CUDA cores: the work per site is
// W^2 * npair * b complex MACs plus the list length, far from a dense GEMM shape.
#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

template <class C>
__global__ void __launch_bounds__(128) ldos_list_kernel(int b, int n, int os, int w, int Rb, int NB, int Q, int W,
                                                        int nimp, int npair, const int2 *__restrict__ pairs,
                                                        const int *__restrict__ off, const int *__restrict__ eu,
                                                        const typename real_of<C>::type *__restrict__ ef,
                                                        const C *__restrict__ box, const C *__restrict__ T,
                                                        const double *__restrict__ term1, double scale,
                                                        float *__restrict__ out32, double *__restrict__ out64)
{
    using Rl = typename real_of<C>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *V = reinterpret_cast<C *>(smem_raw);                  // [W][b][b]
    Rl *Cv = reinterpret_cast<Rl *>(V + (size_t)W * b * b);  // [W * npair] for one d1
    const int site = blockIdx.x, ei = blockIdx.y, e = ei / nimp;
    const int i = site / n, j = site % n, n2 = n >> 1;
    const int px = i - n2, py = j - n2;
    const int bb = b * b, side = 2 * w + 1;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    const C *Te = T + (size_t)ei * bb;
    // V(d1) = T G0(-(p+d1))
    for (int t = threadIdx.x; t < W * bb; t += blockDim.x) {
        const int d = t / bb, a = (t / b) % b, c = t % b;
        const int dx = d / side - w, dy = d % side - w;
        const C *g = boxe + ((size_t)(-px - dx + Rb) * NB + (-py - dy + Rb)) * bb;
        Rl re = 0, im = 0;
        for (int k = 0; k < b; k++) {
            const C tv = __ldg(Te + a * b + k), gv = __ldg(g + k * b + c);
            re += tv.x * gv.x - tv.y * gv.y;
            im += tv.x * gv.y + tv.y * gv.x;
        }
        V[t] = cmake<C>(re, im);
    }
    Rl acc[4] = {0, 0, 0, 0};   // sub-pixels q = threadIdx.x + 128 k, Q <= 512
    const int nitem = W * npair;
    for (int d1 = 0; d1 < W; d1++) {
        __syncthreads();   // V complete (first pass) / Cv of the previous d1 consumed
        for (int t = threadIdx.x; t < nitem; t += blockDim.x) {
            const int d2 = t / npair;
            const int2 pr = pairs[t % npair];   // (o1, o2)
            const int dx = d2 / side - w, dy = d2 % side - w;
            const C *g = boxe + ((size_t)(px + dx + Rb) * NB + (py + dy + Rb)) * bb + pr.y * b;
            const C *v = V + (size_t)d1 * bb + pr.x;
            Rl im = 0;
            for (int a = 0; a < b; a++) {
                const C gv = __ldg(g + a), vv = v[a * b];
                im += gv.x * vv.y + gv.y * vv.x;
            }
            Cv[t] = im;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = threadIdx.x + 128 * k;
            if (q < Q) {
                const int s0 = off[d1 * Q + q], s1 = off[d1 * Q + q + 1];
                Rl a = 0;
                for (int s = s0; s < s1; s++) a += __ldg(ef + s) * Cv[__ldg(eu + s)];
                acc[k] += a;
            }
        }
    }
    const int wn = n * os;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int q = threadIdx.x + 128 * k;
        if (q < Q) {
            const int qx = q / os, qy = q % os;
            const int x = i * os + qx, y = j * os + qy;
            const double rho = (-term1[(size_t)e * Q + q] - (double)acc[k]) * scale;
            const size_t oi = ((size_t)ei * wn + y) * wn + x;
            if (out64) out64[oi] = rho;
            if (out32) out32[oi] = (float)rho;
        }
    }
}

// term1_L(q) per energy: grid (Q, ne), threads over d1 and the entries of (d1, q).
template <class C>
__global__ void __launch_bounds__(128) term1_list_kernel(int b, int w, int Rb, int NB, int Q, int W, int npair,
                                                         const int2 *__restrict__ pairs, const int *__restrict__ off,
                                                         const int *__restrict__ eu, const double *__restrict__ ef,
                                                         const C *__restrict__ box, double *__restrict__ term1)
{
    const int q = blockIdx.x, e = blockIdx.y;
    const int bb = b * b, side = 2 * w + 1;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    double acc = 0.0;
    for (int d1 = 0; d1 < W; d1++) {
        const int s0 = off[d1 * Q + q], s1 = off[d1 * Q + q + 1];
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            const int u = eu[s], d2 = u / npair;
            const int2 pr = pairs[u % npair];
            const int rx = d2 / side - d1 / side, ry = d2 % side - d1 % side;
            const C g = boxe[((size_t)(rx + Rb) * NB + (ry + Rb)) * bb + pr.y * b + pr.x];
            acc += ef[s] * (double)g.y;
        }
    }
    __shared__ double red[128];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) term1[(size_t)e * Q + q] = red[0];
}

// dynamic shared memory of ldos_list_kernel: V [W][b][b] complex + C [W * npair] real
size_t list_smem_bytes(const cqpi_handle *h, bool fp64)
{
    const size_t cs = fp64 ? sizeof(double2) : sizeof(float2), rs = fp64 ? sizeof(double) : sizeof(float);
    return (size_t)h->W * h->b * h->b * cs + (size_t)h->W * h->list_npair * rs;
}

cudaError_t configure_list(cqpi_handle *h)
{
    cudaError_t e = cudaFuncSetAttribute(ldos_list_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)list_smem_bytes(h, true));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(ldos_list_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)list_smem_bytes(h, false));
}

void launch_term1_list(cqpi_handle *h, int ne, const void *box, double *term1)
{
    dim3 grid(h->Q, ne);
    if (h->precision == CQPI_PREC_FP64)
        term1_list_kernel<double2><<<grid, 128, 0, h->stream>>>(h->b, h->w, h->Rb, h->NB, h->Q, h->W, h->list_npair,
                                                                h->d_list_pair, h->d_list_off, h->d_list_u,
                                                                h->d_list_f, (const double2 *)box, term1);
    else
        term1_list_kernel<float2><<<grid, 128, 0, h->stream>>>(h->b, h->w, h->Rb, h->NB, h->Q, h->W, h->list_npair,
                                                               h->d_list_pair, h->d_list_off, h->d_list_u, h->d_list_f,
                                                               (const float2 *)box, term1);
    h->launches++;
}

void launch_ldos_list(cqpi_handle *h, int ne, const void *box, const void *T, const double *term1, float *o32,
                      double *o64)
{
    dim3 grid(h->n * h->n, ne * h->nimp);
    const size_t smem = list_smem_bytes(h, h->precision == CQPI_PREC_FP64);
    if (h->precision == CQPI_PREC_FP64)
        ldos_list_kernel<double2><<<grid, 128, smem, h->stream>>>(
            h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp, h->list_npair, h->d_list_pair, h->d_list_off,
            h->d_list_u, h->d_list_f, (const double2 *)box, (const double2 *)T, term1, (double)h->out_scale, o32, o64);
    else
        ldos_list_kernel<float2><<<grid, 128, smem, h->stream>>>(
            h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp, h->list_npair, h->d_list_pair, h->d_list_off,
            h->d_list_u, h->d_list_f32, (const float2 *)box, (const float2 *)T, term1, (double)h->out_scale, o32, o64);
    h->launches++;
}

}  // namespace cqpi
