// surface.cu -- surface / bulk Green's function of a layered model (green=surface|bulk).
//
// Replaces tmatrix::calcsurfacegreensfunction (src/qpi.cc:488-554) with
// tightbind::setmatrix(k, H, kzdepinplane | kzdepoutofplane) (src/tightbinding.cc:184-207) and
// tightbindingcontext::calcgreensfunctioninv (src/tightbinding.h:75-85).  Per k-point:
//   eps_s = in-plane H(k) of the surface model (R_z = 0 terms, with the Fermi-energy diagonal),
//   eps_b = in-plane H(k) of the bulk model, alpha = bulk terms with R_z < 0 (no diagonal),
//   beta = alpha^H, then the decimation
//     g = (w + i eta - eps_b)^-1
//     eps_s += alpha g beta,  eps_b += alpha g beta + beta g alpha,
//     alpha = alpha g alpha,  beta = beta g beta
//   while |alpha|_F > epserr or |beta|_F > epserr, and G0(k) = (w + i eta - eps_s|b)^-1.
// The k-dependent matrices are built once per model (surface_mats_kernel, FP64, [3][k][b*b])
// and the decimation runs one thread per (k-point, energy) in FP64 (b x b matrices in local
// memory); the G0(k) planes go to the same transforms as the eigen-based G0(k).  The loop is
// bounded (the reference's is not): a k-point still above epserr after CQPI_SURFACE_MAX_ITER
// doublings sets status bit 2.  Roofline: FP64 pipe (about 14 b^3 complex MACs per iteration).
#include <algorithm>
#include <cstdlib>

#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

constexpr int CQPI_SURFACE_MAX_ITER = 200;   // CQPI_SURFACE_MAX_ITER=n in the environment lowers it (tests)

// eps_s, eps_b, alpha for every k-point; terms: (rx, ry, o1, o2, anti) + (t_re, t_im)
__global__ void __launch_bounds__(128) surface_mats_kernel(int b, int kp, int ns, const int4 *__restrict__ ts_i,
                                                           const double2 *__restrict__ ts_t, int nb,
                                                           const int4 *__restrict__ tb_i,
                                                           const double2 *__restrict__ tb_t, int no,
                                                           const int4 *__restrict__ to_i,
                                                           const double2 *__restrict__ to_t, const int *anti_s,
                                                           const int *anti_b, const int *anti_o, double efermi,
                                                           int scmax, double2 *__restrict__ mats)
{
    const long long nk = (long long)kp * kp;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    const int i = (int)(k / kp), j = (int)(k % kp), cut = kp >> 1;
    // k-grid of tmatrix::calchamiltonian (src/qpi.cc:465-466)
    const double x = (i > cut) ? ((double)i - kp) / kp : (double)i / kp;
    const double y = (j > cut) ? ((double)j - kp) / kp : (double)j / kp;
    const int bb = b * b;
    for (int s = 0; s < 3; s++) {
        double2 *M = mats + ((size_t)s * nk + k) * bb;
        for (int e = 0; e < bb; e++) M[e] = make_double2(0.0, 0.0);
        if (s < 2)
            for (int d = 0; d < b; d++) M[d * b + d].x = d < scmax ? -efermi : efermi;
        const int n = s == 0 ? ns : (s == 1 ? nb : no);
        const int4 *ti = s == 0 ? ts_i : (s == 1 ? tb_i : to_i);
        const double2 *tt = s == 0 ? ts_t : (s == 1 ? tb_t : to_t);
        const int *an = s == 0 ? anti_s : (s == 1 ? anti_b : anti_o);
        for (int h = 0; h < n; h++) {
            const int4 q = ti[h];
            double sn, cs;
            sincospi(2.0 * ((double)q.x * x + (double)q.y * y), &sn, &cs);
            if (an[h]) sn = -sn;
            const double2 t = tt[h];
            double2 &v = M[q.z * b + q.w];
            v.x += t.x * cs - t.y * sn;
            v.y += t.x * sn + t.y * cs;
        }
    }
}

template <int B>
__device__ __forceinline__ void zmm(int b, const double2 *A, const double2 *Bm, double2 *C)
{
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int q = 0; q < b; q++) s = cadd(s, cmul(A[r * b + q], Bm[q * b + c]));
            C[r * b + c] = s;
        }
}

// inv = (w + i eta - H)^-1 by Gauss-Jordan with partial pivoting; W is scratch
template <int B>
__device__ void zresolvent(int b, const double2 *H, double w, double eta, double2 *W, double2 *inv)
{
    for (int e = 0; e < b * b; e++) {
        W[e] = make_double2(-H[e].x, -H[e].y);
        inv[e] = make_double2(0.0, 0.0);
    }
    for (int d = 0; d < b; d++) {
        W[d * b + d].x += w;
        W[d * b + d].y += eta;
        inv[d * b + d].x = 1.0;
    }
    for (int c = 0; c < b; c++) {
        int piv = c;
        double best = -1.0;
        for (int r = c; r < b; r++) {
            const double a = W[r * b + c].x * W[r * b + c].x + W[r * b + c].y * W[r * b + c].y;
            if (a > best) { best = a; piv = r; }
        }
        if (piv != c)
            for (int q = 0; q < b; q++) {
                double2 t = W[c * b + q]; W[c * b + q] = W[piv * b + q]; W[piv * b + q] = t;
                t = inv[c * b + q]; inv[c * b + q] = inv[piv * b + q]; inv[piv * b + q] = t;
            }
        const double2 p = W[c * b + c];
        const double pd = p.x * p.x + p.y * p.y;
        const double2 pinv = make_double2(p.x / pd, -p.y / pd);
        for (int q = 0; q < b; q++) {
            W[c * b + q] = cmul(W[c * b + q], pinv);
            inv[c * b + q] = cmul(inv[c * b + q], pinv);
        }
        for (int r = 0; r < b; r++) {
            if (r == c) continue;
            const double2 f = W[r * b + c];
            for (int q = 0; q < b; q++) {
                W[r * b + q] = csub(W[r * b + q], cmul(f, W[c * b + q]));
                inv[r * b + q] = csub(inv[r * b + q], cmul(f, inv[c * b + q]));
            }
        }
    }
}

template <int B>
__device__ __forceinline__ double zfrob(int b, const double2 *A)
{
    double v = 0.0;
    for (int e = 0; e < b * b; e++) v += A[e].x * A[e].x + A[e].y * A[e].y;
    return sqrt(v);   // matnorm, src/qpi.cc:55-61
}

// One thread per (k-point, energy): decimation and G0(k) planes g0k[e][o*b+a][k].
template <int B, class C>
__global__ void __launch_bounds__(128) surface_greens_kernel(int b, long long nk, int surface, int max_iter,
                                                             double eta, double epserr,
                                                             const double *__restrict__ energies,
                                                             const double2 *__restrict__ mats, C *__restrict__ g0k,
                                                             int *status)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    const int e = blockIdx.y;
    const int bb = b * b;
    const double w = energies[e];
    double2 es[B * B], eb[B * B], al[B * B], be[B * B], g[B * B], t1[B * B], t2[B * B];
    for (int q = 0; q < bb; q++) {
        es[q] = mats[k * bb + q];
        eb[q] = mats[((size_t)nk + k) * bb + q];
        al[q] = mats[((size_t)2 * nk + k) * bb + q];
    }
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) be[r * b + c] = make_double2(al[c * b + r].x, -al[c * b + r].y);
    int it = 0;
    bool more = true;
    while (more && it < max_iter) {
        zresolvent<B>(b, eb, w, eta, t1, g);
        zmm<B>(b, g, be, t1);
        zmm<B>(b, al, t1, t2);                        // alpha g beta
        for (int q = 0; q < bb; q++) { es[q] = cadd(es[q], t2[q]); eb[q] = cadd(eb[q], t2[q]); }
        zmm<B>(b, g, al, t1);
        zmm<B>(b, be, t1, t2);                        // beta g alpha
        for (int q = 0; q < bb; q++) eb[q] = cadd(eb[q], t2[q]);
        zmm<B>(b, al, t1, t2);                        // alpha g alpha (t1 = g alpha)
        for (int q = 0; q < bb; q++) al[q] = t2[q];
        zmm<B>(b, g, be, t1);
        zmm<B>(b, be, t1, t2);                        // beta g beta
        for (int q = 0; q < bb; q++) be[q] = t2[q];
        it++;
        more = zfrob<B>(b, al) > epserr || zfrob<B>(b, be) > epserr;
    }
    if (more) atomicOr(status, 4);
    zresolvent<B>(b, surface ? es : eb, w, eta, t1, g);
    C *out = g0k + (size_t)e * bb * nk + k;
    for (int q = 0; q < bb; q++) out[(size_t)q * nk] = cmake<C>(g[q].x, g[q].y);
}

void launch_surface_mats(cqpi_handle *h)
{
    const long long nk = (long long)h->kp * h->kp;
    const SurfaceTerms &s = h->surf;
    surface_mats_kernel<<<cdiv(nk, 128), 128, 0, h->stream>>>(
        h->b, h->kp, s.ns, s.d_i + s.off_s, s.d_t + s.off_s, s.nb, s.d_i + s.off_b, s.d_t + s.off_b, s.no,
        s.d_i + s.off_o, s.d_t + s.off_o, s.d_anti + s.off_s, s.d_anti + s.off_b, s.d_anti + s.off_o, h->efermi,
        h->scmax, h->surf.d_mats);
    h->launches++;
}

template <int B>
static void launch_surface_t(cqpi_handle *h, int ne, const double *d_energies)
{
    const long long nk = (long long)h->kp * h->kp;
    dim3 grid(cdiv(nk, 128), ne);
    const int surface = h->gmode == CQPI_GREEN_SURFACE ? 1 : 0;
    const char *mi = getenv("CQPI_SURFACE_MAX_ITER");
    const int max_iter = mi ? std::max(1, std::min(CQPI_SURFACE_MAX_ITER, atoi(mi))) : CQPI_SURFACE_MAX_ITER;
    if (h->precision == CQPI_PREC_FP64)
        surface_greens_kernel<B, double2><<<grid, 128, 0, h->stream>>>(h->b, nk, surface, max_iter, h->eta, h->epserr,
                                                                       d_energies, h->surf.d_mats, h->ws.g0k,
                                                                       h->d_status);
    else
        surface_greens_kernel<B, float2><<<grid, 128, 0, h->stream>>>(h->b, nk, surface, max_iter, h->eta, h->epserr,
                                                                      d_energies, h->surf.d_mats, h->ws.g0k32,
                                                                      h->d_status);
    h->launches++;
}

void launch_greens_surface(cqpi_handle *h, int ne, const double *d_energies)
{
    const int b = h->b;
    if (b <= 1) launch_surface_t<1>(h, ne, d_energies);
    else if (b <= 2) launch_surface_t<2>(h, ne, d_energies);
    else if (b <= 3) launch_surface_t<3>(h, ne, d_energies);
    else if (b <= 4) launch_surface_t<4>(h, ne, d_energies);
    else if (b <= 6) launch_surface_t<6>(h, ne, d_energies);
    else launch_surface_t<8>(h, ne, d_energies);
}

}  // namespace cqpi
