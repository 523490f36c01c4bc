// spectral.cu -- k-space outputs: spectral function, unfolded spectral function, density of
// states (output=spf|uspf, dosfile).
//
//   spf   tmatrix::calcspf(maxband, shift) (src/qpi.cc:659-683): map[x][y] = -sum_{l<m} Im G0(k)_ll
//         at k = ((x + kp/2) mod kp, (y + kp/2) mod kp) on an n x n k-grid (kpoints = lattice);
//   uspf  tmatrix::calcuspf (src/qpi.cc:735-775): map[i][j] = -sum_{k,l} p_k p_l
//         Im(G0(ki,kj)[l][k] e^{2 pi i (kx (x_k - x_l) + ky (y_k - y_l))}) with kx = (i - n/2)/kp,
//         ki = ((i + n/2) mod n) mod kp; with spin the two blocks of maxband/2 orbitals;
//   dos   tmatrix::calcdos (src/qpi.cc:856-862): -sum_{i<m} Im G0(R=0)_ii, read from the centre
//         of the G0(R) box of each energy.
// G0(k) comes from the FP64 eigen cache (normal Green's function) or from the G0(k) planes
// of the surface / bulk decimation.  One thread per map pixel; tiny next to the LDOS.
#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

// G0(k)[l][c] = sum_n U[l][n] conj(U[c][n]) / (w - e_n + i eta) from the FP64 eigen cache
struct EigG0 {
    const double *eval;
    const double2 *evec;
    long long nk;
    int b;
    double eta;
    __device__ double2 operator()(int e, double w, long long k, int l, int c) const
    {
        (void)e;
        double2 s = make_double2(0.0, 0.0);
        for (int n = 0; n < b; n++) {
            const double dr = w - eval[(size_t)n * nk + k];
            const double den = dr * dr + eta * eta;
            const double2 f = make_double2(dr / den, -eta / den);
            const double2 ul = evec[((size_t)l * b + n) * nk + k], uc = evec[((size_t)c * b + n) * nk + k];
            const double2 x = cmul(ul, f);
            s.x += x.x * uc.x + x.y * uc.y;   // x * conj(uc)
            s.y += x.y * uc.x - x.x * uc.y;
        }
        return s;
    }
};

// G0(k) planes g0k[e][l*b+c][k] written by the surface / bulk decimation
template <class C>
struct PlaneG0 {
    const C *g0k;
    long long nk;
    int b;
    __device__ double2 operator()(int e, double w, long long k, int l, int c) const
    {
        (void)w;
        return to_d2(g0k[((size_t)e * b * b + (size_t)l * b + c) * nk + k]);
    }
};

// kind 0: spf, 1: uspf.  out[(e * n + y) * n + x] = map[x][y] (IDL order)
template <class Src>
__global__ void __launch_bounds__(128) spectral_kernel(int kind, int n, int kp, int maxband, int spin, Src src,
                                                       const double *__restrict__ energies, int e_base,
                                                       const double *__restrict__ pos, const double *__restrict__ pre,
                                                       double *__restrict__ out)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= n * n) return;
    const int e = blockIdx.y;
    const double w = energies[e];
    const int x = pix % n, y = pix / n;
    double tr = 0.0;
    if (kind == 0) {
        const int ks = kp >> 1;
        const long long k = (long long)((x + ks) % kp) * kp + (y + ks) % kp;
        for (int l = 0; l < maxband; l++) tr -= src(e, w, k, l, l).y;
    } else {
        const int h = n >> 1;
        const double kx = (double)(x - h) / kp, ky = (double)(y - h) / kp;
        const long long k = (long long)(((x + h) % n) % kp) * kp + ((y + h) % n) % kp;
        const int nblk = spin ? 2 : 1, mb = spin ? maxband >> 1 : maxband;
        for (int blk = 0; blk < nblk; blk++)
            for (int a = 0; a < mb; a++)
                for (int l = 0; l < mb; l++) {
                    const int ka = blk * mb + a, la = blk * mb + l;
                    double sn, cs;
                    sincospi(2.0 * (kx * (pos[2 * ka] - pos[2 * la]) + ky * (pos[2 * ka + 1] - pos[2 * la + 1])), &sn, &cs);
                    const double2 g = src(e, w, k, la, ka);
                    tr -= pre[ka] * pre[la] * (g.x * sn + g.y * cs);   // Im(g e^{i phi})
                }
    }
    out[((size_t)(e_base + e) * n + y) * n + x] = tr;
}

template <class C>
__global__ void dos_kernel(int ne, int NB, int Rb, int b, int maxband, const C *__restrict__ box, double *__restrict__ dos)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const C *g = box + (((size_t)e * NB + Rb) * NB + Rb) * b * b;
    double s = 0.0;
    for (int i = 0; i < maxband; i++) s -= (double)g[i * b + i].y;
    dos[e] = s;
}

void launch_spectral(cqpi_handle *h, int kind, int ne, int e_base, const double *d_energies, int maxband,
                     const double *d_pos, const double *d_pre, double *out)
{
    const long long nk = (long long)h->kp * h->kp;
    dim3 grid(cdiv((long long)h->n * h->n, 128), ne);
    if (h->gmode == CQPI_GREEN_NORMAL) {
        const EigG0 src = {h->d_eval, h->d_evec, nk, h->b, h->eta};
        spectral_kernel<EigG0><<<grid, 128, 0, h->stream>>>(kind, h->n, h->kp, maxband, h->spin, src, d_energies,
                                                            e_base, d_pos, d_pre, out);
    } else if (h->precision == CQPI_PREC_FP64) {
        const PlaneG0<double2> src = {h->ws.g0k, nk, h->b};
        spectral_kernel<PlaneG0<double2>><<<grid, 128, 0, h->stream>>>(kind, h->n, h->kp, maxband, h->spin, src,
                                                                       d_energies, e_base, d_pos, d_pre, out);
    } else {
        const PlaneG0<float2> src = {h->ws.g0k32, nk, h->b};
        spectral_kernel<PlaneG0<float2>><<<grid, 128, 0, h->stream>>>(kind, h->n, h->kp, maxband, h->spin, src,
                                                                      d_energies, e_base, d_pos, d_pre, out);
    }
    h->launches++;
}

void launch_dos(cqpi_handle *h, int ne, int maxband, double *dos)
{
    if (h->precision == CQPI_PREC_FP64)
        dos_kernel<double2><<<cdiv(ne, 64), 64, 0, h->stream>>>(ne, h->NB, h->Rb, h->b, maxband, h->ws.box, dos);
    else
        dos_kernel<float2><<<cdiv(ne, 64), 64, 0, h->stream>>>(ne, h->NB, h->Rb, h->b, maxband, h->ws.box32, dos);
    h->launches++;
}

}  // namespace cqpi
