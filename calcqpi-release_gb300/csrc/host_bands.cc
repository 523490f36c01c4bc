// host_bands.cc -- the band-structure histogram of the bsfile keyword (CPU only).
//
// Replaces tightbind::calcbst3dhisthr(fname, pix, le, ue, layers, oversamp)
// (src/tightbinding.cc:1158-1193) as the driver calls it (src/calcqpi.cc:308-326).  The
// reference computes this side output on the host cores once per run, before the energy loop;
// so does this file, with one std::thread per host core over rows of pixels.  Per k-point of
// the (pix * oversamp)^2 grid k = (io / (pix*oversamp - 1) - 1/2, jo / (pix*oversamp - 1) - 1/2, 0):
//   H(k) = diag(-efermi for the first scmaxbands orbitals, +efermi after) + sum_terms
//          t e^{+-2 pi i (rx kx + ry ky)} (minus for the conjugated terms of a BdG model),
//          read through its lower triangle as gsl_eigen_hermv does;
//   its eigenvalues (cyclic complex Jacobi, this file's own);
//   every eigenvalue ev with le - 2 bin < ev < ue + 2 bin (bin = (ue - le) / (layers - 1))
//   adds the Lorentzian L(E_l - ev), L(x) = (w / 2) / (x^2 + w^2 / 4) / pi, w = 2 (ue - le) /
//   layers, to the layers l = round((ev - le) / (ue - le) (layers - 1)) + {-1, 0, 1} inside
//   [0, layers) of pixel (io / oversamp, jo / oversamp), E_l the layer energy of idl::getbias.
// Each pixel is summed by one thread in the reference's order (io, then jo, then the bands,
// here in ascending order); the reference's OpenMP loop over io can split the rows of one
// pixel between threads that then add into it concurrently, which this loop does not.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <thread>
#include <vector>

#include "cqpi.h"
#include "cqpi_host.h"

namespace {

using cplx = std::complex<double>;

// Eigenvalues of the Hermitian matrix whose lower triangle (and diagonal) A holds, by cyclic
// Jacobi rotations: a phase makes A[p][q] real, then the real rotation of the 2x2 block
// zeroes it (Numerical Recipes' form of the angle).  A is overwritten.
void hermitian_eigenvalues(std::vector<cplx> &A, int b, double *ev)
{
    for (int i = 0; i < b; i++) {
        A[i * b + i] = cplx(A[i * b + i].real(), 0.0);
        for (int j = 0; j < i; j++) A[j * b + i] = std::conj(A[i * b + j]);
    }
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < b; i++) {
            diag += std::norm(A[i * b + i]);
            for (int j = i + 1; j < b; j++) off += std::norm(A[i * b + j]);
        }
        if (off <= 1e-32 * diag || off == 0.0) break;
        for (int p = 0; p < b; p++)
            for (int q = p + 1; q < b; q++) {
                const cplx g = A[p * b + q];
                const double r = std::abs(g);
                if (r == 0.0) continue;
                const cplx uc = std::conj(g) / r;   // multiplies column q: A[p][q] becomes r
                const double app = A[p * b + p].real(), aqq = A[q * b + q].real();
                const double theta = (aqq - app) / (2.0 * r);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < b; k++) {
                    if (k == p || k == q) continue;
                    const cplx akp = A[k * b + p], akq = A[k * b + q] * uc;
                    const cplx nkp = c * akp - s * akq, nkq = s * akp + c * akq;
                    A[k * b + p] = nkp;
                    A[p * b + k] = std::conj(nkp);
                    A[k * b + q] = nkq;
                    A[q * b + k] = std::conj(nkq);
                }
                A[p * b + p] = cplx(app - t * r, 0.0);
                A[q * b + q] = cplx(aqq + t * r, 0.0);
                A[p * b + q] = A[q * b + p] = cplx(0.0, 0.0);
            }
    }
    for (int i = 0; i < b; i++) ev[i] = A[i * b + i].real();
    std::sort(ev, ev + b);
}

}  // namespace

extern "C" {

int cqpi_band_histogram(const cqpi_model *m, int32_t pix, int32_t oversamp, double le, double ue, int32_t layers,
                        double *out)
{
    if (!m || !out || pix < 1 || oversamp < 1 || layers < 1 || !(ue > le) || m->bands < 1 || m->nhops < 0 ||
        (m->nhops > 0 && (!m->R || !m->orb || !m->t)))
        return CQPI_ERR_ARG;
    for (int64_t h = 0; h < m->nhops; h++)
        if (m->orb[2 * h] < 0 || m->orb[2 * h] >= m->bands || m->orb[2 * h + 1] < 0 || m->orb[2 * h + 1] >= m->bands)
            return CQPI_ERR_ARG;
    const int b = m->bands;
    const long long ospix = (long long)pix * oversamp;
    const size_t plane = (size_t)pix * pix;
    std::fill(out, out + plane * (size_t)layers, 0.0);
    // one layer: every eigenvalue counts, into that layer (the reference's bin is infinite then)
    const double bin = layers > 1 ? (ue - le) / (layers - 1.0) : INFINITY;
    const double w = (ue - le) / layers * 2.0;
    auto lorentz = [w](double x) { return w / 2.0 / (x * x + w * w / 4.0) / M_PI; };
    auto layer_energy = [&](int l) { return layers == 1 ? le : (ue - le) * l / (layers - 1.0) + le; };
    const double kstep = ospix > 1 ? 1.0 / (double)(ospix - 1) : 0.0;
    std::atomic<int> next_row(0);
    auto worker = [&]() {
        std::vector<cplx> H((size_t)b * b);
        std::vector<double> ev(b);
        for (int i = next_row++; i < pix; i = next_row++)
            for (long long io = (long long)i * oversamp; io < (long long)(i + 1) * oversamp; io++)
                for (long long jo = 0; jo < ospix; jo++) {
                    const long long j = jo / oversamp;
                    const double kx = kstep * (double)io - 0.5, ky = kstep * (double)jo - 0.5;
                    std::fill(H.begin(), H.end(), cplx(0.0, 0.0));
                    for (int d = 0; d < b; d++) H[d * b + d] = cplx(d < m->scmaxbands ? -m->efermi : m->efermi, 0.0);
                    for (int64_t h = 0; h < m->nhops; h++) {
                        const double ph = 2.0 * M_PI * (m->R[3 * h] * kx + m->R[3 * h + 1] * ky);
                        const bool anti = m->anti && m->anti[h];
                        const cplx e(std::cos(ph), anti ? -std::sin(ph) : std::sin(ph));
                        H[m->orb[2 * h] * b + m->orb[2 * h + 1]] += cplx(m->t[2 * h], m->t[2 * h + 1]) * e;
                    }
                    hermitian_eigenvalues(H, b, ev.data());
                    for (int l = 0; l < b; l++) {
                        const double e = ev[l];
                        if (!(e > le - 2.0 * bin && e < ue + 2.0 * bin)) continue;
                        const int lay = layers > 1 ? (int)std::round((e - le) / (ue - le) * (layers - 1.0)) : 0;
                        for (int nl = lay - 1; nl <= lay + 1; nl++)
                            if (nl >= 0 && nl < layers)
                                out[(size_t)nl * plane + (size_t)j * pix + (size_t)i] += lorentz(layer_energy(nl) - e);
                    }
                }
    };
    const unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), (unsigned)pix));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (std::thread &t : pool) t.join();
    return CQPI_OK;
}

}  // extern "C"
