// gb300qpi.h -- the reference-side GPU backend for the GB300 engine: a GPUQPI
// (include/gpuqpi.h:18-32 of the reference) that forwards every call to libcqpi.so's C ABI.
//
// A maintainer adds this header to the reference's sources and one branch per constructor to
// tmatrix::allocgpumem (src/qpi.cc:290-321), next to the CUDA / Metal / HIP ones:
//     #elif _GB300
//     gpuqpi = (GPUQPI *)new GB300QPI(wanniern, kpoints, n, window, oversamp, bands, maxband, spin, wf);
//     ...    = (GPUQPI *)new GB300QPI(wanniern, kpoints, n, window, oversamp, bands, flags);
//     ...    = (GPUQPI *)new GB300QPI(kpoints, n, bands, maxbands, spin, pos, prearr);
// includes it after "gpuqpi.h" (src/qpi.cc:31-44), builds with -D_GB300 -D_GPU and links
// -lcqpi.  The reference then runs its own tmatrix (model, eigen-solve, G0, FFT, T) on the CPU
// and the LDOS contraction on the GB300: the A/B harness of the narrow seam.
//
// Semantics follow the reference's CUDA backend (src/qpicudakernel.cu:383-704): wannierldos /
// wannierjosephson / wannierldoslist start the contraction of one energy asynchronously from
// the host T-matrix and the host G0(R) grid; retrieveResult waits and copies the map, with
// map(x, y) at ldos[y * wanniern + x] in the flat form.  The contraction runs in FP64.
// Differences: GPUQPI's methods return nothing, so a failing call throws std::runtime_error
// with the engine's message (the CUDA backend prints and exits, src/qpicudakernel.cu:372-380);
// the k-space outputs (spf, uspf) are served by the wide seam (cqpi_spf / cqpi_uspf compute
// G0(k) on the GPU themselves) and throw on this seam.
#ifndef GB300QPI_H
#define GB300QPI_H

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cqpi.h"

class GB300QPI : public GPUQPI {
    cqpi_handle *h_ = nullptr;
    size_t kpoints_ = 0, bands_ = 0, wanniern_ = 0;
    bool josephson_ = false;
    std::vector<double> g0buf_, tbuf_, map_;

    void check(int rc, const char *what)
    {
        if (rc != CQPI_OK)
            throw std::runtime_error(std::string("GB300QPI: ") + what + ": " +
                                     (h_ ? cqpi_last_error(h_) : cqpi_status_string(rc)));
    }

    // the seam needs no model: T and G0(R) come from the reference's tmatrix each call
    void create(size_t n, size_t window, size_t oversamp, size_t maxband, bool spin)
    {
        const cqpi_model m = {(int32_t)bands_, (int32_t)bands_, 0.0, 0, nullptr, nullptr, nullptr, nullptr};
        const cqpi_params p = {(int32_t)n, (int32_t)kpoints_, (int32_t)oversamp, (int32_t)window, (int32_t)maxband,
                               spin ? 1 : 0, 0.0, CQPI_PREC_FP64};
        check(cqpi_create(&m, &p, &h_), "cqpi_create");
        g0buf_.resize(kpoints_ * kpoints_ * bands_ * bands_ * 2);
        tbuf_.resize(bands_ * bands_ * 2);
    }

    void set_orbitals(size_t window, size_t oversamp, size_t maxband, std::vector<wannierfunctions> *wf)
    {
        const size_t side = (2 * window + 1) * oversamp;
        std::vector<double> cube(maxband * side * side, 0.0);
        std::vector<uint8_t> zero(maxband, 1);
        for (size_t o = 0; wf && o < maxband; o++) {
            zero[o] = (*wf)[o].iszero() ? 1 : 0;
            if (!zero[o])
                for (size_t i = 0; i < side; i++)
                    for (size_t j = 0; j < side; j++) cube[(o * side + i) * side + j] = (*wf)[o].getwave_cached(i, j);
        }
        check(cqpi_set_orbitals(h_, cube.data(), (int32_t)maxband, (int32_t)side, zero.data()), "cqpi_set_orbitals");
    }

    void copy_in(gsl_matrix_complex *scat, std::vector<std::vector<gsl_matrix_complex *> > &g0)
    {
        for (size_t a = 0; a < bands_; a++)
            for (size_t o = 0; o < bands_; o++) {
                const gsl_complex c = gsl_matrix_complex_get(scat, a, o);
                tbuf_[2 * (a * bands_ + o)] = GSL_REAL(c);
                tbuf_[2 * (a * bands_ + o) + 1] = GSL_IMAG(c);
            }
        const size_t bb = bands_ * bands_;
        for (size_t x = 0; x < kpoints_; x++)
            for (size_t y = 0; y < kpoints_; y++) {
                const gsl_matrix_complex *M = g0[x][y];
                double *dst = &g0buf_[(x * kpoints_ + y) * bb * 2];
                if (M->tda == bands_) {
                    memcpy(dst, M->data, sizeof(double) * 2 * bb);
                } else {
                    for (size_t a = 0; a < bands_; a++)
                        for (size_t o = 0; o < bands_; o++) {
                            const gsl_complex c = gsl_matrix_complex_get(M, a, o);
                            dst[2 * (a * bands_ + o)] = GSL_REAL(c);
                            dst[2 * (a * bands_ + o) + 1] = GSL_IMAG(c);
                        }
                }
            }
    }

    void josephson(bool on)
    {
        if (on != josephson_) {
            // deltat / etat only shape cqpi_run's own tip factor; on this seam the tip comes per call
            check(cqpi_set_josephson(h_, on ? 1 : 0, 0.001, 0.0), "cqpi_set_josephson");
            josephson_ = on;
        }
    }

    const std::vector<double> &result()
    {
        map_.resize(wanniern_ * wanniern_);
        check(cqpi_retrieve_result(h_, map_.data()), "cqpi_retrieve_result");
        return map_;
    }

public:
    // LDOS and Josephson modes (CudaQPI(wanniern, kpoints, n, window, oversamp, bands, maxband, spin, wf))
    GB300QPI(size_t wanniern, size_t kpoints, size_t n, size_t window, size_t oversamp, size_t bands, size_t maxband,
             bool spin, std::vector<wannierfunctions> &wf)
        : kpoints_(kpoints), bands_(bands), wanniern_(wanniern)
    {
        create(n, window, oversamp, maxband, spin);
        set_orbitals(window, oversamp, maxband, &wf);
    }

    // proximity-list mode (CudaQPI(wanniern, kpoints, n, window, oversamp, bands, flaglist &)):
    // the list carries the orbital products, so the orbitals stay zero
    GB300QPI(size_t wanniern, size_t kpoints, size_t n, size_t window, size_t oversamp, size_t bands, flaglist &fl)
        : kpoints_(kpoints), bands_(bands), wanniern_(wanniern)
    {
        create(n, window, oversamp, bands, false);
        set_orbitals(window, oversamp, bands, nullptr);
        std::vector<int32_t> ent;
        std::vector<double> fac;
        const size_t wins = 2 * window + 1;
        for (size_t a = 0; a < wins; a++)
            for (size_t b = 0; b < wins; b++)
                for (size_t c = 0; c < wins; c++)
                    for (size_t d = 0; d < wins; d++)
                        for (const flaglistentry &e : fl[a][b][c][d]) {
                            const int32_t list = (int32_t)(((a * wins + b) * wins + c) * wins + d);
                            ent.insert(ent.end(), {list, (int32_t)e.i, (int32_t)e.j, (int32_t)e.o1, (int32_t)e.o2});
                            fac.push_back(e.factor);
                        }
        check(cqpi_set_list(h_, (int64_t)fac.size(), ent.data(), fac.data()), "cqpi_set_list");
    }

    // k-space outputs (CudaQPI(kpoints, n, bands, maxbands, spin, pos, prearr)): served by the
    // wide seam; the object exists so that allocgpumem succeeds, its spf / uspf throw
    GB300QPI(size_t kpoints, size_t n, size_t bands, size_t maxbands, bool spin, std::vector<std::vector<double> > &pos,
             std::vector<double> &prearr)
        : kpoints_(kpoints), bands_(bands), wanniern_(n)
    {
        (void)maxbands;
        (void)spin;
        (void)pos;
        (void)prearr;
    }

    void printinfo(ostream &os) { os << "Running continuum QPI on GB300 (" << cqpi_version() << ")." << endl; }

    void wannierldos(gsl_matrix_complex *scat, std::vector<std::vector<gsl_matrix_complex *> > &g0)
    {
        josephson(false);
        copy_in(scat, g0);
        check(cqpi_wannierldos(h_, tbuf_.data(), g0buf_.data()), "cqpi_wannierldos");
    }

    void wannierjosephson(gsl_matrix_complex *scat, std::vector<std::vector<gsl_matrix_complex *> > &g0,
                          gsl_complex tip)
    {
        josephson(true);
        copy_in(scat, g0);
        const double t[2] = {GSL_REAL(tip), GSL_IMAG(tip)};
        check(cqpi_wannierjosephson(h_, tbuf_.data(), g0buf_.data(), t), "cqpi_wannierjosephson");
    }

    void wannierldoslist(gsl_matrix_complex *scat, std::vector<std::vector<gsl_matrix_complex *> > &g0)
    {
        copy_in(scat, g0);
        check(cqpi_wannierldoslist(h_, tbuf_.data(), g0buf_.data()), "cqpi_wannierldoslist");
    }

    void spf(std::vector<std::vector<gsl_matrix_complex *> > &)
    {
        throw std::runtime_error("GB300QPI: spf runs through the wide seam (cqpi_spf)");
    }
    void uspf(std::vector<std::vector<gsl_matrix_complex *> > &)
    {
        throw std::runtime_error("GB300QPI: uspf runs through the wide seam (cqpi_uspf)");
    }

    void retrieveResult(std::vector<std::vector<double> > &ldos)
    {
        const std::vector<double> &t = result();
        ldos.resize(wanniern_);
        for (size_t x = 0; x < wanniern_; x++) {
            ldos[x].resize(wanniern_);
            for (size_t y = 0; y < wanniern_; y++) ldos[x][y] = t[y * wanniern_ + x];
        }
    }
    void retrieveResult(idl &map, size_t layer)
    {
        const std::vector<double> &t = result();
        for (size_t x = 0; x < wanniern_; x++)
            for (size_t y = 0; y < wanniern_; y++) map.set(x, y, layer, t[y * wanniern_ + x]);
    }
    void retrieveResult(double *ldos) { check(cqpi_retrieve_result(h_, ldos), "cqpi_retrieve_result"); }

    ~GB300QPI()
    {
        if (h_) cqpi_destroy(h_);
    }
};

#endif
