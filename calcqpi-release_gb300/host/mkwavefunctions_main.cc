// mkwavefunctions_main.cc -- `mkwavefunctions <configfile>`: the reference's orbital-file
// tool (src/mkwavefunctions.cc:72-436) on the project's host library.  It writes the
// tip-overlap orbital cache, (2 window + 1) oversamp pixels square per orbital, as an IDL
// file that calcqpi reads back with idlorbitalfile=.
//
// Keywords and defaults follow the reference (window 2, oversamp 4, radius 0.5, angle 0,
// zheight 5).  Exactly one orbital source is used, in the reference's order of precedence:
//   modorbitalfiles  XSF files placed per orbital (orbitals = file indices, modpos[k],
//                    pos[i], angle / anglearr, zheight, basisvector[0/1] in Angstrom)
//                    (:184-226);
//   idlorbitalfile   an IDL orbital file, scaled by prearr (:228-255);
//   orbitals         analytic Slater-type orbitals (radius / radarr, angle / anglearr,
//                    phiarr, prearr, pos[i], zheight, basisvector[0/1]) (:256-300);
//   orbitalfiles     XSF files with a global shift, centred pixels, prearr (:301-324);
//   idlorbitalfiles  IDL orbital files interpolated pixel by pixel at 'interpolate' between
//                    'values' with 'interpmethod' (:325-393).
// then the boundary check (checkwavefunctions, :115-128), 'reorder', 'double' and the
// mkwffile output with its comment line (:394-433).
//
// Where the reference reads out of bounds or aborts (an index in 'orbitals' or 'reorder'
// past the list, fewer 'values' than files, files of different sizes, a point outside the
// 'values' range, an unknown orbital name, no orbital source) this tool stops with an
// error message and exit code 1 instead.
#include <cmath>
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "config.h"
#include "cqpi.h"
#include "cqpi_host.h"
#include "log.h"

namespace {

using cqpi_cli::Log;
using Cache = std::vector<double>;   // side x side, [i][j]

void help()
{
    std::cerr << "mkwavefunctions (" << cqpi_version() << ")\n\n"
              << "Syntax:\nmkwavefunctions configfile\n\n"
              << "Parameters of the configuration file:\n"
              << " logfile, tbfile, mkwffile (output), oversamp (4), window (2)\n"
              << "Slater-type orbitals:\n"
              << " orbitals, radius (0.5), radarr, angle (0.0), anglearr, phiarr, prearr, pos[i], zheight (5.0),\n"
              << " basisvector[0], basisvector[1]\n"
              << "DFT / Wannier90 orbitals:\n"
              << " orbitalfiles (XSF), shift, prearr, zheight; idlorbitalfile, prearr\n"
              << " modorbitalfiles (XSF), modpos[k], orbitals (file indices), pos[i], angle, anglearr, zheight\n"
              << "Interpolation of orbital files:\n"
              << " idlorbitalfiles, values, interpolate (0.5),\n"
              << " interpmethod (linear, polynomial, cspline, cspline_periodic, akima, akima_periodic, steffen)\n"
              << "Reorganising orbitals:\n"
              << " double, reorder\n";
}

struct IdlOrbitals {
    cqpi_idl_header hdr;
    std::vector<float> raw;   // [k][y][x]
    float at(size_t i, size_t j, size_t k) const { return raw[(k * hdr.size[1] + j) * hdr.size[0] + i]; }
};

bool load_idl(const std::string &path, IdlOrbitals &o)
{
    if (cqpi_idl_read_header(path.c_str(), &o.hdr) != CQPI_OK) return false;
    o.raw.resize((size_t)o.hdr.size[0] * o.hdr.size[1] * o.hdr.size[2]);
    return cqpi_idl_read(path.c_str(), o.raw.data(), (int64_t)o.raw.size()) == CQPI_OK;
}

void check_wavefunctions(Log &log, const std::vector<Cache> &wfs, size_t side)
{
    double worst = 0.0;
    log << "Checking wave functions:\n";
    for (size_t o = 0; o < wfs.size(); o++) {
        double mx = 0.0, bnd = 0.0;
        for (size_t i = 0; i < side; i++)
            for (size_t j = 0; j < side; j++) {
                const double v = std::fabs(wfs[o][i * side + j]);
                mx = std::max(mx, v);
                if (i == 0 || j == 0 || i == side - 1 || j == side - 1) bnd = std::max(bnd, v);
            }
        const double ratio = bnd / mx;
        log << " Wave function " << o << ": Max:" << mx << ", Max at boundary: " << bnd << ", Ratio: " << ratio << "\n";
        if (ratio > worst) worst = ratio;
    }
    log << "---------------------------\nMaximum rel. value at boundary: " << worst << "\n";
    if (worst > 0.05) log << "Warning: boundary too close, use larger window size!\n";
}

std::vector<double> pos_of(InputFile &lf, size_t i, bool &found)
{
    std::ostringstream key;
    key << "pos[" << i << "]";
    found = lf.has(key.str());
    std::vector<double> p;
    if (found) p = lf.vec(key.str());
    p.resize(3, 0.0);
    return p;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        help();
        return 0;
    }
    long window = 2, oversamp = 4;
    double radius = 0.5, angle = 0.0, zheight = 5.0;
    Log log;
    std::ostringstream cfgerr;
    InputFile lf(argv[1], cfgerr);
    if (!lf.ok()) {
        std::cerr << cfgerr.str();
        return 1;
    }
    if (lf.has("logfile")) log.open_append(lf.str("logfile"));
    log << "mkwavefunctions (" << cqpi_version() << "), setting wave functions from " << argv[1] << "\n";
    if (!cfgerr.str().empty()) log << "Error while reading configuration file:\n" << cfgerr.str();
    if (!lf.has("mkwffile")) {
        log << "No output file specified, exiting.\n";
        return 1;
    }
    if (lf.has("oversamp")) oversamp = lf.ivalue("oversamp");
    if (lf.has("window")) window = lf.ivalue("window");
    log << "Parameters of calculation:\n"
        << "         window               : " << window << "\n"
        << "         oversamp             : " << oversamp << "\n";
    if (window < 0 || oversamp < 1) {
        log << "Error: window must be >= 0 and oversamp >= 1.\n";
        return 1;
    }
    const size_t side = (size_t)(2 * window + 1) * (size_t)oversamp;
    double basis[4];
    const double *bptr = nullptr;
    if (lf.has("basisvector[0]")) {
        std::vector<double> b0 = lf.vec("basisvector[0]");
        b0.resize(2, 0.0);
        if (!lf.has("basisvector[1]")) {
            log << "Error: only one basis vector specified.\n";
            return 1;
        }
        std::vector<double> b1 = lf.vec("basisvector[1]");
        b1.resize(2, 0.0);
        basis[0] = b0[0]; basis[1] = b0[1]; basis[2] = b1[0]; basis[3] = b1[1];
        bptr = basis;
        log << "Using basis vectors (" << b0[0] << "," << b0[1] << "), (" << b1[0] << "," << b1[1] << ").\n";
    }

    std::vector<Cache> wfs;
    if (lf.has("modorbitalfiles")) {
        log << "Using Wannier90/XSF-orbitals for vacuum overlap (mod code).\n";
        const std::vector<std::string> files = lf.strlist("modorbitalfiles");
        std::vector<std::vector<double>> modshift(files.size(), std::vector<double>(3, 0.0));
        for (size_t k = 0; k < files.size(); k++) {
            log << "Loading wave function file " << files[k] << ".\n";
            std::ostringstream key;
            key << "modpos[" << k << "]";
            if (lf.has(key.str())) {
                std::vector<double> p = lf.vec(key.str());
                p.resize(3, 0.0);
                for (int a = 0; a < 3; a++) modshift[k][a] = -p[a];
            }
        }
        const std::vector<double> orbitals = lf.vec("orbitals");
        if (lf.has("angle")) angle = lf.value("angle");
        if (lf.has("zheight")) zheight = lf.value("zheight");
        std::vector<double> anglearr;
        if (lf.has("anglearr")) anglearr = lf.vec("anglearr");
        anglearr.resize(orbitals.size(), 0.0);
        struct Placed { double x, y, h, theta; };
        std::vector<Placed> placed;
        for (size_t i = 0; i < orbitals.size(); i++) {
            const double on = orbitals[i];
            if (!(on >= 0.0) || (size_t)on >= files.size()) {
                log << "Error: orbital " << i << " refers to modorbitalfiles entry " << on << ", but only "
                    << files.size() << " are given.\n";
                return 1;
            }
            const size_t k = (size_t)on;
            bool found;
            const std::vector<double> p = pos_of(lf, i, found);
            const Placed pl = {p[0], p[1], zheight - p[2], (angle + anglearr[i]) * M_PI / 180.0};
            Cache a(side * side);
            if (cqpi_xsf_orbital_cache_mod(files[k].c_str(), modshift[k].data(), bptr, pl.h, pl.x, pl.y, pl.theta,
                                           1.0, (int32_t)window, (int32_t)oversamp, a.data()) != CQPI_OK) {
                log << cqpi_host_last_error() << "\nError loading wave function file " << files[k] << "\n";
                return 1;
            }
            wfs.push_back(a);
            placed.push_back(pl);
        }
        log << "Parameters for Wannier functions:\n";
        for (size_t i = 0; i < placed.size(); i++)
            log << "Orbital " << i << ": @(" << placed[i].x << "," << placed[i].y << "), height " << placed[i].h
                << ", angle theta " << placed[i].theta * 180.0 / M_PI << "deg\n";
    } else if (lf.has("idlorbitalfile")) {
        const std::string of = lf.str("idlorbitalfile");
        log << "Using IDL orbital file for vacuum overlap.\nLoading wave function file " << of << ".\n";
        IdlOrbitals o;
        if (!load_idl(of, o)) {
            log << cqpi_host_last_error() << "\nError loading orbitals from file " << of << ", exiting.\n";
            return 1;
        }
        const size_t xs = o.hdr.size[0], ys = o.hdr.size[1], orbs = o.hdr.size[2];
        std::vector<double> prearr;
        if (lf.has("prearr")) prearr = lf.vec("prearr");
        prearr.resize(orbs, 1.0);
        if (xs != ys || xs != side) {
            log << "Orbital functions in " << of << " have unsuitable dimensions.\n";
            return 1;
        }
        for (size_t k = 0; k < orbs; k++) {
            Cache a(side * side);
            for (size_t i = 0; i < xs; i++)
                for (size_t j = 0; j < ys; j++) a[i * ys + j] = prearr[k] * (double)o.at(i, j, k);
            wfs.push_back(a);
        }
    } else if (lf.has("orbitals")) {
        const std::vector<std::string> orbitals = lf.list("orbitals");
        std::vector<double> radarr;
        if (lf.has("radius")) radius = lf.value("radius");
        if (lf.has("radarr")) radarr = lf.vec("radarr");
        if (lf.has("angle")) angle = lf.value("angle");
        if (lf.has("zheight")) zheight = lf.value("zheight");
        {
            std::ostringstream r;
            if (radarr.empty()) r << radius;
            for (size_t i = 0; i < radarr.size(); i++) r << (i ? " " : "") << radarr[i];
            log << "Using gaussian orbitals for vacuum overlap.\n    Parameters:\n"
                << "             Radius:         " << r.str() << "\n"
                << "             Rotation angle: " << angle << "\n"
                << "             Height:         " << zheight << "\n";
        }
        std::vector<double> anglearr, phiarr, prearr;
        if (lf.has("anglearr")) anglearr = lf.vec("anglearr");
        anglearr.resize(orbitals.size(), 0.0);
        if (lf.has("phiarr")) phiarr = lf.vec("phiarr");
        phiarr.resize(orbitals.size(), 0.0);
        if (lf.has("prearr")) prearr = lf.vec("prearr");
        prearr.resize(orbitals.size(), 1.0);
        log << "Parameters for Wannier functions:\n";
        struct Spec { double r, x, y, h, theta, phi; };
        std::vector<Spec> specs;
        for (size_t i = 0; i < orbitals.size(); i++) {
            if (!cqpi_orbital_known(orbitals[i].c_str())) {
                log << "Unknown orbital type " << orbitals[i] << " - exiting.\n";
                return 1;
            }
            bool found;
            const std::vector<double> p = pos_of(lf, i, found);
            const double r = radarr.empty() ? radius : radarr[i % radarr.size()];
            specs.push_back({r, p[0], p[1], zheight - p[2], (angle + anglearr[i]) * M_PI / 180.0,
                             phiarr[i] * M_PI / 180.0});
            const std::string nm = orbitals[i] == "z" ? "zero" : orbitals[i];
            log << "Orbital " << i << ": " << nm << "@(" << p[0] << "," << p[1] << "), height " << zheight - p[2]
                << ", angle theta " << specs[i].theta * 180.0 / M_PI << "deg, phi " << phiarr[i] << " deg, radius="
                << r << "\n";
        }
        log << "Precalculating wave functions.\n";
        for (size_t i = 0; i < specs.size(); i++) {
            Cache a(side * side);
            cqpi_orbital_cache_basis(orbitals[i].c_str(), specs[i].r, specs[i].h, specs[i].x, specs[i].y,
                                     specs[i].theta, specs[i].phi, prearr[i], bptr, (int32_t)window,
                                     (int32_t)oversamp, a.data());
            wfs.push_back(a);
        }
        log << "Done.\n";
    } else if (lf.has("orbitalfiles")) {
        if (lf.has("zheight")) zheight = lf.value("zheight");
        log << "Using Wannier90/XSF-orbitals for vacuum overlap.\n    Parameters:\n"
            << "             zheight:         " << zheight << "\n";
        const std::vector<std::string> files = lf.strlist("orbitalfiles");
        std::vector<double> prearr;
        if (lf.has("prearr")) prearr = lf.vec("prearr");
        prearr.resize(files.size(), 1.0);
        std::vector<double> shift(3, 0.0);
        if (lf.has("shift")) {
            shift = lf.vec("shift");
            shift.resize(3, 0.0);
        }
        log << "Applying global shift of (" << shift[0] << "," << shift[1] << "," << shift[2] << ")\n";
        for (size_t i = 0; i < files.size(); i++) {
            log << "Loading wave function file " << files[i] << ".\n";
            Cache a(side * side);
            if (cqpi_xsf_orbital_cache_shifted(files[i].c_str(), shift.data(), 1, zheight, (int32_t)window,
                                               (int32_t)oversamp, prearr[i], a.data()) != CQPI_OK) {
                log << cqpi_host_last_error() << "\nError loading wave function file " << files[i] << "\n";
                return 1;
            }
            wfs.push_back(a);
        }
    } else if (lf.has("idlorbitalfiles")) {
        const std::vector<std::string> files = lf.strlist("idlorbitalfiles");
        const size_t nf = files.size();
        std::string method = "linear";
        std::vector<double> values;
        double x = 0.5;
        if (lf.has("values")) values = lf.vec("values");
        else
            for (size_t i = 0; i < nf; i++) values.push_back(nf > 1 ? (double)i / (double)(nf - 1) : 0.0);
        if (lf.has("interpolate")) x = lf.value("interpolate");
        if (lf.has("interpmethod")) {
            const std::string im = lf.str("interpmethod");
            log << "Setting interpolation method to " << im << "\n";
            if (cqpi_interp_known(im.c_str())) method = im;
            else log << "Unknown interpolation method '" << im << "'\n";
        }
        if (values.size() < nf) {
            log << "Error: " << values.size() << " values for " << nf << " orbital files.\n";
            return 1;
        }
        std::vector<IdlOrbitals> in(nf);
        for (size_t f = 0; f < nf; f++) {
            log << "Loading orbital file " << files[f] << "\n";
            if (!load_idl(files[f], in[f])) {
                log << cqpi_host_last_error() << "\nError loading orbitals from file " << files[f] << ", exiting.\n";
                return 1;
            }
            for (int a = 0; a < 3; a++)
                if (in[f].hdr.size[a] != in[0].hdr.size[a]) {
                    log << "Error: orbital file " << files[f] << " differs in size from " << files[0] << ".\n";
                    return 1;
                }
        }
        if (nf == 0) {
            log << "Error: no orbital files to interpolate.\n";
            return 1;
        }
        log << "Interpolating model at value " << x << "\n";
        const size_t xs = in[0].hdr.size[0], ys = in[0].hdr.size[1], orbs = in[0].hdr.size[2];
        log << "Using interpolation type " << method << "\n";
        if (xs != ys || xs != side) {
            log << "Orbital functions in have unsuitable dimensions.\n";
            return 1;
        }
        std::vector<double> yv(nf);
        for (size_t k = 0; k < orbs; k++) {
            Cache a(side * side);
            for (size_t i = 0; i < xs; i++)
                for (size_t j = 0; j < ys; j++) {
                    for (size_t f = 0; f < nf; f++) yv[f] = (double)in[f].at(i, j, k);
                    if (cqpi_interp_eval(method.c_str(), (int32_t)nf, values.data(), yv.data(), 1, &x,
                                         &a[i * ys + j]) != CQPI_OK) {
                        log << "Error: interpolation '" << method << "' of " << nf << " files at " << x
                            << " failed (values must increase, x must lie within them, and the method needs enough"
                               " files).\n";
                        return 1;
                    }
                }
            wfs.push_back(a);
        }
    }
    if (wfs.empty()) {
        log << "No orbitals specified (modorbitalfiles=, idlorbitalfile=, orbitals=, orbitalfiles= or "
               "idlorbitalfiles=) - exiting.\n";
        return 1;
    }
    check_wavefunctions(log, wfs, side);
    if (lf.has("reorder")) {
        log << "Reordering orbitals.\n";
        const std::vector<double> ro = lf.vec("reorder");
        std::vector<Cache> nw;
        for (double v : ro) {
            if (!(v >= 0.0) || (size_t)v >= wfs.size()) {
                log << "Error: reorder index " << v << " out of range (" << wfs.size() << " orbitals).\n";
                return 1;
            }
            nw.push_back(wfs[(size_t)v]);
        }
        wfs.swap(nw);
    }
    if (lf.has("double")) {
        log << "Duplicating orbitals for spin-polarized calculation.\n";
        const size_t n0 = wfs.size();
        for (size_t i = 0; i < n0; i++) wfs.push_back(wfs[i]);
    }
    std::string tbfile;
    if (lf.has("tbfile")) tbfile = lf.str("tbfile");
    const std::string out = lf.str("mkwffile");
    std::vector<float> d(side * side * wfs.size());
    for (size_t l = 0; l < wfs.size(); l++)
        for (size_t i = 0; i < side; i++)
            for (size_t j = 0; j < side; j++) d[(l * side + j) * side + i] = (float)wfs[l][i * side + j];
    std::ostringstream c;
    c << "Wannier function file for " << tbfile << " with window=" << window << ", oversamp=" << oversamp
      << ", zheight=" << zheight;
    const double sr[2] = {1.0, 1.0}, of[2] = {0.0, 0.0}, bi[2] = {0.0, 0.0};
    log << "Writing wave function file to " << out << "\n";
    if (cqpi_idl_write(out.c_str(), c.str().c_str(), nullptr, (int32_t)side, (int32_t)side, (int32_t)wfs.size(), sr,
                       of, bi, 0.0, d.data()) != CQPI_OK) {
        log << cqpi_host_last_error() << "\n";
        return 1;
    }
    std::ostringstream un;
    lf.report_unused(un);
    if (!un.str().empty()) std::cerr << un.str();
    return 0;
}
