// calcqpi_main.cc -- `calcqpi <inputfile>`: the drop-in CLI of the reference's driver,
// running on the GB300 engine through the C ABI.
//
// Mirrors src/calcqpi.cc:131-811: the keywords and defaults (:133-137), model load
// (:277-292), surface-layer model and green=normal|surface|bulk with epserr (:203-209,
// :293-307, :683-688), scattering setup (:254-272, :393-395), the output modes
// wannier, josephson (:225, :249-251 deltat/etat, :451-460, :643-646, :705-709), spf / uspf
// (:333-334, :465-482, :647-652, :712-717) and nomode, the dosfile (:336-391), orbital setup
// from idlorbitalfile (:483-518), analytic orbitals (:519-576) or XSF orbitalfiles
// (:577-600), wffile output (:602-618), the proximity list of the threshold / spinarr
// keywords (:238, :619-635, :700-701), the map idl(n, n, layers, 2, 2, lenergy, henergy, 0,
// -1, -1) with its comment line (:638-656), layer energies idl::getbias (src/idl.cc:969-973)
// and the final save (:779-783), and the band-structure histogram of bsfile (:308-326, computed
// on the host cores as the reference does).  Extensions: precision=fp64|mixed,
// and flush / resume, which write the map group by group as the layers finish and continue
// an interrupted run from the layers already on disk.
#include <unistd.h>
#include <pwd.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "config.h"
#include "log.h"
#include "cqpi.h"
#include "cqpi_host.h"

using cplx = std::complex<double>;

namespace {

using cqpi_cli::Log;

struct Section {
    std::string name;
    double wall = 0.0, cpu = 0.0;
};

class Timings {
    std::vector<Section> secs_;
    std::chrono::steady_clock::time_point last_ = std::chrono::steady_clock::now();
    double lastcpu_ = cpu_now();
    static double cpu_now()
    {
        timespec ts;
        clock_gettime(CLOCK_PROCESS_CPUTIME_ID, &ts);
        return ts.tv_sec + 1e-9 * ts.tv_nsec;
    }

public:
    void add(const std::string &name)
    {
        auto now = std::chrono::steady_clock::now();
        double c = cpu_now();
        double w = std::chrono::duration<double>(now - last_).count(), dc = c - lastcpu_;
        last_ = now;
        lastcpu_ = c;
        for (auto &s : secs_)
            if (s.name == name) {
                s.wall += w;
                s.cpu += dc;
                return;
            }
        secs_.push_back({name, w, dc});
    }
    void print(Log &log) const
    {
        double tw = 0, tc = 0;
        for (auto &s : secs_) { tw += s.wall; tc += s.cpu; }
        log << "Summary of timings: \n";
        log << "     Section                            CPU time (s)            Real time (s)\n";
        for (auto &s : secs_) {
            std::ostringstream l;
            l << "     " << std::setw(33) << std::left << s.name << " " << std::setw(12) << std::right << std::fixed
              << std::setprecision(6) << s.cpu << " (" << std::setprecision(1) << std::setw(5)
              << (tc > 0 ? 100.0 * s.cpu / tc : 0.0) << "%)   " << std::setprecision(6) << std::setw(12) << s.wall
              << " (" << std::setprecision(1) << std::setw(5) << (tw > 0 ? 100.0 * s.wall / tw : 0.0) << "%)\n";
            log << l.str();
        }
        std::ostringstream l;
        l << "     Total time elapsed                " << std::fixed << std::setprecision(6) << std::setw(12) << tc
          << "           " << std::setw(12) << tw << "\n";
        log << l.str();
    }
};

void help()
{
    std::cerr << "calcqpi (GB300 continuum-LDOS engine, " << cqpi_version() << ")\n\n"
              << "Syntax:\ncalcqpi configfile\n\n"
              << "Keywords of the continuum-LDOS (wannier) path:\n"
              << " tbfile, qpifile, output (wannier, josephson, spf, uspf, nomode), logfile, wffile, dosfile,\n"
              << " doslayers (101), dosenergies ((-0.1,0.1)),\n"
              << " lattice (201), oversamp (4), energies (-1,1), layers (21), kpoints (=lattice),\n"
              << " green (normal|surface|bulk), stbfile, epserr (1e-5), fermi (0), scattering, phase ((1,0)), eta (0.005), spin, scmodel, magscat,\n"
              << " window (2; 0 = from the orbital range), radius (0.5), angle, anglearr, prearr, orbitals,\n"
              << " pos[i], zheight (5.0), idlorbitalfile, orbitalfiles, deltat (0.001), etat (=eta), threshold,\n"
              << " spinarr, bsfile, bslattice (201), bsoversamp (8), bsenergies ((-0.1,0.1)), bslayers (21)\n"
              << "Extensions: precision (fp64|mixed), flush (true: write each group of layers as it is done),\n"
              << " resume (true: continue a flushed run, computing only the layers not yet on disk)\n";
}

double getbias(double lb, double hb, size_t layers, size_t k)
{
    if (layers == 1) return lb;
    return (hb - lb) * (double)k / ((double)layers - 1.0) + lb;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        help();
        return 0;
    }
    size_t n = 201, layers = 21, oversamp = 4, window = 2, kpoints = 0;
    bool spin = false, scmodel = false;
    double lenergy = -1.0, henergy = 1.0, eta = 0.005, efermi = 0.0, radius = 0.5, angle = 0.0, zheight = 5.0,
           magscat = 0.0;
    cplx scatphase(1.0, 0.0);
    std::string tbfile, qpifile;
    std::vector<cplx> scattering;
    Timings timings;
    Log log;

    std::ostringstream cfgerr;
    InputFile lf(argv[1], cfgerr);
    if (!lf.ok()) {
        std::cerr << cfgerr.str();
        return 1;
    }
    if (lf.has("logfile")) log.open_append(lf.str("logfile"));
    log << "calcqpi (" << cqpi_version() << ")\n"
        << "New calculation started, using configuration from " << argv[1] << "\n";
    {
        char host[256] = {0};
        gethostname(host, sizeof host - 1);
        struct passwd *pw = getpwuid(geteuid());
        log << "Running on one GB300 GPU as user " << (pw ? pw->pw_name : "") << " on machine " << host << "\n";
    }
    if (!cfgerr.str().empty()) log << "Error while reading configuration file:\n" << cfgerr.str();

    if (lf.has("tbfile")) tbfile = lf.str("tbfile");
    else {
        log << "No tightbinding model specified ... exiting.\n";
        return 1;
    }
    std::string stbfile;
    if (lf.has("stbfile")) stbfile = lf.str("stbfile");
    if (lf.has("fermi")) efermi = lf.value("fermi");
    double epserr = 1e-5;
    if (lf.has("epserr")) epserr = lf.value("epserr");
    int gmode = CQPI_GREEN_NORMAL;   // green keyword (src/calcqpi.cc:206-209)
    if (lf.has("green")) {
        std::string g = lf.field("green");
        if (g == "surface") gmode = CQPI_GREEN_SURFACE;
        else if (g == "bulk") gmode = CQPI_GREEN_BULK;
        else if (g != "normal") log << "Invalid value for green: " << g << "\n";
    }
    if (lf.has("spin")) {
        std::string s = lf.field("spin");
        if (s == "true") spin = true;
        else if (s == "false") spin = false;
        else log << "Invalid value for spin: " << s << "\n";
    }
    if (lf.has("scmodel")) {
        std::string s = lf.field("scmodel");
        if (s == "true") scmodel = true;
        else if (s == "false") scmodel = false;
        else log << "Invalid value for scmodel: " << s << "\n";
    }
    // output mode (src/calcqpi.cc:127,221-229)
    enum { OUT_WANNIER, OUT_JOSEPHSON, OUT_SPF, OUT_USPF, OUT_NONE } outmode = OUT_WANNIER;
    if (lf.has("output")) {
        std::string o = lf.field("output");
        if (o == "josephson") outmode = OUT_JOSEPHSON;
        else if (o == "spf") outmode = OUT_SPF;
        else if (o == "uspf") outmode = OUT_USPF;
        else if (o == "nomode") outmode = OUT_NONE;
        else if (o != "wannier") {
            log << "Unrecognized output mode.";
            return 1;
        }
    }
    if (lf.has("qpifile")) qpifile = lf.str("qpifile");
    if (lf.has("lattice")) n = lf.ivalue("lattice");
    if (lf.has("oversamp")) oversamp = lf.ivalue("oversamp");
    if (lf.has("window")) window = lf.ivalue("window");
    // proximity list of the wannier mode (src/calcqpi.cc:238, :619-635, :700-701)
    double threshold = NAN;
    if (lf.has("threshold")) threshold = lf.value("threshold");
    if (lf.has("layers")) layers = lf.ivalue("layers");
    if (lf.has("energies")) {
        std::vector<double> e = lf.vec("energies");
        if (e.size() >= 2) { lenergy = e[0]; henergy = e[1]; }
    }
    if (lf.has("eta")) eta = lf.value("eta");
    // tip of the josephson mode: broadening defaults to the sample's (src/calcqpi.cc:249-251)
    double etat = NAN, deltat = 0.001;
    if (lf.has("etat")) etat = lf.value("etat");
    if (std::isnan(etat)) etat = eta;
    if (lf.has("deltat")) deltat = lf.value("deltat");
    if (lf.has("kpoints")) kpoints = lf.ivalue("kpoints");
    if (!kpoints) kpoints = n;
    if (outmode == OUT_SPF) kpoints = n;   // src/calcqpi.cc:333-334
    const bool josephson = outmode == OUT_JOSEPHSON;
    const bool kspace = outmode == OUT_SPF || outmode == OUT_USPF || outmode == OUT_NONE;   // no orbitals needed
    if (lf.has("phase")) {
        std::vector<double> ph = lf.vec("phase");
        ph.resize(2, 0.0);
        scatphase = cplx(ph[0], ph[1]);
        log << "Using scattering phase (" << ph[0] << "," << ph[1] << ")\n";
    }
    if (lf.has("scattering")) {
        std::vector<double> sl = lf.vec("scattering");
        for (double s : sl) scattering.push_back(s * scatphase);
        log << "Scattering: \n";
        std::ostringstream l;
        for (size_t i = 0; i < scattering.size(); i++)
            l << (i ? ",(" : "(") << scattering[i].real() << "," << scattering[i].imag() << ")";
        log << l.str() << "\n";
    }
    if (lf.has("magscat")) magscat = lf.value("magscat");
    // density of states file (src/calcqpi.cc:336-391)
    std::string dosfile;
    size_t doslayers = 101;
    double doslenergy = -0.1, doshenergy = 0.1;
    if (lf.has("dosfile")) {
        dosfile = lf.str("dosfile");
        if (lf.has("doslayers")) doslayers = lf.ivalue("doslayers");
        if (lf.has("dosenergies")) {
            std::vector<double> de = lf.vec("dosenergies");
            de.resize(2, 0.0);
            doslenergy = de[0];
            doshenergy = de[1];
        }
    }

    log << "Loading TB model " << tbfile << "\n";
    cqpi_hr *hr = nullptr;
    if (cqpi_read_hr(tbfile.c_str(), scmodel ? 1 : 0, &hr) != CQPI_OK) {
        log << cqpi_host_last_error() << "\n" << "Error loading TB model from " << tbfile << ", exiting.\n";
        return 1;
    }
    log << "Loading tb model from " << hr->name << " with " << hr->bands << " orbitals and " << hr->nrpts
        << " hopping terms.\n";
    const size_t bands = (size_t)hr->bands;
    size_t maxbands;
    if (scmodel) {
        maxbands = bands >> 1;
        log << "Assuming TB model to be superconducting, only first half of bands used.\n";
        size_t sl = scattering.size();
        if (sl == maxbands)
            for (size_t i = 0; i < sl; i++) scattering.push_back((-1.0 + 2.0 * magscat) * scattering[i]);
    } else {
        maxbands = bands;
    }
    // surface-layer model and the principal-layer check (src/calcqpi.cc:293-307)
    cqpi_hr *shr = nullptr;
    if (!stbfile.empty()) {
        log << "Loading surface TB model " << stbfile << "\n";
        if (cqpi_read_hr(stbfile.c_str(), scmodel ? 1 : 0, &shr) != CQPI_OK) {
            log << cqpi_host_last_error() << "\n" << "Error loading surface TB model from " << stbfile << ", exiting.\n";
            return 1;
        }
    }
    if (gmode != CQPI_GREEN_NORMAL) {
        auto principal = [](const cqpi_hr *m) {
            for (int64_t i = 0; i < m->nhops; i++)
                if (std::abs(m->R[3 * i + 2]) > 1 && (m->t[2 * i] != 0.0 || m->t[2 * i + 1] != 0.0)) return false;
            return true;
        };
        if (!principal(hr))
            log << "Warning: Tight-binding model in file " << tbfile << " is not in principal layer form.\n";
        if (shr && !principal(shr))
            log << "Warning: Surface tight-binding model in file " << stbfile << " is not in principal layer form.\n";
    }
    // band-structure histogram (src/calcqpi.cc:308-326), on the host cores as the reference
    if (lf.has("bsfile")) {
        size_t bslattice = 201, bslayers = 21, bsoversamp = 8;
        double bslenergy = -0.1, bshenergy = 0.1;
        const std::string bsfile = lf.str("bsfile");
        if (lf.has("bslayers")) bslayers = lf.ivalue("bslayers");
        if (lf.has("bsenergies")) {
            std::vector<double> be = lf.vec("bsenergies");
            be.resize(2, 0.0);
            bslenergy = be[0];
            bshenergy = be[1];
        }
        if (lf.has("bslattice")) bslattice = lf.ivalue("bslattice");
        if (lf.has("bsoversamp")) bsoversamp = lf.ivalue("bsoversamp");
        log << "Calculating band structure histogram in energy range (" << bslenergy << "," << bshenergy << ") with "
            << bslayers << " layers and oversampling " << bsoversamp << ".\n";
        const cqpi_model bm = {hr->bands, hr->scmaxbands, efermi, hr->nhops, hr->R, hr->orb, hr->t, hr->anti};
        std::vector<double> hist(bslattice * bslattice * bslayers);
        if (cqpi_band_histogram(&bm, (int32_t)bslattice, (int32_t)bsoversamp, bslenergy, bshenergy, (int32_t)bslayers,
                                hist.data()) != CQPI_OK) {
            log << "Error: invalid band-structure histogram parameters.\n";
            return 1;
        }
        const std::vector<float> hf(hist.begin(), hist.end());
        const double sr[2] = {1.0, 1.0}, of[2] = {-0.5, -0.5}, bi[2] = {bslenergy, bshenergy};
        if (cqpi_idl_write(bsfile.c_str(), hr->name, nullptr, (int32_t)bslattice, (int32_t)bslattice,
                           (int32_t)bslayers, sr, of, bi, 0.0, hf.data()) != CQPI_OK)
            log << "Error writing to stream.\n" << cqpi_host_last_error() << "\n";
        log << "... done and saved to " << bsfile << ".\n";
        timings.add("Bandstructure calculation");
    }
    double maxhop = 0.0;
    for (int64_t i = 0; i < hr->nhops; i++) maxhop = std::max(maxhop, std::hypot(hr->t[2 * i], hr->t[2 * i + 1]));
    if (maxhop / n < eta)
        log << "Note: Broadening eta (" << eta << ") large compared to maximum hopping (" << maxhop
            << ") at given k-point resolution (hopping/kpoints=" << maxhop / kpoints << ").\n";

    // scattering vector (tmatrix::setscatteringphase, src/qpi.h:107-130)
    std::vector<double> vscat(2 * bands, 0.0);
    for (size_t i = 0; i < bands; i++) {
        cplx v = scattering.empty() ? scatphase : (i < scattering.size() ? scattering[i] : cplx(0.0, 0.0));
        vscat[2 * i] = v.real();
        vscat[2 * i + 1] = v.imag();
    }
    {
        std::ostringstream l;
        l << "Parameters of calculation:\n"
          << "         Tight-binding model  : " << tbfile << "\n"
          << "         Surface tight-binding model: " << stbfile << "\n"
          << "         Output file for QPI  : " << qpifile << "\n"
          << "         Bands:               : " << maxbands << "\n"
          << "         Lattice              : " << n << "x" << n << "\n"
          << "         kpoints              : " << kpoints << "x" << kpoints << "\n"
          << "         energy range         : (" << lenergy << "," << henergy << ")\n"
          << "         energy layers        : " << layers << "\n"
          << "         Fermi energy         : " << efermi << "\n"
          << "         broadening parameter : " << eta << "\n"
          << "         window               : " << window << "\n"
          << "         oversamp             : " << oversamp << "\n"
          << "         epserr               : " << epserr << "\n";
        if (!std::isnan(threshold)) l << "         threshold            : " << threshold << "\n";
        l << "         Green's function     : "
          << (gmode == CQPI_GREEN_SURFACE ? "surface" : gmode == CQPI_GREEN_BULK ? "bulk" : "normal") << "\n"
          << (spin ? "         spin-polarized calculation\n" : "         paramagnetic calculation\n");
        log << l.str();
    }
    if (josephson) {
        std::ostringstream l;
        l << "QPI calculations in Josephson-mode.\n   using deltat=" << deltat << ", etat=" << etat << ".\n";
        log << l.str();
        if (!scmodel) {
            log << "Error: Calculation in josephson-mode with scmodel=false makes no sense - exiting.\n";
            return 1;
        }
    } else if (outmode == OUT_WANNIER) {
        log << "QPI calculations in Wannier-mode (cLDOS).\n";
    } else if (outmode == OUT_SPF) {
        log << "Calculations of spectral function.\n";
    } else if (outmode == OUT_USPF) {
        log << "Calculations of unfolded spectral function.\n";
    }
    // band positions of the unfolded spectral function (src/calcqpi.cc:465-478)
    std::vector<double> uspf_pos;
    if (outmode == OUT_USPF)
        for (size_t i = 0; i < maxbands; i++) {
            std::ostringstream key;
            key << "pos[" << i << "]";
            if (lf.has(key.str())) {
                std::vector<double> pos = lf.vec(key.str());
                pos.resize(2, 0.0);
                uspf_pos.push_back(pos[0]);
                uspf_pos.push_back(pos[1]);
            } else {
                uspf_pos.push_back(0.0);
                uspf_pos.push_back(0.0);
                log << "No position found for band " << i << ", using (0,0,0).\n";
            }
        }

    // ---------------------------------------------------------------- orbitals
    std::vector<double> prearr;
    if (lf.has("prearr")) prearr = lf.vec("prearr");
    prearr.resize(maxbands, 1.0);
    const std::vector<double> uspf_pre = prearr;   // before the orbital setups resize it
    std::vector<std::vector<double>> wfs;   // each (2w+1)os squared
    std::vector<uint8_t> zero;
    size_t side = 0;
    if (lf.has("idlorbitalfile")) {
        std::string of = lf.str("idlorbitalfile");
        log << "Using IDL orbital file for vacuum overlap.\nLoading wave function file " << of << ".\n";
        cqpi_idl_header hd;
        if (cqpi_idl_read_header(of.c_str(), &hd) != CQPI_OK) {
            log << "Error loading orbitals from file " << of << ", exiting.\n";
            return 1;
        }
        const size_t xs = hd.size[0], ys = hd.size[1], orbs = hd.size[2];
        prearr.resize(orbs, 1.0);
        if (xs != ys || xs != (2 * window + 1) * oversamp) {
            log << "Orbital functions in " << of << " have unsuitable dimensions.\n";
            return 1;
        }
        std::vector<float> raw(xs * ys * orbs);
        if (cqpi_idl_read(of.c_str(), raw.data(), (int64_t)raw.size()) != CQPI_OK) {
            log << "Error loading orbitals from file " << of << ", exiting.\n";
            return 1;
        }
        side = xs;
        for (size_t k = 0; k < orbs; k++) {
            std::vector<double> a(xs * ys);
            for (size_t i = 0; i < xs; i++)
                for (size_t j = 0; j < ys; j++) a[i * ys + j] = prearr[k] * (double)raw[(k * ys + j) * xs + i];
            wfs.push_back(a);
            zero.push_back(0);
        }
        if ((maxbands >> 1) == orbs && spin) {
            log << "Found half as many orbitals as needed in spin-polarized calculation, duplicating wave function set.\n";
            for (size_t k = 0; k < orbs; k++) { wfs.push_back(wfs[k]); zero.push_back(0); }
        } else if (maxbands > orbs) {
            log << "Warning: Fewer number of orbitals in " << of << " than there are bands, padding with zeros.\n";
            for (size_t i = orbs; i < maxbands; i++) { wfs.push_back(std::vector<double>(xs * ys, 0.0)); zero.push_back(1); }
        }
    } else if (lf.has("orbitals")) {
        std::vector<std::string> orbitals = lf.list("orbitals");
        if (lf.has("radius")) radius = lf.value("radius");
        if (lf.has("angle")) angle = lf.value("angle");
        if (lf.has("zheight")) zheight = lf.value("zheight");
        log << "Using gaussian orbitals for vacuum overlap.\n    Parameters:\n"
            << "             Radius:         " << radius << "\n"
            << "             Rotation angle: " << angle << "\n"
            << "             Height:         " << zheight << "\n";
        std::vector<double> anglearr;
        if (lf.has("anglearr")) anglearr = lf.vec("anglearr");
        anglearr.resize(orbitals.size(), 0.0);
        prearr.resize(orbitals.size(), 1.0);
        struct Spec { std::string name; double height, x, y, theta, pre; };
        std::vector<Spec> specs;
        for (size_t i = 0; i < orbitals.size(); i++) {
            if (!cqpi_orbital_known(orbitals[i].c_str())) {
                log << "Unknown orbital type " << orbitals[i] << " - exiting.\n";
                return 1;
            }
            std::ostringstream key;
            key << "pos[" << i << "]";
            double th = (angle + anglearr[i]) * M_PI / 180.0;
            if (lf.has(key.str())) {
                std::vector<double> pos = lf.vec(key.str());
                pos.resize(3, 0.0);
                specs.push_back({orbitals[i], zheight - pos[2], pos[0], pos[1], th, prearr[i]});
            } else {
                specs.push_back({orbitals[i], zheight, 0.0, 0.0, th, prearr[i]});
            }
        }
        if ((maxbands >> 1) == orbitals.size() && spin) {
            log << "Found half as many orbitals as needed in spin-polarized calculation, duplicating wave function set.\n";
            const size_t k0 = specs.size();
            for (size_t k = 0; k < k0; k++) specs.push_back(specs[k]);
        } else if (orbitals.size() < maxbands) {
            log << "Warning: Fewer number of orbitals specified than there are bands, padding with zeros.\n";
            for (size_t i = orbitals.size(); i < maxbands; i++) specs.push_back({"z", zheight, 0.0, 0.0, 0.0, 0.0});
        }
        log << "Parameters for Wannier functions:\n";
        for (size_t i = 0; i < specs.size(); i++) {
            std::string nm = specs[i].name == "z" ? "zero" : specs[i].name;
            log << "Orbital " << i << ": " << nm << "@(" << specs[i].x << "," << specs[i].y << "), height "
                << specs[i].height << ", theta " << specs[i].theta * 180.0 / M_PI << "deg \n";
        }
        if (window) {
            double val = radius * std::sqrt(std::log(100.0) + std::abs(zheight));
            log << "Recommended window size for r=" << radius << ": " << std::ceil(val * val - zheight * zheight)
                << "\nchosen window size: " << window << "\n";
        } else {
            for (auto &s : specs) {
                (void)s;
                double nw = std::ceil(radius * std::sqrt(std::log(1.0 / 0.01)));
                if (nw > window) window = (size_t)nw;
            }
            log << "Using recommended window size for r=" << radius << ": " << window << "\n";
        }
        log << "Precalculating wave functions.\n";
        side = (2 * window + 1) * oversamp;
        for (auto &s : specs) {
            std::vector<double> a(side * side);
            cqpi_orbital_cache(s.name.c_str(), radius, s.height, s.x, s.y, s.theta, 0.0, s.pre, (int32_t)window,
                               (int32_t)oversamp, a.data());
            wfs.push_back(a);
            zero.push_back(s.name == "z");
        }
        log << "Done.\n";
        double mx = 0.0;
        for (size_t o = 0; o < wfs.size(); o++) {
            if (zero[o]) continue;
            double m = 0.0, bnd = 0.0;
            for (size_t i = 0; i < side; i++)
                for (size_t j = 0; j < side; j++) {
                    double v = std::abs(wfs[o][i * side + j]);
                    m = std::max(m, v);
                    if (i == 0 || j == 0 || i == side - 1 || j == side - 1) bnd = std::max(bnd, v);
                }
            if (m > 0) mx = std::max(mx, bnd / m);
        }
        log << "Maximum rel. value at boundary: " << mx << "\n";
        if (mx > 0.05) log << "Warning: boundary too close, use larger window size!\n";
    } else if (lf.has("orbitalfiles")) {
        // DFT / Wannier90 orbitals from XSF files (src/calcqpi.cc:577-600)
        if (lf.has("zheight")) zheight = lf.value("zheight");
        {
            std::ostringstream l;
            l << "Using Wannier90/XSF-orbitals for vacuum overlap.\n    Parameters:\n"
              << "             zheight:         " << zheight << "\n";
            log << l.str();
        }
        std::vector<std::string> files = lf.strlist("orbitalfiles");
        prearr.resize(files.size(), 1.0);
        side = (2 * window + 1) * oversamp;
        for (size_t i = 0; i < files.size(); i++) {
            log << "Loading wave function file " << files[i] << ".\n";
            std::vector<double> a(side * side);
            if (cqpi_xsf_orbital_cache(files[i].c_str(), zheight, (int32_t)window, (int32_t)oversamp, prearr[i],
                                       a.data()) != CQPI_OK) {
                log << cqpi_host_last_error() << "\nError loading wave function file " << files[i] << "\n";
                return 1;
            }
            wfs.push_back(a);
            zero.push_back(0);
        }
        if ((maxbands >> 1) == files.size() && spin) {
            log << "Found half as many orbitals as needed in spin-polarized calculation, duplicating wave function set.\n";
            for (size_t k = 0; k < files.size(); k++) { wfs.push_back(wfs[k]); zero.push_back(0); }
        } else if (files.size() < maxbands) {
            log << "Fewer number of orbital files specified than there are bands, padding with zeros.\n";
            // the reference counts the padding from its (empty) analytic orbital list, so
            // maxbands zero orbitals follow the files (src/calcqpi.cc:596-599); kept, since
            // the wffile output shows them
            for (size_t i = 0; i < maxbands; i++) { wfs.push_back(std::vector<double>(side * side, 0.0)); zero.push_back(1); }
        }
    } else if (!kspace) {
        log << "No orbitals specified (orbitals=, idlorbitalfile= or orbitalfiles=) - exiting.\n";
        return 1;
    }
    if (lf.has("wffile")) {
        std::vector<float> d(side * side * wfs.size());
        for (size_t l = 0; l < wfs.size(); l++)
            for (size_t i = 0; i < side; i++)
                for (size_t j = 0; j < side; j++) d[(l * side + j) * side + i] = (float)wfs[l][i * side + j];
        std::ostringstream c;
        c << "Wannier function file for " << tbfile << " with window=" << window << " and oversamp=" << oversamp;
        const double sr[2] = {1.0, 1.0}, of[2] = {0.0, 0.0}, bi[2] = {0.0, 0.0};
        log << "Writing wave function file to " << lf.str("wffile") << "\n";
        cqpi_idl_write(lf.str("wffile").c_str(), c.str().c_str(), nullptr, (int32_t)side, (int32_t)side,
                       (int32_t)wfs.size(), sr, of, bi, 0.0, d.data());
    }
    if (wfs.size() < maxbands && !kspace) {
        log << "Fewer orbitals than bands - exiting.\n";
        return 1;
    }

    // ---------------------------------------------------------------- engine
    if (outmode == OUT_NONE && dosfile.empty()) {
        // nothing left for the GPU (output=nomode: at most the band-structure histogram and
        // the wffile above)
        cqpi_hr_free(hr);
        if (shr) cqpi_hr_free(shr);
        timings.print(log);
        return 0;
    }
    cqpi_model model = {hr->bands, hr->scmaxbands, efermi, hr->nhops, hr->R, hr->orb, hr->t, hr->anti};
    cqpi_params par = {(int32_t)n, (int32_t)kpoints, (int32_t)oversamp, (int32_t)window, (int32_t)maxbands,
                       spin ? 1 : 0, eta, CQPI_PREC_FP64};
    if (lf.has("precision")) {
        std::string p = lf.field("precision");
        if (p == "mixed") par.precision = CQPI_PREC_MIXED;
        else if (p != "fp64") log << "Invalid value for precision: " << p << "\n";
    }
    cqpi_handle *h = nullptr;
    int rc = cqpi_create(&model, &par, &h);
    if (rc != CQPI_OK) {
        log << "Error: engine creation failed: " << cqpi_status_string(rc) << "\n";
        return 1;
    }
    std::vector<double> wflat(wfs.size() * side * side);
    for (size_t o = 0; o < wfs.size(); o++) std::copy(wfs[o].begin(), wfs[o].end(), wflat.begin() + o * side * side);
    if (wfs.size() >= maxbands) rc = cqpi_set_orbitals(h, wflat.data(), (int32_t)wfs.size(), (int32_t)side, zero.data());
    if (rc == CQPI_OK) rc = cqpi_set_scattering(h, vscat.data());
    if (rc == CQPI_OK && !std::isnan(threshold)) {
        log << "Creating threshold list ... done\n";
        std::vector<int32_t> spinarr;
        const bool use_spinarr = lf.has("spinarr");
        if (use_spinarr)
            for (double v : lf.vec("spinarr")) spinarr.push_back((int32_t)v);
        int64_t count = 0;
        rc = cqpi_set_threshold(h, threshold, use_spinarr ? spinarr.data() : nullptr, (int32_t)spinarr.size(), &count);
        if (rc == CQPI_OK) {
            const double w1 = 2.0 * window + 1.0;
            const double entries = w1 * w1 * w1 * w1 * oversamp * oversamp * wfs.size() * wfs.size();
            std::ostringstream l;
            l << "Threshold list has " << count << "/" << (size_t)entries << " entries (" << count / entries * 100.0
              << "%), requiring " << std::fixed << std::setprecision(2)
              << count * 40.0 / 1024.0 / 1024.0 / 1024.0 << "GB of memory.\n";
            log << l.str();
        }
    }
    if (rc == CQPI_OK && josephson) rc = cqpi_set_josephson(h, 1, deltat, etat);
    if (rc == CQPI_OK && gmode != CQPI_GREEN_NORMAL) {
        cqpi_model sm = {};
        if (shr) sm = {shr->bands, shr->scmaxbands, efermi, shr->nhops, shr->R, shr->orb, shr->t, shr->anti};
        rc = cqpi_set_greens(h, gmode, epserr, shr ? &sm : nullptr);
    }
    if (rc != CQPI_OK) {
        log << "Error: " << cqpi_last_error(h) << "\n";
        cqpi_destroy(h);
        return 1;
    }
    if (!dosfile.empty()) {
        std::ostringstream l;
        l << "Calculating density of states in energy range (" << doslenergy << "," << doshenergy << ") with "
          << doslayers << " layers.\n";
        log << l.str();
        const double step = (doshenergy - doslenergy) / doslayers;
        std::vector<double> de(doslayers), dv(doslayers);
        for (size_t k = 0; k < doslayers; k++) de[k] = doslenergy + k * step;
        rc = cqpi_dos(h, de.data(), (int32_t)doslayers, (int32_t)maxbands, dv.data());
        if (rc != CQPI_OK) {
            log << "Error: " << cqpi_last_error(h) << "\n";
            cqpi_destroy(h);
            return 1;
        }
        std::ofstream dosout(dosfile.c_str());
        for (size_t k = 0; k < doslayers; k++) dosout << doslenergy + k * step << " " << dv[k] << std::endl;
        log << "... done and saved to " << dosfile << ".\n";
        timings.add("Calculation of density of states");
    }
    if (outmode == OUT_NONE) {
        cqpi_destroy(h);
        cqpi_hr_free(hr);
        if (shr) cqpi_hr_free(shr);
        timings.print(log);
        return 0;
    }
    // maps: lattice*oversamp pixels per side for the real-space modes, lattice for the
    // spectral functions (src/calcqpi.cc:638-656)
    const size_t wn = kspace ? n : n * oversamp;
    std::ostringstream comment;
    if (outmode == OUT_SPF) comment << "SPF calculation for " << hr->name;
    else if (outmode == OUT_USPF) comment << "USPF calculation for " << hr->name << " with kpoints=" << kpoints;
    else
        comment << (josephson ? "Josephson calculation for " : "CQPI calculation for ") << hr->name << " with window="
                << window << " and oversamp=" << oversamp;
    timings.add("Initialization of calculation");

    std::vector<double> energies(layers);
    for (size_t k = 0; k < layers; k++) energies[k] = getbias(lenergy, henergy, layers, k);
    const double sr[2] = {2.0, 2.0}, of[2] = {-1.0, -1.0}, bi[2] = {lenergy, henergy};

    // flush=true / resume=true (an extension; the reference writes the map once at the end):
    // each group of layers goes into qpifile as soon as it is computed and its indices are
    // appended to <qpifile>.progress; resume=true continues such a run, computing only the
    // layers that file does not list.  The finished file equals the one-shot output.
    const bool resume = lf.has("resume") && lf.field("resume") == "true";
    const bool flush = resume || (lf.has("flush") && lf.field("flush") == "true");
    const std::string progress = qpifile + ".progress";
    std::vector<uint8_t> done(layers, 0);
    if (flush) {
        bool reuse = false;
        if (resume) {
            cqpi_idl_header hd;
            std::ifstream pf(progress.c_str());
            if (pf && cqpi_idl_read_header(qpifile.c_str(), &hd) == CQPI_OK) {
                // the header holds the energies as the stream printed them
                auto printed = [](double v) {
                    std::ostringstream o;
                    o << v;
                    return o.str();
                };
                if ((size_t)hd.size[0] != wn || (size_t)hd.size[1] != wn || (size_t)hd.size[2] != layers ||
                    printed(hd.bias[0]) != printed(lenergy) || printed(hd.bias[1]) != printed(henergy) ||
                    comment.str() != hd.name) {
                    log << "Error: " << qpifile << " does not belong to this calculation (size, energies or model"
                        << " differ); not resuming over it.\n";
                    cqpi_destroy(h);
                    return 1;
                }
                long k;
                while (pf >> k)
                    if (k >= 0 && (size_t)k < layers) done[(size_t)k] = 1;
                reuse = true;
                size_t nd = 0;
                for (uint8_t d : done) nd += d;
                log << "Resuming " << qpifile << ": " << nd << " of " << layers << " layers already computed.\n";
            } else {
                log << "Nothing to resume (" << qpifile << " or " << progress << " missing), starting afresh.\n";
            }
        }
        if (!reuse) {
            if (cqpi_idl_create(qpifile.c_str(), comment.str().c_str(), nullptr, (int32_t)wn, (int32_t)wn,
                                (int32_t)layers, sr, of, bi, 0.0) != CQPI_OK) {
                log << "Error writing to stream.\n" << cqpi_host_last_error() << "\n";
                cqpi_destroy(h);
                return 1;
            }
            std::ofstream(progress.c_str(), std::ios::trunc);
        }
    }
    // without flush all layers stay in host memory until the final save; with flush one
    // group at a time
    const size_t group = 16;
    std::vector<float> maps(wn * wn * (flush ? std::min(group, layers) : layers));
    // energies go through the engine in groups of consecutive layers still to compute, so
    // that progress is reported (and flushed) per group
    for (size_t k0 = 0; k0 < layers;) {
        if (done[k0]) {
            k0++;
            continue;
        }
        size_t ne = 1;
        while (k0 + ne < layers && ne < group && !done[k0 + ne]) ne++;
        for (size_t k = k0; k < k0 + ne; k++) {
            std::ostringstream l;
            l << "Calculating layer " << k << " at energy " << std::fixed << std::setprecision(4) << energies[k] << "\n";
            log << l.str();
        }
        float *dst = maps.data() + (flush ? 0 : k0 * wn * wn);
        if (outmode == OUT_SPF)
            rc = cqpi_spf(h, energies.data() + k0, (int32_t)ne, (int32_t)maxbands, dst, nullptr);
        else if (outmode == OUT_USPF)
            rc = cqpi_uspf(h, energies.data() + k0, (int32_t)ne, (int32_t)maxbands, uspf_pos.data(), uspf_pre.data(),
                           dst, nullptr);
        else
            rc = cqpi_run(h, energies.data() + k0, (int32_t)ne, dst, nullptr, 0);
        if (rc != CQPI_OK) {
            log << "Error: " << cqpi_last_error(h) << "\n";
            cqpi_destroy(h);
            return 1;
        }
        timings.add("Calculation of CLDOS");
        if (flush) {
            if (cqpi_idl_write_layers(qpifile.c_str(), (int32_t)k0, (int32_t)ne, dst) != CQPI_OK) {
                log << "Error writing to stream.\n" << cqpi_host_last_error() << "\n";
                cqpi_destroy(h);
                return 1;
            }
            std::ofstream pf(progress.c_str(), std::ios::app);
            for (size_t k = k0; k < k0 + ne; k++) pf << k << "\n";
            timings.add("Saving data");
        }
        k0 += ne;
    }
    if (flush) {
        log << "Calculation finished.\nAll layers saved to " << qpifile << "\n";
        std::remove(progress.c_str());
    } else {
        log << "Calculation finished.\nSaving to " << qpifile << "\n";
        rc = cqpi_idl_write(qpifile.c_str(), comment.str().c_str(), nullptr, (int32_t)wn, (int32_t)wn, (int32_t)layers,
                            sr, of, bi, 0.0, maps.data());
        if (rc != CQPI_OK) log << "Error writing to stream.\n" << cqpi_host_last_error() << "\n";
    }
    log << "Done.\n";
    timings.add("Saving data");
    cqpi_destroy(h);
    cqpi_hr_free(hr);
    if (shr) cqpi_hr_free(shr);
    timings.print(log);
    std::ostringstream un;
    lf.report_unused(un);
    if (!un.str().empty()) std::cerr << un.str();
    return 0;
}
