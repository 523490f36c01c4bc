// refdump.cc -- project-written harness around the reference's own classes
// (tightbind, tmatrix, wannierfunctions from src/tightbinding.cc, src/qpi.cc,
// src/wannierfunctions.cc).  TEST INFRASTRUCTURE ONLY: oracle/build_ref.sh links
// it into oracle/_ref/refdump, and tests/golden/make_golden.py runs it to record
// full-precision (float64) golden LDOS maps -- the reference CLI itself stores
// float32 only (src/idl.cc:78-97).
//
// It drives the classes the way src/calcqpi.cc:335-395,483-518,655-760 does for
// output=wannier, green=normal, with orbitals given as a float64 cube (the
// idlorbitalfile route, wannierfunctions.cc:489-498) padded with zero orbitals.
//
// With a trailing "J deltat etat" it runs the josephson mode instead
// (src/calcqpi.cc:705-709: per-energy tip factor, tmatrix::calcwannierjosephson); with
// "T threshold" the proximity-list form of the wannier mode (mkthresholdlist with maxband
// and spin, src/calcqpi.cc:619-630,700-701), with "S threshold k s_0 .. s_k-1" the same
// with a spinarr (mkthresholdlist(..., spinarr)).
//
// With "X height k file_0 prefact_0 ..." the orbitals are the XSF files, loaded by the
// reference's wannierfunctions(file, height, window, oversamp, prefact) (the orbitalfiles
// keyword); wfbin is then ignored.  With "G surface|bulk epserr stbfile" the Green's function
// is tmatrix::calcsurfacegreensfunction (green=surface|bulk, "-" = no stbfile).  "P" writes
// the spectral function (tmatrix::calcspf, output=spf; pass os = 1 and kp = n), "U k x y pre
// ..." the unfolded one (tmatrix::calcuspf with k band positions and prefactors); no G0(R),
// dos written as 0.
//
// usage: refdump <hrfile> <wfbin> <out> n kp os w eta efermi spin maxband layers
//                lenergy henergy scmodel nscat [vre vim]... [J deltat etat | T thr | S thr k s...]
//                [X height k file prefact ...] [G surface|bulk epserr stbfile|-]
//                [P | U k x_0 y_0 pre_0 ...]
// wfbin: int32 norb, int32 side, float64 [norb][side][side]
// out:   per layer: float64 dos (tmatrix::calcdos), float64 ldos[y][x]
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <string>
#include <vector>
#include <complex>
#include <iostream>

#include "mpidefs.h"
#include "idl.h"
#include "tightbinding.h"
#include "qpi.h"

using namespace std;

int main(int argc, char **argv)
{
    if (argc < 18) {
        cerr << "usage: refdump hr wfbin out n kp os w eta efermi spin maxband layers lenergy henergy scmodel nscat [vre vim]..." << endl;
        return 2;
    }
    const char *hr = argv[1], *wfbin = argv[2], *outp = argv[3];
    size_t n = atoi(argv[4]), kp = atoi(argv[5]), os = atoi(argv[6]), w = atoi(argv[7]);
    double eta = atof(argv[8]), efermi = atof(argv[9]);
    bool spin = atoi(argv[10]) != 0;
    size_t maxband = atoi(argv[11]), layers = atoi(argv[12]);
    double le = atof(argv[13]), he = atof(argv[14]);
    bool scmodel = atoi(argv[15]) != 0;
    int nscat = atoi(argv[16]);
    vector<complex<double> > scat;
    for (int i = 0; i < nscat; i++) scat.push_back(complex<double>(atof(argv[17 + 2 * i]), atof(argv[18 + 2 * i])));
    // trailing options: J deltat etat | T thr | S thr k s_0 .. s_k-1 | X height k file_0 .. file_k-1
    bool josephson = false, listmode = false;
    double deltat = 0.0, etat = 0.0, threshold = 0.0, xsfheight = 0.0;
    vector<int> spinarr;
    vector<string> xsffiles;
    vector<double> xsfpre;
    int gmode = 0;              // 1 surface, 2 bulk Green's function (src/calcqpi.cc:683-688)
    int spfmode = 0;            // 1 output=spf, 2 output=uspf (src/calcqpi.cc:712-717)
    vector<vector<double> > uspos;
    vector<double> uspre;
    double epserr = 1e-5;
    string stbfile = "-";
    for (int a = 17 + 2 * nscat; a < argc;) {
        const string opt = argv[a];
        if (opt == "J" && a + 2 < argc) {
            josephson = true; deltat = atof(argv[a + 1]); etat = atof(argv[a + 2]); a += 3;
        } else if (opt == "T" && a + 1 < argc) {
            listmode = true; threshold = atof(argv[a + 1]); a += 2;
        } else if (opt == "S" && a + 2 < argc) {
            listmode = true; threshold = atof(argv[a + 1]);
            const int k = atoi(argv[a + 2]);
            for (int i = 0; i < k; i++) spinarr.push_back(atoi(argv[a + 3 + i]));
            a += 3 + k;
        } else if (opt == "P") {
            spfmode = 1;
            a += 1;
        } else if (opt == "U" && a + 1 < argc) {
            spfmode = 2;
            const int k = atoi(argv[a + 1]);
            for (int i = 0; i < k; i++) {
                uspos.push_back(vector<double>{atof(argv[a + 2 + 3 * i]), atof(argv[a + 3 + 3 * i]), 0.0});
                uspre.push_back(atof(argv[a + 4 + 3 * i]));
            }
            a += 2 + 3 * k;
        } else if (opt == "G" && a + 3 < argc) {
            gmode = string(argv[a + 1]) == "surface" ? 1 : 2;
            epserr = atof(argv[a + 2]);
            stbfile = argv[a + 3];
            a += 4;
        } else if (opt == "X" && a + 2 < argc) {
            xsfheight = atof(argv[a + 1]);
            const int k = atoi(argv[a + 2]);
            for (int i = 0; i < k; i++) {
                xsffiles.push_back(argv[a + 3 + 2 * i]);
                xsfpre.push_back(atof(argv[a + 4 + 2 * i]));
            }
            a += 3 + 2 * k;
        } else {
            cerr << "unknown option " << opt << endl;
            return 2;
        }
    }

    tightbind *model = new tightbind(string(hr), efermi, scmodel);
    if (!*model) { cerr << "model load failed" << endl; return 1; }
    tightbind *smodel = nullptr;
    if (gmode && stbfile != "-") {
        smodel = new tightbind(stbfile, efermi, scmodel);
        if (!*smodel) { cerr << "surface model load failed" << endl; return 1; }
    }
    vector<wannierfunctions> wfs;
    size_t norb = 0;
    if (!xsffiles.empty()) {
        // orbitalfiles: wannierfunctions(file, zheight, window, oversamp, prefact) as the driver
        // builds them (src/calcqpi.cc:577-590)
        for (size_t i = 0; i < xsffiles.size(); i++) {
            wfs.push_back(wannierfunctions(xsffiles[i], xsfheight, w, os, xsfpre[i]));
            if (!wfs.back()) { cerr << "XSF load failed: " << xsffiles[i] << endl; return 1; }
        }
        norb = xsffiles.size();
    } else {
        FILE *f = fopen(wfbin, "rb");
        if (!f) return 1;
        int nf = 0, side = 0;
        if (fread(&nf, 4, 1, f) != 1 || fread(&side, 4, 1, f) != 1) return 1;
        vector<vector<double> > arr(side, vector<double>(side, 0.0));
        for (int o = 0; o < nf; o++) {
            for (int i = 0; i < side; i++)
                for (int j = 0; j < side; j++)
                    if (fread(&arr[i][j], 8, 1, f) != 1) return 1;
            wfs.push_back(wannierfunctions(arr, 1.0));
        }
        fclose(f);
        norb = nf;
    }
    if (spin && (maxband >> 1) == norb) {
        for (size_t k = 0; k < norb; k++) wfs.push_back(wfs[k]);   // src/calcqpi.cc:592-595
        norb *= 2;
    }
    for (size_t i = norb; i < maxband; i++) wfs.push_back(wannierfunctions("z", 0.5, 5.0, 0.0, 0.0, 0.0, 0.0, 0.0));

    tmatrix *tm = new tmatrix(model, n, kp, eta, spin);
    if (scat.size() > 0) tm->setscatteringphase(scat);
    else tm->setscatteringphase(complex<double>(1.0, 0.0));
    flaglist fls;
    if (listmode) {
        size_t count = spinarr.empty() ? mkthresholdlist(fls, wfs, w, os, threshold, maxband, spin)
                                       : mkthresholdlist(fls, wfs, w, os, threshold, spinarr);
        cerr << "threshold list entries " << count << endl;
    }
    idl ldosmap(n * os, n * os, layers, 2.0, 2.0, le, he, 0.0, -1.0, -1.0);
    size_t wn = n * os;
    vector<double> buf(wn * wn);
    FILE *o = fopen(outp, "wb");
    for (size_t k = 0; k < layers; k++) {
        double energy = ldosmap.getbias(k);
        if (gmode) tm->calcsurfacegreensfunction(energy, epserr, gmode == 1, smodel);
        else tm->setgreensfunction(energy);
        double dos = 0.0;
        if (!spfmode) {
            tm->calcrealspacegreensfunction();
            dos = tm->calcdos(maxband);
        }
        if (spfmode == 1) {
            tm->calcspf(maxband);
        } else if (spfmode == 2) {
            tm->calcuspf(maxband, uspos, uspre);
        } else if (josephson) {
            gsl_complex ocomp = gsl_complex_rect(energy, etat);
            gsl_complex tip = gsl_complex_div(gsl_complex_rect(0.0, -copysign(1.0, energy) * M_PI * deltat),
                                              gsl_complex_sqrt(gsl_complex_sub_real(gsl_complex_mul(ocomp, ocomp),
                                                                                    deltat * deltat)));
            tm->calcwannierjosephson(os, w, wfs, tip);
        } else if (listmode) {
            tm->calcwannierldos(os, w, fls);
        } else {
            tm->calcwannierldos(os, w, wfs, maxband);
        }
        tm->ldos2array(buf.data());
        fwrite(&dos, 8, 1, o);
        fwrite(buf.data(), 8, wn * wn, o);
    }
    fclose(o);
    delete tm;
    delete model;
    return 0;
}
