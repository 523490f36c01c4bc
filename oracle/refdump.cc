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
// usage: refdump <hrfile> <wfbin> <out> n kp os w eta efermi spin maxband layers
//                lenergy henergy scmodel nscat [vre vim]... [J deltat etat | T thr | S thr k s...]
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
    const int ja = 17 + 2 * nscat;
    const bool josephson = argc >= ja + 3 && string(argv[ja]) == "J";
    const double deltat = josephson ? atof(argv[ja + 1]) : 0.0, etat = josephson ? atof(argv[ja + 2]) : 0.0;
    const bool listmode = argc >= ja + 2 && (string(argv[ja]) == "T" || string(argv[ja]) == "S");
    const double threshold = listmode ? atof(argv[ja + 1]) : 0.0;
    vector<int> spinarr;
    if (listmode && string(argv[ja]) == "S") {
        int k = atoi(argv[ja + 2]);
        for (int i = 0; i < k; i++) spinarr.push_back(atoi(argv[ja + 3 + i]));
    }

    tightbind *model = new tightbind(string(hr), efermi, scmodel);
    if (!*model) { cerr << "model load failed" << endl; return 1; }
    FILE *f = fopen(wfbin, "rb");
    if (!f) return 1;
    int norb = 0, side = 0;
    if (fread(&norb, 4, 1, f) != 1 || fread(&side, 4, 1, f) != 1) return 1;
    vector<wannierfunctions> wfs;
    vector<vector<double> > arr(side, vector<double>(side, 0.0));
    for (int o = 0; o < norb; o++) {
        for (int i = 0; i < side; i++)
            for (int j = 0; j < side; j++)
                if (fread(&arr[i][j], 8, 1, f) != 1) return 1;
        wfs.push_back(wannierfunctions(arr, 1.0));
    }
    fclose(f);
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
        tm->setgreensfunction(energy);
        tm->calcrealspacegreensfunction();
        double dos = tm->calcdos(maxband);
        if (josephson) {
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
