// seam_check.cc -- builds the GB300QPI backend (calcqpi-release_gb300/seam/gb300qpi.h) against
// the reference's own GPUQPI interface (include/gpuqpi.h) and links it with the reference's
// objects and libcqpi.so.  Test infrastructure: oracle/build_ref.sh compiles it into
// oracle/_ref/ from the reference's headers.
//
//   seam_check          prints "linked": every virtual member of the backend was compiled and
//                       resolved (the three factories below instantiate its vtable)
//   seam_check create   constructs the LDOS-mode backend; where no GPU is usable the engine's
//                       error must arrive as a std::runtime_error, not as an exit
#define _GPU
#include <cstdio>
#include <exception>

#include "qpi.h"
#include "gb300qpi.h"

static GPUQPI *make_ldos(size_t wn, size_t kp, size_t n, size_t w, size_t os, size_t b, size_t m, bool spin,
                         vector<wannierfunctions> &wf)
{
    return new GB300QPI(wn, kp, n, w, os, b, m, spin, wf);
}

static GPUQPI *make_list(size_t wn, size_t kp, size_t n, size_t w, size_t os, size_t b, flaglist &fl)
{
    return new GB300QPI(wn, kp, n, w, os, b, fl);
}

static GPUQPI *make_kspace(size_t kp, size_t n, size_t b, size_t m, bool spin, vector<vector<double> > &pos,
                           vector<double> &pre)
{
    return new GB300QPI(kp, n, b, m, spin, pos, pre);
}

int main(int argc, char **argv)
{
    GPUQPI *(*volatile f1)(size_t, size_t, size_t, size_t, size_t, size_t, size_t, bool,
                           vector<wannierfunctions> &) = make_ldos;
    GPUQPI *(*volatile f2)(size_t, size_t, size_t, size_t, size_t, size_t, flaglist &) = make_list;
    GPUQPI *(*volatile f3)(size_t, size_t, size_t, size_t, bool, vector<vector<double> > &, vector<double> &) =
        make_kspace;
    if (argc > 1 && std::string(argv[1]) == "create") {
        vector<vector<double> > cube(12, vector<double>(12, 0.0));
        cube[6][6] = 1.0;
        vector<wannierfunctions> wf(1, wannierfunctions(cube));
        try {
            GPUQPI *g = f1(24, 8, 8, 1, 4, 1, 1, false, wf);
            g->printinfo(cout);
            delete g;
            printf("created\n");
        } catch (const std::exception &e) {
            printf("threw: %s\n", e.what());
        }
    }
    (void)f2;
    (void)f3;
    printf("linked\n");
    return 0;
}
