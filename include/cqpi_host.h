/*
 * cqpi_host.h -- host-side (CPU-only) part of the libcqpi.so C ABI: the input and
 * output formats of the reference's continuum-LDOS path.  None of these calls
 * touches the GPU.
 */
#ifndef CQPI_HOST_H
#define CQPI_HOST_H

#include <stdint.h>

#include "cqpi.h"   /* cqpi_model */

#ifdef __cplusplus
extern "C" {
#endif

/* Parsed Wannier90 _hr.dat, owned by the library (free with cqpi_hr_free). */
typedef struct {
    char name[512];       /* first line of the file, up to the first CR/LF */
    int32_t bands;        /* num_wann */
    int32_t scmaxbands;   /* bands, or bands/2 when read with scmodel */
    int32_t nrpts;
    int64_t nhops;
    int32_t *R;           /* [nhops][3] */
    int32_t *orb;         /* [nhops][2], 0-based */
    double *t;            /* [nhops][2], divided by the degeneracy of its R */
    uint8_t *anti;        /* [nhops]: both orbitals in the hole half (scmodel) */
} cqpi_hr;

/* Replaces tightbind::tightbind(file, fermi, scmodel) -> readfile
 * (src/tightbinding.cc:70-149, 151-161): same line grammar, degeneracy list read
 * across lines, degeneracy index advancing when (Rx,Ry,Rz) changes, 1-based
 * orbital indices.  Errors (missing file, bad line, orbital index out of range)
 * return CQPI_ERR_ARG with a message in cqpi_host_last_error(). */
int cqpi_read_hr(const char *path, int32_t scmodel, cqpi_hr **out);
void cqpi_hr_free(cqpi_hr *hr);

/* 1 if 'name' is one of the reference's analytic orbital names
 * (s px py pz dx2 dxy dxz dyz dr2 fy3x2 fxyz fyz2 fz3 fxz2 fzx2 fxx2 n z). */
int cqpi_orbital_known(const char *name);
/* Replaces wannierfunctions(name, width, height, xpos, ypos, theta, phi, prefact)
 * followed by precalculate(window, oversamp) (src/wannierfunctions.cc:21-221,
 * 433-442): out[i][j] = getwave(i/os - w - 0.5, j/os - w - 0.5), side (2w+1)*os,
 * Slater radial part exp(-r/width), evaluated at z = -height. */
int cqpi_orbital_cache(const char *name, double width, double height, double xpos, double ypos, double theta,
                       double phi, double prefact, int32_t window, int32_t oversamp, double *out);

/* Replaces wannierfunctions(filename, height, window, oversamp, prefact) with its XSF
 * reader xcfloader (src/wannierfunctions.cc:444-463, src/loadxcf.cc:37-345), the
 * orbitalfiles keyword: out[i][j] = prefact * value of the XSF 3D data grid at the lattice
 * point (i/os - w, j/os - w) (CONVVEC to Cartesian, nearest grid point, zero outside) and at
 * z = height above the highest atom of PRIMCOORD (below the lowest for height < 0; height 0
 * gives zeros), side (2w+1)*os.  A file that cannot be read (missing, no data grid, no
 * CONVVEC, malformed block) returns CQPI_ERR_ARG with the reason in cqpi_host_last_error(). */
int cqpi_xsf_orbital_cache(const char *path, double height, int32_t window, int32_t oversamp, double prefact,
                           double *out);

/* The orbital sources of the orbital-file tool mkwavefunctions (src/mkwavefunctions.cc):
 *
 * cqpi_orbital_cache_basis: wannierfunctions(basisvectors, name, ...) + precalculate, its
 * 'orbitals' keyword (:241-300, src/wannierfunctions.cc:126-221): as cqpi_orbital_cache with
 * the shifted in-plane point taken to x b0 + y b1 before the rotation (basis = {b0x, b0y, b1x,
 * b1y}, the basisvector[0] and [1] keywords); basis NULL is the unit basis.
 *
 * cqpi_xsf_orbital_cache_shifted: wannierfunctions(filename, shift, height, window,
 * oversamp, prefact, centre) (src/wannierfunctions.cc:465-487), its 'orbitalfiles' keyword
 * (:301-324): as cqpi_xsf_orbital_cache with the XSF grid origin moved by shift[3]
 * (Cartesian) and, for centre != 0, the lattice points at (i/os - w - 0.5, j/os - w - 0.5).
 *
 * cqpi_xsf_orbital_cache_mod: wannierfunctions(basisvectors, xcfloader, window, oversamp,
 * height, xpos, ypos, theta) with xcfloader::getcartmodvalue (src/wannierfunctions.cc:
 * 500-520, src/loadxcf.cc:268-290), its 'modorbitalfiles' keyword (:184-226):
 * out[i][j] = prefact * grid value at the Cartesian point R(theta) B (i/os - w - xpos,
 * j/os - w - ypos) (B the basis, or the unit matrix when NULL; R the rotation about z), with
 * the grid origin moved by modshift[3] (the tool passes -modpos[k]), at z = height above the
 * highest atom (below the lowest for height < 0).
 *
 * Unreadable files return CQPI_ERR_ARG with the reason in cqpi_host_last_error(). */
int cqpi_orbital_cache_basis(const char *name, double width, double height, double xpos, double ypos, double theta,
                             double phi, double prefact, const double *basis, int32_t window, int32_t oversamp,
                             double *out);
int cqpi_xsf_orbital_cache_shifted(const char *path, const double *shift, int32_t centre, double height,
                                   int32_t window, int32_t oversamp, double prefact, double *out);
int cqpi_xsf_orbital_cache_mod(const char *path, const double *modshift, const double *basis, double height,
                               double xpos, double ypos, double theta, double prefact, int32_t window,
                               int32_t oversamp, double *out);

/* One-dimensional interpolation of mkwavefunctions' interpolate() (src/mkwavefunctions.cc:
 * 39-70, GSL gsl_interp_init / gsl_interp_eval): y[q] = f(x[q]) for the curve f of 'method'
 * ("linear", "polynomial", "cspline", "cspline_periodic", "akima", "akima_periodic",
 * "steffen") through (xa[i], ya[i]), i < n.  CQPI_ERR_ARG for an unknown method, fewer points
 * than the method needs, x values that do not strictly increase, or a point outside
 * [xa[0], xa[n-1]] (where GSL's default error handler aborts the reference). */
int cqpi_interp_known(const char *method);
int cqpi_interp_eval(const char *method, int32_t n, const double *xa, const double *ya, int32_t count,
                     const double *x, double *y);

/* Band-structure histogram of the bsfile keyword: replaces tightbind::calcbst3dhisthr(fname,
 * pix, le, ue, layers, oversamp) (src/tightbinding.cc:1158-1193; driver src/calcqpi.cc:308-326).
 * Eigenvalues of H(k) (the model's terms with the Fermi-energy diagonal, all R_z at k_z = 0)
 * on the (pix*oversamp)^2 grid k = (io, jo) / (pix*oversamp - 1) - 1/2, each adding a
 * Lorentzian of width 2 (ue - le) / layers to the three nearest of the layers energies
 * le .. ue in pixel (io / oversamp, jo / oversamp).  out[layers][pix][pix] (x fastest, the
 * IDL order of idl(pix, pix, layers, 1, 1, le, ue, 0, -0.5, -0.5)).  CPU only, on all host
 * cores, as the reference computes it.  CQPI_ERR_ARG unless ue > le, pix, oversamp and layers
 * are positive and the model's orbital indices lie inside its bands. */
int cqpi_band_histogram(const cqpi_model *m, int32_t pix, int32_t oversamp, double le, double ue, int32_t layers,
                        double *out);

/* IDL map header (src/idl.h:41-60). */
typedef struct {
    char name[1024];
    char date[256];
    int32_t size[3];
    double scan_range[2], offset[2], bias[2], setpoint;
    int64_t data_offset;  /* byte offset of the float32 data */
} cqpi_idl_header;

/* Replaces idl::write (src/idl.cc:78-97): 12 header lines formatted like
 * std::ostream defaults, then float32 data with x fastest, then y, then layer.
 * date == NULL writes ctime() of now, as the idl constructor does (src/idl.cc:670-672). */
int cqpi_idl_write(const char *path, const char *name, const char *date, int32_t sx, int32_t sy, int32_t sz,
                   const double *scan_range, const double *offset, const double *bias, double setpoint,
                   const float *data);
/* The same file written layer by layer (the calcqpi CLI's flush / resume keywords, an
 * extension: the reference writes the map once at the end, src/calcqpi.cc:779-783).
 * cqpi_idl_create writes the header of cqpi_idl_write and zero data for sz layers;
 * cqpi_idl_write_layers overwrites layers k0 .. k0+nk-1 (sx*sy floats each, x fastest) of an
 * existing file in place.  Layers outside the file return CQPI_ERR_ARG. */
int cqpi_idl_create(const char *path, const char *name, const char *date, int32_t sx, int32_t sy, int32_t sz,
                    const double *scan_range, const double *offset, const double *bias, double setpoint);
int cqpi_idl_write_layers(const char *path, int32_t k0, int32_t nk, const float *data);
/* Replaces idl::read (src/idl.cc:50-76). */
int cqpi_idl_read_header(const char *path, cqpi_idl_header *hdr);
int cqpi_idl_read(const char *path, float *data, int64_t count);

/* The message of the last failing host call made by the calling thread (valid until that
 * thread's next failing host call). */
const char *cqpi_host_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
