/*
 * cqpi_host.h -- host-side (CPU-only) part of the libcqpi.so C ABI: the input and
 * output formats of the reference's continuum-LDOS path.  None of these calls
 * touches the GPU.
 */
#ifndef CQPI_HOST_H
#define CQPI_HOST_H

#include <stdint.h>

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
/* Replaces idl::read (src/idl.cc:50-76). */
int cqpi_idl_read_header(const char *path, cqpi_idl_header *hdr);
int cqpi_idl_read(const char *path, float *data, int64_t count);

const char *cqpi_host_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
