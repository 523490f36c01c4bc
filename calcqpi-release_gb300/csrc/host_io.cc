// host_io.cc -- host-side input/output of the drop-in, exported through the C ABI:
//   cqpi_read_hr        Wannier90 _hr.dat reader   (tightbind::readfile, src/tightbinding.cc:70-149)
//   cqpi_orbital_cache  analytic orbital cache    (wannierfunctions::precalculate + getwave,
//                                                  src/wannierfunctions.cc:21-221,433-442)
//   cqpi_orbital_cache_basis  the same with lattice basis vectors (mkwavefunctions)
//   cqpi_xsf_orbital_cache  XSF orbital cache   (xcfloader + wannierfunctions(file, ...),
//                                                  src/loadxcf.cc:37-345, src/wannierfunctions.cc:444-463)
//   cqpi_xsf_orbital_cache_shifted / _mod  the XSF forms of mkwavefunctions (orbitalfiles with
//                       shift, modorbitalfiles; src/wannierfunctions.cc:465-520)
//   cqpi_idl_write / cqpi_idl_read_header / cqpi_idl_read
//                       IDL map container          (idl::write / idl::read, src/idl.cc:50-97)
//   cqpi_idl_create / cqpi_idl_write_layers  the same file written layer by layer (the
//                       CLI's flush / resume keywords)
// These run on the CPU only; none of them touches the GPU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "cqpi.h"
#include "cqpi_host.h"

namespace {

// per calling thread, so that host calls from several threads each read their own message
thread_local std::string g_host_err;

int host_fail(int code, const std::string &m)
{
    g_host_err = m;
    return code;
}

}  // namespace

extern "C" {

const char *cqpi_host_last_error(void) { return g_host_err.c_str(); }

int cqpi_read_hr(const char *path, int32_t scmodel, cqpi_hr **out)
{
    if (!path || !out) return host_fail(CQPI_ERR_ARG, "null argument");
    *out = nullptr;
    std::ifstream is(path);
    if (!is) return host_fail(CQPI_ERR_ARG, std::string("cannot read or open input file ") + path);
    std::string buf;
    size_t lineno = 0;
    std::string name;
    int bands = 0, nrpts = 0;
    if (!std::getline(is, buf)) return host_fail(CQPI_ERR_ARG, "empty _hr.dat");
    lineno++;
    name = buf.substr(0, buf.find_first_of("\n\r"));
    if (!std::getline(is, buf)) return host_fail(CQPI_ERR_ARG, "missing num_wann line");
    lineno++;
    std::istringstream(buf) >> bands;
    if (!std::getline(is, buf)) return host_fail(CQPI_ERR_ARG, "missing nrpts line");
    lineno++;
    std::istringstream(buf) >> nrpts;
    if (bands < 1 || nrpts < 0) return host_fail(CQPI_ERR_ARG, "invalid num_wann / nrpts");
    const int scmax = scmodel ? (bands >> 1) : bands;
    // degeneracies: integer tokens read across lines until nrpts are found
    std::vector<long> degs;
    degs.reserve(nrpts);
    size_t pos = 0;
    while ((int)degs.size() < nrpts) {
        if (!pos) {
            if (!std::getline(is, buf)) return host_fail(CQPI_ERR_ARG, "unexpected end of file in degeneracies");
            lineno++;
            pos = buf.find_first_of("0123456789", 0);
            if (pos == std::string::npos) return host_fail(CQPI_ERR_ARG, "error in input file in line " + std::to_string(lineno));
        }
        size_t npos = buf.find_first_of(" \t", pos);
        size_t len = (npos != std::string::npos) ? npos - pos : buf.length() - pos;
        npos = buf.find_first_of("0123456789", npos);
        std::istringstream iss(buf.substr(pos, len));
        long d;
        iss >> d;
        if (iss.fail()) return host_fail(CQPI_ERR_ARG, "error in input file in line " + std::to_string(lineno) + ": " + buf);
        degs.push_back(d);
        pos = (npos != std::string::npos) ? npos : 0;
    }
    // hopping lines: x y z u v re im; the degeneracy index advances whenever (x,y,z) changes
    std::vector<int32_t> R, orb;
    std::vector<double> t;
    std::vector<uint8_t> anti;
    size_t k = 0;
    int ox = 0, oy = 0, oz = 0;
    while (std::getline(is, buf)) {
        lineno++;
        if (buf.empty()) continue;
        std::istringstream iss(buf);
        int x, y, z;
        long u, v;
        double hr, hc;
        iss >> x >> y >> z >> u >> v >> hr >> hc;
        if (iss.fail()) return host_fail(CQPI_ERR_ARG, "error in input file in line " + std::to_string(lineno) + ": " + buf);
        if (k == 0 || x != ox || y != oy || z != oz) {
            k++;
            ox = x; oy = y; oz = z;
        }
        if (k > degs.size()) return host_fail(CQPI_ERR_ARG, "more R vectors than degeneracies (line " + std::to_string(lineno) + ")");
        if (u <= 0 || v <= 0 || u > bands || v > bands)
            return host_fail(CQPI_ERR_ARG, "invalid orbital index in line " + std::to_string(lineno));
        const double dg = (double)degs[k - 1];
        R.push_back(x); R.push_back(y); R.push_back(z);
        orb.push_back((int32_t)(u - 1)); orb.push_back((int32_t)(v - 1));
        t.push_back(hr / dg); t.push_back(hc / dg);
        anti.push_back(((u - 1) >= scmax) && ((v - 1) >= scmax));
    }
    cqpi_hr *hr = (cqpi_hr *)calloc(1, sizeof(cqpi_hr));
    if (!hr) return host_fail(CQPI_ERR_ALLOC, "out of memory");
    snprintf(hr->name, sizeof hr->name, "%s", name.c_str());
    hr->bands = bands;
    hr->scmaxbands = scmax;
    hr->nrpts = nrpts;
    hr->nhops = (int64_t)anti.size();
    size_t nh = anti.size() ? anti.size() : 1;
    hr->R = (int32_t *)malloc(sizeof(int32_t) * 3 * nh);
    hr->orb = (int32_t *)malloc(sizeof(int32_t) * 2 * nh);
    hr->t = (double *)malloc(sizeof(double) * 2 * nh);
    hr->anti = (uint8_t *)malloc(nh);
    if (!hr->R || !hr->orb || !hr->t || !hr->anti) {
        cqpi_hr_free(hr);
        return host_fail(CQPI_ERR_ALLOC, "out of memory");
    }
    if (!anti.empty()) {
        memcpy(hr->R, R.data(), sizeof(int32_t) * R.size());
        memcpy(hr->orb, orb.data(), sizeof(int32_t) * orb.size());
        memcpy(hr->t, t.data(), sizeof(double) * t.size());
        memcpy(hr->anti, anti.data(), anti.size());
    }
    *out = hr;
    return CQPI_OK;
}

void cqpi_hr_free(cqpi_hr *hr)
{
    if (!hr) return;
    free(hr->R);
    free(hr->orb);
    free(hr->t);
    free(hr->anti);
    free(hr);
}

// ------------------------------------------------------------------ orbitals
static int orbital_type(const char *name)
{
    static const char *names[] = {"s", "px", "py", "pz", "dx2", "dxy", "dxz", "dyz", "dr2", "fy3x2", "fxyz",
                                  "fyz2", "fz3", "fxz2", "fzx2", "fxx2", "n", "z"};
    for (int i = 0; i < 18; i++)
        if (!strcmp(name, names[i])) return i;
    return -1;
}

int cqpi_orbital_known(const char *name) { return name && orbital_type(name) >= 0; }

// Value of orbital 'type' at (x, y): z = 0 shifted by -height (tip plane below the
// orbital centre, src/wannierfunctions.cc:127-130), the in-plane point taken through the
// basis vectors when given (wannierfunctions::transform, src/wannierfunctions.h:41-45:
// (x, y) -> x b0 + y b1, basis = {b0x, b0y, b1x, b1y}), optional rotation for non-s types.
static double orbital_value(int type, double x, double y, double width, double height, double xpos, double ypos,
                            double theta, double phi, double prefact, double symmetry, const double *basis)
{
    double z = 0.0;
    x -= xpos; y -= ypos; z -= height;
    if (type == 17) return 0.0;
    if (basis) {
        const double a = x, b = y;
        x = basis[0] * a + basis[2] * b;
        y = basis[1] * a + basis[3] * b;
    }
    if (type != 0 && (theta != 0.0 || phi != 0.0)) {
        const double xc = x, yc = y, zc = z;
        x = xc * cos(theta) + yc * sin(theta) * cos(phi) + zc * sin(theta) * sin(phi);
        y = -xc * sin(theta) + yc * cos(theta) * cos(phi) + zc * cos(theta) * sin(phi);
        z = -sin(phi) * yc + cos(phi) * zc;
    }
    const double r = sqrt(x * x + y * y + z * z);
    const double ex = prefact * exp(-r / width);
    if (type == 0) return ex / sqrt(4.0 * M_PI);
    if (type == 16) {
        const double sc = cos(symmetry * atan2(x, y) / 2.0);
        return ex * sc * sc * r / width;
    }
    if (r == 0.0) return 0.0;
    switch (type) {
    case 1: return ex * x / r * sqrt(3.0 / 4.0 / M_PI);
    case 2: return ex * y / r * sqrt(3.0 / 4.0 / M_PI);
    case 3: return ex * z / r * sqrt(3.0 / 4.0 / M_PI);
    case 4: return ex * (x * x - y * y) / 2.0 / r / r * sqrt(15.0 / 4.0 / M_PI);
    case 5: return ex * x * y / r / r * sqrt(15.0 / 4.0 / M_PI);
    case 6: return ex * x * z / r / r * sqrt(15.0 / 4.0 / M_PI);
    case 7: return ex * y * z / r / r * sqrt(15.0 / 4.0 / M_PI);
    case 8: return ex * (3.0 * z * z - r * r) / 4.0 / r / r * sqrt(5.0 / M_PI);
    case 9: return ex * y * (3.0 * x * x - y * y) / 4.0 / r / r / r * sqrt(35.0 / 2.0 / M_PI);
    case 10: return ex * x * y * z / r / r / r * sqrt(105.0 / 4.0 / M_PI);
    case 11: return ex * y * (5.0 * z * z - r * r) / r / r / r / 4.0 * sqrt(21.0 / 2.0 / M_PI);
    case 12: return ex * (5.0 * z * z * z - 3.0 * z * r * r) / r / r / r / 4.0 * sqrt(7.0 / M_PI);
    case 13: return ex * x * (5.0 * z * z - r * r) / 4.0 / r / r / r * sqrt(21.0 / 2.0 / M_PI);
    case 14: return ex * z * (x * x - y * y) / r / r / r / 4.0 * sqrt(105.0 / M_PI);
    case 15: return ex * x * (x * x - 3.0 * y * y) / 4.0 / r / r / r * sqrt(35.0 / 2.0 / M_PI);
    }
    return NAN;
}

int cqpi_orbital_cache(const char *name, double width, double height, double xpos, double ypos, double theta,
                       double phi, double prefact, int32_t window, int32_t oversamp, double *out)
{
    return cqpi_orbital_cache_basis(name, width, height, xpos, ypos, theta, phi, prefact, nullptr, window, oversamp,
                                    out);
}

int cqpi_orbital_cache_basis(const char *name, double width, double height, double xpos, double ypos, double theta,
                             double phi, double prefact, const double *basis, int32_t window, int32_t oversamp,
                             double *out)
{
    const int type = name ? orbital_type(name) : -1;
    if (type < 0) return host_fail(CQPI_ERR_ARG, std::string("unknown orbital type ") + (name ? name : "(null)"));
    if (!out || window < 0 || oversamp < 1) return host_fail(CQPI_ERR_ARG, "invalid orbital cache arguments");
    const int n = (2 * window + 1) * oversamp;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            out[(size_t)i * n + j] = orbital_value(type, (double)i / oversamp - (double)window - 0.5,
                                                   (double)j / oversamp - (double)window - 0.5, width, height, xpos,
                                                   ypos, theta, phi, prefact, 4.0, basis);
    return CQPI_OK;
}

// ------------------------------------------------------------------ IDL files
// idl::write's header (src/idl.cc:78-97): 12 lines formatted like std::ostream defaults
static void idl_header(std::ostream &os, const char *name, const char *date, int32_t sx, int32_t sy, int32_t sz,
                       const double *scan_range, const double *offset, const double *bias, double setpoint)
{
    std::string d;
    if (date) d = date;
    else {
        time_t tt = time(nullptr);
        d = ctime(&tt);
        d.resize(d.length() - 1);
    }
    os << (name ? name : "") << std::endl << d << std::endl << (size_t)sx << std::endl << (size_t)sy << std::endl
       << (size_t)sz << std::endl << scan_range[0] << std::endl << scan_range[1] << std::endl << offset[0] << std::endl
       << offset[1] << std::endl << bias[0] << std::endl << bias[1] << std::endl << setpoint << std::endl;
}

int cqpi_idl_write(const char *path, const char *name, const char *date, int32_t sx, int32_t sy, int32_t sz,
                   const double *scan_range, const double *offset, const double *bias, double setpoint,
                   const float *data)
{
    if (!path || sx < 0 || sy < 0 || sz < 0 || (!data && (size_t)sx * sy * sz != 0))
        return host_fail(CQPI_ERR_ARG, "invalid IDL arguments");
    std::ofstream os(path, std::ios::binary);
    if (!os) return host_fail(CQPI_ERR_ARG, std::string("error while opening file ") + path + " for writing");
    idl_header(os, name, date, sx, sy, sz, scan_range, offset, bias, setpoint);
    os.write((const char *)data, (std::streamsize)(sizeof(float) * (size_t)sx * sy * sz));
    if (!os) return host_fail(CQPI_ERR_ARG, std::string("error writing to ") + path);
    return CQPI_OK;
}

int cqpi_idl_create(const char *path, const char *name, const char *date, int32_t sx, int32_t sy, int32_t sz,
                    const double *scan_range, const double *offset, const double *bias, double setpoint)
{
    if (!path || sx < 0 || sy < 0 || sz < 0) return host_fail(CQPI_ERR_ARG, "invalid IDL arguments");
    std::ofstream os(path, std::ios::binary | std::ios::trunc);
    if (!os) return host_fail(CQPI_ERR_ARG, std::string("error while opening file ") + path + " for writing");
    idl_header(os, name, date, sx, sy, sz, scan_range, offset, bias, setpoint);
    // the data region reads as zeros: extend the file to its full length by writing its last
    // byte (the file system leaves the rest as a hole instead of writing gigabytes of zeros)
    const size_t bytes = sizeof(float) * (size_t)sx * sy * sz;
    if (bytes) {
        os.seekp((std::streamoff)(bytes - 1), std::ios::cur);
        os.put('\0');
    }
    if (!os) return host_fail(CQPI_ERR_ARG, std::string("error writing to ") + path);
    return CQPI_OK;
}

int cqpi_idl_write_layers(const char *path, int32_t k0, int32_t nk, const float *data)
{
    cqpi_idl_header h;
    int rc = cqpi_idl_read_header(path, &h);
    if (rc) return rc;
    if (!data || k0 < 0 || nk < 0 || (int64_t)k0 + nk > h.size[2])
        return host_fail(CQPI_ERR_ARG, "layers outside the IDL file");
    const size_t plane = (size_t)h.size[0] * h.size[1];
    std::fstream fs(path, std::ios::binary | std::ios::in | std::ios::out);
    if (!fs) return host_fail(CQPI_ERR_ARG, std::string("error while opening file ") + path + " for writing");
    fs.seekp(h.data_offset + (std::streamoff)(sizeof(float) * plane * (size_t)k0));
    fs.write((const char *)data, (std::streamsize)(sizeof(float) * plane * (size_t)nk));
    fs.flush();
    if (!fs) return host_fail(CQPI_ERR_ARG, std::string("error writing to ") + path);
    return CQPI_OK;
}

int cqpi_idl_read_header(const char *path, cqpi_idl_header *hdr)
{
    if (!path || !hdr) return host_fail(CQPI_ERR_ARG, "null argument");
    std::ifstream is(path, std::ios::binary);
    if (!is) return host_fail(CQPI_ERR_ARG, std::string("cannot open ") + path);
    std::string name, date;
    std::getline(is, name);
    std::getline(is, date);
    size_t s0, s1, s2;
    is >> s0 >> s1 >> s2 >> hdr->scan_range[0] >> hdr->scan_range[1] >> hdr->offset[0] >> hdr->offset[1] >>
        hdr->bias[0] >> hdr->bias[1] >> hdr->setpoint;
    if (!is) return host_fail(CQPI_ERR_ARG, std::string("error reading header of ") + path);
    is.ignore(1, '\n');
    // a corrupt header must not produce wrapped sizes: each dimension fits int32, the data
    // size in bytes fits int64, and the data lies inside the file
    const uint64_t lim = (uint64_t)INT32_MAX;
    if ((uint64_t)s0 > lim || (uint64_t)s1 > lim || (uint64_t)s2 > lim)
        return host_fail(CQPI_ERR_ARG, std::string("IDL dimensions out of range in ") + path);
    const uint64_t plane = (uint64_t)s0 * (uint64_t)s1;   // < 2^62
    const uint64_t maxel = (uint64_t)INT64_MAX / sizeof(float);
    if (s2 != 0 && plane > maxel / (uint64_t)s2)
        return host_fail(CQPI_ERR_ARG, std::string("IDL data size overflows in ") + path);
    const uint64_t bytes = plane * (uint64_t)s2 * sizeof(float);
    const std::streamoff off = is.tellg();
    if (off < 0) return host_fail(CQPI_ERR_ARG, std::string("error reading header of ") + path);
    is.seekg(0, std::ios::end);
    const std::streamoff end = is.tellg();
    if (end < off || (uint64_t)(end - off) < bytes)
        return host_fail(CQPI_ERR_ARG, std::string("IDL data region shorter than the header's dimensions in ") + path);
    snprintf(hdr->name, sizeof hdr->name, "%s", name.c_str());
    snprintf(hdr->date, sizeof hdr->date, "%s", date.c_str());
    hdr->size[0] = (int32_t)s0;
    hdr->size[1] = (int32_t)s1;
    hdr->size[2] = (int32_t)s2;
    hdr->data_offset = (int64_t)off;
    return CQPI_OK;
}

int cqpi_idl_read(const char *path, float *data, int64_t count)
{
    cqpi_idl_header h;
    int rc = cqpi_idl_read_header(path, &h);
    if (rc) return rc;
    const int64_t n = (int64_t)h.size[0] * h.size[1] * h.size[2];
    if (!data || count < n) return host_fail(CQPI_ERR_ARG, "IDL data buffer too small");
    std::ifstream is(path, std::ios::binary);
    is.seekg(h.data_offset);
    is.read((char *)data, (std::streamsize)(sizeof(float) * n));
    if (!is) return host_fail(CQPI_ERR_ARG, std::string("error reading data of ") + path);
    return CQPI_OK;
}

// ------------------------------------------------------------------ XSF orbitals
// The XSF reader of the orbitalfiles keyword, as xcfloader reads a file (src/loadxcf.cc:
// 37-185): a line counts only when a newline ends it; '#' anywhere makes the rest of the
// line a comment; CRYSTAL enables PRIMVEC / CONVVEC / PRIMCOORD; in the data grid a value
// starts at one of "+-0123456789" and ends at a blank, and a value that runs to the end of
// its line makes the reader take the next line.  Values are stored cube[i][j][k], x fastest
// in the file.
struct XsfGrid {
    size_t xs = 0, ys = 0, zs = 0;
    std::vector<double> cube;                  // [i][j][k]
    double origin[3] = {0, 0, 0};
    double axis[3][3] = {};                    // spanning vectors
    double convvec[3][3] = {};
    bool has_convvec = false, has_grid = false, error = false;
    std::vector<double> atom_z;
};

static bool xsf_next(std::istream &is, std::string &line)
{
    std::getline(is, line);
    return !is.eof();
}

static bool xsf_read(const char *path, XsfGrid &g, std::string &err)
{
    std::ifstream is(path);
    if (!is) {
        err = std::string("Could not open file ") + path;
        return false;
    }
    std::string line;
    bool crystal = false;
    while (xsf_next(is, line)) {
        if (line.find('#') != std::string::npos) continue;
        if (line.find("CRYSTAL") != std::string::npos) {
            crystal = true;
        } else if (crystal && (line.find("PRIMVEC") != std::string::npos ||
                               line.find("CONVVEC") != std::string::npos)) {
            const bool conv = line.find("CONVVEC") != std::string::npos;
            for (int r = 0; r < 3; r++) {
                std::string pl;
                std::getline(is, pl);
                std::istringstream iss(pl);
                double v[3] = {0, 0, 0};
                iss >> v[0] >> v[1] >> v[2];
                if (conv)
                    for (int c = 0; c < 3; c++) g.convvec[r][c] = v[c];
            }
            if (conv) g.has_convvec = true;
        } else if (crystal && line.find("PRIMCOORD") != std::string::npos) {
            std::string pl;
            std::getline(is, pl);
            std::istringstream iss(pl);
            size_t natoms = 0, type = 0;
            iss >> natoms >> type;
            for (size_t a = 0; a < natoms; a++) {
                std::getline(is, pl);
                std::istringstream ia(pl);
                std::string name;
                double x = 0, y = 0, z = 0;
                ia >> name >> x >> y >> z;
                g.atom_z.push_back(z);
            }
        } else if (line.find("BEGIN_BLOCK_DATAGRID_3D") != std::string::npos) {
            std::string pl, kw;
            std::getline(is, pl);
            { std::istringstream iss(pl); kw.clear(); iss >> kw; }
            if (kw != "3D_field") g.error = true;
            std::getline(is, pl);
            { std::istringstream iss(pl); kw.clear(); iss >> kw; }
            if (kw != "BEGIN_DATAGRID_3D_UNKNOWN") g.error = true;
            std::getline(is, pl);
            { std::istringstream iss(pl); iss >> g.xs >> g.ys >> g.zs; }
            if (g.xs == 0 || g.ys == 0 || g.zs == 0 || g.xs * g.ys * g.zs > ((size_t)1 << 31)) {
                err = std::string("invalid data grid size in ") + path;
                return false;
            }
            std::getline(is, pl);
            { std::istringstream iss(pl); iss >> g.origin[0] >> g.origin[1] >> g.origin[2]; }
            for (int r = 0; r < 3; r++) {
                std::getline(is, pl);
                std::istringstream iss(pl);
                iss >> g.axis[r][0] >> g.axis[r][1] >> g.axis[r][2];
            }
            g.cube.assign(g.xs * g.ys * g.zs, 0.0);
            std::getline(is, line);
            size_t npos = 0;
            for (size_t k = 0; k < g.zs; k++)
                for (size_t j = 0; j < g.ys; j++)
                    for (size_t i = 0; i < g.xs; i++) {
                        const size_t pos = line.find_first_of("+-0123456789", npos);
                        if (pos == std::string::npos) {
                            err = std::string("cannot parse data line of ") + path;
                            return false;
                        }
                        npos = line.find_first_of(" \t", pos);
                        const bool reload = npos == std::string::npos;
                        std::istringstream niss(line.substr(pos, reload ? std::string::npos : npos - pos));
                        double v = 0.0;
                        niss >> v;
                        g.cube[(i * g.ys + j) * g.zs + k] = v;
                        if (reload) {
                            std::getline(is, line);
                            npos = 0;
                        }
                    }
            if (line.find("END_DATAGRID_3D") == std::string::npos) g.error = true;
            std::getline(is, line);
            if (line.find("END_BLOCK_DATAGRID_3D") == std::string::npos) g.error = true;
            g.has_grid = true;
        }
    }
    if (g.error) err = std::string("malformed data grid block in ") + path;
    else if (!g.has_grid) err = std::string("no 3D data grid in ") + path;
    else if (!g.has_convvec) err = std::string("no CONVVEC in ") + path;
    return !g.error && g.has_grid && g.has_convvec;
}

// xcfloader::operator() (src/loadxcf.cc:221-238) at the Cartesian point (x, y, z): fractional
// grid coordinates by solving [a0 a1 a2] f = r - origin - shift (Gaussian elimination with
// partial pivoting), nearest grid point round(f * n), zero outside the grid.  A NaN height
// (getzheight(0)) gives zero.
static double xsf_cart_value(const XsfGrid &g, double x, double y, double z, const double *shift)
{
    const double r[3] = {x - g.origin[0] - shift[0], y - g.origin[1] - shift[1], z - g.origin[2] - shift[2]};
    double A[3][4];
    for (int row = 0; row < 3; row++) {
        for (int c = 0; c < 3; c++) A[row][c] = g.axis[c][row];
        A[row][3] = r[row];
    }
    for (int c = 0; c < 3; c++) {
        int piv = c;
        for (int row = c + 1; row < 3; row++)
            if (std::fabs(A[row][c]) > std::fabs(A[piv][c])) piv = row;
        if (piv != c)
            for (int k = 0; k < 4; k++) std::swap(A[c][k], A[piv][k]);
        if (A[c][c] == 0.0) return 0.0;
        for (int row = c + 1; row < 3; row++) {
            const double m = A[row][c] / A[c][c];
            for (int k = c; k < 4; k++) A[row][k] -= m * A[c][k];
        }
    }
    double f[3];
    for (int c = 2; c >= 0; c--) {
        double v = A[c][3];
        for (int k = c + 1; k < 3; k++) v -= A[c][k] * f[k];
        f[c] = v / A[c][c];
    }
    const size_t n[3] = {g.xs, g.ys, g.zs};
    long long idx[3];
    for (int a = 0; a < 3; a++) {
        const double v = f[a] * (double)n[a];
        if (!std::isfinite(v) || std::fabs(v) > 4e18) return 0.0;
        idx[a] = (long long)std::round(v);
        if (idx[a] < 0 || (size_t)idx[a] >= n[a]) return 0.0;
    }
    return g.cube[((size_t)idx[0] * g.ys + (size_t)idx[1]) * g.zs + (size_t)idx[2]];
}

// xcfloader::getvalue (src/loadxcf.cc:330-332): lattice units -> Cartesian with CONVVEC
static double xsf_value(const XsfGrid &g, double xu, double yu, double z, const double *shift)
{
    return xsf_cart_value(g, xu * g.convvec[0][0] + yu * g.convvec[1][0], xu * g.convvec[0][1] + yu * g.convvec[1][1],
                          z, shift);
}

// xcfloader::getzheight (src/loadxcf.cc:334-348): above the highest / below the lowest atom
static double xsf_zheight(const XsfGrid &g, double height)
{
    double z = NAN;
    if (height > 0.0 && !g.atom_z.empty()) {
        z = g.atom_z[0];
        for (double v : g.atom_z) z = std::max(z, v);
        z += height;
    } else if (height < 0.0 && !g.atom_z.empty()) {
        z = g.atom_z[0];
        for (double v : g.atom_z) z = std::min(z, v);
        z += height;
    }
    return z;
}

int cqpi_xsf_orbital_cache(const char *path, double height, int32_t window, int32_t oversamp, double prefact,
                           double *out)
{
    const double zero[3] = {0.0, 0.0, 0.0};
    return cqpi_xsf_orbital_cache_shifted(path, zero, 0, height, window, oversamp, prefact, out);
}

int cqpi_xsf_orbital_cache_shifted(const char *path, const double *shift, int32_t centre, double height,
                                   int32_t window, int32_t oversamp, double prefact, double *out)
{
    if (!path || !out || !shift || window < 0 || oversamp < 1)
        return host_fail(CQPI_ERR_ARG, "invalid XSF orbital arguments");
    XsfGrid g;
    std::string err;
    if (!xsf_read(path, g, err)) return host_fail(CQPI_ERR_ARG, err);
    const double z = xsf_zheight(g, height), ofs = centre ? 0.5 : 0.0;
    const int n = (2 * window + 1) * oversamp;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            out[(size_t)i * n + j] = prefact * xsf_value(g, (double)i / oversamp - (double)window - ofs,
                                                         (double)j / oversamp - (double)window - ofs, z, shift);
    return CQPI_OK;
}

int cqpi_xsf_orbital_cache_mod(const char *path, const double *modshift, const double *basis, double height,
                               double xpos, double ypos, double theta, double prefact, int32_t window,
                               int32_t oversamp, double *out)
{
    if (!path || !out || !modshift || window < 0 || oversamp < 1)
        return host_fail(CQPI_ERR_ARG, "invalid XSF orbital arguments");
    XsfGrid g;
    std::string err;
    if (!xsf_read(path, g, err)) return host_fail(CQPI_ERR_ARG, err);
    const double z = xsf_zheight(g, height), cs = cos(theta), sn = sin(theta);
    const int n = (2 * window + 1) * oversamp;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            // wannierfunctions(ucv, xcfloader, ...) (src/wannierfunctions.cc:500-520): shift,
            // basis, then xcfloader::getcartmodvalue (src/loadxcf.cc:268-290): rotation by theta
            double x = (double)i / oversamp - (double)window - xpos, y = (double)j / oversamp - (double)window - ypos;
            if (basis) {
                const double a = x, b = y;
                x = basis[0] * a + basis[2] * b;
                y = basis[1] * a + basis[3] * b;
            }
            const double xr = x * cs - y * sn, yr = x * sn + y * cs;
            out[(size_t)i * n + j] = prefact * xsf_cart_value(g, xr, yr, z, modshift);
        }
    return CQPI_OK;
}

}  // extern "C"
