"""Restatements of the reference's input/output formats (oracle, test infrastructure only).

Only tests/, the smoke check and bench.py's CPU-baseline leg import this module, as
the checker of the engine's C++ host code.  Nothing in the product imports it.

* ``read_hr``      -- tightbind::readfile, src/tightbinding.cc:70-149
* ``read_idl`` / ``write_idl`` -- idl::read / idl::write, src/idl.cc:50-97
* ``LoadConfig``   -- loadconfig, include/parser.h:24-197
* ``read_xsf`` / ``xsf_orbital_cache`` -- xcfloader (src/loadxcf.cc:37-345) and the XSF
  constructor of wannierfunctions (src/wannierfunctions.cc:444-463); ``write_xsf`` writes
  the fixture files
"""
from __future__ import annotations

import math
import re
import time

import numpy as np

_DIGITS = "0123456789"


def _find_first_of(s: str, chars: str, pos: int = 0) -> int:
    for i in range(max(pos, 0), len(s)):
        if s[i] in chars:
            return i
    return -1


class _Extract:
    """Formatted extraction like ``std::istringstream >> int/double``: skip blanks, then
    take the longest prefix that forms a number (so '1-2.0e+00' yields 1, then -2.0)."""
    _INT = re.compile(r"[+-]?\d+")
    _REAL = re.compile(r"[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)")

    def __init__(self, s):
        self.s, self.p = s, 0

    def _take(self, rx):
        while self.p < len(self.s) and self.s[self.p] in " \t\r\n\v\f":
            self.p += 1
        m = rx.match(self.s, self.p)
        if not m:
            raise ValueError("no number at %d" % self.p)
        self.p = m.end()
        return m.group(0)

    def integer(self):
        return int(self._take(self._INT))

    def real(self):
        return float(self._take(self._REAL))


def read_hr(text: str, scmodel: bool = False):
    """Parse a Wannier90 ``_hr.dat`` the way tightbinding.cc:70-149 does.

    Returns dict(name, bands, R[h,3], orb[h,2] (0-based), t[h] complex (divided by the
    degeneracy), anti[h] bool).  Raises ValueError where the reference sets its error flag
    or exits (invalid orbital index, tightbinding.cc:139-141).
    """
    lines = text.split("\n")
    li = 0

    def getline():
        nonlocal li
        if li >= len(lines):
            raise ValueError("unexpected end of file")
        s = lines[li]
        li += 1
        return s

    name = getline()
    cut = _find_first_of(name, "\n\r")
    if cut >= 0:
        name = name[:cut]
    bands = int(getline().split()[0])
    nrpts = int(getline().split()[0])
    scmax = bands >> 1 if scmodel else bands
    degs = []
    buf, pos = "", 0
    while len(degs) < nrpts:
        if pos == 0:
            buf = getline()
            pos = _find_first_of(buf, _DIGITS, 0)
            if pos < 0:
                raise ValueError("degeneracy line without digits")
        npos = _find_first_of(buf, " \t", pos)
        ln = (npos - pos) if npos >= 0 else len(buf) - pos
        npos = _find_first_of(buf, _DIGITS, npos) if npos >= 0 else -1
        tok = buf[pos:pos + ln].split()
        if not tok:
            raise ValueError("bad degeneracy entry")
        degs.append(int(tok[0]))
        pos = npos if npos >= 0 else 0
    R, orb, t, anti = [], [], [], []
    k = 0
    prev = None
    while li < len(lines):
        s = lines[li]
        li += 1
        if len(s) == 0:
            continue
        sc = _Extract(s)
        try:
            x, y, z, u, v = sc.integer(), sc.integer(), sc.integer(), sc.integer(), sc.integer()
            hr, hc = sc.real(), sc.real()
        except ValueError:
            raise ValueError(f"bad hopping line: {s!r}")
        if k == 0 or (x, y, z) != prev:
            k += 1
            prev = (x, y, z)
        if k - 1 >= len(degs):
            raise ValueError("more R vectors than degeneracies")
        d = float(degs[k - 1])
        if u <= 0 or v <= 0 or u > bands or v > bands:
            raise ValueError("invalid orbital index")
        R.append((x, y, z))
        orb.append((u - 1, v - 1))
        t.append(complex(hr / d, hc / d))
        anti.append((u - 1) >= scmax and (v - 1) >= scmax)
    return dict(name=name, bands=bands,
                R=np.array(R, dtype=np.int32).reshape(-1, 3),
                orb=np.array(orb, dtype=np.int32).reshape(-1, 2),
                t=np.array(t, dtype=np.complex128),
                anti=np.array(anti, dtype=bool), scmaxbands=scmax)


def write_hr(path, name: str, bands: int, terms: dict, degeneracy=None):
    """Write a ``_hr.dat`` (Wannier90 layout).

    ``terms`` maps (Rx, Ry, Rz) -> complex [bands, bands] hopping matrix; ``degeneracy``
    maps R -> integer weight (default 1).  Stored values are hopping * weight so the
    reader's division by the degeneracy returns the hopping."""
    keys = sorted(terms)
    deg = {k: 1 for k in keys} if degeneracy is None else degeneracy
    out = [name, f"{bands:12d}", f"{len(keys):12d}"]
    degs = [f"{deg[k]:5d}" for k in keys]
    for i in range(0, len(degs), 15):
        out.append("".join(degs[i:i + 15]))
    for key in keys:
        mat = terms[key] * deg[key]
        for v in range(bands):
            for u in range(bands):
                c = mat[u, v]
                out.append(f"{key[0]:5d}{key[1]:5d}{key[2]:5d}{u + 1:5d}{v + 1:5d}"
                           f"{c.real:22.15e}{c.imag:22.15e}")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def cxx_double(x: float) -> str:
    """Format a double like ``std::ostream << double`` with default flags (%g, precision 6)."""
    if math.isnan(x):
        return "nan" if math.copysign(1.0, x) > 0 else "-nan"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return "%g" % x


def idl_bias(lb: float, hb: float, layers: int, k: int) -> float:
    """idl::getbias, src/idl.cc:969-973."""
    if layers == 1:
        return lb
    return (hb - lb) * k / (layers - 1.0) + lb


def write_idl(path, data_kyx: np.ndarray, name: str, scan_range=(2.0, 2.0), offset=(-1.0, -1.0),
              bias=(0.0, 0.0), setpoint=0.0, date: str | None = None):
    """idl::write, src/idl.cc:78-97: 12 text lines, then float32 data layer-major, y, x fastest."""
    z, y, x = data_kyx.shape
    if date is None:
        date = time.ctime()
    head = [name, date, str(x), str(y), str(z), cxx_double(scan_range[0]), cxx_double(scan_range[1]),
            cxx_double(offset[0]), cxx_double(offset[1]), cxx_double(bias[0]), cxx_double(bias[1]),
            cxx_double(setpoint)]
    with open(path, "wb") as fh:
        fh.write(("\n".join(head) + "\n").encode())
        fh.write(np.ascontiguousarray(data_kyx, dtype="<f4").tobytes())


def read_idl(path):
    """idl::read, src/idl.cc:50-76.  Returns (header dict, data[z][y][x] float32)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    pos = 0
    lines = []
    for _ in range(2):
        e = raw.index(b"\n", pos)
        lines.append(raw[pos:e].decode(errors="replace"))
        pos = e + 1
    vals = []
    while len(vals) < 10:
        while raw[pos:pos + 1].isspace():
            pos += 1
        e = pos
        while e < len(raw) and not raw[e:e + 1].isspace():
            e += 1
        vals.append(raw[pos:e].decode())
        pos = e
    pos += 1  # is.ignore(1,'\n')
    x, y, z = int(vals[0]), int(vals[1]), int(vals[2])
    hdr = dict(name=lines[0], date=lines[1], size=(x, y, z),
               scan_range=(float(vals[3]), float(vals[4])), offset=(float(vals[5]), float(vals[6])),
               bias=(float(vals[7]), float(vals[8])), setpoint=float(vals[9]))
    data = np.frombuffer(raw, dtype="<f4", count=x * y * z, offset=pos).reshape(z, y, x)
    return hdr, data


class LoadConfig:
    """loadconfig, include/parser.h:24-197 (non-line mode)."""

    def __init__(self, text: str):
        self.name, self.field, self.comments = [], [], []
        self.warnings = []
        for line in text.split("\n"):
            if len(line) == 0:
                continue
            h = line.find("#")
            if h >= 0:
                self.comments.append(line[h + 1:])
                line = line[:h]
            eq, sc = line.find("="), line.find(";")
            if eq >= 0 and sc >= 0:
                self.name.append(line[:eq])
                self.field.append(line[eq + 1:sc])
            elif eq >= 0 or sc >= 0:
                self.warnings.append(line)
        self.used = [0] * len(self.name)

    def probefield(self, key):
        for i, n in enumerate(self.name):
            if n == key:
                self.used[i] += 1
                return True
        return False

    def getfield(self, key):
        val = ""
        for i, n in enumerate(self.name):
            if n == key:
                self.used[i] += 1
                val = self.field[i]
        if not val:
            return ""
        s = len(val) - len(val.lstrip(" \t"))
        e = len(val.rstrip(" \t"))
        if e <= s:
            return val[s:]
        return val[s:e]

    @staticmethod
    def _field2string(v):
        f, l = v.find('"'), v.rfind('"')
        return v[f + 1:l] if f >= 0 and l >= 0 else ""

    def getstring(self, key):
        return self._field2string(self.getfield(key))

    def getvalue(self, key):
        v = self.getfield(key)
        return _atof(v) if v else float("nan")

    def getintvalue(self, key):
        v = self.getfield(key)
        return _atoi(v) if v else 0

    def getlist(self, key):
        v = self.getfield(key)
        f, l = v.find("("), v.rfind(")")
        out = []
        if f >= 0 and l >= 0:
            idx = f + 1
            while True:
                nidx = _find_first_of(v, ",)", idx)
                out.append(v[idx:nidx].strip(" \t"))
                idx = nidx + 1
                if nidx == l:
                    break
        return out

    def getvector(self, key):
        return [_atof(s) for s in self.getlist(key)]

    def unused(self):
        return [self.name[i] for i, u in enumerate(self.used) if not u]


def _atof(s: str) -> float:
    s = s.lstrip(" \t\n")
    best = 0.0
    for e in range(len(s), 0, -1):
        try:
            return float(s[:e])
        except ValueError:
            continue
    return best


def _atoi(s: str) -> int:
    s = s.lstrip(" \t\n")
    e = 0
    if e < len(s) and s[e] in "+-":
        e += 1
    while e < len(s) and s[e].isdigit():
        e += 1
    try:
        return int(s[:e])
    except ValueError:
        return 0


# --------------------------------------------------------------------------- XSF orbitals
class Xsf:
    """XSF file as xcfloader::readfile keeps it (src/loadxcf.cc:37-185): comments, PRIMVEC,
    CONVVEC, PRIMCOORD atoms, and the first 3D data grid cube[i][j][k] (x fastest in the
    file) with its origin and spanning vectors.  ``error`` mirrors xcfloader::error."""

    def __init__(self):
        self.comments, self.primvec, self.convvec, self.atoms, self.coords = [], [], [], [], []
        self.origin, self.axes = [], []
        self.shape = (0, 0, 0)
        self.cube = None
        self.error = False


def read_xsf(path) -> Xsf:
    """xcfloader::readfile restated: a line counts only when a newline ends it
    (``while(!eof) { getline; if(!eof) ... }``); '#' anywhere makes the rest a comment;
    CRYSTAL enables PRIMVEC / CONVVEC / PRIMCOORD; the data grid is tokenised as the
    reference does (a token starts at one of '+-0123456789' and ends at a blank; a token
    that runs to the end of its line loads the next line)."""
    x = Xsf()
    with open(path, "r", newline="") as fh:
        text = fh.read()
    parts = text.split("\n")
    lines = parts[:-1]          # the last piece has no newline after it
    it = iter(lines)
    pos_line = [0]

    def nxt():
        pos_line[0] += 1
        try:
            return next(it)
        except StopIteration:
            return ""

    crystal = False
    while True:
        try:
            line = next(it)
        except StopIteration:
            break
        pos_line[0] += 1
        h = line.find("#")
        if h >= 0:
            x.comments.append(line[h + 1:])
            continue
        if "CRYSTAL" in line:
            crystal = True
        elif crystal and "PRIMVEC" in line:
            for _ in range(3):
                e = _Extract(nxt())
                x.primvec.append([e.real(), e.real(), e.real()])
        elif crystal and "CONVVEC" in line:
            for _ in range(3):
                e = _Extract(nxt())
                x.convvec.append([e.real(), e.real(), e.real()])
        elif crystal and "PRIMCOORD" in line:
            e = _Extract(nxt())
            natoms = e.integer()
            for _ in range(natoms):
                toks = nxt().split()
                x.atoms.append(toks[0])
                x.coords.append([float(toks[1]), float(toks[2]), float(toks[3])])
        elif "BEGIN_BLOCK_DATAGRID_3D" in line:
            t = nxt().split()
            if not t or t[0] != "3D_field":
                x.error = True
            t = nxt().split()
            if not t or t[0] != "BEGIN_DATAGRID_3D_UNKNOWN":
                x.error = True
            e = _Extract(nxt())
            xs, ys, zs = e.integer(), e.integer(), e.integer()
            x.shape = (xs, ys, zs)
            e = _Extract(nxt())
            x.origin = [e.real(), e.real(), e.real()]
            for _ in range(3):
                e = _Extract(nxt())
                x.axes.append([e.real(), e.real(), e.real()])
            cube = np.zeros((xs, ys, zs))
            line = nxt()
            npos = 0
            for k in range(zs):
                for j in range(ys):
                    for i in range(xs):
                        p = _find_first_of(line, "+-0123456789", npos)
                        if p < 0:
                            x.error = True
                            x.cube = cube
                            return x
                        npos = _find_first_of(line, " \t", p)
                        reload = npos < 0
                        tok = line[p:] if reload else line[p:npos]
                        try:
                            cube[i, j, k] = _Extract(tok).real()
                        except ValueError:
                            cube[i, j, k] = 0.0
                        if reload:
                            line = nxt()
                            npos = 0
            x.cube = cube
            if "END_DATAGRID_3D" not in line:
                x.error = True
            if "END_BLOCK_DATAGRID_3D" not in nxt():
                x.error = True
    return x


def _cround(v: float) -> int:
    """C's round(): half away from zero (abs(v) - floor(abs(v)) is exact in binary)."""
    a = abs(v)
    r = math.floor(a)
    if a - r >= 0.5:
        r += 1
    return int(r) if v >= 0 else -int(r)


def xsf_value(x: Xsf, xu: float, yu: float, z: float) -> float:
    """xcfloader::getvalue + operator() (src/loadxcf.cc:187-202,326-328): lattice units ->
    Cartesian with CONVVEC, fractional grid coordinates from the spanning vectors, nearest
    grid point round(f * n), zero outside the grid (and for a NaN height)."""
    cx = xu * x.convvec[0][0] + yu * x.convvec[1][0]
    cy = xu * x.convvec[0][1] + yu * x.convvec[1][1]
    b = np.array([cx, cy, z]) - np.array(x.origin)
    M = np.array(x.axes, dtype=np.float64).T          # columns: spanning vectors
    f = np.linalg.solve(M, b)
    if not np.all(np.isfinite(f)):
        return 0.0
    idx = [_cround(v * n) for v, n in zip(f, x.shape)]
    if all(0 <= idx[a] < x.shape[a] for a in range(3)):
        return float(x.cube[idx[0], idx[1], idx[2]])
    return 0.0


def xsf_zheight(x: Xsf, height: float) -> float:
    """xcfloader::getzheight (src/loadxcf.cc:330-345)."""
    if height > 0.0:
        return max(c[2] for c in x.coords) + height
    if height < 0.0:
        return min(c[2] for c in x.coords) + height
    return float("nan")


def xsf_orbital_cache(path, height, window, oversamp, prefact=1.0) -> np.ndarray:
    """wannierfunctions(filename, height, window, oversamp, prefact)
    (src/wannierfunctions.cc:444-463): cache[i][j] = prefact * getvalue(i/os - w, j/os - w,
    zheight), side (2w+1) os -- no half-cell shift, unlike the analytic orbitals."""
    x = read_xsf(path)
    if x.error:
        raise ValueError("XSF file could not be read: %s" % path)
    z = xsf_zheight(x, height)
    n = (2 * window + 1) * oversamp
    out = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            out[i, j] = prefact * xsf_value(x, i / oversamp - window, j / oversamp - window, z)
    return out


def write_xsf(path, cube: np.ndarray, origin, axes, convvec, atoms, comment="generated", per_line=6):
    """An XSF file (CRYSTAL, PRIMVEC = CONVVEC, PRIMCOORD, one 3D data grid) that the
    reference's reader accepts: values x fastest, a newline after every per_line values and
    after the last one, no trailing blanks."""
    xs, ys, zs = cube.shape
    out = ["# " + comment, "CRYSTAL", "PRIMVEC"]
    out += ["%.10f %.10f %.10f" % tuple(v) for v in convvec]
    out.append("CONVVEC")
    out += ["%.10f %.10f %.10f" % tuple(v) for v in convvec]
    out.append("PRIMCOORD")
    out.append("%d 1" % len(atoms))
    out += ["%s %.10f %.10f %.10f" % (a[0], a[1], a[2], a[3]) for a in atoms]
    out += ["BEGIN_BLOCK_DATAGRID_3D", "3D_field", "BEGIN_DATAGRID_3D_UNKNOWN", "%d %d %d" % (xs, ys, zs),
            "%.10f %.10f %.10f" % tuple(origin)]
    out += ["%.10f %.10f %.10f" % tuple(v) for v in axes]
    vals = ["%.8e" % v for v in np.transpose(cube, (2, 1, 0)).reshape(-1)]
    for s in range(0, len(vals), per_line):
        out.append(" ".join(vals[s:s + per_line]))
    out += ["END_DATAGRID_3D", "END_BLOCK_DATAGRID_3D"]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
