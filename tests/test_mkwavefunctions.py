"""The orbital-file tool mkwavefunctions (host/mkwavefunctions_main.cc) against the
reference's own tool (src/mkwavefunctions.cc, built from its sources by oracle/build_ref.sh):
golden configurations under tests/golden/mkwf_*/ cover every orbital source (analytic orbitals
with lattice basis vectors, XSF files with a shift, XSF files placed per orbital, an IDL file,
interpolation between IDL files with each method), reorder and double.  The interpolation
itself (cqpi_interp_eval) is also checked against scipy's implementations of the same
published methods.  CPU only: the tool never touches the GPU."""
import ctypes
import glob
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from oracle import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = sorted(os.path.basename(d) for d in glob.glob(os.path.join(GOLDEN, "mkwf_*")))
CONFIGS = [(c, k) for c in CASES for k in json.load(open(os.path.join(GOLDEN, c, "meta.json")))["configs"]]


def _tool(built_lib):
    return os.path.join(os.path.dirname(built_lib["lib"]), "mkwavefunctions")


def _run(built_lib, cwd, cfg):
    return subprocess.run([_tool(built_lib), cfg], cwd=cwd, capture_output=True, text=True, timeout=120)


def _strip_time(line):
    return re.sub(r"^\d{4}-\d\d-\d\d\.\d\d:\d\d:\d\d ", "", line)


@pytest.mark.parametrize("case,k", CONFIGS)
def test_tool_matches_reference(built_lib, tmp_path, case, k):
    src = os.path.join(GOLDEN, case)
    d = tmp_path / case
    shutil.copytree(src, d)
    cfg = (d / ("input_%s.cfg" % k)).read_text().replace('mkwffile="ref_%s.idl";' % k, 'mkwffile="ours.idl";')
    (d / "ours.cfg").write_text(cfg)
    r = _run(built_lib, d, "ours.cfg")
    assert r.returncode == 0, r.stdout + r.stderr
    hr, ref = F.read_idl(os.path.join(src, "ref_%s.idl" % k))
    ho, ours = F.read_idl(str(d / "ours.idl"))
    for key in ("name", "size", "scan_range", "offset", "bias", "setpoint"):
        assert ho[key] == hr[key], (key, ho[key], hr[key])
    exact = json.load(open(os.path.join(src, "meta.json")))["configs"][k]["exact"]
    if exact:
        np.testing.assert_array_equal(ours, ref)
        # the boundary check prints the same figures
        want = [_strip_time(l) for l in open(os.path.join(src, "ref_%s.txt" % k)) if "Wave function" in l
                or "Maximum rel." in l]
        got = [_strip_time(l + "\n") for l in r.stdout.splitlines() if "Wave function" in l or "Maximum rel." in l]
        assert got == want
    else:
        # a different but equivalent linear solve / evaluation order: float32 rounding at most
        scale = float(np.abs(ref).max())
        assert np.abs(ours.astype(np.float64) - ref).max() <= 1e-6 * scale


def _interp(lib, method, xa, ya, x):
    xa = np.ascontiguousarray(xa, np.float64)
    ya = np.ascontiguousarray(ya, np.float64)
    x = np.ascontiguousarray(np.atleast_1d(x), np.float64)
    y = np.zeros_like(x)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.cqpi_interp_eval(method.encode(), len(xa), xa.ctypes.data_as(dp), ya.ctypes.data_as(dp), len(x),
                              x.ctypes.data_as(dp), y.ctypes.data_as(dp))
    return rc, y


@pytest.fixture(scope="module")
def hostlib(built_lib):
    lib = ctypes.CDLL(built_lib["lib"])
    lib.cqpi_interp_eval.restype = ctypes.c_int
    lib.cqpi_interp_eval.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def _data(seed, n=7):
    rng = np.random.default_rng(seed)
    xa = np.cumsum(rng.uniform(0.2, 1.0, n))
    ya = rng.normal(size=n)
    x = np.concatenate([np.linspace(xa[0], xa[-1], 41), xa])
    return xa, ya, x


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_interp_against_scipy(hostlib, seed):
    si = pytest.importorskip("scipy.interpolate")
    xa, ya, x = _data(seed)
    checks = {
        "linear": np.interp(x, xa, ya),
        "polynomial": si.BarycentricInterpolator(xa, ya)(x),
        "cspline": si.CubicSpline(xa, ya, bc_type="natural")(x),
        "akima": si.Akima1DInterpolator(xa, ya)(x),
    }
    yp = ya.copy()
    yp[-1] = yp[0]
    checks["cspline_periodic"] = None
    for m, want in checks.items():
        if m == "cspline_periodic":
            rc, got = _interp(hostlib, m, xa, yp, x)
            want = si.CubicSpline(xa, yp, bc_type="periodic")(x)
        else:
            rc, got = _interp(hostlib, m, xa, ya, x)
        assert rc == 0, m
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-10 * np.abs(want).max(), err_msg=m)
    # every method passes through the data points
    for m in ("linear", "polynomial", "cspline", "akima", "akima_periodic", "steffen"):
        rc, got = _interp(hostlib, m, xa, ya, xa)
        np.testing.assert_allclose(got, ya, rtol=1e-12, atol=1e-12, err_msg=m)


def test_interp_steffen_is_monotone(hostlib):
    # Steffen's interpolant never overshoots monotone data; the cubic spline does here
    xa = np.array([0.0, 1.0, 1.5, 3.0, 3.2, 5.0])
    ya = np.array([0.0, 0.1, 2.0, 2.1, 5.0, 5.05])
    x = np.linspace(0.0, 5.0, 2001)
    rc, y = _interp(hostlib, "steffen", xa, ya, x)
    assert rc == 0
    assert np.all(np.diff(y) >= -1e-14)
    rc, yc = _interp(hostlib, "cspline", xa, ya, x)
    assert np.any(np.diff(yc) < 0)


def test_interp_akima_periodic_continues_slopes(hostlib):
    # periodic data sampled from a periodic function: the periodic Akima curve has the same
    # slope at both ends, the plain one need not
    xa = np.linspace(0.0, 1.0, 9)
    ya = np.sin(2 * np.pi * xa) + 0.3 * np.cos(4 * np.pi * xa)
    h = 1e-6
    _, yl = _interp(hostlib, "akima_periodic", xa, ya, np.array([0.0, h]))
    _, yr = _interp(hostlib, "akima_periodic", xa, ya, np.array([1.0 - h, 1.0]))
    assert abs((yl[1] - yl[0]) / h - (yr[1] - yr[0]) / h) < 1e-4


def test_interp_errors(hostlib):
    xa, ya, _ = _data(4)
    assert _interp(hostlib, "linear", xa, ya, xa[-1] + 1e-9)[0] != 0        # outside the range
    assert _interp(hostlib, "linear", xa, ya, xa[0] - 1e-9)[0] != 0
    assert _interp(hostlib, "bogus", xa, ya, xa[0])[0] != 0                 # unknown method
    assert _interp(hostlib, "akima", xa[:4], ya[:4], xa[0])[0] != 0         # akima needs 5 points
    assert _interp(hostlib, "cspline", xa[:2], ya[:2], xa[0])[0] != 0       # cspline needs 3
    bad = xa.copy()
    bad[3] = bad[2]
    assert _interp(hostlib, "linear", bad, ya, xa[0])[0] != 0               # not strictly increasing


def _case_copy(tmp_path, case):
    d = tmp_path / case
    shutil.copytree(os.path.join(GOLDEN, case), d)
    return d


def test_tool_errors(built_lib, tmp_path):
    d = _case_copy(tmp_path, "mkwf_mod")
    base = (d / "input_plain.cfg").read_text()
    # an orbital index past the modorbitalfiles list (the reference reads past its vector)
    (d / "a.cfg").write_text(base.replace("orbitals=(0,0);", "orbitals=(0,1);"))
    r = _run(built_lib, d, "a.cfg")
    assert r.returncode == 1 and "modorbitalfiles" in r.stdout
    # reorder past the orbital list
    (d / "b.cfg").write_text(base + "reorder=(0,2);\n")
    r = _run(built_lib, d, "b.cfg")
    assert r.returncode == 1 and "reorder" in r.stdout
    # no output file
    (d / "c.cfg").write_text(base.replace('mkwffile="ref_plain.idl";', ""))
    r = _run(built_lib, d, "c.cfg")
    assert r.returncode == 1 and "No output file" in r.stdout
    # no orbital source
    (d / "e.cfg").write_text('mkwffile="x.idl";\nwindow=1;\n')
    r = _run(built_lib, d, "e.cfg")
    assert r.returncode == 1 and "No orbitals specified" in r.stdout
    # interpolation outside the values (GSL's default error handler aborts the reference)
    di = _case_copy(tmp_path, "mkwf_interp")
    cfg = (di / "input_linear.cfg").read_text().replace("interpolate=0.35;", "interpolate=1.5;")
    (di / "f.cfg").write_text(cfg)
    r = _run(built_lib, di, "f.cfg")
    assert r.returncode == 1 and "interpolation" in r.stdout
    # only one basis vector
    da = _case_copy(tmp_path, "mkwf_analytic")
    cfg = (da / "input_basis.cfg").read_text().replace("basisvector[1]=(0.5,0.866);", "")
    (da / "g.cfg").write_text(cfg)
    r = _run(built_lib, da, "g.cfg")
    assert r.returncode == 1 and "only one basis vector" in r.stdout


def test_tool_output_feeds_calcqpi_orbitals(built_lib, tmp_path):
    """The tool's file is an idlorbitalfile: its layers are the caches the host library builds
    for the same analytic keywords (cqpi_orbital_cache_basis with the unit basis)."""
    d = _case_copy(tmp_path, "mkwf_analytic")
    r = _run(built_lib, d, "input_plain.cfg")
    assert r.returncode == 0
    _, data = F.read_idl(str(d / "ref_plain.idl"))
    lib = ctypes.CDLL(built_lib["lib"])
    dp = ctypes.POINTER(ctypes.c_double)
    lib.cqpi_orbital_cache_basis.argtypes = [ctypes.c_char_p] + [ctypes.c_double] * 7 + [ctypes.c_void_p,
                                                                                        ctypes.c_int32,
                                                                                        ctypes.c_int32, dp]
    side = 3 * 5
    out = np.zeros(side * side)
    # orbital 2: dr2 at pos (0.1, -0.1, 0.3), radius 0.8, angle 12 deg, zheight 0.9
    rc = lib.cqpi_orbital_cache_basis(b"dr2", 0.8, 0.9 - 0.3, 0.1, -0.1, 12 * np.pi / 180, 0.0, 1.0, None, 1, 5,
                                      out.ctypes.data_as(dp))
    assert rc == 0
    np.testing.assert_array_equal(data[2].T, out.reshape(side, side).astype(np.float32))


def test_python_bindings(built_lib, tmp_path):
    """cqpi.host binds the tool's host functions: the same caches as the C ABI calls above."""
    from cqpi import host
    side = 3 * 5
    a = host.orbital_cache_basis("dr2", 1, 5, width=0.8, height=0.6, xpos=0.1, ypos=-0.1,
                                 theta=12 * np.pi / 180)
    b = host.orbital_cache("dr2", 1, 5, width=0.8, height=0.6, xpos=0.1, ypos=-0.1, theta=12 * np.pi / 180)
    assert a.shape == (side, side) and np.array_equal(a, b)
    sheared = host.orbital_cache_basis("dxy", 1, 5, width=0.8, height=0.6, basis=((1.0, 0.0), (0.5, 0.866)))
    assert not np.array_equal(sheared, host.orbital_cache("dxy", 1, 5, width=0.8, height=0.6))
    xsf = os.path.join(GOLDEN, "mkwf_xsf", "orb0.xsf")
    c0 = host.xsf_orbital_cache_shifted(xsf, 0.7, 2, 3, shift=(0.0, 0.0, 0.0), centre=False)
    np.testing.assert_array_equal(c0, host.xsf_orbital_cache(xsf, 0.7, 2, 3))
    m0 = host.xsf_orbital_cache_mod(xsf, 0.7, 2, 3)
    assert m0.shape == (15, 15) and np.abs(m0).max() > 0
    y = host.interp_eval("linear", [0.0, 1.0, 2.0], [0.0, 2.0, 0.0], [0.5, 1.5])
    np.testing.assert_allclose(y, [1.0, 1.0])
    with pytest.raises(host.HostError):
        host.interp_eval("linear", [0.0, 1.0], [0.0, 1.0], 2.0)

