"""CPU tests of libcqpi.so: exported symbols and the host-side C ABI (no GPU calls)."""
import os
import re
import subprocess

import numpy as np
import pytest

from golden_cases import NAMES, load
from oracle import formats as F
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("cqpi.h", "cqpi_host.h"):
        with open(os.path.join(ROOT, "include", h)) as fh:
            txt = fh.read()
        names |= set(re.findall(r"\b(cqpi_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_loads_and_exports_every_declared_symbol(built_lib):
    import cqpi
    L = cqpi.load()
    for name in sorted(_declared()):
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib["lib"]], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cqpi_[a-z0-9_]+)", out))
    assert _declared() <= exported
    assert L.cqpi_version().decode().startswith("cqpi-gb300")


@pytest.mark.parametrize("name", NAMES)
def test_read_hr_matches_restatement(built_lib, name):
    from cqpi import host
    d, meta, ref = load(name)
    path = os.path.join(d, "model_hr.dat")
    sc = meta.get("scmodel", False)
    got = host.read_hr(path, sc)
    with open(path) as fh:
        exp = F.read_hr(fh.read(), sc)
    assert got["bands"] == exp["bands"] and got["name"] == exp["name"]
    assert np.array_equal(got["R"], exp["R"]) and np.array_equal(got["orb"], exp["orb"])
    assert np.array_equal(got["t"], exp["t"]) and np.array_equal(got["anti"], exp["anti"])


def test_read_hr_errors(built_lib, tmp_path):
    from cqpi import host
    with pytest.raises(host.HostError):
        host.read_hr(str(tmp_path / "missing_hr.dat"))
    bad = tmp_path / "bad_hr.dat"
    bad.write_text("name\n1\n1\n    1\n    0    0    0    2    1  1.0  0.0\n")   # orbital index 2 > 1 band
    with pytest.raises(host.HostError):
        host.read_hr(str(bad))
    bad.write_text("name\n1\n1\n    1\n    0    0    0    1    1  x  0.0\n")
    with pytest.raises(host.HostError):
        host.read_hr(str(bad))
    ok = tmp_path / "ok_hr.dat"
    # two R vectors, degeneracies on two lines, value split across the degeneracy
    ok.write_text("demo\n1\n2\n    4\n    2\n    1    0    0    1    1  -4.0  0.0\n"
                  "   -1    0    0    1    1-4.0 2.0\n")
    hr = host.read_hr(str(ok))
    assert np.allclose(hr["t"], [-1.0, -2.0 + 1.0j])


@pytest.mark.parametrize("name", ["s", "px", "py", "pz", "dx2", "dxy", "dxz", "dyz", "dr2", "fy3x2", "fxyz",
                                  "fyz2", "fz3", "fxz2", "fzx2", "fxx2", "n", "z"])
def test_orbital_cache_matches_restatement(built_lib, name):
    from cqpi import host
    kw = dict(width=0.45, height=0.7, xpos=0.1, ypos=-0.2, theta=0.3, phi=0.0, prefact=1.3)
    got = host.orbital_cache(name, 2, 5, **kw)
    exp = O.orbital_cache(name, 2, 5, **kw)
    assert np.abs(got - exp).max() <= 1e-14 * max(1.0, np.abs(exp).max())


def test_orbital_cache_matches_reference_wffile(built_lib):
    from cqpi import host
    d, meta, ref = load("c2_analytic")
    hdr, data = F.read_idl(os.path.join(d, "ref_wf.idl"))
    spec = meta["orbitals"][1]
    for o, nm in enumerate(spec["names"]):
        got = host.orbital_cache(nm, meta["w"], meta["os"], width=spec["radius"], height=spec["zheight"])
        assert np.abs(got.astype(np.float32).T - data[o]).max() <= 1e-7 * np.abs(data[o]).max()


def test_idl_layerwise_equals_oneshot(built_lib, tmp_path):
    """cqpi_idl_create + cqpi_idl_write_layers (the CLI's flush / resume) give the file that
    cqpi_idl_write gives in one go, whatever order the layer groups arrive in."""
    from cqpi import host
    rng = np.random.default_rng(3)
    data = rng.normal(size=(7, 5, 6)).astype(np.float32)
    kw = dict(scan_range=(2.0, 2.0), offset=(-1.0, -1.0), bias=(-0.1, 0.1), date="Thu Jan  1 00:00:00 2026")
    host.idl_write(tmp_path / "one.idl", data, "CQPI calculation for m with window=2 and oversamp=4", **kw)
    host.idl_create(tmp_path / "lay.idl", data.shape, "CQPI calculation for m with window=2 and oversamp=4", **kw)
    _, z = host.idl_read(tmp_path / "lay.idl")
    assert z.shape == data.shape and not z.any()
    for k0, k1 in ((4, 7), (0, 2), (2, 4)):
        host.idl_write_layers(tmp_path / "lay.idl", k0, data[k0:k1])
    assert (tmp_path / "lay.idl").read_bytes() == (tmp_path / "one.idl").read_bytes()
    with pytest.raises(host.HostError):
        host.idl_write_layers(tmp_path / "lay.idl", 6, data[:2])   # past the last layer


def test_idl_roundtrip_and_reference_bytes(built_lib, tmp_path):
    from cqpi import host
    for name in NAMES:
        d, meta, ref = load(name)
        path = os.path.join(d, "ref_qpi.idl")
        hdr, data = host.idl_read(path)
        hdr2, data2 = F.read_idl(path)
        assert np.array_equal(data, data2) and hdr["size"] == hdr2["size"] and hdr["name"] == hdr2["name"]
        out = tmp_path / f"{name}.idl"
        host.idl_write(out, data, hdr["name"], hdr["scan_range"], hdr["offset"], hdr["bias"], hdr["setpoint"],
                       date=hdr["date"])
        assert out.read_bytes() == open(path, "rb").read()


def test_cli_josephson_needs_scmodel(built_lib, tmp_path):
    """output=josephson with scmodel=false stops before any device work, with the
    reference's message (src/calcqpi.cc:458-461)."""
    import shutil
    d, meta, ref = load("c1_idl")
    for f in ("model_hr.dat", "orbitals.idl", "input.cfg"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    with open(tmp_path / "input.cfg", "a") as fh:
        fh.write("output=josephson;\ndeltat=0.01;\n")
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Josephson-mode" in r.stdout and "using deltat=0.01, etat=0.05." in r.stdout
    assert "josephson-mode with scmodel=false makes no sense" in r.stdout


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("xsf")])
def test_xsf_orbital_cache_matches_restatement(built_lib, name):
    """cqpi_xsf_orbital_cache (C++) against the restatement of xcfloader + the XSF
    wannierfunctions constructor, which the golden tests pin to the reference."""
    from cqpi import host as Hh
    d, meta, ref = load(name)
    spec = meta["orbitals"][1]
    pre = spec.get("prearr", [1.0] * len(spec["names"]))
    for q in range(len(spec["names"])):
        path = os.path.join(d, "orb%d.xsf" % q)
        got = Hh.xsf_orbital_cache(path, spec["zheight"], meta["w"], meta["os"], pre[q])
        want = F.xsf_orbital_cache(path, spec["zheight"], meta["w"], meta["os"], pre[q])
        assert np.array_equal(got, want)
        assert np.array_equal(got, ref["wf"][q])


def test_xsf_errors(built_lib, tmp_path):
    from cqpi import host as Hh
    with pytest.raises(Hh.HostError):
        Hh.xsf_orbital_cache(str(tmp_path / "missing.xsf"), 0.5, 1, 2)
    d, meta, ref = load("xsf_t2g")
    txt = open(os.path.join(d, "orb0.xsf")).read()
    bad = tmp_path / "bad.xsf"
    bad.write_text(txt.replace("3D_field", "2D_field"))
    with pytest.raises(Hh.HostError):
        Hh.xsf_orbital_cache(str(bad), 0.5, 1, 2)
    noconv = tmp_path / "noconv.xsf"
    lines = txt.split("\n")
    i = lines.index("CONVVEC")
    noconv.write_text("\n".join(lines[:i] + lines[i + 4:]))
    with pytest.raises(Hh.HostError):
        Hh.xsf_orbital_cache(str(noconv), 0.5, 1, 2)
    # height 0: the reference's getzheight returns NaN; the cache is zero
    assert not Hh.xsf_orbital_cache(os.path.join(d, "orb0.xsf"), 0.0, 1, 2).any()


def test_cli_orbitalfiles_missing_file(built_lib, tmp_path):
    """orbitalfiles with a file that cannot be read stops before any device work."""
    import shutil
    d, meta, ref = load("xsf_t2g")
    for f in ("model_hr.dat", "input.cfg", "orb0.xsf", "orb2.xsf"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Using Wannier90/XSF-orbitals for vacuum overlap." in r.stdout
    assert "Error loading wave function file orb1.xsf" in r.stdout
