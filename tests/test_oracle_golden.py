"""Pin the oracle to the reference: golden outputs of the reference's own sources."""
import os

import numpy as np
import pytest

from golden_cases import NAMES, energies, josephson, load, uspf_pos, uspf_pre
from oracle import formats as F
from oracle import oracle as O


def _model(d, meta):
    with open(os.path.join(d, "model_hr.dat")) as fh:
        hr = F.read_hr(fh.read(), scmodel=meta.get("scmodel", False))
    return O.Model.from_hr(hr, efermi=meta.get("fermi", 0.0))


def _smodel(d, meta):
    if not meta.get("surface_model"):
        return None
    with open(os.path.join(d, "surf_hr.dat")) as fh:
        hr = F.read_hr(fh.read(), scmodel=meta.get("scmodel", False))
    return O.Model.from_hr(hr, efermi=meta.get("fermi", 0.0))


def _g0r(m, meta, d, e, cache):
    if meta.get("green"):
        return O.realspace(O.surface_greens_k(m, meta["kp"], e, meta["eta"], meta.get("epserr", 1e-5),
                                              meta["green"] == "surface", _smodel(d, meta)))
    if "eig" not in cache:
        cache["eig"] = O.bands(m, meta["kp"])
    ev, U = cache["eig"]
    return O.realspace(O.greens_k(ev, U, meta["kp"], e, meta["eta"]))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_float64(name):
    d, meta, ref = load(name)
    m = _model(d, meta)
    E = energies(meta)
    out = meta.get("output", "wannier")
    kp = meta["n"] if out == "spf" else meta["kp"]
    maps = O.run(m, meta["n"], kp, meta["os"], meta["w"], meta["eta"], E, ref["vscat"], ref["wf"],
                 ref["zero"], m=meta["maxband"], spin=meta.get("spin", False), josephson=josephson(meta),
                 threshold=meta.get("threshold"), spinarr=meta.get("spinarr"), green=meta.get("green"),
                 epserr=meta.get("epserr", 1e-5), smodel=_smodel(d, meta), output=out, pos=uspf_pos(meta),
                 prearr=uspf_pre(meta))
    err = np.abs(maps - ref["ldos"]).max() / np.abs(ref["ldos"]).max()
    assert err < 1e-10, err
    if out in ("spf", "uspf"):
        return
    # tmatrix::calcdos = -sum_i<maxband Im G0(R=0)_ii  (src/qpi.cc:856-862)
    cache = {}
    for k, e in enumerate(E):
        g00 = _g0r(m, meta, d, e, cache)[0, 0]
        dos = -np.imag(np.diag(g00))[:meta["maxband"]].sum()
        assert abs(dos - ref["dos"][k]) < 1e-12 * max(1.0, abs(ref["dos"][k]))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_cli_float32(name):
    d, meta, ref = load(name)
    hdr, data = F.read_idl(os.path.join(d, "ref_qpi.idl"))
    # spectral functions are lattice x lattice maps (src/calcqpi.cc:647-652)
    wn = meta["n"] * (1 if meta.get("output") in ("spf", "uspf") else meta["os"])
    assert hdr["size"] == (wn, wn, meta["layers"])
    # the CLI's float32 map is the float64 map rounded (src/idl.cc:90-92)
    assert np.array_equal(data, ref["ldos"].astype(np.float32)) or \
        np.abs(data - ref["ldos"]).max() <= 2e-7 * np.abs(ref["ldos"]).max()


def test_numpy_restatement_matches_reference():
    for name in ["c2_pad", "edge_odd", "scmodel"]:
        d, meta, ref = load(name)
        m = _model(d, meta)
        E = energies(meta)
        for k, e in enumerate(E):
            g0r = O.np_greens_r(m, meta["kp"], e, meta["eta"])
            T = O.tmatrix(ref["vscat"], g0r[0, 0])
            got = O.np_wannier_ldos(meta["n"], meta["kp"], meta["os"], meta["w"], meta["maxband"],
                                    meta.get("spin", False), T, g0r, ref["wf"], ref["zero"]).T
            err = np.abs(got - ref["ldos"][k]).max() / np.abs(ref["ldos"][k]).max()
            assert err < 1e-10, (name, err)


@pytest.mark.parametrize("name", [n for n in NAMES if os.path.exists(os.path.join(
    os.path.dirname(os.path.abspath(__file__)), "golden", n, "ref_wf.idl"))])
def test_orbital_cache_matches_reference(name):
    d, meta, ref = load(name)
    hdr, data = F.read_idl(os.path.join(d, "ref_wf.idl"))
    norb = ref["wf"].shape[0]
    cube = np.transpose(data, (0, 2, 1))[:norb]   # file [orb][y][x] -> [orb][x][y]
    assert np.abs(cube - ref["wf"].astype(np.float32)).max() <= 1e-7 * max(np.abs(ref["wf"]).max(), 1e-30)
    assert hdr["name"].startswith("Wannier function file for model_hr.dat with window=")


def test_idl_writer_reproduces_reference_bytes():
    for name in NAMES:
        d, meta, ref = load(name)
        path = os.path.join(d, "ref_qpi.idl")
        hdr, data = F.read_idl(path)
        tmp = os.path.join(d, "_tmp.idl")
        try:
            F.write_idl(tmp, data, hdr["name"], hdr["scan_range"], hdr["offset"], hdr["bias"], hdr["setpoint"],
                        date=hdr["date"])
            with open(tmp, "rb") as a, open(path, "rb") as b:
                assert a.read() == b.read()
        finally:
            os.remove(tmp)


def test_config_restatement_reads_inputs():
    d, meta, ref = load("edge_odd")
    with open(os.path.join(d, "input.cfg")) as fh:
        lf = F.LoadConfig(fh.read())
    assert lf.getintvalue("lattice") == meta["n"]
    assert lf.getvector("phase") == [0.5, 0.3]
    assert lf.getstring("tbfile") == "model_hr.dat"
    assert lf.getlist("orbitals") == ["s"]
    assert lf.getvector("pos[0]") == [0.1, 0.2, 0.1]
    assert "wffile" in lf.unused()
    bad = F.LoadConfig("lattice=3\nx = 4;\n# c=1;\nkpoints=8;\nkpoints=16;\n")
    assert bad.warnings == ["lattice=3"]
    assert not bad.probefield("x")          # keys are not trimmed (include/parser.h:44)
    assert bad.getintvalue("kpoints") == 16  # the last value wins (include/parser.h:117-121)


def test_josephson_tip_matches_complex_arithmetic():
    """The tip factor of src/calcqpi.cc:705-708 against numpy's principal square root,
    including energies near zero and below the tip gap."""
    for e in [-0.3, -0.02, -1e-9, 0.0, 1e-9, 0.004, 0.02, 0.5]:
        for dt, et in [(0.001, 0.005), (0.02, 0.01), (0.05, 1e-4)]:
            want = 1j * (-np.copysign(1.0, e) * np.pi * dt) / np.sqrt(complex(e, et) ** 2 - dt * dt)
            got = O.josephson_tip(e, dt, et)
            assert abs(got - want) <= 1e-14 * abs(want), (e, dt, et, got, want)


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("threshold")])
def test_threshold_list_count_matches_reference_log(name):
    """mkthresholdlist restated: the entry count the reference's CLI logged."""
    import re
    d, meta, ref = load(name)
    with open(os.path.join(d, "ref_stdout.txt")) as fh:
        want = int(re.search(r"Threshold list has (\d+)/", fh.read()).group(1))
    wz = ref["wf"] * (1 - ref["zero"][:len(ref["wf"]), None, None])
    ent, fac = O.threshold_list(meta["w"], meta["os"], wz, meta["threshold"], meta["maxband"],
                                meta.get("spin", False), meta.get("spinarr"))
    assert len(fac) == want


def test_dosfile_matches_reference_text():
    """dosfile (src/calcqpi.cc:336-391): energies dosl + k (dosh - dosl) / doslayers and
    -sum_i<maxband Im G0(R=0)_ii, written with the stream's default 6 significant digits."""
    d, meta, ref = load("dos_c2")
    m = _model(d, meta)
    dl, dh = meta["dosfile"]["energies"]
    L = meta["dosfile"]["layers"]
    step = (dh - dl) / L
    ev, U = O.bands(m, meta["kp"])
    lines = []
    for k in range(L):
        e = dl + k * step
        g00 = O.realspace(O.greens_k(ev, U, meta["kp"], e, meta["eta"]))[0, 0]
        dos = -np.imag(np.diag(g00))[:meta["maxband"]].sum()
        lines.append("%s %s" % (F.cxx_double(e), F.cxx_double(dos)))
    with open(os.path.join(d, "ref_dos.txt")) as fh:
        assert fh.read().splitlines() == lines
