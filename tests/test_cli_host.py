"""calcqpi CLI runs that need no GPU (output=nomode creates no engine), against the reference's
own outputs:

  * the band-structure histogram of the bsfile keyword (cqpi_band_histogram, on the host cores
    as the reference's driver computes it): tests/golden/bs_*/ from tightbind::calcbst3dhisthr
    (src/tightbinding.cc:1158-1193) through the reference CLI (a 3-band model with a Fermi
    energy, a BdG model with conjugated hole terms, a layered model with R_z != 0 terms), and
    the oracle's restatement (oracle.band_histogram), itself pinned on those outputs;
  * the orbital setup and wffile output of every golden case that has one (analytic, IDL and
    XSF orbitals, padding, spin duplication).
"""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = sorted(os.path.basename(d) for d in glob.glob(os.path.join(GOLDEN, "bs_*")))


@pytest.mark.parametrize("case", CASES)
def test_cli_bsfile_matches_reference(built_lib, tmp_path, case):
    src = os.path.join(GOLDEN, case)
    for f in ("model_hr.dat", "input.cfg"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    cfg = (tmp_path / "input.cfg").read_text().replace('bsfile="ref_bs.idl";', 'bsfile="ours.idl";')
    (tmp_path / "input.cfg").write_text(cfg)
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "... done and saved to ours.idl." in r.stdout
    hr, ref = F.read_idl(os.path.join(src, "ref_bs.idl"))
    ho, ours = F.read_idl(str(tmp_path / "ours.idl"))
    for key in ("name", "size", "scan_range", "offset", "bias", "setpoint"):
        assert ho[key] == hr[key], (key, ho[key], hr[key])
    assert np.abs(ref).max() > 0
    # eigenvalues from a different Jacobi order: agreement to float32 rounding
    assert np.abs(ours.astype(np.float64) - ref).max() <= 1e-6 * np.abs(ref).max()


def _oracle_model(case, scmodel, efermi):
    from oracle import oracle as O
    with open(os.path.join(GOLDEN, case, "model_hr.dat")) as fh:
        hr = F.read_hr(fh.read(), scmodel=scmodel)
    return O.Model.from_hr(hr, efermi=efermi)


def _bs_keys(case):
    """(pix, oversamp, le, ue, layers, scmodel, efermi) of a golden case's input.cfg."""
    kv = {}
    for line in open(os.path.join(GOLDEN, case, "input.cfg")):
        if "=" in line and not line.startswith("#"):
            k, v = line.split("=", 1)
            kv[k.strip()] = v.strip().rstrip(";")
    le, ue = (float(x) for x in kv["bsenergies"].strip("()").split(","))
    return (int(kv["bslattice"]), int(kv["bsoversamp"]), le, ue, int(kv["bslayers"]),
            kv.get("scmodel") == "true", float(kv.get("fermi", 0.0)))


@pytest.mark.parametrize("case", CASES)
def test_oracle_histogram_matches_reference(case):
    """Pins the oracle's restatement (oracle.band_histogram) on the reference's outputs."""
    from oracle import oracle as O
    pix, os_, le, ue, layers, scmodel, efermi = _bs_keys(case)
    got = O.band_histogram(_oracle_model(case, scmodel, efermi), pix, os_, le, ue, layers)
    _, ref = F.read_idl(os.path.join(GOLDEN, case, "ref_bs.idl"))
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()


def test_band_histogram_matches_oracle(built_lib):
    """cqpi_band_histogram against the oracle on a model and range no golden uses."""
    from oracle import oracle as O
    om = _oracle_model("bs_bdg", True, 0.02)
    from cqpi import host
    pix, os_, le, ue, layers = 6, 3, -0.3, 0.3, 9
    out = host.band_histogram(om, pix, os_, le, ue, layers)
    want = O.band_histogram(om, pix, os_, le, ue, layers)
    assert np.abs(want).max() > 0
    np.testing.assert_allclose(out, want, rtol=1e-10, atol=1e-12 * np.abs(want).max())


def _wf_cases():
    from golden_cases import NAMES
    return [n for n in NAMES if os.path.exists(os.path.join(GOLDEN, n, "ref_wf.idl"))]


@pytest.mark.parametrize("name", _wf_cases())
def test_cli_wffile_matches_reference_without_gpu(built_lib, tmp_path, name):
    """The orbital setup of the CLI (analytic, IDL and XSF orbitals, padding, spin duplication)
    and its wffile output, in an output=nomode run that needs no GPU, against the reference's
    wffile of the same golden case."""
    src = os.path.join(GOLDEN, name)
    for f in os.listdir(src):
        if f in ("model_hr.dat", "surf_hr.dat", "orbitals.idl") or f.endswith(".xsf"):
            shutil.copy(os.path.join(src, f), tmp_path / f)
    lines = []
    for line in open(os.path.join(src, "input.cfg")):
        key = line.split("=")[0].strip()
        if key in ("output", "dosfile", "qpifile"):
            continue
        lines.append(line.rstrip("\n").replace('wffile="ref_wf.idl";', 'wffile="ours_wf.idl";'))
    lines.append("output=nomode;")
    (tmp_path / "input.cfg").write_text("\n".join(lines) + "\n")
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    hw, dw = F.read_idl(str(tmp_path / "ours_wf.idl"))
    hr, dr = F.read_idl(os.path.join(src, "ref_wf.idl"))
    for key in ("name", "size", "scan_range", "offset", "bias", "setpoint"):
        assert hw[key] == hr[key], (key, hw[key], hr[key])
    assert np.abs(dw - dr).max() <= 1e-7 * max(np.abs(dr).max(), 1e-30)


def test_cli_bsfile_rejects_an_empty_energy_range(built_lib, tmp_path):
    src = os.path.join(GOLDEN, "bs_t2g")
    for f in ("model_hr.dat", "input.cfg"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    cfg = (tmp_path / "input.cfg").read_text().replace("bsenergies=(-0.6,0.4);", "bsenergies=(0.4,-0.6);")
    (tmp_path / "input.cfg").write_text(cfg)
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "band-structure histogram" in r.stdout


def _ref_keywords(prog):
    with open(os.path.join(GOLDEN, "ref_%s_keywords.txt" % prog)) as fh:
        return {l.strip() for l in fh if l.strip() and not l.startswith("#")}


def _read_keywords(source):
    """Keys our program looks up (InputFile::has / field / str / value / ivalue / vec / list /
    strlist with a literal name)."""
    import re
    with open(source) as fh:
        return set(re.findall(r'lf\.(?:has|field|str|value|ivalue|vec|list|strlist)\("([^"]+)"\)', fh.read()))


@pytest.mark.parametrize("prog,source", [("calcqpi", "calcqpi_main.cc"),
                                         ("mkwavefunctions", "mkwavefunctions_main.cc")])
def test_every_reference_keyword_is_read(prog, source):
    """Every keyword the reference's program reads (tests/golden/ref_<prog>_keywords.txt, taken
    from its sources) is read by ours: a reference input file loses nothing."""
    ours = _read_keywords(os.path.join(os.path.dirname(HERE), "calcqpi-release_gb300", "host", source))
    missing = sorted(_ref_keywords(prog) - ours)
    assert not missing, missing
