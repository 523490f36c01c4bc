"""The calcqpi CLI (drop-in for the reference's `calcqpi inputfile`) on every golden case."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from golden_cases import NAMES, load
from oracle import formats as F

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", NAMES)
def test_cli_reproduces_reference_output(built_lib, name, tmp_path):
    d, meta, ref = load(name)
    for f in os.listdir(d):
        if f in ("model_hr.dat", "surf_hr.dat", "orbitals.idl", "input.cfg") or f.endswith(".xsf"):
            shutil.copy(os.path.join(d, f), tmp_path / f)
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got_path, ref_path = tmp_path / "ref_qpi.idl", os.path.join(d, "ref_qpi.idl")
    with open(got_path, "rb") as a, open(ref_path, "rb") as b:
        ga, gb = a.read().split(b"\n", 12), b.read().split(b"\n", 12)
    # header: identical except line 2 (ctime of the run)
    assert ga[0] == gb[0] and ga[2:12] == gb[2:12]
    hg, dg = F.read_idl(got_path)
    hr_, dr = F.read_idl(ref_path)
    assert dg.shape == dr.shape
    err = np.abs(dg.astype(np.float64) - dr).max() / np.abs(dr).max()
    assert err <= 2e-7, err
    if os.path.exists(os.path.join(d, "ref_dos.txt")):
        with open(tmp_path / "ref_dos.txt") as a, open(os.path.join(d, "ref_dos.txt")) as b:
            assert a.read() == b.read()
    if os.path.exists(os.path.join(d, "ref_wf.idl")):
        hw, dw = F.read_idl(tmp_path / "ref_wf.idl")
        hw0, dw0 = F.read_idl(os.path.join(d, "ref_wf.idl"))
        assert hw["name"] == hw0["name"] and dw.shape == dw0.shape
        assert np.abs(dw - dw0).max() <= 1e-7 * np.abs(dw0).max()


def test_cli_flush_and_resume(built_lib, tmp_path):
    """flush=true writes the map group by group; an interrupted run (here: the progress file
    cut back to layer 0 and the other layers zeroed on disk) continues with resume=true,
    computing only the missing layers, and ends with the map of a one-shot run."""
    d, meta, ref = load("c2_analytic")
    for f in ("model_hr.dat", "input.cfg"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    base = (tmp_path / "input.cfg").read_text()
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    oneshot = (tmp_path / "ref_qpi.idl").read_bytes()
    _, full = F.read_idl(tmp_path / "ref_qpi.idl")
    assert full.shape[0] >= 2
    (tmp_path / "f.cfg").write_text(base.replace('qpifile="ref_qpi.idl";', 'qpifile="flush.idl";') + "flush=true;\n")
    r = subprocess.run([built_lib["cli"], "f.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert not (tmp_path / "flush.idl.progress").exists()
    got = (tmp_path / "flush.idl").read_bytes()
    # identical header except the run date, identical data
    assert got.split(b"\n", 12)[2:] == oneshot.split(b"\n", 12)[2:]
    # interrupt: only layer 0 is on disk
    from cqpi import host
    host.idl_write_layers(tmp_path / "flush.idl", 1, np.zeros_like(full[1:]))
    (tmp_path / "flush.idl.progress").write_text("0\n")
    (tmp_path / "r.cfg").write_text(base.replace('qpifile="ref_qpi.idl";', 'qpifile="flush.idl";') + "resume=true;\n")
    r = subprocess.run([built_lib["cli"], "r.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "1 of %d layers already computed" % full.shape[0] in r.stdout
    assert "Calculating layer 0 " not in r.stdout and "Calculating layer 1 " in r.stdout
    _, res = F.read_idl(tmp_path / "flush.idl")
    assert np.array_equal(res[0], full[0])
    assert np.abs(res.astype(np.float64) - full).max() <= 2e-7 * np.abs(full).max()
    # a file of another calculation is not resumed over
    (tmp_path / "flush.idl.progress").write_text("0\n")
    cfg = base.replace('qpifile="ref_qpi.idl";', 'qpifile="flush.idl";') + "resume=true;\n"
    cfg = re.sub(r"layers=(\d+);", lambda m: "layers=%d;" % (int(m.group(1)) + 1), cfg)
    (tmp_path / "x.cfg").write_text(cfg)
    r = subprocess.run([built_lib["cli"], "x.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "does not belong" in r.stdout
