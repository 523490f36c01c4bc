"""The calcqpi CLI (drop-in for the reference's `calcqpi inputfile`) on every golden case."""
import os
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


def test_cli_rejects_out_of_scope_modes(built_lib, tmp_path):
    d, meta, ref = load("c1_idl")
    for f in ("model_hr.dat", "orbitals.idl", "input.cfg"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    with open(tmp_path / "input.cfg", "a") as fh:
        fh.write('bsfile="bs.idl";\n')
    r = subprocess.run([built_lib["cli"], "input.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "not supported" in r.stdout
