"""GPU: surface / bulk Green's functions (green=surface|bulk, stbfile, epserr;
tmatrix::calcsurfacegreensfunction, src/qpi.cc:488-554).

* FP64 engine against the reference's float64 maps (golden fixtures) to 1e-10 relative;
* mixed engine against them to 1e-6;
* the G0(R) box against the oracle's decimation;
* switching back to the eigen-based G0, non-convergence reported as a status, refusals.
"""
import os

import numpy as np
import pytest

from golden_cases import energies, load

pytestmark = pytest.mark.gpu

SURF = ["surface_c1", "bulk_t2g", "surface_t2g"]


def _models(d, meta):
    from oracle import formats as F
    from oracle import oracle as O
    with open(os.path.join(d, "model_hr.dat")) as fh:
        m = O.Model.from_hr(F.read_hr(fh.read()), efermi=meta.get("fermi", 0.0))
    sm = None
    if meta.get("surface_model"):
        with open(os.path.join(d, "surf_hr.dat")) as fh:
            sm = O.Model.from_hr(F.read_hr(fh.read()), efermi=meta.get("fermi", 0.0))
    return m, sm


def _engine(name, precision):
    import cqpi
    d, meta, ref = load(name)
    m, sm = _models(d, meta)
    eng = cqpi.Engine(m, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=meta["maxband"],
                      precision=precision)
    eng.set_orbitals(ref["wf"], ref["zero"])
    eng.set_scattering(ref["vscat"])
    eng.set_greens(meta["green"], meta.get("epserr", 1e-5), sm)
    return eng, meta, ref, m, sm


@pytest.mark.parametrize("name", SURF)
def test_surface_fp64_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, *_ = _engine(name, cqpi.PREC_FP64)
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    err = np.abs(got - ref["ldos"]).max() / np.abs(ref["ldos"]).max()
    assert err < 1e-10, err
    eng.close()


@pytest.mark.parametrize("name", SURF)
def test_surface_mixed_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, *_ = _engine(name, cqpi.PREC_MIXED)
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    for k in range(len(got)):
        err = np.abs(got[k] - ref["ldos"][k]).max() / np.abs(ref["ldos"][k]).max()
        assert err <= 1e-6, (k, err)
    eng.close()


def test_surface_box_matches_oracle(built_lib):
    from oracle import oracle as O
    eng, meta, ref, m, sm = _engine("surface_c1", 0)
    kp = meta["kp"]
    e = energies(meta)[0]
    box, rb = eng.greens_box(e)
    g0r = O.realspace(O.surface_greens_k(m, kp, e, meta["eta"], meta.get("epserr", 1e-5), True, sm))
    idx = np.arange(-rb, rb + 1) % kp
    want = g0r[np.ix_(idx, idx)]
    assert np.abs(box - want).max() <= 1e-12 * np.abs(want).max()
    eng.close()


def test_surface_mode_switches_back_and_reports_non_convergence(built_lib, monkeypatch):
    import cqpi
    eng, meta, ref, m, sm = _engine("bulk_t2g", cqpi.PREC_FP64)
    E = energies(meta)
    a = eng.run(E, f32=False, f64=True)
    eng.set_greens("normal")
    normal = eng.run(E, f32=False, f64=True)
    plain = cqpi.Engine(m, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], precision=cqpi.PREC_FP64)
    plain.set_orbitals(ref["wf"], ref["zero"])
    plain.set_scattering(ref["vscat"])
    assert np.array_equal(normal, plain.run(E, f32=False, f64=True))
    plain.close()
    eng.set_greens("bulk", meta.get("epserr", 1e-5))
    monkeypatch.setenv("CQPI_SURFACE_MAX_ITER", "1")     # one doubling: not yet below epserr
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.run(E, f32=False, f64=True)
    assert ex.value.code == cqpi.ERR_NOT_CONVERGED
    monkeypatch.delenv("CQPI_SURFACE_MAX_ITER")
    assert np.array_equal(eng.run(E, f32=False, f64=True), a)
    wn = meta["n"] * meta["os"]
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.adjoint(E, np.zeros((len(E), 1, wn, wn), np.float32))
    assert ex.value.code == cqpi.ERR_NOT_SUPPORTED
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.get_bands()
    assert ex.value.code == cqpi.ERR_NOT_SUPPORTED
    eng.close()
