"""GPU: the proximity-list form of the LDOS (threshold / spinarr keywords,
tmatrix::calcwannierldos(os, w, flaglist), src/qpi.cc:1085-1134).

* FP64 engine against the reference's float64 maps (golden fixtures) to 1e-10 relative;
* mixed engine (FP32 G0(R), T and list sums, FP64 term1) against them to 1e-6;
* threshold 0 keeps every non-zero term: equal to the full window sum;
* the narrow seam GPUQPI::wannierldoslist against the oracle to 1e-12;
* list counts, rebuild on new orbitals, refused calls.
"""
import os
import re

import numpy as np
import pytest

from golden_cases import energies, load

pytestmark = pytest.mark.gpu

THR = ["threshold_c2", "threshold_spin", "threshold_spinarr"]


def _engine(name, precision):
    import cqpi
    from oracle import formats as F
    from oracle import oracle as O
    d, meta, ref = load(name)
    with open(os.path.join(d, "model_hr.dat")) as fh:
        hr = F.read_hr(fh.read(), scmodel=meta.get("scmodel", False))
    m = O.Model.from_hr(hr, efermi=meta.get("fermi", 0.0))
    eng = cqpi.Engine(m, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=meta["maxband"],
                      spin=meta.get("spin", False), precision=precision)
    eng.set_orbitals(ref["wf"], ref["zero"])
    eng.set_scattering(ref["vscat"])
    count = eng.set_threshold(meta["threshold"], meta.get("spinarr"))
    return eng, meta, ref, m, d, count


@pytest.mark.parametrize("name", THR)
def test_threshold_fp64_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, m, d, count = _engine(name, cqpi.PREC_FP64)
    with open(os.path.join(d, "ref_stdout.txt")) as fh:
        assert count == int(re.search(r"Threshold list has (\d+)/", fh.read()).group(1))
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    err = np.abs(got - ref["ldos"]).max() / np.abs(ref["ldos"]).max()
    assert err < 1e-10, err
    eng.close()


@pytest.mark.parametrize("name", THR)
def test_threshold_mixed_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, *_ = _engine(name, cqpi.PREC_MIXED)
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    for k in range(len(got)):
        err = np.abs(got[k] - ref["ldos"][k]).max() / np.abs(ref["ldos"][k]).max()
        assert err <= 1e-6, (k, err)
    eng.close()


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
@pytest.mark.parametrize("name", ["c2", "c3"])
def test_threshold_zero_equals_full_sum(built_lib, name, precision, tol):
    import cqpi
    from cases import case
    m, p, wf, z, v, E = case(name)
    full = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                       precision=cqpi.PREC_FP64)
    full.set_orbitals(wf, z)
    full.set_scattering(v)
    ref = full.run(E, f32=False, f64=True)
    full.close()
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                      precision=precision)
    eng.set_orbitals(wf, z)
    eng.set_scattering(v)
    assert eng.set_threshold(0.0) > 0
    got = eng.run(E, f32=False, f64=True)
    for e in range(len(E)):
        err = np.abs(got[e, 0] - ref[e, 0]).max() / np.abs(ref[e, 0]).max()
        assert err <= tol, (e, err)
    # NaN switches back to the full window sum
    eng.set_threshold(None)
    back = eng.run(E, f32=False, f64=True)
    if precision == 0:
        assert np.array_equal(back, ref)
    eng.close()


def test_threshold_seam_matches_oracle(built_lib):
    """GPUQPI::wannierldoslist + retrieveResult with the oracle's G0(R), T and list."""
    from oracle import oracle as O
    eng, meta, ref, m, d, count = _engine("threshold_c2", 0)
    kp = meta["kp"]
    ev, U = O.bands(m, kp)
    e = energies(meta)[1]
    g0r = O.realspace(O.greens_k(ev, U, kp, e, meta["eta"]))
    T = O.tmatrix(ref["vscat"], g0r[0, 0])
    ent, fac = O.threshold_list(meta["w"], meta["os"], ref["wf"], meta["threshold"], meta["maxband"])
    assert len(fac) == count
    eng.wannierldoslist(T, g0r)
    got = eng.retrieve_result()
    want = O.wannier_ldos_list(meta["n"], kp, meta["os"], meta["w"], T, g0r, ent, fac).T
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    eng.close()


def test_threshold_rebuilt_on_new_orbitals_and_refusals(built_lib):
    import cqpi
    eng, meta, ref, m, d, count = _engine("threshold_c2", cqpi.PREC_MIXED)
    E = energies(meta)
    a = eng.run(E, f32=False, f64=True)
    eng.set_orbitals(0.5 * ref["wf"], ref["zero"])     # same list (relative threshold), maps x 1/4
    b = eng.run(E, f32=False, f64=True)
    assert np.abs(4 * b - a).max() <= 1e-6 * np.abs(a).max()
    wn = meta["n"] * meta["os"]
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.adjoint(E, np.zeros((len(E), 1, wn, wn), np.float32))
    assert ex.value.code == cqpi.ERR_NOT_SUPPORTED
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.autotune(E)
    assert ex.value.code == cqpi.ERR_NOT_SUPPORTED
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.wannierldos(np.eye(m.bands), np.zeros((meta["kp"], meta["kp"], m.bands, m.bands)))
    assert ex.value.code == cqpi.ERR_STATE
    eng.close()


def test_explicit_list_equals_threshold_list(built_lib):
    """cqpi_set_list with the oracle's mkthresholdlist entries (the form the reference's
    list-mode GPU backend receives) gives the same maps as cqpi_set_threshold, and survives
    new orbitals unchanged."""
    import cqpi
    from oracle import oracle as O
    eng, meta, ref, m, d, count = _engine("threshold_spin", cqpi.PREC_FP64)
    E = energies(meta)
    a = eng.run(E, f32=False, f64=True)
    wz = ref["wf"] * (1 - ref["zero"][:len(ref["wf"]), None, None])
    ent, fac = O.threshold_list(meta["w"], meta["os"], wz, meta["threshold"], meta["maxband"], True)
    eng.set_list(ent, fac)
    b = eng.run(E, f32=False, f64=True)
    assert np.array_equal(a, b)
    eng.set_orbitals(2.0 * ref["wf"], ref["zero"])      # an explicit list is not rebuilt
    c = eng.run(E, f32=False, f64=True)
    assert np.array_equal(a, c)
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.set_list(np.array([[0, 0, 0, 0, eng.bands]]), np.array([1.0]))
    assert ex.value.code == cqpi.ERR_ARG
    eng.close()
