"""GPU: Josephson mode (output=josephson, tmatrix::calcwannierjosephson, src/qpi.cc:953-1033).

* FP64 engine against the reference's own float64 maps (golden fixtures) to 1e-10 relative;
* mixed-precision engine (FP32 CUDA-core contraction, FP64 term1) against them to 1e-6;
* the narrow seam GPUQPI::wannierjosephson against the oracle to 1e-12;
* the mode's argument and state errors.
"""
import os

import numpy as np
import pytest

from golden_cases import energies, josephson, load

pytestmark = pytest.mark.gpu

JOS = ["josephson", "josephson_t2g", "josephson_spin"]


def _model(d, meta):
    from oracle import formats as F
    from oracle import oracle as O
    with open(os.path.join(d, "model_hr.dat")) as fh:
        hr = F.read_hr(fh.read(), scmodel=True)
    return O.Model.from_hr(hr, efermi=meta.get("fermi", 0.0))


def _engine(name, precision):
    import cqpi
    d, meta, ref = load(name)
    m = _model(d, meta)
    eng = cqpi.Engine(m, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=meta["maxband"],
                      spin=meta.get("spin", False), precision=precision)
    eng.set_orbitals(ref["wf"], ref["zero"])
    eng.set_scattering(ref["vscat"])
    dt, et = josephson(meta)
    eng.set_josephson(dt, et)
    return eng, meta, ref, m


@pytest.mark.parametrize("name", JOS)
def test_josephson_fp64_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, _ = _engine(name, cqpi.PREC_FP64)
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    err = np.abs(got - ref["ldos"]).max() / np.abs(ref["ldos"]).max()
    assert err < 1e-10, err
    eng.close()


@pytest.mark.parametrize("name", JOS)
def test_josephson_mixed_matches_reference(built_lib, name):
    import cqpi
    eng, meta, ref, _ = _engine(name, cqpi.PREC_MIXED)
    got = eng.run(energies(meta), f32=False, f64=True)[:, 0]
    for k in range(len(got)):
        err = np.abs(got[k] - ref["ldos"][k]).max() / np.abs(ref["ldos"][k]).max()
        assert err <= 1e-6, (k, err)
    # one spin block: the tcgen05 direct-window kernel; two: FP32 CUDA cores
    assert eng.contraction_kind() == ("fp32" if meta.get("spin") else "tcgen05")
    eng.close()


def test_josephson_seam_matches_oracle(built_lib):
    """GPUQPI::wannierjosephson(scat, g0, tip) + retrieveResult with the oracle's G0(R), T, tip."""
    from oracle import oracle as O
    eng, meta, ref, m = _engine("josephson_t2g", 0)
    kp = meta["kp"]
    ev, U = O.bands(m, kp)
    e = energies(meta)[0]
    g0r = O.realspace(O.greens_k(ev, U, kp, e, meta["eta"]))
    T = O.tmatrix(ref["vscat"], g0r[0, 0])
    tip = O.josephson_tip(e, *josephson(meta))
    eng.wannierjosephson(T, g0r, tip)
    got = eng.retrieve_result()
    want = O.wannier_josephson(meta["n"], kp, meta["os"], meta["w"], False, T, g0r, ref["wf"], tip, ref["zero"]).T
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    eng.close()


def test_josephson_mode_toggles_back_to_ldos(built_lib):
    import cqpi
    eng, meta, ref, m = _engine("josephson", cqpi.PREC_FP64)
    E = energies(meta)
    j1 = eng.run(E, f32=False, f64=True)
    eng.set_josephson(enable=False)
    ldos = eng.run(E, f32=False, f64=True)
    eng.set_josephson(*josephson(meta))
    j2 = eng.run(E, f32=False, f64=True)
    assert np.array_equal(j1, j2)
    plain = cqpi.Engine(m, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=meta["maxband"],
                        precision=cqpi.PREC_FP64)
    plain.set_orbitals(ref["wf"], ref["zero"])
    plain.set_scattering(ref["vscat"])
    assert np.array_equal(ldos, plain.run(E, f32=False, f64=True))
    plain.close()
    eng.close()


def test_josephson_errors(built_lib):
    import cqpi
    from cases import case
    # odd band count (the C2 model: 3 bands)
    m, p, wf, z, v, E = case("c2")
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"])
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.set_josephson(0.01)
    assert ex.value.code == cqpi.ERR_ARG
    eng.close()
    # maxband other than bands/2
    d, meta, ref = load("josephson_t2g")
    mm = _model(d, meta)
    eng = cqpi.Engine(mm, meta["n"], meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=mm.bands)
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.set_josephson(0.01)
    assert ex.value.code == cqpi.ERR_ARG
    eng.close()
    # the adjoint, fields of view and the plain seam are refused in Josephson mode
    eng, meta, ref, m = _engine("josephson_t2g", cqpi.PREC_MIXED)
    E = energies(meta)
    wn = meta["n"] * meta["os"]
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.adjoint(E, np.zeros((len(E), 1, wn, wn), np.float32))
    assert ex.value.code == cqpi.ERR_NOT_SUPPORTED
    with pytest.raises(cqpi.CqpiError) as ex:
        eng.wannierldos(np.eye(m.bands), np.zeros((meta["kp"], meta["kp"], m.bands, m.bands)))
    assert ex.value.code == cqpi.ERR_STATE
    eng.close()


def _bdg_c2_engine(precision, lattice=24, kpoints=256, contraction=None, monkeypatch=None):
    import cqpi
    from cqpi import workloads as W
    if contraction:
        monkeypatch.setenv("CQPI_CONTRACTION", contraction)
    c, m, wf = W.config("CJ")
    eng = cqpi.Engine(m, lattice, kpoints, c.oversamp, c.window, 0.01, maxband=3, precision=precision)
    eng.set_orbitals(wf)
    eng.set_scattering(np.array(c.scattering, complex))
    eng.set_josephson(0.001, 0.01)
    if contraction:
        monkeypatch.delenv("CQPI_CONTRACTION")
    return eng


def test_josephson_tensor_cores_on_bdg_t2g(built_lib, monkeypatch):
    """6-band BdG t2g model, C2 orbitals and window: the tcgen05 Josephson contraction against
    the FP64 engine (1e-6) and against the FP32 CUDA-core kernel.  (At E = 0 this model's
    Josephson map vanishes to rounding, ~1e-18, so a relative bar is meaningless there.)"""
    import cqpi
    E = np.array([-0.08, -0.02, 0.006, 0.03, 0.09])
    e64 = _bdg_c2_engine(cqpi.PREC_FP64)
    ref = e64.run(E, f32=False, f64=True)
    e64.close()
    tc = _bdg_c2_engine(cqpi.PREC_MIXED)
    assert tc.contraction_kind() == "tcgen05"
    got = tc.run(E, f32=False, f64=True)
    tc.close()
    f32 = _bdg_c2_engine(cqpi.PREC_MIXED, contraction="fp32", monkeypatch=monkeypatch)
    assert f32.contraction_kind() == "fp32"
    g32 = f32.run(E, f32=False, f64=True)
    f32.close()
    for e in range(len(E)):
        scale = np.abs(ref[e, 0]).max()
        assert np.abs(got[e, 0] - ref[e, 0]).max() <= 1e-6 * scale, (E[e], np.abs(got[e, 0] - ref[e, 0]).max() / scale)
        assert np.abs(g32[e, 0] - ref[e, 0]).max() <= 1e-6 * scale


def test_josephson_fields_of_view_crop_full_maps(built_lib):
    """cqpi_run_fov in the Josephson mode: every map equals the centred crop of cqpi_run's."""
    import cqpi
    import torch
    E = np.array([-0.05, 0.04])
    eng = _bdg_c2_engine(cqpi.PREC_MIXED)
    full = eng.run(E, f32=True, f64=False)
    fov = np.array([[8], [16]], np.int32)
    os_ = 10
    tot = int(sum((f * os_) ** 2 for f in fov.reshape(-1)))
    buf = torch.zeros(tot, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    eng.run_fov(E, fov, buf.data_ptr())
    eng.synchronize()
    flat = buf.cpu().numpy()
    off, n = 0, 24
    for k, f in enumerate(fov.reshape(-1)):
        w = f * os_
        got = flat[off:off + w * w].reshape(w, w)
        lo = (n // 2 - f // 2) * os_
        assert np.array_equal(got, full[k, 0, lo:lo + w, lo:lo + w])
        off += w * w
    eng.close()


def test_josephson_bulk_and_piecewise_fetch_agree(built_lib, monkeypatch):
    """6-band columns (1.4 KB) are fetched by one bulk copy each; fetched instead as 8-byte
    cp.async pieces (CQPI_TC_NBULK=0), or half and half, the staged values and so the maps
    are the same bit for bit."""
    import cqpi
    E = np.array([-0.07, 0.02, 0.05])
    eng = _bdg_c2_engine(cqpi.PREC_MIXED)
    assert eng.contraction_kind() == "tcgen05"
    bulk = eng.run(E, f32=True, f64=False)
    for nb in ("0", "5"):
        monkeypatch.setenv("CQPI_TC_NBULK", nb)
        assert np.array_equal(eng.run(E, f32=True, f64=False), bulk), nb
    eng.close()


def test_josephson_bulk_fetch_timeout_is_reported_and_handle_recovers(built_lib, monkeypatch):
    """Fault injection without a GPU fault on the bulk-copy producer: with CQPI_TEST_STALL=1
    the MMA warp waits (bounded) on a barrier nothing arrives on, the producer times out on
    its next window-empty wait with bulk copies of later tiles in flight, waits (bounded) for
    them to land and returns; the call reports CQPI_ERR_TIMEOUT and the handle then runs
    normally.  (8 energies: 576 tiles, so every block has more tiles than the two window
    buffers that need no window-empty wait.)"""
    import cqpi
    E = np.linspace(-0.06, 0.06, 8)
    eng = _bdg_c2_engine(cqpi.PREC_MIXED)
    assert eng.contraction_kind() == "tcgen05"
    good = eng.run(E, f32=True, f64=False)
    monkeypatch.setenv("CQPI_TEST_STALL", "1")
    with pytest.raises(cqpi.CqpiError) as ei:
        eng.run(E, f32=True, f64=False)
    assert ei.value.code == cqpi.ERR_TIMEOUT
    monkeypatch.delenv("CQPI_TEST_STALL")
    assert np.array_equal(eng.run(E, f32=True, f64=False), good)
    eng.close()
