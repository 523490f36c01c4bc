"""GPU: k-space outputs -- spectral function (output=spf), unfolded spectral function
(output=uspf) and the density of states (dosfile) -- against the reference's float64 maps
(golden fixtures) and the oracle."""
import os

import numpy as np
import pytest

from golden_cases import energies, load, uspf_pos, uspf_pre

pytestmark = pytest.mark.gpu


def _engine(name, precision, kp=None):
    import cqpi
    from oracle import formats as F
    from oracle import oracle as O
    d, meta, ref = load(name)
    with open(os.path.join(d, "model_hr.dat")) as fh:
        m = O.Model.from_hr(F.read_hr(fh.read()), efermi=meta.get("fermi", 0.0))
    eng = cqpi.Engine(m, meta["n"], kp or meta["kp"], meta["os"], meta["w"], meta["eta"], maxband=meta["maxband"],
                      precision=precision)
    return eng, meta, ref, m


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["spf_t2g", "uspf_t2g", "uspf_rect"])
def test_spectral_matches_reference(built_lib, name, precision):
    eng, meta, ref, m = _engine(name, precision)
    E = energies(meta)
    if meta["output"] == "spf":
        got = eng.spf(E)
    else:
        got = eng.uspf(E, np.array(uspf_pos(meta)), np.array(uspf_pre(meta)))
    err = np.abs(got - ref["ldos"]).max() / np.abs(ref["ldos"]).max()
    assert err < 1e-10, err          # both precisions read the FP64 eigen cache
    eng.close()


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_dos_matches_oracle(built_lib, precision, tol):
    from oracle import oracle as O
    eng, meta, ref, m = _engine("dos_c2", precision)
    dl, dh = meta["dosfile"]["energies"]
    L = meta["dosfile"]["layers"]
    E = np.array([dl + k * (dh - dl) / L for k in range(L)])
    got = eng.dos(E)
    ev, U = O.bands(m, meta["kp"])
    want = np.array([-np.imag(np.diag(O.realspace(O.greens_k(ev, U, meta["kp"], e, meta["eta"]))[0, 0]))
                     [:meta["maxband"]].sum() for e in E])
    assert np.abs(got - want).max() <= tol * np.abs(want).max()
    # the golden's own layer: tmatrix::calcdos of the reference
    assert abs(eng.dos(energies(meta))[0] - ref["dos"][0]) <= tol * abs(ref["dos"][0])
    eng.close()


def test_spectral_with_surface_greens(built_lib):
    """spf and dos follow the handle's Green's function (here the surface decimation)."""
    import cqpi
    from oracle import formats as F
    from oracle import oracle as O
    d, meta, ref = load("surface_c1")
    with open(os.path.join(d, "model_hr.dat")) as fh:
        m = O.Model.from_hr(F.read_hr(fh.read()))
    with open(os.path.join(d, "surf_hr.dat")) as fh:
        sm = O.Model.from_hr(F.read_hr(fh.read()))
    n = meta["kp"]
    eng = cqpi.Engine(m, n, n, meta["os"], meta["w"], meta["eta"], precision=cqpi.PREC_FP64)
    eng.set_greens("surface", 1e-5, sm)
    E = np.array([-0.3, 0.1])
    got = eng.spf(E)
    dos = eng.dos(E)
    for k, e in enumerate(E):
        g0k = O.surface_greens_k(m, n, e, meta["eta"], 1e-5, True, sm)
        want = O.spf(g0k, 1).T
        assert np.abs(got[k] - want).max() <= 1e-12 * np.abs(want).max()
        wd = -np.imag(O.realspace(g0k)[0, 0, 0, 0])
        assert abs(dos[k] - wd) <= 1e-12 * abs(wd)
    eng.close()
