"""GPU parity: every stage of the CUDA path against the CPU oracle (FP64 path)."""
import numpy as np
import pytest

from cases import case

pytestmark = pytest.mark.gpu

CASES = ["c1", "c1_odd", "c2", "c2_zero", "c3"]


def _engine(name, precision=0):
    import cqpi
    m, p, wf, z, v, E = case(name)
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                      precision=precision)
    eng.set_orbitals(wf, z)
    eng.set_scattering(v)
    return eng, (m, p, wf, z, v, E)


def _oracle_model(m):
    from oracle import oracle as O
    return O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)


def _relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_bands_reconstruct_hamiltonian(built_lib, name):
    from oracle import oracle as O
    eng, (m, p, *_rest) = _engine(name)
    ev, U = eng.get_bands()
    H = O.np_hk_grid(_oracle_model(m), p["kpoints"]).reshape(-1, m.bands, m.bands)
    rec = np.einsum("kon,kn,kan->koa", U, ev, U.conj())
    assert np.abs(rec - H).max() < 1e-12 * max(1.0, np.abs(H).max())
    eye = np.einsum("kon,koa->kna", U.conj(), U)
    assert np.abs(eye - np.eye(m.bands)).max() < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_greens_box_and_tmatrix(built_lib, name):
    from oracle import oracle as O
    eng, (m, p, wf, z, v, E) = _engine(name)
    om = _oracle_model(m)
    kp = p["kpoints"]
    ev, U = O.bands(om, kp)
    for e in E:
        g0r = O.realspace(O.greens_k(ev, U, kp, e, p["eta"]))
        box, rb = eng.greens_box(e)
        idx = (np.arange(-rb, rb + 1)) % kp
        ref = g0r[np.ix_(idx, idx)]
        assert _relerr(box, ref) < 1e-12
        T = eng.tmatrix(e)
        Tref = O.tmatrix(v, g0r[0, 0])
        assert _relerr(T, Tref) < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_ldos_fp64_vs_oracle(built_lib, name):
    from oracle import oracle as O
    eng, (m, p, wf, z, v, E) = _engine(name)
    o32, o64 = eng.run(E, f32=True, f64=True)
    ref = O.run(_oracle_model(m), p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], E, v, wf, z,
                spin=p["spin"])
    assert o64.shape == (len(E), 1, p["lattice"] * p["oversamp"], p["lattice"] * p["oversamp"])
    assert _relerr(o64[:, 0], ref) < 1e-10
    assert np.array_equal(o32, o64.astype(np.float32))
    assert eng.kernel_launches() > 0


def test_narrow_seam_gpuqpi(built_lib):
    """GPUQPI::wannierldos + retrieveResult(double*) with the oracle's G0(R) and T."""
    from oracle import oracle as O
    eng, (m, p, wf, z, v, E) = _engine("c2")
    om = _oracle_model(m)
    kp = p["kpoints"]
    ev, U = O.bands(om, kp)
    g0r = O.realspace(O.greens_k(ev, U, kp, E[0], p["eta"]))
    T = O.tmatrix(v, g0r[0, 0])
    eng.wannierldos(T, g0r)
    got = eng.retrieve_result()
    ref = O.wannier_ldos(p["lattice"], kp, p["oversamp"], p["window"], m.bands, False, T, g0r, wf).T
    assert _relerr(got, ref) < 1e-12


def test_multiple_impurities_match_single(built_lib):
    import cqpi
    eng, (m, p, wf, z, v, E) = _engine("c2")
    rng = np.random.default_rng(7)
    A = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    Vh = 0.2 * (A + A.conj().T)
    Vs = np.stack([np.diag(v), Vh])
    eng.set_impurities(Vs)
    both = eng.run(E, f32=False, f64=True)
    eng.set_scattering(v)
    one = eng.run(E, f32=False, f64=True)
    assert np.abs(both[:, 0] - one[:, 0]).max() == 0.0
    assert np.abs(both[:, 1] - both[:, 0]).max() > 0.0


def test_errors_are_status_codes(built_lib):
    import cqpi
    m, p, wf, z, v, E = case("c1")
    with pytest.raises(cqpi.CqpiError) as ei:
        cqpi.Engine(m, 40, 12, 2, 2, 0.01)   # lattice/2 + window > kp, kp not a power of two
    assert ei.value.code == cqpi.ERR_DOMAIN
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"])
    with pytest.raises(cqpi.CqpiError) as ei:
        eng.run(E)
    assert ei.value.code == cqpi.ERR_STATE
    with pytest.raises(cqpi.CqpiError) as ei:
        eng.set_orbitals(np.zeros((1, 5, 5)))
    assert ei.value.code == cqpi.ERR_ARG
