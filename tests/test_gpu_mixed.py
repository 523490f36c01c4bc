"""GPU: the mixed-precision path against the FP64 path and the oracle.

Tolerance (the spec bar): max|rho - rho64| / max|rho64| <= 1e-6 per map.
"""
import numpy as np
import pytest

from cases import case

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _run(name, precision):
    import cqpi
    m, p, wf, z, v, E = case(name)
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                      precision=precision)
    eng.set_orbitals(wf, z)
    eng.set_scattering(v)
    return eng.run(E, f32=False, f64=True), (m, p, wf, z, v, E)


@pytest.mark.parametrize("name", ["c1", "c1_odd", "c2", "c2_zero", "c3"])
def test_mixed_matches_fp64_and_oracle(built_lib, name):
    import cqpi
    from oracle import oracle as O
    mixed, (m, p, wf, z, v, E) = _run(name, cqpi.PREC_MIXED)
    fp64, _ = _run(name, cqpi.PREC_FP64)
    for e in range(len(E)):
        ref = fp64[e, 0]
        err = np.abs(mixed[e, 0] - ref).max() / np.abs(ref).max()
        assert err <= TOL, (name, e, err)
    om = O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)
    orc = O.run(om, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], E, v, wf, z, spin=p["spin"])
    assert np.abs(mixed[:, 0] - orc).max() / np.abs(orc).max() <= TOL


def test_mixed_c2_physics(built_lib):
    """C2 model and orbitals with the C2 k-grid and eta (sharp poles), a 32^2-site field of view."""
    import cqpi
    from cqpi import workloads as W
    c, m, wf = W.config("C2")
    E = np.array([-0.1, -0.03, 0.0, 0.05, 0.1])
    out = {}
    for prec in (cqpi.PREC_FP64, cqpi.PREC_MIXED):
        eng = cqpi.Engine(m, 32, c.kpoints, c.oversamp, c.window, c.eta, precision=prec)
        eng.set_orbitals(wf)
        eng.set_scattering(np.array(c.scattering, complex))
        out[prec] = eng.run(E, f32=False, f64=True)
        eng.close()
    for e in range(len(E)):
        ref = out[cqpi.PREC_FP64][e, 0]
        err = np.abs(out[cqpi.PREC_MIXED][e, 0] - ref).max() / np.abs(ref).max()
        assert err <= TOL, (E[e], err)


@pytest.mark.parametrize("name", ["c1", "c1_odd", "c2", "c2_zero", "c3"])
def test_tensor_core_contraction_matches_cuda_core(built_lib, name, monkeypatch):
    """The tcgen05 (split-FP16 x3) contraction against the FP32 CUDA-core contraction and FP64."""
    import cqpi
    tc, _ = _run(name, cqpi.PREC_MIXED)
    monkeypatch.setenv("CQPI_CONTRACTION", "fp32")
    cc, _ = _run(name, cqpi.PREC_MIXED)
    fp64, _ = _run(name, cqpi.PREC_FP64)
    for e in range(tc.shape[0]):
        ref = fp64[e, 0]
        assert np.abs(tc[e, 0] - ref).max() / np.abs(ref).max() <= TOL
        assert np.abs(tc[e, 0] - cc[e, 0]).max() / np.abs(ref).max() <= TOL


def test_tensor_core_kernel_selected(built_lib):
    import cqpi
    from cqpi import workloads as W
    c, m, wf = W.config("C2")
    eng = cqpi.Engine(m, 16, 64, c.oversamp, c.window, c.eta, precision=cqpi.PREC_MIXED)
    assert eng.contraction_kind() == "tcgen05"
    eng64 = cqpi.Engine(m, 16, 64, c.oversamp, c.window, c.eta, precision=cqpi.PREC_FP64)
    assert eng64.contraction_kind() == "fp64"


def test_tensor_core_multi_impurity(built_lib):
    """Several impurities share u and s; each map must equal its single-impurity run (to the
    mixed-precision bar: one impurity folds T into the s operand, several apply it in the
    epilogue)."""
    import cqpi
    m, p, wf, z, v, E = case("c2")
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"],
                      precision=cqpi.PREC_MIXED)
    eng.set_orbitals(wf, z)
    rng = np.random.default_rng(3)
    A = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    Vs = np.stack([np.diag(v), 0.2 * (A + A.conj().T), np.diag([0.7, -0.2, 0.1])])
    eng.set_impurities(Vs)
    allm = eng.run(E, f32=False, f64=True)
    for k in range(len(Vs)):
        eng.set_impurities(Vs[k:k + 1])
        one = eng.run(E, f32=False, f64=True)
        assert np.abs(allm[:, k] - one[:, 0]).max() <= 1e-6 * np.abs(one).max()


@pytest.mark.parametrize("name", ["c1", "c2", "c2_zero"])
def test_fused_greens_fft_matches_unfused(built_lib, name, monkeypatch):
    """The fused FP32 G0(k) + pruned FFT gives the same G0(R) box as the two-kernel path."""
    import cqpi
    m, p, wf, z, v, E = case(name)

    def box(env):
        if env:
            monkeypatch.setenv("CQPI_GREENS", env)
        else:
            monkeypatch.delenv("CQPI_GREENS", raising=False)
        eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                          precision=cqpi.PREC_MIXED)
        eng.set_orbitals(wf, z)
        return [eng.greens_box(e)[0] for e in E]

    fused, unfused = box(None), box("unfused")
    for a, b in zip(fused, unfused):
        assert np.abs(a - b).max() <= 2e-6 * np.abs(b).max()


@pytest.mark.parametrize("kp,lattice", [(64, 16), (256, 24), (1024, 20), (128, 160)])
def test_register_row_fft_matches_radix2(built_lib, kp, lattice, monkeypatch):
    """Four-step register row and column transforms vs the radix-2 shared-memory transforms
    (the last case has a box wider than the k-grid and takes the radix-2 path in both runs)."""
    import cqpi
    from cqpi import workloads as W
    m = W.t2g_c2()
    wf = W.t2g_orbitals_c2(2, 3)

    def box(force):
        if force:
            monkeypatch.setenv("CQPI_ROWFFT", "radix2")
            monkeypatch.setenv("CQPI_COLFFT", "radix2")
        else:
            monkeypatch.delenv("CQPI_ROWFFT", raising=False)
            monkeypatch.delenv("CQPI_COLFFT", raising=False)
        eng = cqpi.Engine(m, lattice, kp, 3, 2, 0.01, precision=cqpi.PREC_MIXED)
        eng.set_orbitals(wf)
        return eng.greens_box(0.037)[0]

    a, b = box(False), box(True)
    assert np.abs(a - b).max() <= 2e-6 * np.abs(b).max()


@pytest.mark.parametrize("bands,real", [(1, True), (2, True), (3, True), (3, False)])
def test_persistent_row_fft_matches_per_row_kernel(built_lib, bands, real, monkeypatch):
    """kp = 1024, up to 3 bands: the persistent G0 + row transform (a resident grid walking
    (row, energy) items) vs the one-block-per-row kernel (CQPI_ROWFFT=classic), with the
    reciprocity planes (real hoppings) and with all b^2 planes (hoppings given a complex
    phase e^{i theta.R}, which keeps H Hermitian)."""
    import cqpi
    from cqpi import workloads as W
    terms = {}
    for R, M in W.t2g_c2().terms().items():
        ph = 1.0 if real else np.exp(1j * (0.3 * R[0] - 0.2 * R[1]))
        terms[R] = M[:bands, :bands] * ph
    m = W._from_terms(terms, bands, "t2g subset")
    wf = W.t2g_orbitals_c2(2, 3)[:bands]

    def box(classic):
        if classic:
            monkeypatch.setenv("CQPI_ROWFFT", "classic")
        else:
            monkeypatch.delenv("CQPI_ROWFFT", raising=False)
        eng = cqpi.Engine(m, 16, 1024, 3, 2, 0.01, precision=cqpi.PREC_MIXED)
        eng.set_orbitals(wf)
        out = [eng.greens_box(e)[0] for e in (-0.05, 0.037)]
        eng.close()
        return out

    for a, b in zip(box(False), box(True)):
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


@pytest.mark.parametrize("name", ["c1", "c2", "c2_zero"])
def test_pipelined_contraction_matches_serial(built_lib, name, monkeypatch):
    """Software-pipelined tcgen05 kernel (double-buffered B and accumulators) vs the serial one."""
    import cqpi
    pipe, _ = _run(name, cqpi.PREC_MIXED)
    monkeypatch.setenv("CQPI_TC_PIPE", "0")
    serial, _ = _run(name, cqpi.PREC_MIXED)
    assert np.abs(pipe - serial).max() <= 1e-7 * np.abs(serial).max()


@pytest.mark.parametrize("name", ["c1", "c1_odd", "c2", "c2_zero"])
def test_window_contraction_matches_gathered(built_lib, name, monkeypatch):
    """Direct-window tcgen05 kernel (fp16 windows addressed by the MMA descriptors) vs the
    kernel that gathers the B operand per tile."""
    import cqpi
    win, _ = _run(name, cqpi.PREC_MIXED)
    monkeypatch.setenv("CQPI_TC_ATMEM", "1")
    win_smem_a, _ = _run(name, cqpi.PREC_MIXED)
    monkeypatch.delenv("CQPI_TC_ATMEM")
    monkeypatch.setenv("CQPI_TC_WINDOW", "0")
    gathered, _ = _run(name, cqpi.PREC_MIXED)
    # Phi read from tensor memory or from shared memory: the same products in the same order
    assert np.abs(win - win_smem_a).max() <= 1e-7 * np.abs(gathered).max()
    assert np.abs(win - gathered).max() <= 5e-7 * np.abs(gathered).max()


@pytest.mark.parametrize("lattice,window,oversamp", [(40, 3, 5), (33, 2, 10), (24, 4, 3)])
def test_window_contraction_tiles_and_k_steps(built_lib, lattice, window, oversamp, monkeypatch):
    """Several tiles per site row with a ragged last tile, and windows whose K rows need
    more than one 16-wide k-step, against the FP64 path."""
    import cqpi
    from cqpi import workloads as W
    m = W.t2g_c2()
    wf = W.t2g_orbitals_c2(window, oversamp)
    E = np.array([-0.04, 0.013])
    out = {}
    for prec in (cqpi.PREC_FP64, cqpi.PREC_MIXED):
        eng = cqpi.Engine(m, lattice, 64, oversamp, window, 0.01, precision=prec)
        eng.set_orbitals(wf)
        eng.set_scattering(np.array([0.3, 0.3, 0.3], complex))
        out[prec] = eng.run(E, f32=False, f64=True)
        eng.close()
    ref = out[cqpi.PREC_FP64]
    for e in range(len(E)):
        err = np.abs(out[cqpi.PREC_MIXED][e, 0] - ref[e, 0]).max() / np.abs(ref[e, 0]).max()
        assert err <= TOL, (lattice, window, oversamp, E[e], err)


@pytest.mark.parametrize("name", ["c1", "c2", "c2_zero"])
def test_time_reversal_matches_full_solve(built_lib, name, monkeypatch):
    """Real hoppings: the eigen-solve of half the k-grid plus H(-k) = conj(H(k)) gives the
    maps of the full solve (FP64 path to rounding, mixed path to its tolerance)."""
    import cqpi
    half64, _ = _run(name, cqpi.PREC_FP64)
    halfmx, _ = _run(name, cqpi.PREC_MIXED)
    monkeypatch.setenv("CQPI_TIME_REVERSAL", "0")
    full64, _ = _run(name, cqpi.PREC_FP64)
    fullmx, _ = _run(name, cqpi.PREC_MIXED)
    assert np.abs(half64 - full64).max() <= 1e-12 * np.abs(full64).max()
    assert np.abs(halfmx - fullmx).max() <= 1e-6 * np.abs(fullmx).max()


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_spin_block_reduction_matches_full_spin_path(built_lib, precision, tol, monkeypatch):
    """Spin-degenerate model (decoupled, identical spin blocks; same orbitals and V per
    block): the reduced run (twice the mb-band maps) equals the full 2mb-band spin run."""
    import cqpi
    red, _ = _run("c3", precision)
    monkeypatch.setenv("CQPI_SPIN_REDUCE", "0")
    full, _ = _run("c3", precision)
    assert np.abs(red - full).max() <= tol * np.abs(full).max()


def test_spin_block_reduction_only_for_identical_blocks(built_lib):
    """A potential that differs between the spin blocks keeps the full spin path, whose maps
    match the FP64 path and the oracle."""
    import cqpi
    from oracle import oracle as O
    m, p, wf, z, v, E = case("c3")
    v = np.asarray(v, complex).copy()
    v[5:] *= 0.5                      # spin-dependent scattering
    out = {}
    for prec in (cqpi.PREC_FP64, cqpi.PREC_MIXED):
        eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=True,
                          precision=prec)
        eng.set_orbitals(wf, z)
        eng.set_scattering(v)
        out[prec] = eng.run(E, f32=False, f64=True)
        eng.close()
    om = O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)
    orc = O.run(om, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], E, v, wf, z, spin=True)
    assert np.abs(out[cqpi.PREC_FP64][:, 0] - orc).max() <= 1e-10 * np.abs(orc).max()
    assert np.abs(out[cqpi.PREC_MIXED][:, 0] - orc).max() <= TOL * np.abs(orc).max()
