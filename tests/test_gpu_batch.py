"""GPU: batched maps with a field of view per map (cqpi_run_fov) and CUDA-graph replay.

A map of field of view f is the centred f x f-site crop of the full-field map (the LDOS at a
site does not depend on how many sites are computed), so the batched maps must equal the
crops of cqpi_run's maps exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(lattice=24, kp=64, os_=5, w=2, nimp=3, seed=4):
    import cqpi
    from cqpi import workloads as W
    m = W.t2g_c2()
    eng = cqpi.Engine(m, lattice, kp, os_, w, 0.01, precision=cqpi.PREC_MIXED)
    eng.set_orbitals(W.t2g_orbitals_c2(w, os_))
    rng = np.random.default_rng(seed)
    Vs = []
    for k in range(nimp):
        if k % 2 == 0:
            Vs.append(rng.uniform(-1, 1) * np.eye(3))
        else:
            A = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
            Vs.append(0.2 * (A + A.conj().T))
    eng.set_impurities(np.stack(Vs))
    return eng


def _crops(full, fov, os_, lattice):
    n2 = lattice >> 1
    out = []
    nE, nimp = full.shape[:2]
    for e in range(nE):
        for i in range(nimp):
            f = fov[e * nimp + i]
            s0 = (n2 - (f >> 1)) * os_
            out.append(full[e, i, s0:s0 + f * os_, s0:s0 + f * os_].ravel())
    return np.concatenate(out)


def test_run_fov_maps_are_crops_of_full_maps(built_lib):
    torch = pytest.importorskip("torch")
    eng = _engine()
    if eng.contraction_kind() != "tcgen05":
        pytest.skip("tensor-core contraction not selected")
    E = np.array([-0.05, -0.01, 0.02, 0.06, 0.08])
    rng = np.random.default_rng(1)
    fov = rng.choice([5, 8, 12, 17, 24], size=len(E) * eng.nimp).astype(np.int32)
    full = eng.run(E)
    total = int(np.sum((fov * eng.oversamp) ** 2))
    buf = torch.full((total,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    eng.run_fov(E, fov, buf.data_ptr())
    eng.synchronize()
    got = buf.cpu().numpy()
    ref = _crops(full, fov, eng.oversamp, eng.lattice)
    assert np.array_equal(got, ref)
    eng.close()


def test_graph_replay_matches_direct_calls(built_lib):
    torch = pytest.importorskip("torch")
    eng = _engine()
    if eng.contraction_kind() != "tcgen05":
        pytest.skip("tensor-core contraction not selected")
    E = np.linspace(-0.08, 0.08, 7)
    fov = np.full(len(E) * eng.nimp, 16, np.int32)
    fov[::2] = 9
    total = int(np.sum((fov * eng.oversamp) ** 2))
    direct = torch.empty((total,), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    eng.solve_bands()
    eng.run_fov(E, fov, direct.data_ptr())        # allocates every buffer
    eng.synchronize()
    graphed = torch.zeros((total,), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    eng.graph_begin()
    eng.run_fov(E, fov, graphed.data_ptr())
    eng.graph_end()
    n0 = eng.kernel_launches()
    for _ in range(2):
        eng.graph_launch()
    eng.synchronize()
    assert eng.kernel_launches() > n0
    assert torch.equal(direct, graphed)
    eng.close()


def test_device_wait_timeout_is_reported_and_handle_recovers(built_lib, monkeypatch):
    """Fault injection without a GPU fault: with CQPI_TEST_STALL=1 the contraction waits
    (bounded, ~0.3 ms) on a barrier nothing arrives on; every warp role takes the time-out
    path, frees its tensor memory and returns, the call reports CQPI_ERR_TIMEOUT, and the
    same handle then runs normally."""
    import cqpi
    eng = _engine()
    if eng.contraction_kind() != "tcgen05":
        pytest.skip("tensor-core contraction not selected")
    E = np.array([-0.03, 0.01, 0.05])
    good = eng.run(E)
    monkeypatch.setenv("CQPI_TEST_STALL", "1")
    with pytest.raises(cqpi.CqpiError) as ei:
        eng.run(E)
    assert ei.value.code == cqpi.ERR_TIMEOUT
    monkeypatch.delenv("CQPI_TEST_STALL")
    again = eng.run(E)
    assert np.array_equal(again, good)
    eng.close()


def test_bulk_column_fetch_keeps_the_maps(built_lib, monkeypatch):
    """The 3-band kernel's bulk-copy variant (one copy per raw window column, taken when
    autotuning finds it faster) stages the same values as the cp.async pieces: identical
    maps, also with only some columns in bulk."""
    eng = _engine()
    if eng.contraction_kind() != "tcgen05":
        pytest.skip("tensor-core contraction not selected")
    E = np.array([-0.04, 0.02, 0.07])
    pieces = eng.run(E)
    for nb in ("1000", "7"):
        monkeypatch.setenv("CQPI_TC_NBULK", nb)
        assert np.array_equal(eng.run(E), pieces), nb
    eng.close()


def test_autotune_keeps_the_maps(built_lib):
    """Tile shapes change the work split, not the arithmetic of a map value: after the
    autotuner picks a shape the maps are identical to the default shape's."""
    eng = _engine()
    if eng.contraction_kind() != "tcgen05":
        pytest.skip("tensor-core contraction not selected")
    E = np.linspace(-0.06, 0.06, 9)
    before = eng.run(E)
    ms, n = eng.autotune(E)
    assert n >= 1 and ms > 0
    after = eng.run(E)
    assert np.array_equal(before, after)
    eng.close()
