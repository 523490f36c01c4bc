"""GPU: the adjoint (cqpi_adjoint) against finite differences of the FP64 forward.

L = sum W * rho with a fixed random weight map W = dL/drho.  A direction keeps H(k)
Hermitian: a hopping term and its partner (-R, orbitals swapped) move by conjugate amounts.
The directional derivative from the adjoint is sum Re(conj(g) * delta) with
g = dL/dRe z + i dL/dIm z.
  * central differences, h = 1e-6: both precisions to 1e-5 relative (their truncation error
    alone is ~1e-7..1e-6 relative here: eta makes L sharply curved in t);
  * fourth-order differences (h = 4e-6): the FP64 adjoint to 1e-7 relative.
"""
import numpy as np
import pytest

from cases import case

pytestmark = pytest.mark.gpu

def _engine(m, p, wf, z, v, precision):
    import cqpi
    eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], spin=p["spin"],
                      precision=precision)
    eng.set_orbitals(wf, z)
    if np.ndim(v) == 1:
        eng.set_scattering(v)
    else:
        eng.set_impurities(v)
    return eng


def _hermitian_direction(m, rng):
    """Random complex change of every hopping term with its Hermitian partner conjugated."""
    R = np.asarray(m.R).reshape(-1, 3)
    orb = np.asarray(m.orb).reshape(-1, 2)
    anti = np.asarray(m.anti, bool) if getattr(m, "anti", None) is not None else np.zeros(len(m.t), bool)
    key = {(R[i, 0], R[i, 1], orb[i, 0], orb[i, 1], anti[i]): i for i in range(len(m.t))}
    d = np.zeros(len(m.t), complex)
    done = np.zeros(len(m.t), bool)
    for i in range(len(m.t)):
        if done[i]:
            continue
        j = key.get((-R[i, 0], -R[i, 1], orb[i, 1], orb[i, 0], anti[i]))
        if j is None:
            continue
        if j == i:
            d[i] = rng.normal()          # self-partner: real change
        else:
            d[i] = rng.normal() + 1j * rng.normal()
            d[j] = np.conj(d[i])
            done[j] = True
        done[i] = True
    return d


def _loss(eng, E, Wt):
    return float(np.sum(eng.run(E, f32=False, f64=True) * Wt))


def _fd(loss_at, h, order):
    if order == 2:
        return (loss_at(h) - loss_at(-h)) / (2 * h)
    return (8 * (loss_at(h) - loss_at(-h)) - (loss_at(2 * h) - loss_at(-2 * h))) / (12 * h)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("prec,h,order,tol", [(0, 1e-6, 2, 1e-5), (1, 1e-6, 2, 1e-5), (0, 4e-6, 4, 1e-7)])
def test_adjoint_hoppings_and_v_match_fd(built_lib, name, prec, h, order, tol):
    import cqpi
    m, p, wf, z, v, E = case(name)
    b = m.bands
    rng = np.random.default_rng(11)
    # full impurity matrix (an extension of the diagonal reference potential)
    V = np.diag(np.asarray(v, complex).reshape(-1)) + 0.05 * (rng.normal(size=(b, b)) + 1j * rng.normal(size=(b, b)))
    V = V[None]
    eng = _engine(m, p, wf, z, V, prec)
    wn = p["lattice"] * p["oversamp"]
    Wt = rng.normal(size=(len(E), 1, wn, wn)).astype(np.float32)
    gt, gv = eng.adjoint(E, Wt)
    eng.close()

    ref = _engine(m, p, wf, z, V, cqpi.PREC_FP64)
    t0 = np.asarray(m.t, complex)
    for trial in range(2):
        d = _hermitian_direction(m, rng)

        def lt(x):
            ref.set_hoppings(t0 + x * d)
            return _loss(ref, E, Wt)

        fd = _fd(lt, h, order)
        ad = float(np.sum((np.conj(gt) * d).real))
        assert abs(ad - fd) <= tol * abs(fd) + 1e-12, (name, prec, trial, ad, fd)
    ref.set_hoppings(t0)
    for trial in range(2):
        dV = rng.normal(size=(1, b, b)) + 1j * rng.normal(size=(1, b, b))

        def lv(x):
            ref.set_impurities(V + x * dV)
            return _loss(ref, E, Wt)

        fd = _fd(lv, h, order)
        ad = float(np.sum((np.conj(gv) * dV).real))
        assert abs(ad - fd) <= tol * abs(fd) + 1e-12, (name, prec, trial, ad, fd)
    ref.close()


def test_adjoint_matches_fd_of_the_oracle(built_lib):
    """The adjoint of the GPU engine against fourth-order differences of the CPU
    restatement of the reference's path (FP64 throughout)."""
    import cqpi
    from oracle import oracle as O
    m, p, wf, z, v, E = case("c1")
    rng = np.random.default_rng(5)
    eng = _engine(m, p, wf, z, v, cqpi.PREC_FP64)
    wn = p["lattice"] * p["oversamp"]
    Wt = rng.normal(size=(len(E), 1, wn, wn)).astype(np.float32)
    gt, _ = eng.adjoint(E, Wt)
    eng.close()
    d = _hermitian_direction(m, rng)
    t0 = np.asarray(m.t, complex)

    def loss(t):
        om = O.Model(m.bands, m.R, m.orb, t, m.anti, m.efermi, m.scmaxbands)
        maps = O.run(om, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"], E, v, wf, z)
        return float(np.sum(maps * Wt[:, 0]))

    h = 4e-6
    fd = (8 * (loss(t0 + h * d) - loss(t0 - h * d)) - (loss(t0 + 2 * h * d) - loss(t0 - 2 * h * d))) / (12 * h)
    ad = float(np.sum((np.conj(gt) * d).real))
    assert abs(ad - fd) <= 1e-7 * abs(fd) + 1e-12, (ad, fd)


def test_set_hoppings_rebuilds_bands(built_lib):
    """set_hoppings with the model's own amplitudes reproduces the original maps, and a
    changed model changes them."""
    import cqpi
    m, p, wf, z, v, E = case("c2")
    eng = _engine(m, p, wf, z, v, cqpi.PREC_FP64)
    a = eng.run(E, f32=False, f64=True)
    t0 = np.asarray(m.t, complex)
    eng.set_hoppings(1.1 * t0)
    b_ = eng.run(E, f32=False, f64=True)
    eng.set_hoppings(t0)
    c = eng.run(E, f32=False, f64=True)
    assert np.abs(a - c).max() <= 1e-13 * np.abs(a).max()
    assert np.abs(a - b_).max() > 1e-3 * np.abs(a).max()
    eng.close()


@pytest.mark.parametrize("kp,lattice", [(64, 8), (256, 12)])
def test_adjoint_register_rows_match_radix2(built_lib, kp, lattice, monkeypatch):
    """Mixed handle: the box -> k-grid columns and rows of the adjoint by the four-step
    register transforms (several columns per block) give the gradients of the radix-2
    one-column-per-block kernels (CQPI_ADJ_ROWS=radix2) to FP32 rounding."""
    import cqpi
    from cqpi import workloads as W
    m = W.t2g_c2()
    wf = W.t2g_orbitals_c2(2, 3)
    rng = np.random.default_rng(17)
    E = np.array([-0.06, 0.021])
    Wt = rng.normal(size=(len(E), 1, lattice * 3, lattice * 3)).astype(np.float32)
    out = []
    for env in (None, "radix2"):
        if env:
            monkeypatch.setenv("CQPI_ADJ_ROWS", env)
        else:
            monkeypatch.delenv("CQPI_ADJ_ROWS", raising=False)
        eng = cqpi.Engine(m, lattice, kp, 3, 2, 0.01, precision=cqpi.PREC_MIXED)
        eng.set_orbitals(wf)
        eng.set_scattering(np.array([0.3, 0.3, 0.5], complex))
        out.append(eng.adjoint(E, Wt))
        eng.close()
    (gt, gv), (rt, rv) = out
    assert np.abs(gt - rt).max() <= 1e-5 * np.abs(rt).max()
    assert np.abs(gv - rv).max() <= 1e-5 * np.abs(rv).max()


@pytest.mark.parametrize("kind", ["c1", "c2", "c5_cell", "impurities"])
def test_adjoint_tensor_core_contraction_matches_cuda_cores(built_lib, kind, monkeypatch):
    """Mixed handle: the contraction adjoint on the tensor cores (split-fp16 x 3 products,
    adjoint_mma.cu) against the CUDA-core warp-per-site kernel (CQPI_ADJ_MMA=0): the same
    gradients to FP32 rounding, for 1 and 3 bands, a C5-sized cell (10x10 sub-pixels, 75 window
    entries) and two impurities."""
    import cqpi
    from cqpi import workloads as W
    rng = np.random.default_rng(23)
    A = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))

    def engine():
        if kind in ("c1", "c2"):
            m, p, wf, z, v, E = case(kind)
            eng = cqpi.Engine(m, p["lattice"], p["kpoints"], p["oversamp"], p["window"], p["eta"],
                              precision=cqpi.PREC_MIXED)
            eng.set_orbitals(wf, z)
            eng.set_scattering(v)
            return eng, E, p["lattice"] * p["oversamp"], 1
        eng = cqpi.Engine(W.t2g_c2(), 8, 64, 10, 2, 0.01, precision=cqpi.PREC_MIXED)
        eng.set_orbitals(W.t2g_orbitals_c2(2, 10))
        if kind == "impurities":
            eng.set_impurities(np.stack([np.diag([0.3, 0.3, 0.5]), 0.2 * (A + A.conj().T)]).astype(complex))
            return eng, np.array([-0.05, 0.03]), 80, 2
        eng.set_scattering(np.array([0.3, 0.3, 0.5], complex))
        return eng, np.array([-0.05, 0.03]), 80, 1

    Wt = None
    out = []
    for env in (None, "0"):
        if env:
            monkeypatch.setenv("CQPI_ADJ_MMA", env)
        else:
            monkeypatch.delenv("CQPI_ADJ_MMA", raising=False)
        eng, E, wn, nimp = engine()
        if Wt is None:
            Wt = rng.normal(size=(len(E), nimp, wn, wn)).astype(np.float32)
        out.append(eng.adjoint(E, Wt))
        eng.close()
    (gt, gv), (rt, rv) = out
    assert np.abs(gt - rt).max() <= 1e-5 * np.abs(rt).max()
    assert np.abs(gv - rv).max() <= 1e-5 * np.abs(rv).max()
