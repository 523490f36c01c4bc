"""Known answers that pin the oracle independently of the reference's goldens (CPU only).

  * the local lattice Green's function of the nearest-neighbour square lattice outside the
    band: G0(R=0, w) = 2 / (pi w) K(m = (4t / w)^2), K the complete elliptic integral of the
    first kind (the k-sum of tightbind::calcgreensfunction + the FFT of
    tmatrix::calcrealspacegreensfunction, src/tightbinding.cc:282-289, src/qpi.cc:557-578);
  * one band, scalar V: T = V / (1 - V G0(0)) (tmatrix::setscatteringmatrix, src/qpi.cc:833-854);
  * V = 0: T = 0 and the map is the term-1 tile of one unit cell repeated over the field of
    view (tmatrix::calcwannierldos, src/qpi.cc:876-950);
  * reciprocity with real hoppings: G0(R)[a][o] = G0(-R)[o][a];
  * the surface / bulk decimation on a semi-infinite chain: the closed forms;
  * a C4v model with a centred impurity and an s-like orbital: the map is symmetric under
    x <-> y, inversion and 90-degree rotation about the impurity pixel (inside the field of
    view; the wrapped outermost pixel row has no partner).
"""
import numpy as np
import pytest

from cqpi import workloads as W
from oracle import oracle as O


def _model(m):
    return O.Model(m.bands, m.R, m.orb, m.t, None, m.efermi, m.scmaxbands)


@pytest.mark.parametrize("w", [5.0, -4.6, 6.5])
def test_square_lattice_green_function_is_the_elliptic_integral(w):
    special = pytest.importorskip("scipy.special")
    terms = {(r[0], r[1], 0): np.array([[-1.0 + 0j]]) for r in [(1, 0), (-1, 0), (0, 1), (0, -1)]}
    nn = W._from_terms(terms, 1, "nearest-neighbour square lattice, t=-1")
    kp = 256
    ev, U = O.bands(_model(nn), kp)
    g00 = O.realspace(O.greens_k(ev, U, kp, w, 1e-9))[0, 0][0, 0]
    exact = 2.0 / (np.pi * w) * special.ellipk((4.0 / w) ** 2)
    assert abs(g00 - exact) <= 1e-8 * abs(exact)


def test_scalar_t_matrix():
    for g00, v in ((0.3 - 0.2j, 0.7), (-1.1 - 0.05j, -0.4), (0.02 - 2.0j, 3.0)):
        T = O.tmatrix(np.array([v], complex), np.array([[g00]]))
        assert T.shape == (1, 1)
        assert abs(T[0, 0] - v / (1 - v * g00)) <= 1e-14 * abs(T[0, 0])


def test_reciprocity_with_real_hoppings():
    c, m, _ = W.config("C2")
    assert np.all(np.abs(np.imag(m.t)) == 0)
    kp = 32
    ev, U = O.bands(_model(m), kp)
    g = O.realspace(O.greens_k(ev, U, kp, 0.05, 0.02))
    x = np.arange(kp)
    gm = g[np.ix_((-x) % kp, (-x) % kp)]                 # G0(-R)
    assert np.abs(g - np.swapaxes(gm, -1, -2)).max() <= 1e-13 * np.abs(g).max()


@pytest.fixture(scope="module")
def c1_maps():
    m = W.square_c1()
    n, kp, os_, w = 16, 64, 4, 2
    wf = W.gaussian_c1(w, os_)
    ev, U = O.bands(_model(m), kp)
    g0r = O.realspace(O.greens_k(ev, U, kp, 0.1, 0.05))
    mp0 = O.wannier_ldos(n, kp, os_, w, 1, False, np.zeros((1, 1), complex), g0r, wf)
    T = O.tmatrix(np.array([0.5], complex), g0r[0, 0])
    mp = O.wannier_ldos(n, kp, os_, w, 1, False, T, g0r, wf)
    return n, os_, mp0, mp


def test_zero_potential_repeats_the_unit_cell_tile(c1_maps):
    n, os_, mp0, mp = c1_maps
    assert mp0.shape == (n * os_, n * os_)
    np.testing.assert_array_equal(mp0, np.tile(mp0[:os_, :os_], (n, n)))
    assert np.abs(mp - mp0).max() > 1e-3 * np.abs(mp0).max()      # the impurity changes the map


def test_c4v_symmetry_about_the_impurity(c1_maps):
    n, os_, mp0, mp = c1_maps
    tol = 1e-13 * np.abs(mp).max()
    assert np.abs(mp - mp.T).max() <= tol
    c = (n // 2) * os_ + os_ // 2                  # pixel of the impurity site's centre
    idx = np.arange(c - (n // 2 - 1) * os_, c + (n // 2 - 1) * os_ + 1)
    sub = mp[np.ix_(idx, idx)]
    assert np.abs(sub - sub[::-1, ::-1]).max() <= tol
    assert np.abs(sub - np.rot90(sub)).max() <= tol


@pytest.mark.parametrize("w,eta", [(0.7, 0.05), (2.5, 0.05), (-1.3, 0.2)])
def test_semi_infinite_chain_surface_and_bulk_green_functions(w, eta):
    """Only inter-layer hopping t: every k-point is a semi-infinite chain, whose surface and
    bulk Green's functions are (z - sqrt(z^2 - 4t^2)) / (2t^2) and 1 / sqrt(z^2 - 4t^2), the
    roots with Im G < 0 (the decimation of tmatrix::calcsurfacegreensfunction,
    src/qpi.cc:488-554)."""
    t = -1.0
    m = O.Model(1, [[0, 0, 1], [0, 0, -1]], [[0, 0], [0, 0]], [t, t])
    z = w + 1j * eta
    r = np.sqrt(z * z - 4 * t * t)
    surf = [g for g in ((z - r) / (2 * t * t), (z + r) / (2 * t * t)) if g.imag < 0][0]
    bulk = [g for g in (1 / r, -1 / r) if g.imag < 0][0]
    gs = O.surface_greens_k(m, 4, w, eta, 1e-12, True)
    gb = O.surface_greens_k(m, 4, w, eta, 1e-12, False)
    assert np.abs(gs - surf).max() <= 1e-12 * abs(surf)
    assert np.abs(gb - bulk).max() <= 1e-12 * abs(bulk)
