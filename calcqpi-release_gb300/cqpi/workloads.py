"""Seeded synthetic workloads: tight-binding models and orbital cubes.

The reference ships no example inputs, so the five benchmark configurations are
generated here (``numpy.random.default_rng(seed)``):

* C1  square lattice, 1 orbital, NN t=-1.0, NNN t'=0.3 eV; normalised 3D Gaussian
      orbital sigma=0.3a at z=0.5a.
* C2  square-lattice t2g model (dxz, dyz, dxy), hoppings to 3rd neighbours drawn
      N(0, 0.25 eV), C4 symmetry and Hermiticity enforced, seed 2; orbitals are the
      d angular parts times a radial Gaussian sigma=0.4a at z=0.6a.
* C3  triangular lattice, 5 orbitals (s, px, py, dx2-y2, dxy) to 4th neighbours,
      C6 symmetry and Hermiticity enforced, seed 3, spin-degenerate (10 bands);
      orbitals are Gaussian-radial s/p/d mixtures with seed-drawn coefficients.
* C4  the C2 model with a batch of energies x impurities x fields of view.
* C5  the C2 model, 128x128 sites, 41 energies (fitting harness).

Models are returned as hopping lists in the layout of the reference's
``hoppingterm`` vector (src/tightbinding.h:111-164): R[h,3], orb[h,2] (0-based),
t[h] complex, already divided by the Wannier90 degeneracy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class TBModel:
    bands: int
    R: np.ndarray
    orb: np.ndarray
    t: np.ndarray
    anti: np.ndarray = None
    efermi: float = 0.0
    scmaxbands: int = None
    name: str = "model"

    def __post_init__(self):
        self.R = np.ascontiguousarray(self.R, np.int32).reshape(-1, 3)
        self.orb = np.ascontiguousarray(self.orb, np.int32).reshape(-1, 2)
        self.t = np.ascontiguousarray(self.t, np.complex128).reshape(-1)
        if self.anti is None:
            self.anti = np.zeros(len(self.t), np.uint8)
        self.anti = np.ascontiguousarray(self.anti, np.uint8)
        if self.scmaxbands is None:
            self.scmaxbands = self.bands

    def terms(self) -> dict:
        """Hopping matrices keyed by R (for writing a _hr.dat)."""
        out = {}
        for h in range(len(self.t)):
            key = tuple(int(v) for v in self.R[h])
            if key not in out:
                out[key] = np.zeros((self.bands, self.bands), np.complex128)
            out[key][self.orb[h, 0], self.orb[h, 1]] += self.t[h]
        return out


def _from_terms(terms: dict, bands: int, name: str, drop_zero=True) -> TBModel:
    R, orb, t = [], [], []
    for key in sorted(terms):
        M = terms[key]
        for v in range(bands):
            for u in range(bands):
                if drop_zero and M[u, v] == 0:
                    continue
                R.append((key[0], key[1], key[2] if len(key) > 2 else 0))
                orb.append((u, v))
                t.append(M[u, v])
    return TBModel(bands, np.array(R), np.array(orb), np.array(t), name=name)


def square_c1() -> TBModel:
    """C1: one orbital, NN t=-1.0 eV, NNN t'=0.3 eV, mu=0."""
    terms = {}
    for r in [(1, 0), (-1, 0), (0, 1), (0, -1)]:
        terms[(r[0], r[1], 0)] = np.array([[-1.0 + 0j]])
    for r in [(1, 1), (1, -1), (-1, 1), (-1, -1)]:
        terms[(r[0], r[1], 0)] = np.array([[0.3 + 0j]])
    return _from_terms(terms, 1, "square lattice, t=-1.0, t'=0.3 (C1)")


def _symmetrise(raw: dict, ops, bands) -> dict:
    """t'(r) = 1/|G| sum_g D(g) t(g^-1 r) D(g)^T, then Hermiticity t(-r) = t(r)^H."""
    keys = set(raw)
    for op, _ in ops:
        keys |= {op(k) for k in raw}
    keys |= {(-k[0], -k[1]) for k in keys}
    sym = {}
    for k in keys:
        acc = np.zeros((bands, bands), np.complex128)
        for op, D in ops:
            # find r' with op(r') == k  (op is a bijection on the lattice)
            src = None
            for r0 in raw:
                if op(r0) == k:
                    src = r0
                    break
            if src is not None:
                acc += D @ raw[src] @ D.T
        sym[k] = acc / len(ops)
    herm = {}
    for k in keys:
        mk = (-k[0], -k[1])
        herm[k] = 0.5 * (sym[k] + sym[mk].conj().T)
    return herm


def t2g_c2(seed: int = 2, sigma: float = 0.25) -> TBModel:
    """C2: dxz, dyz, dxy on a square lattice, hoppings to 3rd neighbours ~ N(0, sigma)."""
    rng = np.random.default_rng(seed)
    shells = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (1, -1), (-1, 1), (-1, -1),
              (2, 0), (0, 2), (-2, 0), (0, -2)]
    raw = {r: rng.normal(0.0, sigma, size=(3, 3)) + 0j for r in shells}
    # 90 degree rotation (x,y) -> (-y,x); on (dxz, dyz, dxy): dxz->dyz, dyz->-dxz, dxy->-dxy
    D = np.array([[0, -1, 0], [1, 0, 0], [0, 0, -1]], dtype=np.float64)
    ops = []
    Dn = np.eye(3)
    for n in range(4):
        def op(r, n=n):
            x, y = r
            for _ in range(n):
                x, y = -y, x
            return (x, y)
        ops.append((op, Dn.copy()))
        Dn = D @ Dn
    sym = _symmetrise(raw, ops, 3)
    terms = {(k[0], k[1], 0): v for k, v in sym.items()}
    return _from_terms(terms, 3, "t2g square lattice, seed %d (C2)" % seed)


def bdg(base: TBModel, D, name: str = None) -> TBModel:
    """Bogoliubov-de Gennes form of an electron model for scmodel=true: electron block t(R),
    hole block -conj(t(R)) (the hole Hamiltonian -H(-k)^*), on-site pairing matrix D between
    the blocks; Hermitian whenever the electron model is.  Bands 2b, the particle block first."""
    b = base.bands
    terms = {}
    for R, M in base.terms().items():
        T = np.zeros((2 * b, 2 * b), np.complex128)
        T[:b, :b] = M
        T[b:, b:] = -np.conj(M)
        terms[R] = T
    T0 = terms.get((0, 0, 0), np.zeros((2 * b, 2 * b), np.complex128)).copy()
    T0[:b, b:] += D
    T0[b:, :b] += np.conj(np.asarray(D)).T
    terms[(0, 0, 0)] = T0
    m = _from_terms(terms, 2 * b, name or ("BdG " + base.name))
    m.scmaxbands = b
    return m


def bdg_t2g_c2(seed: int = 2) -> TBModel:
    """Six-band BdG form of the C2 t2g model with an orbital-dependent on-site pairing
    (0.04, 0.04, 0.06 eV on the diagonal, 0.01 eV between dxz and dyz)."""
    D = np.diag([0.04, 0.04, 0.06]).astype(np.complex128)
    D[0, 1] = D[1, 0] = 0.01
    return bdg(t2g_c2(seed), D, "BdG t2g square lattice, seed %d (CJ)" % seed)


def t2g_layered_c2(seed: int = 9) -> TBModel:
    """The C2 model stacked into layers (principal-layer form): in-plane terms at R_z = 0,
    seeded interlayer couplings at R_z = +1 (on site and along x) and their Hermitian partners
    at R_z = -1, for the surface / bulk Green's functions."""
    rng = np.random.default_rng(seed)
    terms = {k: v.copy() for k, v in t2g_c2().terms().items()}
    tz = {(0, 0): 0.15 * (rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))),
          (1, 0): 0.05 * rng.normal(size=(3, 3)) + 0j}
    for (rx, ry), M in tz.items():
        terms[(rx, ry, 1)] = terms.get((rx, ry, 1), 0) + M
        terms[(-rx, -ry, -1)] = terms.get((-rx, -ry, -1), 0) + np.conj(M).T
    return _from_terms(terms, 3, "layered t2g square lattice, seed %d (CS)" % seed)


def t2g_c2_parametrisation(seed: int = 2, sigma: float = 0.25):
    """Independent hopping amplitudes of the C2 model family: the symmetrisation of
    t2g_c2 is linear in the raw shell matrices, so every C4-symmetric Hermitian model with
    the same terms is t = B p for a real orthonormal basis B of that map's range.
    Returns (model, B [nterms][P], p0) with model.t == B @ p0."""
    model = t2g_c2(seed, sigma)
    shells = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (1, -1), (-1, 1), (-1, -1),
              (2, 0), (0, 2), (-2, 0), (0, -2)]
    D = np.array([[0, -1, 0], [1, 0, 0], [0, 0, -1]], dtype=np.float64)
    ops = []
    Dn = np.eye(3)
    for n in range(4):
        def op(r, n=n):
            x, y = r
            for _ in range(n):
                x, y = -y, x
            return (x, y)
        ops.append((op, Dn.copy()))
        Dn = D @ Dn
    index = {(int(model.R[i, 0]), int(model.R[i, 1]), int(model.orb[i, 0]), int(model.orb[i, 1])): i
             for i in range(len(model.t))}
    cols = []
    for s_ in shells:
        for u in range(3):
            for v in range(3):
                raw = {r: np.zeros((3, 3), np.complex128) for r in shells}
                raw[s_][u, v] = 1.0
                sym = _symmetrise(raw, ops, 3)
                col = np.zeros(len(model.t))
                for k, M in sym.items():
                    for a_ in range(3):
                        for c_ in range(3):
                            i = index.get((k[0], k[1], a_, c_))
                            if i is not None:
                                col[i] = M[a_, c_].real
                cols.append(col)
    J = np.array(cols).T
    Uj, S, _ = np.linalg.svd(J, full_matrices=False)
    rank = int(np.sum(S > 1e-10 * S[0]))
    B = Uj[:, :rank]
    p0 = B.T @ model.t.real
    return model, B, p0


def _rot2(th):
    return np.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])


def triangular_c3(seed: int = 3, sigma: float = 0.15, spin: bool = True) -> TBModel:
    """C3: (s, px, py, dx2-y2, dxy) on a triangular lattice to 4th neighbours, C6-symmetric.
    With ``spin`` the model is doubled block-diagonally (10 bands)."""
    rng = np.random.default_rng(seed)
    raw = {}
    for n1 in range(-3, 4):
        for n2 in range(-3, 4):
            d2 = n1 * n1 + n1 * n2 + n2 * n2
            if d2 in (0, 1, 3, 4, 7):
                raw[(n1, n2)] = rng.normal(0.0, sigma, size=(5, 5)) + 0j
    # 60 degree rotation: a1 -> a2, a2 -> a2 - a1, i.e. (n1, n2) -> (-n2, n1 + n2)
    ops = []
    for n in range(6):
        th = n * math.pi / 3.0
        D = np.zeros((5, 5))
        D[0, 0] = 1.0
        D[1:3, 1:3] = _rot2(th)
        D[3:5, 3:5] = _rot2(2 * th)

        def op(r, n=n):
            a, b = r
            for _ in range(n):
                a, b = -b, a + b
            return (a, b)
        ops.append((op, D))
    sym = _symmetrise(raw, ops, 5)
    b = 10 if spin else 5
    terms = {}
    for k, v in sym.items():
        M = np.zeros((b, b), np.complex128)
        M[:5, :5] = v
        if spin:
            M[5:, 5:] = v
        terms[(k[0], k[1], 0)] = M
    return _from_terms(terms, b, "triangular 5-orbital%s, seed %d (C3)" % (" x spin" if spin else "", seed))


# ----------------------------------------------------------------------------- orbitals
def grid(window: int, oversamp: int, centre: float = 0.5):
    """Cache grid of wannierfunctions::precalculate (src/wannierfunctions.cc:433-442):
    point i sits at reduced coordinate i/os - w - 0.5."""
    side = (2 * window + 1) * oversamp
    g = np.arange(side) / oversamp - float(window) - centre
    return np.meshgrid(g, g, indexing="ij")


def gaussian_c1(window=2, oversamp=8, sigma=0.3, z=0.5) -> np.ndarray:
    """Normalised 3D Gaussian psi(r) = (pi sigma^2)^(-3/4) exp(-r^2 / (2 sigma^2)) at height z."""
    X, Y = grid(window, oversamp)
    r2 = X * X + Y * Y + z * z
    return ((math.pi * sigma * sigma) ** -0.75 * np.exp(-r2 / (2 * sigma * sigma)))[None]


def _radial(r2, sigma):
    norm = math.sqrt(4.0 / (math.sqrt(math.pi) * sigma ** 3))
    return norm * np.exp(-r2 / (2 * sigma * sigma))


def t2g_orbitals_c2(window=2, oversamp=10, sigma=0.4, z=0.6) -> np.ndarray:
    """dxz, dyz, dxy: real-harmonic angular part times a radial Gaussian, at height z."""
    X, Y = grid(window, oversamp)
    r2 = X * X + Y * Y + z * z
    c = math.sqrt(15.0 / 4.0 / math.pi)
    rad = _radial(r2, sigma)
    return np.stack([c * X * z / r2 * rad, c * Y * z / r2 * rad, c * X * Y / r2 * rad])


def tri_orbitals_c3(window=2, oversamp=6, seed=3, sigma=0.45, z=0.6) -> np.ndarray:
    """Five orbitals on the triangular lattice (basis a1=(1,0), a2=(1/2, sqrt3/2)): each a
    seed-drawn mixture of s, p, d angular parts times a radial Gaussian."""
    rng = np.random.default_rng(seed + 100)
    U, V = grid(window, oversamp)
    X = U + 0.5 * V
    Y = (math.sqrt(3.0) / 2.0) * V
    r2 = X * X + Y * Y + z * z
    r = np.sqrt(r2)
    rad = _radial(r2, sigma)
    basis = [
        np.full_like(X, 1.0 / math.sqrt(4 * math.pi)),
        math.sqrt(3 / (4 * math.pi)) * X / r,
        math.sqrt(3 / (4 * math.pi)) * Y / r,
        math.sqrt(3 / (4 * math.pi)) * z / r,
        math.sqrt(15 / (16 * math.pi)) * (X * X - Y * Y) / r2,
        math.sqrt(15 / (4 * math.pi)) * X * Y / r2,
        math.sqrt(5 / (16 * math.pi)) * (3 * z * z - r2) / r2,
    ]
    out = []
    for o in range(5):
        c = rng.normal(0.0, 0.3, size=len(basis))
        c[[0, 1, 2, 4, 5][o]] += 1.0
        ang = sum(ci * bi for ci, bi in zip(c, basis))
        out.append(ang * rad)
    return np.stack(out)


# ----------------------------------------------------------------------------- configs
@dataclass
class Config:
    name: str
    lattice: int
    kpoints: int
    oversamp: int
    window: int
    layers: int
    energies: tuple
    eta: float
    scattering: tuple
    spin: bool = False
    efermi: float = 0.0
    extra: dict = field(default_factory=dict)

    @property
    def pixels_per_energy(self):
        return (self.lattice * self.oversamp) ** 2

    def energy_list(self):
        lo, hi = self.energies
        L = self.layers
        if L == 1:
            return np.array([lo])
        return np.array([(hi - lo) * k / (L - 1.0) + lo for k in range(L)])


def config(name: str) -> tuple:
    """(Config, TBModel, orbital cube [m, side, side]) for C1, C2, C3, C5, CJ (Josephson) or CS
    (surface Green's function)."""
    if name == "C1":
        c = Config("C1", 64, 256, 8, 2, 21, (-0.2, 0.2), 0.005, (0.5,))
        return c, square_c1(), gaussian_c1(c.window, c.oversamp)
    if name == "C2":
        c = Config("C2", 256, 1024, 10, 2, 101, (-0.1, 0.1), 0.002, (0.3, 0.3, 0.5))
        return c, t2g_c2(), t2g_orbitals_c2(c.window, c.oversamp)
    if name == "C3":
        c = Config("C3", 512, 2048, 6, 2, 64, (-0.1, 0.1), 0.001, tuple([1.0] * 10), spin=True)
        orbs = tri_orbitals_c3(c.window, c.oversamp)
        return c, triangular_c3(), np.concatenate([orbs, orbs])
    if name == "CJ":
        # Josephson mode (output=josephson) on the BdG form of the C2 model: C2 grid and field of
        # view, tip gap 1 meV (the reference's default deltat), tip broadening = eta; scattering
        # duplicated into the hole block with magscat = 0 (src/calcqpi.cc:281-286)
        c = Config("CJ", 256, 1024, 10, 2, 101, (-0.1, 0.1), 0.002, (0.3, 0.3, 0.5, -0.3, -0.3, -0.5),
                   extra={"josephson": (0.001, 0.002), "maxband": 3})
        return c, bdg_t2g_c2(), t2g_orbitals_c2(c.window, c.oversamp)
    if name == "CS":
        # surface Green's function (green=surface) of the layered C2 model: C2 grid and field of
        # view, 21 energies
        c = Config("CS", 256, 1024, 10, 2, 21, (-0.1, 0.1), 0.002, (0.3, 0.3, 0.5),
                   extra={"green": "surface", "epserr": 1e-5})
        return c, t2g_layered_c2(), t2g_orbitals_c2(c.window, c.oversamp)
    if name == "C5":
        c = Config("C5", 128, 1024, 10, 2, 41, (-0.1, 0.1), 0.002, (0.3, 0.3, 0.5))
        return c, t2g_c2(), t2g_orbitals_c2(c.window, c.oversamp)
    raise KeyError(name)
