"""CPU oracle for the CalcQPI continuum-LDOS path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference leg
may import this module -- as the checker, or as the timed CPU baseline -- never the
product.  It wraps two independent restatements of the reference's CPU algorithm:

* ``liboracle.so`` built from ``oracle/cqpi_oracle.c`` (OpenMP C, direct O(W^2) form of
  src/qpi.cc:876-950, the same loop nest as the reference), and
* ``np_*`` functions: a NumPy/SciPy restatement (``numpy.linalg.eigh``, ``numpy.fft``)
  used to cross-check the C restatement on small cases.

Parity pin: both are checked in tests/test_oracle.py against golden outputs of the
reference's own sources (tests/golden/, written by tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile oracle/cqpi_oracle.c into oracle/_build/liboracle.so (gcc -O2 -fopenmp)."""
    src = os.path.join(HERE, "cqpi_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.c_void_p
            i32, i64, dbl = ctypes.c_int, ctypes.c_int64, ctypes.c_double
            L.orc_hk.argtypes = [i32, i64, P, P, P, P, dbl, i32, dbl, dbl, P]
            L.orc_bands.argtypes = [i32, i64, P, P, P, P, dbl, i32, i32, P, P]
            L.orc_greens_k.argtypes = [i32, i32, P, P, dbl, dbl, P]
            L.orc_fft_backward_2d.argtypes = [i32, i32, P]
            L.orc_tmatrix.argtypes = [i32, P, P, P]
            L.orc_tmatrix.restype = i32
            L.orc_wannier_ldos.argtypes = [i32, i32, i32, i32, i32, i32, i32, P, P, P, P, P, i32, i32]
            L.orc_wannier_josephson.argtypes = [i32, i32, i32, i32, i32, i32, P, P, P, P, dbl, dbl, P, i32, i32]
            L.orc_josephson_tip.argtypes = [dbl, dbl, dbl, P]
            L.orc_threshold_list.argtypes = [i32, i32, i32, P, dbl, i32, i32, P, P, P, i64]
            L.orc_threshold_list.restype = i64
            L.orc_wannier_ldos_list.argtypes = [i32, i32, i32, i32, i32, P, P, i64, P, P, P, i32, i32]
            L.orc_surface_greens_k.argtypes = [i32, i32, i64, P, P, P, P, i64, P, P, P, P, i64, P, P, P, P,
                                               dbl, i32, dbl, dbl, dbl, i32, i32, P]
            L.orc_surface_greens_k.restype = i64
            L.orc_num_threads.restype = i32
            L.orc_set_threads.argtypes = [i32]
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Model:
    """Tight-binding model as parsed by tightbind::readfile (src/tightbinding.cc:70-149)."""

    def __init__(self, bands, R, orb, t, anti=None, efermi=0.0, scmaxbands=None, name="model"):
        self.bands = int(bands)
        self.R = np.ascontiguousarray(R, dtype=np.int32).reshape(-1, 3)
        self.orb = np.ascontiguousarray(orb, dtype=np.int32).reshape(-1, 2)
        self.t = np.ascontiguousarray(t, dtype=np.complex128).reshape(-1)
        self.anti = np.ascontiguousarray(
            np.zeros(len(self.t), bool) if anti is None else anti, dtype=np.uint8)
        self.efermi = float(efermi)
        self.scmaxbands = self.bands if scmaxbands is None else int(scmaxbands)
        self.name = name

    @classmethod
    def from_hr(cls, parsed, efermi=0.0):
        return cls(parsed["bands"], parsed["R"], parsed["orb"], parsed["t"], parsed["anti"],
                   efermi, parsed["scmaxbands"], parsed["name"])


# --------------------------------------------------------------------------- C oracle
def hk(model: Model, kx: float, ky: float) -> np.ndarray:
    H = np.zeros((model.bands, model.bands), np.complex128)
    lib().orc_hk(model.bands, len(model.t), _p(model.R), _p(model.orb), _p(model.t), _p(model.anti),
                 model.efermi, model.scmaxbands, kx, ky, _p(H))
    return H


def bands(model: Model, kp: int):
    """tmatrix::calchamiltonian, src/qpi.cc:454-475.  eval[kp*kp, b], evec[kp*kp, b, b]."""
    b = model.bands
    ev = np.zeros((kp * kp, b), np.float64)
    U = np.zeros((kp * kp, b, b), np.complex128)
    lib().orc_bands(b, len(model.t), _p(model.R), _p(model.orb), _p(model.t), _p(model.anti),
                    model.efermi, model.scmaxbands, kp, _p(ev), _p(U))
    return ev, U


def greens_k(ev, U, kp: int, omega: float, eta: float) -> np.ndarray:
    """tightbinding.cc:282-289 over all k (qpi.cc:478-486).  Returns g0[kp, kp, b, b]."""
    b = ev.shape[1]
    g = np.zeros((kp, kp, b, b), np.complex128)
    lib().orc_greens_k(b, kp, _p(ev), _p(U), omega, eta, _p(g))
    return g


def realspace(g0k: np.ndarray) -> np.ndarray:
    """tmatrix::calcrealspacegreensfunction, src/qpi.cc:557-578 (returns a new array)."""
    g = np.ascontiguousarray(g0k, dtype=np.complex128).copy()
    kp, b = g.shape[0], g.shape[2]
    lib().orc_fft_backward_2d(kp, b, _p(g))
    return g


def tmatrix(vscat, g00) -> np.ndarray:
    """tmatrix::setscatteringmatrix, src/qpi.cc:833-854."""
    v = np.ascontiguousarray(vscat, dtype=np.complex128)
    g = np.ascontiguousarray(g00, dtype=np.complex128)
    b = len(v)
    T = np.zeros((b, b), np.complex128)
    rc = lib().orc_tmatrix(b, _p(v), _p(g), _p(T))
    if rc != 0:
        raise ZeroDivisionError("singular 1 - V G0(0)")
    return T


def wannier_ldos(n, kp, os_, w, m, spin, T, g0r, wf, wf_zero=None, rows=None) -> np.ndarray:
    """tmatrix::calcwannierldos (CPU), src/qpi.cc:876-950.  Returns ldos[x][y] (float64)."""
    b = g0r.shape[2]
    wf = np.ascontiguousarray(wf, dtype=np.float64)
    z = np.ascontiguousarray(np.zeros(wf.shape[0], np.uint8) if wf_zero is None else wf_zero, dtype=np.uint8)
    T = np.ascontiguousarray(T, dtype=np.complex128)
    g0r = np.ascontiguousarray(g0r, dtype=np.complex128)
    out = np.zeros((n * os_, n * os_), np.float64)
    r0, r1 = (0, n) if rows is None else rows
    lib().orc_wannier_ldos(n, kp, b, os_, w, m, int(bool(spin)), _p(T), _p(g0r), _p(wf), _p(z), _p(out),
                           r0, r1)
    return out


def josephson_tip(energy, deltat, etat) -> complex:
    """The driver's Josephson tip factor, src/calcqpi.cc:705-708."""
    t = np.zeros(2, np.float64)
    lib().orc_josephson_tip(float(energy), float(deltat), float(etat), _p(t))
    return complex(t[0], t[1])


def wannier_josephson(n, kp, os_, w, spin, T, g0r, wf, tip, wf_zero=None, rows=None) -> np.ndarray:
    """tmatrix::calcwannierjosephson (CPU), src/qpi.cc:953-1033.  Returns ldos[x][y] (float64)."""
    b = g0r.shape[2]
    wf = np.ascontiguousarray(wf, dtype=np.float64)
    z = np.ascontiguousarray(np.zeros(wf.shape[0], np.uint8) if wf_zero is None else wf_zero, dtype=np.uint8)
    if wf.shape[0] < b >> 1:
        raise ValueError("Josephson mode needs bands/2 orbitals")
    T = np.ascontiguousarray(T, dtype=np.complex128)
    g0r = np.ascontiguousarray(g0r, dtype=np.complex128)
    out = np.zeros((n * os_, n * os_), np.float64)
    r0, r1 = (0, n) if rows is None else rows
    lib().orc_wannier_josephson(n, kp, b, os_, w, int(bool(spin)), _p(T), _p(g0r), _p(wf), _p(z),
                                float(tip.real), float(tip.imag), _p(out), r0, r1)
    return out


def threshold_list(w, os_, wf, threshold, maxband=0, spin=False, spinarr=None):
    """mkthresholdlist, src/qpi.cc:139-253: (entries [k][5] int32 = (list, i, j, o1, o2),
    factors [k]), lists contiguous in the reference's order."""
    wf = np.ascontiguousarray(wf, dtype=np.float64)
    sa = None
    if spinarr is not None:   # spinarr.resize(orbitals, 0), qpi.cc:217
        sa = np.zeros(wf.shape[0], np.int32)
        k = min(len(spinarr), wf.shape[0])
        sa[:k] = np.asarray(spinarr, np.int32)[:k]
    args = (w, os_, wf.shape[0], _p(wf), float(threshold), int(maxband), int(bool(spin)),
            None if sa is None else _p(sa))
    n = lib().orc_threshold_list(*args, None, None, 0)
    ent = np.zeros((max(n, 1), 5), np.int32)
    fac = np.zeros(max(n, 1), np.float64)
    lib().orc_threshold_list(*args, _p(ent), _p(fac), n)
    return ent[:n], fac[:n]


def wannier_ldos_list(n, kp, os_, w, T, g0r, ent, fac, rows=None) -> np.ndarray:
    """tmatrix::calcwannierldos(os, w, flaglist) (CPU), src/qpi.cc:1085-1134; ldos[x][y]."""
    b = g0r.shape[2]
    T = np.ascontiguousarray(T, dtype=np.complex128)
    g0r = np.ascontiguousarray(g0r, dtype=np.complex128)
    ent = np.ascontiguousarray(ent, dtype=np.int32)
    fac = np.ascontiguousarray(fac, dtype=np.float64)
    out = np.zeros((n * os_, n * os_), np.float64)
    r0, r1 = (0, n) if rows is None else rows
    lib().orc_wannier_ldos_list(n, kp, b, os_, w, _p(T), _p(g0r), len(fac), _p(ent), _p(fac), _p(out), r0, r1)
    return out


def _split(model: Model, sel):
    R = np.ascontiguousarray(model.R[sel])
    o = np.ascontiguousarray(model.orb[sel])
    t = np.ascontiguousarray(model.t[sel])
    a = np.ascontiguousarray(model.anti[sel])
    return len(t), R, o, t, a


def surface_greens_k(model: Model, kp: int, omega: float, eta: float, epserr: float, surface: bool,
                     smodel: Model = None, max_iter: int = 1000) -> np.ndarray:
    """tmatrix::calcsurfacegreensfunction, src/qpi.cc:488-554 (green=surface / bulk):
    g0[kp, kp, b, b].  Raises if a k-point does not converge within max_iter."""
    b = model.bands
    nb_, Rb, ob, tb, ab = _split(model, model.R[:, 2] == 0)
    no, Ro, oo, to, ao = _split(model, model.R[:, 2] < 0)
    if smodel is not None:
        ns, Rs, os_, ts, as_ = _split(smodel, smodel.R[:, 2] == 0)
    else:
        ns, Rs, os_, ts, as_ = -1, Rb, ob, tb, ab
    g = np.zeros((kp, kp, b, b), np.complex128)
    bad = lib().orc_surface_greens_k(b, kp, nb_, _p(Rb), _p(ob), _p(tb), _p(ab), no, _p(Ro), _p(oo), _p(to),
                                     _p(ao), ns, _p(Rs), _p(os_), _p(ts), _p(as_), model.efermi,
                                     model.scmaxbands, omega, eta, epserr, int(bool(surface)), max_iter, _p(g))
    if bad:
        raise RuntimeError("%d k-points did not converge" % bad)
    return g


def spf(g0k: np.ndarray, maxband: int, shift: bool = True) -> np.ndarray:
    """tmatrix::calcspf, src/qpi.cc:659-683: ldos[x][y] = -sum_{l<maxband} Im G0(k)_ll with
    k = (x + kp/2) mod kp (shift)."""
    kp = g0k.shape[0]
    tr = -np.imag(np.einsum("ijll->ij", g0k[:, :, :maxband, :maxband]))
    ks = kp >> 1 if shift else 0
    idx = (np.arange(kp) + ks) % kp
    return tr[np.ix_(idx, idx)]


def band_histogram(model: "Model", pix: int, oversamp: int, le: float, ue: float, layers: int) -> np.ndarray:
    """tightbind::calcbst3dhisthr(fname, pix, le, ue, layers, oversamp),
    src/tightbinding.cc:1158-1193 (the driver's bsfile, src/calcqpi.cc:308-326): eigenvalues
    (numpy.linalg.eigvalsh on the lower triangle, as gsl_eigen_hermv reads it) of H(k) with the
    Fermi-energy diagonal (tightbind::setmatrix, src/tightbinding.cc:210-219; all terms at
    k_z = 0) on the (pix*oversamp)^2 grid k = (io, jo) / (pix*oversamp - 1) - 1/2; each
    eigenvalue within two bins of [le, ue] adds the Lorentzian of width w = 2 (ue - le) / layers
    (class lorentzian, src/tightbinding.h:42-49) at the layer energies (idl::getbias) to the
    nearest layer and its two neighbours (idl::getbiasindex) of pixel (io/oversamp,
    jo/oversamp).  Returns [layers][y][x]."""
    b = model.bands
    R = np.asarray(model.R).reshape(-1, 3)
    orb = np.asarray(model.orb).reshape(-1, 2)
    t = np.asarray(model.t, np.complex128).reshape(-1)
    anti = np.asarray(model.anti if model.anti is not None else np.zeros(len(t)), bool).reshape(-1)
    scmax = model.scmaxbands if model.scmaxbands is not None else b
    osp = pix * oversamp
    out = np.zeros((layers, pix, pix))
    binsize = (ue - le) / (layers - 1) if layers > 1 else np.inf
    w = (ue - le) / layers * 2.0
    diag = np.array([-model.efermi if d < scmax else model.efermi for d in range(b)], np.complex128)
    for io in range(osp):
        for jo in range(osp):
            kx, ky = io / (osp - 1) - 0.5, jo / (osp - 1) - 0.5
            H = np.diag(diag)
            ph = 2 * np.pi * (R[:, 0] * kx + R[:, 1] * ky)
            np.add.at(H, (orb[:, 0], orb[:, 1]), t * np.exp(1j * np.where(anti, -ph, ph)))
            for e in np.linalg.eigvalsh(H, UPLO="L"):
                if not (le - 2 * binsize < e < ue + 2 * binsize):
                    continue
                lay = int(np.round((e - le) / (ue - le) * (layers - 1))) if layers > 1 else 0
                for nl in (lay - 1, lay, lay + 1):
                    if 0 <= nl < layers:
                        x = ((ue - le) * nl / (layers - 1) + le if layers > 1 else le) - e
                        out[nl, jo // oversamp, io // oversamp] += w / 2 / (x * x + w * w / 4) / np.pi
    return out


def uspf(g0k: np.ndarray, n: int, maxband: int, pos, prearr, spin: bool = False) -> np.ndarray:
    """tmatrix::calcuspf, src/qpi.cc:735-775: the spectral function unfolded with the orbital
    positions, ldos[i][j] = -sum_{k,l} pre_k pre_l Im(G0(ki,kj)[l][k] e^{2 pi i (kx dx + ky dy)}),
    dx = pos_k - pos_l, kx = (i - n/2)/kp, ki = ((i + n/2) mod n) mod kp (spin: two blocks)."""
    kp = g0k.shape[0]
    h = n >> 1
    out = np.zeros((n, n))
    pos = np.asarray(pos, np.float64)
    pre = np.asarray(prearr, np.float64)
    blocks = [range(0, maxband >> 1), range(maxband >> 1, 2 * (maxband >> 1))] if spin else [range(maxband)]
    for i in range(n):
        kx = (i - h) / kp
        ki = ((i + h) % n) % kp
        for j in range(n):
            ky = (j - h) / kp
            kj = ((j + h) % n) % kp
            tr = 0.0
            for blk in blocks:
                for k in blk:
                    for l in blk:
                        ph = np.exp(1j * 2.0 * np.pi * (kx * (pos[k][0] - pos[l][0]) + ky * (pos[k][1] - pos[l][1])))
                        tr -= pre[k] * pre[l] * np.imag(g0k[ki, kj, l, k] * ph)
            out[i, j] = tr
    return out


def set_threads(nt: int):
    lib().orc_set_threads(int(nt))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def run(model: Model, n, kp, os_, w, eta, energies, vscat, wf, wf_zero=None, m=None, spin=False, josephson=None,
        threshold=None, spinarr=None, green=None, epserr=1e-5, smodel=None, output="wannier", pos=None,
        prearr=None):
    """The reference's wannier-mode energy loop (src/calcqpi.cc:673-760, normal Green's
    function): eigen once, then per energy G0(k) -> G0(R) -> T -> LDOS.  Returns maps in
    IDL file order [layer][y][x], float64.  josephson=(deltat, etat) runs the driver's
    josephson mode instead (calcqpi.cc:705-709); threshold (and spinarr) the proximity-list
    form of the wannier mode (calcqpi.cc:619-635,700-701)."""
    m = model.bands if m is None else m
    ev, U = bands(model, kp) if green not in ("surface", "bulk") else (None, None)
    maps = []
    if threshold is not None and josephson is None:
        wz = np.asarray(wf, np.float64) if wf_zero is None else \
            np.asarray(wf, np.float64) * (1 - np.asarray(wf_zero, np.float64)[:len(wf), None, None])
        ent, fac = threshold_list(w, os_, wz, threshold, m, spin, spinarr)
    if output in ("spf", "uspf"):   # src/calcqpi.cc:675-717: G0(k) only, no transform
        for e in energies:
            if green in ("surface", "bulk"):
                g0k = surface_greens_k(model, kp, e, eta, epserr, green == "surface", smodel)
            else:
                g0k = greens_k(ev, U, kp, e, eta)
            if output == "spf":
                maps.append(spf(g0k, m).T)
            else:
                maps.append(uspf(g0k, n, m, pos, prearr, spin).T)
        return np.stack(maps)
    for e in energies:
        if green in ("surface", "bulk"):   # src/calcqpi.cc:675-693
            g0r = realspace(surface_greens_k(model, kp, e, eta, epserr, green == "surface", smodel))
        else:
            g0r = realspace(greens_k(ev, U, kp, e, eta))
        T = tmatrix(vscat, g0r[0, 0])
        if threshold is not None and josephson is None:
            maps.append(wannier_ldos_list(n, kp, os_, w, T, g0r, ent, fac).T)
        elif josephson is not None:
            tip = josephson_tip(e, josephson[0], josephson[1])
            maps.append(wannier_josephson(n, kp, os_, w, spin, T, g0r, wf, tip, wf_zero).T)
        else:
            maps.append(wannier_ldos(n, kp, os_, w, m, spin, T, g0r, wf, wf_zero).T)
    return np.stack(maps)


# --------------------------------------------------------------------------- NumPy cross-check
def np_hk_grid(model: Model, kp: int) -> np.ndarray:
    cut = kp >> 1
    i = np.arange(kp)
    x = np.where(i > cut, (i - kp) / kp, i / kp)
    KX, KY = np.meshgrid(x, x, indexing="ij")
    b = model.bands
    H = np.zeros((kp, kp, b, b), np.complex128)
    for d in range(b):
        H[:, :, d, d] = -model.efermi if d < model.scmaxbands else model.efermi
    for h in range(len(model.t)):
        ph = 2 * np.pi * (model.R[h, 0] * KX + model.R[h, 1] * KY)
        if model.anti[h]:
            ph = -ph
        H[:, :, model.orb[h, 0], model.orb[h, 1]] += model.t[h] * np.exp(1j * ph)
    return H


def np_greens_r(model: Model, kp: int, omega: float, eta: float) -> np.ndarray:
    """G0(R) via eigh + numpy.fft, with the reference's sign and scale (qpi.cc:557-578)."""
    H = np_hk_grid(model, kp)
    ev, U = np.linalg.eigh(H)
    fac = 1.0 / (omega - ev + 1j * eta)
    G = np.einsum("xyon,xyn,xyan->xyoa", U, fac, U.conj())
    return np.fft.ifft2(G, axes=(0, 1))


def np_wannier_ldos(n, kp, os_, w, m, spin, T, g0r, wf, wf_zero=None) -> np.ndarray:
    """Direct double window sum of qpi.cc:889-948, vectorised over sub-pixels."""
    b = g0r.shape[2]
    wn = n * os_
    z = np.zeros(wf.shape[0], bool) if wf_zero is None else np.asarray(wf_zero, bool)
    out = np.zeros((wn, wn))
    n2 = n >> 1
    if spin:
        sb = m >> 1
        blocks = [range(0, sb), range(sb, 2 * sb)]
    else:
        blocks = [range(0, m)]
    offs = [(a, c) for a in range(-w, w + 1) for c in range(-w, w + 1)]
    sub = np.arange(os_)
    for i in range(n):
        for j in range(n):
            ip, jp = i - n2, j - n2
            acc = np.zeros((os_, os_))
            for d1 in offs:
                buf = T @ g0r[(-(ip + d1[0])) % kp, (-(jp + d1[1])) % kp]
                x1 = sub + w * os_ - d1[0] * os_
                y1 = sub + w * os_ - d1[1] * os_
                for d2 in offs:
                    cl = g0r[(ip + d2[0]) % kp, (jp + d2[1]) % kp] @ buf
                    gd = g0r[(d2[0] - d1[0]) % kp, (d2[1] - d1[1]) % kp]
                    x2 = sub + w * os_ - d2[0] * os_
                    y2 = sub + w * os_ - d2[1] * os_
                    for blk in blocks:
                        for o1 in blk:
                            if z[o1]:
                                continue
                            for o2 in blk:
                                if z[o2]:
                                    continue
                                f = wf[o1][np.ix_(x1, y1)] * wf[o2][np.ix_(x2, y2)]
                                acc -= (cl[o2, o1].imag + gd[o2, o1].imag) * f
            out[i * os_:(i + 1) * os_, j * os_:(j + 1) * os_] = acc
    return out


# --------------------------------------------------------------------------- orbitals
ORBITAL_NAMES = ["s", "px", "py", "pz", "dx2", "dxy", "dxz", "dyz", "dr2", "fy3x2", "fxyz", "fyz2",
                 "fz3", "fxz2", "fzx2", "fxx2", "n", "z"]


def orbital_value(name, x, y, width, height, xpos=0.0, ypos=0.0, theta=0.0, phi=0.0, prefact=1.0,
                  symmetry=4.0):
    """wannierfunctions::getwave(x,y), src/wannierfunctions.cc:126-221 with the orbital
    formulas of :21-124 (Slater radial exp(-r/width) times real angular parts)."""
    x = np.asarray(x, np.float64) - xpos
    y = np.asarray(y, np.float64) - ypos
    z = np.zeros_like(x) - height
    if name == "z":
        return np.zeros_like(x)
    if name != "s" and (theta != 0.0 or phi != 0.0):
        xc, yc, zc = x, y, z
        x = xc * np.cos(theta) + yc * np.sin(theta) * np.cos(phi) + zc * np.sin(theta) * np.sin(phi)
        y = -xc * np.sin(theta) + yc * np.cos(theta) * np.cos(phi) + zc * np.cos(theta) * np.sin(phi)
        z = -np.sin(phi) * yc + np.cos(phi) * zc
    r = np.sqrt(x * x + y * y + z * z)
    ex = prefact * np.exp(-r / width)
    with np.errstate(divide="ignore", invalid="ignore"):
        if name == "s":
            v = ex / np.sqrt(4.0 * np.pi)
            return v
        if name == "n":
            sc = np.cos(symmetry * np.arctan2(x, y) / 2.0)
            return ex * sc * sc * r / width
        table = {
            "px": lambda: x / r * np.sqrt(3.0 / 4.0 / np.pi),
            "py": lambda: y / r * np.sqrt(3.0 / 4.0 / np.pi),
            "pz": lambda: z / r * np.sqrt(3.0 / 4.0 / np.pi),
            "dx2": lambda: (x * x - y * y) / 2.0 / r / r * np.sqrt(15.0 / 4.0 / np.pi),
            "dxy": lambda: x * y / r / r * np.sqrt(15.0 / 4.0 / np.pi),
            "dxz": lambda: x * z / r / r * np.sqrt(15.0 / 4.0 / np.pi),
            "dyz": lambda: y * z / r / r * np.sqrt(15.0 / 4.0 / np.pi),
            "dr2": lambda: (3.0 * z * z - r * r) / 4.0 / r / r * np.sqrt(5.0 / np.pi),
            "fy3x2": lambda: y * (3.0 * x * x - y * y) / 4.0 / r / r / r * np.sqrt(35.0 / 2.0 / np.pi),
            "fxyz": lambda: x * y * z / r / r / r * np.sqrt(105.0 / 4.0 / np.pi),
            "fyz2": lambda: y * (5.0 * z * z - r * r) / r / r / r / 4.0 * np.sqrt(21.0 / 2.0 / np.pi),
            "fz3": lambda: (5.0 * z * z * z - 3.0 * z * r * r) / r / r / r / 4.0 * np.sqrt(7.0 / np.pi),
            "fxz2": lambda: x * (5.0 * z * z - r * r) / 4.0 / r / r / r * np.sqrt(21.0 / 2.0 / np.pi),
            "fzx2": lambda: z * (x * x - y * y) / r / r / r / 4.0 * np.sqrt(105.0 / np.pi),
            "fxx2": lambda: x * (x * x - 3.0 * y * y) / 4.0 / r / r / r * np.sqrt(35.0 / 2.0 / np.pi),
        }
        ang = table[name]()
    return np.where(r == 0.0, 0.0, ex * ang)


def orbital_cache(name, window, oversamp, **kw) -> np.ndarray:
    """wannierfunctions::precalculate, src/wannierfunctions.cc:433-442."""
    side = (2 * window + 1) * oversamp
    i = np.arange(side, dtype=np.float64)
    g = i / oversamp - float(window) - 0.5
    X, Y = np.meshgrid(g, g, indexing="ij")
    return orbital_value(name, X, Y, **kw)
