"""Python binding of libcqpi.so (the engine's C ABI, include/cqpi.h) via ctypes.

This is a thin wrapper for tests, the benchmark and the fitting harness; the drop-in
product is the C ABI itself and the calcqpi CLI.  Every call goes to the CUDA library;
there is no CPU fallback: if the library is missing or no GPU is visible, the calls
raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libcqpi.so")

(OK, ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_DOMAIN, ERR_SINGULAR, ERR_STATE, ERR_NOT_SUPPORTED, ERR_NO_DEVICE, ERR_TIMEOUT,
 ERR_NOT_CONVERGED) = range(11)
GREEN_NORMAL, GREEN_SURFACE, GREEN_BULK = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1

EXPORTED = [
    "cqpi_create", "cqpi_destroy", "cqpi_last_error", "cqpi_status_string", "cqpi_version",
    "cqpi_set_orbitals", "cqpi_set_scattering", "cqpi_set_impurities", "cqpi_solve_bands", "cqpi_run",
    "cqpi_wannierldos", "cqpi_retrieve_result", "cqpi_get_bands", "cqpi_get_greens_box", "cqpi_get_tmatrix",
    "cqpi_get_stream", "cqpi_synchronize", "cqpi_kernel_launches", "cqpi_stage_times", "cqpi_measure_fma_peak",
    "cqpi_contraction_kind", "cqpi_realspace_greens_noalloc", "cqpi_set_hoppings", "cqpi_adjoint", "cqpi_run_fov",
    "cqpi_graph_begin", "cqpi_graph_end", "cqpi_graph_launch", "cqpi_autotune", "cqpi_set_josephson",
    "cqpi_wannierjosephson", "cqpi_set_threshold", "cqpi_wannierldoslist", "cqpi_set_list", "cqpi_set_greens",
    "cqpi_spf", "cqpi_uspf", "cqpi_dos",
]


class CqpiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cqpi status {code}: {msg}")
        self.code = code


class _Model(ctypes.Structure):
    _fields_ = [("bands", ctypes.c_int32), ("scmaxbands", ctypes.c_int32), ("efermi", ctypes.c_double),
                ("nhops", ctypes.c_int64), ("R", ctypes.c_void_p), ("orb", ctypes.c_void_p),
                ("t", ctypes.c_void_p), ("anti", ctypes.c_void_p)]


class _Params(ctypes.Structure):
    _fields_ = [("lattice", ctypes.c_int32), ("kpoints", ctypes.c_int32), ("oversamp", ctypes.c_int32),
                ("window", ctypes.c_int32), ("maxband", ctypes.c_int32), ("spin", ctypes.c_int32),
                ("eta", ctypes.c_double), ("precision", ctypes.c_int32)]


_lib = None


def library_path() -> str:
    return LIB_PATH


def load():
    """Load libcqpi.so (build it first with cqpi_build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libcqpi.so not built ({LIB_PATH}); run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    P, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    L.cqpi_create.argtypes = [ctypes.POINTER(_Model), ctypes.POINTER(_Params), ctypes.POINTER(P)]
    L.cqpi_destroy.argtypes = [P]
    L.cqpi_last_error.argtypes = [P]
    L.cqpi_last_error.restype = ctypes.c_char_p
    L.cqpi_status_string.argtypes = [ctypes.c_int]
    L.cqpi_status_string.restype = ctypes.c_char_p
    L.cqpi_version.restype = ctypes.c_char_p
    L.cqpi_set_orbitals.argtypes = [P, P, i32, i32, P]
    L.cqpi_set_scattering.argtypes = [P, P]
    L.cqpi_set_impurities.argtypes = [P, P, i32]
    L.cqpi_solve_bands.argtypes = [P]
    L.cqpi_run.argtypes = [P, P, i32, P, P, i32]
    L.cqpi_wannierldos.argtypes = [P, P, P]
    L.cqpi_retrieve_result.argtypes = [P, P]
    L.cqpi_get_bands.argtypes = [P, P, P]
    L.cqpi_get_greens_box.argtypes = [P, dbl, P, ctypes.POINTER(i32)]
    L.cqpi_get_tmatrix.argtypes = [P, dbl, P]
    L.cqpi_get_stream.argtypes = [P, ctypes.POINTER(P)]
    L.cqpi_synchronize.argtypes = [P]
    L.cqpi_kernel_launches.argtypes = [P, ctypes.POINTER(i64)]
    L.cqpi_stage_times.argtypes = [P, P]
    L.cqpi_measure_fma_peak.argtypes = [i32, ctypes.POINTER(dbl)]
    L.cqpi_contraction_kind.argtypes = [P, ctypes.POINTER(i32)]
    L.cqpi_realspace_greens_noalloc.argtypes = [P, i32, i32, i32, P, P]
    L.cqpi_set_hoppings.argtypes = [P, P]
    L.cqpi_run_fov.argtypes = [P, P, i32, P, P, i32]
    L.cqpi_graph_begin.argtypes = [P]
    L.cqpi_graph_end.argtypes = [P]
    L.cqpi_graph_launch.argtypes = [P]
    L.cqpi_autotune.argtypes = [P, P, i32, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(i32)]
    L.cqpi_adjoint.argtypes = [P, P, i32, P, i32, P, P]
    L.cqpi_set_josephson.argtypes = [P, i32, dbl, dbl]
    L.cqpi_wannierjosephson.argtypes = [P, P, P, P]
    L.cqpi_set_threshold.argtypes = [P, dbl, P, i32, ctypes.POINTER(i64)]
    L.cqpi_wannierldoslist.argtypes = [P, P, P]
    L.cqpi_set_list.argtypes = [P, i64, P, P]
    L.cqpi_set_greens.argtypes = [P, i32, dbl, P]
    L.cqpi_spf.argtypes = [P, P, i32, i32, P, P]
    L.cqpi_uspf.argtypes = [P, P, i32, i32, P, P, P, P]
    L.cqpi_dos.argtypes = [P, P, i32, i32, P]
    _lib = L
    return L


def measure_fma_peak(kind: str) -> float:
    """Measured CUDA-core FMA peak in TFLOP/s ('fp64' or 'fp32')."""
    L = load()
    v = ctypes.c_double()
    rc = L.cqpi_measure_fma_peak({"fp64": 0, "fp32": 1}[kind], ctypes.byref(v))
    if rc != OK:
        raise CqpiError(rc, L.cqpi_status_string(rc).decode())
    return v.value


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Engine:
    """One engine handle: a model, the run parameters, the eigen cache and device buffers."""

    def __init__(self, model, lattice, kpoints, oversamp, window, eta, maxband=None, spin=False,
                 precision=PREC_FP64):
        L = load()
        self.bands = int(model.bands)
        self.lattice, self.kpoints, self.oversamp, self.window = int(lattice), int(kpoints), int(oversamp), int(window)
        self.maxband = self.bands if maxband is None else int(maxband)
        self.spin = bool(spin)
        self.eta = float(eta)
        self.wn = self.lattice * self.oversamp
        self.side = (2 * self.window + 1) * self.oversamp
        self.nimp = 1
        self.nhops = len(model.t)
        self._R = np.ascontiguousarray(model.R, np.int32)
        self._orb = np.ascontiguousarray(model.orb, np.int32)
        self._t = np.ascontiguousarray(np.asarray(model.t, np.complex128).view(np.float64))
        self._anti = np.ascontiguousarray(model.anti, np.uint8)
        m = _Model(self.bands, int(getattr(model, "scmaxbands", self.bands)), float(getattr(model, "efermi", 0.0)),
                   len(model.t), _ptr(self._R), _ptr(self._orb), _ptr(self._t), _ptr(self._anti))
        p = _Params(self.lattice, self.kpoints, self.oversamp, self.window, self.maxband, int(self.spin), float(eta),
                    int(precision))
        h = ctypes.c_void_p()
        rc = L.cqpi_create(ctypes.byref(m), ctypes.byref(p), ctypes.byref(h))
        if rc != OK:
            raise CqpiError(rc, L.cqpi_status_string(rc).decode())
        self._h = h
        self._L = L

    def _check(self, rc):
        if rc != OK:
            raise CqpiError(rc, self._L.cqpi_last_error(self._h).decode() or self._L.cqpi_status_string(rc).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.cqpi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- inputs
    def set_orbitals(self, wf, is_zero=None):
        wf = np.ascontiguousarray(wf, np.float64)
        z = None if is_zero is None else np.ascontiguousarray(is_zero, np.uint8)
        self._check(self._L.cqpi_set_orbitals(self._h, _ptr(wf), wf.shape[0], wf.shape[1], _ptr(z)))

    def set_scattering(self, vscat):
        v = np.ascontiguousarray(np.asarray(vscat, np.complex128).view(np.float64))
        self._check(self._L.cqpi_set_scattering(self._h, _ptr(v)))
        self.nimp = 1

    def set_impurities(self, V):
        V = np.ascontiguousarray(np.asarray(V, np.complex128).reshape(-1, self.bands, self.bands))
        self._check(self._L.cqpi_set_impurities(self._h, _ptr(V.view(np.float64)), V.shape[0]))
        self.nimp = V.shape[0]

    def set_hoppings(self, t):
        """New complex amplitudes for the model's hopping terms (same order as model.t)."""
        t = np.ascontiguousarray(np.asarray(t, np.complex128).reshape(-1))
        assert len(t) == self.nhops
        self._t = np.ascontiguousarray(t.view(np.float64))
        self._check(self._L.cqpi_set_hoppings(self._h, _ptr(self._t)))

    # -- compute
    def solve_bands(self):
        self._check(self._L.cqpi_solve_bands(self._h))

    def run(self, energies, f32=True, f64=False, out32=None):
        """Host maps [nE][nimp][wn][wn] (float32 and/or float64).  ``out32`` may be a
        preallocated (e.g. page-locked) float32 array to receive the maps."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        shape = (len(e), self.nimp, self.wn, self.wn)
        if out32 is not None:
            assert out32.dtype == np.float32 and out32.size == int(np.prod(shape)) and out32.flags.c_contiguous
        o32 = (out32.reshape(shape) if out32 is not None else np.empty(shape, np.float32)) if f32 else None
        o64 = np.empty(shape, np.float64) if f64 else None
        self._check(self._L.cqpi_run(self._h, _ptr(e), len(e), _ptr(o32), _ptr(o64), 0))
        if f32 and f64:
            return o32, o64
        return o32 if f32 else o64

    def run_device(self, energies, ptr32=None, ptr64=None):
        """Asynchronous run into device buffers (raw pointers, e.g. torch tensor.data_ptr())."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        self._check(self._L.cqpi_run(self._h, _ptr(e), len(e), ptr32, ptr64, 1))

    def adjoint(self, energies, dL_dmaps=None, dev_ptr=None):
        """Reverse-mode derivative of run(): dL/drho (host float32 [nE][nimp][wn][wn], or a
        device pointer to that layout) -> (dL/dt complex [nhops], dL/dV complex
        [nimp][b][b]) with dL/dz = dL/dRe z + i dL/dIm z."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        gt = np.zeros(2 * self.nhops, np.float64)
        gv = np.zeros(2 * self.nimp * self.bands * self.bands, np.float64)
        if dev_ptr is not None:
            rc = self._L.cqpi_adjoint(self._h, _ptr(e), len(e), dev_ptr, 1, _ptr(gt), _ptr(gv))
        else:
            w = np.ascontiguousarray(dL_dmaps, np.float32)
            assert w.size == len(e) * self.nimp * self.wn * self.wn
            rc = self._L.cqpi_adjoint(self._h, _ptr(e), len(e), _ptr(w), 0, _ptr(gt), _ptr(gv))
        self._check(rc)
        return gt.view(np.complex128), gv.view(np.complex128).reshape(self.nimp, self.bands, self.bands)

    def run_fov(self, energies, fov, ptr32):
        """Asynchronous batched run with a field of view per (energy, impurity) map into a
        device buffer (packed maps, see cqpi_run_fov)."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        self._fov = np.ascontiguousarray(fov, np.int32).reshape(-1)
        assert len(self._fov) == len(e) * self.nimp
        self._check(self._L.cqpi_run_fov(self._h, _ptr(e), len(e), _ptr(self._fov), ptr32, 1))

    def autotune(self, energies):
        """Time every valid contraction tile shape on the first energy batch and keep the
        fastest; returns (ms per batch with the chosen shape, shapes timed)."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        ms = ctypes.c_float()
        n = ctypes.c_int32()
        self._check(self._L.cqpi_autotune(self._h, _ptr(e), len(e), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_josephson(self, deltat=0.001, etat=None, enable=True):
        """Josephson mode (output=josephson): tip gap deltat, tip broadening etat (default
        the sample's eta, as the reference's driver)."""
        et = self.eta if etat is None else etat
        self._check(self._L.cqpi_set_josephson(self._h, int(bool(enable)), float(deltat), float(et)))

    def set_threshold(self, threshold, spinarr=None) -> int:
        """Proximity-list form of the LDOS (threshold keyword); None or NaN: the full sum.
        Returns the list's entry count."""
        c = ctypes.c_int64()
        thr = float("nan") if threshold is None else float(threshold)
        sa = None if spinarr is None else np.ascontiguousarray(np.asarray(spinarr, np.int32))
        self._check(self._L.cqpi_set_threshold(self._h, thr, None if sa is None else _ptr(sa),
                                               0 if sa is None else len(sa), ctypes.byref(c)))
        return c.value

    def set_greens(self, mode, epserr=1e-5, surface_model=None):
        """Green's function: GREEN_NORMAL, GREEN_SURFACE or GREEN_BULK (green keyword), with
        an optional surface-layer model (stbfile)."""
        if isinstance(mode, str):
            mode = {"normal": GREEN_NORMAL, "surface": GREEN_SURFACE, "bulk": GREEN_BULK}[mode]
        sm = None
        if surface_model is not None:
            self._sR = np.ascontiguousarray(surface_model.R, np.int32)
            self._so = np.ascontiguousarray(surface_model.orb, np.int32)
            self._st = np.ascontiguousarray(np.asarray(surface_model.t, np.complex128).view(np.float64))
            self._sa = np.ascontiguousarray(surface_model.anti, np.uint8)
            self._sm = _Model(int(surface_model.bands), int(getattr(surface_model, "scmaxbands", surface_model.bands)),
                              float(getattr(surface_model, "efermi", 0.0)), len(surface_model.t), _ptr(self._sR),
                              _ptr(self._so), _ptr(self._st), _ptr(self._sa))
            sm = ctypes.byref(self._sm)
        self._check(self._L.cqpi_set_greens(self._h, int(mode), float(epserr), sm))

    def spf(self, energies, maxband=None):
        """Spectral function maps [nE][lattice][lattice] (float64, IDL order)."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        out = np.empty((len(e), self.lattice, self.lattice), np.float64)
        self._check(self._L.cqpi_spf(self._h, _ptr(e), len(e), int(maxband or self.maxband), None, _ptr(out)))
        return out

    def uspf(self, energies, pos, prearr, maxband=None):
        """Unfolded spectral function maps [nE][lattice][lattice] (float64, IDL order)."""
        m = int(maxband or self.maxband)
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        p = np.ascontiguousarray(np.asarray(pos, np.float64)[:, :2].reshape(m, 2))
        q = np.ascontiguousarray(np.asarray(prearr, np.float64).reshape(m))
        out = np.empty((len(e), self.lattice, self.lattice), np.float64)
        self._check(self._L.cqpi_uspf(self._h, _ptr(e), len(e), m, _ptr(p), _ptr(q), None, _ptr(out)))
        return out

    def dos(self, energies, maxband=None):
        """-sum_i<maxband Im G0(R=0)_ii per energy."""
        e = np.ascontiguousarray(energies, np.float64).reshape(-1)
        out = np.empty(len(e), np.float64)
        self._check(self._L.cqpi_dos(self._h, _ptr(e), len(e), int(maxband or self.maxband), _ptr(out)))
        return out

    def set_list(self, ent, factor):
        """Explicit proximity list: ent[k] = (list, i, j, o1, o2), factor[k]."""
        ent = np.ascontiguousarray(np.asarray(ent, np.int32).reshape(-1, 5))
        fac = np.ascontiguousarray(np.asarray(factor, np.float64).reshape(-1))
        assert len(ent) == len(fac)
        self._check(self._L.cqpi_set_list(self._h, len(fac), _ptr(ent), _ptr(fac)))

    def graph_begin(self):
        self._check(self._L.cqpi_graph_begin(self._h))

    def graph_end(self):
        self._check(self._L.cqpi_graph_end(self._h))

    def graph_launch(self):
        self._check(self._L.cqpi_graph_launch(self._h))

    # -- narrow seam
    def wannierldos(self, T, g0r):
        T = np.ascontiguousarray(np.asarray(T, np.complex128))
        g = np.ascontiguousarray(np.asarray(g0r, np.complex128))
        self._check(self._L.cqpi_wannierldos(self._h, _ptr(T.view(np.float64)), _ptr(g.view(np.float64))))

    def wannierjosephson(self, T, g0r, tip):
        T = np.ascontiguousarray(np.asarray(T, np.complex128))
        g = np.ascontiguousarray(np.asarray(g0r, np.complex128))
        tp = np.array([complex(tip).real, complex(tip).imag], np.float64)
        self._check(self._L.cqpi_wannierjosephson(self._h, _ptr(T.view(np.float64)), _ptr(g.view(np.float64)),
                                                  _ptr(tp)))

    def wannierldoslist(self, T, g0r):
        T = np.ascontiguousarray(np.asarray(T, np.complex128))
        g = np.ascontiguousarray(np.asarray(g0r, np.complex128))
        self._check(self._L.cqpi_wannierldoslist(self._h, _ptr(T.view(np.float64)), _ptr(g.view(np.float64))))

    def retrieve_result(self):
        out = np.empty((self.wn, self.wn), np.float64)
        self._check(self._L.cqpi_retrieve_result(self._h, _ptr(out)))
        return out

    # -- stage access
    def get_bands(self):
        nk = self.kpoints ** 2
        ev = np.empty((nk, self.bands), np.float64)
        U = np.empty((nk, self.bands, self.bands), np.complex128)
        self._check(self._L.cqpi_get_bands(self._h, _ptr(ev), _ptr(U.view(np.float64))))
        return ev, U

    def greens_box(self, energy):
        rb = ctypes.c_int32()
        self._check(self._L.cqpi_get_greens_box(self._h, float(energy), None, ctypes.byref(rb)))
        nb = 2 * rb.value + 1
        box = np.empty((nb, nb, self.bands, self.bands), np.complex128)
        self._check(self._L.cqpi_get_greens_box(self._h, float(energy), _ptr(box.view(np.float64)), ctypes.byref(rb)))
        return box, rb.value

    def tmatrix(self, energy):
        T = np.empty((self.bands, self.bands), np.complex128)
        self._check(self._L.cqpi_get_tmatrix(self._h, float(energy), _ptr(T.view(np.float64))))
        return T

    # -- runtime
    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(self._L.cqpi_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def synchronize(self):
        self._check(self._L.cqpi_synchronize(self._h))

    def kernel_launches(self) -> int:
        c = ctypes.c_int64()
        self._check(self._L.cqpi_kernel_launches(self._h, ctypes.byref(c)))
        return c.value

    def contraction_kind(self) -> str:
        """Which contraction kernel the handle uses: 'fp64', 'fp32' (CUDA cores) or 'tcgen05'."""
        k = ctypes.c_int32()
        self._check(self._L.cqpi_contraction_kind(self._h, ctypes.byref(k)))
        return {0: "fp64", 1: "fp32", 2: "tcgen05"}[k.value]

    def stage_times(self):
        t = np.zeros(5, np.float32)
        self._check(self._L.cqpi_stage_times(self._h, _ptr(t)))
        return dict(zip(["bands", "greens", "tmatrix", "ldos", "total"], t.tolist()))
