"""ctypes wrappers of the host-side (CPU-only) C ABI in include/cqpi_host.h."""
from __future__ import annotations

import ctypes

import numpy as np

from . import load


class _HR(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 512), ("bands", ctypes.c_int32), ("scmaxbands", ctypes.c_int32),
                ("nrpts", ctypes.c_int32), ("nhops", ctypes.c_int64), ("R", ctypes.POINTER(ctypes.c_int32)),
                ("orb", ctypes.POINTER(ctypes.c_int32)), ("t", ctypes.POINTER(ctypes.c_double)),
                ("anti", ctypes.POINTER(ctypes.c_uint8))]


class _IDLHeader(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 1024), ("date", ctypes.c_char * 256), ("size", ctypes.c_int32 * 3),
                ("scan_range", ctypes.c_double * 2), ("offset", ctypes.c_double * 2), ("bias", ctypes.c_double * 2),
                ("setpoint", ctypes.c_double), ("data_offset", ctypes.c_int64)]


def _lib():
    L = load()
    if not getattr(L, "_host_ready", False):
        P = ctypes.c_void_p
        L.cqpi_read_hr.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.POINTER(_HR))]
        L.cqpi_hr_free.argtypes = [ctypes.POINTER(_HR)]
        L.cqpi_orbital_known.argtypes = [ctypes.c_char_p]
        L.cqpi_orbital_cache.argtypes = [ctypes.c_char_p] + [ctypes.c_double] * 7 + [ctypes.c_int32, ctypes.c_int32, P]
        L.cqpi_idl_write.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, P, P, P, ctypes.c_double, P]
        L.cqpi_xsf_orbital_cache.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_double, P]
        L.cqpi_idl_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32, P, P, P, ctypes.c_double]
        L.cqpi_idl_write_layers.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, P]
        L.cqpi_idl_read_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(_IDLHeader)]
        L.cqpi_idl_read.argtypes = [ctypes.c_char_p, P, ctypes.c_int64]
        L.cqpi_orbital_cache_basis.argtypes = [ctypes.c_char_p] + [ctypes.c_double] * 7 + [P, ctypes.c_int32,
                                                                                         ctypes.c_int32, P]
        L.cqpi_xsf_orbital_cache_shifted.argtypes = [ctypes.c_char_p, P, ctypes.c_int32, ctypes.c_double,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_double, P]
        L.cqpi_xsf_orbital_cache_mod.argtypes = [ctypes.c_char_p, P, P] + [ctypes.c_double] * 5 + [ctypes.c_int32,
                                                                                                 ctypes.c_int32, P]
        L.cqpi_band_histogram.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int32, P]
        L.cqpi_interp_known.argtypes = [ctypes.c_char_p]
        L.cqpi_interp_eval.argtypes = [ctypes.c_char_p, ctypes.c_int32, P, P, ctypes.c_int32, P, P]
        L.cqpi_host_last_error.restype = ctypes.c_char_p
        L._host_ready = True
    return L


class HostError(RuntimeError):
    pass


def _err(L, rc):
    raise HostError(f"status {rc}: {L.cqpi_host_last_error().decode()}")


def read_hr(path: str, scmodel: bool = False) -> dict:
    L = _lib()
    p = ctypes.POINTER(_HR)()
    rc = L.cqpi_read_hr(path.encode(), int(scmodel), ctypes.byref(p))
    if rc:
        _err(L, rc)
    hr = p.contents
    n = hr.nhops
    out = dict(name=hr.name.decode(), bands=hr.bands, scmaxbands=hr.scmaxbands, nrpts=hr.nrpts,
               R=np.ctypeslib.as_array(hr.R, (n, 3)).copy() if n else np.zeros((0, 3), np.int32),
               orb=np.ctypeslib.as_array(hr.orb, (n, 2)).copy() if n else np.zeros((0, 2), np.int32),
               t=(np.ctypeslib.as_array(hr.t, (n, 2)).copy().view(np.complex128).reshape(-1)) if n
               else np.zeros(0, np.complex128),
               anti=np.ctypeslib.as_array(hr.anti, (n,)).astype(bool) if n else np.zeros(0, bool))
    L.cqpi_hr_free(p)
    return out


def orbital_cache(name, window, oversamp, width=0.5, height=5.0, xpos=0.0, ypos=0.0, theta=0.0, phi=0.0,
                  prefact=1.0) -> np.ndarray:
    L = _lib()
    side = (2 * window + 1) * oversamp
    out = np.empty((side, side), np.float64)
    rc = L.cqpi_orbital_cache(name.encode(), width, height, xpos, ypos, theta, phi, prefact, window, oversamp,
                              out.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)
    return out


def xsf_orbital_cache(path, height, window, oversamp, prefact=1.0) -> np.ndarray:
    """Orbital cache [side][side] from an XSF file (the orbitalfiles keyword)."""
    L = _lib()
    side = (2 * window + 1) * oversamp
    out = np.empty((side, side), np.float64)
    rc = L.cqpi_xsf_orbital_cache(str(path).encode(), float(height), window, oversamp, float(prefact),
                                  out.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)
    return out


def _vec(v, n):
    """A float64 array of n values (or None for NULL)."""
    if v is None:
        return None
    a = np.ascontiguousarray(np.asarray(v, np.float64).reshape(-1))
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def orbital_cache_basis(name, window, oversamp, width=0.5, height=5.0, xpos=0.0, ypos=0.0, theta=0.0, phi=0.0,
                        prefact=1.0, basis=None) -> np.ndarray:
    """Analytic orbital cache with lattice basis vectors basis = ((b0x, b0y), (b1x, b1y)) or
    None (mkwavefunctions' 'orbitals' source)."""
    L = _lib()
    side = (2 * window + 1) * oversamp
    out = np.empty((side, side), np.float64)
    b = _vec(basis, 4)
    rc = L.cqpi_orbital_cache_basis(name.encode(), width, height, xpos, ypos, theta, phi, prefact, _ptr(b), window,
                                    oversamp, out.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)
    return out


def xsf_orbital_cache_shifted(path, height, window, oversamp, shift=(0.0, 0.0, 0.0), prefact=1.0,
                              centre=True) -> np.ndarray:
    """XSF orbital cache with the grid moved by shift and centred pixels (mkwavefunctions'
    'orbitalfiles' source)."""
    L = _lib()
    side = (2 * window + 1) * oversamp
    out = np.empty((side, side), np.float64)
    sh = _vec(shift, 3)
    rc = L.cqpi_xsf_orbital_cache_shifted(str(path).encode(), _ptr(sh), 1 if centre else 0, height, window, oversamp,
                                          prefact, out.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)
    return out


def xsf_orbital_cache_mod(path, height, window, oversamp, modshift=(0.0, 0.0, 0.0), basis=None, xpos=0.0, ypos=0.0,
                          theta=0.0, prefact=1.0) -> np.ndarray:
    """XSF orbital placed at (xpos, ypos), rotated by theta, with the grid moved by modshift
    (mkwavefunctions' 'modorbitalfiles' source)."""
    L = _lib()
    side = (2 * window + 1) * oversamp
    out = np.empty((side, side), np.float64)
    sh, b = _vec(modshift, 3), _vec(basis, 4)
    rc = L.cqpi_xsf_orbital_cache_mod(str(path).encode(), _ptr(sh), _ptr(b), height, xpos, ypos, theta, prefact,
                                      window, oversamp, out.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)
    return out


def interp_eval(method, xa, ya, x) -> np.ndarray:
    """One-dimensional interpolation of mkwavefunctions (GSL's methods by name)."""
    L = _lib()
    xa = np.ascontiguousarray(xa, np.float64)
    ya = np.ascontiguousarray(ya, np.float64)
    xs = np.ascontiguousarray(np.atleast_1d(x), np.float64)
    if xa.shape != ya.shape:
        raise ValueError("xa and ya differ in length")
    y = np.empty_like(xs)
    rc = L.cqpi_interp_eval(method.encode(), xa.size, _ptr(xa), _ptr(ya), xs.size, _ptr(xs), _ptr(y))
    if rc:
        raise HostError(f"status {rc}: interpolation '{method}' rejected its input (method, point count, "
                        "increasing x values, x inside the data range)")
    return y


def band_histogram(model, pix, oversamp, le, ue, layers) -> np.ndarray:
    """The bsfile band-structure histogram [layers][pix][pix] of a model with fields bands, R,
    orb, t (complex), anti and optionally efermi, scmaxbands (cqpi.workloads.TBModel, the
    oracle's Model, or the dict of read_hr)."""
    from . import _Model
    L = _lib()
    get = (lambda k, d=None: model.get(k, d)) if isinstance(model, dict) else (lambda k, d=None: getattr(model, k, d))
    bands = int(get("bands"))
    R = np.ascontiguousarray(np.asarray(get("R")).reshape(-1, 3), np.int32)
    orb = np.ascontiguousarray(np.asarray(get("orb")).reshape(-1, 2), np.int32)
    tc = np.asarray(get("t"), np.complex128).reshape(-1)
    t = np.ascontiguousarray(np.stack([tc.real, tc.imag], -1), np.float64)
    anti_v = get("anti")
    anti = np.ascontiguousarray(np.zeros(len(tc)) if anti_v is None else np.asarray(anti_v).reshape(-1), np.uint8)
    scmax = get("scmaxbands")
    m = _Model(bands, bands if scmax is None else int(scmax), float(get("efermi", 0.0) or 0.0), len(tc),
               R.ctypes.data, orb.ctypes.data, t.ctypes.data, anti.ctypes.data)
    out = np.empty((layers, pix, pix), np.float64)
    rc = L.cqpi_band_histogram(ctypes.addressof(m), pix, oversamp, le, ue, layers, _ptr(out))
    if rc:
        raise HostError(f"status {rc}: invalid band-structure histogram arguments")
    return out


def idl_write(path, data_kyx, name, scan_range=(2.0, 2.0), offset=(-1.0, -1.0), bias=(0.0, 0.0), setpoint=0.0,
              date=None):
    L = _lib()
    d = np.ascontiguousarray(data_kyx, np.float32)
    z, y, x = d.shape
    sr, of, bi = (np.array(v, np.float64) for v in (scan_range, offset, bias))
    rc = L.cqpi_idl_write(str(path).encode(), name.encode(), None if date is None else date.encode(), x, y, z,
                          sr.ctypes.data_as(ctypes.c_void_p), of.ctypes.data_as(ctypes.c_void_p),
                          bi.ctypes.data_as(ctypes.c_void_p), setpoint, d.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)


def idl_create(path, shape_kyx, name, scan_range=(2.0, 2.0), offset=(-1.0, -1.0), bias=(0.0, 0.0), setpoint=0.0,
               date=None):
    """An IDL file of shape (layers, y, x) with zero data, for idl_write_layers."""
    L = _lib()
    z, y, x = shape_kyx
    sr, of, bi = (np.array(v, np.float64) for v in (scan_range, offset, bias))
    rc = L.cqpi_idl_create(str(path).encode(), name.encode(), None if date is None else date.encode(), x, y, z,
                           sr.ctypes.data_as(ctypes.c_void_p), of.ctypes.data_as(ctypes.c_void_p),
                           bi.ctypes.data_as(ctypes.c_void_p), setpoint)
    if rc:
        _err(L, rc)


def idl_write_layers(path, k0, data_kyx):
    """Overwrite layers k0 .. k0 + len(data_kyx) - 1 of an existing IDL file in place."""
    L = _lib()
    d = np.ascontiguousarray(data_kyx, np.float32)
    rc = L.cqpi_idl_write_layers(str(path).encode(), int(k0), d.shape[0], d.ctypes.data_as(ctypes.c_void_p))
    if rc:
        _err(L, rc)


def idl_read(path):
    L = _lib()
    h = _IDLHeader()
    rc = L.cqpi_idl_read_header(str(path).encode(), ctypes.byref(h))
    if rc:
        _err(L, rc)
    x, y, z = h.size
    data = np.empty((z, y, x), np.float32)
    rc = L.cqpi_idl_read(str(path).encode(), data.ctypes.data_as(ctypes.c_void_p), data.size)
    if rc:
        _err(L, rc)
    hdr = dict(name=h.name.decode(), date=h.date.decode(), size=(x, y, z), scan_range=tuple(h.scan_range),
               offset=tuple(h.offset), bias=tuple(h.bias), setpoint=h.setpoint)
    return hdr, data
