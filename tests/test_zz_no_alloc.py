"""GPU test of cqpi_realspace_greens_noalloc, the entry point that allocates nothing.

It is for callers that cannot call cudaMalloc (work enqueued during a CUDA stream
capture, hosts with a fixed pre-allocated device budget).  The tests call it through the
C ABI on two energies in a row -- the second call reuses the fixed scratch array the
first one left behind -- and compare each box with the one the regular handle-based
entry point (cqpi_get_greens_box, FP64 path) returns for the same model and energy, on a
power-of-two k-grid (radix-2 transform) and on one that is not (direct transform).  The
device's free memory must not change across the second call, and a call recorded inside a
stream capture must replay to the same box.  Buffers for the test's own input and output
come from torch; the entry point itself allocates nothing.  This file is collected last so
that a failing run stops after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from cases import case

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _setup(name):
    import cqpi
    from oracle import oracle as O
    m, p, wf, z, v, E = case(name)
    kp, eta = p["kpoints"], p["eta"]
    eng = cqpi.Engine(m, p["lattice"], kp, p["oversamp"], p["window"], eta, spin=p["spin"],
                      precision=cqpi.PREC_FP64)
    om = O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)
    ev, U = O.bands(om, kp)
    return eng, m.bands, kp, eta, ev, U


def _g0k_device(O, ev, U, kp, energy, eta):
    import torch
    g0k = np.ascontiguousarray(O.greens_k(ev, U, kp, energy, eta))   # [kp][kp][b][b]
    return torch.from_numpy(g0k.view(np.float64).reshape(-1).copy()).cuda()


@pytest.mark.parametrize("name", ["c2", "c1_odd"])   # kpoints 16 (radix-2) and 12 (direct)
def test_noalloc_greens_box_matches_handle(built_lib, name):
    import torch
    import cqpi
    from oracle import oracle as O

    eng, b, kp, eta, ev, U = _setup(name)
    L = cqpi.load()
    for k, energy in enumerate((-0.07, 0.11)):       # two calls in a row
        ref, rb = eng.greens_box(energy)              # existing entry point
        nb = 2 * rb + 1
        dev_in = _g0k_device(O, ev, U, kp, energy, eta)
        dev_out = torch.full((nb * nb * b * b * 2,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(dev_in.data_ptr()), kp, b, rb,
                                             ctypes.c_void_p(dev_out.data_ptr()), None)
        assert rc == cqpi.OK
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        if k == 1:
            # the call after the first one on this device takes no device memory
            assert free1 == free0, (free0, free1)
        got = dev_out.cpu().numpy().view(np.complex128).reshape(nb, nb, b, b)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < TOL, err
    eng.close()


def test_noalloc_inside_stream_capture(built_lib):
    """A first call outside any capture, then one recorded into a CUDA graph (cudaMalloc
    would be an error there) and replayed: the replay writes the same box."""
    import torch
    import cqpi
    from oracle import oracle as O

    eng, b, kp, eta, ev, U = _setup("c2")
    L = cqpi.load()
    ref0, rb = eng.greens_box(-0.04)
    ref1, _ = eng.greens_box(0.06)
    nb = 2 * rb + 1
    in0 = _g0k_device(O, ev, U, kp, -0.04, eta)
    in1 = _g0k_device(O, ev, U, kp, 0.06, eta)
    out0 = torch.full((nb * nb * b * b * 2,), float("nan"), dtype=torch.float64, device="cuda")
    out1 = torch.full_like(out0, float("nan"))
    torch.cuda.synchronize()
    assert L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(in0.data_ptr()), kp, b, rb,
                                           ctypes.c_void_p(out0.data_ptr()), None) == cqpi.OK
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g.capture_begin()
        rc = L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(in1.data_ptr()), kp, b, rb,
                                             ctypes.c_void_p(out1.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        g.capture_end()
    assert rc == cqpi.OK
    torch.cuda.synchronize()
    assert torch.isnan(out1).all()                    # recorded, not yet run
    g.replay()
    torch.cuda.synchronize()
    for out, ref in ((out0, ref0), (out1, ref1)):
        got = out.cpu().numpy().view(np.complex128).reshape(nb, nb, b, b)
        assert np.abs(got - ref).max() / np.abs(ref).max() < TOL
    eng.close()


def test_noalloc_rejects_oversized_requests(built_lib):
    import cqpi
    L = cqpi.load()
    # bands^2 * kpoints * (2rb+1) = 9 * 1024 * 261 complex doubles > 16 MiB of scratch
    rc = L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(16), 1024, 3, 130, ctypes.c_void_p(16), None)
    assert rc == cqpi.ERR_NOT_SUPPORTED
    rc = L.cqpi_realspace_greens_noalloc(None, 16, 1, 2, None, None)
    assert rc == cqpi.ERR_ARG
