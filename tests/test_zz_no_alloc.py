"""GPU test of cqpi_realspace_greens_noalloc, the entry point that allocates nothing.

It is for callers that cannot call cudaMalloc (work enqueued during a CUDA stream
capture, hosts with a fixed pre-allocated device budget).  The test calls it through the
C ABI on two energies in a row -- the second call reuses the fixed scratch array the
first one left behind -- and compares each box with the one the regular handle-based
entry point (cqpi_get_greens_box, FP64 path) returns for the same model and energy.
Buffers for the test's own input and output come from torch; the entry point itself
allocates nothing.  This file is collected last so that a failing run stops after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

from cases import case

pytestmark = pytest.mark.gpu


def test_noalloc_greens_box_matches_handle(built_lib):
    import torch
    import cqpi
    from oracle import oracle as O

    m, p, wf, z, v, E = case("c2")
    kp, eta = p["kpoints"], p["eta"]
    eng = cqpi.Engine(m, p["lattice"], kp, p["oversamp"], p["window"], eta, precision=cqpi.PREC_FP64)
    om = O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)
    ev, U = O.bands(om, kp)
    L = cqpi.load()
    b = m.bands
    for energy in (-0.07, 0.11):                      # two calls in a row
        ref, rb = eng.greens_box(energy)              # existing entry point
        nb = 2 * rb + 1
        g0k = np.ascontiguousarray(O.greens_k(ev, U, kp, energy, eta))   # [kp][kp][b][b]
        dev_in = torch.from_numpy(g0k.view(np.float64).reshape(-1).copy()).cuda()
        dev_out = torch.full((nb * nb * b * b * 2,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(dev_in.data_ptr()), kp, b, rb,
                                             ctypes.c_void_p(dev_out.data_ptr()), None)
        assert rc == cqpi.OK
        torch.cuda.synchronize()
        got = dev_out.cpu().numpy().view(np.complex128).reshape(nb, nb, b, b)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 1e-12, err


def test_noalloc_rejects_oversized_requests(built_lib):
    import cqpi
    L = cqpi.load()
    # bands^2 * kpoints * (2rb+1) = 9 * 1024 * 261 complex doubles > 16 MiB of scratch
    rc = L.cqpi_realspace_greens_noalloc(ctypes.c_void_p(16), 1024, 3, 130, ctypes.c_void_p(16), None)
    assert rc == cqpi.ERR_NOT_SUPPORTED
    rc = L.cqpi_realspace_greens_noalloc(None, 16, 1, 2, None, None)
    assert rc == cqpi.ERR_ARG
