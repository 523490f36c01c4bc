"""GPU: the fitting harness (torch.autograd.Function over cqpi_run / cqpi_adjoint).

The QPI loss gradient through the adjoint against central differences of the same loss
evaluated with the FP64 engine, and a short Adam run that lowers the loss.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMALL = dict(lattice=16, kpoints=64, oversamp=4, window=2, energies=np.array([-0.05, 0.0, 0.04]), eta=0.02)


def test_qpi_loss_gradient_matches_fd(built_lib):
    torch = pytest.importorskip("torch")
    import cqpi
    from cqpi import fit as F
    f64 = F.QPIFit(precision=cqpi.PREC_FP64, **SMALL)
    p_true, target = F.target_maps(f64)
    loss0, gp, gV = F.gradient(f64, f64.p0, f64.V0.real, target)
    rng = np.random.default_rng(3)

    def loss_at(p, V):
        with torch.no_grad():
            return float(F.qpi_loss(f64.maps(p, V), target))

    h = 1e-6
    for _ in range(2):
        d = rng.normal(size=f64.p0.shape)
        fd = (loss_at(f64.p0 + h * d, f64.V0.real) - loss_at(f64.p0 - h * d, f64.V0.real)) / (2 * h)
        assert abs(float(gp @ d) - fd) <= 1e-5 * abs(fd), (float(gp @ d), fd)
    dV = rng.normal(size=(3, 3))
    fd = (loss_at(f64.p0, f64.V0.real + h * dV) - loss_at(f64.p0, f64.V0.real - h * dV)) / (2 * h)
    assert abs(float(np.sum(gV * dV)) - fd) <= 1e-5 * abs(fd), (float(np.sum(gV * dV)), fd)
    f64.close()


def test_adam_lowers_the_qpi_loss(built_lib):
    pytest.importorskip("torch")
    from cqpi import fit as F
    fm = F.QPIFit(**SMALL)
    p_true, target = F.target_maps(fm)
    p, V, losses = F.run_adam(fm, target, steps=30, lr=2e-3)
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])
    fm.close()
