"""Fitting harness around the engine's adjoint (outside the drop-in path).

Loss (per energy, summed): || |FFT2(rho_w)| - target_w ||^2, the QPI magnitude of every
LDOS map against target maps.  Parameters: the independent real amplitudes p of a
symmetric model family (t = B p, see workloads.t2g_c2_parametrisation) and the impurity
matrix V.  ``LDOSMaps`` is a torch.autograd.Function whose forward runs the engine
(cqpi_set_hoppings / cqpi_set_impurities / cqpi_run into a CUDA tensor) and whose backward
calls cqpi_adjoint on the incoming dL/drho; torch does only the loss (FFT, abs, square) and
the optimiser.
"""
import time

import numpy as np

from . import Engine, PREC_FP64, PREC_MIXED
from . import workloads as W


def _torch():
    import torch
    return torch


class QPIFit:
    """One engine plus the fixed pieces of a fit: energies, parametrisation, orbitals."""

    def __init__(self, lattice=128, kpoints=1024, oversamp=10, window=2, energies=None, eta=0.002,
                 seed=2, precision=PREC_MIXED, V=None):
        self.model, self.B, self.p0 = W.t2g_c2_parametrisation(seed)
        self.energies = np.linspace(-0.1, 0.1, 41) if energies is None else np.asarray(energies, np.float64)
        self.eng = Engine(self.model, lattice, kpoints, oversamp, window, eta, precision=precision)
        self.eng.set_orbitals(W.t2g_orbitals_c2(window, oversamp))
        b = self.model.bands
        self.V0 = np.diag([0.3, 0.3, 0.5]).astype(np.complex128) if V is None else np.asarray(V, np.complex128)
        self.eng.set_impurities(self.V0[None])
        self.wn = lattice * oversamp
        self.bands = b
        self.precision = precision
        self.timing = {"forward": [], "adjoint": []}

    def hoppings(self, p):
        return self.B @ np.asarray(p, np.float64)

    def set_params(self, p, V):
        self.eng.set_hoppings(self.hoppings(p).astype(np.complex128))
        self.eng.set_impurities(np.asarray(V, np.complex128).reshape(1, self.bands, self.bands))

    def maps(self, p, V):
        """rho for parameters (p, V) as a CUDA tensor [nE][1][wn][wn] (no autograd): float32
        from the mixed engine, float64 from the FP64 engine."""
        torch = _torch()
        self.set_params(p, V)
        fp64 = self.precision == PREC_FP64
        out = torch.empty((len(self.energies), 1, self.wn, self.wn), dtype=torch.float64 if fp64 else torch.float32,
                          device="cuda")
        torch.cuda.synchronize()
        if fp64:
            self.eng.run_device(self.energies, ptr64=out.data_ptr())
        else:
            self.eng.run_device(self.energies, ptr32=out.data_ptr())
        self.eng.synchronize()
        return out

    def close(self):
        self.eng.close()


def _ldos_function():
    torch = _torch()

    class LDOSMaps(torch.autograd.Function):
        @staticmethod
        def forward(ctx, p, Vr, fit):
            t0 = time.perf_counter()
            V = Vr.detach().cpu().numpy()
            out = fit.maps(p.detach().cpu().numpy(), V)
            fit.timing["forward"].append(time.perf_counter() - t0)
            ctx.fit = fit
            return out

        @staticmethod
        def backward(ctx, g):
            fit = ctx.fit
            t0 = time.perf_counter()
            g = g.contiguous().to(torch.float32)
            torch.cuda.synchronize()          # g is complete before the engine's stream reads it
            gt, gv = fit.eng.adjoint(fit.energies, dev_ptr=g.data_ptr())
            fit.timing["adjoint"].append(time.perf_counter() - t0)
            # t = B p with real p: dL/dp = B^T dL/dRe t; V real: dL/dV = dL/dRe V
            gp = torch.from_numpy(fit.B.T @ gt.real)
            gV = torch.from_numpy(np.ascontiguousarray(gv[0].real))
            return gp, gV, None

    return LDOSMaps


def qpi_loss(maps, target, dtype=None):
    """sum over energies of || |FFT2(rho)| - target ||^2 (target: [nE][wn][wn] magnitudes).
    dtype: the transform's real type (torch.float64 by default; torch.float32 runs the FFT in
    single precision, the sum in double)."""
    torch = _torch()
    dt = torch.float64 if dtype is None else dtype
    q = torch.abs(torch.fft.fft2(maps[:, 0].to(dt)))
    return torch.sum(((q - target.to(dt)) ** 2).to(torch.float64))


def target_maps(fit, rel=0.05, seed=7):
    """Target QPI magnitudes from seed-perturbed amplitudes p* = p0 (1 + rel N(0,1))."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    p_true = fit.p0 * (1.0 + rel * rng.normal(size=fit.p0.shape))
    with torch.no_grad():
        m = fit.maps(p_true, fit.V0.real)
        tgt = torch.abs(torch.fft.fft2(m[:, 0].to(torch.float64)))
    return p_true, tgt


def run_adam(fit, target, steps=200, lr=2e-3, fit_v=True, log=None, loss_dtype="float32", V_init=None):
    """Adam on (p, V) from p0 / V0 (or V_init); returns (p, V, losses).  fit_v: optimise the
    3x3 impurity matrix too; loss_dtype: the QPI loss's FFT precision ("float32": the
    transform in single precision, the sum in double; "float64")."""
    torch = _torch()
    LDOSMaps = _ldos_function()
    dt = torch.float32 if loss_dtype == "float32" else torch.float64
    p = torch.tensor(fit.p0.copy(), dtype=torch.float64, requires_grad=True)
    V0 = fit.V0.real if V_init is None else np.asarray(V_init, np.float64)
    Vr = torch.tensor(V0.copy(), dtype=torch.float64, requires_grad=fit_v)
    opt = torch.optim.Adam([p, Vr] if fit_v else [p], lr=lr)
    losses = []
    for it in range(steps):
        opt.zero_grad()
        maps = LDOSMaps.apply(p, Vr, fit)
        loss = qpi_loss(maps, target, dt)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
        if log is not None and (it % 20 == 0 or it == steps - 1):
            log(it, losses[-1])
    return p.detach().numpy(), Vr.detach().numpy(), losses


def gradient(fit, p, V, target):
    """(loss, dL/dp, dL/dV) at (p, V) through the adjoint."""
    torch = _torch()
    LDOSMaps = _ldos_function()
    pt = torch.tensor(np.asarray(p, np.float64), requires_grad=True)
    Vt = torch.tensor(np.asarray(V, np.float64), requires_grad=True)
    loss = qpi_loss(LDOSMaps.apply(pt, Vt, fit), target)
    loss.backward()
    return float(loss.detach()), pt.grad.numpy(), Vt.grad.numpy()


def gauss_newton(fit, p, V, h_rel=1e-4, h_abs=1e-5):
    """Gauss-Newton matrix J^T J of the QPI magnitudes F(x) = |FFT2 rho(x)| (every energy and
    pixel) at x = (p, V) -- the p amplitudes, then the nine real entries of V -- with J by
    central differences of the engine's maps (step h_rel |x_i|, at least h_abs), the
    transforms and the products in FP64.  Returns (JtJ [n][n], x)."""
    torch = _torch()
    x = np.concatenate([np.asarray(p, np.float64), np.asarray(V, np.float64).reshape(-1)])
    npar = len(x)
    npp = len(p)

    def F(xx):
        m = fit.maps(xx[:npp], xx[npp:].reshape(fit.bands, fit.bands))
        return torch.abs(torch.fft.fft2(m[:, 0].to(torch.float64))).reshape(-1).to(torch.float32)

    cols = []
    for i in range(npar):
        h = max(h_rel * abs(x[i]), h_abs)
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        cols.append((F(xp) - F(xm)) / (2.0 * h))
    J = torch.stack(cols, dim=1)                       # [outputs][npar] float32 on the device
    JtJ = np.zeros((npar, npar))
    step = 1 << 22
    for r0 in range(0, J.shape[0], step):              # FP64 products, chunked over the outputs
        Jc = J[r0:r0 + step].to(torch.float64)
        JtJ += (Jc.T @ Jc).cpu().numpy()
    del J, cols
    return JtJ, x


def identifiability(JtJ, x_true, x_start, x_fit):
    """Eigen-directions of J^T J (descending eigenvalues) and, per direction, the parameter
    error of the start and of the fit projected on it: how much of the start's error the fit
    removed in the well-constrained directions and which directions the maps do not constrain."""
    lam, vec = np.linalg.eigh(JtJ)
    order = np.argsort(lam)[::-1]
    lam, vec = lam[order], vec[:, order]
    d0, d1 = vec.T @ (x_start - x_true), vec.T @ (x_fit - x_true)
    return {"eigenvalues_rel": (lam / lam[0]).tolist(),
            "start_error_per_direction": np.abs(d0).tolist(),
            "fit_error_per_direction": np.abs(d1).tolist(),
            "fit_over_start_per_direction": (np.abs(d1) / np.maximum(np.abs(d0), 1e-300)).tolist()}


def loss_at(fit, x, target):
    """The QPI loss (FP64 transform) at x = (p, V)."""
    npp = len(fit.p0)
    m = fit.maps(x[:npp], x[npp:].reshape(fit.bands, fit.bands))
    return float(qpi_loss(m, target))


def gauss_newton_fit(fit, target, x0, iters=6, log=None):
    """Levenberg-Marquardt iterations on x = (p, V) for the QPI loss: J^T J from central
    differences of the maps (gauss_newton), the gradient 2 J^T r from the adjoint (gradient),
    the step -(J^T J + mu lambda_max I)^-1 J^T r with the damping mu chosen among 10^-8 ..
    10^-1 as the one that lowers the loss most (the loss is far from quadratic: sharp poles
    and |FFT| magnitudes); stops when no damping lowers the loss.  Returns (x, losses)."""
    npp = len(fit.p0)
    b = fit.bands
    x = np.asarray(x0, np.float64).copy()
    losses = [loss_at(fit, x, target)]
    for it in range(iters):
        JtJ, _ = gauss_newton(fit, x[:npp], x[npp:].reshape(b, b))
        _, gp, gV = gradient(fit, x[:npp], x[npp:].reshape(b, b), target)
        g = np.concatenate([gp, np.asarray(gV).reshape(-1)])
        lam_max = float(np.linalg.eigvalsh(JtJ).max())
        best = None
        for mu in (1e-8, 1e-6, 1e-4, 1e-3, 1e-2, 1e-1):
            step = -np.linalg.solve(JtJ + mu * lam_max * np.eye(len(x)), 0.5 * g)
            l = loss_at(fit, x + step, target)
            if l < losses[-1] and (best is None or l < best[0]):
                best = (l, step)
        if best is None:
            break
        x = x + best[1]
        losses.append(best[0])
        if log is not None:
            log(it, best[0])
    return x, losses
