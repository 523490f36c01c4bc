"""Small parity cases shared by the GPU tests (sizes the oracle finishes in seconds)."""
import numpy as np

from cqpi import workloads as W


def case(name):
    """(model, params dict, wf [norb][side][side], is_zero, vscat, energies)."""
    if name == "c1":
        m = W.square_c1()
        p = dict(lattice=12, kpoints=32, oversamp=4, window=2, eta=0.05, spin=False)
        wf = W.gaussian_c1(2, 4)
        return m, p, wf, None, np.array([0.5 + 0j]), np.array([-0.2, 0.0, 0.2])
    if name == "c1_odd":   # odd lattice, non power-of-two k-grid, complex phase
        m = W.square_c1()
        p = dict(lattice=7, kpoints=12, oversamp=3, window=1, eta=0.03, spin=False)
        wf = W.gaussian_c1(1, 3)
        return m, p, wf, None, np.array([0.5 * np.exp(0.3j)]), np.array([-0.1, 0.15])
    if name == "c2":
        m = W.t2g_c2()
        p = dict(lattice=8, kpoints=16, oversamp=3, window=2, eta=0.02, spin=False)
        wf = W.t2g_orbitals_c2(2, 3)
        return m, p, wf, None, np.array([0.3, 0.3, 0.5], complex), np.array([-0.1, 0.1])
    if name == "c2_zero":  # a padded zero orbital ('z'), src/calcqpi.cc:514-518
        m = W.t2g_c2()
        p = dict(lattice=6, kpoints=16, oversamp=2, window=1, eta=0.02, spin=False)
        wf = W.t2g_orbitals_c2(1, 2)
        wf[2] = 123.0  # must be ignored
        return m, p, wf, np.array([0, 0, 1], np.uint8), np.array([0.3, 0.3, 0.5], complex), np.array([0.05])
    if name == "c3":
        m = W.triangular_c3()
        p = dict(lattice=6, kpoints=12, oversamp=2, window=1, eta=0.02, spin=True)
        orbs = W.tri_orbitals_c3(1, 2)
        wf = np.concatenate([orbs, orbs])
        return m, p, wf, None, np.ones(10, complex), np.array([0.0])
    raise KeyError(name)
