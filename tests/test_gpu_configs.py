"""GPU parity at the benchmarked configurations: the CUDA path against the oracle.

The oracle is the CPU restatement of the reference's wannier-mode energy loop
(src/calcqpi.cc:673-760: tmatrix::calchamiltonian, setgreensfunction,
calcrealspacegreensfunction, setscatteringmatrix and calcwannierldos, src/qpi.cc:454-950;
calcwannierjosephson, src/qpi.cc:953-1033, for the Josephson configuration).  The
configurations are the benchmarked ones at their own k-grids and broadenings -- the
sharp-pole regime where the FP32 Green's function, the FP32 transform and the split-FP16
contraction of the mixed path are at risk:

  C1  exactly as benchmarked: 1 orbital, lattice 64, k-grid 256^2, 8x8 px/cell, window 2,
      21 energies in [-0.2, 0.2] eV, eta 5 meV, V = 0.5 eV;
  C2  the t2g model at k-grid 1024^2 and eta 2 meV on a 24^2-site field of view
      (10x10 px/cell), five energies, one of them eta/2 above a band minimum;
  C3  the triangular 5-orbital x spin model at k-grid 2048^2 and eta 1 meV, spin pairing,
      on a 12^2-site field of view (6x6 px/cell), two energies (one eta/2 above a band
      minimum);
  CJ  Josephson mode on the 6-band BdG t2g model at k-grid 1024^2 and eta 2 meV on a
      16^2-site field of view, three energies (one eta/2 above a band minimum).

Tolerances, per map, relative to the map's largest value: FP64 path 1e-10; mixed path
1e-6 (the mixed-precision bar), written max|rho - rho_oracle| / max|rho_oracle|.
"""
import functools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-6}


def _setup(name):
    """(Config with the test's field of view, model, orbitals, energies)."""
    from cqpi import workloads as W
    from oracle import oracle as O
    c, m, wf = W.config(name)
    om = O.Model(m.bands, m.R, m.orb, m.t, m.anti, m.efermi, m.scmaxbands)
    if name == "C1":
        return c, om, wf, c.energy_list(), None
    ev, U = O.bands(om, c.kpoints)
    # the band minimum closest to the Fermi level: E = e_min + eta/2 puts a pole within eta of
    # a grid point
    mins = ev.min(axis=0)
    e_ext = float(mins[np.argmin(np.abs(mins))]) + 0.5 * c.eta
    if name == "C2":
        c.lattice = 24
        E = np.array([-0.1, -0.02, 0.05, 0.1, e_ext])
    elif name == "C3":
        c.lattice = 12
        E = np.array([-0.05, e_ext])
    else:  # CJ; E = 0 is left out: this model's Josephson map vanishes there to rounding
        c.lattice = 16
        E = np.array([-0.06, 0.03, e_ext])
    return c, om, wf, E, (ev, U)


@functools.lru_cache(maxsize=None)
def _oracle(name):
    """Oracle maps [nE][y][x] float64 of a configuration (computed once per test session)."""
    from oracle import oracle as O
    c, om, wf, E, eig = _setup(name)
    v = np.array(c.scattering, complex)
    jos = c.extra.get("josephson")
    m = c.extra.get("maxband", om.bands)
    if eig is None:
        return c, om, wf, E, O.run(om, c.lattice, c.kpoints, c.oversamp, c.window, c.eta, E, v, wf, m=m, spin=c.spin)
    ev, U = eig
    maps = []
    for e in E:   # the energy loop of O.run with the eigen-solve reused
        g0r = O.realspace(O.greens_k(ev, U, c.kpoints, e, c.eta))
        T = O.tmatrix(v, g0r[0, 0])
        if jos:
            tip = O.josephson_tip(e, *jos)
            maps.append(O.wannier_josephson(c.lattice, c.kpoints, c.oversamp, c.window, c.spin, T, g0r, wf, tip).T)
        else:
            maps.append(O.wannier_ldos(c.lattice, c.kpoints, c.oversamp, c.window, m, c.spin, T, g0r, wf).T)
        del g0r
    return c, om, wf, E, np.stack(maps)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["C1", "C2", "C3", "CJ"])
def test_config_matches_oracle(built_lib, name, prec):
    import cqpi
    c, om, wf, E, ref = _oracle(name)
    eng = cqpi.Engine(om, c.lattice, c.kpoints, c.oversamp, c.window, c.eta, maxband=c.extra.get("maxband"),
                      spin=c.spin, precision=cqpi.PREC_FP64 if prec == "fp64" else cqpi.PREC_MIXED)
    eng.set_orbitals(wf)
    eng.set_scattering(np.array(c.scattering, complex))
    if "josephson" in c.extra:
        eng.set_josephson(*c.extra["josephson"])
    got = eng.run(E, f32=False, f64=True)[:, 0]
    kind = eng.contraction_kind()
    eng.close()
    if prec == "mixed" and name != "C1":
        # one spin block after the spin-degenerate reduction (C3) and the one-block Josephson
        # form (CJ) contract on the tensor cores
        assert kind == "tcgen05", kind
    errs = [float(np.abs(got[k] - ref[k]).max() / np.abs(ref[k]).max()) for k in range(len(E))]
    assert max(errs) <= TOL[prec], (name, prec, errs)
