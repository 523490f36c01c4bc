"""Generate the golden fixtures under tests/golden/<case>/ from the reference itself.

The reference ships no tests or example data, so its known answers are recorded here:
for each case this script writes seeded inputs (a _hr.dat, an IDL orbital file or
analytic orbital keywords, a calcqpi input file), runs the reference CLI built from its
own sources (oracle/_ref/calcqpi, see oracle/build_ref.sh) and the float64 harness
oracle/_ref/refdump, and stores:

  model_hr.dat, orbitals.idl (when used), input.cfg   the inputs
  ref_qpi.idl                                         the reference's output map (float32)
  ref_wf.idl                                          the reference's wffile output (analytic cases)
  ref_ldos64.npz                                      float64 maps + tmatrix::calcdos per layer
  meta.json                                           the parameters

The bs_* cases record band-structure histograms (bsfile, output=nomode) of the reference's
CLI.  The mkwf_* cases do the same for the orbital-file tool (oracle/_ref/mkwavefunctions): the
inputs, input_<k>.cfg, the reference's IDL output ref_<k>.idl and its log ref_<k>.txt.

Run from the repository root:
    CQPI_REFERENCE=<reference checkout> python tests/golden/make_golden.py [case ...]
(requires the reference sources; CQPI_REFERENCE names the folder that holds src/qpi.cc).
"""
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "calcqpi-release_gb300"))

from cqpi import workloads as W  # noqa: E402
from oracle import formats as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def bdg_c1(delta=0.1):
    """Two-band BdG form of the C1 model: electron block t(R), hole block -t(R),
    on-site pairing delta (for scmodel=true)."""
    base = W.square_c1().terms()
    terms = {}
    for R, M in base.items():
        T = np.zeros((2, 2), complex)
        T[0, 0] = M[0, 0]
        T[1, 1] = -M[0, 0]
        terms[R] = T
    T0 = np.zeros((2, 2), complex)
    T0[0, 1] = T0[1, 0] = delta
    terms[(0, 0, 0)] = T0
    return terms


def bdg(base: dict, D: np.ndarray) -> dict:
    """BdG form of an electron model: electron block t(R), hole block -conj(t(R)) (the
    hole Hamiltonian -H(-k)^*), on-site pairing matrix D between the blocks (for
    scmodel=true).  Hermitian whenever the electron model is."""
    b = next(iter(base.values())).shape[0]
    terms = {}
    for R, M in base.items():
        T = np.zeros((2 * b, 2 * b), complex)
        T[:b, :b] = M
        T[b:, b:] = -np.conj(M)
        terms[R] = T
    T0 = terms.get((0, 0, 0), np.zeros((2 * b, 2 * b), complex)).copy()
    T0[:b, b:] += D
    T0[b:, :b] += np.conj(D).T
    terms[(0, 0, 0)] = T0
    return terms


def bdg_t2g():
    """Six-band BdG form of the C2 t2g model with an orbital-dependent on-site pairing."""
    D = np.diag([0.04, 0.04, 0.06]).astype(complex)
    D[0, 1] = D[1, 0] = 0.01
    return bdg(W.t2g_c2().terms(), D)


def bdg_spin():
    """Four-band BdG form of a spinful one-orbital square lattice (orbitals up, down; a
    Zeeman splitting of 0.05 on site) with equal-spin pairing 0.08 so that both spin
    blocks of the Josephson sum are non-zero."""
    base = {}
    for R, M in W.square_c1().terms().items():
        base[R] = M[0, 0] * np.eye(2, dtype=complex)
    T0 = base.get((0, 0, 0), np.zeros((2, 2), complex)).copy()
    T0 += np.diag([0.05, -0.05])
    base[(0, 0, 0)] = T0
    return bdg(base, 0.08 * np.eye(2, dtype=complex))


def stacked(base: dict, tz: dict) -> dict:
    """A layered model: the in-plane terms of base plus interlayer terms tz[(rx, ry)] at
    R_z = +1 and their Hermitian partners at R_z = -1 (principal-layer form)."""
    terms = {k: v.copy() for k, v in base.items()}
    for (rx, ry), M in tz.items():
        terms[(rx, ry, 1)] = terms.get((rx, ry, 1), 0) + M
        terms[(-rx, -ry, -1)] = terms.get((-rx, -ry, -1), 0) + np.conj(M).T
    return terms


def c1_layered():
    return stacked(W.square_c1().terms(), {(0, 0): np.array([[-0.4 + 0j]]), (1, 0): np.array([[0.1 + 0j]]),
                                           (-1, 0): np.array([[0.1 + 0j]])})


def c1_surface_layer():
    """The surface layer of c1_layered: in-plane hoppings with a 0.2 eV on-site shift."""
    terms = {k: v.copy() for k, v in W.square_c1().terms().items()}
    terms[(0, 0, 0)] = terms.get((0, 0, 0), np.zeros((1, 1), complex)) + 0.2
    return terms


def t2g_layered(seed=9):
    rng = np.random.default_rng(seed)
    tz = {(0, 0): 0.15 * (rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))),
          (1, 0): 0.05 * rng.normal(size=(3, 3)) + 0j}
    return stacked(W.t2g_c2().terms(), tz)


CASES = {
    "c1_idl": dict(model="c1", deg=2, n=12, kp=32, os=4, w=2, layers=3, energies=(-0.2, 0.2), eta=0.05,
                   scattering=(0.5,), orbitals=("idl", "gauss")),
    "c2_analytic": dict(model="c2", n=8, kp=16, os=3, w=2, layers=2, energies=(-0.1, 0.1), eta=0.02,
                        scattering=(0.3, 0.3, 0.5),
                        orbitals=("analytic", dict(names=["dxz", "dyz", "dxy"], radius=0.4, zheight=0.6))),
    "c3_spin": dict(model="c3", n=6, kp=12, os=2, w=1, layers=2, energies=(-0.05, 0.05), eta=0.02, spin=True,
                    orbitals=("idl", "tri5")),
    "edge_odd": dict(model="c1", fermi=0.1, phase=(0.5, 0.3), n=7, kp=12, os=3, w=1, layers=1,
                     energies=(0.05, 0.3), eta=0.03,
                     orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5, angle=30.0,
                                                pos={0: (0.1, 0.2, 0.1)}, prearr=(0.8,)))),
    "c2_pad": dict(model="c2", n=6, kp=16, os=2, w=1, layers=2, energies=(-0.1, 0.1), eta=0.02,
                   scattering=(0.3, 0.3, 0.5), orbitals=("idl", "t2g2")),
    "scmodel": dict(model="bdg", scmodel=True, magscat=0.25, n=8, kp=16, os=2, w=1, layers=2,
                    energies=(-0.1, 0.1), eta=0.03, scattering=(0.5,),
                    orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "josephson": dict(model="bdg", scmodel=True, magscat=0.25, n=8, kp=16, os=2, w=1, layers=3,
                      energies=(-0.12, 0.09), eta=0.03, scattering=(0.5,), josephson=(0.02, 0.01),
                      orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "josephson_t2g": dict(model="bdg_t2g", scmodel=True, magscat=0.0, n=6, kp=16, os=2, w=1, layers=2,
                          energies=(-0.06, 0.05), eta=0.02, scattering=(0.3, 0.3, 0.5), josephson=(None, None),
                          orbitals=("analytic", dict(names=["dxz", "dyz", "dxy"], radius=0.4, zheight=0.6))),
    "josephson_spin": dict(model="bdg_spin", scmodel=True, spin=True, magscat=0.1, n=6, kp=12, os=2, w=1,
                           layers=2, energies=(-0.1, 0.07), eta=0.03, scattering=(0.4,), josephson=(0.05, 0.02),
                           orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "threshold_c2": dict(model="c2", n=6, kp=16, os=3, w=2, layers=2, energies=(-0.1, 0.1), eta=0.02,
                         scattering=(0.3, 0.3, 0.5), threshold=0.05,
                         orbitals=("analytic", dict(names=["dxz", "dyz", "dxy"], radius=0.4, zheight=0.6))),
    "threshold_spin": dict(model="c3", n=6, kp=12, os=2, w=1, layers=2, energies=(-0.05, 0.05), eta=0.02,
                           spin=True, threshold=0.02, orbitals=("idl", "tri5")),
    "threshold_spinarr": dict(model="c2", n=5, kp=16, os=2, w=1, layers=2, energies=(-0.08, 0.06), eta=0.02,
                              scattering=(0.3, 0.3, 0.5), threshold=0.0, spinarr=(1, 0, 1),
                              orbitals=("idl", "t2g3")),
    "xsf_t2g": dict(model="c2", n=6, kp=16, os=3, w=2, layers=2, energies=(-0.1, 0.1), eta=0.02,
                    scattering=(0.3, 0.3, 0.5), orbitals=("xsf", dict(names=["dxz", "dyz", "dxy"], zheight=0.5))),
    "xsf_pad": dict(model="c2", n=5, kp=16, os=2, w=1, layers=2, energies=(-0.08, 0.05), eta=0.02,
                    scattering=(0.3, 0.3, 0.5),
                    orbitals=("xsf", dict(names=["dxz", "dxy"], zheight=0.75, prearr=(0.7, 1.3)))),
    "surface_c1": dict(model="c1z", green="surface", surface_model=True, n=8, kp=16, os=2, w=1, layers=2,
                       energies=(-0.3, 0.4), eta=0.05, scattering=(0.5,),
                       orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "bulk_t2g": dict(model="t2gz", green="bulk", epserr=1e-7, n=6, kp=16, os=2, w=1, layers=2,
                     energies=(-0.1, 0.15), eta=0.03, scattering=(0.3, 0.3, 0.5), orbitals=("idl", "t2g3")),
    "surface_t2g": dict(model="t2gz", green="surface", n=6, kp=16, os=2, w=1, layers=1,
                        energies=(0.05, 0.05), eta=0.03, scattering=(0.3, 0.3, 0.5), orbitals=("idl", "t2g3")),
    "spf_t2g": dict(model="c2", output="spf", n=16, kp=16, os=2, w=1, layers=2, energies=(-0.1, 0.1), eta=0.02,
                    scattering=(0.3, 0.3, 0.5), orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "uspf_t2g": dict(model="c2", output="uspf", n=16, kp=16, os=2, w=1, layers=2, energies=(-0.05, 0.08),
                     eta=0.02, scattering=(0.3, 0.3, 0.5), pos={0: (0.1, 0.2), 1: (-0.2, 0.1)},
                     prearr=(1.0, 0.8, 1.2), orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "uspf_rect": dict(model="c1", output="uspf", n=12, kp=16, os=2, w=1, layers=1, energies=(0.2, 0.2), eta=0.05,
                      scattering=(0.5,), pos={0: (0.25, 0.0)},
                      orbitals=("analytic", dict(names=["s"], radius=0.3, zheight=0.5))),
    "dos_c2": dict(model="c2", n=6, kp=16, os=2, w=1, layers=1, energies=(0.02, 0.02), eta=0.02,
                   scattering=(0.3, 0.3, 0.5), dosfile=dict(layers=7, energies=(-0.2, 0.25)),
                   orbitals=("idl", "t2g3")),
    "wrap": dict(model="c1", n=20, kp=8, os=2, w=1, layers=1, energies=(0.1, 0.1), eta=0.05, scattering=(0.7,),
                 orbitals=("analytic", dict(names=["px"], radius=0.35, zheight=0.4, angle=20.0))),
}


def model_terms(c):
    if c["model"] == "c1":
        m = W.square_c1()
        return m.name, m.bands, m.terms()
    if c["model"] == "c2":
        m = W.t2g_c2()
        return m.name, m.bands, m.terms()
    if c["model"] == "c3":
        m = W.triangular_c3()
        return m.name, m.bands, m.terms()
    if c["model"] == "bdg":
        return "BdG square lattice (scmodel)", 2, bdg_c1()
    if c["model"] == "c1z":
        return "layered square lattice", 1, c1_layered()
    if c["model"] == "t2gz":
        return "layered t2g square lattice", 3, t2g_layered()
    if c["model"] == "bdg_t2g":
        return "BdG t2g model (scmodel)", 6, bdg_t2g()
    if c["model"] == "bdg_spin":
        return "BdG spinful square lattice (scmodel)", 4, bdg_spin()
    raise KeyError(c["model"])


def orbital_cube(kind, w, os_):
    if kind == "gauss":
        return W.gaussian_c1(w, os_)
    if kind == "tri5":
        return W.tri_orbitals_c3(w, os_)
    if kind == "t2g2":
        return W.t2g_orbitals_c2(w, os_)[:2]
    if kind == "t2g3":
        return W.t2g_orbitals_c2(w, os_)
    raise KeyError(kind)


XSF_GRID = dict(origin=(-2.5, -2.5, -1.0), axes=((5.0, 0.0, 0.0), (0.0, 5.0, 0.0), (0.0, 0.0, 4.0)),
                shape=(40, 40, 16), convvec=((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 8.0)))


def xsf_cubes(names, seed=5, sigma=0.6, grid=None):
    """Seeded Wannier-like orbitals on the XSF grid: d angular part (centred on the atom at
    the origin) times a Gaussian, plus 5% seeded noise so that no symmetry hides an index
    error.  Grid points r = origin + (i/xs, j/ys, k/zs) . axes, as the reference reads them."""
    g = grid or XSF_GRID
    xs, ys, zs = g["shape"]
    i, j, k = np.meshgrid(np.arange(xs), np.arange(ys), np.arange(zs), indexing="ij")
    X = g["origin"][0] + g["axes"][0][0] * i / xs
    Y = g["origin"][1] + g["axes"][1][1] * j / ys
    Z = g["origin"][2] + g["axes"][2][2] * k / zs
    rad = np.exp(-(X * X + Y * Y + Z * Z) / sigma ** 2)
    ang = {"dxz": X * Z, "dyz": Y * Z, "dxy": X * Y, "s": np.ones_like(X), "pz": Z}
    rng = np.random.default_rng(seed)
    return [ang[nm] * rad * (1.0 + 0.05 * rng.normal(size=X.shape)) for nm in names]


def fmt_list(v):
    return "(" + ",".join(repr(float(x)) for x in v) + ")"


def make_case(name, c):
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    mname, bands, terms = model_terms(c)
    deg = None
    if c.get("deg"):
        deg = {k: c["deg"] for k in terms}
    F.write_hr(os.path.join(d, "model_hr.dat"), mname, bands, terms, deg)
    w, os_, n, kp = c["w"], c["os"], c["n"], c["kp"]
    scmodel = c.get("scmodel", False)
    spin = c.get("spin", False)
    maxband = bands >> 1 if scmodel else bands
    jos = c.get("josephson")
    outmode = c.get("output", "josephson" if jos else "wannier")
    lines = ['tbfile="model_hr.dat";', 'qpifile="ref_qpi.idl";', f"output={outmode};",
             f"lattice={n};", f"kpoints={kp};", f"oversamp={os_};", f"window={w};", f"layers={c['layers']};",
             f"energies={fmt_list(c['energies'])};", f"eta={c['eta']!r};"]
    if "fermi" in c:
        lines.append(f"fermi={c['fermi']!r};")
    if "phase" in c:
        lines.append(f"phase={fmt_list(c['phase'])};")
    if "scattering" in c:
        lines.append(f"scattering={fmt_list(c['scattering'])};")
    if "green" in c:
        lines.append(f"green={c['green']};")
        if "epserr" in c:
            lines.append(f"epserr={c['epserr']!r};")
        if c.get("surface_model"):
            F.write_hr(os.path.join(d, "surf_hr.dat"), "surface layer", bands, c1_surface_layer(), None)
            lines.append('stbfile="surf_hr.dat";')
    if "threshold" in c:
        lines.append(f"threshold={c['threshold']!r};")
    if outmode == "uspf":
        for i, pxy in c.get("pos", {}).items():
            lines.append(f"pos[{i}]={fmt_list(pxy)};")
        if "prearr" in c:
            lines.append(f"prearr={fmt_list(c['prearr'])};")
    if "dosfile" in c:
        lines.append('dosfile="ref_dos.txt";')
        lines.append(f"doslayers={c['dosfile']['layers']};")
        lines.append(f"dosenergies={fmt_list(c['dosfile']['energies'])};")
    if "spinarr" in c:
        lines.append("spinarr=(" + ",".join(str(int(v)) for v in c["spinarr"]) + ");")
    if jos:
        if jos[0] is not None:
            lines.append(f"deltat={jos[0]!r};")
        if jos[1] is not None:
            lines.append(f"etat={jos[1]!r};")
    if spin:
        lines.append("spin=true;")
    if scmodel:
        lines.append("scmodel=true;")
        lines.append(f"magscat={c['magscat']!r};")
    kind, spec = c["orbitals"]
    side = (2 * w + 1) * os_
    if kind == "idl":
        cube = orbital_cube(spec, w, os_).astype(np.float32)
        # file layout data[x][y][orbital] written x fastest (idl.cc:78-97): [orb][y][x]
        F.write_idl(os.path.join(d, "orbitals.idl"), np.ascontiguousarray(np.transpose(cube, (0, 2, 1))),
                    "orbital cube", scan_range=(1.0, 1.0), offset=(0.0, 0.0), bias=(0.0, 0.0),
                    date="Thu Jan  1 00:00:00 2026")
        lines.append('idlorbitalfile="orbitals.idl";')
        wf64 = cube.astype(np.float64)
        if spin and (maxband >> 1) == wf64.shape[0]:
            wf64 = np.concatenate([wf64, wf64])
        zero = np.zeros(max(maxband, wf64.shape[0]), np.uint8)
        if wf64.shape[0] < maxband:
            zero[wf64.shape[0]:] = 1
            wf64 = np.concatenate([wf64, np.zeros((maxband - wf64.shape[0], side, side))])
    elif kind == "xsf":
        names = spec["names"]
        files = []
        for q, cube in enumerate(xsf_cubes(names)):
            fn = "orb%d.xsf" % q
            F.write_xsf(os.path.join(d, fn), cube, XSF_GRID["origin"], XSF_GRID["axes"], XSF_GRID["convvec"],
                        [("Fe", 0.0, 0.0, 0.0)], comment="seeded %s-like orbital" % names[q])
            files.append(fn)
        lines.append("orbitalfiles=(" + ",".join('"%s"' % fn for fn in files) + ");")
        lines.append(f"zheight={spec['zheight']!r};")
        pre = spec.get("prearr", (1.0,) * len(files))
        if "prearr" in spec:
            lines.append(f"prearr={fmt_list(pre)};")
        # with fewer files than bands the reference appends zero orbitals without a cache and
        # its wffile output then crashes (segmentation fault): ask for wffile only otherwise
        if len(files) >= maxband or (spin and (maxband >> 1) == len(files)):
            lines.append('wffile="ref_wf.idl";')
        wf64 = np.stack([F.xsf_orbital_cache(os.path.join(d, fn), spec["zheight"], w, os_, pre[q])
                         for q, fn in enumerate(files)])
        # the driver pads with maxband zero orbitals when fewer files than bands are given
        # (src/calcqpi.cc:596-599 counts from the empty analytic orbital list)
        zero = np.zeros(wf64.shape[0], np.uint8)
        if spin and (maxband >> 1) == len(files):
            wf64 = np.concatenate([wf64, wf64])
            zero = np.zeros(wf64.shape[0], np.uint8)
        elif len(files) < maxband:
            wf64 = np.concatenate([wf64, np.zeros((maxband, side, side))])
            zero = np.concatenate([zero, np.ones(maxband, np.uint8)])
        xsf_args = ["X", repr(spec["zheight"]), str(len(files))]
        for q, fn in enumerate(files):
            xsf_args += [os.path.join(d, fn), repr(float(pre[q]))]
    else:
        names = spec["names"]
        lines.append("orbitals=(" + ",".join(names) + ");")
        lines.append(f"radius={spec['radius']!r};")
        lines.append(f"zheight={spec['zheight']!r};")
        if "angle" in spec:
            lines.append(f"angle={spec['angle']!r};")
        for i, p in spec.get("pos", {}).items():
            lines.append(f"pos[{i}]={fmt_list(p)};")
        if "prearr" in spec:
            lines.append(f"prearr={fmt_list(spec['prearr'])};")
        lines.append('wffile="ref_wf.idl";')
        cubes = []
        for i, nm in enumerate(names):
            # pos[i] lines (orbital spec, or the uspf band positions) also place the orbitals
            pos = tuple({**c.get("pos", {}), **spec.get("pos", {})}.get(i, (0.0, 0.0, 0.0)))
            pos = pos + (0.0,) * (3 - len(pos))
            pre = spec.get("prearr", (1.0,) * len(names))[i] if i < len(spec.get("prearr", ())) else 1.0
            cubes.append(O.orbital_cache(nm, w, os_, width=spec["radius"], height=spec["zheight"] - pos[2],
                                         xpos=pos[0], ypos=pos[1],
                                         theta=spec.get("angle", 0.0) * np.pi / 180.0, prefact=pre))
        wf64 = np.stack(cubes)
        zero = np.zeros(max(maxband, wf64.shape[0]), np.uint8)
        if spin and (maxband >> 1) == len(names):
            wf64 = np.concatenate([wf64, wf64])
        elif wf64.shape[0] < maxband:
            zero[wf64.shape[0]:] = 1
            wf64 = np.concatenate([wf64, np.zeros((maxband - wf64.shape[0], side, side))])
    with open(os.path.join(d, "input.cfg"), "w") as fh:
        fh.write("# golden case %s (generated by tests/golden/make_golden.py)\n" % name)
        fh.write("\n".join(lines) + "\n")
    # reference CLI
    r = subprocess.run([os.path.join(REF, "calcqpi"), "input.cfg"], cwd=d, capture_output=True, text=True,
                       timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: reference failed\n{r.stdout}\n{r.stderr}")
    # float64 harness
    scat = [complex(v) for v in c.get("scattering", ())]
    phase = complex(*c.get("phase", (1.0, 0.0)))
    scat = [s * phase for s in scat]
    if scmodel and len(scat) == maxband:
        scat = scat + [(-1.0 + 2.0 * c["magscat"]) * s for s in scat]
    vscat = [scat[i] if i < len(scat) else 0j for i in range(bands)] if scat else [phase] * bands
    wfbin = os.path.join(d, "_wf.bin")
    with open(wfbin, "wb") as fh:
        fh.write(np.array([wf64.shape[0], side], np.int32).tobytes())
        fh.write(np.ascontiguousarray(wf64 * (1 - zero[:wf64.shape[0], None, None])).tobytes())
    outbin = os.path.join(d, "_ldos.bin")
    spfm = outmode in ("spf", "uspf")
    os_run = 1 if spfm else os_
    kp_run = n if outmode == "spf" else kp          # output=spf runs on an n x n k-grid (src/calcqpi.cc:333-334)
    args = [os.path.join(REF, "refdump"), os.path.join(d, "model_hr.dat"), wfbin, outbin, str(n), str(kp_run),
            str(os_run),
            str(w), repr(c["eta"]), repr(c.get("fermi", 0.0)), str(int(spin)), str(maxband), str(c["layers"]),
            repr(c["energies"][0]), repr(c["energies"][1]), str(int(scmodel)), str(len(vscat))]
    for v in vscat:
        args += [repr(v.real), repr(v.imag)]
    if kind == "xsf":
        args += xsf_args
    if "green" in c:
        args += ["G", c["green"], repr(c.get("epserr", 1e-5)),
                 os.path.join(d, "surf_hr.dat") if c.get("surface_model") else "-"]
    if "threshold" in c and not jos:
        if "spinarr" in c:
            args += ["S", repr(c["threshold"]), str(len(c["spinarr"]))] + [str(int(v)) for v in c["spinarr"]]
        else:
            args += ["T", repr(c["threshold"])]
    if outmode == "spf":
        args += ["P"]
    elif outmode == "uspf":
        args += ["U", str(maxband)]
        pre = list(c.get("prearr", ())) + [1.0] * maxband
        for i in range(maxband):
            pxy = c.get("pos", {}).get(i, (0.0, 0.0))
            args += [repr(float(pxy[0])), repr(float(pxy[1])), repr(float(pre[i]))]
    if jos:
        # the driver's defaults: deltat 0.001, etat = eta (src/calcqpi.cc:137,249-251)
        args += ["J", repr(0.001 if jos[0] is None else jos[0]), repr(c["eta"] if jos[1] is None else jos[1])]
    r2 = subprocess.run(args, capture_output=True, text=True, timeout=600)
    if r2.returncode != 0:
        raise RuntimeError(f"{name}: refdump failed\n{r2.stderr}")
    wn = n * os_run
    raw = np.fromfile(outbin, np.float64).reshape(c["layers"], 1 + wn * wn)
    np.savez_compressed(os.path.join(d, "ref_ldos64.npz"), dos=raw[:, 0], ldos=raw[:, 1:].reshape(-1, wn, wn),
                        vscat=np.array(vscat), wf=wf64, zero=zero)
    os.remove(wfbin)
    os.remove(outbin)
    meta = dict(c)
    meta["bands"] = bands
    meta["maxband"] = maxband
    meta["orbitals"] = [kind, spec]
    with open(os.path.join(d, "meta.json"), "w") as fh:
        json.dump(meta, fh, indent=1, default=str)
    with open(os.path.join(d, "ref_stdout.txt"), "w") as fh:
        fh.write(r.stdout + r.stderr)
    print(name, "ok", wn, "x", wn, "x", c["layers"])


# ------------------------------------------------------------------ mkwavefunctions
MKWF_XSF_GRID = dict(XSF_GRID, shape=(28, 28, 10))
# Cases of the orbital-file tool: tests/golden/mkwf_<case>/ holds the inputs, one
# input_<k>.cfg per configuration, the reference's outputs ref_<k>.idl and its log
# ref_<k>.txt (oracle/_ref/mkwavefunctions, built from src/mkwavefunctions.cc).
MKWF_INTERP_METHODS = ("linear", "polynomial", "cspline", "cspline_periodic", "akima", "akima_periodic", "steffen")

MKWF_CASES = {
    # analytic orbitals with every per-orbital keyword, lattice basis vectors, reorder, double
    "mkwf_analytic": dict(kind="analytic", configs={
        "basis": ["window=2;", "oversamp=4;", "orbitals=(dxy,dx2,pz,s,fxyz,n);", "radarr=(0.5,0.7,0.6);",
                  "anglearr=(10,0,30,0,5,20);", "phiarr=(0,20,0,0,15,0);", "prearr=(1.0,0.5,2.0);",
                  "pos[1]=(0.25,0.1,0.2);", "pos[4]=(-0.2,0.3);", "basisvector[0]=(1,0);",
                  "basisvector[1]=(0.5,0.866);", "zheight=1.5;", "reorder=(2,0,1,5,4,3);", "double=1;"],
        "plain": ["window=1;", "oversamp=5;", "orbitals=(dxz,dyz,dr2,fy3x2,z);", "radius=0.8;", "angle=12;",
                  "zheight=0.9;", "pos[2]=(0.1,-0.1,0.3);"],
    }),
    # XSF orbitals with a global shift and centred pixels (orbitalfiles)
    "mkwf_xsf": dict(kind="xsf", names=("dxz", "dyz", "dxy"), configs={
        "shift": ["window=2;", "oversamp=3;", 'orbitalfiles=("orb0.xsf","orb1.xsf","orb2.xsf");',
                  "shift=(0.3,-0.2,0.1);", "prearr=(1.0,-0.5,2.0);", "zheight=0.7;"],
        "noshift": ["window=1;", "oversamp=4;", 'orbitalfiles=("orb2.xsf","orb0.xsf");', "zheight=-0.4;"],
    }),
    # XSF orbitals placed per orbital (modorbitalfiles): file indices, modpos, pos, rotation,
    # basis vectors in Angstrom
    "mkwf_mod": dict(kind="xsf", names=("dxz", "dxy"), configs={
        "basis": ["window=2;", "oversamp=3;", 'modorbitalfiles=("orb0.xsf","orb1.xsf");',
                  "modpos[0]=(0.2,0.1,0.0);", "modpos[1]=(-0.1,0.3,0.2);", "orbitals=(0,1,1);",
                  "pos[1]=(0.25,0.25,0.1);", "pos[2]=(0.5,0);", "angle=15;", "anglearr=(0,10,45);",
                  "zheight=0.6;", "basisvector[0]=(0.9,0.0);", "basisvector[1]=(0.45,0.78);"],
        "plain": ["window=1;", "oversamp=4;", 'modorbitalfiles=("orb1.xsf");', "orbitals=(0,0);",
                  "anglearr=(0,90);", "zheight=0.5;"],
    }),
    # an IDL orbital file scaled by prearr (idlorbitalfile)
    "mkwf_idl": dict(kind="idl", configs={
        "prearr": ["window=2;", "oversamp=3;", 'idlorbitalfile="orbitals.idl";', "prearr=(2.0,-1.0);",
                   "double=1;"],
    }),
    # pixel-wise interpolation between five IDL orbital files (idlorbitalfiles)
    "mkwf_interp": dict(kind="interp", configs={
        m: ["window=1;", "oversamp=4;",
            'idlorbitalfiles=("in0.idl","in1.idl","in2.idl","in3.idl","in4.idl");',
            "values=(0.0,0.2,0.5,0.7,1.0);", "interpolate=0.35;", 'interpmethod="%s";' % m]
        for m in MKWF_INTERP_METHODS
    } | {"default": ["window=1;", "oversamp=4;",
                     'idlorbitalfiles=("in0.idl","in1.idl","in2.idl","in3.idl","in4.idl");']}),
}


def _write_idl_cube(path, cube):
    """cube[orbital][i][j] -> IDL data x fastest ([orb][y][x] in the file)."""
    F.write_idl(path, np.ascontiguousarray(np.transpose(np.asarray(cube, np.float32), (0, 2, 1))), "orbital cube",
                scan_range=(1.0, 1.0), offset=(0.0, 0.0), bias=(0.0, 0.0), date="Thu Jan  1 00:00:00 2026")


def make_mkwf_case(name, c):
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    rng = np.random.default_rng(17)
    if c["kind"] == "xsf":
        g = MKWF_XSF_GRID
        for q, cube in enumerate(xsf_cubes(c["names"], seed=11, grid=g)):
            F.write_xsf(os.path.join(d, "orb%d.xsf" % q), cube, g["origin"], g["axes"], g["convvec"], [("Fe", 0.0, 0.0, 0.0), ("O", 0.3, 0.2, -0.4)],
                        comment="seeded %s-like orbital" % c["names"][q])
    elif c["kind"] == "idl":
        side = 5 * 3
        _write_idl_cube(os.path.join(d, "orbitals.idl"), rng.normal(size=(2, side, side)))
    elif c["kind"] == "interp":
        side = 3 * 4
        base = rng.normal(size=(2, side, side))
        # a smooth, non-monotone family in the parameter plus seeded noise per file
        for q, v in enumerate((0.0, 0.2, 0.5, 0.7, 1.0)):
            cube = base * np.cos(2.0 * v) + 0.3 * np.sin(5.0 * v) + 0.05 * rng.normal(size=base.shape)
            _write_idl_cube(os.path.join(d, "in%d.idl" % q), cube)
    meta = {"configs": {}}
    for k, lines in c["configs"].items():
        cfg = ["# mkwavefunctions golden case %s/%s (generated by tests/golden/make_golden.py)" % (name, k),
               'tbfile="model_hr.dat";', 'mkwffile="ref_%s.idl";' % k] + lines
        with open(os.path.join(d, "input_%s.cfg" % k), "w") as fh:
            fh.write("\n".join(cfg) + "\n")
        r = subprocess.run([os.path.join(REF, "mkwavefunctions"), "input_%s.cfg" % k], cwd=d, capture_output=True,
                           text=True, timeout=120)
        if r.returncode != 0:
            raise RuntimeError("reference mkwavefunctions failed for %s/%s:\n%s%s" % (name, k, r.stdout, r.stderr))
        with open(os.path.join(d, "ref_%s.txt" % k), "w") as fh:
            fh.write(r.stdout)
        meta["configs"][k] = {"exact": c["kind"] != "interp"}
    with open(os.path.join(d, "meta.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    print("golden", name, "configs", list(c["configs"]))


# ------------------------------------------------------------------ bsfile
# Band-structure histograms (tightbind::calcbst3dhisthr through the driver's bsfile keyword,
# output=nomode): tests/golden/bs_<case>/ holds model_hr.dat, input.cfg, the reference's
# ref_bs.idl and its log.  The reference runs single-threaded: its OpenMP loop can let two
# threads add into one pixel at once.
BS_CASES = {
    "bs_t2g": dict(model="t2g", keys=["bslattice=24;", "bsoversamp=3;", "bsenergies=(-0.6,0.4);",
                                       "bslayers=15;", "fermi=0.05;"]),
    "bs_bdg": dict(model="bdg_t2g", keys=["scmodel=true;", "bslattice=16;", "bsoversamp=4;",
                                          "bsenergies=(-0.3,0.3);", "bslayers=9;"]),
    "bs_layered": dict(model="c1_layered", keys=["bslattice=20;", "bsoversamp=2;", "bsenergies=(-2.0,2.0);",
                                                 "bslayers=31;"]),
}


def make_bs_case(name, c):
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    terms = {"t2g": lambda: W.t2g_c2().terms(), "bdg_t2g": bdg_t2g, "c1_layered": c1_layered}[c["model"]]()
    bands = next(iter(terms.values())).shape[0]
    F.write_hr(os.path.join(d, "model_hr.dat"), "band-structure case %s" % name, bands, terms, None)
    cfg = ["# band-structure histogram case %s (generated by tests/golden/make_golden.py)" % name,
           'tbfile="model_hr.dat";', "output=nomode;", 'bsfile="ref_bs.idl";'] + c["keys"]
    with open(os.path.join(d, "input.cfg"), "w") as fh:
        fh.write("\n".join(cfg) + "\n")
    r = subprocess.run([os.path.join(REF, "calcqpi"), "input.cfg"], cwd=d, capture_output=True, text=True,
                       timeout=600, env=dict(os.environ, OMP_NUM_THREADS="1"))
    if r.returncode != 0 or not os.path.exists(os.path.join(d, "ref_bs.idl")):
        raise RuntimeError("reference bsfile run failed for %s:\n%s%s" % (name, r.stdout, r.stderr))
    with open(os.path.join(d, "ref_stdout.txt"), "w") as fh:
        fh.write(r.stdout)
    print("golden", name)


# ------------------------------------------------------------------ keywords
def write_keywords():
    """The input keywords the reference's programs read (loadconfig::probefield with a literal
    name in src/calcqpi.cc and src/mkwavefunctions.cc), one per line, for the keyword
    coverage test of the CLI and the orbital-file tool."""
    import re
    root = reference_root()
    for prog in ("calcqpi", "mkwavefunctions"):
        with open(os.path.join(root, "src", prog + ".cc")) as fh:
            names = sorted(set(re.findall(r'probefield\("([^"]+)"\)', fh.read())))
        with open(os.path.join(HERE, "ref_%s_keywords.txt" % prog), "w") as fh:
            fh.write("# keywords read by src/%s.cc (generated by tests/golden/make_golden.py)\n" % prog)
            fh.write("\n".join(names) + "\n")
        print("keywords", prog, len(names))


def reference_root():
    """The reference checkout whose sources the fixtures are generated from: the
    CQPI_REFERENCE environment variable (required; there is no default location)."""
    root = os.environ.get("CQPI_REFERENCE")
    if not root or not os.path.isfile(os.path.join(root, "src", "qpi.cc")):
        raise SystemExit("set CQPI_REFERENCE to the reference checkout (the folder holding src/qpi.cc)")
    return root


if __name__ == "__main__":
    if not os.path.exists(os.path.join(REF, "mkwavefunctions")):
        subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), reference_root()])
    names = [a for a in sys.argv[1:] if a != "keywords"]
    if not sys.argv[1:] or "keywords" in sys.argv[1:]:
        write_keywords()
    if not sys.argv[1:]:
        names = list(CASES) + list(MKWF_CASES) + list(BS_CASES)
    for nm in names:
        if nm in MKWF_CASES:
            make_mkwf_case(nm, MKWF_CASES[nm])
        elif nm in BS_CASES:
            make_bs_case(nm, BS_CASES[nm])
        else:
            make_case(nm, CASES[nm])
