"""Time the reference's own CPU build (oracle/_ref/calcqpi, compiled from its sources with the
project-written GSL/FFTW layer by oracle/build_ref.sh) against the oracle port that the
benchmark's cpu_baseline uses, on the same host, for one energy of the C2 workload
(t2g model, kpoints 1024, oversamp 10, window 2) on an n x n field of view.

TEST INFRASTRUCTURE ONLY (build container: oracle/_ref is an x86 build from the reference's
sources, which do not exist on the GPU machine).  The reference's per-energy cost is taken from
its own "Calculation of CLDOS" real time: (layers=3 - layers=1) / 2, which removes the
eigen-solve of layer 0.  The port's is G0(k) + FFT + T + the direct LDOS loop for one energy.

Usage: python oracle/time_ref_vs_port.py [n]   (default 64; prints one line per arm)
"""
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# the script's own folder would shadow the oracle package with oracle/oracle.py
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path[:0] = [ROOT, os.path.join(ROOT, "calcqpi-release_gb300")]

from cqpi import workloads as W  # noqa: E402
from oracle import formats as F  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cldos_real_seconds(stdout: str) -> float:
    line = [l for l in stdout.splitlines() if "Calculation of CLDOS" in l][0]
    d, h, m, s, us = (int(x) for x in re.findall(r"(\d+)d,\s+(\d+)h,\s+(\d+)m,\s+(\d+)s\s+(\d+)μs", line)[1])
    return ((d * 24 + h) * 60 + m) * 60 + s + us * 1e-6


def main(n=64):
    c, m, wf = W.config("C2")
    threads = os.cpu_count()
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    with tempfile.TemporaryDirectory() as d:
        F.write_hr(os.path.join(d, "model_hr.dat"), "C2", m.bands, W.t2g_c2().terms(), None)
        F.write_idl(os.path.join(d, "orbitals.idl"),
                    np.ascontiguousarray(np.transpose(wf.astype(np.float32), (0, 2, 1))), "orbitals",
                    scan_range=(1.0, 1.0), offset=(0.0, 0.0), bias=(0.0, 0.0))

        def run(layers):
            cfg = ['tbfile="model_hr.dat";', 'qpifile="q.idl";', "output=wannier;", f"lattice={n};",
                   f"kpoints={c.kpoints};", f"oversamp={c.oversamp};", f"window={c.window};", f"layers={layers};",
                   "energies=(-0.1,0.1);", f"eta={c.eta};", "scattering=(0.3,0.3,0.5);",
                   'idlorbitalfile="orbitals.idl";']
            with open(os.path.join(d, "in.cfg"), "w") as fh:
                fh.write("\n".join(cfg) + "\n")
            r = subprocess.run([os.path.join(HERE, "_ref", "calcqpi"), "in.cfg"], cwd=d, env=env,
                               capture_output=True, text=True, check=True)
            return cldos_real_seconds(r.stdout)

        t_ref = (run(3) - run(1)) / 2
    om = O.Model(m.bands, m.R, m.orb, m.t, None, m.efermi, m.scmaxbands)
    ev, U = O.bands(om, c.kpoints)
    t0 = time.perf_counter()
    g0r = O.realspace(O.greens_k(ev, U, c.kpoints, 0.0, c.eta))
    T = O.tmatrix(np.array(c.scattering, complex), g0r[0, 0])
    O.wannier_ldos(n, c.kpoints, c.oversamp, c.window, m.bands, c.spin, T, g0r, wf, rows=(0, n))
    t_port = time.perf_counter() - t0
    pix = (n * c.oversamp) ** 2
    print(f"reference build ({threads} threads): {t_ref:.2f} s/energy, {pix / t_ref:.3e} pixel*E/s")
    print(f"oracle port ({O.num_threads()} threads): {t_port:.2f} s/energy, {pix / t_port:.3e} pixel*E/s")
    print(f"port / reference speed: {t_ref / t_port:.2f}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 64)
