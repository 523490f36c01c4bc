#!/usr/bin/env python
"""Benchmark of the continuum-LDOS path (pixel*energies/s) on the 3-orbital t2g model.

Workload (default --config C2): square-lattice t2g model (dxz, dyz, dxy), hoppings to
3rd neighbours N(0, 0.25 eV) with C4 symmetry (seed 2), V = diag(0.3, 0.3, 0.5) eV,
k-grid 1024^2, field of view 256^2 sites, 10x10 pixels per cell, 101 energies in
[-0.1, 0.1] eV, eta = 2 meV.  Synthetic inputs generated from seeds (no dataset).

One step = one complete job: H(k) + eigen-solve of all 1024^2 k-points, then for each
of the 101 energies G0(k) -> pruned FFT -> T-matrix -> LDOS map; the maps (101 x
2560^2 float32 = 2.6 GB) are written to HBM.  Inputs and outputs are far larger than
the 129 MB L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
  python bench.py --impl reference ...   # the reference's CPU algorithm on host cores

Under torchrun (N > 1) every rank runs the same job on its own GPU (replicas: energies,
impurities and fields of view are independent units; there is no data-path
collective); the time is the max over ranks and value is the sum of all ranks' work.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "calcqpi-release_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "LDOS pixel*energies/s"
UNIT = "pixel*energies/s"


def ldos_flops_per_pixel_energy(b, m, W, spin, josephson=False):
    """Algorithmic FLOPs of the factored contraction per pixel*energy:
    8*W*m_eff*b (u and s, complex x real MACs) + 8*b^2 (T s) + 4*b (Im u.Ts) per spin block;
    the Josephson form adds Re u.Ts (4*b) and the tip product (3)."""
    nblk = 2 if spin else 1
    mb = (m >> 1) if spin else m
    return nblk * (8 * W * mb * b + 8 * b * b + 4 * b + (4 * b + 3 if josephson else 0))


def workload_desc(name, c, m, nE):
    kind = {"C1": "square 1-orbital lattice", "C2": "t2g 3-orbital square lattice",
            "C3": "triangular 5-orbital x spin lattice", "C5": "t2g 3-orbital square lattice",
            "CJ": "Josephson mode (output=josephson) on the 6-band BdG t2g square lattice",
            "CS": "surface Green's function (green=surface) of the layered t2g lattice"}.get(name, name)
    return (f"{name}: {kind}, k-grid {c.kpoints}^2, FOV {c.lattice}^2 sites, {c.oversamp}x{c.oversamp} px/cell, "
            f"{nE} energies, eta={c.eta}")


def make_engine(cqpi, c, m, wf, vscat, prec):
    """Engine of a workload with its orbitals, scattering and (CJ) Josephson tip."""
    eng = cqpi.Engine(m, c.lattice, c.kpoints, c.oversamp, c.window, c.eta, maxband=c.extra.get("maxband"),
                      spin=c.spin, precision=prec)
    eng.set_orbitals(wf)
    eng.set_scattering(vscat)
    if "josephson" in c.extra:
        eng.set_josephson(*c.extra["josephson"])
    if "green" in c.extra:
        eng.set_greens(c.extra["green"], c.extra.get("epserr", 1e-5))
    return eng


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax = max(smax, float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            os.remove(self.path)
        except Exception:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def cpu_sample(cfg_name, target_s=8.0, threads=None):
    """Time the reference's CPU algorithm (oracle port of src/qpi.cc:478-950) on one
    energy of the workload: G0(k) + FFT + T on the full k-grid, the direct LDOS loop
    on the first R site rows, R chosen for ~target_s seconds.  Returns (pixel*E/s
    extrapolated to the full energy, cores, description)."""
    from cqpi import workloads as W
    from oracle import oracle as O
    if threads:
        O.set_threads(threads)
    c, m, wf = W.config(cfg_name)
    om = O.Model(m.bands, m.R, m.orb, m.t, None, m.efermi, m.scmaxbands)
    # the eigen-solve is once per run in the reference and not part of the sample
    ev, U = O.bands(om, c.kpoints) if not c.extra.get("green") else (None, None)
    e = float(c.energy_list()[len(c.energy_list()) // 2])
    t0 = time.perf_counter()
    if c.extra.get("green"):   # tmatrix::calcsurfacegreensfunction, src/qpi.cc:488-554
        g0k = O.surface_greens_k(om, c.kpoints, e, c.eta, c.extra.get("epserr", 1e-5), c.extra["green"] == "surface")
    else:
        g0k = O.greens_k(ev, U, c.kpoints, e, c.eta)
    g0r = O.realspace(g0k)
    T = O.tmatrix(np.array(c.scattering, complex), g0r[0, 0])
    tg = time.perf_counter() - t0
    jos = c.extra.get("josephson")
    tip = O.josephson_tip(e, *jos) if jos else None

    def contraction(rows):
        if jos:   # tmatrix::calcwannierjosephson, src/qpi.cc:953-1033
            return O.wannier_josephson(c.lattice, c.kpoints, c.oversamp, c.window, c.spin, T, g0r, wf, tip, rows=rows)
        return O.wannier_ldos(c.lattice, c.kpoints, c.oversamp, c.window, m.bands, c.spin, T, g0r, wf, rows=rows)

    t0 = time.perf_counter()
    contraction((0, 2))
    t2 = time.perf_counter() - t0
    rows = int(max(2, min(c.lattice, round(2 * target_s / max(t2, 1e-3)))))
    t0 = time.perf_counter()
    contraction((0, rows))
    tl = time.perf_counter() - t0
    t_energy = tg + tl * c.lattice / rows
    value = c.pixels_per_energy / t_energy
    desc = (f"{cfg_name}, 1 energy: G0(k)+FFT+T on the full {c.kpoints}^2 k-grid ({tg:.2f} s) + direct LDOS "
            f"loop on {rows}/{c.lattice} site rows ({tl:.2f} s), extrapolated to the full energy "
            f"({c.pixels_per_energy} pixels); eigen-solve excluded as in the reference's layer-0 timing")
    return value, O.num_threads(), desc


def max_over_ranks(x, dist, device):
    """The largest x over all ranks of the process group (every rank passes its own x and gets
    the maximum back); x itself without a process group.  Replicas finish when the slowest
    one does, so the job's time is the maximum."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, work_per_rank, seconds):
    """Units all ranks processed per second: each of the world replicas did work_per_rank
    units (weak scaling), and the job took the slowest rank's time."""
    return world * work_per_rank / seconds


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    vals = []
    desc, cores = "", 1
    for i in range(args.warmup + args.steps):
        v, cores, desc = cpu_sample(args.config, target_s=args.cpu_seconds / 2)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{args.config} continuum LDOS (reference CPU algorithm, oracle port)"
                                   if args.config != "CJ" else
                                   "CJ Josephson-mode maps (reference CPU algorithm, oracle port)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    world, rank, local = dist_setup()
    import torch
    import cqpi_build
    cqpi_build.build()
    import cqpi
    from cqpi import workloads as W
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    prec = cqpi.PREC_MIXED if args.precision == "mixed" else cqpi.PREC_FP64
    c, m, wf = W.config(args.config)
    if args.fov:                 # reduced field of view (profiling captures); the headline uses the config's
        c.lattice = args.fov
    E = c.energy_list()
    if args.energies:
        E = np.linspace(E[0], E[-1], args.energies)
    nE = len(E)
    vscat = np.array(c.scattering, complex)
    if len(vscat) < m.bands:
        vscat = np.concatenate([vscat, np.zeros(m.bands - len(vscat), complex)])
    eng = make_engine(cqpi, c, m, wf, vscat, prec)
    wn = c.lattice * c.oversamp
    out = torch.empty((nE, 1, wn, wn), dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(eng.stream)

    stage_acc = {"bands": 0.0, "greens": 0.0, "tmatrix": 0.0, "ldos": 0.0, "total": 0.0}

    tune = None
    if prec != cqpi.PREC_FP64 and eng.contraction_kind() == "tcgen05" and not args.no_autotune:
        try:
            ms_t, n_t = eng.autotune(E)
            tune = {"shapes_timed": n_t, "batch_ms": ms_t}
        except cqpi.CqpiError:
            tune = None

    def step():
        eng.solve_bands()
        eng.run_device(E, ptr32=out.data_ptr())

    for _ in range(args.warmup):
        step()
    eng.synchronize()
    eng.stage_times()           # clears the warm-up intervals
    launches0 = eng.kernel_launches()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    ev1.synchronize()
    eng.synchronize()
    stage_acc.update(eng.stage_times())   # CUDA-event totals of the K timed steps
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = eng.kernel_launches() - launches0
    ms = max_over_ranks(ms, dist, "cuda")
    work_per_rank = c.pixels_per_energy * nE
    value = whole_job_rate(world, work_per_rank, ms / 1e3)

    # e2e through the public API with host buffers, as a serving host would call it: one
    # handle; every step uploads the model's hopping amplitudes, the orbitals and the
    # scattering potential from host arrays (so the eigen-solve is redone), runs all energies
    # and reads the maps back into page-locked host memory.
    host_out = torch.empty((nE * wn * wn,), dtype=torch.float32, pin_memory=True).numpy()
    t_host = np.ascontiguousarray(np.asarray(m.t, np.complex128))
    h2d = t_host.nbytes + wf.nbytes + vscat.nbytes + E.nbytes
    d2h = host_out.nbytes
    e2e_steps = max(3, min(args.steps, 7))
    e2 = make_engine(cqpi, c, m, wf, vscat, prec)

    def e2e_step():
        e2.set_hoppings(t_host)
        e2.set_orbitals(wf)
        e2.set_scattering(vscat)
        e2.run(E, out32=host_out)

    e2e_step()
    barrier()
    # every step is timed on its own and the median is kept: the device-to-host leg shares
    # the host's memory system with other jobs on the machine, which adds rare stalls of tens
    # of milliseconds to single steps
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    barrier()
    e2e_s = statistics.median(e2e_times)
    e2.close()
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    e2e_value = whole_job_rate(world, work_per_rank, e2e_s)

    # roofline of the dominant kernel (the LDOS contraction)
    peaks, peak_src = measured_peaks()
    F = ldos_flops_per_pixel_energy(m.bands, c.extra.get("maxband", m.bands), (2 * c.window + 1) ** 2, c.spin,
                                    "josephson" in c.extra)
    ldos_ms = stage_acc["ldos"] / args.steps
    achieved = F * work_per_rank / (ldos_ms / 1e3) / 1e12
    if prec == cqpi.PREC_FP64:
        peak = cqpi.measure_fma_peak("fp64")
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "measured DFMA loop (cqpi_measure_fma_peak), not in MEASURED_PEAKS.json"}
    elif eng.contraction_kind() == "tcgen05":
        peak = peaks.get("bf16_tflops", 1900.0)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": f"bf16 dense burst, {peak_src} (fp16 kind::f16 runs at the same rate)"}
    else:
        peak = cqpi.measure_fma_peak("fp32")
        roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": "measured FFMA loop (cqpi_measure_fma_peak), not in MEASURED_PEAKS.json"}
    roof["kernel"] = "ldos contraction"
    roof["flop_per_pixel_energy"] = F
    roof["traffic"] = None
    if (args.config == "C2" and not args.fov and not args.energies and prec != cqpi.PREC_FP64
            and eng.contraction_kind() == "tcgen05"):
        # dram__bytes_read.sum + dram__bytes_write.sum of one contraction launch of 32 energies
        # on a 192^2-site field of view (one ncu capture: profiles/launches_c2_mixed.md), scaled
        # to this 256^2-site launch by the pixels it writes and the window sites it reads
        roof["traffic"] = (178.1e6 + 414.6e6) * (256.0 / 192.0) ** 2
        roof["traffic_note"] = ("bytes per contraction launch of 32 energies (ncu, 192^2-site launch x 1.78); "
                                "algorithmic: the u windows from 32 G0(R) boxes and the s windows from 32 T G0(R) "
                                "boxes (2 x 157 MB) + 32 maps (839 MB)")
    roof["stage_ms_per_step"] = {k: v / args.steps for k, v in stage_acc.items()}

    # accuracy and speed of the all-FP64 path on the same workload (the metric's comparison)
    fp64_info = None
    if prec != cqpi.PREC_FP64 and not args.no_fp64_check:
        fp64_info = fp64_check(cqpi, c, m, wf, vscat, E, lambda sub: out[sub].double().cpu().numpy(), 5)
        fp64_info["mixed_over_fp64"] = value / world / fp64_info["fp64_path_value"]

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == cqpi.PREC_FP64 else f"mixed: f64 eigen/T/term1, f32 G0+FFT, {eng.contraction_kind()} contraction",
            "data": "synthetic (seeded model and orbitals)",
            "config": {"workload": workload_desc(args.config, c, m, nE), "precision": args.precision,
                       "parallelism": f"replicas x{world}",
                       "l2": (f"inputs/outputs larger than L2 ({nE * wn * wn * 4 / 1e9:.1f} GB of maps, "
                              f"{c.kpoints ** 2 * (16 * m.bands ** 2 + 8 * m.bands) / 1e6:.0f} MB eigen cache per step)")},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": e2e_steps, "statistic": "median of per-step wall times",
                    "ms_per_step": [round(1e3 * t, 3) for t in e2e_times]},
            "gpu_launches": int(launches), "roofline": roof}
    if tune is not None:
        line["config"]["autotune"] = tune
    if fp64_info is not None:
        line["accuracy"] = fp64_info
    if clk is not None:
        line["clocks"] = clk
    if rank == 0 and args.adjoint_steps > 0 and prec != cqpi.PREC_FP64:
        line["adjoint"] = adjoint_rate(args.adjoint_steps)
    # the other workloads of the series, each measured the same way (device outputs, CUDA
    # events on the engine's stream) with its error against the FP64 path
    if rank == 0 and world == 1 and not args.no_extras and args.config == "C2" and not args.fov and not args.energies:
        extras = {}
        for nm, n_check in (("C3", 2), ("CJ", 3)):
            extras[nm] = workload_measure(nm, 3, 2, n_check)
        f4, _ = c4_measure(3, 2, not args.no_autotune)
        extras["C4"] = {"workload": f4["config"]["workload"], "ms_per_job": f4["ms_per_step"], "value": f4["value"],
                        "unit": UNIT, "latency_ms_per_map": f4["latency_ms_per_map"], "maps": f4["config"]["maps"],
                        "pixel_energies": f4["config"]["pixel_energies"]}
        line["extras"] = extras
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, desc = cpu_sample(args.config, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def c4_workload(seed=4):
    """C4: the C2 model with 256 energies in [-0.1, 0.1] eV x 12 impurities (6 scalar
    V = v*1, v ~ U(-1, 1) eV; 6 random Hermitian 3x3 V, entries ~ N(0, 0.2) eV) and a field of
    view per map drawn from {64, 128, 256, 384} sites per side (seeded)."""
    rng = np.random.default_rng(seed)
    Vs = []
    for k in range(12):
        if k < 6:
            Vs.append(rng.uniform(-1.0, 1.0) * np.eye(3, dtype=complex))
        else:
            A = rng.normal(0.0, 0.2, size=(3, 3)) + 1j * rng.normal(0.0, 0.2, size=(3, 3))
            Vs.append(0.5 * (A + A.conj().T))
    E = np.linspace(-0.1, 0.1, 256)
    fov = rng.choice([64, 128, 256, 384], size=len(E) * 12).astype(np.int32)
    return E, np.stack(Vs), fov


def c4_measure(steps, warmup, autotune=True):
    """Batched workload: all energies, impurities and uneven fields of view of one job as
    one captured CUDA graph of cqpi_run_fov calls (chunks of 32 energies into a reused
    device output ring); per-map latency from single-energy calls (12 maps each).  Returns
    (line fields, clocks)."""
    import torch
    import cqpi
    from cqpi import workloads as W
    c, m, wf = W.config("C2")
    E, Vs, fov = c4_workload()
    nimp, os_ = len(Vs), c.oversamp
    eng = cqpi.Engine(m, 384, c.kpoints, os_, c.window, c.eta, precision=cqpi.PREC_MIXED)
    eng.set_orbitals(wf)
    eng.set_impurities(Vs)
    chunk = 32
    sizes = (fov.astype(np.int64) * os_) ** 2
    per_chunk = [int(sizes[e0 * nimp:(e0 + chunk) * nimp].sum()) for e0 in range(0, len(E), chunk)]
    buf = torch.empty((max(per_chunk),), dtype=torch.float32, device="cuda")
    pix = float(sizes.sum())

    def job():
        for e0 in range(0, len(E), chunk):
            eng.run_fov(E[e0:e0 + chunk], fov[e0 * nimp:(e0 + chunk) * nimp], buf.data_ptr())

    eng.solve_bands()
    tune = None
    if autotune:
        ms_t, n_t = eng.autotune(E[:32])
        tune = {"shapes_timed": n_t, "batch_ms": ms_t}
    job()                                   # allocates every buffer
    eng.synchronize()
    eng.graph_begin()
    job()
    eng.graph_end()
    stream = torch.cuda.ExternalStream(eng.stream)
    for _ in range(warmup):
        eng.solve_bands()
        eng.graph_launch()
    eng.synchronize()
    launches0 = eng.kernel_launches()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        eng.solve_bands()
        eng.graph_launch()
    ev1.record(stream)
    ev1.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / steps
    launches = eng.kernel_launches() - launches0
    # per-map latency: one energy (its 12 maps) per call, CUDA events around each call
    lat = []
    one = torch.empty((int(max(sizes[e * nimp:(e + 1) * nimp].sum() for e in range(len(E)))),), dtype=torch.float32,
                      device="cuda")
    for e in range(len(E)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.run_fov(E[e:e + 1], fov[e * nimp:(e + 1) * nimp], one.data_ptr())
        b.record(stream)
        lat.append((a, b))
    eng.synchronize()
    per_call = np.array([a.elapsed_time(b) for a, b in lat])
    per_map = np.repeat(per_call, nimp)
    kind = eng.contraction_kind()
    eng.close()
    fields = {"value": pix / (ms / 1e3), "ms_per_step": ms, "gpu_launches": int(launches),
              "dtype": f"mixed: f64 eigen/T/term1, f32 G0+FFT, {kind} contraction",
              "config": {"workload": "C4: C2 t2g model, k-grid 1024^2, 256 energies x 12 impurities (6 scalar, 6 "
                                     "Hermitian 3x3), field of view per map from {64,128,256,384}^2 sites, 10x10 "
                                     "px/cell, one CUDA graph of cqpi_run_fov chunks (32 energies)",
                         "maps": int(len(fov)), "pixel_energies": pix, "mean_pixels_per_map": pix / len(fov),
                         "autotune": tune, "l2": "outputs far larger than L2"},
              "latency_ms_per_map": {"p50": float(np.percentile(per_map, 50)), "p99": float(np.percentile(per_map, 99)),
                                     "definition": "duration of the single-energy call (12 maps) that produced the map"}}
    return fields, clk


def run_c4(args):
    import torch
    import cqpi_build
    cqpi_build.build()
    torch.cuda.set_device(0)
    f, clk = c4_measure(args.steps, args.warmup, not args.no_autotune)
    line = {"metric": METRIC, "value": f["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": f["dtype"], "data": "synthetic (seeded model, impurities and fields of view)",
            "config": f["config"], "gpu_launches": f["gpu_launches"], "latency_ms_per_map": f["latency_ms_per_map"]}
    if clk is not None:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)
    return 0


def fp64_check(cqpi, c, m, wf, vscat, E, maps, n_check):
    """Per-map relative errors of the mixed maps (host [nE][wn][wn]) against the engine's
    FP64 path on n_check energies spread over the list; maps that vanish to rounding in FP64
    (the Josephson map at E = 0) are reported against the largest checked map."""
    sub = np.linspace(0, len(E) - 1, n_check).astype(int)
    with make_engine(cqpi, c, m, wf, vscat, cqpi.PREC_FP64) as e64:
        ref = e64.run(E[sub], f32=False, f64=True)
        t0 = time.perf_counter()
        e64.solve_bands()
        e64.run(E[sub], f32=False, f64=False)
        t64 = time.perf_counter() - t0
    got = maps(sub)
    gmax = max(float(np.abs(ref[i, 0]).max()) for i in range(len(sub)))
    live = [i for i in range(len(sub)) if np.abs(ref[i, 0]).max() > 1e-9 * gmax]
    zero = [i for i in range(len(sub)) if i not in live]
    errs = [float(np.abs(got[i, 0] - ref[i, 0]).max() / np.abs(ref[i, 0]).max()) for i in live]
    rms = [float(np.sqrt(np.mean((got[i, 0] - ref[i, 0]) ** 2) / np.mean(ref[i, 0] ** 2))) for i in live]
    info = {"max_rel_err_vs_fp64": max(errs), "rms_rel_err_vs_fp64": max(rms),
            "rel_err_definitions": "max|rho-rho64|/max|rho64| and rms(rho-rho64)/rms(rho64) per map, worst map",
            "per_map_max_rel_err": errs, "energies_checked": [float(x) for x in E[sub]], "tolerance": 1e-6,
            "fp64_path_value": len(sub) * c.pixels_per_energy / t64}
    if zero:
        info["vanishing_maps"] = {"energies": [float(E[sub][i]) for i in zero],
                                  "max_abs_err_over_largest_map": max(float(np.abs(got[i, 0] - ref[i, 0]).max()) / gmax
                                                                      for i in zero)}
    return info


def workload_measure(name, steps, warmup, n_check):
    """ms per job (eigen-solve + every energy, device outputs), pixel*E/s and the error
    against the FP64 path of one workload of the C-series, for the extra objects of the
    default line."""
    import torch
    import cqpi
    from cqpi import workloads as W
    c, m, wf = W.config(name)
    E = c.energy_list()
    vscat = np.array(c.scattering, complex)
    if len(vscat) < m.bands:
        vscat = np.concatenate([vscat, np.zeros(m.bands - len(vscat), complex)])
    eng = make_engine(cqpi, c, m, wf, vscat, cqpi.PREC_MIXED)
    wn = c.lattice * c.oversamp
    out = torch.empty((len(E), 1, wn, wn), dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(eng.stream)

    def step():
        eng.solve_bands()
        eng.run_device(E, ptr32=out.data_ptr())

    for _ in range(warmup):
        step()
    eng.synchronize()
    eng.stage_times()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    stages = {k: v / steps for k, v in eng.stage_times().items()}
    kind = eng.contraction_kind()
    eng.close()
    res = {"workload": workload_desc(name, c, m, len(E)), "ms_per_job": ms,
           "value": c.pixels_per_energy * len(E) / (ms / 1e3), "unit": UNIT, "contraction": kind,
           "stage_ms_per_job": stages, "steps": steps, "warmup": warmup}
    res["accuracy"] = fp64_check(cqpi, c, m, wf, vscat, E, lambda sub: out[sub].double().cpu().numpy(), n_check)
    del out
    return res


def adjoint_rate(steps, analysis=False):
    """Differentiation workload (C5): QPI loss sum_w || |FFT2 rho_w| - target_w ||^2 on the
    C2 model family with a 128^2-site FOV, 10x10 px/cell, 41 energies in [-0.1, 0.1] eV,
    eta = 2 meV, k-grid 1024^2; target from amplitudes perturbed by 5% (seed 7); gradient
    w.r.t. the 20 independent hopping amplitudes and V through cqpi_adjoint; Adam steps.
    One iteration = forward (eigen-solve + 41 maps) + loss + adjoint + optimiser step."""
    from cqpi import fit as F
    fm = F.QPIFit()
    p_true, target = F.target_maps(fm)
    F.run_adam(fm, target, steps=1)                       # warm-up (plans, workspaces)
    fm.timing = {"forward": [], "adjoint": []}
    t0 = time.perf_counter()
    p, V, losses = F.run_adam(fm, target, steps=steps)
    dt = (time.perf_counter() - t0) / steps
    err0 = float(np.linalg.norm(fm.p0 - p_true) / np.linalg.norm(p_true))
    err1 = float(np.linalg.norm(p - p_true) / np.linalg.norm(p_true))
    out = {"metric": "adjoint grad s/it", "value": dt, "unit": "s/it", "higher_is_better": False,
           "steps": steps, "forward_s": float(statistics.median(fm.timing["forward"])),
           "adjoint_s": float(statistics.median(fm.timing["adjoint"])),
           "loss_first": losses[0], "loss_last": losses[-1], "param_rel_err_start": err0, "param_rel_err_end": err1,
           "V_rel_err_end": float(np.linalg.norm(V - fm.V0.real) / np.linalg.norm(fm.V0.real)),
           "config": "C5: t2g C2 family, 20 hopping amplitudes + 3x3 V (both optimised), FOV 128^2, 10x10 px/cell, "
                     "41 energies, k-grid 1024^2, eta=0.002, mixed forward, QPI loss FFT in FP32 (sum in FP64), "
                     "adjoint checked vs FD in the tests"}
    if analysis:
        # Gauss-Newton matrix of the QPI magnitudes at the true parameters: which parameter
        # directions the 41 maps constrain, and how much of the start's error the fit removed
        # along each of them
        JtJ, x_true = F.gauss_newton(fm, p_true, fm.V0.real)
        x_start = np.concatenate([fm.p0, fm.V0.real.reshape(-1)])
        x_fit = np.concatenate([p, np.asarray(V).reshape(-1)])
        out["gauss_newton"] = F.identifiability(JtJ, x_true, x_start, x_fit)
        # the same least-squares problem solved by Gauss-Newton steps (adjoint gradient, J^T J
        # from differences of the maps) from the same start, for comparison with Adam
        t0 = time.perf_counter()
        x_gn, gn_losses = F.gauss_newton_fit(fm, target, x_start, iters=6)
        out["gauss_newton_fit"] = {"iterations": len(gn_losses) - 1, "seconds": time.perf_counter() - t0,
                                   "losses": gn_losses,
                                   "param_rel_err_end": float(np.linalg.norm(x_gn[:len(fm.p0)] - p_true) /
                                                              np.linalg.norm(p_true)),
                                   "per_direction": F.identifiability(JtJ, x_true, x_start, x_gn)}
    fm.close()
    return out


def run_c5(args):
    """The differentiation workload alone: Adam steps of the fit (args.adjoint_steps) and the
    Gauss-Newton analysis of what the maps constrain."""
    import torch
    import cqpi_build
    cqpi_build.build()
    torch.cuda.set_device(0)
    out = adjoint_rate(max(1, args.adjoint_steps), analysis=True)
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="C2")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the C3 / CJ / C4 objects of the default line")
    ap.add_argument("--no-autotune", action="store_true", help="keep the rule-based contraction tile shape")
    ap.add_argument("--fov", type=int, default=0, help="override the field of view (sites per side) for small captures")
    ap.add_argument("--energies", type=int, default=0, help="override the number of energies for small captures")
    ap.add_argument("--adjoint-steps", type=int, default=3,
                    help="Adam iterations of the C5 differentiation workload timed for 'adjoint grad s/it' (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "C4":
        return run_c4(args)
    if args.config == "C5":
        return run_c5(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
