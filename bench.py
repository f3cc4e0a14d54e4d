#!/usr/bin/env python3
"""Benchmark of the GB300 leapfrog: link-updates/s and the fraction of the HBM
roofline for the precision form of the Yang-Mills leapfrog (SU(3), 128^3
periodic lattice, dt = 0.05, FP32 links and E with re-unitarisation every 10
steps, FP64 compensated reductions), with the plain FP64 GPU path on the same
lattice beside it.

One step = storeFields + updateGrid over the whole lattice (3 * 128^3 link
updates).  ``value`` is timed with CUDA events on the handle's own stream over
K steps with the fields resident in HBM (inputs are larger than L2: the links
alone are 453 MB).  ``e2e`` is the same metric through the public C ABI with
host buffers: upload of the initial U and E from pinned memory, the K steps
with the BulkQuantities row of every step read back to the host
(opx_step_measured; ``e2e.step_then_reduce`` makes the same run as one
opx_step + opx_reduce call pair per step), and the download of the final U
and E, all inside the timed region;
``e2e.per_call_copy`` is FieldSolver.step as a per-call drop-in whose host grid
stays authoritative (U and E copied in, E and Unext copied out on every call).

Beside the headline line: the batching form (256 SU(2) events in one
persistent launch) and the CPIC collision form (SU(2) FP64, 256 x 64^2, two MV
nuclei, 300 steps with per-step diagnostics, oracle check of the first steps).

``--impl reference`` times the CPU implementation of the path: the reference
(Java) cannot be built or run on this machine, so its FP64 restatement (the
oracle, C + OpenMP over all host threads) stands in; every step updates a
bounded slab of the same lattice.

Multi-GPU: the path is one lattice per GPU; N ranks run N independent
replicas (weak scaling), with a barrier and max-over-ranks timing.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: ncolors, dims, precision, reunit_every, dt, sigma (A and E), bytes per link update
    "su3_fp32_128": dict(nc=3, dims=(128, 128, 128), prec="f32", reunit=10, dt=0.05, sigma=0.2, bpl=208,
                         label="SU(3) pure Yang-Mills leapfrog, 128^3 periodic, dt=0.05, FP32 links/E, "
                               "reunitarisation every 10 steps, reductions accumulated in FP64"),
    "su3_fp32_96": dict(nc=3, dims=(96, 96, 96), prec="f32", reunit=10, dt=0.05, sigma=0.2, bpl=208,
                        label="SU(3) pure Yang-Mills leapfrog, 96^3 periodic (profiling size), FP32"),
    "su3_fp64_128": dict(nc=3, dims=(128, 128, 128), prec="f64", reunit=0, dt=0.05, sigma=0.2, bpl=416,
                         label="SU(3) pure Yang-Mills leapfrog, 128^3 periodic, dt=0.05, FP64"),
    "su2_fp64_32": dict(nc=2, dims=(32, 32, 32), prec="f64", reunit=0, dt=0.05, sigma=0.1, bpl=112,
                        label="SU(2) pure Yang-Mills leapfrog, 32^3 periodic, dt=0.05, FP64"),
    "su2_fp32_128": dict(nc=2, dims=(128, 128, 128), prec="f32", reunit=10, dt=0.05, sigma=0.1, bpl=56,
                         label="SU(2) pure Yang-Mills leapfrog, 128^3 periodic, dt=0.05, FP32"),
}
SEED = 20261203
METRIC = "link-updates/s"


class nvtx_range:
    """NVTX range around a bench phase (ncu --nvtx --nvtx-include <name>/ selects
    the kernels launched inside it); a no-op when NVTX is unavailable."""

    def __init__(self, name):
        self.name = name
        try:
            import torch.cuda.nvtx as nv
            self.nv = nv
        except Exception:
            self.nv = None

    def __enter__(self):
        if self.nv is not None:
            self.nv.range_push(self.name)
        return self

    def __exit__(self, *exc):
        if self.nv is not None:
            self.nv.range_pop()
        return False


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    """Barrier and max-reduction across ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self, backend):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64,
                         device="cuda" if self.td.get_backend() == "nccl" else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_for(workload, key="dram_bytes_per_launch"):
    """DRAM bytes per launch of the leapfrog kernel (or another figure, `key`)
    from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        v = d.get(workload)
        if isinstance(v, dict):
            return v.get(key)
        return v if key == "dram_bytes_per_launch" else None
    return None


def make_handle(w, prec_name, device):
    import openpixi_gb300 as opx
    prec = opx.OPX_F32 if prec_name == "f32" else opx.OPX_F64
    return opx.Handle(w["nc"], w["dims"], a=1.0, dt=w["dt"], g=1.0, precision=prec,
                      reunit_every=w["reunit"] if prec_name == "f32" else 0, device=device)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo; Arm hosts report
    the implementer and part numbers there)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        info = open("/proc/cpuinfo").read()
    except OSError:
        return "unknown"
    for line in info.splitlines():
        if line.lower().startswith("model name"):
            return line.split(":", 1)[1].strip()
    impl = [ln.split(":", 1)[1].strip() for ln in info.splitlines() if ln.startswith("CPU implementer")]
    part = [ln.split(":", 1)[1].strip() for ln in info.splitlines() if ln.startswith("CPU part")]
    return f"Arm implementer {impl[0]} part {part[0]}" if impl and part else "unknown"


def cpu_baseline(w, U_ref, E_ref, target_s=12.0):
    """The oracle (FP64 restatement of the reference update, C + OpenMP) on a bounded
    sample of the same lattice: whole-lattice steps, or a leading slab of sites when
    one step would exceed the time budget."""
    import oracle
    g = oracle.OracleGrid(w["nc"], w["dims"], a=1.0, dt=w["dt"], g=1.0)
    g.U[...] = U_ref
    g.E[...] = E_ref
    g.update_links()
    nth = cpu_threads()
    plane = w["dims"][1] * w["dims"][2]
    t = time.perf_counter()
    g.update_grid_range_omp(0, plane, nth)
    per_plane = max(time.perf_counter() - t, 1e-6)
    planes = int(max(1, min(w["dims"][0], target_s / per_plane)))
    sites = planes * plane
    t = time.perf_counter()
    g.update_grid_range_omp(0, sites, nth)
    el = time.perf_counter() - t
    return {"value": 3.0 * sites / el, "unit": METRIC, "cores": nth, "kind": "port",
            "cpu_model": cpu_model(), "build": "gcc -O3 -fopenmp -ffp-contract=off",
            "sample": f"one leapfrog update of {planes} of {w['dims'][0]} x0-planes ({sites} sites, "
                      f"{3 * sites} link updates) of the same lattice, FP64, {nth} OpenMP threads, {el:.2f} s"}


def run_reference(args, w, wname):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    g = oracle.OracleGrid(w["nc"], w["dims"], a=1.0, dt=w["dt"], g=1.0)
    g.random_fields(SEED, w["sigma"], w["sigma"])
    g.update_links()
    nth = cpu_threads()
    plane = w["dims"][1] * w["dims"][2]
    t = time.perf_counter()
    g.update_grid_range_omp(0, plane, nth)
    per_plane = max(time.perf_counter() - t, 1e-6)
    budget = 150.0 / max(1, args.steps + args.warmup)  # whole run within a few minutes
    planes = int(max(1, min(w["dims"][0], budget / per_plane)))
    sites = planes * plane
    for _ in range(args.warmup):
        g.update_grid_range_omp(0, sites, nth)
    t = time.perf_counter()
    for _ in range(args.steps):
        g.store_fields()
        g.update_grid_range_omp(0, sites, nth)
    el = time.perf_counter() - t
    value = 3.0 * sites * args.steps / el
    sample = (f"each step: one leapfrog update (FastTYMSolver.CombinedUpdate restated in C, FP64) of "
              f"{planes} of {w['dims'][0]} x0-planes ({sites} sites) of the same lattice; "
              f"{nth} OpenMP threads; the Java reference cannot run here (no JDK)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_for(w, wname),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": nth, "kind": "port",
                             "cpu_model": cpu_model(), "build": "gcc -O3 -fopenmp -ffp-contract=off",
                             "sample": sample},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def config_for(w, wname):
    return {"workload": wname, "description": w["label"], "lattice": list(w["dims"]), "ncolors": w["nc"],
            "dt": w["dt"], "a": 1.0, "g": 1.0, "reunit_every": w["reunit"], "precision": w["prec"],
            "initial_fields": f"seeded Gaussian A and E (sigma={w['sigma']}), E projected onto Gauss's law "
                              f"in FP64 on the device",
            "l2": "inputs larger than L2 (links alone exceed 129 MB)" if np.prod(w["dims"]) >= 64 ** 3
            else "lattice fits in L2", "parallelism": "replicas (one lattice per GPU)"}


def bench_batch(device, nc=2, nsteps=200, nev=256, seed=SEED):
    """Batching form: 256 events of cubic sizes drawn uniformly from
    {16,24,32,40,48}^3 (SU(2), the configured workload; SU(3) with the same
    sizes, seeds and widths beside it), FP32 with reunitarisation every 10
    steps, 200 steps in one persistent launch replayed from a CUDA graph
    (autotuned cluster / block size), against the plain FP64 single-lattice path
    looping over the same events (GPU time of each event's 200 steps, summed),
    which also gives the batch's energy error after 200 steps (max over the
    events)."""
    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    rng = np.random.default_rng(seed)
    sizes = [int(x) for x in rng.choice([16, 24, 32, 40, 48], nev)]
    dims = [(L, L, L) for L in sizes]
    bpl = 56 if nc == 2 else 208
    b = opx.Batch(nc, dims, dt=0.05, precision=N.OPX_F32, reunit_every=10, device=device)
    b.init_random([seed + 1000 + q for q in range(nev)], 0.1, 0.1, tol=1e-24)
    b.initialize()
    init = [(b.download(q, N.FIELD_U), b.download(q, N.FIELD_E)) for q in range(nev)]
    cluster, block = b.autotune(steps=5)  # restores the fields
    b.run(nsteps)  # instantiates the graph
    obs_first = b.reduce()  # the events after their first nsteps steps
    b.run(nsteps)
    l0 = b.kernel_launches
    ms = b.time_run(nsteps)
    launches = b.kernel_launches - l0
    links = 3 * sum(L ** 3 for L in sizes)
    obs = b.reduce()
    # plain FP64 path, one lattice at a time, from the same initial fields: its
    # time, and the FP32 batch's energy error after nsteps steps against it
    handles = {}
    ms64 = 0.0
    derr = 0.0
    for q, d in enumerate(dims):
        h = handles.get(d)
        if h is None:
            h = handles[d] = opx.Handle(nc, d, dt=0.05, precision=N.OPX_F64, device=device)
        h.upload(N.FIELD_U, init[q][0])
        h.upload(N.FIELD_E, init[q][1])
        h.initialize()
        ms64 += h.time_steps(nsteps)
        o = h.reduce()
        e64 = o.e2_total + o.b2_total
        derr = max(derr, abs(obs_first[q].e2_total + obs_first[q].b2_total - e64) / abs(e64))
    for h in handles.values():
        h.close()
    peak, _ = hbm_peak()
    lu = links * nsteps / (ms / 1000.0)
    b.close()
    return {"group": f"SU({nc})", "events": nev, "steps": nsteps,
            "lattice_sizes": "L^3, L uniform in {16,24,32,40,48}",
            "link_updates_per_step": links, "ms": ms, "events_per_s": nev / (ms / 1000.0),
            "link_updates_per_s": lu, "roofline_frac": bpl * lu / 1e9 / peak, "bytes_per_link": bpl,
            "fp64_loop_ms": ms64, "fp64_loop_events_per_s": nev / (ms64 / 1000.0),
            "speedup_vs_fp64_loop": ms64 / ms, "cluster": cluster, "block": block, "graph": True,
            "gpu_launches": launches, "max_gauss": max(o.gauss for o in obs),
            "energy_rel_err_vs_fp64": derr}


CGC_DIMS = (256, 64, 64)


def cgc_nuclei():
    """Two MV nuclei of the CPIC collision workload (YamlMVModel defaults for the
    UV cutoff 4.44, coherence length 0 and IR coefficient 0)."""
    base = {"direction": 0, "width": 4.0, "mu": 0.5, "use_seed": 1, "uvt": 4.44, "coherence": 0.0, "ir": 0.0}
    return [dict(base, orientation=1, location=64.0, seed=1), dict(base, orientation=-1, location=192.0, seed=2)]


def bench_cgc(device, nsteps=300, oracle_steps=2):
    """CPIC collision form: SU(2) FP64, lattice 256 x 64^2 (beam along dimension 0),
    a = 1, dt = 0.5, g = 1, two MV nuclei (mu = 0.5, width 4, seeds 1 and 2) with
    round(a/dt) = 2 NGP particles per cell; 300 steps of Simulation.step with the
    ProjectedEnergyDensity (4 x 256) and BulkQuantities diagnostics every step.
    The oracle repeats the initial condition and the first steps at full size on
    the host for a parity check."""
    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    h = opx.Handle(2, CGC_DIMS, a=1.0, dt=0.5, g=1.0, precision=N.OPX_F64, device=device)
    h.synchronize()
    t = time.perf_counter()
    h.cgc_mv(cgc_nuclei())
    h.synchronize()
    ic_ms = 1000.0 * (time.perf_counter() - t)
    np_ = h.np
    h.initialize()
    U0, E0 = h.download(N.FIELD_U), h.download(N.FIELD_E)
    P0 = h.particles_download()
    h.set_profiling(True)
    obs0 = h.reduce()
    e0 = obs0.e2_total + obs0.b2_total
    gmax = obs0.gauss
    proj = []
    h.synchronize()
    t = time.perf_counter()
    with nvtx_range("cgc_steps"):
        for _ in range(nsteps):
            h.step(1)
            o = h.reduce()
            proj.append(h.projected_energy(0))
            gmax = max(gmax, o.gauss)
    h.synchronize()
    wall_ms = 1000.0 * (time.perf_counter() - t)
    ms, counts = h.phase_times()
    h.set_profiling(False)
    obs = h.reduce()
    e1 = obs.e2_total + obs.b2_total
    links = 3 * int(np.prod(CGC_DIMS))
    step_ms = (ms[N.PHASE_EOM] + ms[N.PHASE_CPIC]) / nsteps
    peak, _ = hbm_peak()
    lu = links / (step_ms / 1000.0)
    # algorithmic bytes of the particle phases per step (SU(2) FP64): per particle
    # the state read (pos, vel, Q0, Q1: 96 B, direction 1 B) and written (pos0,
    # pos1, Q0, Q1: 96 B) and, on a cell change, one Unext link (32 B; with
    # |v| = 1 and dt = a/2 every particle changes cell every other step); per
    # site the rho (24 B) and J (72 B) written
    cpic_bytes = np_ * (193 + 0.5 * 32) + int(np.prod(CGC_DIMS)) * 96
    cpic_ms = ms[N.PHASE_CPIC] / nsteps
    out = {"workload": "SU(2) CPIC collision, 256x64^2, dt=0.5, 2 MV nuclei, FP64", "particles": np_,
           "steps": nsteps, "ic_ms": ic_ms, "wall_ms_with_diagnostics": wall_ms,
           "ms_per_step_device": step_ms, "eom_ms_per_step": ms[N.PHASE_EOM] / nsteps,
           "cpic_ms_per_step": ms[N.PHASE_CPIC] / nsteps, "diagnostics_ms_per_step": ms[N.PHASE_DIA] / nsteps,
           "link_updates_per_s": lu, "particle_updates_per_s": np_ / (cpic_ms / 1000.0),
           "cpic_bytes_per_step": cpic_bytes, "roofline_frac_cpic": cpic_bytes / (cpic_ms / 1000.0) / 1e9 / peak,
           "roofline_frac_eom": 136.0 * links / (ms[N.PHASE_EOM] / nsteps / 1000.0) / 1e9 / peak,
           "bytes_per_link": 136, "max_gauss_mean_sq": gmax, "energy_start": e0, "energy_end": e1,
           "projected_energy_rows": [4, CGC_DIMS[0]], "final_T_el_sum": float(proj[-1][0].sum())}
    # the same collision with super particles (temporal optimized cgc ngp)
    try:
        hs = opx.Handle(2, CGC_DIMS, a=1.0, dt=0.5, g=1.0, precision=N.OPX_F64, device=device)
        hs.synchronize()
        t = time.perf_counter()
        hs.cgc_mv_super(cgc_nuclei())
        hs.synchronize()
        sic = 1000.0 * (time.perf_counter() - t)
        hs.initialize()
        hs.set_profiling(True)
        hs.step(nsteps)
        sms, _ = hs.phase_times()
        hs.set_profiling(False)
        so = hs.reduce()
        charges = sum(hs.super_download(k)["n"] for k in range(hs.super_groups)) * 2
        out["super_particles"] = {
            "groups": hs.super_groups, "charges": charges, "ic_ms": sic,
            "eom_ms_per_step": sms[N.PHASE_EOM] / nsteps, "cpic_ms_per_step": sms[N.PHASE_CPIC] / nsteps,
            "energy_end": so.e2_total + so.b2_total, "gauss_end": so.gauss,
            "energy_end_rel_to_ngp": abs(so.e2_total + so.b2_total - e1) / e1}
        hs.close()
    except Exception as e:
        out["super_particles"] = f"skipped: {e}"
    # oracle at full size: the initial condition and the first steps
    if oracle_steps <= 0:
        h.close()
        return out
    try:
        import oracle
        from oracle import cgc as ocgc
        from oracle import OracleSimulation
        g = oracle.OracleGrid(2, CGC_DIMS, dt=0.5)
        nus = [ocgc.MVNucleus(orientation=n["orientation"], location=n["location"], width=n["width"], mu=n["mu"],
                              seed=n["seed"]) for n in cgc_nuclei()]
        t = time.perf_counter()
        P, _ = ocgc.cgc_mv(g, nus)
        ic_cpu = time.perf_counter() - t
        sim = OracleSimulation(g, P)
        sim.initialize()
        h2 = opx.Handle(2, CGC_DIMS, a=1.0, dt=0.5, g=1.0, precision=N.OPX_F64, device=device)
        h2.upload(N.FIELD_U, U0)
        h2.upload(N.FIELD_E, E0)
        h2.particles_upload(P0["pos0"], P0["pos1"], P0["vel"], P0["Q0"], P0["Q1"], P0["dir"])
        h2.initialize()
        ic_err = float(np.max(np.abs(U0 - g.U)))
        t = time.perf_counter()
        for _ in range(oracle_steps):
            sim.step()
        step_cpu = (time.perf_counter() - t) / oracle_steps
        h2.step(oracle_steps)
        du = float(np.max(np.abs(h2.download(N.FIELD_U) - g.U)))
        de = float(np.max(np.abs(h2.download(N.FIELD_E) - g.E)) / max(np.abs(g.E).max(), 1e-300))
        h2.close()
        out.update({"oracle_particles": int(P.n), "oracle_ic_s": ic_cpu, "oracle_ms_per_step_1thread": 1000 * step_cpu,
                    "oracle_ic_max_abs_dU": ic_err, "oracle_steps": oracle_steps,
                    "oracle_max_abs_dU_after": du, "oracle_max_rel_dE_after": de})
    except Exception as e:  # the measurement stands without the check
        out["oracle_check"] = f"skipped: {e}"
    h.close()
    return out


def bench_differentiation(device, ndir=64):
    """Differentiation form: SU(2), 64^3, dt = 0.05, 200 steps, FP32 forward with
    FP64 checkpoints every 14 steps, objective the mean energy density over the
    central 16^3; the gradient w.r.t. the initial E checked on 64 seeded random
    directions against central differences (h = 1e-4 along the unit-norm
    direction) of FP64 forward runs and against the FP64 tangent-linear run."""
    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    dims, nsteps, ckpt = (64, 64, 64), 200, 14
    lo, hi = (24, 24, 24), (39, 39, 39)
    h64 = opx.Handle(2, dims, dt=0.05, precision=N.OPX_F64, device=device)
    h64.init_random(SEED + 5, 0.1, 0.1)
    h64.gauss_project(1e-24)
    h32 = opx.Handle(2, dims, dt=0.05, precision=N.OPX_F32, reunit_every=10, device=device)
    h32.upload(N.FIELD_U, h64.download(N.FIELD_U))
    h32.upload(N.FIELD_E, h64.download(N.FIELD_E))
    h32.synchronize()
    t = time.perf_counter()
    J32, g32 = h32.energy_gradient(nsteps, ckpt, lo, hi)
    t32 = time.perf_counter() - t
    t = time.perf_counter()
    J64, g64 = h64.energy_gradient(nsteps, ckpt, lo, hi)
    t64 = time.perf_counter() - t
    rng = np.random.default_rng(64)
    worst = {"fd": 0.0, "fd_rms": 0.0, "rich_rms": 0.0, "tl": 0.0, "f32_vs_tl": 0.0}
    t = time.perf_counter()
    for _ in range(ndir):
        d = rng.normal(size=g64.shape)  # unit RMS per component
        adj = float((g64 * d).sum())
        nrm = float(np.sqrt((d * d).sum()))

        def cfd(eps, dd):
            return (h64.energy_objective(nsteps, lo, hi, dd, eps) - h64.energy_objective(nsteps, lo, hi, dd, -eps)) / (2 * eps)
        # the unit-norm direction d/|d| with h = 1e-4
        fd = cfd(1e-4, d / nrm) * nrm
        # the unit-RMS direction with h = 1e-4 moves every E component by ~1e-4
        # (1e-3 of its width): the O(h^2) truncation of the central difference
        # shows, and the Richardson combination removes it
        fd_rms = cfd(1e-4, d)
        rich_rms = (4.0 * cfd(5e-5, d) - fd_rms) / 3.0
        _, dJ = h64.energy_tangent(nsteps, d, lo, hi)
        worst["fd"] = max(worst["fd"], abs(fd - adj) / abs(adj))
        worst["fd_rms"] = max(worst["fd_rms"], abs(fd_rms - adj) / abs(adj))
        worst["rich_rms"] = max(worst["rich_rms"], abs(rich_rms - adj) / abs(adj))
        worst["tl"] = max(worst["tl"], abs(adj - dJ) / abs(dJ))
        worst["f32_vs_tl"] = max(worst["f32_vs_tl"], abs(float((g32 * d).sum()) - dJ) / abs(dJ))
    tcheck = time.perf_counter() - t
    # the other objective / input pairs on the same workload, checked on 8
    # unit-norm directions each (central differences h = 1e-4, tangent-linear)
    forms = {}
    for name, kind, wrt in (("anisotropy_wrt_E", N.OBJ_ANISOTROPY, N.WRT_E),
                            ("energy_wrt_rho", N.OBJ_ENERGY, N.WRT_RHO),
                            ("anisotropy_wrt_rho", N.OBJ_ANISOTROPY, N.WRT_RHO)):
        t = time.perf_counter()
        Jf, gf = h64.objective_gradient(nsteps, ckpt, kind, 0, lo, hi, wrt)
        tg = time.perf_counter() - t
        wf = {"fd": 0.0, "tl": 0.0}
        rng_f = np.random.default_rng(100 + kind + 2 * wrt)
        for _ in range(8):
            d = rng_f.normal(size=gf.shape)
            d /= np.linalg.norm(d)
            adj = float((gf * d).sum())
            kw = {"dE": d} if wrt == N.WRT_E else {"drho": d}
            fd = (h64.objective_value(nsteps, kind, 0, lo, hi, h=1e-4, **kw) -
                  h64.objective_value(nsteps, kind, 0, lo, hi, h=-1e-4, **kw)) / 2e-4
            _, dJ = h64.objective_tangent(nsteps, kind, 0, lo, hi, **kw)
            wf["fd"] = max(wf["fd"], abs(fd - adj) / abs(adj))
            wf["tl"] = max(wf["tl"], abs(adj - dJ) / abs(dJ))
        forms[name] = {"J": Jf, "gradient_s_fp64_forward": tg, "directions": 8,
                       "worst_rel_vs_central_fd": wf["fd"], "worst_rel_vs_tangent_linear": wf["tl"]}
    h64.close()
    h32.close()
    return {"workload": "SU(2) 64^3, 200 steps, dt=0.05, ckpt 14, central 16^3 energy density",
            "other_forms": forms,
            "other_forms_note": "anisotropy = sum P_L / sum P_T of the projected components over the same box, "
                                "longitudinal direction 0; rho enters through the Gauss projection of the "
                                "initial E (dJ/drho = K^+ div dJ/dE_0)",
            "J": J64, "gradient_s_fp32_forward": t32, "gradient_s_fp64_forward": t64,
            "directions": ndir, "worst_rel_vs_central_fd": worst["fd"],
            "worst_rel_vs_central_fd_unit_rms_direction": worst["fd_rms"],
            "worst_rel_vs_richardson_fd_unit_rms_direction": worst["rich_rms"],
            "worst_rel_vs_tangent_linear": worst["tl"],
            "worst_rel_fp32_forward_vs_tangent_linear": worst["f32_vs_tl"],
            "fp32_forward_objective_rel_diff": abs(J32 - J64) / abs(J64), "check_s": tcheck,
            "bars": {"fd": 1e-5, "tl": 1e-9},
            "fp32_note": "the FP32-forward gradient is the exact adjoint of the FP32 trajectory's checkpoints; "
                         "it differs from the FP64 gradient by the FP32 rounding that 200 steps of the "
                         "nonlinear dynamics amplify (the objective itself differs by "
                         "fp32_forward_objective_rel_diff), so no parity bar applies to it",
            "fd_note": "central differences with h = 1e-4 along the unit-norm direction; along the "
                       "unit-RMS direction the same h leaves the O(h^2) truncation visible"}


def bench_configs(device):
    """Parity legs at full size: the plain SU(2) FP64 workload (32^3, 100
    steps) against the oracle per link; the SU(3) FP32 form against the FP64 GPU
    run on 128^3 x 500 steps (energy and per link) and against the oracle on a
    32^3 lattice of the same generator."""
    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    import oracle
    out = {}
    # SU(2) FP64 32^3 x 100 steps against the oracle
    g = oracle.OracleGrid(2, (32, 32, 32), dt=0.05)
    g.random_fields(SEED + 1, 0.1, 0.1)
    g.gauss_project(1e-26)
    h = opx.Handle(2, g.dims, dt=0.05, precision=N.OPX_F64, device=device)
    h.upload(N.FIELD_U, g.U)
    h.upload(N.FIELD_E, g.E)
    h.initialize()
    sim = oracle.OracleSimulation(g)
    sim.initialize()
    t = time.perf_counter()
    for _ in range(100):
        sim.step()
    t_orc = time.perf_counter() - t
    ms = h.time_steps(100)
    U, E = h.download(N.FIELD_U), h.download(N.FIELD_E)
    du = np.linalg.norm((U - g.U).reshape(-1, 4), axis=1).max()
    ev = E.reshape(-1, 3)
    eo = g.E.reshape(-1, 3)
    de = (np.linalg.norm(ev - eo, axis=1) / np.maximum(np.linalg.norm(eo, axis=1), np.sqrt((eo ** 2).sum(1).mean()))).max()
    bo, bd = g.bulk(), h.reduce()
    out["su2_fp64_32_parity"] = {"steps": 100, "gpu_ms_per_step": ms / 100, "oracle_s_1thread": t_orc,
                                  "max_rel_link_err": float(du), "max_rel_E_err": float(de),
                                  "energy_rel_err": abs(bd.e2_total + bd.b2_total - bo[11] - bo[12]) / (bo[11] + bo[12]),
                                  "gauss": bd.gauss, "bar": 1e-10}
    h.close()
    # SU(3) FP32 against FP64 on the full lattice, and against the oracle on 32^3
    res = {}
    for dims, nsteps, key in (((128, 128, 128), 500, "gpu_fp64_128"), ((32, 32, 32), 500, "oracle_32")):
        h64 = opx.Handle(3, dims, dt=0.05, precision=N.OPX_F64, device=device)
        h64.init_random(SEED + 3, 0.2, 0.2)
        h64.gauss_project(1e-26)
        h32 = opx.Handle(3, dims, dt=0.05, precision=N.OPX_F32, reunit_every=10, device=device)
        U0, E0 = h64.download(N.FIELD_U), h64.download(N.FIELD_E)
        h32.upload(N.FIELD_U, U0)
        h32.upload(N.FIELD_E, E0)
        h32.initialize()
        if key == "oracle_32":
            ref = oracle.OracleGrid(3, dims, dt=0.05)
            ref.U[...] = U0
            ref.E[...] = E0
            ref.update_links()
            nth = cpu_threads()
            e_ref0 = ref.bulk()
            for _ in range(nsteps):
                ref.store_fields()
                ref.update_grid_omp(nth)
            h32.step(nsteps)
            b = ref.bulk()
            Ur, e_ref = ref.U, b[11] + b[12]
        else:
            h64.initialize()
            h64.step(nsteps)
            h32.step(nsteps)
            o = h64.reduce()
            Ur, e_ref = h64.download(N.FIELD_U), o.e2_total + o.b2_total
        o32 = h32.reduce()
        U32 = h32.download(N.FIELD_U)
        d = np.linalg.norm((U32 - Ur).reshape(-1, 18), axis=1) / np.linalg.norm(Ur.reshape(-1, 18), axis=1)
        res[key] = {"lattice": list(dims), "steps": nsteps, "energy_rel_err": abs(o32.e2_total + o32.b2_total - e_ref) / e_ref,
                    "max_rel_link_err": float(d.max()), "mean_rel_link_err": float(d.mean())}
        h64.close()
        h32.close()
    out["su3_fp32_errors"] = res
    return out


# the lattice-size sweep: (ncolors, precision, reunit_every, sigma, bytes per link update, L)
SWEEP = [(3, "f32", 10, 0.2, 208, (48, 64, 96, 128, 160, 192, 256)),
         (2, "f32", 10, 0.1, 56, (64, 128, 192, 256)),
         (2, "f64", 0, 0.1, 112, (32, 128))]


def bench_sweep(device, steps=50, warmup=5):
    """Lattice-size sweep of the single-lattice leapfrog: per form and L^3
    periodic lattice (dt = 0.05, seeded fields), the best of three
    opx_time_steps runs (CUDA events on the handle's stream) of `steps` steps
    after `warmup` steps; one JSON line per row, with the fraction of the
    measured copy bandwidth at the form's algorithmic bytes per link update."""
    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    peak, peak_kind = hbm_peak()
    for nc, prec, reunit, sigma, bpl, sizes in SWEEP:
        for L in sizes:
            h = opx.Handle(nc, (L, L, L), dt=0.05, precision=N.OPX_F32 if prec == "f32" else N.OPX_F64,
                           reunit_every=reunit, device=device)
            h.init_random(SEED, sigma, sigma)
            h.initialize()
            h.step(warmup)
            ms = min(h.time_steps(steps) for _ in range(3)) / steps
            links = 3 * L ** 3
            print(json.dumps({"form": f"SU({nc}) {prec.upper()}", "L": L, "ms_per_step": ms,
                              "g_link_updates_per_s": links / ms / 1e6,
                              "hbm_roofline_frac": bpl * links / (ms * 1e-3) / (peak * 1e9),
                              "bytes_per_link_update": bpl, "peak_gbs": peak, "peak": peak_kind}), flush=True)
            h.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="su3_fp32_128", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-cgc", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    # one leg alone (profiling runs): the CPIC collision (`--leg-steps` steps with
    # its diagnostics, no oracle check) or the batched form (SU(`--batch-nc`),
    # `--batch-events` events, `--leg-steps` steps); prints that leg's JSON.
    # `--leg sweep`: the lattice-size sweep, one JSON line per form and size
    ap.add_argument("--leg", default="all", choices=["all", "cgc", "batch", "sweep"])
    ap.add_argument("--leg-steps", type=int, default=20)
    ap.add_argument("--batch-nc", type=int, default=3, choices=[2, 3])
    ap.add_argument("--batch-events", type=int, default=64)
    args = ap.parse_args()
    if args.leg == "cgc":
        print(json.dumps(bench_cgc(0, nsteps=args.leg_steps, oracle_steps=0)), flush=True)
        return 0
    if args.leg == "batch":
        print(json.dumps(bench_batch(0, nc=args.batch_nc, nsteps=args.leg_steps, nev=args.batch_events)), flush=True)
        return 0
    if args.leg == "sweep":
        bench_sweep(0)
        return 0
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w, args.workload)

    import openpixi_gb300 as opx
    from openpixi_gb300 import _native as N
    rank, world, local = dist_env()
    device = local
    dist = Dist("nccl" if world > 1 else "gloo")
    V = int(np.prod(w["dims"]))
    links = 3 * V

    # ---- set-up (untimed): seeded fields, Gauss projection in FP64, Unext
    h = make_handle(w, w["prec"], device)
    h.init_random(SEED + rank, w["sigma"], w["sigma"])
    cg_it, g2 = h.gauss_project(1e-24 if w["prec"] == "f32" else 1e-26, 5000)
    U_host = opx.PinnedArray((V, 3, h.ng))
    E_host = opx.PinnedArray((V, 3, h.na_ref))
    h.download(N.FIELD_U, out=U_host.array)
    h.download(N.FIELD_E, out=E_host.array)
    h.initialize()
    o0 = h.reduce()
    for _ in range(args.warmup):
        h.step(1)
    h.synchronize()

    # ---- timed region: K steps, fields resident in HBM, CUDA events on the handle's stream
    clocks = ClockSampler(device)
    clocks.start()
    l0 = h.kernel_launches
    dist.barrier()
    h.synchronize()
    with nvtx_range("timed_steps"):
        ms = h.time_steps(args.steps)
        h.synchronize()
    dist.barrier()
    launches = h.kernel_launches - l0
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = world * links * args.steps / (ms_max / 1000.0)
    o1 = h.reduce()
    e0, e1 = o0.e2_total + o0.b2_total, o1.e2_total + o1.b2_total

    # ---- roofline of the leapfrog kernel.  The timed region holds exactly one
    # launch of it per step (the CUDA events bracket only those launches), so its
    # average launch duration is the region's time over the steps; the same
    # kernel timed launch by launch afterwards is reported beside it.
    t_launch = ms_max / args.steps / 1000.0
    h.set_profiling(True)
    nprof = min(args.steps, 50)
    h.step(nprof)
    pms, pn = h.phase_times()
    h.set_profiling(False)
    t_each = pms[N.PHASE_EOM] / max(pn[N.PHASE_EOM], 1) / 1000.0
    peak, peak_kind = hbm_peak()
    achieved = w["bpl"] * links / t_launch / 1e9
    traffic = traffic_for(args.workload)
    kname = "k_update_grid_su3f_pair" if (w["nc"] == 3 and w["prec"] == "f32") else "k_update_grid"
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_link": w["bpl"], "links_per_launch": links,
                "kernel": kname, "launch_ms": t_launch * 1000.0, "launch_ms_one_by_one": t_each * 1000.0}
    # the FP32 FMA pipe's floor for the same launch (ncu FMA-pipe time at 100 %
    # busy): the kernel is bound by it before HBM, so its fraction is beside the HBM one
    fma_floor = traffic_for(args.workload, "fma_pipe_floor_ms")
    if fma_floor:
        roofline["fma_pipe_floor_ms"] = fma_floor
        roofline["frac_of_fma_pipe_floor"] = fma_floor / (t_launch * 1000.0)
        roofline["hbm_frac_at_fma_pipe_floor"] = achieved * (t_launch * 1000.0) / fma_floor / peak

    # ---- the BulkQuantities reduction (one pass: E^2, B^2 from U and Unext, Gauss, rho^2)
    h.set_profiling(True)
    with nvtx_range("reduce"):
        for _ in range(10):
            h.reduce()
    rms, rn = h.phase_times()
    h.set_profiling(False)
    reduce_ms = rms[N.PHASE_DIA] / max(rn[N.PHASE_DIA], 1)
    # the reduction right after one step, as in a per-step diagnostics loop: B^2
    # of U comes from the previous reduction's B^2 of Unext (one full reduction
    # first, its mean time taken out)
    h.set_profiling(True)
    h.reduce()
    with nvtx_range("step_reduce"):
        for _ in range(10):
            h.step(1)
            h.reduce()
    rms, rn = h.phase_times()
    h.set_profiling(False)
    reduce_after_step_ms = (rms[N.PHASE_DIA] - reduce_ms) / max(rn[N.PHASE_DIA] - 1, 1)

    # ---- the plain FP64 GPU path on the same lattice (same initial fields)
    fp64 = None
    if w["prec"] == "f32":
        h64 = make_handle(w, "f64", device)
        h64.upload(N.FIELD_U, U_host.array)
        h64.upload(N.FIELD_E, E_host.array)
        h64.initialize()
        h64.step(3)
        n64 = max(5, min(args.steps, 20))
        ms64 = h64.time_steps(n64)
        v64 = links * n64 / (ms64 / 1000.0)
        fp64 = {"value": v64 * world, "unit": METRIC, "steps": n64,
                "fp32_over_fp64": value / (v64 * world)}
        h64.close()

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        h2 = make_handle(w, w["prec"], device)
        he = (h2.ng + h2.na_ref) * 8 * links
        obs_bytes = 13 * 8
        def run(measured):
            U0, E0 = U_host.array.copy(), E_host.array.copy()
            dist.barrier()
            t = time.perf_counter()
            h2.upload(N.FIELD_U, U_host.array)
            h2.upload(N.FIELD_E, E_host.array)
            h2.initialize()
            t_in = time.perf_counter()
            if measured:
                with nvtx_range("e2e_measured"):
                    rows = h2.step_measured(args.steps)
            else:
                rows = []
                for k in range(args.steps):
                    h2.step(1)
                    rows.append(h2.reduce())
            t_loop = time.perf_counter()
            h2.download(N.FIELD_U, out=U_host.array)
            h2.download(N.FIELD_E, out=E_host.array)
            t_out = time.perf_counter()
            el = dist.max(t_out - t)
            U_host.array[...] = U0
            E_host.array[...] = E0
            return {"value": world * links * args.steps / el, "unit": METRIC,
                    "upload_ms": (t_in - t) * 1e3, "loop_ms_per_step": (t_loop - t_in) * 1e3 / args.steps,
                    "download_ms": (t_out - t_loop) * 1e3,
                    "h2d_bytes_per_step": he / args.steps,
                    "d2h_bytes_per_step": obs_bytes + he / args.steps}, rows

        plain, rows_p = run(False)
        meas, rows_m = run(True)
        # the two forms must report the same observables (FP32 rounding of the per-site terms)
        dev = max(abs(a.e2_total + a.b2_total - b.e2_total - b.b2_total) / abs(b.e2_total + b.b2_total)
                  for a, b in zip(rows_m, rows_p))
        meas["energy_rel_diff_vs_step_then_reduce"] = dev
        plain["note"] = ("opx_step(ctx, 1) then opx_reduce on every step (FieldSolver.step and "
                         "BulkQuantitiesInTime as separate drop-in calls)")
        e2e = dict(meas)
        e2e["note"] = ("MainBatch's loop with BulkQuantitiesInTime every step through the C ABI "
                       "(opx_step_measured: the BulkQuantities row of every step, 13 FP64 values, copied "
                       "to pinned host memory as each step completes; the step kernel forms the per-site "
                       "terms); initial U,E uploaded from pinned host memory and final U,E downloaded inside "
                       "the timed region")
        e2e["step_then_reduce"] = plain
        # FieldSolver.step as a per-call drop-in with the host grid authoritative:
        # every call uploads U and E and downloads E and Unext (reference layout, FP64 host arrays)
        ncall = max(3, min(args.steps, 20))
        Un_host = opx.PinnedArray((V, 3, h2.ng))
        h2.upload(N.FIELD_U, U_host.array)
        h2.upload(N.FIELD_E, E_host.array)
        h2.synchronize()
        dist.barrier()
        t = time.perf_counter()
        for k in range(ncall):
            h2.upload(N.FIELD_U, U_host.array if k == 0 else Un_host.array)
            h2.upload(N.FIELD_E, E_host.array)
            h2.update_grid()
            h2.download(N.FIELD_E, out=E_host.array)
            h2.download(N.FIELD_UNEXT, out=Un_host.array)
        el = dist.max(time.perf_counter() - t)
        e2e["per_call_copy"] = {"value": world * links * ncall / el, "unit": METRIC, "calls": ncall,
                                "h2d_bytes_per_step": he, "d2h_bytes_per_step": he,
                                "note": "each FieldSolver.step call copies the whole grid state in and out"}
        Un_host.free()
        h2.close()

    # the collision leg runs before the batched one: measured after the batched
    # leg (13 GB of batch stores and snapshots allocated and freed, 2560 FP64
    # event runs) its particle phases and diagnostics took 2.5x and 1.9x as
    # long per step in the same process
    cgc = None
    if not args.no_cgc and args.workload == "su3_fp32_128":
        cgc = bench_cgc(device)

    batched = None
    if not args.no_batch and args.workload == "su3_fp32_128":
        batched = bench_batch(device, nc=2)
        batched["su3"] = bench_batch(device, nc=3)

    configs = None
    if rank == 0 and not args.no_configs and args.workload == "su3_fp32_128":
        try:
            configs = bench_configs(device)
            configs["su2_64_differentiation"] = bench_differentiation(device)
        except Exception as e:  # the headline stands without the extra legs
            configs = {"skipped": str(e)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, U_host.array, E_host.array)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": w["prec"], "data": "synthetic",
                "config": config_for(w, args.workload), "roofline": roofline, "cpu_baseline": cpu,
                "e2e": e2e, "gpu_launches": launches, "clocks": clk, "fp64_plain": fp64, "batched": batched,
                "cgc_collision": cgc, "configs": configs,
                "reduce_ms": reduce_ms, "reduce_after_step_ms": reduce_after_step_ms,
                "energy_rel_change_over_run": abs(e1 - e0) / e0, "gauss_violation_end": o1.gauss,
                "ic": {"cg_iterations": cg_it, "mean_g2_after_projection": g2}}
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
