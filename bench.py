"""EAM MD throughput benchmark (atom-steps/s).

Workload: the 2,048,000-atom random 50/50 A/B alloy (FCC 80^3, a = 3.615 A,
seed 1, 0.05 A Gaussian noise, 600 K velocities) on the analytic EAM of
mapp4py_gb300.synth (setfl, nr = nrho = 5000, cutoff 5.5 A), NVT with the
Nose-Hoover chain, dt = 1 fs, skin 0.5 A, mixed precision (FP32 pair math,
FP64 state and reductions).  One step = one MD step of the whole cell.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Each rank runs its own replica of the cell on its own GPU (the path has no
data exchange between cells); value = atoms * steps * N / max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EAM MD atom-steps/s"
N_CELLS = (80, 80, 80)
T_K = 600.0
REF_BUDGET_S = 60  # CPU seconds of the reference arm's timed sample
# kernels in one step's CUDA graph: FP64 step_open, kick_drift, com_skin, 7 rebuild-chain, density,
# force, kick2; mixed step_open32, integrate32, 7 rebuild-chain, density32, force32, close32
KERNELS_PER_STEP = {"fp64": 13, "mixed": 12}
# how the sums of the pair terms are carried (the line's dtype in words)
ACCUMULATION = {
    "mixed": "FP32 pair terms; per-atom density, force and pair energy in compensated FP32 (Kahan) "
             "within a lane, exact FP32 two-sums across an atom's lanes, FP64 per atom and across "
             "blocks; virial in plain FP32 per thread (a few hundred terms), FP64 across threads",
    "fp64": "FP64 throughout",
}


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(name):
    """Per-launch DRAM bytes of a kernel from its committed ncu summary
    (a line 'dram_bytes_per_launch: <bytes>' in profiles/<name>.md)."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    try:
        for line in open(p):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while timing."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, dist=None, device=None):
    """The largest value of x over all ranks (x itself without a process group)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(natoms, steps, world, ms):
    """Whole-job atom-steps/s: every rank advances its own replica of natoms."""
    return natoms * steps * world / (ms / 1000.0)


def guarded(leg):
    """leg() or, if it raises, {"error": <type: message>}."""
    try:
        return leg()
    except Exception as ex:
        return {"error": "%s: %s" % (type(ex).__name__, ex)}


def workload_config(natoms, cells, world):
    """The workload both arms run (the arithmetic is the line's `precision`
    and `dtype`, outside the config, so the two arms' configs compare equal)."""
    return {"workload": "EAM NVT MD, %d-atom A/B alloy (FCC %d^3, seed 1)" % (natoms, cells),
            "natoms": natoms, "dt_fs": 1.0, "T_K": T_K,
            "parallelism": "replicas x%d" % world, "global_batch": None, "seq_len": None,
            "l2": l2_note(natoms)}


def l2_note(natoms):
    """How the timed steps stand to the 129 MB L2 (no flush between steps:
    the neighbour list is read twice per step)."""
    mb = natoms * 78 * 4 / 1e6
    if mb > 129.0:
        return "inputs larger than L2 (the neighbour list alone is ~%.0f MB)" % mb
    return "inputs smaller than L2 (neighbour list ~%.0f MB; a profiling size, not the workload)" % mb


def make_cell(cells=80):
    from mapp4py_gb300 import synth

    return synth.alloy((cells, cells, cells), xB=0.5, sigma=0.05, T=T_K, seed=1)


def write_potential(d):
    from mapp4py_gb300 import synth

    return synth.write_setfl(os.path.join(d, "AB.setfl"), ("A", "B"))


def cpu_baseline(path, cell, threads, steps=5, natoms_cap=256000):
    """The oracle's multi-threaded restatement on a bounded sample: the
    first FCC 40^3 block (256,000 atoms) of the same alloy, same noise and
    temperature, `steps` NVT steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mapp4py_gb300 import synth

    c = synth.alloy((40, 40, 40), xB=0.5, sigma=0.05, T=T_K, seed=1)
    e = O.Eam.setfl(path)
    o = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5, pair_wise=False)
    o.v = c.v
    o.nvt_run(T_K, synth.FS, synth.KB, steps, threads=threads)
    secs = o.loop_seconds
    return {"value": c.natoms * steps / secs, "unit": "atom-steps/s", "cores": threads, "kind": "port",
            "sample": "%d NVT steps of a 256,000-atom (FCC 40^3) block of the same alloy, full-list OpenMP "
                      "restatement of ForceFieldEAM/MDNVT, step loop only" % steps}


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores: the oracle's full-list
    OpenMP restatement of ForceFieldEAM/MDNVT (pinned to the reference itself
    by the ref_*.npz fixtures), FP64, on the whole workload cell."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        path = write_potential(d)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        from mapp4py_gb300 import synth

        c = make_cell(args.cells)
        e = O.Eam.setfl(path)
        o = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5, pair_wise=False)
        o.v = c.v
        o.nvt_run(T_K, synth.FS, synth.KB, args.warmup, threads=threads)
        # a bounded sample: as many of the requested steps as fit in about a
        # minute at the warm-up's pace
        per_step = o.loop_seconds / max(1, args.warmup)
        steps = max(1, min(args.steps, int(REF_BUDGET_S / max(per_step, 1e-9))))
        o.nvt_run(T_K, synth.FS, synth.KB, steps, threads=threads)
        secs = o.loop_seconds
    value = c.natoms * steps / secs
    sample = ("%d NVT steps (of %d requested; a sample bounded to ~%d s) of the whole %d-atom cell after %d "
              "warm-up steps, on %d host threads: the oracle's OpenMP restatement of the reference's CPU path, "
              "FP64; the reference itself builds only where its sources are (x86 here, not on this host)"
              % (steps, args.steps, REF_BUDGET_S, c.natoms, args.warmup, threads))
    config = workload_config(c.natoms, args.cells, world)
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "impl": "reference", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "precision": "fp64",
            "data": "synthetic", "config": config,
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_batch(args, ff, torch):
    """512 independent A/B alloy cells (log-uniform 500-32,000 atoms, random
    composition, vacancies, temperatures 100-1200 K) advanced together.  A
    3-step warm-up run, then the timed run: its args.batch_steps steps of
    every cell are one CUDA graph, launched once; device-timed like the main
    line."""
    from mapp4py_gb300 import _lib, synth

    cells, temps = synth.batch_cells(args.batch_cells, seed=7)
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    b.set_v(np.concatenate([c.v for c in cells]))
    tpa, unroll, tune = b.autotune()
    K, W = args.batch_steps, 3
    b.nvt_begin(temps, synth.FS, synth.KB, W)
    b.nvt_steps(W)
    b.nvt_end(W)
    b.nvt_begin(temps, synth.FS, synth.KB, K)  # captures the K steps as one graph
    stream = torch.cuda.ExternalStream(b.stream())
    b.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.nvt_steps(K)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    b.nvt_end(K)
    st = b.stats()
    return {"workload": "%d independent cells, %d atoms (%d-%d per cell), NVT at 100-1200 K, mixed precision"
                        % (len(cells), b.n, int(b.natoms.min()), int(b.natoms.max())),
            "value": b.n * K / (ms / 1000.0), "unit": "atom-steps/s", "steps": K, "ms_per_step": ms / K,
            "graph_launches": 1 if K <= 512 else -(-K // 512), "rebuilds_in_run": st["rebuilds"],
            "lanes_per_atom": tpa, "entries_per_step": unroll, "atoms_per_chunk": b.chunk_atoms,
            "force_entries_per_step": b.tuning()["force_entries_per_step"],
            "autotune_ms": {"%d,%d,%d" % k: round(v, 4) for k, v in tune.items()}}


def run_lbfgs(args, ff):
    """L-BFGS time to max|F| < 1e-4 eV/A, the learned diagonal initial inverse
    Hessian against plain L-BFGS (scalar gamma); m = 10, back-tracking line
    search, mixed precision (FP32 forces; line-search energy differences
    formed pair by pair, FP32 energy differences for steps beyond the skin).
      c4: the 253,489-atom cell (A/B alloy, FCC 40^3, 1 % vacancies, 0.15 A
          noise, seed 3), to the tolerance or args.lbfgs_cap iterations
      c5: args.c5_cells cells of 1,000-16,000 atoms (log-uniform), random
          composition, 0-3 % vacancies, strain up to +-2 %, noise
          U(0.05, 0.2) A, relaxed together as one batch, each cell to the
          tolerance or args.c5_cap iterations
    max_dx (the largest atom move of a step, MinLBFGS's max_dx) is
    args.lbfgs_dx for both.  Each system is autotuned before its timed run,
    as md.atoms tunes mixed systems of 50,000 atoms or more."""
    from mapp4py_gb300 import _lib, precond, synth

    net = precond.load()
    dx = args.lbfgs_dx

    def c4(cap):
        c = synth.alloy((args.lbfgs_n,) * 3, xB=0.5, sigma=0.15, vac=0.01, seed=3)
        res = {"natoms": c.natoms, "iteration_cap": cap, "max_dx": dx}
        for name in ("plain", "learned"):
            s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
            s.build()
            s.autotune()  # as md.atoms does for a mixed system of 50,000 atoms or more
            s.sync()
            t0 = time.perf_counter()
            if name == "plain":
                r = s.lbfgs_run(m=10, e_tol=0.0, max_dx=dx, f_tol=1e-4, nsteps=cap)
            else:
                r = _lib.lbfgs_run_precond(s, net, m=10, e_tol=0.0, max_dx=dx, f_tol=1e-4, nsteps=cap)
            secs = time.perf_counter() - t0
            res[name] = {"seconds": secs, "converged": r["err"] == 100, "stop_code": r["err"], "iterations": r["niter"],
                         "fmax": r["fmax"], "energy_calls": r["n_energy"], "force_calls": r["n_force"],
                         "ms_per_iteration": 1000.0 * secs / max(1, r["niter"])}
        res["wall_ratio_plain_over_learned"] = res["plain"]["seconds"] / res["learned"]["seconds"]
        return res

    def c5(ncell, cap):
        cells, _ = synth.batch_cells(ncell, seed=11, nmin=1000, nmax=16000, vac=(0.0, 0.03), sigma=(0.05, 0.2),
                                     strain=0.02)
        res = {"cells": ncell, "natoms": int(sum(x.natoms for x in cells)), "iteration_cap": cap, "max_dx": dx}
        for name in ("plain", "learned"):
            b = _lib.Batch(ff, [(x.H, x.x, x.elem) for x in cells], cells[0].masses)
            b.autotune()  # chunk, lanes per atom and unrolling for the batch's own cells
            b.sync()
            t0 = time.perf_counter()
            r = b.lbfgs_run(m=10, max_dx=dx, f_tol=1e-4, nsteps=cap, net=None if name == "plain" else net)
            secs = time.perf_counter() - t0
            its = np.array([q["niter"] for q in r])
            codes = {}
            for q in r:
                codes[str(q["err"])] = codes.get(str(q["err"]), 0) + 1
            res[name] = {"seconds": secs, "cells_converged": int(sum(q["err"] == 100 for q in r)), "stop_codes": codes,
                         "iterations_max": int(its.max()), "iterations_median": float(np.median(its)),
                         "energy_calls": int(sum(q["n_energy"] for q in r)),
                         "force_calls": int(sum(q["n_force"] for q in r))}
        res["wall_ratio_plain_over_learned"] = res["plain"]["seconds"] / res["learned"]["seconds"]
        return res

    out = {"metric": "L-BFGS time to max|F| < 1e-4 eV/A, learned vs plain", "unit": "s",
           "stop_code_legend": {"100": "max|F| below the tolerance", "5": "iteration cap",
                                "3": "line search: step below min_alpha", "1": "line search: not downhill",
                                "2": "line search: zero gradient", "4": "energy change below e_tol",
                                "7": "bracketing: step above its maximum",
                                "8": "bracketing: not downhill"},
           "network": "33-64-64-3 BF16 MLP trained on 201,814 FD Hessian diagonals (precond_net.npz)"}
    if args.lbfgs_cap > 0:
        out["c4"] = c4(args.lbfgs_cap)
    if args.c5_cells > 0:
        out["c5"] = c5(args.c5_cells, args.c5_cap)
    return out


def run_accuracy(args, ff, path, cell, torch):
    """The FP64 path on the same 2,048,000-atom cell (throughput), the mixed
    path's error against it (force RMS, energy per atom), and the NVE energy
    drift of both paths (run_nve)."""
    from mapp4py_gb300 import _lib, synth

    out = {}
    s64 = _lib.System(ff, cell.H, cell.x, cell.elem, cell.masses, precision=_lib.FP64)
    s64.set_v(cell.v)
    K = 10
    s64.nvt_begin(T_K, synth.FS, synth.KB, K + 3)
    st = torch.cuda.ExternalStream(s64.stream())
    s64.nvt_steps(3)
    s64.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    s64.nvt_steps(K)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / K
    s64.nvt_end(K + 3)
    out["fp64"] = {"value": cell.natoms / (ms / 1000.0), "unit": "atom-steps/s", "ms_per_step": ms, "steps": K}
    # the FP64 path's own roof: its pair kernels are bound by the FP64 pipe,
    # not by HBM
    out["fp64"]["roof"] = guarded(lambda: {
        "bound": "fp64 pipe", "fma_rate_tflops": _lib.fp64_fma_rate(),
        "source": "mappg_fp64_fma_rate: independent FP64 FMA chains on every SM, CUDA events"})
    # error of the mixed path against FP64 on the starting configuration
    a = _lib.System(ff, cell.H, cell.x, cell.elem, cell.masses, precision=_lib.FP64)
    b = _lib.System(ff, cell.H, cell.x, cell.elem, cell.masses, precision=_lib.MIXED)
    pa, _ = a.force()
    pb, _ = b.force()
    fa, fb = a.get_f(), b.get_f()
    out["mixed_vs_fp64"] = {"force_rms_eV_per_A": float(np.sqrt(np.mean(np.sum((fa - fb) ** 2, axis=1)))),
                            "force_max_eV_per_A": float(np.max(np.abs(fa - fb))),
                            "energy_eV_per_atom": float(abs(pa - pb) / cell.natoms)}
    del a, b
    out["nve"] = run_nve(args, path)
    return out


def run_nve(args, ff_path):
    """NVE energy drift (t_relax = inf, dt = 1 fs) over args.nve_ps
    picoseconds, mixed and FP64, on the 4,000-atom single-element FCC cell
    of the plain FP64 workload (300 K start).  The 50/50 alloy of the MD
    workload is metastable under this potential: NVE runs of it (and of the
    single-element crystal from 600 K) collapse within a few ps into a denser
    structure (rows 78 -> 125 entries, 0.7-1 eV/atom released; the oracle
    shows the same), so a drift over tens of ps is only meaningful on a cell
    that stays crystalline.  Drift = slope of a straight-line fit of the
    total energy per atom."""
    from mapp4py_gb300 import _lib, synth

    c = synth.md_single((10, 10, 10), T=300.0, seed=0)
    ff1 = _lib.ForceField.setfl(ff_path, ["A"])
    out = {"workload": "%d-atom single-element FCC 10^3, 300 K start" % c.natoms, "dt_fs": 1.0}
    for name, prec in (("mixed", _lib.MIXED), ("fp64", _lib.FP64)):
        nsteps = int(round(args.nve_ps * 1000))
        s = _lib.System(ff1, c.H, c.x, c.elem, c.masses, precision=prec)
        s.set_v(c.v)
        t0 = time.perf_counter()
        th, _ = s.nvt_run(300.0, synth.FS, synth.KB, nsteps, t_relax=float("inf"), thermo=True)
        secs = time.perf_counter() - t0
        etot = (th[:, 0] + 0.5 * (th[:, 2] + th[:, 5] + th[:, 7])) / c.natoms
        t_ns = np.arange(nsteps + 1) * 1e-6
        slope = np.polyfit(t_ns, etot, 1)[0]
        out[name] = {"steps": nsteps, "span_ns": nsteps * 1e-6, "drift_eV_per_atom_per_ns": float(slope),
                     "max_deviation_eV_per_atom": float(np.max(np.abs(etot - etot[0]))),
                     "T_end_K": float(th[-1, 1]), "seconds": secs}
    return out


def run_c1(args, ff_path, torch):
    """The reference's CPU-runnable case: 4,000 atoms, FCC 10^3, NVE 100
    steps, FP64, on the GPU and on the oracle (1 thread and all threads)."""
    from mapp4py_gb300 import _lib, synth

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    c = synth.md_single((10, 10, 10), T=300.0, seed=0)
    ff1 = _lib.ForceField.setfl(ff_path, ["A"])  # the single-element case: element A of the file
    s = _lib.System(ff1, c.H, c.x, c.elem, c.masses)
    s.set_v(c.v)
    s.nvt_run(300.0, synth.FS, synth.KB, 5, t_relax=float("inf"))  # warm-up (graph, first launches)
    s = _lib.System(ff1, c.H, c.x, c.elem, c.masses)
    s.set_v(c.v)
    tpa, _, _ = s.autotune()  # lanes per atom for this small FP64 system
    s.nvt_begin(300.0, synth.FS, synth.KB, 100, t_relax=float("inf"))
    st = torch.cuda.ExternalStream(s.stream())
    s.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    s.nvt_steps(100)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    s.nvt_end(100)
    out = {"workload": "4000-atom FCC 10^3, NVE 100 steps, FP64", "gpu": c.natoms * 100 / (ms / 1000.0),
           "lanes_per_atom": tpa}
    e = O.Eam.setfl(ff_path)
    masses = np.full(e.nelem, c.masses[0])  # one mass per element of the file (all atoms are A)
    for name, threads in (("oracle_1_thread", 0), ("oracle_all_threads", os.cpu_count() or 1)):
        o = O.System(e, c.H, c.x, c.elem, masses, pair_wise=threads == 0)
        o.v = c.v
        o.nvt_run(300.0, synth.FS, synth.KB, 100, t_relax=float("inf"), threads=threads)
        out[name] = c.natoms * 100 / o.loop_seconds
    out["unit"] = "atom-steps/s"
    out["cores"] = os.cpu_count() or 1
    return out


def run_gpu(args, rank, world, local_rank):
    import torch

    from mapp4py_gb300 import _lib, md, synth

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    K, W = args.steps, args.warmup
    tmp = tempfile.TemporaryDirectory()
    path = write_potential(tmp.name)
    cell = make_cell(args.cells)
    N = cell.natoms
    ff = _lib.ForceField.setfl(path)
    prec = _lib.MIXED if args.precision == "mixed" else _lib.FP64
    sysm = _lib.System(ff, cell.H, cell.x, cell.elem, cell.masses, skin=0.5, precision=prec)
    sysm.set_v(cell.v)
    tpa, unroll, tune_ms = sysm.autotune()  # lanes per atom, entries per step of the density/force kernels
    dt = synth.FS
    sysm.nvt_begin(T_K, dt, synth.KB, W + K, t_relax=100.0 * dt, L=3, niters=1)
    stream = torch.cuda.ExternalStream(sysm.stream())
    sysm.nvt_steps(W)
    sysm.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local_rank)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sysm.nvt_steps(K)
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    sysm.nvt_end(K + W)
    ms = max_over_ranks(ms, dist, "cuda")
    value = throughput(N, K, world, ms)
    st = sysm.stats()
    kbar = st["mean_row_x1000"] / 1000.0

    # dominant kernels timed alone with CUDA events on the library's stream
    def time_kernel(what, reps=20):
        for _ in range(3):
            sysm.enqueue(what)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            sysm.enqueue(what)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    sysm.enqueue(0)
    t_density = time_kernel(0)
    t_force = time_kernel(1)
    # algorithmic bytes per launch (per atom: the row of 4*K entries plus the
    # atom's own streams; neighbour gathers are served by L2)
    if prec == _lib.MIXED:
        b_force = N * (4 * kbar + 16 + 1 + 4 + 12)   # row, q32 (position, F'), elem, count, f32 write
        b_density = N * (4 * kbar + 16 + 1 + 4 + 16 + 4)  # row, p32, elem, count, q32 write, rho32 write
    else:
        b_force = N * (4 * kbar + 24 + 8 + 1 + 4 + 4 + 24)   # row, x, dF, elem, count, bins, f
        b_density = N * (4 * kbar + 24 + 1 + 4 + 4 + 8 + 8)
    peak, peak_kind = peaks()
    achieved = b_force / (t_force / 1000.0) / 1e9
    prof = "k_force_mixed_alloy_2048000" if prec == _lib.MIXED else "k_force_fp64_alloy_2048000"
    traffic = traffic_from_profiles(prof)
    roof = {"bound": "hbm", "kernel": "k_force", "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "bytes_per_launch": b_force, "ms_per_launch": t_force,
            "density_kernel": {"ms_per_launch": t_density, "bytes_per_launch": b_density,
                               "achieved": b_density / (t_density / 1000.0) / 1e9},
            "step_bytes_per_atom": 8 * kbar + 305, "mean_row": kbar,
            "step_frac": (8 * kbar + 305) * value / world / 1e9 / peak}

    # end to end: md.nvt(T,dt).run(atoms, 1) per step through the public API,
    # positions and velocities in pinned host memory, copied in and out
    E = max(1, min(K, args.e2e_steps))
    xh = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    vh = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    xh[:] = cell.x
    vh[:] = cell.v
    at = md.atoms(cell.H, xh, cell.elem, elems=("A", "B"), masses=cell.masses, x_d=vh)
    at.x, at.x_d = xh, vh  # keep the pinned buffers
    at.f = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()  # refilled in place
    at.kB = synth.KB
    at.precision = args.precision
    at.ff = ff
    nv = md.nvt(T_K, dt)
    nv.ntally = 0
    nv.run(at, 1)  # warm-up call (system creation)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(E):
        nv.run(at, 1)
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    te = max_over_ranks(te, dist, "cuda")
    e2e = {"value": throughput(N, E, world, 1000.0 * te), "unit": "atom-steps/s", "h2d_bytes_per_step": 48 * N,
           "d2h_bytes_per_step": 72 * N, "steps": E,
           "call": "mapp4py_gb300.md.nvt(600,1fs).run(atoms,1): x,v in; x,v,f out (pinned); skin test "
                   "(list rebuilt when an atom moved more than skin/2) + opening force call + one step per "
                   "call, as MDNVT::run"}

    # the legs beside the headline: each reports its own failure in the line
    # instead of taking the measured headline down with it
    batched = None if args.batch_steps <= 0 else guarded(lambda: run_batch(args, ff, torch))
    lbfgs = None if args.lbfgs_cap <= 0 and args.c5_cells <= 0 else guarded(lambda: run_lbfgs(args, ff))
    extras = None
    if args.extras and rank == 0:
        extras = guarded(lambda: run_accuracy(args, ff, path, cell, torch))
        if "error" in extras:
            extras = {"accuracy_error": extras["error"]}
        if not args.no_cpu:
            extras["c1"] = guarded(lambda: run_c1(args, path, torch))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64acc" if prec == _lib.MIXED else "f64", "precision": args.precision,
                "accumulation": ACCUMULATION[args.precision],
                "data": "synthetic",
                "config": workload_config(N, args.cells, world),
                "tuning": dict(sysm.tuning(), entries_per_step=unroll,
                               autotune_ms={"%d,%d" % k: round(v, 4) for k, v in tune_ms.items()}),
                "roofline": roof, "clocks": clk, "e2e": e2e, "gpu_launches": KERNELS_PER_STEP[args.precision] * K,
                "neighbor": {"rebuilds_in_run": st["rebuilds"], "max_row": st["max_row"], "capacity": st["capacity"]}}
        if batched is not None:
            line["batched"] = batched
        if lbfgs is not None:
            line["lbfgs"] = lbfgs
        if extras is not None:
            line.update(extras)
        if not args.no_cpu and world == 1:
            try:
                line["cpu_baseline"] = cpu_baseline(path, cell, os.cpu_count() or 1)
            except Exception as ex:  # reported, not fatal
                line["cpu_baseline"] = {"value": None, "error": str(ex)}
            cpu = line["cpu_baseline"].get("value")
            if cpu and "fp64" in line:
                # the same FP64 arithmetic on both sides: GPU FP64 path against the CPU port
                line["fp64_gpu_vs_cpu"] = {"gpu_fp64": line["fp64"]["value"], "cpu_fp64": cpu,
                                           "ratio": line["fp64"]["value"] / cpu}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    tmp.cleanup()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="mapp", choices=["mapp", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=500,
                    help="steps of the 512-cell batch measurement (0 skips it)")
    ap.add_argument("--batch-cells", type=int, default=512)
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the FP64 run, the mixed-vs-FP64 error, the NVE drift and the 4,000-atom case")
    ap.add_argument("--nve-ps", type=float, default=50.0,
                    help="length of the mixed-precision NVE drift run in ps (1 fs steps)")
    ap.add_argument("--lbfgs-cap", type=int, default=20000,
                    help="iteration cap of the 253,489-atom L-BFGS comparison (0 skips it)")
    ap.add_argument("--lbfgs-n", type=int, default=40, help="FCC repeats per side of that cell")
    ap.add_argument("--lbfgs-dx", type=float, default=1.0, help="max_dx of the L-BFGS runs (A)")
    ap.add_argument("--c5-cells", type=int, default=128,
                    help="cells of the batched L-BFGS comparison, the first cells of the 1024-cell recipe "
                         "(0 skips it; all 1024 take about 6 min per arm)")
    ap.add_argument("--c5-cap", type=int, default=8000, help="iteration cap per cell of the batched comparison")
    ap.add_argument("--cells", type=int, default=N_CELLS[0],
                    help="FCC repeats per side (80 = the 2,048,000-atom workload; smaller for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", args.gpus)
    local_rank = env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
