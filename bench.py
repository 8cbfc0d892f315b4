#!/usr/bin/env python3
"""Benchmark of the GB300 explicit MPM step (one JSON line on stdout).

Workload (default): the 3-D soil slope -- 20 m high, 45 degrees, 0.1 m
particle spacing jittered by +-1% from a fixed seed (1.2 M particles), grid
cell 0.2 m, Drucker-Prager (c = 10 kPa, phi = 20 deg), gravity, GIMP shape
functions, USF. A "step" is one explicit time step of the whole scene.

  value      particle-steps/s of the mixed-precision form, state resident in
             HBM, CUDA-graph replay, timed with CUDA events on the library's
             stream (inputs are larger than L2, no flush needed);
  fp64       the plain FP64 form (bit-identical to the CPU oracle) on the same
             steps, and the mixed form's error against it;
  e2e        the same metric through the C ABI from page-locked host arrays:
             context creation (host->device upload of the particle state), the
             steps with the per-step scalar read-back the host loop needs for
             its exit test, and the read-back of the particle state;
  roofline   the dominant kernel's algorithmic bytes / its event-timed duration;
  cpu_baseline  the CPU oracle (a restatement of the reference step) on a
             bounded sample of the same workload on this host's cores.

`--impl reference` times the reference's CPU step (the oracle port; the
Fortran reference cannot be compiled on these machines) with one replica per
host core.

Multi-GPU: scenes are independent, so N GPUs run N replicas (weak scaling,
no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mpm3d-f90_gb300"))

WORKLOADS = {
    # name: (deck factory kwargs, description)
    "soil_slope": ("soil slope 20 m 45 deg, 0.1 m spacing, GIMP, Drucker-Prager, USF",),
    "taylor_bar": ("Taylor bar R 3.2 mm L 32.4 mm, 0.4 mm spacing, linear, Johnson-Cook + EOS, USF",),
    "dam_break": ("dam break 4x2x2 m in 10x2x4 m tank, 1 cm spacing, B-spline, null + EOS 4, MUSL",),
    "granular_column": ("granular column r 0.5 m H 1 m, 2.307 mm spacing, 512x512x256 grid of 4 mm, GIMP, "
                        "Drucker-Prager phi 30 c 0, MUSL",),
}


def make_deck(workload: str, scale: float = 1.0) -> str:
    from mpm3d_gb300 import decks

    if workload == "soil_slope":
        return decks.soil_slope(dp=0.1 * scale, width=3.0)
    if workload == "taylor_bar":
        return decks.taylor_bar(dp=4e-4 * scale)
    if workload == "dam_break":
        return decks.dam_break(dp=0.01 * scale, h=0.02 * scale)
    if workload == "granular_column":
        return decks.granular_column(scale)[0]
    raise SystemExit(f"unknown workload {workload}")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region:
    the sampler runs every 20 ms from before the region (the first sample is
    awaited, so sampling is live when the region starts), each line is
    stamped with the host clock when it arrives, and only the lines that
    arrived between the region's start and shortly after its end are kept."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.perf_counter() + 5.0
            while not self.lines and time.perf_counter() < deadline and self.proc.poll() is None:
                time.sleep(0.005)
        except OSError:
            self.proc = None
        self.t0 = time.perf_counter()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self) -> dict:
        self.t1 = time.perf_counter()
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)  # a sample taken at the end of the region is still in the pipe
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        inside = [ln for t, ln in self.lines if self.t0 <= t <= self.t1 + 0.05]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in inside:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": 20,
                "region_ms": round((self.t1 - self.t0) * 1e3, 1)}


def rel_err(a, b) -> float:
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b)))


def disp_err(xm, xf, x0) -> float:
    """Position error relative to the motion: max |(Xm - X0) - (Xf - X0)| /
    max |Xf - X0| (positions stay FP64 in the mixed form, so an error relative
    to the coordinates themselves would say nothing)."""
    import numpy as np

    dm = np.asarray(xm, dtype=np.float64) - x0
    df = np.asarray(xf, dtype=np.float64) - x0
    s = float(np.max(np.abs(df)))
    return float(np.max(np.abs(dm - df)) / s) if s > 0 else float(np.max(np.abs(dm - df)))


def form_errors(mixed: dict, fp64: dict, x0) -> dict:
    """Mixed-form error against the FP64 form on the same deck after the same
    steps: nodal momentum, particle stress (mean and deviatoric), particle
    displacement; each max |a - b| / max |b| over the field."""
    return {"nodal_momentum_rel": rel_err(mixed["PXg"], fp64["PXg"]),
            "particle_stress_rel": max(rel_err(mixed["SM"], fp64["SM"]), rel_err(mixed["SD"], fp64["SD"])),
            "displacement_rel": disp_err(mixed["Xp"], fp64["Xp"], x0)}


ERR_FIELDS = ("PXg", "Mg", "SM", "SD", "Xp", "VXp")


def run_to(s, total: int) -> None:
    """Advance a context to step `total` (graph replay) and wait for it."""
    done = int(s.scalars()["istep"])
    if total > done:
        s.run(total - done, graph=True)
    s.sync()


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def dominant_kernel(stats: list, steps: int) -> dict:
    best = max(stats, key=lambda s: s["total_ms"])
    return dict(best, avg_ms=best["total_ms"] / max(1, best["launches"]))


def kernel_bytes(kernel: str, np_: int, nn_active: float, usf: bool = True) -> float:
    """Algorithmic bytes of one launch of a kernel of the mixed (batched) step:
    the particle and node fields it must touch, each read once and written
    once, at their stored widths (FP64 position, velocity, mass, energy, grid;
    FP32 stress state). Sort keys, permutation and per-step scratch are
    implementation overhead and are not counted."""
    if kernel == "p2g_mass_scatter":
        # read x, mass, v; add node mass + momentum
        return np_ * (24 + 8 + 24) + nn_active * 32
    if kernel == "p2g_force_scatter":
        # read x, sigma * vol (6), external force (3); add node force
        return np_ * (24 + 36) + nn_active * 24
    if kernel == "p2g_mass":
        # node finalize: node mass + momentum written (+ velocity under USF)
        return nn_active * (32 + (12 if usf else 0))
    if kernel == "p2g_force_integrate":
        # node finalize: read mass + momentum, write force, momentum, velocity, acceleration
        return nn_active * (32 + 24 + 24 + 24)
    if kernel == "stress_update":
        # read x, vol, SM, SD, q, ie, cp, epeff, sig_y; write vol, SM, SD, q,
        # ie, seqv, epeff; node velocity read once; under USF the kernel also
        # stages the force input (read mass, point loads; write sigma * vol
        # and the external force)
        staged = np_ * (8 + 24 + 36) if usf else 0
        return np_ * (24 + 4 * 13 + 8) + np_ * (4 * 11 + 8) + nn_active * 12 + staged
    if kernel == "g2p_position":
        # read x, v; write x, v; node velocity and acceleration read once
        return np_ * 96 + nn_active * 24
    if kernel == "permute":
        return np_ * 2 * (6 * 8 + 6 * 8 + 16 * 4 + 1 + 2 + 2 + 4)
    return np_ * 100.0


def profiled_fp64_ops(workload: str, kernel: str, particles: int):
    """Executed FP64 operations per launch of an FP64-form kernel (adds and
    multiplies count 1, fused multiply-adds 2), from one ncu capture
    summarised in profiles/ (lines 'fp64_ops: <workload> <kernel> <ops>
    <particles>'), scaled to this run's particle count; None without one."""
    import glob
    import re

    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"fp64_ops:\s+(\S+)\s+(\S+)\s+([0-9.eE+]+)\s+([0-9]+)", line.strip())
                if m and m.group(1) == workload and m.group(2) == kernel:
                    return float(m.group(3)) * particles / float(m.group(4))
    return None


def fp64_roofline(args, device: int, kernels: list, steps: int, npart: int) -> dict:
    """The FP64 forms' ceiling is the FP64 pipe: the measured FMA rate of
    this device (mpm_fp64_ceiling) and, per FP64 kernel, its executed FP64
    flops per launch (ncu capture in profiles/) over its event-timed
    duration."""
    import mpm3d_gb300 as m

    ceil = m.fp64_ceiling(device)
    peak = ceil["fp64_tflops"]
    per = {}
    for k in kernels:
        if not k["launches"]:
            continue
        avg_ms = k["total_ms"] / k["launches"]
        ops = profiled_fp64_ops(args.workload, k["kernel"], npart)
        ach = ops / (avg_ms / 1e3) / 1e12 if ops else None
        per[k["kernel"]] = {"ms_per_step": round(k["total_ms"] / steps, 4),
                            "fp64_tflops": ach, "frac": (ach / peak) if ach else None}
    return {"bound": "fp64", "unit": "TFLOP/s", "peak": peak, "peak_source": "measured (mpm_fp64_ceiling)",
            "ddiv_per_s": ceil["ddiv_per_s"], "kernels": per}


def profiled_traffic(workload: str, kernel: str, particles: int):
    """DRAM bytes per launch (dram__bytes_read + write) of a step category,
    from one ncu capture summarised in profiles/ (lines 'traffic_bytes:
    <workload> <category> <bytes> <particles>'), scaled to this run's particle
    count (the per-particle traffic of these kernels does not depend on the
    count); None when the workload has no capture."""
    import glob
    import re

    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"traffic_bytes:\s+(\S+)\s+(\S+)\s+([0-9.eE+]+)\s+([0-9]+)", line.strip())
                if m and m.group(1) == workload and m.group(2) == kernel:
                    return float(m.group(3)) * particles / float(m.group(4))
    return None


class Replicas:
    """Multi-GPU runs are replicas: one process per GPU (torchrun), each
    advancing its own copy of the workload; the only cross-rank traffic is a
    barrier around the timed region and the max of the timings (gloo, host
    side; no collective on the data path)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo", init_method="env://")
            self.dist = dist

    def barrier(self) -> None:
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None


def aggregate_rate(units_per_rank: float, world: int, steps: int, ms_max: float) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world * steps / (ms_max / 1e3)


def workload_config(args, npart: int, grid_nodes: int, world: int) -> dict:
    """The config object of both arms (the same workload, so the same dict)."""
    return {"workload": f"{args.workload}: {WORKLOADS[args.workload][0]}", "particles": npart,
            "grid_nodes": grid_nodes, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (no flush)"}


def run_ours(args) -> dict:
    import numpy as np
    import mpm3d_gb300 as m

    rep = Replicas()
    world, rank, local = rep.world, rep.rank, rep.local
    text = make_deck(args.workload, args.scale)
    with tempfile.NamedTemporaryFile("w", suffix=".mpm", delete=False) as f:
        f.write(text)
        deck_path = f.name
    deck = m.Deck.load(deck_path)
    os.unlink(deck_path)
    npart = deck.nb_particle

    barrier = rep.barrier
    max_over_ranks = rep.max

    results = {}
    states = {}
    ctxs = {}
    x0 = deck.particles()["Xp"]
    for form in (("mixed",) if args.no_fp64 else ("fp64", "mixed")):
        s = m.MpmStep(deck, precision=form, device=local)
        s.run(args.warmup, graph=True)
        s.sync()
        barrier()
        sampler = ClockSampler(local) if form == "mixed" else None
        if sampler:
            sampler.start()
        ms = s.time_steps(args.steps, graph=True)
        s.sync()
        clocks = sampler.stop() if sampler else None
        ms = max_over_ranks(ms)
        barrier()
        results[form] = {"ms": ms, "clocks": clocks, "device_bytes": s.device_bytes(),
                         "alg_bytes_step": s.algorithmic_bytes(), "scalars": s.scalars()}
        states[form] = {f: s.download(f) for f in ERR_FIELDS}
        # per-kernel timing over a second, profiled run of the same length
        s.profile(True)
        s.time_steps(args.steps, graph=True)
        results[form]["kernels"] = s.kernel_stats()
        s.profile(False)
        ctxs[form] = s
    err = None
    if "fp64" in states:
        err = dict(form_errors(states["mixed"], states["fp64"], x0), steps=args.warmup + args.steps)
    # the FP64 form with CUDA's libm and contraction (within 1e-10 of the
    # oracle on glibc): the faster of the two plain FP64 forms
    native = None
    if not args.no_fp64:
        if args.target_steps <= 0:  # the strict context is not needed again: free its memory first
            ctxs.pop("fp64").close()
        try:
            s = m.MpmStep(deck, precision="native", device=local)
        except m.MpmError as e:  # (a workload that fits one FP64 context, not two)
            s = None
            native = {"skipped": str(e)}
        if s is not None:
            s.run(args.warmup, graph=True)
            s.sync()
            barrier()
            ms_n = max_over_ranks(s.time_steps(args.steps, graph=True))
            s.close()
            native = {"value": aggregate_rate(npart, world, args.steps, ms_n), "ms_per_step": ms_n / args.steps}
    # error at the workload's own length: both forms advanced from the same
    # deck to the same step, outside the timed regions
    target_c2 = None
    if "fp64" in ctxs and args.target_steps > 0:
        t0 = time.perf_counter()
        fin = {}
        for form in ("fp64", "mixed"):
            run_to(ctxs[form], args.target_steps)
            fin[form] = {f: ctxs[form].download(f) for f in ERR_FIELDS}
        # the FP64 form's own response to input noise the size of one FP32
        # rounding: the same deck with every initial coordinate perturbed by
        # a seeded relative 1e-7, run to the same step
        pert = m.MpmStep(deck, precision="fp64", device=local)
        xp = pert.download("Xp")
        pert.upload("Xp", xp * (1.0 + 1e-7 * np.random.default_rng(7).uniform(-1.0, 1.0, size=xp.shape)))
        run_to(pert, args.target_steps)
        fin["perturbed"] = {f: pert.download(f) for f in ERR_FIELDS}
        pert.close()
        target_c2 = {"steps": args.target_steps,
                     "max_error": form_errors(fin["mixed"], fin["fp64"], x0),
                     "fp64_perturbed_1e-7": form_errors(fin["perturbed"], fin["fp64"], x0),
                     "wall_s": round(time.perf_counter() - t0, 1)}
    for c in ctxs.values():
        c.close()

    # end to end through the C ABI from host buffers: the deck's particle
    # arrays and the result buffers are page-locked once, before the timed
    # region, as a host program would allocate them
    if args.no_e2e:
        t_e2e, h2d, d2h = float("nan"), 0, 0
    if not args.no_e2e:
        res_fields = ("Xp", "VXp", "SM", "SD")
        deck.pin(True)
        bufs = {f: m.pinned_empty(m.COMPONENTS.get(f, 1) * npart) for f in res_fields}
        t0 = time.perf_counter()
        e2 = m.MpmStep(deck, precision="mixed", device=local)
        h2d = npart * 8 * (1 + 3 + 3 + 3)  # mass, Xp, VXp, FXp uploaded
        for _ in range(args.steps):
            e2.step()
            e2.scalars()  # the host loop's exit test needs CurrentTime every step
        out = [e2.download(f, out=bufs[f]) for f in res_fields]
        t_e2e = time.perf_counter() - t0
        d2h = args.steps * 16 * 8 + sum(o.nbytes for o in out)
        e2.close()
        deck.pin(False)
        t_e2e = max_over_ranks(t_e2e)

    mixed, fp64 = results["mixed"], results.get("fp64")
    value = aggregate_rate(npart, world, args.steps, mixed["ms"])
    fp64_value = aggregate_rate(npart, world, args.steps, fp64["ms"]) if fp64 else None
    peaks = measured_peaks()
    dom = dominant_kernel(mixed["kernels"], args.steps)
    nn_active = mixed["scalars"]["active_nodes"]
    kb = kernel_bytes(dom["kernel"], npart, nn_active)
    achieved = kb / (dom["avg_ms"] / 1e3) / 1e9
    line = {
        "metric": "particle-steps/s (mixed precision vs plain FP64 GPU, stated error)",
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mixed["ms"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 particle / f64 grid (mixed)",
        "data": "synthetic (seeded deck generator)",
        "config": workload_config(args, npart, int(mixed["scalars"]["nb_gridnode"]), world),
        "graph": True,
        "fp64": ({"value": fp64_value, "ms_per_step": fp64["ms"] / args.steps, "dtype": "f64",
                  "parity": "bit-identical to the CPU oracle (tests/test_gpu_parity.py)",
                  "speedup_mixed_over_fp64": value / fp64_value,
                  "native": native,
                  "speedup_mixed_over_fp64_native": value / native["value"] if native and "value" in native else None}
                 if fp64 else None),
        "error_vs_fp64": err,
        "e2e": {"value": npart * world * args.steps / t_e2e, "unit": "particle-steps/s",
                "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps},
        "roofline": {"bound": "hbm", "kernel": dom["kernel"], "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "traffic": profiled_traffic(args.workload, dom["kernel"], npart), "algorithmic_bytes": kb,
                     "avg_launch_ms": dom["avg_ms"]},
        "step_alg_gbs": mixed["alg_bytes_step"] / (mixed["ms"] / args.steps / 1e3) / 1e9,
        "kernels_mixed": {k["kernel"]: round(k["total_ms"] / args.steps, 4) for k in mixed["kernels"] if k["launches"]},
        "kernels_fp64": ({k["kernel"]: round(k["total_ms"] / args.steps, 4) for k in fp64["kernels"] if k["launches"]}
                         if fp64 else None),
        "gpu_launches": sum(k["launches"] for k in mixed["kernels"]),
        "clocks": mixed["clocks"],
    }
    target = {}
    if target_c2 is not None:
        fastest = max(fp64_value, native["value"]) if native and "value" in native else fp64_value
        target[args.workload] = dict(target_c2, ratio_mixed_over_fp64=value / fastest,
                                    fp64_form_compared="fastest of strict / native",
                                    error_reference="FP64 strict form (bit-identical to the oracle)")
    if fp64 is not None:
        line["fp64"]["roofline"] = fp64_roofline(args, local, fp64["kernels"], args.steps, npart)
    if world == 1 and args.serve_scenes > 0:
        line["serving"], target_c4 = run_serving(args, local)
        if target_c4 is not None:
            target["serving_scenes"] = target_c4
    if target:
        line["target"] = target
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(text, args.cpu_steps, npart)
    rep.close()
    return line if rank == 0 else None


def run_serving(args, device: int) -> dict:
    """Serving workload: scenes (Cook membrane panels and cantilever soft
    beams, SGMP, MUSL, neo-Hookean; particle counts log-uniform in 2k..400k;
    E log-uniform in 1..100 MPa, nu uniform in 0.3..0.49) arriving as a
    Poisson process, each run for a fixed step count through the serving
    runtime (HBM-budget admission, batched chunks, CUDA graphs, launch-shape
    autotuning). Reports scene latency (submit to retirement) percentiles and
    the aggregate particle-step rate over the run."""
    import numpy as np
    import mpm3d_gb300 as m
    from mpm3d_gb300 import decks

    rng = np.random.default_rng(0x5E4E)
    gen = [decks.serving_scene(rng) for _ in range(args.serve_scenes)]
    dks = [m.Deck.parse(t) for t, _, _ in gen]
    nps = np.array([n for _, n, _ in gen], dtype=np.float64)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, size=len(dks)))
    out = {"fifo": serve_scenes(args, device, dks, nps, arrivals, "fifo", 0)}
    if args.serve_cap > 0:
        # a resident-particle cap bounds the batch a scene shares the device
        # with: FIFO with the cap bounds the tail, least-work-first with it
        # trades the tail for the median
        out["fifo_capped"] = serve_scenes(args, device, dks, nps, arrivals, "fifo", args.serve_cap)
        out["shortest_capped"] = serve_scenes(args, device, dks, nps, arrivals, "shortest", args.serve_cap)
    target = None
    if args.target_stride > 0:
        target = serving_vs_fp64(args, device, dks, nps, out["fifo"]["particle_steps_per_s"])
    if not args.no_cpu_baseline:
        out["cpu_baseline_per_scene"] = serving_cpu_baseline()
    return out, target


def serving_cpu_baseline(steps: int = 2) -> list:
    """The oracle (the CPU port of the reference step, one core) on serving
    scenes of each kind at 2k, 40k and 400k particles: a bounded sample of
    `steps` timed steps after one untimed step, per scene."""
    import numpy as np
    from mpm3d_gb300 import decks

    out = []
    for kind in ("cook", "beam"):
        for n in (2000, 40000, 400000):
            text, npart, _ = decks.serving_scene(np.random.default_rng(n), n, n, kind=kind)
            cb = cpu_baseline(text, steps, npart)
            out.append({"kind": kind, "particles": npart, "particle_steps_per_s": cb["value"], "cores": 1,
                        "sample": cb["sample"]})
    return out


def serving_vs_fp64(args, device: int, dks, nps, served_rate: float) -> dict:
    """The serving scenes through the plain FP64 forms: every target_stride-th
    scene of the stream, one context per scene, run for the scenes' step
    count (CUDA events, graph replay); the FP64 rate of the scene mix is the
    sampled particle-steps over the summed FP64 time. The same scenes run
    alone in the mixed form (bit-identical to their results in the batch,
    tests/test_gpu_batch.py) give the per-scene error against the FP64 strict
    form after the full step count."""
    import numpy as np
    import mpm3d_gb300 as m

    idx = list(range(0, len(dks), args.target_stride))
    steps = args.serve_steps
    work, t_strict, t_native = 0.0, 0.0, 0.0
    worst = {"nodal_momentum_rel": 0.0, "particle_stress_rel": 0.0, "displacement_rel": 0.0}
    per_scene = []
    t0 = time.perf_counter()
    for k in idx:
        d = dks[k]
        x0 = d.particles()["Xp"]
        f = m.MpmStep(d, precision="fp64", device=device)
        t_strict += f.time_steps(steps, graph=True)
        f.sync()
        ref = {fl: f.download(fl) for fl in ERR_FIELDS}
        f.close()
        nat = m.MpmStep(d, precision="native", device=device)
        t_native += nat.time_steps(steps, graph=True)
        nat.close()
        mx = m.MpmStep(d, precision="mixed", device=device)
        mx.run(steps, graph=True)
        mx.sync()
        got = {fl: mx.download(fl) for fl in ERR_FIELDS}
        mx.close()
        e = form_errors(got, ref, x0)
        per_scene.append([int(nps[k])] + [float("%.3g" % e[q]) for q in worst])
        for q in worst:
            worst[q] = max(worst[q], e[q])
        work += float(nps[k]) * steps
    strict_rate = work / (t_strict / 1e3)
    native_rate = work / (t_native / 1e3)
    fastest = max(strict_rate, native_rate)
    return {"scenes_sampled": len(idx), "of_scenes": len(dks), "stride": args.target_stride, "steps": steps,
            "fp64_strict_particle_steps_per_s": strict_rate, "fp64_native_particle_steps_per_s": native_rate,
            "served_particle_steps_per_s": served_rate, "ratio_served_over_fp64": served_rate / fastest,
            "fp64_form_compared": "fastest of strict / native", "max_error": worst,
            "error_reference": "FP64 strict form, each scene alone",
            "per_scene_np_mom_stress_disp": per_scene, "wall_s": round(time.perf_counter() - t0, 1)}


def serve_scenes(args, device: int, dks, nps, arrivals, policy: str, cap: int) -> dict:
    import numpy as np
    import mpm3d_gb300 as m

    # the device loop returns when a scene finishes, or after at least
    # chunk_steps steps when a submission is waiting
    with m.Server(device=device, chunk_steps=25, autotune=True, policy=policy, max_resident_particles=cap) as srv:
        tickets = []
        t0 = time.perf_counter()
        for k, d in enumerate(dks):
            wait = arrivals[k] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            tickets.append(srv.submit(d, args.serve_steps))
        for t in tickets:
            srv.wait(t)
        wall = time.perf_counter() - t0
        res = [srv.result(t) for t in tickets]
        st = srv.stats()
        shape = srv.launch_shape()
    lat = np.array([r["latency_ms"] for r in res])
    queue = np.array([r["queue_ms"] for r in res])
    return {
        "scenes": len(dks), "steps_per_scene": args.serve_steps, "arrival_rate_per_s": args.serve_rate,
        "policy": policy, "max_resident_particles": cap,
        "particles_min_max_mean": [int(nps.min()), int(nps.max()), float(nps.mean())],
        "p50_latency_ms": float(np.percentile(lat, 50)), "p99_latency_ms": float(np.percentile(lat, 99)),
        "mean_queue_ms": float(queue.mean()), "makespan_s": wall,
        "particle_steps_per_s": float(nps.sum() * args.serve_steps / wall),
        "gpu_busy_frac": st["busy_ms"] / 1e3 / wall, "device_loops": int(st["chunks"]),
        "device_loop": True, "autotuned_launch_shape": shape,
        "peak_resident_bytes": int(st["peak_resident_bytes"]),
    }


def cpu_baseline(text: str, steps: int, npart: int, cores: int = 1) -> dict:
    """The oracle (a port of the reference step) on this host, bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    o = oracle.Oracle(deck_text=text)
    o.run(1)
    t0 = time.perf_counter()
    o.run(steps)
    t = time.perf_counter() - t0
    o.close()
    return {"value": npart * steps / t, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} steps of the full workload ({npart} particles) after 1 untimed step"}


def _replica(args_tuple):
    """One CPU replica of the reference arm: warm-up steps, then up to
    `steps` timed steps, stopping early once `budget_s` seconds are spent."""
    text, warm, steps, budget_s = args_tuple
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    o = oracle.Oracle(deck_text=text)
    o.run(warm)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        o.run(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return time.perf_counter() - t0, o.nb_particle, done, o.nb_gridnode


def run_reference(args) -> dict:
    """Reference arm: the CPU step (oracle port), one replica per host core,
    each running the --warmup / --steps of the workload (bounded: a replica
    stops timing once --ref-budget seconds are spent)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import multiprocessing as mp

    text = make_deck(args.workload, args.scale)
    cores = args.ref_cores or os.cpu_count() or 1
    steps = args.ref_steps or args.steps
    warm = args.ref_warmup if args.ref_warmup >= 0 else args.warmup
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_replica, [(text, warm, steps, args.ref_budget)] * cores)
    t = max(r[0] for r in res)
    npart = res[0][1]
    done = [r[2] for r in res]
    value = npart * sum(done) / t
    return {
        "impl": "reference",
        "metric": "particle-steps/s (mixed precision vs plain FP64 GPU, stated error)",
        "value": value, "unit": "particle-steps/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": min(done), "warmup": warm, "ms_per_step": t / max(1, min(done)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded deck generator)",
        "config": workload_config(args, npart, int(res[0][3]), int(os.environ.get("WORLD_SIZE", "1"))),
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{min(done)}-{max(done)} timed steps per replica (of {steps} asked, "
                                   f"{args.ref_budget:.0f} s budget) after {warm} warm-up steps, "
                                   f"{cores} independent replicas of the full workload"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_run(args) -> None:
    """A few steps of the workload in one form, launched kernel by kernel, for
    ncu captures of single kernels (the timed bench replays graphs)."""
    import mpm3d_gb300 as m

    d = m.Deck.parse(make_deck(args.workload, args.scale))
    s = m.MpmStep(d, precision=args.profile_form, device=0)
    s.run(args.profile_steps, graph=False)
    s.sync()
    print(f"{args.workload} x{args.scale}: {d.nb_particle} particles, {args.profile_steps} {args.profile_form} steps")
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="soil_slope", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=float, default=1.0, help="particle spacing multiplier (1 = full size)")
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 form (large workloads)")
    ap.add_argument("--ref-steps", type=int, default=0, help="reference arm steps (0 = --steps)")
    ap.add_argument("--ref-warmup", type=int, default=-1, help="reference arm warm-up steps (-1 = --warmup)")
    ap.add_argument("--ref-budget", type=float, default=90.0, help="reference arm: seconds of timed steps per replica")
    ap.add_argument("--ref-cores", type=int, default=0)
    ap.add_argument("--serve-scenes", type=int, default=256, help="serving workload scenes (0 = skip)")
    ap.add_argument("--serve-steps", type=int, default=500)
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate (scenes/s)")
    ap.add_argument("--serve-cap", type=int, default=2_000_000,
                    help="resident particle cap of the shortest-work-first serving run (0 = FIFO run only)")
    ap.add_argument("--target-steps", type=int, default=5000,
                    help="mixed-vs-FP64 error after this many steps of the workload (0 = skip)")
    ap.add_argument("--target-stride", type=int, default=8,
                    help="serving scenes also run through the FP64 forms: every n-th scene (0 = skip)")
    ap.add_argument("--profile-form", default="", choices=["", "mixed", "fp64", "native"],
                    help="profiling harness for ncu: only run --profile-steps steps of the workload in this form, "
                         "one kernel launch at a time (no graph), and exit; prints no bench line")
    ap.add_argument("--profile-steps", type=int, default=4)
    args = ap.parse_args()
    if args.profile_form:
        profile_run(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
