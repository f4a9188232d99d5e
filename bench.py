"""Benchmark of tlaloque's hydrodynamic step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl tlq|reference]
                    [--workload wind256|wind128|sedov128|sod|clumpy<N>|cloud128|cloud256|ensemble48]

A "step" is one full iteration of the reference's main loop
(source/mainHD.f90:74-99: CFL dt, two HLLC stages, ghost fill, winds, point
gravity, artificial viscosity, cooling) over the whole mesh.  The metric is
zone-updates/s = interior cells x steps / time.

* value      device-resident, headline form (mixed precision + the learned
             cooling surrogate when the workload cools, else mixed): K steps
             through the C ABI (tlq_advance with per-kernel CUDA events) with
             the state already in HBM, timed with CUDA events on the
             library's stream; `forms` holds the plain FP64 form and the
             mixed form measured the same way, the speed-ups, and each form's
             relative L1 density error and total-energy drift against FP64
             after W+K steps (the surrogate against FP64 with the exact
             integrator it falls back to); `surrogate` its training and
             fallback rate (the network is trained on the GPU first), and
             `surrogate.active` the same forms on the clumpy medium, where
             the network cools a quarter of a million cells a step;
* ensemble   (wind256) the 48-member ensemble in the batched persistent
             form for --ens-steps steps, against its members one after
             another (same form; plain FP64 with the exact integrator);
* e2e        the same metric end to end through the C ABI with host
             buffers: per step tlq_upload (pinned host -> device + layout
             conversion + calc_prims/dt), tlq_step, tlq_download;
* roofline   the dominant kernel's algorithmic bytes per launch / its
             average CUDA-event duration, against the measured HBM peak;
* cpu_baseline  the oracle restatement on the host cores (bounded sample).

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement: the Fortran reference has no compiler on this pool) on
all host cores, same workload and metric.  With N > 1 ranks (torchrun) each
rank advances an independent replica of the workload (the step has no data
path shared between meshes); value = all ranks' zone-updates / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "zone-updates/s on 1 GB300 at 256³ (mixed+surrogate vs plain FP64 at ≤1% L1 err); HBM GB/s"
UNIT = "zone-updates/s"

# FP64 operations per zone-update of the reference algorithm by kind,
# counted by the oracle's counting build at each workload's size (one step
# after the first): python -m oracle.flops_report --wind-n 256 --sedov-n 128.
# cmp: comparisons (DSETP, issued on the FP64 pipe like an add).
FP64_OPS_PER_ZONE = {
    "wind256": {"add": 475.28, "mul": 442.29, "div": 89.98, "sqrt": 15.24, "cmp": 71.93},
    "sedov128": {"add": 386.23, "mul": 322.22, "div": 52.77, "sqrt": 13.28, "cmp": 66.61},
    "sod": {"add": 560.05, "mul": 648.96, "div": 109.46, "sqrt": 19.82, "cmp": 95.83},
}


def fp64_pipe_bound(ops: dict, rate: dict) -> dict:
    """The plain FP64 step's compute roofline from the op counts and the FP64
    pipe's measured rates (tlq_measure_fp64_rate): every add, multiply and
    comparison takes one FMA slot (the FP64 kernels are built without
    contraction), an IEEE division or square root the FMA-slot cost measured
    for it; zone-updates/s at a fully busy pipe = FMA rate / slots."""
    div_cost = rate["fma_per_s"] / rate["div_per_s"]
    sqrt_cost = rate["fma_per_s"] / rate["sqrt_per_s"]
    slots = ops["add"] + ops["mul"] + ops["cmp"] + ops["div"] * div_cost + ops["sqrt"] * sqrt_cost
    return {"fma_slots_per_zone": slots, "div_fma_slots": div_cost, "sqrt_fma_slots": sqrt_cost,
            "zone_updates_per_s_bound": rate["fma_per_s"] / slots}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def make_workload(name: str):
    from tlaloque_gb300 import problems, tlq
    if name == "wind256":
        cfg, U0 = problems.wind_bubble(256)
        desc = ("radiative wind-blown bubble 256^3, (8 pc)^3 box, HLLC + van Leer, spherical wind (R = 4 dx, "
                "1e-6 Msun/yr, 2000 km/s), 10 Msun point mass, sub-cycled tabulated cooling, outflow")
    elif name == "wind128":
        cfg, U0 = problems.wind_bubble(128)
        desc = "radiative wind-blown bubble 128^3 (the 256^3 workload at half resolution)"
    elif name == "sedov128":
        cfg, U0 = problems.sedov(128)
        desc = "3-D Sedov-Taylor blast 128^3, HLLC + van Leer, outflow"
    elif name.startswith("clumpy") and name[6:].isdigit():
        n = int(name[6:])
        cfg, U0 = problems.clumpy(n)
        desc = (f"clumpy radiative medium {n}^3, periodic (8 pc)^3, lognormal density (sigma ln n = 1, mean "
                "1 cm^-3, k^-5/3), log T uniform 1e3-1e8 K, rms Mach 2, HLLC + van Leer, sub-cycled tabulated "
                "cooling")
    elif name == "sod":
        cfg, U0 = problems.sod_tube()
        desc = "Sod shock tube 256x4x4, HLL, gamma 1.4, outflow"
    elif name in ("cloud128", "cloud256"):
        n = int(name[5:])
        cfg, U0 = problems.gravitating_cloud(n)
        desc = (f"self-gravitating cloud {n}^3 (the reference's -DGRAV MultiGrid before each stage, multipole faces "
                "every 10 steps): (4 pc)^3, 1 pc sphere n = 500 cm^-3, T = 50 K, pressure-matched medium 100x "
                "thinner, HLLC + van Leer, outflow")
    else:
        raise SystemExit(f"unknown workload {name}")
    return cfg, U0, desc


def bytes_per_zone(cfg, mixed: bool = False) -> dict:
    """HBM bytes per zone-update of each stage kernel.  "alg": the scheme's
    compulsory state traffic -- stage 1 reads U (40 B FP64) and writes UPP,
    stage 2 reads UPP and U and writes the new U; UPP is FP32 (20 B) in the
    mixed form, FP64 (40 B) in the plain one; point gravity reads the
    potential (8 B) in each stage.  "moved": what the kernels must move on top
    of that: the mixed form's viscosity term, eta Lap(U), formed by stage 1
    from the U planes it streams and read by stage 2 (FP32, 20 B each way);
    the plain form's carried cooled pressure (8 B each way).  Ghost and halo
    re-reads are not counted (they lower the achieved fraction).  With the
    surrogate the cooling passes read and write only the cells stage 2 queued
    (those cooling beyond a single step): their bytes scale with those cells,
    not with the mesh, and are not counted per zone-update."""
    from tlaloque_gb300 import tlq
    grav = 8 if ((cfg.masses is not None and len(cfg.masses) > 0) or getattr(cfg, "self_gravity", 0)) else 0
    upp = 20 if mixed else 40
    alg = {"stage1": 40 + upp + grav, "stage2": upp + 40 + 40 + grav}
    extra = 20 if mixed else (8 if cfg.cooling != tlq.COOL_NONE else 0)
    moved = {k: v + extra for k, v in alg.items()}
    return {"alg": {**alg, "step": alg["stage1"] + alg["stage2"]},
            "moved": {**moved, "step": moved["stage1"] + moved["stage2"]}}


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region.
    start() returns once the first sample has arrived (nvidia-smi takes a
    few hundred ms to start), so the sampler is already running when timing
    begins; begin()/end() bracket the timed region on the host clock and
    stop() summarises the samples that arrived inside it."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None
        self.first = threading.Event()
        self.t0 = self.t1 = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        self.first.wait(timeout=5.0)
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.monotonic(), parts))
                self.first.set()

    def begin(self):
        self.t0 = time.monotonic()

    def end(self):
        self.t1 = time.monotonic()

    def stop(self):
        if self.t1 is None:
            self.end()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        t0 = self.t0 if self.t0 is not None else float("-inf")
        inside = [s for t, s in self.samples if t0 <= t <= self.t1]
        where = "timed region"
        if not inside and self.samples:
            # the region was shorter than the sampling interval: the sample closest to it
            mid = 0.5 * (t0 + self.t1) if self.t0 is not None else self.t1
            inside = [min(self.samples, key=lambda ts: abs(ts[0] - mid))[1]]
            where = "nearest sample to the timed region (shorter than the sampling interval)"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in inside if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in inside if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for s in inside for q in range(4) if s[5 + q].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "sampled": where,
                "region_s": round(self.t1 - t0, 4) if self.t0 is not None else None}


# ---------------------------------------------------------------------------
def cpu_oracle_rate(cfg, U0, budget_s: float, nthreads: int, min_steps: int = 2, max_steps: int = 10 ** 6,
                    warm: int = 1):
    """Time the oracle restatement on the host: zone-updates/s over a bounded
    number of steps of the same workload (steps until budget_s elapses)."""
    from oracle.oracle import Run
    from oracle.oracle import params_from_config as oracle_params
    run = Run(oracle_params(cfg, nthreads=nthreads), U0)
    run.run(warm)  # first touch of the arrays (and the workload's first, heavier step)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        run.run(1)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= min_steps and el >= budget_s:
            break
    el = time.perf_counter() - t0
    return cfg.cells * steps / el, steps, el


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local, dist


def allmax(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def ensemble_members(n: int = 48, seed: int = 2024):
    """The ensemble workload: n wind bubbles, sizes uniform from
    {48, 64, 96, 128}^3, wind speed log-uniform in 500-3000 km/s, ambient
    density log-uniform in 0.1-10 cm^-3 (seeded); mixed precision with the
    learned cooling surrogate (exact-integrator fallback)."""
    from tlaloque_gb300 import problems, tlq
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        size = int(rng.choice([48, 64, 96, 128]))
        vw = float(np.exp(rng.uniform(np.log(500.0), np.log(3000.0))))
        namb = float(np.exp(rng.uniform(np.log(0.1), np.log(10.0))))
        cfg, U0 = problems.wind_bubble(size, vw_kms=vw, n_amb=namb)
        cfg = tlq.Config(**{**cfg.__dict__, "precision": tlq.PREC_MIXED, "cooling": tlq.COOL_MLP,
                            "cool_sub_frac": 2e-3})
        out.append((cfg, U0))
    return out


def ensemble_record(steps, warmup, net, world, dist):
    """The ensemble's 48 wind bubbles advanced by the batched persistent step
    (one launch per stage over all members' tiles, graph-replayed step,
    z-chunks from the autotuner) for `steps` timed steps after `warmup`,
    against the same members stepped one context after another, in the same
    form and in plain FP64 with the exact cooling integrator.  net: the
    cooling surrogate's weights (the members share the table and physics)."""
    import tempfile

    from tlaloque_gb300 import tlq
    members = ensemble_members()
    cells = sum(c.cells for c, _ in members)
    b = tlq.Batch([c for c, _ in members])
    for m, (cfg, U0) in zip(b.members, members):
        m.set_cooling_surrogate(*net)
        U1 = U0.copy(order="F")
        m.borders(U1, 1)
        m.upload(U1)
    cache = os.path.join(tempfile.gettempdir(), "tlq_autotune.json")
    t0 = time.perf_counter()
    chosen = b.autotune(cache, steps=3)
    tune_s = time.perf_counter() - t0
    b.run(warmup)
    b.synchronize()
    barrier(dist)
    b.enable_timing(True)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))).start()
    sampler.begin()
    b.run(steps)
    b.synchronize()
    sampler.end()
    clocks = sampler.stop()
    st = b.stats()
    ms = allmax(dist, st.ms_per_step * steps)
    status = b.status()
    b.close()

    def one_after_another(over, with_net):
        tot = 0.0
        for cfg, U0 in members:
            with tlq.Context(tlq.Config(**{**cfg.__dict__, **over})) as ctx:
                if with_net:
                    ctx.set_cooling_surrogate(*net)
                U1 = U0.copy(order="F")
                ctx.borders(U1, 1)
                ctx.upload(U1)
                ctx.advance(warmup)
                ctx.enable_timing(True)
                ctx.advance(steps)
                s = ctx.stats()
                tot += (s.ms_stage1 + s.ms_stage2 + s.ms_cool) * steps
        return tot
    seq_ms = one_after_another({}, True)  # per-member graphs, the same form
    # what the reference computes: plain FP64 with the exact integrator
    seq64_ms = one_after_another({"precision": tlq.PREC_FP64, "cooling": tlq.COOL_EXACT}, False)
    return {"value": world * cells * steps / (ms / 1e3), "unit": UNIT, "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "cells": cells, "members": len(members), "items": st.items,
            "persistent_blocks": st.blocks, "zlen_chosen": sorted(set(chosen)), "autotune_s": tune_s,
            "members_failed": int(sum(1 for x in status if x != 0)),
            "sequential": {"value": cells * steps / (seq_ms / 1e3), "ms_per_step": seq_ms / steps,
                           "path": "each member alone, its own graph-replayed step, one after another"},
            "speedup_vs_sequential": seq_ms / ms,
            "sequential_fp64": {"value": cells * steps / (seq64_ms / 1e3), "ms_per_step": seq64_ms / steps,
                                "path": "each member alone in the plain FP64 form with the exact cooling "
                                        "integrator (closed form), one after another"},
            "speedup_vs_sequential_fp64": seq64_ms / ms,
            "gpu_launches": st.launches_per_step * steps, "clocks": clocks}


ENSEMBLE_WORKLOAD = ("ensemble of 48 wind bubbles, sizes uniform from {48,64,96,128}^3, v_w log-uniform "
                     "500-3000 km/s, n log-uniform 0.1-10 cm^-3, mixed precision + learned cooling surrogate")


def run_ensemble(args, world, rank, dist):
    """The ensemble workload as the bench's own line (--workload ensemble48)."""
    import torch
    from tlaloque_gb300 import build as tbuild
    from tlaloque_gb300 import tlq
    tbuild.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    members = ensemble_members()
    with tlq.Context(members[0][0]) as tctx:  # one network: the members share the cooling table and physics
        rep = tctx.train_cooling_surrogate(nsamples=args.train_samples, epochs=args.train_epochs)
        net = tctx.get_cooling_surrogate()
    r = ensemble_record(args.steps, args.warmup, net, world, dist)
    line = {"metric": "zone-updates/s of a 48-member wind-bubble ensemble on 1 GB300 (batched persistent step)",
            "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": ENSEMBLE_WORKLOAD, "surrogate_training_ms": rep["ms_generate"] + rep["ms_train"],
                       "cells": r["cells"], "members": r["members"], "items": r["items"],
                       "persistent_blocks": r["persistent_blocks"], "zlen_chosen": r["zlen_chosen"],
                       "autotune_s": r["autotune_s"], "l2": "the members' state (~6 GB) exceeds L2"},
            **{k: r[k] for k in ("members_failed", "sequential", "speedup_vs_sequential", "sequential_fp64",
                                 "speedup_vs_sequential_fp64", "gpu_launches", "clocks")}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_reference(args, world, rank, dist):
    """The reference algorithm on the host cores (oracle restatement)."""
    if rank != 0:
        return
    cfg, U0, desc = make_workload(args.workload)
    ncores = os.cpu_count() or 1
    from oracle.oracle import Run
    from oracle.oracle import params_from_config as oracle_params
    run = Run(oracle_params(cfg, nthreads=ncores), U0)
    run.run(args.warmup)
    t0 = time.perf_counter()
    run.run(args.steps)
    el = time.perf_counter() - t0
    value = cfg.cells * args.steps / el
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "mesh": [cfg.nx, cfg.ny, cfg.nz], "parallelism": "replicas"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                         "sample": f"{args.steps} full steps of the workload after {args.warmup} warm-up steps "
                                   f"(oracle restatement, OpenMP over {ncores} host threads; the Fortran reference "
                                   "cannot be compiled on this pool: no Fortran compiler)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tlq", choices=["tlq", "reference"])
    ap.add_argument("--workload", default="wind256")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--train-samples", type=int, default=20_000_000, help="surrogate training pairs")
    ap.add_argument("--train-epochs", type=int, default=30, help="surrogate training epochs")
    ap.add_argument("--clumpy-n", type=int, default=256, help="mesh of the surrogate-active record")
    ap.add_argument("--sur-steps", type=int, default=100, help="timed steps of the surrogate-active record")
    ap.add_argument("--no-surrogate-active", action="store_true")
    ap.add_argument("--ens-steps", type=int, default=10, help="timed steps of the ensemble record")
    ap.add_argument("--no-ensemble", action="store_true", help="leave out the ensemble record")
    ap.add_argument("--sur-tol", type=float, default=1e-3, help="residual tolerance of the surrogate-active record")
    ap.add_argument("--mlp-tol", type=float, default=1e-3, help="residual tolerance of the workload's surrogate form")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        barrier(dist)
        return
    if args.workload == "ensemble48":
        run_ensemble(args, world, rank, dist)
        barrier(dist)
        return

    import torch
    from tlaloque_gb300 import build as tbuild
    from tlaloque_gb300 import problems, tlq
    tbuild.build()
    torch.cuda.set_device(local)
    cfg, U0, desc = make_workload(args.workload)
    cfg.device = local
    peak, peak_kind = load_peaks()
    stream = torch.cuda.Stream()
    forms = {}
    ensemble = None
    import tempfile
    tune_cache = os.path.join(tempfile.gettempdir(), "tlq_autotune.json")

    def measure(precision, steps, sample_clocks, net=None, base=None, tune=True, **over):
        """W warm-up + K timed steps of one form from the initial state of the
        workload (base: another workload's (cfg, U0))."""
        bcfg, bU0 = base if base is not None else (cfg, U0)
        c = tlq.Config(**{**bcfg.__dict__, "precision": precision, **over})
        ctx = tlq.Context(c)
        ctx.set_stream(stream.cuda_stream)
        if net is not None:
            ctx.set_cooling_surrogate(*net)
        U1 = bU0.copy(order="F")
        ctx.borders(U1, 1)          # mainHD.f90:38
        ctx.upload(U1)
        # z-chunk of the stage grid (state restored)
        zlen = ctx.autotune(tune_cache, steps=3) if tune else ctx.tiling()
        ctx.advance(args.warmup)    # warm-up (builds the CUDA graphs)
        ctx.synchronize()
        st0 = ctx.stats()
        sampler = ClockSampler(local).start() if sample_clocks else None
        ctx.enable_timing(True)
        barrier(dist)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if sampler:
            sampler.begin()
        with torch.cuda.stream(stream):
            e0.record(stream)
            ctx.advance(steps)
            e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.end()
        barrier(dist)
        ms = e0.elapsed_time(e1)
        clocks = sampler.stop() if sampler else None
        st = ctx.stats()
        ctx.enable_timing(False)
        t_sim, it_sim, dt_sim, status = ctx.time()
        W = bcfg.zeros()
        ctx.download(None, W)
        sums = ctx.conserved_sums()
        ms_max = allmax(dist, ms)
        return {"ctx": ctx, "ms": ms_max, "value": world * bcfg.cells * steps / (ms_max / 1e3), "k1": st.ms_stage1,
                "k2": st.ms_stage2, "kc": st.ms_cool, "kg": st.ms_grav, "sim": {"t": t_sim, "it": it_sim, "dt": dt_sim, "status": status},
                "rho": W[0, 2:-2, 2:-2, 2:-2].copy(), "E": float(sums[4]), "clocks": clocks,
                "cool": (st.cool_mlp - st0.cool_mlp, st.cool_fallback - st0.cool_fallback,
                         st.cool_single - st0.cool_single), "zlen": zlen}

    def form(m):
        d = {"value": m["value"], "ms_per_step": m["ms"] / args.steps, "ms_stage1": m["k1"], "ms_stage2": m["k2"],
             "zlen": m["zlen"]}
        if m["kc"] > 0:
            d["ms_cool_passes"] = m["kc"]
        if m["kg"] > 0:
            d["ms_multigrid"] = m["kg"]  # both solves of a step (ms_stage1/2: the stage kernels alone)
        return d

    def accuracy(a, b):
        """a against b after the same W+K steps: relative L1 density error and
        total-energy drift scaled to 100 steps."""
        nst = args.warmup + args.steps
        return {"after_steps": nst, "l1_rho_rel": float(np.sum(np.abs(a["rho"] - b["rho"])) / np.sum(np.abs(b["rho"]))),
                "energy_drift_rel_per_100_steps": abs(a["E"] - b["E"]) / abs(b["E"]) * (100.0 / nst)}

    def surrogate_active(net, sub):
        """The surrogate doing real work: a clumpy radiative medium (lognormal
        density, log T uniform over 1e3-1e8 K, rms Mach 2; the wind bubble's
        cooling curve and physics, so the same network) where a few per cent
        of the cells cool stiffly every step.  W warm-up + S timed steps of
        mixed + surrogate, of the mixed form with the exact integrator's
        closed form alone, and of the judge (plain FP64, exact integrator);
        accuracy after the W + S steps."""
        ccfg, cU0 = problems.clumpy(args.clumpy_n)
        nst = args.sur_steps
        judge = measure(tlq.PREC_FP64, nst, False, base=(ccfg, cU0), tune=False, cooling=tlq.COOL_EXACT, **sub)
        judge["ctx"].close()
        closed = measure(tlq.PREC_MIXED, nst, False, base=(ccfg, cU0), cooling=tlq.COOL_EXACT, **sub)
        closed["ctx"].close()
        act = measure(tlq.PREC_MIXED, nst, False, net=net, base=(ccfg, cU0), cooling=tlq.COOL_MLP,
                      cool_mlp_tol=args.sur_tol, **sub)
        act["ctx"].close()

        def acc(a):
            n_all = args.warmup + nst
            return {"after_steps": n_all,
                    "l1_rho_rel": float(np.sum(np.abs(a["rho"] - judge["rho"])) / np.sum(np.abs(judge["rho"]))),
                    "energy_drift_rel_per_100_steps": abs(a["E"] - judge["E"]) / abs(judge["E"]) * (100.0 / n_all)}
        nm, nf, ns = act["cool"]
        return {"workload": f"clumpy radiative medium {args.clumpy_n}^3, periodic (8 pc)^3, lognormal density "
                            "(sigma ln n = 1, mean 1 cm^-3, k^-5/3), log T uniform 1e3-1e8 K, rms Mach 2, the wind bubble's "
                            "cooling curve; HLLC + van Leer",
                "mesh": [ccfg.nx, ccfg.ny, ccfg.nz], "warmup": args.warmup, "steps": nst,
                "cool_mlp_tol": args.sur_tol,
                "tol_note": "the residual tolerance of an accepted prediction, |T_pred - T_exact| / T (the north "
                            "star's a-posteriori check at 1e-3)",
                "value": act["value"], "unit": UNIT, "ms_per_step": act["ms"] / nst, "ms_stage1": act["k1"],
                "ms_stage2": act["k2"], "ms_cool_passes": act["kc"],
                "timed_cell_steps_network": nm, "timed_cell_steps_exact": nf, "timed_cell_steps_single_step": ns,
                "network_cells_per_step": nm / nst, "fallback_rate": nf / max(1, nm + nf),
                "vs_fp64_exact": acc(act),
                "fp64_exact": {"value": judge["value"], "ms_per_step": judge["ms"] / nst},
                "speedup_vs_fp64_exact": act["value"] / judge["value"],
                "mixed_exact_closed_form": {"value": closed["value"], "ms_per_step": closed["ms"] / nst,
                                            "ms_cool_in_stage2": closed["k2"], "vs_fp64_exact": acc(closed)}}

    cooling = cfg.cooling != tlq.COOL_NONE
    f64 = measure(tlq.PREC_FP64, args.steps, False)
    f64["ctx"].close()
    mix = measure(tlq.PREC_MIXED, args.steps, not cooling)
    forms = {"fp64": form(f64), "mixed": form(mix), "speedup_mixed_vs_fp64": mix["value"] / f64["value"],
             "mixed_vs_fp64": accuracy(mix, f64)}
    # the plain form's bound: the FP64 pipe (measured here, with the oracle's
    # op counts) next to its HBM fraction
    bpz64 = bytes_per_zone(cfg)["alg"]
    forms["fp64"]["roofline"] = {
        "hbm_achieved_gbs": bpz64["step"] * f64["value"] / 1e9,
        "hbm_frac": bpz64["step"] * f64["value"] / 1e9 / peak}
    ops = FP64_OPS_PER_ZONE.get(args.workload)
    if ops:
        rate = tlq.measure_fp64_rate(local)
        b = fp64_pipe_bound(ops, rate)
        forms["fp64"]["roofline"].update({
            "bound": "fp64 pipe", "fp64_ops_per_zone": ops,
            "fp64_rate_measured": {**rate, "how": "tlq_measure_fp64_rate: independent FMA / IEEE divide / IEEE "
                                                 "square-root chains, 8 blocks of 256 threads per SM, CUDA events"},
            **b, "fp64_pipe_frac": f64["value"] / b["zone_updates_per_s_bound"]})
    head = mix
    surrogate = None
    if cooling:
        # the learned cooling surrogate: trained here on the GPU for this
        # workload's cooling table and physics; its fallback (and the FP64
        # step it is compared with) is the exact integrator, fine sub-cycling
        mix["ctx"].close()
        # the judge: the exact integrator (the reference's single exponential
        # step up to a cooling number of 2e-3, the closed form above it)
        sub = {"cool_sub_frac": 2e-3}
        with tlq.Context(cfg) as tctx:
            rep = tctx.train_cooling_surrogate(nsamples=args.train_samples, epochs=args.train_epochs)
            net = tctx.get_cooling_surrogate()
        f64x = measure(tlq.PREC_FP64, args.steps, False, cooling=tlq.COOL_EXACT, **sub)
        f64x["ctx"].close()
        sur = measure(tlq.PREC_MIXED, args.steps, True, net=net, cooling=tlq.COOL_MLP, cool_mlp_tol=args.mlp_tol,
                      **sub)
        nm, nf, ns = sur["cool"]
        forms["fp64_exact_cooling"] = form(f64x)
        forms["mixed_surrogate"] = form(sur)
        forms["speedup_mixed_surrogate_vs_fp64"] = sur["value"] / f64["value"]
        forms["mixed_surrogate_vs_fp64_exact_cooling"] = accuracy(sur, f64x)
        surrogate = {"train": {k: rep[k] for k in ("ms_generate", "ms_train", "steps", "val_accept", "val_p99_rel_T",
                                                    "val_rmse_y")},
                     "cool_mlp_tol": args.mlp_tol,
                     "timed_cell_steps_network": nm, "timed_cell_steps_fallback": nf,
                     "timed_cell_steps_single_step": ns,
                     "fallback_rate": nf / max(1, nm + nf),
                     "fallback_note": "of the cooling cell-steps with tau above the single-step limit (the "
                                      "network's domain), the share cooled by the exact integrator: outside the "
                                      "training box or failing the residual check; cells with smaller tau take "
                                      "the exact integrator's single exponential step directly (single_step)"}
        head = sur
        if not args.no_surrogate_active:
            surrogate["active"] = surrogate_active(net, sub)
        if not args.no_ensemble and args.workload == "wind256":
            # the batched form on the ensemble workload (its own line: --workload ensemble48)
            ensemble = {"workload": ENSEMBLE_WORKLOAD, **ensemble_record(args.ens_steps, args.warmup, net, world,
                                                                          dist)}
    value = head["value"]
    ms_max = head["ms"]
    mix = head

    k1, k2 = mix["k1"], mix["k2"]
    dom = "stage2" if k2 >= k1 else "stage1"
    kms = max(k1, k2)
    bpz = bytes_per_zone(cfg, mixed=True)
    bpz_m = bpz["alg"]
    achieved = bpz_m[dom] * cfg.cells / (kms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": f"stage_kernel_mixed<{2 if dom == 'stage2' else 1}>",
                "ms_cool_passes": mix["kc"],
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)" if peak_kind == "measured"
                else peak_kind,
                "traffic": None, "bytes_per_zone": bpz_m, "bytes_per_zone_moved": bpz["moved"],
                "achieved_moved": bpz["moved"][dom] * cfg.cells / (kms / 1e3) / 1e9,
                "ms_stage1": k1, "ms_stage2": k2}
    if mix["kg"] > 0:
        roofline["ms_multigrid"] = mix["kg"]
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tr = json.load(f).get(args.workload, {}).get("mixed_" + dom)
            if tr:
                roofline["traffic"] = tr["bytes_per_launch"] * cfg.cells / tr["cells"]
    except Exception:
        pass

    # ---- end to end through the C ABI with pinned host buffers -------------
    ctx = mix["ctx"]
    host = torch.empty((cfg.nz + 4, cfg.ny + 4, cfg.nx + 4, 5), dtype=torch.float64, pin_memory=True)
    Uh = host.numpy().transpose(3, 2, 1, 0)
    ctx.download(Uh, None)
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        ctx.upload(Uh)
        ctx.step()
        ctx.download(Uh, None)
    el = time.perf_counter() - t0
    barrier(dist)
    el = allmax(dist, el)
    e2e = {"value": world * cfg.cells * args.e2e_steps / el, "unit": UNIT,
           "h2d_bytes_per_step": int(Uh.nbytes), "d2h_bytes_per_step": int(Uh.nbytes),
           "ms_per_step": 1e3 * el / args.e2e_steps,
           "path": "tlq_upload(pinned host U) + tlq_step + tlq_download(U) per step, "
                   + ("mixed + surrogate form" if surrogate else "mixed form")}
    ctx.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": desc, "mesh": [cfg.nx, cfg.ny, cfg.nz],
                   "form": ("mixed + learned cooling surrogate (BF16 tensor-core MLP, exact-integrator fallback): "
                            if surrogate else "mixed: ")
                           + "FP32 reconstruction, Riemann fluxes, sources; FP64 state, "
                             "accumulation, high-Mach pressure recovery and dt",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (each state array 0.7 GB; 3 arrays touched per step)",
                   "sim": mix["sim"]},
        "forms": forms, "surrogate": surrogate, "e2e": e2e, "roofline": roofline, "clocks": mix["clocks"],
        "gpu_launches": (5 if surrogate else 2) * args.steps,
        "hbm_gbs_step": bpz_m["step"] * cfg.cells * args.steps / (ms_max / 1e3) / 1e9,
    }
    if ensemble is not None:
        line["ensemble"] = ensemble
    if rank == 0 and not args.no_cpu_baseline:
        ncores = os.cpu_count() or 1
        rate, steps, secs = cpu_oracle_rate(cfg, U0, args.cpu_budget, ncores)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": ncores, "kind": "port",
                                "sample": f"{steps} full steps of the same workload ({secs:.1f} s) on the oracle "
                                          f"restatement, OpenMP over {ncores} host threads"}
        # the same restatement on one core (the reference itself is serial)
        rate1, steps1, secs1 = cpu_oracle_rate(cfg, U0, 0.0, 1, min_steps=1)
        line["cpu_baseline"]["serial"] = {"value": rate1, "unit": UNIT, "cores": 1,
                                          "sample": f"{steps1} full step ({secs1:.1f} s) after one warm-up step"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
