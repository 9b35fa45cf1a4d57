#!/usr/bin/env python
"""Benchmark: SSA reaction events/s of the dimerization ensemble on one GB300.

A step is one pass of the direct method over the whole ensemble: 1e5
independent dimerization trajectories (gene, mRNA, protein, dimer; x0 =
(1, 0, 0, 0); rates 25, 1000, 0.001, 0.1, 1; tmax = 1, 101 regular samples),
about 1.7e9 reaction events.  ``value`` times the kernel on HBM-resident
inputs (CUDA events on the launching stream, L2 flushed between steps);
``e2e`` times the C-ABI host call ``rb_ensemble_run`` from page-locked host
buffers, copies included.  ``--impl reference`` times the CPU restatement of
the reference on all host cores instead.  Under torchrun each rank simulates
its own 1e5 trajectories (weak scaling; seeds keyed by global trajectory id).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DIMER = dict(
    name="dimer",
    desc=("dimerization ensemble: gene,mRNA,protein,dimer x0=(1,0,0,0); G->G+M 25, M->M+P 1000, "
          "2P->D 0.001, M->0 0.1, P->0 1; tmax=1.0, nb_steps=100"),
    S=4,
    reactions=[(25.0, [1, 0, 0, 0], [0, 1, 0, 0]), (1000.0, [0, 1, 0, 0], [0, 0, 1, 0]),
               (0.001, [0, 0, 2, 0], [0, 0, -2, 1]), (0.1, [0, 1, 0, 0], [0, -1, 0, 0]),
               (1.0, [0, 0, 1, 0], [0, 0, -1, 0])],
    x0=[1, 0, 0, 0], tmax=1.0, nb_steps=100, n_traj=100_000, cpu_sample=20_000,
)
SIR = dict(
    name="sir",
    desc="SIR: S,I,R x0=(999,1,0); S+I->2I 1e-4, I->R 0.01; tmax=250, nb_steps=250",
    S=3,
    reactions=[(1e-4, [1, 1, 0], [-1, 1, 0]), (0.01, [0, 1, 0], [0, -1, 1])],
    x0=[999, 1, 0], tmax=250.0, nb_steps=250, n_traj=10_000, cpu_sample=10_000,
)


def random_network(seed: int, S: int, R: int, rate_lo: float = 1e-4, rate_hi: float = 1e1, x0_mean: float = 200.0):
    """Random mass-action network that keeps its activity: reactions take 0-2
    reactant molecules (order <= 2) and mostly give back as many product
    molecules (conversions A -> B, exchanges A + B -> C + D), with a few
    inflows, degradations and bindings, so stoichiometries stay in {-2..2};
    rate constants log-uniform in [rate_lo, rate_hi]; counts Poisson(x0_mean)."""
    rng = np.random.default_rng(seed)
    reactions = []
    for _ in range(R):
        order = int(rng.choice([0, 1, 2], p=[0.05, 0.5, 0.45]))
        if order == 0:
            n_prod = 1
        elif order == 1:
            n_prod = 1 if rng.random() < 0.9 else 0
        else:
            n_prod = 2 if rng.random() < 0.9 else 1
        exps = [0] * S
        diff = [0] * S
        for sp in rng.integers(0, S, size=order):
            exps[int(sp)] += 1
            diff[int(sp)] -= 1
        for sp in rng.integers(0, S, size=n_prod):
            diff[int(sp)] += 1
        k = float(np.exp(rng.uniform(np.log(rate_lo), np.log(rate_hi))))
        reactions.append((k, exps, diff))
    x0 = rng.poisson(x0_mean, size=S).astype(np.int64).tolist()
    return reactions, x0


_LR, _LX0 = random_network(20260104, 200, 1000)
LARGE = dict(
    name="large",
    desc=("large random mass-action network: 200 species, 1000 reactions, reactant order <= 2, rates "
          "log-uniform in [1e-4, 1e1], x0 ~ Poisson(200) (seed 20260104); one warp per trajectory; "
          "tmax = 1.5 (~1e5 events per trajectory), nb_steps = 100"),
    S=200, reactions=_LR, x0=_LX0, tmax=1.5, nb_steps=100, n_traj=10_000, cpu_sample=32, sparse=True,
)


def vilar_workload() -> dict:
    """The reference's Vilar oscillator benchmark (benchmarks/benches/vilar/vilar.py:1-41),
    read from the committed golden extract: 9 species in the order the run-time API
    names them (first appearance), 16 mass-action reactions, x0 Da = Dr = 1,
    tmax 200, nb_steps 200.  The reference times 100 trajectories of it."""
    d = json.loads((ROOT / "tests/golden/reference_goldens.json").read_text())["vilar"]
    names: list[str] = []
    for r in d["reactions"]:
        for s in r["reactants"] + r["products"]:
            if s not in names:
                names.append(s)
    reactions = []
    for r in d["reactions"]:
        e = [r["reactants"].count(s) for s in names]
        reactions.append((r["rate"], e, [r["products"].count(s) - x for s, x in zip(names, e)]))
    run = d["run"]
    return dict(
        name="vilar",
        desc=(f"Vilar oscillator ({len(names)} species, {len(reactions)} reactions, parameters of the "
              f"reference benchmark), x0 Da=Dr=1, tmax={run['tmax']:g}, nb_steps={run['nb_steps']}"),
        S=len(names), species=names, reactions=reactions,
        x0=[run["init"].get(s, 0) for s in names], tmax=run["tmax"], nb_steps=run["nb_steps"],
        n_traj=65_536, cpu_sample=256, calib_n=run["n_traj"],
        # published wall time of the reference's own 100-trajectory run (rebopy, run-time API)
        calib_published_s=5.811,
    )


VILAR = vilar_workload()
WORKLOADS = {"dimer": DIMER, "sir": SIR, "large": LARGE, "vilar": VILAR}

BATCH = dict(
    name="batch",
    desc=("heterogeneous batch in one CUDA graph around one persistent launch: 4096 Michaelis-Menten sets (E+S<->ES->E+P, rates log-uniform "
          "in [1e-3, 1e1], E0 ~ U[10, 100], S0 ~ U[100, 1000], tmax 1) and 1024 random mass-action networks "
          "(8-64 species, 16-256 reactions, order <= 2, stoichiometry in {-2..2}, counts ~ U[0, 500], tmax 1e-3); "
          "64 trajectories each, nb_steps 100 (seed 20260105)"),
    n_mm=4096, n_rand=1024, traj=64, nb_steps=100, tmax_mm=1.0, tmax_rand=1e-3, cpu_every=64,
)
MM_REACTIONS = [([1, 1, 0, 0], [-1, -1, 1, 0]), ([0, 0, 1, 0], [1, 1, -1, 0]), ([0, 0, 1, 0], [1, 0, -1, 1])]


def batch_items(seed: int = 20260105):
    """Items of the heterogeneous batch: ("mm", rates, x0) and ("rand", reactions, x0)."""
    rng = np.random.default_rng(seed)
    items = []
    for _ in range(BATCH["n_mm"]):
        rates = np.exp(rng.uniform(np.log(1e-3), np.log(1e1), 3))
        items.append(("mm", rates, [int(rng.integers(10, 101)), int(rng.integers(100, 1001)), 0, 0]))
    for k in range(BATCH["n_rand"]):
        S, R = int(rng.integers(8, 65)), int(rng.integers(16, 257))
        reactions, _ = random_network(seed * 7919 + k, S, R)
        items.append(("rand", reactions, rng.integers(0, 501, size=S).tolist()))
    return items


def batch_seeds(step: int, j: int) -> np.ndarray:
    """Seeds of batch item j at bench step `step`."""
    return seeds_for(step, 100000 + j, BATCH["traj"])


def make_batch(rb, items, want_events: bool = False, copy: bool = True):
    """The heterogeneous batch of `items` (see batch_items) as one rb.Batch:
    every Michaelis-Menten set shares one network with its own rate constants,
    every random network is its own; seeds of step 0; copy=False reads results
    where the batch keeps them.  Returns (batch, networks)."""
    b = rb.Batch()
    mm = rb.Network(4)
    for e, d in MM_REACTIONS:
        mm.add_reaction(rb.Rate.lma(1.0, e), d)
    nets = [mm]
    for j, (kind, spec, x0) in enumerate(items):
        seeds = batch_seeds(0, j)
        if kind == "mm":
            b.add(mm, x0, seeds, BATCH["tmax_mm"], BATCH["nb_steps"], rates=spec, want_events=want_events,
                  copy=copy)
        else:
            net = rb.Network(len(x0))
            for k, e, d in spec:
                net.add_reaction(rb.Rate.lma(k, e), d)
            nets.append(net)
            b.add(net, x0, seeds, BATCH["tmax_rand"], BATCH["nb_steps"], want_events=want_events, copy=copy)
    return b, nets


def batch_oracle_net(O, item):
    """The oracle's copy of a batch item's network (the reference's sparse form
    for the random networks) and its horizon."""
    kind, spec, x0 = item
    if kind == "mm":
        net = O.OracleNet(4)
        for (e, d), k in zip(MM_REACTIONS, spec):
            net.add_lma(k, e, d)
        return net, BATCH["tmax_mm"]
    net = O.OracleNet(len(x0))
    for k, e, d in spec:
        net.add_lma_sparse(k, [(i, x) for i, x in enumerate(e) if x], d)
    return net, BATCH["tmax_rand"]


def f_event(w) -> int:
    """Algorithmic binary64 operations per event of the direct method with full
    recompute: sum of reactant orders (LMA multiplies) + R (running sum) + R
    (choice compares) + 4 (U scaling, total*U, Exp1/total, clock add)."""
    R = len(w["reactions"])
    return sum(sum(e) for _, e, _ in w["reactions"]) + 2 * R + 4


def seeds_for(rank: int, step: int, n: int) -> np.ndarray:
    rng = np.random.default_rng([20260101, rank, step])
    return rng.integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock, power and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines: list[str] = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU side
def oracle_net_of(O, w):
    net = O.OracleNet(w["S"])
    for k, e, d in w["reactions"]:
        if w.get("sparse"):  # Rate::lma_sparse: the reference's form for large networks
            net.add_lma_sparse(k, [(i, x) for i, x in enumerate(e) if x], d)
        else:
            net.add_lma(k, e, d)
    return net


def cpu_reference(w, n_traj: int, steps: int, warmup: int, threads: int) -> dict:
    """The oracle port of the reference's CPU path: `steps` timed passes over
    n_traj trajectories of workload w on `threads` threads."""
    from oracle import oracle as O

    net = oracle_net_of(O, w)
    tot_ev, tot_s = 0, 0.0
    for step in range(warmup + steps):
        seeds = seeds_for(0, 1000 + step, n_traj)
        t0 = time.perf_counter()
        _, _, ev, _ = net.run_ensemble(w["x0"], seeds, w["tmax"], w["nb_steps"], n_threads=threads)
        dt = time.perf_counter() - t0
        if step >= warmup:
            tot_ev += ev
            tot_s += dt
    return {"value": tot_ev / tot_s, "events": tot_ev, "seconds": tot_s}


def oracle_build_flags() -> str:
    from oracle import oracle as O

    return " ".join(O.compile_flags())


def workload_config(w, n: int) -> dict:
    """The `config` both arms report for workload w at n trajectories."""
    return {"workload": w["desc"], "n_traj": n, "nb_steps": w["nb_steps"], "tmax": w["tmax"],
            "rng": "reference stream: xoshiro256++/SplitMix64 seeds, ziggurat Exp1",
            "l2": "GPU arm: 256 MB written between timed steps (L2 flush)"}


def run_reference_arm(args, w):
    """The reference's CPU path (oracle port, all host cores) on the same
    workload as the GPU arm: every step simulates all w['n_traj'] trajectories."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.n_traj or w["n_traj"]
    r = cpu_reference(w, n, args.steps, args.warmup, threads)
    sample = (f"all {n} trajectories of the workload per step ({w['name']}), oracle port of the reference's "
              f"CPU path, {threads} threads, gcc {oracle_build_flags()}")
    line = {
        "impl": "reference", "metric": "SSA reaction events/sec", "value": r["value"], "unit": "events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * r["seconds"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+int64", "data": "synthetic",
        "config": workload_config(w, n),
        "cpu_baseline": {"value": r["value"], "unit": "events/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": r["value"], "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def reduce_over_ranks(dist, seconds: float, events: float, device: str):
    """Whole-job timing: the slowest rank's seconds and the sum of all ranks'
    events (no data-path collective; trajectories never cross ranks)."""
    if dist is None:
        return seconds, events
    import torch

    t = torch.tensor([seconds, events], dtype=torch.float64, device=device)
    m = t.clone()
    dist.all_reduce(m[:1], op=dist.ReduceOp.MAX)
    dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
    return float(m[0]), float(t[1])


def shard_seeds(rank: int, step: int, n: int) -> np.ndarray:
    """Rank `rank`'s trajectories of a step: its own seeds (weak scaling).  A
    trajectory's stream depends on its seed alone, so any sharding of a seed
    list reproduces the unsharded ensemble."""
    return seeds_for(rank, step, n)


# ---------------------------------------------------------------- GPU side
# Kernel that runs each mapping (rb_run_stats.mapping) and what it is.
MAPPINGS = {
    5: ("ssa_warp_kernel", "warp per trajectory: lanes share the reaction list, only the propensities a firing "
                           "touches re-evaluated, float-pair scan, exact binary64 fold for close choices and "
                           "re-runs of undecided intervals"),
    4: ("rbg_net_kernel", "thread per trajectory, kernel generated for the network and compiled at run time "
                          "(NVRTC); float-pair speculation with exact binary64 re-runs; lanes go to the "
                          "trajectories whose clocks lag furthest behind"),
    3: ("ssa_spec_kernel", "thread per trajectory, packed-descriptor speculative kernel"),
    2: ("ssa_fast_kernel", "thread per trajectory, lockstep exact integer-binary64 kernel"),
    0: ("ssa_thread_kernel", "thread per trajectory, generic exact kernel"),
}


def read_profile(kernel: str, workload: str) -> dict:
    """Per-launch figures (``key: value`` lines) of the committed ncu summary
    of `kernel` on `workload` (profiles/<kernel>_<workload>.md)."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.md"
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        if ":" in line and not line.startswith(("#", "|", " ")):
            k, v = line.split(":", 1)
            try:
                out[k.strip()] = float(v.strip().split()[0])
            except (ValueError, IndexError):
                pass
    return out


def release_host_memory():
    """Between workloads: drop the previous one's page-locked host buffers,
    which torch's host allocator would otherwise keep cached (gigabytes after
    the large-network workload), so each workload starts from the same state."""
    import gc

    import torch

    gc.collect()
    torch.cuda.synchronize()
    empty = getattr(torch._C, "_host_emptyCache", None)
    if empty is not None:
        empty()


def hbm_peak() -> tuple[float, str]:
    """Measured HBM copy bandwidth (GB/s) of the GB300s, else the fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s (of fallback)"


def roofline(kname: str, wname: str, events_per_launch: float, launch_s: float, sample_bytes: float,
             sm_mhz, sms: int, fe: int, dfma_per_s: float | None) -> dict:
    """Roofline of the dominant kernel.  The SSA is a chain of dependent steps
    per trajectory with no reuse to stage: the bound is instruction issue
    (4 schedulers x 32 lanes per SM per clock) over the thread instructions the
    kernel executes per event, measured by ncu on the same kernel and workload
    (the committed profile).  HBM carries only the samples (algorithmic bytes:
    the sample array written once); the FP64-equivalent figure is the direct
    method's binary64 work per event against the DFMA rate measured live, a
    speed-up over an FP64-pipe-bound kernel, not a roofline fraction."""
    prof = read_profile(kname, wname)
    out = {"bound": "issue", "achieved": None, "peak": None, "unit": "T thread-instructions/s", "frac": None,
           "traffic": prof.get("traffic_bytes_per_launch"), "kernel": kname}
    tipe = prof.get("thread_inst_per_event")
    if tipe and sm_mhz:
        peak = sms * 4 * 32 * sm_mhz * 1e6 / 1e12
        ach = tipe * events_per_launch / launch_s / 1e12
        out.update(achieved=ach, peak=peak, frac=ach / peak, thread_inst_per_event=tipe,
                   peak_source=f"{sms} SMs x 4 schedulers x 32 lanes x the SM clock sampled in this run",
                   inst_source=f"profiles/{kname}_{wname}.md (ncu, same kernel and workload)")
    hp, hsrc = hbm_peak()
    out["hbm"] = {"algorithmic_bytes": sample_bytes, "achieved_gbs": sample_bytes / launch_s / 1e9,
                  "peak_gbs": hp, "frac": sample_bytes / launch_s / 1e9 / hp, "peak_source": hsrc,
                  "traffic_vs_algorithmic": (prof["traffic_bytes_per_launch"] / sample_bytes
                                             if prof.get("traffic_bytes_per_launch") and sample_bytes else None)}
    if dfma_per_s:
        ach64 = events_per_launch * fe / launch_s / 1e9
        out["fp64_equivalent"] = {"ops_per_event": fe, "achieved_gops": ach64, "dfma_rate_gops": dfma_per_s / 1e9,
                                  "speedup_over_fp64_pipe": ach64 / (dfma_per_s / 1e9),
                                  "note": "binary64 work done exactly on the FP32/integer pipes"}
    return out


def measure_workload(args, w, steps: int, warmup: int, n: int | None = None, dist=None, rank: int = 0,
                     local: int = 0, cpu: bool = True, fp64_rate: bool = False) -> dict:
    """Device time (HBM-resident inputs, L2 flushed between steps) and end to
    end time (C-ABI host call from page-locked buffers, copies inside) of
    `steps` passes over workload w; the CPU port on a bounded sample beside it."""
    import torch

    import rebop_gb300 as rb
    from rebop_gb300._lib import lib as rblib

    world = 1 if dist is None else dist.get_world_size()

    def barrier():
        if dist is not None:
            dist.barrier()

    net = rb.Network(w["S"])
    for k, e, d in w["reactions"]:
        net.add_reaction(rb.Rate.lma(k, e), d)
    n = n or w["n_traj"]
    NT, S = w["nb_steps"] + 1, w["S"]
    stream = torch.cuda.current_stream()
    sid = stream.cuda_stream
    d_x0 = torch.tensor(w["x0"], dtype=torch.int64, device="cuda")
    d_seeds = [torch.from_numpy(shard_seeds(rank, s, n).view(np.int64)).cuda() for s in range(warmup + steps)]
    d_out = torch.empty((NT, S, n), dtype=torch.int64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def launch(seeds):
        net.run_ensemble_device(n, d_x0.data_ptr(), False, seeds.data_ptr(), w["tmax"], w["nb_steps"],
                                d_out.data_ptr(), stream=sid)

    # the autotuner picks the kernel and launch shape for this network and
    # ensemble size (pilot runs, outside the timed region)
    tuning = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tr = net.tune(w["x0"], n, w["tmax"], w["nb_steps"])
        tuning = {"best": tr["best"], "trials": tr["trials"], "seconds": time.perf_counter() - t0}
    for s in range(warmup):
        launch(d_seeds[s])
    torch.cuda.synchronize()
    dfma = rblib.rbg_internal_fp64_fma_rate(sid) if fp64_rate else None  # DFMA instructions / s, live

    vis = [v for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    clocks = ClockSampler(int(vis[local]) if local < len(vis) and vis[local].strip().isdigit() else local)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    events_per_step = []
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    for s in range(steps):
        flush.zero_()  # L2 flush between timed steps (256 MB > 129 MB L2)
        ev0[s].record(stream)
        launch(d_seeds[warmup + s])
        ev1[s].record(stream)
        events_per_step.append(net.last_events())
    torch.cuda.synchronize()
    barrier()
    t_wall = time.perf_counter() - t_wall0
    step_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    dev_s = sum(step_ms) / 1e3
    ev_total = sum(events_per_step)
    dev_s_all, ev_all = reduce_over_ranks(dist, dev_s, float(ev_total), "cuda")

    # end to end: the C-ABI host call with page-locked buffers, copies in the timed region
    pin_out = torch.empty((NT, S, n), dtype=torch.int64, pin_memory=True).numpy()
    pin_seeds = [torch.from_numpy(seeds_for(rank, 500 + s, n).view(np.int64)).pin_memory().numpy().view(np.uint64)
                 for s in range(steps + 1)]
    x0_host = np.asarray(w["x0"], dtype=np.int64)
    net.run_ensemble(x0_host, pin_seeds[0], w["tmax"], w["nb_steps"], out=pin_out, want_events=False)
    barrier()
    e2e_ev, e2e_s, h2d, d2h, k_ms = 0, 0.0, 0, 0, 0.0
    for s in range(steps):
        t0 = time.perf_counter()
        res = net.run_ensemble(x0_host, pin_seeds[1 + s], w["tmax"], w["nb_steps"], out=pin_out,
                               want_events=False)
        e2e_s += time.perf_counter() - t0
        e2e_ev += res.total_events
        h2d, d2h = res.stats["h2d_bytes"], res.stats["d2h_bytes"]
        k_ms += res.stats["kernel_ms"]
    clk = clocks.stop()
    e2e_s_all, e2e_ev_all = reduce_over_ranks(dist, e2e_s, float(e2e_ev), "cuda")

    mapping = int(res.stats["mapping"])
    kname, kdesc = MAPPINGS.get(mapping, ("?", "?"))
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    rl = roofline(kname, w["name"], ev_total / steps, dev_s / steps, NT * S * n * 8.0, clk.get("sm_mhz"), sms,
                  f_event(w), dfma)

    cpu_b = None
    if cpu and rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        nb = args.cpu_sample or w["cpu_sample"]
        r = cpu_reference(w, nb, 1, 0, threads)
        # one core as well, on a sample of about a second
        n1 = max(1, min(nb, int(nb * 1.0 / max(r["seconds"] * threads, 1e-9))))
        r1 = cpu_reference(w, n1, 1, 0, 1)
        cpu_b = {"value": r["value"], "unit": "events/s", "cores": threads, "kind": "port",
                 "sample": f"{nb} trajectories of the same workload, oracle port of the reference CPU path, "
                           f"{threads} threads, gcc {oracle_build_flags()}",
                 "value_1core": r1["value"], "sample_1core": f"{n1} trajectories on one thread"}
    return {
        "value": ev_all / dev_s_all, "unit": "events/s", "steps": steps, "warmup": warmup,
        "ms_per_step": 1e3 * dev_s_all / steps, "events_per_step": ev_total / steps, "wall_s": t_wall,
        "e2e": {"value": e2e_ev_all / e2e_s_all, "unit": "events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e2e_s / steps,
                "kernel_ms_per_step": k_ms / steps},
        "gpu_launches": steps, "roofline": rl, "cpu_baseline": cpu_b, "clocks": clk,
        "kernel": kname, "mapping": kdesc, "n_traj": n, "tuning": tuning,
        "_net": net, "_x0": x0_host, "_world": world,
    }


def run_ours(args, w):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    m = measure_workload(args, w, args.steps, args.warmup, n=args.n_traj or None, dist=dist, rank=rank,
                         local=local, cpu=not args.no_cpu_baseline, fp64_rate=True)

    calib = None
    if rank == 0 and w.get("calib_n"):
        # the reference's own benchmark size: calib_n trajectories through the
        # host API (host buffers, copies inside the timed region)
        nc = int(w["calib_n"])
        cs = seeds_for(rank, 900, nc)
        net, x0_host = m["_net"], m["_x0"]
        net.run_ensemble(x0_host, cs, w["tmax"], w["nb_steps"], want_events=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = net.run_ensemble(x0_host, cs, w["tmax"], w["nb_steps"], want_events=True)
        c_s = time.perf_counter() - t0
        calib = {"n_traj": nc, "seconds": c_s, "events": int(rc.total_events),
                 "published_reference_s": w["calib_published_s"],
                 "note": "wall time of the reference's own run size through the host API on one GPU; "
                         "the published figure is the reference's rebopy run on its authors' CPU"}
        if not args.no_cpu_baseline:
            # single-thread slope of the oracle port, the unit the reference's
            # benchmark quotes (ms per trajectory on one core)
            r1 = cpu_reference(w, 16, 1, 0, 1)
            calib["cpu_port_1thread_ms_per_traj"] = 1e3 * r1["seconds"] / 16

    # the other configurations, a few steps each, beside the headline (one GPU only)
    subs = {}
    if rank == 0 and world == 1 and args.workloads != "none":
        for name in [x for x in args.workloads.split(",") if x and x != w["name"]]:
            release_host_memory()
            if name == "batch":
                subs[name] = measure_batch(args, min(args.steps, 3), min(args.warmup, 2),
                                           cpu=not args.no_cpu_baseline)
            elif name == "surrogate":
                subs[name] = measure_surrogate(args)
            else:
                sw = WORKLOADS[name]
                st, wu = SUB_STEPS.get(name, (3, 2))
                r = measure_workload(args, sw, min(args.steps, st), min(args.warmup, wu),
                                     cpu=not args.no_cpu_baseline)
                r["config"] = workload_config(sw, r["n_traj"])
                subs[name] = {k: v for k, v in r.items() if not k.startswith("_")}

    if rank == 0:
        line = {
            "metric": "SSA reaction events/sec", "value": m["value"], "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+int64",
            "data": "synthetic",
            "config": workload_config(w, m["n_traj"]),
            "events_per_step": m["events_per_step"], "kernel": m["kernel"], "mapping": m["mapping"],
            "wall_s": m["wall_s"],
            "e2e": m["e2e"], "gpu_launches": m["gpu_launches"], "roofline": m["roofline"],
            "cpu_baseline": m["cpu_baseline"], "clocks": m["clocks"], "tuning": m["tuning"],
        }
        if calib is not None:
            line["reference_benchmark_run"] = calib
        if subs:
            line["workloads"] = subs
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# steps / warm-up of the configurations run beside the headline
SUB_STEPS = {"sir": (5, 3), "large": (2, 1), "vilar": (2, 1)}


def _batch_cpu(items, every: int, traj: int, threads: int):
    """Oracle on every `every`-th item of each kind: events/s on `threads` threads."""
    from oracle import oracle as O

    ev_tot, t_tot = 0, 0.0
    for j, item in enumerate(items):
        if j % every:
            continue
        net, tmax = batch_oracle_net(O, item)
        x0 = item[2]
        seeds = seeds_for(0, 7000 + j, traj)
        t0 = time.perf_counter()
        _, _, ev, _ = net.run_ensemble(x0, seeds, tmax, BATCH["nb_steps"], n_threads=threads)
        t_tot += time.perf_counter() - t0
        ev_tot += ev
    return ev_tot / t_tot, ev_tot, t_tot


def measure_batch(args, steps: int, warmup: int, cpu: bool = True) -> dict:
    import torch

    import rebop_gb300 as rb

    items = batch_items()
    b, nets = make_batch(rb, items, copy=False)  # results read in place, as a serving caller would
    n_own, n_persistent = b.plan()
    for s in range(warmup):
        b.run()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    dev_ms, wall, events, h2d, d2h, launches = 0.0, 0.0, 0, 0, 0, 0
    parts = {"in_ms": 0.0, "kernels_ms": 0.0, "out_ms": 0.0}
    for s in range(steps):
        for j in range(len(items)):
            b.seeds(j)[:] = batch_seeds(1 + s, j)
        t0 = time.perf_counter()
        st = b.run()
        wall += time.perf_counter() - t0
        dev_ms += st["kernel_ms"]
        events += st["events"]
        launches += st["kernel_launches"]
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
        for k, v in b.times().items():
            parts[k] += v / steps
    clk = clocks.stop()
    torch.cuda.synchronize()
    cpu_b = None
    if cpu:
        threads = os.cpu_count() or 1
        v, _, _ = _batch_cpu(items, BATCH["cpu_every"] * 4, BATCH["traj"], threads)
        cpu_b = {"value": v, "unit": "events/s", "cores": threads, "kind": "port",
                 "sample": f"every {BATCH['cpu_every'] * 4}th item of each kind, oracle port, {threads} threads"}
    # value: the kernels' device time inside the graph (inputs resident in HBM,
    # results left there); the copies in and out and the host-side staging are
    # in e2e, and the whole graph's device time is reported beside it
    kern_ms = parts["kernels_ms"] * steps if parts["kernels_ms"] > 0 else dev_ms
    return {
        "value": events / (kern_ms / 1e3), "unit": "events/s", "steps": steps, "warmup": warmup,
        "ms_per_step": kern_ms / steps,
        "config": {"workload": BATCH["desc"], "items": len(items), "traj_per_item": BATCH["traj"],
                   "trajectories": len(items) * BATCH["traj"],
                   "events_per_step": events / steps, "own_launches": n_own, "persistent_items": n_persistent,
                   "mode": os.environ.get("RB_BATCH_MODE", "persistent"),
                   "timing": ("value: device time of the graph's kernels (CUDA events recorded as graph nodes); "
                              "e2e: wall time of Batch.run (input staging, the graph with its input copy and its "
                              "copy of every result into page-locked host memory, where the caller reads them)"),
                   "graph_ms_per_step": dev_ms / steps,
                   "graph_parts_ms": parts,
                   "l2": "inputs and outputs far above L2 are copied in every step"},
        "e2e": {"value": events / wall, "unit": "events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches, "cpu_baseline": cpu_b, "clocks": clk,
    }


def run_batch(args):
    import torch

    items = batch_items()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        threads = os.cpu_count() or 1
        v, ev, t = _batch_cpu(items, BATCH["cpu_every"], BATCH["traj"], threads)
        print(json.dumps({"impl": "reference", "metric": "SSA reaction events/sec", "value": v, "unit": "events/s",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * t,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+int64",
                          "data": "synthetic", "config": {"workload": BATCH["desc"]},
                          "cpu_baseline": {"value": v, "unit": "events/s", "cores": threads, "kind": "port",
                                           "sample": f"every {BATCH['cpu_every']}th item of each kind, oracle port"},
                          "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.n_traj:
        BATCH["traj"] = args.n_traj  # trajectories per item (a smaller case for profiling)
    m = measure_batch(args, args.steps, args.warmup, cpu=not args.no_cpu_baseline)
    line = {"metric": "SSA reaction events/sec", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+int64", "data": "synthetic", **m}
    print(json.dumps(line), flush=True)


SURROGATE = dict(
    name="surrogate",
    desc=("learned surrogate of the dimer ensemble: 2^22 training tuples generated by the engine, one per "
          "trajectory (5 rate factors 10^U[-1,1] around 25, 1000, 0.001, 0.1, 1; t drawn from the 101-point grid "
          "of [0, 1]); rate-equation baseline per query; MLP 8 -> 4 x 256 SiLU -> count-aware head per species "
          "(classes for counts 0..30, an 8-component Gaussian mixture over the log-count residual above), BF16 "
          "weights, FP32 accumulation; held-out points judged against fresh SSA batches"),
    n_traj=1 << 22, epochs=20, batch=4096, lr=2e-3, n_points=128, n_ssa=1000, n_points_big=64, n_ssa_big=10000,
    n_queries=1_000_000, draws=1000,
)


def measure_surrogate(args) -> dict:
    import torch

    from rebop_gb300 import surrogate as sg

    w = SURROGATE
    t0 = time.perf_counter()
    x, y, _ = sg.generate(w["n_traj"], seed=20260106)
    t_gen = time.perf_counter() - t0
    model = sg.MDN(seed=0)
    t0 = time.perf_counter()
    model.fit(x, y, epochs=w["epochs"], batch=w["batch"], lr=w["lr"])
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    val = sg.Surrogate(model, tol=0.01).validate(w["n_points"], w["n_ssa"], seed=7)
    sur = sg.Surrogate(model, tol=0.01)
    big = sur.validate(w["n_points_big"], w["n_ssa_big"], seed=8)
    # throughput: queries answered by the surrogate (rate equations, one forward
    # pass and `draws` samples each) against queries answered by the SSA engine
    # (`draws` trajectories each)
    rng = np.random.default_rng(9)
    q = np.concatenate([rng.uniform(-1, 1, (w["n_queries"], 5)), rng.integers(1, 101, (w["n_queries"], 1)) / 100],
                       axis=1).astype(np.float32)
    Q = torch.from_numpy(q).cuda()
    chunk = 65536  # queries per call (1000 draws each: 524 MB of draws)
    for s in range(0, 2 * chunk, chunk):  # warm-up
        model.sample_counts(Q[s:s + chunk], w["draws"])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_q = 262144
    e0.record()
    for s in range(0, n_q, chunk):
        model.sample_counts(Q[s:s + chunk], w["draws"])
    e1.record()
    torch.cuda.synchronize()
    sur_qps = n_q / (e0.elapsed_time(e1) / 1e3)
    e0.record()
    for s in range(0, w["n_queries"], 65536):
        model.predict_params(Q[s:s + 65536])
    e1.record()
    torch.cuda.synchronize()
    param_qps = w["n_queries"] / (e0.elapsed_time(e1) / 1e3)
    ssa_qps = w["n_points"] / (val["ssa_kernel_ms"] / 1e3)
    gemm_tflops = gemm_figures(model.tc_err)
    model.check_errors()
    answered = sur.answer(q[:100000]).mean()
    med = lambda a: float(np.median(a))  # noqa: E731
    ok = (big["w1"] <= 0.01).all(axis=1)
    return {
        "metric": "surrogate queries/s (1000 draws each) vs plain GPU SSA queries/s (1000 trajectories each)",
        "value": sur_qps, "unit": "queries/s", "steps": 1, "warmup": 1, "ms_per_step": 1e3 * n_q / sur_qps,
        "dtype": "bf16 weights, fp32 accumulation", "data": "synthetic (engine-generated)",
        "config": {"workload": w["desc"], "training_tuples": int(x.shape[0]), "epochs": w["epochs"],
                   "generate_s": t_gen, "train_s": t_train},
        "ssa_queries_per_s": ssa_qps, "speedup_vs_ssa": sur_qps / ssa_qps, "params_only_queries_per_s": param_qps,
        "accuracy_1e3": {
            "points": w["n_points"], "model_draws": val["model_draws"],
            "median_w1_rel": [med(val["w1"][:, 0]), med(val["w1"][:, 1])],
            "median_w1_rel_ssa_vs_ssa": [med(val["w1_floor"][:, 0]), med(val["w1_floor"][:, 1])],
            "fraction_w1_within_1pct": float(np.mean((val["w1"] <= 0.01).all(axis=1))),
            "fraction_w1_within_1pct_ssa_vs_ssa": float(np.mean((val["w1_floor"] <= 0.01).all(axis=1))),
            "median_ks": [med(val["ks"][:, 0]), med(val["ks"][:, 1])]},
        "accuracy_1e4": {
            "points": w["n_points_big"], "model_draws": big["model_draws"],
            "median_w1_rel": [med(big["w1"][:, 0]), med(big["w1"][:, 1])],
            "median_w1_rel_ssa_vs_ssa": [med(big["w1_floor"][:, 0]), med(big["w1_floor"][:, 1])],
            "fraction_w1_within_1pct": float(np.mean(ok)),
            "fraction_w1_within_1pct_ssa_vs_ssa": float(np.mean((big["w1_floor"] <= 0.01).all(axis=1))),
            "fraction_w1_within_1pct_per_species": [float(np.mean(big["w1"][:, 0] <= 0.01)),
                                                     float(np.mean(big["w1"][:, 1] <= 0.01))],
            "median_ks": [med(big["ks"][:, 0]), med(big["ks"][:, 1])]},
        "answered_by_surrogate": float(answered),
        "gemm_4096x256x256_tflops": gemm_tflops,
    }


def gemm_figures(err_flag, reps: int = 50) -> dict:
    """TFLOP/s of the training GEMM shape (4096 x 256 x 256, BF16 in, FP32 out)
    on each tensor-core path: tc05_tma (operands by cp.async.bulk.tensor),
    tc05_staged (the same MMAs, operands staged by vector loads,
    RB_GEMM_TMA=0) and mma (mma.sync); `reps` back-to-back launches each,
    CUDA events on the launching stream."""
    import torch

    from rebop_gb300._lib import check, lib

    ga = torch.randn(4096, 256, device="cuda").to(torch.bfloat16)
    gb = torch.randn(256, 256, device="cuda").to(torch.bfloat16)
    gc = torch.empty(4096, 256, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    for name in ("tc05_tma", "tc05_staged", "mma"):
        if name == "tc05_staged":
            os.environ["RB_GEMM_TMA"] = "0"
        for rep in range(reps + 10):
            if rep == 10:
                e0.record()
            if name != "mma":
                check(lib.rbg_mdn_gemm_tc05(ga.data_ptr(), 256, 0, gb.data_ptr(), 256, 1, gc.data_ptr(), 256, 4096,
                                            256, 256, 0.0, err_flag.data_ptr(), st))
            else:
                check(lib.rbg_mdn_gemm(ga.data_ptr(), 256, 0, gb.data_ptr(), 256, 1, gc.data_ptr(), 256, 4096, 256,
                                       256, 0.0, st))
        e1.record()
        torch.cuda.synchronize()
        os.environ.pop("RB_GEMM_TMA", None)
        out[name] = reps * 2 * 4096 * 256 * 256 / (e0.elapsed_time(e1) / 1e3) / 1e12
    return out


def run_gemm(args):
    """The surrogate's GEMM alone: one JSON line of TFLOP/s per tensor-core path."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    reps = max(args.steps, 1) * 50
    f = gemm_figures(err, reps)
    if int(err.item()):
        raise RuntimeError("tcgen05 GEMM: a completion wait ran out")
    try:
        peak, src = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"]), \
            "MEASURED_PEAKS.json bf16_tflops (burst, of measured)"
    except (OSError, ValueError, KeyError):
        peak, src = 1900.0, "fallback 1.9 PFLOP/s (of fallback)"
    # the fused inference kernel on the same network shape (random weights):
    # 65 536 queries per launch, the whole MLP in one kernel
    from rebop_gb300 import surrogate as sg

    model = sg.MDN(seed=0)
    F = torch.randn(65536, sg.N_IN, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for rep in range(reps // 10 + 5):
        if rep == 5:
            e0.record()
        model.infer(F)
    e1.record()
    torch.cuda.synchronize()
    model.check_errors()
    n_inf = reps // 10
    inf_s = e0.elapsed_time(e1) / 1e3 / n_inf
    flop = 2.0 * 65536 * (sg.N_IN * 256 + 3 * 256 * 256 + 256 * model.n_out)
    f["fused_inference"] = {"queries_per_s": 65536 / inf_s, "us_per_launch": inf_s * 1e6, "tflops": flop / inf_s / 1e12}
    v = f["tc05_tma"]
    print(json.dumps({"metric": "BF16 GEMM TFLOP/s, 4096 x 256 x 256, FP32 accumulate", "value": v,
                      "unit": "TFLOP/s", "n_gpus": 1, "steps": reps, "warmup": 10, "higher_is_better": True,
                      "dtype": "bf16", "data": "synthetic", "paths": f,
                      "roofline": {"bound": "tensor", "achieved": v, "peak": peak, "unit": "TFLOP/s",
                                   "frac": v / peak, "peak_source": src,
                                   "note": "0.54 GFLOP per launch: launch- and latency-bound at this size"}}),
          flush=True)


def run_surrogate(args):
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    m = measure_surrogate(args)
    line = {"metric": m.pop("metric"), "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "gpu_launches": None, **m}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch", "surrogate", "gemm"], default="dimer")
    ap.add_argument("--n-traj", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner's pilot runs")
    # the batch first: measured after the SIR and large-network CPU baselines,
    # its 2.77 GB result copy into page-locked memory ran up to 7x slower
    ap.add_argument("--workloads", default="batch,sir,large,surrogate",
                    help="configurations measured beside the headline (comma list, or 'none')")
    args = ap.parse_args()
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "gemm":
        if args.impl == "ours":
            run_gemm(args)
        elif int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no GEMM"}), flush=True)
        return
    if args.workload == "surrogate":
        if args.impl == "reference":
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned surrogate; "
                                  "its plain SSA answers the same queries in the surrogate line "
                                  "(ssa_queries_per_s)"}), flush=True)
            return
        run_surrogate(args)
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference_arm(args, w)
    else:
        run_ours(args, w)


if __name__ == "__main__":
    main()
