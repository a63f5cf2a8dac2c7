"""Benchmark of the SIS force/integration hot path on GB300.

Metric: bead*steps/s of the mixed-precision path (FP32 pair/bonded terms,
FP64 accumulation and integration) next to the plain FP64 GPU path, at the
stated force error against FP64.

Workload (default, single GPU): the crowded single-system run -- 200 chains
x 500 nt (100,000 beads), seeded random sequences and random-coil starts
placed without overlap in a cubic PBC box at 10 mM nucleotide, 150 mM salt,
300 K, sis.ff parameters, base-pair model 1.  Inputs are synthetic (no
dataset is involved).

A bench "step" is one block of MD steps (``--md-steps``, default 100) of all
instances; L2 is flushed (512 MiB write) between timed blocks.  Positions,
velocities and the noise state stay resident in HBM for ``value``; ``e2e``
runs the same blocks through the public C ABI with host buffers: every block
uploads x, v and the GJF-2GJ noise term from pinned host memory and reads the
positions back.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bead·steps/s batched-FP32 vs plain-FP64 on 1 GB300 at stated force err; p99 job ms"
UNIT = "bead*steps/s"
WORKLOADS = {
    "serve": "Poisson job stream (continuous batching): lengths log-U[20,2000] nt, steps log-U[1e4,1e6] x steps-scale, "
             "T U[280,360] K, salt U[20,500] mM",
    "crowded": "200 chains x 500 nt (100,000 beads), cubic PBC box at 10 mM nucleotide, 150 mM salt, 300 K; "
               "random-coil start with non-bonded pairs >= 10 A apart",
    "uneven": "256 independent chains, lengths U[20,500], salt U[20,500] mM, T U[280,340] K",
    "remd": "64 replicas x 120 nt, T geometric 280-360 K",
    "chain64": "one 64-nt chain, 300 K, 150 mM, no PBC",
}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


RELAXED = ROOT / "sis_gb300" / "data" / "crowded_relaxed.npz"


def make_system(name, seed_offset=0):
    """The workload's system.  The crowded box starts from its relaxed
    positions (sis_gb300/data/crowded_relaxed.npz, written by make_relaxed.py)
    when they are present, so that every arm starts from the same state."""
    from sis_gb300.coil import crowded_box, remd_batch, single_chain, uneven_batch
    from sis_gb300.inputs import read_ff

    ff = read_ff(ROOT / "sis_gb300" / "data" / "sis.ff")
    if name == "crowded":
        if RELAXED.exists():
            # every rank: the same relaxed box (its ranks differ in their noise)
            seed_offset = 0
        sysm = crowded_box(ff, 200, 500, 0.01, seed=1002 + seed_offset)
        if RELAXED.exists():
            x = np.load(RELAXED)["xyz"].astype(np.float64)
            if x.shape == (sysm.nmp, 3):
                sysm.instances[0].xyz = x
                sysm.relaxed_start = True
        return sysm
    if name == "uneven":
        return uneven_batch(ff, 256, seed=1004 + seed_offset)
    if name == "remd":
        return remd_batch(ff, 64, 120, seed=1003 + seed_offset)
    return single_chain(ff, 64, seed=1001 + seed_offset)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the region starts once the sampler is producing samples
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.n0 = len(self.lines)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # samples taken during the region (the last one before it as well, if the region was shorter than a period)
        for l in self.lines[max(0, getattr(self, "n0", 0) - 1):]:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def list_stats(eng):
    """List entries per bead in the reference's convention (WCA + DH + bp half lists)."""
    tot = {0: 0, 1: 0, 2: 0}
    for k in range(eng.n_inst):
        for kind in (0, 1, 2):
            tot[kind] += len(eng.get_list(k, kind))
    return tot


def run_gpu(args):
    from sis_gb300 import FP64, MIXED
    from sis_gb300.engine import Engine

    rank, world, local = dist_env()
    sysm = make_system(args.workload, seed_offset=rank)
    S = args.md_steps
    N = sysm.nmp
    eng = Engine(sysm, precision=MIXED, seed=2024 + rank)
    if args.lanes:  # fixed lanes per bead (no autotuning): reproducible launch sequences for profiling
        eng.set_lanes(args.lanes)
    if args.no_graphs:  # every kernel launched from the host (what per-kernel profilers can see)
        eng.set_graphs(False)
    if args.overlap >= 0:
        eng.set_overlap(bool(args.overlap))
    eng.init_velocities()
    relaxed = getattr(sysm, "relaxed_start", False)
    relax = args.relax if args.relax >= 0 else (500 if relaxed else 3000)
    if relaxed:
        # the relaxed start: velocities from the noise, then free dynamics
        eng.set_force_cap(args.force_cap)
        eng.step(relax)
    else:
        # equilibrate before timing (force-capped, then free dynamics; neither
        # is timed): a coil start is far from equilibrium
        eng.relax(capped_steps=relax, fmax=1000.0, free_steps=relax)
    # singularity guard for the production steps: the cosine dihedral force of
    # the model (force_dih_cos.F90) diverges as a bond angle reaches 180 degrees;
    # a per-bead cap far above thermal forces keeps such events finite
    eng.set_force_cap(args.force_cap)
    # replica exchange (64 replicas of one 120-nt chain): an attempt every exchange_interval
    # MD steps, odd and even patterns alternating, inside the timed region
    remd = args.workload == "remd"
    rx = {"since": 0, "attempts": 0, "accepted": 0}
    if remd:
        eng.remd_init([inst.tempK for inst in sysm.instances])

    def advance():
        eng.step(S)
        if remd:
            rx["since"] += S
            if rx["since"] >= args.exchange_interval:
                _, acc = eng.remd_exchange(rx["attempts"] % 2)
                rx["attempts"] += 1
                rx["accepted"] += acc
                rx["since"] = 0

    for _ in range(args.warmup):
        eng.flush_l2()
        advance()
    launches0 = eng.kernel_launches()
    st0 = eng.stats()
    cap0 = st0["capped"]
    rx0 = dict(rx)
    times = []
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            eng.flush_l2()
            eng.event(0)
            advance()
            eng.event(1)
            times.append(eng.elapsed_ms(0, 1))
    rx_timed = {"attempts": rx["attempts"] - rx0["attempts"], "accepted": rx["accepted"] - rx0["accepted"]}
    launches = eng.kernel_launches() - launches0
    st1 = eng.stats()
    total_ms = max_over_ranks(sum(times), world)
    value = world * N * S * args.steps / (total_ms * 1e-3)

    # roofline of the pair and update kernels (k_pairs_cl + k_step_mixed, one
    # after the other under CUDA events on the stream that launches them).
    # Algorithmic bytes per bead and MD step: k_pairs_cl reads the bead's
    # mirror (16), its share of the cluster records (20 per j-cluster per
    # 8 beads) and writes its pair force (16); k_step_mixed reads the pair
    # and bonded forces (16 + 16), reads and clears the base-pair sum
    # (32 + 32), reads and writes FP64 x, v, beta (2 x 72), reads the
    # coefficients (32), the mirror at the last rebuild (16) and the bead
    # record (16), and writes the mirror and residual (32).
    prof_steps = min(200, S * args.steps)
    ms3 = eng.step_profiled(prof_steps)
    lst = list_stats(eng)
    L = (lst[0] + lst[1] + lst[2]) / N
    C = st1["cluster_pairs"] / max(1, st1["i_clusters"])
    bytes_per_bead = 16 + 20 * C / 8 + 16 + 336
    step_ms = ms3[1] / prof_steps
    achieved = N * bytes_per_bead / (step_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    rebuilds = st1["rebuilds"] - st0["rebuilds"]
    k_rebuild = (S * args.steps * len(sysm.instances)) / rebuilds if rebuilds else None
    traffic = None
    tf = ROOT / "profiles" / f"step_kernels_{args.workload}_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("bytes_per_launch")

    # plain FP64 GPU path on the same state, and the force error against it
    x, v, a = eng.get_state(-1)
    e64 = Engine(sysm, precision=FP64, seed=2024 + rank)
    e64.set_state(-1, x, v, a)
    e64.set_force_cap(args.force_cap)
    f64 = np.concatenate([e64.force(k) for k in range(e64.n_inst)])
    eng.set_state(-1, x, v, a)
    f32 = np.concatenate([eng.force(k) for k in range(eng.n_inst)])
    err = float(np.sqrt(np.mean(np.sum((f32 - f64) ** 2, axis=1)) / np.mean(np.sum(f64 ** 2, axis=1))))
    e64.step(S)
    t64 = []
    for _ in range(max(2, args.steps // 3)):
        e64.flush_l2()
        e64.event(0)
        e64.step(S)
        e64.event(1)
        t64.append(e64.elapsed_ms(0, 1))
    fp64_value = world * N * S * len(t64) / (max_over_ranks(sum(t64), world) * 1e-3)
    e64.close()

    # end to end through the C ABI with host buffers
    x, v, a = eng.get_state(-1)
    e2e_t = []
    for _ in range(args.steps):
        eng.flush_l2()
        eng.synchronize()
        t0 = time.perf_counter()
        eng.set_state(-1, x, v, a)
        advance()
        x, v, a = eng.get_state(-1)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sum(e2e_t), world)
    e2e_value = world * N * S * args.steps / e2e_s
    cfg = {"workload": args.workload, "description": WORKLOADS[args.workload], "n_beads": N,
           "n_instances": len(sysm.instances), "md_steps_per_step": S, "precision": "FP32 terms / FP64 accumulate+integrate",
           "list_entries_per_bead": round(L, 3), "steps_per_rebuild": k_rebuild, "lanes_per_bead": st1["lanes_per_bead"], "pair_kernel_beside_bonded": bool(st1["overlap"]), "bp_blocks": st1["bp_blocks"],
           "small_blocks": st1["small_blocks"], "small_threads": st1["small_threads"],
           "l2": "flushed between timed steps (512 MiB write)", "fp64_value": fp64_value,
           "speedup_vs_fp64": value / fp64_value, "force_rms_rel_err_vs_fp64": err,
           "start": "relaxed positions of sis_gb300/data/crowded_relaxed.npz" if relaxed else "random coil",
           "relax_steps": {"force_capped": 0 if relaxed else relax, "free": relax},
           "force_cap": args.force_cap, "capped_bead_steps": st1["capped"] - cap0,
           "launches_before_timed": int(launches0), "step_graphs": not args.no_graphs,
           **({"exchange_interval": args.exchange_interval, "exchange_attempts_timed": rx_timed["attempts"],
               "exchange_pairs_accepted_timed": rx_timed["accepted"]} if remd else {}),
           "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32+fp64", "data": "synthetic (seeded sequences and random-coil starts)", "config": cfg,
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * 32 * N, "d2h_bytes_per_step": 3 * 32 * N},
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": traffic, "peak_kind": peak_kind,
                        "kernel": "k_pairs_cl + k_step_mixed", "kernel_ms": step_ms,
                        "bonded_bp_ms": ms3[0] / prof_steps, "trigger_rebuild_ms": ms3[2] / prof_steps,
                        "bytes_per_bead_step": bytes_per_bead, "j_clusters_per_i_cluster": C},
           "clocks": clk.summary()}
    eng.close()
    if not args.no_sub and args.workload == "crowded":
        # the batched-chain workload the >= 20x target is stated on, and the serving stream
        cfg["uneven"] = uneven_record(args, rank, world)
        cfg["serve"] = serve_record(args, rank, world)
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(args, sysm)
    return out, rank


def uneven_record(args, rank, world):
    """The uneven batch (256 chains of U[20,500] nt, each with its own salt and
    temperature, no PBC), the workload the >= 20x target is stated on: mixed
    path against the plain FP64 path from the same state, L2 flushed between
    timed blocks, max over ranks.  The same protocol as the --workload uneven
    line: 3000 capped + 3000 free relaxation steps from the random coils,
    --warmup untimed and --steps timed blocks of --md-steps MD steps."""
    from sis_gb300 import FP64, MIXED
    from sis_gb300.engine import Engine

    sysm = make_system("uneven", seed_offset=rank)
    N, S = sysm.nmp, args.md_steps
    eng = Engine(sysm, precision=MIXED, seed=2024 + rank)
    eng.init_velocities()
    eng.relax(capped_steps=3000, fmax=1000.0, free_steps=3000)
    eng.set_force_cap(args.force_cap)
    for _ in range(max(3, args.warmup)):
        eng.flush_l2()
        eng.step(S)
    st0 = eng.stats()
    t = []
    for _ in range(max(1, args.steps)):
        eng.flush_l2()
        eng.event(0)
        eng.step(S)
        eng.event(1)
        t.append(eng.elapsed_ms(0, 1))
    st1 = eng.stats()
    ms = max_over_ranks(sum(t), world)
    value = world * N * S * len(t) / (ms * 1e-3)
    x, v, a = eng.get_state(-1)
    e64 = Engine(sysm, precision=FP64, seed=2024 + rank)
    e64.set_state(-1, x, v, a)
    e64.set_force_cap(args.force_cap)
    f64 = np.concatenate([e64.force(k) for k in range(e64.n_inst)])
    f32 = np.concatenate([eng.force(k) for k in range(eng.n_inst)])
    err = float(np.sqrt(np.mean(np.sum((f32 - f64) ** 2, axis=1)) / np.mean(np.sum(f64 ** 2, axis=1))))
    e64.step(S)
    t64 = []
    for _ in range(3):
        e64.flush_l2()
        e64.event(0)
        e64.step(S)
        e64.event(1)
        t64.append(e64.elapsed_ms(0, 1))
    v64 = world * N * S * len(t64) / (max_over_ranks(sum(t64), world) * 1e-3)
    e64.close()
    eng.close()
    reb = st1["rebuilds"] - st0["rebuilds"]
    return {"description": WORKLOADS["uneven"], "n_beads": N, "n_instances": len(sysm.instances), "value": value,
            "unit": UNIT, "ms_per_md_step": ms / (len(t) * S), "fp64_value": v64, "speedup_vs_fp64": value / v64,
            "target_speedup_vs_fp64": 20.0, "force_rms_rel_err_vs_fp64": err,
            "steps_per_rebuild": S * len(t) * len(sysm.instances) / reb if reb else None,
            "lanes_per_bead": st1["lanes_per_bead"], "small_blocks": st1["small_blocks"], "small_threads": st1["small_threads"],
            "timed_blocks": len(t), "md_steps_per_block": S,
            "relax_steps": {"force_capped": 3000, "free": 3000}, "l2": "flushed between timed blocks (512 MiB write)"}


def serve_record(args, rank, world, seconds=4.0, scale=0.01):
    """The serving stream at a stated scale: Poisson arrivals at --serve-rate
    jobs/s for `seconds`, every job's step count times `scale`; latency is
    arrival to completion."""
    summ, cfg, value, _ = serve_run(args, rank, world, seconds, scale)
    return {"description": WORKLOADS["serve"], "arrival_rate_per_s": args.serve_rate, "arrival_window_s": seconds,
            "steps_scale": scale, "jobs": cfg["jobs"], "jobs_completed": summ["jobs"], "jobs_failed": summ["failed"],
            "p50_latency_ms": summ["p50_ms"], "p99_latency_ms": summ["p99_ms"],
            "offered_bead_steps_per_s": cfg["offered_bead_steps_per_s"], "achieved_bead_steps_per_s": value, "unit": UNIT}


class CpuSampler:
    """The FP64 oracle (C++ restatement of the reference, OpenMP over all host
    threads) on up to 8 instances of the workload, from the workload's start
    (for the crowded box its relaxed positions, the GPU arm's start too) with
    velocities from the oracle's own MT19937 + polar Box-Muller noise.  Its
    lists are built once (untimed); each sample then runs MD until the
    displacement trigger has rebuilt the lists once, so the reference's O(N^2)
    rebuild enters at its natural rate: one rebuild per rebuild interval."""

    def __init__(self, sysm, seed=1234):
        from oracle.oracle import Oracle

        self.cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(self.cores))
        n_inst = len(sysm.instances)
        insts = range(0, n_inst, max(1, n_inst // 8)) if n_inst > 8 else range(n_inst)
        self.oracles = []
        for k in insts:
            o = Oracle.from_instance(sysm, k)
            o.seed_streams(seed + k)  # MT19937 stream as init_mts.F90 derives it
            o.md_init()
            o.init_velocities()
            self.oracles.append(o)
        self.start = ("relaxed positions (sis_gb300/data/crowded_relaxed.npz)" if getattr(sysm, "relaxed_start", False)
                      else "the workload's start")

    def sample(self, max_seconds=30.0, max_steps=4000, chunk=10):
        """Per instance: steps in chunks until a rebuild happened (or the caps)."""
        bead_steps, secs, steps, rebuilds = 0, 0.0, 0, 0
        for o in self.oracles:
            t0 = time.perf_counter()
            s = r = 0
            while r == 0 and s < max_steps and time.perf_counter() - t0 < max_seconds:
                r += o.run(chunk)
                s += chunk
            secs += time.perf_counter() - t0
            bead_steps += o.nmp * s
            steps += s
            rebuilds += r
        return bead_steps, secs, steps, rebuilds

    def describe(self, steps, rebuilds):
        n = sum(o.nmp for o in self.oracles)
        return (f"{steps} MD steps over {len(self.oracles)} instance(s) ({n} beads) from {self.start}, velocities from the "
                f"oracle's MT19937 noise, after one untimed rebuild interval; each sample ran until the displacement trigger "
                f"rebuilt its lists ({rebuilds} O(N^2) rebuilds timed); FP64 C++ restatement of the reference with OpenMP")


def cpu_samples(sysm, n_samples, warmup=1):
    """Timed samples of the CPU sampler after `warmup` untimed ones (the first
    leaves the start's transient and ends right after a rebuild)."""
    smp = CpuSampler(sysm)
    for w in range(warmup):
        smp.sample() if w == 0 else smp.sample(max_steps=2)
    tot_bs, tot_s, tot_steps, tot_reb = 0, 0.0, 0, 0
    for _ in range(n_samples):
        bs, secs, steps, reb = smp.sample()
        tot_bs, tot_s, tot_steps, tot_reb = tot_bs + bs, tot_s + secs, tot_steps + steps, tot_reb + reb
    return smp, tot_bs, tot_s, tot_steps, tot_reb


def cpu_baseline(args, sysm):
    smp, bs, secs, steps, reb = cpu_samples(sysm, 1)
    return {"value": bs / secs, "unit": UNIT, "cores": smp.cores, "kind": "port", "sample": smp.describe(steps, reb),
            "steps_per_rebuild": steps / reb if reb else None}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return None, rank
    sysm = make_system(args.workload)
    # warm-up: the first sample leaves the start's transient and ends right
    # after a rebuild, so every timed sample spans one rebuild interval
    smp, tot_bs, tot_s, tot_steps, tot_reb = cpu_samples(sysm, args.steps, args.warmup)
    value = tot_bs / tot_s
    cb = {"value": value, "unit": UNIT, "cores": smp.cores, "kind": "port", "sample": smp.describe(tot_steps, tot_reb),
          "steps_per_rebuild": tot_steps / tot_reb if tot_reb else None}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp64", "data": "synthetic (seeded sequences and random-coil starts)", "impl": "reference",
           "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "n_beads": sysm.nmp,
                      "start": smp.start, "steps_per_rebuild": cb["steps_per_rebuild"],
                      "note": "Fortran reference unavailable on this box (no Fortran compiler, toml-f not vendored); "
                              "timed arm is the FP64 C++ restatement of its algorithms"},
           "cpu_baseline": cb, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out, rank


def serve_run(args, rank, world, seconds, scale):
    from sis_gb300.coil import sis_options
    from sis_gb300.inputs import read_ff
    from sis_gb300.serve import Server, job_stream

    ff = read_ff(ROOT / "sis_gb300" / "data" / "sis.ff")
    jobs = job_stream(1005 + rank, args.serve_rate, seconds, steps_scale=scale)
    # one block per slot on the per-block kernel: 144 slots fill the 152 SMs
    classes = [(128, 32), (512, 48), (2048, 64)]
    # warm-up session (graph capture, first-touch of every pool), not timed
    warm = Server(ff, sis_options(), classes=classes, seed=2024 + rank, force_cap=args.force_cap)
    warm.run(job_stream(7, 20.0, 0.5, steps_scale=scale))
    warm.close()
    srv = Server(ff, sis_options(), classes=classes, seed=2024 + rank, force_cap=args.force_cap)
    barrier(world)
    with Clocks(dist_env()[2]) as clk:
        srv.run(jobs)
    summ = srv.summary()
    done_bead_steps = sum(r.job.nmp * r.job.nsteps for r in srv.results)
    srv.close()
    offered = sum(j.nmp * j.nsteps for j in jobs) / seconds
    # every rank serves its own stream; the slowest rank's wall time bounds the job
    value = world * done_bead_steps / max_over_ranks(summ["wall_s"], world)
    cfg = {"workload": "serve", "description": WORKLOADS["serve"], "jobs": len(jobs), "arrival_rate_per_s": args.serve_rate,
           "arrival_window_s": seconds, "steps_scale": scale,
           "offered_bead_steps_per_s": offered, "p50_latency_ms": summ["p50_ms"], "p99_latency_ms": summ["p99_ms"],
           "jobs_completed": summ["jobs"], "jobs_failed": summ["failed"], "force_cap": args.force_cap,
           "pool_classes": [{"capacity": c, "slots": n} for c, n in classes], "precision": "FP32 terms / FP64 accumulate+integrate",
           "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}
    return summ, cfg, value, (clk, jobs)


def run_serve(args):
    """The serving workload, scaled: Poisson arrivals at --serve-rate jobs/s for
    --serve-seconds, each job's step count times --serve-steps-scale; pools of
    slots in three length classes; latency = arrival to completion."""
    rank, world, local = dist_env()
    summ, cfg, value, (clk, jobs) = serve_run(args, rank, world, args.serve_seconds, args.serve_steps_scale)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 1,
           "ms_per_step": summ["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32+fp64", "data": "synthetic (seeded sequences and random-coil starts, Poisson arrivals)", "config": cfg,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(sum(j.nmp * 24 for j in jobs)),
                   "d2h_bytes_per_step": int(sum(j.nmp * 96 for j in jobs))},
           "clocks": clk.summary()}
    return out, rank


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="crowded", choices=list(WORKLOADS))
    ap.add_argument("--md-steps", type=int, default=100)
    ap.add_argument("--relax", type=int, default=-1,
                    help="relaxation steps before timing (-1: 500 free steps from a relaxed start, else 3000 capped + 3000 free)")
    ap.add_argument("--no-sub", action="store_true", help="leave out the uneven-batch and serving records of the default line")
    ap.add_argument("--force-cap", type=float, default=1000.0)
    ap.add_argument("--lanes", type=int, default=0, help="lanes per bead of the step kernel (0: autotune)")
    ap.add_argument("--no-graphs", action="store_true", help="launch every kernel from the host instead of step graphs")
    ap.add_argument("--overlap", type=int, default=-1, help="1/0: pair-force kernel beside the bonded pass or not (-1: the autotuner chooses)")
    ap.add_argument("--exchange-interval", type=int, default=1000, help="MD steps between replica-exchange attempts (remd)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="job arrivals per second (serve)")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window in seconds (serve)")
    ap.add_argument("--serve-steps-scale", type=float, default=0.01, help="factor on every job's step count (serve)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.impl == "reference":
        out, rank = run_reference(args)
    elif args.workload == "serve":
        out, rank = run_serve(args)
    else:
        out, rank = run_gpu(args)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
