"""Continuous-batching simulation service.

Jobs (sequence, initial structure, temperature, salt, step count) arrive
while others run.  Device memory is held by pools of slots: a pool is one
context whose instances all have the same bead capacity, so a pool's
footprint is fixed when it is created and the pools together stay inside an
HBM budget.  A job is admitted into a free slot of the smallest pool that
fits it as soon as one is free (sis_gpu_load_slot rewrites the slot in
place), advances with every other job of its pool in the same launches, and
leaves its slot when its own step count is reached; pools run on their own
CUDA streams from their own host threads, so their work overlaps on the
device.  A job's noise stream is keyed by (job id, local bead, steps since
admission), so its trajectory is the same alone and in the mix.

Trajectory frames are copied from the device at each job's save interval and
written to its DCD file by a writer thread.  The service reports each job's
completion latency (arrival to last step) and the aggregate bead-steps/s.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import dcd
from ._abi import SisError
from .engine import Engine
from .model import MIXED, Chain, ForceField, Instance, Options, System

# resident bytes per bead slot (FP64 state, mirror, coefficients, forces,
# pair list at the default capacity): the pool sizing estimate
BYTES_PER_BEAD = 4096


@dataclass
class Job:
    id: int
    chains: List[Chain]
    xyz: np.ndarray
    tempK: float
    salt: float
    nsteps: int
    arrival: float = 0.0  # seconds after the service starts
    save_interval: int = 0  # MD steps between DCD frames (0: none)
    dcd_path: Optional[str] = None

    @property
    def nmp(self) -> int:
        return int(sum(len(c) for c in self.chains))


@dataclass
class Result:
    job: Job
    xyz: np.ndarray
    admitted: float
    finished: float
    frames: int = 0
    failed: bool = False  # the job's coordinates became non-finite

    @property
    def latency(self) -> float:
        return self.finished - self.job.arrival


class SlotPool:
    """One context of n_slots instances of `capacity` beads each."""

    def __init__(self, ff: ForceField, opts: Options, capacity: int, n_slots: int, seed: int = 1,
                 precision: int = MIXED, lanes: int = 8, force_cap: float = 0.0):
        self.capacity, self.n_slots = capacity, n_slots
        filler = [Chain(np.array([4], dtype=np.int32)) for _ in range(capacity)]
        insts = [Instance(list(filler), tempK=300.0, ionic_strength=0.15, xyz=np.zeros((capacity, 3)),
                          has_charge=np.zeros(capacity, dtype=bool)) for _ in range(n_slots)]
        self.eng = Engine(System(ff, opts, insts), precision=precision, seed=seed)
        self.eng.set_lanes(lanes)
        if force_cap > 0.0:  # per-bead force bound, a guard against singular geometries
            self.eng.set_force_cap(force_cap)
        for k in range(n_slots):
            self.eng.load_slot(k, [], 300.0, 0.15, 0, None)
        self.free = list(range(n_slots))
        self.active: Dict[int, dict] = {}
        self.step_count = 0

    def admit(self, job: Job) -> int:
        slot = self.free.pop(0)
        self.eng.load_slot(slot, job.chains, job.tempK, job.salt, job.id & 0x7fffffff, job.xyz, init_velocities=True)
        self.active[slot] = {"job": job, "left": job.nsteps, "done": 0}
        return slot

    def retire(self, slot: int) -> np.ndarray:
        job = self.active.pop(slot)["job"]
        x = self.eng.get_state(slot)[0][:job.nmp].copy()
        self.eng.load_slot(slot, [], 300.0, 0.15, 0, None)
        self.free.append(slot)
        return x

    def next_chunk(self, max_chunk: int) -> int:
        """Steps until the first job finishes or saves a frame."""
        n = max_chunk
        for a in self.active.values():
            n = min(n, a["left"])
            si = a["job"].save_interval
            if si:
                n = min(n, si - a["done"] % si)
        return max(1, n)

    def step(self, n: int):
        # sis_gpu_step reports an error after all n steps have run
        try:
            self.eng.step(n)
        finally:
            self.step_count += n
            for a in self.active.values():
                a["left"] -= n
                a["done"] += n

    def close(self):
        self.eng.close()


class Server:
    """Pools by capacity class; jobs go to the smallest class that fits."""

    def __init__(self, ff: ForceField, opts: Options, classes: Sequence[tuple], seed: int = 1, precision: int = MIXED,
                 max_chunk: int = 2000, hbm_budget: Optional[float] = None, force_cap: float = 0.0):
        """classes: (capacity, n_slots) pairs; with hbm_budget (bytes), n_slots
        is scaled down so that the pools fit in the budget."""
        classes = sorted(classes)
        if hbm_budget is not None:
            need = sum(c * s for c, s in classes) * BYTES_PER_BEAD
            if need > hbm_budget:
                f = hbm_budget / need
                classes = [(c, max(1, int(s * f))) for c, s in classes]
        self.pools = [SlotPool(ff, opts, c, s, seed=seed, precision=precision, force_cap=force_cap) for c, s in classes]
        self.max_chunk = max_chunk
        self.results: List[Result] = []
        self._lock = threading.Lock()
        self._writer_q: "queue.Queue" = queue.Queue()

    def _pool_for(self, job: Job) -> int:
        for p, pool in enumerate(self.pools):
            if pool.capacity >= job.nmp:
                return p
        raise ValueError(f"job {job.id} ({job.nmp} beads) exceeds every slot capacity")

    def _writer(self):
        files = {}
        while True:
            item = self._writer_q.get()
            if item is None:
                break
            kind, job, payload = item
            if kind == "open":
                f = open(job.dcd_path, "wb")
                dcd.write_header(f, job.nmp, False)
                files[job.id] = f
            elif kind == "frame":
                dcd.write_frame(files[job.id], payload)
            else:
                files.pop(job.id).close()

    def _run_pool(self, p: int, pending: List[Job], t0: float):
        pool = self.pools[p]
        frames: Dict[int, int] = {}
        while pending or pool.active:
            now = time.perf_counter() - t0
            while pool.free and pending and pending[0].arrival <= now:
                job = pending.pop(0)
                slot = pool.admit(job)
                pool.active[slot]["admitted"] = time.perf_counter() - t0
                frames[job.id] = 0
                if job.dcd_path and job.save_interval:
                    self._writer_q.put(("open", job, None))
            if not pool.active:
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                continue
            n = pool.next_chunk(self.max_chunk)
            try:
                pool.step(n)
            except SisError as e:
                if e.code != -4:
                    raise
                # retire the jobs whose coordinates became non-finite
                bad = [k for k in pool.active if not np.all(np.isfinite(pool.eng.get_state(k)[0]))]
                if not bad:
                    raise
                for slot in bad:
                    job = pool.active[slot]["job"]
                    admitted = pool.active[slot]["admitted"]
                    pool.retire(slot)
                    if job.dcd_path and job.save_interval:
                        self._writer_q.put(("close", job, None))
                    with self._lock:
                        self.results.append(Result(job, np.full((job.nmp, 3), np.nan), admitted, time.perf_counter() - t0,
                                                   frames[job.id], failed=True))
                continue
            for slot in list(pool.active):
                a = pool.active[slot]
                job = a["job"]
                if job.dcd_path and job.save_interval and a["done"] % job.save_interval == 0:
                    self._writer_q.put(("frame", job, pool.eng.get_state(slot)[0][:job.nmp].copy()))
                    frames[job.id] += 1
                if a["left"] == 0:
                    admitted = a["admitted"]
                    x = pool.retire(slot)
                    if job.dcd_path and job.save_interval:
                        self._writer_q.put(("close", job, None))
                    with self._lock:
                        self.results.append(Result(job, x, admitted, time.perf_counter() - t0, frames[job.id]))

    def run(self, jobs: Sequence[Job]) -> List[Result]:
        """Serves `jobs` (arrival times relative to now) until all are done."""
        per_pool: List[List[Job]] = [[] for _ in self.pools]
        for job in sorted(jobs, key=lambda j: j.arrival):
            per_pool[self._pool_for(job)].append(job)
        writer = threading.Thread(target=self._writer, daemon=True)
        writer.start()
        t0 = time.perf_counter()
        threads = [threading.Thread(target=self._run_pool, args=(p, per_pool[p], t0)) for p in range(len(self.pools))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        self._writer_q.put(None)
        writer.join()
        self.wall = time.perf_counter() - t0
        return self.results

    def summary(self) -> dict:
        ok = [r for r in self.results if not r.failed]
        lat = np.array([r.latency for r in ok])
        bead_steps = sum(r.job.nmp * r.job.nsteps for r in ok)
        return {"jobs": len(ok), "failed": len(self.results) - len(ok), "wall_s": self.wall,
                "bead_steps_per_s": bead_steps / self.wall,
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None}

    def close(self):
        for pool in self.pools:
            pool.close()


def job_stream(ff_seed: int, rate: float, seconds: float, lmin: int = 20, lmax: int = 2000, smin: float = 1e4,
               smax: float = 1e6, tmin: float = 280.0, tmax: float = 360.0, salt_min: float = 0.02, salt_max: float = 0.5,
               steps_scale: float = 1.0, max_len: Optional[int] = None) -> List[Job]:
    """Poisson arrivals at `rate` jobs/s for `seconds`: lengths log-uniform in
    [lmin, lmax], steps log-uniform in [smin, smax] (times steps_scale), T and
    salt uniform; seeded sequences and random-coil starts whose non-bonded
    pairs are at least the WCA sigma apart."""
    from .coil import random_coil, random_sequence

    rng = np.random.default_rng(ff_seed)
    jobs, t, k = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        n = int(round(np.exp(rng.uniform(np.log(lmin), np.log(lmax)))))
        if max_len:
            n = min(n, max_len)
        steps = max(1, int(round(np.exp(rng.uniform(np.log(smin), np.log(smax))) * steps_scale)))
        jobs.append(Job(k, [Chain(random_sequence(rng, n))], random_coil(rng, n, rmin=10.0), float(rng.uniform(tmin, tmax)),
                        float(rng.uniform(salt_min, salt_max)), steps, arrival=t))
        k += 1
    return jobs
