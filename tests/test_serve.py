"""Continuous batching (sis_gpu_load_slot, sis_gb300.serve): a job gives the
same result alone and admitted into a running pool next to other jobs.

The mixed path is deterministic per instance (FP32 lane sums in a fixed
order, exact fixed-point base-pair sums, per-instance lists and trigger), the
filler beads of a slot join no term, and a job's noise is keyed by its own
stream and its steps since admission; so the states agree bit for bit.
"""
import numpy as np
import pytest

from sis_gb300 import MIXED
from sis_gb300.coil import random_coil, random_sequence, sis_options
from sis_gb300.dcd import read_dcd
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, System
from sis_gb300.serve import Job, Server, SlotPool

pytestmark = pytest.mark.gpu
SEED = 11


def make_job(rng, k, n, nsteps, arrival=0.0):
    return Job(k, [Chain(random_sequence(rng, n))], random_coil(rng, n, rmin=10.0), float(rng.uniform(280, 360)),
               float(rng.uniform(0.02, 0.5)), nsteps, arrival=arrival)


def alone(ff, opts, job):
    eng = Engine(System(ff, opts, [Instance(job.chains, tempK=job.tempK, ionic_strength=job.salt, xyz=job.xyz)]),
                 precision=MIXED, seed=SEED, streams=[job.id & 0x7fffffff])
    eng.set_lanes(8)
    eng.init_velocities()
    eng.step(job.nsteps)
    x = eng.get_state(0)[0]
    eng.close()
    return x


def test_job_same_alone_and_in_mix(sis_ff):
    opts = sis_options()
    rng = np.random.default_rng(5)
    a, b, c = make_job(rng, 1, 40, 200), make_job(rng, 2, 64, 120), make_job(rng, 3, 23, 57)
    pool = SlotPool(sis_ff, opts, capacity=96, n_slots=3, seed=SEED)
    sa = pool.admit(a)
    pool.step(40)
    sb = pool.admit(b)
    pool.step(60)
    sc = pool.admit(c)
    pool.step(57)  # c: 57 steps
    xc = pool.retire(sc)
    pool.step(3)  # b: 120 steps
    xb = pool.retire(sb)
    pool.step(40)  # a: 200 steps
    xa = pool.retire(sa)
    assert sorted(pool.free) == [0, 1, 2]
    pool.close()
    for job, x in ((a, xa), (b, xb), (c, xc)):
        assert np.array_equal(x, alone(sis_ff, opts, job)), job.id


def test_server_serves_a_stream(sis_ff, tmp_path):
    opts = sis_options()
    rng = np.random.default_rng(8)
    jobs = []
    for k in range(12):
        n = int(rng.integers(20, 180))
        job = make_job(rng, 100 + k, n, int(rng.integers(100, 400)), arrival=0.02 * k)
        job.save_interval = 50
        job.dcd_path = str(tmp_path / f"job{job.id}.dcd")
        jobs.append(job)
    srv = Server(sis_ff, opts, classes=[(64, 3), (192, 2)], seed=SEED, max_chunk=64)
    res = srv.run(jobs)
    summ = srv.summary()
    srv.close()
    assert len(res) == len(jobs)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0 and summ["bead_steps_per_s"] > 0
    by_id = {r.job.id: r for r in res}
    for job in jobs[:3]:
        r = by_id[job.id]
        assert r.finished >= r.admitted >= job.arrival
        assert np.array_equal(r.xyz, alone(sis_ff, opts, job))
        frames, _ = read_dcd(job.dcd_path)
        assert len(frames) == job.nsteps // 50 == r.frames
        if len(frames):
            assert np.allclose(frames[-1], r.xyz, atol=1e-3) or job.nsteps % 50 != 0
