"""The serving host logic (sis_gb300.serve) on the CPU, over a stand-in
engine whose beads move by one unit per step: pool choice by capacity, the
HBM budget, step chunks that end where a job finishes or saves a frame,
DCD frames per job, failed jobs retired while the others finish, and the
summary.  The device side of serving is tested on the GPU in test_serve.py."""
import numpy as np
import pytest

from sis_gb300 import serve
from sis_gb300._abi import SisError
from sis_gb300.dcd import read_dcd
from sis_gb300.model import Chain, Options


class SlotEngine:
    """One pool context: slot k holds a job's coordinates; every step adds 1
    to all of them.  A slot loaded with a stream in ``poison`` turns
    non-finite at its first step, and the step then reports it as the
    device does (SIS_ERR_NONFINITE after the steps ran)."""
    poison = set()
    made = []

    def __init__(self, system, precision=0, seed=1):
        self.cap = system.instances[0].nmp
        self.x = np.zeros((len(system.instances), self.cap, 3))
        self.stream = [0] * len(system.instances)
        self.steps = []
        SlotEngine.made.append(self)

    def set_lanes(self, lanes):
        pass

    def set_force_cap(self, f):
        pass

    def load_slot(self, k, chains, tempK, salt, stream, xyz, init_velocities=False):
        self.x[k] = 0.0
        if xyz is not None:
            self.x[k, :len(xyz)] = xyz
        self.stream[k] = stream

    def step(self, n):
        self.steps.append(n)
        self.x += n
        bad = [k for k, s in enumerate(self.stream) if s in self.poison]
        for k in bad:
            self.x[k] = np.nan
        if bad:
            raise SisError(-4, "non-finite displacement")

    def get_state(self, k):
        return self.x[k].copy(), None, None

    def close(self):
        pass


def _job(i, n, steps, arrival=0.0, save=0, path=None):
    return serve.Job(i, [Chain(np.zeros(n, dtype=np.int32))], np.zeros((n, 3)), 300.0, 0.15, steps,
                     arrival=arrival, save_interval=save, dcd_path=path)


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(serve, "Engine", SlotEngine)
    SlotEngine.made = []
    SlotEngine.poison = set()
    return SlotEngine


def test_jobs_go_to_the_smallest_pool_that_fits(fake):
    srv = serve.Server(None, Options(), [(64, 2), (16, 2)], max_chunk=100)
    assert [p.capacity for p in srv.pools] == [16, 64]
    assert srv._pool_for(_job(0, 16, 1)) == 0 and srv._pool_for(_job(1, 17, 1)) == 1
    with pytest.raises(ValueError, match="exceeds every slot capacity"):
        srv._pool_for(_job(2, 65, 1))


def test_hbm_budget_scales_the_slots_down(fake):
    budget = (16 * 8 + 64 * 8) * serve.BYTES_PER_BEAD / 4
    srv = serve.Server(None, Options(), [(16, 8), (64, 8)], hbm_budget=budget)
    assert [(p.capacity, p.n_slots) for p in srv.pools] == [(16, 2), (64, 2)]


def test_chunks_end_where_a_job_finishes_or_saves(fake):
    pool = serve.SlotPool(None, Options(), 8, 3)
    pool.admit(_job(0, 4, 250, save=40))
    pool.admit(_job(1, 8, 90))
    assert pool.next_chunk(1000) == 40
    pool.step(40)
    assert pool.next_chunk(1000) == 40
    pool.step(40)
    assert pool.next_chunk(1000) == 10  # job 1 ends at 90
    pool.step(10)
    x = pool.retire(1)
    assert x.shape == (8, 3) and np.all(x == 90.0)
    assert pool.free == [2, 1] and pool.next_chunk(1000) == 30
    assert pool.next_chunk(7) == 7


def test_serving_run_frames_and_results(fake, tmp_path):
    jobs = [_job(0, 10, 300, save=100, path=str(tmp_path / "j0.dcd")), _job(1, 30, 120, arrival=0.01),
            _job(2, 12, 50, save=25, path=str(tmp_path / "j2.dcd")), _job(3, 5, 80, arrival=0.02)]
    srv = serve.Server(None, Options(), [(16, 2), (32, 1)], max_chunk=64)
    res = srv.run(jobs)
    by_id = {r.job.id: r for r in res}
    assert sorted(by_id) == [0, 1, 2, 3] and not any(r.failed for r in res)
    for r in res:
        # every bead moved by the job's own step count, whatever it shared a launch with
        assert np.all(r.xyz == r.job.nsteps) and r.latency >= 0.0 and r.finished >= r.admitted
    frames, _ = read_dcd(tmp_path / "j0.dcd")
    assert by_id[0].frames == 3 and frames.shape == (3, 10, 3)
    assert np.allclose(frames[:, 0, 0], [100.0, 200.0, 300.0])
    frames2, _ = read_dcd(tmp_path / "j2.dcd")
    assert by_id[2].frames == 2 and np.allclose(frames2[:, 0, 0], [25.0, 50.0])
    assert all(n <= 64 for e in fake.made for n in e.steps)
    s = srv.summary()
    assert s["jobs"] == 4 and s["failed"] == 0
    assert s["bead_steps_per_s"] == pytest.approx((10 * 300 + 30 * 120 + 12 * 50 + 5 * 80) / srv.wall)
    assert s["p50_ms"] <= s["p99_ms"]


def test_a_failed_job_is_retired_and_the_others_finish(fake):
    fake.poison = {1}
    jobs = [_job(0, 8, 100), _job(1, 8, 100), _job(2, 8, 100, arrival=0.01)]
    srv = serve.Server(None, Options(), [(8, 2)], max_chunk=50)
    res = {r.job.id: r for r in srv.run(jobs)}
    assert res[1].failed and np.all(np.isnan(res[1].xyz))
    assert not res[0].failed and not res[2].failed
    assert srv.summary()["failed"] == 1 and srv.summary()["jobs"] == 2
