"""The MD job (sis_gb300.job_md) and the files around it.

CPU, against a stand-in engine that records every call:
* the job runs the steps between two events as one Engine.step call and
  still acts at exactly the steps of job_md.F90's one-step-at-a-time loop
  (restated below): frames, restart files, replica label table and
  exchanges (alternating pair patterns), annealing and timed Rg-bias
  stages, tweezers records;
* a STOP_SIS file or the wall-clock limit stops the run at the next check
  step, after writing the restart file;
* a restarted run writes no step-0 frame and resumes its annealing stage
  and replica labels;
* .rep, .twz, schedule files and the .out optional columns; .rst readers
  refuse truncated or inconsistent files.
GPU: the annealing temperature update and a short job on the real engine.
"""
import os
import struct
from pathlib import Path

import numpy as np
import pytest

from sis_gb300 import job_md
from sis_gb300.job_md import MdControl, MdJob
from sis_gb300.model import ForceRampPair
from sis_gb300.outputs import (RepFile, TwzFile, fortran_g, read_out, read_rst, read_schedule, restart_engine,
                               write_rst)


# ------------------------------------------------------------ stand-in
class _Opts:
    flg_ele = True


class _Inst:
    def __init__(self, n, tempK, box=None):
        self.n, self.tempK, self.ionic_strength, self.box = n, tempK, 0.15, box


class _System:
    def __init__(self, insts):
        self.opts = _Opts()
        self.instances = insts


class FakeEngine:
    """Records what the job asks for, with the step it was at.  The
    coordinates of bead i at step s are (s, i, 0), so a record of positions
    names the step it was taken at."""

    def __init__(self, n_inst=1, n=5, temps=None, fr=None, box=None):
        temps = temps or [300.0] * n_inst
        self.system = _System([_Inst(n, t, box) for t in temps])
        self.n_inst = n_inst
        self.offsets = np.arange(n_inst + 1) * n
        self.n = n * n_inst
        self.s = 0
        self.log = []
        self.steps = []
        self.fr = fr or {}
        self.rg_state = {}
        self.labels = None

    def nmp(self, inst=-1):
        return self.n if inst < 0 else int(self.offsets[inst + 1] - self.offsets[inst])

    def get_step(self):
        return self.s

    def set_step(self, s):
        self.s = s

    def set_state(self, inst, x=None, v=None, a=None):
        self.log.append(("set_state", self.s))

    def step(self, n):
        assert n > 0
        self.steps.append(n)
        self.s += n

    def get_state(self, inst=-1):
        x = np.zeros((self.nmp(inst), 3))
        x[:, 0] = self.s
        x[:, 1] = np.arange(x.shape[0]) % self.nmp(0)
        return x, 0.5 * x, 0.25 * x

    def energy_sumup(self, k, tK):
        if k == 0:
            self.log.append(("save", self.s))
        return np.array([self.s + 0.5] + [float(i) for i in range(1, 11)])

    def energy_kinetic(self, k):
        return 1.25

    def rg(self, k):
        return np.array([7.5])

    def get_list(self, k, kind):
        return np.array([[3, 10, 0, 0, 0, 0, 0]], dtype=np.int32)

    def get_bp_status(self, k):
        return np.array([1], dtype=np.uint8)

    def get_bp_energies(self, k):
        return np.array([-2.5])

    def set_condition(self, k, tK, ionic):
        if self.labels is None:
            self.log.append(("cond", self.s, k, tK))
        self.system.instances[k].tempK = tK

    def neighbor_list(self, inst=-1):
        self.log.append(("nl", self.s))

    def set_temperature(self, inst, tK):
        self.log.append(("temp", self.s, tK))
        for i in self.system.instances:
            i.tempK = tK

    def set_rg_bias(self, inst, k, rg0, flat=False, off=False):
        self.log.append(("rg", self.s, k, rg0, flat))
        for q in range(self.n_inst):
            self.rg_state[q] = (k, rg0, flat)

    def rg_bias(self, inst):
        return self.rg_state.get(inst)

    def tweezers(self, inst):
        return [], self.fr.get(inst, [])

    def optional_terms(self):
        return {"stage": False, "twz": bool(self.fr), "rg": bool(self.rg_state), "rest": False}

    def remd_init(self, temps):
        self.temps = list(temps)
        self.labels = [self.temps.index(i.tempK) for i in self.system.instances]

    def remd_exchange(self, parity):
        self.log.append(("exch", self.s, parity))
        # swap every pair of labels of the pattern
        lab2rep = {lab: r for r, lab in enumerate(self.labels)}
        for l in range(parity, self.n_inst - 1, 2):
            a, b = lab2rep[l], lab2rep[l + 1]
            self.labels[a], self.labels[b] = l + 1, l
        return np.array(self.labels, dtype=np.int32), (self.n_inst - parity) // 2


# ------------------------------------------- the reference's loop, restated
def reference_events(c, istep, restarted=False, nrep=0, twz=False, stop_at=None, ianneal0=None):
    """Events of job_md.F90:360-680 taken one step at a time.  stop_at(step)
    says whether the stop check of that step finds a reason to stop;
    ianneal0 is the annealing stage a restart file holds."""
    ev = [("nl", istep)]
    anneal_on, ianneal, next_anneal = c.anneal is not None, 1, None
    if c.anneal is not None:
        # main.F90:97: set up at the first stage's temperature
        ev.append(("cond", istep, 0, c.anneal[0][1]))
        n = len(c.anneal)
        if istep >= c.anneal[-1][0]:
            ianneal, anneal_on = n, False
        elif restarted and ianneal0 is not None:
            ianneal = ianneal0
        ev.append(("temp", istep, c.anneal[ianneal - 1][1]))
        if ianneal < n:
            next_anneal = c.anneal[ianneal][0]
    itrg, next_trg = 1, None
    if c.timed_bias_rg is not None:
        n = len(c.timed_bias_rg)
        if istep >= c.timed_bias_rg[-1][0]:
            itrg = n
        ev.append(("rg", istep, *c.timed_bias_rg[itrg - 1][1:], False))
        if itrg < n:
            next_trg = c.timed_bias_rg[itrg][0]
    if not restarted:
        ev.append(("save", istep))
    nexch = 0
    while istep < c.nstep:
        istep += 1
        if twz and istep % c.nstep_save == 0:
            ev.append(("twz", istep))
        if istep % c.nstep_save == 0:
            ev.append(("save", istep))
        if nrep and c.nstep_rep_exchange > 0:
            if c.nstep_rep_save > 0 and istep % c.nstep_rep_save == 0:
                ev.append(("rep", istep))
            if istep % c.nstep_rep_exchange == 0:
                ev.append(("exch", istep, nexch % 2))
                nexch += 1
        if anneal_on and next_anneal is not None and istep + 1 == next_anneal:
            ianneal += 1
            ev.append(("temp", istep, c.anneal[ianneal - 1][1]))
            if ianneal < len(c.anneal):
                next_anneal = c.anneal[ianneal][0]
            else:
                anneal_on = False
        if next_trg is not None and istep + 1 == next_trg:
            itrg += 1
            ev.append(("rg", istep, *c.timed_bias_rg[itrg - 1][1:], False))
            next_trg = c.timed_bias_rg[itrg][0] if itrg < len(c.timed_bias_rg) else None
        stop = istep % c.nstep_check_stop == 0 and stop_at is not None and stop_at(istep)
        if istep % c.nstep_save_rst == 0 or stop:
            ev.append(("rst", istep))
        if stop:
            break
    return ev


def _run(tmp_path, monkeypatch, c, eng, **kw):
    rst_log = []
    real = job_md.write_rst

    def logged(path, step, *a, **k):
        if str(path).endswith(("_0001.rst", "md.rst")):
            rst_log.append(("rst", step))
        return real(path, step, *a, **k)

    monkeypatch.setattr(job_md, "write_rst", logged)
    job = MdJob(eng, str(tmp_path / "md"), c, log=lambda s: None, **kw)
    why = job.run()
    got = list(eng.log)
    twz = tmp_path / "md.twz"
    if twz.exists():
        got += [("twz", int(line.split()[0])) for line in twz.read_text().splitlines()[1:]
                if line.split()[1] == "1"]
    got += [("rep", int(line.split()[0])) for line in
            ((tmp_path / "md.rep").read_text().splitlines() if (tmp_path / "md.rep").exists() else [])]
    return why, got + rst_log, job


def _order(ev):
    kind = {"cond": 0, "nl": 0, "temp": 0, "rg": 0, "twz": 1, "save": 2, "rep": 3, "exch": 4, "rst": 5}
    return sorted(ev, key=lambda e: (e[1], kind[e[0]], e[2:]))


CASES = [
    MdControl(nstep=1000, nstep_save=100, nstep_save_rst=250, nstep_check_stop=300),
    MdControl(nstep=997, nstep_save=70, nstep_check_stop=1000, anneal=[(0, 400.0), (150, 350.0), (400, 300.0)]),
    MdControl(nstep=600, nstep_save=50, nstep_save_rst=600, timed_bias_rg=[(0, 1.0, 20.0), (101, 2.0, 15.0),
                                                                          (102, 3.0, 12.0), (300, 0.5, 30.0)]),
    MdControl(nstep=15, nstep_save=1, nstep_save_rst=4, nstep_check_stop=3, anneal=[(0, 300.0), (1, 310.0),
                                                                                   (2, 320.0)]),
]


@pytest.mark.parametrize("c", CASES)
def test_events_match_the_one_step_loop(c, tmp_path, monkeypatch):
    eng = FakeEngine()
    why, got, _ = _run(tmp_path, monkeypatch, c, eng)
    assert why == "end"
    assert _order(got) == _order(reference_events(c, 0))
    # every Engine.step call stays between two events
    assert sum(eng.steps) == c.nstep
    assert len(eng.steps) <= c.nstep // c.nstep_save + len(got) + 1


def test_random_schedules_match_the_one_step_loop(tmp_path, monkeypatch):
    """40 seeded random controls, with and without annealing, timed Rg
    bias, tweezers records, replicas and a STOP_SIS file."""
    rng = np.random.default_rng(11)
    fr = [ForceRampPair(1, 5, (0.3, 0.2), ((0.0, 0.0, 20.0), (60.0, 5.0, 25.0)), ((0.01, 0.0, 0.0), (0.0, 0.0, 0.0)))]
    for case in range(40):
        d = tmp_path / f"c{case}"
        d.mkdir()
        nstep = int(rng.integers(1, 400))
        kw = dict(nstep=nstep, nstep_save=int(rng.integers(1, 60)), nstep_save_rst=int(rng.integers(1, 200)),
                  nstep_check_stop=int(rng.integers(1, 150)), step_progress=int(rng.integers(0, 50)))
        nrep = 0
        if rng.random() < 0.4:
            steps = sorted(set(int(v) for v in rng.integers(0, nstep + 5, size=int(rng.integers(1, 5)))))
            kw["anneal"] = [(st, 300.0 + 5 * k) for k, st in enumerate(steps)]
        elif rng.random() < 0.5:
            nrep = int(rng.integers(2, 5))
            kw["nstep_rep_exchange"] = int(rng.integers(1, 40))
            kw["nstep_rep_save"] = int(rng.integers(0, 40))
        if rng.random() < 0.4 and not nrep:
            steps = sorted(set(int(v) for v in rng.integers(0, nstep + 5, size=int(rng.integers(1, 5)))))
            kw["timed_bias_rg"] = [(st, 1.0 + k, 10.0 + k) for k, st in enumerate(steps)]
        twz = rng.random() < 0.3
        kw["out_twz"] = twz
        stop = rng.random() < 0.2
        if stop:
            (d / "STOP_SIS").write_text("")
        c = MdControl(**kw)
        temps = [300.0 + 10 * k for k in range(nrep)] if nrep else None
        eng = FakeEngine(n_inst=max(nrep, 1), temps=temps, fr={0: fr} if twz else None)
        monkeypatch.undo()
        why, got, _ = _run(d, monkeypatch, c, eng, replica_temps=temps)
        want = reference_events(c, 0, nrep=nrep, twz=twz, stop_at=(lambda s: True) if stop else None)
        assert _order(got) == _order(want), (case, kw)
        assert why == ("stop_file" if stop and c.nstep >= c.nstep_check_stop else "end")


def test_replica_exchange_events_and_label_table(tmp_path, monkeypatch):
    c = MdControl(nstep=400, nstep_save=100, nstep_rep_exchange=30, nstep_rep_save=60, nstep_check_stop=1000)
    temps = [300.0, 310.0, 320.0, 330.0]
    eng = FakeEngine(n_inst=4, temps=[310.0, 300.0, 330.0, 320.0])
    why, got, job = _run(tmp_path, monkeypatch, c, eng, replica_temps=temps)
    assert _order(got) == _order(reference_events(c, 0, nrep=4))
    # files per replica: prefix_0001 ... (init_out_files.F90:62-64)
    assert sorted(p.name for p in tmp_path.glob("md_*.out")) == [f"md_000{k}.out" for k in range(1, 5)]
    rep = (tmp_path / "md.rep").read_text().splitlines()
    # written before the exchange of step 60, after the one of step 30
    assert rep[0] == "          60     1     2     3     4"
    # the .out rows carry each replica's label and the label's temperature
    cols = read_out(tmp_path / "md_0001.out")
    assert list(cols["R"][:1]) == [2] and list(cols["T"][:1]) == [310.0]
    r = read_rst(tmp_path / "md_0001.rst")
    assert r.rep2lab == [lab + 1 for lab in job.labels]


def test_stop_file_stops_at_the_next_check_and_writes_the_restart(tmp_path, monkeypatch):
    (tmp_path / "STOP_SIS").write_text("")
    c = MdControl(nstep=1000, nstep_save=40, nstep_save_rst=1000, nstep_check_stop=150)
    msgs = []
    eng = FakeEngine()
    why = MdJob(eng, str(tmp_path / "md"), c, log=msgs.append).run()
    assert why == "stop_file" and eng.s == 150
    assert msgs == ["STOP_SIS file was found at step           150. Stop the job."]
    assert read_rst(tmp_path / "md.rst").step == 150
    assert list(read_out(tmp_path / "md.out")["nframe"]) == [0, 40, 80, 120]
    eng2 = FakeEngine()
    _, got, _ = _run(tmp_path, monkeypatch, c, eng2)
    assert _order(got) == _order(reference_events(c, 0, stop_at=lambda s: True))


def test_wall_time_limit(tmp_path, monkeypatch):
    """The limit is whole seconds (stop_wall_time_hour x 3600); the clock is
    read at the check steps only."""
    eng = FakeEngine()
    clock = lambda: eng.s * 2.0  # two seconds per step  # noqa: E731
    c = MdControl(nstep=10000, nstep_save=500, nstep_check_stop=100, stop_wall_time_hour=0.1)  # 360 s
    msgs = []
    why = MdJob(eng, str(tmp_path / "md"), c, clock=clock, log=msgs.append).run()
    assert why == "wall_time" and eng.s == 200  # 400 s > 360 s at the check of step 200
    assert msgs == ["Wall-clock time limit reached at step           200. Stop the job."]
    assert read_rst(tmp_path / "md.rst").step == 200


def test_threaded_and_inline_writers_write_the_same_files(tmp_path):
    fr = [ForceRampPair(1, 5, (0.3, 0.2), ((0.0, 0.0, 20.0), (60.0, 5.0, 25.0)), ((0.01, 0.0, 0.0), (0.0, 0.0, 0.0)))]
    c = MdControl(nstep=500, nstep_save=25, nstep_save_rst=100, nstep_rep_exchange=10, nstep_rep_save=20,
                  out_twz=True, out_bpall=True, out_bpe=True)
    files = {}
    for threaded in (False, True):
        d = tmp_path / str(threaded)
        d.mkdir()
        eng = FakeEngine(n_inst=2, temps=[300.0, 310.0], fr={0: fr})
        MdJob(eng, str(d / "md"), c, replica_temps=[300.0, 310.0], log=lambda s: None,
              threaded_writer=threaded).run()
        files[threaded] = {p.name: p.read_bytes() for p in sorted(d.iterdir())}
    assert files[False] == files[True]
    assert sorted(files[True]) == ["md.rep", "md.twz"] + [f"md_000{k}.{x}" for k in (1, 2) for x in
                                                          ("bp", "bpall", "bpe", "dcd", "out", "rst")]


def test_a_failed_write_is_raised(tmp_path, monkeypatch):
    from sis_gb300 import outputs
    calls = []
    real = outputs.OutFile.write

    def failing(self, *a, **k):
        calls.append(1)
        if len(calls) == 3:
            raise OSError("disk full")
        return real(self, *a, **k)

    monkeypatch.setattr(outputs.OutFile, "write", failing)
    c = MdControl(nstep=200, nstep_save=10)
    with pytest.raises(OSError, match="disk full"):
        MdJob(FakeEngine(), str(tmp_path / "md"), c, log=lambda s: None).run()
    assert len(calls) == 3  # the writes after the failed one are dropped


def test_progress_lines(tmp_path):
    """progress.F90: a five-line header, then per [Progress] step the step,
    million steps per day since the previous line and since the start, and
    the hours left at the average rate."""
    eng = FakeEngine()
    clock = lambda: eng.s * (0.864 if eng.s <= 200 else 1.728)  # noqa: E731
    msgs = []
    c = MdControl(nstep=400, nstep_save=400, nstep_check_stop=1000, step_progress=100)
    MdJob(eng, str(tmp_path / "md"), c, clock=clock, log=msgs.append).run()
    assert msgs[:5] == ["# PROGRESS", "#1: step", "#2: million steps / day (latest cycle)",
                        "#3: million steps / day (averaged)", "#4: remaining time / hours"]
    # 100 steps per 86.4 s is 0.1 million steps per day; 300 steps left
    # at that rate are 0.072 hours
    assert msgs[5] == "         100 " + fortran_g(0.1) + " " + fortran_g(0.1) + "    0.1"
    assert msgs[6] == "         200 " + fortran_g(0.1) + " " + fortran_g(0.1) + "    0.0"
    # step 300 at 518.4 s: the last 100 steps took 345.6 s (0.025 million
    # steps per day), all 300 took 518.4 s (0.05)
    assert msgs[7].split() == ["300", "0.250000E-01", "0.500000E-01", "0.0"]
    assert [m.split()[0] for m in msgs[5:]] == ["100", "200", "300", "400"]


def test_restart_resumes_annealing_stage_and_skips_the_first_frame(tmp_path, monkeypatch):
    c = MdControl(nstep=500, nstep_save=100, nstep_check_stop=1000,
                  anneal=[(0, 400.0), (150, 350.0), (400, 300.0)])
    eng = FakeEngine()
    MdJob(eng, str(tmp_path / "md"), MdControl(**{**c.__dict__, "nstep": 300}), log=lambda s: None).run()
    r = read_rst(tmp_path / "md.rst")
    assert r.step == 300 and r.ianneal == 2  # stage 2 is on until step 399
    eng2 = FakeEngine()
    restart_engine(eng2, tmp_path / "md.rst")
    assert eng2.log == [("set_state", 0)] and eng2.s == 300
    eng2.log.clear()
    out2 = tmp_path / "b"
    out2.mkdir()
    why, got, _ = _run(out2, monkeypatch, c, eng2, restart=r)
    assert why == "end"
    want = reference_events(c, 300, restarted=True, ianneal0=2)
    assert _order(got) == _order(want)
    assert ("temp", 300, 350.0) in want and ("temp", 399, 300.0) in want
    assert list(read_out(out2 / "md.out")["nframe"]) == [400, 500]
    # past the last stage the file holds no annealing block
    assert read_rst(out2 / "md.rst").ianneal is None


def test_replica_labels_restored_from_the_restart(tmp_path, monkeypatch):
    temps = [300.0, 310.0, 320.0]
    x = np.zeros((5, 3))
    write_rst(tmp_path / "r.rst", 90, x, x, x, grep=1, rep2lab=[3, 1, 2])
    r = read_rst(tmp_path / "r.rst")
    eng = FakeEngine(n_inst=3, temps=[300.0, 310.0, 320.0])
    eng.set_step(90)
    job = MdJob(eng, str(tmp_path / "md"), MdControl(nstep=100, nstep_save=10, nstep_rep_exchange=1000),
                replica_temps=temps, restart=r, log=lambda s: None)
    assert job.labels == [2, 0, 1]
    assert [i.tempK for i in eng.system.instances] == [320.0, 300.0, 310.0]


def test_twz_records_take_the_positions_the_step_starts_from(tmp_path, monkeypatch):
    fr = [ForceRampPair(1, 5, (0.3, 0.2), ((0.0, 0.0, 20.0), (60.0, 5.0, 25.0)), ((0.01, 0.0, 0.0), (-0.02, 0.01, 0.0)))]
    c = MdControl(nstep=300, nstep_save=100, nstep_check_stop=1000, out_twz=True)
    eng = FakeEngine(fr={0: fr})
    why, got, _ = _run(tmp_path, monkeypatch, c, eng)
    assert _order(got) == _order(reference_events(c, 0, twz=True))
    lines = (tmp_path / "md.twz").read_text().splitlines()
    assert lines[0] == TwzFile.HEADER
    # the restart file keeps where the traps started
    assert np.array_equal(read_rst(tmp_path / "md.rst").twz_init[1], [fr[0].init])
    # the record of step 200: beads at step 199, traps at step 200
    x = np.zeros((5, 3))
    x[:, 0] = 199
    x[:, 1] = np.arange(5)
    p = tmp_path / "expect.twz"
    w = TwzFile(p)
    w.write(200, x, fr)
    w.close()
    assert lines[2] == p.read_text().splitlines()[1]
    f = lines[2].split()
    p1 = np.array([0.0, 0.0, 20.0]) + 200 * np.array([0.01, 0.0, 0.0])
    d1 = np.linalg.norm(p1 - x[0])
    assert float(f[4]) == pytest.approx(d1, rel=1e-7)
    assert float(f[6]) == pytest.approx(0.3 * d1 / (job_md_pn()), rel=1e-7)


def job_md_pn():
    # kcal/mol/A -> pN: JOUL2KCAL_MOL x 1e-22
    return (1.0 / 4184.0) * 6.02214076e23 * 1.0e-22


def test_twz_line_format(tmp_path):
    fr = [ForceRampPair(1, 2, (1.0, 2.0), ((0.0, 0.0, 0.0), (10.0, 0.0, 0.0)), ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0)))]
    x = np.array([[0.0, 3.0, 4.0], [10.0, 0.0, 0.0]])
    p = tmp_path / "a.twz"
    w = TwzFile(p)
    w.write(7, x, fr)
    w.close()
    line = p.read_text().splitlines()[1]
    # (i13, x, i3, 6(x, g15.8))
    assert line[:17] == "            7   1"
    vals = [10.0, np.sqrt(125.0), 5.0, 0.0, 5.0 / job_md_pn(), 0.0]
    assert line[17:] == "".join(" " + fortran_g(v, 15, 8) for v in vals)
    assert len(line) == 13 + 1 + 3 + 6 * 16


def test_twz_uses_the_minimum_image():
    from sis_gb300.outputs import pbc_vec_d
    v = pbc_vec_d([1.0, 99.0, 50.0], [99.0, 1.0, 0.0], [100.0, 100.0, 100.0])
    assert np.array_equal(v, [2.0, -2.0, 50.0])


def test_rep_file_format(tmp_path):
    p = tmp_path / "a.rep"
    w = RepFile(p)
    w.write(123, [1, 2, 3])
    w.write(10 ** 13, [12345, 2])
    w.close()
    assert p.read_text() == "         123     1     2     3\n************ 12345     2\n"


def test_schedule_files(tmp_path):
    p = tmp_path / "anneal.txt"
    p.write_text("0 400.0\n1000, 350.0 extra ignored\n\n2000\n300.0\n")
    assert read_schedule(p, 2) == [(0, 400.0), (1000, 350.0), (2000, 300.0)]
    p.write_text("0 1.0 20.0\n500 2.0 15.0\n")
    assert read_schedule(p, 3) == [(0, 1.0, 20.0), (500, 2.0, 15.0)]
    for bad, n in (("0 -1.0\n", 2), ("-5 300.0\n", 2), ("0 -1.0 20.0\n", 3), ("0 1.0 0.0\n", 3), ("0 x\n", 2),
                   ("0\n", 2)):
        p.write_text(bad)
        with pytest.raises(ValueError):
            read_schedule(p, n)


def test_control_validation():
    with pytest.raises(ValueError):
        MdControl(nstep=10, nstep_save=0)
    with pytest.raises(ValueError):
        MdControl(nstep=10, nstep_save=1, anneal=[(0, -1.0)])
    with pytest.raises(ValueError):
        MdControl(nstep=10, nstep_save=1, timed_bias_rg=[(0, 1.0, 0.0)])
    assert MdControl(nstep=10, nstep_save=5).nstep_save_rst == 5
    with pytest.raises(ValueError):
        MdJob(FakeEngine(), "x", MdControl(nstep=10, nstep_save=5, nstep_rep_exchange=2))


def test_out_optional_columns(tmp_path):
    from sis_gb300.outputs import OutFile
    p = tmp_path / "a.out"
    w = OutFile(p, ele=True, stage=True, twz=True, rg=True, rest=True)
    w.write(5, 300.0, 1.0, [float(i) for i in range(11)], rg=12.5)
    w.close()
    head, row = p.read_text().splitlines()
    assert head.endswith(" (10)Eele      (11)Estage    (12)Etweezers (13)Erg       (14)Rg        (15)Erest    ")
    vals = row.split()
    assert [float(v) for v in vals[-6:]] == [6.0, 7.0, 8.0, 9.0, 12.5, 10.0]
    cols = read_out(p)
    assert list(cols)[-6:] == ["Eele", "Estage", "Etweezers", "Erg", "Rg", "Erest"]


# --------------------------------------------------------- .rst robustness
def _rst_bytes(tmp_path):
    x = np.arange(12.0).reshape(4, 3)
    p = tmp_path / "ok.rst"
    write_rst(p, 77, x, x, x, ianneal=2, box=[10.0, 10.0, 10.0])
    return p.read_bytes()


def test_rst_anneal_block(tmp_path):
    b = _rst_bytes(tmp_path)
    # STEP block, then ANNEAL (id 2, size 4, stage)
    assert struct.unpack("<iii", b[20:32]) == (2, 4, 2)
    r = read_rst(tmp_path / "ok.rst")
    assert r.ianneal == 2 and r.step == 77


@pytest.mark.parametrize("cut", [3, 8, 19, 40, -1])
def test_truncated_rst_raises(tmp_path, cut):
    b = _rst_bytes(tmp_path)
    p = tmp_path / "bad.rst"
    p.write_bytes(b[:cut])
    with pytest.raises(ValueError):
        read_rst(p)


def test_inconsistent_rst_raises(tmp_path):
    b = bytearray(_rst_bytes(tmp_path))
    off = 20 + 12  # the XYZ block header
    assert struct.unpack_from("<ii", b, off)[0] == 3
    bad = bytearray(b)
    struct.pack_into("<i", bad, off + 12, 5)  # nmp 5 for 4 beads of payload
    (tmp_path / "bad.rst").write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="beads"):
        read_rst(tmp_path / "bad.rst")
    bad = bytearray(b)
    struct.pack_into("<i", bad, 4, 13)  # step block size
    (tmp_path / "bad.rst").write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        read_rst(tmp_path / "bad.rst")
    (tmp_path / "empty.rst").write_bytes(b"")
    with pytest.raises(ValueError, match="no step block"):
        read_rst(tmp_path / "empty.rst")


def test_restart_engine_checks_the_bead_count(tmp_path):
    x = np.zeros((4, 3))
    write_rst(tmp_path / "a.rst", 5, x, x, x)
    with pytest.raises(ValueError, match="4 beads, the instance has 5"):
        restart_engine(FakeEngineWithState(), tmp_path / "a.rst")
    with pytest.raises(ValueError, match="replica 2"):
        restart_engine(FakeEngineWithState(), tmp_path / "a.rst", grep=2)


class FakeEngineWithState(FakeEngine):
    def set_state(self, inst, x, v, a):
        raise AssertionError("must not be reached")


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_set_temperature_moves_the_noise_and_leaves_electrostatics(sis_ff):
    from sis_gb300 import FP64
    from sis_gb300.coil import single_chain
    from sis_gb300.engine import Engine

    sysm = single_chain(sis_ff, n=24, seed=2)
    eng = Engine(sysm, precision=FP64)
    ele0, md0 = eng.get_ele(0), eng.get_md_coef(0)
    eng.set_temperature(-1, 4.0 * 300.0)
    assert np.array_equal(eng.get_ele(0), ele0)
    md1 = eng.get_md_coef(0)
    assert np.array_equal(md1[:, :3], md0[:, :3])
    assert np.allclose(md1[:, 3], 2.0 * md0[:, 3], rtol=1e-14)
    # set_condition moves both
    eng.set_condition(0, 1200.0, sysm.instances[0].ionic_strength)
    assert not np.array_equal(eng.get_ele(0), ele0)


@pytest.mark.gpu
def test_job_on_the_engine(sis_ff, tmp_path):
    """A short annealed job: the files hold what the engine computed, and a
    job stopped by a STOP_SIS file at step 50 and restarted from its .rst
    ends bit for bit where a job that reloads its own state at step 50 does
    (a loaded state rebuilds the lists, and list order enters the sums; the
    lanes and the overlap are fixed so that both engines sum alike)."""
    from sis_gb300 import FP64
    from sis_gb300.coil import single_chain
    from sis_gb300.dcd import read_dcd
    from sis_gb300.engine import Engine

    sysm = single_chain(sis_ff, n=24, seed=2)
    anneal = [(0, 320.0), (60, 300.0)]

    def engine():
        e = Engine(sysm, precision=FP64, seed=4)
        e.set_lanes(2)
        e.set_overlap(False)
        e.set_force_cap(1000.0)
        return e

    quiet = dict(log=lambda s: None)
    a = engine()
    a.init_velocities()
    x0 = a.get_state(0)
    a.set_state(0, *x0)
    c50 = MdControl(nstep=50, nstep_save=20, nstep_save_rst=50, anneal=anneal)
    assert MdJob(a, str(tmp_path / "a"), c50, **quiet).run() == "end"
    ra = read_rst(tmp_path / "a.rst")
    assert ra.step == 50 and ra.ianneal == 1
    a.set_state(0, *a.get_state(0))
    c = MdControl(nstep=100, nstep_save=20, nstep_save_rst=50, anneal=anneal)
    assert MdJob(a, str(tmp_path / "a2"), c, restart=ra, **quiet).run() == "end"
    assert list(read_out(tmp_path / "a.out")["nframe"]) == [0, 20, 40]
    cols = read_out(tmp_path / "a2.out")
    assert list(cols["nframe"]) == [60, 80, 100]
    assert list(cols["T"]) == [300.0, 300.0, 300.0]
    assert list(read_out(tmp_path / "a.out")["T"]) == [320.0, 320.0, 320.0]
    frames, _ = read_dcd(tmp_path / "a2.dcd")
    assert frames.shape == (3, 24, 3)
    assert np.allclose(frames[-1], a.get_state(0)[0], atol=1e-4)
    # stopped at 50 by a STOP_SIS file, then restarted in a fresh context
    (tmp_path / "b").mkdir()
    b = engine()
    b.set_state(0, *x0)
    (tmp_path / "b" / "STOP_SIS").write_text("")
    cb = MdControl(nstep=100, nstep_save=20, nstep_save_rst=50, nstep_check_stop=50, anneal=anneal)
    assert MdJob(b, str(tmp_path / "b" / "b"), cb, **quiet).run() == "stop_file"
    os.remove(tmp_path / "b" / "STOP_SIS")
    r = read_rst(tmp_path / "b" / "b.rst")
    assert r.step == 50 and r.ianneal == 1
    assert np.array_equal(r.xyz[1], ra.xyz[1]) and np.array_equal(r.velos[1], ra.velos[1])
    b2 = engine()
    restart_engine(b2, tmp_path / "b" / "b.rst")
    assert MdJob(b2, str(tmp_path / "b" / "b2"), cb, restart=r, **quiet).run() == "end"
    assert list(read_out(Path(tmp_path / "b" / "b2.out"))["nframe"]) == [60, 80, 100]
    for u, w in zip(a.get_state(0), b2.get_state(0)):
        assert np.array_equal(u, w)


def test_replicas_must_start_on_rungs():
    with pytest.raises(ValueError, match="not rungs"):
        MdJob(FakeEngine(n_inst=2, temps=[300.0, 305.0]), "x", MdControl(nstep=10, nstep_save=5),
              replica_temps=[300.0, 310.0])


def test_restart_files_keep_the_noise_key(tmp_path):
    """With an engine that has a Philox key, every replica's .rst holds the
    key and that replica's stream, and restart_engine checks them."""
    eng = FakeEngine(n_inst=2, temps=[300.0, 310.0])
    eng.seed, eng.streams = 77, [5, 9]
    MdJob(eng, str(tmp_path / "md"), MdControl(nstep=20, nstep_save=10), log=lambda s: None).run()
    assert read_rst(tmp_path / "md_0001.rst").noise == {1: (77, 5)}
    assert read_rst(tmp_path / "md_0002.rst").noise == {2: (77, 9)}
    other = FakeEngine(n_inst=2)
    other.seed, other.streams = 77, [5, 9]
    restart_engine(other, tmp_path / "md_0002.rst", inst=1, grep=2)
    other.streams = [5, 5]
    with pytest.raises(ValueError, match="noise key"):
        restart_engine(other, tmp_path / "md_0002.rst", inst=1, grep=2)
