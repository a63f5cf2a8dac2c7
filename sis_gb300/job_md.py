"""The MD job around an Engine: the loop control of job_md.F90.

The reference's main loop (src/job_md.F90:360-680) takes one step at a time
and, after each, checks a row of intervals: frames to .out/.bp/.bpall/.bpe/
.dcd every ``nstep_save`` (:462-507), the replica label table every
``nstep_rep_save`` and an exchange every ``nstep_rep_exchange`` (:509-560),
the next annealing stage (:597-611) and timed Rg-bias stage (:613-627), a
progress line every ``[Progress] step`` (:629-635, progress.F90), a
``STOP_SIS`` file beside the output prefix and the wall-clock limit every
``nstep_check_stop`` (:637-654), and a restart file every ``nstep_save_rst``
or when it stops (:659-676).  :class:`MdJob` does the same checks, but runs
the steps between two of these events as one ``Engine.step`` call, so the
device runs whole captured step graphs and the host only wakes at the steps
where the reference would do something.

File names follow init_out_files.F90:59-139: ``prefix.out`` etc. for one
instance, ``prefix_0001.out`` ... (replica number + 10**4, last four digits)
for several, and ``prefix.rep`` / ``prefix.twz``.
"""
from __future__ import annotations

import os
import queue
import threading
import time
from dataclasses import dataclass
from typing import Callable, Optional, Sequence, Tuple

import numpy as np

from . import dcd
from .outputs import (BpeFile, BpFile, OutFile, RepFile, Restart, TwzFile, fortran_f, fortran_g, fortran_i,
                      write_rst)

# const.F90 FILENAME_DIGIT_REPLICA
FILENAME_DIGIT_REPLICA = 4

STOP_END, STOP_FILE, STOP_WALL = "end", "stop_file", "wall_time"


@dataclass
class MdControl:
    """The [MD] and [Replica] settings the loop uses (read_input.F90:380-440)."""
    nstep: int
    nstep_save: int
    nstep_save_rst: Optional[int] = None  # default: nstep_save (read_input.F90:391)
    nstep_check_stop: int = 10000  # read_input.F90:431
    stop_wall_time_hour: float = -1.0  # < 0: no limit (read_input.F90:417-428)
    nstep_rep_exchange: int = 0  # 0: no exchange
    nstep_rep_save: int = 0
    anneal: Optional[Sequence[Tuple[int, float]]] = None  # (step, tempK) rows, read_anneal.F90
    timed_bias_rg: Optional[Sequence[Tuple[int, float, float]]] = None  # (step, k, rg0) rows
    out_bp: bool = True
    out_bpall: bool = False
    out_bpe: bool = False
    out_dcd: bool = True
    out_rst: bool = True
    out_twz: bool = False
    fix_com_origin: bool = False
    step_progress: int = 0  # [Progress] step; 0: no progress lines

    def __post_init__(self):
        if self.nstep < 0 or self.nstep_save <= 0 or self.nstep_check_stop <= 0:
            raise ValueError("nstep >= 0, nstep_save > 0 and nstep_check_stop > 0 are required")
        if self.nstep_save_rst is None:
            self.nstep_save_rst = self.nstep_save
        if self.nstep_save_rst <= 0:
            raise ValueError("nstep_save_rst must be positive")
        if self.step_progress < 0:
            raise ValueError("step_progress must be >= 0")
        if self.anneal is not None:
            if len(self.anneal) == 0:
                raise ValueError("an annealing schedule needs at least one row")
            if any(s < 0 or t <= 0.0 for s, t in self.anneal):
                raise ValueError("annealing rows need step >= 0 and tempK > 0")
        if self.timed_bias_rg is not None:
            if len(self.timed_bias_rg) == 0:
                raise ValueError("a timed Rg-bias schedule needs at least one row")
            if any(s < 0 or k < 0.0 or r0 <= 0.0 for s, k, r0 in self.timed_bias_rg):
                raise ValueError("timed Rg-bias rows need step >= 0, k >= 0 and rg0 > 0")


class _Writer:
    """Runs the file writes of a job in order, on one host thread (or
    inline).  At most ``depth`` writes wait, so a slow disk holds the steps
    back instead of filling memory.  The first write that fails stops the
    others and is raised by the next ``put`` or by ``close``."""

    def __init__(self, threaded: bool, depth: int = 8):
        self.err: Optional[BaseException] = None
        self.q: Optional[queue.Queue] = queue.Queue(maxsize=depth) if threaded else None
        if self.q is not None:
            self.t = threading.Thread(target=self._run, name="md-writer", daemon=True)
            self.t.start()

    def _run(self):
        while True:
            fn = self.q.get()
            if fn is None:
                return
            if self.err is None:
                try:
                    fn()
                except BaseException as e:  # noqa: BLE001 - handed to the caller
                    self.err = e

    def put(self, fn: Callable[[], None]):
        if self.err is not None:
            raise self.err
        if self.q is None:
            fn()
        else:
            self.q.put(fn)

    def close(self):
        if self.q is not None:
            self.q.put(None)
            self.t.join()
            self.q = None
        if self.err is not None:
            raise self.err


def _next_multiple(istep: int, n: int) -> int:
    return (istep // n + 1) * n


class MdJob:
    """Runs ``control.nstep`` steps of every instance of an Engine and
    writes the reference's output files under ``prefix``; messages and
    progress lines go to ``log``.

    ``replica_temps``: the temperature ladder of replica exchange (one rung
    per instance, by label; ``Engine.remd_init`` is called with it).
    ``restart``: the Restart the engine was loaded from (outputs.read_rst and
    restart_engine); a restarted job writes no frame at its first step and
    resumes the annealing stage and the replica labels the file holds.
    ``reset_step`` starts the step count at 0 whatever the file holds.
    ``clock``: wall-clock seconds
    (time.monotonic), measured from the job's construction.  The optional
    .out columns and the .twz file follow the terms set on the engine.
    With ``threaded_writer`` the files are formatted and written on a host
    thread while the device takes the next steps (the values are read from
    the device first, at the step they belong to)."""

    def __init__(self, eng, prefix: str, control: MdControl, replica_temps: Optional[Sequence[float]] = None,
                 restart: Optional[Restart] = None, reset_step: bool = False,
                 clock: Callable[[], float] = time.monotonic, log: Callable[[str], None] = print,
                 threaded_writer: bool = True):
        self.eng, self.prefix, self.c = eng, str(prefix), control
        self.threaded_writer = threaded_writer
        self.clock, self.log = clock, log
        self.t0 = clock()
        self.n_inst = eng.n_inst
        self.restart = restart
        self.replica = replica_temps is not None
        if self.replica:
            self.temps = [float(t) for t in replica_temps]
            if restart is not None and restart.rep2lab is not None:
                # read_rst.F90 REPLICA block: every replica resumes at its label's rung
                if sorted(restart.rep2lab) != list(range(1, self.n_inst + 1)):
                    raise ValueError("the restart file's replica table does not match the instances")
                for k, lab in enumerate(restart.rep2lab):
                    inst = eng.system.instances[k]
                    eng.set_condition(k, self.temps[lab - 1], inst.ionic_strength)
            off = [float(i.tempK) for i in eng.system.instances if float(i.tempK) not in self.temps]
            if off:
                raise ValueError(f"every replica must start on a rung of replica_temps; {off} are not rungs")
            eng.remd_init(self.temps)
            self.labels = [self.temps.index(float(i.tempK)) for i in eng.system.instances]
        elif self.c.nstep_rep_exchange > 0:
            raise ValueError("replica exchange needs replica_temps")
        if reset_step:
            eng.set_step(0)
        self.istep = eng.get_step()
        self.n_exchange = 0
        self.n_accepted = 0
        # the wall time of read_input.F90:427 is whole seconds
        self.stop_wall_sec = int(self.c.stop_wall_time_hour * 3600.0) if self.c.stop_wall_time_hour > 0 else -1
        d = os.path.dirname(self.prefix)
        self.stop_file = os.path.join(d, "STOP_SIS") if d else "STOP_SIS"
        self._files_open = False

    # ------------------------------------------------------------- files
    def base(self, inst: int) -> str:
        if self.n_inst > 1 or self.replica:
            crep = str(inst + 1 + 10 ** FILENAME_DIGIT_REPLICA)
            return f"{self.prefix}_{crep[-FILENAME_DIGIT_REPLICA:]}"
        return self.prefix

    def _open(self):
        c, eng = self.c, self.eng
        terms = eng.optional_terms()
        if c.timed_bias_rg is not None:
            terms["rg"] = True
        flags = dict(ele=bool(eng.system.opts.flg_ele), **terms)
        self.out = [OutFile(self.base(k) + ".out", replica=self.replica, **flags) for k in range(self.n_inst)]
        self.bp = [BpFile(self.base(k) + ".bp") if c.out_bp else None for k in range(self.n_inst)]
        self.bpall = [BpFile(self.base(k) + ".bpall", all_formed=True) if c.out_bpall else None
                      for k in range(self.n_inst)]
        self.bpe = [BpeFile(self.base(k) + ".bpe") if c.out_bpe else None for k in range(self.n_inst)]
        self.dcd = []
        for k in range(self.n_inst):
            if c.out_dcd:
                f = open(self.base(k) + ".dcd", "wb")
                dcd.write_header(f, eng.nmp(k), self._box(k) is not None)
                self.dcd.append(f)
            else:
                self.dcd.append(None)
        self.rep = RepFile(self.prefix + ".rep") if self.replica else None
        fr_any = any(len(eng.tweezers(k)[1]) for k in range(self.n_inst))
        self.twz = TwzFile(self.prefix + ".twz") if c.out_twz and fr_any else None
        self.writer = _Writer(self.threaded_writer)
        self._files_open = True

    def close(self):
        """Waits for the writer, then closes every file; a write that failed
        in the writer is raised here."""
        if not self._files_open:
            return
        try:
            self.writer.close()
        finally:
            for group in (self.out, self.bp, self.bpall, self.bpe, self.dcd):
                for w in group:
                    if w is not None:
                        w.close()
            for w in (self.rep, self.twz):
                if w is not None:
                    w.close()
            self._files_open = False

    # ---------------------------------------------------------- helpers
    def _box(self, inst: int):
        return self.eng.system.instances[inst].box

    def temp_of(self, inst: int) -> float:
        if self.replica:
            return self.temps[self.labels[inst]]
        return float(self.eng.system.instances[inst].tempK)

    def save_frames(self):
        """job_md.F90:487-507: energies, then .out, .bp files and the DCD
        frame of every instance.  The device values are read here; the
        formatting and writing go to the writer."""
        eng, step = self.eng, self.istep
        xyz = eng.get_state(-1)[0] if self.c.out_dcd else None
        rows = []
        for k in range(self.n_inst):
            tK = self.temp_of(k)
            e = eng.energy_sumup(k, tK)
            rg = float(eng.rg(k)[0]) if self.out[k].rg else 0.0
            label = self.labels[k] + 1 if self.replica else None
            bp = None
            if self.bp[k] is not None or self.bpall[k] is not None or self.bpe[k] is not None:
                bp = (eng.get_list(k, 2), eng.get_bp_status(k), eng.get_bp_energies(k))
            rows.append((tK, e, eng.energy_kinetic(k), rg, label, bp))
        o = eng.offsets

        def write():
            for k, (tK, e, ekin, rg, label, bp) in enumerate(rows):
                self.out[k].write(step, tK, ekin, e, rep_label=label, rg=rg)
                if bp is not None:
                    for w in (self.bp[k], self.bpall[k], self.bpe[k]):
                        if w is not None:
                            w.write_frame(*bp, tK)
                if self.dcd[k] is not None:
                    dcd.write_frame(self.dcd[k], xyz[o[k]:o[k + 1]], self._box(k), self.c.fix_com_origin)

        self.writer.put(write)

    def write_restart(self):
        eng, step = self.eng, self.istep
        x, v, a = eng.get_state(-1)
        o = eng.offsets
        rep2lab = [lab + 1 for lab in self.labels] if self.replica else None
        ianneal = self.ianneal if self.anneal_on else None
        boxes = [self._box(k) for k in range(self.n_inst)]
        # write_rst.F90:98-111: the force-ramp traps' starting positions
        twz = [np.array([t.init for t in eng.tweezers(k)[1]], dtype=np.float64).reshape(-1, 2, 3)
               for k in range(self.n_inst)]
        noise = [(eng.seed, eng.streams[k]) if hasattr(eng, "seed") else None for k in range(self.n_inst)]

        def write():
            for k in range(self.n_inst):
                s = slice(o[k], o[k + 1])
                write_rst(self.base(k) + ".rst", step, x[s], v[s], a[s], grep=k + 1, box=boxes[k],
                          rep2lab=rep2lab if k == 0 else None, ianneal=ianneal, twz_init=twz[k], noise=noise[k])

        self.writer.put(write)

    def write_twz(self, step: int):
        """The .twz lines the reference writes from the force evaluation of
        ``step``: beads where that step starts, traps at ``step``."""
        if self.twz is None:
            return
        x = self.eng.get_state(-1)[0]
        o = self.eng.offsets
        fr = [list(self.eng.tweezers(k)[1]) for k in range(self.n_inst)]

        def write():
            for k in range(self.n_inst):
                if fr[k]:
                    self.twz.write(step, x[o[k]:o[k + 1]], fr[k], self._box(k))

        self.writer.put(write)

    # ----------------------------------------------------------- progress
    def _progress_init(self):
        """progress.F90 progress_init: the header of the progress lines."""
        for line in ("# PROGRESS", "#1: step", "#2: million steps / day (latest cycle)",
                     "#3: million steps / day (averaged)", "#4: remaining time / hours"):
            self.log(line)
        self._p_ini = self._p_pre = (self.istep, self.clock())

    def _progress_update(self):
        """progress.F90 progress_update: ``(i12,1x,g13.6,1x,g13.6,1x,f6.1)``
        of the step, million steps per day since the previous line and since
        the start, and the hours left at the average rate."""
        now = self.clock()
        day = 86400.0

        def rate(ref):
            dt = (now - ref[1]) / day
            return (self.istep - ref[0]) / 1.0e6 / dt if dt > 0 else float("inf")

        r_pre, r_ini = rate(self._p_pre), rate(self._p_ini)
        left = (self.c.nstep - self.istep) / 1.0e6 / r_ini * 24.0 if r_ini > 0 else float("inf")
        self.log(fortran_i(self.istep, 12) + " " + fortran_g(r_pre) + " " + fortran_g(r_ini) + " "
                 + fortran_f(left, 6, 1))
        self._p_pre = (self.istep, now)

    # ---------------------------------------------------------- schedules
    def _setup_condition(self):
        """main.F90:97: with an annealing schedule the run is set up at the
        first stage's temperature, electrostatics (set_ele) included; the
        later stages move only the noise and base-pair temperatures."""
        sch = self.c.anneal
        if sch is None:
            return
        if self.replica:
            raise ValueError("an annealing schedule does not work with replica exchange")
        for k, inst in enumerate(self.eng.system.instances):
            self.eng.set_condition(k, sch[0][1], inst.ionic_strength)

    def _setup_anneal(self):
        """job_md.F90:206-230: the stage the run starts in."""
        sch = self.c.anneal
        self.anneal_on = sch is not None  # opt_anneal > 0
        self.ianneal = 1
        self.next_anneal = None
        if sch is None:
            return
        n = len(sch)
        if self.istep >= sch[-1][0]:
            self.ianneal = n
            self.anneal_on = False
        elif self.restart is not None and self.restart.ianneal is not None:
            self.ianneal = int(self.restart.ianneal)
            if not 1 <= self.ianneal <= n:
                raise ValueError(f"the restart file's annealing stage {self.ianneal} is not in the schedule")
        self.eng.set_temperature(-1, sch[self.ianneal - 1][1])
        if self.ianneal < n:
            self.next_anneal = sch[self.ianneal][0]

    def _setup_timed_rg(self):
        """job_md.F90:232-265: the timed Rg-bias stage the run starts in."""
        sch = self.c.timed_bias_rg
        self.itrg = 1
        self.next_trg = None
        if sch is None:
            return
        if self.replica:
            raise ValueError("a timed Rg bias does not work with replica exchange")
        n = len(sch)
        if self.istep >= sch[-1][0]:
            self.itrg = n
        elif self.restart is not None:
            while self.itrg < n and sch[self.itrg][0] <= self.istep:
                self.itrg += 1
        cur = self.eng.rg_bias(0)
        self.rg_flat = bool(cur[2]) if cur is not None else False
        _, k, r0 = sch[self.itrg - 1]
        self.eng.set_rg_bias(-1, k, r0, flat=self.rg_flat)
        if self.itrg < n:
            self.next_trg = sch[self.itrg][0]

    # ---------------------------------------------------------------- run
    def _next_event(self) -> int:
        c, i = self.c, self.istep
        cand = [c.nstep, _next_multiple(i, c.nstep_save), _next_multiple(i, c.nstep_check_stop),
                _next_multiple(i, c.nstep_save_rst)]
        if self.twz is not None:
            # the step before a save step, for the .twz record of that step
            cand.append(_next_multiple(i + 1, c.nstep_save) - 1)
        if c.step_progress > 0:
            cand.append(_next_multiple(i, c.step_progress))
        if self.replica and c.nstep_rep_exchange > 0:
            cand.append(_next_multiple(i, c.nstep_rep_exchange))
            if c.nstep_rep_save > 0:
                cand.append(_next_multiple(i, c.nstep_rep_save))
        for nxt in (self.next_anneal, self.next_trg):
            if nxt is not None and nxt - 1 > i:
                cand.append(nxt - 1)
        return min(v for v in cand if v > i)

    def _check_stop(self) -> Optional[str]:
        if os.path.exists(self.stop_file):
            return STOP_FILE
        if self.stop_wall_sec > 0 and self.clock() - self.t0 > self.stop_wall_sec:
            return STOP_WALL
        return None

    def run(self) -> str:
        """Steps to control.nstep or until a stop condition; returns
        ``"end"``, ``"stop_file"`` or ``"wall_time"``."""
        c, eng = self.c, self.eng
        self._setup_condition()
        # job_md.F90:195-199: every replica's lists are built as the job starts
        eng.neighbor_list(-1)
        self._setup_anneal()
        self._setup_timed_rg()
        self._open()
        try:
            if self.restart is None:
                # job_md.F90:332-338: the frame of step 0
                self.save_frames()
            if c.step_progress > 0:
                self._progress_init()
            why = STOP_END
            while self.istep < c.nstep:
                if self.twz is not None and (self.istep + 1) % c.nstep_save == 0:
                    self.write_twz(self.istep + 1)
                nxt = self._next_event()
                eng.step(nxt - self.istep)
                self.istep = nxt
                i = self.istep
                if i % c.nstep_save == 0:
                    self.save_frames()
                if self.replica and c.nstep_rep_exchange > 0:
                    if c.nstep_rep_save > 0 and i % c.nstep_rep_save == 0:
                        labs = [lab + 1 for lab in self.labels]
                        self.writer.put(lambda i=i, labs=labs: self.rep.write(i, labs))
                    if i % c.nstep_rep_exchange == 0:
                        r2l, acc = eng.remd_exchange(self.n_exchange % 2)
                        self.labels = [int(v) for v in r2l]
                        self.n_exchange += 1
                        self.n_accepted += acc
                if self.next_anneal is not None and i + 1 == self.next_anneal:
                    self.ianneal += 1
                    eng.set_temperature(-1, c.anneal[self.ianneal - 1][1])
                    if self.ianneal < len(c.anneal):
                        self.next_anneal = c.anneal[self.ianneal][0]
                    else:
                        self.next_anneal = None
                        self.anneal_on = False
                if self.next_trg is not None and i + 1 == self.next_trg:
                    self.itrg += 1
                    _, k, r0 = c.timed_bias_rg[self.itrg - 1]
                    eng.set_rg_bias(-1, k, r0, flat=self.rg_flat)
                    self.next_trg = c.timed_bias_rg[self.itrg][0] if self.itrg < len(c.timed_bias_rg) else None
                if c.step_progress > 0 and i % c.step_progress == 0:
                    self._progress_update()
                stop = self._check_stop() if i % c.nstep_check_stop == 0 else None
                if c.out_rst and (i % c.nstep_save_rst == 0 or stop):
                    self.write_restart()
                if stop:
                    why = stop
                    if stop == STOP_FILE:
                        self.log(f"STOP_SIS file was found at step {i:13d}. Stop the job.")
                    else:
                        self.log(f"Wall-clock time limit reached at step {i:13d}. Stop the job.")
                    break
            return why
        finally:
            self.close()
