"""The force check of job_check_force.F90: forces against the central
difference of the total energy, bead by bead.

The reference jitters the structure by up to ``small`` per coordinate, takes
``force``, then moves each coordinate by +/-``small`` in turn and calls
``energy_sumup`` twice, 6 N serial energy evaluations.  Here the 6 N
displaced copies are instances of one context (in batches of at most
``max_beads`` beads), so their lists and energies are built in the same
launches; the forces come from one more context holding the jittered
structure.  The report lines are the reference's
(job_check_force.F90:64-76).
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence, TextIO, Tuple

import numpy as np

from .engine import Engine
from .model import FP64, Instance, System
from .outputs import ENE_TOTAL, fortran_f, fortran_g, fortran_i


def _engine(system: System, xyz_list, precision: int, setup: Optional[Callable[[Engine], None]]) -> Engine:
    i0 = system.instances[0]
    insts = [Instance(list(i0.chains), tempK=i0.tempK, ionic_strength=i0.ionic_strength, box=i0.box, xyz=x,
                      has_charge=i0.has_charge) for x in xyz_list]
    eng = Engine(System(system.ff, system.opts, insts), precision=precision)
    if setup is not None:
        setup(eng)
    eng.neighbor_list(-1)
    return eng


def check_force(system: System, small: float = 0.001, jitter: Optional[np.ndarray] = None, seed: int = 0,
                precision: int = FP64, setup: Optional[Callable[[Engine], None]] = None,
                out: Optional[TextIO] = None, log: Callable[[str], None] = print,
                max_beads: int = 2_000_000) -> Tuple[np.ndarray, np.ndarray]:
    """(f_energy, f_force), both (nmp, 3), for the first instance of
    ``system`` (its xyz).  ``jitter``: the (nmp, 3) uniforms in (0, 1) that
    scale ``small`` for the initial displacement (the reference draws them
    with genrand_double3); by default a seeded numpy stream.  ``setup`` is
    called on every engine made (optional terms, lanes).  Per bead the two
    report lines go to ``out``; beads whose difference exceeds ``small`` in
    any coordinate are also passed to ``log``."""
    inst = system.instances[0]
    x = np.asarray(inst.xyz, dtype=np.float64).copy()
    n = x.shape[0]
    if jitter is None:
        rng = np.random.default_rng(seed)
        jitter = rng.random((n, 3))
        jitter[jitter == 0.0] = 0.5
    x += small * np.asarray(jitter, dtype=np.float64).reshape(n, 3)

    eng = _engine(system, [x], precision, setup)
    try:
        f_force = eng.force(0)
    finally:
        eng.close()

    # displaced copies: (bead, axis, sign) in the reference's loop order
    e_tot = np.empty((n, 3, 2))
    per = max(1, int(max_beads) // max(n, 1))
    jobs = [(i, a, s) for i in range(n) for a in range(3) for s in (0, 1)]
    for c0 in range(0, len(jobs), per):
        chunk = jobs[c0:c0 + per]
        frames = []
        for i, a, s in chunk:
            y = x.copy()
            y[i, a] = x[i, a] + (small if s == 0 else -small)
            frames.append(y)
        eng = _engine(system, frames, precision, setup)
        try:
            for k, (i, a, s) in enumerate(chunk):
                e_tot[i, a, s] = eng.energy_sumup(k)[ENE_TOTAL]
        finally:
            eng.close()
    f_energy = -(e_tot[:, :, 0] - e_tot[:, :, 1]) / (2.0 * small)

    if out is not None:
        out.write("".join(line + "\n" for line in check_force_lines(f_energy, f_force)))
    for i in range(n):
        diff = f_energy[i] - f_force[i]
        if np.any(np.abs(diff) > small):
            # job_check_force.F90:74-76, to the terminal
            log("f_energy - f_force " + fortran_i(i + 1, 6) + "".join(" " + fortran_f(v, 11, 4) for v in diff))
    return f_energy, f_force


def check_force_lines(f_energy: np.ndarray, f_force: np.ndarray) -> Sequence[str]:
    """The two report lines per bead as the reference writes them to .out."""
    lines = []
    for i in range(f_energy.shape[0]):
        diff = f_energy[i] - f_force[i]
        lines.append("imp=" + fortran_i(i + 1, 6) + "  f_energy" + "".join(" " + fortran_g(v, 11, 4) for v in f_energy[i])
                     + "  f_force=" + "".join(" " + fortran_g(v, 11, 4) for v in f_force[i]))
        lines.append("f_energy - f_force" + fortran_i(i + 1, 6) + "".join(fortran_f(v, 11, 4) for v in diff))
    return lines
